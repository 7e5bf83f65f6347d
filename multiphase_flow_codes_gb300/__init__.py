"""GB300 lattice Boltzmann engine for particle-laden turbulence.

D3Q19 MRT with finite-size moving spheres (interpolated bounce-back,
momentum exchange, lubrication, refilling) and low-wavenumber stochastic
forcing, as hand-written CUDA kernels for sm_103a behind the C ABI of
``include/lbm.h``.  ``engine.LBMBox`` is the Python face of that ABI.
"""

from ._capi import LBMError, lbm_config  # noqa: F401
from .engine import LBMBox  # noqa: F401

__all__ = ["LBMBox", "LBMError", "lbm_config"]
