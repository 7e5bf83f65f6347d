"""GB300 lattice Boltzmann engine for particle-laden turbulence.

D3Q19 MRT with finite-size moving spheres (interpolated bounce-back,
momentum exchange, lubrication, refilling) and low-wavenumber stochastic
forcing, as hand-written CUDA kernels for sm_103a behind the C ABI of
``include/lbm.h``.  ``engine.LBMBox`` is the Python face of that ABI.

The package imports its submodules on first use, so that the seeded input
generators (``inputs``) can be used without loading the engine.
"""

from __future__ import annotations

import importlib

__all__ = ["LBMBox", "LBMError", "lbm_config"]


def __getattr__(name):
    if name == "LBMBox":
        return importlib.import_module(".engine", __name__).LBMBox
    if name in ("LBMError", "lbm_config"):
        return getattr(importlib.import_module("._capi", __name__), name)
    raise AttributeError(name)
