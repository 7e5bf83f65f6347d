"""Density pre-relaxation of a new run (lbm_prerelax) against the oracle.

B/main.f90:86-108 repeats collision_MRT, streaming and rhoupdat with the
velocity field held at its initial value until the density stops changing
(max |rho - rho_previous| <= rhoepsl) or the counter passes 15000.  The test
runs the same loop on the CPU oracle's per-subroutine entries and compares
the exit counter, the last difference and the populations.
"""

import numpy as np
import pytest

from conftest import relerr
from test_gpu_parity import TOL64

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import inputs

pytestmark = pytest.mark.gpu


def oracle_prerelax(o, eps, max_iter):
    istep = 0
    while True:
        o.collision_MRT()
        o.streaming()
        rhop = np.array(o.rho, copy=True)
        o.rhoupdat()
        err = float(np.abs(np.asarray(o.rho) - rhop).max())
        if err <= eps or istep > max_iter:
            return istep, err
        istep += 1


@pytest.mark.parametrize("preset,shape,urms,eps,max_iter", [
    (capi.LBM_PRESET_BOX, (32, 32, 32), 0.03, 1e-7, 400),
    (capi.LBM_PRESET_BOX, (24, 20, 28), 0.05, 1e-12, 30),     # stops on the counter
    (capi.LBM_PRESET_CHANNEL, (24, 32, 20), 0.02, 1e-7, 400),
])
def test_prerelax_matches_oracle(require_gpu, oracle_mod, preset, shape, urms, eps, max_iter):
    from multiphase_flow_codes_gb300.engine import LBMBox
    nx, ny, nz = shape
    cfg = capi.config_init(preset, nx, ny, nz, 0, 4.0, 1.0)
    u = inputs.spectral_velocity(nx, 4.0, urms, ny=ny, nz=nz, seed=77)
    if preset == capi.LBM_PRESET_CHANNEL:
        # no flow through the walls at x = 0 and x = nx
        u = (u[0] * 0.0, u[1], u[2])
    o = oracle_mod.OracleBox(cfg)
    o.initpop(*u)
    o.rhoupdat()
    box = LBMBox(cfg)
    box.initpop(*u)
    box.rhoupdat()
    it_o, err_o = oracle_prerelax(o, eps, max_iter)
    it_g, err_g = box.prerelax(eps, max_iter)
    assert it_g == it_o
    # a difference of two densities: its error is set by the densities' size
    assert abs(err_g - err_o) <= 1e-12 * float(np.abs(np.asarray(o.rho)).max())
    assert relerr(box.get_f(), o.f) <= TOL64
    rho_g = box.get_macro()[0]
    assert relerr(rho_g, o.rho) <= TOL64


def test_prerelax_at_rest_exits_at_once(require_gpu):
    """The reference's own new-run setting: u = 0, so the first difference is 0."""
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 16, 16, 16, 0, 4.0, 1.0)
    box = LBMBox(cfg)
    z = np.zeros((16, 16, 16))
    box.initpop(z, z, z)
    box.rhoupdat()
    assert box.prerelax(1e-5, 15000) == (0, 0.0)
