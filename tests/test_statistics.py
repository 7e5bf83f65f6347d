"""On-device statistics (lbm_statistics, lbm_particle_slip) against the
numpy restatement of statistc in oracle/statistics.py, on the GPU's own
velocity field."""

import numpy as np
import pytest

from conftest import relerr
from test_gpu_parity import make_pair

from multiphase_flow_codes_gb300 import _capi as capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,shape", [(capi.LBM_PREC_F64, (32, 32, 32)),
                                             (capi.LBM_PREC_F32, (32, 32, 32)),
                                             (capi.LBM_PREC_F64, (40, 24, 32))])
def test_spectrum_matches_numpy(require_gpu, oracle_mod, precision, shape):
    from oracle import statistics
    _, box = make_pair(oracle_mod, shape=shape, npart=2, rad=4.0, precision=precision)
    box.step(3)
    st = box.statistics()
    _, ux, uy, uz = box.get_macro()
    ek, dk, out = statistics.spectrum(ux, uy, uz, box.cfg.visc)
    assert len(st["ek"]) == len(ek) == int(shape[0] / 2 - 1.5)
    assert relerr(st["ek"], ek) <= 1e-12
    assert relerr(st["dk"], dk) <= 1e-12
    assert abs(st["energy"] - out[1]) <= 1e-12 * out[1]
    assert abs(st["dissipation"] - out[2]) <= 1e-12 * out[2]
    assert abs(st["skewness"] - out[3]) <= 1e-9 * max(1.0, abs(out[3]))
    assert abs(st["flatness"] - out[4]) <= 1e-9 * out[4]
    # deterministic: the same state gives the same bits
    st2 = box.statistics()
    assert np.array_equal(st2["ek"], st["ek"]) and st2["skewness"] == st["skewness"]


def test_particle_slip_matches_numpy(require_gpu, oracle_mod):
    from oracle import statistics
    rng = np.random.default_rng(11)
    wp = rng.uniform(-0.02, 0.02, (3, 3))
    _, box = make_pair(oracle_mod, shape=(32, 32, 32), npart=3, rad=4.0, wp=wp)
    box.step(2)
    slip = box.particle_slip(5.0, 7.0)
    _, ux, uy, uz = box.get_macro()
    _, isn = box.get_flags()
    p = box.get_particles()
    ref = statistics.particle_slip(ux, uy, uz, isn, p["ypglb"], p["wp"], 5.0, 7.0)
    assert np.abs(slip - ref).max() <= 1e-13
