"""rmsstat and diag (B/saveload.f90:1530-1730, 1342-1400) on the device
against the numpy restatement (oracle/statistics.py), on the GPU's own
macroscopic fields and on the oracle's after the same steps."""

import numpy as np
import pytest

from conftest import relerr
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,npart", [((32, 32, 32), 3), ((36, 24, 20), 0)])
def test_rmsstat_and_diag(require_gpu, oracle_mod, shape, npart):
    from oracle import statistics as ost
    o, box = make_pair(oracle_mod, shape=shape, npart=npart, rad=4.0, rhopart=2.5, urms=0.04)
    for _ in range(3):
        o.step(1)
        box.step(1)
    rho, ux, uy, uz = box.get_macro()
    _, isn = box.get_flags()
    p = box.get_particles()
    wp = p["wp"] if npart else None
    om = p["omgp"] if npart else None
    got = np.array(list(box.rmsstat().values()))
    want = ost.rmsstat(ux, uy, uz, isn, wp, om)
    assert got[0] == want[0]                      # fluid node count, exact
    assert np.allclose(got, want, rtol=1e-11, atol=1e-13)
    if npart:
        assert np.abs(got[10:18]).max() > 0       # particle columns filled
    else:
        assert np.all(got[10:18] == 0) and np.all(got[26:34] == 0)
    d = box.diag()
    dw = ost.diag(ux, uy, uz, isn, wp, om)
    assert relerr(d["vmax"], dw[0]) <= 1e-15
    assert (d["idwp"], d["idomgp"]) == (dw[1], dw[3])
    assert relerr([d["wpmax"], d["omgpmax"]], [dw[2], dw[4]]) <= 1e-15
    # the oracle's own fields after the same steps (FP64 contract)
    want_o = ost.rmsstat(np.asarray(o.ux), np.asarray(o.uy), np.asarray(o.uz),
                         np.asarray(o.isnodes), wp, om)
    assert np.allclose(got, want_o, rtol=1e-10, atol=1e-13)


@pytest.mark.parametrize("fluid_only", [False, True])
def test_channel_profiles(require_gpu, oracle_mod, fluid_only):
    from oracle import statistics as ost
    from multiphase_flow_codes_gb300 import _capi as capi
    o, box = make_pair(oracle_mod, preset=capi.LBM_PRESET_CHANNEL, shape=(32, 24, 20), npart=2,
                       rad=4.0, rhopart=1.0, urms=0.0)
    for _ in range(20):
        o.step(1)
        box.step(1)
    rho, ux, uy, uz = box.get_macro()
    _, isn = box.get_flags()
    cfg = box.cfg
    ustar = float(np.sqrt(cfg.force_y * cfg.nx / (2.0 * cfg.rho0)))
    got = box.channel_profiles(fluid_only)
    want = ost.channel_profiles(rho, ux, uy, uz, isn, ustar, cfg.visc, fluid_only)
    assert got.shape == want.shape == (32, 15 if fluid_only else 13)
    # variances and stresses are differences of mean squares: their error is
    # set by the squared means they cancel
    scale = np.abs(want).max(axis=0) + 1e-300
    usq = np.abs(want[:, 2:5]).max() ** 2
    scale[5:11] += usq
    scale[12] += np.abs(want[:, 11]).max() ** 2
    assert np.all(np.abs(got - want) <= 1e-11 * scale)
    # the same against the oracle's own fields (FP64 contract)
    want_o = ost.channel_profiles(np.asarray(o.rho), np.asarray(o.ux), np.asarray(o.uy),
                                  np.asarray(o.uz), np.asarray(o.isnodes), ustar, cfg.visc,
                                  fluid_only)
    assert np.all(np.abs(got - want_o) <= 1e-9 * scale)
    if fluid_only:
        assert np.all(got[:, 13] <= 1.0) and np.any(got[:, 13] < 1.0)
