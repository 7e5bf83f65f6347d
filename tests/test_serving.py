"""The serving loop (lbm_server_*): admission by HBM footprint, continuous
batching, and the same result for a request alone and in a mix."""

import ctypes as C

import numpy as np
import pytest

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import serving

pytestmark = pytest.mark.gpu


def _run(reqs, budget=8 << 30, max_active=16, chunk=8):
    with serving.LBMServer(budget, max_active, chunk) as srv:
        ids = [srv.submit(r) for r in reqs]
        return [srv.wait(i, timeout=300.0) for i in ids]


def test_request_same_alone_and_in_mix(require_gpu):
    target = serving.request(24, 32, 20, 13, wall_axis=1, npart=3, seed=7)
    others = [serving.request(32, 24, 28, 9, wall_axis=1, npart=2, seed=8),
              serving.request(40, 16, 24, 22, wall_axis=1, npart=0, seed=9),
              serving.request(16, 32, 16, 5, wall_axis=1, npart=1, seed=10),
              serving.request(24, 24, 24, 17, wall_axis=-1, npart=2, seed=11)]
    alone = _run([target])[0]
    mixed = _run(others[:2] + [target] + others[2:], chunk=6)[2]
    assert alone.state == mixed.state == serving.REQ_DONE
    assert alone.steps_done == mixed.steps_done == 13
    assert mixed.batched == 1
    assert list(alone.summary) == list(mixed.summary)


def test_wall_axis_relabelling(require_gpu):
    """Walls normal to y are the engine's x walls with the axes relabelled."""
    a = _run([serving.request(24, 32, 20, 8, wall_axis=1, npart=2, seed=5)])[0]
    b = _run([serving.request(32, 24, 20, 8, wall_axis=0, npart=2, seed=5)])[0]
    assert a.state == b.state == serving.REQ_DONE
    sa, sb = list(a.summary), list(b.summary)
    assert sa[0] == sb[0] and sa[4] == sb[4] and sa[5] == sb[5]
    assert sa[2] == sb[1] and sa[1] == sb[2] and sa[3] == sb[3]   # momentum x <-> y


def test_admission_by_footprint(require_gpu):
    """A budget that holds one solve at a time runs them one after another."""
    reqs = [serving.request(32, 32, 32, 6, wall_axis=1, seed=s) for s in (1, 2, 3)]
    lib = capi.lib()
    cfg = capi.config_init(capi.LBM_PRESET_CHANNEL, 32, 32, 32, 0, 4.0, 1.0)
    cfg.precision = capi.LBM_PREC_F32
    fp = C.c_uint64(0)
    assert lib.lbm_footprint(C.byref(cfg), C.byref(fp)) == capi.LBM_OK
    budget = int(fp.value * 1.9) + 32 * 32 * 32 * 48
    res = _run(reqs, budget=budget)
    assert all(r.state == serving.REQ_DONE for r in res)
    for r0, r1 in zip(res, res[1:]):
        assert r1.t_start >= r0.t_done - 1e-9


def test_oversized_request_rejected(require_gpu):
    with serving.LBMServer(1 << 20, 4, 8) as srv:
        with pytest.raises(capi.LBMError):
            srv.submit(serving.request(64, 64, 64, 10))


def test_served_fields_match_standalone_and_oracle(require_gpu, oracle_mod):
    """A request served in a mix, its context kept and taken afterwards:
    its final populations and particles equal a standalone LBMBox run of the
    same request bit for bit, and agree with the FP64 oracle started from
    the same initial state within the FP32 tolerance."""
    from conftest import relerr
    from multiphase_flow_codes_gb300.engine import LBMBox
    steps, seed, npart = 12, 21, 3
    target = serving.request(24, 32, 20, steps, wall_axis=1, npart=npart, seed=seed, u_rms=0.03,
                             keep_state=True)
    others = [serving.request(32, 24, 28, 9, wall_axis=1, npart=2, seed=8),
              serving.request(24, 24, 24, 17, wall_axis=-1, npart=2, seed=11)]
    with serving.LBMServer(8 << 30, 16, 4) as srv:
        ids = [srv.submit(r) for r in others[:1] + [target] + others[1:]]
        res = [srv.wait(i, timeout=300.0) for i in ids]
        assert all(r.state == serving.REQ_DONE for r in res)
        served = srv.take(ids[1])
    assert (served.nx, served.ny, served.nz) == (32, 24, 20)  # walls normal to engine x
    f_served = served.get_f()
    p_served = served.get_particles()
    served.close()

    cfg = capi.config_init(capi.LBM_PRESET_CHANNEL, 32, 24, 20, npart, 4.0, 1.0)
    cfg.precision = capi.LBM_PREC_F32
    box = LBMBox(cfg)
    box.init_spectral(4.0, 0.03, seed)
    box.macrovar()
    box.init_particles(npart, seed=seed % 2147483646 + 1)
    f0 = box.get_f()
    y0 = box.get_particles()["ypglb"]
    box.step(steps)
    assert np.array_equal(box.get_f(), f_served)
    for k in ("ypglb", "wp", "omgp", "fHIp"):
        assert np.array_equal(box.get_particles()[k], p_served[k]), k
    box.close()

    ocfg = capi.config_init(capi.LBM_PRESET_CHANNEL, 32, 24, 20, npart, 4.0, 1.0)
    o = oracle_mod.OracleBox(ocfg)
    o.f[...] = f0
    o.macrovar()
    o.release_particles(y0)
    assert o.step(steps) == 0
    assert relerr(f_served, o.f) <= 1e-5
    assert relerr(p_served["ypglb"], o.ypglb[:npart]) <= 1e-9
