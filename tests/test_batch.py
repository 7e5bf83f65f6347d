"""Batched boxes (lbm_batch_*): one persistent stream + collide kernel for
boxes of different sizes, per-box forcing and particles, graph replay.

A box must give the same bits in any batch (the per-node arithmetic is the
same and every reduction has a fixed order), the graph replay must equal
direct launches, and the batched FP32 path stays within the FP32-shifted
contract of the FP64 oracle."""

import numpy as np
import pytest

from conftest import relerr
from test_gpu_parity import TOL32, make_pair

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import inputs

pytestmark = pytest.mark.gpu


def make_box(n, npart, rad, seed, precision=capi.LBM_PREC_F32, preset=capi.LBM_PRESET_BOX,
             shape=None):
    from multiphase_flow_codes_gb300.engine import LBMBox
    nx, ny, nz = shape or (n, n, n)
    cfg = capi.config_init(preset, nx, ny, nz, npart, rad, 2.5)
    cfg.precision = precision
    box = LBMBox(cfg)
    u = inputs.spectral_velocity(nx, 4.0, 0.03, seed=seed, ny=ny, nz=nz)
    box.initpop(*u)
    box.macrovar()
    if npart:
        box.release_particles(inputs.initpartpos(nx, ny, nz, npart, rad, seed=seed + 1,
                                                 channel=preset == capi.LBM_PRESET_CHANNEL))
    return box


SPECS = [(32, 2, 3.5, 101), (48, 3, 4.0, 202), (64, 0, 4.0, 303), (36, 1, 3.0, 404)]


def run_batch(specs, steps, graph, schedule=None):
    from multiphase_flow_codes_gb300.engine import LBMBatch
    boxes = [make_box(*s) for s in specs]
    with LBMBatch(boxes) as b:
        if schedule:
            b.set_schedule(*schedule)
        b.step(steps, graph=graph)
        b.synchronize()
    out = [(bx.get_f(), bx.get_particles()) for bx in boxes]
    for bx in boxes:
        bx.close()
    return out


def test_batch_same_as_alone_and_graph_same_as_direct(require_gpu):
    together = run_batch(SPECS, 13, graph=True)
    direct = run_batch(SPECS, 13, graph=False)
    for (f1, p1), (f2, p2) in zip(together, direct):
        assert np.array_equal(f1, f2)
        assert np.array_equal(p1["ypglb"], p2["ypglb"]) and np.array_equal(p1["fHIp"], p2["fHIp"])
    for spec, (f, p) in zip(SPECS, together):
        alone = run_batch([spec], 13, graph=True)[0]
        assert np.array_equal(alone[0], f)
        assert np.array_equal(alone[1]["fHIp"], p["fHIp"])


@pytest.mark.parametrize("schedule", [(2, 1, 1), (4, 2, 0), (8, 4, 0), (6, 2, 2)])
def test_batch_schedules_agree(require_gpu, schedule):
    ref = run_batch(SPECS[:2], 7, graph=False, schedule=(2, 1, 0))
    got = run_batch(SPECS[:2], 7, graph=False, schedule=schedule)
    for (f1, _), (f2, _) in zip(ref, got):
        assert np.array_equal(f1, f2)


def test_batch_box_close_to_standalone_step(require_gpu):
    """Batched and standalone FP32 kernels differ only in rounding."""
    spec = SPECS[1]
    alone = make_box(*spec)
    alone.step(8)
    f_alone = alone.get_f()
    alone.close()
    f_batch = run_batch([spec, SPECS[0]], 8, graph=True)[0][0]
    assert relerr(f_batch, f_alone) <= 1e-5


def test_batch_fp32_within_contract_of_oracle(require_gpu, oracle_mod):
    from multiphase_flow_codes_gb300.engine import LBMBatch
    o, box = make_pair(oracle_mod, shape=(32, 32, 32), npart=2, rad=4.0, rhopart=2.5,
                       precision=capi.LBM_PREC_F32)
    other = make_box(*SPECS[1])
    with LBMBatch([box, other]) as b:
        b.step(10, graph=True)
        b.synchronize()
    o.step(10)
    assert relerr(box.get_f(), o.f) <= TOL32


def test_batch_channel(require_gpu, oracle_mod):
    from multiphase_flow_codes_gb300.engine import LBMBatch
    o, box = make_pair(oracle_mod, preset=capi.LBM_PRESET_CHANNEL, shape=(24, 20, 16), npart=2,
                       rad=3.5, rhopart=1.0, precision=capi.LBM_PREC_F32)
    other = make_box(0, 0, 4.0, 7, preset=capi.LBM_PRESET_CHANNEL, shape=(32, 24, 20))
    with LBMBatch([box, other]) as b:
        b.step(6, graph=True)
        b.synchronize()
    o.step(6)
    assert relerr(box.get_f(), o.f) <= TOL32


def test_batch_rejects(require_gpu):
    from multiphase_flow_codes_gb300 import LBMError
    from multiphase_flow_codes_gb300.engine import LBMBatch
    a = make_box(32, 0, 4.0, 1)
    b64 = make_box(32, 0, 4.0, 2, precision=capi.LBM_PREC_F64)
    with pytest.raises(LBMError):
        LBMBatch([a, b64])
    big = make_box(0, 0, 4.0, 3, shape=(136, 8, 8))
    with pytest.raises(LBMError):
        LBMBatch([a, big])
    c = make_box(32, 0, 4.0, 4)
    c.step(1)                      # one step ahead of a
    with LBMBatch([a, c]) as bt:
        with pytest.raises(LBMError):
            bt.step(1)
    with pytest.raises(LBMError):
        LBMBatch([a, a])


def test_batch_forcing_state_follows_the_steps(require_gpu):
    """The forcing that a batch runs one step ahead is invisible from outside
    and undone when the batch ends: a box stepped 8 times in a batch and 4
    more alone equals the same box stepped 12 times alone."""
    from multiphase_flow_codes_gb300.engine import LBMBatch
    ref = make_box(*SPECS[0])
    ref.step(12)
    a = make_box(*SPECS[0])
    other = make_box(*SPECS[2])
    with LBMBatch([a, other]) as b:
        b.step(8, graph=True)
        b.synchronize()
        s_in = a.get_forcing_state()
    a.step(4)
    assert relerr(a.get_f(), ref.get_f()) <= 1e-5
    s_out = a.get_forcing_state()
    s_ref = ref.get_forcing_state()
    assert s_out[0] == s_ref[0] and s_out[1] == s_ref[1]
    assert np.array_equal(s_out[2], s_ref[2])
    r8 = make_box(*SPECS[0])
    r8.step(8)
    s8 = r8.get_forcing_state()
    assert s_in[0] == s8[0] and s_in[1] == s8[1] and np.array_equal(s_in[2], s8[2])


def test_batch_led_by_a_box_without_particles(require_gpu):
    """Boxes with and without spheres share the flag-buffer parity."""
    specs = [SPECS[2], SPECS[0], SPECS[1]]       # first box has no particles
    together = run_batch(specs, 9, graph=True)
    for spec, (f, p) in zip(specs, together):
        alone = run_batch([spec], 9, graph=False)[0]
        assert np.array_equal(alone[0], f)
        assert np.array_equal(alone[1]["fHIp"], p["fHIp"])
