"""The staged stream+collide kernel (rows moved by bulk copies through shared
memory) against the direct kernel and the CPU oracle.

Both variants run the same per-node arithmetic, so FP64 results agree with
the oracle within the path's 1e-12 and with each other to rounding; the
x-row wrap, the y/z destination rows and the row ranges of the persistent
CTAs are exercised on boxes whose sides differ and are not powers of two.
"""

import numpy as np
import pytest

from conftest import relerr
from test_gpu_parity import TOL64, TOL32, make_pair

from multiphase_flow_codes_gb300 import _capi as capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,stages,ctas", [
    ((32, 32, 32), 0, 0),
    ((36, 20, 28), 2, 1),
    ((100, 12, 16), 3, 2),
    ((64, 48, 40), 4, 0),
])
def test_staged_fp64_matches_oracle(require_gpu, oracle_mod, shape, stages, ctas):
    o, box = make_pair(oracle_mod, shape=shape, npart=2 if min(shape) >= 16 else 0, rad=3.5)
    box.set_variant(capi.LBM_VARIANT_STAGED, stages, 0, ctas)
    v, s, _, c = box.variant()
    assert v == capi.LBM_VARIANT_STAGED and s >= 2 and c >= 1
    for _ in range(6):
        o.step(1)
        box.step(1)
    assert relerr(box.get_f(), o.f) <= TOL64


@pytest.mark.parametrize("precision,variant,groups", [
    (capi.LBM_PREC_F64, capi.LBM_VARIANT_STAGED, 0),
    (capi.LBM_PREC_F32, capi.LBM_VARIANT_STAGED, 0),
    (capi.LBM_PREC_F32, capi.LBM_VARIANT_STAGED_X2, 1),
])
def test_staged_equals_direct(require_gpu, oracle_mod, precision, variant, groups):
    _, a = make_pair(oracle_mod, shape=(48, 40, 32), npart=3, rad=4.0, precision=precision)
    _, b = make_pair(oracle_mod, shape=(48, 40, 32), npart=3, rad=4.0, precision=precision)
    a.set_variant(capi.LBM_VARIANT_DIRECT)
    b.set_variant(variant, 3, groups, 0)
    a.step(5)
    b.step(5)
    fa, fb = a.get_f(), b.get_f()
    tol = 1e-14 if precision == capi.LBM_PREC_F64 else 1e-6
    assert relerr(fb, fa) <= tol
    pa, pb = a.get_particles(), b.get_particles()
    assert relerr(pb["ypglb"], pa["ypglb"]) <= (1e-15 if precision == capi.LBM_PREC_F64 else 1e-9)


@pytest.mark.parametrize("stages,groups", [(2, 2), (4, 2), (4, 4), (8, 4), (6, 3)])
def test_x2_consumer_groups(require_gpu, oracle_mod, stages, groups):
    """Several rows in the collision at once: each stage stays with one group."""
    _, a = make_pair(oracle_mod, shape=(128, 24, 20), npart=2, rad=4.0,
                     precision=capi.LBM_PREC_F32)
    _, b = make_pair(oracle_mod, shape=(128, 24, 20), npart=2, rad=4.0,
                     precision=capi.LBM_PREC_F32)
    a.set_variant(capi.LBM_VARIANT_DIRECT)
    b.set_variant(capi.LBM_VARIANT_STAGED_X2, stages, groups, 0)
    assert b.variant()[:3] == (capi.LBM_VARIANT_STAGED_X2, stages, groups)
    a.step(4)
    b.step(4)
    assert relerr(b.get_f(), a.get_f()) <= 1e-6


def test_x2_rejects_ambiguous_schedules(require_gpu):
    """A stage shared by two consumer groups (stages not a multiple of groups)."""
    from multiphase_flow_codes_gb300 import LBMError
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 128, 24, 20, 0, 4.0, 1.0)
    cfg.precision = capi.LBM_PREC_F32
    box = LBMBox(cfg)
    for stages, groups in [(3, 2), (2, 4), (6, 4)]:
        with pytest.raises(LBMError):
            box.set_variant(capi.LBM_VARIANT_STAGED_X2, stages, groups, 0)


@pytest.mark.parametrize("variant,shape", [
    (capi.LBM_VARIANT_STAGED, (32, 32, 32)),
    (capi.LBM_VARIANT_STAGED_X2, (32, 32, 32)),
    (capi.LBM_VARIANT_STAGED_X2, (100, 12, 16)),
    (capi.LBM_VARIANT_STAGED_X2, (136, 16, 12)),
])
def test_staged_fp32_within_contract(require_gpu, oracle_mod, variant, shape):
    o, box = make_pair(oracle_mod, shape=shape, precision=capi.LBM_PREC_F32)
    box.set_variant(variant)
    for _ in range(10):
        o.step(1)
        box.step(1)
    assert relerr(box.get_f(), o.f) <= TOL32


def test_autotune_keeps_state(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod, shape=(64, 32, 32), npart=2, rad=3.5)
    box.step(2)
    o.step(2)
    f0 = box.get_f()
    ms = box.autotune(reps=2)
    assert ms > 0
    assert np.array_equal(box.get_f(), f0)
    v = box.variant()[0]
    assert v in (capi.LBM_VARIANT_DIRECT, capi.LBM_VARIANT_STAGED)
    box.step(3)
    o.step(3)
    assert relerr(box.get_f(), o.f) <= TOL64


@pytest.mark.parametrize("variant", [capi.LBM_VARIANT_DIRECT, capi.LBM_VARIANT_STAGED])
def test_channel_variants_match_oracle(require_gpu, oracle_mod, variant):
    """x walls: the halfway bounce-back stores of both variants."""
    o, box = make_pair(oracle_mod, preset=capi.LBM_PRESET_CHANNEL, shape=(24, 20, 16), npart=2,
                       rad=3.5, rhopart=1.0)
    box.set_variant(variant)
    for _ in range(5):
        o.step(1)
        box.step(1)
    assert relerr(box.get_f(), o.f) <= TOL64


@pytest.mark.parametrize("variant", [capi.LBM_VARIANT_DIRECT, capi.LBM_VARIANT_STAGED,
                                     capi.LBM_VARIANT_STAGED_X2])
def test_channel_fp32_variants(require_gpu, oracle_mod, variant):
    o, box = make_pair(oracle_mod, preset=capi.LBM_PRESET_CHANNEL, shape=(24, 20, 16), npart=2,
                       rad=3.5, rhopart=1.0, precision=capi.LBM_PREC_F32)
    box.set_variant(variant)
    for _ in range(5):
        o.step(1)
        box.step(1)
    assert relerr(box.get_f(), o.f) <= TOL32


def test_staged_rejected_where_it_does_not_apply(require_gpu):
    from multiphase_flow_codes_gb300 import LBMError
    from multiphase_flow_codes_gb300.engine import LBMBox
    odd = LBMBox(capi.config_init(capi.LBM_PRESET_BOX, 30, 24, 24, 0, 4.0, 1.0))
    assert odd.variant()[0] == capi.LBM_VARIANT_DIRECT
    with pytest.raises(LBMError):
        odd.set_variant(capi.LBM_VARIANT_STAGED, 2)
    with pytest.raises(LBMError):
        odd.set_variant(7)
    f64 = LBMBox(capi.config_init(capi.LBM_PRESET_BOX, 32, 24, 24, 0, 4.0, 1.0))
    with pytest.raises(LBMError):
        f64.set_variant(capi.LBM_VARIANT_STAGED_X2)
