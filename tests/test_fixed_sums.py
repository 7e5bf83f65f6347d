"""FP64 collision with exact fixed-point moment sums (lbm_set_sums).

The fused FP64 kernels compute the integer-coefficient sums of the moment
transforms in 64-bit fixed point and keep every other operation in FP64.
These tests hold that path to the FP64 contract against the CPU oracle, to
rounding against the all-FP64 arithmetic, and exercise the nodes it hands
back to the FP64 path: populations of 1/8 and more, and (staged kernel, FP64
storage) quiescent nodes whose populations are all below 2^-12.  The direct
kernel's fused steps keep the populations in 64-bit fixed point at 2^-58:
absolute resolution 3.5e-18, the FP64 rounding of the largest deviations of
a flowing field, but absolute rather than relative for tiny deviations.
"""

import numpy as np
import pytest

from conftest import relerr
from test_gpu_parity import TOL64, make_pair

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import inputs

pytestmark = pytest.mark.gpu


def test_fp64_contexts_default_to_integer_sums(require_gpu):
    from multiphase_flow_codes_gb300 import LBMError
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 16, 16, 16, 0, 4.0, 1.0)
    box = LBMBox(cfg)
    assert box.sums() == capi.LBM_SUMS_INTEGER
    box.set_sums(capi.LBM_SUMS_FIXED)
    assert box.sums() == capi.LBM_SUMS_FIXED
    box.set_sums(capi.LBM_SUMS_FLOAT)
    assert box.sums() == capi.LBM_SUMS_FLOAT
    with pytest.raises(LBMError):
        box.set_sums(7)
    cfg.precision = capi.LBM_PREC_F32
    b32 = LBMBox(cfg)
    assert b32.sums() == capi.LBM_SUMS_FLOAT
    with pytest.raises(LBMError):
        b32.set_sums(capi.LBM_SUMS_FIXED)


@pytest.mark.parametrize("mode", [capi.LBM_SUMS_FIXED, capi.LBM_SUMS_INTEGER])
@pytest.mark.parametrize("variant", [capi.LBM_VARIANT_DIRECT, capi.LBM_VARIANT_STAGED])
@pytest.mark.parametrize("preset,shape", [
    (capi.LBM_PRESET_BOX, (48, 40, 32)),
    (capi.LBM_PRESET_CHANNEL, (32, 40, 24)),
])
def test_fixed_sums_match_oracle_and_fp64(require_gpu, oracle_mod, variant, preset, shape, mode):
    if preset == capi.LBM_PRESET_CHANNEL and variant == capi.LBM_VARIANT_STAGED:
        pytest.skip("the staged kernel serves periodic boxes")
    o, fx = make_pair(oracle_mod, preset=preset, shape=shape, npart=3, rad=4.0, rhopart=2.5)
    _, fl = make_pair(oracle_mod, preset=preset, shape=shape, npart=3, rad=4.0, rhopart=2.5)
    for b in (fx, fl):
        b.set_variant(variant)
    fl.set_sums(capi.LBM_SUMS_FLOAT)
    fx.set_sums(mode)
    assert fx.sums() == mode
    for _ in range(10):
        o.step(1)
        fx.step(1)
        fl.step(1)
    assert relerr(fx.get_f(), o.f) <= TOL64
    assert relerr(fx.get_f(), fl.get_f()) <= 1e-13
    px, pl = fx.get_particles(), fl.get_particles()
    assert relerr(px["ypglb"], pl["ypglb"]) <= 1e-14
    assert relerr(px["fHIp"], pl["fHIp"]) <= 1e-11


@pytest.mark.parametrize("variant,mode", [(capi.LBM_VARIANT_DIRECT, capi.LBM_SUMS_FIXED),
                                          (capi.LBM_VARIANT_STAGED, capi.LBM_SUMS_FIXED),
                                          (capi.LBM_VARIANT_DIRECT, capi.LBM_SUMS_INTEGER)])
def test_fixed_sums_hand_back_out_of_range_nodes(require_gpu, oracle_mod, variant, mode):
    """One half of the box moves fast enough for populations of 1/8 and
    more; the other half is at rest with a 1e-9 density ripple, all its
    populations far below 2^-12.  The fast nodes take the FP64 path in both
    kernels.  The staged kernel (FP64 storage) also hands the quiescent nodes
    to the FP64 path, which keeps FP64's relative precision there; the direct
    kernel stores them in fixed point, to a few units of its absolute
    resolution 2^-58 over three steps (bound: 2^-54)."""
    from multiphase_flow_codes_gb300.engine import LBMBox
    n = 32
    cfg = capi.config_init(capi.LBM_PRESET_BOX, n, n, n, 0, 4.0, 1.0)
    ux, uy, uz = inputs.spectral_velocity(n, 4.0, 0.25, seed=5)
    rest = np.zeros((n, n, n), dtype=bool)
    rest[: n // 2] = True
    for u in (ux, uy, uz):
        u[rest] = 0.0
    o = oracle_mod.OracleBox(cfg)
    o.initpop(ux, uy, uz)
    f0 = o.f.copy()
    # a tiny density ripple over the resting half (populations ~1e-10)
    ripple = 1e-9 * np.sin(2 * np.pi * np.arange(n) / n)[None, None, :] * rest
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    f0 = f0 + w[:, None, None, None] * ripple[None]
    assert np.abs(f0).max() >= 0.125
    boxes = []
    for m in (mode, capi.LBM_SUMS_FLOAT):
        b = LBMBox(cfg)
        b.set_f(f0.copy())
        b.macrovar()
        b.set_variant(variant)
        b.set_sums(m)
        b.step(3)
        boxes.append(b.get_f())
    fxd, fld = boxes
    assert relerr(fxd, fld) <= 1e-13
    # the resting half against its own magnitude
    far = rest.copy()
    far[: 3] = False
    far[n // 2 - 3: n // 2] = False
    a, b = fxd[:, far], fld[:, far]
    assert np.abs(b).max() > 0
    if variant == capi.LBM_VARIANT_STAGED:
        assert relerr(a, b) <= 1e-13
    else:
        assert np.abs(a - b).max() <= 2.0 ** -54


def test_force_cache_across_mixed_steps(require_gpu, oracle_mod):
    """The FP64 direct kernel keeps each step's body force per node for the
    next step's velocity.  Steps through other paths in between (the unfused
    subroutines, the staged kernel, a timing run of the autotuner) must leave
    no stale field behind: the run stays on the oracle's trajectory."""
    o, box = make_pair(oracle_mod, shape=(40, 32, 36), npart=2, rad=4.0, rhopart=2.5)
    box.set_variant(capi.LBM_VARIANT_DIRECT)
    plan = ["fused", "fused", "unfused", "fused", "fused", "staged", "fused", "tune", "fused",
            "fused"]
    for what in plan:
        if what == "unfused":
            box.step_unfused(1)
        elif what == "staged":
            box.set_variant(capi.LBM_VARIANT_STAGED)
            box.step(1)
            box.set_variant(capi.LBM_VARIANT_DIRECT)
        elif what == "tune":
            box.autotune(1)
            box.set_variant(capi.LBM_VARIANT_DIRECT)
            box.step(1)
        else:
            box.step(1)
        o.step(1)
    assert relerr(box.get_f(), o.f) <= TOL64
