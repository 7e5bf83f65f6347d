"""Populations stored in 64-bit fixed point between the FP64 plain path's
fused steps (g.pop_fixed): reads of the state between steps convert the
buffer back to FP64 and the next fused step converts it again, so any mix of
steps and reads stays on the oracle's trajectory; values the fixed point
cannot hold are reported, not wrapped.  Every failure here is made on the
host side (an input the fixed point cannot represent); the kernels report it
through the context's status word.
"""

import numpy as np
import pytest

from conftest import relerr
from test_gpu_parity import TOL64, make_pair

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import LBMError

pytestmark = pytest.mark.gpu


def test_reads_between_fused_steps_keep_parity(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod, shape=(36, 32, 32), npart=3, rad=4.0, rhopart=2.5)
    box.set_variant(capi.LBM_VARIANT_DIRECT)
    reads = [lambda: box.get_f(), lambda: box.get_macro(), lambda: box.diag(),
             lambda: box.mass_momentum(), lambda: box.summary(), lambda: None]
    for s in range(12):
        box.step(1)
        o.step(1)
        reads[s % len(reads)]()
    assert relerr(box.get_f(), o.f) <= TOL64
    # a read right after a step returns that step's populations
    box.step(1)
    o.step(1)
    assert relerr(box.get_f(), o.f) <= TOL64


def test_population_beyond_fixed_range_reported(require_gpu, oracle_mod):
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 16, 16, 16, 0, 4.0, 1.0)
    box = LBMBox(cfg)
    f = np.zeros((19, 16, 16, 16))
    f[3, 5, 6, 7] = 40.0  # |f| >= 32: not representable at 2^-58 in 64 bits
    box.set_f(f)
    box.macrovar()
    box.set_variant(capi.LBM_VARIANT_DIRECT)
    with pytest.raises(LBMError) as e:
        for _ in range(4):  # a step reports the status of the steps before it
            box.step(1)
            box.synchronize()
    assert e.value.code == capi.LBM_ERR_NONFINITE


def test_forcing_beyond_fixed_range_reported(require_gpu):
    """Forcing amplitudes whose row coefficients reach 2^-7 leave the
    fixed-point force range: the step reports LBM_ERR_STATE."""
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 16, 16, 16, 0, 4.0, 1.0)
    box = LBMBox(cfg)
    box.set_f(np.zeros((19, 16, 16, 16)))
    box.macrovar()
    iseedf, iyf, ivf, b = box.get_forcing_state()
    box.set_forcing_state(iseedf, iyf, ivf, np.full_like(b, 10.0))
    with pytest.raises(LBMError) as e:
        for _ in range(4):
            box.step(1)
            box.synchronize()
    assert e.value.code == capi.LBM_ERR_STATE
