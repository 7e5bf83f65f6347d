"""lbm_mass_momentum_noalloc: the allocation-free mass/momentum reduction.

It serves callers that cannot allocate device memory (a solver that has
reserved the GPU's memory for its own state, or a runtime that hands out
pointers from its own pool): they pass their own device buffers and the
library works in a fixed static scratch array.  This test calls it through
the C ABI on a device array that the test allocates, twice in a row, and
checks both results against the context-based lbm_mass_momentum.

This file is named so that pytest collects it last.
"""

import ctypes as C

import numpy as np
import pytest

from multiphase_flow_codes_gb300 import _capi as capi

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def test_noalloc_matches_mass_momentum(require_gpu, engine_lib):
    import torch
    from multiphase_flow_codes_gb300.engine import LBMBox

    nx, ny, nz = 24, 20, 18
    rng = np.random.default_rng(11)
    f = 0.05 * rng.standard_normal((19, nz, ny, nx))
    f[1] += 0.01  # a nonzero net momentum
    cfg = capi.config_init(capi.LBM_PRESET_BOX, nx, ny, nz, 0, 4.0, 2.5)
    box = LBMBox(cfg)
    box.set_f(f)
    ref = box.mass_momentum()
    box.close()

    dev_f = torch.from_numpy(f).to("cuda")
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        rc = engine_lib.lbm_mass_momentum_noalloc(C.c_void_p(dev_f.data_ptr()), nx, ny, nz,
                                                  C.c_void_p(out.data_ptr()), None)
        assert rc == capi.LBM_OK
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() <= RTOL * scale, (call, got, ref)


def test_noalloc_rejects_too_many_planes(require_gpu, engine_lib):
    import torch
    dummy = torch.zeros(19, dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    rc = engine_lib.lbm_mass_momentum_noalloc(C.c_void_p(dummy.data_ptr()), 1, 1, 4097,
                                              C.c_void_p(out.data_ptr()), None)
    assert rc == capi.LBM_ERR_ARG
