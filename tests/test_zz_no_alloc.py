"""lbm_mass_momentum_noalloc: the allocation-free mass/momentum reduction.

It serves callers that cannot allocate device memory (a solver that has
reserved the GPU's memory for its own state, or a runtime that hands out
pointers from its own pool): they pass their own device buffers and the
library works in a fixed static scratch array.  These tests call it through
the C ABI on device arrays that the test allocates and check each result
against an exactly rounded numpy sum and against the context-based
lbm_mass_momentum:

* two calls in a row, the second on another field with fewer planes, so a
  call that read the first call's leftover plane sums would be caught;
* a call on a caller's stream (not the default stream);
* the largest plane count the scratch array holds, and one more (rejected).

This file is named so that pytest collects it last.
"""

import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

from multiphase_flow_codes_gb300 import _capi as capi

pytestmark = pytest.mark.gpu

RTOL = 1e-12
MAX_PLANES = int(re.search(r"#define\s+LBM_NOALLOC_MAX_PLANES\s+(\d+)",
                           (Path(__file__).resolve().parents[1] / "include" / "lbm.h").read_text()).group(1))
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0], dtype=np.float64)
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1], dtype=np.float64)
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1], dtype=np.float64)


def exact_totals(f):
    """(sum f, sum cx f, sum cy f, sum cz f) rounded once (math.fsum), and the
    sum of |f| that bounds a summation's rounding."""
    flat = f.reshape(19, -1)
    out = []
    for c in (np.ones(19), CX, CY, CZ):
        out.append(math.fsum((c[:, None] * flat).ravel()))
    return np.array(out), float(np.abs(flat).sum())


def call(engine_lib, dev_f, dims, out, stream=None):
    nx, ny, nz = dims
    return engine_lib.lbm_mass_momentum_noalloc(C.c_void_p(dev_f.data_ptr()), nx, ny, nz,
                                                C.c_void_p(out.data_ptr()),
                                                None if stream is None else C.c_void_p(stream))


def field(rng, dims, scale, drift):
    nx, ny, nz = dims
    f = scale * rng.standard_normal((19, nz, ny, nx))
    f[1] += drift  # a nonzero net momentum
    return f


def test_noalloc_two_calls_against_numpy_and_engine(require_gpu, engine_lib):
    import torch
    from multiphase_flow_codes_gb300.engine import LBMBox

    rng = np.random.default_rng(11)
    d1, d2 = (24, 20, 18), (16, 12, 7)
    f1 = field(rng, d1, 0.05, 0.01)
    f2 = field(rng, d2, 0.2, -0.03)
    cfg = capi.config_init(capi.LBM_PRESET_BOX, *d1, 0, 4.0, 2.5)
    box = LBMBox(cfg)
    box.set_f(f1)
    ref_engine = box.mass_momentum()
    box.close()

    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    for f, dims in ((f1, d1), (f2, d2)):
        dev_f = torch.from_numpy(f).to("cuda")
        torch.cuda.synchronize()
        assert call(engine_lib, dev_f, dims, out) == capi.LBM_OK
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        exact, bound = exact_totals(f)
        assert np.abs(got - exact).max() <= RTOL * bound, (dims, got, exact)
        if f is f1:
            assert np.abs(got - ref_engine).max() <= RTOL * bound, (got, ref_engine)


def test_noalloc_on_a_caller_stream(require_gpu, engine_lib):
    import torch
    rng = np.random.default_rng(12)
    dims = (32, 8, 40)
    f = field(rng, dims, 0.05, 0.02)
    exact, bound = exact_totals(f)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        dev_f = torch.from_numpy(f).to("cuda", non_blocking=False)
        out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    s.synchronize()
    assert call(engine_lib, dev_f, dims, out, s.cuda_stream) == capi.LBM_OK
    s.synchronize()
    got = out.cpu().numpy()
    assert np.abs(got - exact).max() <= RTOL * bound, (got, exact)


def test_noalloc_plane_limit(require_gpu, engine_lib):
    import torch
    nz = MAX_PLANES
    rng = np.random.default_rng(13)
    dims = (2, 2, nz)
    f = field(rng, dims, 0.05, 0.01)
    exact, bound = exact_totals(f)
    dev_f = torch.from_numpy(f).to("cuda")
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    assert call(engine_lib, dev_f, dims, out) == capi.LBM_OK
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.abs(got - exact).max() <= RTOL * bound, (got, exact)
    # one plane more than the scratch array holds is refused before any launch
    assert call(engine_lib, dev_f, (1, 2, nz + 1), out) == capi.LBM_ERR_ARG
