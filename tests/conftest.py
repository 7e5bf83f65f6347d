import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def engine_lib():
    """The CUDA engine library, built in-tree if it is missing."""
    from multiphase_flow_codes_gb300 import build
    build.build()
    from multiphase_flow_codes_gb300 import _capi
    return _capi.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def gpu_available() -> bool:
    try:
        import ctypes
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            import torch
            return torch.cuda.is_available()
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def require_gpu():
    if not gpu_available():
        pytest.fail("GPU test selected but no CUDA device is visible")


CIX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CIY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
CIZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
IPOPP = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15])


def relerr(a, b):
    """max-norm relative difference ||a - b||_inf / ||b||_inf"""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def oracle_links(o):
    """Dense oracle link arrays -> sorted (particle, node, ipop, alpha) table."""
    il = o.ilink
    q, k, j, i = np.nonzero(il > 0)
    node = i + o.nx * (j + o.ny * k)
    part = o.mlink[q, k, j, i]
    alpha = o.alink[q, k, j, i]
    ipop = q + 1
    order = np.lexsort((ipop, node, part))
    return part[order], node[order], ipop[order], alpha[order]


def gpu_links(box):
    node, ipop, part, alpha = box.get_links()
    order = np.lexsort((ipop, node, part))
    return part[order], node[order], ipop[order], alpha[order]


def link_term_scale(o, links):
    """Per particle, the sum over its links of 2 |f| of the two populations a
    link exchanges (the magnitude of the momentum-exchange terms whose sum
    is fHIp), from the oracle's post-step populations."""
    part, node, ipop, _ = links
    f = o.f.reshape(19, -1)
    mag = np.abs(f[ipop, node]) + np.abs(f[IPOPP[ipop], node])
    s = np.zeros(o.npmax)
    np.add.at(s, part - 1, 2.0 * mag)
    return s
