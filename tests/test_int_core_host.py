"""The FP64 plain path's two fixed-point collision cores on the host.

The all-integer core (velocity and force products as exact 128-bit integer
products, the FP64 contexts' default) and the core that keeps those products
in FP64 compute the same collision; the integer core rounds each product
once, the other converts FP64 values whose rounding the inverse transform
multiplies by up to 30, so their post-collision populations (at 2^-58 =
3.5e-18) agree to about 3e-17 (measured: 3.1e-17, nine units).  States beyond the
integer core's ranges (|u| >= 1/4) are declined by it and taken by the FP64
path in the kernel; its ranges are the narrower ones, so the FP64 core takes
every state the integer core takes.  Built for the host with nvcc from the header the
kernels use (tests/host/int_core_check.cu); no GPU is needed.
"""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_integer_core_matches_fp64_product_core(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc"
                                    if Path("/usr/local/cuda/bin/nvcc").exists() else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = tmp_path / "int_core_check"
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-O2",
                    "-I", str(ROOT / "include"),
                    "-I", str(ROOT / "multiphase_flow_codes_gb300" / "csrc"),
                    str(ROOT / "tests" / "host" / "int_core_check.cu"), "-o", str(exe)],
                   check=True, capture_output=True, timeout=600)
    out = subprocess.run([str(exe), "60000"], check=True, capture_output=True, text=True,
                         timeout=600).stdout.split("\n")
    rows = [ln.split() for ln in out if ln.strip()]
    rng_row = rows.pop(0)
    assert rng_row[0] == "range" and int(rng_row[1]) == 0, rng_row  # high-word test == 64-bit test
    assert len(rows) == 2
    for mrt, maxd, dec_int, dec_fp, int_only, fp_only, n in rows:
        assert float(maxd) <= 16 * 2.0 ** -58, (mrt, maxd)
        # the integer core's ranges are the narrower: what it takes, the FP64
        # core takes too; it declines more of the fast states
        assert int(fp_only) == 0, (mrt, fp_only)
        assert int(dec_int) >= int(dec_fp) > 0, (mrt, dec_int, dec_fp)
