"""Regenerate the golden fixtures in this directory.

The reference has no test vectors of its own and cannot be compiled here,
so these fixtures come from the package's independent Python restatements of
the reference's generators (they pin the CPU oracle and guard against
regressions):
  ran1.npz                 first 500 draws of ranff/ranpp (Park-Miller with
                           Bays-Durham shuffle, B/gaussian.f90:374-404,
                           B/partlib.f90:83-115) for seeds 232300 and 12345
  positions_box64_p16.npz  initpartpos (B/partlib.f90:1-80) for a 64^3 box,
                           16 spheres of radius 4.5, mingap 2, seed 12345
Run: python tests/golden/make_golden.py
"""

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from multiphase_flow_codes_gb300 import inputs  # noqa: E402


def main():
    out = {}
    for seed in (232300, 12345):
        r = inputs.Ran1(seed)
        out[f"s{seed}"] = np.array([r() for _ in range(500)])
    np.savez(HERE / "ran1.npz", **out)
    y = inputs.initpartpos(64, 64, 64, 16, 4.5, 2.0, seed=12345)
    np.savez(HERE / "positions_box64_p16.npz", ypglb=y)


if __name__ == "__main__":
    main()
