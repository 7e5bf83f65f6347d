"""Golden vectors from the reference's own Fortran (run through oracle/fortran).

The reference ships no test vectors and no Fortran compiler exists here; its
hot-path sources are translated to C++ and run on one process by
oracle/fortran (see oracle/fortran/build.py).  This script records small
fixtures of those runs so the oracle stays pinned where the reference's
sources are absent:

  reference_box24_p2.npz      3DBox...: 24^3, 2 spheres R = 4 (density 2.5),
                              seeded velocity (inputs.spectral_velocity, seed
                              54321, k0 4, u_rms 0.03), spheres from
                              initpartpos (seed 12345) moving with given
                              velocities, 5 full steps
  reference_channel24_p2.npz  3DChannel...: 24 x 28 x 20, walls at x = 0 and
                              x = 24, 2 spheres R = 4, 5 full steps
  reference_initpartvel.npz   initpartvel of both programs on a 24 x 20 x 16
                              grid: the seeded velocity (spectral_velocity,
                              seed 54321, k0 3, u_rms 0.04) interpolated at
                              13 centres in every halo case of trilinear

Each holds the particle vectors, the solid-node ids (isnodes, 1-based as
the reference), the number of links, the forcing generator's state (box),
and the populations at 4096 seeded positions.
Run: python tests/golden/make_reference_golden.py [name ...]   (needs the
reference; with names, only those fixtures)
"""

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from multiphase_flow_codes_gb300 import inputs  # noqa: E402
from oracle import refrun  # noqa: E402

WP = np.array([[0.03, -0.02, 0.01], [-0.01, 0.04, -0.03]])
OMGP = np.array([[0.0, 0.004, -0.002], [0.003, 0.0, 0.001]])
STEPS = 5


def sample_index(shape, n=4096, seed=99):
    rng = np.random.default_rng(seed)
    return rng.integers(0, int(np.prod(shape)), n)


def record(R, name, box: bool):
    F = refrun.fields(R)
    idx = sample_index(F["f"].shape)
    out = {"f_sample": F["f"].reshape(-1)[idx], "f_index": idx,
           "isnodes": F["isnodes"].astype(np.int16), "nlinks": int((F["ilink"] > 0).sum())}
    for k in ("ypglb", "wp", "omgp", "fHIp", "flubp", "torqp"):
        out[k] = F[k]
    if box:
        out["iseedf"] = R["iseedf"]
        out["iyf"] = R["iyf"]
        out["ivf"] = R["ivf"].copy()
    np.savez_compressed(HERE / name, **out)


INTERP = np.array([
    [10.3, 9.7, 7.2], [0.2, 5.3, 6.6], [23.8, 6.1, 3.3], [7.7, 0.3, 8.1], [11.1, 19.6, 9.9],
    [3.3, 4.4, 0.1], [5.5, 7.5, 15.7], [0.1, 0.2, 0.3], [23.9, 19.9, 15.9], [12.0, 0.4, 15.6],
    [6.0, 19.7, 0.2], [2.2, 19.8, 15.8], [4.5, 5.5, 6.5]])


def interp_centres(channel: bool, nx: int = 24):
    pos = INTERP.copy()
    if channel:  # x cells inside the walls
        pos[:, 0] = np.clip(pos[:, 0], 0.6, nx - 0.6)
    return pos


def record_initpartvel():
    shape = (24, 20, 16)
    u = inputs.spectral_velocity(shape[0], 3.0, 0.04, seed=54321, ny=shape[1], nz=shape[2])
    out = {}
    for prog in ("box", "channel"):
        pos = interp_centres(prog == "channel", shape[0])
        n = pos.shape[0]
        if prog == "box":
            R = refrun.box_program(shape[0], n, 1.0, 1.0, ny=shape[1], nz=shape[2])
        else:
            R = refrun.channel_program(*shape, n, 1.0, 1.0)
        refrun.set_velocity(R, *u)
        R["istep"] = 1
        R.call("initpartpos")
        R["ypglb"] = pos.T
        R["yp"][:, :n] = pos.T
        R.call("initpartvel")
        out[f"pos_{prog}"] = pos
        out[f"wp_{prog}"] = R["wp"].T.copy()
    np.savez_compressed(HERE / "reference_initpartvel.npz", **out)


def main(only=()):
    if not only or "initpartvel" in only:
        record_initpartvel()
    if only and "runs" not in only:
        return
    n = 24
    R = refrun.box_program(n, 2, 4.0, 2.5)
    refrun.set_velocity(R, *inputs.spectral_velocity(n, 4.0, 0.03, seed=54321))
    R.call("initpop")
    R.call("macrovar")
    refrun.release(R, WP, OMGP)
    for s in range(1, STEPS + 1):
        refrun.step(R, s)
    record(R, "reference_box24_p2.npz", True)

    shape = (24, 28, 20)
    R = refrun.channel_program(*shape, 2, 4.0, 1.0)
    refrun.set_velocity(R, *inputs.spectral_velocity(shape[0], 4.0, 0.03, seed=54321,
                                                      ny=shape[1], nz=shape[2]))
    R.call("forcing")
    R.call("initpop")
    R.call("macrovar")
    refrun.release(R, WP, OMGP)
    for s in range(1, STEPS + 1):
        refrun.step(R, s, forcing=False)
    record(R, "reference_channel24_p2.npz", False)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
