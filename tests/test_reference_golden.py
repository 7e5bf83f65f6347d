"""The oracle against golden vectors recorded from the reference's own
Fortran (tests/golden/make_reference_golden.py, run through oracle/fortran).

These need neither the reference's sources nor a GPU: the oracle repeats
the recorded runs and must match the channel run bit for bit and the box
run within 1e-13 (the box's stochastic force comes from FFTs in the
reference and from direct mode sums in the oracle)."""

from pathlib import Path

import numpy as np
import pytest

from conftest import relerr

from multiphase_flow_codes_gb300 import inputs

GOLDEN = Path(__file__).resolve().parent / "golden"
WP = np.array([[0.03, -0.02, 0.01], [-0.01, 0.04, -0.03]])
OMGP = np.array([[0.0, 0.004, -0.002], [0.003, 0.0, 0.001]])


def check(o, g, tol):
    f = o.f.reshape(-1)[g["f_index"]]
    assert relerr(f, g["f_sample"]) <= tol
    isn = np.where(o.isnodes >= 0, o.isnodes + 1, o.isnodes)
    assert np.array_equal(isn, g["isnodes"])
    assert int((o.ilink > 0).sum()) == int(g["nlinks"])
    for k in ("ypglb", "wp", "omgp", "fHIp", "flubp", "torqp"):
        assert relerr(getattr(o, k)[:2], g[k]) <= tol, k


@pytest.mark.parametrize("kind", ["box", "channel"])
def test_oracle_matches_reference_golden(oracle_mod, kind):
    from oracle import config as ocfg
    if kind == "box":
        g = np.load(GOLDEN / "reference_box24_p2.npz")
        shape, preset, rhop = (24, 24, 24), ocfg.PRESET_BOX, 2.5
    else:
        g = np.load(GOLDEN / "reference_channel24_p2.npz")
        shape, preset, rhop = (24, 28, 20), ocfg.PRESET_CHANNEL, 1.0
    cfg = ocfg.config_init(preset, *shape, 2, 4.0, rhop)
    if kind == "box":
        # the box program's para derives visc = anu vscale ny / (2 pi)
        cfg.visc = 0.0945 * 2.037183272e-3 * shape[1] / (2.0 * np.pi)
    o = oracle_mod.OracleBox(cfg)
    o.initpop(*inputs.spectral_velocity(shape[0], 4.0, 0.03, seed=54321, ny=shape[1],
                                        nz=shape[2]))
    o.macrovar()
    y = inputs.initpartpos(*shape, 2, 4.0, cfg.mingap, seed=12345,
                           channel=kind == "channel", mingap_w=cfg.mingap_w)
    o.release_particles(y, WP, OMGP)
    assert o.step(5) == 0
    if kind == "box":
        assert o.iseedf == int(g["iseedf"]) and o.iyf == int(g["iyf"])
        assert np.array_equal(o.ivf, g["ivf"])
    check(o, g, 1e-13 if kind == "box" else 0.0)


@pytest.mark.parametrize("kind", ["box", "channel"])
def test_oracle_initpartvel_matches_reference_golden(oracle_mod, kind):
    """initpartvel's trilinear interpolation, bit for bit, at centres in
    every halo case (reference_initpartvel.npz)."""
    from oracle import config as ocfg
    g = np.load(GOLDEN / "reference_initpartvel.npz")
    pos = g[f"pos_{kind}"]
    shape = (24, 20, 16)
    preset = ocfg.PRESET_BOX if kind == "box" else ocfg.PRESET_CHANNEL
    cfg = ocfg.config_init(preset, *shape, pos.shape[0], 1.0, 1.0)
    o = oracle_mod.OracleBox(cfg)
    u = inputs.spectral_velocity(shape[0], 3.0, 0.04, seed=54321, ny=shape[1], nz=shape[2])
    for c, a in zip(("ux", "uy", "uz"), u):
        getattr(o, c)[...] = a
    assert np.array_equal(o.initpartvel(pos), g[f"wp_{kind}"])
