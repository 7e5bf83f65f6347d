"""The oracle pinned against the reference's own Fortran.

The reference's hot-path sources (3DBox_Forced_HI_Turbulence_Moving_Particles_LBM
and 3DChannel_Decaying_HIT_Finite_Size_Moving_Particles) are translated to
C++ by oracle/fortran and run on one process (oracle/refrun.py drives them in
the order of their main programs).  The C++ restatement that the GPU tests
use as their checker (oracle/lbm_oracle.cpp) must reproduce them:

* the channel program bit for bit: populations, solid flags, links, link
  fractions and particle state, every step;
* the box program bit for bit in everything but the stochastic force, which
  the reference synthesises with three FFTs (FFTW 2) and the restatement by
  direct evaluation of its 50 modes: the forcing generator's state is equal,
  the force fields agree to 1e-13 of their maximum, and the populations and
  particle state that follow agree to 1e-13.

Particle ids are 1-based in the reference and 0-based in the restatement.
These tests need the reference's sources (or the translation generated from
them); without either they skip.
"""

import numpy as np
import pytest

from conftest import relerr

from multiphase_flow_codes_gb300 import inputs

refrun = pytest.importorskip("oracle.refrun")


def need(prog):
    if not refrun.available(prog):
        pytest.skip(f"the reference's {prog} program is not available here")


def ids_ref(a):
    """0-based particle ids of the restatement -> the reference's 1-based ids."""
    return np.where(a >= 0, a + 1, a)


def compare(R, o, npart, tol_f, tol_p, exact_links=True):
    F = refrun.fields(R)
    out = {"f": relerr(o.f, F["f"])}
    assert np.array_equal(o.ibnodes, F["ibnodes"])
    assert np.array_equal(ids_ref(o.isnodes), F["isnodes"])
    assert np.array_equal(o.ilink, F["ilink"])
    assert np.array_equal(ids_ref(o.mlink), F["mlink"])
    out["alpha"] = float(np.abs(o.alink - F["alink"]).max())
    for k in ("ypglb", "wp", "omgp", "fHIp", "flubp", "torqp"):
        out[k] = relerr(getattr(o, k)[:npart], F[k])
    assert out["f"] <= tol_f, out
    assert out["alpha"] <= (0.0 if exact_links else 1e-15), out
    for k in ("ypglb", "wp", "omgp", "fHIp", "flubp", "torqp"):
        assert out[k] <= tol_p, (k, out)
    return out


def box_pair(oracle_mod, n, npart, rad, rhopart, wp=None, omgp=None, positions=None):
    from oracle import config as ocfg
    R = refrun.box_program(n, npart, rad, rhopart)
    cfg = ocfg.config_init(ocfg.PRESET_BOX, n, n, n, npart, rad, rhopart)
    cfg.visc = R["visc"]  # para derives visc from anu, vscale and ny
    o = oracle_mod.OracleBox(cfg)
    u = inputs.spectral_velocity(n, 4.0, 0.03)
    refrun.set_velocity(R, *u)
    R.call("initpop")
    o.initpop(*u)
    R.call("macrovar")
    o.macrovar()
    assert np.array_equal(o.f, refrun.fields(R)["f"])  # initpop and macrovar bit for bit
    refrun.release(R, wp, omgp, positions)
    y = R["ypglb"].T.copy()
    o.release_particles(y, wp, omgp)
    return R, o


def test_box_ten_steps(oracle_mod):
    """32^3 box, 4 spheres R = 4.5, density ratio 5, 10 full steps."""
    need("box")
    R, o = box_pair(oracle_mod, 32, 4, 4.5, 5.0)
    y0 = inputs.initpartpos(32, 32, 32, 4, 4.5)
    assert np.array_equal(R["ypglb"].T, y0)  # initpartpos / ranpp bit for bit
    for s in range(1, 11):
        refrun.step(R, s)
        o.step(1)
        assert R["iseedf"] == o.iseedf and R["iyf"] == o.iyf
        assert np.array_equal(R["ivf"], o.ivf)
        F = refrun.fields(R)
        for c, k in (("fx", "force_realx"), ("fy", "force_realy"), ("fz", "force_realz")):
            assert relerr(getattr(o, c), F[k]) <= 1e-13, (s, c)
        compare(R, o, 4, 1e-13, 1e-13)


def test_box_moving_spheres_refill_and_lubrication(oracle_mod):
    """Spheres launched with translation and spin (nodes uncovered and
    refilled every step) and a pair inside the lubrication range."""
    need("box")
    rng = np.random.default_rng(7)
    wp = rng.uniform(-0.08, 0.08, (4, 3))
    om = rng.uniform(-0.01, 0.01, (4, 3))
    pos = np.array([[10.2, 12.3, 11.9], [18.8, 12.6, 12.1], [22.0, 25.0, 5.0], [5.5, 26.0, 24.0]])
    R, o = box_pair(oracle_mod, 32, 4, 4.0, 2.5, wp, om, pos)
    refilled = 0
    for s in range(1, 11):
        before = o.ibnodes.copy()
        refrun.step(R, s)
        o.step(1)
        refilled += int(((before > 0) & (o.ibnodes < 0)).sum())
        if s == 1:
            assert np.abs(o.flubp[:2]).max() > 0
        compare(R, o, 4, 1e-13, 1e-13)
    assert refilled > 0


def channel_pair(oracle_mod, shape, npart, rad, rhopart, wp=None, positions=None):
    from oracle import config as ocfg
    nx, ny, nz = shape
    R = refrun.channel_program(nx, ny, nz, npart, rad, rhopart)
    cfg = ocfg.config_init(ocfg.PRESET_CHANNEL, nx, ny, nz, npart, rad, rhopart)
    assert cfg.visc == R["visc"] and cfg.force_y == R["force_in_y"]
    o = oracle_mod.OracleBox(cfg)
    u = inputs.spectral_velocity(nx, 4.0, 0.03, ny=ny, nz=nz)
    refrun.set_velocity(R, *u)
    R.call("forcing")  # once, before the loop (3DChannel.../main.f90:151)
    R.call("initpop")
    o.initpop(*u)
    R.call("macrovar")
    o.macrovar()
    assert np.array_equal(o.f, refrun.fields(R)["f"])
    refrun.release(R, wp, None, positions)
    o.release_particles(R["ypglb"].T.copy(), wp)
    return R, o


def test_channel_ten_steps_bit_exact(oracle_mod):
    """30 x 36 x 28 channel, walls at x = 0 and x = 30, 4 spheres with
    random velocities: the restatement reproduces every bit."""
    need("channel")
    rng = np.random.default_rng(3)
    wp = rng.uniform(-0.05, 0.05, (4, 3))
    R, o = channel_pair(oracle_mod, (30, 36, 28), 4, 4.0, 1.0, wp)
    y0 = inputs.initpartpos(30, 36, 28, 4, 4.0, channel=True)
    assert np.array_equal(R["ypglb"].T, y0)
    for s in range(1, 11):
        refrun.step(R, s, forcing=False)
        o.step(1)
        compare(R, o, 4, 0.0, 0.0)


def test_channel_wall_lubrication_bit_exact(oracle_mod):
    """Spheres inside the particle-wall lubrication range of both walls
    (3DChannel.../partlib.f90:2317-2356) and a pair inside the
    particle-particle range."""
    need("channel")
    pos = np.array([[5.1, 8.3, 7.7], [36 - 5.4, 30.2, 20.6], [18.0, 20.0, 9.0],
                    [18.3, 29.1, 9.4]])
    wp = np.array([[-0.01, 0.0, 0.0], [0.01, 0.0, 0.0], [0.0, 0.01, 0.0], [0.0, -0.01, 0.0]])
    R, o = channel_pair(oracle_mod, (36, 40, 32), 4, 4.0, 1.0, wp, pos)
    for s in range(1, 11):
        refrun.step(R, s, forcing=False)
        o.step(1)
        if s == 1:
            assert np.all(np.abs(o.flubp[:4]).max(axis=1) > 0)
        compare(R, o, 4, 0.0, 0.0)


def test_channel_initvel(oracle_mod):
    """The channel's initvel (log-law mean flow) against its numpy
    restatement, which the GPU's lbm_init_channel is tested against."""
    need("channel")
    from oracle import initial
    for shape in ((64, 24, 16), (30, 36, 28)):
        R = refrun.channel_program(*shape, 2, 4.0, 1.0)
        R.call("initvel")
        F = refrun.fields(R)
        u = initial.channel_loglaw(*shape, R["visc"])
        for a, b in zip(u, (F["ux"], F["uy"], F["uz"])):
            assert np.array_equal(a, b), shape


def test_box_rhoupdat(oracle_mod):
    """The pre-relaxation's density update (3DBox.../collision.f90:213-229)."""
    need("box")
    R, o = box_pair(oracle_mod, 24, 1, 4.0, 2.5)
    for _ in range(2):
        R.call("collision_mrt")
        o.collision_MRT()
        R.call("streaming")
        o.streaming()
        R.call("rhoupdat")
        o.rhoupdat()
    F = refrun.fields(R)
    assert np.array_equal(o.rho, F["rho"])
    assert relerr(o.f, F["f"]) == 0.0


INTERP_BOX = np.array([
    [10.3, 9.7, 7.2], [0.2, 5.3, 6.6], [23.8, 6.1, 3.3], [7.7, 0.3, 8.1], [11.1, 19.6, 9.9],
    [3.3, 4.4, 0.1], [5.5, 7.5, 15.7], [0.1, 0.2, 0.3], [23.9, 19.9, 15.9], [12.0, 0.4, 15.6],
    [6.0, 19.7, 0.2], [2.2, 19.8, 15.8], [4.5, 5.5, 6.5]])


def interp_pair(oracle_mod, prog, shape, positions):
    """The reference program and the restatement with a random velocity
    field and the given centres after initpartpos's local lists."""
    from oracle import config as ocfg
    nx, ny, nz = shape
    n = positions.shape[0]
    if prog == "box":
        R = refrun.box_program(nx, n, 1.0, 1.0, ny=ny, nz=nz)
        cfg = ocfg.config_init(ocfg.PRESET_BOX, nx, ny, nz, n, 1.0, 1.0)
    else:
        R = refrun.channel_program(nx, ny, nz, n, 1.0, 1.0)
        cfg = ocfg.config_init(ocfg.PRESET_CHANNEL, nx, ny, nz, n, 1.0, 1.0)
    o = oracle_mod.OracleBox(cfg)
    rng = np.random.default_rng(nx * 7 + ny)
    u = [rng.standard_normal((nz, ny, nx)) * 0.05 for _ in range(3)]
    refrun.set_velocity(R, *u)
    for c, a in zip(("ux", "uy", "uz"), u):
        getattr(o, c)[...] = a
    R["istep"] = 1
    R.call("initpartpos")
    assert np.array_equal(R["ipglb"][:R["nps"]], np.arange(1, n + 1))
    R["ypglb"] = positions.T
    R["yp"][:, :n] = positions.T
    return R, o


@pytest.mark.parametrize("prog", ["box", "channel"])
def test_initpartvel(oracle_mod, prog):
    """initpartvel (trilinear interpolation of u at the centres,
    3DBox.../partlib.f90:177-263, 320-831; channel 182-268, 325-836) bit for
    bit, with centres in every halo case of trilinear: below the first and
    above the last node along each axis, the corners, a centre on a node."""
    need(prog)
    shape = (24, 20, 16)
    pos = INTERP_BOX.copy()
    if prog == "channel":  # x cells inside the walls (the reference has no x image there)
        pos[:, 0] = np.clip(pos[:, 0], 0.6, shape[0] - 0.6)
    R, o = interp_pair(oracle_mod, prog, shape, pos)
    R.call("initpartvel")
    got = o.initpartvel(pos)
    assert np.array_equal(got, R["wp"].T)
    assert np.abs(got).max() > 0


def test_initpartvel_channel_rejects_wall_cells(oracle_mod):
    from oracle import config as ocfg
    cfg = ocfg.config_init(ocfg.PRESET_CHANNEL, 24, 20, 16, 2, 1.0, 1.0)
    o = oracle_mod.OracleBox(cfg)
    with pytest.raises(ValueError):
        o.initpartvel(np.array([[5.0, 5.0, 5.0], [0.4, 5.0, 5.0]]))
    with pytest.raises(ValueError):
        o.initpartvel(np.array([[23.6, 5.0, 5.0]]))
