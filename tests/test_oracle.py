"""CPU tests of the oracle (the C++ restatement of the reference time step).

The reference ships no tests or golden vectors and cannot be compiled here,
so the oracle is checked against independent restatements and invariants:
  * the Park-Miller/Bays-Durham generator against an independent Python
    restatement, and particle placement against the Python initpartpos;
  * the forcing's direct mode synthesis against numpy's inverse FFT of the
    spectral array FORCING places (gaussian.f90:557-601);
  * streaming against numpy rolls, channel halfway bounce-back included;
  * collision: mass conservation, momentum change equal to the body force,
    equilibrium fixed point (all-equal rates);
  * link geometry against a vectorised numpy restatement;
  * lubrication: equal and opposite pair forces;
  * channel Poiseuille flow against the analytic parabola.
"""

import math

import numpy as np
import pytest

from conftest import CIX, CIY, CIZ, IPOPP

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import inputs


def box_cfg(engine_lib, n=16, npart=0, rad=4.5, rhopart=5.0, preset=capi.LBM_PRESET_BOX, shape=None):
    nx, ny, nz = shape or (n, n, n)
    return capi.config_init(preset, nx, ny, nz, npart, rad, rhopart)


def test_ran1_matches_python_restatement(oracle_mod):
    for seed in (232300, 12345, 1):
        got = oracle_mod.ran1_sequence(seed, 3000)
        r = inputs.Ran1(seed)
        ref = np.array([r() for _ in range(3000)])
        assert np.array_equal(got, ref)
        assert got.min() > 0.0 and got.max() < 1.0


# Park & Miller, "Random number generators: good ones are hard to find",
# CACM 31 (1988): the minimal standard x_{k+1} = 16807 x_k mod (2^31 - 1)
# started from x_0 = 1 has x_10000 = 1043618065.
PARK_MILLER_X10000 = 1043618065


def test_park_miller_known_answer(oracle_mod):
    """The core of ranff/ranpp (3DBox.../gaussian.f90:385-397) is the minimal
    standard generator: its state after the shuffle table's 40-step warm-up
    and 9960 draws is the published 10,000th value from seed 1, in the
    oracle and in the Python restatement."""
    assert oracle_mod.ran1_state(1, 9960) == PARK_MILLER_X10000
    r = inputs.Ran1(1)
    for _ in range(9960):
        r()
    assert r.idum == PARK_MILLER_X10000
    # and every other state is the closed form 16807^k mod (2^31 - 1)
    for n in (1, 2, 450, 4500):
        assert oracle_mod.ran1_state(232300, n) == 232300 * pow(16807, 40 + n, 2**31 - 1) % (2**31 - 1)


def test_ran1_golden(oracle_mod):
    g = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "ran1.npz")
    for seed in (232300, 12345):
        assert np.array_equal(oracle_mod.ran1_sequence(seed, g[f"s{seed}"].size), g[f"s{seed}"])


@pytest.mark.parametrize("preset", [capi.LBM_PRESET_BOX, capi.LBM_PRESET_CHANNEL])
def test_initpartpos_matches_python(engine_lib, oracle_mod, preset):
    n, npart, rad = 48, 20, 4.0
    cfg = box_cfg(engine_lib, n, npart, rad, preset=preset)
    o = oracle_mod.OracleBox(cfg)
    assert o.initpartpos(npart) == 0
    py = inputs.initpartpos(n, n, n, npart, rad, channel=(preset == capi.LBM_PRESET_CHANNEL))
    assert np.array_equal(o.ypglb[:npart], py)


def test_initpartpos_golden():
    g = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "positions_box64_p16.npz")
    y = inputs.initpartpos(64, 64, 64, 16, 4.5)
    assert np.array_equal(y, g["ypglb"])


def spectral_field(o, a):
    """numpy restatement of FORCING's spectral placement + mpifft3DCR."""
    nx, ny, nz = o.nx, o.ny, o.nz
    C = np.zeros((nz, ny, nx // 2 + 1), dtype=np.complex128)
    kvals = [0, 1, 2, -2, -1]
    A = a.reshape(5, 5, 6)  # Fortran (6,5,5) -> [k][j][i]
    for k in range(5):
        for j in range(5):
            for kx in range(3):
                C[kvals[k] % nz, kvals[j] % ny, kx] = A[k, j, 2 * kx] + 1j * A[k, j, 2 * kx + 1]
    return np.fft.irfftn(C, s=(nz, ny, nx), axes=(0, 1, 2)) * (nx * ny * nz)


def test_forcing_direct_synthesis_equals_fft(engine_lib, oracle_mod):
    cfg = box_cfg(engine_lib, 16)
    o = oracle_mod.OracleBox(cfg)
    for _ in range(5):
        o.FORCING()
    for comp, arr in (("a1r", o.fx), ("a2r", o.fy), ("a3r", o.fz)):
        ref = spectral_field(o, getattr(o, comp))
        assert np.abs(arr - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs(o.fx).max() > 0


def test_forcing_modes_are_solenoidal(engine_lib, oracle_mod):
    cfg = box_cfg(engine_lib, 32)
    o = oracle_mod.OracleBox(cfg)
    for _ in range(3):
        o.FORCING()
    kx = np.array([0, 0, 1, 1, 2, 2], dtype=float)
    kv = np.array([0, 1, 2, -2, -1], dtype=float)
    A = [getattr(o, c).reshape(5, 5, 6) for c in ("a1r", "a2r", "a3r")]
    div = A[0] * kx[None, None, :] + A[1] * kv[None, :, None] + A[2] * kv[:, None, None]
    assert np.abs(div).max() <= 1e-14 * max(np.abs(A[0]).max(), 1e-300)


def test_streaming_is_periodic_translation(engine_lib, oracle_mod):
    cfg = box_cfg(engine_lib, shape=(12, 10, 8))
    o = oracle_mod.OracleBox(cfg)
    rng = np.random.default_rng(0)
    f0 = rng.standard_normal(o.f.shape)
    o.f[...] = f0
    o.streaming()
    for q in range(19):
        ref = np.roll(f0[q], shift=(CIZ[q], CIY[q], CIX[q]), axis=(0, 1, 2))
        assert np.array_equal(o.f[q], ref)


def test_channel_streaming_halfway_bounce_back(engine_lib, oracle_mod):
    cfg = box_cfg(engine_lib, preset=capi.LBM_PRESET_CHANNEL, shape=(12, 10, 8))
    o = oracle_mod.OracleBox(cfg)
    rng = np.random.default_rng(1)
    f0 = rng.standard_normal(o.f.shape)
    o.f[...] = f0
    o.streaming()
    for q in range(19):
        ref = np.roll(f0[q], shift=(CIZ[q], CIY[q], CIX[q]), axis=(0, 1, 2))
        if CIX[q] == 1:
            ref[:, :, 0] = f0[IPOPP[q], :, :, 0]
        if CIX[q] == -1:
            ref[:, :, -1] = f0[IPOPP[q], :, :, -1]
        assert np.array_equal(o.f[q], ref)


def test_collision_conserves_mass_and_adds_force(engine_lib, oracle_mod):
    cfg = box_cfg(engine_lib, 8)
    o = oracle_mod.OracleBox(cfg)
    rng = np.random.default_rng(2)
    u = [0.03 * rng.standard_normal((8, 8, 8)) for _ in range(3)]
    o.initpop(*u)
    o.f[...] += 1e-3 * rng.standard_normal(o.f.shape)
    F = [1e-4 * rng.standard_normal((8, 8, 8)) for _ in range(3)]
    o.fx[...], o.fy[...], o.fz[...] = F
    o.macrovar()
    f_in = o.f.copy()
    o.collision_MRT()
    dm = (o.f - f_in).sum(axis=0)
    assert np.abs(dm).max() <= 1e-15
    for c, Fc in zip((CIX, CIY, CIZ), F):
        dj = np.tensordot(c, o.f - f_in, axes=(0, 0))
        assert np.abs(dj - Fc).max() <= 1e-15


def test_collision_equilibrium_fixed_point(engine_lib, oracle_mod):
    """With all rates equal (MRT type 2) the incompressible equilibrium of
    initpop is a fixed point of the collision when F = 0."""
    cfg = box_cfg(engine_lib, 8)
    cfg.mrt_type = 2
    o = oracle_mod.OracleBox(cfg)
    rng = np.random.default_rng(3)
    u = [0.04 * rng.standard_normal((8, 8, 8)) for _ in range(3)]
    o.initpop(*u)
    o.macrovar()
    f_in = o.f.copy()
    o.collision_MRT()
    assert np.abs(o.f - f_in).max() <= 1e-15


def numpy_links(y, n, rad):
    """Vectorised restatement of the solid test and link geometry for a
    periodic box (minimum image by rounding)."""
    c = (np.arange(n) + 0.5)
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    isn = -np.ones((n, n, n), dtype=np.int32)
    links = {}
    for p, (xc, yc, zc) in enumerate(y):
        dx = X - xc
        dx -= n * np.round(dx / n)
        dy = Y - yc
        dy -= n * np.round(dy / n)
        dz = Z - zc
        dz -= n * np.round(dz / n)
        r2 = dx * dx + dy * dy + dz * dz
        solid = r2 - rad * rad <= 0
        isn[solid] = p
        near = (~solid) & (r2 <= (rad + 2) ** 2)
        for q in range(1, 19):
            x1, y1, z1 = dx + CIX[q], dy + CIY[q], dz + CIZ[q]
            inside = near & (x1 * x1 + y1 * y1 + z1 * z1 - rad * rad <= 0)
            kk, jj, ii = np.nonzero(inside)
            for k, j, i in zip(kk, jj, ii):
                x0 = np.array([dx[k, j, i], dy[k, j, i], dz[k, j, i]])
                x1v = x0 + np.array([CIX[q], CIY[q], CIZ[q]])
                # |x1 + (x0 - x1) t|^2 = R^2, alpha = 1 - t
                a = float(np.dot(x0 - x1v, x0 - x1v))
                b = float(np.dot(x1v, x0 - x1v))
                cc = float(np.dot(x1v, x1v) - rad * rad)
                t = (-b + math.sqrt(b * b - a * cc)) / a
                links[(p, int(i + n * (j + n * k)), q)] = 1.0 - t
    return isn, links


def test_links_match_numpy_geometry(engine_lib, oracle_mod):
    n, rad = 32, 4.5
    cfg = box_cfg(engine_lib, n, 5, rad)
    o = oracle_mod.OracleBox(cfg)
    y = np.array([[3.3, 30.1, 16.7], [16.2, 16.9, 0.3], [28.7, 6.25, 9.9],
                  [10.1, 11.2, 24.6], [22.4, 25.8, 27.1]])
    o.release_particles(y)
    isn, links = numpy_links(y, n, rad)
    assert np.array_equal(o.isnodes, isn)
    q, k, j, i = np.nonzero(o.ilink > 0)
    got = {(int(o.mlink[a, b, c, d]), int(d + n * (c + n * b)), int(a + 1)): float(o.alink[a, b, c, d])
           for a, b, c, d in zip(q, k, j, i)}
    assert set(got) == set(links)
    assert max(abs(got[key] - links[key]) for key in got) <= 1e-12
    assert all(0.0 <= v <= 1.0 for v in got.values())


def test_lubrication_equal_and_opposite(engine_lib, oracle_mod):
    n, rad = 40, 4.0
    cfg = box_cfg(engine_lib, n, 4, rad, rhopart=2.5)
    o = oracle_mod.OracleBox(cfg)
    # two close pairs, one across the periodic boundary
    y = np.array([[10.0, 10.0, 10.0], [18.6, 10.4, 10.2], [1.0, 30.0, 20.0], [38.5, 30.2, 20.1]])
    o.release_particles(y)
    o.beads_lubforce()
    fl = o.flubp[:4]
    assert np.abs(fl.sum(axis=0)).max() <= 1e-18
    assert np.abs(fl[0]).max() > 0 and np.abs(fl[2]).max() > 0
    # repulsive: particle 0 pushed away from particle 1 (-x)
    assert fl[0, 0] < 0 < fl[1, 0]


@pytest.mark.timeout(300)
def test_channel_poiseuille(engine_lib, oracle_mod):
    """Halfway bounce-back walls with a constant body force: the steady
    profile is the parabola u(x) = F x (H - x) / (2 nu), H = nx.  With all
    rates equal to 1/tau and tau = 1/2 + sqrt(3/16) the halfway wall sits
    exactly midway between nodes, so the lattice solution is the parabola
    itself (other tau leave a known uniform slip of order (tau - 1/2)^2)."""
    nx, ny, nz = 16, 4, 4
    cfg = box_cfg(engine_lib, preset=capi.LBM_PRESET_CHANNEL, shape=(nx, ny, nz))
    tau = 0.5 + math.sqrt(3.0 / 16.0)
    cfg.visc = (tau - 0.5) / 3.0
    cfg.force_y = 1e-6
    o = oracle_mod.OracleBox(cfg)
    o.macrovar()
    o.step(6000)
    x = np.arange(nx) + 0.5
    uy = o.uy[0, 0, :]
    ref = cfg.force_y * x * (nx - x) / (2 * cfg.visc)
    assert np.abs(uy - ref).max() <= 1e-12 * ref.max()
    assert np.abs(o.ux).max() <= 1e-18 and np.abs(o.uz).max() <= 1e-18


def test_statistics_single_mode():
    """One Fourier mode u_x = A cos(2 pi (k1 y + k2 z) / n): all energy A^2/4
    in shell int(|k| + 1/2), dissipation 2 nu |q|^2 E."""
    from oracle import statistics
    n = 16
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    A, k1, k2 = 0.03, 2, 1
    ux = A * np.cos(2 * np.pi * (k1 * y + k2 * z) / n)
    zero = np.zeros_like(ux)
    ek, dk, out = statistics.spectrum(ux, zero, zero, visc=0.0036)
    shell = int(np.sqrt(k1 * k1 + k2 * k2) + 0.5)
    assert abs(ek[shell - 1] - A * A / 4) < 1e-15
    assert np.abs(np.delete(ek, shell - 1)).max() < 1e-18
    q2 = (2 * np.pi / n) ** 2 * (k1 * k1 + k2 * k2)
    assert abs(dk[shell - 1] - 2 * 0.0036 * q2 * A * A / 4) < 1e-16
    assert abs(out[1] - 0.5 * (ux ** 2).mean()) < 1e-15   # Parseval: E = <u^2>/2
    assert out[0] == int(n / 2 - 1.5)
