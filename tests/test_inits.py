"""Initial conditions made by the engine.

* ``lbm_init_particles``: initpartpos (3DBox.../partlib.f90:1-80, channel
  3DChannel.../partlib.f90:10-24) with the ranpp generator must place the
  spheres bit for bit where the Python restatement ``inputs.initpartpos``
  and the oracle place them.
* ``lbm_init_spectral``: the seeded solenoidal Gaussian field behind
  initpop, made in initvel's steps (3DBox.../initial.f90:55-116): the same
  seed gives the same bits, another seed another field; zero mean, rms
  u_rms, divergence-free, no Nyquist or beyond-nek modes, and every shell's
  energy exactly on the workload's spectrum k^4 exp(-2 (k/k0)^2).
* ``lbm_init_channel``: initvel of the channel program (the log-law mean
  flow, 3DChannel.../initial.f90:57-126) against its numpy restatement.
* ``lbm_initpartvel`` / ``lbm_release_particles``: initpartvel's trilinear
  interpolation of u at the centres (3DBox.../partlib.f90:177-263, 320-831)
  bit for bit against the oracle's restatement (itself pinned bit for bit to
  the reference's Fortran) on the engine's own velocity field, with centres
  in every halo case; the release block (initpartvel, omgp = 0, links) and
  the rejection of centres whose cell leaves the grid.
"""

import numpy as np
import pytest

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("preset,shape,npart,rad", [
    (capi.LBM_PRESET_BOX, (64, 64, 64), 16, 4.5),
    (capi.LBM_PRESET_BOX, (48, 40, 56), 30, 4.0),
    (capi.LBM_PRESET_CHANNEL, (40, 64, 48), 20, 4.0),
])
def test_init_particles_bit_exact(require_gpu, oracle_mod, preset, shape, npart, rad):
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(preset, *shape, npart, rad, 2.5)
    chan = preset == capi.LBM_PRESET_CHANNEL
    ref = inputs.initpartpos(*shape, npart, rad, cfg.mingap, seed=12345, channel=chan,
                             mingap_w=cfg.mingap_w)
    o = oracle_mod.OracleBox(cfg)
    assert o.initpartpos(npart) == 0
    assert np.array_equal(o.ypglb[:npart], ref)
    box = LBMBox(cfg)
    box.init_particles(npart, seed=12345)
    p = box.get_particles()
    assert np.array_equal(p["ypglb"], ref)
    assert not p["wp"].any() and not p["omgp"].any()
    box.close()


def _field(box):
    box.macrovar()
    _, ux, uy, uz = box.get_macro()
    return np.stack([ux, uy, uz])


def test_init_spectral_properties(require_gpu):
    from multiphase_flow_codes_gb300.engine import LBMBox
    from oracle import statistics as ost
    n, k0, urms = 48, 4.0, 0.03
    cfg = capi.config_init(capi.LBM_PRESET_BOX, n, n, n, 0, 4.0, 2.5)
    cfg.forcing = capi.LBM_FORCING_NONE  # macrovar's u is then sum c f, no F/2
    box = LBMBox(cfg)
    box.init_spectral(k0, urms, 54321)
    u1 = _field(box)
    stats = box.statistics()
    box.init_spectral(k0, urms, 54321)
    u2 = _field(box)
    box.init_spectral(k0, urms, 54322)
    u3 = _field(box)
    box.close()
    assert np.array_equal(u1, u2)                      # same seed, same bits
    assert np.abs(u1 - u3).max() > 0.1 * urms          # another seed, another field
    assert np.abs(u1.mean(axis=(1, 2, 3))).max() <= 1e-15
    rms = np.sqrt((u1 ** 2).sum(axis=0).mean() / 3.0)
    assert abs(rms / urms - 1.0) <= 1e-12, rms
    uh = np.fft.rfftn(u1, axes=(1, 2, 3))
    kz = np.fft.fftfreq(n, 1.0 / n)[:, None, None]
    ky = np.fft.fftfreq(n, 1.0 / n)[None, :, None]
    kx = np.arange(n // 2 + 1)[None, None, :]
    kk = np.sqrt(kx * kx + ky * ky + kz * kz + 0.0)
    amp = np.sqrt((np.abs(uh) ** 2).sum(axis=0))
    # divergence-free, relative to |k| |u^|
    div = kx * uh[0] + ky * uh[1] + kz * uh[2]
    assert np.abs(div).max() <= 1e-12 * (kk * amp).max()
    # no Nyquist modes and nothing beyond shell nek
    nek = int(n / 2 - 1.5)
    nyq = (kx == n // 2) | (np.abs(ky) == n // 2) | (np.abs(kz) == n // 2) | ((kk + 0.5).astype(int) > nek)
    assert np.broadcast_to(amp, nyq.shape)[nyq].max() <= 1e-12 * amp.max()
    # every shell on the spectrum: E(ik) / (ik^4 exp(-2 (ik/k0)^2)) is one constant
    ek, _, _ = ost.spectrum(*u1, cfg.visc)
    ik = np.arange(1, nek + 1, dtype=np.float64)
    ratio = ek / (ik ** 4 * np.exp(-2.0 * (ik / k0) ** 2))
    resolved = ek >= 1e-6 * ek.max()  # shells far below the peak carry FFT rounding
    assert resolved.sum() >= 8
    assert np.abs(ratio[resolved] / ratio[0] - 1.0).max() <= 1e-10, ratio
    # and the engine's own statistc agrees with the numpy spectrum
    assert np.abs(stats["ek"] - ek).max() <= 1e-12 * ek.max()


def test_init_channel_loglaw(require_gpu):
    from multiphase_flow_codes_gb300.engine import LBMBox
    from oracle import initial
    for shape in ((64, 24, 16), (45, 20, 12)):
        cfg = capi.config_init(capi.LBM_PRESET_CHANNEL, *shape, 0, 4.0, 1.0)
        cfg.forcing = capi.LBM_FORCING_NONE  # macrovar's u is then sum c f, no F/2
        box = LBMBox(cfg)
        box.init_channel()
        u = _field(box)
        box.close()
        ref = np.stack(initial.channel_loglaw(*shape, cfg.visc))
        assert np.abs(u - ref).max() <= 1e-15 * np.abs(ref).max() + 1e-18, shape
        assert ref[1].max() > 0.0


# centres in every halo case of trilinear on a 24 x 20 x 16 grid: below the
# first and above the last node along each axis, corners, a centre on a node
INTERP = np.array([
    [10.3, 9.7, 7.2], [0.2, 5.3, 6.6], [23.8, 6.1, 3.3], [7.7, 0.3, 8.1], [11.1, 19.6, 9.9],
    [3.3, 4.4, 0.1], [5.5, 7.5, 15.7], [0.1, 0.2, 0.3], [23.9, 19.9, 15.9], [12.0, 0.4, 15.6],
    [6.0, 19.7, 0.2], [2.2, 19.8, 15.8], [4.5, 5.5, 6.5]])


def _interp_box(oracle_mod, preset, precision):
    from multiphase_flow_codes_gb300.engine import LBMBox
    shape = (24, 20, 16)
    cfg = capi.config_init(preset, *shape, len(INTERP), 1.0, 2.5)
    cfg.precision = precision
    box = LBMBox(cfg)
    u = inputs.spectral_velocity(shape[0], 3.0, 0.04, ny=shape[1], nz=shape[2])
    box.initpop(*u)
    box.macrovar()
    _, ux, uy, uz = box.get_macro()
    o = oracle_mod.OracleBox(cfg)
    o.ux[...] = ux
    o.uy[...] = uy
    o.uz[...] = uz
    pos = INTERP.copy()
    if preset == capi.LBM_PRESET_CHANNEL:
        pos[:, 0] = np.clip(pos[:, 0], 0.6, shape[0] - 0.6)
    return box, o, pos


@pytest.mark.parametrize("preset", [capi.LBM_PRESET_BOX, capi.LBM_PRESET_CHANNEL])
@pytest.mark.parametrize("precision", [capi.LBM_PREC_F64, capi.LBM_PREC_F32])
def test_initpartvel_bit_exact(require_gpu, oracle_mod, preset, precision):
    box, o, pos = _interp_box(oracle_mod, preset, precision)
    got = box.initpartvel(pos)
    ref = o.initpartvel(pos)
    assert np.abs(ref).max() > 0
    assert np.array_equal(got, ref), np.abs(got - ref).max()
    assert box.npart == 0  # the context's particles are not changed
    box.close()


def test_release_particles_in_the_flow(require_gpu, oracle_mod):
    """The reference's release block: wp interpolated, omgp = 0, flags and
    links as the oracle builds them for those centres and velocities."""
    from conftest import gpu_links, oracle_links
    box, o, pos = _interp_box(oracle_mod, capi.LBM_PRESET_BOX, capi.LBM_PREC_F64)
    pos = pos[[0, 4, 8]]  # three spheres of radius 1 far apart
    box.release_particles(pos, wp="fluid")
    p = box.get_particles()
    wp = o.initpartvel(pos)
    assert np.array_equal(p["ypglb"], pos)
    assert np.array_equal(p["wp"], wp)
    assert not p["omgp"].any()
    o.release_particles(pos, wp)
    po, no, qo, _ = oracle_links(o)
    pg, ng, qg, _ = gpu_links(box)
    assert np.array_equal(po, pg) and np.array_equal(no, ng) and np.array_equal(qo, qg)
    box.close()


@pytest.mark.parametrize("preset,centre", [
    (capi.LBM_PRESET_CHANNEL, [0.4, 5.0, 5.0]),
    (capi.LBM_PRESET_CHANNEL, [23.5, 5.0, 5.0]),
    (capi.LBM_PRESET_BOX, [24.6, 5.0, 5.0]),
    (capi.LBM_PRESET_BOX, [5.0, -0.6, 5.0]),
    (capi.LBM_PRESET_BOX, [5.0, 5.0, float("nan")]),
])
def test_initpartvel_rejects_cells_off_the_grid(require_gpu, oracle_mod, preset, centre):
    box, o, _ = _interp_box(oracle_mod, preset, capi.LBM_PREC_F64)
    pos = np.array([[5.0, 5.0, 5.0], centre])
    with pytest.raises(capi.LBMError) as e:
        box.initpartvel(pos)
    assert e.value.code == capi.LBM_ERR_ARG
    with pytest.raises(ValueError):
        o.initpartvel(pos)
    assert box.initpartvel(pos[:1]).shape == (1, 3)  # the context stays usable
    box.close()


def test_initpartvel_at_a_released_sphere_gives_its_velocity(require_gpu, oracle_mod):
    """Inside a resolved sphere macrovar sets u = w_p + omega x r
    (3DBox.../collision.f90:278-329), a linear field that trilinear
    interpolation reproduces: u at the centre is w_p."""
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 32, 32, 32, 2, 4.0, 2.5)
    box = LBMBox(cfg)
    u = inputs.spectral_velocity(32, 4.0, 0.03)
    box.initpop(*u)
    box.macrovar()
    pos = np.array([[8.3, 9.1, 20.6], [24.2, 22.7, 7.4]])
    wp = np.array([[0.01, -0.02, 0.005], [-0.015, 0.004, 0.02]])
    om = np.array([[0.002, -0.001, 0.003], [0.0, 0.004, -0.002]])
    box.release_particles(pos, wp, om)
    box.macrovar()
    got = box.initpartvel(pos)
    assert np.abs(got - wp).max() <= 1e-15, np.abs(got - wp).max()
    box.close()
