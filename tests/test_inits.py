"""Initial conditions made by the engine.

* ``lbm_init_particles``: initpartpos (3DBox.../partlib.f90:1-80, channel
  3DChannel.../partlib.f90:10-24) with the ranpp generator must place the
  spheres bit for bit where the Python restatement ``inputs.initpartpos``
  and the oracle place them.
* ``lbm_init_spectral``: the seeded solenoidal Gaussian field behind
  initpop: the same seed gives the same bits, another seed another field;
  zero mean, per-component rms u_rms, divergence-free, and the energy in
  the spectrum's peak shells well above the far tail.
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
    n, k0, urms = 48, 4.0, 0.03
    cfg = capi.config_init(capi.LBM_PRESET_BOX, n, n, n, 0, 4.0, 2.5)
    box = LBMBox(cfg)
    box.init_spectral(k0, urms, 54321)
    u1 = _field(box)
    box.init_spectral(k0, urms, 54321)
    u2 = _field(box)
    box.init_spectral(k0, urms, 54322)
    u3 = _field(box)
    box.close()
    assert np.array_equal(u1, u2)                      # same seed, same bits
    assert np.abs(u1 - u3).max() > 0.1 * urms          # another seed, another field
    assert np.abs(u1.mean(axis=(1, 2, 3))).max() <= 1e-13
    rms = np.sqrt((u1 ** 2).mean(axis=(1, 2, 3)))
    assert np.abs(rms / urms - 1.0).max() <= 1e-12, rms
    # divergence in spectral space, relative to |k| |u^|
    uh = np.fft.rfftn(u1, axes=(1, 2, 3))
    kz = np.fft.fftfreq(n, 1.0 / n)[:, None, None]
    ky = np.fft.fftfreq(n, 1.0 / n)[None, :, None]
    kx = np.arange(n // 2 + 1)[None, None, :]
    ny_ok = (np.abs(kz) < n // 2) & (np.abs(ky) < n // 2) & (kx < n // 2)
    div = kx * uh[0] + ky * uh[1] + kz * uh[2]
    kk = np.sqrt(kx * kx + ky * ky + kz * kz + 0.0)
    mag = kk * np.sqrt((np.abs(uh) ** 2).sum(axis=0))
    assert (np.abs(div)[ny_ok]).max() <= 1e-10 * mag.max()
    # spectrum shape E(k) ~ k^4 exp(-2 (k/k0)^2): the peak shells (k near k0)
    # hold far more energy than shells at 3 k0
    e = (np.abs(uh) ** 2).sum(axis=0)
    shell = (kk + 0.5).astype(int)
    ek = np.bincount(shell.ravel(), weights=e.ravel(), minlength=n)
    assert ek[int(k0)] > 1e3 * ek[int(3 * k0)]
    assert ek[0] <= 1e-20 * ek.max()
