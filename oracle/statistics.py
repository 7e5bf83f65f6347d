"""CPU restatement of statistc's spectrum and moments (numpy).

TEST INFRASTRUCTURE ONLY: the GPU statistics entry (lbm_statistics) is
checked against this.  It follows 3DBox_Forced_HI_Turbulence_Moving_Particles_LBM/
saveload.f90:1111-1338 with the wavenumbers of gaussian.f90:40-73 and the
forward transform of mpifft.f90:52-108 (normalised by 1/N per axis):

  E(ik)  = sum over the half spectrum kx >= 0, shell int(|k| + 1/2) = ik,
           of |u^|^2 with the kx = 0 plane weighted 1/2;
  D(ik)  = the same sum of 2 nu |q|^2 |u^|^2, q = 2 pi (kx/nx, ky/ny, kz/nz)
           (the reference keeps integer k and folds (2 pi / n)^2 into dscale);
  ik = 1 .. nek, nek = int(nx/2 - 1.5) (para.f90:83);
  skewness / flatness of statistc, which sums wx^p + wy^p + wx^p
  (saveload.f90:1181-1193) with w_a the spectral derivative d u_a / d x_a
  (the Nyquist wavenumber of each axis dropped, so w_a is real).
Parity unpinned against the reference itself (FFTW 2 and MPI are absent).
"""

from __future__ import annotations

import numpy as np


def _signed(n: int) -> np.ndarray:
    k = np.arange(n)
    return np.where(k <= n // 2, k, k - n)


def spectrum(ux: np.ndarray, uy: np.ndarray, uz: np.ndarray, visc: float):
    """(ek, dk, out) as lbm_statistics returns them; fields are (nz, ny, nx)."""
    nz, ny, nx = ux.shape
    N = nx * ny * nz
    nek = int(nx / 2 - 1.5)
    v = [np.fft.rfftn(u, axes=(0, 1, 2)) / N for u in (ux, uy, uz)]
    kx = np.arange(nx // 2 + 1)[None, None, :]
    ky = _signed(ny)[None, :, None]
    kz = _signed(nz)[:, None, None]
    k2 = kx * kx + ky * ky + kz * kz
    shell = (np.sqrt(k2.astype(np.float64)) + 0.5).astype(np.int64)
    s = sum(np.abs(c) ** 2 for c in v)
    s = np.where(kx == 0, 0.5 * s, s)
    q2 = (2 * np.pi * kx / nx) ** 2 + (2 * np.pi * ky / ny) ** 2 + (2 * np.pi * kz / nz) ** 2
    d = 2.0 * visc * q2 * s
    sh = np.broadcast_to(shell, s.shape)
    ek = np.zeros(nek)
    dk = np.zeros(nek)
    for ik in range(1, nek + 1):
        m = sh == ik
        ek[ik - 1] = s[m].sum()
        dk[ik - 1] = d[m].sum()
    # derivative moments (integer wavenumbers, as statistc; Nyquist dropped)
    kxd = np.where(2 * kx == nx, 0, kx)
    kyd = np.where(2 * ky == ny, 0, ky)
    wx = np.fft.irfftn(1j * np.broadcast_to(kxd, v[0].shape) * v[0] * N, s=(nz, ny, nx), axes=(0, 1, 2))
    wy = np.fft.irfftn(1j * np.broadcast_to(kyd, v[1].shape) * v[1] * N, s=(nz, ny, nx), axes=(0, 1, 2))
    cc2 = ((wx ** 2 + wy ** 2 + wx ** 2) / 3.0).mean()
    cc3 = ((wx ** 3 + wy ** 3 + wx ** 3) / 3.0).mean()
    cc4 = ((wx ** 4 + wy ** 4 + wx ** 4) / 3.0).mean()
    qq = ek.sum()
    out = np.array([nek, qq, dk.sum(), cc3 / cc2 ** 1.5 if cc2 > 0 else 0.0,
                    cc4 / cc2 ** 2 if cc2 > 0 else 0.0, np.sqrt(2.0 * qq / 3.0)])
    return ek, dk, out


def particle_slip(ux, uy, uz, isnodes, ypglb, wp, r_in, r_out, channel=False):
    """w_p minus the mean fluid velocity on the shell r_in <= r <= r_out."""
    nz, ny, nx = ux.shape
    zc, yc, xc = np.meshgrid(np.arange(nz) + 0.5, np.arange(ny) + 0.5, np.arange(nx) + 0.5,
                             indexing="ij")
    out = np.zeros_like(np.asarray(ypglb, dtype=np.float64))
    for p, (x0, y0, z0) in enumerate(ypglb):
        def near(d, n):
            return np.where(d > 0.5 * n, d - n, np.where(d < -0.5 * n, d + n, d))
        dx = (xc - x0) if channel else near(xc - x0, nx)
        dy, dz = near(yc - y0, ny), near(zc - z0, nz)
        r2 = dx * dx + dy * dy + dz * dz
        m = (r2 >= r_in * r_in) & (r2 <= r_out * r_out) & (isnodes < 0)
        cnt = max(int(m.sum()), 1)
        out[p] = np.asarray(wp[p]) - np.array([ux[m].sum(), uy[m].sum(), uz[m].sum()]) / cnt
    return out


def vorticity(ux, uy, uz):
    """vortcalc (saveload.f90:3411-3450): the spectral curl with integer
    wavenumbers, Nyquist modes dropped; fields (nz, ny, nx)."""
    nz, ny, nx = ux.shape
    v = [np.fft.rfftn(u, axes=(0, 1, 2)) for u in (ux, uy, uz)]
    kx = np.arange(nx // 2 + 1)[None, None, :]
    ky = _signed(ny)[None, :, None]
    kz = _signed(nz)[:, None, None]
    kx = np.where(2 * kx == nx, 0, kx)
    ky = np.where(2 * ky == ny, 0, ky)
    kz = np.where(2 * kz == nz, 0, kz)
    wx = 1j * (ky * v[2] - kz * v[1])
    wy = 1j * (kz * v[0] - kx * v[2])
    wz = 1j * (kx * v[1] - ky * v[0])
    return tuple(np.fft.irfftn(w, s=(nz, ny, nx), axes=(0, 1, 2)) for w in (wx, wy, wz))


def rmsstat(ux, uy, uz, isnodes, wp=None, omgp=None):
    """The 36 columns of rms.dat after the time (saveload.f90:1530-1730)."""
    nz, ny, nx = ux.shape
    fl = np.asarray(isnodes) < 0
    nf = int(fl.sum())

    def mean_rms(a, b, c):
        m = [x[fl].sum() / nf for x in (a, b, c)]
        r = [np.sqrt(((x - mx) ** 2)[fl].sum() / nf) for x, mx in zip((a, b, c), m)]
        return m, r

    um, ur = mean_rms(ux, uy, uz)
    om, orr = mean_rms(*vorticity(ux, uy, uz))
    norm = lambda a, b, c: np.sqrt(a * a + b * b + c * c)
    if wp is not None and len(wp):
        wp = np.asarray(wp).reshape(-1, 3)
        omgp = np.asarray(omgp).reshape(-1, 3)
        n = wp.shape[0]
        wm = [wp[:, c].sum() / n for c in range(3)]
        wr = [np.sqrt(((wp[:, c] - wm[c]) ** 2).sum() / n) for c in range(3)]
        pm = [omgp[:, c].sum() / n for c in range(3)]
        pr = [np.sqrt(((omgp[:, c] - pm[c]) ** 2).sum() / n) for c in range(3)]
    else:
        wm = wr = pm = pr = [0.0, 0.0, 0.0]
    velfrms, omgfrms = norm(*ur), norm(*orr)
    return np.array([nf, nf / float(nx ** 3), *um, *ur, velfrms, norm(*um), *wm, *wr, norm(*wr),
                     norm(*wm), *om, *orr, omgfrms / 2.0, norm(*om), *pm, *pr, norm(*pr),
                     norm(pm[0], pm[1], pm[0]), omgfrms ** 2, velfrms ** 2])


def diag(ux, uy, uz, isnodes, wp=None, omgp=None):
    """diag's columns after the time (saveload.f90:1342-1400)."""
    vel = np.sqrt(ux * ux + uy * uy + uz * uz)
    vel = np.where(np.asarray(isnodes) >= 0, 0.0, vel)
    out = [float(vel.max()), 0, 0.0, 0, 0.0]
    if wp is not None and len(wp):
        wm = np.sqrt((np.asarray(wp).reshape(-1, 3) ** 2).sum(axis=1))
        om = np.sqrt((np.asarray(omgp).reshape(-1, 3) ** 2).sum(axis=1))
        out[1:] = [int(np.argmax(wm)) + 1, float(wm.max()), int(np.argmax(om)) + 1, float(om.max())]
    return out


def channel_profiles(rho, ux, uy, uz, isnodes, ustar, visc, fluid_only=False):
    """statistc / statistc2 of the channel (C/saveload.f90:1136-1428); fields
    (nz, ny, nx), rows per x-plane."""
    nz, ny, nx = ux.shape
    ystar = visc / ustar
    rows = []
    fl = np.asarray(isnodes) < 0
    for i in range(1, nx + 1):
        sl = (slice(None), slice(None), i - 1)
        m = fl[sl] if fluid_only else np.ones((nz, ny), dtype=bool)
        cnt = float(m.sum()) if fluid_only else float(ny * nz)
        S = lambda a: a[sl][m].sum()
        u, v, w = S(ux) / cnt / ustar, S(uy) / cnt / ustar, S(uz) / cnt / ustar
        us2 = ustar * ustar
        pm = S(rho) / cnt / us2
        yplus = ((nx - i) + 0.5) / ystar if i > nx // 2 else (i - 0.5) / ystar
        row = [i - 0.5, yplus, u, v, w,
               S(ux * ux) / cnt / us2 - u * u, S(uy * uy) / cnt / us2 - v * v,
               S(uz * uz) / cnt / us2 - w * w,
               S(ux * uz) / cnt / us2 - u * w, S(ux * uy) / cnt / us2 - u * v,
               S(uy * uz) / cnt / us2 - v * w,
               pm, S(rho * rho) / cnt / us2 ** 2 - pm * pm]
        if fluid_only:
            row += [cnt / (ny * nz), 1.0 - cnt / (ny * nz)]
        rows.append(row)
    return np.array(rows)
