"""Seeded synthetic inputs: initial velocity fields and particle positions.

The reference starts its runs from a spectral random velocity field
(``initvel``, 3DBox.../initial.f90:55-116, FFTW-based) and draws particle
centres with its own Park-Miller generator (``initpartpos`` / ``ranpp``,
3DBox.../partlib.f90:1-115).  The velocity field here is a seeded
divergence-free Gaussian field with a prescribed energy spectrum (numpy);
the particle positions follow ``initpartpos`` exactly (same generator, same
re-draw of overlapping particles), so they are identical for the same seed.
"""

from __future__ import annotations

import math

import numpy as np

# Park-Miller / Bays-Durham constants (ranpp, partlib.f90:89-92)
_IA, _IM, _IQ, _IR, _NTAB = 16807, 2147483647, 127773, 2836, 32
_NDIV = 1 + (_IM - 1) // _NTAB
_AM = 1.0 / _IM
_RNMX = 1.0 - 1.2e-7


class Ran1:
    """The ``ranpp``/``ranff`` generator (Numerical Recipes ran1).

    All integer arithmetic stays inside int32 range, so Python ints
    reproduce the Fortran results exactly."""

    def __init__(self, seed: int):
        self.idum = -abs(int(seed))
        self.iy = 0
        self.iv = [0] * _NTAB

    def __call__(self) -> float:
        if self.idum <= 0 or self.iy == 0:
            self.idum = max(-self.idum, 1)
            for j in range(_NTAB + 8, 0, -1):
                k = self.idum // _IQ  # idum > 0 here, so floor == Fortran truncation
                self.idum = _IA * (self.idum - k * _IQ) - _IR * k
                if self.idum < 0:
                    self.idum += _IM
                if j <= _NTAB:
                    self.iv[j - 1] = self.idum
            self.iy = self.iv[0]
        k = self.idum // _IQ  # idum > 0 here, so floor == Fortran truncation
        self.idum = _IA * (self.idum - k * _IQ) - _IR * k
        if self.idum < 0:
            self.idum += _IM
        j = self.iy // _NDIV
        self.iy = self.iv[j]
        self.iv[j] = self.idum
        return min(_AM * float(self.iy), _RNMX)


def _near(c: float, p: float, n: int, nh: int) -> float:
    if c - p > nh:
        c = c - n
    if c - p < -nh:
        c = c + n
    return c


def initpartpos(nx: int, ny: int, nz: int, npart: int, rad: float, mingap: float = 2.0,
                seed: int = 12345, channel: bool = False, mingap_w: float = 2.0,
                max_rounds: int = 100000) -> np.ndarray:
    """Particle centres as ``initpartpos`` draws them: uniform in the box
    (the channel keeps ``rad + mingap_w`` from the x walls), re-drawing every
    particle that comes within ``mingap`` of a later one (``ovlpchk`` with
    ``istep00 = 0``, partlib.f90:118-171).  Returns ``(npart, 3)``."""
    rng = Ran1(seed)
    y = np.zeros((npart, 3))
    flag = [1] * npart
    radpgap = rad + mingap_w
    nxh, nyh, nzh = nx // 2, ny // 2, nz // 2
    for _ in range(max_rounds):
        for ip in range(npart):
            if flag[ip] > 0:
                if channel:
                    y[ip, 0] = radpgap + (float(nx) - 2.0 * radpgap) * rng()
                else:
                    y[ip, 0] = float(nx) * rng()
                y[ip, 1] = float(ny) * rng()
                y[ip, 2] = float(nz) * rng()
        flag = [0] * npart
        for idp in range(npart - 1):
            xc, yc, zc = y[idp]
            for ii in range(idp + 1, npart):
                xb, yb, zb = y[ii]
                if not channel:
                    xb = _near(xb, xc, nx, nxh)
                yb = _near(yb, yc, ny, nyh)
                zb = _near(zb, zc, nz, nzh)
                dx, dy, dz = xc - xb, yc - yb, zc - zb
                dist = math.sqrt(dx * dx + dy * dy + dz * dz)
                if dist - 2.0 * rad - mingap < 0.0:
                    flag[idp] = 1
                    break
        if not any(flag):
            return y
    raise RuntimeError("could not place particles without overlap")


def spectral_velocity(n: int, k0: float, urms: float, seed: int = 54321,
                      ny: int | None = None, nz: int | None = None):
    """Seeded solenoidal Gaussian velocity field with energy spectrum
    E(k) ~ k^4 exp(-2 (k/k0)^2), rescaled to a per-component rms ``urms``.

    Returns (ux, uy, uz), each ``(nz, ny, nx)`` float64, zero mean."""
    nx = n
    ny = ny or n
    nz = nz or n
    rng = np.random.default_rng(seed)
    kz = np.fft.fftfreq(nz) * nz
    ky = np.fft.fftfreq(ny) * ny
    kx = np.fft.rfftfreq(nx) * nx
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    K2 = KX * KX + KY * KY + KZ * KZ
    shape = (3,) + K2.shape
    c = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    kv = np.stack([KX, KY, KZ])
    K2s = np.where(K2 == 0, 1.0, K2)
    div = (kv * c).sum(axis=0) / K2s
    c = c - kv * div
    K = np.sqrt(K2)
    Ek = K ** 4 * np.exp(-2.0 * (K / k0) ** 2)
    amp = np.sqrt(Ek / np.where(K2 == 0, 1.0, K2))
    amp[K2 == 0] = 0.0
    c = c * amp
    u = np.fft.irfftn(c, s=(nz, ny, nx), axes=(1, 2, 3))
    u -= u.mean(axis=(1, 2, 3), keepdims=True)
    rms = math.sqrt(float((u * u).sum(axis=0).mean()) / 3.0)
    u *= urms / rms
    return u[0].copy(), u[1].copy(), u[2].copy()
