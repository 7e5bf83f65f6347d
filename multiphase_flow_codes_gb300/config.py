"""Workload presets: the five benchmark configurations of this path.

Each preset returns an ``lbm_config`` (reference defaults from
``lbm_config_init``) plus the seeded initial condition recipe.  Values follow
the reference where the workload does not state them: stochastic forcing
with the reference amplitude constants (var = 447.31 (vscale tscale)^2,
tf = 0.038/tscale, vscale = 2.037183272e-3, gaussian.f90:196-199,
para.f90:37), MRT rates of MRTtype 1 for the box and all-1/tau (MRTtype 2)
for the channel, lubrication constants of para.f90:244-245.
"""

from __future__ import annotations

from dataclasses import dataclass, field

from . import _capi as capi


@dataclass
class Workload:
    name: str
    cfg: capi.lbm_config
    npart: int
    k0: float
    urms: float
    steps: int
    flow_seed: int = 54321      # var_inc.f90:19
    particle_seed: int = 12345  # para.f90:247
    extra: dict = field(default_factory=dict)


def box(n: int, npart: int, rad: float, rhopart: float, k0: float, urms: float, steps: int,
        precision: int = capi.LBM_PREC_F64, name: str = "", ny: int | None = None,
        nz: int | None = None) -> Workload:
    cfg = capi.config_init(capi.LBM_PRESET_BOX, n, ny or n, nz or n, npart, rad, rhopart)
    cfg.visc = 0.0036  # tau = 3 visc + 0.5 = 0.5108
    cfg.precision = precision
    return Workload(name or f"box{n}", cfg, npart, k0, urms, steps)


def channel(nx: int, ny: int, nz: int, npart: int, rad: float = 4.0, rhopart: float = 1.0,
            steps: int = 200, precision: int = capi.LBM_PREC_F32, name: str = "") -> Workload:
    cfg = capi.config_init(capi.LBM_PRESET_CHANNEL, nx, ny, nz, npart, rad, rhopart)
    cfg.precision = precision
    return Workload(name or f"channel{nx}x{ny}x{nz}", cfg, npart, 4.0, 0.0, steps)


def box64_p16_f64() -> Workload:
    """64^3 periodic box, 16 spheres R = 4.5, density ratio 5, u_rms 0.03,
    spectrum peak k0 = 4, 1000 steps, FP64."""
    return box(64, 16, 4.5, 5.0, 4.0, 0.03, 1000, name="box64_p16_f64")


def box256_p1000_f64() -> Workload:
    """256^3 periodic box, 1000 spheres R = 4, density ratio 2.5, u_rms 0.04,
    k0 = 8, 2000 steps, FP64: the roofline workload."""
    return box(256, 1000, 4.0, 2.5, 8.0, 0.04, 2000, name="box256_p1000_f64")


def box256_p1000_f32() -> Workload:
    """The 256^3, 1000-sphere box with populations stored and collided in FP32."""
    w = box(256, 1000, 4.0, 2.5, 8.0, 0.04, 2000, precision=capi.LBM_PREC_F32,
            name="box256_p1000_f32")
    return w
