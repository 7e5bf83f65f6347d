"""Configuration of the CPU restatement, independent of the engine library.

TEST INFRASTRUCTURE ONLY.  The CPU-timed reference leg of ``bench.py`` must
not load the engine's shared library, so the oracle builds its own copy of
the parameter block that ``include/lbm.h`` declares (``struct lbm_config``)
from the reference's constants:

* rates and seeds: ``3DBox.../para.f90:20`` (iseedf 232300), ``:37``
  (vscale), ``:96`` (MRTtype 1), ``:237-247`` (gscale, rhog, stiffness,
  iseedp 12345); lubrication scale ``partlib.f90:2260``;
* the channel: ``3DChannel.../para.f90:14-19`` (Rstar 180, ustar, force),
  ``:67`` (MRTtype 2), ``partlib.f90:2409`` (volp * force_in_y in y).

A CPU test checks that every field equals what the engine's
``lbm_config_init`` writes for the same arguments.
"""

from __future__ import annotations

import ctypes as C
import math

PRESET_BOX, PRESET_CHANNEL = 0, 1
PREC_F64, PREC_F32 = 0, 1
BC_PERIODIC, BC_XWALLS = 0, 1
FORCING_NONE, FORCING_STOCHASTIC, FORCING_CONSTANT = 0, 1, 2


class lbm_config(C.Structure):
    """``struct lbm_config`` of include/lbm.h (field order and types)."""

    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("npart_max", C.c_int32), ("mrt_type", C.c_int32), ("boundary", C.c_int32),
        ("forcing", C.c_int32), ("precision", C.c_int32), ("iseedf", C.c_int32),
        ("iseedp", C.c_int32), ("link_capacity", C.c_int32), ("reserved_i", C.c_int32 * 5),
        ("visc", C.c_double), ("rho0", C.c_double), ("rhopart", C.c_double), ("rad", C.c_double),
        ("mingap", C.c_double), ("mingap_w", C.c_double), ("vscale", C.c_double),
        ("force_y", C.c_double), ("fpc", C.c_double), ("stf0", C.c_double), ("stf1", C.c_double),
        ("stf0_w", C.c_double), ("stf1_w", C.c_double), ("body_force_y", C.c_double),
        ("reserved_d", C.c_double * 6),
    ]


def config_init(preset: int, nx: int, ny: int, nz: int, npart: int, rad: float,
                rhopart: float) -> lbm_config:
    """The reference's parameters for an nx*ny*nz box or x-walled channel."""
    if nx < 4 or ny < 4 or nz < 4 or npart < 0 or preset not in (PRESET_BOX, PRESET_CHANNEL):
        raise ValueError("config_init: bad arguments")
    c = lbm_config()
    pi = 4.0 * math.atan(1.0)
    c.nx, c.ny, c.nz = nx, ny, nz
    c.npart_max = npart
    c.precision = PREC_F64
    c.iseedf = 232300
    c.iseedp = 12345
    c.visc = 0.0036
    c.rho0 = 1.0
    c.rhopart = rhopart
    c.rad = rad
    c.mingap = 2.0
    c.mingap_w = 2.0
    c.vscale = 2.037183272e-3
    c.stf0, c.stf1 = 0.025, 0.002
    c.stf0_w, c.stf1_w = 0.025, 0.002
    volp = 4.0 / 3.0 * pi * (rad * rad * rad)
    if preset == PRESET_BOX:
        c.mrt_type = 1
        c.boundary = BC_PERIODIC
        c.forcing = FORCING_STOCHASTIC
        gscale = 10000.0 / 4.0
        c.fpc = volp * c.rho0 * 9.8 / gscale
        rhog = 0.0
        c.body_force_y = -(volp * rhog)
    else:
        c.mrt_type = 2
        c.boundary = BC_XWALLS
        c.forcing = FORCING_CONSTANT
        rstar = 180.0
        ustar = 2.0 * rstar * c.visc / float(nx)
        force_in_y = 2.0 * c.rho0 * ustar * ustar / float(nx)
        ystar = c.visc / ustar
        c.force_y = force_in_y * 1.0
        g_lbm = ustar * ustar / ystar
        c.fpc = volp * c.rho0 * g_lbm
        c.body_force_y = volp * force_in_y
    return c


# Benchmark workloads by name: (preset, edge, particles, radius, density
# ratio, spectrum peak k0, u_rms).
WORKLOADS = {
    "box64_p16_f64": (PRESET_BOX, 64, 16, 4.5, 5.0, 4.0, 0.03),
    "box256_p1000_f64": (PRESET_BOX, 256, 1000, 4.0, 2.5, 8.0, 0.04),
    "box256_p1000_f32": (PRESET_BOX, 256, 1000, 4.0, 2.5, 8.0, 0.04),
}


def workload_config(name: str):
    """(lbm_config, npart, k0, u_rms) of a named workload, FP64 populations."""
    preset, n, npart, rad, ratio, k0, urms = WORKLOADS[name]
    c = config_init(preset, n, n, n, npart, rad, ratio)
    return c, npart, k0, urms
