"""ctypes binding of ``liblbm_gb300.so`` (the C ABI declared in include/lbm.h).

Loading fails loudly: there is no CPU fallback behind this package.  The
library must have been built (``multiphase_flow_codes_gb300.build.build()``)
for the engine to run, and every compute entry point needs a CUDA device.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "liblbm_gb300.so"

# status codes (lbm.h)
LBM_OK = 0
LBM_ERR_ARG = -1
LBM_ERR_CUDA = -2
LBM_ERR_OVERLAP = -3
LBM_ERR_CAPACITY = -4
LBM_ERR_ALPHA = -5
LBM_ERR_NONFINITE = -6
LBM_ERR_TIMEOUT = -7
LBM_ERR_STATE = -8
LBM_ERR_NOMEM = -9

LBM_PREC_F64, LBM_PREC_F32 = 0, 1
LBM_BC_PERIODIC, LBM_BC_XWALLS = 0, 1
LBM_FORCING_NONE, LBM_FORCING_STOCHASTIC, LBM_FORCING_CONSTANT = 0, 1, 2
LBM_PRESET_BOX, LBM_PRESET_CHANNEL = 0, 1
LBM_VARIANT_DIRECT, LBM_VARIANT_STAGED, LBM_VARIANT_STAGED_X2 = 1, 2, 3
LBM_SUMS_FLOAT, LBM_SUMS_FIXED, LBM_SUMS_INTEGER = 0, 1, 2


class lbm_config(C.Structure):
    """Mirror of ``struct lbm_config`` in include/lbm.h (field order matters)."""

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

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("reserved")}


class LBMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (code {code})")
        self.code = code


_lib = None

_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)

# symbol -> (restype, argtypes); every symbol declared in include/lbm.h
SIGNATURES = {
    "lbm_config_init": (C.c_int, [C.POINTER(lbm_config), C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_int, C.c_double, C.c_double]),
    "lbm_create": (C.c_int, [C.POINTER(lbm_config), C.POINTER(_P)]),
    "lbm_destroy": (C.c_int, [_P]),
    "lbm_last_error": (C.c_char_p, [_P]),
    "lbm_version": (C.c_int, []),
    "lbm_footprint": (C.c_int, [C.POINTER(lbm_config), C.POINTER(C.c_uint64)]),
    "lbm_set_stream": (C.c_int, [_P, _P]),
    "lbm_synchronize": (C.c_int, [_P]),
    "lbm_upload_f": (C.c_int, [_P, _D]),
    "lbm_download_f": (C.c_int, [_P, _D]),
    "lbm_upload_f_soa": (C.c_int, [_P, _D]),
    "lbm_download_f_soa": (C.c_int, [_P, _D]),
    "lbm_initpop": (C.c_int, [_P, _D, _D, _D]),
    "lbm_download_macro": (C.c_int, [_P, _D, _D, _D, _D]),
    "lbm_download_force": (C.c_int, [_P, _D, _D, _D]),
    "lbm_upload_particles": (C.c_int, [_P, C.c_int, _D, _D, _D]),
    "lbm_initpartvel": (C.c_int, [_P, C.c_int, _D, _D]),
    "lbm_release_particles": (C.c_int, [_P, C.c_int, _D]),
    "lbm_download_particles": (C.c_int, [_P, _D, _D, _D, _D, _D, _D]),
    "lbm_download_flags": (C.c_int, [_P, _I, _I]),
    "lbm_download_links": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_int64), _I, _I, _I, _D]),
    "lbm_forcing_state": (C.c_int, [_P, C.c_int, _I, _I, _I, _D]),
    "lbm_forcing": (C.c_int, [_P]),
    "lbm_collision_mrt": (C.c_int, [_P]),
    "lbm_beads_collision": (C.c_int, [_P]),
    "lbm_streaming": (C.c_int, [_P]),
    "lbm_beads_lubforce": (C.c_int, [_P]),
    "lbm_beads_move": (C.c_int, [_P]),
    "lbm_beads_redistribute": (C.c_int, [_P]),
    "lbm_beads_links": (C.c_int, [_P]),
    "lbm_beads_filling": (C.c_int, [_P]),
    "lbm_macrovar": (C.c_int, [_P]),
    "lbm_rhoupdat": (C.c_int, [_P]),
    "lbm_rmsstat": (C.c_int, [_P, _D]),
    "lbm_diag": (C.c_int, [_P, _D]),
    "lbm_channel_profiles": (C.c_int, [_P, C.c_int, C.c_double, _D]),
    "lbm_particle_state": (C.c_int, [_P, C.c_int, C.c_int, _D, C.POINTER(C.c_int32)]),
    "lbm_prerelax": (C.c_int, [_P, C.c_double, C.c_int, C.POINTER(C.c_int), _D]),
    "lbm_step": (C.c_int, [_P, C.c_int]),
    "lbm_mass_momentum": (C.c_int, [_P, _D]),
    "lbm_profile": (C.c_int, [_P, C.c_int]),
    "lbm_profile_read": (C.c_int, [_P, C.c_int, _D, C.POINTER(C.c_int64)]),
    "lbm_kernel_launches": (C.c_int64, []),
    "lbm_mass_momentum_noalloc": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P]),
    "lbm_fma_throughput": (C.c_int, [C.c_int, _D]),
    "lbm_set_variant": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int]),
    "lbm_set_sums": (C.c_int, [_P, C.c_int]),
    "lbm_get_sums": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "lbm_get_variant": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int)]),
    "lbm_autotune": (C.c_int, [_P, C.c_int, _D]),
    "lbm_statistics": (C.c_int, [_P, C.c_int, _D, _D, _D]),
    "lbm_init_spectral": (C.c_int, [_P, C.c_double, C.c_double, C.c_uint64]),
    "lbm_init_particles": (C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    "lbm_place_particles": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P]),
    "lbm_init_channel": (C.c_int, [_P]),
    "lbm_summary": (C.c_int, [_P, _D]),
    "lbm_particle_slip": (C.c_int, [_P, C.c_double, C.c_double, _D]),
    "lbm_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "lbm_batch_destroy": (C.c_int, [_P]),
    "lbm_batch_last_error": (C.c_char_p, [_P]),
    "lbm_batch_step": (C.c_int, [_P, C.c_int, C.c_int]),
    "lbm_batch_synchronize": (C.c_int, [_P]),
    "lbm_batch_wait": (C.c_int, [_P]),
    "lbm_batch_set_schedule": (C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    "lbm_batch_get_schedule": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]),
    "lbm_batch_autotune": (C.c_int, [_P, C.c_int, _D]),
    "lbm_batch_nodes": (C.c_int64, [_P]),
    "lbm_batch_set_stream": (C.c_int, [_P, _P]),
    "lbm_server_create": (C.c_int, [C.c_uint64, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "lbm_server_submit": (C.c_int, [_P, _P, C.POINTER(C.c_int64)]),
    "lbm_server_result": (C.c_int, [_P, C.c_int64, _P]),
    "lbm_server_wait": (C.c_int, [_P, C.c_int64, C.c_double]),
    "lbm_server_stats": (C.c_int, [_P, _D]),
    "lbm_server_destroy": (C.c_int, [_P]),
    "lbm_server_take": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_void_p)]),
    "lbm_get_config": (C.c_int, [_P, C.POINTER(lbm_config)]),
    "lbm_particle_count": (C.c_int, [_P, C.POINTER(C.c_int)]),
}

PHASES = ("stream_collide", "bounce", "particles", "links", "filling", "forcing")


def lib() -> C.CDLL:
    """Load the engine library (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA engine first "
                "(python -m multiphase_flow_codes_gb300.build)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and (a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"])
    return a.ctypes.data_as(_D)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and (a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"])
    return a.ctypes.data_as(_I)


def config_init(preset: int, nx: int, ny: int, nz: int, npart: int, rad: float,
                rhopart: float) -> lbm_config:
    cfg = lbm_config()
    rc = lib().lbm_config_init(C.byref(cfg), preset, nx, ny, nz, npart, rad, rhopart)
    if rc != LBM_OK:
        raise LBMError(rc, "lbm_config_init rejected the arguments")
    return cfg


def place_particles(cfg: lbm_config, npart: int, seed: int, max_rounds: int = 0) -> np.ndarray:
    """initpartpos on the host (lbm_place_particles): centres ``(npart, 3)``."""
    y = np.zeros((npart, 3), dtype=np.float64)
    rc = lib().lbm_place_particles(C.byref(cfg), npart, seed, max_rounds,
                                   y.ctypes.data_as(C.c_void_p))
    if rc != LBM_OK:
        raise LBMError(rc, "lbm_place_particles")
    return y


def footprint(cfg: lbm_config) -> int:
    out = C.c_uint64(0)
    rc = lib().lbm_footprint(C.byref(cfg), C.byref(out))
    if rc != LBM_OK:
        raise LBMError(rc, "lbm_footprint")
    return int(out.value)
