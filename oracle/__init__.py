"""CPU oracle: ctypes wrapper of the C++ restatement in lbm_oracle.cpp.

TEST INFRASTRUCTURE ONLY.  The parity tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` compare the engine with it; the engine
never calls it.

Parity pinned against the reference itself: the reference (Fortran + MPI +
FFTW 2, no Fortran compiler here) is translated to C++ by ``oracle/fortran``
and run on one process (``oracle.refrun``); tests/test_reference_pin.py and
tests/test_reference_golden.py hold this restatement to that run.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liblbm_oracle.so"

_lib = None


def build(force: bool = False) -> Path:
    src = HERE / "lbm_oracle.cpp"
    hdr = HERE.parent / "include" / "lbm.h"
    if force or not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def build_reference() -> dict:
    """The reference's own programs, translated and compiled into
    oracle/_ref/ (where its sources or the generated translation exist)."""
    from .fortran import build as rbuild
    return rbuild.build_all()


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.c_void_p]
        L.orc_destroy.argtypes = [P]
        L.orc_field.restype = P
        L.orc_field.argtypes = [P, C.c_char_p]
        for name in ("orc_forcing", "orc_collision_mrt", "orc_beads_collision", "orc_streaming",
                     "orc_beads_lubforce", "orc_beads_move", "orc_beads_links", "orc_beads_filling",
                     "orc_macrovar", "orc_rhoupdat", "orc_initpop"):
            getattr(L, name).argtypes = [P]
            getattr(L, name).restype = None
        L.orc_beads_redistribute.argtypes = [P]
        L.orc_beads_redistribute.restype = C.c_int
        L.orc_error.argtypes = [P]
        L.orc_npart.argtypes = [P]
        L.orc_initpartpos.argtypes = [P, C.c_int]
        L.orc_initpartvel.argtypes = [P, C.c_int]
        L.orc_initpartvel.restype = C.c_int
        L.orc_release.argtypes = [P, C.c_int]
        L.orc_release.restype = None
        L.orc_restore.argtypes = [P, C.c_int]
        L.orc_restore.restype = None
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = None
        L.orc_step.argtypes = [P, C.c_int]
        L.orc_ran1_sequence.argtypes = [C.c_int32, C.c_int, C.POINTER(C.c_double)]
        L.orc_ran1_sequence.restype = None
        L.orc_ran1_state.argtypes = [C.c_int32, C.c_int]
        L.orc_ran1_state.restype = C.c_int32
        _lib = L
    return _lib


def set_threads(n: int):
    """Host threads of the restatement's parallel loops."""
    lib().orc_set_threads(int(n))


def ran1_sequence(seed: int, n: int) -> np.ndarray:
    out = np.empty(n)
    lib().orc_ran1_sequence(seed, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def ran1_state(seed: int, n: int) -> int:
    """The Park-Miller state after n ran1 draws from seed (see lbm_oracle.cpp)."""
    return int(lib().orc_ran1_state(seed, n))


class OracleBox:
    """The reference's var_inc state on the CPU, with its subroutines.

    Node arrays are (nz, ny, nx) views, populations (19, nz, ny, nx),
    dense link arrays (18, nz, ny, nx) (ilink(ipop) at index ipop-1),
    particle vectors (npart_max, 3).  Views alias the C++ state."""

    NODE = ("rho", "ux", "uy", "uz", "fx", "fy", "fz")
    INODE = ("ibnodes", "isnodes", "ibnodes0", "isnodes0")
    PART = ("ypglb", "ypglbp", "wp", "wpp", "omgp", "omgpp", "dwdt", "domgdt", "forcep",
            "forcepp", "torqp", "torqpp", "thetap", "fHIp", "flubp")

    def __init__(self, cfg):
        self._cfg = cfg
        self.nx, self.ny, self.nz = cfg.nx, cfg.ny, cfg.nz
        self._L = lib()
        self._h = self._L.orc_create(C.addressof(cfg))
        self.npmax = max(cfg.npart_max, 0)

    def close(self):
        if self._h:
            self._L.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _view(self, name: str, dtype, shape):
        p = self._L.orc_field(self._h, name.encode())
        if not p:
            raise KeyError(name)
        n = int(np.prod(shape))
        ct = C.c_double if dtype == np.float64 else C.c_int32
        arr = np.ctypeslib.as_array((ct * n).from_address(p))
        return arr.reshape(shape)

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        sh = (self.nz, self.ny, self.nx)
        if name == "f":
            return self._view("f", np.float64, (19,) + sh)
        if name in self.NODE:
            return self._view(name, np.float64, sh)
        if name in self.INODE:
            return self._view(name, np.int32, sh)
        if name in ("ilink", "mlink"):
            return self._view(name, np.int32, (18,) + sh)
        if name == "alink":
            return self._view(name, np.float64, (18,) + sh)
        if name in self.PART:
            return self._view(name, np.float64, (self.npmax, 3))
        if name in ("b1r", "b2r", "b3r", "a1r", "a2r", "a3r"):
            return self._view(name, np.float64, (150,))
        if name == "ivf":
            return self._view(name, np.int32, (32,))
        if name in ("iseedf", "iyf"):
            return int(self._view(name, np.int32, (1,))[0])
        raise AttributeError(name)

    @property
    def error(self) -> int:
        return self._L.orc_error(self._h)

    # reference subroutines
    def FORCING(self): self._L.orc_forcing(self._h)
    def collision_MRT(self): self._L.orc_collision_mrt(self._h)
    def beads_collision(self): self._L.orc_beads_collision(self._h)
    def streaming(self): self._L.orc_streaming(self._h)
    def beads_lubforce(self): self._L.orc_beads_lubforce(self._h)
    def beads_move(self): self._L.orc_beads_move(self._h)
    def beads_redistribute(self) -> int: return self._L.orc_beads_redistribute(self._h)
    def beads_links(self): self._L.orc_beads_links(self._h)
    def beads_filling(self): self._L.orc_beads_filling(self._h)
    def macrovar(self): self._L.orc_macrovar(self._h)
    def rhoupdat(self): self._L.orc_rhoupdat(self._h)

    def initpop(self, ux, uy, uz):
        self.ux[...] = ux
        self.uy[...] = uy
        self.uz[...] = uz
        self._L.orc_initpop(self._h)

    def initpartpos(self, npart: int) -> int:
        return self._L.orc_initpartpos(self._h, npart)

    def initpartvel(self, ypglb) -> np.ndarray:
        """wp at the given centres from the current ux, uy, uz (initpartvel,
        B/partlib.f90:177-263); returns wp (npart, 3).  ValueError for a
        centre whose cell leaves the grid (a channel's: within 0.5 of a
        wall)."""
        y = np.asarray(ypglb, dtype=np.float64).reshape(-1, 3)
        n = y.shape[0]
        self.ypglb[:n] = y
        bad = self._L.orc_initpartvel(self._h, n)
        if bad >= 0:
            raise ValueError(f"particle {bad}: centre outside the interpolation range")
        return self.wp[:n].copy()

    def release_particles(self, ypglb, wp=None, omgp=None):
        y = np.asarray(ypglb, dtype=np.float64).reshape(-1, 3)
        n = y.shape[0]
        self.ypglb[:n] = y
        self.wp[:n] = 0.0 if wp is None else wp
        self.omgp[:n] = 0.0 if omgp is None else omgp
        self._L.orc_release(self._h, n)

    def restore_particles(self, state: dict):
        """Restart: set every (3, npart) particle vector (names as var_inc),
        then rebuild the flags and links (B/main.f90:129-132)."""
        n = int(np.asarray(state["ypglb"]).reshape(-1, 3).shape[0])
        for k in self.PART:
            if k in state:
                getattr(self, k)[:n] = np.asarray(state[k]).reshape(n, 3)
        self._L.orc_restore(self._h, n)

    def set_forcing_state(self, iseedf: int, iyf: int, ivf, b):
        self._view("iseedf", np.int32, (1,))[0] = iseedf
        self._view("iyf", np.int32, (1,))[0] = iyf
        self.ivf[:] = np.asarray(ivf, dtype=np.int32)
        b = np.asarray(b, dtype=np.float64).reshape(450)
        self.b1r[:] = b[:150]
        self.b2r[:] = b[150:300]
        self.b3r[:] = b[300:]

    def step(self, nsteps: int = 1) -> int:
        return self._L.orc_step(self._h, nsteps)
