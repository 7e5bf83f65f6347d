"""The reference's own Fortran, translated and run on the CPU (test infrastructure).

``RefProgram`` loads a library built by ``oracle/fortran/build.py`` from the
reference's source files and exposes its module variables (var_inc) by name
as numpy views in Fortran order, plus its argument-free subroutines by name.
Tests drive it in the order of the reference's main program to pin the C++
restatement (``oracle.OracleBox``) against the reference itself.  Nothing in
the engine uses it.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from .fortran import build as rbuild

_DT = {0: np.int32, 1: np.int64, 2: np.float64, 3: np.complex128, 4: np.bool_}
_CT = {0: C.c_int32, 1: C.c_int64, 2: C.c_double, 4: C.c_bool}


def available(prog: str = "box") -> bool:
    try:
        return rbuild.build(prog) is not None
    except Exception:
        return False


class RefProgram:
    """One translated reference program (one process, single domain).  A
    library holds one program state per process, so one instance per
    process at a time."""

    _loaded = {}

    def __init__(self, prog: str = "box", overrides: dict | None = None):
        lib = rbuild.build(prog)
        if lib is None:
            raise RuntimeError(f"the reference program {prog!r} is not available")
        if prog not in RefProgram._loaded:
            L = C.CDLL(str(lib))
            ns = f"ref_{prog}"
            for fn, res, args in (("_error", C.c_char_p, []),
                                  ("_override", None, [C.c_char_p, C.c_double]),
                                  ("_clear_overrides", None, []),
                                  ("_init", C.c_int, []),
                                  ("_call", C.c_int, [C.c_char_p]),
                                  ("_var", C.c_int, [C.c_char_p, C.POINTER(C.c_int),
                                                     C.POINTER(C.c_int),
                                                     C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                                     C.POINTER(C.c_void_p)])):
                f = getattr(L, ns + fn)
                f.restype = res
                f.argtypes = args
            RefProgram._loaded[prog] = (L, ns)
        self._L, self._ns = RefProgram._loaded[prog]
        self._fn = lambda s: getattr(self._L, self._ns + s)  # noqa: E731
        self._fn("_clear_overrides")()
        for k, v in (overrides or {}).items():
            self._fn("_override")(k.encode(), float(v))
        if self._fn("_init")() != 0:
            raise RuntimeError(self.error())

    def error(self) -> str:
        return self._fn("_error")().decode()

    def call(self, name: str):
        rc = self._fn("_call")(name.lower().encode())
        if rc != 0:
            raise RuntimeError(f"{name}: {self.error()}")

    def _info(self, name: str):
        t, r = C.c_int(), C.c_int()
        lb = (C.c_int64 * 7)()
        ub = (C.c_int64 * 7)()
        p = C.c_void_p()
        rc = self._fn("_var")(name.lower().encode(), C.byref(t), C.byref(r), lb, ub, C.byref(p))
        if rc != 0:
            raise KeyError(f"{name} (code {rc})")
        return t.value, r.value, list(lb[:r.value]), list(ub[:r.value]), p.value

    def __getitem__(self, name: str):
        """Module variable: a numpy view in Fortran order for arrays (index 0
        is the lower bound), a Python value for scalars."""
        t, r, lb, ub, p = self._info(name)
        if r == 0:
            return _CT[t].from_address(p).value
        shape = tuple(u - l + 1 for l, u in zip(lb, ub))
        n = int(np.prod(shape))
        buf = (C.c_char * (n * np.dtype(_DT[t]).itemsize)).from_address(p)
        return np.frombuffer(buf, dtype=_DT[t]).reshape(shape, order="F")

    def __setitem__(self, name: str, value):
        t, r, lb, ub, p = self._info(name)
        if r == 0:
            _CT[t].from_address(p).value = value
        else:
            self[name][...] = value

    def bounds(self, name: str):
        _, _, lb, ub, _ = self._info(name)
        return lb, ub


# ---- the reference's main program, step by step ---------------------------
# 3DBox.../main.f90:50-62 and 3DChannel.../main.f90:40-47: MPI start-up on
# one process, FFTW plans (box), para, allocarray, wave (box).

def box_program(nx: int, npart: int, rad: float, rhopart: float, ny=None, nz=None) -> RefProgram:
    """The box program set up for an nx*ny*nz domain with npart spheres."""
    ov = {"nx": nx, "ny": ny or nx, "nz": nz or nx, "npart": npart, "rad": rad,
          "rhopart": rhopart}
    R = RefProgram("box", ov)
    R["myid"] = 0
    R["nproc"] = 1
    for s in ("set_plan1d_rc", "set_plan1d_cc", "para", "allocarray", "wave"):
        R.call(s)
    return R


def channel_program(nx: int, ny: int, nz: int, npart: int, rad: float,
                    rhopart: float) -> RefProgram:
    """The channel program (walls at x = 0 and x = nx) with particles
    released at the first step."""
    ov = {"nx8": nx + 1, "nx": nx, "ny": ny, "nz": nz, "nx7": nz, "npart": npart, "rad": rad,
          "rhopart": rhopart, "irelease": 1}
    R = RefProgram("channel", ov)
    R["myid"] = 0
    R["nproc"] = 1
    for s in ("para", "allocarray"):
        R.call(s)
    return R


def set_velocity(R: RefProgram, ux, uy, uz):
    """ux, uy, uz from (nz, ny, nx) arrays into var_inc's (lx, ly, lz)."""
    for k, a in zip(("ux", "uy", "uz"), (ux, uy, uz)):
        R[k] = np.transpose(np.asarray(a), (2, 1, 0))


def release(R: RefProgram, wp=None, omgp=None, positions=None):
    """Particle release of main.f90 at istep = irelease: initpartpos (or, with
    `positions`, its local lists with the given centres in place of its
    draw), the velocities (initpartvel/initpartomg replaced by the given
    values; the workloads start at rest), beads_links."""
    R["istep"] = 1
    R["istep00"] = 0
    R.call("initpartpos")
    n = R["ypglb"].shape[1]
    if positions is not None:
        y = np.asarray(positions, dtype=np.float64).reshape(n, 3).T
        ids = R["ipglb"][:R["nps"]]
        if not np.array_equal(ids, np.arange(1, n + 1)):
            raise RuntimeError("one process should hold every particle in order")
        R["ypglb"] = y
        R["yp"][:, :n] = y
    R["wp"] = 0.0 if wp is None else np.asarray(wp, dtype=np.float64).reshape(n, 3).T
    R["omgp"] = 0.0 if omgp is None else np.asarray(omgp, dtype=np.float64).reshape(n, 3).T
    R.call("beads_links")
    R["istep00"] = 1


def step(R: RefProgram, istep: int, forcing: bool = True):
    """One pass of the main loop (3DBox.../main.f90:172-188; the channel's
    main.f90:187-204 calls FORCING once before its loop)."""
    R["istep"] = istep
    seq = ("forcing",) if forcing else ()
    seq += ("collision_mrt", "beads_collision", "streaming", "beads_lubforce", "beads_move",
            "beads_redistribute", "beads_links", "beads_filling", "macrovar")
    for s in seq:
        R.call(s)


def fields(R: RefProgram) -> dict:
    """var_inc's state in the oracle's layout: populations (19, nz, ny, nx),
    node arrays (nz, ny, nx), links (18, nz, ny, nx), particle vectors
    (npart, 3).  Particle ids are the reference's (1-based)."""
    out = {"f": np.transpose(R["f"], (0, 3, 2, 1)).copy()}
    for k in ("rho", "ux", "uy", "uz", "ibnodes", "isnodes", "force_realx", "force_realy",
              "force_realz"):
        try:
            out[k] = np.transpose(R[k], (2, 1, 0)).copy()
        except KeyError:
            pass
    for k in ("ilink", "mlink", "alink"):
        out[k] = np.transpose(R[k], (0, 3, 2, 1)).copy()
    for k in ("ypglb", "wp", "omgp", "fHIp", "flubp", "torqp"):
        out[k] = R[k].T.copy()
    return out
