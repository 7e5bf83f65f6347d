"""Host-side mirror of the reference's per-step call surface.

``LBMBox`` wraps one ``lbm_ctx`` (one box on one GPU).  Its methods carry
the names of the Fortran subroutines that the reference main loop calls
(3DBox_Forced_HI_Turbulence_Moving_Particles_LBM/main.f90:172-188), each
leaving the device state as that subroutine leaves var_inc's arrays:

    FORCING  collision_MRT  beads_collision  streaming  beads_lubforce
    beads_move  beads_redistribute  beads_links  beads_filling  macrovar

``step(n)`` runs that whole sequence ``n`` times through the fused GPU
path.  Errors that stop the reference (particle overlap, for instance)
raise ``LBMError`` instead.

Array conventions (numpy):
  populations  ``(19, nz, ny, nx)`` float64 (structure of arrays); the
               reference's own ``f(0:18, lx, ly, lz)`` is available through
               ``get_f_fortran`` / ``set_f_fortran``
  node fields  ``(nz, ny, nx)``
  particles    ``(npart, 3)`` float64 (= the reference's ``(3, npart)``)
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as capi
from ._capi import LBMError, dptr, iptr


class LBMBox:
    def __init__(self, cfg: capi.lbm_config):
        self.cfg = cfg
        self.nx, self.ny, self.nz = cfg.nx, cfg.ny, cfg.nz
        self.N = self.nx * self.ny * self.nz
        self._L = capi.lib()
        h = C.c_void_p()
        rc = self._L.lbm_create(C.byref(cfg), C.byref(h))
        if rc != capi.LBM_OK:
            raise LBMError(rc, "lbm_create failed (is a CUDA device present?)")
        self._h = h
        self.npart = 0

    @classmethod
    def adopt(cls, handle) -> "LBMBox":
        """An LBMBox around an existing context (e.g. one taken from the
        server), which it now owns."""
        box = cls.__new__(cls)
        box._L = capi.lib()
        cfg = capi.lbm_config()
        rc = box._L.lbm_get_config(handle, C.byref(cfg))
        if rc != capi.LBM_OK:
            raise LBMError(rc, "lbm_get_config")
        n = C.c_int(0)
        box._L.lbm_particle_count(handle, C.byref(n))
        box.cfg = cfg
        box.nx, box.ny, box.nz = cfg.nx, cfg.ny, cfg.nz
        box.N = box.nx * box.ny * box.nz
        box._h = handle
        box.npart = int(n.value)
        return box

    # ---- lifetime ------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.lbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def _ck(self, rc: int, what: str):
        if rc != capi.LBM_OK:
            msg = self._L.lbm_last_error(self._h)
            raise LBMError(rc, f"{what}: {msg.decode() if msg else ''}")

    def synchronize(self):
        self._ck(self._L.lbm_synchronize(self._h), "lbm_synchronize")

    def set_stream(self, stream_ptr: int):
        """Run all work of this box on the given cudaStream_t (an integer)."""
        self._ck(self._L.lbm_set_stream(self._h, C.c_void_p(stream_ptr)), "set_stream")

    def profile(self, enable: bool = True):
        """Start (and clear) or stop per-phase CUDA-event timing of step()."""
        self._ck(self._L.lbm_profile(self._h, 1 if enable else 0), "profile")

    def profile_read(self) -> dict:
        """{phase: (total ms, timed intervals)} since profile(True)."""
        out = {}
        for i, name in enumerate(capi.PHASES):
            ms = C.c_double(0.0)
            n = C.c_int64(0)
            self._ck(self._L.lbm_profile_read(self._h, i, C.byref(ms), C.byref(n)), "profile_read")
            out[name] = (ms.value, int(n.value))
        return out

    @staticmethod
    def kernel_launches() -> int:
        return int(capi.lib().lbm_kernel_launches())

    # ---- populations -----------------------------------------------------
    def set_f(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(19, self.nz, self.ny, self.nx)
        self._ck(self._L.lbm_upload_f_soa(self._h, dptr(f)), "upload_f")

    def get_f(self) -> np.ndarray:
        out = np.empty((19, self.nz, self.ny, self.nx), dtype=np.float64)
        self._ck(self._L.lbm_download_f_soa(self._h, dptr(out)), "download_f")
        return out

    def set_f_fortran(self, f: np.ndarray):
        """f(0:18, lx, ly, lz) as the reference stores it (population fastest)."""
        f = np.asfortranarray(f, dtype=np.float64)
        assert f.shape == (19, self.nx, self.ny, self.nz)
        self._ck(self._L.lbm_upload_f(self._h, dptr(f)), "upload_f")

    def get_f_fortran(self) -> np.ndarray:
        out = np.empty((19, self.nx, self.ny, self.nz), dtype=np.float64, order="F")
        self._ck(self._L.lbm_download_f(self._h, dptr(out)), "download_f")
        return out

    def initpop(self, ux: np.ndarray, uy: np.ndarray, uz: np.ndarray):
        """initpop (initial.f90:3-28) from a (nz, ny, nx) velocity field."""
        a = [np.ascontiguousarray(u, dtype=np.float64).reshape(self.nz, self.ny, self.nx)
             for u in (ux, uy, uz)]
        self._ck(self._L.lbm_initpop(self._h, dptr(a[0]), dptr(a[1]), dptr(a[2])), "initpop")

    def get_macro(self):
        """(rho, ux, uy, uz) as left by the last macrovar, each (nz, ny, nx)."""
        out = [np.empty((self.nz, self.ny, self.nx)) for _ in range(4)]
        self._ck(self._L.lbm_download_macro(self._h, *map(dptr, out)), "download_macro")
        return tuple(out)

    def get_force(self):
        out = [np.empty((self.nz, self.ny, self.nx)) for _ in range(3)]
        self._ck(self._L.lbm_download_force(self._h, *map(dptr, out)), "download_force")
        return tuple(out)

    def mass_momentum(self) -> np.ndarray:
        out = np.zeros(4)
        self._ck(self._L.lbm_mass_momentum(self._h, dptr(out)), "mass_momentum")
        return out

    def init_spectral(self, k0: float, u_rms: float, seed: int):
        """initpop from a seeded divergence-free Gaussian field made on the GPU."""
        self._ck(self._L.lbm_init_spectral(self._h, float(k0), float(u_rms), int(seed)),
                 "init_spectral")

    def init_channel(self):
        """initpop from the channel's log-law initial velocity (initvel of
        3DChannel.../initial.f90:57-126)."""
        self._ck(self._L.lbm_init_channel(self._h), "init_channel")

    def init_particles(self, npart: int, seed: int = 12345, max_rounds: int = 0):
        """initpartpos with the ranpp generator, particles at rest."""
        self._ck(self._L.lbm_init_particles(self._h, int(npart), int(seed), int(max_rounds)),
                 "init_particles")
        self.npart = int(npart)

    def summary(self) -> np.ndarray:
        """[mass, momentum x, y, z, population checksum, kinetic energy]."""
        out = np.zeros(6)
        self._ck(self._L.lbm_summary(self._h, dptr(out)), "summary")
        return out

    def statistics(self, nshell: int | None = None) -> dict:
        """statistc's spectrum and moments of the current velocity
        (saveload.f90:1111-1338): ek, dk per shell and the totals."""
        n = int(self.nx / 2 - 1.5) if nshell is None else int(nshell)
        ek = np.zeros(max(n, 1))
        dk = np.zeros(max(n, 1))
        out = np.zeros(6)
        self._ck(self._L.lbm_statistics(self._h, n, dptr(ek), dptr(dk), dptr(out)), "statistics")
        nek = int(out[0])
        return {"ek": ek[:min(n, nek)], "dk": dk[:min(n, nek)], "energy": out[1],
                "dissipation": out[2], "skewness": out[3], "flatness": out[4], "uprime": out[5]}

    def particle_slip(self, r_in: float, r_out: float) -> np.ndarray:
        """(npart, 3) slip: w_p minus the mean fluid velocity on the shell
        r_in <= r <= r_out around each centre."""
        out = np.zeros((max(self.npart, 0), 3))
        if self.npart:
            self._ck(self._L.lbm_particle_slip(self._h, float(r_in), float(r_out), dptr(out)),
                     "particle_slip")
        return out

    RMS_COLUMNS = ("nf", "portionf", "uxmn", "uymn", "uzmn", "uxrms", "uyrms", "uzrms", "velfrms",
                   "velfmn", "wpxmn", "wpymn", "wpzmn", "wpxrms", "wpyrms", "wpzrms", "velprms",
                   "velpmn", "oxmn", "oymn", "ozmn", "oxrms", "oyrms", "ozrms", "omgfrms_half",
                   "omgfmn", "omgpxmn", "omgpymn", "omgpzmn", "omgpxrms", "omgpyrms", "omgpzrms",
                   "omgprms", "omgpmn", "omgfrms2", "velfrms2")

    def rmsstat(self) -> dict:
        """rmsstat's columns (saveload.f90:1530-1730) by name."""
        out = np.zeros(36)
        self._ck(self._L.lbm_rmsstat(self._h, dptr(out)), "rmsstat")
        return dict(zip(self.RMS_COLUMNS, out.tolist()))

    def channel_profiles(self, fluid_only: bool = False, ustar: float = 0.0) -> np.ndarray:
        """statistc / statistc2 profiles of the channel (C/saveload.f90:1136-1428):
        (nx, 13) or (nx, 15) rows of profiles.dat / profiles2.dat."""
        ncol = 15 if fluid_only else 13
        out = np.zeros((self.nx, ncol))
        self._ck(self._L.lbm_channel_profiles(self._h, int(bool(fluid_only)), float(ustar), dptr(out)),
                 "channel_profiles")
        return out

    def diag(self) -> dict:
        """diag's columns (saveload.f90:1342-1400)."""
        out = np.zeros(5)
        self._ck(self._L.lbm_diag(self._h, dptr(out)), "diag")
        return {"vmax": out[0], "idwp": int(out[1]), "wpmax": out[2], "idomgp": int(out[3]),
                "omgpmax": out[4]}

    # ---- particles -------------------------------------------------------
    def initpartvel(self, ypglb: np.ndarray) -> np.ndarray:
        """The fluid velocity at the centres (npart, 3) by trilinear
        interpolation of u (initpartvel, partlib.f90:177-263); the context's
        particles are not changed."""
        y = np.ascontiguousarray(ypglb, dtype=np.float64).reshape(-1, 3)
        w = np.zeros_like(y)
        self._ck(self._L.lbm_initpartvel(self._h, y.shape[0], dptr(y), dptr(w)), "initpartvel")
        return w

    def release_particles(self, ypglb: np.ndarray, wp: np.ndarray | str | None = None,
                          omgp: np.ndarray | None = None):
        """Release spheres at the centres (npart, 3): with wp = "fluid" the
        reference's release block (initpartvel, omgp = 0, beads_links),
        otherwise the given velocities (None: at rest)."""
        y = np.ascontiguousarray(ypglb, dtype=np.float64).reshape(-1, 3)
        n = y.shape[0]
        if isinstance(wp, str):
            if wp != "fluid" or omgp is not None:
                raise ValueError('wp is an array, None or "fluid" (with omgp None)')
            self._ck(self._L.lbm_release_particles(self._h, n, dptr(y)), "release_particles")
            self.npart = n
            return
        w = np.zeros_like(y) if wp is None else np.ascontiguousarray(wp, dtype=np.float64).reshape(n, 3)
        o = np.zeros_like(y) if omgp is None else np.ascontiguousarray(omgp, dtype=np.float64).reshape(n, 3)
        self._ck(self._L.lbm_upload_particles(self._h, n, dptr(y), dptr(w), dptr(o)),
                 "upload_particles")
        self.npart = n

    def get_particles(self) -> dict:
        n = max(self.npart, 0)
        arrs = {k: np.zeros((n, 3)) for k in ("ypglb", "wp", "omgp", "fHIp", "flubp", "torqp")}
        if n:
            self._ck(self._L.lbm_download_particles(
                self._h, *(dptr(arrs[k]) for k in ("ypglb", "wp", "omgp", "fHIp", "flubp", "torqp"))),
                "download_particles")
        return arrs

    # the 15 (3, npart) vectors of var_inc, in lbm_particle_state's order
    PARTICLE_VECTORS = ("ypglb", "ypglbp", "wp", "wpp", "omgp", "omgpp", "dwdt", "domgdt",
                        "forcep", "forcepp", "torqp", "torqpp", "thetap", "fHIp", "flubp")

    def get_particle_state(self) -> dict:
        """Every particle vector, (npart, 3) each, and 'first_move'."""
        n = max(self.npart, 0)
        buf = np.zeros((15, n, 3))
        fm = C.c_int32(0)
        self._ck(self._L.lbm_particle_state(self._h, 0, n, dptr(buf), C.byref(fm)),
                 "particle_state")
        out = {k: buf[i].copy() for i, k in enumerate(self.PARTICLE_VECTORS)}
        out["first_move"] = int(fm.value)
        return out

    def set_particle_state(self, state: dict, first_move: int = 0):
        """Set the particle vectors given in `state` (others zero) and rebuild
        the flags and links from ypglb."""
        y = np.asarray(state["ypglb"], dtype=np.float64).reshape(-1, 3)
        n = y.shape[0]
        buf = np.zeros((15, n, 3))
        for i, k in enumerate(self.PARTICLE_VECTORS):
            if k in state:
                buf[i] = np.asarray(state[k], dtype=np.float64).reshape(n, 3)
        fm = C.c_int32(int(first_move))
        self._ck(self._L.lbm_particle_state(self._h, 1, n, dptr(buf), C.byref(fm)),
                 "particle_state")
        self.npart = n

    def get_flags(self):
        ib = np.empty((self.nz, self.ny, self.nx), dtype=np.int32)
        isn = np.empty((self.nz, self.ny, self.nx), dtype=np.int32)
        self._ck(self._L.lbm_download_flags(self._h, iptr(ib), iptr(isn)), "download_flags")
        return ib, isn

    def get_links(self):
        """(node, ipop, particle, alpha) of every boundary link."""
        n = C.c_int64(0)
        self._ck(self._L.lbm_download_links(self._h, 0, C.byref(n), None, None, None, None), "links")
        m = int(n.value)
        node = np.empty(m, dtype=np.int32)
        ipop = np.empty(m, dtype=np.int32)
        part = np.empty(m, dtype=np.int32)
        alpha = np.empty(m, dtype=np.float64)
        if m:
            self._ck(self._L.lbm_download_links(self._h, m, C.byref(n), iptr(node), iptr(ipop),
                                                iptr(part), dptr(alpha)), "links")
        return node, ipop, part, alpha

    # ---- forcing state ---------------------------------------------------
    def get_forcing_state(self):
        iseed = C.c_int32(0)
        iy = C.c_int32(0)
        iv = np.zeros(32, dtype=np.int32)
        b = np.zeros(450)
        self._ck(self._L.lbm_forcing_state(self._h, 0, C.byref(iseed), C.byref(iy), iptr(iv), dptr(b)),
                 "forcing_state")
        return int(iseed.value), int(iy.value), iv, b

    def set_forcing_state(self, iseedf: int, iyf: int, ivf: np.ndarray, b: np.ndarray):
        iseed = C.c_int32(iseedf)
        iy = C.c_int32(iyf)
        iv = np.ascontiguousarray(ivf, dtype=np.int32)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        self._ck(self._L.lbm_forcing_state(self._h, 1, C.byref(iseed), C.byref(iy), iptr(iv), dptr(bb)),
                 "forcing_state")

    # ---- the reference's subroutines ----------------------------------------
    def FORCING(self):
        self._ck(self._L.lbm_forcing(self._h), "FORCING")

    def collision_MRT(self):
        self._ck(self._L.lbm_collision_mrt(self._h), "collision_MRT")

    def beads_collision(self):
        self._ck(self._L.lbm_beads_collision(self._h), "beads_collision")

    def streaming(self):
        self._ck(self._L.lbm_streaming(self._h), "streaming")

    def beads_lubforce(self):
        self._ck(self._L.lbm_beads_lubforce(self._h), "beads_lubforce")

    def beads_move(self):
        self._ck(self._L.lbm_beads_move(self._h), "beads_move")

    def beads_redistribute(self):
        self._ck(self._L.lbm_beads_redistribute(self._h), "beads_redistribute")

    def beads_links(self):
        self._ck(self._L.lbm_beads_links(self._h), "beads_links")

    def beads_filling(self):
        self._ck(self._L.lbm_beads_filling(self._h), "beads_filling")

    def macrovar(self):
        self._ck(self._L.lbm_macrovar(self._h), "macrovar")

    def rhoupdat(self):
        self._ck(self._L.lbm_rhoupdat(self._h), "rhoupdat")

    def prerelax(self, eps: float = 1e-5, max_iter: int = 15000) -> tuple:
        """Density pre-relaxation of a new run (main.f90:86-108); returns
        (iterations counter at exit, last max |rho - rho_previous|)."""
        it, err = C.c_int(0), C.c_double(0.0)
        self._ck(self._L.lbm_prerelax(self._h, float(eps), int(max_iter), C.byref(it),
                                      C.byref(err)), "prerelax")
        return it.value, err.value

    def step(self, nsteps: int = 1):
        """The time step of main.f90:172-188, ``nsteps`` times (fused path)."""
        self._ck(self._L.lbm_step(self._h, int(nsteps)), "step")

    # ---- kernel selection -------------------------------------------------
    def set_variant(self, variant: int, stages: int = 0, groups: int = 0, ctas_per_sm: int = 0):
        """Pick the stream+collide kernel (capi.LBM_VARIANT_*) and its schedule."""
        self._ck(self._L.lbm_set_variant(self._h, int(variant), int(stages), int(groups),
                                         int(ctas_per_sm)), "set_variant")

    def variant(self) -> tuple:
        """(variant, stages, groups, ctas_per_sm) of the stream+collide kernel in use."""
        v, s, g, c = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        self._ck(self._L.lbm_get_variant(self._h, C.byref(v), C.byref(s), C.byref(g), C.byref(c)),
                 "get_variant")
        return v.value, s.value, g.value, c.value

    def set_sums(self, mode: int):
        """Arithmetic of the collision (capi.LBM_SUMS_*): FIXED (FP64 default)
        computes the integer-coefficient moment sums exactly in fixed point."""
        self._ck(self._L.lbm_set_sums(self._h, int(mode)), "set_sums")

    def sums(self) -> int:
        m = C.c_int(0)
        self._ck(self._L.lbm_get_sums(self._h, C.byref(m)), "get_sums")
        return m.value

    def autotune(self, reps: int = 5) -> float:
        """Time every applicable stream+collide variant on the current state
        (without advancing it), keep the fastest; returns its ms per launch."""
        ms = C.c_double(0.0)
        self._ck(self._L.lbm_autotune(self._h, int(reps), C.byref(ms)), "autotune")
        return ms.value

    def step_unfused(self, nsteps: int = 1):
        """The same sequence, one reference subroutine per call."""
        for _ in range(nsteps):
            self.FORCING()
            self.collision_MRT()
            if self.npart:
                self.beads_collision()
            self.streaming()
            if self.npart:
                self.beads_lubforce()
                self.beads_move()
                self.beads_redistribute()
                self.beads_links()
                self.beads_filling()
            self.macrovar()


class LBMBatch:
    """Several LBMBox contexts advanced together (lbm_batch_*): one persistent
    stream + collide kernel for all boxes, FORCING and the particle
    subroutines of each box on the box's own stream, whole cycles of steps
    replayed from a captured CUDA graph."""

    def __init__(self, boxes: list):
        self.boxes = list(boxes)          # keeps the contexts alive
        self._L = capi.lib()
        arr = (C.c_void_p * len(self.boxes))(*[b.handle.value for b in self.boxes])
        h = C.c_void_p()
        rc = self._L.lbm_batch_create(arr, len(self.boxes), C.byref(h))
        if rc != capi.LBM_OK:
            msg = self._L.lbm_last_error(self.boxes[0].handle)
            raise LBMError(rc, f"lbm_batch_create: {msg.decode() if msg else ''}")
        self._h = h

    def _ck(self, rc: int, what: str):
        if rc != capi.LBM_OK:
            msg = self._L.lbm_batch_last_error(self._h)
            raise LBMError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "_h", None):
            self._L.lbm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def nodes(self) -> int:
        return int(self._L.lbm_batch_nodes(self._h))

    def step(self, nsteps: int = 1, graph: bool = True):
        self._ck(self._L.lbm_batch_step(self._h, int(nsteps), 1 if graph else 0), "batch_step")

    def synchronize(self):
        self._ck(self._L.lbm_batch_synchronize(self._h), "batch_synchronize")

    def set_stream(self, stream_ptr: int):
        """Enqueue batch steps on this cudaStream_t (an integer)."""
        self._ck(self._L.lbm_batch_set_stream(self._h, C.c_void_p(stream_ptr)), "batch_set_stream")

    def set_schedule(self, stages: int, groups: int, ctas_per_sm: int = 0):
        self._ck(self._L.lbm_batch_set_schedule(self._h, int(stages), int(groups), int(ctas_per_sm)),
                 "batch_set_schedule")

    def schedule(self) -> tuple:
        s, g, c = C.c_int(0), C.c_int(0), C.c_int(0)
        self._ck(self._L.lbm_batch_get_schedule(self._h, C.byref(s), C.byref(g), C.byref(c)),
                 "batch_get_schedule")
        return s.value, g.value, c.value

    def autotune(self, reps: int = 3) -> float:
        ms = C.c_double(0.0)
        self._ck(self._L.lbm_batch_autotune(self._h, int(reps), C.byref(ms)), "batch_autotune")
        return ms.value
