"""Error of the FP32-shifted populations against the FP64 plain path.

The FP32 form stores and collides the populations in single precision as
deviations f_i - w_i rho0 (which the reference's own populations already
are, initial.f90:14-26) and keeps FP64 for the particle force and torque
sums, the Newton-Euler update and the mass balance.  ``error_report`` runs
both precisions from the same seeded initial state side by side on the GPU
and, at each checkpoint step, compares the quantities the workload names:

  energy spectrum E(k)      statistc's shells (lbm_statistics)
  dissipation rate          sum of 2 nu |k|^2 E(k)
  mean particle slip        w_p minus the mean fluid velocity on the shell
                            R + 1 <= r <= R + 3 (lbm_particle_slip)
  per-particle force        fHIp, root mean square over the particles

The FP64 GPU path is itself held to the CPU oracle within 1e-12 by the
parity tests, so it stands for the FP64 oracle at sizes where running the
oracle for thousands of steps is out of reach.

Beside each FP32 row the report gives the FP64 floor: a second FP64 box
whose collision sums are done in plain FP64 instead of exact fixed point,
so it differs from the first only by FP64 rounding.  Whatever grows between
those two is the turbulence amplifying rounding differences, not FP32; an
FP32 error far above the floor is FP32's own.  The population difference
is also split into nodes whose solid flags agree in both runs and nodes
where a sphere covers a node in one run and not in the other, and
``storage_rounding`` measures what rounding the stored populations to FP32
does by itself to one FP64 step (the force sum over a sphere's links
cancels to about 1 % of its terms, so the populations' FP32 rounding shows
in the force amplified about 100 times).
"""

from __future__ import annotations

import numpy as np

from . import _capi as capi
from .engine import LBMBox


def _rel(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b|| / ||b|| (2-norm)."""
    nb = float(np.sqrt((np.asarray(b) ** 2).sum()))
    return float(np.sqrt(((np.asarray(a) - np.asarray(b)) ** 2).sum()) / nb) if nb > 0 else 0.0


def compare(s32: dict, s64: dict, p32: dict, p64: dict, slip32: np.ndarray,
            slip64: np.ndarray) -> dict:
    """Relative errors of one checkpoint (FP32 against FP64)."""
    e32, e64 = s32["ek"], s64["ek"]
    resolved = e64 >= 1e-6 * e64.max() if e64.size else e64 > 0
    out = {
        "spectrum_rel_l2": _rel(e32, e64),
        "spectrum_max_rel": float(np.max(np.abs(e32 - e64)[resolved] / e64[resolved]))
        if resolved.any() else 0.0,
        "energy_rel": abs(s32["energy"] - s64["energy"]) / s64["energy"],
        "dissipation_rel": abs(s32["dissipation"] - s64["dissipation"]) / s64["dissipation"],
    }
    if p64["fHIp"].size:
        out["force_rms_rel"] = _rel(p32["fHIp"], p64["fHIp"])
        m32 = np.linalg.norm(slip32, axis=1).mean()
        m64 = np.linalg.norm(slip64, axis=1).mean()
        out["mean_slip_rel"] = float(abs(m32 - m64) / m64) if m64 > 0 else 0.0
        out["slip_rms_rel"] = _rel(slip32, slip64)
        out["mean_slip_fp64"] = float(m64)
    return out


def population_split(b_test: LBMBox, b_ref: LBMBox) -> dict:
    """Max-norm population difference (relative to max |f_ref|) over the nodes
    whose solid flags agree and over those whose flags differ."""
    f_ref = b_ref.get_f()
    scale = float(np.abs(f_ref).max()) or 1.0
    d = np.abs(b_test.get_f() - f_ref).max(axis=0)
    del f_ref
    _, is_t = b_test.get_flags()
    _, is_r = b_ref.get_flags()
    agree = is_t == is_r
    return {"pop_rel_flags_agree": float(d[agree].max() / scale) if agree.any() else 0.0,
            "pop_rel_flags_differ": float(d[~agree].max() / scale) if (~agree).any() else 0.0,
            "nodes_flags_differ": int((~agree).sum())}


def storage_rounding(cfg64: capi.lbm_config, box64: LBMBox, steps: int = 1) -> dict:
    """The part of the FP32 error that FP32 storage alone causes: two FP64
    copies of `box64`'s current state, one with its populations rounded to
    single precision, stepped `steps` steps in FP64 and compared (particle
    force RMS, populations).  Both copies are set up the same way (state,
    particle vectors, forcing generator), so their difference is the
    rounding of the stored populations and nothing else."""
    f = box64.get_f()
    part = box64.get_particle_state()
    first = part.pop("first_move")
    forcing = box64.get_forcing_state()
    copies = []
    try:
        for rounded in (False, True):
            b = LBMBox(cfg64)
            copies.append(b)
            b.set_f(f.astype(np.float32).astype(np.float64) if rounded else f)
            b.macrovar()
            if box64.npart:
                b.set_particle_state(part, first)
            b.set_forcing_state(*forcing)
            b.step(steps)
        pa, pb = (b.get_particles() for b in copies)
        out = {"steps": steps, "pop_rel": float(np.abs(copies[1].get_f() - copies[0].get_f()).max()
                                                / np.abs(f).max())}
        if box64.npart:
            out["force_rms_rel"] = _rel(pb["fHIp"], pa["fHIp"])
        return out
    finally:
        for b in copies:
            b.close()


def error_report(cfg64: capi.lbm_config, u, ypglb: np.ndarray,
                 checkpoints=(10, 100, 2000), stream_ptr: int | None = None,
                 floor: bool = True, split_at=(10, 100)) -> list:
    """Step an FP64 and an FP32 copy of the same box (and, with `floor`, a
    second FP64 copy with plain-FP64 collision sums) to each checkpoint and
    compare them there; returns one dict per checkpoint with the FP32 errors
    and, under "fp64_floor", the FP64-against-FP64 errors."""
    cfg32 = type(cfg64).from_buffer_copy(cfg64)
    cfg32.precision = capi.LBM_PREC_F32
    cfg64 = type(cfg64).from_buffer_copy(cfg64)
    cfg64.precision = capi.LBM_PREC_F64
    boxes = [LBMBox(cfg64), LBMBox(cfg32)]
    if floor:
        boxes.append(LBMBox(cfg64))
        boxes[2].set_sums(capi.LBM_SUMS_FLOAT if boxes[0].sums() != capi.LBM_SUMS_FLOAT
                          else capi.LBM_SUMS_FIXED)
    r_in, r_out = cfg64.rad + 1.0, cfg64.rad + 3.0
    try:
        for b in boxes:
            if stream_ptr is not None:
                b.set_stream(stream_ptr)
            b.initpop(*u)
            b.macrovar()
            if len(ypglb):
                b.release_particles(ypglb)
        done = 0
        rows = []
        for cp in sorted(checkpoints):
            for b in boxes:
                b.step(cp - done)
            done = cp
            stats = [b.statistics() for b in boxes]
            parts = [b.get_particles() for b in boxes]
            if len(ypglb):
                slips = [b.particle_slip(r_in, r_out) for b in boxes]
            else:
                slips = [np.zeros((0, 3))] * len(boxes)
            row = {"step": cp}
            row.update(compare(stats[1], stats[0], parts[1], parts[0], slips[1], slips[0]))
            if cp in split_at:
                row.update(population_split(boxes[1], boxes[0]))
                row["fp32_storage_only"] = storage_rounding(cfg64, boxes[0])
            if floor:
                fl = compare(stats[2], stats[0], parts[2], parts[0], slips[2], slips[0])
                if cp in split_at:
                    fl.update(population_split(boxes[2], boxes[0]))
                row["fp64_floor"] = fl
            rows.append(row)
        return rows
    finally:
        for b in boxes:
            b.close()
