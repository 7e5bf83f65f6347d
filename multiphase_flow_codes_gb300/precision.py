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


def error_report(cfg64: capi.lbm_config, u, ypglb: np.ndarray,
                 checkpoints=(10, 100, 2000), stream_ptr: int | None = None) -> list:
    """Step an FP64 and an FP32 copy of the same box to each checkpoint and
    compare them there; returns one dict per checkpoint."""
    cfg32 = type(cfg64).from_buffer_copy(cfg64)
    cfg32.precision = capi.LBM_PREC_F32
    cfg64 = type(cfg64).from_buffer_copy(cfg64)
    cfg64.precision = capi.LBM_PREC_F64
    boxes = [LBMBox(cfg64), LBMBox(cfg32)]
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
            s64, s32 = (b.statistics() for b in boxes)
            p64, p32 = (b.get_particles() for b in boxes)
            if len(ypglb):
                sl64, sl32 = (b.particle_slip(r_in, r_out) for b in boxes)
            else:
                sl64 = sl32 = np.zeros((0, 3))
            row = {"step": cp}
            row.update(compare(s32, s64, p32, p64, sl32, sl64))
            rows.append(row)
        return rows
    finally:
        for b in boxes:
            b.close()
