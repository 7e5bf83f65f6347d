"""One small run of every kernel the library launches, for profiling.

Runs, on cuda:0: the FP64 plain path (the collision arithmetic given on the
command line, default integer) and the FP32-shifted path of a 128^3 box
with 150 spheres (three full steps each, then the macroscopic fields, the
statistics, the mass/momentum diagnostics and initpartvel at the centres),
a batch of three boxes of uneven sizes (two steps), the per-subroutine
entries once, and the allocation-free reduction.  ``python -m multiphase_flow_codes_gb300.kernels_tour``
under a profiler gives one launch list covering lbm_step, lbm_batch_step,
lbm_statistics and the rest.  Inputs are seeded; nothing is checked here.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as capi
from . import config, inputs
from .engine import LBMBatch, LBMBox


def main(n: int = 128, npart: int = 150, steps: int = 3, sums: int = capi.LBM_SUMS_INTEGER):
    u = inputs.spectral_velocity(n, 4.0, 0.03)
    y = inputs.initpartpos(n, n, n, npart, 4.0)
    for prec in (capi.LBM_PREC_F64, capi.LBM_PREC_F32):
        wl = config.box(n, npart, 4.0, 2.5, 4.0, 0.03, steps, precision=prec)
        box = LBMBox(wl.cfg)
        if prec == capi.LBM_PREC_F64:
            box.set_sums(sums)
        box.initpop(*u)
        box.macrovar()
        box.release_particles(y)
        box.step(steps)
        box.get_macro()
        box.statistics()
        box.rmsstat()
        box.mass_momentum()
        box.particle_slip(5.0, 7.0)
        box.initpartvel(y)
        box.step_unfused(1)
        box.synchronize()
        if prec == capi.LBM_PREC_F64:
            import torch
            f = torch.from_numpy(box.get_f()).to("cuda")
            out = torch.zeros(4, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            capi.lib().lbm_mass_momentum_noalloc(C.c_void_p(f.data_ptr()), n, n, n,
                                                 C.c_void_p(out.data_ptr()), None)
            torch.cuda.synchronize()
            del f
        box.close()
    boxes = []
    for e, p in ((64, 12), (96, 30), (48, 4)):
        cfg = capi.config_init(capi.LBM_PRESET_BOX, e, e, e, p, 4.0, 2.5)
        cfg.precision = capi.LBM_PREC_F32
        b = LBMBox(cfg)
        b.init_spectral(4.0, 0.03, 7 + e)
        b.macrovar()
        b.init_particles(p)
        boxes.append(b)
    batch = LBMBatch(boxes)
    batch.step(2, graph=False)
    batch.synchronize()
    batch.close()
    for b in boxes:
        b.close()


if __name__ == "__main__":
    import sys
    modes = {"fixed": capi.LBM_SUMS_FIXED, "integer": capi.LBM_SUMS_INTEGER,
             "float": capi.LBM_SUMS_FLOAT}
    main(sums=modes[sys.argv[1]] if len(sys.argv) > 1 else capi.LBM_SUMS_INTEGER)
