"""Batched ensemble: many independent boxes of uneven sizes in one batch.

The workload: 48 periodic boxes, cubic edge drawn uniformly from
{32, 48, 64, 96, 128}, 0 to 64 spheres each with one radius per box drawn
uniformly from [3, 6], FP32-shifted populations, seeded initial fields as in
the 64^3 case (E(k) ~ k^4 exp(-2 (k/4)^2), u_rms 0.03).  Spheres are capped
at a solid volume fraction of 15 % so that the reference's placement
(initpartpos with a gap of 2) can succeed in the small boxes.

``run`` builds the boxes, splits them into a few batches stepped
concurrently on their own streams, lets the batch autotuner pick each
batch's schedule, and times whole steps of all boxes (graph replays of
6-step cycles) with CUDA events joined over the streams.
"""

from __future__ import annotations

import math
import time

import numpy as np

from . import _capi as capi
from . import inputs
from .engine import LBMBatch, LBMBox

EDGES = (32, 48, 64, 96, 128)


def specs(nboxes: int = 48, seed: int = 3003, max_fraction: float = 0.15) -> list:
    """(edge, npart, radius, flow seed, particle seed) of each box."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nboxes):
        n = int(rng.choice(EDGES))
        npart = int(rng.integers(0, 65))
        rad = float(rng.uniform(3.0, 6.0))
        cap = int(max_fraction * n ** 3 / (4.0 / 3.0 * math.pi * rad ** 3))
        out.append((n, min(npart, cap), rad, 54321 + i, 12345 + i))
    return out


def make_boxes(box_specs: list, precision: int = capi.LBM_PREC_F32) -> list:
    boxes = []
    for n, npart, rad, fseed, pseed in box_specs:
        cfg = capi.config_init(capi.LBM_PRESET_BOX, n, n, n, max(npart, 0), rad, 2.5)
        cfg.precision = precision
        b = LBMBox(cfg)
        b.initpop(*inputs.spectral_velocity(n, 4.0, 0.03, seed=fseed))
        b.macrovar()
        if npart:
            b.release_particles(inputs.initpartpos(n, n, n, npart, rad, seed=pseed))
        boxes.append(b)
    return boxes


def split(box_specs: list, parts: int) -> list:
    """Indices of the boxes in `parts` groups of about equal node counts
    (largest first into the lightest group)."""
    order = sorted(range(len(box_specs)), key=lambda i: -box_specs[i][0] ** 3)
    groups = [[] for _ in range(max(1, min(parts, len(box_specs))))]
    load = [0] * len(groups)
    for i in order:
        g = load.index(min(load))
        groups[g].append(i)
        load[g] += box_specs[i][0] ** 3
    return [sorted(g) for g in groups]


def run(steps: int = 500, warmup: int = 6, nboxes: int = 48, tune_reps: int = 3,
        concurrent: int = 3) -> dict:
    """Time `steps` steps of the ensemble; returns the figures of one run.

    The boxes form `concurrent` batches of about equal node counts, each on
    its own stream: while one batch's particle kernels (latency-bound) run,
    another batch's stream + collide kernel (bandwidth-bound) keeps HBM busy.
    Steps go in whole 6-step graph cycles, interleaved over the batches."""
    import torch
    sp = specs(nboxes)
    t0 = time.perf_counter()
    boxes = make_boxes(sp)
    setup_s = time.perf_counter() - t0
    groups = split(sp, concurrent)
    batches = [LBMBatch([boxes[i] for i in g]) for g in groups]
    try:
        kernel_ms = [b.autotune(tune_reps) for b in batches]
        scheds = [b.schedule() for b in batches]
        streams = [torch.cuda.Stream() for _ in batches]
        for b, st in zip(batches, streams):
            b.set_stream(st.cuda_stream)
        for b in batches:
            b.step(warmup, graph=True)
        for b in batches:
            b.synchronize()
        nodes = sum(b.nodes for b in batches)
        cycles = max(1, steps // 6)
        steps = 6 * cycles
        base = torch.cuda.Stream()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        ends = [torch.cuda.Event() for _ in batches]
        torch.cuda.synchronize()
        l0 = LBMBox.kernel_launches()
        e0.record(base)
        for st in streams:
            st.wait_event(e0)
        for _ in range(cycles):
            for b in batches:
                b.step(6, graph=True)
        for ev, st in zip(ends, streams):
            ev.record(st)
            base.wait_event(ev)
        e1.record(base)
        e1.synchronize()
        for b in batches:
            b.synchronize()
        wall = e0.elapsed_time(e1) / 1e3
        launches = LBMBox.kernel_launches() - l0
        alg = [2 * 19 * 4 * b.nodes for b in batches]
        return {
            "boxes": nboxes, "steps": steps, "nodes": nodes,
            "particles": int(sum(s[1] for s in sp)),
            "edges": {str(e): sum(1 for s in sp if s[0] == e) for e in EDGES},
            "value": nodes * steps / wall / 1e6, "unit": "MLUPS",
            "ms_per_step": wall * 1e3 / steps,
            "concurrent_batches": len(batches),
            "kernel": {"name": "k_fused_batch_x2",
                       "schedule": [{"stages": s[0], "groups": s[1], "ctas_per_sm": s[2]}
                                    for s in scheds],
                       "ms_per_launch": kernel_ms, "alg_bytes": alg,
                       "achieved_gbs": [a / (m / 1e3) / 1e9 for a, m in zip(alg, kernel_ms)]},
            "gpu_launches": launches,
            "setup_s": setup_s,
            "how": f"{len(batches)} lbm_batches of about equal node counts, each on its own stream "
                   "(one group's particle kernels overlap another's stream + collide); autotuned "
                   "schedules; 6-step cycles replayed from CUDA graphs; CUDA events around all "
                   "streams",
        }
    finally:
        for b in batches:
            b.close()
        for b in boxes:
            b.close()


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="time the batched ensemble")
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=6)
    ap.add_argument("--boxes", type=int, default=48)
    ap.add_argument("--tune-reps", type=int, default=3)
    ap.add_argument("--concurrent", type=int, default=3)
    a = ap.parse_args()
    print(json.dumps(run(a.steps, a.warmup, a.boxes, a.tune_reps, a.concurrent)))
