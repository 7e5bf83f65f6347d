#!/usr/bin/env python
"""Benchmark of the particle-laden D3Q19 MRT time step on GB300.

Workload (default, ``box256_p1000_f64``): periodic 256^3 box, forced
homogeneous isotropic turbulence (stochastic low-wavenumber forcing), 1000
spheres of radius 4 with density ratio 2.5, FP64 populations; synthetic
seeded initial field (E(k) ~ k^4 exp(-2 (k/8)^2), u_rms = 0.04).  A "step"
is one full time step of the reference main loop (FORCING ... macrovar).

Metric: MLUPS = lattice nodes x steps / s / 1e6 (all nodes, fluid and solid).

Printed JSON line (rank 0):
  value      device-resident throughput, K steps timed with CUDA events
  e2e        the same metric through the C ABI with host buffers: upload of
             the reference-layout populations and particles from pinned
             memory, K C-ABI step calls each followed by a read-back of the
             particle state, download of the final populations
  roofline   the fused stream+collide kernel: algorithmic bytes per launch
             (2 x 19 x sizeof(real) per node) / its CUDA-event time, against
             the measured HBM copy bandwidth
  fp32_shifted  the same workload with FP32 populations, its roofline and
             its difference from the FP64 run after the timed steps
  cpu_baseline  the CPU restatement (OpenMP, all host cores) on a bounded
             sample of the same workload

``--impl reference`` times the CPU restatement of the reference's algorithm
(the reference itself is Fortran + MPI + FFTW 2 with no toolchain on the
GPU host) on the same workload with all host cores.

With --gpus N under torchrun every rank advances an independent replica of
the box (the path does not shard); value = all ranks' node updates / the
slowest rank's time.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

HBM_FALLBACK = 6800.0  # GB/s, used only if the measured peaks file is absent


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


def profile_figures() -> dict:
    p = ROOT / "profiles" / "ncu_figures.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs(wl):
    from multiphase_flow_codes_gb300 import inputs
    c = wl.cfg
    u = inputs.spectral_velocity(c.nx, wl.k0, wl.urms, seed=wl.flow_seed, ny=c.ny, nz=c.nz)
    y = inputs.initpartpos(c.nx, c.ny, c.nz, wl.npart, c.rad, c.mingap, seed=wl.particle_seed) \
        if wl.npart else np.zeros((0, 3))
    return u, y


def initial_f(u):
    """initpop (initial.f90:14-26) on the host: f = w_i (3 c.u + 4.5 (c.u)^2 - 1.5 u^2)."""
    cx = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0], dtype=np.float64)
    cy = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1], dtype=np.float64)
    cz = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1], dtype=np.float64)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    ux, uy, uz = u
    usqr = 1.5 * (ux * ux + uy * uy + uz * uz)
    f = np.empty((19,) + ux.shape)
    for q in range(19):
        G = cx[q] * ux + cy[q] * uy + cz[q] * uz
        f[q] = w[q] * (3.0 * G + 4.5 * G * G - usqr)
    return f


def run_device(wl, u, y, steps, warmup, device, want_f=False, variant=None, sums=None):
    """Device-resident timing of `steps` C-ABI step calls."""
    import torch
    from multiphase_flow_codes_gb300 import _capi as capi
    from multiphase_flow_codes_gb300.engine import LBMBox
    box = LBMBox(wl.cfg)
    if sums is not None and wl.cfg.precision == capi.LBM_PREC_F64:
        box.set_sums(sums)
    stream = torch.cuda.Stream(device=device)
    box.set_stream(stream.cuda_stream)
    box.initpop(*u)
    box.macrovar()
    if wl.npart:
        box.release_particles(y)
    if variant is None:
        box.autotune(reps=3)      # pick the stream+collide variant on this state
    else:
        box.set_variant(*variant)
    variant = box.variant()
    for _ in range(warmup):
        box.step(1)
    box.synchronize()
    box.profile(True)
    l0 = box.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    e0.record(stream)
    for _ in range(steps):
        box.step(1)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    launches = box.kernel_launches() - l0
    phases = box.profile_read()
    box.profile(False)
    box.synchronize()
    f = box.get_f() if want_f else None
    parts = box.get_particles() if (want_f and wl.npart) else None
    box.close()
    return ms, launches, phases, f, parts, variant


def sc_achieved(phases, alg_bytes):
    """Algorithmic GB/s of the stream + collide kernel: its bytes per launch
    over the mean CUDA-event duration of its launches in the timed region."""
    sc_ms, sc_n = phases["stream_collide"]
    if not sc_n:
        return None
    return alg_bytes / (sc_ms / sc_n / 1e3) / 1e9


def kernel_name(variant, fixed=False, integer=False):
    v, st, groups, per_sm = variant
    if v == 3:
        return (f"k_fused_staged_x2 (stream + MRT collide + forcing, FP32 pairs on f32x2; "
                f"{st} stages, {groups} consumer groups, {per_sm} CTAs/SM)")
    if v == 2:
        return f"k_fused_staged (stream + MRT collide + forcing; {st} stages, {per_sm} CTAs/SM)"
    if fixed and integer:
        return ("k_fused_fixed (stream + MRT collide + forcing; direct, populations and forces in "
                "64-bit fixed point, integer collision core, FP64 body-force series)")
    if fixed:
        return ("k_fused_fixed (stream + MRT collide + forcing; direct, populations and forces in "
                "64-bit fixed point)")
    return "k_fused (stream + MRT collide + forcing; direct)"


def run_e2e(wl, f0_fortran, y, steps, device, variant=None, sums=None):
    """End to end through the C ABI with host buffers (see module doc)."""
    import torch
    from multiphase_flow_codes_gb300 import _capi as capi
    from multiphase_flow_codes_gb300.engine import LBMBox
    box = LBMBox(wl.cfg)
    if sums is not None and wl.cfg.precision == capi.LBM_PREC_F64:
        box.set_sums(sums)
    if variant is not None:
        box.set_variant(*variant)
    npart = y.shape[0]
    pin = torch.empty(f0_fortran.size, dtype=torch.float64, pin_memory=True).numpy()
    hf = np.ndarray(f0_fortran.shape, dtype=np.float64, buffer=pin, order="F")
    hf[...] = f0_fortran
    py = torch.empty(max(npart, 1) * 3, dtype=torch.float64, pin_memory=True).numpy()[: npart * 3].reshape(npart, 3)
    py[...] = y
    outs = {k: torch.empty(max(npart, 1) * 3, dtype=torch.float64, pin_memory=True).numpy()[: npart * 3].reshape(npart, 3)
            for k in ("ypglb", "wp", "fHIp", "torqp")}
    hout = torch.empty(f0_fortran.size, dtype=torch.float64, pin_memory=True).numpy()
    hfo = np.ndarray(f0_fortran.shape, dtype=np.float64, buffer=hout, order="F")
    import ctypes as C
    from multiphase_flow_codes_gb300._capi import dptr
    L = box._L
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    box._ck(L.lbm_upload_f(box.handle, dptr(hf)), "upload_f")
    box._ck(L.lbm_macrovar(box.handle), "macrovar")
    if npart:
        zero = np.zeros_like(py)
        box._ck(L.lbm_upload_particles(box.handle, npart, dptr(py), dptr(zero), dptr(zero)), "upload_particles")
    for _ in range(steps):
        box._ck(L.lbm_step(box.handle, 1), "step")
        if npart:
            box._ck(L.lbm_download_particles(box.handle, dptr(outs["ypglb"]), dptr(outs["wp"]), None,
                                             dptr(outs["fHIp"]), None, dptr(outs["torqp"])), "particles")
    box._ck(L.lbm_download_f(box.handle, dptr(hfo)), "download_f")
    t1 = time.perf_counter()
    box.close()
    h2d = f0_fortran.nbytes + npart * 3 * 8 * 3
    d2h = f0_fortran.nbytes + steps * npart * 3 * 8 * 4
    return (t1 - t0) * 1e3, h2d / steps, d2h / steps


def cpu_oracle(wl, u, y, steps, threads=None):
    """The CPU restatement on `steps` full steps of the workload."""
    import oracle
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
        oracle.set_threads(threads)
    o = oracle.OracleBox(wl.cfg)
    o.initpop(*u)
    o.macrovar()
    if wl.npart:
        o.release_particles(y)
    t0 = time.perf_counter()
    rc = o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    if rc:
        raise RuntimeError(f"oracle step failed with {rc}")
    return dt


def workload(name: str):
    """box64_p16_f64, box256_p1000_f64, box256_p1000_f32, or
    box{n}[x{ny}x{nz}]_p{npart}_{f64|f32} (radius 4, density ratio 2.5)."""
    from multiphase_flow_codes_gb300 import _capi as capi
    from multiphase_flow_codes_gb300 import config
    table = {"box64_p16_f64": config.box64_p16_f64, "box256_p1000_f64": config.box256_p1000_f64,
             "box256_p1000_f32": config.box256_p1000_f32}
    if name in table:
        return table[name]()
    import re
    m = re.fullmatch(r"box(\d+)(?:x(\d+)x(\d+))?_p(\d+)_(f64|f32)", name)
    if not m:
        raise SystemExit(f"unknown workload {name}")
    n, npart = int(m.group(1)), int(m.group(4))
    ny = int(m.group(2)) if m.group(2) else n
    nz = int(m.group(3)) if m.group(3) else n
    prec = capi.LBM_PREC_F64 if m.group(5) == "f64" else capi.LBM_PREC_F32
    return config.box(n, npart, 4.0, 2.5, 8.0 if n >= 256 else 4.0, 0.04, 2000, precision=prec,
                      name=name, ny=ny, nz=nz)


def describe(name, c, npart, k0, urms, dtype, world):
    """The JSON line's config block."""
    N = c.nx * c.ny * c.nz
    return {"workload": name, "grid": [c.nx, c.ny, c.nz], "particles": npart,
            "radius": c.rad, "density_ratio": c.rhopart, "k0": k0, "u_rms": urms,
            "forcing": "stochastic low-k (|k| < sqrt 8)", "mrt_type": c.mrt_type,
            "l2": "inputs larger than L2 (populations %.2f GB)" % (2 * 19 * N * (8 if dtype == "f64" else 4) / 1e9),
            "parallelism": f"replicas x{world}"}


def reference_arm(args):
    """--impl reference: the CPU restatement of the reference's time step.

    Loads nothing of the engine: the parameter block comes from the
    oracle's own restatement of the reference constants (oracle/config.py),
    the seeded inputs from the numpy generators, the timed steps from the
    oracle library.  Under torchrun only rank 0 runs."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import re
    import oracle
    from oracle import config as ocfg
    from multiphase_flow_codes_gb300 import inputs
    name = args.workload
    if name in ocfg.WORKLOADS:
        c, npart, k0, urms = ocfg.workload_config(name)
    else:
        m = re.fullmatch(r"box(\d+)_p(\d+)_(f64|f32)", name)
        if not m:
            raise SystemExit(f"unknown workload {name}")
        n, npart = int(m.group(1)), int(m.group(2))
        k0, urms = (8.0 if n >= 256 else 4.0), 0.04
        c = ocfg.config_init(ocfg.PRESET_BOX, n, n, n, npart, 4.0, 2.5)
    N = c.nx * c.ny * c.nz
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    u = inputs.spectral_velocity(c.nx, k0, urms, seed=54321, ny=c.ny, nz=c.nz)
    y = inputs.initpartpos(c.nx, c.ny, c.nz, npart, c.rad, c.mingap, seed=12345) \
        if npart else np.zeros((0, 3))
    o = oracle.OracleBox(c)
    o.initpop(*u)
    o.macrovar()
    if npart:
        o.release_particles(y)
    steps = max(1, min(args.steps, args.ref_max_steps))
    warm = max(0, min(args.warmup, args.ref_max_steps - steps))
    if warm:
        rc = o.step(warm)
        if rc:
            raise RuntimeError(f"oracle step failed with {rc}")
    t0 = time.perf_counter()
    rc = o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    if rc:
        raise RuntimeError(f"oracle step failed with {rc}")
    v = N * steps / dt / 1e6
    line = {"impl": "reference", "metric": "MLUPS", "value": v, "unit": "MLUPS",
            "n_gpus": 0, "steps": steps, "warmup": warm, "ms_per_step": dt * 1e3 / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic seeded", "config": describe(name, c, npart, k0, urms, "f64", 1),
            "cpu_baseline": {"value": v, "unit": "MLUPS", "cores": cores, "kind": "port",
                             "sample": f"{steps} full steps of {name} after {warm} untimed ones (CPU "
                                       "restatement of the reference, OpenMP over all host cores; the "
                                       "Fortran/MPI/FFTW2 reference has no toolchain on this host)"},
            "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="box256_p1000_f64")
    ap.add_argument("--cpu-steps", type=int, default=2, help="CPU baseline sample (full steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-one-core-steps", type=int, default=1,
                    help="CPU baseline also on one thread for this many steps (0: skip)")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--fp32-report", default="10,100,2000",
                    help="steps at which the FP32-shifted run is compared with FP64 "
                         "('' to skip)")
    ap.add_argument("--batch-steps", type=int, default=500,
                    help="steps of the 48-box batched ensemble (0: skip it)")
    ap.add_argument("--serve-seconds", type=float, default=30.0,
                    help="window of the Poisson serving run (0: skip it)")
    ap.add_argument("--serve-rate", type=float, default=6.0,
                    help="requests per second (6: the highest rate measured with a flat p99 "
                         "over 600 s; 20: the overload case)")
    ap.add_argument("--serve-window", type=float, default=10.0,
                    help="seconds per latency window of the serving run")
    ap.add_argument("--no-fp64-float", action="store_true",
                    help="skip the all-FP64 (--sums float) comparison run of the FP64 workload")
    ap.add_argument("--sums", choices=["fixed", "float", "integer"], default="integer",
                    help="FP64 collision arithmetic: integer-coefficient moment sums exact in "
                         "64-bit fixed point with FP64 products (fixed), all in FP64 (float), or "
                         "the velocity and force products as integer products too (integer, the "
                         "default)")
    ap.add_argument("--variant", default=None,
                    help="stream+collide kernel as 'variant,stages,groups,ctas_per_sm' "
                         "(default: autotuned on the workload)")
    ap.add_argument("--ref-max-steps", type=int, default=200,
                    help="--impl reference: at most this many full CPU steps (warm-up included)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    if args.impl == "reference":
        reference_arm(args)
        return

    from multiphase_flow_codes_gb300.replicas import Replicas
    rep = Replicas("nccl")
    world, rank, local = rep.world, rep.rank, rep.local
    wl = workload(args.workload)
    c = wl.cfg
    N = c.nx * c.ny * c.nz
    from multiphase_flow_codes_gb300 import _capi as capi
    dtype = "f64" if c.precision == capi.LBM_PREC_F64 else "f32"
    cfg_desc = describe(wl.name, c, wl.npart, wl.k0, wl.urms, dtype, world)
    if dtype == "f64":
        cfg_desc["collision_sums"] = {
            "fixed": "integer-coefficient moment sums exact in 64-bit fixed point, products FP64",
            "integer": "moment sums exact in 64-bit fixed point, velocity and force products as "
                       "exact 128-bit integer products; body-force series in FP64, rounded once to "
                       "fixed point",
            "float": "all FP64"}[args.sums]

    import torch
    torch.cuda.set_device(local)
    from multiphase_flow_codes_gb300 import build as b
    b.build()
    u, y = make_inputs(wl)

    sampler = ClockSampler(local)
    rep.barrier()
    torch.cuda.synchronize()
    sampler.start()
    fixed = tuple(int(v) for v in args.variant.split(",")) if args.variant else None
    sums = {"fixed": capi.LBM_SUMS_FIXED, "float": capi.LBM_SUMS_FLOAT,
            "integer": capi.LBM_SUMS_INTEGER}[args.sums]
    ms, launches, phases, f64, p64, variant = run_device(wl, u, y, args.steps, args.warmup, local,
                                                         want_f=not args.no_fp32, variant=fixed,
                                                         sums=sums)
    clocks = sampler.stop()
    rate, t_s = rep.rate(N * args.steps, ms / 1e3)
    t_ms = t_s * 1e3
    value = rate / 1e6

    peaks = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", HBM_FALLBACK))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    esz = 8 if dtype == "f64" else 4
    alg_bytes = 2 * 19 * esz * N
    achieved = sc_achieved(phases, alg_bytes)
    figs = profile_figures()
    key = f"fused_{dtype}_{c.nx}" + ({"fixed": "_fx", "integer": "_int"}.get(args.sums, "")
                                      if dtype == "f64" else "")
    traffic = None
    if key in figs and figs[key].get("dram_bytes_per_node"):
        traffic = figs[key]["dram_bytes_per_node"] * N
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
            "kernel": kernel_name(variant, dtype == "f64" and args.sums != "float",
                                  args.sums == "integer"),
            "alg_bytes_per_launch": alg_bytes, "peak_source": peak_src}
    fp64 = {}
    if dtype == "f64" and key in figs and figs[key].get("pipes"):
        # the integer collision core's compute roofline is the integer pipes,
        # from the ncu capture (FP64 only in the body-force series)
        fp64 = {"fp64_inst_per_node": figs[key].get("fp64_inst_per_node", 0.0),
                "pipes_pct_of_peak": figs[key]["pipes"], "capture": figs[key].get("capture"),
                "note": "integer collision core, FP64 body-force series: bound by the ALU pipe "
                        "(fixed-point sums, 128-bit products, range tests), not by FP64 or HBM"}
    elif dtype == "f64" and key in figs and figs[key].get("fp64_flop_per_node") and phases["stream_collide"][1]:
        sc_ms, sc_n = phases["stream_collide"]
        import ctypes as C
        peak = C.c_double(0.0)
        rc = capi.lib().lbm_fma_throughput(capi.LBM_PREC_F64, C.byref(peak))
        fp64_peak = peak.value if rc == 0 and peak.value > 0 else None
        per_s = N / (sc_ms / sc_n / 1e3)
        tf = figs[key]["fp64_flop_per_node"] * per_s / 1e12
        # the FMA probe issues one FP64 instruction per two flops
        ti = figs[key].get("fp64_inst_per_node", 0.0) * per_s / 1e12
        fp64 = {"achieved_tflops": tf, "peak_tflops": fp64_peak,
                "frac": tf / fp64_peak if fp64_peak else None, "unit": "TFLOP/s",
                "flop_per_node": figs[key]["fp64_flop_per_node"],
                "fp64_inst_per_node": figs[key].get("fp64_inst_per_node"),
                "issue_frac": (2 * ti / fp64_peak) if (fp64_peak and ti) else None,
                "note": "FP64 FMA peak measured live on this GPU (lbm_fma_throughput); FP64 flops "
                        "and instructions per node from the ncu counters; issue_frac = FP64 "
                        "instructions per second over the probe's FMA instructions per second. "
                        "The FP64 kernel is bound by its FP64 and integer instruction issue"}

    line = {"metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic seeded (no dataset)", "config": cfg_desc, "roofline": roof,
            "gpu_launches": launches, "clocks": clocks,
            "phase_ms_per_step": {k: (v[0] / args.steps) for k, v in phases.items()}}
    if fp64:
        line["fp64_roofline"] = fp64

    # end to end right after the device-resident run, before the FP32, ensemble and
    # serving runs (whose host threads and device state it should not share)
    if not args.no_e2e:
        f0 = initial_f(u)
        f0_fortran = np.asfortranarray(np.transpose(f0, (0, 3, 2, 1)))
        del f0
        e_ms, h2d, d2h = run_e2e(wl, f0_fortran, y, args.steps, local, variant, sums)
        e_rate, _ = rep.rate(N * args.steps, e_ms / 1e3)
        line["e2e"] = {"value": e_rate / 1e6, "unit": "MLUPS",
                       "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "how": "C ABI: lbm_upload_f (Fortran layout, pinned host) + particles, "
                              f"{args.steps} x (lbm_step + particle read-back), lbm_download_f"}

    # the same FP64 steps with every collision operation and the stored
    # populations in plain FP64 (no fixed point anywhere), for comparison
    if dtype == "f64" and args.sums != "float" and not args.no_fp64_float:
        msf, lf, phf, _, _, vf = run_device(wl, u, y, args.steps, args.warmup, local,
                                            variant=variant, sums=capi.LBM_SUMS_FLOAT)
        achf = sc_achieved(phf, alg_bytes)
        ratef, _ = rep.rate(N * args.steps, msf / 1e3)
        line["fp64_all_float"] = {
            "value": ratef / 1e6, "unit": "MLUPS", "ms_per_step": msf / args.steps,
            "roofline": {"bound": "hbm", "achieved": achf, "peak": hbm, "unit": "GB/s",
                         "frac": (achf / hbm) if achf else None,
                         "kernel": kernel_name(vf, False, False)},
            "phase_ms_per_step": {k: (v[0] / args.steps) for k, v in phf.items()},
            "how": "the workload's steps with LBM_SUMS_FLOAT: FP64 collision arithmetic and FP64 "
                   "population storage throughout (the reference's own arithmetic)"}

    if not args.no_fp32 and dtype == "f64":
        from multiphase_flow_codes_gb300 import config
        wl32 = config.box256_p1000_f32() if args.workload == "box256_p1000_f64" else workload(args.workload)
        if wl32.cfg.precision != capi.LBM_PREC_F32:
            wl32.cfg.precision = capi.LBM_PREC_F32
        ms32, l32, ph32, f32, p32, variant32 = run_device(wl32, u, y, args.steps, args.warmup, local, want_f=True)
        ach32 = sc_achieved(ph32, 2 * 19 * 4 * N)
        err = float(np.abs(f32 - f64).max() / np.abs(f64).max())
        ferr = None
        if p64 is not None and p32 is not None and wl.npart:
            ferr = float(np.sqrt(((p32["fHIp"] - p64["fHIp"]) ** 2).mean() / (p64["fHIp"] ** 2).mean()))
        line["fp32_shifted"] = {
            "value": N * args.steps * world / (ms32 / 1e3) / 1e6, "unit": "MLUPS",
            "ms_per_step": ms32 / args.steps, "vs_fp64": (N * args.steps / (ms32 / 1e3)) / (N * args.steps / (ms / 1e3)),
            "roofline": {"bound": "hbm", "achieved": ach32, "peak": hbm, "unit": "GB/s",
                         "frac": (ach32 / hbm) if ach32 else None, "kernel": kernel_name(variant32),
                         "traffic": (figs.get(f"fused_f32_{c.nx}", {}).get("dram_bytes_per_node") or 0) * N or None},
            "rel_err_f_vs_fp64": err, "rel_rms_particle_force_vs_fp64": ferr,
            "error_after_steps": args.warmup + args.steps,
            "phase_ms_per_step": {k: (v[0] / args.steps) for k, v in ph32.items()}}
        del f32
        if args.fp32_report and rank == 0:
            from multiphase_flow_codes_gb300 import precision
            cps = [int(v) for v in args.fp32_report.split(",") if v]
            line["fp32_shifted"]["error_vs_fp64"] = {
                "checkpoints": precision.error_report(wl.cfg, u, y, cps),
                "target": 1e-5,
                "how": "FP32-shifted and FP64 boxes stepped side by side from the same seeded state; "
                       "E(k) and dissipation from lbm_statistics, slip on the R+1..R+3 fluid shell, "
                       "fHIp RMS over particles"}

    if args.batch_steps > 0 and rank == 0 and args.workload == "box256_p1000_f64":
        from multiphase_flow_codes_gb300 import ensemble
        be = ensemble.run(steps=args.batch_steps)
        k = be["kernel"]
        # each batch's kernel timed alone by its autotuner; bytes over time summed
        agg = sum(k["alg_bytes"]) / (sum(k["ms_per_launch"]) / 1e3) / 1e9
        k["roofline"] = {"bound": "hbm", "achieved": agg, "peak": hbm, "unit": "GB/s",
                         "frac": agg / hbm}
        line["batched_ensemble"] = be

    if args.serve_seconds > 0 and rank == 0 and args.workload == "box256_p1000_f64":
        from multiphase_flow_codes_gb300 import serving
        sv = serving.poisson_run(rate=args.serve_rate, duration=args.serve_seconds,
                                 window=args.serve_window)
        sv["how"] = ("native lbm_server loop: Poisson arrivals, admission by lbm_footprint within a "
                     "96 GiB budget, up to 96 resident solves, continuous batching of the FP32 channel "
                     "solves into batched stream+collide launches, 50-step chunks; latency = done - "
                     "submit; after the window the queue is drained and counted")
        line["serving"] = sv

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        dt = cpu_oracle(wl, u, y, args.cpu_steps, cores)
        line["cpu_baseline"] = {"value": N * args.cpu_steps / dt / 1e6, "unit": "MLUPS", "cores": cores,
                                "kind": "port",
                                "sample": f"{args.cpu_steps} full steps of {wl.name} on the CPU "
                                          "restatement (OpenMP)"}
        if args.cpu_one_core_steps > 0:
            dt1 = cpu_oracle(wl, u, y, args.cpu_one_core_steps, 1)
            line["cpu_baseline"]["one_core"] = {
                "value": N * args.cpu_one_core_steps / dt1 / 1e6, "unit": "MLUPS", "cores": 1,
                "sample": f"{args.cpu_one_core_steps} full step(s) of {wl.name}, one thread"}
    rep.barrier()
    if rep.leader:
        print(json.dumps(line), flush=True)
    rep.close()


if __name__ == "__main__":
    main()
