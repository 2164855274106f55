#!/usr/bin/env python
"""Benchmark of the FastS solve step on GB300.

Workload (the configuration the headline metric is quoted on): laminar
Taylor-Green vortex on a 256^3 periodic box, Re 1600, Mach 0.1, AUSM+(P) o3,
implicit dual time stepping with 4 LU-SGS sub-iterations, FP64.  A "step" is
one physical time step (all sub-iterations).  Synthetic data generated by
fast_gb300.cases (the reference's benchmarks use no public dataset).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Prints one JSON line.  `value` = Mcell-updates/s with the state resident in
HBM, device-timed with CUDA events on the solver stream; `e2e` = the same
metric through fasts._compute with host arrays (levels n, n-1 copied in, the
new level copied out every step).  The state (>= 700 MB) is larger than L2,
so no flush is needed between steps.  Multi-GPU: replicas (one independent
case per GPU, weak scaling), value = all ranks' cell updates / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mcell-updates/s; time to 1e-10 residual drop, mixed vs FP64; adjoint/primal cost"
UNIT = "Mcell-updates/s"
# compulsory FP64 traffic per cell and launch group (8 B words, NEQ = 5):
# residual (W^p, W^n, W^{n-1} in, drodm out) = 160 B; LU-SGS lower + upper
# (drodm, W^p, coe in / increment, W^{p+1} out) = 320 B per sub-iteration.
ALG_BYTES = {"residual": 160.0, "lu_sgs": 320.0}
# DRAM bytes per cell and launch group measured with ncu (dram__bytes_read.sum
# + dram__bytes_write.sum of every kernel of the group, one sub-iteration of
# the 160^3 case, FP64): LU-SGS = lu_gather (2.75 GB) + the dataflow sweep
# with one CTA per SM (5.05 GB) over 4.10 M cells; the plane-ordered records
# (64 words a cell) are written once and read by both sweeps, so the traffic
# scales with the cell count.  residual = three face_flux launches
# (1.01 GB) + assemble (1.03 GB).
DRAM_BYTES = {"residual": 497.0, "lu_sgs": 1904.0}
# FP64 arithmetic instructions per cell and launch group (thread level,
# DADD + DMUL + DFMA counted by ncu, `smsp__sass_thread_inst_executed_op_d*`,
# 160^3, a sub-iteration after the first): residual = face_flux i + j + k
# (197 + 196 + 197) + assemble (78); LU-SGS = lu_gather (109) + lower and
# upper sweep (260) + lu_newton (35).  The in-place sweeps of later
# sub-iterations also rebuild the k+1 entries and do the Newton update, so
# for LU-SGS this is a floor.  A DADD or DMUL issues at the DFMA rate, so the
# instruction peak is half the measured FP64 FMA FLOP rate.
FP64_INST = {"residual": 668.0, "lu_sgs": 404.0}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=256)
    p.add_argument("--ss", type=int, default=4)
    p.add_argument("--cpu-n", type=int, default=None,
                   help="CPU sample size (cells per side; default: the workload's)")
    p.add_argument("--no-ttc", action="store_true",
                   help="skip the time-to-1e-10 part of the default line")
    p.add_argument("--no-adjoint", action="store_true",
                   help="skip the adjoint/primal part of the default line")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-mixed", action="store_true",
                   help="skip the FP32-sweep steps reported beside the FP64 value")
    p.add_argument("--ttc", action="store_true",
                   help="time to a 1e-10 Newton residual drop, FP64 vs mixed sweeps")
    p.add_argument("--ttc-n", type=int, default=256)
    p.add_argument("--ttc-max", type=int, default=100, help="max sub-iterations per step")
    p.add_argument("--workload", default="tgv",
                   choices=["tgv", "channel", "batch", "adjoint", "vortex"],
                   help="tgv: the headline 256^3 case; channel: 48-block SA channel; "
                        "batch: 64 independent Taylor-Green cases; adjoint: gradient of the "
                        "C-grid wall force (cost against the primal, tangent and FD checks); "
                        "vortex: isentropic vortex 128x128x4, Roe + minmod, RK3 at CFL 0.5, "
                        "timed over --vortex-steps steps")
    p.add_argument("--vortex-steps", type=int, default=200)
    p.add_argument("--adj-nsteps", type=int, default=400, help="adjoint workload: RK3 steps")
    p.add_argument("--adj-ckpt", type=int, default=20, help="adjoint workload: checkpoint period")
    p.add_argument("--adj-graph", type=int, default=1, choices=[0, 1],
                   help="adjoint workload: replay the driver loops as CUDA graphs")
    p.add_argument("--adj-checks", type=int, default=1, choices=[0, 1],
                   help="adjoint workload: tangent / FD checks and the per-group breakdown")
    p.add_argument("--slope", default="o3", choices=["o3", "o3sc"],
                   help="tgv workload: MUSCL slope of the AUSM+(P) faces (o3sc adds the shock sensor)")
    p.add_argument("--lu-mode", type=int, default=2, choices=[0, 1, 2],
                   help="LU-SGS schedule: 2 dataflow (default), 1 grid barrier, 0 plane launches")
    p.add_argument("--lu-prefetch", type=int, default=1, choices=[0, 1],
                   help="dataflow LU-SGS sweep: L2 prefetch of each chunk's operands")
    p.add_argument("--compute-graph", type=int, default=1, choices=[0, 1],
                   help="record each fgb_compute signature as a CUDA graph and replay it")
    p.add_argument("--lu-grid", type=int, default=0,
                   help="LU-SGS sweep CTAs (0: every resident slot)")
    p.add_argument("--lu-precision", type=int, default=64, choices=[64, 32],
                   help="64: plain FP64 path; 32: FP32 LU-SGS sweeps (mixed precision)")
    return p.parse_args()


# ----------------------------------------------------------- distributed
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


def replica_throughput(d, cells, steps, ms):
    """Whole-job Mcell-updates/s of N independent replicas (one case per
    rank, no collective on the data path): every rank's cell updates over
    the slowest rank's time.  Returns (value, max ms over ranks)."""
    ms_max = d.max(ms)
    return d.world * cells * steps / (ms_max * 1e-3) / 1e6, ms_max


# ----------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi sampling during the timed region (every 200 ms)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU side
def cpu_sample(n, ss, steps=1, min_seconds=0.0, slope="o3", warmup=0):
    """The oracle (C restatement of the FastS kernels, OpenMP on every host
    core, one LU-SGS block per thread as FastS does) on the n^3 Taylor-Green
    workload: `warmup` untimed physical steps, then `steps` timed ones,
    continued until `min_seconds` of CPU time have elapsed.  Returns
    (Mcell-updates/s, threads, seconds, steps, per-step seconds)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    from fast_gb300 import cases, fasts
    threads = os.cpu_count() or 1
    t = cases.taylor_green(n=n, ss_iteration=ss, slope=slope,
                           numb={"temporal_scheme": "implicit", "ss_iteration": ss,
                                 "modulo_verif": 200})
    m = fasts.prepare(t)
    c = oracle.Case(fasts.zone_data(t, m))
    del t, m
    oracle.set_threads(threads)
    oracle.load().or_set_lu_tiles(threads)
    c.apply_bc(0)
    c.apply_bc(1)
    it = 0
    for _ in range(warmup):
        it += 1
        c.compute(it, 1, ss + 1, 1, modulo_verif=200)
    per = []
    t0 = time.perf_counter()
    while len(per) < steps or (time.perf_counter() - t0 < min_seconds and len(per) < 10000):
        it += 1
        t1 = time.perf_counter()
        c.compute(it, 1, ss + 1, 1, modulo_verif=200)
        per.append(time.perf_counter() - t1)
    dt = time.perf_counter() - t0
    oracle.load().or_set_lu_tiles(1)
    return n ** 3 * len(per) / dt / 1e6, threads, dt, len(per), per


def run_reference(args, d: Dist):
    """The reference arm: FastS's OpenMP CPU path on the host cores.  FastS
    itself cannot be built here (no Fortran compiler, no Cassiopee), so the
    oracle port of its kernels stands in for it (kind "port"), on the same
    workload as our arm (n^3 Taylor-Green, same numerics), one physical step
    per timed step."""
    if d.rank != 0:
        return
    n = args.n
    value, threads, secs, nst, per = cpu_sample(n, args.ss, args.steps, slope=args.slope,
                                                warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / nst, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"taylor_green_{n}^3_ausmpred_{args.slope}_implicit_lusgs_ss{args.ss}",
                   "cells": n ** 3, "sub_iterations": args.ss, "lu_precision": 64,
                   "parallelism": f"host OpenMP x{threads}", "same_config": True},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"taylor_green {n}^3 (the full workload), {nst} physical "
                                   f"steps of {args.ss} LU-SGS sub-iterations, one LU block "
                                   f"per thread, after {args.warmup} untimed steps"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- GPU side
def run_ours(args, d: Dist):
    import json as _json
    from fast_gb300 import cases, fasts, fastc
    from fast_gb300 import _native
    dev = d.local
    n, ss = args.n, args.ss
    cells = n ** 3
    peaks = {}
    pf = ROOT / "MEASURED_PEAKS.json"
    if pf.exists():
        peaks = _json.loads(pf.read_text())
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_kind = "measured" if "hbm_gbs" in peaks else "fallback"

    # FastS defaults: residual check every 200 steps (modulo_verif)
    t = cases.taylor_green(n=n, ss_iteration=ss, slope=args.slope,
                           numb={"temporal_scheme": "implicit", "ss_iteration": ss,
                                 "modulo_verif": 200})
    t, tc, metrics = fasts.warmup(t, None, device=dev, gpu_resident=True)
    s = fasts.HOOK["solver"]
    s.set_option("lu_precision", args.lu_precision)
    s.set_option("lu_mode", args.lu_mode)
    s.set_option("lu_grid", args.lu_grid)
    s.set_option("lu_prefetch", args.lu_prefetch)
    s.set_option("compute_graph", args.compute_graph)
    it = 1
    for _ in range(args.warmup):
        fasts._compute(t, metrics, it)
        it += 1
    s.synchronize()

    # ---- device-resident timed region
    clocks = Clocks(dev)
    d.barrier()
    s.synchronize()
    l0 = s.launch_count()
    clocks.start()
    s.timer_start()
    for _ in range(args.steps):
        fasts._compute(t, metrics, it)
        it += 1
    ms = s.timer_stop()
    clk = clocks.stop()
    launches = s.launch_count() - l0
    tuned = s.get_option("lu_tuned")
    lu_sched = {"lu_mode": args.lu_mode, "autotuned": lu_choice(tuned),
                "trial_ms": lu_trials(s, 64) if tuned >= 0 else None}
    d.barrier()
    value, ms_max = replica_throughput(d, cells, args.steps, ms)

    # ---- the same steps with FP32 LU-SGS sweeps (FP64 residual, update and
    # norms): reported beside the FP64 value, not part of it
    mixed = None
    if args.lu_precision == 64 and not args.no_mixed:
        s.set_option("lu_precision", 32)
        fasts._compute(t, metrics, it)   # untimed: first FP32 solve builds its work arrays
        it += 1
        d.barrier()
        s.synchronize()
        s.timer_start()
        for _ in range(args.steps):
            fasts._compute(t, metrics, it)
            it += 1
        ms32 = s.timer_stop()
        d.barrier()
        v32, ms32_max = replica_throughput(d, cells, args.steps, ms32)
        t32 = s.get_option("lu_tuned32")
        mixed = {"value": v32, "unit": UNIT, "ms_per_step": ms32_max / args.steps,
                 "dtype": "f64+f32-sweeps",
                 "lu_autotuned": lu_choice(t32),
                 "lu_trial_ms": lu_trials(s, 32) if t32 >= 0 else None}
        s.set_option("lu_precision", 64)
        fasts._compute(t, metrics, it)   # back on the FP64 path before the profiled step
        it += 1

    # ---- per-kernel groups (separate profiled step; not part of `value`)
    s.set_option("profile", 1)
    s.kernel_stats(reset=True)
    fasts._compute(t, metrics, it)
    it += 1
    stats = s.kernel_stats(reset=True)
    s.set_option("profile", 0)
    groups = {"residual": ("face_flux", "assemble_bdf"), "lu_sgs": ("lu_sgs",)}
    gt = {}
    for g, names in groups.items():
        cnt = max((stats.get(nm, (0, 0.0))[0] for nm in names), default=0)
        tot = sum(stats.get(nm, (0, 0.0))[1] for nm in names)
        if cnt:
            gt[g] = (cnt, tot)
    dom = max(gt, key=lambda g: gt[g][1])
    cnt, tot = gt[dom]
    avg_ms = tot / cnt
    achieved = ALG_BYTES[dom] * cells / (avg_ms * 1e-3) / 1e9
    fp64 = _native.fp64_peak_gflops(dev)
    total_prof = sum(v[1] for v in stats.values())
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": achieved / hbm_peak,
        "traffic": DRAM_BYTES[dom] * cells if args.lu_precision == 64 else None,
        "traffic_source": "ncu at 160^3, bytes per cell scaled to this cell count",
        "peak_source": peak_kind,
        "avg_launch_ms": avg_ms,
        "fp64_fma_peak_gflops_measured": fp64,
        "fp64_issue": {
            "unit": "G FP64 instructions/s (DADD + DMUL + DFMA, thread level)",
            "peak": fp64 / 2.0,
            "inst_per_cell": FP64_INST,
            "achieved": {g: FP64_INST[g] * cells / (gt[g][1] / gt[g][0] * 1e-3) / 1e9 for g in gt},
            "frac": {g: FP64_INST[g] * cells / (gt[g][1] / gt[g][0] * 1e-3) / 1e9 / (fp64 / 2.0)
                     for g in gt},
        } if args.lu_precision == 64 else None,
        "kernel_share": {k: round(v[1] / total_prof, 4) for k, v in stats.items()},
    }

    # ---- end to end through the public API with host arrays
    e2e = None
    if not args.no_e2e:
        fasts._syncHost(t)
        fasts.HOOK["gpu_resident"] = False
        nd = (n + 4) ** 3
        k2 = args.steps
        fasts._compute(t, metrics, it)   # untimed first call (page-in)
        it += 1
        d.barrier()
        t0 = time.perf_counter()
        for _ in range(k2):
            fasts._compute(t, metrics, it)
            it += 1
        s.synchronize()
        el = d.max(time.perf_counter() - t0)
        e2e = {"value": d.world * cells * k2 / el / 1e6, "unit": UNIT,
               "h2d_bytes_per_step": 2 * 5 * nd * 8, "d2h_bytes_per_step": 5 * nd * 8,
               "steps": k2, "timer": "host wall clock around fasts._compute"}

    s.close()
    fasts.HOOK = None

    # ---- the other two parts of the metric (rank 0, N = 1 line only)
    ttc = adj = None
    if d.rank == 0 and d.world == 1 and not args.no_ttc and args.lu_precision == 64:
        ttc = ttc_measure(args.ttc_n, args.ttc_max)
        if mixed is not None:
            mixed["error_vs_fp64"] = ttc.pop("error_mixed_vs_fp64")
            mixed["time_to_1e-10_speedup_vs_fp64"] = ttc["speedup_mixed_vs_fp64"]
    if d.rank == 0 and d.world == 1 and not args.no_adjoint:
        adj = adjoint_measure(args, checks=True)

    cpu = None
    if d.rank == 0 and not args.no_cpu:
        cn = args.cpu_n or n
        v, threads, sec, nst, _ = cpu_sample(cn, ss, 1, min_seconds=10.0, slope=args.slope)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"taylor_green {cn}^3, {nst} physical steps ({ss} LU-SGS "
                         f"sub-iterations each), {sec:.1f} s, one LU block per thread"}
    d.barrier()
    if d.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": d.world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.lu_precision == 64 else "f64+f32-sweeps",
            "data": "synthetic",
            "config": {"workload": f"taylor_green_{n}^3_ausmpred_{args.slope}_implicit_lusgs_ss{ss}",
                       "lu_precision": args.lu_precision,
                       "cells": cells, "global_batch": d.world, "sub_iterations": ss,
                       "parallelism": f"replicas x{d.world}",
                       "l2": "state (>=700 MB) larger than L2; no flush"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": launches,
            "kernel_ms_per_step": {k: v[1] for k, v in stats.items()},
            "lu_schedule": lu_sched,
            "mixed_precision": mixed,
            "ttc": ttc,
            "adjoint": adj,
        }
        print(json.dumps(line), flush=True)


def lu_choice(v):
    """The LU-SGS autotuner's choice from get_option("lu_tuned"):
    1000 x warps per CTA (dataflow) + 10 x lu_mode + CTAs per SM."""
    if v < 0:
        return None
    v = int(v)
    out = {"lu_mode": (v % 1000) // 10, "ctas_per_sm": v % 10}
    if v // 1000:
        out["warps_per_cta"] = v // 1000
    return out


def lu_trials(s, prec):
    """The autotuner's trial times (ms) of the first LU group: grid barrier;
    dataflow 8 warps x 1, 2, 4 CTAs per SM; dataflow 4 warps x 1, 2."""
    names = ["grid_barrier", "flow_8w_x1", "flow_8w_x2", "flow_8w_x4", "flow_4w_x1", "flow_4w_x2"]
    return {n: round(s.get_option(f"lu_trial_ms{prec}_{c}"), 3) for c, n in enumerate(names)}


def run_multizone(args):
    """Workloads beside the headline, on one GPU, one solver: the 48-block
    Spalart-Allmaras channel (2.1 M cells, 1-to-1 interfaces), 64 independent
    Taylor-Green cases (48^3..96^3), or the isentropic vortex of 128 x 128 x 4
    cells (explicit RK3 at CFL 0.5; 2.2 M state bytes per level, so it runs
    from L2 and is bound by launches, not HBM).  Zones run one after another within each
    sub-step; interfaces and BCs are filled after every sub-step.  Value =
    interior cells of all zones x physical steps / device time."""
    import numpy as np
    from fast_gb300 import cases, fasts
    steps = args.steps
    if args.workload == "channel":
        t, tc = cases.sa_channel(ss_iteration=args.ss, modulo_verif=200)
        name = f"sa_channel_48_blocks_ausmpred_o3_implicit_lusgs_ss{args.ss}"
    elif args.workload == "vortex":
        t, tc = cases.isentropic_vortex(cfl=0.5), None
        name = "isentropic_vortex_128x128x4_roe_minmod_rk3_cfl0.5"
        steps = args.vortex_steps
    else:
        t, _ = cases.tgv_batch(ss_iteration=args.ss, modulo_verif=200)
        tc = None
        name = f"tgv_batch_64_cases_ausmpred_o3_implicit_lusgs_ss{args.ss}"
    t, tc, metrics = fasts.warmup(t, tc, gpu_resident=True)
    s = fasts.HOOK["solver"]
    s.set_option("lu_precision", args.lu_precision)
    s.set_option("lu_mode", args.lu_mode)
    s.set_option("lu_grid", args.lu_grid)
    s.set_option("lu_prefetch", args.lu_prefetch)
    s.set_option("compute_graph", args.compute_graph)
    cells = sum(int(np.prod(z[1][:, 0] - 1 - 4)) for z in fasts.HOOK["zones"])
    it = 1
    for _ in range(args.warmup):
        fasts._compute(t, metrics, it)
        it += 1
    s.synchronize()
    clocks = Clocks(0)
    l0 = s.launch_count()
    clocks.start()
    s.timer_start()
    for _ in range(steps):
        fasts._compute(t, metrics, it)
        it += 1
    ms = s.timer_stop()
    clk = clocks.stop()
    launches = s.launch_count() - l0
    s.set_option("profile", 1)
    s.kernel_stats(reset=True)
    fasts._compute(t, metrics, it)
    stats = s.kernel_stats(reset=True)
    s.set_option("profile", 0)
    line = {"metric": METRIC, "value": cells * steps / (ms * 1e-3) / 1e6, "unit": UNIT,
            "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if args.lu_precision == 64 else "f64+f32-sweeps", "data": "synthetic",
            "config": {"workload": name, "zones": len(fasts.HOOK["zones"]), "cells": cells,
                       "lu_precision": args.lu_precision, "sub_iterations": args.ss,
                       "compute_graph": args.compute_graph},
            "clocks": clk, "gpu_launches": launches,
            "kernel_ms_per_step": {k: v[1] for k, v in stats.items()}}
    print(json.dumps(line), flush=True)


def adjoint_measure(args, checks=True):
    """Adjoint / primal cost on the differentiation case: C-grid 385 x 129,
    8 Hicks-Henne amplitudes + M_inf, Roe + van Albada, RK3, 400 steps,
    checkpoints every 20.  Times (CUDA-synchronised wall clock of the
    device work) of the primal run and of the adjoint (recomputation +
    reverse sweep), the gradient, its agreement with the forward-mode tangent
    along two directions and with central differences (h = 1e-6, 1e-7)."""
    import numpy as np
    import torch
    from fast_gb300 import adjoint as A
    case = A.CGridCase(nsteps=args.adj_nsteps, ckpt=args.adj_ckpt)
    case.graph = bool(args.adj_graph)
    alpha = torch.from_numpy(np.random.default_rng(4).uniform(-0.005, 0.005, 8))
    mach = torch.tensor(0.7, dtype=torch.float64)
    for _ in range(max(1, min(args.warmup, 3))):
        A.gradient(case, alpha, mach)
    prim, adj = [], []
    for _ in range(max(1, min(args.steps, 5))):
        J, ga, gm = A.gradient(case, alpha, mach)
        prim.append(case.timing["primal_s"])
        adj.append(case.timing["adjoint_s"])
    grad = np.concatenate([ga, [gm]])
    tp, ta = float(np.median(prim)), float(np.median(adj))
    out = {"value": ta / tp, "unit": "x primal", "higher_is_better": False,
           "primal_s": tp, "adjoint_s": ta, "J": J, "gradient": grad.tolist(),
           "workload": f"cgrid_385x129_roe_vanalbada_rk3_{case.nsteps}_steps_ckpt{case.ckpt}",
           "parameters": "8 Hicks-Henne amplitudes + M_inf", "cuda_graphs": case.graph}
    if checks:
        rng = np.random.default_rng(5)
        tang = []
        for _ in range(2):
            dd = rng.standard_normal(9)
            dJ = A.tangent(case, alpha, mach, torch.from_numpy(dd[:8]),
                           torch.tensor(dd[8], dtype=torch.float64))
            tang.append(abs(dJ - grad @ dd) / abs(dJ))
        scale = float(np.max(np.abs(grad)))
        fd6 = A.fd_gradient(case, alpha, mach, h=1e-6)
        fd7 = A.fd_gradient(case, alpha, mach, h=1e-7)
        out.update({"tangent_rel_err": tang,
                    "fd_rel_err_h1e-6": float(np.max(np.abs(fd6 - grad)) / scale),
                    "fd_rel_err_h1e-7": float(np.max(np.abs(fd7 - grad)) / scale),
                    "fd_rel_err_per_component_h1e-7":
                        (np.abs(fd7 - grad) / np.maximum(np.abs(grad), 1e-300)).tolist()})
    return out


def run_adjoint(args):
    """--workload adjoint: the adjoint/primal line on its own, with the
    per-group breakdown of one adjoint (stream launches, CUDA events)."""
    import numpy as np
    import torch
    from fast_gb300 import adjoint as A
    out = adjoint_measure(args, checks=bool(args.adj_checks))
    if args.adj_checks:
        case = A.CGridCase(nsteps=args.adj_nsteps, ckpt=args.adj_ckpt)
        case.profile = True
        alpha = torch.from_numpy(np.random.default_rng(4).uniform(-0.005, 0.005, 8))
        A.gradient(case, alpha, torch.tensor(0.7, dtype=torch.float64))
        out["eager_profiled_groups_ms"] = case.timing.get("groups_ms", {})
    line = {"metric": "adjoint/primal cost", "value": out.pop("value"), "unit": out.pop("unit"),
            "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": out.pop("workload"), "parameters": out.pop("parameters"),
                       "mach": 0.7, "cuda_graphs": out.pop("cuda_graphs")}, **out}
    print(json.dumps(line), flush=True)


def ttc_measure(n, ttc_max):
    """Time to a 1e-10 drop of the Newton residual within one physical step.

    One BDF2 step (after one BDF1 step) of the n^3 Taylor-Green case with up
    to ttc_max LU-SGS sub-iterations, residual norms (FP64, computed by the GPU
    as cprdu3s1 does) recorded at every sub-iteration.  The drop is that of
    the system residual, sqrt(sum_e L2_e(k)^2) / sqrt(sum_e L2_e(1)^2) over
    the 5 equations (the w-momentum residual of the Taylor-Green vortex starts
    far below the others, so a per-equation maximum says little; the
    per-equation drops are reported as well); time = sub-iterations to reach
    1e-10 x measured time per sub-iteration.  FP64 sweeps vs FP32 sweeps (the
    residual, the update and the norms stay FP64).  Both runs continue to
    ttc_max sub-iterations, past the 1e-10 drop; the error of the mixed
    final state against the FP64 one is reported per variable, as the largest
    cell difference over the variable's largest magnitude (interior cells)."""
    from fast_gb300 import cases, fasts
    from fast_gb300 import fastc, pytree as I
    import numpy as np
    out = {}
    for prec in (64, 32):
        t = cases.taylor_green(n=n, ss_iteration=ttc_max,
                               numb={"temporal_scheme": "implicit",
                                     "ss_iteration": ttc_max, "modulo_verif": 1})
        t, tc, metrics = fasts.warmup(t, None, gpu_resident=True)
        s = fasts.HOOK["solver"]
        s.set_option("lu_precision", prec)
        fasts._compute(t, metrics, 1)          # BDF1 step
        s.synchronize()
        s.timer_start()
        fasts._compute(t, metrics, 2)          # BDF2 step, timed
        ms = s.timer_stop()
        r = s.residuals(0)                     # (2*neq, nit)
        l2 = r[:5]
        tot = np.sqrt(np.sum(l2 * l2, axis=0))
        drop = tot / tot[0]
        per_eq = l2 / np.where(l2[:, :1] > 0, l2[:, :1], 1.0)
        nit = l2.shape[1]
        ms_it = ms / nit
        hit = np.nonzero(drop <= 1e-10)[0]
        k = int(hit[0]) + 1 if hit.size else None
        fasts._syncHost(t)
        out[prec] = {"sub_iterations_to_1e-10": k, "sub_iterations_run": int(nit),
                     "ms_per_sub_iteration": ms_it,
                     "time_to_1e-10_ms": (k * ms_it) if k else None,
                     "best_drop": float(drop.min()),
                     "drop_history": [float(x) for x in drop],
                     "initial_l2_per_equation": [float(x) for x in l2[:, 0]],
                     "final_drop_per_equation": [float(x) for x in per_eq[:, -1]]}
        z = I.getZones(t)[0]
        pi = I.getNodeFromName1(I.getNodeFromName1(z, ".Solver#ownData"), "Parameter_int")[1]
        ni, nj, nk = (int(pi[20 + d]) for d in range(3))
        q = fastc.compactArray(z, "").reshape(5, nk + 4, nj + 4, ni + 4)
        out[prec]["_state"] = q[:, 2:-2, 2:-2, 2:-2].copy()
        s.close()
        fasts.HOOK = None
    a, b = out[64].pop("_state"), out[32].pop("_state")
    names = ("density", "velocity_x", "velocity_y", "velocity_z", "temperature")
    err = {nm: float(np.max(np.abs(b[v] - a[v])) / np.max(np.abs(a[v])))
           for v, nm in enumerate(names)}
    t64, t32 = out[64]["time_to_1e-10_ms"], out[32]["time_to_1e-10_ms"]
    return {"workload": f"taylor_green_{n}^3_ausmpred_o3_bdf2_one_step",
            "fp64": out[64], "mixed": out[32],
            "speedup_mixed_vs_fp64": (t64 / t32) if (t64 and t32) else None,
            "error_mixed_vs_fp64": {"per_variable_max_abs_over_scale": err,
                                    "max": max(err.values()),
                                    "at": f"both after {out[64]['sub_iterations_run']} "
                                          f"sub-iterations (past the 1e-10 drop)"}}


def run_ttc(args):
    """--ttc: the time-to-1e-10 line on its own."""
    r = ttc_measure(args.ttc_n, args.ttc_max)
    line = {"metric": "time to 1e-10 residual drop (one BDF2 step)", "unit": "ms",
            "higher_is_better": False, "config": {"workload": r.pop("workload")}, **r}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.ttc:
        run_ttc(args)
        return
    if args.workload == "adjoint" and args.impl == "ours":
        run_adjoint(args)
        return
    if args.workload != "tgv" and args.impl == "ours":
        run_multizone(args)
        return
    d = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, d)
        else:
            run_ours(args, d)
    finally:
        d.close()


if __name__ == "__main__":
    main()
