"""Benchmark of the GB300 2D GKS / WENO-AO-DF / S2O4 step.

Workload (one "step" = one full two-stage S2O4 step of every interior cell): the 2D
four-quadrant Riemann problem on [0,1]^2 at 1024 x 1024 cells, WENO7-AO-DF in
characteristic variables with 3 Gauss points per face, GKS flux with c1 = 0.05, c2 = 1,
outflow boundaries, CFL 0.5 -- the reference's PlanarShock setup at the benchmark size.
Seeded synthetic initial data; no dataset is involved.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``value`` is cell-updates/s of the plain FP64 path with the state
resident in HBM (CUDA events on the solver's stream, L2 flushed between steps, summed
over K steps, max over ranks); ``e2e`` is the same metric through the C ABI with host
buffers (upload, step, download every step).  ``variants`` reports the FP32-bulk path and
its density deviation from the FP64 run.  ``--impl reference`` times the CPU
implementation of the same step on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "high-order-solver_gb300"))

N_CELLS = 1024
ORDER = 7
WORKLOAD = "riemann2d_1024x1024_weno7ao_df_char_gp3_gks_s2o4"
METRIC = "cell-updates/s per S2O4 step"
# FP64 operations one face-kernel launch executes per face (2 x DFMA + DADD + DMUL, counted
# by ncu on the 256^2 case), and the algorithmic HBM bytes of one face-kernel launch per
# face: W (32 B) + two DF indicators (16 B) read, stage flux (32 B) + face alpha (8 B)
# written, stage-0 partial written or read (32 B).
FLOP_PER_FACE = 24028.0
BYTES_PER_FACE = 120.0
# dram__bytes_read + write per face of one face-kernel launch (ncu, 256^2 case: 4.02 MB / 65,792)
TRAFFIC_PER_FACE = 61.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_CELLS, help=argparse.SUPPRESS)
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-problem batched sweep")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def run_reference(args):
    """CPU implementation of the same step on all host cores (oracle/_ref where the
    reference compiled on this host, else the repository's restatement)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "tests"))
    from hos_gb300 import cases
    from oracle_lib import CpuStep, ORACLE_DIR

    kind = "reference" if (ORACLE_DIR / "_ref" / "libhosref.so").exists() else "port"
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    pb, con, prim = cases.riemann2d(args.n, order=ORDER)
    cpu = CpuStep("ref" if kind == "reference" else "oracle").init(pb, threads=cores)
    cpu.set_state(con, prim)
    t0 = time.perf_counter()
    cpu.step()
    one = time.perf_counter() - t0
    n = args.n
    if (args.steps + args.warmup) * one > 150.0:  # keep the run within a few minutes
        n = 256
        pb, con, prim = cases.riemann2d(n, order=ORDER)
        cpu = CpuStep("ref" if kind == "reference" else "oracle").init(pb, threads=cores)
        cpu.set_state(con, prim)
    for _ in range(args.warmup):
        cpu.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu.step()
    el = time.perf_counter() - t0
    v = n * n * args.steps / el
    sample = f"{n}x{n} Riemann WENO7-AO-DF, {args.steps} S2O4 steps after {args.warmup} warm-up"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD if n == N_CELLS else WORKLOAD.replace("1024x1024", f"{n}x{n}"),
                       "cells": n * n, "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_sample():
    """The oracle timed on the host cores on a bounded sample (256^2, ~10 s of CPU work)."""
    sys.path.insert(0, str(ROOT / "tests"))
    from hos_gb300 import cases
    from oracle_lib import CpuStep, ORACLE_DIR

    kind = "reference" if (ORACLE_DIR / "_ref" / "libhosref.so").exists() else "port"
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    n = 256
    pb, con, prim = cases.riemann2d(n, order=ORDER)
    cpu = CpuStep("ref" if kind == "reference" else "oracle").init(pb, threads=cores)
    cpu.set_state(con, prim)
    cpu.step()
    steps, el = 0, 0.0
    t0 = time.perf_counter()
    while el < 8.0 and steps < 200:
        cpu.step()
        steps += 1
        el = time.perf_counter() - t0
    return {"value": n * n * steps / el, "unit": "cell-updates/s", "cores": cores, "kind": kind,
            "sample": f"{n}x{n} Riemann WENO7-AO-DF, {steps} S2O4 steps after 1 warm-up"}


def batch_leg(dev, precision, count=64, seed=0, max_steps=4000):
    """The batched sweep: ``count`` seeded shock-vortex / wedge problems (sides 128..768) in one
    batch, face-tile shapes chosen by the autotuner, every step one CUDA-graph replay.  Runs
    every problem to its end time; an event recorded after each step gives each problem's time
    to solution (the end of the last step it was active in)."""
    import torch

    from hos_gb300 import cases
    from hos_gb300.solver import Batch2D

    sweep = cases.batch_sweep(count=count, seed=seed)
    b = Batch2D([x[0] for x in sweep], [x[3] for x in sweep], precision)
    for k, x in enumerate(sweep):
        b.set_state(k, x[1], x[2])
    t0 = time.perf_counter()
    chosen, tune_ms = b.autotune(reps=3)
    tune_s = time.perf_counter() - t0
    ext = torch.cuda.ExternalStream(b.stream, device=dev)
    b.advance(1, graph=True)          # instantiates the graph (batch step index 0)
    for k, x in enumerate(sweep):     # back to the initial states
        b.set_state(k, x[1], x[2])
    base = 1
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    evs = []
    while len(evs) < max_steps:
        for _ in range(25):
            b.advance(1, graph=True)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(ext)
            evs.append(ev)
        if b.status(failed=True)[0] == 0:
            break
    torch.cuda.synchronize(dev)
    act, t, last, failed = b.status(failed=True)
    b.close()
    cells = np.array([x[0].nodex * x[0].nodey for x in sweep], dtype=np.float64)
    nsteps = last - base + 1          # steps each problem took (a failed one: up to its bad step)
    tts = np.array([e0.elapsed_time(evs[int(n) - 1]) / 1e3 for n in nsteps])
    done = ~failed
    total = e0.elapsed_time(evs[int(nsteps.max()) - 1]) / 1e3
    return {"problems": count, "seed": seed, "cells": int(cells.sum()),
            "value": float((cells * nsteps).sum() / total), "unit": "cell-updates/s",
            "wall_s": total, "batch_steps": int(nsteps.max()), "unfinished": int(act),
            "blown_up": int(failed.sum()),
            "blown_up_problems": [sweep[k][4] for k in np.flatnonzero(failed)],
            "steps_per_problem": {"min": int(nsteps.min()), "max": int(nsteps.max())},
            "time_to_solution_s": {"p50": float(np.percentile(tts[done], 50)),
                                   "p99": float(np.percentile(tts[done], 99)), "max": float(tts[done].max()),
                                   "over": "problems that reached their end time"},
            "tiles": {"x": "x".join(map(str, Batch2D.SHAPES[chosen[0]])),
                      "y": "x".join(map(str, Batch2D.SHAPES[chosen[1]]))},
            "autotune_ms": tune_ms.round(3).tolist(), "autotune_s": tune_s, "graph": True,
            "launches_per_step": 1 + 2 * 4, "gate": "off"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import torch.distributed as dist

    from hos_gb300 import cases
    from hos_gb300.solver import FP32, FP64, Solver2D

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.n
    pb, con, prim = cases.riemann2d(n, order=ORDER)
    cells = pb.nodex * pb.nodey

    # 256 MB buffer written between timed steps to flush the 129 MB L2
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def timed_steps(solver, k, w):
        ext = torch.cuda.ExternalStream(solver.stream, device=dev)
        for _ in range(w):
            solver.advance(1, 1e30, graph=True)
        solver.sync()
        total = 0.0
        evs = []
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize(dev)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
            solver.advance(1, 1e30, graph=True)
            b.record(ext)
            evs.append((a, b))
        solver.sync()
        for a, b in evs:
            total += a.elapsed_time(b) / 1e3
        return total

    # ---- plain FP64 path, state resident in HBM ----
    s64 = Solver2D(pb, FP64)
    s64.set_state(con, prim)
    with ClockSampler(local) as clk:
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)
        t64 = timed_steps(s64, args.steps, args.warmup)
        torch.cuda.synchronize(dev)
    if ws > 1:
        tt = torch.tensor([t64], device=dev, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t64 = float(tt.item())
    value = ws * cells * args.steps / t64
    rho64 = s64.get_state()["convar"][..., 0]
    # per-kernel device times of a few steps (L2 flushed before each)
    prof = []
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize(dev)
        prof.append(s64.profile_step(1e30))
    kern_ms = {k: float(np.mean([p[k] for p in prof])) for k in prof[0]}
    face_ms = float(np.mean([kern_ms[k] for k in ("face_x0", "face_y0", "face_x1", "face_y1")]))

    # ---- FP32-bulk path (FP64 state / accumulation), same steps, deviation vs FP64 ----
    s32 = Solver2D(pb, FP32)
    s32.set_state(con, prim)
    t32 = timed_steps(s32, args.steps, args.warmup)
    rho32 = s32.get_state()["convar"][..., 0]
    g = pb.ghost
    a, b = rho64[g:-g, g:-g], rho32[g:-g, g:-g]
    l1_dev = float(np.abs(a - b).mean() / np.abs(a).mean())
    linf_dev = float(np.abs(a - b).max() / np.abs(a).max())
    s32.close()

    # ---- end to end through the C ABI with pinned host buffers ----
    host_in = torch.from_numpy(np.ascontiguousarray(con.reshape(-1))).pin_memory()
    host_prim = torch.from_numpy(np.ascontiguousarray(prim.reshape(-1))).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    lib = s64._lib
    dp = ctypes.POINTER(ctypes.c_double)
    pin = ctypes.cast(host_in.data_ptr(), dp)
    ppr = ctypes.cast(host_prim.data_ptr(), dp)
    pout = ctypes.cast(host_out.data_ptr(), dp)
    ke = max(3, args.steps // 2)
    for _ in range(1):
        lib.hos2d_set_state(s64._h, pin, ppr)
        s64.step(1e30)
        lib.hos2d_get_state(s64._h, pout, None, None, None)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(ke):
        assert lib.hos2d_set_state(s64._h, pin, ppr) == 0
        s64.step(1e30)
        assert lib.hos2d_get_state(s64._h, pout, None, None, None) == 0
    te = time.perf_counter() - t0
    e2e_value = ws * cells * ke / te
    s64.close()

    hbm_peak, hbm_src = peaks()
    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return

    # FP64 peak measured here by cuBLAS DGEMM (the denominator of the compute roofline)
    m = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    torch.matmul(m, m)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        torch.matmul(m, m)
    e1.record()
    torch.cuda.synchronize(dev)
    dgemm_tflops = 3 * 2 * 4096 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12

    ms = 1e3 * t64 / args.steps
    faces_per_launch = (pb.nodex + 1) * pb.nodey
    achieved_gbs = BYTES_PER_FACE * faces_per_launch / (face_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": cells, "order": ORDER, "gauss_points": 3,
                   "characteristic": True, "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "flushed between timed steps (256 MB write)"},
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": int(2 * host_in.numel() * 8),
                "d2h_bytes_per_step": int(host_out.numel() * 8)},
        "gpu_launches": args.steps * 9,
        "roofline": {"kernel": "face_kernel<double,7,x|y>", "bound": "fp64", "unit": "TFLOP/s",
                     "achieved": None, "peak": dgemm_tflops,
                     "peak_source": "cuBLAS DGEMM 4096^3 measured in this run", "frac": None,
                     "traffic": TRAFFIC_PER_FACE * faces_per_launch, "launch_ms": face_ms,
                     "hbm": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                             "frac": achieved_gbs / hbm_peak, "peak_source": hbm_src}},
        "variants": {"fp32_bulk": {"value": cells * args.steps / t32, "unit": "cell-updates/s",
                                   "speedup_vs_fp64": t64 / t32, "rho_rel_l1_vs_fp64": l1_dev,
                                   "rho_rel_linf_vs_fp64": linf_dev}},
        "kernels_ms": kern_ms,
        "clocks": clk.summary(),
    }
    if FLOP_PER_FACE:
        ach = FLOP_PER_FACE * faces_per_launch / (face_ms / 1e3) / 1e12
        line["roofline"]["achieved"] = ach
        line["roofline"]["frac"] = ach / dgemm_tflops
    if ws == 1:
        line["cpu_baseline"] = cpu_baseline_sample()
    if not args.no_batch:
        line["variants"]["batch64_fp32"] = batch_leg(dev, FP32)
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
