"""Benchmark of the GB300 2D GKS / WENO-AO-DF / S2O4 step.

Workload (one "step" = one full two-stage S2O4 step of every interior cell): the 2D
four-quadrant Riemann problem on [0,1]^2 at 1024 x 1024 cells, WENO7-AO-DF in
characteristic variables with 3 Gauss points per face, GKS flux with c1 = 0.05, c2 = 1,
outflow boundaries, CFL 0.5 -- the reference's PlanarShock setup at the benchmark size.
Seeded synthetic initial data; no dataset is involved.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``value`` is cell-updates/s of the gated FP32 form (reconstruction,
flux and the learned gate in FP32/BF16; state, stage combination and CFL in FP64) with the
state resident in HBM (CUDA events on the solver's stream, L2 flushed between steps, summed
over K steps, max over ranks); ``plain_fp64`` is the plain FP64 path on the same data and
``accuracy`` the density deviation between them after the same steps.  The gate is trained
first on the solver's own 256^2 / 512^2 random-quadrant runs.  ``e2e`` is the headline metric
through the C ABI with host buffers (upload, step, download every step).  ``--impl reference``
times the CPU implementation of the same step on the host cores.
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
METRIC = "cell-updates/s per S2O4 step: gated FP32 vs plain FP64 on GB300 at stated L1 error"
# FP64 operations one face-kernel launch executes per face (2 x DFMA + DADD + DMUL, counted
# by ncu on the 256^2 case), and the algorithmic HBM bytes of one face-kernel launch per
# face: W (32 B) + two DF indicators (16 B) read, stage flux (32 B) + face alpha (8 B)
# written, stage-0 partial written or read (32 B).
FLOP_PER_FACE = 24028.0
BYTES_PER_FACE = 120.0
# dram__bytes_read + write per face of one face-kernel launch (ncu, 256^2 case: 4.02 MB / 65,792)
TRAFFIC_PER_FACE = 61.0
# FP32 operations (2 x FFMA + FADD + FMUL) one gated FP32 face-kernel launch (TMA staging,
# 16 x 16-face tiles) executes per face, and its DRAM traffic per face averaged over the
# stage-0 and stage-1 launches (ncu, --case gated1024: 1024^2 Riemann WENO7, 7.04e9 flop and
# 46-71 MB per launch over 1,049,600 faces)
FP32_FLOP_PER_FACE_GATED = 6716.0
TRAFFIC_PER_FACE_FP32 = 55.7
AUDIT_LOG2 = 10   # audit one warp in 1024 of predicted-smooth cells with full weights
N_3D = 256        # cells per side of the 3D Taylor-Green leg
# 3D point kernel (tangential point sweep + GKS3D at 4 Gauss points + FP64 stage combination):
# flop per face (2 x FMA + ADD + MUL; ncu, 64^3 TGV) of the FP32 and FP64 builds, and the FP32
# build's DRAM bytes per face
FP32_FLOP_PER_FACE_POINT3 = 28400.0
FP64_FLOP_PER_FACE_POINT3 = 37100.0
TRAFFIC_PER_FACE_POINT3 = 289.0
# the gated FP32 point kernel on the Taylor-Green vortex (every face flagged smooth; ncu, 64^3):
# flop per face and DRAM bytes per face
GATED_FLOP_PER_FACE_POINT3 = 17440.0
GATED_TRAFFIC_PER_FACE_POINT3 = 290.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_CELLS, help=argparse.SUPPRESS)
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-problem batched sweep")
    ap.add_argument("--no-3d", action="store_true", help="skip the 3D Taylor-Green leg")
    ap.add_argument("--no-endtime", action="store_true", help="skip the 1024^2 end-time accuracy leg")
    ap.add_argument("--batch-failures", action="store_true",
                    help="run every problem the gated FP32 batch loses to a blow-up alone: plain FP64 on the GPU "
                         "and the FP64 restatement on the host cores, with the step where each stops")
    ap.add_argument("--endtime", action="store_true",
                    help="accuracy studies at the end times instead of the bench line: 1024^2 Riemann to "
                         "t = 0.25 and 64^3 Taylor-Green to t = 10 (FP64, FP32 bulk, gated FP32)")
    ap.add_argument("--endtime-256", action="store_true", help="with --endtime: also gated FP32 256^3 to t = 10")
    ap.add_argument("--case", choices=["gated256", "gated1024", "tgv3d64"], default=None,
                    help="small profiling case: gated256 = gate trained as in the bench, then 21 plain FP32 "
                         "and 21 gated FP32 steps of the 256^2 WENO7 Riemann problem; gated1024 = the same "
                         "gate, then 2 gated FP32 steps of the 1024^2 problem; tgv3d64 = 2 FP32 and "
                         "1 FP64 steps of the 64^3 Taylor-Green vortex in NVTX ranges fp32 / fp64")
    return ap.parse_args()


def dist_env():
    from hos_gb300 import replicas
    return replicas.env()


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


def batch_leg(dev, precision, count=64, seed=0, max_steps=4000, gate=None, threshold=0.0):
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
    if gate is not None:
        b.set_gate(gate, threshold, audit_log2=AUDIT_LOG2)
    ext = torch.cuda.ExternalStream(b.stream, device=dev)
    b.advance(1, graph=True)          # instantiates the graph (batch step index 0)
    for k, x in enumerate(sweep):     # back to the initial states
        b.set_state(k, x[1], x[2])
    base = 1
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    evs = []
    # the drivers' first-order step 0 (e.g. src/2Dproblem.cpp:940-945), then WENO5-AO-DF
    b.set_reconstruction(True)
    b.advance(1, graph=True)
    ev = torch.cuda.Event(enable_timing=True)
    ev.record(ext)
    evs.append(ev)
    b.set_reconstruction(False)
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
    gst = b.gate_stats() if gate is not None else None
    b.close()
    cells = np.array([x[0].nodex * x[0].nodey for x in sweep], dtype=np.float64)
    nsteps = last - base + 1          # steps each problem took (a failed one: up to its bad step)
    tts = np.array([e0.elapsed_time(evs[int(n) - 1]) / 1e3 for n in nsteps])
    done = ~failed
    total = e0.elapsed_time(evs[int(nsteps.max()) - 1]) / 1e3
    # the aggregate counts the steps of the problems that reached their end time only
    return {"problems": count, "seed": seed, "cells": int(cells.sum()),
            "value": float((cells * nsteps)[done].sum() / total), "unit": "cell-updates/s",
            "value_over": "cell updates of the problems that reached their end time / wall time of the batch",
            "first_order_step0": True,
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
            "launches_per_step": 1 + 2 * (4 + (gate is not None)),
            "gate": "off" if gst is None else {
                "linear_path_fraction": (gst["smooth_x"] + gst["smooth_y"]) / max(1, gst["cells_x"] + gst["cells_y"]),
                "audited": gst["audited"], "audit_false_negative_rate": gst["false_neg"] / max(1, gst["audited"]),
                "aposteriori_rejections": gst["fallback"]}}


def endtime2d_leg(gate, rep, n=N_CELLS, tstop=0.25):
    """The four-quadrant Riemann problem at n^2 (WENO7-AO-DF, characteristic, 3 Gauss points) run
    to its end time t = 0.25 in plain FP64, plain FP32 bulk and gated FP32 from the same initial
    data: density deviation of each FP32 form from FP64 at t = 0.25 (relative L1 and L-inf over
    the interior cells), steps taken, and the gate's activity over the whole gated run (linear-path
    fraction, audits, false negatives among the audited, a-posteriori rejections).  Steps are
    graph replays; the time step is the solver's own CFL, clipped to the end time."""
    from hos_gb300 import cases
    from hos_gb300.solver import FP32, FP64, Solver2D

    pb, con, prim = cases.riemann2d(n, order=ORDER)
    g = pb.ghost
    rho, runs = {}, {}
    for name, prec, gated in (("fp64", FP64, False), ("fp32", FP32, False), ("gated", FP32, True),
                              ("gated_every_stage", FP32, True)):
        s = Solver2D(pb, prec)
        s.set_state(con, prim)
        if gated:
            s.set_gate(gate, rep.threshold, audit_log2=AUDIT_LOG2)
            s.set_gate_reuse(name == "gated")
            s.gate_stats(reset=True)
        t0 = time.perf_counter()
        steps = 0
        t, _ = s.sync()
        while t < tstop:
            s.advance(1, tstop, graph=True)
            steps += 1
            if steps % 16 == 0 or steps > 1000:
                t, _ = s.sync()
        t, _ = s.sync()
        wall = time.perf_counter() - t0
        rho[name] = s.get_state()["convar"][g:-g, g:-g, 0]
        runs[name] = {"steps": steps, "t": t, "wall_s": wall}
        if gated:
            st = s.gate_stats()
            cells = max(1, st["cells_x"] + st["cells_y"])
            fc = s.gate_audit_check()
            runs[name]["gate"] = {"linear_path_fraction": (st["smooth_x"] + st["smooth_y"]) / cells,
                                  "audited": st["audited"], "audit_false_negatives": st["false_neg"],
                                  "audit_false_negative_rate": st["false_neg"] / max(1, st["audited"]),
                                  "aposteriori_rejections": st["fallback"],
                                  # what the check did with the audited false negatives' linear
                                  # reconstructions: accepted (wrongly) or sent back to WENO-AO
                                  "false_negative_linear_reconstructions": fc["fn_linear"],
                                  "false_negative_accepted_by_check": fc["fn_linear_accepted"]}
        s.close()

    def rel(a, b, norm):
        d = np.abs(a - b)
        return float(d.mean() / np.abs(b).mean()) if norm == 1 else float(d.max() / np.abs(b).max())

    return {"grid": f"{n}x{n}", "t_end": tstop, "runs": runs,
            "rho_rel_l1_gated_vs_fp64": rel(rho["gated"], rho["fp64"], 1),
            "rho_rel_linf_gated_vs_fp64": rel(rho["gated"], rho["fp64"], 0),
            "rho_rel_l1_fp32_vs_fp64": rel(rho["fp32"], rho["fp64"], 1),
            "rho_rel_linf_fp32_vs_fp64": rel(rho["fp32"], rho["fp64"], 0),
            "rho_rel_l1_gated_vs_fp32": rel(rho["gated"], rho["fp32"], 1),
            "cells_off_by_1e-2_gated": float((np.abs(rho["gated"] - rho["fp64"]) > 1e-2 * np.abs(rho["fp64"])).mean()),
            "gated": "network at stage 0, its flags dilated by one cell at stage 1 (hos2d_set_gate_reuse)",
            "rho_rel_l1_gated_every_stage_vs_fp64": rel(rho["gated_every_stage"], rho["fp64"], 1),
            "rho_rel_linf_gated_every_stage_vs_fp64": rel(rho["gated_every_stage"], rho["fp64"], 0),
            "target": "rho_rel_l1_gated_vs_fp64 <= 1e-3"}


def endtime3d_leg(gate, rep, n=64, tstop=10.0, every=0.25, forms=("fp64", "fp32", "gated")):
    """The Taylor-Green vortex at n^3 (Re 1600, Mach 0.1, Pr 0.71; WENO5-AO, GKS3D with the
    Navier-Stokes collision time, S2O4) run to t = 10 in each form from the same initial data,
    stopping at the same checkpoints every ``every`` time units (the last step before each
    checkpoint is clipped to it, as the end time is): kinetic energy <rho |u|^2 / 2> at every
    checkpoint, the dissipation rate -dKE/dt from central differences of those, their largest
    deviation from FP64 (KE relative to the initial KE, the rate relative to FP64's peak rate),
    density deviation at t = 10, and the gate's activity per checkpoint interval."""
    from hos_gb300 import cases
    from hos_gb300.solver import FP32, FP64, Solver3D

    pb, con = cases.tgv3d(n)
    g = pb.ghost
    marks = np.round(np.arange(every, tstop + 0.5 * every, every), 10)
    ke, rho, runs = {}, {}, {}
    for name in forms:
        prec = FP64 if name == "fp64" else FP32
        s = Solver3D(pb, prec)
        s.set_state(con)
        if name == "gated":
            s.set_gate(gate, rep.threshold, audit_log2=AUDIT_LOG2)
            s.gate_stats(reset=True)
        kk, acts = [], []
        t0 = time.perf_counter()
        steps = 0

        def energy():
            st = s.get_state()["convar"][g:-g, g:-g, g:-g]
            return 0.5 * float(((st[..., 1] ** 2 + st[..., 2] ** 2 + st[..., 3] ** 2) / st[..., 0]).mean()), st

        kk.append(energy()[0])
        for tm in marks:
            steps += s.run(float(tm), check_every=20)
            e, st = energy()
            kk.append(e)
            if name == "gated":
                gs = s.gate_stats(reset=True)
                cells = max(1, gs["cells_x"] + gs["cells_y"] + gs["cells_z"])
                acts.append({"t": float(tm),
                             "linear_fraction": (gs["smooth_x"] + gs["smooth_y"] + gs["smooth_z"]) / cells,
                             "audited": gs["audited"], "false_neg": gs["false_neg"], "fallback": gs["fallback"]})
        runs[name] = {"steps_upper_bound": steps, "wall_s": time.perf_counter() - t0, "t": s.sync()[0]}
        if acts:
            runs[name]["gate_by_interval"] = acts
        rho[name] = st[..., 0].copy()
        ke[name] = np.array(kk)
        s.close()
    tt = np.concatenate([[0.0], marks])
    out = {"grid": f"{n}^3", "t_end": tstop, "checkpoint_every": every, "runs": runs,
           "t": tt.tolist(), "kinetic_energy": {k: v.tolist() for k, v in ke.items()}}
    eps = {k: (-(v[2:] - v[:-2]) / (tt[2:] - tt[:-2])) for k, v in ke.items()}
    out["dissipation_rate"] = {k: v.tolist() for k, v in eps.items()}
    out["dissipation_rate_t"] = tt[1:-1].tolist()
    if "fp64" in ke:
        for k in ke:
            if k == "fp64":
                continue
            out[f"kinetic_energy_rel_dev_max_{k}"] = float(np.abs(ke[k] - ke["fp64"]).max() / ke["fp64"][0])
            out[f"dissipation_rate_rel_dev_max_{k}"] = float(np.abs(eps[k] - eps["fp64"]).max()
                                                             / np.abs(eps["fp64"]).max())
            out[f"rho_rel_l1_{k}_vs_fp64"] = float(np.abs(rho[k] - rho["fp64"]).mean() / np.abs(rho["fp64"]).mean())
        out["dissipation_peak_fp64"] = {"t": float(out["dissipation_rate_t"][int(np.argmax(eps["fp64"]))]),
                                        "rate": float(eps["fp64"].max())}
    return out


def _steps_until_blowup(step, tstop, blowup, max_steps=20000, budget_s=None):
    """Steps of a driver loop (first-order step 0, then the scheme) until t >= tstop or a blow-up
    (an exception of type ``blowup``).  step(k) runs step k and returns the time after it.
    Returns (steps taken, blew_up, t after the last good step, seconds); blew_up is None when the
    time budget ran out first."""
    t0 = time.perf_counter()
    k, t = 0, 0.0
    while t < tstop and k < max_steps:
        try:
            t = step(k)
        except blowup:
            return k + 1, True, t, time.perf_counter() - t0
        k += 1
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            return k, None, t, time.perf_counter() - t0
    return k, False, t, time.perf_counter() - t0


def batch_failures_main(args):
    """The problems of the 64-problem sweep that the gated FP32 batch loses to a blow-up, each run
    alone from the same initial data with the drivers' first-order step 0: the plain FP64 GPU
    solver, the gated FP32 solver, and the FP64 restatement of the reference's algorithm on the
    host cores (at most ~120 s per problem).  Prints one JSON line with the step at which each
    stops (negative density / pressure) or its end."""
    import torch

    sys.path.insert(0, str(ROOT / "tests"))
    from hos_gb300 import cases, gate_train
    from hos_gb300.solver import FP32, FP64, HosBlowUp, Solver2D
    from oracle_lib import CpuStep

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    gate5, rep5 = gate_train.train(order=5, sizes=(256, 512), seeds=range(4), steps=120, sample_log2=5,
                                   train_steps=3000, batch=4096)
    res = batch_leg(dev, FP32, gate=gate5, threshold=rep5.threshold)
    sweep = {x[4]: x for x in cases.batch_sweep(count=64, seed=0)}
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    out = []
    for label in res["blown_up_problems"]:
        pb, con, prim, tstop, _ = sweep[label]
        row = {"problem": label, "t_end": tstop}
        for name, prec, gated in (("gpu_fp64", FP64, False), ("gpu_fp32_gated", FP32, True)):
            s = Solver2D(pb, prec)
            s.set_state(con, prim)
            if gated:
                s.set_gate(gate5, rep5.threshold, audit_log2=AUDIT_LOG2)

            def step(k, s=s):
                s.set_reconstruction(k == 0)
                s.step(tstop)
                return s.sync()[0]

            n, bad, t, sec = _steps_until_blowup(step, tstop, HosBlowUp)
            row[name] = {"steps": n, "blew_up": bad, "t": t}
            s.close()
        o = CpuStep("oracle").init(pb, threads=cores)
        o.set_state(con, prim)

        def ostep(k):
            o.fn("set_first_order")(1 if k == 0 else 0)
            o.step(tstop)
            return o.t

        # the restatement reports its blow-up status as a RuntimeError
        n, bad, t, sec = _steps_until_blowup(ostep, tstop, RuntimeError, budget_s=120.0)
        row["cpu_fp64_restatement"] = {"steps": n, "blew_up": bad, "t": t, "seconds": sec, "threads": cores}
        out.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    gate5.close()
    print(json.dumps({"mode": "batch_failures", "batch": {k: res[k] for k in ("blown_up", "value", "wall_s")},
                      "problems": out}), flush=True)


def endtime_main(args):
    """--endtime: the accuracy studies at the configurations' end times, one JSON line: the 2D
    Riemann problem at 1024^2 to t = 0.25 and the Taylor-Green vortex at 64^3 to t = 10 (FP64,
    FP32 bulk, gated FP32), then gated FP32 alone at 256^3 to t = 10 for its throughput and
    kinetic-energy curve."""
    import torch

    from hos_gb300 import gate_train

    torch.cuda.set_device(0)
    out = {"mode": "endtime"}
    t0 = time.perf_counter()
    gate, rep = gate_train.train(order=ORDER, sizes=(256, 512), seeds=range(4), steps=120, sample_log2=5,
                                 train_steps=3000, batch=4096)
    out["gate2d"] = {"train_s": time.perf_counter() - t0, "threshold": rep.threshold, "heldout": rep.heldout}
    out["riemann2d"] = endtime2d_leg(gate, rep)
    print(json.dumps({"riemann2d": out["riemann2d"]}), flush=True)
    gate.close()
    t0 = time.perf_counter()
    gate3, rep3 = gate_train.train3d()
    out["gate3d"] = {"train_s": time.perf_counter() - t0, "threshold": rep3.threshold, "heldout": rep3.heldout}
    out["tgv3d_64"] = endtime3d_leg(gate3, rep3, n=64)
    print(json.dumps({"tgv3d_64": out["tgv3d_64"]}), flush=True)
    if args.endtime_256:
        out["tgv3d_256_gated"] = endtime3d_leg(gate3, rep3, n=256, every=0.5, forms=("gated",))
        r = out["tgv3d_256_gated"]["runs"]["gated"]
        r["cell_updates_per_s_upper_bound"] = 256 ** 3 * r["steps_upper_bound"] / r["wall_s"]
    gate3.close()
    print(json.dumps(out), flush=True)


def vortex_leg(sizes=(50, 100, 200, 400)):
    """The isentropic vortex on the periodic [0, 10]^2 (unit freestream, strength 5, WENO5-AO-DF,
    characteristic, CFL 0.5) run to t = 2 in FP64 and in FP32 bulk at each size: density L1 / L-inf
    error against the exact solution (the initial vortex moved by (2, 2)), the FP32 path's
    deviation from FP64, the L1 / L-inf convergence order between the sizes, and the throughput
    of the whole run (graph-captured steps, wall time by CUDA-synchronised host clock)."""
    from hos_gb300 import cases
    from hos_gb300.solver import FP32, FP64, Solver2D

    out = {"workload": "isentropic_vortex_periodic10_weno5ao_df_char_gp2_t2", "sizes": {}}
    l1, linf = {}, {}
    for n in sizes:
        pb, con, prim = cases.isentropic_vortex(n, order=5)
        _, exact, _ = cases.isentropic_vortex(n, order=5, center=(7.0, 7.0))
        g = pb.ghost
        ex = exact[g:-g, g:-g, 0]
        row = {}
        rho = {}
        for name, prec in (("fp64", FP64), ("fp32_bulk", FP32)):
            # the run to t = 2 one step per call counts the steps; a second run queues exactly
            # that many steps behind one synchronisation for the throughput
            s = Solver2D(pb, prec)
            s.set_state(con, prim)
            nsteps = s.run(2.0, graph=True, check_every=1)
            r = s.get_state()["convar"][g:-g, g:-g, 0]
            s.close()
            s = Solver2D(pb, prec)
            s.set_state(con, prim)
            s.sync()
            t0 = time.perf_counter()
            s.advance(nsteps, 2.0, graph=True)
            s.sync()
            wall = time.perf_counter() - t0
            s.close()
            e = np.abs(r - ex)
            rho[name] = r
            row[name] = {"l1": float(e.mean()), "linf": float(e.max()), "steps": int(nsteps),
                         "cell_updates_per_s": pb.nodex * pb.nodey * nsteps / wall}
        d = np.abs(rho["fp32_bulk"] - rho["fp64"])
        row["rho_rel_l1_fp32_vs_fp64"] = float(d.mean() / np.abs(rho["fp64"]).mean())
        row["rho_rel_linf_fp32_vs_fp64"] = float(d.max() / np.abs(rho["fp64"]).max())
        out["sizes"][f"{n}x{n}"] = row
        l1[n], linf[n] = row["fp64"]["l1"], row["fp64"]["linf"]
    # orders between consecutive sizes; from 200^2 on the error nears the floor of the initial
    # data's non-periodic tail (a velocity jump of up to 2.4e-5 across the boundary)
    out["order_fp64"] = {f"{a}-{b}": {"l1": float(np.log2(l1[a] / l1[b]) / np.log2(b / a)),
                                      "linf": float(np.log2(linf[a] / linf[b]) / np.log2(b / a))}
                         for a, b in zip(sizes, sizes[1:])}
    return out


def tgv3d_leg(torch, dev, flush, steps, warmup, fp32_peak, fp64_peak, n=N_3D, n512=True):
    """3D Taylor-Green vortex, n^3 cells (WENO5-AO on 2 x 2 Gauss points per face, GKS3D with
    the Navier-Stokes collision time, S2O4): gated FP32 bulk (the learned gate trained on the
    solver's own 3D runs first, outside the timed region), plain FP32 bulk and FP64, state
    resident in HBM, CUDA events on the solver's stream, L2 flushed between timed steps;
    density, kinetic-energy and dissipation-rate deviation from FP64 over 20 steps at 128^3;
    512^3 throughput; the 3D restatement timed on the host cores."""
    from hos_gb300 import cases, gate_train
    from hos_gb300.solver import FP32, FP64, Solver3D

    t0 = time.perf_counter()
    gate, rep = gate_train.train3d()
    train_s = time.perf_counter() - t0

    pb, con = cases.tgv3d(n)
    cells = n ** 3
    out = {"workload": f"tgv3d_{n}^3_re1600_ma0.1_pr0.71_weno5ao_char_4gp_gks3d_ns_s2o4", "cells": cells}

    def timed(prec, k, w, gated=False):
        s = Solver3D(pb, prec)
        s.set_state(con)
        if gated:
            s.set_gate(gate, rep.threshold, audit_log2=AUDIT_LOG2)
        ext = torch.cuda.ExternalStream(s.stream, device=dev)
        s.advance(w)
        s.sync()
        evs = []
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize(dev)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
            s.advance(1)
            b.record(ext)
            evs.append((a, b))
        s.sync()
        t = sum(a.elapsed_time(b) / 1e3 for a, b in evs)
        flush.zero_()
        torch.cuda.synchronize(dev)
        prof = s.profile_step()
        st = s.gate_stats() if gated else None
        s.close()
        return t, prof, st

    tg, profg, statsg = timed(FP32, steps, warmup, gated=True)
    t32, prof32, _ = timed(FP32, steps, warmup)
    k64 = min(steps, 2)
    t64, prof64, _ = timed(FP64, k64, 1)
    cells_g = statsg["cells_x"] + statsg["cells_y"] + statsg["cells_z"]
    out["gated_fp32"] = {"value": cells * steps / tg, "unit": "cell-updates/s", "ms_per_step": 1e3 * tg / steps,
                         "steps": steps, "warmup": warmup, "kernels_ms": profg,
                         "gate": {"train_s": train_s, "samples": rep.samples, "threshold": rep.threshold,
                                  "heldout": rep.heldout, "audit_log2": AUDIT_LOG2,
                                  "smooth_fraction": (statsg["smooth_x"] + statsg["smooth_y"] + statsg["smooth_z"])
                                  / max(cells_g, 1),
                                  "audited": statsg["audited"], "false_neg": statsg["false_neg"],
                                  "fallback_faces": statsg["fallback"]}}
    out["gated_speedup_vs_fp64"] = (t64 / k64) / (tg / steps)
    out["gated_speedup_vs_fp32"] = t32 / tg
    out["fp32_bulk"] = {"value": cells * steps / t32, "unit": "cell-updates/s", "ms_per_step": 1e3 * t32 / steps,
                        "steps": steps, "warmup": warmup, "kernels_ms": prof32}
    out["fp64"] = {"value": cells * k64 / t64, "unit": "cell-updates/s", "ms_per_step": 1e3 * t64 / k64,
                   "steps": k64, "warmup": 1, "kernels_ms": prof64}
    out["fp32_speedup"] = (t64 / k64) / (t32 / steps)
    faces = (n + 1) * n * n
    for name, prof, flop, peak, unit_peak in (("gated_fp32", profg, GATED_FLOP_PER_FACE_POINT3, fp32_peak, "SGEMM"),
                                              ("fp32_bulk", prof32, FP32_FLOP_PER_FACE_POINT3, fp32_peak, "SGEMM"),
                                              ("fp64", prof64, FP64_FLOP_PER_FACE_POINT3, fp64_peak, "DGEMM")):
        ms = float(np.mean([v for k, v in prof.items() if k.startswith("point")]))
        ach = flop * faces / (ms / 1e3) / 1e12
        kern = {"gated_fp32": "point3_kernel<float, gated>", "fp32_bulk": "point3_kernel<float>"}.get(name, "point3_kernel<double>")
        out[name]["roofline"] = {"kernel": kern, "bound": "fp64" if name == "fp64" else "fp32", "unit": "TFLOP/s",
                                 "achieved": ach, "peak": peak, "frac": ach / peak,
                                 "peak_source": f"cuBLAS {unit_peak} measured in this run",
                                 "flop_per_face": flop, "launch_ms": ms,
                                 "traffic": {"fp32_bulk": TRAFFIC_PER_FACE_POINT3 * faces,
                                             "gated_fp32": GATED_TRAFFIC_PER_FACE_POINT3 * faces}.get(name)}
    # FP32 bulk (plain and gated) against FP64 from the same initial data, 128^3, 20 steps:
    # density deviation, kinetic energy <rho |u|^2 / 2> and its dissipation rate -dKE/dt
    pa, ca = cases.tgv3d(128)
    rho, ke, ts = {}, {}, {}
    for name, prec in (("fp64", FP64), ("fp32", FP32), ("gated", FP32)):
        s = Solver3D(pa, prec)
        s.set_state(ca)
        if name == "gated":
            s.set_gate(gate, rep.threshold, audit_log2=AUDIT_LOG2)
        kk, tt = [], []
        for i in range(21):
            st = s.get_state()["convar"][3:-3, 3:-3, 3:-3]
            kk.append(0.5 * float(((st[..., 1] ** 2 + st[..., 2] ** 2 + st[..., 3] ** 2) / st[..., 0]).mean()))
            tt.append(s.sync()[0])
            if i < 20:
                s.advance(1)
        rho[name] = st[..., 0]
        ke[name], ts[name] = np.array(kk), np.array(tt)
        s.close()
    eps = {k: -np.diff(ke[k]) / np.diff(ts[k]) for k in ke}
    out["accuracy"] = {"grid": "128^3", "steps": 20, "t": float(ts["fp64"][-1]),
                       "rho_rel_l1_fp32_vs_fp64": float(np.abs(rho["fp32"] - rho["fp64"]).mean()
                                                        / np.abs(rho["fp64"]).mean()),
                       "kinetic_energy_rel_dev_max": float(np.abs(ke["fp32"] - ke["fp64"]).max() / ke["fp64"][0]),
                       "dissipation_rate_rel_dev_max": float(np.abs(eps["fp32"] - eps["fp64"]).max()
                                                             / np.abs(eps["fp64"]).max()),
                       "kinetic_energy_ratio_fp64": float(ke["fp64"][-1] / ke["fp64"][0]),
                       "rho_rel_l1_gated_vs_fp64": float(np.abs(rho["gated"] - rho["fp64"]).mean()
                                                         / np.abs(rho["fp64"]).mean()),
                       "kinetic_energy_rel_dev_max_gated": float(np.abs(ke["gated"] - ke["fp64"]).max()
                                                                 / ke["fp64"][0]),
                       "dissipation_rate_rel_dev_max_gated": float(np.abs(eps["gated"] - eps["fp64"]).max()
                                                                   / np.abs(eps["fp64"]).max())}
    # 512^3: FP32 bulk (1 warm-up, 2 timed steps) and FP64 (1 timed step, ~45 s)
    if n512:
        pb5, con5 = cases.tgv3d(512)
        big = {}
        for name, prec, k, w in (("gated_fp32", FP32, 2, 1), ("fp32_bulk", FP32, 2, 1), ("fp64", FP64, 1, 0)):
            s = Solver3D(pb5, prec)
            s.set_state(con5)
            if name == "gated_fp32":
                s.set_gate(gate, rep.threshold, audit_log2=AUDIT_LOG2)
            ext = torch.cuda.ExternalStream(s.stream, device=dev)
            s.advance(w)
            s.sync()
            flush.zero_()
            torch.cuda.synchronize(dev)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(ext)
            s.advance(k)
            b.record(ext)
            s.sync()
            t = a.elapsed_time(b) / 1e3
            big[name] = {"value": 512 ** 3 * k / t, "unit": "cell-updates/s", "ms_per_step": 1e3 * t / k,
                         "steps": k, "warmup": w}
            s.close()
        del con5
        big["fp32_speedup"] = big["fp32_bulk"]["value"] / big["fp64"]["value"]
        big["gated_speedup_vs_fp64"] = big["gated_fp32"]["value"] / big["fp64"]["value"]
        out["n512"] = big
    # the 3D restatement on the host cores, bounded sample
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_lib import CpuStep3D
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    pc, cc = cases.tgv3d(32)
    cpu = CpuStep3D().init(pc)
    cpu.set_state(cc)
    cpu.step()
    nst, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < 8.0 and nst < 50:
        cpu.step()
        nst += 1
    el = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": 32 ** 3 * nst / el, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                           "sample": f"32^3 Taylor-Green, {nst} S2O4 steps after 1 warm-up (OpenMP)"}
    gate.close()
    return out


def sgemm_tflops(torch, dev):
    """FP32 (no TF32) cuBLAS GEMM throughput: the FP32-pipe peak the gated kernels are held to."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    m = torch.randn(8192, 8192, dtype=torch.float32, device=dev)
    torch.matmul(m, m)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        torch.matmul(m, m)
    e1.record()
    torch.cuda.synchronize(dev)
    torch.backends.cuda.matmul.allow_tf32 = prev
    return 5 * 2 * 8192 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12


def dgemm_tflops(torch, dev):
    m = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    torch.matmul(m, m)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        torch.matmul(m, m)
    e1.record()
    torch.cuda.synchronize(dev)
    return 3 * 2 * 4096 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12


def profile_case(n=256, steps=21, plain=True):
    """The launches the ncu summaries under profiles/ capture (see --case): the steps run inside
    NVTX ranges "plain" and "gated" so that ncu --nvtx-include selects them."""
    import torch

    from hos_gb300 import cases, gate_train
    from hos_gb300.solver import FP32, Solver2D

    gate, rep = gate_train.train(order=ORDER, sizes=(256, 512), seeds=range(4), steps=120, sample_log2=5,
                                 train_steps=3000, batch=4096)
    pb, con, prim = cases.riemann2d(n, order=ORDER)
    for gated in ((False, True) if plain else (True,)):
        s = Solver2D(pb, FP32)
        s.set_state(con, prim)
        if gated:
            s.set_gate(gate, rep.threshold, audit_log2=AUDIT_LOG2)
            s.set_gate_reuse(True)
        torch.cuda.nvtx.range_push("gated" if gated else "plain")
        s.advance(steps, 1e30, graph=False)
        s.sync()
        torch.cuda.nvtx.range_pop()
        print("gated" if gated else "plain", s.gate_stats() if gated else "", flush=True)
        s.close()
    gate.close()


def profile_case_3d():
    """The launches of the 3D ncu summaries: 64^3 Taylor-Green, 2 FP32 steps in NVTX range
    "fp32", 2 gated FP32 steps in "gated" (a gate trained on 32^3 runs first), then 1 FP64 step
    in "fp64"."""
    import torch

    from hos_gb300 import cases, gate_train
    from hos_gb300.solver import FP32, FP64, Solver3D

    gate, rep = gate_train.train3d(sizes=(32,), seeds=range(2), steps=20, train_steps=800, capacity=1 << 20)
    pb, con = cases.tgv3d(64)
    for name, prec, k in (("fp32", FP32, 2), ("gated", FP32, 2), ("fp64", FP64, 1)):
        s = Solver3D(pb, prec)
        s.set_state(con)
        if name == "gated":
            s.set_gate(gate, rep.threshold, audit_log2=AUDIT_LOG2)
        torch.cuda.nvtx.range_push(name)
        s.advance(k)
        s.sync()
        torch.cuda.nvtx.range_pop()
        print(name, s.sync(), s.gate_stats() if name == "gated" else "", flush=True)
        s.close()
    gate.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.endtime:
        endtime_main(args)
        return
    if args.batch_failures:
        batch_failures_main(args)
        return
    if args.case == "gated256":
        profile_case()
        return
    if args.case == "gated1024":
        profile_case(1024, 2, plain=False)
        return
    if args.case == "tgv3d64":
        profile_case_3d()
        return
    import torch
    import torch.distributed as dist

    from hos_gb300 import cases, gate_train, replicas
    from hos_gb300.solver import FP32, FP64, Solver2D

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.n
    pb, con, prim = cases.riemann2d(n, order=ORDER)
    cells = pb.nodex * pb.nodey
    g = pb.ghost

    # 256 MB buffer written between timed steps to flush the 129 MB L2
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def timed_steps(solver, k, w):
        ext = torch.cuda.ExternalStream(solver.stream, device=dev)
        for _ in range(w):
            solver.advance(1, 1e30, graph=True)
        solver.sync()
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
        return sum(a.elapsed_time(b) / 1e3 for a, b in evs)

    def kernel_ms(solver, reps=3):
        prof = []
        for _ in range(reps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            prof.append(solver.profile_step(1e30))
        return {k: float(np.mean([q[k] for q in prof])) for k in prof[0]}

    # ---- the learned gate, trained on the solver's own 256^2 / 512^2 random-quadrant runs ----
    t0 = time.perf_counter()
    gate, rep = gate_train.train(order=ORDER, sizes=(256, 512), seeds=range(4), steps=120, sample_log2=5,
                                 train_steps=3000, batch=4096)
    train_s = time.perf_counter() - t0

    def run(precision, gated, clk=None):
        s = Solver2D(pb, precision)
        s.set_state(con, prim)
        if gated:
            s.set_gate(gate, rep.threshold, audit_log2=AUDIT_LOG2)
            s.set_gate_reuse(True)   # the network at stage 0; stage 1 takes its flags dilated
        replicas.barrier(ws)
        torch.cuda.synchronize(dev)
        t = timed_steps(s, args.steps, args.warmup)
        torch.cuda.synchronize(dev)
        return s, replicas.max_over_ranks(t, ws, dev)

    # ---- gated FP32 (the headline), plain FP64 and plain FP32 on the same initial data ----
    with ClockSampler(local) as clk:
        sg, tg = run(FP32, True)
        gstats = sg.gate_stats()
        kern_g = kernel_ms(sg)
        rho_g = sg.get_state()["convar"][g:-g, g:-g, 0]
        s64, t64 = run(FP64, False)
        kern_64 = kernel_ms(s64)
        rho_64 = s64.get_state()["convar"][g:-g, g:-g, 0]
        s32, t32 = run(FP32, False)
        kern_32 = kernel_ms(s32)
        rho_32 = s32.get_state()["convar"][g:-g, g:-g, 0]
    s64.close()
    s32.close()

    # deviation at the configuration's end time: every form run to t = 0.25 from the same data
    end_time = endtime2d_leg(gate, rep, n=n) if not args.no_endtime else None

    def dev_l1(a, b):
        return float(np.abs(a - b).mean() / np.abs(b).mean())

    def dev_linf(a, b):
        return float(np.abs(a - b).max() / np.abs(b).max())

    # ---- end to end through the C ABI with pinned host buffers (gated FP32 solver) ----
    host_in = torch.from_numpy(np.ascontiguousarray(con.reshape(-1))).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    lib = sg._lib
    dp = ctypes.POINTER(ctypes.c_double)
    pin = ctypes.cast(host_in.data_ptr(), dp)
    pout = ctypes.cast(host_out.data_ptr(), dp)
    ke = max(3, args.steps)
    # each step uploads the conserved state (the library derives the primitives the first CFL
    # reads, as Convar_to_Primvar does), steps, and downloads the conserved state
    lib.hos2d_set_state(sg._h, pin, None)
    sg.advance(1, 1e30, graph=True)
    lib.hos2d_get_state(sg._h, pout, None, None, None)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(ke):
        assert lib.hos2d_set_state(sg._h, pin, None) == 0
        sg.advance(1, 1e30, graph=True)
        assert lib.hos2d_get_state(sg._h, pout, None, None, None) == 0
    te = time.perf_counter() - t0
    e2e_value = ws * cells * ke / te
    # where the end-to-end step goes (outside the timed loop: a synchronize after the step
    # separates it from the download)
    split = {"set_state": [], "step": [], "get_state": []}
    for _ in range(ke):
        ta = time.perf_counter()
        assert lib.hos2d_set_state(sg._h, pin, None) == 0
        tb = time.perf_counter()
        sg.advance(1, 1e30, graph=True)
        torch.cuda.synchronize(dev)
        tc = time.perf_counter()
        assert lib.hos2d_get_state(sg._h, pout, None, None, None) == 0
        td = time.perf_counter()
        split["set_state"].append(tb - ta)
        split["step"].append(tc - tb)
        split["get_state"].append(td - tc)
    e2e_split = {k + "_ms": round(1e3 * float(np.median(v)), 4) for k, v in split.items()}
    launches = args.steps * sg.launches_per_step
    sg.close()

    hbm_peak, hbm_src = peaks()
    if rank != 0:
        gate.close()
        if ws > 1:
            dist.destroy_process_group()
        return

    fp32_peak = sgemm_tflops(torch, dev)
    fp64_peak = dgemm_tflops(torch, dev)
    faces = (pb.nodex + 1) * pb.nodey
    face_g = float(np.mean([kern_g[k] for k in ("face_x0", "face_y0", "face_x1", "face_y1")]))
    face_64 = float(np.mean([kern_64[k] for k in ("face_x0", "face_y0", "face_x1", "face_y1")]))
    fl_g = FP32_FLOP_PER_FACE_GATED * faces / (face_g / 1e3) / 1e12
    fl_64 = FLOP_PER_FACE * faces / (face_64 / 1e3) / 1e12
    bytes_gbs = BYTES_PER_FACE * faces / (face_g / 1e3) / 1e9
    smooth = (gstats["smooth_x"] + gstats["smooth_y"]) / max(1, gstats["cells_x"] + gstats["cells_y"])
    line = {
        "metric": METRIC, "value": replicas.aggregate_rate(ws, cells * args.steps, tg), "unit": "cell-updates/s",
        "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tg / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 reconstruction/flux/gate (bf16 MLP on tensor cores); f64 state, stage combination, CFL",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": cells, "order": ORDER, "gauss_points": 3,
                   "characteristic": True, "form": "gated FP32 (learned gate) vs plain FP64",
                   "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "flushed between timed steps (256 MB write)",
                   "gate_training": "seeded random-quadrant runs at 256^2 and 512^2 (4 seeds each, 120 steps)",
                   "gate_stages": "network at stage 0, its flags dilated by one cell at stage 1"},
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": int(host_in.numel() * 8),
                "d2h_bytes_per_step": int(host_out.numel() * 8), "split": e2e_split},
        "gpu_launches": launches,
        "roofline": {"kernel": "face_kernel_tma<7,x|y,gated>", "bound": "fp32", "unit": "TFLOP/s",
                     "achieved": fl_g, "peak": fp32_peak, "frac": fl_g / fp32_peak,
                     "peak_source": "cuBLAS SGEMM 8192^3 (no TF32) measured in this run",
                     "flop_per_face": FP32_FLOP_PER_FACE_GATED, "launch_ms": face_g,
                     "traffic": TRAFFIC_PER_FACE_FP32 * faces,
                     "hbm": {"achieved": bytes_gbs, "peak": hbm_peak, "unit": "GB/s",
                             "frac": bytes_gbs / hbm_peak, "peak_source": hbm_src}},
        "plain_fp64": {"value": ws * cells * args.steps / t64, "unit": "cell-updates/s",
                       "ms_per_step": 1e3 * t64 / args.steps, "gated_fp32_speedup": t64 / tg,
                       "roofline": {"kernel": "face_kernel<double,7,x|y>", "bound": "fp64", "unit": "TFLOP/s",
                                    "achieved": fl_64, "peak": fp64_peak, "frac": fl_64 / fp64_peak,
                                    "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                                    "flop_per_face": FLOP_PER_FACE, "launch_ms": face_64,
                                    "traffic": TRAFFIC_PER_FACE * faces}},
        "accuracy": {"steps_compared": args.steps + args.warmup,
                     "rho_rel_l1_gated_vs_fp64": dev_l1(rho_g, rho_64),
                     "rho_rel_linf_gated_vs_fp64": dev_linf(rho_g, rho_64),
                     "rho_rel_l1_fp32_vs_fp64": dev_l1(rho_32, rho_64),
                     "rho_rel_l1_gated_vs_fp32": dev_l1(rho_g, rho_32),
                     "end_time": end_time},
        "gate": {"train_s": train_s, "samples": rep.samples, "smooth_label_fraction": rep.smooth_fraction,
                 "threshold": rep.threshold, "heldout": rep.heldout,
                 "linear_path_fraction": smooth, "audited": gstats["audited"],
                 "audit_false_negative_rate": gstats["false_neg"] / max(1, gstats["audited"]),
                 "aposteriori_rejections": gstats["fallback"], "audit_rate": 2.0 ** -AUDIT_LOG2},
        "variants": {"fp32_bulk": {"value": cells * args.steps / t32, "unit": "cell-updates/s",
                                   "ms_per_step": 1e3 * t32 / args.steps, "gated_speedup": t32 / tg}},
        "kernels_ms": {"gated_fp32": kern_g, "fp32": kern_32, "fp64": kern_64},
        "clocks": clk.summary(),
    }
    if ws == 1:
        line["cpu_baseline"] = cpu_baseline_sample()
    line["variants"]["vortex2d"] = vortex_leg()
    if not args.no_3d:
        line["variants"]["tgv3d"] = tgv3d_leg(torch, dev, flush, args.steps, args.warmup, fp32_peak, fp64_peak)
    if not args.no_batch:
        # the sweep runs WENO5: its gate is trained the same way on WENO5 runs
        gate5, rep5 = gate_train.train(order=5, sizes=(256, 512), seeds=range(4), steps=120, sample_log2=5,
                                       train_steps=3000, batch=4096)
        line["variants"]["batch64_fp32_gated"] = batch_leg(dev, FP32, gate=gate5, threshold=rep5.threshold)
        line["variants"]["batch64_fp32_gated"]["gate_heldout"] = rep5.heldout
        gate5.close()
    gate.close()
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
