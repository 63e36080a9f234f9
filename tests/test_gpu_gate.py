"""The learned gate on the GPU: features and labels against the CPU oracle, the tensor-core
forward pass and the training gradients against the CPU statement of the network, training,
and the gated FP32 solver's deviation from the plain FP32 solver."""
import sys
from pathlib import Path

import numpy as np
import pytest

from hos_gb300 import cases, gate_train
from hos_gb300.solver import FP32, FP64, Gate, HosBlowUp, HosError, Solver2D
from oracle_lib import gate_cells

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import gate_oracle as go  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build()


@pytest.fixture(scope="module")
def trained():
    g, rep = gate_train.train(order=7, sizes=(64, 128), seeds=range(3), steps=60, sample_log2=2,
                              train_steps=1500, batch=2048, capacity=1 << 21, fn_target=0.01)
    yield g, rep
    g.close()


@pytest.fixture(scope="module")
def trained5():
    g, rep = gate_train.train(order=5, sizes=(128, 256), seeds=range(3), steps=80, sample_log2=3,
                              train_steps=2000, batch=4096, capacity=1 << 21)
    yield g, rep
    g.close()


def _state_after(pb, con, prim, steps):
    s = Solver2D(pb, FP32)
    s.set_state(con, prim)
    s.advance(steps, 1e30)
    s.sync()
    return s


def test_gate_features_and_labels_match_oracle():
    pb, con, prim = cases.riemann2d(32, order=7)
    s = _state_after(pb, con, prim, 3)
    s.boundary()   # ghost cells of the current state, as the gate sees them
    st = s.get_state()
    g = Gate(capacity=1 << 16)
    g.collect(s, 0)
    smp = g.samples()
    s.close()
    g.close()
    f, d = gate_cells(pb, st["convar"], st["alpha_x"], st["alpha_y"])
    cell = smp[:, 18].astype(np.int64)
    dirs = smp[:, 19].astype(np.int64)
    of = f.reshape(-1, 2, 16)[cell, dirs]
    od = d.reshape(-1, 2)[cell, dirs]
    assert (od >= 0).all() and len(smp) == int((d >= 0).sum())
    # FP32 features: indicators of stencils whose variation is near the 1e-5 normalisation floor
    # carry the primitives' FP32 rounding, so the bound is on the distribution
    err = np.abs(smp[:, :16] - of)
    assert np.percentile(err, 99) <= 5e-2 and np.median(err) <= 1e-4
    clear = np.abs(od - 0.02) > 0.005               # labels away from the threshold
    agree = (smp[clear, 16] > 0.5) == (od[clear] <= 0.02)
    assert agree.mean() >= 0.99


def test_gate_forward_and_gradient_match_cpu_oracle():
    rng = np.random.default_rng(3)
    n = 1000
    smp = np.zeros((n, 20), np.float32)
    smp[:, :15] = rng.random((n, 15))
    smp[:, 16] = rng.random(n) > 0.5
    g = Gate(capacity=n, seed=7)
    g.set_samples(smp)
    p = g.params
    z = g.forward(0, n)
    zo, _ = go.forward(p, smp[:, :16])
    assert np.abs(z - zo).max() <= 1e-2 * max(1.0, np.abs(zo).max())
    grad, loss = g.gradient(0, n, 1.0, 4.0)
    lo, go_ = go.loss_grad(p, smp[:, :16], smp[:, 16], 1.0, 4.0)
    g.close()
    cos = float(grad @ go_ / (np.linalg.norm(grad) * np.linalg.norm(go_)))
    assert cos >= 0.9999 and np.linalg.norm(grad - go_) <= 1e-2 * np.linalg.norm(go_)
    assert abs(loss - lo) <= 1e-4 * abs(lo)


def test_gate_training_learns_and_beats_a_tau_threshold(trained):
    g, rep = trained
    h = rep.heldout
    assert rep.samples > 20000 and 0.2 < rep.smooth_fraction < 0.99
    assert h["false_negative_rate"] <= 0.01 + 1e-9 and h["coverage"] >= 0.3, h
    # the method without the network: a threshold on the normalised tau of density and pressure,
    # tuned on the same held-out samples to the same coverage
    s = g.samples()
    held = s[np.arange(len(s)) % 10 == 0]
    y = held[:, 16] > 0.5
    tau = np.maximum(held[:, 6], held[:, 13])
    k = int(h["coverage"] * len(held))
    pick = np.argsort(tau)[:k]
    fn_tau = float((~y[pick]).mean())
    assert h["false_negative_rate"] <= fn_tau, (h, fn_tau)


def test_gated_solver_deviation_and_coverage(trained):
    g, rep = trained
    pb, con, prim = cases.riemann2d(128, order=7)
    a = Solver2D(pb, FP32)
    a.set_state(con, prim)
    b = Solver2D(pb, FP32)
    b.set_state(con, prim)
    b.set_gate(g, rep.threshold, audit_log2=2)
    for s in (a, b):
        s.advance(40, 1e30)
        s.sync()
    ra, rb = a.get_state()["convar"][..., 0], b.get_state()["convar"][..., 0]
    st = b.gate_stats()
    fc = b.gate_audit_check()
    a.close()
    b.close()
    # the audited false negatives are flagged for the face kernels, which count what the
    # a-posteriori check does with their linear reconstructions
    assert fc["fn_linear_accepted"] <= fc["fn_linear"], fc
    assert st["false_neg"] == 0 or fc["fn_linear"] > 0, (st, fc)
    gh = pb.ghost
    ra, rb = ra[gh:-gh, gh:-gh], rb[gh:-gh, gh:-gh]
    assert np.abs(ra - rb).mean() / np.abs(ra).mean() <= 1e-3
    cov = (st["smooth_x"] + st["smooth_y"]) / (st["cells_x"] + st["cells_y"])
    assert cov >= 0.3, st
    assert st["audited"] > 100 and st["false_neg"] / st["audited"] <= 0.05, st


def test_gate_flags_reused_at_the_second_stage(trained):
    """hos2d_set_gate_reuse: the network runs at stage 0 only and stage 1 takes its flags dilated
    by one cell.  The step is the same number of launches; the gated run with reused flags stays as
    close to plain FP32 as the gate run at every stage, and predicts no more cells smooth at
    stage 1 than the network did at stage 0 (the dilation only clears flags)."""
    g, rep = trained
    pb, con, prim = cases.riemann2d(128, order=7)
    runs = {}
    for name, gated, reuse in (("fp32", False, False), ("every", True, False), ("reuse", True, True)):
        s = Solver2D(pb, FP32)
        s.set_state(con, prim)
        if gated:
            s.set_gate(g, rep.threshold, audit_log2=2)
            s.set_gate_reuse(reuse)
        n = s.launches_per_step
        s.advance(40, 1e30)
        s.sync()
        runs[name] = (s.get_state()["convar"][..., 0], s.gate_stats() if gated else None, n)
        s.close()
    gh = pb.ghost
    ref = runs["fp32"][0][gh:-gh, gh:-gh]
    dev = {k: np.abs(runs[k][0][gh:-gh, gh:-gh] - ref).mean() / np.abs(ref).mean() for k in ("every", "reuse")}
    assert dev["reuse"] <= 1e-3 and dev["reuse"] <= 2.0 * dev["every"] + 1e-7, dev
    assert runs["reuse"][2] == runs["every"][2]
    st = runs["reuse"][1]
    # the network ran at stage 0 only: half the cells of the every-stage run were classified
    assert st["cells_x"] * 2 == runs["every"][1]["cells_x"], (st, runs["every"][1])


def test_gate_needs_the_fp32_path():
    pb, con, prim = cases.riemann2d(16, order=5)
    s = Solver2D(pb, FP64)
    g = Gate(capacity=16)
    with pytest.raises(HosError, match="FP32"):
        s.set_gate(g)
    s.close()
    g.close()


def _run(pb, con, prim, precision, steps, gate=None, threshold=0.0, slack=None):
    s = Solver2D(pb, precision)
    s.set_state(con, prim)
    if gate is not None:
        s.set_gate(gate, threshold, audit_log2=10)
        if slack is not None:
            s.set_gate_check(slack)
    try:
        s.advance(steps, 1e30, graph=True)
        s.sync()
        rho = s.get_state()["convar"][pb.ghost:-pb.ghost, pb.ghost:-pb.ghost, 0]
    except HosBlowUp:
        rho = None
    s.close()
    return rho


def _ms_per_step(pb, con, prim, gate=None, threshold=0.0, steps=40):
    import time
    s = Solver2D(pb, FP32)
    s.set_state(con, prim)
    if gate is not None:
        s.set_gate(gate, threshold, audit_log2=10)
    s.advance(5, 1e30, graph=True)
    s.sync()
    t0 = time.perf_counter()
    s.advance(steps, 1e30, graph=True)
    s.sync()
    ms = 1e3 * (time.perf_counter() - t0) / steps
    s.close()
    return ms


def test_gate_gains_over_the_method_without_it(trained5):
    """What the trained network gains over the method without it, on the 512^2 quadrant problem
    (WENO5-AO-DF, characteristic, 80 steps):
      speed    -- the gated FP32 step is faster than the plain FP32 step, which runs the full
                  WENO-AO weights everywhere;
      accuracy -- its density deviation from FP64 is far below that of linear weights
                  everywhere, both as the reference's own wenotype = linear (non-DF WENO5-AO)
                  and as a gate that sends every cell down the linear path."""
    g, rep = trained5
    pb, con, prim = cases.riemann2d(512, order=5)
    ref = _run(pb, con, prim, FP64, 80)
    dev = lambda r: np.inf if r is None else float(np.abs(r - ref).mean() / np.abs(ref).mean())
    gated = dev(_run(pb, con, prim, FP32, 80, g, rep.threshold))
    always = dev(_run(pb, con, prim, FP32, 80, g, -1e30, slack=10.0))
    pb_lin, _, _ = cases.riemann2d(512, order=5)
    pb_lin.use_df, pb_lin.wenotype = False, "linear"
    linear = dev(_run(pb_lin, con, prim, FP32, 80))
    assert gated <= 1e-3 and gated < 0.2 * linear and gated < 0.2 * always, (gated, linear, always)
    t_plain = _ms_per_step(pb, con, prim)
    t_gated = _ms_per_step(pb, con, prim, g, rep.threshold)
    assert t_gated < t_plain, (t_gated, t_plain)
