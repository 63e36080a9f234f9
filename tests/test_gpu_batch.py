"""Batched 2D problems (config 4 of the benchmark definition): every problem of a batch of
uneven sizes and kinds must equal the single-problem solver bit for bit, across tile
shapes chosen by the autotuner, graph replay and per-problem stop times."""
import numpy as np
import pytest

from hos_gb300 import cases
from hos_gb300.solver import FP32, FP64, Batch2D, Solver2D

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build()


def _mixed(order=5):
    return [cases.wedge2d(96, 24, mach=4.0, order=order),
            cases.shock_vortex2d(40, mach=2.5, strength=0.3, order=order),
            cases.random_riemann2d(56, seed=7, order=order),
            cases.isentropic_vortex(48, order=order),
            cases.wedge2d(64, 16, mach=10.0, order=order)]


def _single(pb, con, prim, nsteps, tstop, precision):
    s = Solver2D(pb, precision)
    s.set_state(con, prim)
    for _ in range(nsteps):
        s.step(tstop)
    t, _ = s.sync()
    st = s.get_state()
    s.close()
    return st, t


@pytest.mark.parametrize("precision", [FP64, FP32])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_equals_single_problem_solver(precision, graph):
    probs = _mixed()
    tstops = [0.01, 1e30, 0.02, 1e30, 1e30]
    b = Batch2D([p[0] for p in probs], tstops, precision)
    for k, (pb, con, prim) in enumerate(probs):
        b.set_state(k, con, prim)
    chosen, ms = b.autotune(reps=1)
    assert all(0 <= c < 3 for c in chosen)
    b.advance(6, graph=graph)
    act, t, last = b.status()
    for k, (pb, con, prim) in enumerate(probs):
        ref, tref = _single(pb, con, prim, 6, tstops[k], precision)
        got = b.get_state(k)
        _close(got["convar"], ref["convar"], precision, k)
        _close(got["alpha_x"][..., None], ref["alpha_x"][..., None], precision, k)
        assert t[k] == pytest.approx(tref, rel=1e-13 if precision == FP64 else 1e-6)
    b.close()


def _close(got, ref, precision, what=None):
    """The batched face kernels are separate instantiations of the single-problem kernel's
    tile code; nvcc contracts multiply-adds differently in them, so the two agree to rounding:
    relative to each variable's scale 1e-13 in FP64, 1e-5 in FP32 (a few steps of FP32 rounding
    carried through shocks)."""
    scale = np.maximum(np.abs(ref).max(axis=(0, 1)), 1e-300)
    tol = 1e-13 if precision == FP64 else 1e-5
    assert (np.abs(got - ref) / scale).max() <= tol, what


def test_batch_problems_stop_at_their_own_time():
    probs = _mixed()
    pb, con, prim = probs[2]
    b = Batch2D([pb, pb], [0.003, 1e30], FP64)
    b.set_state(0, con, prim)
    b.set_state(1, con, prim)
    b.advance(20)
    act, t, last = b.status()
    assert act == 1 and t[0] >= 0.003 and last[0] < last[1] == 19
    b.close()


@pytest.mark.parametrize("order", [7, 9])
@pytest.mark.parametrize("precision", [FP64, FP32])
def test_batch_weno7_weno9_default_shape(order, precision):
    """Orders 7 and 9 batch with the default 8 x 16 tile only; they agree with the
    single-problem solver to rounding (see _close)."""
    probs = [cases.random_riemann2d(40, seed=s, order=order) for s in (1, 2)]
    b = Batch2D([p[0] for p in probs], [1e30, 1e30], precision)
    for k, (pb, con, prim) in enumerate(probs):
        b.set_state(k, con, prim)
    chosen, ms = b.autotune(reps=1)
    assert chosen == (0, 0) and (ms[:, 1:] < 0).all()
    b.advance(2)
    for k, (pb, con, prim) in enumerate(probs):
        ref, _ = _single(pb, con, prim, 2, 1e30, precision)
        _close(b.get_state(k)["convar"], ref["convar"], precision, k)
    b.close()


def test_blown_up_problem_stops_alone_at_the_oracles_step():
    """A Mach 9 shock hit by a vortex of strength 0.3 drives the reference algorithm to a
    negative pressure (the oracle reports it); in a batch that problem stops at the same step
    and the problem beside it runs on unchanged."""
    from oracle_lib import CpuStep

    bad_pb, bad_con, bad_prim = cases.shock_vortex2d(40, mach=9.0, strength=0.3)
    cpu = CpuStep("oracle").init(bad_pb)
    cpu.set_state(bad_con, bad_prim)
    fail_step = None
    for n in range(60):
        try:
            cpu.step()
        except RuntimeError:
            fail_step = n
            break
    assert fail_step is not None
    good = cases.random_riemann2d(40, seed=3, order=5)
    b = Batch2D([bad_pb, good[0]], [1e30, 1e30], FP64)
    b.set_state(0, bad_con, bad_prim)
    b.set_state(1, good[1], good[2])
    b.advance(fail_step + 5)
    act, t, last, failed = b.status(failed=True)
    assert failed.tolist() == [True, False] and act == 1
    assert last[0] == fail_step and last[1] == fail_step + 4
    from hos_gb300.solver import HosBlowUp
    with pytest.raises(HosBlowUp):
        b.status()
    ref, _ = _single(good[0], good[1], good[2], fail_step + 5, 1e30, FP64)
    _close(b.get_state(1)["convar"], ref["convar"], FP64)
    b.close()


def test_gated_batch_matches_gated_single_problem_solver():
    from hos_gb300 import gate_train
    g, rep = gate_train.train(order=5, sizes=(64,), seeds=range(2), steps=40, sample_log2=1, train_steps=600,
                              batch=1024, capacity=1 << 19)
    probs = _mixed()[:4]
    b = Batch2D([p[0] for p in probs], [1e30] * len(probs), FP32)
    for k, (pb, con, prim) in enumerate(probs):
        b.set_state(k, con, prim)
    b.autotune(reps=1)
    b.set_gate(g, rep.threshold, audit_log2=2)
    b.advance(5, graph=True)
    st = b.gate_stats()
    assert st["smooth_x"] > 0 and st["cells_x"] >= st["smooth_x"]
    for k, (pb, con, prim) in enumerate(probs):
        s = Solver2D(pb, FP32)
        s.set_state(con, prim)
        s.set_gate(g, rep.threshold, audit_log2=2)
        for _ in range(5):
            s.step(1e30)
        s.sync()
        ref = s.get_state()["convar"]
        s.close()
        # the gate's features are compiled into two kernels; nvcc may contract their
        # multiply-adds differently, and a cell whose logit sits at the threshold can then
        # take the other (equally valid) path: equal up to such cells
        got = b.get_state(k)["convar"]
        gh = pb.ghost
        a_, r_ = got[gh:-gh, gh:-gh, 0], ref[gh:-gh, gh:-gh, 0]
        assert np.abs(a_ - r_).mean() / np.abs(r_).mean() <= 1e-5, k
    b.close()
    g.close()
