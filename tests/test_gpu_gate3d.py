"""The learned gate on the 3D FP32-bulk path: its inputs and labels against the CPU oracle
(oracle/gate_oracle.py), training on the solver's own 3D runs, and gated runs against the
FP64 and plain FP32 paths."""
import sys
from pathlib import Path

import numpy as np
import pytest

from hos_gb300 import cases, gate_train
from hos_gb300.solver import FP32, FP64, Gate, Solver3D

pytestmark = pytest.mark.gpu
sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import gate_oracle  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build()


@pytest.fixture(scope="module")
def trained():
    g, rep = gate_train.train3d(sizes=(32,), seeds=range(2), steps=20, sample_log2=2, train_steps=800, batch=2048,
                                capacity=1 << 20)
    yield g, rep
    g.close()


def test_gate3d_inputs_and_labels_match_the_oracle():
    pb, con = cases.random_octants3d(12, seed=3)
    s = Solver3D(pb, FP32)
    s.set_state(con)
    s.advance(2)
    g = Gate(capacity=1 << 16, seed=1)
    g.collect3d(s, sample_log2=0)           # every cell whose stencil fits, three axes
    st = s.get_state()["convar"]
    s.close()
    smp = g.samples()
    g.close()
    assert len(smp) > 3 * 12 ** 3
    rng = np.random.default_rng(0)
    shape = pb.shape
    ferr, agree, near = [], 0, 0
    for r in smp[rng.choice(len(smp), 400, replace=False)]:
        c, ax = int(r[18]), int(r[19])
        cell = np.unravel_index(c, shape)
        f = gate_oracle.features3d(st, cell, ax)
        ferr.append(np.abs(f - r[:16]).max())
        d = gate_oracle.distance3d(st, cell, ax)
        if abs(d - 0.02) > 0.005:
            agree += (d <= 0.02) == (r[16] > 0.5)
            near += 1
    assert np.percentile(ferr, 99) <= 5e-2
    assert agree >= 0.99 * near


def test_gate3d_training_calibrates_false_negatives(trained):
    g, rep = trained
    assert rep.samples > 10000
    assert 0.05 < rep.smooth_fraction < 0.98
    assert rep.heldout["false_negative_rate"] <= 0.02
    assert rep.heldout["coverage"] > 0.05


def test_gated_fp32_3d_stays_close_to_fp64(trained):
    g, rep = trained
    pb, con = cases.tgv3d(32)
    out = {}
    for name, prec, gated in (("fp64", FP64, False), ("fp32", FP32, False), ("gated", FP32, True)):
        s = Solver3D(pb, prec)
        s.set_state(con)
        if gated:
            s.set_gate(g, rep.threshold, audit_log2=2)
        s.advance(8)
        out[name] = s.get_state()["convar"][3:-3, 3:-3, 3:-3]
        if gated:
            st = s.gate_stats()
        s.close()
    dev = np.abs(out["gated"][..., 0] - out["fp64"][..., 0]).mean() / np.abs(out["fp64"][..., 0]).mean()
    assert dev < 1e-4
    cells = st["cells_x"] + st["cells_y"] + st["cells_z"]
    smooth = st["smooth_x"] + st["smooth_y"] + st["smooth_z"]
    assert cells > 0 and smooth / cells > 0.5          # the smooth vortex takes the linear path
    assert st["false_neg"] <= max(1, 0.02 * st["audited"])


def test_gate3d_marking_nothing_equals_plain_fp32(trained):
    g, _ = trained
    pb, con = cases.random_octants3d(16, seed=7)
    res = []
    for thr in (None, 1e30):
        s = Solver3D(pb, FP32)
        s.set_state(con)
        if thr is not None:
            s.set_gate(g, thr, audit_log2=31)
        s.advance(3)
        res.append(s.get_state()["convar"])
        st = s.gate_stats() if thr is not None else None
        s.close()
    assert st["smooth_x"] + st["smooth_y"] + st["smooth_z"] == 0
    scale = np.abs(res[0]).max(axis=(0, 1, 2))
    assert (np.abs(res[1] - res[0]) / scale).max() <= 1e-6


def test_gated_3d_shock_box_rejects_and_stays_bounded(trained):
    """Sharp octant fronts: flagged reconstructions failing the check fall back to WENO-AO, and
    the gated run stays within FP32 noise of the plain FP32 run in L1."""
    g, rep = trained
    pb, con = cases.random_octants3d(24, seed=11)
    res = []
    for gated in (False, True):
        s = Solver3D(pb, FP32)
        s.set_state(con)
        if gated:
            s.set_gate(g, rep.threshold, audit_log2=4)
        s.advance(6)
        res.append(s.get_state()["convar"][3:-3, 3:-3, 3:-3, 0])
        s.close()
    dev = np.abs(res[1] - res[0]).mean() / np.abs(res[0]).mean()
    assert dev < 1e-3
