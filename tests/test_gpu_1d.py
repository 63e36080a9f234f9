"""GPU parity of the 1D step (config 1: Sod, plus WENO7/9 and the accuracy case) against the
oracle and the reference's golden vectors; tolerance 1e-12 relative L-inf for FP64."""
from pathlib import Path

import numpy as np
import pytest

from hos_gb300 import cases
from hos_gb300.solver import FP32, FP64, Solver1D
from oracle_lib import CpuStep1D

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build()


def _rel(a, b, g):
    a, b = a[g:-g], b[g:-g]
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLDEN.glob("sod1d_*.npz")))
def test_gpu1d_matches_reference_golden(name):
    from test_oracle1d_cpu import _problem
    pb, _ = _problem(name)
    gold = np.load(GOLDEN / f"{name}.npz")
    s = Solver1D(pb, FP64)
    s.set_state(gold["convar0"])
    dts = []
    for _ in range(3):
        s.step(0.2)
        dts.append(s.sync()[1])
    st = s.get_state()
    np.testing.assert_allclose(dts, gold["dts"], rtol=1e-14)
    assert _rel(st["convar"], gold["convar3"], pb.ghost) <= 1e-12
    assert np.abs(st["alpha"] - gold["alpha3"]).max() <= 1e-9 * max(1.0, np.abs(gold["alpha3"]).max())
    steps = s.run(0.2)  # steps since set_state
    t, _ = s.sync()
    end = s.get_state()["convar"]
    s.close()
    assert steps == int(gold["steps"])
    assert abs(t - float(gold["t_end"])) <= 1e-15
    # full run (hundreds of steps through the shock): agreement stays at round-off level
    assert _rel(end, gold["convar_end"], pb.ghost) <= 1e-10


@pytest.mark.parametrize("bc", ["free", "reflect", "periodic"])
def test_gpu1d_vs_oracle_boundaries(bc):
    pb, con = cases.sod1d(300, order=7)
    pb.bc = (bc, bc)
    o = CpuStep1D("oracle").init(pb)
    o.set_state(con)
    for _ in range(5):
        o.step(0.2)
    s = Solver1D(pb, FP64)
    s.set_state(con)
    for _ in range(5):
        s.step(0.2)
    s.sync()
    got = s.get_state()["convar"]
    s.close()
    assert _rel(got, o.state()["convar"], pb.ghost) <= 1e-12


def test_gpu1d_accuracy_case():
    pb, con = cases.sinwave1d(40)
    s = Solver1D(pb, FP64)
    s.set_state(con)
    s.run(2.0)
    g = pb.ghost
    e = np.abs(s.get_state()["convar"][g:-g, 0] - con[g:-g, 0])
    s.close()
    gold = np.load(GOLDEN / "sinwave1d_w5_accuracy.npz")["n40"]
    assert abs(e.mean() - gold[0]) <= 1e-9 * gold[0] + 1e-15


def test_gpu1d_fp32_close_to_fp64():
    pb, con = cases.sod1d(1000)
    a, b = Solver1D(pb, FP64), Solver1D(pb, FP32)
    for s in (a, b):
        s.set_state(con)
        s.run(0.2)
    ra, rb = a.get_state()["convar"][5:-5, 0], b.get_state()["convar"][5:-5, 0]
    a.close()
    b.close()
    assert np.abs(ra - rb).mean() / np.abs(ra).mean() <= 1e-4


@pytest.mark.parametrize("wenotype", ["wenoz", "wenojs", "linear"])
def test_gpu1d_nodf_wenotype_vs_oracle(wenotype):
    """Non-DF WENO5-AO every step with each wenotype weight choice against the oracle."""
    pb, con = cases.sod1d(200, order=5)
    pb.df_mode, pb.wenotype = 0, wenotype
    o = CpuStep1D("oracle").init(pb)
    o.set_state(con)
    s = Solver1D(pb, FP64)
    s.set_state(con)
    for _ in range(3):
        o.step(0.2)
        s.step(0.2)
    s.sync()
    got = s.get_state()["convar"]
    s.close()
    assert _rel(got, o.state()["convar"], pb.ghost) <= 1e-12
