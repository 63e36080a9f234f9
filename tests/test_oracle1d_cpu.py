"""1D oracle: bit-for-bit against the reference's golden vectors (Sod, config 1 of the
benchmark definition, and the reference's 1D accuracy known-answer test) and against the
compiled reference where its checkout exists."""
from pathlib import Path

import numpy as np
import pytest

from hos_gb300 import cases
from oracle_lib import CpuStep1D, ref_available

GOLDEN = Path(__file__).resolve().parent / "golden"
SOD = sorted(p.stem for p in GOLDEN.glob("sod1d_*.npz"))


def _problem(name):
    n = int(name.rsplit("_", 1)[1])
    order = int(name.split("_")[1][1])
    return cases.sod1d(n, order=order, characteristic="char" in name)


@pytest.mark.parametrize("name", SOD)
def test_oracle1d_matches_golden(name):
    pb, con = _problem(name)
    gold = np.load(GOLDEN / f"{name}.npz")
    assert np.array_equal(con[pb.ghost:-pb.ghost], gold["convar0"][pb.ghost:-pb.ghost])
    o = CpuStep1D("oracle").init(pb)
    o.set_state(gold["convar0"])
    dts = [o.step(0.2) for _ in range(3)]
    s3 = o.state()
    assert np.array_equal(np.array(dts), gold["dts"])
    g = pb.ghost
    assert np.array_equal(s3["convar"][g:-g], gold["convar3"][g:-g])
    assert np.array_equal(s3["alpha"], gold["alpha3"])
    o.run(0.2)
    assert o.nstep == int(gold["steps"]) and o.t == float(gold["t_end"])
    assert np.array_equal(o.state()["convar"][g:-g], gold["convar_end"][g:-g])


def test_oracle1d_accuracy_known_answer():
    """accuracy_sinwave_1d (src/1Dproblem.cpp:519-735): WENO5-AO-DF, t = 2, L1 order -> 5."""
    gold = np.load(GOLDEN / "sinwave1d_w5_accuracy.npz")
    errs = []
    for n in (10, 20, 40):
        pb, con = cases.sinwave1d(n)
        o = CpuStep1D("oracle").init(pb)
        o.set_state(con)
        o.run(2.0)
        g = pb.ghost
        e = np.abs(o.state()["convar"][g:-g, 0] - con[g:-g, 0])
        err = np.array([e.mean(), np.sqrt((e * e).mean()), e.max()])
        np.testing.assert_allclose(err, gold[f"n{n}"], rtol=1e-12)
        errs.append(err[0])
    assert np.log2(errs[1] / errs[2]) > 4.9


@pytest.mark.skipif(not ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("order,charac,bc", [(5, True, "reflect"), (7, False, "periodic"), (9, True, "free")])
def test_oracle1d_matches_reference_bitwise(order, charac, bc):
    pb, con = cases.sod1d(120, order=order, characteristic=charac)
    pb.bc = (bc, bc)
    a = CpuStep1D("ref").init(pb)
    b = CpuStep1D("oracle").init(pb)
    a.set_state(con)
    b.set_state(con)
    for _ in range(40):
        assert a.step(0.2) == b.step(0.2)
    g = pb.ghost
    assert np.array_equal(a.state()["convar"][g:-g], b.state()["convar"][g:-g])
    assert np.array_equal(a.state()["alpha"], b.state()["alpha"])


@pytest.mark.skipif(not ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("wenotype", ["wenojs", "linear"])
def test_oracle1d_wenotype_matches_reference_bitwise(wenotype):
    """The Sod driver's non-DF WENO5-AO steps under the other wenotype weights
    (weno_5th_ao_left / _right, src/reconstruction.cpp:161-360, honour all three)."""
    pb, con = cases.sod1d(120, order=5)
    pb.df_mode, pb.wenotype = 0, wenotype
    a = CpuStep1D("ref").init(pb)
    b = CpuStep1D("oracle").init(pb)
    a.set_state(con)
    b.set_state(con)
    for _ in range(20):
        assert a.step(0.2) == b.step(0.2)
    g = pb.ghost
    assert np.array_equal(a.state()["convar"][g:-g], b.state()["convar"][g:-g])
