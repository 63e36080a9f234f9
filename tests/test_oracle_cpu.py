"""CPU tests of the oracle: pinned bit-for-bit against the compiled reference (where the
reference checkout exists) and against the reference-generated golden vectors."""
from pathlib import Path

import numpy as np
import pytest

from hos_gb300 import cases
from oracle_lib import CpuStep, interior, ref_available, rel_linf

GOLDEN = Path(__file__).resolve().parent / "golden"
STEP_CASES = sorted(p.stem for p in GOLDEN.glob("*.npz") if "accuracy" not in p.stem and "1d" not in p.stem
              and not p.stem.startswith("ref3d"))


def first_order_steps(name):
    """steps run with first-order reconstruction at the start of a golden case"""
    return 1 if name.startswith(("fo_", "ns_", "rt_")) else 0


def with_source(name):
    """cases whose stage update is Update_with_source (the RT_instability driver)"""
    return name.startswith("rt_")


def _problem(name):
    n = int(name.rsplit("_", 1)[1])
    if name.startswith("riemann"):
        order = int(name.split("_")[1][1])
        return cases.riemann2d(n, order=order, characteristic="char" in name)
    if name.startswith("rriemann"):
        seed = int(name.split("_")[2][1:])
        return cases.random_riemann2d(n, seed=seed, order=7)
    if name.startswith("vortex"):
        return cases.isentropic_vortex(n, order=5, images=False)   # the fixture's initial data
    if name.startswith("sinwave"):
        return cases.sinwave2d(n, order=9)
    if name.startswith("fo_"):
        # fo_w<order>_<bc>_<n>: seeded random quadrants, first-order reconstruction at step 0
        # then WENO-AO-DF (the drivers' is_using_df_factor switch, src/2Dproblem.cpp:733-745)
        _, w, bc, _ = name.split("_")
        pb, con, prim = cases.random_riemann2d(n, seed=int(w[1]), order=int(w[1]))
        pb.bc = (bc,) * 4
        return pb, con, prim
    if name.startswith("nodf_"):
        # nodf_w5_<wenotype>_<bc>_<n>: seeded random quadrants with the drivers' default slots
        # WENO5_AO_normal / WENO5_AO_tangent (is_using_df_factor = false): non-DF WENO5-AO with
        # Z-type ("z") or Jiang-Shu ("js") weights; "cons" runs conservative variables, periodic
        _, _, wt, bc, _ = name.split("_")
        pb, con, prim = cases.random_riemann2d(n, seed=50 + len(wt) + len(bc), order=5)
        pb.use_df, pb.wenotype = False, {"z": "wenoz", "js": "wenojs"}[wt]
        if bc == "cons":
            pb.characteristic, bc = False, "periodic"
        pb.bc = (bc,) * 4
        return pb, con, prim
    if name.startswith("lfns_"):
        # lfns_w<order>_<variant>_<n>: LF2D with the Navier-Stokes collision time, i.e. with its
        # viscous term NS_by_central_difference_prim_2D (src/flux_function.cpp:720-754)
        #   mu    : Mu = 2e-3, Pr = 0.72, free sides
        #   nu    : Nu = 1e-3 (Mu unset), Pr = 1, periodic
        #   walls : Mu = 1e-2, no-slip walls moving at the bcprim velocities (the dt cap decides)
        _, w, variant, _ = name.split("_")
        order = int(w[1])
        pb, con, prim = cases.random_riemann2d(n, seed=30 + order, order=order)
        pb.flux, pb.tau_type = "LF", 1
        if variant == "mu":
            pb.mu, pb.prandtl = 2e-3, 0.72
        elif variant == "nu":
            pb.mu, pb.nu, pb.bc = -1.0, 1e-3, ("periodic",) * 4
        else:
            pb.mu, pb.bc = 1e-2, ("noslip",) * 4
            pb.bc_prim = ((0.0, 0.0, 0.2, 0.0), (0.0, 0.0, -0.1, 0.0), (0.0, 0.3, 0.0, 0.0), (0.0, -0.25, 0.0, 0.0))
        return pb, con, prim
    if name.startswith("rt_"):
        # rt_w5_<nodex>: the RT_instability set-up, first-order step 0, gravity source
        return cases.rt2d(n, order=5)
    if name.startswith("ns_"):
        # ns_w<order>_<variant>_<n>: Navier-Stokes collision time, first-order step 0
        #   noslip : the viscous_sod_shock_problem set-up (src/2Dproblem.cpp:1095-1160): no-slip
        #            adiabatic left/right/bottom, reflecting top, Mu = 1e-3, c2 = 9
        #   wall   : moving no-slip walls, Prandtl fix (Pr = 0.72), Mu = 0.01, c2 = 1
        #   cap    : as wall with Mu = 0.05, c2 = 9: the viscous dt cap decides every step
        #   nu     : kinematic viscosity Nu = 2e-3 (Mu unset), periodic
        _, w, variant, _ = name.split("_")
        order = int(w[1])
        pb, con, prim = cases.random_riemann2d(n, seed=order, order=order)
        pb.tau_type, pb.c2_euler = 1, 9.0
        if variant == "noslip":
            pb.bc, pb.mu = ("noslip", "noslip", "noslip", "reflect"), 1e-3
        elif variant in ("wall", "cap"):
            pb.bc, pb.prandtl_fix, pb.prandtl = ("noslip",) * 4, True, 0.72
            pb.mu, pb.c2_euler = (0.01, 1.0) if variant == "wall" else (0.05, 9.0)
            pb.bc_prim = ((0.0, 0.0, 0.2, 0.0), (0.0, 0.0, -0.1, 0.0), (0.0, 0.3, 0.0, 0.0), (0.0, -0.25, 0.0, 0.0))
        else:
            pb.bc, pb.mu, pb.nu = ("periodic",) * 4, -1.0, 2e-3
        return pb, con, prim
    if name.startswith("tmarch"):
        # tmarch_<integrator>_<flux>_w<order>_<n>: the quadrant problem with another time
        # marching / flux choice
        _, integ, flux, w, _ = name.split("_")
        pb, con, prim = cases.riemann2d(n, order=int(w[1]))
        pb.integrator, pb.flux = integ.upper(), flux.upper()
        return pb, con, prim
    raise KeyError(name)


@pytest.mark.parametrize("name", STEP_CASES)
def test_golden_initial_data_reproduced(name):
    pb, con, prim = _problem(name)
    gold = np.load(GOLDEN / f"{name}.npz")
    assert np.array_equal(interior(pb, gold["convar0"]), interior(pb, con))


@pytest.mark.parametrize("name", STEP_CASES)
def test_oracle_matches_golden_bitwise(name):
    pb, _, _ = _problem(name)
    gold = np.load(GOLDEN / f"{name}.npz")
    o = CpuStep("oracle").init(pb, threads=4)
    o.set_state(gold["convar0"], gold["primvar0"])
    o.fn("set_source")(1 if with_source(name) else 0)
    fo = first_order_steps(name)
    dts = []
    for k in range(3):
        o.fn("set_first_order")(1 if k < fo else 0)
        dts.append(o.step())
        if k == 0:
            s1 = o.state()
    s3 = o.state()
    assert np.array_equal(np.array(dts), gold["dts"])
    for k, s in (("1", s1), ("3", s3)):
        assert np.array_equal(interior(pb, s["convar"]), interior(pb, gold["convar" + k]))
        assert np.array_equal(s["alpha_x"], gold["alpha_x" + k])
        assert np.array_equal(s["alpha_y"], gold["alpha_y" + k])


@pytest.mark.skipif(not ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("order,charac,bc,wenotype", [
    (5, True, "free", None), (7, True, "free", None), (9, True, "free", None), (9, False, "free", None),
    (7, True, "reflect", None), (5, False, "periodic", None), (7, True, "inflow", None),
    (5, True, "free", "wenoz"), (5, True, "reflect", "wenojs"), (5, False, "periodic", "wenoz"),
    (5, False, "free", "wenojs"),
])
def test_oracle_matches_reference_bitwise(order, charac, bc, wenotype):
    """The restatement equals the compiled reference bit for bit; a wenotype selects the
    reference's default non-DF WENO5-AO slots (is_using_df_factor = false)."""
    pb, con, prim = cases.random_riemann2d(18, seed=order * 10 + len(bc), order=order)
    pb.characteristic = charac
    if wenotype:
        pb.use_df, pb.wenotype = False, wenotype
    if bc == "inflow":
        pb.bc = ("inflow", "free", "reflect", "free")
        pb.bc_prim = ((1.2, 0.8, 0.1, 1.1), (0,) * 4, (0,) * 4, (0,) * 4)
    else:
        pb.bc = (bc,) * 4
    a = CpuStep("ref").init(pb)
    b = CpuStep("oracle").init(pb)
    a.set_state(con, prim)
    b.set_state(con, prim)
    for _ in range(4):
        assert a.step() == b.step()
    sa, sb = a.state(), b.state()
    assert np.array_equal(interior(pb, sa["convar"]), interior(pb, sb["convar"]))
    assert np.array_equal(sa["alpha_x"], sb["alpha_x"])
    assert np.array_equal(sa["alpha_y"], sb["alpha_y"])
    for d in (0, 1):
        ga, gb = a.gauss(d), b.gauss(d)
        g = pb.ghost
        sl = (slice(g, g + pb.nodex), slice(g, g + pb.nodey))
        assert np.array_equal(ga[sl], gb[sl])


@pytest.mark.skipif(not ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("name", ["lfns_w5_mu_18", "lfns_w7_nu_18", "lfns_w9_walls_18"])
def test_oracle_lf_viscous_term_matches_reference_bitwise(name):
    """LF2D + NS_by_central_difference_prim_2D against the reference run by the harness, which
    fills the centre states the reference computes only for GKS2D."""
    pb, con, prim = _problem(name)
    a = CpuStep("ref").init(pb)
    b = CpuStep("oracle").init(pb)
    a.set_state(con, prim)
    b.set_state(con, prim)
    for _ in range(4):
        assert a.step() == b.step()
    sa, sb = a.state(), b.state()
    assert np.array_equal(interior(pb, sa["convar"]), interior(pb, sb["convar"]))
    assert np.array_equal(sa["alpha_x"], sb["alpha_x"])


def test_oracle_lf_viscous_term_acts():
    """The viscous term changes the LF2D step of a smooth flow (it is not silently dropped)."""
    pb, con, prim = cases.isentropic_vortex(24, order=5)
    pb.flux, pb.mu = "LF", 1e-2
    out = []
    for tau in (0, 1):
        pb.tau_type = tau
        o = CpuStep("oracle").init(pb)
        o.set_state(con, prim)
        for _ in range(3):
            o.step()
        out.append(o.state()["convar"])
    assert rel_linf(out[1], out[0], pb) > 1e-5


def _sinwave_errors(n):
    pb, con, prim = cases.sinwave2d(n, order=9)
    o = CpuStep("oracle").init(pb)
    o.set_state(con, prim)
    while o.t < 2.0:
        o.step(2.0)
    e = np.abs(interior(pb, o.state()["convar"][..., 0]) - interior(pb, prim[..., 0]))
    return np.array([e.mean(), np.sqrt((e * e).mean()), e.max()])


def test_oracle_2d_accuracy_known_answer():
    """The reference's 2D accuracy driver (sinwave_2d, WENO9-AO-DF, 4 Gauss-Lobatto points,
    src/2Dproblem.cpp:1347-1603): error norms at t = 2 equal the reference's, and the L1
    order between 10^2 and 20^2 is above 9 as the reference reports."""
    gold = np.load(GOLDEN / "sinwave_w9_accuracy.npz")
    e10, e20 = _sinwave_errors(10), _sinwave_errors(20)
    np.testing.assert_allclose(e10, gold["n10"], rtol=1e-12)
    np.testing.assert_allclose(e20, gold["n20"], rtol=1e-12)
    assert np.log2(e10[0] / e20[0]) > 9.0


def test_oracle_conserves_on_periodic_domain():
    pb, con, prim = cases.isentropic_vortex(24, order=5)
    o = CpuStep("oracle").init(pb, threads=4)
    o.set_state(con, prim)
    tot0 = interior(pb, con).sum(axis=(0, 1))
    for _ in range(5):
        o.step()
    tot = interior(pb, o.state()["convar"]).sum(axis=(0, 1))
    assert np.all(np.abs(tot - tot0) <= 1e-12 * np.abs(tot0).max())


@pytest.mark.skipif(not ref_available(), reason="reference checkout not present")
def test_oracle_wedge_boundary_matches_reference_bitwise():
    """Double-Mach-reflection boundary (boundaryforDoubleMach, src/2Dproblem.cpp:1029-1093,
    Mach 10) on nodex = nodey (the reference's Update_alpha bound is only in range there)."""
    pb, con, prim = cases.wedge2d(24, 24, mach=10.0, order=5)
    a = CpuStep("ref").init(pb)
    b = CpuStep("oracle").init(pb)
    a.set_state(con, prim)
    b.set_state(con, prim)
    for _ in range(6):
        assert a.step(0.2) == b.step(0.2)
    assert np.array_equal(a.state()["convar"], b.state()["convar"])


def test_oblique_shock_states_reduce_to_reference_constants():
    post, pre, speed = cases.oblique_shock_states(10.0)
    import math
    assert post == (8.0, 4.125 * math.sqrt(3), -4.125, 116.5) and pre == (1.4, 0.0, 0.0, 1.0)
    # the general Rankine-Hugoniot branch agrees with the literal Mach-10 constants
    rho1, p1, g = 1.4, 1.0, 1.4
    m2 = 100.0
    assert abs(rho1 * (g + 1) * m2 / ((g - 1) * m2 + 2) - 8.0) < 1e-12
    assert abs(p1 * (2 * g * m2 - (g - 1)) / (g + 1) - 116.5) < 1e-12


@pytest.mark.parametrize("name", ["nodf_w5_z_free_24", "nodf_w5_z_cons_20"])
def test_nodf_scheme_amplifies_rounding(name):
    """The non-DF WENO5-AO (epsilon 1e-10 in the weights, the big-stencil indicator as a raw
    quadratic form with coefficients ~1e5) carries a 1e-15 relative perturbation of the initial
    state past 1e-13 within three steps, where the DF variant of the same data stays near 1e-15:
    that bounds how closely any other arithmetic can follow the reference there."""
    pb, con, prim = _problem(name)
    dev = {}
    for df in (False, True):
        pb.use_df = df
        runs = []
        for eps in (0.0, 1e-15):
            o = CpuStep("oracle").init(pb, threads=4)
            o.set_state(con * (1 + eps * np.sin(np.arange(con.size).reshape(con.shape))), prim)
            for _ in range(3):
                o.step()
            runs.append(o.state()["convar"])
        dev[df] = rel_linf(runs[1], runs[0], pb)
    assert dev[False] > 1e-13 and dev[True] < 1e-14, dev


def test_viscous_cap_case_amplifies_rounding():
    """In the viscous-cap case the algorithm amplifies rounding: a 1e-15 relative perturbation
    of the initial state grows past 1e-13 within three steps (the GKS time coefficients
    with tau_num >> dt cancel), which bounds how closely any other arithmetic can follow it."""
    pb, con, prim = _problem("ns_w7_cap_24")
    runs = []
    for eps in (0.0, 1e-15):
        o = CpuStep("oracle").init(pb, threads=4)
        o.set_state(con * (1 + eps * np.sin(np.arange(con.size).reshape(con.shape))), prim)
        for k in range(3):
            o.fn("set_first_order")(1 if k == 0 else 0)
            o.step()
        runs.append(o.state()["convar"])
    assert rel_linf(runs[1], runs[0], pb) > 1e-13
