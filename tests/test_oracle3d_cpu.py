"""The 3D restatement (oracle/hos_oracle3d.cpp), checked on the CPU.

The reference's own 3D path does not run as shipped: its Gauss-point arrays are never
allocated.  oracle/ref_driver3d.cpp allocates them and runs the reference's own 3D
functions unmodified (CubicTube's loop).  The restatement is pinned as follows:
  * with the reference's own conventions switched on (pressure in GKS3D's lambda slots,
    order-reduction flags of lines and points that stay set), it equals the reference's 3D
    code bit for bit (golden vectors tests/golden/ref3d_*.npz, and the compiled reference
    where the checkout exists); switching them off is the only difference to the default;
  * one-dimensional data along x, y or z gives the 1D restatement's result, which is itself
    bit-exact with the compiled reference (test_oracle1d_cpu.py), to rounding: this covers
    the normal reconstruction, every GKS3D term, the update, the CFL and the frame rotations;
  * a smooth periodic 3D wave converges at the scheme's order, which the tangential line and
    point reconstructions at the 2x2 Gauss points must reach;
  * mass, momentum and energy are conserved on a periodic box;
  * a state symmetric under the cyclic permutation of the axes stays symmetric.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle_lib import CpuStep1D, CpuStep3D, ref_available

from hos_gb300.params import DF_NEVER, Problem1D, Problem3D

G = 3
GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"
REF3D_CASES = ["ref3d_smooth_free_12", "ref3d_cubicsod_free_12", "ref3d_smooth_cons_ns_10"]


def _grid3(pb):
    xc = pb.left + (np.arange(pb.shape[0]) - G + 0.5) * pb.dx
    yc = pb.down + (np.arange(pb.shape[1]) - G + 0.5) * pb.dy
    zc = pb.back + (np.arange(pb.shape[2]) - G + 0.5) * pb.dz
    return np.meshgrid(xc, yc, zc, indexing="ij")


def _state3(rho, u, v, w, p, gamma=1.4):
    return np.stack([rho, rho * u, rho * v, rho * w, p / (gamma - 1) + 0.5 * rho * (u * u + v * v + w * w)], -1)


def ref3d_problem(name):
    """The 3D cases the reference's own code is run on (free sides: the reference's only 3D
    boundary), as (problem, convar, steps).
      smooth_free   : a smooth seeded field, characteristic variables, Euler, 3 steps
      cubicsod_free : CubicTube's box (src/3Dproblem.cpp:174-219), 1 step (with the pressure
                      in the lambda slots the reference blows up in its second step)
      smooth_cons_ns: the smooth field in conservative variables, NS collision time with
                      Mu = 2e-3, 3 steps"""
    n = int(name.rsplit("_", 1)[1])
    kw = dict(nodex=n, nodey=n, nodez=n, ghost=G, bc=("free",) * 6, c1_euler=0.05, c2_euler=1.0)
    if "cubicsod" in name:
        pb = Problem3D(**kw)
        X, Y, Z = _grid3(pb)
        inside = (np.abs(X - 0.5) < 0.2) & (np.abs(Y - 0.5) < 0.2) & (np.abs(Z - 0.5) < 0.2)
        zero = np.zeros(pb.shape)
        return pb, _state3(np.where(inside, 1.0, 0.125), zero, zero, zero, np.where(inside, 1.0, 0.1)), 1
    if "cons_ns" in name:
        kw.update(characteristic=False, tau_type=1, mu=2e-3)
    pb = Problem3D(**kw)
    X, Y, Z = _grid3(pb)
    k = 2 * np.pi
    a = np.random.default_rng(n).uniform(-0.4, 0.4, 12)
    rho = 1.0 + 0.2 * np.sin(k * X + a[0]) * np.cos(k * Y + a[1]) + 0.1 * np.sin(k * Z + a[2])
    u = 0.3 * np.sin(k * Y + a[3])
    v = 0.3 * np.sin(k * Z + a[5])
    w = 0.3 * np.sin(k * X + a[7])
    p = 1.0 + 0.2 * np.cos(k * (X + Y) + a[9])
    return pb, _state3(rho, u, v, w, p), 3


def _run_conventions(kind, pb, W, steps):
    c = CpuStep3D(kind).init(pb)
    if kind == "oracle":
        c.fn("set_reference_conventions")(1)
    c.set_state(W)
    dts, states = [], []
    for _ in range(steps):
        dts.append(c.step())
        states.append(c.state()["convar"])
    return c, np.array(dts), states


@pytest.mark.parametrize("name", REF3D_CASES)
def test_3d_restatement_matches_reference_golden_bitwise(name):
    """With the reference's conventions the restatement reproduces the reference's own 3D
    functions' outputs (tests/golden/ref3d_*.npz, made by tests/golden/make_golden.py) bit for
    bit: every time step and every interior state."""
    pb, W, steps = ref3d_problem(name)
    gold = np.load(GOLDEN / f"{name}.npz")
    assert np.array_equal(W[G:-G, G:-G, G:-G], gold["convar0"][G:-G, G:-G, G:-G])
    c, dts, states = _run_conventions("oracle", pb, gold["convar0"], steps)
    assert np.array_equal(dts, gold["dts"])
    for k, st in enumerate(states):
        assert np.array_equal(st[G:-G, G:-G, G:-G], gold[f"convar{k + 1}"][G:-G, G:-G, G:-G]), k
    c.fn("reduced_count").restype = ctypes.c_longlong
    assert c.fn("reduced_count")() == 0   # no order reduction on the faces the fluxes use


@pytest.mark.skipif(not ref_available(), reason="reference checkout not present")
def test_3d_restatement_matches_compiled_reference_bitwise():
    pb, W, _ = ref3d_problem("ref3d_smooth_free_12")
    _, da, sa = _run_conventions("ref", pb, W, 6)
    _, db, sb = _run_conventions("oracle", pb, W, 6)
    assert np.array_equal(da, db)
    for a, b in zip(sa, sb):
        assert np.array_equal(a[G:-G, G:-G, G:-G], b[G:-G, G:-G, G:-G])


def test_3d_reference_conventions_differ_from_the_default():
    """The two conventions are the only switch between the pinned and the default restatement;
    with the pressure in the lambda slots the step is a different (wrong) one."""
    pb, W, _ = ref3d_problem("ref3d_smooth_free_12")
    _, _, sa = _run_conventions("oracle", pb, W, 1)
    d = CpuStep3D("oracle").init(pb)
    d.fn("set_reference_conventions")(0)
    d.set_state(W)
    d.step()
    b = d.state()["convar"]
    assert np.abs(sa[0] - b)[G:-G, G:-G, G:-G].max() > 1e-6


def _sod_1d(n, c1, c2):
    p1 = Problem1D(nodex=n, order=5, df_mode=DF_NEVER, update_alpha=False, ghost=G, K=4,
                   c1_euler=c1, c2_euler=c2)
    x = (np.arange(p1.nx) - G + 0.5) / n
    rho = np.where(x < 0.5, 1.0, 0.125)
    p = np.where(x < 0.5, 1.0, 0.1)
    u = np.where(x < 0.5, 0.3, -0.2)
    return p1, np.stack([rho, rho * u, p / 0.4 + 0.5 * rho * u * u], -1)


def _embed(pb, W1, axis):
    W3 = np.zeros(pb.shape + (5,))
    shp = [1, 1, 1]
    shp[axis] = W1.shape[0]
    W3[..., 0] = W1[:, 0].reshape(shp)
    W3[..., 1 + axis] = W1[:, 1].reshape(shp)
    W3[..., 4] = W1[:, 2].reshape(shp)
    return W3


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("c1,c2,half_tau_of_dt", [(0.05, 1.0, 1), (0.0, 0.0, 0)])
def test_3d_on_1d_data_matches_the_1d_restatement(axis, c1, c2, half_tau_of_dt):
    n = 40
    p1, W1 = _sod_1d(n, c1, c2)
    o1 = CpuStep1D().init(p1)
    o1.set_state(W1)
    dims = [4, 4, 4]
    dims[axis] = n
    pb = Problem3D(nodex=dims[0], nodey=dims[1], nodez=dims[2], ghost=G, c1_euler=c1, c2_euler=c2)
    o3 = CpuStep3D().init(pb)
    o3.fn("set_half_tau_of_dt")(half_tau_of_dt)
    try:
        for _ in range(5):
            # the 1D CFL reads the fresh state, the 3D one the lagged primitives: start each
            # step from the same state with fresh primitives
            o3.set_state(_embed(pb, o1.state()["convar"].copy(), axis))
            dt3 = o3.step()
            dt1 = o1.step()
            assert dt3 == pytest.approx(dt1, rel=1e-14)
            W1n = o1.state()["convar"][G:G + n]
            W3n = o3.state()["convar"][G:-G, G:-G, G:-G]
            # uniform across the two tangential directions, no tangential momentum
            others = tuple(a for a in range(3) if a != axis)
            assert np.ptp(W3n, axis=others).max() == 0.0
            assert max(np.abs(W3n[..., 1 + a]).max() for a in others) < 1e-15
            idx = [0, 0, 0]
            idx[axis] = slice(None)
            line = W3n[tuple(idx)]
            got = np.stack([line[:, 0], line[:, 1 + axis], line[:, 4]], -1)
            assert np.abs(got - W1n).max() / np.abs(W1n).max() < 1e-11
    finally:
        o3.fn("set_half_tau_of_dt")(0)


def _wave(n, t=0.0):
    """cell averages of rho = 1 + 0.2 sin(2 pi (x + y + z - 3t)), u = v = w = 1, p = 1"""
    pb = Problem3D(nodex=n, nodey=n, nodez=n, ghost=G, bc=("periodic",) * 6, c1_euler=0.0, c2_euler=0.0)
    h = 1.0 / n
    xc = (np.arange(pb.shape[0]) - G + 0.5) * h
    X, Y, Z = np.meshgrid(xc, xc, xc, indexing="ij")
    fac = (np.sin(np.pi * h) / (np.pi * h)) ** 3
    return pb, 1.0 + 0.2 * fac * np.sin(2 * np.pi * (X + Y + Z - 3 * t))


def _wave_state(pb, rho):
    W = np.zeros(pb.shape + (5,))
    W[..., 0] = rho
    W[..., 1] = W[..., 2] = W[..., 3] = rho
    W[..., 4] = 1.0 / 0.4 + 1.5 * rho
    return W


def test_3d_smooth_wave_converges_at_high_order():
    errs = []
    for n in (8, 16):
        pb, rho = _wave(n)
        o = CpuStep3D().init(pb)
        o.set_state(_wave_state(pb, rho))
        while o.t < 0.1:
            o.step(0.1)
        _, exact = _wave(n, o.t)
        got = o.state()["convar"][G:-G, G:-G, G:-G, 0]
        errs.append(np.abs(got - exact[G:-G, G:-G, G:-G]).mean())
    order = np.log2(errs[0] / errs[1])
    assert order > 4.5, (errs, order)


def _random_periodic(n, seed):
    rng = np.random.default_rng(seed)
    pb = Problem3D(nodex=n, nodey=n, nodez=n, ghost=G, bc=("periodic",) * 6)
    h = 1.0 / n
    xc = (np.arange(pb.shape[0]) - G + 0.5) * h
    X, Y, Z = np.meshgrid(xc, xc, xc, indexing="ij")
    k = 2 * np.pi
    a = rng.uniform(-0.3, 0.3, size=12)
    rho = 1.0 + 0.2 * np.sin(k * X + a[0]) * np.cos(k * Y + a[1]) + 0.1 * np.sin(k * Z + a[2])
    u = 0.4 * np.sin(k * Y + a[3]) + a[4]
    v = 0.4 * np.sin(k * Z + a[5]) + a[6]
    w = 0.4 * np.sin(k * X + a[7]) + a[8]
    p = 1.0 + 0.2 * np.cos(k * (X + Y) + a[9]) + a[10]
    W = np.stack([rho, rho * u, rho * v, rho * w, p / 0.4 + 0.5 * rho * (u * u + v * v + w * w)], -1)
    return pb, W


def test_3d_periodic_box_conserves_mass_momentum_energy():
    pb, W = _random_periodic(10, 3)
    o = CpuStep3D().init(pb)
    o.set_state(W)
    s0 = W[G:-G, G:-G, G:-G].sum(axis=(0, 1, 2))
    for _ in range(3):
        o.step()
    s1 = o.state()["convar"][G:-G, G:-G, G:-G].sum(axis=(0, 1, 2))
    assert np.abs(s1 - s0).max() / np.abs(W[G:-G, G:-G, G:-G]).sum(axis=(0, 1, 2)).max() < 1e-13


def test_3d_mirror_symmetry_in_each_axis():
    """A state even under x -> -x (with u odd), and likewise in y and z, stays so.  (The
    sweep order of the tangential reconstruction -- lines then points: y then z on x faces,
    -x then z on y faces, y then -x on z faces -- is part of the scheme, so the scheme is not
    symmetric under axis permutations, only under reflections.)"""
    n = 10
    pb = Problem3D(nodex=n, nodey=n, nodez=n, ghost=G, bc=("periodic",) * 6)
    h = 1.0 / n
    xc = (np.arange(pb.shape[0]) - G + 0.5) * h
    X, Y, Z = np.meshgrid(xc, xc, xc, indexing="ij")
    k = 2 * np.pi
    cx, cy, cz = np.cos(k * X), np.cos(k * Y), np.cos(k * Z)
    rho = 1.0 + 0.2 * cx * np.cos(2 * k * Y) * cz + 0.05 * cy
    u = 0.3 * np.sin(k * X) * cy * cz
    v = 0.2 * cx * np.sin(k * Y) * cz
    w = 0.1 * cx * cy * np.sin(k * Z)
    p = 1.0 + 0.1 * cx * cy * cz + 0.05 * np.cos(2 * k * Z)
    W = np.stack([rho, rho * u, rho * v, rho * w, p / 0.4 + 0.5 * rho * (u * u + v * v + w * w)], -1)
    o = CpuStep3D().init(pb)
    o.set_state(W)
    for _ in range(2):
        o.step()
    out = o.state()["convar"][G:-G, G:-G, G:-G]
    for ax in range(3):
        m = np.flip(out, axis=ax).copy()
        m[..., 1 + ax] = -m[..., 1 + ax]
        assert np.abs(m - out).max() / np.abs(out).max() < 1e-12, ax


def test_3d_prandtl_fix_corrects_the_energy_flux_only():
    """The Prandtl-number correction adds (1/Pr - 1) q to the energy flux (q: the heat flux of
    the equilibrium part's slopes, GKS2D's form with the third velocity component): mass and
    momentum fluxes of a stage are unchanged, the energy flux moves, and Pr = 1 changes
    nothing."""
    from hos_gb300.params import TAU_NS
    fl = {}
    for name, fix, pr in (("off", False, 1.0), ("pr1", True, 1.0), ("pr071", True, 0.71)):
        pb, W = _random_periodic(8, 5)
        pb.tau_type, pb.mu, pb.c2_euler = TAU_NS, 0.01, 1.0
        pb.prandtl_fix, pb.prandtl = fix, pr
        o = CpuStep3D().init(pb)
        o.set_state(W)
        dt = o.lib.oracle3d_begin_step(ctypes.c_double(1e30), ctypes.c_double(0.0))
        assert o.fn("stage")(0, ctypes.c_double(dt)) == 0
        nf = (pb.nodex + 1) * pb.nodey * pb.nodez
        out = np.zeros(nf * 2 * 10)
        o.fn("get_flux")(0, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        fl[name] = out.reshape(nf, 2, 10)[:, 0, :]
    assert np.array_equal(fl["off"], fl["pr1"])
    a, b = fl["off"], fl["pr071"]
    assert np.array_equal(a[:, [0, 1, 2, 3, 5, 6, 7, 8]], b[:, [0, 1, 2, 3, 5, 6, 7, 8]])
    assert np.abs(a[:, 4] - b[:, 4]).max() > 1e-10 * np.abs(a[:, 4]).max()
