"""GPU parity of the 3D step (WENO5-AO on 2 x 2 Gauss points, GKS3D, S2O4) against the 3D
restatement (oracle/hos_oracle3d.cpp), which the CPU suite pins against the 1D restatement.
FP64: relative L-inf <= 1e-11 after a few steps (the GPU contracts multiply-adds and uses
reciprocals, so agreement is to rounding, not bitwise).  FP32 bulk: relative L1 <= 1e-5."""
import numpy as np
import pytest

from hos_gb300.params import TAU_NS, Problem3D
from hos_gb300.solver import FP32, FP64, HosError, Solver3D
from oracle_lib import CpuStep3D

pytestmark = pytest.mark.gpu
G = 3


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build()


def _grid(pb):
    xc = pb.left + (np.arange(pb.shape[0]) - G + 0.5) * pb.dx
    yc = pb.down + (np.arange(pb.shape[1]) - G + 0.5) * pb.dy
    zc = pb.back + (np.arange(pb.shape[2]) - G + 0.5) * pb.dz
    return np.meshgrid(xc, yc, zc, indexing="ij")


def _state(rho, u, v, w, p, gamma=1.4):
    return np.stack([rho, rho * u, rho * v, rho * w, p / (gamma - 1) + 0.5 * rho * (u * u + v * v + w * w)], -1)


def smooth_periodic(n=(12, 10, 8), seed=0, **kw):
    pb = Problem3D(nodex=n[0], nodey=n[1], nodez=n[2], ghost=G, bc=("periodic",) * 6, **kw)
    X, Y, Z = _grid(pb)
    rng = np.random.default_rng(seed)
    a = rng.uniform(-0.4, 0.4, size=12)
    k = 2 * np.pi
    rho = 1.0 + 0.2 * np.sin(k * X + a[0]) * np.cos(k * Y + a[1]) + 0.1 * np.sin(k * Z + a[2])
    u = 0.4 * np.sin(k * Y + a[3]) + a[4]
    v = 0.4 * np.sin(k * Z + a[5]) + a[6]
    w = 0.4 * np.sin(k * X + a[7]) + a[8]
    p = 1.0 + 0.2 * np.cos(k * (X + Y) + a[9]) + 0.1 * np.sin(k * Z) + a[10]
    return pb, _state(rho, u, v, w, p)


def cubic_sod(n=16, **kw):
    """the reference's CubicTube initial state (src/3Dproblem.cpp:174-219): a box of
    (1, 0, 0, 0, 1) inside |x - 0.5|, |y - 0.5|, |z - 0.5| < 0.2, (0.125, 0, 0, 0, 0.1) outside"""
    pb = Problem3D(nodex=n, nodey=n, nodez=n, ghost=G, **kw)
    X, Y, Z = _grid(pb)
    inside = (np.abs(X - 0.5) < 0.2) & (np.abs(Y - 0.5) < 0.2) & (np.abs(Z - 0.5) < 0.2)
    rho = np.where(inside, 1.0, 0.125)
    p = np.where(inside, 1.0, 0.1)
    zero = np.zeros_like(rho)
    return pb, _state(rho, zero, zero, zero, p)


def _interior(a):
    return a[G:-G, G:-G, G:-G]


def _compare(pb, W, steps, precision=FP64):
    o = CpuStep3D().init(pb)
    o.set_state(W)
    s = Solver3D(pb, precision)
    s.set_state(W)
    dts = []
    for _ in range(steps):
        dto = o.step()
        s.step()
        dts.append((s.sync()[1], dto))
    got = s.get_state()["convar"]
    ref = o.state()["convar"]
    s.close()
    return _interior(got), _interior(ref), np.array(dts)


@pytest.mark.parametrize("case", ["periodic", "periodic_conservative", "periodic_ns", "periodic_ns_prandtl",
                                  "cubic_sod_free", "cubic_sod_reflect"])
def test_gpu3d_fp64_matches_oracle(case):
    if case == "periodic":
        pb, W = smooth_periodic()
    elif case == "periodic_conservative":
        pb, W = smooth_periodic(seed=1, characteristic=False)
    elif case == "periodic_ns":
        pb, W = smooth_periodic(seed=2, tau_type=TAU_NS, mu=0.01, c2_euler=1.0)
    elif case == "periodic_ns_prandtl":
        pb, W = smooth_periodic(seed=4, tau_type=TAU_NS, mu=0.01, c2_euler=1.0, prandtl_fix=True, prandtl=0.71)
    elif case == "cubic_sod_free":
        pb, W = cubic_sod()
    else:
        pb, W = cubic_sod(bc=("reflect",) * 6)
    got, ref, dts = _compare(pb, W, 3)
    np.testing.assert_allclose(dts[:, 0], dts[:, 1], rtol=1e-13)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-11


@pytest.mark.parametrize("name", ["ref3d_smooth_free_12", "ref3d_cubicsod_free_12", "ref3d_smooth_cons_ns_10"])
def test_gpu3d_reference_convention_matches_reference_golden(name):
    """The GPU with the reference's own GKS3D convention (gks3d_pressure_slot: pressure where
    lambda belongs) against the outputs of the reference's 3D functions (tests/golden/ref3d_*,
    run by oracle/ref_driver3d.cpp): 1e-12 relative L-inf after the first step, 1e-11 after
    three, every dt to 1e-13.  No order reduction occurs on the faces the fluxes use there,
    so the reference's never-cleared reduction flags do not enter."""
    from pathlib import Path

    from test_oracle3d_cpu import ref3d_problem

    pb, _, steps = ref3d_problem(name)
    pb.gks3d_pressure_slot = True
    gold = np.load(Path(__file__).resolve().parent / "golden" / f"{name}.npz")
    s = Solver3D(pb, FP64)
    s.set_state(gold["convar0"])
    for k in range(steps):
        s.step()
        dt = s.sync()[1]
        np.testing.assert_allclose(dt, gold["dts"][k], rtol=1e-13)
        got, ref = _interior(s.get_state()["convar"]), _interior(gold[f"convar{k + 1}"])
        assert np.abs(got - ref).max() / np.abs(ref).max() <= (1e-12 if k == 0 else 1e-11), k
    s.close()


def test_gpu3d_reference_convention_needs_fp64():
    from test_oracle3d_cpu import ref3d_problem

    pb, _, _ = ref3d_problem("ref3d_smooth_free_12")
    pb.gks3d_pressure_slot = True
    with pytest.raises(HosError):
        Solver3D(pb, FP32)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_gpu3d_sod_along_each_axis_matches_oracle(axis):
    dims = [4, 4, 4]
    dims[axis] = 48
    pb = Problem3D(nodex=dims[0], nodey=dims[1], nodez=dims[2], ghost=G)
    X, Y, Z = _grid(pb)
    x = (X, Y, Z)[axis]
    rho = np.where(x < 0.5, 1.0, 0.125)
    p = np.where(x < 0.5, 1.0, 0.1)
    vel = [np.zeros_like(rho)] * 3
    vel[axis] = np.where(x < 0.5, 0.3, -0.2)
    W = _state(rho, vel[0], vel[1], vel[2], p)
    got, ref, _ = _compare(pb, W, 5)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-11


def test_gpu3d_stage_api_equals_step():
    pb, W = smooth_periodic(seed=3)
    a = Solver3D(pb, FP64)
    b = Solver3D(pb, FP64)
    a.set_state(W)
    b.set_state(W)
    for _ in range(2):
        a.step()
        b.begin_step(1e30)
        b.stage(0)
        b.stage(1)
    assert np.array_equal(a.get_state()["convar"], b.get_state()["convar"])
    a.close()
    b.close()


def test_gpu3d_periodic_conservation_and_stop_time():
    pb, W = smooth_periodic(n=(16, 16, 16), seed=4)
    s = Solver3D(pb, FP64)
    s.set_state(W)
    s0 = _interior(W).sum(axis=(0, 1, 2))
    steps = s.run(0.02)
    t, _ = s.sync()
    assert t == pytest.approx(0.02 + 1e-16, abs=1e-15) and steps >= 2
    s1 = _interior(s.get_state()["convar"]).sum(axis=(0, 1, 2))
    assert np.abs(s1 - s0).max() / np.abs(_interior(W)).sum(axis=(0, 1, 2)).max() < 1e-13
    s.close()


def test_gpu3d_fp32_bulk_close_to_fp64():
    pb, W = smooth_periodic(n=(16, 16, 16), seed=5)
    res = []
    for prec in (FP64, FP32):
        s = Solver3D(pb, prec)
        s.set_state(W)
        s.advance(5)
        res.append(_interior(s.get_state()["convar"]))
        s.close()
    rel_l1 = np.abs(res[1] - res[0]).sum() / np.abs(res[0]).sum()
    assert rel_l1 < 1e-5


def test_gpu3d_primvar_output_and_initial_primitives():
    pb, W = smooth_periodic(seed=6)
    s = Solver3D(pb, FP64)
    rho = W[..., 0]
    prim = np.stack([rho, W[..., 1] / rho, W[..., 2] / rho, W[..., 3] / rho,
                     0.4 * (W[..., 4] - 0.5 * (W[..., 1] ** 2 + W[..., 2] ** 2 + W[..., 3] ** 2) / rho)], -1)
    s.set_state(W, prim)
    out = s.get_state(primvar=True)
    assert np.allclose(out["primvar"], prim, rtol=1e-13, atol=1e-13)
    s.close()


def test_gpu3d_rejects_bad_configuration():
    with pytest.raises(HosError):
        Solver3D(Problem3D(nodex=8, nodey=8, nodez=8, ghost=2), FP64)
    with pytest.raises(HosError):
        Solver3D(Problem3D(nodex=8, nodey=8, nodez=8, bc=("periodic", "free", "free", "free", "free", "free")), FP64)
