"""hos2d_step_static: the allocation-free step, for callers that may not allocate device memory
once running (a code that reserves its whole HBM budget at start-up, or runs under a fixed
memory quota on a shared GPU).  The caller owns the state; the step's scratch is a fixed
static device array inside the library.

Checks, through the C ABI, that two calls in a row give the same states and DF indicators as
the allocating entry point (hos2d_create + hos2d_step) fed the same time steps -- FP64 within
the 1e-12 relative L-inf tolerance of the parity tests, FP32 within the 2e-6 the TMA-staged and
converting FP32 kernels are held to -- with the Euler and the Navier-Stokes collision times,
and that problems or settings the step does not run are rejected.  This file is collected last
on purpose and must pass alone or after the other tests."""
import ctypes

import numpy as np
import pytest

from hos_gb300 import cases
from hos_gb300.params import Params2D
from hos_gb300.solver import FP32, FP64, Solver2D, load

pytestmark = pytest.mark.gpu
TOL = {FP64: 1e-12, FP32: 2e-6}


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge
    ge.build()
    lib = load()
    lib.hos2d_step_static.argtypes = [ctypes.POINTER(Params2D), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
    lib.hos_static_last_error.restype = ctypes.c_char_p
    return lib


def _soa(aos, nx, ny):
    return np.ascontiguousarray(aos.reshape(nx * ny, 4).T)


def _ns_walls():
    """Navier-Stokes collision time with the Prandtl fix, inflow / reflecting sides."""
    pb, con, prim = cases.random_riemann2d(48, seed=7, order=5)
    pb.tau_type, pb.mu, pb.c2_euler, pb.prandtl_fix, pb.prandtl = 1, 5e-3, 1.0, True, 0.72
    pb.bc = ("inflow", "free", "reflect", "reflect")
    pb.bc_prim = ((1.2, 0.8, 0.1, 1.0), (0.0,) * 4, (0.0,) * 4, (0.0,) * 4)
    return pb, con, prim


MAKERS = {"riemann_w7": lambda: cases.riemann2d(96, order=7),
          "vortex_w5": lambda: cases.isentropic_vortex(64, order=5),
          "ns_prandtl_w5": _ns_walls}


@pytest.mark.parametrize("precision", [FP64, FP32], ids=["fp64", "fp32"])
@pytest.mark.parametrize("case", list(MAKERS))
def test_static_step_matches_allocating_step(lib, case, precision):
    import torch

    pb, con, prim = MAKERS[case]()
    nx, ny, g = pb.nx, pb.ny, pb.ghost
    # existing entry point: allocating solver, record the two steps' dt and states
    s = Solver2D(pb, precision)
    s.set_state(con, prim)
    dts, states = [], []
    for _ in range(2):
        s.step(1e30)
        dts.append(s.sync()[1])
        st = s.get_state()
        states.append((st["convar"], st["alpha_x"], st["alpha_y"]))
    s.close()
    # new entry point on caller-owned device buffers (the test allocates them, the call does not)
    dev = torch.device("cuda", 0)
    W = torch.from_numpy(_soa(con, nx, ny)).to(dev)
    ax = torch.zeros(nx * ny, dtype=torch.float64, device=dev)
    ay = torch.zeros(nx * ny, dtype=torch.float64, device=dev)
    p = pb.to_c()
    stream = torch.cuda.current_stream(dev)
    for k in range(2):
        rc = lib.hos2d_step_static(ctypes.byref(p), precision, W.data_ptr(), ax.data_ptr(), ay.data_ptr(), dts[k],
                                   ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.hos_static_last_error()
        torch.cuda.synchronize(dev)
        got = W.cpu().numpy().T.reshape(nx, ny, 4)
        ref = states[k][0]
        err = np.abs(got - ref)[g:-g, g:-g].max() / np.abs(ref[g:-g, g:-g]).max()
        assert err <= TOL[precision], (k, err)
        # the DF indicators: an indicator below 2 is zeroed, so where rounding moves one across
        # that threshold the two entry points may differ by one O(1) value; FP64 may not
        for a_dev, a_ref in ((ax, states[k][1]), (ay, states[k][2])):
            ga = a_dev.cpu().numpy().reshape(nx, ny)
            d = np.abs(ga - a_ref)
            if precision == FP64:
                assert d.max() <= TOL[FP64] * max(1.0, np.abs(a_ref).max()), d.max()
            else:
                assert (d > 1e-4 * max(1.0, np.abs(a_ref).max())).mean() <= 1e-3


def _rejected(lib, pb, what):
    p = pb.to_c()
    rc = lib.hos2d_step_static(ctypes.byref(p), FP64, ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1),
                               1e-3, None)
    assert rc == 2, what
    return lib.hos_static_last_error()


def test_static_step_rejects_oversized_problem(lib):
    pb, _, _ = cases.riemann2d(300, order=5)
    assert b"static scratch limit" in _rejected(lib, pb, "nodex 300")
    pb, _, _ = cases.riemann2d(64, order=5)
    pb.ghost = 6
    assert b"static scratch limit" in _rejected(lib, pb, "ghost 6")


def test_static_step_rejects_settings_it_does_not_run(lib):
    pb, _, _ = cases.riemann2d(32, order=5)
    pb.bc = ("free", "free", "noslip", "free")
    assert b"boundaries" in _rejected(lib, pb, "no-slip side")
    pb, _, _ = cases.wedge2d(64, 32, mach=4.0, order=5)
    assert b"boundaries" in _rejected(lib, pb, "wedge")
    pb, _, _ = cases.riemann2d(32, order=5)
    pb.integrator = "RK3"
    assert b"S2O4" in _rejected(lib, pb, "RK3")
    pb, _, _ = cases.riemann2d(32, order=5)
    pb.use_df = False
    assert b"use_df" in _rejected(lib, pb, "non-DF")
