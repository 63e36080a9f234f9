"""hos2d_step_static: the allocation-free step, for callers that may not allocate device
memory once running (a code that reserves its whole HBM budget at start-up, or runs under a
fixed memory quota on a shared GPU).  The caller owns the state; the step's scratch is a
fixed static device array inside the library.

Checks, through the C ABI, that two calls in a row give the same states as the allocating
entry point (hos2d_create + hos2d_step) fed the same time steps, within the 1e-12 relative
L-inf tolerance of the parity tests, and that an oversized problem is rejected.  This file
is collected last on purpose and must pass alone or after the other tests."""
import ctypes

import numpy as np
import pytest

from hos_gb300 import cases
from hos_gb300.params import Params2D
from hos_gb300.solver import FP64, Solver2D, load

pytestmark = pytest.mark.gpu
TOL = 1e-12


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


@pytest.mark.parametrize("maker", [lambda: cases.riemann2d(96, order=7), lambda: cases.isentropic_vortex(64, order=5)])
def test_static_step_matches_allocating_step(lib, maker):
    import torch

    pb, con, prim = maker()
    nx, ny = pb.nx, pb.ny
    # existing entry point: allocating solver, record the two steps' dt and states
    s = Solver2D(pb, FP64)
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
        rc = lib.hos2d_step_static(ctypes.byref(p), FP64, W.data_ptr(), ax.data_ptr(), ay.data_ptr(), dts[k],
                                   ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.hos_static_last_error()
        torch.cuda.synchronize(dev)
        got = W.cpu().numpy().T.reshape(nx, ny, 4)
        ref = states[k][0]
        g = pb.ghost
        err = np.abs(got - ref)[g:-g, g:-g].max() / np.abs(ref[g:-g, g:-g]).max()
        assert err <= TOL, (k, err)
        ga = ax.cpu().numpy().reshape(nx, ny)
        assert np.abs(ga - states[k][1]).max() <= 1e-9 * max(1.0, np.abs(states[k][1]).max())


def test_static_step_rejects_oversized_problem(lib):
    pb, _, _ = cases.riemann2d(300, order=5)
    p = pb.to_c()
    rc = lib.hos2d_step_static(ctypes.byref(p), FP64, ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1),
                               1e-3, None)
    assert rc == 2
    assert b"static scratch limit" in lib.hos_static_last_error()
