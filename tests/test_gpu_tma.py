"""TMA tile staging of the FP32 face kernels.

The FP32 solvers keep an FP32 mirror of the state with rows padded to a 32-byte pitch and
stage each face tile (conserved variables, both DF indicators, stencil halo) from it with one
cp.async.bulk.tensor load.  The allocation-free step (hos2d_step_static) runs the same FP32
face computation but loads its tiles from the FP64 state with ordinary loads, converting on
the fly.  Fed the same state and time step, both must produce the same FP32 stage results:
the staged values are the same roundings of the same FP64 numbers.  The grids cover every
order, row lengths that are and are not multiples of the pitch, tiles that hang over the
upper edge in both directions, and every boundary kind the tile halo reads."""
import ctypes

import numpy as np
import pytest

from hos_gb300 import cases
from hos_gb300.params import Params2D
from hos_gb300.solver import FP32, Solver2D, load

pytestmark = pytest.mark.gpu
# Same FP32 arithmetic on the same inputs; the two kernels are separate instantiations, so
# the compiler may contract a few multiply-adds differently: a few FP32 ulps of the state's
# increment, far below the FP32 path's own deviation from FP64 (~1e-7 relative).
TOL = 2e-6


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


def _problem(order, nodex, nodey, bc, seed):
    pb, con, prim = cases.random_riemann2d(max(nodex, nodey), seed=seed, order=order)
    pb.nodex, pb.nodey = nodex, nodey
    pb.right = pb.left + (pb.right - pb.left) * nodex / max(nodex, nodey)
    pb.up = pb.down + (pb.up - pb.down) * nodey / max(nodex, nodey)
    con = np.ascontiguousarray(con[: pb.nx, : pb.ny])
    prim = np.ascontiguousarray(prim[: pb.nx, : pb.ny])
    pb.bc = bc
    return pb, con, prim


CASES = [
    (5, 64, 64, ("free",) * 4),
    (7, 45, 37, ("free",) * 4),                                  # ny = 47: pitch pads 1 cell
    (7, 40, 61, ("periodic",) * 4),
    (9, 33, 50, ("reflect", "free", "periodic", "periodic")),
    (9, 96, 17, ("free", "reflect", "reflect", "free")),
    (5, 23, 130, ("periodic", "periodic", "free", "reflect")),
]


@pytest.mark.parametrize("order,nodex,nodey,bc", CASES)
def test_tma_staged_fp32_step_equals_converting_fp32_step(lib, order, nodex, nodey, bc):
    import torch

    pb, con, prim = _problem(order, nodex, nodey, bc, seed=order * 100 + nodey)
    nx, ny = pb.nx, pb.ny
    s = Solver2D(pb, FP32)
    s.set_state(con, prim)
    dts, states = [], []
    for _ in range(2):
        s.step(1e30)
        dts.append(s.sync()[1])
        st = s.get_state()
        states.append(st["convar"])
    s.close()

    dev = torch.device("cuda", 0)
    W = torch.from_numpy(_soa(con, nx, ny)).to(dev)
    ax = torch.zeros(nx * ny, dtype=torch.float64, device=dev)
    ay = torch.zeros(nx * ny, dtype=torch.float64, device=dev)
    p = pb.to_c()
    stream = torch.cuda.current_stream(dev)
    g = pb.ghost
    for k in range(2):
        rc = lib.hos2d_step_static(ctypes.byref(p), FP32, W.data_ptr(), ax.data_ptr(), ay.data_ptr(), dts[k],
                                   ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.hos_static_last_error()
        torch.cuda.synchronize(dev)
        got = W.cpu().numpy().T.reshape(nx, ny, 4)
        ref = states[k]
        scale = np.abs(ref[g:-g, g:-g]).max()
        err = np.abs(got - ref)[g:-g, g:-g].max() / scale
        assert err <= TOL, (k, err)
