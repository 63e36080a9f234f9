"""The device-side waits of the FP32 solvers (TMA tile loads, the gate's tensor-core MMAs)
are bounded: a wait that runs out reports HOS_E_TIMEOUT instead of hanging the GPU.  The
self-test waits on a barrier nothing completes; the wait gives up within seconds and the CUDA
context stays usable: a solver created afterwards steps normally."""
import ctypes
import time

import pytest

from hos_gb300 import cases
from hos_gb300.solver import FP32, Solver2D, load

pytestmark = pytest.mark.gpu
HOS_E_TIMEOUT = 6


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build()


def test_bounded_wait_gives_up_and_reports():
    lib = load()
    lib.hos_last_error.restype = ctypes.c_char_p
    t0 = time.perf_counter()
    rc = lib.hos_wait_limit_selftest()
    took = time.perf_counter() - t0
    assert rc == HOS_E_TIMEOUT, (rc, lib.hos_last_error())
    assert took < 60.0
    pb, con, prim = cases.riemann2d(32, order=5)
    s = Solver2D(pb, FP32)
    s.set_state(con, prim)
    s.advance(2, 1e30)
    t, dt = s.sync()
    s.close()
    assert t > 0 and dt > 0
