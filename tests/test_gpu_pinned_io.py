"""Host-facing transfers with pinned host buffers.  hos2d_set_state reads a pinned buffer over
the host link from its upload kernel, and hos2d_get_state writes one from its transposition
kernel; pageable buffers go through a device staging copy.  Both routes give the same state,
primitives, time and time step, bit for bit, and a pinned buffer that starts inside its
allocation (an offset view) works the same way."""
import ctypes

import numpy as np
import pytest

from hos_gb300 import cases
from hos_gb300.solver import FP32, FP64, Solver2D

pytestmark = pytest.mark.gpu

_DP = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build()


def _run(pb, con, prim, precision, pinned, offset=0):
    import torch
    n = con.size
    if pinned:
        # one pinned allocation per buffer, the solver's view starting `offset` doubles in
        buf_in = torch.zeros(n + offset, dtype=torch.float64).pin_memory()
        buf_in[offset:] = torch.from_numpy(np.ascontiguousarray(con.reshape(-1)))
        buf_c = torch.zeros(n + offset, dtype=torch.float64).pin_memory()
        buf_p = torch.zeros(n + offset, dtype=torch.float64).pin_memory()
        ptr = lambda t: ctypes.cast(t.data_ptr() + 8 * offset, _DP)
        src, dst_c, dst_p = ptr(buf_in), ptr(buf_c), ptr(buf_p)
    else:
        c = np.ascontiguousarray(con.reshape(-1))
        out_c, out_p = np.zeros(n), np.zeros(n)
        src, dst_c, dst_p = c.ctypes.data_as(_DP), out_c.ctypes.data_as(_DP), out_p.ctypes.data_as(_DP)
    s = Solver2D(pb, precision)
    try:
        assert s._lib.hos2d_set_state(s._h, src, None) == 0
        s.advance(3, 1e30)
        t, dt = s.sync()
        assert s._lib.hos2d_get_state(s._h, dst_c, dst_p, None, None) == 0
    finally:
        s.close()
    if pinned:
        out_c = buf_c[offset:].numpy().copy()
        out_p = buf_p[offset:].numpy().copy()
        assert not buf_c[:offset].any() and not buf_p[:offset].any()   # nothing written before the view
    return out_c, out_p, t, dt


@pytest.mark.parametrize("precision", [FP64, FP32], ids=["fp64", "fp32"])
def test_pinned_and_pageable_transfers_agree(precision):
    pb, con, prim = cases.riemann2d(64, order=5)
    a = _run(pb, con, prim, precision, pinned=False)
    b = _run(pb, con, prim, precision, pinned=True)
    c = _run(pb, con, prim, precision, pinned=True, offset=3)   # 8-byte aligned view
    for other in (b, c):
        assert np.array_equal(a[0], other[0]) and np.array_equal(a[1], other[1])
        assert a[2:] == other[2:]
    assert a[2] > 0 and a[3] > 0 and np.isfinite(a[0]).all()
