"""CPU tests of the C ABI boundary: the library loads without a GPU, exports every
function include/hos_gb300.h declares, the ctypes struct matches the C struct layout, and
calls fail with a status code (no crash, no CPU fallback) when no GPU is present."""
import ctypes

import numpy as np
import re
import subprocess
import textwrap
from pathlib import Path

import pytest

from hos_gb300 import cases
from hos_gb300.params import GAUSS_POINTS, Params2D, Problem2D
from hos_gb300 import solver as hs

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "hos_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^(?:int|void\*|const char\*|void)\s+\*?(hos\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from hos_gb300 import build as hb
    hb.build()  # incremental: recompiles only when a source is newer than the library
    return ctypes.CDLL(str(hs.library_path()))


def test_header_declares_the_step_api():
    names = declared_functions()
    for n in ("hos2d_create", "hos2d_destroy", "hos2d_set_state", "hos2d_get_state", "hos2d_begin_step",
              "hos2d_boundary", "hos2d_stage", "hos2d_step", "hos2d_advance", "hos2d_sync", "hos_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_params_struct_layout_matches_c(tmp_path):
    fields = [f[0] for f in Params2D._fields_]
    src = "#include <stdio.h>\n#include <stddef.h>\n#include \"hos_gb300.h\"\nint main(void){\n"
    src += 'printf("%zu\\n", sizeof(hos_params2d));\n'
    for f in fields:
        src += f'printf("%zu\\n", offsetof(hos_params2d, {f}));\n'
    src += "return 0;}\n"
    c = tmp_path / "layout.c"
    c.write_text(src)
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(c), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(Params2D)
    for f, off in zip(fields, out[1:]):
        assert getattr(Params2D, f).offset == off, f


@pytest.mark.parametrize("order", [5, 7, 9])
def test_problem_to_c(order):
    pb = Problem2D(nodex=64, nodey=48, order=order, bc=("periodic", "periodic", "reflect", "inflow"),
                   bc_prim=((0,) * 4, (0,) * 4, (0,) * 4, (1.0, 0.5, 0.0, 1.0)))
    p = pb.to_c()
    assert (p.nodex, p.nodey, p.order, p.gausspoint) == (64, 48, order, GAUSS_POINTS[order])
    assert list(p.bc) == [1, 1, 2, 3]
    assert p.bc_prim[3][1] == 0.5
    assert pb.nx == 74 and pb.ny == 58


def test_cases_shapes_and_positivity():
    for pb, con, prim in (cases.riemann2d(32, order=7), cases.isentropic_vortex(20), cases.sinwave2d(12)):
        assert con.shape == (pb.nx, pb.ny, 4) and prim.shape == con.shape
        assert (prim[..., 0] > 0).all() and (prim[..., 3] > 0).all()


def _no_gpu():
    try:
        import torch
        return not torch.cuda.is_available()
    except Exception:
        return True


@pytest.mark.skipif(not _no_gpu(), reason="checks the no-GPU error path")
def test_create_without_gpu_fails_loudly():
    pb, _, _ = cases.riemann2d(16, order=5)
    with pytest.raises(hs.HosError) as ei:
        hs.Solver2D(pb)
    assert "hos error 3" in str(ei.value)


def test_bad_config_rejected_before_touching_cuda(lib):
    pb = Problem2D(nodex=16, nodey=16, order=5)
    p = pb.to_c()
    p.gausspoint = 3  # WENO5 writes two Gauss points only
    h = ctypes.c_void_p()
    lib.hos2d_create.argtypes = [ctypes.POINTER(Params2D), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    assert lib.hos2d_create(ctypes.byref(p), 0, ctypes.byref(h)) == hs.HOS_E_CONFIG
    p.gausspoint = 2
    p.use_df = 0
    p.wenotype = 3  # HOS_WENO_Z, HOS_WENO_JS, HOS_WENO_LINEAR only
    assert lib.hos2d_create(ctypes.byref(p), 0, ctypes.byref(h)) == hs.HOS_E_CONFIG
    # the non-DF scheme (the drivers' default slots) exists for WENO5 only
    p7 = Problem2D(nodex=16, nodey=16, order=7, use_df=False).to_c()
    assert lib.hos2d_create(ctypes.byref(p7), 0, ctypes.byref(h)) == hs.HOS_E_CONFIG


def test_batch_sweep_is_seeded_and_in_range():
    from hos_gb300 import cases

    a = cases.batch_sweep(count=8, seed=5)
    b = cases.batch_sweep(count=8, seed=5)
    assert [x[4] for x in a] == [x[4] for x in b]
    for k, (pb, con, prim, tstop, label) in enumerate(a):
        assert 128 <= pb.nodex <= 768 and pb.nodex % 4 == 0
        assert pb.nodey == pb.nodex // (2 if k % 2 == 0 else 4)
        assert abs(pb.dx - pb.dy) < 1e-15 and tstop > 0
        assert con.shape == (pb.nx, pb.ny, 4) and np.isfinite(con).all() and (con[..., 0] > 0).all()
