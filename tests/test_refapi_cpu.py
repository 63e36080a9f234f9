"""The reference's C++ function-level API (libhos_ref.so, include/hos_ref_api.h) on the CPU:
its class layouts equal the reference's, a driver compiled against the reference's own headers
links against it, and the reference-API fixtures are pinned by the oracle.  Tests that need the
reference checkout skip without it."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
REF_INCLUDE = Path(os.environ.get("HOS_REFERENCE", "/root/reference")) / "include"
PKG = ROOT / "high-order-solver_gb300" / "hos_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden" / "refapi"

LAYOUT_SRC = r"""
#include <cstddef>
#include <cstdio>
#define P(c, m) std::printf(#c "." #m " %zu\n", offsetof(c, m));
#define S(c) std::printf(#c " %zu\n", sizeof(c));
int main() {
    S(Block1d) S(Fluid1d) S(Point1d) S(Flux1d) S(Interface1d)
    S(Block2d) S(Point2d) S(Fluid2d) S(Flux2d) S(Recon2d) S(Interface2d) S(Flux2d_gauss)
    P(Block1d, timecoefficient) P(Block1d, t) P(Block1d, CFL) P(Block1d, dt) P(Block1d, step)
    P(Fluid1d, convar) P(Fluid1d, convar_old) P(Fluid1d, alpha) P(Interface1d, flux)
    P(Block2d, nx) P(Block2d, ny) P(Block2d, dx) P(Block2d, left) P(Block2d, stages)
    P(Block2d, timecoefficient) P(Block2d, t) P(Block2d, CFL) P(Block2d, dt) P(Block2d, step)
    P(Block2d, T) P(Block2d, outputperstep)
    P(Fluid2d, primvar) P(Fluid2d, convar) P(Fluid2d, convar_old) P(Fluid2d, res)
    P(Fluid2d, node) P(Fluid2d, alpha_x) P(Fluid2d, alpha_y) P(Fluid2d, direction) P(Fluid2d, Sw1)
    P(Flux2d, f) P(Flux2d, derf) P(Flux2d, normal) P(Recon2d, center) P(Recon2d, normal)
    P(Interface2d, gauss) P(Interface2d, length) P(Point2d, der1y) P(Point2d, is_reduce_order)
    std::printf("Euler %d NS %d characteristic %d wenoz %d gks2nd_2d %d all_collisionn %d\n",
                (int)Euler, (int)NS, (int)characteristic, (int)wenoz, (int)gks2nd_2d, (int)all_collisionn);
    return 0;
}
"""


def _layout(tmp: Path, include_line: str, flags: list) -> str:
    src = tmp / "layout.cpp"
    src.write_text(include_line + "\n" + LAYOUT_SRC)
    exe = tmp / "layout"
    subprocess.run(["g++", "-std=c++17", "-w", "-Wno-invalid-offsetof", *flags, str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


@pytest.mark.skipif(not REF_INCLUDE.exists(), reason="reference checkout absent")
def test_class_layouts_equal_the_reference(tmp_path):
    ours = _layout(tmp_path, '#include "hos_ref_types.h"', [f"-I{ROOT / 'include'}"])
    ref = _layout(tmp_path, '#include "fluid_mesh.h"\n#include "reconstruction.h"', [f"-I{REF_INCLUDE}"])
    assert ours == ref


def _lib_built():
    import __graft_entry__ as ge
    ge.build()
    return PKG / "libhos_ref.so"


@pytest.mark.skipif(not REF_INCLUDE.exists(), reason="reference checkout absent")
@pytest.mark.parametrize("driver", ["driver2d", "driver1d"])
def test_driver_compiled_with_reference_headers_links_against_libhos_ref(tmp_path, driver):
    """A driver compiled against the reference's own headers resolves every reference-API
    symbol it uses (mangled C++ names) from libhos_ref.so: a link-level drop-in."""
    _lib_built()
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-w", "-DHOS_DRIVER_WITH_REFERENCE", f"-I{REF_INCLUDE}",
                        str(ROOT / "tests" / "refapi" / f"{driver}.cpp"), "-o", str(tmp_path / driver),
                        f"-L{PKG}", "-lhos_ref", "-lhos_gb300", f"-Wl,-rpath,{PKG}", "-Wl,--no-undefined"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_driver_reports_a_missing_gpu_as_the_reference_api_error(tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the GPU tests run this driver")
    _lib_built()
    from hos_gb300 import cases
    from refapi_lib import build_driver, config2d, run2d

    exe = build_driver("driver2d", tmp_path)
    pb, con, prim = cases.riemann2d(16, order=5)
    with pytest.raises(RuntimeError, match=r"driver failed \(3\): hos_ref_error 3"):
        run2d(exe, pb, con, prim, config2d(pb, 1))


@pytest.mark.parametrize("name", ["refapi_riemann_w7_24", "refapi_rt_w5_12", "refapi_fo_w9_reflect_20",
                                  "refapi_ns_noslip_w5_20", "refapi_inflow_reflect_w5_20", "refapi_vortex_w9_20",
                                  "refapi_nodf_riemann_w5_20", "refapi_nodf_js_periodic_w5_20"])
def test_refapi_fixture_equals_the_oracle(name):
    """The reference run of the same driver loop equals the oracle bit for bit."""
    from oracle_lib import CpuStep
    from refapi_lib import refapi_cases_2d

    (pb, _, _), steps = next((c, s) for n, c, s in refapi_cases_2d() if n == name)
    gold = np.load(GOLDEN / f"{name}.npz")
    o = CpuStep("oracle").init(pb)
    o.set_state(gold["convar0"], gold["primvar0"])
    o.fn("set_source")(1 if getattr(pb, "source", False) else 0)
    fo = getattr(pb, "first_order_steps", 0)
    dts = []
    for k in range(steps):
        o.fn("set_first_order")(1 if k < fo else 0)
        dts.append(o.step())
    st = o.state()
    assert np.array_equal(np.array(dts), gold["dts"])
    assert np.array_equal(st["convar"], gold["convar"])
    assert np.array_equal(st["alpha_x"], gold["alpha_x"]) and np.array_equal(st["alpha_y"], gold["alpha_y"])


def test_refapi_sod_fixture_equals_the_oracle():
    from hos_gb300 import cases
    from oracle_lib import CpuStep1D

    gold = np.load(GOLDEN / "refapi_sod1d_1000.npz")
    pb, _ = cases.sod1d(1000)
    o = CpuStep1D("oracle").init(pb)
    o.set_state(gold["convar0"])
    o.run(0.2)
    st = o.state()
    assert np.array_equal(st["convar"], gold["convar"])


@pytest.mark.skipif(not REF_INCLUDE.exists(), reason="reference checkout absent")
def test_output_writers_are_byte_identical_to_the_reference(tmp_path):
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "refdrivers"], check=True, capture_output=True)
    _lib_built()
    ours = tmp_path / "outputs_ours"
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "refapi" / "outputs.cpp"),
                    "-o", str(ours), f"-L{PKG}", "-lhos_ref", "-lhos_gb300", f"-Wl,-rpath,{PKG}"], check=True)
    outs = {}
    for name, exe in (("ref", ROOT / "oracle" / "_ref" / "outputs"), ("ours", ours)):
        run = tmp_path / name / "run"
        (tmp_path / name / "data").mkdir(parents=True)
        run.mkdir()
        subprocess.run([str(exe)], cwd=run, check=True, capture_output=True)
        outs[name] = {p.name: p.read_bytes() for p in (tmp_path / name / "data").iterdir()}
    assert set(outs["ref"]) == {"R.txt", "R-42.txt", "error.txt"}
    assert outs["ours"] == outs["ref"]
