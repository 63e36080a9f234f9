"""Build and run the reference-API drivers of tests/refapi (test infrastructure).

``driver2d.cpp`` / ``driver1d.cpp`` are problem drivers written against the reference's own
C++ function-level API.  ``build_driver`` links one against libhos_ref.so (the GPU path);
oracle/Makefile's ``refdrivers`` target links the same source against the reference's own
objects (only where the reference checkout exists), and tests/golden/make_golden.py stores
those reference runs as fixtures.
"""
from __future__ import annotations

import subprocess
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "high-order-solver_gb300" / "hos_gb300"
DRIVER_DIR = Path(__file__).resolve().parent / "refapi"
BC_NAMES = {0: "free", 1: "periodic", 2: "reflect", 3: "inflow", 6: "noslip"}


def build_driver(name: str, out_dir: Path) -> Path:
    """Compile tests/refapi/<name>.cpp against include/hos_ref_api.h and libhos_ref.so."""
    exe = Path(out_dir) / name
    cmd = ["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(DRIVER_DIR / f"{name}.cpp"), "-o", str(exe),
           f"-L{PKG}", "-lhos_ref", "-lhos_gb300", f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stderr}")
    return exe


def config2d(pb, steps: int, tstop: float = 1e30, precision: int = 0, mirror: int = 1) -> str:
    bc = [b if isinstance(b, str) else BC_NAMES[b] for b in pb.bc]
    bc = ["reflect" if b == "reflective" else "free" if b == "outflow" else b for b in bc]
    lines = [f"nodex {pb.nodex}", f"nodey {pb.nodey}", f"ghost {pb.ghost}", f"order {pb.order}",
             f"characteristic {int(pb.characteristic)}", f"K {pb.K}", f"gamma {pb.gamma!r}",
             f"c1 {pb.c1_euler!r}", f"c2 {pb.c2_euler!r}", f"cfl {pb.cfl!r}", f"left {pb.left!r}",
             f"right {pb.right!r}", f"down {pb.down!r}", f"up {pb.up!r}", "bc " + " ".join(bc),
             f"steps {steps}", f"tstop {tstop!r}", f"precision {precision}", f"mirror {mirror}"]
    if not getattr(pb, "use_df", True):
        lines += ["df 0", "wenotype " + {"wenoz": "z", "wenojs": "js", "linear": "linear"}[pb.wenotype]]
    if getattr(pb, "first_order_steps", 0):
        lines.append(f"first_order_steps {pb.first_order_steps}")
    if getattr(pb, "source", False):
        lines.append("source 1")
    if getattr(pb, "tau_type", 0):
        lines += [f"tau_type {pb.tau_type}", f"mu {pb.mu!r}", f"nu {pb.nu!r}",
                  f"prandtl_fix {int(pb.prandtl_fix)}", f"pr {pb.prandtl!r}"]
    bp = []
    for s in range(4):
        if bc[s] in ("inflow", "noslip"):
            bp += [str(s)] + [repr(float(v)) for v in pb.bc_prim[s]]
    if bp:
        lines.append("bcprim " + " ".join(bp))
    return "\n".join(lines) + "\n"


def config1d(pb, steps: int, df: str, tstop: float = 1e30, precision: int = 0, mirror: int = 1) -> str:
    bc = [b if isinstance(b, str) else BC_NAMES[b] for b in pb.bc]
    lines = [f"nodex {pb.nodex}", f"ghost {pb.ghost}", f"order {pb.order}",
             f"characteristic {int(pb.characteristic)}", f"df {df}", f"K {pb.K}", f"gamma {pb.gamma!r}",
             f"c1 {pb.c1_euler!r}", f"c2 {pb.c2_euler!r}", f"cfl {pb.cfl!r}", f"left {pb.left!r}",
             f"right {pb.right!r}", "bc " + " ".join(bc), f"steps {steps}", f"tstop {tstop!r}",
             f"precision {precision}", f"mirror {mirror}"]
    return "\n".join(lines) + "\n"


def run2d(exe: Path, pb, con, prim, config: str) -> dict:
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        (d / "c.txt").write_text(config)
        np.concatenate([np.ascontiguousarray(con, np.float64).ravel(),
                        np.ascontiguousarray(prim, np.float64).ravel()]).tofile(d / "in.bin")
        r = subprocess.run([str(exe), str(d / "c.txt"), str(d / "in.bin"), str(d / "out.bin")],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver failed ({r.returncode}): {r.stderr.strip()}")
        out = np.fromfile(d / "out.bin")
    n = pb.nx * pb.ny
    k = 0
    res = {}
    for key, size, shape in (("convar", 4 * n, (pb.nx, pb.ny, 4)), ("primvar", 4 * n, (pb.nx, pb.ny, 4)),
                             ("alpha_x", n, (pb.nx, pb.ny)), ("alpha_y", n, (pb.nx, pb.ny))):
        res[key] = out[k:k + size].reshape(shape)
        k += size
    res["t"], res["steps"], res["dts"] = out[k], int(out[k + 1]), out[k + 2:]
    return res


def run1d(exe: Path, pb, con, config: str) -> dict:
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        (d / "c.txt").write_text(config)
        np.ascontiguousarray(con, np.float64).ravel().tofile(d / "in.bin")
        r = subprocess.run([str(exe), str(d / "c.txt"), str(d / "in.bin"), str(d / "out.bin")],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver failed ({r.returncode}): {r.stderr.strip()}")
        out = np.fromfile(d / "out.bin")
    n = pb.nx
    return {"convar": out[:3 * n].reshape(n, 3), "alpha": out[3 * n:4 * n], "t": out[4 * n],
            "steps": int(out[4 * n + 1]), "dts": out[4 * n + 2:]}


def refapi_cases_2d():
    """(name, case, steps) of the 2D reference-API fixtures.  All grids have nodex <= nodey:
    the reference's Update_alpha runs its j loop to nodex (src/reconstruction.cpp:1528), which
    for nodex > nodey writes past the rows it owns, so such grids have no reference result."""
    from hos_gb300 import cases
    inflow = cases.riemann2d(20, order=5)
    inflow[0].bc = ("inflow", "free", "reflect", "reflect")
    inflow[0].bc_prim = ((1.2, 0.8, 0.1, 1.0), (0.0,) * 4, (0.0,) * 4, (0.0,) * 4)
    fo = cases.random_riemann2d(20, seed=9, order=9)
    fo[0].bc = ("reflect",) * 4
    fo[0].first_order_steps = 1     # the drivers' first-order step 0 (e.g. doubleMach)
    # the viscous_sod_shock_problem loop (src/2Dproblem.cpp:1095-1283): NS collision time,
    # no-slip adiabatic left / right / bottom, reflecting top, first-order step 0, WENO5-AO-DF
    ns = cases.random_riemann2d(20, seed=5, order=5)
    ns[0].bc = ("noslip", "noslip", "noslip", "reflect")
    ns[0].tau_type, ns[0].mu, ns[0].c2_euler = 1, 1e-3, 9.0
    ns[0].first_order_steps = 1
    # the RT_instability loop (src/2Dproblem.cpp:699-763): RT_boundary, Update_with_source
    rt = cases.rt2d(12)
    rt[0].source, rt[0].first_order_steps = True, 1
    # PlanarShock with the reference's default is_using_df_factor = false: the slots stay
    # WENO5_AO_normal / WENO5_AO_tangent (non-DF WENO5-AO, Z-type weights), no Update_alpha
    nodf = cases.riemann2d(20, order=5)
    nodf[0].use_df = False
    nodf_js = cases.random_riemann2d(20, seed=21, order=5)
    nodf_js[0].use_df, nodf_js[0].wenotype, nodf_js[0].bc = False, "wenojs", ("periodic",) * 4
    return [("refapi_riemann_w7_24", cases.riemann2d(24, order=7), 5),
            ("refapi_rt_w5_12", rt, 4),
            ("refapi_fo_w9_reflect_20", fo, 4),
            ("refapi_ns_noslip_w5_20", ns, 4),
            ("refapi_inflow_reflect_w5_20", inflow, 5),
            ("refapi_vortex_w9_20", cases.isentropic_vortex(20, order=9), 3),
            ("refapi_nodf_riemann_w5_20", nodf, 5),
            ("refapi_nodf_js_periodic_w5_20", nodf_js, 4)]
