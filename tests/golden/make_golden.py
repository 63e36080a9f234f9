"""Generate the golden vectors under tests/golden/ by running the COMPILED REFERENCE
(oracle/_ref/libhosref.so, built from the reference sources by oracle/Makefile) on small
seeded cases.  Run from the repository root where the reference checkout exists:

    python tests/golden/make_golden.py

Each case stores the initial conserved/primitive state, the reference state (convar,
alpha_x, alpha_y) after 1 and after 3 S2O4 steps, and the three time steps ("fo_" cases run
step 0 with First_order_normal / First_order_tangent, as the drivers do when
is_using_df_factor is set; "ns_" cases use the Navier-Stokes collision time, no-slip walls
and the Prandtl fix, also with a first-order step 0; "rt_" is the RT_instability loop with
Update_with_source; "nodf_" cases run the drivers' default non-DF WENO5-AO slots with
is_using_df_factor = false and the Z-type or Jiang-Shu weights).

tests/golden/refapi/ holds runs of the reference-API drivers (tests/refapi/driver2d.cpp,
driver1d.cpp) linked against the reference's own objects (oracle/Makefile, refdrivers): the
input state, the Fluid arrays after the run and every dt; the 1D entry is the complete Sod
run of the benchmark definition (1000 cells to t = 0.2).  The 2D
accuracy entries store the reference's own known-answer test (sinwave_2d,
src/2Dproblem.cpp:1347-1603): L1/L2/Linf density errors at t = 2 on 10^2 and 20^2 meshes.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "high-order-solver_gb300"))
sys.path.insert(0, str(ROOT / "tests"))

from hos_gb300 import cases  # noqa: E402
from oracle_lib import CpuStep, CpuStep1D  # noqa: E402

OUT = Path(__file__).resolve().parent


def step_cases():
    yield "riemann_w5_char_24", cases.riemann2d(24, order=5)
    yield "riemann_w7_char_24", cases.riemann2d(24, order=7)
    yield "riemann_w9_char_24", cases.riemann2d(24, order=9)
    yield "riemann_w7_cons_24", cases.riemann2d(24, order=7, characteristic=False)
    yield "rriemann_w7_s11_20", cases.random_riemann2d(20, seed=11, order=7)
    yield "vortex_w5_char_20", cases.isentropic_vortex(20, order=5)
    yield "sinwave_w9_cons_16", cases.sinwave2d(16, order=9)
    from test_oracle_cpu import _problem
    for name in ("tmarch_s1o1_gks_w5_24", "tmarch_s1o2_gks_w5_24", "tmarch_rk2_gks_w7_24",
                 "tmarch_rk3_lf_w5_24", "tmarch_rk4_gks_w9_24", "tmarch_s2o4_lf_w7_24"):
        yield name, _problem(name)
    for name in ("fo_w5_free_24", "fo_w7_periodic_24", "fo_w9_reflect_24",
                 "ns_w5_noslip_24", "ns_w7_wall_24", "ns_w7_cap_24", "ns_w9_nu_24", "rt_w5_12",
                 "nodf_w5_z_free_24", "nodf_w5_js_reflect_24", "nodf_w5_z_cons_20",
                 "lfns_w5_mu_24", "lfns_w7_nu_24", "lfns_w9_walls_24"):
        yield name, _problem(name)


def sinwave_errors(n, tstop=2.0):
    pb, con, prim = cases.sinwave2d(n, order=9)
    r = CpuStep("ref").init(pb)
    r.set_state(con, prim)
    while r.t < tstop:
        r.step(tstop)
    rho = r.state()["convar"][..., 0]
    g = pb.ghost
    exact = prim[..., 0]  # exact cell averages are periodic in t = 2 (one period)
    e = np.abs(rho - exact)[g:-g, g:-g]
    return np.array([e.mean(), np.sqrt((e * e).mean()), e.max()])


def sinwave1d_errors(n, tstop=2.0):
    """1D accuracy driver (accuracy_sinwave_1d, src/1Dproblem.cpp:519-735): L1/L2/Linf of rho."""
    pb, con = cases.sinwave1d(n)
    r = CpuStep1D("ref").init(pb)
    r.set_state(con)
    r.run(tstop)
    g = pb.ghost
    e = np.abs(r.state()["convar"][g:-g, 0] - con[g:-g, 0])
    return np.array([e.mean(), np.sqrt((e * e).mean()), e.max()])


def one_d():
    """Config 1 of the benchmark definition: 1D Sod, 1000 cells, run to t = 0.2 (plus small
    variants), and the reference's 1D known-answer test at 10/20/40/80 cells."""
    for name, (pb, con), tstop in (("sod1d_w5_char_1000", cases.sod1d(1000), 0.2),
                                   ("sod1d_w7_char_200", cases.sod1d(200, order=7), 0.2),
                                   ("sod1d_w9_char_200", cases.sod1d(200, order=9), 0.2),
                                   ("sod1d_w5_cons_200", cases.sod1d(200, characteristic=False), 0.2)):
        r = CpuStep1D("ref").init(pb)
        r.set_state(con)
        dts = [r.step(tstop) for _ in range(3)]
        s3 = r.state()
        n = 3 + r.run(tstop)
        s = r.state()
        np.savez_compressed(OUT / f"{name}.npz", convar0=con, convar3=s3["convar"], alpha3=s3["alpha"],
                            dts=np.array(dts), convar_end=s["convar"], alpha_end=s["alpha"],
                            t_end=np.array(r.t), steps=np.array(r.nstep))
        print(name, r.nstep, r.t)
    errs = {f"n{n}": sinwave1d_errors(n) for n in (10, 20, 40, 80)}
    np.savez_compressed(OUT / "sinwave1d_w5_accuracy.npz", **errs)
    print(errs)


def refapi():
    import subprocess

    from refapi_lib import config1d, config2d, refapi_cases_2d, run1d, run2d

    subprocess.run(["make", "-C", str(ROOT / "oracle"), "refdrivers"], check=True, capture_output=True)
    d2 = ROOT / "oracle" / "_ref" / "driver2d"
    d1 = ROOT / "oracle" / "_ref" / "driver1d"
    out = OUT / "refapi"
    out.mkdir(exist_ok=True)
    for name, (pb, con, prim), steps in refapi_cases_2d():
        r = run2d(d2, pb, con, prim, config2d(pb, steps))
        np.savez_compressed(out / f"{name}.npz", convar0=con, primvar0=prim, steps_asked=steps,
                            **{k: np.asarray(v) for k, v in r.items()})
        print(name, r["steps"], r["dts"])
    pb, con = cases.sod1d(1000)
    r = run1d(d1, pb, con, config1d(pb, 100000, "switch", tstop=0.2))
    np.savez_compressed(out / "refapi_sod1d_1000.npz", convar0=con, **{k: np.asarray(v) for k, v in r.items()})
    print("refapi_sod1d_1000", r["steps"], r["t"])


def three_d():
    """The reference's own 3D functions run by oracle/ref_driver3d.cpp (which allocates the
    Gauss-point arrays the reference leaves unallocated): initial state, every step's state
    and dt of the cases of test_oracle3d_cpu.ref3d_problem."""
    from oracle_lib import CpuStep3D
    from test_oracle3d_cpu import REF3D_CASES, ref3d_problem
    for name in REF3D_CASES:
        pb, W, steps = ref3d_problem(name)
        r = CpuStep3D("ref").init(pb)
        r.set_state(W)
        out = {"convar0": W}
        dts = []
        for k in range(steps):
            dts.append(r.step())
            out[f"convar{k + 1}"] = r.state()["convar"]
        np.savez_compressed(OUT / f"{name}.npz", dts=np.array(dts), **out)
        print(name, dts)


def main(only=None):
    if only == "refapi":
        refapi()
        return
    if only == "ref3d":
        three_d()
        return
    for name, (pb, con, prim) in step_cases():
        if only and not name.startswith(only):
            continue
        from test_oracle_cpu import first_order_steps, with_source
        r = CpuStep("ref").init(pb)
        r.set_state(con, prim)
        r.fn("set_source")(1 if with_source(name) else 0)
        fo = first_order_steps(name)
        dts = []
        for k in range(3):
            r.fn("set_first_order")(1 if k < fo else 0)
            dts.append(r.step())
            if k == 0:
                s1 = r.state()
        s3 = r.state()
        np.savez_compressed(OUT / f"{name}.npz", convar0=con, primvar0=prim,
                            convar1=s1["convar"], alpha_x1=s1["alpha_x"], alpha_y1=s1["alpha_y"],
                            convar3=s3["convar"], alpha_x3=s3["alpha_x"], alpha_y3=s3["alpha_y"],
                            dts=np.array(dts))
        print(name, dts)
    if only:
        return
    errs = {f"n{n}": sinwave_errors(n) for n in (10, 20)}
    np.savez_compressed(OUT / "sinwave_w9_accuracy.npz", **errs)
    print(errs)
    one_d()
    refapi()
    three_d()


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
