"""ctypes binding of the C ABI in include/hos_gb300.h.

``Solver2D`` mirrors the reference's function-level stage API for this path
(src/2Dproblem.cpp:128-157 in XJTUZhangHong/high-order-solver):

    reference                                  this binding
    CopyFluid_new_to_old + Get_CFL             Solver2D.get_cfl / begin_step
    left/right/down/upboundary(...)            Solver2D.boundary
    Convar_to_Primvar ... Update_alpha          Solver2D.stage(i)
    loop body of the driver                    Solver2D.step
    (blow-up exit(0) in Convar_to_Primvar)     HosBlowUp raised by sync()

State arrays use the reference's cell order (i * ny + j, 4 doubles per cell).  There is no
CPU fallback: without the CUDA library every call raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from .params import Params1D, Params2D, Params3D, Problem1D, Problem2D, Problem3D

HOS_OK, HOS_E_BLOWUP, HOS_E_CONFIG, HOS_E_CUDA, HOS_E_ARG, HOS_E_NOMEM = range(6)
FP64, FP32 = 0, 1

_LIB = None
_DP = ctypes.POINTER(ctypes.c_double)


class HosError(RuntimeError):
    pass


class HosBlowUp(HosError):
    """Negative density or pressure (or NaN) where the reference calls exit(0)
    (Convar_to_Primvar, src/basic_function.cpp:752-773)."""


def library_path() -> Path:
    return Path(__file__).resolve().parent / "libhos_gb300.so"


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the CUDA library; raises if it has not been built (no fallback path)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = Path(path) if path else library_path()
    if not p.exists():
        raise HosError(f"{p} is missing: build it with __graft_entry__.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(str(p))
    vp = ctypes.c_void_p
    lib.hos2d_create.argtypes = [ctypes.POINTER(Params2D), ctypes.c_int, ctypes.POINTER(vp)]
    lib.hos2d_destroy.argtypes = [vp]
    lib.hos2d_dims.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.hos2d_set_state.argtypes = [vp, _DP, _DP]
    lib.hos2d_set_state_device.argtypes = [vp, vp, vp]
    lib.hos2d_get_state.argtypes = [vp, _DP, _DP, _DP, _DP]
    lib.hos2d_set_alpha.argtypes = [vp, _DP, _DP]
    lib.hos2d_begin_step.argtypes = [vp, ctypes.c_double]
    lib.hos2d_boundary.argtypes = [vp]
    lib.hos2d_stage.argtypes = [vp, ctypes.c_int]
    lib.hos2d_step.argtypes = [vp, ctypes.c_double]
    lib.hos2d_advance.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    lib.hos2d_sync.argtypes = [vp, _DP, _DP]
    lib.hos2d_launches_per_step.argtypes = [vp]
    lib.hos2d_profile_step.argtypes = [vp, ctypes.c_double, _DP]
    lib.hos2d_set_reconstruction.argtypes = [vp, ctypes.c_int]
    lib.hos2d_set_source.argtypes = [vp, ctypes.c_int]
    lib.hos2d_stream.argtypes = [vp]
    lib.hos2d_stream.restype = vp
    lib.hos_last_error.restype = ctypes.c_char_p
    lib.hos1d_create.argtypes = [ctypes.POINTER(Params1D), ctypes.c_int, ctypes.POINTER(vp)]
    lib.hos1d_destroy.argtypes = [vp]
    lib.hos1d_set_state.argtypes = [vp, _DP]
    lib.hos1d_get_state.argtypes = [vp, _DP, _DP]
    lib.hos1d_step.argtypes = [vp, ctypes.c_double]
    lib.hos1d_run.argtypes = [vp, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.hos1d_sync.argtypes = [vp, _DP, _DP]
    lib.hos1d_last_error.restype = ctypes.c_char_p
    lib.hos_batch2d_create.argtypes = [ctypes.POINTER(Params2D), _DP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
    lib.hos_batch2d_destroy.argtypes = [vp]
    lib.hos_batch2d_set_state.argtypes = [vp, ctypes.c_int, _DP, _DP]
    lib.hos_batch2d_get_state.argtypes = [vp, ctypes.c_int, _DP, _DP, _DP]
    lib.hos_batch2d_autotune.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _DP]
    lib.hos_batch2d_advance.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    lib.hos_batch2d_status.argtypes = [vp, ctypes.POINTER(ctypes.c_int), _DP, ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_int)]
    lib.hos_batch2d_cells.argtypes = [vp]
    lib.hos_batch2d_cells.restype = ctypes.c_longlong
    lib.hos_batch2d_stream.argtypes = [vp]
    lib.hos_batch2d_stream.restype = vp
    lib.hos_batch2d_last_error.restype = ctypes.c_char_p
    _FP = ctypes.POINTER(ctypes.c_float)
    _ULL = ctypes.POINTER(ctypes.c_ulonglong)
    lib.hos_gate_create.argtypes = [ctypes.c_ulonglong, ctypes.c_uint, ctypes.POINTER(vp)]
    lib.hos_gate_destroy.argtypes = [vp]
    lib.hos_gate_get_params.argtypes = [vp, _FP]
    lib.hos_gate_set_params.argtypes = [vp, _FP]
    lib.hos_gate_collect.argtypes = [vp, vp, ctypes.c_int]
    lib.hos_gate_sample_count.argtypes = [vp, _ULL]
    lib.hos_gate_get_samples.argtypes = [vp, _FP, ctypes.c_ulonglong]
    lib.hos_gate_set_samples.argtypes = [vp, _FP, ctypes.c_ulonglong]
    lib.hos_gate_clear_samples.argtypes = [vp]
    lib.hos_gate_gradient.argtypes = [vp, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_float, ctypes.c_float, _FP, _DP]
    lib.hos_gate_forward.argtypes = [vp, ctypes.c_ulonglong, ctypes.c_int, _FP]
    lib.hos_gate_train.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_uint, _DP]
    lib.hos_gate_last_error.restype = ctypes.c_char_p
    lib.hos2d_set_gate.argtypes = [vp, vp, ctypes.c_float, ctypes.c_int]
    lib.hos2d_set_gate_check.argtypes = [vp, ctypes.c_double]
    lib.hos_batch2d_set_gate.argtypes = [vp, vp, ctypes.c_float, ctypes.c_int]
    lib.hos_batch2d_set_reconstruction.argtypes = [vp, ctypes.c_int]
    lib.hos_batch2d_gate_stats.argtypes = [vp, _ULL, ctypes.c_int]
    lib.hos2d_gate_stats.argtypes = [vp, _ULL, ctypes.c_int]
    lib.hos2d_gate_audit_check.argtypes = [vp, _ULL]
    lib.hos3d_create.argtypes = [ctypes.POINTER(Params3D), ctypes.c_int, ctypes.POINTER(vp)]
    lib.hos3d_destroy.argtypes = [vp]
    lib.hos3d_set_state.argtypes = [vp, _DP, _DP]
    lib.hos3d_get_state.argtypes = [vp, _DP, _DP]
    lib.hos3d_step.argtypes = [vp, ctypes.c_double]
    lib.hos3d_advance.argtypes = [vp, ctypes.c_int, ctypes.c_double]
    lib.hos3d_sync.argtypes = [vp, _DP, _DP]
    lib.hos3d_begin_step.argtypes = [vp, ctypes.c_double]
    lib.hos3d_stage.argtypes = [vp, ctypes.c_int]
    lib.hos3d_set_time.argtypes = [vp, ctypes.c_double]
    lib.hos3d_stream.argtypes = [vp, ctypes.POINTER(vp)]
    lib.hos3d_profile_step.argtypes = [vp, ctypes.c_double, _FP, ctypes.c_int]
    lib.hos3d_set_gate.argtypes = [vp, vp, ctypes.c_float, ctypes.c_int]
    lib.hos3d_gate_stats.argtypes = [vp, _ULL, ctypes.c_int]
    lib.hos_gate_collect3d.argtypes = [vp, vp, ctypes.c_int]
    lib.hos3d_last_error.restype = ctypes.c_char_p
    _LIB = lib
    return lib


def _check(code: int) -> None:
    if code == HOS_OK:
        return
    msg = load().hos_last_error().decode(errors="replace")
    if code == HOS_E_BLOWUP:
        raise HosBlowUp(msg)
    raise HosError(f"hos error {code}: {msg}")


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(_DP)


class Solver2D:
    """One 2D problem resident on the current CUDA device."""

    def __init__(self, problem: Problem2D, precision: int = FP64):
        self.problem = problem
        self.precision = precision
        self._lib = load()
        self._params = problem.to_c()
        h = ctypes.c_void_p()
        _check(self._lib.hos2d_create(ctypes.byref(self._params), precision, ctypes.byref(h)))
        self._h = h
        nx, ny = ctypes.c_int(), ctypes.c_int()
        _check(self._lib.hos2d_dims(h, ctypes.byref(nx), ctypes.byref(ny)))
        self.nx, self.ny = nx.value, ny.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hos2d_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    # -- state ---------------------------------------------------------------------------
    def set_state(self, convar: np.ndarray, primvar: np.ndarray | None = None) -> None:
        c = np.ascontiguousarray(convar, dtype=np.float64).reshape(-1)
        if c.size != self.nx * self.ny * 4:
            raise ValueError("convar must hold nx*ny*4 values")
        p = None if primvar is None else np.ascontiguousarray(primvar, dtype=np.float64).reshape(-1)
        _check(self._lib.hos2d_set_state(self._h, _ptr(c), _ptr(p)))

    def set_state_device(self, convar_soa_ptr: int, primvar_soa_ptr: int | None = None) -> None:
        _check(self._lib.hos2d_set_state_device(self._h, ctypes.c_void_p(convar_soa_ptr),
                                                 ctypes.c_void_p(primvar_soa_ptr or 0) if primvar_soa_ptr else None))

    def set_reconstruction(self, first_order: bool) -> None:
        """First_order_normal / _tangent (True) or the WENO-AO scheme (False) for the following
        stages: the reference drivers' step-0 switch (src/2Dproblem.cpp:733-745)."""
        _check(self._lib.hos2d_set_reconstruction(self._h, 1 if first_order else 0))

    def set_source(self, on: bool) -> None:
        """Update_with_source (gravity along +y, the RT_instability driver) as the stage update."""
        _check(self._lib.hos2d_set_source(self._h, 1 if on else 0))

    def set_alpha(self, alpha_x: np.ndarray, alpha_y: np.ndarray) -> None:
        ax = np.ascontiguousarray(alpha_x, dtype=np.float64).reshape(-1)
        ay = np.ascontiguousarray(alpha_y, dtype=np.float64).reshape(-1)
        if ax.size != self.nx * self.ny or ay.size != self.nx * self.ny:
            raise ValueError("alpha arrays must hold nx*ny values")
        _check(self._lib.hos2d_set_alpha(self._h, _ptr(ax), _ptr(ay)))

    def get_state(self, primvar: bool = False):
        n = self.nx * self.ny
        c = np.empty(4 * n)
        p = np.empty(4 * n) if primvar else None
        ax = np.empty(n)
        ay = np.empty(n)
        _check(self._lib.hos2d_get_state(self._h, _ptr(c), _ptr(p), _ptr(ax), _ptr(ay)))
        out = dict(convar=c.reshape(self.nx, self.ny, 4), alpha_x=ax.reshape(self.nx, self.ny),
                   alpha_y=ay.reshape(self.nx, self.ny))
        if primvar:
            out["primvar"] = p.reshape(self.nx, self.ny, 4)
        return out

    # -- the reference's stage-level API --------------------------------------------------
    def begin_step(self, tstop: float) -> None:
        _check(self._lib.hos2d_begin_step(self._h, tstop))

    def get_cfl(self, tstop: float) -> float:
        """CopyFluid_new_to_old + Get_CFL; returns this step's dt (synchronises)."""
        self.begin_step(tstop)
        return self.sync()[1]

    def boundary(self) -> None:
        _check(self._lib.hos2d_boundary(self._h))

    def stage(self, i: int) -> None:
        _check(self._lib.hos2d_stage(self._h, i))

    def step(self, tstop: float) -> None:
        _check(self._lib.hos2d_step(self._h, tstop))

    def advance(self, nsteps: int, tstop: float, graph: bool = True) -> None:
        _check(self._lib.hos2d_advance(self._h, nsteps, tstop, 1 if graph else 0))

    def sync(self) -> tuple[float, float]:
        t, dt = ctypes.c_double(), ctypes.c_double()
        _check(self._lib.hos2d_sync(self._h, ctypes.byref(t), ctypes.byref(dt)))
        return t.value, dt.value

    def profile_step(self, tstop: float = 1e30) -> dict:
        """One step with events between launches: device milliseconds per kernel."""
        ms = np.zeros(11)
        _check(self._lib.hos2d_profile_step(self._h, tstop, _ptr(ms)))
        names = ["begin_step"] + [f"{k}{st}" for st in (0, 1) for k in ("bc_fill", "gate", "face_x", "face_y", "update")]
        return dict(zip(names, ms.tolist()))

    @property
    def launches_per_step(self) -> int:
        return int(self._lib.hos2d_launches_per_step(self._h))

    @property
    def stream(self) -> int:
        return int(self._lib.hos2d_stream(self._h) or 0)

    def set_gate(self, gate: "Gate | None", threshold: float = 0.0, audit_log2: int = 6) -> None:
        """Attach a copy of a learned gate (FP32 solvers); None detaches it."""
        _check(self._lib.hos2d_set_gate(self._h, gate._h if gate is not None else None, threshold, audit_log2))

    def set_gate_reuse(self, reuse: bool) -> None:
        """Run the gate's network at the first stage of each step only and give the later stages
        its flags dilated by one cell along each flag's axis (hos2d_set_gate_reuse)."""
        _check(self._lib.hos2d_set_gate_reuse(self._h, 1 if reuse else 0))

    def set_gate_check(self, slack: float) -> None:
        """Widening of the linear path's a-posteriori range check (fraction of the range)."""
        _check(self._lib.hos2d_set_gate_check(self._h, slack))

    def gate_stats(self, reset: bool = False) -> dict:
        v = (ctypes.c_ulonglong * 8)()
        _check(self._lib.hos2d_gate_stats(self._h, v, 1 if reset else 0))
        keys = ("cells_x", "cells_y", "smooth_x", "smooth_y", "audited", "false_neg", "fallback", "unused")
        return dict(zip(keys, (int(x) for x in v)))

    def gate_audit_check(self) -> dict:
        """Linear reconstructions in cell-directions an audit found not smooth, and how many of
        them the a-posteriori check accepted (hos2d_gate_audit_check)."""
        v = (ctypes.c_ulonglong * 2)()
        _check(self._lib.hos2d_gate_audit_check(self._h, v))
        return {"fn_linear": int(v[0]), "fn_linear_accepted": int(v[1])}

    def run(self, tstop: float, max_steps: int = 10**9, graph: bool = True, check_every: int = 50) -> int:
        """Advance until t >= tstop (the driver's while loop); returns steps taken."""
        steps = 0
        t, _ = self.sync()
        while t < tstop and steps < max_steps:
            k = min(check_every, max_steps - steps)
            self.advance(k, tstop, graph=graph)
            steps += k
            t, _ = self.sync()
        return steps


def _check1(code: int) -> None:
    if code == HOS_OK:
        return
    msg = load().hos1d_last_error().decode(errors="replace")
    if code == HOS_E_BLOWUP:
        raise HosBlowUp(msg)
    raise HosError(f"hos error {code}: {msg}")


class Solver1D:
    """One 1D problem resident on the current CUDA device (the reference's 1D drivers)."""

    def __init__(self, problem: Problem1D, precision: int = FP64):
        self.problem = problem
        self._lib = load()
        self._params = problem.to_c()
        h = ctypes.c_void_p()
        _check1(self._lib.hos1d_create(ctypes.byref(self._params), precision, ctypes.byref(h)))
        self._h = h
        self.nx = problem.nx

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hos1d_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, convar: np.ndarray) -> None:
        c = np.ascontiguousarray(convar, dtype=np.float64).reshape(-1)
        if c.size != 3 * self.nx:
            raise ValueError("convar must hold nx*3 values")
        _check1(self._lib.hos1d_set_state(self._h, _ptr(c)))

    def get_state(self):
        c = np.empty(3 * self.nx)
        a = np.empty(self.nx)
        _check1(self._lib.hos1d_get_state(self._h, _ptr(c), _ptr(a)))
        return dict(convar=c.reshape(self.nx, 3), alpha=a)

    def step(self, tstop: float) -> None:
        _check1(self._lib.hos1d_step(self._h, tstop))

    def run(self, tstop: float, max_steps: int = 10**9) -> int:
        n = ctypes.c_int()
        _check1(self._lib.hos1d_run(self._h, tstop, max_steps, ctypes.byref(n)))
        return n.value

    def sync(self) -> tuple[float, float]:
        t, dt = ctypes.c_double(), ctypes.c_double()
        _check1(self._lib.hos1d_sync(self._h, ctypes.byref(t), ctypes.byref(dt)))
        return t.value, dt.value


def _check3(code: int) -> None:
    if code == HOS_OK:
        return
    msg = load().hos3d_last_error().decode(errors="replace")
    if code == HOS_E_BLOWUP:
        raise HosBlowUp(msg)
    raise HosError(f"hos error {code}: {msg}")


class Solver3D:
    """One 3D problem resident on the current CUDA device (the reference's CubicTube loop,
    src/3Dproblem.cpp:125-157): WENO5-AO on 2 x 2 Gauss points per face, GKS3D, S2O4.
    State arrays use the reference's cell order ((i * ny + j) * nz + k, 5 doubles per cell)."""

    PROFILE_KEYS = ["begin_step"] + [f"{k}{s}" for s in (0, 1) for k in
                                     ("bc", "gate", "face_x", "line_x", "point_x", "face_y", "line_y", "point_y",
                                      "face_z", "line_z", "point_z", "update")]

    def __init__(self, problem: Problem3D, precision: int = FP64):
        self.problem = problem
        self._lib = load()
        self._params = problem.to_c()
        h = ctypes.c_void_p()
        _check3(self._lib.hos3d_create(ctypes.byref(self._params), precision, ctypes.byref(h)))
        self._h = h
        self.shape = problem.shape

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hos3d_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def _n(self) -> int:
        return self.shape[0] * self.shape[1] * self.shape[2]

    def set_state(self, convar: np.ndarray, primvar: np.ndarray | None = None) -> None:
        c = np.ascontiguousarray(convar, dtype=np.float64).reshape(-1)
        if c.size != 5 * self._n():
            raise ValueError("convar must hold nx*ny*nz*5 values")
        p = None if primvar is None else np.ascontiguousarray(primvar, dtype=np.float64).reshape(-1)
        _check3(self._lib.hos3d_set_state(self._h, _ptr(c), _ptr(p)))

    def get_state(self, primvar: bool = False):
        c = np.empty(5 * self._n())
        p = np.empty(5 * self._n()) if primvar else None
        _check3(self._lib.hos3d_get_state(self._h, _ptr(c), _ptr(p)))
        out = dict(convar=c.reshape(*self.shape, 5))
        if primvar:
            out["primvar"] = p.reshape(*self.shape, 5)
        return out

    def step(self, tstop: float = 1e30) -> None:
        _check3(self._lib.hos3d_step(self._h, tstop))

    def advance(self, nsteps: int, tstop: float = 1e30) -> None:
        _check3(self._lib.hos3d_advance(self._h, nsteps, tstop))

    def begin_step(self, tstop: float = 1e30) -> None:
        _check3(self._lib.hos3d_begin_step(self._h, tstop))

    def stage(self, i: int) -> None:
        _check3(self._lib.hos3d_stage(self._h, i))

    def sync(self) -> tuple[float, float]:
        t, dt = ctypes.c_double(), ctypes.c_double()
        _check3(self._lib.hos3d_sync(self._h, ctypes.byref(t), ctypes.byref(dt)))
        return t.value, dt.value

    def set_time(self, t: float) -> None:
        _check3(self._lib.hos3d_set_time(self._h, t))

    @property
    def stream(self) -> int:
        v = ctypes.c_void_p()
        _check3(self._lib.hos3d_stream(self._h, ctypes.byref(v)))
        return v.value or 0

    def profile_step(self, tstop: float = 1e30) -> dict:
        ms = (ctypes.c_float * 25)()
        _check3(self._lib.hos3d_profile_step(self._h, tstop, ms, 25))
        return dict(zip(self.PROFILE_KEYS, [float(x) for x in ms]))

    def set_gate(self, gate: "Gate | None", threshold: float = 0.0, audit_log2: int = 10) -> None:
        _check3(self._lib.hos3d_set_gate(self._h, gate._h if gate is not None else None, threshold, audit_log2))

    GATE_KEYS = ["cells_x", "cells_y", "cells_z", "smooth_x", "smooth_y", "smooth_z", "audited", "false_neg",
                 "fallback", "unused"]

    def gate_stats(self, reset: bool = False) -> dict:
        v = (ctypes.c_ulonglong * 10)()
        _check3(self._lib.hos3d_gate_stats(self._h, v, 1 if reset else 0))
        return dict(zip(self.GATE_KEYS, [int(x) for x in v]))

    def run(self, tstop: float, max_steps: int = 10**9, check_every: int = 20) -> int:
        steps = 0
        t, _ = self.sync()
        while t < tstop and steps < max_steps:
            k = min(check_every, max_steps - steps)
            self.advance(k, tstop)
            steps += k
            t, _ = self.sync()
        return steps


def _checkb(code: int) -> None:
    if code == HOS_OK:
        return
    msg = load().hos_batch2d_last_error().decode(errors="replace")
    if code == HOS_E_BLOWUP:
        raise HosBlowUp(msg)
    raise HosError(f"hos error {code}: {msg}")


class Batch2D:
    """Independent 2D problems advanced together (one launch per phase for the batch)."""

    SHAPES = ((8, 16), (16, 16), (16, 8))   # face-tile shapes (normal x tangential); 16 x 16: WENO5 only

    def __init__(self, problems, tstops, precision: int = FP64):
        self._lib = load()
        self.problems = list(problems)
        arr = (Params2D * len(self.problems))(*[p.to_c() for p in self.problems])
        ts = np.ascontiguousarray(tstops, dtype=np.float64)
        h = ctypes.c_void_p()
        _checkb(self._lib.hos_batch2d_create(arr, _ptr(ts), len(self.problems), precision, ctypes.byref(h)))
        self._h = h
        self.count = len(self.problems)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hos_batch2d_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, k: int, convar: np.ndarray, primvar: np.ndarray | None = None) -> None:
        c = np.ascontiguousarray(convar, dtype=np.float64).reshape(-1)
        p = None if primvar is None else np.ascontiguousarray(primvar, dtype=np.float64).reshape(-1)
        _checkb(self._lib.hos_batch2d_set_state(self._h, k, _ptr(c), _ptr(p)))

    def get_state(self, k: int):
        pb = self.problems[k]
        c = np.empty(pb.nx * pb.ny * 4)
        ax = np.empty(pb.nx * pb.ny)
        ay = np.empty(pb.nx * pb.ny)
        _checkb(self._lib.hos_batch2d_get_state(self._h, k, _ptr(c), _ptr(ax), _ptr(ay)))
        return dict(convar=c.reshape(pb.nx, pb.ny, 4), alpha_x=ax.reshape(pb.nx, pb.ny),
                    alpha_y=ay.reshape(pb.nx, pb.ny))

    def autotune(self, reps: int = 3):
        ch = (ctypes.c_int * 2)()
        ms = np.zeros(6)
        _checkb(self._lib.hos_batch2d_autotune(self._h, reps, ch, _ptr(ms)))
        return tuple(ch), ms.reshape(2, 3)

    def advance(self, nsteps: int, graph: bool = True) -> None:
        _checkb(self._lib.hos_batch2d_advance(self._h, nsteps, 1 if graph else 0))

    def status(self, failed: bool = False):
        """(problems still running, t per problem, batch step index of each problem's last
        step[, per-problem failure flags]).  Without ``failed`` a blown-up problem raises
        HosBlowUp; with it, the flags say which problems stopped on a bad state."""
        act = ctypes.c_int()
        t = np.empty(self.count)
        last = (ctypes.c_int * self.count)()
        bad = (ctypes.c_int * self.count)() if failed else None
        _checkb(self._lib.hos_batch2d_status(self._h, ctypes.byref(act), _ptr(t), last, bad))
        if failed:
            return act.value, t, np.array(last[:]), np.array(bad[:], dtype=bool)
        return act.value, t, np.array(last[:])

    def set_reconstruction(self, first_order: bool) -> None:
        """First-order reconstruction for the following steps of every problem (the drivers'
        step 0) or the WENO-AO scheme."""
        _checkb(self._lib.hos_batch2d_set_reconstruction(self._h, 1 if first_order else 0))

    def set_gate(self, gate, threshold: float = 0.0, audit_log2: int = 10) -> None:
        """Attach a copy of a learned gate (FP32 batches); None detaches it."""
        _checkb(self._lib.hos_batch2d_set_gate(self._h, gate._h if gate is not None else None, threshold, audit_log2))

    def gate_stats(self, reset: bool = False) -> dict:
        v = (ctypes.c_ulonglong * 8)()
        _checkb(self._lib.hos_batch2d_gate_stats(self._h, v, 1 if reset else 0))
        keys = ("cells_x", "cells_y", "smooth_x", "smooth_y", "audited", "false_neg", "fallback", "unused")
        return dict(zip(keys, (int(x) for x in v)))

    @property
    def cells(self) -> int:
        return int(self._lib.hos_batch2d_cells(self._h))

    @property
    def stream(self) -> int:
        return int(self._lib.hos_batch2d_stream(self._h) or 0)


def _checkg(code: int) -> None:
    if code == HOS_OK:
        return
    msg = load().hos_gate_last_error().decode(errors="replace") or load().hos_last_error().decode(errors="replace")
    raise HosError(msg)


class Gate:
    """The learned smoothness gate: a 16-32-32-1 MLP trained on the GPU on labels the solver
    writes from its own states (``collect``)."""

    FEATURES = 16
    SAMPLE = 20
    PARAMS = 1633

    def __init__(self, capacity: int = 1 << 22, seed: int = 1):
        self._lib = load()
        h = ctypes.c_void_p()
        _checkg(self._lib.hos_gate_create(capacity, seed, ctypes.byref(h)))
        self._h = h
        self.capacity = capacity

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.hos_gate_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        out = np.empty(self.PARAMS, np.float32)
        _checkg(self._lib.hos_gate_get_params(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    @params.setter
    def params(self, value) -> None:
        v = np.ascontiguousarray(value, np.float32)
        assert v.size == self.PARAMS
        _checkg(self._lib.hos_gate_set_params(self._h, v.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def collect(self, solver: "Solver2D", sample_log2: int = 4) -> None:
        _check(self._lib.hos_gate_collect(self._h, solver._h, sample_log2))

    def collect3d(self, solver: "Solver3D", sample_log2: int = 4) -> None:
        """Samples of a 3D solver's state: features along x, y and z of sampled cells."""
        _check3(self._lib.hos_gate_collect3d(self._h, solver._h, sample_log2))

    @property
    def count(self) -> int:
        n = ctypes.c_ulonglong()
        _checkg(self._lib.hos_gate_sample_count(self._h, ctypes.byref(n)))
        return int(n.value)

    def samples(self) -> np.ndarray:
        n = self.count
        out = np.empty((n, self.SAMPLE), np.float32)
        _checkg(self._lib.hos_gate_get_samples(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n))
        return out

    def set_samples(self, s: np.ndarray) -> None:
        s = np.ascontiguousarray(s, np.float32).reshape(-1, self.SAMPLE)
        _checkg(self._lib.hos_gate_set_samples(self._h, s.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(s)))

    def clear(self) -> None:
        _checkg(self._lib.hos_gate_clear_samples(self._h))

    def gradient(self, first: int, n: int, w_pos: float = 1.0, w_neg: float = 4.0):
        g = np.empty(self.PARAMS, np.float32)
        loss = ctypes.c_double()
        _checkg(self._lib.hos_gate_gradient(self._h, first, n, w_pos, w_neg,
                                            g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(loss)))
        return g, loss.value

    def forward(self, first: int, n: int) -> np.ndarray:
        z = np.empty(n, np.float32)
        _checkg(self._lib.hos_gate_forward(self._h, first, n, z.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return z

    def train(self, steps: int, batch: int = 4096, lr: float = 3e-3, w_pos: float = 1.0, w_neg: float = 4.0,
              seed: int = 0) -> float:
        loss = ctypes.c_double()
        _checkg(self._lib.hos_gate_train(self._h, steps, batch, lr, w_pos, w_neg, seed, ctypes.byref(loss)))
        return loss.value
