"""Loaders for the two CPU implementations of the 2D step used as checkers:
the repository's FP64 restatement (oracle/liboracle.so) and, where it could be built,
the compiled reference (oracle/_ref/libhosref.so).  Test infrastructure only."""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
ORACLE_DIR = ROOT / "oracle"
REFERENCE = Path(os.environ.get("HOS_REFERENCE", "/root/reference"))
_DP = ctypes.POINTER(ctypes.c_double)


def _make(target=None):
    cmd = ["make", "-s", "-C", str(ORACLE_DIR), f"-j{os.cpu_count() or 4}"]
    if target:
        cmd.append(target)
    subprocess.run(cmd, check=True, capture_output=True)


class CpuStep:
    """One CPU implementation of the 2D step behind the oracle_api.h interface."""

    def __init__(self, kind: str = "oracle"):
        if kind == "oracle":
            path, self.pre = ORACLE_DIR / "liboracle.so", "oracle2d_"
            if not path.exists():
                _make()
        else:
            path, self.pre = ORACLE_DIR / "_ref" / "libhosref.so", "ref2d_"
            if not path.exists():
                if not (REFERENCE / "src").is_dir():
                    raise FileNotFoundError("reference checkout not present")
                _make("ref")
        self.lib = ctypes.CDLL(str(path))
        self.fn("begin_step").restype = ctypes.c_double

    def fn(self, name):
        return getattr(self.lib, self.pre + name)

    def init(self, pb, threads: int | None = None):
        self.pb = pb
        self.params = pb.to_c()
        st = self.fn("init")(ctypes.byref(self.params))
        if st != 0:
            raise RuntimeError(f"init failed: {st}")
        ncpu = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
        self.fn("set_threads")(threads or ncpu)
        self.t = 0.0
        return self

    def set_state(self, convar, primvar=None):
        c = np.ascontiguousarray(convar, dtype=np.float64).reshape(-1)
        p = None if primvar is None else np.ascontiguousarray(primvar, dtype=np.float64).reshape(-1)
        self._keep = (c, p)
        self.fn("set_state")(c.ctypes.data_as(_DP), None if p is None else p.ctypes.data_as(_DP))
        self.t = 0.0

    def step(self, tstop: float = 1e30) -> float:
        dt = ctypes.c_double()
        st = self.fn("step")(ctypes.c_double(tstop), ctypes.c_double(self.t), ctypes.byref(dt))
        if st != 0:
            raise RuntimeError(f"blow-up (status {st})")
        self.t += dt.value
        return dt.value

    def state(self):
        nx, ny = self.pb.nx, self.pb.ny
        c = np.empty(nx * ny * 4)
        p = np.empty(nx * ny * 4)
        ax = np.empty(nx * ny)
        ay = np.empty(nx * ny)
        self.fn("get_state")(c.ctypes.data_as(_DP), p.ctypes.data_as(_DP), ax.ctypes.data_as(_DP), ay.ctypes.data_as(_DP))
        return dict(convar=c.reshape(nx, ny, 4), primvar=p.reshape(nx, ny, 4),
                    alpha_x=ax.reshape(nx, ny), alpha_y=ay.reshape(nx, ny))

    def gauss(self, direction: int):
        nf = (self.pb.nx + 1) * (self.pb.ny + 1)
        gp = self.params.gausspoint
        out = np.empty(nf * gp * 36)
        self.fn("get_gauss")(direction, out.ctypes.data_as(_DP))
        return out.reshape(self.pb.nx + 1, self.pb.ny + 1, gp, 36)


def ref_available() -> bool:
    return (ORACLE_DIR / "_ref" / "libhosref.so").exists() or (REFERENCE / "src").is_dir()


def interior(pb, a):
    g = pb.ghost
    return a[g:g + pb.nodex, g:g + pb.nodey]


def rel_linf(a, b, pb):
    a = interior(pb, a)
    b = interior(pb, b)
    return float(np.abs(a - b).max() / np.abs(b).max())


class CpuStep1D:
    """1D counterpart of CpuStep (oracle1d_* / ref1d_*)."""

    def __init__(self, kind: str = "oracle"):
        base = CpuStep(kind)
        self.lib = base.lib
        self.pre = "oracle1d_" if kind == "oracle" else "ref1d_"

    def fn(self, name):
        return getattr(self.lib, self.pre + name)

    def init(self, pb):
        self.pb = pb
        self.params = pb.to_c()
        if self.fn("init")(ctypes.byref(self.params)) != 0:
            raise RuntimeError("init failed")
        self.t, self.nstep = 0.0, 0
        return self

    def set_state(self, convar):
        c = np.ascontiguousarray(convar, dtype=np.float64).reshape(-1)
        self._keep = c
        self.fn("set_state")(c.ctypes.data_as(_DP))
        self.t, self.nstep = 0.0, 0

    def step(self, tstop: float = 1e30) -> float:
        dt = ctypes.c_double()
        self.fn("step")(ctypes.c_double(tstop), ctypes.c_double(self.t), self.nstep, ctypes.byref(dt))
        self.t += dt.value
        self.nstep += 1
        return dt.value

    def run(self, tstop: float):
        while self.t < tstop:
            self.step(tstop)
        return self.nstep

    def state(self):
        nx = self.pb.nx
        c = np.empty(3 * nx)
        a = np.empty(nx)
        self.fn("get_state")(c.ctypes.data_as(_DP), a.ctypes.data_as(_DP))
        return dict(convar=c.reshape(nx, 3), alpha=a)


def gate_cells(pb, convar, alpha_x=None, alpha_y=None):
    """Oracle gate features [nx, ny, 2, 16] and weight distances [nx, ny, 2] (-1 where the
    stencil leaves the array) of a state, in FP64."""
    cpu = CpuStep("oracle").init(pb)
    n = pb.nx * pb.ny
    c = np.ascontiguousarray(convar, np.float64).reshape(-1)
    ax = np.zeros(n) if alpha_x is None else np.ascontiguousarray(alpha_x, np.float64).reshape(-1)
    ay = np.zeros(n) if alpha_y is None else np.ascontiguousarray(alpha_y, np.float64).reshape(-1)
    feat = np.empty(n * 2 * 16)
    dist = np.empty(n * 2)
    fn = cpu.fn("gate_cells")
    fn(c.ctypes.data_as(_DP), ax.ctypes.data_as(_DP), ay.ctypes.data_as(_DP), feat.ctypes.data_as(_DP),
       dist.ctypes.data_as(_DP))
    return feat.reshape(pb.nx, pb.ny, 2, 16), dist.reshape(pb.nx, pb.ny, 2)


class CpuStep3D:
    """The 3D restatement (oracle3d_*) or, with kind="ref", the compiled reference's own 3D
    functions driven by oracle/ref_driver3d.cpp (ref3d_*)."""

    def __init__(self, kind: str = "oracle"):
        self.lib = CpuStep(kind).lib
        self.pre = "oracle3d_" if kind == "oracle" else "ref3d_"
        self.fn("begin_step").restype = ctypes.c_double

    def fn(self, name):
        return getattr(self.lib, self.pre + name)

    def init(self, pb, threads: int | None = None):
        self.pb = pb
        self.params = pb.to_c()
        if self.fn("init")(ctypes.byref(self.params)) != 0:
            raise RuntimeError("init failed")
        if threads and self.pre == "ref3d_":
            self.fn("set_threads")(threads)
        self.t, self.nstep = 0.0, 0
        return self

    def set_state(self, convar, primvar=None):
        c = np.ascontiguousarray(convar, dtype=np.float64).reshape(-1)
        p = None if primvar is None else np.ascontiguousarray(primvar, dtype=np.float64).reshape(-1)
        self._keep = (c, p)
        self.fn("set_state")(c.ctypes.data_as(_DP), None if p is None else p.ctypes.data_as(_DP))
        self.t, self.nstep = 0.0, 0

    def step(self, tstop: float = 1e30) -> float:
        dt = ctypes.c_double()
        st = self.fn("step")(ctypes.c_double(tstop), ctypes.c_double(self.t), ctypes.byref(dt))
        if st != 0:
            raise RuntimeError(f"3D oracle blew up at t={self.t}")
        self.t += dt.value
        self.nstep += 1
        return dt.value

    def state(self):
        shp = self.pb.shape
        n = shp[0] * shp[1] * shp[2]
        c = np.empty(5 * n)
        p = np.empty(5 * n)
        self.fn("get_state")(c.ctypes.data_as(_DP), p.ctypes.data_as(_DP))
        return dict(convar=c.reshape(*shp, 5), primvar=p.reshape(*shp, 5))
