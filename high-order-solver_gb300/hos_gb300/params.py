"""Problem parameters shared by every implementation of the 2D step.

``Params2D`` is the ctypes mirror of the C struct ``hos_params2d`` declared in
``include/hos_gb300.h``.  Its fields are the knobs the reference sets as globals inside
each problem driver (``src/2Dproblem.cpp:3-60`` in the reference project): mesh size and
ghost layers (Block2d), reconstruction order and variables (cellreconstruction_2D_*,
reconstruction_variable), Gauss points (gausspoint), gas constants (K, Gamma), the
numerical collision-time coefficients (c1_euler, c2_euler), the CFL number and the four
boundary functions.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

BC_FREE, BC_PERIODIC, BC_REFLECT, BC_INFLOW, BC_WEDGE_BOTTOM, BC_WEDGE_TOP, BC_NOSLIP = 0, 1, 2, 3, 4, 5, 6
_BC_NAMES = {"free": BC_FREE, "outflow": BC_FREE, "periodic": BC_PERIODIC,
             "reflect": BC_REFLECT, "reflective": BC_REFLECT, "inflow": BC_INFLOW,
             "wedge_bottom": BC_WEDGE_BOTTOM, "wedge_top": BC_WEDGE_TOP, "noslip": BC_NOSLIP}

# Gauss points per face the reference pairs with each WENO-AO order
# (weno_5th/7th/9th_ao_with_df_2gauss write 2, 3 and 4 points; src/reconstruction.cpp:2700,3093,3489)
GAUSS_POINTS = {5: 2, 7: 3, 9: 4}


class Params2D(ctypes.Structure):
    _fields_ = [
        ("nodex", ctypes.c_int), ("nodey", ctypes.c_int), ("ghost", ctypes.c_int),
        ("order", ctypes.c_int), ("gausspoint", ctypes.c_int),
        ("characteristic", ctypes.c_int), ("use_df", ctypes.c_int), ("K", ctypes.c_int),
        ("gamma", ctypes.c_double), ("c1_euler", ctypes.c_double), ("c2_euler", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("left", ctypes.c_double), ("right", ctypes.c_double),
        ("down", ctypes.c_double), ("up", ctypes.c_double),
        ("bc", ctypes.c_int * 4), ("bc_prim", (ctypes.c_double * 4) * 4),
        ("wedge_x0", ctypes.c_double), ("wedge_top_speed", ctypes.c_double),
        ("wedge_post", ctypes.c_double * 4), ("wedge_pre", ctypes.c_double * 4),
        ("integrator", ctypes.c_int), ("flux", ctypes.c_int),
        ("tau_type", ctypes.c_int), ("mu", ctypes.c_double), ("nu", ctypes.c_double),
        ("prandtl_fix", ctypes.c_int), ("prandtl", ctypes.c_double),
        ("wenotype", ctypes.c_int),
    ]


# weights of the non-DF WENO5-AO scheme (HOS_WENO_* in include/hos_gb300.h)
WENOTYPES = {"wenoz": 0, "wenojs": 1, "linear": 2}

# time-marching methods and fluxes (HOS_INT_*, HOS_FLUX_* in include/hos_gb300.h)
INTEGRATORS = {"S2O4": 0, "S1O1": 1, "S1O2": 2, "RK2": 3, "RK3": 4, "RK4": 5}
STAGES = {0: 2, 1: 1, 2: 1, 3: 2, 4: 3, 5: 4}
FLUXES = {"GKS": 0, "LF": 1}


@dataclass
class Problem2D:
    """A 2D problem: mesh, scheme and boundary choices (one reference problem driver)."""

    nodex: int
    nodey: int
    order: int = 5
    characteristic: bool = True
    ghost: int = 5
    K: int = 3
    gamma: float = 1.4
    c1_euler: float = 0.05
    c2_euler: float = 1.0
    cfl: float = 0.5
    left: float = 0.0
    right: float = 1.0
    down: float = 0.0
    up: float = 1.0
    bc: tuple = ("free", "free", "free", "free")
    bc_prim: tuple = field(default_factory=lambda: ((0.0,) * 4,) * 4)
    # oblique shock on a wedge (the reference's doubleMach boundary)
    wedge_x0: float = 1.0 / 6.0
    wedge_top_speed: float = 0.0
    wedge_post: tuple = (0.0,) * 4
    wedge_pre: tuple = (0.0,) * 4
    # time marching and flux (the reference's timecoe_list_2d / flux_function_2d)
    integrator: str = "S2O4"
    flux: str = "GKS"
    # collision time (tau_type, Mu, Nu) and the Prandtl fix (is_Prandtl_fix, Pr); the
    # reference's defaults Mu = Nu = -1, Pr = 1
    tau_type: int = 0
    mu: float = -1.0
    nu: float = -1.0
    prandtl_fix: bool = False
    prandtl: float = 1.0
    # is_using_df_factor: True the DF variants; False the non-DF WENO5-AO with the wenotype
    # weights ("wenoz", "wenojs" or "linear")
    use_df: bool = True
    wenotype: str = "wenoz"

    @property
    def nx(self) -> int:
        return self.nodex + 2 * self.ghost

    @property
    def ny(self) -> int:
        return self.nodey + 2 * self.ghost

    @property
    def dx(self) -> float:
        return (self.right - self.left) / self.nodex

    @property
    def dy(self) -> float:
        return (self.up - self.down) / self.nodey

    def to_c(self) -> Params2D:
        p = Params2D()
        p.nodex, p.nodey, p.ghost = self.nodex, self.nodey, self.ghost
        p.order = self.order
        p.gausspoint = GAUSS_POINTS[self.order]
        p.characteristic = 1 if self.characteristic else 0
        p.use_df = 1 if self.use_df else 0
        p.wenotype = WENOTYPES[self.wenotype]
        p.K = self.K
        p.gamma, p.c1_euler, p.c2_euler, p.cfl = self.gamma, self.c1_euler, self.c2_euler, self.cfl
        p.left, p.right, p.down, p.up = self.left, self.right, self.down, self.up
        for s in range(4):
            b = self.bc[s]
            p.bc[s] = _BC_NAMES[b] if isinstance(b, str) else int(b)
            for v in range(4):
                p.bc_prim[s][v] = float(self.bc_prim[s][v])
        p.wedge_x0, p.wedge_top_speed = self.wedge_x0, self.wedge_top_speed
        for v in range(4):
            p.wedge_post[v] = float(self.wedge_post[v])
            p.wedge_pre[v] = float(self.wedge_pre[v])
        p.integrator = INTEGRATORS[self.integrator]
        p.flux = FLUXES[self.flux]
        p.tau_type, p.mu, p.nu = int(self.tau_type), float(self.mu), float(self.nu)
        p.prandtl_fix, p.prandtl = 1 if self.prandtl_fix else 0, float(self.prandtl)
        return p


class Params1D(ctypes.Structure):
    """ctypes mirror of hos_params1d (include/hos_gb300.h): the knobs of the reference's 1D
    drivers (SodTubeProblem, accuracy_sinwave_1d, src/1Dproblem.cpp:3-149, 540-640)."""

    _fields_ = [
        ("nodex", ctypes.c_int), ("ghost", ctypes.c_int), ("order", ctypes.c_int),
        ("characteristic", ctypes.c_int), ("df_mode", ctypes.c_int), ("update_alpha", ctypes.c_int),
        ("K", ctypes.c_int), ("gamma", ctypes.c_double), ("c1_euler", ctypes.c_double),
        ("c2_euler", ctypes.c_double), ("cfl", ctypes.c_double), ("left", ctypes.c_double),
        ("right", ctypes.c_double), ("bc", ctypes.c_int * 2), ("wenotype", ctypes.c_int),
    ]


# df_mode values: non-DF WENO5-AO always / DF variant always / non-DF at step 0 then DF
DF_NEVER, DF_ALWAYS, DF_AFTER_FIRST_STEP = 0, 1, 2


@dataclass
class Problem1D:
    """A 1D problem (one reference 1D driver)."""

    nodex: int
    order: int = 5
    characteristic: bool = True
    df_mode: int = DF_AFTER_FIRST_STEP
    update_alpha: bool = True
    ghost: int = 5
    K: int = 4
    gamma: float = 1.4
    c1_euler: float = 0.05
    c2_euler: float = 1.0
    cfl: float = 0.5
    left: float = 0.0
    right: float = 1.0
    bc: tuple = ("free", "free")
    # weights of the non-DF WENO5-AO steps ("wenoz", "wenojs" or "linear")
    wenotype: str = "wenoz"

    @property
    def nx(self) -> int:
        return self.nodex + 2 * self.ghost

    @property
    def dx(self) -> float:
        return (self.right - self.left) / self.nodex

    def to_c(self) -> Params1D:
        p = Params1D()
        p.nodex, p.ghost, p.order = self.nodex, self.ghost, self.order
        p.characteristic = 1 if self.characteristic else 0
        p.df_mode = int(self.df_mode)
        p.update_alpha = 1 if self.update_alpha else 0
        p.wenotype = WENOTYPES[self.wenotype]
        p.K = self.K
        p.gamma, p.c1_euler, p.c2_euler, p.cfl = self.gamma, self.c1_euler, self.c2_euler, self.cfl
        p.left, p.right = self.left, self.right
        for s in range(2):
            b = self.bc[s]
            p.bc[s] = _BC_NAMES[b] if isinstance(b, str) else int(b)
        return p


class Params3D(ctypes.Structure):
    """ctypes mirror of hos_params3d (include/hos_gb300.h): the knobs of the reference's 3D
    driver (CubicTube, src/3Dproblem.cpp:3-66) plus the viscosity of the Navier-Stokes
    collision time (Get_Tau_NS, src/basic_function.cpp:638-661) and periodic sides."""

    _fields_ = [
        ("nodex", ctypes.c_int), ("nodey", ctypes.c_int), ("nodez", ctypes.c_int), ("ghost", ctypes.c_int),
        ("characteristic", ctypes.c_int), ("K", ctypes.c_int),
        ("gamma", ctypes.c_double), ("c1_euler", ctypes.c_double), ("c2_euler", ctypes.c_double),
        ("cfl", ctypes.c_double), ("tau_type", ctypes.c_int), ("mu", ctypes.c_double),
        ("left", ctypes.c_double), ("right", ctypes.c_double), ("down", ctypes.c_double),
        ("up", ctypes.c_double), ("back", ctypes.c_double), ("front", ctypes.c_double),
        ("bc", ctypes.c_int * 6), ("prandtl_fix", ctypes.c_int), ("prandtl", ctypes.c_double),
        ("gks3d_pressure_slot", ctypes.c_int),
    ]


TAU_EULER, TAU_NS = 0, 1


@dataclass
class Problem3D:
    """A 3D problem: WENO5-AO (non-DF) on 2x2 Gauss points per face, GKS3D, S2O4."""

    nodex: int
    nodey: int
    nodez: int
    characteristic: bool = True
    ghost: int = 3
    K: int = 2
    gamma: float = 1.4
    c1_euler: float = 0.05
    c2_euler: float = 1.0
    cfl: float = 0.5
    tau_type: int = TAU_EULER
    mu: float = 0.0
    left: float = 0.0
    right: float = 1.0
    down: float = 0.0
    up: float = 1.0
    back: float = 0.0
    front: float = 1.0
    bc: tuple = ("free",) * 6
    prandtl_fix: bool = False   # Prandtl-number correction of the heat flux ...
    prandtl: float = 1.0        # ... with this Pr
    # the reference's own GKS3D convention (pressure where lambda belongs), FP64 only
    gks3d_pressure_slot: bool = False

    @property
    def shape(self) -> tuple:
        g = 2 * self.ghost
        return (self.nodex + g, self.nodey + g, self.nodez + g)

    @property
    def dx(self) -> float:
        return (self.right - self.left) / self.nodex

    @property
    def dy(self) -> float:
        return (self.up - self.down) / self.nodey

    @property
    def dz(self) -> float:
        return (self.front - self.back) / self.nodez

    def to_c(self) -> Params3D:
        p = Params3D()
        p.nodex, p.nodey, p.nodez, p.ghost = self.nodex, self.nodey, self.nodez, self.ghost
        p.characteristic = 1 if self.characteristic else 0
        p.K = self.K
        p.gamma, p.c1_euler, p.c2_euler, p.cfl = self.gamma, self.c1_euler, self.c2_euler, self.cfl
        p.tau_type, p.mu = int(self.tau_type), float(self.mu)
        p.left, p.right, p.down, p.up, p.back, p.front = (self.left, self.right, self.down, self.up,
                                                          self.back, self.front)
        for s in range(6):
            b = self.bc[s]
            p.bc[s] = _BC_NAMES[b] if isinstance(b, str) else int(b)
        p.prandtl_fix, p.prandtl = 1 if self.prandtl_fix else 0, float(self.prandtl)
        p.gks3d_pressure_slot = 1 if self.gks3d_pressure_slot else 0
        return p
