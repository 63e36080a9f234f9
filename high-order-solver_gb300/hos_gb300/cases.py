"""Initial data for the workloads (seeded, synthetic; no dataset is involved).

Every builder returns ``(problem, convar, primvar)`` with ``convar``/``primvar`` shaped
``(nx, ny, 4)`` over the whole block including ghost cells, cell (i, j) at ``[i, j]`` --
the reference's ``i * ny + j`` order (Fluid2d arrays, ``include/fluid_mesh.h:125-160``).
Ghost cells are filled by clamping to the nearest interior cell; every step's boundary
fill overwrites them before they are read.
"""
from __future__ import annotations

import math

import numpy as np

from .params import DF_ALWAYS, DF_AFTER_FIRST_STEP, TAU_NS, Problem1D, Problem2D, Problem3D


def prim_to_con(prim: np.ndarray, gamma: float) -> np.ndarray:
    """(rho, u, v, p) -> (rho, rho u, rho v, rho E), operand order of Primvar_to_convar_2D
    (src/basic_function.cpp:851-857, Q_densityE :1123-1127)."""
    rho, u, v, p = prim[..., 0], prim[..., 1], prim[..., 2], prim[..., 3]
    out = np.empty_like(prim)
    out[..., 0] = rho
    out[..., 1] = rho * u
    out[..., 2] = rho * v
    out[..., 3] = rho * (p / rho / (gamma - 1) + 0.5 * (u * u + v * v))
    return out


def _fill_ghosts(a: np.ndarray, g: int) -> np.ndarray:
    a[:g] = a[g]
    a[-g:] = a[-g - 1]
    a[:, :g] = a[:, g:g + 1]
    a[:, -g:] = a[:, -g - 1:-g]
    return a


def riemann2d(n: int = 1024, order: int = 7, zones=None, discon=(0.7, 0.7),
              characteristic: bool = True) -> tuple:
    """Four-quadrant Riemann problem on [0,1]^2 with outflow boundaries.

    Zone assignment follows IC_for_riemann_2d (src/2Dproblem.cpp:345-385): zone 1 lower-left,
    zone 2 lower-right, zone 3 upper-right, zone 4 upper-left, tested with the reference's
    ``i - ghost + 1 < discon / dx`` rule.  Default states are the quadrant states of the
    reference's PlanarShock driver (src/2Dproblem.cpp:85-90).
    """
    if zones is None:
        zones = ((0.138, 1.206, 1.206, 0.029), (0.5323, 0.0, 1.206, 0.3),
                 (1.5, 0.0, 0.0, 1.5), (0.5323, 1.206, 0.0, 0.3))
    pb = Problem2D(nodex=n, nodey=n, order=order, characteristic=characteristic,
                   c1_euler=0.05, c2_euler=1.0, cfl=0.5, bc=("free",) * 4)
    g = pb.ghost
    prim = np.zeros((pb.nx, pb.ny, 4))
    ii = (np.arange(pb.nx) - g + 1)[:, None].astype(np.float64)
    jj = (np.arange(pb.ny) - g + 1)[None, :].astype(np.float64)
    lx = ii < discon[0] / pb.dx
    ly = jj < discon[1] / pb.dx
    z = np.asarray(zones, dtype=np.float64)
    for q, mask in enumerate((lx & ly, ~lx & ly, ~lx & ~ly, lx & ~ly)):
        prim[mask] = z[q]
    _fill_ghosts(prim, g)
    return pb, prim_to_con(prim, pb.gamma), prim


def random_riemann2d(n: int, seed: int, order: int = 7) -> tuple:
    """Seeded random quadrant states: rho in [0.1, 2], p in [0.02, 2], u, v in [-1.5, 1.5]."""
    rng = np.random.default_rng(seed)
    zones = []
    for _ in range(4):
        zones.append((rng.uniform(0.1, 2.0), rng.uniform(-1.5, 1.5), rng.uniform(-1.5, 1.5),
                      rng.uniform(0.02, 2.0)))
    disc = (rng.uniform(0.3, 0.7), rng.uniform(0.3, 0.7))
    return riemann2d(n, order=order, zones=zones, discon=disc)


def isentropic_vortex(n: int = 200, order: int = 5, strength: float = 5.0,
                      center=(5.0, 5.0), length: float = 10.0,
                      characteristic: bool = True, images: bool = True) -> tuple:
    """Isentropic vortex on the periodic square [0, L]^2 over a unit freestream
    (rho, u, v, p) = (1, 1, 1, 1); cell averages by 4x4 Gauss-Legendre quadrature.
    The flow is smooth, so the numerical collision time is zero (c1 = c2 = 0) as in the
    reference's smooth accuracy drivers (src/2Dproblem.cpp:1376-1377).

    images: the vortex's perturbations (velocity and the temperature factor e^2) are summed
    over its periodic images at offsets -L, 0, +L in x and y, so the data are periodic to
    round-off (the nearest omitted image lies 15 or more away: e^(-112)).  A single vortex on
    [0, 10]^2 is not periodic: its velocity tail jumps by up to 2.4e-5 across the boundary,
    which bounds the error of any scheme near 4e-7 in L1."""
    pb = Problem2D(nodex=n, nodey=n, order=order, characteristic=characteristic,
                   c1_euler=0.0, c2_euler=0.0, cfl=0.5, left=0.0, right=length,
                   down=0.0, up=length, bc=("periodic",) * 4)
    gamma = pb.gamma
    g = pb.ghost
    xg, wg = np.polynomial.legendre.leggauss(4)
    cons = np.zeros((pb.nx, pb.ny, 4))
    xc = pb.left + (np.arange(pb.nx) - g + 0.5) * pb.dx
    yc = pb.down + (np.arange(pb.ny) - g + 0.5) * pb.dy
    for a, wa in zip(xg, wg):
        for b, wb in zip(xg, wg):
            x = xc[:, None] + 0.5 * pb.dx * a
            y = yc[None, :] + 0.5 * pb.dy * b
            du, dv, dt = 0.0, 0.0, 0.0
            for ox in ((-length, 0.0, length) if images else (0.0,)):
                for oy in ((-length, 0.0, length) if images else (0.0,)):
                    dxv = x - (center[0] + ox)
                    dyv = y - (center[1] + oy)
                    r2 = dxv * dxv + dyv * dyv
                    e = np.exp(0.5 * (1.0 - r2))
                    du = du - strength / (2 * math.pi) * e * dyv
                    dv = dv + strength / (2 * math.pi) * e * dxv
                    dt = dt + (gamma - 1.0) * strength ** 2 / (8 * gamma * math.pi ** 2) * e * e
            t = 1.0 - dt
            rho = t ** (1.0 / (gamma - 1.0))
            prim = np.stack([rho, 1.0 + du, 1.0 + dv, rho * t], axis=-1)
            cons += 0.25 * wa * wb * prim_to_con(prim, gamma)
    from_c = con_to_prim(cons, gamma)
    return pb, cons, from_c


def sinwave2d(n: int = 20, order: int = 9, characteristic: bool = False) -> tuple:
    """Density sine wave advected diagonally on the periodic square [0, 2]^2 (the reference's
    2D accuracy test, ICfor_sinwave_2d, src/2Dproblem.cpp:1527-1564): exact cell averages of
    rho = 1 + 0.2 sin(pi (x + y)), u = v = p = 1."""
    pb = Problem2D(nodex=n, nodey=n, order=order, characteristic=characteristic,
                   c1_euler=0.0, c2_euler=0.0, cfl=0.05, left=0.0, right=2.0, down=0.0,
                   up=2.0, bc=("periodic",) * 4)
    g = pb.ghost
    pi = 3.14159265358979323846
    prim = np.zeros((pb.nx, pb.ny, 4))
    i = np.arange(pb.nx)[:, None]
    j = np.arange(pb.ny)[None, :]
    xl = (i - g) * pb.dx
    xr = (i + 1 - g) * pb.dx
    yl = (j - g) * pb.dy
    yr = (j + 1 - g) * pb.dy
    k1 = np.sin(pi * (xr + yr))
    k2 = np.sin(pi * (xr + yl))
    k3 = np.sin(pi * (xl + yr))
    k4 = np.sin(pi * (xl + yl))
    prim[..., 0] = 1.0 - 0.2 / pi / pi / pb.dx / pb.dy * ((k1 - k2) - (k3 - k4))
    prim[..., 1:] = 1.0
    return pb, prim_to_con(prim, pb.gamma), prim


def con_to_prim(con: np.ndarray, gamma: float) -> np.ndarray:
    """Convar_to_primvar_2D (src/basic_function.cpp:811-817, Pressure :1156-1159)."""
    rho = con[..., 0]
    out = np.empty_like(con)
    out[..., 0] = rho
    out[..., 1] = con[..., 1] / rho
    out[..., 2] = con[..., 2] / rho
    out[..., 3] = (gamma - 1.0) * (con[..., 3] - 0.5 * con[..., 1] * con[..., 1] / rho
                                   - 0.5 * con[..., 2] * con[..., 2] / rho)
    return out


def prim_to_con_1d(prim: np.ndarray, gamma: float) -> np.ndarray:
    """(rho, u, p) -> (rho, rho u, rho E) (Primvar_to_convar_1D, src/basic_function.cpp:844-849)."""
    rho, u, p = prim[..., 0], prim[..., 1], prim[..., 2]
    out = np.empty_like(prim)
    out[..., 0] = rho
    out[..., 1] = rho * u
    out[..., 2] = rho * (p / rho / (gamma - 1) + 0.5 * (u * u))
    return out


def sod1d(n: int = 1000, order: int = 5, characteristic: bool = True) -> tuple:
    """Sod shock tube on [0, 1]: (1, 0, 1) | (0.125, 0, 0.1) at x = 0.5, outflow ends,
    WENO5-AO at step 0 then WENO5-AO-DF, GKS c1 = 0.05, c2 = 1, CFL 0.5 (SodTubeProblem,
    src/1Dproblem.cpp:3-174).  Returns (problem, convar[nx, 3])."""
    pb = Problem1D(nodex=n, order=order, characteristic=characteristic,
                   df_mode=DF_AFTER_FIRST_STEP if order == 5 else DF_ALWAYS, update_alpha=True)
    g = pb.ghost
    prim = np.zeros((pb.nx, 3))
    i = np.arange(pb.nx)
    left = (i - g + 1).astype(np.float64) * pb.dx <= 0.5
    prim[left] = (1.0, 0.0, 1.0)
    prim[~left] = (0.125, 0.0, 0.1)
    prim[:g] = prim[g]
    return pb, prim_to_con_1d(prim, pb.gamma)


def sinwave1d(n: int = 20) -> tuple:
    """The reference's 1D accuracy test (accuracy_sinwave_1d, src/1Dproblem.cpp:540-706):
    exact cell averages of rho = 1 + 0.2 sin(pi x) on the periodic [0, 2], u = p = 1,
    WENO5-AO-DF in conservative variables with the DF indicators never updated, c1 = c2 = 0,
    CFL 0.1.  Returns (problem, convar[nx, 3])."""
    pb = Problem1D(nodex=n, order=5, characteristic=False, df_mode=DF_ALWAYS, update_alpha=False,
                   c1_euler=0.0, c2_euler=0.0, cfl=0.1, left=0.0, right=2.0, bc=("periodic", "periodic"))
    g = pb.ghost
    pi = 3.14159265358979323846
    i = np.arange(pb.nx)
    prim = np.ones((pb.nx, 3))
    prim[:, 0] = 1.0 - 0.2 / pi / pb.dx * (np.cos(pi * (i + 1 - g) * pb.dx) - np.cos(pi * (i - g) * pb.dx))
    return pb, prim_to_con_1d(prim, pb.gamma)


def oblique_shock_states(mach: float, gamma: float = 1.4):
    """Pre- and post-shock primitive states of the double-Mach-reflection setup for a shock of
    Mach number ``mach`` moving at 60 degrees into (1.4, 0, 0, 1) (Rankine-Hugoniot), and the
    speed of its trace along a horizontal line.  Mach 10 returns the reference's literal
    constants (src/2Dproblem.cpp:989-1013, 1031-1035)."""
    if mach == 10.0:
        post = (8.0, 4.125 * math.sqrt(3), -4.125, 116.5)
        return post, (1.4, 0.0, 0.0, 1.0), 20 / math.sqrt(3.0)
    rho1, p1 = 1.4, 1.0
    c1 = math.sqrt(gamma * p1 / rho1)
    m2 = mach * mach
    rho2 = rho1 * (gamma + 1) * m2 / ((gamma - 1) * m2 + 2)
    p2 = p1 * (2 * gamma * m2 - (gamma - 1)) / (gamma + 1)
    un = mach * c1 * (1 - rho1 / rho2)
    post = (rho2, un * math.sqrt(3) / 2, -un / 2, p2)
    return post, (rho1, 0.0, 0.0, p1), 2 * mach * c1 / math.sqrt(3.0)


def wedge2d(nodex: int = 240, nodey: int = 60, mach: float = 10.0, order: int = 5,
            characteristic: bool = True, c1_euler: float = 0.2, c2_euler: float = 1.0) -> tuple:
    """Oblique shock on a wedge: the reference's double Mach reflection (doubleMach,
    ICforDoubleMach, boundaryforDoubleMach; src/2Dproblem.cpp:819-1093) on [0, 4] x [0, 1],
    wall from x = 1/6, parameterised by the shock Mach number."""
    post, pre, speed = oblique_shock_states(mach)
    pb = Problem2D(nodex=nodex, nodey=nodey, order=order, characteristic=characteristic,
                   c1_euler=c1_euler, c2_euler=c2_euler, cfl=0.5, left=0.0, right=4.0, down=0.0, up=1.0,
                   bc=("inflow", "free", "wedge_bottom", "wedge_top"),
                   bc_prim=(post, (0.0,) * 4, (0.0,) * 4, (0.0,) * 4),
                   wedge_x0=1.0 / 6.0, wedge_top_speed=speed, wedge_post=post, wedge_pre=pre)
    g = pb.ghost
    x = pb.left + (np.arange(pb.nx) + 0.5 - g) * pb.dx
    y = pb.down + (np.arange(pb.ny) + 0.5 - g) * pb.dy
    X, Y = np.meshgrid(x, y, indexing="ij")
    behind = (X < 1.0 / 6.0) | (Y > math.sqrt(3) * (X - 1.0 / 6.0))
    prim = np.empty((pb.nx, pb.ny, 4))
    prim[behind] = post
    prim[~behind] = pre
    return pb, prim_to_con(prim, pb.gamma), prim


def shock_vortex2d(n: int = 128, mach: float = 1.5, strength: float = 0.3, order: int = 5,
                   characteristic: bool = True, c1_euler: float = 0.05) -> tuple:
    """Shock-vortex interaction on [0, 2] x [0, 1] (2n x n cells): a stationary normal shock at
    x = 0.5 with upstream Mach ``mach``, upstream state (1, M sqrt(gamma), 0, 1), and an
    isentropic vortex of strength ``strength`` (core radius 0.05, decay 0.204) centred at
    (0.25, 0.5) in the upstream flow; inflow left, outflow right, reflective top and bottom.
    c1_euler: the numerical collision-time coefficient (the reference's drivers take 0.05 for
    the quadrant problems and 0.2 for the Mach-10 double Mach reflection)."""
    gamma = 1.4
    u1 = mach * math.sqrt(gamma)
    m2 = mach * mach
    rho2 = (gamma + 1) * m2 / ((gamma - 1) * m2 + 2)
    p2 = (2 * gamma * m2 - (gamma - 1)) / (gamma + 1)
    up = (1.0, u1, 0.0, 1.0)
    down = (rho2, u1 / rho2, 0.0, p2)
    pb = Problem2D(nodex=2 * n, nodey=n, order=order, characteristic=characteristic,
                   c1_euler=c1_euler, c2_euler=1.0, cfl=0.5, left=0.0, right=2.0, down=0.0, up=1.0,
                   bc=("inflow", "free", "reflect", "reflect"),
                   bc_prim=(up, (0.0,) * 4, (0.0,) * 4, (0.0,) * 4))
    g = pb.ghost
    x = pb.left + (np.arange(pb.nx) + 0.5 - g) * pb.dx
    y = pb.down + (np.arange(pb.ny) + 0.5 - g) * pb.dy
    X, Y = np.meshgrid(x, y, indexing="ij")
    prim = np.empty((pb.nx, pb.ny, 4))
    prim[X < 0.5] = up
    prim[X >= 0.5] = down
    rc, alpha = 0.05, 0.204
    dx_, dy_ = X - 0.25, Y - 0.5
    tau = np.sqrt(dx_ * dx_ + dy_ * dy_) / rc
    e = strength * np.exp(alpha * (1 - tau * tau))
    r = np.maximum(np.sqrt(dx_ * dx_ + dy_ * dy_), 1e-300)
    sin_t, cos_t = dy_ / r, dx_ / r
    T = 1.0 - (gamma - 1) * strength ** 2 * np.exp(2 * alpha * (1 - tau * tau)) / (4 * alpha * gamma)
    m = X < 0.5
    rho = np.where(m, T ** (1 / (gamma - 1)), prim[..., 0])
    prim[..., 1] = np.where(m, u1 + e * tau * sin_t, prim[..., 1])
    prim[..., 2] = np.where(m, -e * tau * cos_t, prim[..., 2])
    prim[..., 3] = np.where(m, rho * T, prim[..., 3])
    prim[..., 0] = rho
    return pb, prim_to_con(prim, pb.gamma), prim


def batch_sweep(count: int = 64, seed: int = 0, side_min: int = 128, side_max: int = 768,
                mach_min: float = 1.5, mach_max: float = 10.0, strength_max: float = 0.5,
                order: int = 5) -> list:
    """A seeded sweep of independent shock-vortex and oblique-shock-on-wedge problems of uneven
    sizes: even entries are shock-vortex problems, odd entries wedges.  The grid side ``s`` (the
    number of cells along x) is drawn uniformly from [side_min, side_max] and rounded to a
    multiple of 4; shock-vortex grids are s x s/2 on [0,2]x[0,1], wedge grids s x s/4 on
    [0,4]x[0,1] (square cells in both).  Shock Mach numbers are uniform in [mach_min, mach_max]
    and vortex strengths uniform in [0, strength_max].  End times are set so that the vortex
    crosses 0.3 of the domain height through the shock (0.3 / u_upstream) and the wedge shock
    trace moves the same distance whatever its Mach number (0.5 / M).  Shocks of Mach 3 and
    above take the reference's strong-shock collision coefficient c1 = 0.2
    (src/2Dproblem.cpp:839-840, the Mach-10 driver), weaker ones the quadrant problems' 0.05;
    the drivers' first-order step 0 is the caller's (Batch2D.set_reconstruction).

    Returns a list of (problem, convar, primvar, tstop, label)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        s = int(rng.integers(side_min, side_max + 1)) // 4 * 4
        mach = float(rng.uniform(mach_min, mach_max))
        if k % 2 == 0:
            strength = float(rng.uniform(0.0, strength_max))
            pb, con, prim = shock_vortex2d(s // 2, mach=mach, strength=strength, order=order,
                                           c1_euler=0.2 if mach >= 3.0 else 0.05)
            tstop = 0.3 / (mach * math.sqrt(pb.gamma))
            label = f"shock_vortex {pb.nodex}x{pb.nodey} M={mach:.2f} eps={strength:.2f}"
        else:
            pb, con, prim = wedge2d(s, s // 4, mach=mach, order=order)
            tstop = 0.5 / mach
            label = f"wedge {pb.nodex}x{pb.nodey} M={mach:.2f}"
        out.append((pb, con, prim, tstop, label))
    return out


def tgv3d(n: int = 256, re: float = 1600.0, mach: float = 0.1, gamma: float = 1.4,
          characteristic: bool = True, prandtl: float | None = 0.71) -> tuple:
    """Taylor-Green vortex on the periodic box [0, 2 pi]^3 (no counterpart among the reference's
    drivers; its 3D path is CubicTube, src/3Dproblem.cpp:3-172): rho = 1,
    u = sin x cos y cos z, v = -cos x sin y cos z, w = 0,
    p = 1/(gamma Ma^2) + (cos 2x + cos 2y)(cos 2z + 2)/16 at the cell centres, Navier-Stokes
    collision time with mu = 1/Re (rho_0 = V_0 = L = 1), Prandtl number Pr through the heat-flux
    correction (prandtl None: the BGK collision's Pr = 1).  Returns (problem, convar)."""
    L = 2.0 * math.pi
    pb = Problem3D(nodex=n, nodey=n, nodez=n, ghost=3, characteristic=characteristic, K=2, gamma=gamma,
                   c1_euler=0.0, c2_euler=1.0, cfl=0.5, tau_type=TAU_NS, mu=1.0 / re,
                   left=0.0, right=L, down=0.0, up=L, back=0.0, front=L, bc=("periodic",) * 6,
                   prandtl_fix=prandtl is not None, prandtl=1.0 if prandtl is None else prandtl)
    h = L / n
    xc = (np.arange(pb.shape[0]) - pb.ghost + 0.5) * h
    X, Y, Z = np.meshgrid(xc, xc, xc, indexing="ij", sparse=True)
    shape = pb.shape
    u = np.broadcast_to(np.sin(X) * np.cos(Y) * np.cos(Z), shape)
    v = np.broadcast_to(-np.cos(X) * np.sin(Y) * np.cos(Z), shape)
    p = np.broadcast_to(1.0 / (gamma * mach * mach) + (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2) / 16, shape)
    con = np.empty(shape + (5,))
    con[..., 0] = 1.0
    con[..., 1] = u
    con[..., 2] = v
    con[..., 3] = 0.0
    con[..., 4] = p / (gamma - 1) + 0.5 * (u * u + v * v)
    return pb, con


def rt2d(nodex: int = 100, order: int = 5) -> tuple:
    """Rayleigh-Taylor set-up of the reference's RT_instability driver (src/2Dproblem.cpp:611-818):
    [0, 0.25] x [0, 1] with nodex x 4 nodex cells, density 2 below y = 0.5 and 1 above,
    hydrostatic pressure p = 2y + 1 / y + 1.5, vertical velocity perturbation
    v = -0.025 c cos(8 pi x); reflecting left/right walls and the fixed bottom (2, 0, 0, 1) and
    top (1, 0, 0, 2.5) states of RT_boundary (src/boundary_condition.cpp:188-242).  The gravity
    source of Update_with_source acts along +y.  Returns (problem, convar, primvar)."""
    gamma = 1.4
    pb = Problem2D(nodex=nodex, nodey=4 * nodex, order=order, ghost=5, K=3, gamma=gamma, c1_euler=0.05,
                   c2_euler=1.0, cfl=0.5, left=0.0, right=0.25, down=0.0, up=1.0,
                   bc=("reflect", "reflect", "inflow", "inflow"),
                   bc_prim=((0.0,) * 4, (0.0,) * 4, (2.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 2.5)))
    g = pb.ghost
    dx, dy = pb.dx, pb.dy
    prim = np.zeros((pb.nx, pb.ny, 4))
    for i in range(g, pb.nx - g):
        x = (i - g + 0.5) * dx
        for j in range(g, pb.ny - g):
            if j - g + 1 < 0.5 / dy:
                p = 2.0 * (j - g + 0.5) * dy + 1.0
                c = math.sqrt(gamma * p / 2.0)
                prim[i, j] = (2.0, 0.0, -0.025 * c * math.cos(8.0 * math.pi * x), p)
            else:
                p = (j - g + 0.5) * dy + 1.5
                c = math.sqrt(gamma * p / 1.0)
                prim[i, j] = (1.0, 0.0, -0.025 * c * math.cos(8.0 * math.pi * x), p)
    prim = _fill_ghosts(prim, g)   # ghosts: filled by the boundaries before first use
    con = prim_to_con(prim, gamma)
    return pb, con, prim


def random_octants3d(n: int, seed: int, characteristic: bool = True) -> tuple:
    """A 3D Riemann problem on [0, 1]^3 for gate training: eight octants around a seeded centre
    with seeded states (rho in [0.3, 2], p in [0.2, 2], u, v, w in [-1, 1]), free sides."""
    rng = np.random.default_rng(seed)
    pb = Problem3D(nodex=n, nodey=n, nodez=n, ghost=3, characteristic=characteristic)
    ctr = rng.uniform(0.35, 0.65, size=3)
    states = np.stack([rng.uniform(0.3, 2.0, 8), rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8),
                       rng.uniform(-1, 1, 8), rng.uniform(0.2, 2.0, 8)], -1)
    xc = (np.arange(pb.shape[0]) - 3 + 0.5) / n
    X, Y, Z = np.meshgrid(xc, xc, xc, indexing="ij", sparse=True)
    octant = (X > ctr[0]).astype(int) * 4 + (Y > ctr[1]).astype(int) * 2 + (Z > ctr[2]).astype(int)
    prim = states[np.broadcast_to(octant, pb.shape)]
    rho, u, v, w, p = (prim[..., q] for q in range(5))
    gamma = pb.gamma
    con = np.stack([rho, rho * u, rho * v, rho * w, p / (gamma - 1) + 0.5 * rho * (u * u + v * v + w * w)], -1)
    return pb, con
