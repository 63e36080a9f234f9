// hos_oracle3d.cpp -- CPU FP64 restatement of the reference's 3D per-step path.
//
// TEST INFRASTRUCTURE ONLY (see oracle_api.h): the checker for the CUDA 3D path.
//
// Restates (file:line in XJTUZhangHong/high-order-solver):
//   step driver .......... src/3Dproblem.cpp:125-157 (CubicTube's loop)
//   CopyFluid_new_to_old . src/basic_function.cpp (3D overload, interior cells)
//   Get_CFL / Dtx_3d ..... src/time_advance.cpp:793-848 (lagged primitives, seed R_c,
//                          viscous cap, +1e-16 clip)
//   boundaries 3D ........ src/boundary_condition.cpp:445-570 (free); periodic and
//                          reflecting sides are added here in the same per-axis form
//   Convar_to_primvar 3D . src/basic_function.cpp:775-800 (interior, blow-up status)
//   face values .......... src/reconstruction.cpp:3698-3722 (cell loop), :3774-3925
//                          (WENO5_AO_splitting_3d, WENO5_AO: non-DF WENO5-AO, epsilon 1e-10)
//   line values .......... src/reconstruction.cpp:3724-3738, :3927-4143
//   point values ......... src/reconstruction.cpp:3740-3752, :4145-4398
//   2-point WENO5-AO ..... src/reconstruction.cpp:2393-2551 (weno_5th_ao_2gauss)
//   GKS3D ................ src/flux_function.cpp:813-1103, Calculate_flux 3D :756-811
//   moments 3D ........... src/basic_function.cpp:189-401 (MMDF3d_left/right/MMDF3d),
//                          :585-601 (A 3D), include/basic_function.h:203-358
//                          (Collision, GL/GR/G_address templates)
//   characteristic 3D .... src/basic_function.cpp:994-1095, rotations :1208-1224
//   collision times ...... src/basic_function.cpp:638-708 (Get_Tau_NS, Get_Tau)
//   S2O4 + Update_gauss .. src/time_advance.cpp:732-741, :850-999
//
// Where this restatement departs from the reference (the reference's 3D path does not run:
// Interface3d::gauss is never allocated, src/basic_function.cpp:1897-1903):
//   * GKS3D converts the face states with Convar_to_primvar_3D and hands the pressure to the
//     Maxwellian moments, the microslope solver and the collision times as if it were
//     lambda = (K+3) rho / (4 (rho E - rho |u|^2 / 2)) (src/flux_function.cpp:831-836, 914).
//     Here lambda is used, as the 1D and 2D GKS do (Convar_to_ULambda_1d/_2d).
//   * The order-reduction flags of lines and points are never cleared in the reference
//     (src/reconstruction.cpp:4124-4132, :4376-4384), so one reduction would make that face
//     first order for the rest of the run; here each reconstruction decides afresh.
//   * The Gauss-point Recon3d array is allocated (4 points per face, weights 1/4).
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle_api.h"
#include "oracle_weno.h"

namespace {

using namespace oracle_weno;

hos3d_params P;
int NX = 0, NY = 0, NZ = 0, G = 0;
double DX = 0, DY = 0, DZ = 0, RC = 0, KK = 0, GAM = 0;
std::vector<double> W, Wold, PR;   // 5 doubles per cell, reference order (i*ny + j)*nz + k

const double TC[2][2][2] = {{{0.5, 1.0 / 8.0}, {0.0, 0.0}}, {{1.0, 1.0 / 6.0}, {0.0, 1.0 / 3.0}}};
// Checker-only switch: the 1D GKS keeps the numerical collision time of dt at the dt/2 level
// (src/flux_function.cpp:16-276) where GKS2D/GKS3D recompute it for dt/2; setting this makes
// the 3D restatement follow the 1D convention so that one-dimensional data can be compared
// with the reference-pinned 1D restatement with every GKS term active.
int HALF_TAU_OF_DT = 0;
// Checker-only switch: the reference's own 3D conventions, the two departures listed at the
// top of this file (pressure in the lambda slot of GKS3D; order-reduction flags of lines and
// points that stay set), so that the restatement can be compared bit for bit with the
// reference's 3D functions run by oracle/ref_driver3d.cpp.
int REF_CONVENTIONS = 0;
// the reference's sticky flags: per direction, line flags over the line grid of
// direction_fluxes (face a, b interior, c with halo 2), point flags per interior face and line
std::vector<unsigned char> LINE_FLAG[3], POINT_FLAG[3];

inline size_t cell(int i, int j, int k) { return ((size_t)i * NY + j) * NZ + k; }

// ---- conversions ------------------------------------------------------------------------
inline void to_prim(double* pr, const double* w) {  // Convar_to_primvar_3D: (rho, u, v, w, p)
    pr[0] = w[0];
    pr[1] = w[1] / w[0];
    pr[2] = w[2] / w[0];
    pr[3] = w[3] / w[0];
    pr[4] = (GAM - 1.0) * (w[4] - 0.5 * w[1] * w[1] / w[0] - 0.5 * w[2] * w[2] / w[0] - 0.5 * w[3] * w[3] / w[0]);
}
inline double lambda3(double rho, double u, double v, double ww, double rhoE) {
    return (KK + 3.0) * 0.25 * (rho / (rhoE - 0.5 * rho * (u * u + v * v + ww * ww)));
}
inline void to_ulambda(double* pr, const double* w) {  // (rho, u, v, w, lambda)
    pr[0] = w[0];
    pr[1] = w[1] / w[0];
    pr[2] = w[2] / w[0];
    pr[3] = w[3] / w[0];
    pr[4] = lambda3(w[0], pr[1], pr[2], pr[3], w[4]);
}
inline bool needs_reduce(const double* w) {  // Check_Order_Reduce_by_Lambda_3D
    double lam = lambda3(w[0], w[1] / w[0], w[2] / w[0], w[3] / w[0], w[4]);
    return lam <= 0.0 || !(lam == lam);
}
// frame of a y face: (u, v, w) -> (v, -u, w); of a z face: (u, v, w) -> (w, v, -u)
inline void to_local(int dir, double* o, const double* w) {
    o[0] = w[0];
    o[4] = w[4];
    if (dir == 0) { o[1] = w[1]; o[2] = w[2]; o[3] = w[3]; }
    else if (dir == 1) { o[1] = w[2]; o[2] = -w[1]; o[3] = w[3]; }
    else { o[1] = w[3]; o[2] = w[2]; o[3] = -w[1]; }
}

void char_base(double* s, const double* pr) {  // Char_base_3D
    double c = std::sqrt(GAM * pr[4] / pr[0]);
    double overc = 1.0 / c;
    double alfa = (GAM - 1.) * 0.5 * overc * overc;
    double u = pr[1], v = pr[2], w = pr[3];
    double r_over = 1 / (GAM - 1);
    double H = 0.5 * (u * u + v * v + w * w) + 0.5 / alfa;
    double t[25] = {H + c * r_over * (u - c), -(u + c * r_over), -v, -w, 1,
                    -2 * H + 4 * r_over * c * c, 2 * u, 2 * v, 2 * w, -2,
                    -2 * v * c * c * r_over, 0, 2 * c * c * r_over, 0, 0,
                    -2 * w * c * c * r_over, 0, 0, 2 * c * c * r_over, 0,
                    H - c * r_over * (u + c), -u + c * r_over, -v, -w, 1};
    for (int i = 0; i < 25; ++i) s[i] = t[i] * alfa;
}
void to_char(double* ch, const double* s, const double* w) {  // Convar_to_char_3D
    for (int i = 0; i < 5; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 5; ++j) acc = acc + s[i * 5 + j] * w[j];
        ch[i] = acc;
    }
}
void from_char(double* w, const double* pr, const double* ch) {  // Char_to_convar_3D
    double c = std::sqrt(GAM * pr[4] / pr[0]);
    double alfa = (GAM - 1.) / (2.0 * c * c);
    double u = pr[1], v = pr[2], ww = pr[3];
    double H = 0.5 * (u * u + v * v + ww * ww) + 0.5 / alfa;
    double s[5][5] = {{1., 1.0, 0.0, 0.0, 1.0},
                      {u - c, u, 0, 0, u + c},
                      {v, v, 1, 0, v},
                      {ww, ww, 0, 1, ww},
                      {H - u * c, 0.5 * (u * u + v * v + ww * ww), v, ww, H + u * c}};
    for (int i = 0; i < 5; ++i) {
        double acc = 0;
        for (int j = 0; j < 5; ++j) acc = acc + s[i][j] * ch[j];
        w[i] = acc;
    }
}

// ---- reconstruction ---------------------------------------------------------------------
// A reconstructed state on one side of a face: value and slopes in the face's frame
// (d[0] normal, d[1] first tangential, d[2] second tangential).
struct Side { double c[5], d[3][5]; };
struct LR { Side l, r; };

// Face values of direction dir at face (a, b, c) of the local (normal, t1, t2) grid: the
// normal WENO5-AO of the cells either side (WENO5_AO, :3803-3925).  The left value comes
// from the left cell's right reconstruction, the right value from the right cell's left one.
// Local grids: x faces (i, j, k); y faces (j, nx-1-i, k); z faces (k, j, nx-1-i), so that the
// first and second tangential sweeps run forward in local indices exactly as the reference's
// line and point loops run along y/-x/y and z/z/-x (:3927-3960, :4145-4163).
struct Grid {
    int dir;
    int n0, n1, n2;  // extents of the local cell grid
    double hn, h1, h2;
    // global cell index of local cell (a, b, c)
    size_t at(int a, int b, int c) const {
        if (dir == 0) return cell(a, b, c);
        if (dir == 1) return cell(NX - 1 - b, a, c);
        return cell(NX - 1 - c, b, a);
    }
};
Grid grid(int dir) {
    Grid g;
    g.dir = dir;
    if (dir == 0) { g.n0 = NX; g.n1 = NY; g.n2 = NZ; g.hn = DX; g.h1 = DY; g.h2 = DZ; }
    else if (dir == 1) { g.n0 = NY; g.n1 = NX; g.n2 = NZ; g.hn = DY; g.h1 = DX; g.h2 = DZ; }
    else { g.n0 = NZ; g.n1 = NY; g.n2 = NX; g.hn = DZ; g.h1 = DY; g.h2 = DX; }
    return g;
}

// One cell of the local grid: its values at its left face (side "r" of face a) and its right
// face (side "l" of face a+1), WENO5_AO (:3803-3925) with the order reduction of the cell.
void cell_faces(const Grid& gr, int a, int b, int c, Side& at_left, Side& at_right) {
    double st[5][5], pr[3][5];
    for (int m = 0; m < 5; ++m) to_local(gr.dir, st[m], &W[5 * gr.at(a - 2 + m, b, c)]);
    for (int m = 0; m < 3; ++m) to_prim(pr[m], st[1 + m]);
    const bool ch = P.characteristic != 0;
    for (int side = 0; side < 2; ++side) {  // 0: left face (weno left), 1: right face
        double base[5];
        for (int v = 0; v < 5; ++v) base[v] = 0.5 * (pr[side == 0 ? 0 : 2][v] + pr[1][v]);
        double s5[5][5];
        if (ch) {
            double sb[25];
            char_base(sb, base);
            for (int m = 0; m < 5; ++m) {
                double t[5];
                to_char(t, sb, st[m]);
                for (int v = 0; v < 5; ++v) s5[v][m] = t[v];
            }
        } else {
            for (int m = 0; m < 5; ++m)
                for (int v = 0; v < 5; ++v) s5[v][m] = st[m][v];
        }
        double var[5], der[5];
        for (int v = 0; v < 5; ++v) weno5_plain(side, s5[v], gr.hn, var[v], der[v]);
        Side& o = side == 0 ? at_left : at_right;
        if (ch) {
            from_char(o.c, base, var);
            from_char(o.d[0], base, der);
        } else {
            for (int v = 0; v < 5; ++v) { o.c[v] = var[v]; o.d[0][v] = der[v]; }
        }
        for (int v = 0; v < 5; ++v) o.d[1][v] = o.d[2][v] = 0.0;
    }
    if (needs_reduce(at_right.c) || needs_reduce(at_left.c)) {
        for (int v = 0; v < 5; ++v) {
            at_left.c[v] = at_right.c[v] = st[2][v];
            at_left.d[0][v] = at_right.d[0][v] = 0.0;
        }
    }
}

// Tangential sweep of one side: from five states along the sweep (stencil[m], m = 0..4,
// centre m = 2) to the two Gauss points of the centre, WENO5_AO_for_line_value (:3963-4108)
// when nd == 1 (values + slope along t1 from convar, der1x carried) and
// WENO5_AO_for_point_value (:4165-4360) when nd == 2 (slope along t2, der1x and der1y carried).
void sweep_side(const Side* const* stencil, int nd, double h, Side* out) {
    const Side& w0 = *stencil[2];
    double base[5];
    to_prim(base, w0.c);
    const bool ch = P.characteristic != 0;
    double sb[25];
    if (ch) char_base(sb, base);
    // quantity q: 0 = convar (value and slope), 1.. = carried slopes d[q-1]
    for (int q = 0; q <= nd; ++q) {
        double s5[5][5];
        for (int m = 0; m < 5; ++m) {
            const double* src = q == 0 ? stencil[m]->c : stencil[m]->d[q - 1];
            if (ch) {
                double t[5];
                to_char(t, sb, src);
                for (int v = 0; v < 5; ++v) s5[v][m] = t[v];
            } else {
                for (int v = 0; v < 5; ++v) s5[v][m] = src[v];
            }
        }
        double g[2][5], gx[2][5];
        for (int v = 0; v < 5; ++v) {
            double gg[2], ggx[2];
            weno5_2gauss(s5[v], h, q == 0, gg, ggx);
            g[0][v] = gg[0];
            g[1][v] = gg[1];
            if (q == 0) { gx[0][v] = ggx[0]; gx[1][v] = ggx[1]; }
        }
        for (int ig = 0; ig < 2; ++ig) {
            double* dst = q == 0 ? out[ig].c : out[ig].d[q - 1];
            if (ch) from_char(dst, base, g[ig]);
            else for (int v = 0; v < 5; ++v) dst[v] = g[ig][v];
            if (q == 0) {
                if (ch) from_char(out[ig].d[nd], base, gx[ig]);
                else for (int v = 0; v < 5; ++v) out[ig].d[nd][v] = gx[ig][v];
            }
        }
    }
    for (int ig = 0; ig < 2; ++ig)
        for (int q = nd + 1; q < 3; ++q)
            for (int v = 0; v < 5; ++v) out[ig].d[q][v] = 0.0;
}

// both sides of a face position, with the order reduction of the sweep (:4110-4142,
// :4362-4397): any non-positive lambda among the two points' left/right values sends both
// points back to the centre state with a zero slope along the sweep
// sticky (reference conventions only): the position's order-reduction flag, read and set as
// the reference's line[0].order_reduce / point[0].order_reduce are (:4124-4132, :4380-4384)
void sweep(const LR* const* stencil, int nd, double h, LR* out, unsigned char* sticky = nullptr) {
    const Side* sl[5];
    const Side* sr[5];
    for (int m = 0; m < 5; ++m) { sl[m] = &stencil[m]->l; sr[m] = &stencil[m]->r; }
    Side ol[2], orr[2];
    sweep_side(sl, nd, h, ol);
    sweep_side(sr, nd, h, orr);
    bool reduce = false;
    for (int ig = 0; ig < 2; ++ig) reduce = reduce || needs_reduce(ol[ig].c) || needs_reduce(orr[ig].c);
    if (sticky) {
        reduce = reduce || *sticky;
        if (reduce) *sticky = 1;
    }
    for (int ig = 0; ig < 2; ++ig) {
        if (reduce) {
            out[ig] = *stencil[2];
            for (int v = 0; v < 5; ++v) { out[ig].l.d[nd][v] = 0.0; out[ig].r.d[nd][v] = 0.0; }
        } else {
            out[ig].l = ol[ig];
            out[ig].r = orr[ig];
        }
    }
}

// ---- GKS3D ------------------------------------------------------------------------------
// Moments of a Maxwellian (MMDF3d_left / _right / MMDF3d, src/basic_function.cpp:189-401):
// whole-space <u^i>, half-space <u^i>_{>0} / <u^i>_{<0}, <v^j>, <w^k>, <xi^2m>.
struct Mom3 {
    double uw[7], up[7], un[7], v[6], w[6], xi[3];
    int kind;  // 0 left (up), 1 right (un), 2 centre (both)
};
inline double AlphaF(double lambda, double u) { return std::erfc(std::sqrt(lambda) * u); }
inline double BetaF(double lambda, double u) {
    double pi = 3.14159265358979323846;
    return std::exp(-lambda * u * u) / std::sqrt(pi * lambda);
}
void mom3(Mom3& m, int kind, double u, double v, double w, double lambda) {
    m.kind = kind;
    m.uw[0] = 1;
    m.uw[1] = u;
    if (kind == 2) {
        m.up[0] = 0.5 * AlphaF(lambda, -u);
        m.un[0] = 0.5 * AlphaF(lambda, u);
        m.up[1] = u * m.up[0] + 0.5 * BetaF(lambda, u);
        m.un[1] = u * m.un[0] - 0.5 * BetaF(lambda, u);
        for (int i = 2; i <= 6; ++i) m.uw[i] = u * m.uw[i - 1] + 0.5 * (i - 1) / lambda * m.uw[i - 2];
        for (int i = 2; i <= 6; ++i) {
            m.up[i] = u * m.up[i - 1] + 0.5 * (i - 1) / lambda * m.up[i - 2];
            m.un[i] = u * m.un[i - 1] + 0.5 * (i - 1) / lambda * m.un[i - 2];
        }
        m.v[0] = 1; m.v[1] = v; m.w[0] = 1; m.w[1] = w;
        for (int i = 2; i <= 5; ++i) {
            m.v[i] = v * m.v[i - 1] + 0.5 * (i - 1) / lambda * m.v[i - 2];
            m.w[i] = w * m.w[i - 1] + 0.5 * (i - 1) / lambda * m.w[i - 2];
        }
        m.xi[0] = 1.0;
        m.xi[1] = 0.5 * KK / lambda;
        m.xi[2] = 0.25 * (KK * KK + 2 * KK) / (lambda * lambda);
        return;
    }
    double ol = 1.0 / lambda;
    double* h = kind == 0 ? m.up : m.un;
    if (kind == 0) {
        h[0] = 0.5 * AlphaF(lambda, -u);
        h[1] = u * h[0] + 0.5 * BetaF(lambda, u);
    } else {
        h[0] = 0.5 * AlphaF(lambda, u);
        h[1] = u * h[0] - 0.5 * BetaF(lambda, u);
    }
    for (int i = 2; i <= 6; ++i) m.uw[i] = u * m.uw[i - 1] + 0.5 * (i - 1) * ol * m.uw[i - 2];
    for (int i = 2; i <= 6; ++i) h[i] = u * h[i - 1] + 0.5 * (i - 1) * ol * h[i - 2];
    m.v[0] = 1; m.v[1] = v; m.w[0] = 1; m.w[1] = w;
    for (int i = 2; i <= 5; ++i) {
        m.v[i] = v * m.v[i - 1] + 0.5 * (i - 1) * ol * m.v[i - 2];
        m.w[i] = w * m.w[i - 1] + 0.5 * (i - 1) * ol * m.w[i - 2];
    }
    m.xi[0] = 1.0;
    m.xi[1] = 0.5 * KK * ol;
    m.xi[2] = 0.25 * (KK * KK + 2 * KK) * ol * ol;
}
// <u^i v^j w^k xi^2m> over the whole (s = 0), positive (1) or negative (2) half space
inline double mt(const Mom3& m, int s, int i, int j, int k, int q) {
    const double* u = s == 0 ? m.uw : s == 1 ? m.up : m.un;
    double r = u[i] * m.v[j] * m.w[k];
    return q == 0 ? r : r * m.xi[q];
}
// <psi a u^nu v^nv w^nw xi^2nx> (GL_address / GR_address / G_address templates)
void gaddr(const Mom3& m, int s, int nu, int nv, int nw, int nx, const double* a, double* psi) {
    auto M = [&](int i, int j, int k, int q) { return mt(m, s, nu + i, nv + j, nw + k, nx + q); };
    psi[0] = a[0] * M(0, 0, 0, 0) + a[1] * M(1, 0, 0, 0) + a[2] * M(0, 1, 0, 0) + a[3] * M(0, 0, 1, 0)
             + a[4] * 0.5 * (M(2, 0, 0, 0) + M(0, 2, 0, 0) + M(0, 0, 2, 0) + M(0, 0, 0, 1));
    psi[1] = a[0] * M(1, 0, 0, 0) + a[1] * M(2, 0, 0, 0) + a[2] * M(1, 1, 0, 0) + a[3] * M(1, 0, 1, 0)
             + a[4] * 0.5 * (M(3, 0, 0, 0) + M(1, 2, 0, 0) + M(1, 0, 2, 0) + M(1, 0, 0, 1));
    psi[2] = a[0] * M(0, 1, 0, 0) + a[1] * M(1, 1, 0, 0) + a[2] * M(0, 2, 0, 0) + a[3] * M(0, 1, 1, 0)
             + a[4] * 0.5 * (M(2, 1, 0, 0) + M(0, 3, 0, 0) + M(0, 1, 2, 0) + M(0, 1, 0, 1));
    psi[3] = a[0] * M(0, 0, 1, 0) + a[1] * M(1, 0, 1, 0) + a[2] * M(0, 1, 1, 0) + a[3] * M(0, 0, 2, 0)
             + a[4] * 0.5 * (M(2, 0, 1, 0) + M(0, 2, 1, 0) + M(0, 0, 3, 0) + M(0, 0, 1, 1));
    psi[4] = 0.5 * (a[0] * (M(2, 0, 0, 0) + M(0, 2, 0, 0) + M(0, 0, 2, 0) + M(0, 0, 0, 1)) +
                    a[1] * (M(3, 0, 0, 0) + M(1, 2, 0, 0) + M(1, 0, 2, 0) + M(1, 0, 0, 1)) +
                    a[2] * (M(2, 1, 0, 0) + M(0, 3, 0, 0) + M(0, 1, 2, 0) + M(0, 1, 0, 1)) +
                    a[3] * (M(2, 0, 1, 0) + M(0, 2, 1, 0) + M(0, 0, 3, 0) + M(0, 0, 1, 1)) +
                    a[4] * 0.5 * (M(4, 0, 0, 0) + M(0, 4, 0, 0) + M(0, 0, 4, 0) + M(0, 0, 0, 2) +
                                  2 * M(2, 2, 0, 0) + 2 * M(2, 0, 2, 0) + 2 * M(2, 0, 0, 1) +
                                  2 * M(0, 2, 2, 0) + 2 * M(0, 2, 0, 1) + 2 * M(0, 0, 2, 1)));
}
// microslope from a slope of the conserved variables (A 3D, src/basic_function.cpp:585-601)
void micro3(double* a, const double* der, const double* pr) {
    const double density = pr[0], u = pr[1], v = pr[2], w = pr[3], lambda = pr[4];
    double overden = 1.0 / density, overlambda = 1.0 / lambda;
    double A = 2 * der[4] * overden - (u * u + v * v + w * w + 0.5 * (KK + 3) * overlambda) * der[0] * overden;
    double B = (der[1] - u * der[0]) * overden;
    double C = (der[2] - v * der[0]) * overden;
    double D = (der[3] - w * der[0]) * overden;
    a[4] = 4 * lambda * lambda / (KK + 3) * (A - 2 * u * B - 2 * v * C - 2 * w * D);
    a[3] = 2 * lambda * D - w * a[4];
    a[2] = 2 * lambda * C - v * a[4];
    a[1] = 2 * lambda * B - u * a[4];
    a[0] = der[0] * overden - u * a[1] - v * a[2] - w * a[3] - 0.5 * a[4] * (u * u + v * v + w * w + 0.5 * (KK + 3) * overlambda);
}
double tau_ns(double d0, double l0) {  // Get_Tau_NS
    if (P.tau_type == 0) return 0.0;
    if (P.mu > 0.0) return 2.0 * P.mu * l0 / d0;
    return 0.0;
}
double tau_num(double dl, double dr, double d0, double ll, double lr, double l0, double dt) {  // Get_Tau
    if (P.tau_type == 0) {
        if (P.c1_euler <= 0 && P.c2_euler <= 0) return 0.0;
        double C = P.c2_euler * std::abs(dl / ll - dr / lr) / std::abs(dl / ll + dr / lr);
        return P.c1_euler * dt + dt * C;
    }
    double tn = P.c2_euler * std::abs(dl / ll - dr / lr) / std::abs(dl / ll + dr / lr) * dt;
    if (tn != tn) tn = 0.0;
    if (P.mu > 0.0) return tn + 2.0 * P.mu * l0 / d0;
    return 0.0;
}
void time_coeffs(double* t, double tau, double tn, double dt) {
    double eta = std::exp(-dt / tn);
    t[0] = tn * (1 - eta);
    t[1] = tn * (eta * (dt + tn) - tn) + tau * tn * (eta - 1);
    t[2] = tau * tn * (eta - 1);
    t[3] = tn * eta + dt - tn;
    t[4] = tn * (tn - eta * (dt + tn) - tau * (eta - 1)) - dt * tau;
    t[5] = 0.5 * dt * dt - tau * tn * (eta - 1) - tau * dt;
}
// GKS3D (src/flux_function.cpp:813-1103) for the S2O4 pair of time levels dt and dt/2:
// f = 4 F(dt/2) - F(dt), derf = 4 (F(dt) - 2 F(dt/2)), in the face's frame
void gks3(const Side& L, const Side& R, double dt, double* f, double* df) {
    double pl[5], prr[5], p0[5];
    // the reference hands Convar_to_primvar_3D's pressure to every lambda slot
    // (src/flux_function.cpp:831-836, 914); the restatement uses lambda
    auto prim_of = REF_CONVENTIONS ? to_prim : to_ulambda;
    prim_of(pl, L.c);
    prim_of(prr, R.c);
    Mom3 ml, mr;
    mom3(ml, 0, pl[1], pl[2], pl[3], pl[4]);
    mom3(mr, 1, prr[1], prr[2], prr[3], prr[4]);
    const double dl = pl[0], dr = prr[0];
    // all-collision centre state (Collision template, include/basic_function.h:203-214)
    double c0[5];
    c0[0] = dl * ml.up[0] + dr * mr.un[0];
    c0[1] = dl * ml.up[1] + dr * mr.un[1];
    c0[2] = dl * ml.v[1] * ml.up[0] + dr * mr.v[1] * mr.un[0];
    c0[3] = dl * ml.w[1] * ml.up[0] + dr * mr.w[1] * mr.un[0];
    c0[4] = 0.5 * dl * (ml.up[2] + ml.up[0] * ml.v[2] + ml.up[0] * ml.w[2] + ml.up[0] * ml.xi[1]) +
            0.5 * dr * (mr.un[2] + mr.un[0] * mr.v[2] + mr.un[0] * mr.w[2] + mr.un[0] * mr.xi[1]);
    double al[3][5], ar[3][5], d0[3][5];
    for (int d = 0; d < 3; ++d) {
        micro3(al[d], L.d[d], pl);
        micro3(ar[d], R.d[d], prr);
        double a0l[5], a0r[5];
        gaddr(ml, 1, 0, 0, 0, 0, al[d], a0l);
        gaddr(mr, 2, 0, 0, 0, 0, ar[d], a0r);
        for (int v = 0; v < 5; ++v) d0[d][v] = dl * a0l[v] + dr * a0r[v];
    }
    prim_of(p0, c0);
    const double tau = tau_ns(p0[0], p0[4]);
    double t[6];
    time_coeffs(t, tau, tau_num(dl, dr, p0[0], pl[4], prr[4], p0[4], dt), dt);
    const double unit[5] = {1, 0.0, 0.0, 0.0, 0.0};
    double glu[5], gru[5];
    gaddr(ml, 1, 1, 0, 0, 0, unit, glu);
    gaddr(mr, 2, 1, 0, 0, 0, unit, gru);
    Mom3 m0;
    mom3(m0, 2, p0[1], p0[2], p0[3], p0[4]);
    double g0u[5];
    gaddr(m0, 0, 1, 0, 0, 0, unit, g0u);
    double lxx[5], rxx[5], lyy[5], ryy[5], lzz[5], rzz[5];
    gaddr(ml, 1, 2, 0, 0, 0, al[0], lxx);
    gaddr(mr, 2, 2, 0, 0, 0, ar[0], rxx);
    gaddr(ml, 1, 1, 1, 0, 0, al[1], lyy);
    gaddr(mr, 2, 1, 1, 0, 0, ar[1], ryy);
    gaddr(ml, 1, 1, 0, 1, 0, al[2], lzz);
    gaddr(mr, 2, 1, 0, 1, 0, ar[2], rzz);
    // time derivatives from the compatibility condition
    double lxu[5], rxu[5], lyv[5], ryv[5], lzw[5], rzw[5];
    gaddr(ml, 0, 1, 0, 0, 0, al[0], lxu);
    gaddr(mr, 0, 1, 0, 0, 0, ar[0], rxu);
    gaddr(ml, 0, 0, 1, 0, 0, al[1], lyv);
    gaddr(mr, 0, 0, 1, 0, 0, ar[1], ryv);
    gaddr(ml, 0, 0, 0, 1, 0, al[2], lzw);
    gaddr(mr, 0, 0, 0, 1, 0, ar[2], rzw);
    double derl[5], derr[5];
    for (int v = 0; v < 5; ++v) {
        derl[v] = -dl * (lxu[v] + lyv[v] + lzw[v]);
        derr[v] = -dr * (rxu[v] + ryv[v] + rzw[v]);
    }
    double Al[5], Ar[5], Alu[5], Aru[5];
    micro3(Al, derl, pl);
    micro3(Ar, derr, prr);
    gaddr(ml, 1, 1, 0, 0, 0, Al, Alu);
    gaddr(mr, 2, 1, 0, 0, 0, Ar, Aru);
    double a0[3][5], a0xu[5], a0xuu[5], a0yv[5], a0yuv[5], a0zw[5], a0zuw[5];
    for (int d = 0; d < 3; ++d) micro3(a0[d], d0[d], p0);
    gaddr(m0, 0, 1, 0, 0, 0, a0[0], a0xu);
    gaddr(m0, 0, 2, 0, 0, 0, a0[0], a0xuu);
    gaddr(m0, 0, 0, 1, 0, 0, a0[1], a0yv);
    gaddr(m0, 0, 1, 1, 0, 0, a0[1], a0yuv);
    gaddr(m0, 0, 0, 0, 1, 0, a0[2], a0zw);
    gaddr(m0, 0, 1, 0, 1, 0, a0[2], a0zuw);
    double derA0[5], A0[5], A0u[5];
    for (int v = 0; v < 5; ++v) derA0[v] = -p0[0] * (a0xu[v] + a0yv[v] + a0zw[v]);
    micro3(A0, derA0, p0);
    gaddr(m0, 0, 1, 0, 0, 0, A0, A0u);
    // Prandtl-number correction of the heat flux: GKS2D's (src/flux_function.cpp:630-636,
    // 678-684; the reference's GKS3D has none) with the third velocity component
    const double prc = P.prandtl_fix ? 1.0 / P.prandtl - 1.0 : 0.0;
    double qs = a0xuu[4] + A0u[4] - p0[1] * (a0xuu[1] + A0u[1]) - p0[2] * (a0xuu[2] + A0u[2]) -
                p0[3] * (a0xuu[3] + A0u[3]);
    double F0[5], F1[5];
    for (int v = 0; v < 5; ++v) {
        F0[v] = dl * t[0] * glu[v] + dr * t[0] * gru[v];
        F0[v] = F0[v] + p0[0] * t[3] * g0u[v];
        F0[v] = F0[v] + t[1] * (dl * (lxx[v] + lyy[v] + lzz[v]) + dr * (rxx[v] + ryy[v] + rzz[v]));
        F0[v] = F0[v] + t[2] * (dl * Alu[v] + dr * Aru[v]);
        F0[v] = F0[v] + p0[0] * t[4] * (a0xuu[v] + a0yuv[v] + a0zuw[v]);
        F0[v] = F0[v] + p0[0] * t[5] * (A0u[v]);
    }
    if (P.prandtl_fix) F0[4] += prc * (qs * (-p0[0] * tau * dt));
    const double dt2 = 0.5 * dt;
    time_coeffs(t, tau, tau_num(dl, dr, p0[0], pl[4], prr[4], p0[4], HALF_TAU_OF_DT ? dt : dt2), dt2);
    for (int v = 0; v < 5; ++v) {
        F1[v] = t[0] * (dl * glu[v] + dr * gru[v]);
        F1[v] = F1[v] + t[1] * (dl * (lxx[v] + lyy[v] + lzz[v]) + dr * (rxx[v] + ryy[v] + rzz[v]));
        F1[v] = F1[v] + t[2] * (dl * Alu[v] + dr * Aru[v]);
        F1[v] = F1[v] + p0[0] * t[3] * g0u[v];
        F1[v] = F1[v] + p0[0] * t[4] * (a0xuu[v] + a0yuv[v] + a0zuw[v]);
        F1[v] = F1[v] + p0[0] * t[5] * (A0u[v]);
    }
    if (P.prandtl_fix) F1[4] += prc * (qs * (-p0[0] * tau * 0.5 * dt));
    for (int v = 0; v < 5; ++v) {
        f[v] = (4.0 * F1[v] - F0[v]);
        df[v] = 4.0 * (F0[v] - 2.0 * F1[v]);
    }
}

// ---- boundaries -------------------------------------------------------------------------
// per-axis source index of ghost index x (free: nearest interior layer; periodic: wrap;
// reflect: mirror), applied x, then y, then z as the driver calls the six side functions
int bc_src(int x, int n, int kind, bool low, bool& flip) {
    flip = false;
    const int g = G;
    if (kind == HOS_BC_PERIODIC) return low ? x + (n - 2 * g) : x - (n - 2 * g);
    if (kind == HOS_BC_REFLECT) {
        flip = true;
        return low ? 2 * g - 1 - x : 2 * (n - g) - 1 - x;
    }
    return low ? g : n - g - 1;
}
void bc3() {
    const int n[3] = {NX, NY, NZ};
    for (int ax = 0; ax < 3; ++ax) {
        for (int i = 0; i < NX; ++i)
            for (int j = 0; j < NY; ++j)
                for (int k = 0; k < NZ; ++k) {
                    int idx[3] = {i, j, k};
                    const int x = idx[ax];
                    if (x >= G && x < n[ax] - G) continue;
                    const bool low = x < G;
                    bool flip;
                    int src[3] = {i, j, k};
                    src[ax] = bc_src(x, n[ax], P.bc[2 * ax + (low ? 0 : 1)], low, flip);
                    double* dst = &W[5 * cell(i, j, k)];
                    const double* s = &W[5 * cell(src[0], src[1], src[2])];
                    for (int v = 0; v < 5; ++v) dst[v] = s[v];
                    if (flip) dst[1 + ax] = -dst[1 + ax];
                }
    }
}

// ---- one stage --------------------------------------------------------------------------
// per direction: face values on the local grid, lines, points, GKS at the four Gauss points;
// stored per face as sum over the points of weight 1/4 x (f, derf) in the face frame
std::vector<double> FXS[3];  // [dir][(face * 2 + stage) * 10 + q]: f[5], derf[5]
std::vector<double> FXP[3];  // per Gauss point: [dir][((face * 2 + stage) * 4 + point) * 10 + q]

struct FaceGrid {
    int na, nb, nc;  // local face grid: normal faces 0..n0-2G (interior faces), tangential interior
};

void direction_fluxes(int dir, int stage, double dt) {
    const Grid gr = grid(dir);
    const int g = G;
    const int nn = gr.n0 - 2 * g + 1, n1 = gr.n1 - 2 * g, n2 = gr.n2 - 2 * g;
    // face values for faces a in [g, n0-g], b in [g-2, n1-g+2), c in [g-2, n2-g+2)
    const int eb = n1 + 4, ec = n2 + 4;
    std::vector<LR> FV((size_t)nn * eb * ec);
    auto fv = [&](int a, int b, int c) -> LR& { return FV[((size_t)(a - g) * eb + (b - g + 2)) * ec + (c - g + 2)]; };
    #pragma omp parallel for collapse(2)
    for (int b = g - 2; b < gr.n1 - g + 2; ++b)
        for (int c = g - 2; c < gr.n2 - g + 2; ++c)
            for (int a = g - 1; a <= gr.n0 - g; ++a) {
                Side atl, atr;
                cell_faces(gr, a, b, c, atl, atr);
                if (a >= g) fv(a, b, c).r = atl;
                if (a + 1 <= gr.n0 - g) fv(a + 1, b, c).l = atr;
            }
    // lines along t1 for b interior, c in the halo
    std::vector<LR> LV((size_t)nn * n1 * ec * 2);
    auto lv = [&](int a, int b, int c, int ig) -> LR& {
        return LV[(((size_t)(a - g) * n1 + (b - g)) * ec + (c - g + 2)) * 2 + ig];
    };
    #pragma omp parallel for collapse(2)
    for (int a = g; a <= gr.n0 - g; ++a)
        for (int b = g; b < gr.n1 - g; ++b)
            for (int c = g - 2; c < gr.n2 - g + 2; ++c) {
                const LR* st[5];
                for (int m = 0; m < 5; ++m) st[m] = &fv(a, b - 2 + m, c);
                LR out[2];
                const size_t li = ((size_t)(a - g) * n1 + (b - g)) * ec + (c - g + 2);
                sweep(st, 1, gr.h1, out, REF_CONVENTIONS ? &LINE_FLAG[dir][li] : nullptr);
                lv(a, b, c, 0) = out[0];
                lv(a, b, c, 1) = out[1];
            }
    // points along t2 and the flux
    std::vector<double>& FX = FXS[dir];
    #pragma omp parallel for collapse(2)
    for (int a = g; a <= gr.n0 - g; ++a)
        for (int b = g; b < gr.n1 - g; ++b)
            for (int c = g; c < gr.n2 - g; ++c) {
                double acc[10] = {0};
                const size_t face = ((size_t)(a - g) * n1 + (b - g)) * n2 + (c - g);
                double* opt = &FXP[dir][(face * 2 + stage) * 4 * 10];
                for (int ig = 0; ig < 2; ++ig) {
                    const LR* st[5];
                    for (int m = 0; m < 5; ++m) st[m] = &lv(a, b, c - 2 + m, ig);
                    LR pt[2];
                    const size_t pi = ((((size_t)(a - g) * n1 + (b - g)) * n2 + (c - g)) * 2) + ig;
                    sweep(st, 2, gr.h2, pt, REF_CONVENTIONS ? &POINT_FLAG[dir][pi] : nullptr);
                    for (int ip = 0; ip < 2; ++ip) {
                        double f[5], df[5];
                        gks3(pt[ip].l, pt[ip].r, dt, f, df);
                        // the reference's Gauss point ig * 2 + ip (gauss[i * sqrt(gausspoint)], :4152-4160)
                        for (int v = 0; v < 5; ++v) {
                            opt[(ig * 2 + ip) * 10 + v] = f[v];
                            opt[(ig * 2 + ip) * 10 + 5 + v] = df[v];
                        }
                        for (int v = 0; v < 5; ++v) {
                            acc[v] += 0.25 * f[v];
                            acc[5 + v] += 0.25 * df[v];
                        }
                    }
                }
                double* o = &FX[(face * 2 + stage) * 10];
                for (int q = 0; q < 10; ++q) o[q] = acc[q];
            }
}

// stage-combined flux of Gauss point m of local face (a, b, c) (interior-relative indices),
// in the face frame: sum over the stages so far of c_f f + c_d derf (Update_gauss,
// src/time_advance.cpp:866-939)
void combined(int dir, int stage, int a, int b, int c, int m, double* loc) {
    const Grid gr = grid(dir);
    const int n1 = gr.n1 - 2 * G, n2 = gr.n2 - 2 * G;
    const size_t face = ((size_t)a * n1 + b) * n2 + c;
    for (int v = 0; v < 5; ++v) {
        double s = 0.0;
        for (int k = 0; k <= stage; ++k) {
            const double* q = &FXP[dir][((face * 2 + k) * 4 + m) * 10];
            s = s + (TC[stage][k][0] * q[v] + TC[stage][k][1] * q[5 + v]);
        }
        loc[v] = s;
    }
}

int stage3(int stage, double dt) {
    bc3();
    // Convar_to_primvar over the interior: the primitives the next Get_CFL reads
    bool ok = true;
    for (int i = G; i < NX - G; ++i)
        for (int j = G; j < NY - G; ++j)
            for (int k = G; k < NZ - G; ++k) {
                double* pr = &PR[5 * cell(i, j, k)];
                to_prim(pr, &W[5 * cell(i, j, k)]);
                if (std::isnan(pr[0]) || std::isnan(pr[4]) || pr[0] < 0 || pr[4] < 0) ok = false;
            }
    if (!ok) return 1;
    for (int dir = 0; dir < 3; ++dir) direction_fluxes(dir, stage, dt);
    const int nx = NX - 2 * G, ny = NY - 2 * G, nz = NZ - 2 * G;
    #pragma omp parallel for collapse(2)
    for (int I = 0; I < nx; ++I)
        for (int J = 0; J < ny; ++J)
            for (int K = 0; K < nz; ++K) {
                // local indices of the six faces: x (I, J, K); y (J, nx-1-I, K); z (K, J, nx-1-I).
                // Per Gauss point the z, y and x face differences are accumulated in that order
                // with weight 1/4, the y and z faces' momentum components rotated back to the
                // global frame as the reference writes them (Update_gauss, :941-996).
                const double odx = 1 / DX, ody = 1 / DY, odz = 1 / DZ, w = 0.25;
                double tot[5];
                for (int v = 0; v < 5; ++v) tot[v] = 0.0;
                for (int m = 0; m < 4; ++m) {
                    double xl[5], xr[5], yl[5], yr[5], zl[5], zr[5];
                    combined(0, stage, I, J, K, m, xl);
                    combined(0, stage, I + 1, J, K, m, xr);
                    combined(1, stage, J, nx - 1 - I, K, m, yl);
                    combined(1, stage, J + 1, nx - 1 - I, K, m, yr);
                    combined(2, stage, K, J, nx - 1 - I, m, zl);
                    combined(2, stage, K + 1, J, nx - 1 - I, m, zr);
                    tot[0] += w * odz * (zl[0] - zr[0]);
                    tot[1] += w * odz * (-zl[3] + zr[3]);
                    tot[2] += w * odz * (zl[2] - zr[2]);
                    tot[3] += w * odz * (zl[1] - zr[1]);
                    tot[4] += w * odz * (zl[4] - zr[4]);
                    tot[0] += w * ody * (yl[0] - yr[0]);
                    tot[1] += w * ody * (-yl[2] + yr[2]);
                    tot[2] += w * ody * (yl[1] - yr[1]);
                    tot[3] += w * ody * (yl[3] - yr[3]);
                    tot[4] += w * ody * (yl[4] - yr[4]);
                    for (int v = 0; v < 5; ++v) tot[v] += w * odx * (xl[v] - xr[v]);
                }
                const size_t cc = cell(I + G, J + G, K + G);
                for (int v = 0; v < 5; ++v) W[5 * cc + v] = Wold[5 * cc + v] + tot[v];
            }
    return 0;
}

}  // namespace

extern "C" {

int oracle3d_init(const hos3d_params* p) {
    P = *p;
    if (p->ghost < 3) return 2;
    G = p->ghost;
    NX = p->nodex + 2 * G;
    NY = p->nodey + 2 * G;
    NZ = p->nodez + 2 * G;
    DX = (p->right - p->left) / p->nodex;
    DY = (p->up - p->down) / p->nodey;
    DZ = (p->front - p->back) / p->nodez;
    RC = DX;
    if (DY < RC) RC = DY;
    if (DZ < RC) RC = DZ;
    KK = p->K;
    GAM = p->gamma;
    const size_t n = (size_t)NX * NY * NZ * 5;
    W.assign(n, 0.0);
    Wold.assign(n, 0.0);
    PR.assign(n, 0.0);
    for (int d = 0; d < 3; ++d) {
        const Grid gr = grid(d);
        FXS[d].assign((size_t)(gr.n0 - 2 * G + 1) * (gr.n1 - 2 * G) * (gr.n2 - 2 * G) * 2 * 10, 0.0);
        FXP[d].assign(FXS[d].size() * 4, 0.0);
    }
    return 0;
}

void oracle3d_free(void) {
    W.clear(); Wold.clear(); PR.clear();
    for (auto& f : FXS) f.clear();
    for (auto& f : FXP) f.clear();
}

void oracle3d_set_state(const double* convar, const double* primvar) {
    const size_t n = (size_t)NX * NY * NZ * 5;
    // a new run: the reference's sticky order-reduction flags start cleared
    for (int d = 0; d < 3; ++d) {
        const Grid gr = grid(d);
        const size_t nn = gr.n0 - 2 * G + 1, n1 = gr.n1 - 2 * G, n2 = gr.n2 - 2 * G;
        LINE_FLAG[d].assign(nn * n1 * (n2 + 4), 0);
        POINT_FLAG[d].assign(nn * n1 * n2 * 2, 0);
    }
    std::memcpy(W.data(), convar, n * sizeof(double));
    if (primvar) std::memcpy(PR.data(), primvar, n * sizeof(double));
    else
        for (size_t c = 0; c < n / 5; ++c) to_prim(&PR[5 * c], &W[5 * c]);
}

void oracle3d_get_state(double* convar, double* primvar) {
    const size_t n = (size_t)NX * NY * NZ * 5;
    if (convar) std::memcpy(convar, W.data(), n * sizeof(double));
    if (primvar) std::memcpy(primvar, PR.data(), n * sizeof(double));
}

// CopyFluid_new_to_old + Get_CFL 3D (lagged primitives, seed R_c, viscous cap, clip)
double oracle3d_begin_step(double tstop, double t) {
    for (int i = G; i < NX - G; ++i)
        for (int j = G; j < NY - G; ++j)
            for (int k = G; k < NZ - G; ++k)
                for (int v = 0; v < 5; ++v) Wold[5 * cell(i, j, k) + v] = W[5 * cell(i, j, k) + v];
    double dt = RC;
    for (int i = G; i < NX - G; ++i)
        for (int j = G; j < NY - G; ++j)
            for (int k = G; k < NZ - G; ++k) {
                const double* pr = &PR[5 * cell(i, j, k)];
                double overden = 1.0 / pr[0];
                double tmp = std::sqrt(pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]) + std::sqrt(GAM * pr[4] * overden);
                if (tmp > P.cfl * RC / dt) dt = P.cfl * RC / tmp;
                if (P.tau_type != 0 && P.mu > 0 && dt > 0.33 * P.cfl * RC * RC * pr[0] / P.mu)
                    dt = 0.33 * P.cfl * RC * RC * pr[0] / P.mu;
            }
    if (t + dt > tstop) dt = tstop - t + 1e-16;
    return dt;
}

int oracle3d_stage(int stage, double dt) { return stage3(stage, dt); }

void oracle3d_set_half_tau_of_dt(int on) { HALF_TAU_OF_DT = on; }

void oracle3d_set_reference_conventions(int on) { REF_CONVENTIONS = on; }

long long oracle3d_reduced_count(void) {
    long long n = 0;
    for (int d = 0; d < 3; ++d) {
        for (unsigned char f : LINE_FLAG[d]) n += f ? 2 : 0;     // both lines of the face
        for (unsigned char f : POINT_FLAG[d]) n += f ? 2 : 0;    // both points of the line
    }
    return n;
}

int oracle3d_step(double tstop, double t, double* dt_out) {
    double dt = oracle3d_begin_step(tstop, t);
    if (dt_out) *dt_out = dt;
    for (int s = 0; s < 2; ++s) {
        int st = stage3(s, dt);
        if (st) return st;
    }
    return 0;
}

// per-face stage fluxes of direction dir, face frame: [face][stage][f 5, derf 5] over the
// interior faces of the local grid (normal, t1, t2)
void oracle3d_get_flux(int dir, double* out) {
    std::memcpy(out, FXS[dir].data(), FXS[dir].size() * sizeof(double));
}

}  // extern "C"
