// hos_oracle2d.cpp -- CPU FP64 restatement of the reference's 2D per-step hot path.
//
// TEST INFRASTRUCTURE ONLY: this is the checker for the CUDA path.  Only tests/, the smoke
// check of __graft_entry__.py and the cpu_baseline leg of bench.py load it.  The product
// (hos_gb300 package and its CUDA library) never includes, links or calls it.
//
// What it restates (file:line in the reference project XJTUZhangHong/high-order-solver):
//   step driver ............ src/2Dproblem.cpp:128-157 (PlanarShock time loop)
//   CopyFluid_new_to_old ... src/basic_function.cpp:1571-1584
//   Get_CFL / Dtx .......... src/time_advance.cpp:264-305
//   boundary conditions .... src/boundary_condition.cpp:66-186, 244-258, 367-442
//   Convar_to_Primvar ...... src/basic_function.cpp:752-773 (blow-up -> status 1, no exit)
//   normal recon (DF) ...... src/reconstruction.cpp:1701-1859 (WENO5), 1861-2028 (WENO7),
//                            2030-2211 (WENO9); scalar kernels :480-657, :750-974, :1072-1364
//   normal recon (non-DF) .. src/reconstruction.cpp:1562-1699 (WENO5_AO_normal, WENO5_AO),
//                            scalar kernels :161-360 with the wenotype choice
//   tangential (non-DF) .... src/reconstruction.cpp:2233-2551 (WENO5_AO_tangent, 2 pts)
//   tangential recon (DF) .. src/reconstruction.cpp:2553-2838 (WENO5, 2 pts),
//                            2840-3174 (WENO7, 3 pts), 3176-3609 (WENO9, 4 pts + Polynomial_9th)
//   positivity fallback .... src/reconstruction.cpp:1439-1449
//   g0 centre state ........ src/reconstruction.cpp:3652-3687 (computed once, inside the flux,
//                            as GKS2D recomputes it anyway: src/flux_function.cpp:369-401)
//   GKS2D flux ............. src/flux_function.cpp:317-343, 345-698
//   Maxwellian moments ..... src/basic_function.cpp:110-187 (MMDF2d), 561-636 (Collision, A,
//                            GL/GR/G_address), 638-719 (Get_Tau*, Alpha, Beta)
//   characteristic vars .... src/basic_function.cpp:923-992
//   S2O4 update ............ src/time_advance.cpp:221-230, 307-474
//   DF factor .............. src/reconstruction.cpp:1451-1534
//
// Arithmetic follows the reference expression by expression (same operand order, x*x for
// pow(x, 2), integer divisions 13/3 == 4 and 781/20 == 39 kept) so that, compiled with
// -ffp-contract=off, it reproduces the reference bit for bit.  Deliberate differences:
//   * Update_alpha's j loop bound uses nodex (src/reconstruction.cpp:1528); this restatement
//     bounds j by min(nodex, nodey), identical on the square grids the workloads use.
//   * No console output, no exit(): errors come back as status codes.
#include "oracle_api.h"
#include "oracle_weno.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

using namespace oracle_weno;

// ----------------------------------------------------------------------------------------
// configuration and state
// ----------------------------------------------------------------------------------------
struct Config {
    hos2d_params p;
    int nx = 0, ny = 0, g = 0, gp = 0;
    double dx = 0, dy = 0;
    double gloc[4] = {0, 0, 0, 0};
    double gw[4] = {0, 0, 0, 0};
    double K = 0, Gamma = 0;
    double tbeg = 0;   // Block2d::t during the step (read by the wedge boundary)
    int stages = 2;
    double tc[5][5][2] = {};   // Block2d::timecoefficient of the time-marching method
    int first_order = 0;       // First_order_normal / _tangent in the reconstruction slots
    int source = 0;            // Update_with_source instead of Update (gravity source)
};
Config C;

struct Point { double convar[4], der1x[4], der1y[4]; };
struct Recon { Point left, right, center; };

std::vector<double> W, Wold, Prim, AX, AY;   // per cell: 4, 4, 4, 1, 1
std::vector<Point> XL, YL;                    // line states: [face][side] (side 0 left, 1 right)
std::vector<Recon> XG, YG;                    // Gauss states: [face][gp]
std::vector<double> XF, YF;                   // flux: [face][stage (4)][gp][8] (f[4], derf[4])
std::vector<double> XX, YX;                   // stage flux combination x[4]: [face][gp][4]

inline int cell(int i, int j) { return i * C.ny + j; }
inline int face(int i, int j) { return i * (C.ny + 1) + j; }

// time-marching coefficients tc[stage][k][f or derf] (S1O1_2D ... RK4_2D,
// src/time_advance.cpp:197-247); RK3 has its own state combination (:476-532)
void set_integrator(int integrator) {
    for (auto& a : C.tc)
        for (auto& b : a) b[0] = b[1] = 0.0;
    switch (integrator) {
        case 0:  // S2O4
            C.stages = 2;
            C.tc[0][0][0] = 0.5; C.tc[0][0][1] = 1.0 / 8.0;
            C.tc[1][0][0] = 1.0; C.tc[1][1][0] = 0.0; C.tc[1][0][1] = 1.0 / 6.0; C.tc[1][1][1] = 1.0 / 3.0;
            break;
        case 1:  // S1O1
            C.stages = 1;
            C.tc[0][0][0] = 1.0; C.tc[0][0][1] = 0.0;
            break;
        case 2:  // S1O2
            C.stages = 1;
            C.tc[0][0][0] = 1.0; C.tc[0][0][1] = 0.5;
            break;
        case 3:  // RK2
            C.stages = 2;
            C.tc[0][0][0] = 1.0; C.tc[1][0][0] = 0.5; C.tc[1][1][0] = 0.5;
            break;
        case 4:  // RK3
            C.stages = 3;
            break;
        default:  // RK4
            C.stages = 4;
            C.tc[0][0][0] = 0.5; C.tc[1][1][0] = 0.5; C.tc[2][2][0] = 1.0;
            C.tc[3][0][0] = 1.0 / 6.0; C.tc[3][1][0] = 1.0 / 3.0; C.tc[3][2][0] = 1.0 / 3.0; C.tc[3][3][0] = 1.0 / 6.0;
    }
}

// ----------------------------------------------------------------------------------------
// conversions (src/basic_function.cpp:811-842, 1102-1177)
// ----------------------------------------------------------------------------------------
inline void to_prim(double* pr, const double* w) {
    pr[0] = w[0];
    pr[1] = w[1] / w[0];
    pr[2] = w[2] / w[0];
    pr[3] = (C.Gamma - 1.0) * (w[3] - 0.5 * w[1] * w[1] / w[0] - 0.5 * w[2] * w[2] / w[0]);
}
inline double lambda_of(double rho, double u, double v, double rhoE) {
    return (C.K + 2.0) * 0.25 * (rho / (rhoE - 0.5 * rho * (u * u + v * v)));
}
inline void to_ulambda(double* pr, const double* w) {
    pr[0] = w[0];
    pr[1] = w[1] / w[0];
    pr[2] = w[2] / w[0];
    pr[3] = lambda_of(w[0], pr[1], pr[2], w[3]);
}
inline void prim_to_con(double* w, const double* pr) {
    w[0] = pr[0];
    w[1] = pr[0] * pr[1];
    w[2] = pr[0] * pr[2];
    w[3] = pr[0] * (pr[3] / pr[0] / (C.Gamma - 1) + 0.5 * (pr[1] * pr[1] + pr[2] * pr[2]));
}
// (u, v) -> (v, -u): y-face quantities in the x-face frame (YchangetoX, :1192-1198)
inline void rot_y_to_x(double* o, const double* w) { o[0] = w[0]; o[1] = w[2]; o[2] = -w[1]; o[3] = w[3]; }
// inverse rotation (XchangetoY, :1200-1206)
inline void rot_x_to_y(double* o, const double* w) { o[0] = w[0]; o[1] = -w[2]; o[2] = w[1]; o[3] = w[3]; }

// characteristic projection with base primitive state (Convar_to_char, :960-992)
inline void to_char(double* ch, const double* base, const double* w) {
    double c = std::sqrt(C.Gamma * base[3] / base[0]);
    double overc = 1.0 / c;
    double alfa = (C.Gamma - 1.0) * 0.5 * overc * overc;
    double u = base[1], v = base[2];
    double s[4][4];
    s[0][0] = 1.0 - alfa * (u * u + v * v); s[0][1] = 2.0 * alfa * u; s[0][2] = 2.0 * alfa * v; s[0][3] = -2.0 * alfa;
    s[1][0] = -v; s[1][1] = 0.; s[1][2] = 1.; s[1][3] = 0.;
    s[2][0] = 0.5 * (-u * overc + alfa * (u * u + v * v)); s[2][1] = 0.5 * overc - alfa * u; s[2][2] = -alfa * v; s[2][3] = alfa;
    s[3][0] = 0.5 * (u * overc + alfa * (u * u + v * v)); s[3][1] = -0.5 * overc - alfa * u; s[3][2] = -alfa * v; s[3][3] = alfa;
    for (int r = 0; r < 4; ++r) {
        double acc = 0;
        for (int k = 0; k < 4; ++k) acc = acc + s[r][k] * w[k];
        ch[r] = acc;
    }
}
// back-projection (Char_to_convar, :958-992 region, right eigenvectors)
inline void from_char(double* w, const double* base, const double* ch) {
    double c = std::sqrt(C.Gamma * base[3] / base[0]);
    double u = base[1], v = base[2];
    double s[4][4];
    s[0][0] = 1.; s[0][1] = 0.0; s[0][2] = 1.0; s[0][3] = 1.0;
    s[1][0] = u; s[1][1] = 0.; s[1][2] = u + c; s[1][3] = u - c;
    s[2][0] = v; s[2][1] = 1.; s[2][2] = v; s[2][3] = v;
    s[3][0] = 0.5 * (u * u + v * v); s[3][1] = v;
    s[3][2] = 0.5 * (u * u + v * v) + c * u + c * c / (C.Gamma - 1.0);
    s[3][3] = 0.5 * (u * u + v * v) - c * u + c * c / (C.Gamma - 1.0);
    for (int r = 0; r < 4; ++r) {
        double acc = 0;
        for (int k = 0; k < 4; ++k) acc = acc + s[r][k] * ch[k];
        w[r] = acc;
    }
}
// positivity check of a reconstructed state (Check_Order_Reduce_by_Lambda_2D, :1439-1449)
inline bool needs_order_reduction(const double* w) {
    double lam = lambda_of(w[0], w[1] / w[0], w[2] / w[0], w[3]);
    return lam <= 0.0 || !(lam == lam);
}

// scalar tangential reconstruction at all Gauss points of one face side
void weno_tangent(int order, const double* s, const double* df, double h, double* g, double* gx) {
    if (!C.p.use_df) {   // non-DF WENO5-AO at the 2 Gauss points (WENO5_AO_tangential, :2244-2391)
        weno5_2gauss(s, h, true, g, gx, C.p.wenotype);
        return;
    }
    double fw[6], p[6], px[6];
    int n = ao_weights(order, s, fw);
    for (int ig = 0; ig < C.gp; ++ig) {
        tangent_points(order, ig, s, df, h, p, px);
        double a = 0.0, b = 0.0;
        for (int k = 0; k < n; ++k) {
            a += fw[k] * p[k];
            b += fw[k] * px[k];
        }
        g[ig] = a;
        gx[ig] = b;
    }
}

// ----------------------------------------------------------------------------------------
// normal reconstruction of one cell in one direction (WENO*_AO_with_df, :1731-1859 etc.)
//   st[k][4]: stencil of cell states (already rotated for y), al[]: DF alpha along it.
//   Lp: value/slope at the cell's left (lower) face, Rp: at its right (upper) face.
// ----------------------------------------------------------------------------------------
void normal_cell(int order, const double (*st)[4], const double* al, double h, Point& Lp, Point& Rp) {
    const int r = order / 2, n = order;
    if (C.first_order) {  // First_order_normal (src/reconstruction.cpp:1537-1560)
        for (int v = 0; v < 4; ++v) {
            Lp.convar[v] = st[r][v];
            Rp.convar[v] = st[r][v];
            Lp.der1x[v] = 0.0;
            Rp.der1x[v] = 0.0;
        }
        return;
    }
    double df[6];
    df_factors(order, al, df);
    double pn1[4], p0[4], pp1[4], bl[4], br[4];
    to_prim(pn1, st[r - 1]);
    to_prim(p0, st[r]);
    to_prim(pp1, st[r + 1]);
    for (int v = 0; v < 4; ++v) {
        bl[v] = 0.5 * (pn1[v] + p0[v]);
        br[v] = 0.5 * (pp1[v] + p0[v]);
    }
    double ch[9][4], s[9], var[4], der[4];
    for (int side = 0; side < 2; ++side) {
        const double* base = side == 0 ? bl : br;
        for (int k = 0; k < n; ++k) {
            if (C.p.characteristic) to_char(ch[k], base, st[k]);
            else for (int v = 0; v < 4; ++v) ch[k][v] = st[k][v];
        }
        for (int v = 0; v < 4; ++v) {
            for (int k = 0; k < n; ++k) s[k] = ch[k][v];
            if (C.p.use_df) weno_normal(order, side, s, df, h, var[v], der[v]);
            else weno5_plain(side, s, h, var[v], der[v], C.p.wenotype);   // WENO5_AO, :1589-1699
        }
        Point& P = side == 0 ? Lp : Rp;
        if (C.p.characteristic) {
            from_char(P.convar, base, var);
            from_char(P.der1x, base, der);
        } else {
            for (int v = 0; v < 4; ++v) { P.convar[v] = var[v]; P.der1x[v] = der[v]; }
        }
    }
    bool rr = needs_order_reduction(Rp.convar);
    bool rl = needs_order_reduction(Lp.convar);
    if (rl || rr) {
        for (int v = 0; v < 4; ++v) {
            Rp.convar[v] = st[r][v];
            Lp.convar[v] = st[r][v];
            Rp.der1x[v] = 0.0;
            Lp.der1x[v] = 0.0;
        }
    }
}

// ----------------------------------------------------------------------------------------
// tangential reconstruction of one face (weno_*th_ao_with_df_tangential, :2578-2791 etc.)
//   ln[k][2]: line states (side 0 = left of face, 1 = right) along the face,
//   a1/a2: DF alpha of the left / right cell column.  Writes gp Gauss states.
//   For order 9 the right side reuses the left side's characteristic projection of the
//   outermost stencil entries, as the reference does (:3318-3327: ren4/rep4 are not
//   re-projected with the right base).
// ----------------------------------------------------------------------------------------
void tangent_face(int order, const Point (*ln)[2], const double* a1, const double* a2, double h, Recon* re) {
    const int r = order / 2, n = order, gp = C.gp;
    if (C.first_order) {  // First_order_tangent (src/reconstruction.cpp:2214-2231)
        for (int side = 0; side < 2; ++side)
            for (int ig = 0; ig < gp; ++ig) {
                Point& P = side == 0 ? re[ig].left : re[ig].right;
                for (int v = 0; v < 4; ++v) {
                    P.convar[v] = ln[r][side].convar[v];
                    P.der1x[v] = ln[r][side].der1x[v];
                    P.der1y[v] = 0.0;
                }
            }
        return;
    }
    double df[2][6];
    df_factors(order, a1, df[0]);
    df_factors(order, a2, df[1]);
    double ch[9][4], s[9];
    for (int side = 0; side < 2; ++side) {
        const Point& w0 = ln[r][side];
        double base[4];
        to_prim(base, w0.convar);
        double var[4][4], der[4][4];
        if (C.p.characteristic) {
            for (int k = 0; k < n; ++k) {
                if (order == 9 && side == 1 && (k == 0 || k == n - 1)) continue;  // reference quirk
                to_char(ch[k], base, ln[k][side].convar);
            }
            for (int v = 0; v < 4; ++v) {
                for (int k = 0; k < n; ++k) s[k] = ch[k][v];
                double g[4], gx[4];
                weno_tangent(order, s, df[side], h, g, gx);
                for (int ig = 0; ig < gp; ++ig) { var[ig][v] = g[ig]; der[ig][v] = gx[ig]; }
            }
            for (int ig = 0; ig < gp; ++ig) {
                Point& P = side == 0 ? re[ig].left : re[ig].right;
                from_char(P.convar, base, var[ig]);
                from_char(P.der1y, base, der[ig]);
            }
        } else {
            for (int v = 0; v < 4; ++v) {
                for (int k = 0; k < n; ++k) s[k] = ln[k][side].convar[v];
                double g[4], gx[4];
                weno_tangent(order, s, df[side], h, g, gx);
                for (int ig = 0; ig < gp; ++ig) {
                    Point& P = side == 0 ? re[ig].left : re[ig].right;
                    P.convar[v] = g[ig];
                    P.der1y[v] = gx[ig];
                }
            }
        }
        // normal slope reconstructed in conservative variables
        for (int v = 0; v < 4; ++v) {
            for (int k = 0; k < n; ++k) s[k] = ln[k][side].der1x[v];
            double g[4], gx[4];
            weno_tangent(order, s, df[side], h, g, gx);
            for (int ig = 0; ig < gp; ++ig) {
                Point& P = side == 0 ? re[ig].left : re[ig].right;
                P.der1x[v] = g[ig];
            }
        }
    }
    for (int side = 0; side < 2; ++side)
        for (int ig = 0; ig < gp; ++ig) {
            Point& P = side == 0 ? re[ig].left : re[ig].right;
            if (needs_order_reduction(P.convar)) {
                const Point& w0 = ln[r][side];
                for (int v = 0; v < 4; ++v) {
                    P.convar[v] = w0.convar[v];
                    P.der1x[v] = w0.der1x[v];
                    P.der1y[v] = 0.0;
                }
            }
        }
}

// ----------------------------------------------------------------------------------------
// Maxwellian moments (MMDF2d, src/basic_function.cpp:110-187)
// ----------------------------------------------------------------------------------------
struct Moments {
    double uwhole[7], uplus[7], uminus[7], vwhole[7];
    double up[7][7][3], un[7][7][3], uv[7][7][3];
    double xi2, xi4;
};
void moments(Moments& m, double u, double v, double lambda) {
    const double pi = 3.14159265358979323846;
    m.uwhole[0] = 1;
    m.uwhole[1] = u;
    m.uplus[0] = 0.5 * std::erfc(std::sqrt(lambda) * -u);
    m.uminus[0] = 1.0 - m.uplus[0];
    m.uplus[1] = u * m.uplus[0] + 0.5 * (std::exp(-lambda * u * u) / std::sqrt(pi * lambda));
    m.uminus[1] = u - m.uplus[1];
    double ol = 1.0 / lambda;
    for (int i = 2; i <= 6; ++i) m.uwhole[i] = u * m.uwhole[i - 1] + 0.5 * (i - 1) * ol * m.uwhole[i - 2];
    for (int i = 2; i <= 6; ++i) {
        m.uplus[i] = u * m.uplus[i - 1] + 0.5 * (i - 1) * ol * m.uplus[i - 2];
        m.uminus[i] = m.uwhole[i] - m.uplus[i];
    }
    m.vwhole[0] = 1;
    m.vwhole[1] = v;
    for (int i = 2; i <= 6; ++i) m.vwhole[i] = v * m.vwhole[i - 1] + 0.5 * (i - 1) * ol * m.vwhole[i - 2];
    m.xi2 = 0.5 * C.K * ol;
    m.xi4 = 0.25 * (C.K * C.K + 2 * C.K) * ol * ol;
    for (int i = 0; i < 7; ++i)
        for (int j = 0; j < 7; ++j)
            for (int k = 0; k < 3; ++k)
                if (i + j + 2 * k <= 6) {
                    if (k == 0) {
                        m.up[i][j][k] = m.uplus[i] * m.vwhole[j];
                        m.un[i][j][k] = m.uminus[i] * m.vwhole[j];
                    } else {
                        double xi = k == 1 ? m.xi2 : m.xi4;
                        m.up[i][j][k] = m.uplus[i] * m.vwhole[j] * xi;
                        m.un[i][j][k] = m.uminus[i] * m.vwhole[j] * xi;
                    }
                    m.uv[i][j][k] = m.up[i][j][k] + m.un[i][j][k];
                }
}
// moment contraction <a psi u^nu v^nv> over a table (GL/GR/G_address, :603-636)
void contract(const double (*M)[7][3], int nu, int nv, const double* a, double* psi) {
    const int u = nu, v = nv;
    psi[0] = a[0] * M[u][v][0] + a[1] * M[u + 1][v][0] + a[2] * M[u][v + 1][0] + a[3] * 0.5 * (M[u + 2][v][0] + M[u][v + 2][0] + M[u][v][1]);
    psi[1] = a[0] * M[u + 1][v][0] + a[1] * M[u + 2][v][0] + a[2] * M[u + 1][v + 1][0] + a[3] * 0.5 * (M[u + 3][v][0] + M[u + 1][v + 2][0] + M[u + 1][v][1]);
    psi[2] = a[0] * M[u][v + 1][0] + a[1] * M[u + 1][v + 1][0] + a[2] * M[u][v + 2][0] + a[3] * 0.5 * (M[u + 2][v + 1][0] + M[u][v + 3][0] + M[u][v + 1][1]);
    psi[3] = 0.5 * (a[0] * (M[u + 2][v][0] + M[u][v + 2][0] + M[u][v][1]) +
                    a[1] * (M[u + 3][v][0] + M[u + 1][v + 2][0] + M[u + 1][v][1]) +
                    a[2] * (M[u + 2][v + 1][0] + M[u][v + 3][0] + M[u][v + 1][1]) +
                    a[3] * 0.5 * (M[u + 4][v][0] + M[u][v + 4][0] + M[u][v][2] + 2 * M[u + 2][v + 2][0] + 2 * M[u + 2][v][1] + 2 * M[u][v + 2][1]));
}
// micro-slope from a macroscopic slope (A, :571-583)
void microslope(double* a, const double* der, const double* prim) {
    double overden = 1.0 / prim[0];
    double R4 = der[3] * overden - 0.5 * (prim[1] * prim[1] + prim[2] * prim[2] + 0.5 * (C.K + 2) / prim[3]) * der[0] * overden;
    double R3 = (der[2] - prim[2] * der[0]) * overden;
    double R2 = (der[1] - prim[1] * der[0]) * overden;
    a[3] = (4.0 / (C.K + 2)) * prim[3] * prim[3] * (2 * R4 - 2 * prim[1] * R2 - 2 * prim[2] * R3);
    a[2] = 2 * prim[3] * R3 - prim[2] * a[3];
    a[1] = 2 * prim[3] * R2 - prim[1] * a[3];
    a[0] = der[0] * overden - prim[1] * a[1] - prim[2] * a[2] - 0.5 * a[3] * (prim[1] * prim[1] + prim[2] * prim[2] + 0.5 * (C.K + 2) / prim[3]);
}
// Get_Tau (src/basic_function.cpp:663-708): Euler numerical collision time, or the
// Navier-Stokes one (numerical part c2 |.| dt plus the physical 2 Mu lambda0 / rho0)
double tau_num(double dl, double dr, double ll, double lr, double dt, double d0 = 0.0, double l0 = 0.0) {
    if (C.p.tau_type == 1) {
        double tn = C.p.c2_euler * std::abs(dl / ll - dr / lr) / std::abs(dl / ll + dr / lr) * dt;
        if (tn != tn) tn = 0.0;
        if ((C.p.mu > 0.0 && C.p.nu > 0.0) || (C.p.mu < 0.0 && C.p.nu < 0.0)) return 0.0;
        if (C.p.mu > 0.0) return tn + 2.0 * C.p.mu * l0 / d0;
        if (C.p.nu > 0.0) return tn + 2 * C.p.nu * l0;
        return 0.0;
    }
    if (C.p.c1_euler <= 0 && C.p.c2_euler <= 0) return 0.0;
    double Cc = C.p.c2_euler * std::abs(dl / ll - dr / lr) / std::abs(dl / ll + dr / lr);
    return C.p.c1_euler * dt + dt * Cc;
}
// Get_Tau_NS (:638-661)
double tau_ns(double d0, double l0) {
    if (C.p.tau_type != 1) return 0.0;
    if (C.p.mu > 0.0) return 2.0 * C.p.mu * l0 / d0;
    if (C.p.nu > 0.0) return 2 * C.p.nu * l0;
    return 0.0;
}

// ----------------------------------------------------------------------------------------
// Centre (g0) state of a Gauss point by collision, with its x and y slopes from the left and
// right micro-slopes (Center_all_collision_2d_multi, src/reconstruction.cpp:3652-3687; GKS2D
// recomputes the same state, src/flux_function.cpp:369-401).  ml, mr: the sides' moments.
// ----------------------------------------------------------------------------------------
void centre_state(Recon& re, const double* pl, const double* pr, const Moments& ml, const Moments& mr) {
    double* w0 = re.center.convar;
    w0[0] = pl[0] * ml.uplus[0] + pr[0] * mr.uminus[0];
    w0[1] = pl[0] * ml.uplus[1] + pr[0] * mr.uminus[1];
    w0[2] = pl[0] * ml.vwhole[1] * ml.uplus[0] + pr[0] * mr.vwhole[1] * mr.uminus[0];
    w0[3] = 0.5 * pl[0] * (ml.uplus[2] + ml.uplus[0] * ml.vwhole[2] + ml.uplus[0] * ml.xi2) +
            0.5 * pr[0] * (mr.uminus[2] + mr.uminus[0] * mr.vwhole[2] + mr.uminus[0] * mr.xi2);
    {
        double alx[4], arx[4], al0x[4], ar0x[4], aly[4], ary[4], al0y[4], ar0y[4];
        microslope(alx, re.left.der1x, pl);
        microslope(arx, re.right.der1x, pr);
        contract(ml.up, 0, 0, alx, al0x);
        contract(mr.un, 0, 0, arx, ar0x);
        microslope(aly, re.left.der1y, pl);
        microslope(ary, re.right.der1y, pr);
        contract(ml.up, 0, 0, aly, al0y);
        contract(mr.un, 0, 0, ary, ar0y);
        for (int v = 0; v < 4; ++v) {
            re.center.der1x[v] = pl[0] * al0x[v] + pr[0] * ar0x[v];
            re.center.der1y[v] = pl[0] * al0y[v] + pr[0] * ar0y[v];
        }
    }
}

// ----------------------------------------------------------------------------------------
// GKS2D at one Gauss point (src/flux_function.cpp:345-698, gks2nd, Euler tau, S2O4 branch):
// centre state by collision (also stored in re.center), the full second-order flux over
// [0, dt] and [0, dt/2], combined into f = 4F(dt/2) - F(dt), derf = 4(F(dt) - 2F(dt/2)).
// ----------------------------------------------------------------------------------------
void gks2d(Recon& re, double dt, double* fo, double* dfo, bool one_level) {
    double pl[4], pr[4], p0[4];
    to_ulambda(pl, re.left.convar);
    to_ulambda(pr, re.right.convar);
    Moments ml, mr;
    moments(ml, pl[1], pl[2], pl[3]);
    moments(mr, pr[1], pr[2], pr[3]);
    centre_state(re, pl, pr, ml, mr);
    to_ulambda(p0, re.center.convar);
    const double tau = tau_ns(p0[0], p0[3]);
    double tn = tau_num(pl[0], pr[0], pl[3], pr[3], dt, p0[0], p0[3]);
    double eta = std::exp(-dt / tn);
    double t[6];
    t[0] = tn * (1 - eta);
    t[1] = tn * (eta * (dt + tn) - tn) + tau * tn * (eta - 1);
    t[2] = tau * tn * (eta - 1);
    t[3] = tn * eta + dt - tn;
    t[4] = tn * (tn - eta * (dt + tn) - tau * (eta - 1)) - dt * tau;
    t[5] = 0.5 * dt * dt - tau * tn * (eta - 1) - tau * dt;
    const double unit[4] = {1, 0.0, 0.0, 0.0};
    double F0[4], F1[4];
    double glu[4], gru[4];
    contract(ml.up, 1, 0, unit, glu);
    contract(mr.un, 1, 0, unit, gru);
    for (int i = 0; i < 4; ++i) F0[i] = pl[0] * t[0] * glu[i] + pr[0] * t[0] * gru[i];
    Moments m0;
    moments(m0, p0[1], p0[2], p0[3]);
    double g0u[4];
    contract(m0.uv, 1, 0, unit, g0u);
    for (int i = 0; i < 4; ++i) F0[i] = F0[i] + p0[0] * t[3] * g0u[i];
    double alx[4], alxuul[4], arx[4], arxuur[4], aly[4], alyuvl[4], ary[4], aryuvr[4];
    microslope(alx, re.left.der1x, pl);
    contract(ml.up, 2, 0, alx, alxuul);
    microslope(arx, re.right.der1x, pr);
    contract(mr.un, 2, 0, arx, arxuur);
    microslope(aly, re.left.der1y, pl);
    contract(ml.up, 1, 1, aly, alyuvl);
    microslope(ary, re.right.der1y, pr);
    contract(mr.un, 1, 1, ary, aryuvr);
    for (int i = 0; i < 4; ++i) F0[i] = F0[i] + t[1] * (pl[0] * (alxuul[i] + alyuvl[i]) + pr[0] * (arxuur[i] + aryuvr[i]));
    double alxu[4], alyv[4], arxu[4], aryv[4];
    contract(ml.uv, 1, 0, alx, alxu);
    contract(mr.uv, 1, 0, arx, arxu);
    contract(ml.uv, 0, 1, aly, alyv);
    contract(mr.uv, 0, 1, ary, aryv);
    double Al[4], Ar[4], dAL[4], dAR[4];
    for (int i = 0; i < 4; ++i) {
        dAL[i] = -pl[0] * (alxu[i] + alyv[i]);
        dAR[i] = -pr[0] * (arxu[i] + aryv[i]);
    }
    microslope(Al, dAL, pl);
    microslope(Ar, dAR, pr);
    double Alul[4], Arur[4];
    contract(ml.up, 1, 0, Al, Alul);
    contract(mr.un, 1, 0, Ar, Arur);
    for (int i = 0; i < 4; ++i) F0[i] = F0[i] + t[2] * (pl[0] * Alul[i] + pr[0] * Arur[i]);
    double a0x[4], a0xu[4], a0xuu[4], a0y[4], a0yv[4], a0yuv[4];
    microslope(a0x, re.center.der1x, p0);
    contract(m0.uv, 1, 0, a0x, a0xu);
    contract(m0.uv, 2, 0, a0x, a0xuu);
    microslope(a0y, re.center.der1y, p0);
    contract(m0.uv, 0, 1, a0y, a0yv);
    contract(m0.uv, 1, 1, a0y, a0yuv);
    for (int i = 0; i < 4; ++i) F0[i] = F0[i] + p0[0] * t[4] * (a0xuu[i] + a0yuv[i]);
    double dA0[4], A0[4], A0u[4];
    for (int i = 0; i < 4; ++i) dA0[i] = -p0[0] * (a0xu[i] + a0yv[i]);
    microslope(A0, dA0, p0);
    contract(m0.uv, 1, 0, A0, A0u);
    for (int i = 0; i < 4; ++i) F0[i] = F0[i] + p0[0] * t[5] * (A0u[i]);
    if (C.p.prandtl_fix) {   // heat-flux correction (:630-636)
        double qs = a0xuu[3] + A0u[3] - p0[1] * (a0xuu[1] + A0u[1]) - p0[2] * (a0xuu[2] + A0u[2]);
        qs *= -p0[0] * tau * dt;
        F0[3] += (1.0 / C.p.prandtl - 1.0) * qs;
    }
    if (one_level) {   // S1O1 takes the dt integral alone (:637-645)
        for (int i = 0; i < 4; ++i) {
            fo[i] = F0[i];
            dfo[i] = 0.0;
        }
        return;
    }
    // second time level dt/2 (:647-676)
    double dt2 = 0.5 * dt;
    tn = tau_num(pl[0], pr[0], pl[3], pr[3], dt2, p0[0], p0[3]);
    eta = std::exp(-dt2 / tn);
    t[0] = tn * (1 - eta);
    t[1] = tn * (eta * (dt2 + tn) - tn) + tau * tn * (eta - 1);
    t[2] = tau * tn * (eta - 1);
    t[3] = tn * eta + dt2 - tn;
    t[4] = tn * (tn - eta * (dt2 + tn) - tau * (eta - 1)) - dt2 * tau;
    t[5] = 0.5 * dt2 * dt2 - tau * tn * (eta - 1) - tau * dt2;
    for (int i = 0; i < 4; ++i) {
        F1[i] = t[0] * (pl[0] * glu[i] + pr[0] * gru[i]);
        F1[i] = F1[i] + t[1] * (pl[0] * (alxuul[i] + alyuvl[i]) + pr[0] * (arxuur[i] + aryuvr[i]));
        F1[i] = F1[i] + t[2] * (pl[0] * Alul[i] + pr[0] * Arur[i]);
        F1[i] = F1[i] + p0[0] * t[3] * g0u[i];
        F1[i] = F1[i] + p0[0] * t[4] * (a0xuu[i] + a0yuv[i]);
        F1[i] = F1[i] + p0[0] * t[5] * (A0u[i]);
    }
    if (C.p.prandtl_fix) {   // (:678-684)
        double qs = a0xuu[3] + A0u[3] - p0[1] * (a0xuu[1] + A0u[1]) - p0[2] * (a0xuu[2] + A0u[2]);
        qs *= -p0[0] * tau * 0.5 * dt;
        F1[3] += (1.0 / C.p.prandtl - 1.0) * qs;
    }
    for (int i = 0; i < 4; ++i) {
        fo[i] = (4.0 * F1[i] - F0[i]);
        dfo[i] = 4.0 * (F0[i] - 2.0 * F1[i]);
    }
}

// LF2D's viscous term (NS_by_central_difference_prim_2D, src/flux_function.cpp:737-754), as
// written: it reads the centre state's entries as (rho, u, v, T) and their slopes, while the
// centre state holds conserved variables (rho, rho u, rho v, rho E) and their slopes; mu = Mu,
// or Nu rho when Nu > 0; the heat-flux factor (K + 4) / (2 Pr).
void ns_central(const Recon& re, double dt, double* fo) {
    double mu = C.p.mu;
    if (C.p.nu > 0) mu = C.p.nu * re.center.convar[0];
    const double u = re.center.convar[1];
    const double v = re.center.convar[2];
    const double ux = re.center.der1x[1];
    const double vx = re.center.der1x[2];
    const double uy = re.center.der1y[1];
    const double vy = re.center.der1y[2];
    const double tau_xx = 2 * mu * ux - 2.0 / 3.0 * mu * (ux + vy);
    const double tau_xy = mu * (uy + vx);
    const double q = u * tau_xx + v * tau_xy + (C.K + 4) / (2 * C.p.prandtl) * mu * re.center.der1x[3];
    fo[1] += tau_xx * dt;
    fo[2] += tau_xy * dt;
    fo[3] += q * dt;
}

// Lax-Friedrichs flux times dt at a Gauss point (LF2D, src/flux_function.cpp:700-735); with
// the Navier-Stokes collision time its viscous term is added.  That term reads the centre
// state, which the reference computes only for GKS2D (Center_all_collision_multi returns for
// other fluxes, src/reconstruction.cpp:3642-3650, and leaves the Gauss points' centre states
// as allocated, uninitialised); here it is the collision state GKS2D would use.
void lf2d(Recon& re, double dt, double* fo, double* dfo) {
    double pl[4], pr[4];
    to_prim(pl, re.left.convar);
    to_prim(pr, re.right.convar);
    const double kl = std::abs(pl[1]) + std::sqrt(C.Gamma * pl[3] / pl[0]);
    const double kr = std::abs(pr[1]) + std::sqrt(C.Gamma * pr[3] / pr[0]);
    const double beta = kr > kl ? kr : kl;
    auto flux = [](const double* q, double* f) {
        f[0] = q[0] * q[1];
        f[1] = q[0] * q[1] * q[1] + q[3];
        f[2] = q[0] * q[1] * q[2];
        const double e = 0.5 * (q[1] * q[1] + q[2] * q[2]) * q[0] + q[3] / (C.Gamma - 1.0);
        f[3] = q[1] * (e + q[3]);
    };
    double fl[4], fr[4];
    flux(pl, fl);
    flux(pr, fr);
    for (int m = 0; m < 4; ++m) {
        fo[m] = 0.5 * ((fl[m] + fr[m]) - beta * (re.right.convar[m] - re.left.convar[m]));
        fo[m] *= dt;
        dfo[m] = 0.0;
    }
    if (C.p.tau_type == 1) {
        double ql[4], qr[4];
        to_ulambda(ql, re.left.convar);
        to_ulambda(qr, re.right.convar);
        Moments ml, mr;
        moments(ml, ql[1], ql[2], ql[3]);
        moments(mr, qr[1], qr[2], qr[3]);
        centre_state(re, ql, qr, ml, mr);
        ns_central(re, dt, fo);
    }
}

// ----------------------------------------------------------------------------------------
// boundary conditions, applied left, right, down, up as the drivers do
// ----------------------------------------------------------------------------------------
void bc_side(int side) {
    const int nx = C.nx, ny = C.ny, g = C.g;
    const int kind = C.p.bc[side];
    auto copy = [&](int dst, int src, int flipv) {
        for (int v = 0; v < 4; ++v) W[4 * dst + v] = W[4 * src + v];
        if (flipv) W[4 * dst + flipv] = -W[4 * src + flipv];
    };
    double inflow[4];
    prim_to_con(inflow, C.p.bc_prim[side]);
    // noslip_adiabatic_boundary_* (src/boundary_condition.cpp:290-365): mirrored cell, density
    // and energy copied, both momentum components 2 rho u_wall - rho u
    auto noslip = [&](int dst, int src) {
        W[4 * dst + 0] = W[4 * src + 0];
        W[4 * dst + 1] = 2 * W[4 * dst + 0] * C.p.bc_prim[side][1] - W[4 * src + 1];
        W[4 * dst + 2] = 2 * W[4 * dst + 0] * C.p.bc_prim[side][2] - W[4 * src + 2];
        W[4 * dst + 3] = W[4 * src + 3];
    };
    if (side == 0 || side == 1) {
        for (int k = 0; k < g; ++k) {
            int i = side == 0 ? g - 1 - k : nx - g + k;  // same sweep order as the reference
            for (int j = 0; j < ny; ++j) {
                int dst = cell(i, j);
                if (kind == HOS_BC_FREE) copy(dst, cell(side == 0 ? i + 1 : i - 1, j), 0);
                else if (kind == HOS_BC_PERIODIC) copy(dst, cell(side == 0 ? i + C.p.nodex : i - C.p.nodex, j), 0);
                else if (kind == HOS_BC_REFLECT) copy(dst, cell(side == 0 ? 2 * g - 1 - i : 2 * nx - 2 * g - 1 - i, j), 1);
                else if (kind == HOS_BC_NOSLIP) noslip(dst, cell(side == 0 ? 2 * g - 1 - i : 2 * nx - 2 * g - 1 - i, j));
                else for (int v = 0; v < 4; ++v) W[4 * dst + v] = inflow[v];
            }
        }
    } else if (kind == HOS_BC_WEDGE_TOP || kind == HOS_BC_WEDGE_BOTTOM) {
        // boundaryforDoubleMach top / bottom parts (src/2Dproblem.cpp:1041-1092), i >= ghost
        double post[4], pre[4];
        prim_to_con(post, C.p.wedge_post);
        prim_to_con(pre, C.p.wedge_pre);
        const double height = C.p.up - C.p.down;
        for (int k = 0; k < g; ++k) {
            const int j = side == 2 ? g - 1 - k : ny - g + k;
            for (int i = g; i < nx; ++i) {
                const int dst = cell(i, j);
                const double coordx = C.p.left + (i + 0.5 - g) * C.dx;
                if (kind == HOS_BC_WEDGE_TOP) {
                    const double* st = coordx < (C.p.wedge_x0 + height / std::sqrt(3.0) + C.p.wedge_top_speed * C.tbeg) ? post : pre;
                    for (int v = 0; v < 4; ++v) W[4 * dst + v] = st[v];
                } else if (coordx < C.p.wedge_x0) {
                    for (int v = 0; v < 4; ++v) W[4 * dst + v] = post[v];
                } else {
                    copy(dst, cell(i, 2 * g - 1 - j), 2);
                }
            }
        }
    } else {
        for (int k = 0; k < g; ++k) {
            int j = side == 2 ? g - 1 - k : ny - g + k;
            for (int i = 0; i < nx; ++i) {
                int dst = cell(i, j);
                if (kind == HOS_BC_FREE) copy(dst, cell(i, side == 2 ? j + 1 : j - 1), 0);
                else if (kind == HOS_BC_PERIODIC) copy(dst, cell(i, side == 2 ? j + C.p.nodey : j - C.p.nodey), 0);
                else if (kind == HOS_BC_REFLECT) copy(dst, cell(i, side == 2 ? 2 * g - 1 - j : 2 * ny - 2 * g - 1 - j), 2);
                else if (kind == HOS_BC_NOSLIP) noslip(dst, cell(i, side == 2 ? 2 * g - 1 - j : 2 * ny - 2 * g - 1 - j));
                else for (int v = 0; v < 4; ++v) W[4 * dst + v] = inflow[v];
            }
        }
    }
}

// ----------------------------------------------------------------------------------------
// DF indicator of a face from its Gauss states (Calculate_alpha_k / Calculate_alpha, :1463-1521)
// ----------------------------------------------------------------------------------------
double alpha_k(const double* pl, const double* pr) {
    double Mln = pl[1] / std::sqrt(C.Gamma * pl[3] / pl[0]);
    double Mlt = pl[2] / std::sqrt(C.Gamma * pl[3] / pl[0]);
    double Mrn = pr[1] / std::sqrt(C.Gamma * pr[3] / pr[0]);
    double Mrt = pr[2] / std::sqrt(C.Gamma * pr[3] / pr[0]);
    double A = std::abs(pl[3] - pr[3]) / pl[3] + std::abs(pl[3] - pr[3]) / pr[3];
    A = A + sq(Mln - Mrn) + sq(Mlt - Mrt);
    return A;
}
double face_alpha(const Recon* re, bool yface) {
    double a[4];
    for (int ig = 0; ig < C.gp; ++ig) {
        double pl[4], pr[4];
        to_prim(pl, re[ig].left.convar);
        to_prim(pr, re[ig].right.convar);
        if (yface) {
            double ql[4], qr[4];
            rot_x_to_y(ql, pl);
            rot_x_to_y(qr, pr);
            a[ig] = alpha_k(ql, qr);
        } else {
            a[ig] = alpha_k(pl, pr);
        }
    }
    double r = 0;
    if (C.gp == 2) r = 0.5 * (a[0] + a[1]);
    if (C.gp == 3) r = (a[0] + a[1] + a[2]) / 3.0;
    if (C.gp == 4) r = 0.25 * (a[0] + a[1] + a[2] + a[3]);
    return r < 2.0 ? 0.0 : r;
}

// ----------------------------------------------------------------------------------------
// learned-gate features and labels (the gate has no counterpart in the reference; this is
// its CPU statement, in FP64, for the tests)
// ----------------------------------------------------------------------------------------
double gate_betas(int order, const double* s, double* beta) {
    int n;
    if (order == 5) {
        n = 4;
        beta3(s, 2, beta);
        beta[3] = 1.0 / 6.0 * (beta[0] + 4.0 * beta[1] + beta[2]) + std::abs(beta[0] - beta[2]);
    } else if (order == 7) {
        n = 5;
        beta3(s, 3, beta);
        beta[3] = 1.0 / 6.0 * (beta[0] + 4.0 * beta[1] + beta[2]) + std::abs(beta[0] - beta[2]);
        beta[4] = beta7(s, 3);
    } else {
        n = 6;
        beta3(s, 4, beta);
        beta[4] = beta7(s, 4);
        double mid;
        beta[5] = beta9(s, &mid);
        beta[3] = mid;
    }
    double tau = 0;
    for (int k = 0; k < n - 1; ++k) tau += std::abs(beta[n - 1] - beta[k]);
    return tau / (n - 1);
}

void gate_linear(int order, double* d) {
    const double h = 0.85;
    if (order == 5) {
        d[0] = (1 - h) * (1 - h) / 2; d[1] = (1 - h) * h; d[2] = d[0]; d[3] = h;
    } else if (order == 7) {
        d[0] = (1 - h) * (1 - h) * (1 - h) / 2; d[1] = (1 - h) * (1 - h) * h; d[2] = d[0];
        d[3] = (1 - h) * h; d[4] = h;
    } else {
        d[0] = (1 - h) * (1 - h) * (1 - h) * (1 - h) / 2; d[1] = (1 - h) * (1 - h) * (1 - h) * h; d[2] = d[0];
        d[3] = (1 - h) * (1 - h) * h; d[4] = (1 - h) * h; d[5] = h;
    }
}

// 7 normalised indicators of one stencil: betas / (sum + tau + 1e-10 c^2), padded to 6, then tau
void gate_indicators(int order, const double* s, double* f) {
    const int n = order == 5 ? 4 : order == 7 ? 5 : 6;
    double beta[6] = {0, 0, 0, 0, 0, 0};
    const double tau = gate_betas(order, s, beta);
    double sum = tau;
    for (int k = 0; k < n; ++k) sum += beta[k];
    const double c = s[order / 2];
    const double inv = 1.0 / (sum + 1e-10 * c * c + 1e-30);
    for (int k = 0; k < 6; ++k) f[k] = k < n ? beta[k] * inv : 0.0;
    f[6] = tau * inv;
}

// largest |omega_k - d_k| of the Z-type AO weights (epsilon 1e-6)
double gate_distance(int order, const double* s) {
    const int n = order == 5 ? 4 : order == 7 ? 5 : 6;
    double beta[6], d[6], a[6], sum = 0;
    const double tau = gate_betas(order, s, beta);
    gate_linear(order, d);
    for (int k = 0; k < n; ++k) {
        const double q = tau / (beta[k] + 1e-6);
        a[k] = d[k] * (1.0 + q * q);
        sum += a[k];
    }
    double dm = 0;
    for (int k = 0; k < n; ++k) dm = std::max(dm, std::abs(a[k] / sum - d[k]));
    return dm;
}

}  // namespace

// ========================================================================================
// C interface
// ========================================================================================
extern "C" {

int oracle2d_init(const hos2d_params* p) {
    C = Config();
    C.p = *p;
    if (!(p->order == 5 || p->order == 7 || p->order == 9)) return 2;
    // the non-DF scheme (WENO5_AO_normal / WENO5_AO_tangent, the drivers' default slots) exists
    // for WENO5 only, and its tangential sweep writes the Gauss points only when gausspoint == 2
    // (src/reconstruction.cpp:2264, :2279)
    if (!p->use_df && p->order != 5) return 2;
    if (p->wenotype < 0 || p->wenotype > 2) return 2;
    const int need_gp = p->order == 5 ? 2 : p->order == 7 ? 3 : 4;
    if (p->gausspoint != need_gp) return 2;
    if (p->ghost < p->order / 2 + 1) return 2;
    C.g = p->ghost;
    C.gp = p->gausspoint;
    C.nx = p->nodex + 2 * p->ghost;
    C.ny = p->nodey + 2 * p->ghost;
    C.dx = (p->right - p->left) / p->nodex;
    C.dy = (p->up - p->down) / p->nodey;
    C.K = p->K;
    C.Gamma = p->gamma;
    if (C.gp == 2) { C.gw[0] = 0.5; C.gw[1] = 0.5; }
    if (C.gp == 3) { C.gw[0] = 4.0 / 9.0; C.gw[1] = 0.5 - 0.5 * C.gw[0]; C.gw[2] = C.gw[1]; }
    if (C.gp == 4) { C.gw[0] = 1.0 / 12.0; C.gw[1] = 1.0 / 12.0; C.gw[2] = 5.0 / 12.0; C.gw[3] = 5.0 / 12.0; }
    const size_t nc = static_cast<size_t>(C.nx) * C.ny;
    const size_t nf = static_cast<size_t>(C.nx + 1) * (C.ny + 1);
    W.assign(4 * nc, 0.0);
    Wold.assign(4 * nc, 0.0);
    Prim.assign(4 * nc, 0.0);
    AX.assign(nc, 0.0);
    AY.assign(nc, 0.0);
    Point z;
    std::memset(&z, 0, sizeof z);
    XL.assign(2 * nf, z);
    YL.assign(2 * nf, z);
    Recon zr;
    std::memset(&zr, 0, sizeof zr);
    XG.assign(nf * C.gp, zr);
    YG.assign(nf * C.gp, zr);
    XF.assign(nf * 4 * C.gp * 8, 0.0);
    YF.assign(nf * 4 * C.gp * 8, 0.0);
    if (p->integrator < 0 || p->integrator > 5 || p->flux < 0 || p->flux > 1) return 2;
    set_integrator(p->integrator);
    XX.assign(nf * C.gp * 4, 0.0);
    YX.assign(nf * C.gp * 4, 0.0);
    return 0;
}

void oracle2d_free(void) {
    std::vector<double>().swap(W);
    std::vector<double>().swap(Wold);
    std::vector<double>().swap(Prim);
    std::vector<Point>().swap(XL);
    std::vector<Point>().swap(YL);
    std::vector<Recon>().swap(XG);
    std::vector<Recon>().swap(YG);
}

void oracle2d_set_threads(int n) { omp_set_num_threads(n); }

void oracle2d_set_first_order(int on) { C.first_order = on ? 1 : 0; }

void oracle2d_set_source(int on) { C.source = on ? 1 : 0; }

void oracle2d_set_state(const double* convar, const double* primvar) {
    const size_t n = static_cast<size_t>(C.nx) * C.ny;
    std::memcpy(W.data(), convar, 4 * n * sizeof(double));
    if (primvar) std::memcpy(Prim.data(), primvar, 4 * n * sizeof(double));
}

void oracle2d_get_state(double* convar, double* primvar, double* alpha_x, double* alpha_y) {
    const size_t n = static_cast<size_t>(C.nx) * C.ny;
    if (convar) std::memcpy(convar, W.data(), 4 * n * sizeof(double));
    if (primvar) std::memcpy(primvar, Prim.data(), 4 * n * sizeof(double));
    if (alpha_x) std::memcpy(alpha_x, AX.data(), n * sizeof(double));
    if (alpha_y) std::memcpy(alpha_y, AY.data(), n * sizeof(double));
}

// CopyFluid_new_to_old + Get_CFL with the primitive state of the previous stage
// (src/time_advance.cpp:264-305)
double oracle2d_begin_step(double tstop, double t) {
    const int g = C.g;
    C.tbeg = t;
#pragma omp parallel for
    for (int i = g; i < g + C.p.nodex; ++i)
        for (int j = g; j < g + C.p.nodey; ++j)
            for (int v = 0; v < 4; ++v) Wold[4 * cell(i, j) + v] = W[4 * cell(i, j) + v];
    double dt = C.dx;
    const double cfl = C.p.cfl;
    auto dtx = [&](double d, double h, const double* pr) {
        double tmp = std::sqrt(pr[1] * pr[1] + pr[2] * pr[2]) + std::sqrt(C.Gamma * pr[3] / pr[0]);
        if (tmp > cfl * h / d) d = cfl * h / tmp;
        // viscous cap (Dtx, src/time_advance.cpp:300-303)
        if (d > 0.25 * cfl * h * h / C.p.mu && C.p.tau_type == 1 && C.p.mu > 0) d = 0.25 * cfl * h * h / C.p.mu;
        return d;
    };
    for (int i = g; i < C.nx - g; ++i)
        for (int j = g; j < C.ny - g; ++j) {
            const double* pr = &Prim[4 * cell(i, j)];
            dt = dtx(dt, C.dx, pr);
            dt = dtx(dt, C.dy, pr);
        }
    if (t + dt > tstop) dt = tstop - t + 1e-16;
    return dt;
}

int oracle2d_stage(int stage, double dt) {
    const int nx = C.nx, ny = C.ny, g = C.g, gp = C.gp, order = C.p.order, r = order / 2;
    for (int s = 0; s < 4; ++s) bc_side(s);
    // Convar_to_Primvar with the blow-up check
    int bad = 0;
#pragma omp parallel for reduction(| : bad)
    for (int c = 0; c < nx * ny; ++c) {
        double* pr = &Prim[4 * c];
        to_prim(pr, &W[4 * c]);
        if (pr[0] < 0 || pr[3] < 0 || std::isnan(pr[0]) || std::isnan(pr[3])) bad |= 1;
    }
    if (bad) return 1;
    // normal reconstruction: x for cells with i in [g-1, nx-g], y for j in [g-1, ny-g]
#pragma omp parallel for
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            double st[9][4], al[9];
            if (i > g - 2 && i < nx - g + 1) {
                for (int k = 0; k < order; ++k) {
                    const int c = cell(i + k - r, j);
                    for (int v = 0; v < 4; ++v) st[k][v] = W[4 * c + v];
                    al[k] = AX[c];
                }
                normal_cell(order, st, al, C.dx, XL[2 * face(i, j) + 1], XL[2 * face(i + 1, j) + 0]);
            }
            if (j > g - 2 && j < ny - g + 1) {
                for (int k = 0; k < order; ++k) {
                    const int c = cell(i, j + k - r);
                    rot_y_to_x(st[k], &W[4 * c]);
                    al[k] = AY[c];
                }
                normal_cell(order, st, al, C.dy, YL[2 * face(i, j) + 1], YL[2 * face(i, j + 1) + 0]);
            }
        }
    // tangential reconstruction for cells in [g-1, n-g+1): x-face (i+1, j), y-face (i, j+1)
#pragma omp parallel for
    for (int i = g - 1; i < nx - g + 1; ++i)
        for (int j = g - 1; j < ny - g + 1; ++j) {
            Point ln[9][2];
            double a1[9], a2[9];
            // x-face (i+1, j): tangent along +y, left cell column i, right column i+1
            for (int k = 0; k < order; ++k) {
                const int f = face(i + 1, j + k - r);
                ln[k][0] = XL[2 * f + 0];
                ln[k][1] = XL[2 * f + 1];
                a1[k] = AY[cell(i, j + k - r)];
                a2[k] = AY[cell(i + 1, j + k - r)];
            }
            tangent_face(order, ln, a1, a2, C.dy, &XG[static_cast<size_t>(face(i + 1, j)) * gp]);
            // y-face (i, j+1): tangent along -x, lower cell row j, upper row j+1
            for (int k = 0; k < order; ++k) {
                const int f = face(i - (k - r), j + 1);
                ln[k][0] = YL[2 * f + 0];
                ln[k][1] = YL[2 * f + 1];
                a1[k] = AX[cell(i - (k - r), j)];
                a2[k] = AX[cell(i - (k - r), j + 1)];
            }
            tangent_face(order, ln, a1, a2, C.dx, &YG[static_cast<size_t>(face(i, j + 1)) * gp]);
        }
    // fluxes (Calculate_flux, src/flux_function.cpp:317-343)
#pragma omp parallel for
    for (int i = g; i < g + C.p.nodex + 1; ++i)
        for (int j = g; j < g + C.p.nodey; ++j)
            for (int ig = 0; ig < gp; ++ig) {
                const size_t f = face(i, j);
                double* o = &XF[((f * 4 + stage) * gp + ig) * 8];
                if (C.p.flux == 1) lf2d(XG[f * gp + ig], dt, o, o + 4);
                else gks2d(XG[f * gp + ig], dt, o, o + 4, C.p.integrator == 1);
            }
#pragma omp parallel for
    for (int i = g; i < g + C.p.nodex; ++i)
        for (int j = g; j < g + C.p.nodey + 1; ++j)
            for (int ig = 0; ig < gp; ++ig) {
                const size_t f = face(i, j);
                double* o = &YF[((f * 4 + stage) * gp + ig) * 8];
                if (C.p.flux == 1) lf2d(YG[f * gp + ig], dt, o, o + 4);
                else gks2d(YG[f * gp + ig], dt, o, o + 4, C.p.integrator == 1);
            }
    // stage combination per face and Gauss point (Update, src/time_advance.cpp:378-428)
    auto combine = [&](std::vector<double>& F, std::vector<double>& X, int i0, int i1, int j0, int j1) {
#pragma omp parallel for
        for (int i = i0; i < i1; ++i)
            for (int j = j0; j < j1; ++j)
                for (int ig = 0; ig < gp; ++ig)
                    for (int v = 0; v < 4; ++v) {
                        const size_t f = face(i, j);
                        double fl = 0.0;
                        if (C.p.integrator == 4) {   // RK3 (:317-372)
                            const double q = F[((f * 4 + stage) * gp + ig) * 8 + v];
                            fl = stage == 0 ? C.gw[ig] * q : stage == 1 ? 0.25 * C.gw[ig] * q : 2.0 / 3.0 * C.gw[ig] * q;
                        } else {
                            for (int k = 0; k < stage + 1; ++k) {
                                const double* q = &F[((f * 4 + k) * gp + ig) * 8];
                                fl = fl + C.gw[ig] * (C.tc[stage][k][0] * q[v] + C.tc[stage][k][1] * q[4 + v]);
                            }
                        }
                        X[(f * gp + ig) * 4 + v] = fl;
                    }
    };
    if (C.source) {
        // Update_with_source (src/time_advance.cpp:534-704) under S2O4: stage 0 takes
        // W = W_old + dt (L + S) with L the Gauss-weighted face fluxes f of the stage (global
        // frame) over dx dt and S = (0, 0, rho, rho v) of the current state; stage 1 leaves W
        if (stage == 0) {
            const double dx = C.dx, dy = C.dy;
#pragma omp parallel for
            for (int i = g; i < g + C.p.nodex; ++i)
                for (int j = g; j < g + C.p.nodey; ++j) {
                    const int c = cell(i, j);
                    const size_t f = face(i, j);
                    double Lw[4] = {0, 0, 0, 0};
                    for (int v = 0; v < 4; ++v)
                        for (int ig = 0; ig < gp; ++ig) {
                            auto xf = [&](size_t ff) {
                                const double* x = &XF[((ff * 4 + stage) * gp + ig) * 8];
                                return v == 1 ? x[1] * 1.0 - x[2] * 0.0 : v == 2 ? x[1] * 0.0 + x[2] * 1.0 : x[v];
                            };
                            auto yf = [&](size_t ff) {
                                const double* x = &YF[((ff * 4 + stage) * gp + ig) * 8];
                                return v == 1 ? x[1] * 0.0 - x[2] * 1.0 : v == 2 ? x[1] * 1.0 + x[2] * 0.0 : x[v];
                            };
                            Lw[v] += C.gw[ig] * ((xf(f) - xf(f + ny + 1)) / dx / dt + (yf(f) - yf(f + 1)) / dy / dt);
                        }
                    const double S[4] = {0.0, 0.0, W[4 * c + 0], W[4 * c + 2]};
                    for (int v = 0; v < 4; ++v) {
                        const double L1 = Lw[v] + S[v];
                        W[4 * c + v] = Wold[4 * c + v] + dt * L1;
                    }
                }
        }
    } else {
    combine(XF, XX, g, g + C.p.nodex + 1, g, g + C.p.nodey);
    combine(YF, YX, g, g + C.p.nodex, g, g + C.p.nodey + 1);
    // Update_with_gauss (src/time_advance.cpp:431-474): y-face fluxes rotate back to the
    // global frame (local (n, t) -> global (-t, n)); x-face rotation is the identity.
    const double area = C.dx * C.dy;
#pragma omp parallel for
    for (int i = g; i < g + C.p.nodex; ++i)
        for (int j = g; j < g + C.p.nodey; ++j) {
            const int c = cell(i, j);
            const size_t f = face(i, j);
            for (int v = 0; v < 4; ++v) {
                const double cur = W[4 * c + v];   // the RK3 stage state (convar_stage1 / _stage2)
                W[4 * c + v] = Wold[4 * c + v];
                double total = 0.0;
                for (int ig = 0; ig < gp; ++ig) {
                    auto yv = [&](size_t ff) {
                        const double* x = &YX[(ff * gp + ig) * 4];
                        return v == 1 ? x[1] * 0.0 - x[2] * 1.0 : v == 2 ? x[1] * 1.0 + x[2] * 0.0 : x[v];
                    };
                    auto xv = [&](size_t ff) {
                        const double* x = &XX[(ff * gp + ig) * 4];
                        return v == 1 ? x[1] * 1.0 - x[2] * 0.0 : v == 2 ? x[1] * 0.0 + x[2] * 1.0 : x[v];
                    };
                    total += C.dx * yv(f);
                    total += -C.dx * yv(f + 1);
                    total += C.dy * xv(f);
                    total += -C.dy * xv(f + ny + 1);
                }
                if (C.p.integrator == 4 && stage == 1)
                    W[4 * c + v] = 0.75 * Wold[4 * c + v] + 0.25 * cur + total / area;
                else if (C.p.integrator == 4 && stage == 2)
                    W[4 * c + v] = 1.0 / 3.0 * Wold[4 * c + v] + 2.0 / 3.0 * cur + total / area;
                else
                    W[4 * c + v] += total / area;
            }
        }
    }
    // DF factor update (Update_alpha, :1523-1534), which the drivers call only with
    // is_using_df_factor set (src/2Dproblem.cpp:154)
    if (!C.p.use_df) return 0;
    const int jend = g + std::min(C.p.nodex, C.p.nodey);
#pragma omp parallel for
    for (int i = g; i < g + C.p.nodex; ++i)
        for (int j = g; j < jend; ++j) {
            const int c = cell(i, j);
            double al = face_alpha(&XG[static_cast<size_t>(face(i, j)) * gp], false);
            double ar = face_alpha(&XG[static_cast<size_t>(face(i + 1, j)) * gp], false);
            double ad = face_alpha(&YG[static_cast<size_t>(face(i, j)) * gp], true);
            double au = face_alpha(&YG[static_cast<size_t>(face(i, j + 1)) * gp], true);
            AX[c] = al + ar;
            AY[c] = ad + au;
        }
    return 0;
}

int oracle2d_step(double tstop, double t, double* dt_out) {
    double dt = oracle2d_begin_step(tstop, t);
    if (dt_out) *dt_out = dt;
    for (int s = 0; s < C.stages; ++s) {
        int st = oracle2d_stage(s, dt);
        if (st) return st;
    }
    return 0;
}

void oracle2d_get_gauss(int dir, double* out) {
    std::vector<Recon>& G = dir == 0 ? XG : YG;
    const size_t nf = static_cast<size_t>(C.nx + 1) * (C.ny + 1);
    for (size_t f = 0; f < nf; ++f)
        for (int ig = 0; ig < C.gp; ++ig) {
            double* o = out + (f * C.gp + ig) * 36;
            const Recon& re = G[f * C.gp + ig];
            const Point* pts[3] = {&re.left, &re.right, &re.center};
            for (int s = 0; s < 3; ++s)
                for (int v = 0; v < 4; ++v) {
                    o[s * 12 + v] = pts[s]->convar[v];
                    o[s * 12 + 4 + v] = pts[s]->der1x[v];
                    o[s * 12 + 8 + v] = pts[s]->der1y[v];
                }
        }
}

void oracle2d_get_flux(int dir, int stage, double* out) {
    std::vector<double>& F = dir == 0 ? XF : YF;
    const size_t nf = static_cast<size_t>(C.nx + 1) * (C.ny + 1);
    for (size_t f = 0; f < nf; ++f)
        for (int ig = 0; ig < C.gp; ++ig)
            for (int k = 0; k < 8; ++k) out[(f * C.gp + ig) * 8 + k] = F[((f * 4 + stage) * C.gp + ig) * 8 + k];
}

// Gate features ([ncell][2][16]) and label distances ([ncell][2]; -1 where the stencil leaves
// the array) of a state (AoS convar, DF indicators), in the configuration of oracle2d_init.
void oracle2d_gate_cells(const double* convar, const double* alpha_x, const double* alpha_y, double* feat,
                         double* dist) {
    const int order = C.p.order, N = order, r = order / 2;
    for (int i = 0; i < C.nx; ++i)
        for (int j = 0; j < C.ny; ++j) {
            const int c = cell(i, j);
            for (int dir = 0; dir < 2; ++dir) {
                double* f = feat + (static_cast<size_t>(c) * 2 + dir) * 16;
                double& dd = dist[static_cast<size_t>(c) * 2 + dir];
                for (int k = 0; k < 16; ++k) f[k] = 0.0;
                const int pos = dir == 0 ? i : j, lim = dir == 0 ? C.nx : C.ny;
                if (pos < r || pos >= lim - r) {
                    dd = -1.0;
                    continue;
                }
                double st[9][4], rho[9], pr[9];
                for (int k = 0; k < N; ++k) {
                    const int q = dir == 0 ? cell(i + k - r, j) : cell(i, j + k - r);
                    if (dir == 0) for (int v = 0; v < 4; ++v) st[k][v] = convar[4 * q + v];
                    else rot_y_to_x(st[k], convar + 4 * q);
                    double pv[4];
                    to_prim(pv, st[k]);
                    rho[k] = pv[0];
                    pr[k] = pv[3];
                }
                gate_indicators(order, rho, f);
                gate_indicators(order, pr, f + 7);
                const double al = dir == 0 ? alpha_x[c] : alpha_y[c];
                f[14] = al / (1.0 + al);
                double pn1[4], p0[4], pp1[4];
                to_prim(pn1, st[r - 1]);
                to_prim(p0, st[r]);
                to_prim(pp1, st[r + 1]);
                double dm = 0;
                for (int side = 0; side < 2; ++side) {
                    double base[4], ch[9][4];
                    for (int v = 0; v < 4; ++v) base[v] = 0.5 * ((side == 0 ? pn1[v] : pp1[v]) + p0[v]);
                    for (int k = 0; k < N; ++k) {
                        if (C.p.characteristic) to_char(ch[k], base, st[k]);
                        else for (int v = 0; v < 4; ++v) ch[k][v] = st[k][v];
                    }
                    for (int v = 0; v < 4; ++v) {
                        double sv[9];
                        for (int k = 0; k < N; ++k) sv[k] = ch[k][v];
                        dm = std::max(dm, gate_distance(order, sv));
                    }
                }
                dd = dm;
            }
        }
}

}  // extern "C"
