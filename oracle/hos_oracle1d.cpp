// hos_oracle1d.cpp -- CPU FP64 restatement of the reference's 1D per-step path.
//
// TEST INFRASTRUCTURE ONLY (see oracle_api.h): the checker for the CUDA 1D path.
//
// Restates (file:line in XJTUZhangHong/high-order-solver):
//   step driver .......... src/1Dproblem.cpp:93-131 (SodTubeProblem), :606-640 (accuracy_sinwave_1d)
//   CopyFluid_new_to_old . src/basic_function.cpp:1559-1569
//   Get_CFL / Dtx 1D ..... src/time_advance.cpp:75-111 (fresh conserved state, +1e-15 clip)
//   boundaries 1D ........ src/boundary_condition.cpp:4-64
//   reconstruction 1D .... src/reconstruction.cpp:46-53 (cell loop), WENO5_AO :85-159,
//                          weno_5th_ao_left/right :161-360 (non-DF, epsilon 1e-10),
//                          WENO5/7/9_AO_with_DF :394-478, :659-748, :976-1070
//   order reduction ...... src/reconstruction.cpp:13-44
//   centre collision ..... src/reconstruction.cpp:1366-1407
//   GKS 1D ............... src/flux_function.cpp:7-276 (the dt/2 level uses tau_num of dt)
//   moments 1D ........... src/basic_function.cpp:16-99 (MMDF1d), 522-559 (G/GL/GR, Microslope)
//   characteristic 1D .... src/basic_function.cpp:868-921
//   S2O4 update 1D ....... src/time_advance.cpp:113-194
//   DF factor 1D ......... src/reconstruction.cpp:362-392
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle_api.h"
#include "oracle_weno.h"

namespace {

using namespace oracle_weno;

hos1d_params P;
int NX = 0, G = 0;
double DX = 0, KK = 0, GAM = 0;
std::vector<double> W, Wold, AL;          // 3 per cell, 3 per cell, 1 per cell
struct Pt { double convar[3], der1[3]; };
struct Itf { Pt left, center, right; };
std::vector<Itf> IF;                        // nx + 1 interfaces
std::vector<double> FL;                     // [face][stage][6]: f[3], derf[3]

const double TC[2][2][2] = {{{0.5, 1.0 / 8.0}, {0.0, 0.0}}, {{1.0, 1.0 / 6.0}, {0.0, 1.0 / 3.0}}};

inline void to_prim(double* pr, const double* w) {  // (rho, u, p)
    pr[0] = w[0];
    pr[1] = w[1] / w[0];
    pr[2] = (GAM - 1.0) * (w[2] - 0.5 * w[1] * w[1] / w[0]);
}
inline double lambda1(double rho, double u, double rhoE) { return (KK + 1.0) * 0.25 * (rho / (rhoE - 0.5 * rho * (u * u))); }
inline void to_ulambda(double* pr, const double* w) {
    pr[0] = w[0];
    pr[1] = w[1] / w[0];
    pr[2] = lambda1(w[0], pr[1], w[2]);
}
void to_char(double* ch, const double* base, const double* w) {
    double c = std::sqrt(GAM * base[2] / base[0]);
    double alfa = (GAM - 1.0) / (2.0 * c * c);
    double u = base[1];
    double s[3][3];
    s[0][0] = alfa * (0.5 * u * u + u * c / (GAM - 1.0));
    s[0][1] = alfa * (-u - c / (GAM - 1.0));
    s[0][2] = alfa;
    s[1][0] = alfa * (-u * u + 2.0 * c * c / (GAM - 1.0));
    s[1][1] = alfa * 2.0 * u;
    s[1][2] = -2.0 * alfa;
    s[2][0] = alfa * (0.5 * u * u - u * c / (GAM - 1.0));
    s[2][1] = alfa * (-u + c / (GAM - 1.0));
    s[2][2] = alfa;
    for (int r = 0; r < 3; ++r) {
        double acc = 0;
        for (int k = 0; k < 3; ++k) acc = acc + s[r][k] * w[k];
        ch[r] = acc;
    }
}
void from_char(double* w, const double* base, const double* ch) {
    double c = std::sqrt(GAM * base[2] / base[0]);
    double u = base[1];
    double h = 0.5 * u * u + c * c / (GAM - 1.0);
    double s[3][3] = {{1.0, 1.0, 1.0}, {u - c, u, u + c}, {h - u * c, u * u / 2.0, h + u * c}};
    for (int r = 0; r < 3; ++r) {
        double acc = 0;
        for (int k = 0; k < 3; ++k) acc = acc + s[r][k] * ch[k];
        w[r] = acc;
    }
}
inline bool needs_reduce(const double* w) {
    double lam = lambda1(w[0], w[1] / w[0], w[2]);
    return lam <= 0.0 || !(lam == lam);
}

// one cell: values and slopes at its left face (L) and right face (R)
void recon_cell(int i, bool df_variant, Pt& L, Pt& R) {
    const int order = P.order, r = order / 2, n = order;
    double st[9][3], al[9], df[6];
    for (int k = 0; k < n; ++k) {
        for (int v = 0; v < 3; ++v) st[k][v] = W[3 * (i + k - r) + v];
        al[k] = AL[i + k - r];
    }
    if (df_variant) df_factors(order, al, df);
    const double h = DX;
    double ch[2][9][3], var[3], der[3];
    double bl[3], br[3];
    if (P.characteristic) {
        double pn1[3], p0[3], pp1[3];
        to_prim(pn1, st[r - 1]);
        to_prim(p0, st[r]);
        to_prim(pp1, st[r + 1]);
        for (int v = 0; v < 3; ++v) {
            bl[v] = 0.5 * (pn1[v] + p0[v]);
            br[v] = 0.5 * (pp1[v] + p0[v]);
        }
        for (int k = 0; k < n; ++k) to_char(ch[0][k], bl, st[k]);
        for (int k = 0; k < n; ++k) {
            // the WENO9 right side keeps the left base's projection of its outermost entries
            // (src/reconstruction.cpp:1050-1061)
            if (order == 9 && (k == 0 || k == n - 1)) {
                for (int v = 0; v < 3; ++v) ch[1][k][v] = ch[0][k][v];
                continue;
            }
            to_char(ch[1][k], br, st[k]);
        }
    } else {
        for (int sd = 0; sd < 2; ++sd)
            for (int k = 0; k < n; ++k)
                for (int v = 0; v < 3; ++v) ch[sd][k][v] = st[k][v];
    }
    for (int sd = 0; sd < 2; ++sd) {
        for (int v = 0; v < 3; ++v) {
            double s[9];
            for (int k = 0; k < n; ++k) s[k] = ch[sd][k][v];
            if (df_variant) weno_normal(order, sd, s, df, h, var[v], der[v]);
            else weno5_plain(sd, s, h, var[v], der[v], P.wenotype);
        }
        Pt& Q = sd == 0 ? L : R;
        if (P.characteristic) {
            from_char(Q.convar, sd == 0 ? bl : br, var);
            from_char(Q.der1, sd == 0 ? bl : br, der);
        } else {
            for (int v = 0; v < 3; ++v) { Q.convar[v] = var[v]; Q.der1[v] = der[v]; }
        }
    }
    bool r0 = needs_reduce(R.convar), r1 = needs_reduce(L.convar);
    if (r0 || r1) {
        for (int v = 0; v < 3; ++v) {
            L.convar[v] = st[r][v];
            R.convar[v] = st[r][v];
            L.der1[v] = 0.0;
            R.der1[v] = 0.0;
        }
    }
}

// 1D Maxwellian moments (MMDF1d, src/basic_function.cpp:16-99)
struct Mom1 { double up[10][4], un[10][4], uw[10][4]; };
void mom1(Mom1& m, double u, double lambda) {
    const double pi = 3.14159265358979323846;
    double uwhole[10], uplus[10], uminus[10];
    uwhole[0] = 1;
    uwhole[1] = u;
    uplus[0] = 0.5 * std::erfc(std::sqrt(lambda) * -u);
    uminus[0] = 0.5 * std::erfc(std::sqrt(lambda) * u);
    const double beta = std::exp(-lambda * u * u) / std::sqrt(pi * lambda);
    uplus[1] = u * uplus[0] + 0.5 * beta;
    uminus[1] = u * uminus[0] - 0.5 * beta;
    for (int i = 2; i <= 9; ++i) uwhole[i] = u * uwhole[i - 1] + 0.5 * (i - 1) / lambda * uwhole[i - 2];
    for (int i = 2; i <= 9; ++i) {
        uplus[i] = u * uplus[i - 1] + 0.5 * (i - 1) / lambda * uplus[i - 2];
        uminus[i] = u * uminus[i - 1] + 0.5 * (i - 1) / lambda * uminus[i - 2];
    }
    const double xi2 = 0.5 * KK / lambda;
    const double xi4 = 0.25 * (KK * KK + 2 * KK) / (lambda * lambda);
    const double xi6 = 0.5 * (KK + 4) / lambda * xi4;
    const double xi[4] = {1.0, xi2, xi4, xi6};
    for (int i = 0; i < 10; ++i)
        for (int k = 0; k < 4; ++k)
            if (i + 2 * k <= 9) {
                m.up[i][k] = k == 0 ? uplus[i] : uplus[i] * xi[k];
                m.un[i][k] = k == 0 ? uminus[i] : uminus[i] * xi[k];
                m.uw[i][k] = k == 0 ? uwhole[i] : uwhole[i] * xi[k];
            }
}
// G / GL / GR (src/basic_function.cpp:522-548) on table M
void g1(const double (*M)[4], int u, int x, const double* a, double* psi) {
    psi[0] = a[0] * M[u][x] + a[1] * M[u + 1][x] + a[2] * 0.5 * (M[u + 2][x] + M[u][x + 1]);
    psi[1] = a[0] * M[u + 1][x] + a[1] * M[u + 2][x] + a[2] * 0.5 * (M[u + 3][x] + M[u + 1][x + 1]);
    psi[2] = 0.5 * (a[0] * (M[u + 2][x] + M[u][x + 1]) + a[1] * (M[u + 3][x] + M[u + 1][x + 1]) +
                    a[2] * 0.5 * (M[u + 4][x] + M[u][x + 2] + 2 * M[u + 2][x + 1]));
}
// Microslope (src/basic_function.cpp:551-559)
void microslope1(double* a, const double* der, const double* prim) {
    double R4 = der[2] / prim[0] - 0.5 * (prim[1] * prim[1] + 0.5 * (KK + 1) / prim[2]) * der[0] / prim[0];
    double R2 = (der[1] - prim[1] * der[0]) / prim[0];
    a[2] = 4 * prim[2] * prim[2] / (KK + 1) * (2 * R4 - 2 * prim[1] * R2);
    a[1] = 2 * prim[2] * R2 - prim[1] * a[2];
    a[0] = der[0] / prim[0] - prim[1] * a[1] - 0.5 * a[2] * (prim[1] * prim[1] + 0.5 * (KK + 1) / prim[2]);
}
double tau_num1(double dl, double dr, double ll, double lr, double dt) {
    if (P.c1_euler <= 0 && P.c2_euler <= 0) return 0.0;
    double Cc = P.c2_euler * std::abs(dl / ll - dr / lr) / std::abs(dl / ll + dr / lr);
    return P.c1_euler * dt + dt * Cc;
}

void gks1(Itf& itf, double dt, double* fo, double* dfo) {
    double pl[3], pr[3], p0[3];
    to_ulambda(pl, itf.left.convar);
    to_ulambda(pr, itf.right.convar);
    Mom1 ml, mr;
    mom1(ml, pl[1], pl[2]);
    mom1(mr, pr[1], pr[2]);
    // centre state (Center_collision, src/reconstruction.cpp:1375-1407)
    {
        const double unit[3] = {1.0, 0.0, 0.0};
        double gl[3], gr[3], axl[3], axr[3], ax0l[3], ax0r[3];
        g1(ml.up, 0, 0, unit, gl);
        g1(mr.un, 0, 0, unit, gr);
        microslope1(axl, itf.left.der1, pl);
        microslope1(axr, itf.right.der1, pr);
        g1(ml.up, 0, 0, axl, ax0l);
        g1(mr.un, 0, 0, axr, ax0r);
        for (int i = 0; i < 3; ++i) {
            itf.center.convar[i] = itf.left.convar[0] * gl[i] + itf.right.convar[0] * gr[i];
            itf.center.der1[i] = itf.left.convar[0] * ax0l[i] + itf.right.convar[0] * ax0r[i];
        }
    }
    to_ulambda(p0, itf.center.convar);
    const double tau = 0.0;
    double tn = tau_num1(pl[0], pr[0], pl[2], pr[2], dt);
    double eta = std::exp(-dt / tn);
    double t[6];
    t[0] = tn * (1 - eta);
    t[1] = tn * (eta * (dt + tn) - tn) + tau * tn * (eta - 1);
    t[2] = tau * tn * (eta - 1);
    t[3] = tn * eta + dt - tn;
    t[4] = tn * (tn - eta * (dt + tn) - tau * (eta - 1)) - dt * tau;
    t[5] = 0.5 * dt * dt - tau * tn * (eta - 1) - tau * dt;
    Mom1 m0;
    mom1(m0, p0[1], p0[2]);
    const double unit[3] = {1, 0.0, 0.0};
    double glu[3], gru[3], g0u[3], F0[3], F1[3];
    g1(ml.up, 1, 0, unit, glu);
    g1(mr.un, 1, 0, unit, gru);
    for (int i = 0; i < 3; ++i) F0[i] = pl[0] * t[0] * glu[i] + pr[0] * t[0] * gru[i];
    g1(m0.uw, 1, 0, unit, g0u);
    for (int i = 0; i < 3; ++i) F0[i] = F0[i] + p0[0] * t[3] * g0u[i];
    double alx[3], arx[3], alxuul[3], arxuur[3];
    microslope1(alx, itf.left.der1, pl);
    g1(ml.up, 2, 0, alx, alxuul);
    microslope1(arx, itf.right.der1, pr);
    g1(mr.un, 2, 0, arx, arxuur);
    for (int i = 0; i < 3; ++i) F0[i] = F0[i] + pl[0] * t[1] * (alxuul[i]) + pr[0] * t[1] * (arxuur[i]);
    double alxu[3], arxu[3], dAL[3], dAR[3], Al[3], Ar[3], Alul[3], Arur[3];
    g1(ml.uw, 1, 0, alx, alxu);
    g1(mr.uw, 1, 0, arx, arxu);
    for (int i = 0; i < 3; ++i) {
        dAL[i] = -pl[0] * (alxu[i]);
        dAR[i] = -pr[0] * (arxu[i]);
    }
    microslope1(Al, dAL, pl);
    microslope1(Ar, dAR, pr);
    g1(ml.up, 1, 0, Al, Alul);
    g1(mr.un, 1, 0, Ar, Arur);
    for (int i = 0; i < 3; ++i) F0[i] = F0[i] + pl[0] * t[2] * (Alul[i]) + pr[0] * t[2] * (Arur[i]);
    double a0x[3], a0xu[3], a0xuu[3], dA0[3], A0[3], A0u[3];
    microslope1(a0x, itf.center.der1, p0);
    g1(m0.uw, 1, 0, a0x, a0xu);
    g1(m0.uw, 2, 0, a0x, a0xuu);
    for (int i = 0; i < 3; ++i) F0[i] = F0[i] + p0[0] * t[4] * (a0xuu[i]);
    for (int i = 0; i < 3; ++i) dA0[i] = -p0[0] * (a0xu[i]);
    microslope1(A0, dA0, p0);
    g1(m0.uw, 1, 0, A0, A0u);
    for (int i = 0; i < 3; ++i) F0[i] = F0[i] + p0[0] * t[5] * (A0u[i]);
    // dt/2 level; the 1D driver evaluates tau_num with dt (src/flux_function.cpp:236)
    const double dt2 = 0.5 * dt;
    tn = tau_num1(pl[0], pr[0], pl[2], pr[2], dt);
    eta = std::exp(-dt2 / tn);
    t[0] = tn * (1 - eta);
    t[1] = tn * (eta * (dt2 + tn) - tn) + tau * tn * (eta - 1);
    t[2] = tau * tn * (eta - 1);
    t[3] = tn * eta + dt2 - tn;
    t[4] = tn * (tn - eta * (dt2 + tn) - tau * (eta - 1)) - dt2 * tau;
    t[5] = 0.5 * dt2 * dt2 - tau * tn * (eta - 1) - tau * dt2;
    for (int i = 0; i < 3; ++i) {
        F1[i] = pl[0] * t[0] * glu[i] + pr[0] * t[0] * gru[i];
        F1[i] = F1[i] + pl[0] * t[1] * (alxuul[i]) + pr[0] * t[1] * (arxuur[i]);
        F1[i] = F1[i] + pl[0] * t[2] * (Alul[i]) + pr[0] * t[2] * (Arur[i]);
        F1[i] = F1[i] + p0[0] * t[3] * g0u[i];
        F1[i] = F1[i] + p0[0] * t[4] * (a0xuu[i]);
        F1[i] = F1[i] + p0[0] * t[5] * (A0u[i]);
    }
    for (int i = 0; i < 3; ++i) {
        fo[i] = (4.0 * F1[i] - F0[i]);
        dfo[i] = 4.0 * (F0[i] - 2.0 * F1[i]);
    }
}

double alpha_k1(const double* pl, const double* pr) {
    double Ml = pl[1] / std::sqrt(GAM * pl[2] / pl[0]);
    double Mr = pr[1] / std::sqrt(GAM * pr[2] / pr[0]);
    double A = std::abs(pl[2] - pr[2]) / pl[2] + std::abs(pl[2] - pr[2]) / pr[2];
    A = A + (Ml - Mr) * (Ml - Mr);
    return A;
}

void bc1() {
    const int nx = NX, g = G;
    for (int side = 0; side < 2; ++side) {
        const int kind = P.bc[side];
        for (int k = 0; k < g; ++k) {
            const int i = side == 0 ? g - 1 - k : nx - g + k;
            int src;
            if (kind == HOS_BC_FREE) src = side == 0 ? i + 1 : i - 1;
            else if (kind == HOS_BC_PERIODIC) src = side == 0 ? i + P.nodex : i - P.nodex;
            else src = side == 0 ? 2 * g - 1 - i : 2 * (nx - g) - 1 - i;
            for (int v = 0; v < 3; ++v) W[3 * i + v] = W[3 * src + v];
            if (kind == HOS_BC_REFLECT) W[3 * i + 1] = -W[3 * src + 1];
        }
    }
}

}  // namespace

extern "C" {

int oracle1d_init(const hos1d_params* p) {
    P = *p;
    if (!(p->order == 5 || p->order == 7 || p->order == 9)) return 2;
    if (p->df_mode != 1 && p->order != 5) return 2;
    if (p->ghost < p->order / 2 + 1) return 2;
    G = p->ghost;
    NX = p->nodex + 2 * G;
    DX = (p->right - p->left) / p->nodex;
    KK = p->K;
    GAM = p->gamma;
    W.assign(3 * NX, 0.0);
    Wold.assign(3 * NX, 0.0);
    AL.assign(NX, 0.0);
    Itf z;
    std::memset(&z, 0, sizeof z);
    IF.assign(NX + 1, z);
    FL.assign((NX + 1) * 2 * 6, 0.0);
    return 0;
}

void oracle1d_set_state(const double* convar) { std::memcpy(W.data(), convar, 3 * NX * sizeof(double)); }

void oracle1d_get_state(double* convar, double* alpha) {
    if (convar) std::memcpy(convar, W.data(), 3 * NX * sizeof(double));
    if (alpha) std::memcpy(alpha, AL.data(), NX * sizeof(double));
}

int oracle1d_step(double tstop, double t, int step, double* dt_out) {
    const int g = G, nx = NX;
    for (int i = g; i < g + P.nodex; ++i)
        for (int v = 0; v < 3; ++v) Wold[3 * i + v] = W[3 * i + v];
    // Get_CFL 1D: fresh conserved state, seeded with dx
    double dt = DX;
    for (int i = 0; i < P.nodex; ++i) {
        double pr[3];
        to_prim(pr, &W[3 * (i + g)]);
        double tmp = std::abs(pr[1]) + std::sqrt(GAM * pr[2] / pr[0]);
        if (tmp > P.cfl * DX / dt) dt = P.cfl * DX / tmp;
    }
    if (t + dt > tstop) dt = tstop - t + 1e-15;
    if (dt_out) *dt_out = dt;
    const bool df = P.df_mode == 1 || (P.df_mode == 2 && step > 0);
    for (int stage = 0; stage < 2; ++stage) {
        bc1();
        for (int i = g - 1; i < nx - g + 1; ++i) recon_cell(i, df, IF[i].right, IF[i + 1].left);
        for (int i = g; i < nx - g + 1; ++i) {
            double* o = &FL[(i * 2 + stage) * 6];
            gks1(IF[i], dt, o, o + 3);
        }
        // stage combination per face (Update 1D, src/time_advance.cpp:170-192) and update
        for (int i = g; i < P.nodex + g; ++i)
            for (int j = 0; j < 3; ++j) {
                double Fi = 0.0, Fi1 = 0.0;
                for (int k = 0; k < stage + 1; ++k) {
                    const double* q = &FL[(i * 2 + k) * 6];
                    const double* q1 = &FL[((i + 1) * 2 + k) * 6];
                    Fi = Fi + TC[stage][k][0] * q[j] + TC[stage][k][1] * q[3 + j];
                    Fi1 = Fi1 + TC[stage][k][0] * q1[j] + TC[stage][k][1] * q1[3 + j];
                }
                W[3 * i + j] = Wold[3 * i + j] + 1.0 / DX * (Fi - Fi1);
            }
        if (P.update_alpha) {
            for (int i = g; i < P.nodex + g; ++i) {
                double a[2];
                for (int s = 0; s < 2; ++s) {
                    double pl[3], pr[3];
                    to_prim(pl, IF[i + s].left.convar);
                    to_prim(pr, IF[i + s].right.convar);
                    a[s] = alpha_k1(pl, pr);
                    a[s] = a[s] < 2.0 ? 0.0 : a[s];
                }
                AL[i] = a[0] + a[1];
            }
        }
    }
    return 0;
}

}  // extern "C"
