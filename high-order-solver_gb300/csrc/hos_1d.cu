// hos_1d.cu -- the 1D step (SodTubeProblem / accuracy_sinwave_1d path of the reference) on
// the GPU, and its C ABI (hos1d_* in include/hos_gb300.h).
//
// One stage = bc1d -> face1d (normal reconstruction of the tile's cells staged in shared
// memory, 1D GKS flux per face, S2O4 stage combination) -> update1d.  One step adds
// begin1d.  Differences of the 1D reference path from 2D that are reproduced here:
//   * CFL from the conserved state at the start of the step (not lagged), seed dx,
//     clip tstop - t + 1e-15 (src/time_advance.cpp:75-111);
//   * non-DF WENO5-AO (epsilon 1e-10, full 5th-order indicator) at step 0 of the Sod driver
//     (src/1Dproblem.cpp:103-106, src/reconstruction.cpp:161-360);
//   * 1D moments: u<0 half-space moments from their own recurrence, divisions by lambda
//     (MMDF1d, src/basic_function.cpp:16-99);
//   * the dt/2 time level evaluates the collision time with dt (src/flux_function.cpp:236);
//   * no blow-up check in the 1D drivers; the status bit is still set on NaN or negative
//     density/pressure so the caller can stop.
#include <cstring>
#include <new>
#include <string>

#include "../../include/hos_gb300.h"
#include "hos_launch.h"

namespace hos {
namespace d1 {

struct Ctl {
    double dt, t;
    unsigned long long cfl_bits;
    unsigned int status, active;
    int step;      // steps completed
    int pad;
};

struct Geo {
    int nx, g, nodex, order, characteristic, df_mode, update_alpha;
    int wenotype;   // weights of the non-DF WENO5-AO steps (HOS_WENO_*)
    double dx, cfl, gamma, K, c1, c2;
    int bc[2];
};

constexpr int TILE = 128;  // faces per CTA

template <class T>
__device__ __forceinline__ void prim1(T* pr, const T* w, T gamma) {
    const T ir = T(1.0) / w[0];
    pr[0] = w[0];
    pr[1] = w[1] * ir;
    pr[2] = (gamma - T(1.0)) * (w[2] - T(0.5) * w[1] * pr[1]);
}
template <class T>
__device__ __forceinline__ T lambda1(T rho, T u, T rhoE, T K) {
    return (K + T(1.0)) * T(0.25) * (rho / (rhoE - T(0.5) * rho * (u * u)));
}
template <class T>
__device__ __forceinline__ bool reduce1(const T* w, T K) {
    T lam = lambda1(w[0], w[1] / w[0], w[2], K);
    return lam <= T(0) || !(lam == lam);
}

// characteristic projection of the 1D Euler system at a base (rho, u, p)
// (Convar_to_char1D / Char_to_convar1D, src/basic_function.cpp:868-921)
template <class T> struct Char1 {
    T s00, s01, s02, s10, s11, s12, s20, s21, s22;
    T u, c, h;
    __device__ __forceinline__ void init(const T* b, T gamma) {
        c = sqrt(gamma * b[2] / b[0]);
        const T alfa = (gamma - T(1.0)) / (T(2.0) * c * c);
        u = b[1];
        const T cg = c / (gamma - T(1.0));
        s00 = alfa * (T(0.5) * u * u + u * cg); s01 = alfa * (-u - cg); s02 = alfa;
        s10 = alfa * (-u * u + T(2.0) * c * cg); s11 = alfa * T(2.0) * u; s12 = T(-2.0) * alfa;
        s20 = alfa * (T(0.5) * u * u - u * cg); s21 = alfa * (-u + cg); s22 = alfa;
        h = T(0.5) * u * u + c * cg;
    }
    __device__ __forceinline__ void to_char(T* ch, const T* w) const {
        ch[0] = s00 * w[0] + s01 * w[1] + s02 * w[2];
        ch[1] = s10 * w[0] + s11 * w[1] + s12 * w[2];
        ch[2] = s20 * w[0] + s21 * w[1] + s22 * w[2];
    }
    __device__ __forceinline__ void from_char(T* w, const T* ch) const {
        w[0] = ch[0] + ch[1] + ch[2];
        w[1] = (u - c) * ch[0] + u * ch[1] + (u + c) * ch[2];
        w[2] = (h - u * c) * ch[0] + T(0.5) * u * u * ch[1] + (h + u * c) * ch[2];
    }
};

// non-DF WENO5-AO weights: weights5 (hos_weno.cuh), epsilon 1e-10, the wenotype weights

// 1D Maxwellian moments (MMDF1d); entries (i, k) = moment_i * xi_k, i <= 6, k <= 2
template <class T> struct Mom1 {
    T up[7], un[7], uw[7], xi2, xi4;
    __device__ __forceinline__ void whole(T u, T lambda, T K) {
        uw[0] = T(1);
        uw[1] = u;
#pragma unroll
        for (int i = 2; i <= 6; ++i) uw[i] = u * uw[i - 1] + T(0.5 * (i - 1)) / lambda * uw[i - 2];
        xi2 = T(0.5) * K / lambda;
        xi4 = T(0.25) * (K * K + T(2) * K) / (lambda * lambda);
    }
    __device__ __forceinline__ void half(T u, T lambda, T K) {
        constexpr double pi = 3.14159265358979323846;
        whole(u, lambda, K);
        const T sl = sqrt(lambda);
        up[0] = T(0.5) * erfc(sl * -u);
        un[0] = T(0.5) * erfc(sl * u);
        const T b = exp(-lambda * u * u) / sqrt(T(pi) * lambda);
        up[1] = u * up[0] + T(0.5) * b;
        un[1] = u * un[0] - T(0.5) * b;
#pragma unroll
        for (int i = 2; i <= 6; ++i) {
            up[i] = u * up[i - 1] + T(0.5 * (i - 1)) / lambda * up[i - 2];
            un[i] = u * un[i - 1] + T(0.5 * (i - 1)) / lambda * un[i - 2];
        }
    }
};
template <class T, int TAB>
__device__ __forceinline__ T M1(const Mom1<T>& m, int i, int k) {
    const T* a = TAB == 0 ? m.up : TAB == 1 ? m.un : m.uw;
    return k == 0 ? a[i] : k == 1 ? a[i] * m.xi2 : a[i] * m.xi4;
}
// G / GL / GR (src/basic_function.cpp:522-548)
template <class T, int TAB, int NU>
__device__ __forceinline__ void g1(const Mom1<T>& m, const T* a, T* psi) {
    constexpr int u = NU;
#define H1(i, k) M1<T, TAB>(m, i, k)
    psi[0] = a[0] * H1(u, 0) + a[1] * H1(u + 1, 0) + a[2] * T(0.5) * (H1(u + 2, 0) + H1(u, 1));
    psi[1] = a[0] * H1(u + 1, 0) + a[1] * H1(u + 2, 0) + a[2] * T(0.5) * (H1(u + 3, 0) + H1(u + 1, 1));
    psi[2] = T(0.5) * (a[0] * (H1(u + 2, 0) + H1(u, 1)) + a[1] * (H1(u + 3, 0) + H1(u + 1, 1)) +
                       a[2] * T(0.5) * (H1(u + 4, 0) + H1(u, 2) + T(2) * H1(u + 2, 1)));
#undef H1
}
// Microslope (src/basic_function.cpp:551-559)
template <class T>
__device__ __forceinline__ void slope1(T* a, const T* der, const T* prim, T K) {
    const T q = prim[1] * prim[1] + T(0.5) * (K + T(1)) / prim[2];
    const T R4 = der[2] / prim[0] - T(0.5) * q * der[0] / prim[0];
    const T R2 = (der[1] - prim[1] * der[0]) / prim[0];
    a[2] = T(4) * prim[2] * prim[2] / (K + T(1)) * (T(2) * R4 - T(2) * prim[1] * R2);
    a[1] = T(2) * prim[2] * R2 - prim[1] * a[2];
    a[0] = der[0] / prim[0] - prim[1] * a[1] - T(0.5) * a[2] * q;
}
template <class T>
__device__ __forceinline__ void ulambda1(T* pr, const T* w, T K) {
    pr[0] = w[0];
    pr[1] = w[1] / w[0];
    pr[2] = lambda1(w[0], pr[1], w[2], K);
}

// 1D GKS flux at a face from left/right states and slopes (GKS, src/flux_function.cpp:16-276,
// centre state by Center_collision, src/reconstruction.cpp:1375-1407; tau = 0)
template <class T>
__device__ void gks1(const T* L, const T* R, T dt, const Geo& geo, T* fo, T* dfo) {
    const T K = T(geo.K);
    T pl[3], pr[3], p0[3], c0[3], c0d[3];
    ulambda1(pl, L, K);
    ulambda1(pr, R, K);
    T glu[3], gru[3], t1l[3], t1r[3];
    {
        Mom1<T> ml, mr;
        ml.half(pl[1], pl[2], K);
        mr.half(pr[1], pr[2], K);
        const T unit[3] = {T(1), T(0), T(0)};
        T gl[3], gr[3], axl[3], axr[3], q0[3], q1[3];
        g1<T, 0, 0>(ml, unit, gl);
        g1<T, 1, 0>(mr, unit, gr);
        slope1(axl, L + 3, pl, K);
        slope1(axr, R + 3, pr, K);
        g1<T, 0, 0>(ml, axl, q0);
        g1<T, 1, 0>(mr, axr, q1);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            c0[i] = L[0] * gl[i] + R[0] * gr[i];
            c0d[i] = L[0] * q0[i] + R[0] * q1[i];
        }
        g1<T, 0, 1>(ml, unit, glu);
        g1<T, 1, 1>(mr, unit, gru);
        g1<T, 0, 2>(ml, axl, t1l);
        g1<T, 1, 2>(mr, axr, t1r);
    }
    ulambda1(p0, c0, K);
    T g0u[3], a0xuu[3], A0u[3];
    {
        Mom1<T> m0;
        m0.whole(p0[1], p0[2], K);
        const T unit[3] = {T(1), T(0), T(0)};
        g1<T, 2, 1>(m0, unit, g0u);
        T a0x[3], a0xu[3], dA0[3], A0[3];
        slope1(a0x, c0d, p0, K);
        g1<T, 2, 1>(m0, a0x, a0xu);
        g1<T, 2, 2>(m0, a0x, a0xuu);
#pragma unroll
        for (int i = 0; i < 3; ++i) dA0[i] = -p0[0] * (a0xu[i]);
        slope1(A0, dA0, p0, K);
        g1<T, 2, 1>(m0, A0, A0u);
    }
    const T c1 = T(geo.c1), c2 = T(geo.c2);
    T tn = T(0);
    if (!(c1 <= T(0) && c2 <= T(0))) {
        const T a = pl[0] / pl[2], b = pr[0] / pr[2];
        tn = c1 * dt + dt * (c2 * fabsT(a - b) / fabsT(a + b));
    }
    T F0[3], F1[3];
    {
        const T eta = exp(-dt / tn);
        const T t0 = tn * (T(1) - eta), t1 = tn * (eta * (dt + tn) - tn), t3 = tn * eta + dt - tn;
        const T t4 = tn * (tn - eta * (dt + tn)), t5 = T(0.5) * dt * dt;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            T f = pl[0] * t0 * glu[i] + pr[0] * t0 * gru[i];
            f = f + p0[0] * t3 * g0u[i];
            f = f + pl[0] * t1 * t1l[i] + pr[0] * t1 * t1r[i];
            f = f + p0[0] * t4 * a0xuu[i];
            f = f + p0[0] * t5 * A0u[i];
            F0[i] = f;
        }
    }
    {
        const T dt2 = T(0.5) * dt;   // tau_num stays that of dt in the 1D reference
        const T eta = exp(-dt2 / tn);
        const T t0 = tn * (T(1) - eta), t1 = tn * (eta * (dt2 + tn) - tn), t3 = tn * eta + dt2 - tn;
        const T t4 = tn * (tn - eta * (dt2 + tn)), t5 = T(0.5) * dt2 * dt2;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            T f = pl[0] * t0 * glu[i] + pr[0] * t0 * gru[i];
            f = f + pl[0] * t1 * t1l[i] + pr[0] * t1 * t1r[i];
            f = f + p0[0] * t3 * g0u[i];
            f = f + p0[0] * t4 * a0xuu[i];
            f = f + p0[0] * t5 * A0u[i];
            F1[i] = f;
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        fo[i] = T(4.0) * F1[i] - F0[i];
        dfo[i] = T(4.0) * (F0[i] - T(2.0) * F1[i]);
    }
}

// DF indicator of a face (Calculate_alpha_k_1d, src/reconstruction.cpp:362-372), thresholded
template <class T>
__device__ __forceinline__ T face_alpha1(const T* L, const T* R, T gamma) {
    T pl[3], pr[3];
    prim1(pl, L, gamma);
    prim1(pr, R, gamma);
    const T Ml = pl[1] / sqrt(gamma * pl[2] / pl[0]);
    const T Mr = pr[1] / sqrt(gamma * pr[2] / pr[0]);
    T A = fabsT(pl[2] - pr[2]) / pl[2] + fabsT(pl[2] - pr[2]) / pr[2];
    A = A + (Ml - Mr) * (Ml - Mr);
    return A < T(2.0) ? T(0.0) : A;
}

struct FaceArgs1 {
    const double* W;
    const double* AL;
    double* FX;   // stage combination per face [3][nodex+1]
    double* FP;   // stage-0 partial [3][nodex+1]
    double* FA;   // face DF indicator [nodex+1]
    const Ctl* ctl;
    int stage;
};

template <class T, int ORDER>
__global__ void __launch_bounds__(TILE) face1d_kernel(FaceArgs1 a, Geo geo) {
    constexpr int r = ORDER / 2, N = ORDER, NW = AO<ORDER>::N;
    if (!a.ctl->active) return;
    __shared__ T lines[TILE][2][6];   // [face][side][convar 3, der 3]
    const int F0 = blockIdx.x * TILE;
    const int g = geo.g, nodex = geo.nodex;
    const T gamma = T(geo.gamma), K = T(geo.K), ih = T(1.0 / geo.dx);
    const bool df = geo.df_mode == 1 || (geo.df_mode == 2 && a.ctl->step > 0);
    // phase 1: cells c = g + F0 - 1 + k for k in [0, TILE]
    for (int k = threadIdx.x; k <= TILE; k += TILE) {
        const int c = g + F0 - 1 + k;
        if (c > g + nodex) continue;
        T st[N][3], al[N];
#pragma unroll
        for (int q = 0; q < N; ++q) {
            const int ci = c + q - r;
#pragma unroll
            for (int v = 0; v < 3; ++v) st[q][v] = T(a.W[v * geo.nx + ci]);
            al[q] = T(a.AL[ci]);
        }
        T dfa[NW];
        if (df) df_factors<T, ORDER>(al, dfa);
        else {
#pragma unroll
            for (int q = 0; q < NW; ++q) dfa[q] = T(1);
        }
        T out[2][6];
        Char1<T> cb[2];
        T ch[2][N][3];
        if (geo.characteristic) {
            T pn1[3], p0[3], pp1[3], b0[3], b1[3];
            prim1(pn1, st[r - 1], gamma);
            prim1(p0, st[r], gamma);
            prim1(pp1, st[r + 1], gamma);
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                b0[v] = T(0.5) * (pn1[v] + p0[v]);
                b1[v] = T(0.5) * (pp1[v] + p0[v]);
            }
            cb[0].init(b0, gamma);
            cb[1].init(b1, gamma);
#pragma unroll
            for (int q = 0; q < N; ++q) {
                cb[0].to_char(ch[0][q], st[q]);
                // WENO9: the right side keeps the left base's projection of its outermost entries
                if (ORDER == 9 && (q == 0 || q == N - 1)) {
#pragma unroll
                    for (int v = 0; v < 3; ++v) ch[1][q][v] = ch[0][q][v];
                } else {
                    cb[1].to_char(ch[1][q], st[q]);
                }
            }
        } else {
#pragma unroll
            for (int sd = 0; sd < 2; ++sd)
#pragma unroll
                for (int q = 0; q < N; ++q)
#pragma unroll
                    for (int v = 0; v < 3; ++v) ch[sd][q][v] = st[q][v];
        }
#pragma unroll
        for (int sd = 0; sd < 2; ++sd) {
            T var[3], der[3];
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                T s[N], fw[NW], p[NW], px[NW];
#pragma unroll
                for (int q = 0; q < N; ++q) s[q] = ch[sd][q][v];
                if (ORDER == 5 && !df) weights5<T>(s, T(1e-10), fw, geo.wenotype);
                else ao_weights<T, ORDER>(s, fw);
                if (sd == 0) normal_face<T, ORDER, 0>(s, dfa, ih, p, px);
                else normal_face<T, ORDER, 1>(s, dfa, ih, p, px);
                T x = T(0), y = T(0);
#pragma unroll
                for (int q = 0; q < NW; ++q) { x += fw[q] * p[q]; y += fw[q] * px[q]; }
                var[v] = x;
                der[v] = y;
            }
            if (geo.characteristic) {
                cb[sd].from_char(out[sd], var);
                cb[sd].from_char(out[sd] + 3, der);
            } else {
#pragma unroll
                for (int v = 0; v < 3; ++v) { out[sd][v] = var[v]; out[sd][3 + v] = der[v]; }
            }
        }
        if (reduce1(out[1], K) || reduce1(out[0], K)) {
#pragma unroll
            for (int sd = 0; sd < 2; ++sd)
#pragma unroll
                for (int v = 0; v < 3; ++v) { out[sd][v] = st[r][v]; out[sd][3 + v] = T(0); }
        }
        // left-face value -> right side of face c; right-face value -> left side of face c+1
        const int fl = c - (g + F0);
        if (fl >= 0 && fl < TILE)
#pragma unroll
            for (int q = 0; q < 6; ++q) lines[fl][1][q] = out[0][q];
        if (fl + 1 >= 0 && fl + 1 < TILE)
#pragma unroll
            for (int q = 0; q < 6; ++q) lines[fl + 1][0][q] = out[1][q];
    }
    __syncthreads();
    // phase 2: GKS flux per face and the S2O4 stage combination (FP64)
    const int f = threadIdx.x, face = F0 + f;
    if (face > nodex) return;
    const size_t nf = (size_t)nodex + 1;
    T Ls[6], Rs[6], fo[3], dfo[3];
#pragma unroll
    for (int q = 0; q < 6; ++q) { Ls[q] = lines[f][0][q]; Rs[q] = lines[f][1][q]; }
    gks1<T>(Ls, Rs, T(a.ctl->dt), geo, fo, dfo);
#pragma unroll
    for (int v = 0; v < 3; ++v) {
        const double fv = double(fo[v]), dv = double(dfo[v]);
        if (a.stage == 0) {
            a.FX[v * nf + face] = 0.5 * fv + (1.0 / 8.0) * dv;
            a.FP[v * nf + face] = 1.0 * fv + (1.0 / 6.0) * dv;
        } else {
            a.FX[v * nf + face] = a.FP[v * nf + face] + (1.0 / 3.0) * dv;
        }
    }
    if (geo.update_alpha) a.FA[face] = double(face_alpha1<T>(Ls, Rs, gamma));
}

__global__ void bc1d_kernel(double* W, Geo geo, const Ctl* ctl) {
    if (ctl && !ctl->active) return;
    const int k = threadIdx.x;
    if (k >= 2 * geo.g) return;
    const int side = k < geo.g ? 0 : 1;
    const int i = side == 0 ? k : geo.nx - 2 * geo.g + k;
    const int kind = geo.bc[side], g = geo.g, nx = geo.nx;
    int src;
    if (kind == HOS_BC_FREE) src = side == 0 ? g : nx - g - 1;
    else if (kind == HOS_BC_PERIODIC) src = side == 0 ? i + geo.nodex : i - geo.nodex;
    else src = side == 0 ? 2 * g - 1 - i : 2 * (nx - g) - 1 - i;
    for (int v = 0; v < 3; ++v) W[v * nx + i] = W[v * nx + src];
    if (kind == HOS_BC_REFLECT) W[nx + i] = -W[nx + src];
}

__device__ __forceinline__ double cfl_candidate1(const double* w, const Geo& geo, bool& bad) {
    double pr[3];
    prim1<double>(pr, w, geo.gamma);
    bad = pr[0] < 0 || pr[2] < 0 || isnan(pr[0]) || isnan(pr[2]);
    const double tmp = fabs(pr[1]) + sqrt(geo.gamma * pr[2] / pr[0]);
    const double q = geo.cfl * geo.dx / tmp;
    return q > 0 ? q : 1e300;
}

__device__ __forceinline__ void reduce_min_bad(double cand, unsigned bad, Ctl* ctl, bool do_cfl) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cand = fmin(cand, __shfl_xor_sync(0xffffffffu, cand, o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (do_cfl && cand < 1e300) atomicMin(&ctl->cfl_bits, (unsigned long long)__double_as_longlong(cand));
        if (bad) atomicOr(&ctl->status, 1u);
    }
}

// W = Wold + (F_i - F_{i+1}) / dx (Update 1D, src/time_advance.cpp:183-192), DF indicators,
// and at stage 1 the CFL candidates of the new state (the next step's Get_CFL)
__global__ void __launch_bounds__(256) update1d_kernel(double* W, double* Wold, double* AL, const double* FX,
                                                       const double* FA, Ctl* ctl, Geo geo, int stage) {
    if (!ctl->active) return;
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    double cand = 1e300;
    unsigned bad = 0;
    if (I < geo.nodex) {
        const int c = I + geo.g, nx = geo.nx;
        const size_t nf = (size_t)geo.nodex + 1;
        double w[3];
        for (int v = 0; v < 3; ++v) {
            double old;
            if (stage == 0) {
                old = W[v * nx + c];
                Wold[v * nx + c] = old;
            } else {
                old = Wold[v * nx + c];
            }
            w[v] = old + 1.0 / geo.dx * (FX[v * nf + I] - FX[v * nf + I + 1]);
            W[v * nx + c] = w[v];
        }
        if (geo.update_alpha) AL[c] = FA[I] + FA[I + 1];
        bool b;
        const double q = cfl_candidate1(w, geo, b);
        bad = b ? 1u : 0u;
        if (stage == 1) cand = q;
    }
    reduce_min_bad(cand, bad, ctl, stage == 1);
}

__global__ void __launch_bounds__(256) cfl1d_init_kernel(const double* W, Ctl* ctl, Geo geo) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    double cand = 1e300;
    unsigned bad = 0;
    if (I < geo.nodex) {
        const int c = I + geo.g;
        double w[3] = {W[c], W[geo.nx + c], W[2 * geo.nx + c]};
        bool b;
        cand = cfl_candidate1(w, geo, b);
        bad = b ? 1u : 0u;
    }
    reduce_min_bad(cand, bad, ctl, true);
}

__global__ void begin1d_kernel(Ctl* ctl, double tstop, double seed, int first) {
    if (!first) ctl->step += ctl->active ? 1 : 0;
    const double t = ctl->t;
    ctl->active = t < tstop ? 1u : 0u;
    double dt = __longlong_as_double((long long)ctl->cfl_bits);
    ctl->cfl_bits = (unsigned long long)__double_as_longlong(seed);
    if (!(t < tstop)) return;
    if (t + dt > tstop) dt = tstop - t + 1e-15;
    ctl->dt = dt;
    ctl->t = t + dt;
}

template <class T, int ORDER>
cudaError_t launch_face(const FaceArgs1& a, const Geo& geo, cudaStream_t s) {
    face1d_kernel<T, ORDER><<<(geo.nodex + 1 + TILE - 1) / TILE, TILE, 0, s>>>(a, geo);
    return cudaGetLastError();
}

thread_local std::string g_err1;
int fail1(int code, const std::string& m) {
    g_err1 = m;
    return code;
}

}  // namespace d1
}  // namespace hos

using namespace hos;
using namespace hos::d1;

struct hos_solver1d {
    hos_params1d p;
    int precision = 0;
    Geo geo;
    cudaStream_t stream = nullptr;
    double *W = nullptr, *Wold = nullptr, *AL = nullptr, *FX = nullptr, *FP = nullptr, *FA = nullptr, *stage = nullptr;
    Ctl* ctl = nullptr;
    bool first = true;
};

namespace {

void free1(hos_solver1d* s) {
    double* b[] = {s->W, s->Wold, s->AL, s->FX, s->FP, s->FA, s->stage};
    for (double* x : b)
        if (x) cudaFree(x);
    if (s->ctl) cudaFree(s->ctl);
    if (s->stream) cudaStreamDestroy(s->stream);
}

int enqueue_begin1(hos_solver1d* s, double tstop) {
    begin1d_kernel<<<1, 1, 0, s->stream>>>(s->ctl, tstop, s->geo.dx, s->first ? 1 : 0);
    s->first = false;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HOS_OK : fail1(HOS_E_CUDA, std::string("begin1d: ") + cudaGetErrorString(e));
}

int enqueue_stage1(hos_solver1d* s, int stage) {
    const Geo& geo = s->geo;
    bc1d_kernel<<<1, 32, 0, s->stream>>>(s->W, geo, s->ctl);
    FaceArgs1 fa{s->W, s->AL, s->FX, s->FP, s->FA, s->ctl, stage};
    cudaError_t e;
    if (s->precision == 0)
        e = geo.order == 5 ? launch_face<double, 5>(fa, geo, s->stream)
          : geo.order == 7 ? launch_face<double, 7>(fa, geo, s->stream)
                           : launch_face<double, 9>(fa, geo, s->stream);
    else
        e = geo.order == 5 ? launch_face<float, 5>(fa, geo, s->stream)
          : geo.order == 7 ? launch_face<float, 7>(fa, geo, s->stream)
                           : launch_face<float, 9>(fa, geo, s->stream);
    if (e != cudaSuccess) return fail1(HOS_E_CUDA, std::string("face1d: ") + cudaGetErrorString(e));
    update1d_kernel<<<(geo.nodex + 255) / 256, 256, 0, s->stream>>>(s->W, s->Wold, s->AL, s->FX, s->FA, s->ctl, geo, stage);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail1(HOS_E_CUDA, std::string("update1d: ") + cudaGetErrorString(e));
    return HOS_OK;
}

int enqueue_step1(hos_solver1d* s, double tstop) {
    int st = enqueue_begin1(s, tstop);
    for (int stage = 0; stage < 2 && !st; ++stage) st = enqueue_stage1(s, stage);
    return st;
}

int check_bc1(const int* bc) {
    for (int k = 0; k < 2; ++k)
        if (bc[k] < 0 || bc[k] > 2) return fail1(HOS_E_CONFIG, "1D boundaries: free, periodic or reflective");
    if ((bc[0] == HOS_BC_PERIODIC) != (bc[1] == HOS_BC_PERIODIC)) return fail1(HOS_E_CONFIG, "periodic boundaries must be paired");
    return HOS_OK;
}

}  // namespace

extern "C" {

const char* hos1d_last_error(void) { return g_err1.c_str(); }

int hos1d_create(const hos_params1d* params, int precision, hos_solver1d** out) {
    if (!params || !out) return fail1(HOS_E_ARG, "null argument");
    const hos_params1d& p = *params;
    if (!(p.order == 5 || p.order == 7 || p.order == 9)) return fail1(HOS_E_CONFIG, "order must be 5, 7 or 9");
    if (p.df_mode != 1 && p.order != 5) return fail1(HOS_E_CONFIG, "the non-DF variant exists for WENO5 only");
    if (p.df_mode < 0 || p.df_mode > 2) return fail1(HOS_E_CONFIG, "bad df_mode");
    if (p.wenotype < HOS_WENO_Z || p.wenotype > HOS_WENO_LINEAR) return fail1(HOS_E_CONFIG, "bad wenotype");
    if (p.ghost < p.order / 2 + 1 || p.nodex < p.ghost) return fail1(HOS_E_CONFIG, "ghost/nodex too small");
    if (p.ghost > 16) return fail1(HOS_E_CONFIG, "ghost must be <= 16");  // one warp fills both ends
    if (int st = check_bc1(p.bc)) return st;
    if (precision != HOS_FP64 && precision != HOS_FP32) return fail1(HOS_E_CONFIG, "bad precision");
    hos_solver1d* s = new (std::nothrow) hos_solver1d();
    if (!s) return fail1(HOS_E_NOMEM, "host allocation");
    s->p = p;
    s->precision = precision;
    Geo& geo = s->geo;
    geo.nx = p.nodex + 2 * p.ghost;
    geo.g = p.ghost;
    geo.nodex = p.nodex;
    geo.order = p.order;
    geo.characteristic = p.characteristic ? 1 : 0;
    geo.df_mode = p.df_mode;
    geo.update_alpha = p.update_alpha ? 1 : 0;
    geo.wenotype = p.wenotype;
    geo.dx = (p.right - p.left) / p.nodex;
    geo.cfl = p.cfl;
    geo.gamma = p.gamma;
    geo.K = p.K;
    geo.c1 = p.c1_euler;
    geo.c2 = p.c2_euler;
    geo.bc[0] = p.bc[0];
    geo.bc[1] = p.bc[1];
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return fail1(HOS_E_CUDA, std::string("stream: ") + cudaGetErrorString(e));
    }
    const size_t nx = geo.nx, nf = (size_t)p.nodex + 1;
    struct { double** q; size_t n; } al[] = {{&s->W, 3 * nx}, {&s->Wold, 3 * nx}, {&s->AL, nx}, {&s->FX, 3 * nf},
                                             {&s->FP, 3 * nf}, {&s->FA, nf}, {&s->stage, 3 * nx}};
    for (auto& a : al) {
        if ((e = cudaMalloc(a.q, a.n * sizeof(double))) != cudaSuccess) {
            free1(s);
            delete s;
            return fail1(HOS_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        cudaMemset(*a.q, 0, a.n * sizeof(double));
    }
    if ((e = cudaMalloc(&s->ctl, sizeof(Ctl))) != cudaSuccess) {
        free1(s);
        delete s;
        return fail1(HOS_E_NOMEM, "cudaMalloc ctl");
    }
    cudaMemset(s->ctl, 0, sizeof(Ctl));
    *out = s;
    return HOS_OK;
}

int hos1d_destroy(hos_solver1d* s) {
    if (!s) return HOS_OK;
    cudaStreamSynchronize(s->stream);
    free1(s);
    delete s;
    return HOS_OK;
}

int hos1d_set_state(hos_solver1d* s, const double* convar) {
    if (!s || !convar) return fail1(HOS_E_ARG, "null argument");
    const int nx = s->geo.nx;
    std::string err;
    // AoS [nx][3] -> SoA [3][nx] on the host side of the copy (nx is small in 1D)
    double* h = new (std::nothrow) double[3 * (size_t)nx];
    if (!h) return fail1(HOS_E_NOMEM, "host staging");
    for (int i = 0; i < nx; ++i)
        for (int v = 0; v < 3; ++v) h[v * nx + i] = convar[3 * i + v];
    cudaError_t e = cudaMemcpyAsync(s->W, h, 3 * nx * sizeof(double), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->AL, 0, nx * sizeof(double), s->stream);
    Ctl c{};
    const double seed = s->geo.dx;
    std::memcpy(&c.cfl_bits, &seed, sizeof seed);
    c.active = 1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->ctl, &c, sizeof c, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
        cfl1d_init_kernel<<<(s->geo.nodex + 255) / 256, 256, 0, s->stream>>>(s->W, s->ctl, s->geo);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    delete[] h;
    if (e != cudaSuccess) return fail1(HOS_E_CUDA, std::string("set_state: ") + cudaGetErrorString(e));
    s->first = true;
    Ctl back;
    cudaMemcpy(&back, s->ctl, sizeof back, cudaMemcpyDeviceToHost);
    if (back.status & 1u) return fail1(HOS_E_BLOWUP, "initial state has negative density/pressure or NaN");
    return HOS_OK;
}

int hos1d_get_state(hos_solver1d* s, double* convar, double* alpha) {
    if (!s) return fail1(HOS_E_ARG, "null solver");
    const int nx = s->geo.nx;
    double* h = new (std::nothrow) double[3 * (size_t)nx];
    if (!h) return fail1(HOS_E_NOMEM, "host staging");
    cudaError_t e = cudaMemcpyAsync(h, s->W, 3 * nx * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess && alpha) e = cudaMemcpyAsync(alpha, s->AL, nx * sizeof(double), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && convar)
        for (int i = 0; i < nx; ++i)
            for (int v = 0; v < 3; ++v) convar[3 * i + v] = h[v * nx + i];
    delete[] h;
    return e == cudaSuccess ? HOS_OK : fail1(HOS_E_CUDA, std::string("get_state: ") + cudaGetErrorString(e));
}

int hos1d_step(hos_solver1d* s, double tstop) {
    if (!s) return fail1(HOS_E_ARG, "null solver");
    return enqueue_step1(s, tstop);
}

int hos1d_begin_step(hos_solver1d* s, double tstop) {
    if (!s) return fail1(HOS_E_ARG, "null solver");
    return enqueue_begin1(s, tstop);
}

int hos1d_stage(hos_solver1d* s, int stage) {
    if (!s) return fail1(HOS_E_ARG, "null solver");
    if (stage != 0 && stage != 1) return fail1(HOS_E_ARG, "stage must be 0 or 1");
    return enqueue_stage1(s, stage);
}

int hos1d_set_boundary(hos_solver1d* s, const int* bc) {
    if (!s || !bc) return fail1(HOS_E_ARG, "null argument");
    if (int st = check_bc1(bc)) return st;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail1(HOS_E_CUDA, std::string("set_boundary: ") + cudaGetErrorString(e));
    s->p.bc[0] = s->geo.bc[0] = bc[0];
    s->p.bc[1] = s->geo.bc[1] = bc[1];
    return HOS_OK;
}

int hos1d_set_alpha(hos_solver1d* s, const double* alpha) {
    if (!s || !alpha) return fail1(HOS_E_ARG, "null argument");
    cudaError_t e = cudaMemcpyAsync(s->AL, alpha, s->geo.nx * sizeof(double), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? HOS_OK : fail1(HOS_E_CUDA, std::string("set_alpha: ") + cudaGetErrorString(e));
}

int hos1d_set_time(hos_solver1d* s, double t) {
    if (!s) return fail1(HOS_E_ARG, "null solver");
    Ctl c;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&c, s->ctl, sizeof c, cudaMemcpyDeviceToHost);
    c.t = t;
    if (e == cudaSuccess) e = cudaMemcpy(s->ctl, &c, sizeof c, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? HOS_OK : fail1(HOS_E_CUDA, std::string("set_time: ") + cudaGetErrorString(e));
}

int hos1d_run(hos_solver1d* s, double tstop, int max_steps, int* steps_done) {
    if (!s) return fail1(HOS_E_ARG, "null solver");
    int n = 0;
    double t = 0;
    for (;;) {
        Ctl c;
        cudaError_t e = cudaStreamSynchronize(s->stream);
        if (e == cudaSuccess) e = cudaMemcpy(&c, s->ctl, sizeof c, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail1(HOS_E_CUDA, std::string("run: ") + cudaGetErrorString(e));
        if (c.status & 1u) return fail1(HOS_E_BLOWUP, "negative density/pressure or NaN in the state");
        t = c.t;
        if (!(t < tstop) || n >= max_steps) break;
        const int k = max_steps - n < 64 ? max_steps - n : 64;
        for (int q = 0; q < k; ++q) {
            int st = enqueue_step1(s, tstop);
            if (st) return st;
        }
        n += k;
    }
    if (steps_done) {
        Ctl c;
        cudaMemcpy(&c, s->ctl, sizeof c, cudaMemcpyDeviceToHost);
        *steps_done = c.step + (c.active ? 1 : 0);
    }
    return HOS_OK;
}

int hos1d_sync(hos_solver1d* s, double* t, double* dt) {
    if (!s) return fail1(HOS_E_ARG, "null solver");
    cudaError_t e = cudaStreamSynchronize(s->stream);
    Ctl c;
    if (e == cudaSuccess) e = cudaMemcpy(&c, s->ctl, sizeof c, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail1(HOS_E_CUDA, std::string("sync: ") + cudaGetErrorString(e));
    if (t) *t = c.t;
    if (dt) *dt = c.dt;
    if (c.status & 1u) return fail1(HOS_E_BLOWUP, "negative density/pressure or NaN in the state");
    return HOS_OK;
}

}  // extern "C"
