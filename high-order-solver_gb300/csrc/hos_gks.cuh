// hos_gks.cuh -- device math of the second-order gas-kinetic (GKS) flux at one Gauss point,
// templated on the compute type T.
//
// Follows GKS2D (src/flux_function.cpp:345-698 in the reference project) for the branch the
// hot path uses: gks2nd, Euler collision time (tau = 0, tau_num from c1/c2), S2O4 (two time
// levels dt and dt/2).  The centre (g0) state is computed once here; the reference computes
// the same collision twice (src/reconstruction.cpp:3652-3687 and again inside GKS2D).
//
// Maxwellian moments <u^i v^j xi^2k> (MMDF2d, src/basic_function.cpp:110-187) are formed on
// the fly from the 1D half/full-space moment recurrences instead of materialising the three
// 7x7x3 tables: the entry (i, j, k) is uplus[i] * vwhole[j] * xi_k exactly as the table
// constructor computes it, so only the entries the contractions touch are ever evaluated.
#pragma once
#include <type_traits>
#include "hos_weno.cuh"

namespace hos {

// half / full space moments of one Maxwellian.  init_half fills the u > 0 / u < 0 moments
// (the left and right states' tables); init_whole only the full-space ones (the centre
// state's table, which GKS2D contracts with G_address alone).
template <class T> struct Mom {
    T up[7], un[7], uw[7], vw[7], xi2, xi4;
    __device__ __forceinline__ void whole(T u, T v, T ol, T K) {
        uw[0] = T(1);
        uw[1] = u;
#pragma unroll
        for (int i = 2; i <= 6; ++i) uw[i] = u * uw[i - 1] + T(0.5 * (i - 1)) * ol * uw[i - 2];
        vw[0] = T(1);
        vw[1] = v;
#pragma unroll
        for (int i = 2; i <= 6; ++i) vw[i] = v * vw[i - 1] + T(0.5 * (i - 1)) * ol * vw[i - 2];
        xi2 = T(0.5) * K * ol;
        xi4 = T(0.25) * (K * K + T(2) * K) * ol * ol;
    }
    __device__ __forceinline__ void init_whole(T u, T v, T lambda, T K) { whole(u, v, T(1.0) / lambda, K); }
    __device__ __forceinline__ void init_half(T u, T v, T lambda, T K) {
        constexpr double pi = 3.14159265358979323846;
        const T ol = T(1.0) / lambda;
        whole(u, v, ol, K);
        up[0] = T(0.5) * ferfc(T(sqrt(lambda) * -u));
        un[0] = T(1.0) - up[0];
        up[1] = u * up[0] + T(0.5) * (fexp(T(-lambda * u * u)) / sqrt(T(pi) * lambda));
        un[1] = u - up[1];
#pragma unroll
        for (int i = 2; i <= 6; ++i) {
            up[i] = u * up[i - 1] + T(0.5 * (i - 1)) * ol * up[i - 2];
            un[i] = uw[i] - up[i];
        }
    }
};

// table selectors: 0 = u > 0 half space, 1 = u < 0 half space, 2 = whole space.  The
// reference's whole-space table is uplus*v + uminus*v, equal to uwhole*v to within one
// rounding; the whole-space recurrence is used directly.
//
// For the paired FP32 type the unit factors vw[0] = uw[0] = 1 are left out (x * 1 == x, but a
// paired multiply is not folded away); the scalar types keep the products as written.
template <class T, int TAB>
__device__ __forceinline__ T M(const Mom<T>& m, int i, int j, int k) {
    if constexpr (std::is_same<T, F2>::value) {
        const T xk = k == 1 ? m.xi2 : m.xi4;
        const T& ui = TAB == 0 ? m.up[i] : TAB == 1 ? m.un[i] : m.uw[i];
        if (TAB == 2 && i == 0) {
            if (j == 0) return k == 0 ? T(1) : xk;
            return k == 0 ? m.vw[j] : T(m.vw[j] * xk);
        }
        if (j == 0) return k == 0 ? ui : T(ui * xk);
        return k == 0 ? T(ui * m.vw[j]) : T(ui * m.vw[j] * xk);
    } else {
        const T xk = k == 0 ? T(1) : k == 1 ? m.xi2 : m.xi4;
        if (TAB == 0) return k == 0 ? m.up[i] * m.vw[j] : m.up[i] * m.vw[j] * xk;
        if (TAB == 1) return k == 0 ? m.un[i] * m.vw[j] : m.un[i] * m.vw[j] * xk;
        return k == 0 ? m.uw[i] * m.vw[j] : m.uw[i] * m.vw[j] * xk;
    }
}

// moment contraction <a psi u^NU v^NV> (GL_address / GR_address / G_address, :603-636)
template <class T, int TAB, int NU, int NV>
__device__ __forceinline__ void contract(const Mom<T>& m, const T* a, T* psi) {
    constexpr int u = NU, v = NV;
#define HM(i, j, k) M<T, TAB>(m, i, j, k)
    psi[0] = a[0] * HM(u, v, 0) + a[1] * HM(u + 1, v, 0) + a[2] * HM(u, v + 1, 0) + a[3] * T(0.5) * (HM(u + 2, v, 0) + HM(u, v + 2, 0) + HM(u, v, 1));
    psi[1] = a[0] * HM(u + 1, v, 0) + a[1] * HM(u + 2, v, 0) + a[2] * HM(u + 1, v + 1, 0) + a[3] * T(0.5) * (HM(u + 3, v, 0) + HM(u + 1, v + 2, 0) + HM(u + 1, v, 1));
    psi[2] = a[0] * HM(u, v + 1, 0) + a[1] * HM(u + 1, v + 1, 0) + a[2] * HM(u, v + 2, 0) + a[3] * T(0.5) * (HM(u + 2, v + 1, 0) + HM(u, v + 3, 0) + HM(u, v + 1, 1));
    psi[3] = T(0.5) * (a[0] * (HM(u + 2, v, 0) + HM(u, v + 2, 0) + HM(u, v, 1)) +
                       a[1] * (HM(u + 3, v, 0) + HM(u + 1, v + 2, 0) + HM(u + 1, v, 1)) +
                       a[2] * (HM(u + 2, v + 1, 0) + HM(u, v + 3, 0) + HM(u, v + 1, 1)) +
                       a[3] * T(0.5) * (HM(u + 4, v, 0) + HM(u, v + 4, 0) + HM(u, v, 2) + T(2) * HM(u + 2, v + 2, 0) +
                                        T(2) * HM(u + 2, v, 1) + T(2) * HM(u, v + 2, 1)));
#undef HM
}

// contraction with a = (1, 0, 0, 0): the moments <psi u^NU v^NV> themselves
template <class T, int TAB, int NU, int NV>
__device__ __forceinline__ void contract_unit(const Mom<T>& m, T* psi) {
    constexpr int u = NU, v = NV;
#define HM(i, j, k) M<T, TAB>(m, i, j, k)
    psi[0] = HM(u, v, 0);
    psi[1] = HM(u + 1, v, 0);
    psi[2] = HM(u, v + 1, 0);
    psi[3] = T(0.5) * (HM(u + 2, v, 0) + HM(u, v + 2, 0) + HM(u, v, 1));
#undef HM
}

// micro-slope a from a macroscopic slope (A, src/basic_function.cpp:571-583);
// K enters through hK = (K + 2) / 2 and c4K = 4 / (K + 2)
template <class T> struct GasK {
    T K, hK, c4K;
    __device__ __forceinline__ explicit GasK(T k) : K(k), hK(T(0.5) * (k + T(2))), c4K(T(4.0) / (k + T(2))) {}
};
template <class T>
__device__ __forceinline__ void microslope(T* a, const T* der, const T* prim, const GasK<T>& gk) {
    const T overden = T(1.0) / prim[0];
    const T q = prim[1] * prim[1] + prim[2] * prim[2] + gk.hK / prim[3];
    const T R4 = der[3] * overden - T(0.5) * q * der[0] * overden;
    const T R3 = (der[2] - prim[2] * der[0]) * overden;
    const T R2 = (der[1] - prim[1] * der[0]) * overden;
    a[3] = gk.c4K * prim[3] * prim[3] * (T(2) * R4 - T(2) * prim[1] * R2 - T(2) * prim[2] * R3);
    a[2] = T(2) * prim[3] * R3 - prim[2] * a[3];
    a[1] = T(2) * prim[3] * R2 - prim[1] * a[3];
    a[0] = der[0] * overden - prim[1] * a[1] - prim[2] * a[2] - T(0.5) * a[3] * q;
}

template <class T>
__device__ __forceinline__ void to_ulambda(T* pr, const T* w, T K) {
    const T ir = T(1.0) / w[0];
    pr[0] = w[0];
    pr[1] = w[1] * ir;
    pr[2] = w[2] * ir;
    pr[3] = lambda_of(w[0], pr[1], pr[2], w[3], K);
}

// Euler-type numerical collision time tau_num = c1 dt + dt C (Get_Tau,
// src/basic_function.cpp:663-708); C depends only on the left/right states, so it is formed
// once for both time levels.
template <class T>
__device__ __forceinline__ T tau_ratio(T dl, T dr, T ll, T lr, T c2) {
    const T a = dl / ll, b = dr / lr;
    return c2 * fabsT(a - b) / fabsT(a + b);
}
template <class T, class S>
__device__ __forceinline__ T tau_num(T Cc, T dt, S c1, S c2) {
    if (c1 <= S(0) && c2 <= S(0)) return T(0.0);
    return T(c1) * dt + dt * Cc;
}

// Gauss-point state: convar[4], der1x[4], der1y[4] of one side
template <class T> struct GState { T w[4], dx[4], dy[4]; };

// The centre (g0) part and the time integration of GKS2D's Euler form at one Gauss point
// (src/flux_function.cpp:410-690 with tau = 0): from the collision state w0 and its slopes c0x,
// c0y, the sides' <u psi> moments gl, gr (SUMMED, the FP32 form: gl already holds rl gl + rr gr,
// gr is unused, and the time levels are folded as described below),
// the <a u^2 + a u v> terms t1s, and the sides' densities rl, rr and lambdas ll, lr.
template <class T, bool SUMMED = false>
__device__ __forceinline__ void gks_tail(const T* w0, const T* c0x, const T* c0y, const T* gl, const T* gr,
                                         const T* t1s, T rl, T rr, T ll, T lr, T dt, T K,
                                         typename ScalarOf<T>::type c1, typename ScalarOf<T>::type c2, T* fo,
                                         T* dfo) {
    const GasK<T> gk(K);
    T p0[4];
    to_ulambda(p0, w0, K);
    T g0u[4], t4s[4], A0u[4];
    {
        Mom<T> m0;
        m0.init_whole(p0[1], p0[2], p0[3], K);
        contract_unit<T, 2, 1, 0>(m0, g0u);
        T a0x[4], a0y[4], a0xu[4], a0xuu[4], a0yv[4], a0yuv[4];
        microslope(a0x, c0x, p0, gk);
        contract<T, 2, 1, 0>(m0, a0x, a0xu);
        contract<T, 2, 2, 0>(m0, a0x, a0xuu);
        microslope(a0y, c0y, p0, gk);
        contract<T, 2, 0, 1>(m0, a0y, a0yv);
        contract<T, 2, 1, 1>(m0, a0y, a0yuv);
        T dA0[4], A0[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            t4s[v] = a0xuu[v] + a0yuv[v];
            dA0[v] = -p0[0] * (a0xu[v] + a0yv[v]);
        }
        microslope(A0, dA0, p0, gk);
        contract<T, 2, 1, 0>(m0, A0, A0u);
    }
    const T Cc = tau_ratio(rl, rr, ll, lr, T(c2));
    if constexpr (SUMMED) {
        // FP32 form.  The Euler collision time is proportional to the time level,
        // tau_num(h) = (c1 + C) h, so exp(-h / tau_num) is the same at h = dt and dt/2 and every
        // time coefficient below scales exactly as h (t0, t3) or h^2 (t1, t4, t5).  In
        // 4 F(dt/2) - F(dt) the h^2 terms cancel and the h terms stay once; in
        // 4 (F(dt) - 2 F(dt/2)) the h terms cancel and the h^2 terms stay twice.  The two
        // results are formed that way, from the dt level alone, without the cancellation.
        const T tn = tau_num(Cc, dt, c1, c2);
        const T eta = fexp(T(-dt / tn));
        const T t0 = tn * (T(1) - eta);
        const T t1 = tn * (eta * (dt + tn) - tn);
        const T t3 = tn * eta + dt - tn;
        const T t4 = tn * (tn - eta * (dt + tn));
        const T r3 = p0[0] * t3, d1 = T(2) * t1, d4 = T(2) * p0[0] * t4, d5 = p0[0] * dt * dt;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            fo[v] = t0 * gl[v] + r3 * g0u[v];
            dfo[v] = d1 * t1s[v] + d4 * t4s[v] + d5 * A0u[v];
        }
        return;
    }
    // time-integration coefficients for tau = 0 (Euler) at dt and dt/2
    T F0[4], F1[4];
    {
        const T tn = tau_num(Cc, dt, c1, c2);
        const T eta = fexp(T(-dt / tn));
        const T t0 = tn * (T(1) - eta);
        const T t1 = tn * (eta * (dt + tn) - tn);
        const T t3 = tn * eta + dt - tn;
        const T t4 = tn * (tn - eta * (dt + tn));
        const T t5 = T(0.5) * dt * dt;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            T f = rl * t0 * gl[v] + rr * t0 * gr[v];
            f = f + p0[0] * t3 * g0u[v];
            f = f + t1 * t1s[v];
            f = f + p0[0] * t4 * t4s[v];
            f = f + p0[0] * t5 * A0u[v];
            F0[v] = f;
        }
    }
    {
        const T dt2 = T(0.5) * dt;
        const T tn = tau_num(Cc, dt2, c1, c2);
        const T eta = fexp(T(-dt2 / tn));
        const T t0 = tn * (T(1) - eta);
        const T t1 = tn * (eta * (dt2 + tn) - tn);
        const T t3 = tn * eta + dt2 - tn;
        const T t4 = tn * (tn - eta * (dt2 + tn));
        const T t5 = T(0.5) * dt2 * dt2;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            T f = t0 * (rl * gl[v] + rr * gr[v]);
            f = f + t1 * t1s[v];
            f = f + p0[0] * t3 * g0u[v];
            f = f + p0[0] * t4 * t4s[v];
            f = f + p0[0] * t5 * A0u[v];
            F1[v] = f;
        }
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        fo[v] = (T(4.0) * F1[v] - F0[v]);
        dfo[v] = T(4.0) * (F0[v] - T(2.0) * F1[v]);
    }
}

// Time-integrated GKS flux at one Gauss point: fo = 4 F(dt/2) - F(dt),
// dfo = 4 (F(dt) - 2 F(dt/2)) (src/flux_function.cpp:686-690).  T = F2 computes two Gauss
// points at once (c1, c2 stay scalars: the launch's collision coefficients).
template <class T>
__device__ __forceinline__ void gks_point(const GState<T>& L, const GState<T>& R, T dt, T K,
                                          typename ScalarOf<T>::type c1, typename ScalarOf<T>::type c2, T* fo,
                                          T* dfo) {
    const GasK<T> gk(K);
    T pl[4], pr[4], p0[4];
    to_ulambda(pl, L.w, K);
    to_ulambda(pr, R.w, K);
    // partial results assembled into the two time levels at the end (same accumulation order
    // as the reference): glu, gru and the <a u^2 + a u v> terms.  With tau = 0 the
    // coefficient t[2] of the <A u> half-space terms is identically zero, so those terms
    // (src/flux_function.cpp:528-567) are not formed.
    T glu[4], gru[4], t1s[4], w0[4], c0x[4], c0y[4];
    {
        Mom<T> ml, mr;
        ml.init_half(pl[1], pl[2], pl[3], K);
        mr.init_half(pr[1], pr[2], pr[3], K);
        // collision (Collision, src/basic_function.cpp:561-569)
        w0[0] = pl[0] * ml.up[0] + pr[0] * mr.un[0];
        w0[1] = pl[0] * ml.up[1] + pr[0] * mr.un[1];
        w0[2] = pl[0] * ml.vw[1] * ml.up[0] + pr[0] * mr.vw[1] * mr.un[0];
        w0[3] = T(0.5) * pl[0] * (ml.up[2] + ml.up[0] * ml.vw[2] + ml.up[0] * ml.xi2) +
                T(0.5) * pr[0] * (mr.un[2] + mr.un[0] * mr.vw[2] + mr.un[0] * mr.xi2);
        T alx[4], arx[4], aly[4], ary[4], q0[4], q1[4], q2[4], q3[4];
        microslope(alx, L.dx, pl, gk);
        microslope(arx, R.dx, pr, gk);
        microslope(aly, L.dy, pl, gk);
        microslope(ary, R.dy, pr, gk);
        contract<T, 0, 0, 0>(ml, alx, q0);
        contract<T, 1, 0, 0>(mr, arx, q1);
        contract<T, 0, 0, 0>(ml, aly, q2);
        contract<T, 1, 0, 0>(mr, ary, q3);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            c0x[v] = pl[0] * q0[v] + pr[0] * q1[v];
            c0y[v] = pl[0] * q2[v] + pr[0] * q3[v];
        }
        contract_unit<T, 0, 1, 0>(ml, glu);
        contract_unit<T, 1, 1, 0>(mr, gru);
        contract<T, 0, 2, 0>(ml, alx, q0);   // alxuul
        contract<T, 1, 2, 0>(mr, arx, q1);   // arxuur
        contract<T, 0, 1, 1>(ml, aly, q2);   // alyuvl
        contract<T, 1, 1, 1>(mr, ary, q3);   // aryuvr
#pragma unroll
        for (int v = 0; v < 4; ++v) t1s[v] = pl[0] * (q0[v] + q2[v]) + pr[0] * (q1[v] + q3[v]);
    }
    gks_tail<T>(w0, c0x, c0y, glu, gru, t1s, pl[0], pr[0], pl[3], pr[3], dt, K, c1, c2, fo, dfo);
}

// FP32 GKS2D (Euler form) at one Gauss point with the two sides in the two lanes of the paired
// FP32 type: lane x carries the left state and the u > 0 half space of its Maxwellian, lane y
// the right state and the u < 0 half space of its own.  The side terms of the collision, its
// slopes and the <u psi> and <a u^2 + a u v> moments are formed on both lanes at once and
// summed across them; the centre part (one state) is scalar.  The u < 0 half-space moments
// follow the same recurrence as the u > 0 ones (0.5 erfc(+sqrt(lambda) u) and the opposite sign
// of the boundary term), not 1 - up and uw - up.
// alpha (not null): the DF indicator contribution of the point (Calculate_alpha_k,
// src/reconstruction.cpp:1463-1476) from the lanes' (rho, u, v, lambda): the pressure is
// beta rho / lambda and the squared sound speed gamma beta / lambda, beta = (gamma - 1)(K + 2) / 4,
// so |pl - pr| / pl + |pl - pr| / pr = |ql - qr| (1 / ql + 1 / qr) with q = rho / lambda, and
// 1 / c = sqrt(lambda / (gamma beta)); the squared Mach differences add normal first (dir 0) or
// tangential first (dir 1), as the reference's y faces do after the rotation back.
__device__ __forceinline__ void gks_point_lr(const GState<float>& L, const GState<float>& R, float dt, float K,
                                             float c1, float c2, float* fo, float* dfo, float gamma = 0.0f,
                                             int dir = 0, float* alpha = nullptr) {
    const F2 Kp(K);
    const GasK<F2> gk(Kp);
    F2 w[4], sx[4], sy[4], ps[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        w[v] = F2(L.w[v], R.w[v]);
        sx[v] = F2(L.dx[v], R.dx[v]);
        sy[v] = F2(L.dy[v], R.dy[v]);
    }
    to_ulambda(ps, w, Kp);
    const F2 r = ps[0];
    auto hs = [](F2 a) { return a.v.x + a.v.y; };
    float w0[4], c0x[4], c0y[4], gs[4], t1s[4];
    {
        constexpr double pi = 3.14159265358979323846;
        Mom<F2> m;   // up[] holds the lanes' half-space moments
        const F2 u = ps[1], lam = ps[3], ol = F2(1.0f) / lam;
        if (alpha) {
            const F2 q = r * ol, iq = F2(1.0f) / q;
            const float igb = 4.0f / (gamma * (gamma - 1.0f) * (K + 2.0f));
            const F2 ic = sqrt(F2(lam * F2(igb)));
            const F2 mn = u * ic, mt = ps[2] * ic;
            const float dn = mn.v.x - mn.v.y, dtg = mt.v.x - mt.v.y;
            const float a = fabsf(q.v.x - q.v.y) * (iq.v.x + iq.v.y);
            *alpha = dir == 0 ? a + dn * dn + dtg * dtg : a + dtg * dtg + dn * dn;
        }
        m.whole(u, ps[2], ol, Kp);
        m.up[0] = F2(0.5f) * ferfc(F2(F2(-1.0f, 1.0f) * sqrt(lam) * u));
        m.up[1] = u * m.up[0] + F2(0.5f, -0.5f) * (fexp(-F2(lam * u * u)) / sqrt(F2(pi) * lam));
#pragma unroll
        for (int i = 2; i <= 6; ++i) m.up[i] = u * m.up[i - 1] + F2(0.5 * (i - 1)) * ol * m.up[i - 2];
        w0[0] = hs(r * m.up[0]);
        w0[1] = hs(r * m.up[1]);
        w0[2] = hs(r * m.vw[1] * m.up[0]);
        w0[3] = hs(F2(0.5f) * r * (m.up[2] + m.up[0] * m.vw[2] + m.up[0] * m.xi2));
        F2 ax[4], ay[4], q[4], q2[4];
        microslope(ax, sx, ps, gk);
        microslope(ay, sy, ps, gk);
        contract<F2, 0, 0, 0>(m, ax, q);
#pragma unroll
        for (int v = 0; v < 4; ++v) c0x[v] = hs(r * q[v]);
        contract<F2, 0, 0, 0>(m, ay, q);
#pragma unroll
        for (int v = 0; v < 4; ++v) c0y[v] = hs(r * q[v]);
        contract_unit<F2, 0, 1, 0>(m, q);
#pragma unroll
        for (int v = 0; v < 4; ++v) gs[v] = hs(r * q[v]);
        contract<F2, 0, 2, 0>(m, ax, q);    // <a_x u^2>
        contract<F2, 0, 1, 1>(m, ay, q2);   // <a_y u v>
#pragma unroll
        for (int v = 0; v < 4; ++v) t1s[v] = hs(r * (q[v] + q2[v]));
    }
    gks_tail<float, true>(w0, c0x, c0y, gs, nullptr, t1s, r.v.x, r.v.y, ps[3].v.x, ps[3].v.y, dt, K, c1, c2, fo,
                          dfo);
}

// Navier-Stokes collision times (tau_type NS): Get_Tau_NS and Get_Tau
// (src/basic_function.cpp:638-708) with viscosity Mu (or Nu when Mu <= 0)
template <class T>
struct NsParam {
    T c2, mu, nu, prc;   // prc: Prandtl fix factor 1/Pr - 1, 0 when the fix is off
};
template <class T>
__device__ __forceinline__ T tau_phys(const NsParam<T>& q, T d0, T l0) {
    if (q.mu > T(0)) return T(2.0) * q.mu * l0 / d0;
    if (q.nu > T(0)) return T(2) * q.nu * l0;
    return T(0);
}
template <class T>
__device__ __forceinline__ T tau_num_ns(const NsParam<T>& q, T ratio, T dt, T d0, T l0) {
    T tn = ratio * dt;   // c2 |rho_l/lambda_l - rho_r/lambda_r| / |... + ...| dt
    if (tn != tn) tn = T(0);
    if ((q.mu > T(0) && q.nu > T(0)) || (q.mu < T(0) && q.nu < T(0))) return T(0);
    if (q.mu > T(0)) return tn + T(2.0) * q.mu * l0 / d0;
    if (q.nu > T(0)) return tn + T(2) * q.nu * l0;
    return T(0);
}

// GKS2D with the Navier-Stokes collision time at one Gauss point: the full set of
// time-integration coefficients with tau != 0 (src/flux_function.cpp:410-690), including the
// <A u> half-space terms of both sides and the Prandtl fix of the energy flux.  The face
// kernel branches between this and the Euler form once per launch (tau_type is uniform).
template <class T>
__device__ __forceinline__ void gks_point_ns(const GState<T>& L, const GState<T>& R, T dt, T K, const NsParam<T> q,
                                          T* fo, T* dfo) {
    const GasK<T> gk(K);
    T pl[4], pr[4], p0[4];
    to_ulambda(pl, L.w, K);
    to_ulambda(pr, R.w, K);
    T glu[4], gru[4], t1s[4], t2s[4], w0[4], c0x[4], c0y[4];
    {
        Mom<T> ml, mr;
        ml.init_half(pl[1], pl[2], pl[3], K);
        mr.init_half(pr[1], pr[2], pr[3], K);
        w0[0] = pl[0] * ml.up[0] + pr[0] * mr.un[0];
        w0[1] = pl[0] * ml.up[1] + pr[0] * mr.un[1];
        w0[2] = pl[0] * ml.vw[1] * ml.up[0] + pr[0] * mr.vw[1] * mr.un[0];
        w0[3] = T(0.5) * pl[0] * (ml.up[2] + ml.up[0] * ml.vw[2] + ml.up[0] * ml.xi2) +
                T(0.5) * pr[0] * (mr.un[2] + mr.un[0] * mr.vw[2] + mr.un[0] * mr.xi2);
        T alx[4], arx[4], aly[4], ary[4], q0[4], q1[4], q2[4], q3[4];
        microslope(alx, L.dx, pl, gk);
        microslope(arx, R.dx, pr, gk);
        microslope(aly, L.dy, pl, gk);
        microslope(ary, R.dy, pr, gk);
        contract<T, 0, 0, 0>(ml, alx, q0);
        contract<T, 1, 0, 0>(mr, arx, q1);
        contract<T, 0, 0, 0>(ml, aly, q2);
        contract<T, 1, 0, 0>(mr, ary, q3);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            c0x[v] = pl[0] * q0[v] + pr[0] * q1[v];
            c0y[v] = pl[0] * q2[v] + pr[0] * q3[v];
        }
        contract_unit<T, 0, 1, 0>(ml, glu);
        contract_unit<T, 1, 1, 0>(mr, gru);
        contract<T, 0, 2, 0>(ml, alx, q0);
        contract<T, 1, 2, 0>(mr, arx, q1);
        contract<T, 0, 1, 1>(ml, aly, q2);
        contract<T, 1, 1, 1>(mr, ary, q3);
#pragma unroll
        for (int v = 0; v < 4; ++v) t1s[v] = pl[0] * (q0[v] + q2[v]) + pr[0] * (q1[v] + q3[v]);
        // time derivatives of the sides' distributions from the compatibility condition,
        // with the whole-space moments of each side's Maxwellian (:528-567)
        T dl[4], dr[4], Al[4], Ar[4];
        contract<T, 2, 1, 0>(ml, alx, q0);
        contract<T, 2, 0, 1>(ml, aly, q2);
        contract<T, 2, 1, 0>(mr, arx, q1);
        contract<T, 2, 0, 1>(mr, ary, q3);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            dl[v] = -pl[0] * (q0[v] + q2[v]);
            dr[v] = -pr[0] * (q1[v] + q3[v]);
        }
        microslope(Al, dl, pl, gk);
        microslope(Ar, dr, pr, gk);
        contract<T, 0, 1, 0>(ml, Al, q0);
        contract<T, 1, 1, 0>(mr, Ar, q1);
#pragma unroll
        for (int v = 0; v < 4; ++v) t2s[v] = pl[0] * q0[v] + pr[0] * q1[v];
    }
    to_ulambda(p0, w0, K);
    T g0u[4], a0xuu[4], t4s[4], A0u[4];
    {
        Mom<T> m0;
        m0.init_whole(p0[1], p0[2], p0[3], K);
        contract_unit<T, 2, 1, 0>(m0, g0u);
        T a0x[4], a0y[4], a0xu[4], a0yv[4], a0yuv[4];
        microslope(a0x, c0x, p0, gk);
        contract<T, 2, 1, 0>(m0, a0x, a0xu);
        contract<T, 2, 2, 0>(m0, a0x, a0xuu);
        microslope(a0y, c0y, p0, gk);
        contract<T, 2, 0, 1>(m0, a0y, a0yv);
        contract<T, 2, 1, 1>(m0, a0y, a0yuv);
        T dA0[4], A0[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            t4s[v] = a0xuu[v] + a0yuv[v];
            dA0[v] = -p0[0] * (a0xu[v] + a0yv[v]);
        }
        microslope(A0, dA0, p0, gk);
        contract<T, 2, 1, 0>(m0, A0, A0u);
    }
    const T tau = tau_phys(q, p0[0], p0[3]);
    const T ratio = tau_ratio(pl[0], pr[0], pl[3], pr[3], q.c2);
    // heat-flux correction of the Prandtl fix (:630-636, :678-684)
    const T qs0 = a0xuu[3] + A0u[3] - p0[1] * (a0xuu[1] + A0u[1]) - p0[2] * (a0xuu[2] + A0u[2]);
    T F[2][4];
#pragma unroll
    for (int lev = 0; lev < 2; ++lev) {
        const T h = lev == 0 ? dt : T(0.5) * dt;
        const T tn = tau_num_ns(q, ratio, h, p0[0], p0[3]);
        const T eta = fexp(T(-h / tn));
        const T t0 = tn * (T(1) - eta);
        const T t1 = tn * (eta * (h + tn) - tn) + tau * tn * (eta - T(1));
        const T t2 = tau * tn * (eta - T(1));
        const T t3 = tn * eta + h - tn;
        const T t4 = tn * (tn - eta * (h + tn) - tau * (eta - T(1))) - h * tau;
        const T t5 = T(0.5) * h * h - tau * tn * (eta - T(1)) - tau * h;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            T f;
            if (lev == 0) {
                f = pl[0] * t0 * glu[v] + pr[0] * t0 * gru[v];
                f = f + p0[0] * t3 * g0u[v];
                f = f + t1 * t1s[v];
                f = f + t2 * t2s[v];
            } else {
                f = t0 * (pl[0] * glu[v] + pr[0] * gru[v]);
                f = f + t1 * t1s[v];
                f = f + t2 * t2s[v];
                f = f + p0[0] * t3 * g0u[v];
            }
            f = f + p0[0] * t4 * t4s[v];
            f = f + p0[0] * t5 * A0u[v];
            F[lev][v] = f;
        }
        if (q.prc != T(0)) F[lev][3] += q.prc * (qs0 * (-p0[0] * tau * h));
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        fo[v] = (T(4.0) * F[1][v] - F[0][v]);
        dfo[v] = T(4.0) * (F[0][v] - T(2.0) * F[1][v]);
    }
}

// Lax-Friedrichs flux times dt of one Gauss point in the face frame (LF2D,
// src/flux_function.cpp:700-735): the larger of |u| + c on the two sides as dissipation.
template <class T>
__device__ __forceinline__ void lf_point(const T* wl, const T* wr, T dt, T gamma, T* f) {
    T pl[4], pr[4];
    to_prim(pl, wl, gamma);
    to_prim(pr, wr, gamma);
    const T kl = fabsT(pl[1]) + sqrt(gamma * pl[3] / pl[0]);
    const T kr = fabsT(pr[1]) + sqrt(gamma * pr[3] / pr[0]);
    const T beta = kr > kl ? kr : kl;
    const T ig = T(1.0) / (gamma - T(1.0));
    T fl[4], fr[4];
    const T* q[2] = {pl, pr};
    T* o[2] = {fl, fr};
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
        const T* p = q[sd];
        o[sd][0] = p[0] * p[1];
        o[sd][1] = p[0] * p[1] * p[1] + p[3];
        o[sd][2] = p[0] * p[1] * p[2];
        const T e = T(0.5) * (p[1] * p[1] + p[2] * p[2]) * p[0] + p[3] * ig;
        o[sd][3] = p[1] * (e + p[3]);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) f[m] = dt * (T(0.5) * ((fl[m] + fr[m]) - beta * (wr[m] - wl[m])));
}


// Centre (g0) state of a Gauss point and its x / y slopes (Center_all_collision_2d_multi,
// src/reconstruction.cpp:3652-3687): the collision of the left and right Maxwellians' half
// spaces and the half-space moments of their micro-slopes, in conserved variables.
template <class T>
__device__ __forceinline__ void centre_state(const GState<T>& L, const GState<T>& R, T K, T* w0, T* c0x, T* c0y) {
    const GasK<T> gk(K);
    T pl[4], pr[4];
    to_ulambda(pl, L.w, K);
    to_ulambda(pr, R.w, K);
    Mom<T> ml, mr;
    ml.init_half(pl[1], pl[2], pl[3], K);
    mr.init_half(pr[1], pr[2], pr[3], K);
    w0[0] = pl[0] * ml.up[0] + pr[0] * mr.un[0];
    w0[1] = pl[0] * ml.up[1] + pr[0] * mr.un[1];
    w0[2] = pl[0] * ml.vw[1] * ml.up[0] + pr[0] * mr.vw[1] * mr.un[0];
    w0[3] = T(0.5) * pl[0] * (ml.up[2] + ml.up[0] * ml.vw[2] + ml.up[0] * ml.xi2) +
            T(0.5) * pr[0] * (mr.un[2] + mr.un[0] * mr.vw[2] + mr.un[0] * mr.xi2);
    T alx[4], arx[4], aly[4], ary[4], q0[4], q1[4], q2[4], q3[4];
    microslope(alx, L.dx, pl, gk);
    microslope(arx, R.dx, pr, gk);
    microslope(aly, L.dy, pl, gk);
    microslope(ary, R.dy, pr, gk);
    contract<T, 0, 0, 0>(ml, alx, q0);
    contract<T, 1, 0, 0>(mr, arx, q1);
    contract<T, 0, 0, 0>(ml, aly, q2);
    contract<T, 1, 0, 0>(mr, ary, q3);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        c0x[v] = pl[0] * q0[v] + pr[0] * q1[v];
        c0y[v] = pl[0] * q2[v] + pr[0] * q3[v];
    }
}

// LF2D's viscous term with the Navier-Stokes collision time (NS_by_central_difference_prim_2D,
// src/flux_function.cpp:737-754) added to the Lax-Friedrichs flux f, as the reference writes
// it: the centre state's entries are read as (rho, u, v, T) and their slopes as slopes of
// those, although the centre state holds conserved variables (rho, rho u, rho v, rho E);
// mu = Mu, or Nu rho when Nu > 0; heat-flux factor (K + 4) / (2 Pr).
template <class T>
__device__ __forceinline__ void lf_viscous(const GState<T>& L, const GState<T>& R, T dt, T K, T mu_c, T nu_c, T pr,
                                           T* f) {
    T w0[4], cx[4], cy[4];
    centre_state<T>(L, R, K, w0, cx, cy);
    T mu = mu_c;
    if (nu_c > T(0)) mu = nu_c * w0[0];
    const T u = w0[1], v = w0[2];
    const T ux = cx[1], vx = cx[2], uy = cy[1], vy = cy[2];
    const T tau_xx = T(2) * mu * ux - T(2.0 / 3.0) * mu * (ux + vy);
    const T tau_xy = mu * (uy + vx);
    const T q = u * tau_xx + v * tau_xy + (K + T(4)) / (T(2) * pr) * mu * cx[3];
    f[1] += tau_xx * dt;
    f[2] += tau_xy * dt;
    f[3] += q * dt;
}

}  // namespace hos
