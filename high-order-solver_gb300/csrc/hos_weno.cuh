// hos_weno.cuh -- device math of the WENO-AO-DF reconstruction, templated on the compute
// type T (double for the plain path, float for the FP32-bulk path).
//
// The formulas are the published WENO-AO(5,3), (7,5,3), (9,7,5,3) reconstructions with the
// discontinuity-feedback (DF) factor, as the reference writes them in
// src/reconstruction.cpp (normal: :480-657, :750-974, :1072-1364; tangential Gauss-point
// forms: :2751-2836, :3021-3174, :3389-3609).  Coefficients and operand order follow the
// reference so that the FP64 instantiation agrees with it to rounding; the integer
// divisions 13/3 == 4 and 781/20 == 39 of its 7th-order indicator are kept.
#pragma once
#include <cuda_runtime.h>
#include "hos_f32x2.cuh"
#include "hos_linear_coef.cuh"

namespace hos {

template <class T> __device__ __forceinline__ T sq(T x) { return x * x; }
template <class T> __device__ __forceinline__ T fabsT(T x) { return x < T(0) ? -x : x; }
template <class T> __device__ __forceinline__ T fmaxT(T a, T b) { return a > b ? a : b; }
template <class T> __device__ __forceinline__ T fminT(T a, T b) { return a < b ? a : b; }

// number of candidate polynomials per order
template <int ORDER> struct AO { static constexpr int N = ORDER == 5 ? 4 : ORDER == 7 ? 5 : 6; };

// ---- conversions (src/basic_function.cpp:811-842, 1102-1177) ----
template <class T>
__device__ __forceinline__ void to_prim(T* pr, const T* w, T gamma) {
    const T ir = T(1.0) / w[0];
    pr[0] = w[0];
    pr[1] = w[1] * ir;
    pr[2] = w[2] * ir;
    pr[3] = (gamma - T(1.0)) * (w[3] - T(0.5) * (w[1] * pr[1] + w[2] * pr[2]));
}
template <class T>
__device__ __forceinline__ T lambda_of(T rho, T u, T v, T rhoE, T K) {
    return (K + T(2.0)) * T(0.25) * (rho / (rhoE - T(0.5) * rho * (u * u + v * v)));
}
template <class T>
__device__ __forceinline__ bool needs_order_reduction(const T* w, T K) {
    const T ir = T(1.0) / w[0];
    T lam = lambda_of(w[0], w[1] * ir, w[2] * ir, w[3], K);
    return lam <= T(0) || !(lam == lam);
}

// ---- characteristic projection (Convar_to_char / Char_to_convar, :923-992) ----
// Left eigenvectors of the x-direction flux Jacobian at a base primitive state, built once
// per base and applied to every stencil entry.
template <class T> struct CharBase {
    T s00, s01, s02, s03, s10, s20, s21, s22, s23, s30, s31, s32, s33;  // left
    T u, v, c, k2, h;                                                     // right
    __device__ __forceinline__ void init(const T* base, T gamma) {
        c = sqrt(gamma * base[3] / base[0]);
        T overc = T(1.0) / c;
        T alfa = (gamma - T(1.0)) * T(0.5) * overc * overc;
        u = base[1];
        v = base[2];
        T q = u * u + v * v;
        s00 = T(1.0) - alfa * q; s01 = T(2.0) * alfa * u; s02 = T(2.0) * alfa * v; s03 = T(-2.0) * alfa;
        s10 = -v;
        s20 = T(0.5) * (-u * overc + alfa * q); s21 = T(0.5) * overc - alfa * u; s22 = -alfa * v; s23 = alfa;
        s30 = T(0.5) * (u * overc + alfa * q); s31 = T(-0.5) * overc - alfa * u; s32 = -alfa * v; s33 = alfa;
        k2 = T(0.5) * q;
        h = c * c / (gamma - T(1.0));
    }
    __device__ __forceinline__ void to_char(T* ch, const T* w) const {
        ch[0] = s00 * w[0] + s01 * w[1] + s02 * w[2] + s03 * w[3];
        ch[1] = s10 * w[0] + w[2];
        ch[2] = s20 * w[0] + s21 * w[1] + s22 * w[2] + s23 * w[3];
        ch[3] = s30 * w[0] + s31 * w[1] + s32 * w[2] + s33 * w[3];
    }
    __device__ __forceinline__ void from_char(T* w, const T* ch) const {
        w[0] = ch[0] + ch[2] + ch[3];
        w[1] = u * ch[0] + (u + c) * ch[2] + (u - c) * ch[3];
        w[2] = v * ch[0] + ch[1] + v * ch[2] + v * ch[3];
        w[3] = k2 * ch[0] + v * ch[1] + (k2 + c * u + h) * ch[2] + (k2 - c * u + h) * ch[3];
    }
};

// ---- smoothness indicators ----
template <class T>
__device__ __forceinline__ void beta3(const T* s, T* b) {
    const T wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
    b[0] = T(13.0 / 12.0) * sq(wn2 - T(2.0) * wn1 + w0) + T(0.25) * sq(wn2 - T(4.0) * wn1 + T(3.0) * w0);
    b[1] = T(13.0 / 12.0) * sq(wn1 - T(2.0) * w0 + wp1) + T(0.25) * sq(wn1 - wp1);
    b[2] = T(13.0 / 12.0) * sq(w0 - T(2.0) * wp1 + wp2) + T(0.25) * sq(T(3.0) * w0 - T(4.0) * wp1 + wp2);
}
// s points at wn3 (7 entries)
template <class T>
__device__ __forceinline__ T beta7(const T* s) {
    const T wn3 = s[0], wn2 = s[1], wn1 = s[2], w0 = s[3], wp1 = s[4], wp2 = s[5], wp3 = s[6];
    T a1, a2, a3, b0, b1, b2, b3;
    a1 = (T(-19) * wn3 + T(87) * wn2 - T(177) * wn1 + T(109) * w0) * T(1.0 / (60.0));
    a2 = (-wn3 + T(4) * wn2 - T(5) * wn1 + T(2) * w0) * T(1.0 / (2));
    a3 = (-wn3 + T(3) * wn2 - T(3) * wn1 + w0) * T(1.0 / (6.0));
    b0 = (a1 + a3 * T(1.0 / (10.0))) * (a1 + a3 * T(1.0 / (10.0))) + T(4) * a2 * a2 + T(39) * a3 * a3;
    a1 = (T(11) * wn2 - T(63) * wn1 + T(33) * w0 + T(19) * wp1) * T(1.0 / (60.0));
    a2 = (wn1 - T(2) * w0 + wp1) * T(1.0 / (2));
    a3 = (-wn2 + T(3) * wn1 - T(3) * w0 + wp1) * T(1.0 / (6.0));
    b1 = (a1 + a3 * T(1.0 / (10.0))) * (a1 + a3 * T(1.0 / (10.0))) + T(4) * a2 * a2 + T(39) * a3 * a3;
    a1 = (T(-19) * wn1 - T(33) * w0 + T(63) * wp1 - T(11) * wp2) * T(1.0 / (60.0));
    a2 = (wn1 - T(2) * w0 + wp1) * T(1.0 / (2));
    a3 = (-wn1 + T(3) * w0 - T(3) * wp1 + wp2) * T(1.0 / (6.0));
    b2 = (a1 + a3 * T(1.0 / (10.0))) * (a1 + a3 * T(1.0 / (10.0))) + T(4) * a2 * a2 + T(39) * a3 * a3;
    a1 = (T(-109) * w0 + T(177) * wp1 - T(87) * wp2 + T(19) * wp3) * T(1.0 / (60.0));
    a2 = (T(2) * w0 - T(5) * wp1 + T(4) * wp2 - wp3) * T(1.0 / (2));
    a3 = (-w0 + T(3) * wp1 - T(3) * wp2 + wp3) * T(1.0 / (6.0));
    b3 = (a1 + a3 * T(1.0 / (10.0))) * (a1 + a3 * T(1.0 / (10.0))) + T(4) * a2 * a2 + T(39) * a3 * a3;
    return T(1.0 / 20.0) * (b0 + T(9.0) * b1 + T(9.0) * b2 + b3) + fabsT(b0 - b1 - b2 + b3);
}
// s points at wn4 (9 entries); b5mid returns the middle quartic indicator
template <class T>
__device__ __forceinline__ T beta9(const T* s, T& b5mid) {
    const T wn4 = s[0], wn3 = s[1], wn2 = s[2], wn1 = s[3], w0 = s[4];
    const T wp1 = s[5], wp2 = s[6], wp3 = s[7], wp4 = s[8];
    T a1, a2, a3, a4, b[5];
#define HOS_B9COMB                                                                          \
    ((a1 + a3 * T(1.0 / (10.0))) * (a1 + a3 * T(1.0 / (10.0))) +                                            \
     T(13.0 / 3.0) * (a2 + T(123.0 / 455.0) * a4) * (a2 + T(123.0 / 455.0) * a4) +          \
     T(781.0 / 20.0) * a3 * a3 + T(1421461.0 / 2275.0) * a4 * a4)
    a1 = (T(-462) * wn1 + T(336) * wn2 - T(146) * wn3 + T(27) * wn4 + T(245) * w0) * T(1.0 / (120.0));
    a2 = (T(-240) * wn1 + T(262) * wn2 - T(128) * wn3 + T(25) * wn4 + T(81) * w0) * T(1.0 / (56.0));
    a3 = (T(-18) * wn1 + T(24) * wn2 - T(14) * wn3 + T(3) * wn4 + T(5) * w0) * T(1.0 / (12.0));
    a4 = (T(-4) * wn1 + T(6) * wn2 - T(4) * wn3 + wn4 + w0) * T(1.0 / (24.0));
    b[0] = HOS_B9COMB;
    a1 = (T(-192) * wn1 + T(66) * wn2 - T(11) * wn3 + T(110) * w0 + T(27) * wp1) * T(1.0 / (120));
    a2 = (T(10) * wn1 + T(12) * wn2 - T(3) * wn3 - T(44) * w0 + T(25) * wp1) * T(1.0 / (56));
    a3 = (T(12) * wn1 - T(6) * wn2 + wn3 - T(10) * w0 + T(3) * wp1) * T(1.0 / (12));
    a4 = (T(6) * wn1 - T(4) * wn2 + wn3 - T(4) * w0 + wp1) * T(1.0 / (24));
    b[1] = HOS_B9COMB;
    a1 = (T(-82) * wn1 + T(11) * wn2 + T(82) * wp1 - T(11) * wp2) * T(1.0 / (120));
    a2 = (T(40) * wn1 - T(3) * wn2 - T(74) * w0 + T(40) * wp1 - T(3) * wp2) * T(1.0 / (56));
    a3 = (T(2) * wn1 - wn2 - T(2) * wp1 + wp2) * T(1.0 / (12));
    a4 = (T(-4) * wn1 + wn2 + T(6) * w0 - T(4) * wp1 + wp2) * T(1.0 / (24));
    b[2] = HOS_B9COMB;
    a1 = (T(-27) * wn1 - T(110) * w0 + T(192) * wp1 - T(66) * wp2 + T(11) * wp3) * T(1.0 / (120));
    a2 = (T(25) * wn1 - T(44) * w0 + T(10) * wp1 + T(12) * wp2 - T(3) * wp3) * T(1.0 / (56));
    a3 = (T(-3) * wn1 + T(10) * w0 - T(12) * wp1 + T(6) * wp2 - wp3) * T(1.0 / (12));
    a4 = (wn1 - T(4) * w0 + T(6) * wp1 - T(4) * wp2 + wp3) * T(1.0 / (24));
    b[3] = HOS_B9COMB;
    a1 = (T(-245) * w0 + T(462) * wp1 - T(336) * wp2 + T(146) * wp3 - T(27) * wp4) * T(1.0 / (120));
    a2 = (T(81) * w0 - T(240) * wp1 + T(262) * wp2 - T(128) * wp3 + T(25) * wp4) * T(1.0 / (56));
    a3 = (T(-5) * w0 + T(18) * wp1 - T(24) * wp2 + T(14) * wp3 - T(3) * wp4) * T(1.0 / (12));
    a4 = (w0 - T(4) * wp1 + T(6) * wp2 - T(4) * wp3 + wp4) * T(1.0 / (24));
    b[4] = HOS_B9COMB;
#undef HOS_B9COMB
    b5mid = b[2];
    return T(1.0 / 70.0) * (b[0] + T(16.0) * b[1] + T(36.0) * b[2] + T(16.0) * b[3] + b[4]) +
           fabsT(b[0] - b[1] - b[3] + b[4]);
}

// Linear weights d_k of the candidate polynomials (0.85 for every level, as the reference sets).
template <int ORDER>
__device__ __forceinline__ void ao_linear(double* dd) {
    constexpr double dhi = 0.85, dlo = 0.85, dav = 0.85;
    if (ORDER == 5) {
        dd[0] = (1.0 - dhi) * (1.0 - dlo) / 2.0; dd[1] = (1.0 - dhi) * dlo;
        dd[2] = (1.0 - dhi) * (1.0 - dlo) / 2.0; dd[3] = dhi;
    } else if (ORDER == 7) {
        dd[0] = (1.0 - dhi) * (1.0 - dlo) * (1.0 - dav) / 2.0; dd[1] = (1.0 - dhi) * (1.0 - dav) * dlo;
        dd[2] = (1.0 - dhi) * (1.0 - dlo) * (1.0 - dav) / 2.0; dd[3] = (1.0 - dhi) * dav; dd[4] = dhi;
    } else {
        dd[0] = (1.0 - dhi) * (1.0 - dlo) * (1.0 - dav) * (1.0 - dav) / 2.0;
        dd[1] = (1.0 - dhi) * (1.0 - dav) * (1.0 - dav) * dlo;
        dd[2] = (1.0 - dhi) * (1.0 - dlo) * (1.0 - dav) * (1.0 - dav) / 2.0;
        dd[3] = (1.0 - dhi) * (1.0 - dav) * dav; dd[4] = (1.0 - dhi) * dav; dd[5] = dhi;
    }
}

// Smoothness indicators beta_k of the candidate stencils (the last one the full stencil) and
// the global indicator tau (mean |beta_top - beta_k|); s holds the ORDER stencil entries.
template <class T, int ORDER>
__device__ __forceinline__ T ao_betas(const T* s, T* beta) {
    constexpr int N = AO<ORDER>::N;
    if (ORDER == 5) {
        beta3<T>(s, beta);
        beta[3] = T(1.0 / 6.0) * (beta[0] + T(4.0) * beta[1] + beta[2]) + fabsT(beta[0] - beta[2]);
    } else if (ORDER == 7) {
        beta3<T>(s + 1, beta);
        beta[3] = T(1.0 / 6.0) * (beta[0] + T(4.0) * beta[1] + beta[2]) + fabsT(beta[0] - beta[2]);
        beta[4] = beta7<T>(s);
    } else {
        beta3<T>(s + 2, beta);
        beta[4] = beta7<T>(s + 1);
        T mid;
        beta[5] = beta9<T>(s, mid);
        beta[3] = mid;
    }
    if (N == 4)
        return T(1.0 / 3.0) * (fabsT(beta[3] - beta[0]) + fabsT(beta[3] - beta[1]) + fabsT(beta[3] - beta[2]));
    if (N == 5)
        return T(0.25) * (fabsT(beta[4] - beta[0]) + fabsT(beta[4] - beta[1]) + fabsT(beta[4] - beta[2]) +
                          fabsT(beta[4] - beta[3]));
    return T(0.2) * (fabsT(beta[5] - beta[0]) + fabsT(beta[5] - beta[1]) + fabsT(beta[5] - beta[2]) +
                     fabsT(beta[5] - beta[3]) + fabsT(beta[5] - beta[4]));
}

// Final adaptive-order weights of the DF variants (epsilon 1e-6, Z-type weights).
template <class T, int ORDER>
__device__ __forceinline__ void ao_weights(const T* s, T* fw) {
    constexpr int N = AO<ORDER>::N;
    double dd[6];
    ao_linear<ORDER>(dd);
    T beta[6];
    const T tau = ao_betas<T, ORDER>(s, beta);
    constexpr int top = N - 1;
    T alpha[6], sum = T(0.0);
#pragma unroll
    for (int k = 0; k < N; ++k) {
        T gd = tau / (beta[k] + T(1e-6));
        alpha[k] = T(dd[k]) * (T(1.0) + gd * gd);
        sum += alpha[k];
    }
    T inv = T(1.0) / sum;
    T wtop = alpha[top] * inv;
    const T wt = wtop * T(1.0 / dd[top]);
    fw[top] = wt;
#pragma unroll
    for (int k = 0; k < top; ++k) fw[k] = alpha[k] * inv - wt * T(dd[k]);
}

// Largest distance max_k |omega_k - d_k| of the normalised nonlinear weights from the linear
// weights: 0 where the reconstruction is the linear (full-stencil) one.
template <class T, int ORDER>
__device__ __forceinline__ T ao_weight_distance(const T* s) {
    constexpr int N = AO<ORDER>::N;
    double dd[6];
    ao_linear<ORDER>(dd);
    T beta[6];
    const T tau = ao_betas<T, ORDER>(s, beta);
    T alpha[6], sum = T(0.0);
#pragma unroll
    for (int k = 0; k < N; ++k) {
        T gd = tau / (beta[k] + T(1e-6));
        alpha[k] = T(dd[k]) * (T(1.0) + gd * gd);
        sum += alpha[k];
    }
    const T inv = T(1.0) / sum;
    T dmax = T(0.0);
#pragma unroll
    for (int k = 0; k < N; ++k) dmax = fmaxT(dmax, fabsT(alpha[k] * inv - T(dd[k])));
    return dmax;
}

// DF factors from the alpha values along the stencil (e.g. :1731-1741, :1898-1909)
template <class T, int ORDER>
__device__ __forceinline__ void df_factors(const T* a, T* df) {
    T s[6];
    if (ORDER == 5) {
        s[0] = a[0] + a[2]; s[1] = a[1] + a[3]; s[2] = a[2] + a[4]; s[3] = a[0] + a[2] + a[4];
    } else if (ORDER == 7) {
        s[0] = a[1] + a[3]; s[1] = a[2] + a[4]; s[2] = a[3] + a[5]; s[3] = a[1] + a[3] + a[5];
        s[4] = a[0] + a[2] + a[4] + a[6];
    } else {
        s[0] = a[2] + a[4]; s[1] = a[3] + a[5]; s[2] = a[4] + a[6]; s[3] = a[2] + a[4] + a[6];
        s[4] = a[1] + a[3] + a[5] + a[7]; s[5] = a[0] + a[2] + a[4] + a[6] + a[8];
    }
#pragma unroll
    for (int k = 0; k < AO<ORDER>::N; ++k) df[k] = s[k] < T(2.0) ? T(1.0) : T(2.0) / s[k];
}

// the full stencil's factor alone (df_factors' last entry, the same arithmetic): the gate's
// linear path needs no other
template <class T, int ORDER>
__device__ __forceinline__ T df_full(const T* a) {
    T s;
    if (ORDER == 5) s = a[0] + a[2] + a[4];
    else if (ORDER == 7) s = a[0] + a[2] + a[4] + a[6];
    else s = a[0] + a[2] + a[4] + a[6] + a[8];
    return s < T(2.0) ? T(1.0) : T(2.0) / s;
}

// ---- candidate polynomials at the left (SIDE 0) or right (SIDE 1) face of the centre cell ----
template <class T, int ORDER, int SIDE>
__device__ __forceinline__ void normal_face(const T* s, const T* df, T ih, T* p, T* px) {
    constexpr int r = ORDER / 2;
    const T w0 = s[r], wn1 = s[r - 1], wn2 = s[r - 2], wp1 = s[r + 1], wp2 = s[r + 2];
    const T wn3 = r >= 3 ? s[r >= 3 ? r - 3 : 0] : T(0), wp3 = r >= 3 ? s[r >= 3 ? r + 3 : 0] : T(0);
    const T wn4 = r >= 4 ? s[0] : T(0), wp4 = r >= 4 ? s[r >= 4 ? r + 4 : 0] : T(0);
    if (SIDE == 0) {
        p[0] = w0 + df[0] * (T(-1.0 / 6.0) * wn2 + T(5.0 / 6.0) * wn1 + T(1.0 / 3.0) * w0 - w0);
        p[1] = w0 + df[1] * (T(1.0 / 3.0) * wn1 + T(5.0 / 6.0) * w0 - T(1.0 / 6.0) * wp1 - w0);
        p[2] = w0 + df[2] * (T(11.0 / 6.0) * w0 - T(7.0 / 6.0) * wp1 + T(1.0 / 3.0) * wp2 - w0);
        p[3] = w0 + df[3] * (T(1.0 / 60.0) * (T(47.0) * w0 + T(27.0) * wn1 - T(3.0) * wn2 - T(13.0) * wp1 + T(2.0) * wp2) - w0);
        px[0] = df[0] * (w0 - wn1) * ih;
        px[1] = df[1] * (w0 - wn1) * ih;
        px[2] = -df[2] * ((T(2.0) * w0 - T(3.0) * wp1 + wp2) * ih);
        px[3] = df[3] * (T(15.0) * w0 - T(15.0) * wn1 + wn2 - wp1) * (T(1.0 / 12.0) * ih);
        if (ORDER >= 7) {
            p[4] = w0 + df[4] * (T(1.0 / 420.0) * (T(319.0) * w0 + T(214.0) * wn1 - T(38.0) * wn2 + T(4.0) * wn3 - T(101.0) * wp1 + T(25.0) * wp2 - T(3.0) * wp3) - w0);
            px[4] = df[4] * (T(245.0) * w0 - T(245.0) * wn1 + T(25.0) * wn2 - T(2.0) * wn3 - T(25.0) * wp1 + T(2.0) * wp2) * (T(1.0 / 180.0) * ih);
        }
        if (ORDER == 9) {
            p[5] = w0 + df[5] * (T(1.0 / 2520.0) * (T(1879.0) * w0 + T(1375.0) * wn1 - T(305.0) * wn2 + T(55.0) * wn3 - T(5.0) * wn4 - T(641.0) * wp1 + T(199.0) * wp2 - T(41.0) * wp3 + T(4.0) * wp4) - w0);
            px[5] = df[5] * (T(7175.0) * w0 - T(7175.0) * wn1 + T(889.0) * wn2 - T(119.0) * wn3 + T(9.0) * wn4 - T(889.0) * wp1 + T(119.0) * wp2 - T(9.0) * wp3) * (T(1.0 / 5040.0) * ih);
        }
    } else {
        p[0] = w0 + df[0] * (T(1.0 / 3.0) * wn2 - T(7.0 / 6.0) * wn1 + T(11.0 / 6.0) * w0 - w0);
        p[1] = w0 + df[1] * (T(-1.0 / 6.0) * wn1 + T(5.0 / 6.0) * w0 + T(1.0 / 3.0) * wp1 - w0);
        p[2] = w0 + df[2] * (T(1.0 / 3.0) * w0 + T(5.0 / 6.0) * wp1 - T(1.0 / 6.0) * wp2 - w0);
        p[3] = w0 + df[3] * (T(1.0 / 60.0) * (T(47.0) * w0 - T(13.0) * wn1 + T(2.0) * wn2 + T(27.0) * wp1 - T(3.0) * wp2) - w0);
        px[0] = df[0] * (T(2.0) * w0 - T(3.0) * wn1 + wn2) * ih;
        px[1] = df[1] * (-w0 + wp1) * ih;
        px[2] = df[2] * (-w0 + wp1) * ih;
        px[3] = df[3] * (T(-15.0) * w0 + wn1 + T(15.0) * wp1 - wp2) * (T(1.0 / 12.0) * ih);
        if (ORDER >= 7) {
            p[4] = w0 + df[4] * (T(1.0 / 420.0) * (T(319.0) * w0 - T(101.0) * wn1 + T(25.0) * wn2 - T(3.0) * wn3 + T(214.0) * wp1 - T(38.0) * wp2 + T(4.0) * wp3) - w0);
            px[4] = df[4] * (T(-245.0) * w0 + T(25.0) * wn1 - T(2.0) * wn2 + T(245.0) * wp1 - T(25.0) * wp2 + T(2.0) * wp3) * (T(1.0 / 180.0) * ih);
        }
        if (ORDER == 9) {
            p[5] = w0 + df[5] * (T(1.0 / 2520.0) * (T(1879.0) * w0 - T(641.0) * wn1 + T(199.0) * wn2 - T(41.0) * wn3 + T(4.0) * wn4 + T(1375.0) * wp1 - T(305.0) * wp2 + T(55.0) * wp3 - T(5.0) * wp4) - w0);
            px[5] = df[5] * (T(-7175.0) * w0 + T(889.0) * wn1 - T(119.0) * wn2 + T(9.0) * wn3 + T(7175.0) * wp1 - T(889.0) * wp2 + T(119.0) * wp3 - T(9.0) * wp4) * (T(1.0 / 5040.0) * ih);
        }
    }
}

// ---- candidate polynomials at Gauss point IG of a face segment ----
template <class T, int ORDER>
__device__ __forceinline__ void tangent_point(int ig, const T* s, const T* df, T ih, T* p, T* px) {
    if (ORDER == 5) {
        const T wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
        constexpr double q = 1.732050807568877294;  // sqrt(3)
        if (ig == 0) {
            p[0] = w0 + df[0] * (w0 - (T(q) * w0) * T(1.0 / (4)) + (T(4) * wn1 - wn2) * T(1.0 / (4 * q)) - w0);
            p[1] = w0 + df[1] * (w0 + (wn1 - wp1) * T(1.0 / (4 * q)) - w0);
            p[2] = w0 + df[2] * (T(1.0 / 12.0) * (T(3 * (4 + q)) * w0 + T(q) * (T(-4) * wp1 + wp2)) - w0);
            p[3] = w0 + df[3] * ((T(4314) * w0 + T(4 + 500 * q) * wn1 - wn2 - T(70 * q) * wn2 + T(4) * wp1 - T(500 * q) * wp1 - wp2 + T(70 * q) * wp2) * T(1.0 / (4320)) - w0);
            px[0] = -df[0] * (T(-9 + q) * w0 - T(2 * (-6 + q)) * wn1 + T(-3 + q) * wn2) * (T(1.0 / 6) * ih);
            px[1] = -df[1] * (T(-2 * q) * w0 + T(3 + q) * wn1 + T(-3 + q) * wp1) * (T(1.0 / 6) * ih);
            px[2] = -df[2] * (T(9 + q) * w0 - T(2 * (6 + q)) * wp1 + T(3 + q) * wp2) * (T(1.0 / 6) * ih);
            px[3] = df[3] * (T(48 * q) * w0 - T(72) * wn1 - T(26 * q) * wn1 + T(9) * wn2 + T(2 * q) * wn2 + T(72) * wp1 - T(26 * q) * wp1 - T(9) * wp2 + T(2 * q) * wp2) * (T(1.0 / 108) * ih);
        } else {
            p[0] = w0 + df[0] * (T(1.0 / 12.0) * (T(3 * (4 + q)) * w0 + T(q) * (T(-4) * wn1 + wn2)) - w0);
            p[1] = w0 + df[1] * (w0 + (-wn1 + wp1) * T(1.0 / (4 * q)) - w0);
            p[2] = w0 + df[2] * (w0 - (T(q) * w0) * T(1.0 / (4)) + (T(4) * wp1 - wp2) * T(1.0 / (4 * q)) - w0);
            p[3] = w0 + df[3] * ((T(4314) * w0 + T(4 - 500 * q) * wn1 - wn2 + T(70 * q) * wn2 + T(4) * wp1 + T(500 * q) * wp1 - wp2 - T(70 * q) * wp2) * T(1.0 / (4320)) - w0);
            px[0] = df[0] * (T(9 + q) * w0 - T(2 * (6 + q)) * wn1 + T(3 + q) * wn2) * (T(1.0 / 6) * ih);
            px[1] = df[1] * (T(-2 * q) * w0 + T(-3 + q) * wn1 + T(3 + q) * wp1) * (T(1.0 / 6) * ih);
            px[2] = df[2] * (T(-9 + q) * w0 - T(2 * (-6 + q)) * wp1 + T(-3 + q) * wp2) * (T(1.0 / 6) * ih);
            px[3] = -df[3] * ((T(48 * q) * w0 + T(72) * wn1 - T(26 * q) * wn1 - T(9) * wn2 + T(2 * q) * wn2 - T(72) * wp1 - T(26 * q) * wp1 + T(9) * wp2 + T(2 * q) * wp2) * (T(1.0 / 108) * ih));
        }
    } else if (ORDER == 7) {
        const T wn3 = s[0], wn2 = s[1], wn1 = s[2], w0 = s[3], wp1 = s[4], wp2 = s[5], wp3 = s[6];
        constexpr double q = 3.872983346207417;  // sqrt(15)
        if (ig == 0) {
            p[0] = w0 + df[0] * ((T(23.0) * w0 + T(2.0) * wn1 - wn2) * T(1.0 / (24.0)) - w0);
            p[1] = w0 + df[1] * ((T(26.0) * w0 - wn1 - wp1) * T(1.0 / (24.0)) - w0);
            p[2] = w0 + df[2] * ((T(23.0) * w0 + T(2.0) * wp1 - wp2) * T(1.0 / (24.0)) - w0);
            p[3] = w0 + df[3] * ((T(2134.0) * w0 - T(116.0) * wn1 + T(9.0) * wn2 - T(116.0) * wp1 + T(9.0) * wp2) * T(1.0 / (1920.0)) - w0);
            p[4] = w0 + df[4] * ((T(121004) * w0 - T(7621) * wn1 + T(954) * wn2 - T(75) * wn3 - T(7621) * wp1 + T(954) * wp2 - T(75) * wp3) * T(1.0 / (107520.0)) - w0);
            px[0] = df[0] * (T(3.0) * w0 - T(4.0) * wn1 + wn2) * (T(1.0 / 2.0) * ih);
            px[1] = df[1] * (-wn1 + wp1) * (T(1.0 / 2.0) * ih);
            px[2] = df[2] * (T(-3.0) * w0 + T(4.0) * wp1 - wp2) * (T(1.0 / 2.0) * ih);
            px[3] = df[3] * (T(-34.0) * wn1 + T(5.0) * wn2 + T(34.0) * wp1 - T(5.0) * wp2) * (T(1.0 / 48.0) * ih);
            px[4] = df[4] * (T(-9455) * wn1 + T(2236) * wn2 - T(259) * wn3 + T(9455) * wp1 - T(2236) * wp2 + T(259) * wp3) * (T(1.0 / 11520.0) * ih);
        } else if (ig == 1) {
            p[0] = w0 + df[0] * ((T(62 - 9 * q) * w0 + T(4 * (-1 + 3 * q)) * wn1 + T(2 - 3 * q) * wn2) * T(1.0 / (60.0)) - w0);
            p[1] = w0 + df[1] * ((T(56) * w0 + T(2 + 3 * q) * wn1 + T(2 - 3 * q) * wp1) * T(1.0 / (60.0)) - w0);
            p[2] = w0 + df[2] * ((T(62 + 9 * q) * w0 - T(4 * (1 + 3 * q)) * wp1 + T(2 + 3 * q) * wp2) * T(1.0 / (60.0)) - w0);
            p[3] = w0 + df[3] * ((T(2186) * w0 + T(4 * (29 + 41 * q)) * wn1 - T(9) * wn2 - T(22 * q) * wn2 + T(116) * wp1 - T(164 * q) * wp1 - T(9) * wp2 + T(22 * q) * wp2) * T(1.0 / (2400.0)) - w0);
            p[4] = w0 + df[4] * ((T(4534440) * w0 + T(5 * (57144 + 78421 * q)) * wn1 - T(35748) * wn2 - T(84364 * q) * wn2 + T(2808) * wn3 + T(9541 * q) * wn3 + T(285720) * wp1 -
                                  T(392105 * q) * wp1 - T(35748) * wp2 + T(84364 * q) * wp2 + T(2808) * wp3 - T(9541 * q) * wp3) * T(1.0 / (5040000.0)) - w0);
            px[0] = df[0] * (-(T(-15 + q) * w0) + T(2 * (-10 + q)) * wn1 - T(-5 + q) * wn2) * (T(1.0 / 10.0) * ih);
            px[1] = df[1] * (T(2 * q) * w0 - T(5 + q) * wn1 - T(-5 + q) * wp1) * (T(1.0 / 10.0) * ih);
            px[2] = df[2] * (-(T(15 + q) * w0) + T(2 * (10 + q)) * wp1 - T(5 + q) * wp2) * (T(1.0 / 10.0) * ih);
            px[3] = df[3] * (T(78 * q) * w0 - T(2 * (95 + 21 * q)) * wn1 + T(20) * wn2 + T(3 * q) * wn2 + T(190) * wp1 - T(42 * q) * wp1 - T(20) * wp2 + T(3 * q) * wp2) * (T(1.0 / 300.0) * ih);
            px[4] = df[4] * (T(103860 * q) * w0 - T(5 * (49925 + 11619 * q)) * wn1 + T(41300) * wn2 + T(6678 * q) * wn2 - T(4325) * wn3 - T(513 * q) * wn3 + T(249625) * wp1 -
                             T(58095 * q) * wp1 - T(41300) * wp2 + T(6678 * q) * wp2 + T(4325) * wp3 - T(513 * q) * wp3) * (T(1.0 / 360000.0) * ih);
        } else {
            p[0] = w0 + df[0] * ((T(62 + 9 * q) * w0 - T(4 * (1 + 3 * q)) * wn1 + T(2 + 3 * q) * wn2) * T(1.0 / (60.0)) - w0);
            p[1] = w0 + df[1] * ((T(56) * w0 + T(2 - 3 * q) * wn1 + T(2 + 3 * q) * wp1) * T(1.0 / (60.0)) - w0);
            p[2] = w0 + df[2] * ((T(62 - 9 * q) * w0 + T(4 * (-1 + 3 * q)) * wp1 + T(2 - 3 * q) * wp2) * T(1.0 / (60.0)) - w0);
            p[3] = w0 + df[3] * ((T(2186) * w0 - T(4 * (-29 + 41 * q)) * wn1 - T(9) * wn2 + T(22 * q) * wn2 + T(116) * wp1 + T(164 * q) * wp1 - T(9) * wp2 - T(22 * q) * wp2) * T(1.0 / (2400.0)) - w0);
            p[4] = w0 + df[4] * ((T(4534440) * w0 - T(5 * (-57144 + 78421 * q)) * wn1 - T(35748) * wn2 + T(84364 * q) * wn2 + T(2808) * wn3 - T(9541 * q) * wn3 + T(285720) * wp1 +
                                  T(392105 * q) * wp1 - T(35748) * wp2 - T(84364 * q) * wp2 + T(2808) * wp3 + T(9541 * q) * wp3) * T(1.0 / (5040000.0)) - w0);
            px[0] = df[0] * (T(15 + q) * w0 - T(2 * (10 + q)) * wn1 + T(5 + q) * wn2) * (T(1.0 / 10.0) * ih);
            px[1] = df[1] * (T(-2 * q) * w0 - T(5 - q) * wn1 + T(5 + q) * wp1) * (T(1.0 / 10.0) * ih);
            px[2] = df[2] * (T(-15 + q) * w0 - T(2 * (-10 + q)) * wp1 + T(-5 + q) * wp2) * (T(1.0 / 10.0) * ih);
            px[3] = df[3] * (T(-78 * q) * w0 + T(2 * (-95 + 21 * q)) * wn1 + T(20) * wn2 - T(3 * q) * wn2 + T(190) * wp1 + T(42 * q) * wp1 - T(20) * wp2 - T(3 * q) * wp2) * (T(1.0 / 300.0) * ih);
            px[4] = df[4] * (T(-103860 * q) * w0 + T(5 * (-49925 + 11619 * q)) * wn1 + T(41300) * wn2 - T(6678 * q) * wn2 - T(4325) * wn3 + T(513 * q) * wn3 + T(249625) * wp1 +
                             T(58095 * q) * wp1 - T(41300) * wp2 - T(6678 * q) * wp2 + T(4325) * wp3 + T(513 * q) * wp3) * (T(1.0 / 360000.0) * ih);
        }
    } else {
        // 9th order: the polynomial family (Polynomial_9th, :3557-3609) at the Lobatto
        // abscissae x = -1, 0, -1/2 - sqrt(5)/10, -1/2 + sqrt(5)/10 of the segment [-1, 0]
        const T wn4 = s[0], wn3 = s[1], wn2 = s[2], wn1 = s[3], w0 = s[4];
        const T wp1 = s[5], wp2 = s[6], wp3 = s[7], wp4 = s[8];
        constexpr double r5 = 2.236067977499790;
        const T x = ig == 0 ? T(-1.0) : ig == 1 ? T(0.0) : ig == 2 ? T(-0.5 - r5 / 10.0) : T(-0.5 + r5 / 10.0);
        const T x2 = x * x, x3 = x * x * x, x4 = x * x * x * x;
        T a3, b3, c3;
        a3 = (T(11) * w0 - T(7) * wn1 + T(2) * wn2) * T(1.0 / (6.0)); b3 = (T(2) * w0 - T(3) * wn1 + wn2); c3 = (w0 - T(2) * wn1 + wn2) * T(1.0 / (2.0));
        p[0] = w0 + df[0] * (a3 + b3 * x + c3 * x * x - w0); px[0] = df[0] * (b3 + T(2.0) * c3 * x) * ih;
        a3 = (T(5) * w0 - wn1 + T(2) * wp1) * T(1.0 / (6.0)); b3 = (-w0 + wp1); c3 = (T(-2) * w0 + wn1 + wp1) * T(1.0 / (2.0));
        p[1] = w0 + df[1] * (a3 + b3 * x + c3 * x * x - w0); px[1] = df[1] * (b3 + T(2.0) * c3 * x) * ih;
        a3 = (T(2) * w0 + T(5) * wp1 - wp2) * T(1.0 / (6.0)); b3 = (-w0 + wp1); c3 = (w0 - T(2) * wp1 + wp2) * T(1.0 / (2.0));
        p[2] = w0 + df[2] * (a3 + b3 * x + c3 * x * x - w0); px[2] = df[2] * (b3 + T(2.0) * c3 * x) * ih;
        T a5, b5, c5, d5, e5;
        a5 = (T(47) * w0 - T(13) * wn1 + T(2) * wn2 + T(27) * wp1 - T(3) * wp2) * T(1.0 / (60.0));
        b5 = (T(-15) * w0 + wn1 + T(15) * wp1 - wp2) * T(1.0 / (12.0));
        c5 = (T(-8) * w0 + T(6) * wn1 - wn2 + T(2) * wp1 + wp2) * T(1.0 / (8.0));
        d5 = (T(3) * w0 - wn1 - T(3) * wp1 + wp2) * T(1.0 / (6.0));
        e5 = (T(6) * w0 - T(4) * wn1 + wn2 - T(4) * wp1 + wp2) * T(1.0 / (24.0));
        p[3] = w0 + df[3] * (a5 + b5 * x + c5 * x2 + d5 * x3 + e5 * x4 - w0);
        px[3] = df[3] * (b5 + T(2.0) * c5 * x + T(3.0) * d5 * x2 + T(4.0) * e5 * x3) * ih;
        T a7, b7, c7, d7, e7, f7, g7;
        a7 = (T(319) * w0 - T(101) * wn1 + T(25) * wn2 - T(3) * wn3 + T(214) * wp1 - T(38) * wp2 + T(4) * wp3) * T(1.0 / (420.0));
        b7 = (T(-245) * w0 + T(25) * wn1 - T(2) * wn2 + T(245) * wp1 - T(25) * wp2 + T(2) * wp3) * T(1.0 / (180.0));
        c7 = (T(-230) * w0 + T(210) * wn1 - T(57) * wn2 + T(7) * wn3 + T(15) * wp1 + T(63) * wp2 - T(8) * wp3) * T(1.0 / (240.0));
        d7 = (T(28) * w0 - T(11) * wn1 + wn2 - T(28) * wp1 + T(11) * wp2 - wp3) * T(1.0 / (36.0));
        e7 = (T(46) * w0 - T(39) * wn1 + T(15) * wn2 - T(2) * wn3 - T(24) * wp1 + T(3) * wp2 + wp3) * T(1.0 / (144.0));
        f7 = (T(-10) * w0 + T(5) * wn1 - wn2 + T(10) * wp1 - T(5) * wp2 + wp3) * T(1.0 / (120.0));
        g7 = (T(-20) * w0 + T(15) * wn1 - T(6) * wn2 + wn3 + T(15) * wp1 - T(6) * wp2 + wp3) * T(1.0 / (720.0));
        const T x5 = x * x * x * x * x, x6 = x * x * x * x * x * x;
        p[4] = w0 + df[4] * (a7 + b7 * x + c7 * x2 + d7 * x3 + e7 * x4 + f7 * x5 + g7 * x6 - w0);
        px[4] = df[4] * (b7 + T(2.0) * c7 * x + T(3.0) * d7 * x2 + T(4.0) * e7 * x3 + T(5.0) * f7 * x4 + T(6.0) * g7 * x5) * ih;
        T a9, b9, c9, d9, e9, f9, g9, h9, i9;
        a9 = (T(1879) * w0 - T(641) * wn1 + T(199) * wn2 - T(41) * wn3 + T(4) * wn4 + T(1375) * wp1 - T(305) * wp2 + T(55) * wp3 - T(5) * wp4) * T(1.0 / (2520.0));
        b9 = (T(-7175) * w0 + T(889) * wn1 - T(119) * wn2 + T(9) * wn3 + T(7175) * wp1 - T(889) * wp2 + T(119) * wp3 - T(9) * wp4) * T(1.0 / (5040.0));
        c9 = (T(-27895) * w0 + T(28679) * wn1 - T(9835) * wn2 + T(2081) * wn3 - T(205) * wn4 - T(2065) * wp1 + T(11459) * wp2 - T(2455) * wp3 + T(236) * wp4) * T(1.0 / (30240.0));
        d9 = (T(1365) * w0 - T(587) * wn1 + T(89) * wn2 - T(7) * wn3 - T(1365) * wp1 + T(587) * wp2 - T(89) * wp3 + T(7) * wp4) * T(1.0 / (1440.0));
        e9 = (T(1174) * w0 - T(1160) * wn1 + T(556) * wn2 - T(128) * wn3 + T(13) * wn4 - T(464) * wp1 - T(68) * wp2 + T(88) * wp3 - T(11) * wp4) * T(1.0 / (3456.0));
        f9 = (T(-75) * w0 + T(41) * wn1 - T(11) * wn2 + wn3 + T(75) * wp1 - T(41) * wp2 + T(11) * wp3 - wp4) * T(1.0 / (480.0));
        g9 = (T(-380) * w0 + T(334) * wn1 - T(170) * wn2 + T(46) * wn3 - T(5) * wn4 + T(250) * wp1 - T(86) * wp2 + T(10) * wp3 + wp4) * T(1.0 / (8640.0));
        h9 = (T(35) * w0 - T(21) * wn1 + T(7) * wn2 - wn3 - T(35) * wp1 + T(21) * wp2 - T(7) * wp3 + wp4) * T(1.0 / (5040.0));
        i9 = (T(70) * w0 - T(56) * wn1 + T(28) * wn2 - T(8) * wn3 + wn4 - T(56) * wp1 + T(28) * wp2 - T(8) * wp3 + wp4) * T(1.0 / (40320.0));
        const T x7 = x6 * x, x8 = x7 * x;
        p[5] = w0 + df[5] * (a9 + b9 * x + c9 * x2 + d9 * x3 + e9 * x4 + f9 * x5 + g9 * x6 + h9 * x7 + i9 * x8 - w0);
        px[5] = df[5] * (b9 + T(2.0) * c9 * x + T(3.0) * d9 * x2 + T(4.0) * e9 * x3 + T(5.0) * f9 * x4 + T(6.0) * g9 * x5 + T(7.0) * h9 * x6 + T(8.0) * i9 * x7) * ih;
    }
}

// ---- the full-stencil (linear-weight) reconstruction of the learned gate's linear path ----
// sum_k c(p, k) s[k] over the nonzero coefficients of row p of a table of hos_linear_coef.cuh
// (C::V: values, C::D: slopes)
template <class T, int N, class C, bool DER>
__device__ __forceinline__ T lin_dot(int p, const T* s) {
    T acc = T(0.0);
    bool first = true;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const double c = DER ? C::D(p, k) : C::V(p, k);
        if (c == 0.0) continue;
        if (first) acc = T(c) * s[k];
        else acc = T(c) * s[k] + acc;
        first = false;
    }
    return acc;
}
// value and slope of the top candidate polynomial with its DF factor at point p of the centre
// cell: w0 + df (P - w0) and df ih P' (dfi = df * ih).  The same polynomial as normal_face /
// tangent_point's last candidate, with the coefficients collected per stencil cell.
template <class T, int N, class C>
__device__ __forceinline__ T lin_value(int p, const T* s, T df) {
    return s[N / 2] + df * (lin_dot<T, N, C, false>(p, s) - s[N / 2]);
}
template <class T, int N, class C>
__device__ __forceinline__ T lin_slope(int p, const T* s, T dfi) {
    return lin_dot<T, N, C, true>(p, s) * dfi;
}

// ---- non-DF WENO5-AO (src/reconstruction.cpp:161-360, 2393-2551): the 3D scheme and the 2D
// drivers' default slots WENO5_AO_normal / WENO5_AO_tangent (is_using_df_factor = false) ----
// nonlinear weights: the reference's WENOtype (HOS_WENO_* of the C ABI)
enum { WENO_Z = 0, WENO_JS = 1, WENO_LINEAR = 2 };
template <class T>
__device__ __forceinline__ T beta5_big(T wn2, T wn1, T w0, T wp1, T wp2) {
    return T(1.0 / 5040.0) * (T(231153) * w0 * w0 + T(104963) * wn1 * wn1 + T(6908) * wn2 * wn2 -
                              T(38947) * wn2 * wp1 + T(104963) * wp1 * wp1 +
                              wn1 * (T(-51001) * wn2 + T(179098) * wp1 - T(38947) * wp2) -
                              T(3) * w0 * (T(99692) * wn1 - T(22641) * wn2 + T(99692) * wp1 - T(22641) * wp2) +
                              T(8209) * wn2 * wp2 - T(51001) * wp1 * wp2 + T(6908) * wp2 * wp2);
}
// final AO weights (linear weights d = {0.01125, 0.1275, 0.01125, 0.85} from dhi = dlo = 0.85);
// wtype: WENO_Z, WENO_JS or WENO_LINEAR (the reference's wenotype, :176-216)
template <class T>
__device__ __forceinline__ void weights5(const T* s, T eps, T* fw, int wtype = WENO_Z) {
    const T d0 = T(0.5) * T(0.15) * T(0.15), d1 = T(0.15) * T(0.85), d3 = T(0.85);
    if (wtype == WENO_LINEAR) {
        // the linear weights select the big-stencil polynomial alone
        fw[0] = T(0); fw[1] = T(0); fw[2] = T(0); fw[3] = T(1);
        return;
    }
    T b[4];
    beta3<T>(s, b);
    if constexpr (sizeof(T) == 4) {
        // the big-stencil indicator expands into terms ~1e5 w^2 that cancel; it depends on
        // differences only, so FP32 evaluates it about the centre value
        b[3] = beta5_big(s[0] - s[2], s[1] - s[2], T(0), s[3] - s[2], s[4] - s[2]);
    } else {
        b[3] = beta5_big(s[0], s[1], s[2], s[3], s[4]);
    }
    const T tau = T(1.0 / 3.0) * (fabsT(b[3] - b[0]) + fabsT(b[3] - b[1]) + fabsT(b[3] - b[2]));
    T al[4];
    const T dd[4] = {d0, d1, d0, d3};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (wtype == WENO_JS) {
            const T e = eps + b[k];
            al[k] = dd[k] / (e * e);
        } else {
            const T q = tau / (b[k] + eps);
            al[k] = dd[k] * (T(1) + q * q);
        }
    }
    const T isum = T(1) / (al[0] + al[1] + al[2] + al[3]);
    const T w3 = al[3] * isum;
    fw[3] = w3 / d3;
#pragma unroll
    for (int k = 0; k < 3; ++k) fw[k] = al[k] * isum - fw[3] * dd[k];
}
// value and slope at the left (side 0) or right (side 1) face of the centre cell, epsilon 1e-10
template <class T>
__device__ __forceinline__ void weno5_face(int side, const T* s, T ih, T& var, T& der, int wtype = WENO_Z) {
    T fw[4];
    weights5<T>(s, T(1e-10), fw, wtype);
    const T wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
    T p[4], px[4];
    if (side == 0) {
        p[0] = T(-1.0 / 6.0) * wn2 + T(5.0 / 6.0) * wn1 + T(1.0 / 3.0) * w0;
        p[1] = T(1.0 / 3.0) * wn1 + T(5.0 / 6.0) * w0 - T(1.0 / 6.0) * wp1;
        p[2] = T(11.0 / 6.0) * w0 - T(7.0 / 6.0) * wp1 + T(1.0 / 3.0) * wp2;
        p[3] = T(1.0 / 60.0) * (T(47) * w0 + T(27) * wn1 - T(3) * wn2 - T(13) * wp1 + T(2) * wp2);
        px[0] = (w0 - wn1) * ih;
        px[1] = px[0];
        px[2] = -(T(2) * w0 - T(3) * wp1 + wp2) * ih;
        px[3] = (T(15) * w0 - T(15) * wn1 + wn2 - wp1) * (T(1.0 / 12.0) * ih);
    } else {
        p[0] = T(1.0 / 3.0) * wn2 - T(7.0 / 6.0) * wn1 + T(11.0 / 6.0) * w0;
        p[1] = T(-1.0 / 6.0) * wn1 + T(5.0 / 6.0) * w0 + T(1.0 / 3.0) * wp1;
        p[2] = T(1.0 / 3.0) * w0 + T(5.0 / 6.0) * wp1 - T(1.0 / 6.0) * wp2;
        p[3] = T(1.0 / 60.0) * (T(47) * w0 - T(13) * wn1 + T(2) * wn2 + T(27) * wp1 - T(3) * wp2);
        px[0] = (T(2) * w0 - T(3) * wn1 + wn2) * ih;
        px[1] = (wp1 - w0) * ih;
        px[2] = px[1];
        px[3] = (T(-15) * w0 + wn1 + T(15) * wp1 - wp2) * (T(1.0 / 12.0) * ih);
    }
    var = fw[0] * p[0] + fw[1] * p[1] + fw[2] * p[2] + fw[3] * p[3];
    der = fw[0] * px[0] + fw[1] * px[1] + fw[2] * px[2] + fw[3] * px[3];
}
// values (and slopes when DER) at the Gauss points -h/(2 sqrt 3) (g0) and +h/(2 sqrt 3) (g1)
// of the centre cell, epsilon 1e-6 (weno_5th_ao_2gauss).  Under wenotype = linear the
// reference leaves its weights unset (:2446-2468 have no linear branch); the linear weights
// are taken here.
template <class T, bool DER>
__device__ __forceinline__ void weno5_2g(const T* s, T ih, T* g, T* gx, int wtype = WENO_Z) {
    T fw[4];
    weights5<T>(s, T(1e-6), fw, wtype);
    const T wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
    const T r3 = T(1.732050807568877294), i4r3 = T(1) / (T(4) * r3);
    // candidate polynomials at g0; g1 is their mirror image
    T p0 = w0 - r3 * w0 * T(0.25) + (T(4) * wn1 - wn2) * i4r3;
    T p1 = w0 + (wn1 - wp1) * i4r3;
    T p2 = T(1.0 / 12.0) * (T(3) * (T(4) + r3) * w0 + r3 * (T(-4) * wp1 + wp2));
    T p3 = (T(4314) * w0 + (T(4) + T(500) * r3) * wn1 - wn2 - T(70) * r3 * wn2 + T(4) * wp1 - T(500) * r3 * wp1 - wp2
            + T(70) * r3 * wp2) * T(1.0 / 4320.0);
    g[0] = fw[0] * p0 + fw[1] * p1 + fw[2] * p2 + fw[3] * p3;
    p0 = T(1.0 / 12.0) * (T(3) * (T(4) + r3) * w0 + r3 * (T(-4) * wn1 + wn2));
    p1 = w0 + (wp1 - wn1) * i4r3;
    p2 = w0 - r3 * w0 * T(0.25) + (T(4) * wp1 - wp2) * i4r3;
    p3 = (T(4314) * w0 + (T(4) - T(500) * r3) * wn1 - wn2 + T(70) * r3 * wn2 + T(4) * wp1 + T(500) * r3 * wp1 - wp2
          - T(70) * r3 * wp2) * T(1.0 / 4320.0);
    g[1] = fw[0] * p0 + fw[1] * p1 + fw[2] * p2 + fw[3] * p3;
    if (DER) {
        const T i6h = ih * T(1.0 / 6.0), i108h = ih * T(1.0 / 108.0);
        T q0 = -((r3 - T(9)) * w0 - T(2) * (r3 - T(6)) * wn1 + (r3 - T(3)) * wn2) * i6h;
        T q1 = -(T(-2) * r3 * w0 + (T(3) + r3) * wn1 + (r3 - T(3)) * wp1) * i6h;
        T q2 = -((T(9) + r3) * w0 - T(2) * (T(6) + r3) * wp1 + (T(3) + r3) * wp2) * i6h;
        T q3 = (T(48) * r3 * w0 - T(72) * wn1 - T(26) * r3 * wn1 + T(9) * wn2 + T(2) * r3 * wn2 + T(72) * wp1
                - T(26) * r3 * wp1 - T(9) * wp2 + T(2) * r3 * wp2) * i108h;
        gx[0] = fw[0] * q0 + fw[1] * q1 + fw[2] * q2 + fw[3] * q3;
        q0 = ((T(9) + r3) * w0 - T(2) * (T(6) + r3) * wn1 + (T(3) + r3) * wn2) * i6h;
        q1 = (T(-2) * r3 * w0 + (r3 - T(3)) * wn1 + (T(3) + r3) * wp1) * i6h;
        q2 = ((r3 - T(9)) * w0 - T(2) * (r3 - T(6)) * wp1 + (r3 - T(3)) * wp2) * i6h;
        q3 = -(T(48) * r3 * w0 + T(72) * wn1 - T(26) * r3 * wn1 - T(9) * wn2 + T(2) * r3 * wn2 - T(72) * wp1
               - T(26) * r3 * wp1 + T(9) * wp2 + T(2) * r3 * wp2) * i108h;
        gx[1] = fw[0] * q0 + fw[1] * q1 + fw[2] * q2 + fw[3] * q3;
    }
}

}  // namespace hos
