// oracle_weno.h -- scalar WENO-AO-DF kernels shared by the 1D and 2D oracle restatements.
// TEST INFRASTRUCTURE ONLY (see oracle_api.h).  Restates src/reconstruction.cpp of the
// reference (normal face values :480-657, :750-974, :1072-1364; Gauss-point values
// :2751-2836, :3021-3174, :3389-3609) with the same operand order.
#pragma once
#include <cmath>

namespace oracle_weno {

// ----------------------------------------------------------------------------------------
// WENO-AO-DF weights.  The linear weights d, smoothness indicators and the Z-type
// nonlinear weights are the published WENO-AO(5,3)/(7,5,3)/(9,7,5,3) construction as the
// reference writes it (e.g. src/reconstruction.cpp:489-521, 763-830, 1087-1187).
// s[] holds the stencil with s[r] the centre cell, r = 2, 3, 4.
// ----------------------------------------------------------------------------------------
inline double sq(double x) { return x * x; }

inline void beta3(const double* s, int r, double* b) {
    const double wn2 = s[r - 2], wn1 = s[r - 1], w0 = s[r], wp1 = s[r + 1], wp2 = s[r + 2];
    b[0] = 13.0 / 12.0 * sq(wn2 - 2.0 * wn1 + w0) + 0.25 * sq(wn2 - 4.0 * wn1 + 3.0 * w0);
    b[1] = 13.0 / 12.0 * sq(wn1 - 2.0 * w0 + wp1) + 0.25 * sq(wn1 - wp1);
    b[2] = 13.0 / 12.0 * sq(w0 - 2.0 * wp1 + wp2) + 0.25 * sq(3.0 * w0 - 4.0 * wp1 + wp2);
}
// 7th-order indicator built from four cubic sub-stencils (:778-806); 13/3 and 781/20 are
// integer divisions in the reference (4 and 39) and are kept as such.
inline double beta7(const double* s, int r) {
    const double wn3 = s[r - 3], wn2 = s[r - 2], wn1 = s[r - 1], w0 = s[r];
    const double wp1 = s[r + 1], wp2 = s[r + 2], wp3 = s[r + 3];
    double a1, a2, a3, b4[4];
    a1 = (-19 * wn3 + 87 * wn2 - 177 * wn1 + 109 * w0) / 60.0;
    a2 = (-wn3 + 4 * wn2 - 5 * wn1 + 2 * w0) / 2;
    a3 = (-wn3 + 3 * wn2 - 3 * wn1 + w0) / 6.0;
    b4[0] = (a1 + a3 / 10.0) * (a1 + a3 / 10.0) + 13 / 3 * a2 * a2 + 781 / 20 * a3 * a3;
    a1 = (11 * wn2 - 63 * wn1 + 33 * w0 + 19 * wp1) / 60.0;
    a2 = (wn1 - 2 * w0 + wp1) / 2;
    a3 = (-wn2 + 3 * wn1 - 3 * w0 + wp1) / 6.0;
    b4[1] = (a1 + a3 / 10.0) * (a1 + a3 / 10.0) + 13 / 3 * a2 * a2 + 781 / 20 * a3 * a3;
    a1 = (-19 * wn1 - 33 * w0 + 63 * wp1 - 11 * wp2) / 60.0;
    a2 = (wn1 - 2 * w0 + wp1) / 2;
    a3 = (-wn1 + 3 * w0 - 3 * wp1 + wp2) / 6.0;
    b4[2] = (a1 + a3 / 10.0) * (a1 + a3 / 10.0) + 13 / 3 * a2 * a2 + 781 / 20 * a3 * a3;
    a1 = (-109 * w0 + 177 * wp1 - 87 * wp2 + 19 * wp3) / 60.0;
    a2 = (2 * w0 - 5 * wp1 + 4 * wp2 - wp3) / 2;
    a3 = (-w0 + 3 * wp1 - 3 * wp2 + wp3) / 6.0;
    b4[3] = (a1 + a3 / 10.0) * (a1 + a3 / 10.0) + 13 / 3 * a2 * a2 + 781 / 20 * a3 * a3;
    return 1.0 / 20.0 * (b4[0] + 9.0 * b4[1] + 9.0 * b4[2] + b4[3]) + std::abs(b4[0] - b4[1] - b4[2] + b4[3]);
}
// 9th-order indicator from five quartic sub-stencils (:1130-1169); returns beta5[2] (the
// 5th-order indicator of this family) through b5mid.
inline double beta9(const double* s, double* b5mid) {
    const double wn4 = s[0], wn3 = s[1], wn2 = s[2], wn1 = s[3], w0 = s[4];
    const double wp1 = s[5], wp2 = s[6], wp3 = s[7], wp4 = s[8];
    double a1, a2, a3, a4, b5[5];
    auto comb = [&]() {
        return (a1 + a3 / 10.0) * (a1 + a3 / 10.0) + 13.0 / 3.0 * (a2 + 123.0 / 455.0 * a4) * (a2 + 123.0 / 455.0 * a4)
               + 781.0 / 20.0 * a3 * a3 + 1421461.0 / 2275.0 * a4 * a4;
    };
    a1 = (-462 * wn1 + 336 * wn2 - 146 * wn3 + 27 * wn4 + 245 * w0) / 120.0;
    a2 = (-240 * wn1 + 262 * wn2 - 128 * wn3 + 25 * wn4 + 81 * w0) / 56.0;
    a3 = (-18 * wn1 + 24 * wn2 - 14 * wn3 + 3 * wn4 + 5 * w0) / 12.0;
    a4 = (-4 * wn1 + 6 * wn2 - 4 * wn3 + wn4 + w0) / 24.0;
    b5[0] = comb();
    a1 = (-192 * wn1 + 66 * wn2 - 11 * wn3 + 110 * w0 + 27 * wp1) / 120;
    a2 = (10 * wn1 + 12 * wn2 - 3 * wn3 - 44 * w0 + 25 * wp1) / 56;
    a3 = (12 * wn1 - 6 * wn2 + wn3 - 10 * w0 + 3 * wp1) / 12;
    a4 = (6 * wn1 - 4 * wn2 + wn3 - 4 * w0 + wp1) / 24;
    b5[1] = comb();
    a1 = (-82 * wn1 + 11 * wn2 + 82 * wp1 - 11 * wp2) / 120;
    a2 = (40 * wn1 - 3 * wn2 - 74 * w0 + 40 * wp1 - 3 * wp2) / 56;
    a3 = (2 * wn1 - wn2 - 2 * wp1 + wp2) / 12;
    a4 = (-4 * wn1 + wn2 + 6 * w0 - 4 * wp1 + wp2) / 24;
    b5[2] = comb();
    a1 = (-27 * wn1 - 110 * w0 + 192 * wp1 - 66 * wp2 + 11 * wp3) / 120;
    a2 = (25 * wn1 - 44 * w0 + 10 * wp1 + 12 * wp2 - 3 * wp3) / 56;
    a3 = (-3 * wn1 + 10 * w0 - 12 * wp1 + 6 * wp2 - wp3) / 12;
    a4 = (wn1 - 4 * w0 + 6 * wp1 - 4 * wp2 + wp3) / 24;
    b5[3] = comb();
    a1 = (-245 * w0 + 462 * wp1 - 336 * wp2 + 146 * wp3 - 27 * wp4) / 120;
    a2 = (81 * w0 - 240 * wp1 + 262 * wp2 - 128 * wp3 + 25 * wp4) / 56;
    a3 = (-5 * w0 + 18 * wp1 - 24 * wp2 + 14 * wp3 - 3 * wp4) / 12;
    a4 = (w0 - 4 * wp1 + 6 * wp2 - 4 * wp3 + wp4) / 24;
    b5[4] = comb();
    *b5mid = b5[2];
    return 1.0 / 70.0 * (b5[0] + 16.0 * b5[1] + 36.0 * b5[2] + 16.0 * b5[3] + b5[4]) + std::abs(b5[0] - b5[1] - b5[3] + b5[4]);
}

// Final AO weights fw[0..n-1] for order 5/7/9 (n = 4/5/6) on stencil s (DF variants,
// epsilon 1e-6).  Returns n.
inline int ao_weights(int order, const double* s, double* fw) {
    const double dhi = 0.85, dlo = 0.85, davg = 0.85, davg1 = 0.85, davg2 = 0.85;
    const double eps = 1e-6;
    double beta[6], d[6];
    int n;
    if (order == 5) {
        n = 4;
        d[0] = (1.0 - dhi) * (1.0 - dlo) / 2.0;
        d[1] = (1.0 - dhi) * dlo;
        d[2] = (1.0 - dhi) * (1.0 - dlo) / 2.0;
        d[3] = dhi;
        beta3(s, 2, beta);
        beta[3] = 1.0 / 6.0 * (beta[0] + 4.0 * beta[1] + beta[2]) + std::abs(beta[0] - beta[2]);
    } else if (order == 7) {
        n = 5;
        d[0] = (1.0 - dhi) * (1.0 - dlo) * (1.0 - davg) / 2.0;
        d[1] = (1.0 - dhi) * (1.0 - davg) * dlo;
        d[2] = (1.0 - dhi) * (1.0 - dlo) * (1.0 - davg) / 2.0;
        d[3] = (1.0 - dhi) * davg;
        d[4] = dhi;
        beta3(s, 3, beta);
        beta[3] = 1.0 / 6.0 * (beta[0] + 4.0 * beta[1] + beta[2]) + std::abs(beta[0] - beta[2]);
        beta[4] = beta7(s, 3);
    } else {
        n = 6;
        d[0] = (1.0 - dhi) * (1.0 - dlo) * (1.0 - davg1) * (1.0 - davg2) / 2.0;
        d[1] = (1.0 - dhi) * (1.0 - davg1) * (1.0 - davg2) * dlo;
        d[2] = (1.0 - dhi) * (1.0 - dlo) * (1.0 - davg1) * (1.0 - davg2) / 2.0;
        d[3] = (1.0 - dhi) * (1.0 - davg2) * davg1;
        d[4] = (1.0 - dhi) * davg2;
        d[5] = dhi;
        beta3(s, 4, beta);
        beta[4] = beta7(s, 4);
        double b5mid;
        beta[5] = beta9(s, &b5mid);
        beta[3] = b5mid;
    }
    const int top = n - 1;
    double tau;
    if (n == 4)
        tau = 1.0 / 3.0 * (std::abs(beta[3] - beta[0]) + std::abs(beta[3] - beta[1]) + std::abs(beta[3] - beta[2]));
    else if (n == 5)
        tau = 0.25 * (std::abs(beta[4] - beta[0]) + std::abs(beta[4] - beta[1]) + std::abs(beta[4] - beta[2]) + std::abs(beta[4] - beta[3]));
    else
        tau = 0.2 * (std::abs(beta[5] - beta[0]) + std::abs(beta[5] - beta[1]) + std::abs(beta[5] - beta[2]) + std::abs(beta[5] - beta[3]) + std::abs(beta[5] - beta[4]));
    double alpha[6], ww[6], sum = 0.0;
    for (int k = 0; k < n; ++k) {
        double gd = tau / (beta[k] + eps);
        alpha[k] = d[k] * (1.0 + gd * gd);
        sum += alpha[k];
    }
    for (int k = 0; k < n; ++k) ww[k] = alpha[k] / sum;
    fw[top] = ww[top] / d[top];
    for (int k = 0; k < top; ++k) fw[k] = ww[k] - ww[top] / d[top] * d[k];
    return n;
}

// DF factors from the alpha values along the stencil (e.g. :1731-1741, :1898-1909, :2074-2087)
inline int df_factors(int order, const double* a, double* df) {
    double s[6];
    int n;
    if (order == 5) {
        n = 4;
        s[0] = a[0] + a[2]; s[1] = a[1] + a[3]; s[2] = a[2] + a[4]; s[3] = a[0] + a[2] + a[4];
    } else if (order == 7) {
        n = 5;
        s[0] = a[1] + a[3]; s[1] = a[2] + a[4]; s[2] = a[3] + a[5]; s[3] = a[1] + a[3] + a[5];
        s[4] = a[0] + a[2] + a[4] + a[6];
    } else {
        n = 6;
        s[0] = a[2] + a[4]; s[1] = a[3] + a[5]; s[2] = a[4] + a[6]; s[3] = a[2] + a[4] + a[6];
        s[4] = a[1] + a[3] + a[5] + a[7]; s[5] = a[0] + a[2] + a[4] + a[6] + a[8];
    }
    for (int k = 0; k < n; ++k) df[k] = s[k] < 2.0 ? 1.0 : 2.0 / s[k];
    return n;
}

// ----------------------------------------------------------------------------------------
// normal (cell-face) candidate polynomials: value and first derivative at the left face
// (x = -1/2 cell) or right face of the centre cell, scaled by the DF factor.
// Left face: :526-536 / :835-847 / :1196-1210; right face: :612-622 / :936-948 / :1341-1355.
// ----------------------------------------------------------------------------------------
inline void normal_face(int order, int side, const double* s, const double* df, double h, double* p, double* px) {
    const int r = order / 2;
    const double w0 = s[r];
    const double wn1 = s[r - 1], wn2 = s[r - 2], wp1 = s[r + 1], wp2 = s[r + 2];
    const double wn3 = r >= 3 ? s[r - 3] : 0, wp3 = r >= 3 ? s[r + 3] : 0;
    const double wn4 = r >= 4 ? s[r - 4] : 0, wp4 = r >= 4 ? s[r + 4] : 0;
    if (side == 0) {
        p[0] = w0 + df[0] * (-1.0 / 6.0 * wn2 + 5.0 / 6.0 * wn1 + 1.0 / 3.0 * w0 - w0);
        p[1] = w0 + df[1] * (1.0 / 3.0 * wn1 + 5.0 / 6.0 * w0 - 1.0 / 6.0 * wp1 - w0);
        p[2] = w0 + df[2] * (11.0 / 6.0 * w0 - 7.0 / 6.0 * wp1 + 1.0 / 3.0 * wp2 - w0);
        p[3] = w0 + df[3] * ((1.0 / 60.0) * (47.0 * w0 + 27.0 * wn1 - 3.0 * wn2 - 13.0 * wp1 + 2.0 * wp2) - w0);
        px[0] = df[0] * (w0 - wn1) / h;
        px[1] = df[1] * (w0 - wn1) / h;
        px[2] = -df[2] * ((2.0 * w0 - 3.0 * wp1 + wp2) / h);
        px[3] = df[3] * (15.0 * w0 - 15.0 * wn1 + wn2 - wp1) / (12.0 * h);
        if (order >= 7) {
            p[4] = w0 + df[4] * ((order == 7 ? 1.0 / 420.0 : (1.0 / 420.0)) * (319.0 * w0 + 214.0 * wn1 - 38.0 * wn2 + 4.0 * wn3 - 101.0 * wp1 + 25.0 * wp2 - 3.0 * wp3) - w0);
            px[4] = df[4] * (245.0 * w0 - 245.0 * wn1 + 25.0 * wn2 - 2.0 * wn3 - 25.0 * wp1 + 2.0 * wp2) / (180.0 * h);
        }
        if (order == 9) {
            p[5] = w0 + df[5] * ((1.0 / 2520.0) * (1879.0 * w0 + 1375.0 * wn1 - 305.0 * wn2 + 55.0 * wn3 - 5.0 * wn4 - 641.0 * wp1 + 199.0 * wp2 - 41.0 * wp3 + 4.0 * wp4) - w0);
            px[5] = df[5] * (7175.0 * w0 - 7175.0 * wn1 + 889.0 * wn2 - 119.0 * wn3 + 9.0 * wn4 - 889.0 * wp1 + 119.0 * wp2 - 9.0 * wp3) / (5040.0 * h);
        }
    } else {
        p[0] = w0 + df[0] * (1.0 / 3.0 * wn2 - 7.0 / 6.0 * wn1 + 11.0 / 6.0 * w0 - w0);
        p[1] = w0 + df[1] * (-1.0 / 6.0 * wn1 + 5.0 / 6.0 * w0 + 1.0 / 3.0 * wp1 - w0);
        p[2] = w0 + df[2] * (1.0 / 3.0 * w0 + 5.0 / 6.0 * wp1 - 1.0 / 6.0 * wp2 - w0);
        p[3] = w0 + df[3] * ((1.0 / 60.0) * (47.0 * w0 - 13.0 * wn1 + 2.0 * wn2 + 27.0 * wp1 - 3.0 * wp2) - w0);
        px[0] = df[0] * (2.0 * w0 - 3.0 * wn1 + wn2) / h;
        px[1] = df[1] * (-w0 + wp1) / h;
        px[2] = df[2] * (-w0 + wp1) / h;
        px[3] = df[3] * (-15.0 * w0 + wn1 + 15.0 * wp1 - wp2) / (12.0 * h);
        if (order >= 7) {
            p[4] = w0 + df[4] * (1.0 / 420.0 * (319.0 * w0 - 101.0 * wn1 + 25.0 * wn2 - 3.0 * wn3 + 214.0 * wp1 - 38.0 * wp2 + 4.0 * wp3) - w0);
            px[4] = df[4] * (-245.0 * w0 + 25.0 * wn1 - 2.0 * wn2 + 245.0 * wp1 - 25.0 * wp2 + 2.0 * wp3) / (180.0 * h);
        }
        if (order == 9) {
            p[5] = w0 + df[5] * ((1.0 / 2520) * (1879.0 * w0 - 641.0 * wn1 + 199.0 * wn2 - 41.0 * wn3 + 4.0 * wn4 + 1375.0 * wp1 - 305.0 * wp2 + 55.0 * wp3 - 5.0 * wp4) - w0);
            px[5] = df[5] * (-7175.0 * w0 + 889.0 * wn1 - 119.0 * wn2 + 9.0 * wn3 + 7175.0 * wp1 - 889.0 * wp2 + 119.0 * wp3 - 9.0 * wp4) / (5040.0 * h);
        }
    }
}

// scalar normal reconstruction: value and slope at one face of the centre cell
inline void weno_normal(int order, int side, const double* s, const double* df, double h, double& var, double& der) {
    double fw[6], p[6], px[6];
    int n = ao_weights(order, s, fw);
    normal_face(order, side, s, df, h, p, px);
    var = 0.0;
    der = 0.0;
    for (int k = 0; k < n; ++k) {
        var += fw[k] * p[k];
        der += fw[k] * px[k];
    }
}

// ----------------------------------------------------------------------------------------
// tangential candidate polynomials at the Gauss points of a face
//   WENO5, 2 Gauss-Legendre points (:2793-2836), WENO7, 3 Gauss-Legendre points (:3093-3173),
//   WENO9, 4 Gauss-Lobatto points via the 9th-order polynomial family (:3489-3609)
// ----------------------------------------------------------------------------------------
inline void tangent_points(int order, int ig, const double* s, const double* df, double h, double* p, double* px) {
    if (order == 5) {
        const double wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
        const double sqrt3 = 1.732050807568877294;
        if (ig == 0) {
            p[0] = w0 + df[0] * (w0 - (sqrt3 * w0) / 4 + (4 * wn1 - wn2) / (4 * sqrt3) - w0);
            p[1] = w0 + df[1] * (w0 + (wn1 - wp1) / (4 * sqrt3) - w0);
            p[2] = w0 + df[2] * ((1.0 / 12.0) * (3 * (4 + sqrt3) * w0 + sqrt3 * (-4 * wp1 + wp2)) - w0);
            p[3] = w0 + df[3] * ((4314 * w0 + (4 + 500 * sqrt3) * wn1 - wn2 - 70 * sqrt3 * wn2 + 4 * wp1 - 500 * sqrt3 * wp1 - wp2 + 70 * sqrt3 * wp2) / 4320 - w0);
            px[0] = -df[0] * ((-9 + sqrt3) * w0 - 2 * (-6 + sqrt3) * wn1 + (-3 + sqrt3) * wn2) / (6 * h);
            px[1] = -df[1] * (-2 * sqrt3 * w0 + (3 + sqrt3) * wn1 + (-3 + sqrt3) * wp1) / (6 * h);
            px[2] = -df[2] * ((9 + sqrt3) * w0 - 2 * (6 + sqrt3) * wp1 + (3 + sqrt3) * wp2) / (6 * h);
            px[3] = df[3] * (48 * sqrt3 * w0 - 72 * wn1 - 26 * sqrt3 * wn1 + 9 * wn2 + 2 * sqrt3 * wn2 + 72 * wp1 - 26 * sqrt3 * wp1 - 9 * wp2 + 2 * sqrt3 * wp2) / (108 * h);
        } else {
            p[0] = w0 + df[0] * ((1.0 / 12.0) * (3 * (4 + sqrt3) * w0 + sqrt3 * (-4 * wn1 + wn2)) - w0);
            p[1] = w0 + df[1] * (w0 + (-wn1 + wp1) / (4 * sqrt3) - w0);
            p[2] = w0 + df[2] * (w0 - (sqrt3 * w0) / 4 + (4 * wp1 - wp2) / (4 * sqrt3) - w0);
            p[3] = w0 + df[3] * ((4314 * w0 + (4 - 500 * sqrt3) * wn1 - wn2 + 70 * sqrt3 * wn2 + 4 * wp1 + 500 * sqrt3 * wp1 - wp2 - 70 * sqrt3 * wp2) / 4320 - w0);
            px[0] = df[0] * ((9 + sqrt3) * w0 - 2 * (6 + sqrt3) * wn1 + (3 + sqrt3) * wn2) / (6 * h);
            px[1] = df[1] * (-2 * sqrt3 * w0 + (-3 + sqrt3) * wn1 + (3 + sqrt3) * wp1) / (6 * h);
            px[2] = df[2] * ((-9 + sqrt3) * w0 - 2 * (-6 + sqrt3) * wp1 + (-3 + sqrt3) * wp2) / (6 * h);
            px[3] = -df[3] * ((48 * sqrt3 * w0 + 72 * wn1 - 26 * sqrt3 * wn1 - 9 * wn2 + 2 * sqrt3 * wn2 - 72 * wp1 - 26 * sqrt3 * wp1 + 9 * wp2 + 2 * sqrt3 * wp2) / (108 * h));
        }
        return;
    }
    if (order == 7) {
        const double wn3 = s[0], wn2 = s[1], wn1 = s[2], w0 = s[3], wp1 = s[4], wp2 = s[5], wp3 = s[6];
        const double sqrt15 = 3.872983346207417;
        if (ig == 0) {
            p[0] = w0 + df[0] * ((23.0 * w0 + 2.0 * wn1 - wn2) / 24.0 - w0);
            p[1] = w0 + df[1] * ((26.0 * w0 - wn1 - wp1) / 24.0 - w0);
            p[2] = w0 + df[2] * ((23.0 * w0 + 2.0 * wp1 - wp2) / 24.0 - w0);
            p[3] = w0 + df[3] * ((2134.0 * w0 - 116.0 * wn1 + 9.0 * wn2 - 116.0 * wp1 + 9.0 * wp2) / 1920.0 - w0);
            p[4] = w0 + df[4] * ((121004 * w0 - 7621 * wn1 + 954 * wn2 - 75 * wn3 - 7621 * wp1 + 954 * wp2 - 75 * wp3) / 107520.0 - w0);
            px[0] = df[0] * (3.0 * w0 - 4.0 * wn1 + wn2) / (2.0 * h);
            px[1] = df[1] * (-wn1 + wp1) / (2.0 * h);
            px[2] = df[2] * (-3.0 * w0 + 4.0 * wp1 - wp2) / (2.0 * h);
            px[3] = df[3] * (-34.0 * wn1 + 5.0 * wn2 + 34.0 * wp1 - 5.0 * wp2) / (48.0 * h);
            px[4] = df[4] * (-9455 * wn1 + 2236 * wn2 - 259 * wn3 + 9455 * wp1 - 2236 * wp2 + 259 * wp3) / (11520.0 * h);
        } else if (ig == 1) {
            p[0] = w0 + df[0] * (((62 - 9 * sqrt15) * w0 + 4 * (-1 + 3 * sqrt15) * wn1 + (2 - 3 * sqrt15) * wn2) / 60.0 - w0);
            p[1] = w0 + df[1] * ((56 * w0 + (2 + 3 * sqrt15) * wn1 + (2 - 3 * sqrt15) * wp1) / 60.0 - w0);
            p[2] = w0 + df[2] * (((62 + 9 * sqrt15) * w0 - 4 * (1 + 3 * sqrt15) * wp1 + (2 + 3 * sqrt15) * wp2) / 60.0 - w0);
            p[3] = w0 + df[3] * ((2186 * w0 + 4 * (29 + 41 * sqrt15) * wn1 - 9 * wn2 - 22 * sqrt15 * wn2 + 116 * wp1 - 164 * sqrt15 * wp1 - 9 * wp2 + 22 * sqrt15 * wp2) / 2400.0 - w0);
            p[4] = w0 + df[4] * ((4534440 * w0 + 5 * (57144 + 78421 * sqrt15) * wn1 - 35748 * wn2 - 84364 * sqrt15 * wn2 + 2808 * wn3 + 9541 * sqrt15 * wn3 + 285720 * wp1 -
                                  392105 * sqrt15 * wp1 - 35748 * wp2 + 84364 * sqrt15 * wp2 + 2808 * wp3 - 9541 * sqrt15 * wp3) / 5040000.0 - w0);
            px[0] = df[0] * (-((-15 + sqrt15) * w0) + 2 * (-10 + sqrt15) * wn1 - (-5 + sqrt15) * wn2) / (10.0 * h);
            px[1] = df[1] * (2 * sqrt15 * w0 - (5 + sqrt15) * wn1 - (-5 + sqrt15) * wp1) / (h * 10.0);
            px[2] = df[2] * (-((15 + sqrt15) * w0) + 2 * (10 + sqrt15) * wp1 - (5 + sqrt15) * wp2) / (10.0 * h);
            px[3] = df[3] * (78 * sqrt15 * w0 - 2 * (95 + 21 * sqrt15) * wn1 + 20 * wn2 + 3 * sqrt15 * wn2 + 190 * wp1 - 42 * sqrt15 * wp1 - 20 * wp2 + 3 * sqrt15 * wp2) / (300.0 * h);
            px[4] = df[4] * (103860 * sqrt15 * w0 - 5 * (49925 + 11619 * sqrt15) * wn1 + 41300 * wn2 + 6678 * sqrt15 * wn2 - 4325 * wn3 - 513 * sqrt15 * wn3 + 249625 * wp1 -
                             58095 * sqrt15 * wp1 - 41300 * wp2 + 6678 * sqrt15 * wp2 + 4325 * wp3 - 513 * sqrt15 * wp3) / (360000.0 * h);
        } else {
            p[0] = w0 + df[0] * (((62 + 9 * sqrt15) * w0 - 4 * (1 + 3 * sqrt15) * wn1 + (2 + 3 * sqrt15) * wn2) / 60.0 - w0);
            p[1] = w0 + df[1] * ((56 * w0 + (2 - 3 * sqrt15) * wn1 + (2 + 3 * sqrt15) * wp1) / 60.0 - w0);
            p[2] = w0 + df[2] * (((62 - 9 * sqrt15) * w0 + 4 * (-1 + 3 * sqrt15) * wp1 + (2 - 3 * sqrt15) * wp2) / 60.0 - w0);
            p[3] = w0 + df[3] * ((2186 * w0 - 4 * (-29 + 41 * sqrt15) * wn1 - 9 * wn2 + 22 * sqrt15 * wn2 + 116 * wp1 + 164 * sqrt15 * wp1 - 9 * wp2 - 22 * sqrt15 * wp2) / 2400.0 - w0);
            p[4] = w0 + df[4] * ((4534440 * w0 - 5 * (-57144 + 78421 * sqrt15) * wn1 - 35748 * wn2 + 84364 * sqrt15 * wn2 + 2808 * wn3 - 9541 * sqrt15 * wn3 + 285720 * wp1 +
                                  392105 * sqrt15 * wp1 - 35748 * wp2 - 84364 * sqrt15 * wp2 + 2808 * wp3 + 9541 * sqrt15 * wp3) / 5040000.0 - w0);
            px[0] = df[0] * ((15 + sqrt15) * w0 - 2 * (10 + sqrt15) * wn1 + (5 + sqrt15) * wn2) / (10.0 * h);
            px[1] = df[1] * (-2 * sqrt15 * w0 - (5 - sqrt15) * wn1 + (5 + sqrt15) * wp1) / (h * 10.0);
            px[2] = df[2] * ((-15 + sqrt15) * w0 - 2 * (-10 + sqrt15) * wp1 + (-5 + sqrt15) * wp2) / (10.0 * h);
            px[3] = df[3] * (-78 * sqrt15 * w0 + 2 * (-95 + 21 * sqrt15) * wn1 + 20 * wn2 - 3 * sqrt15 * wn2 + 190 * wp1 + 42 * sqrt15 * wp1 - 20 * wp2 - 3 * sqrt15 * wp2) / (300.0 * h);
            px[4] = df[4] * (-103860 * sqrt15 * w0 + 5 * (-49925 + 11619 * sqrt15) * wn1 + 41300 * wn2 - 6678 * sqrt15 * wn2 - 4325 * wn3 + 513 * sqrt15 * wn3 + 249625 * wp1 +
                             58095 * sqrt15 * wp1 - 41300 * wp2 - 6678 * sqrt15 * wp2 + 4325 * wp3 + 513 * sqrt15 * wp3) / (360000.0 * h);
        }
        return;
    }
    // order 9: the polynomial family evaluated at the Lobatto abscissae
    // x = -1, 0, -1/2 - sqrt5/10, -1/2 + sqrt5/10 of the face segment [-1, 0] (:3494-3543)
    const double wn4 = s[0], wn3 = s[1], wn2 = s[2], wn1 = s[3], w0 = s[4];
    const double wp1 = s[5], wp2 = s[6], wp3 = s[7], wp4 = s[8];
    const double sqrt5 = 2.236067977499790;
    double x = ig == 0 ? -1.0 : ig == 1 ? 0.0 : ig == 2 ? -0.5 - sqrt5 / 10.0 : -0.5 + sqrt5 / 10.0;
    double a3, b3, c3;
    a3 = (11 * w0 - 7 * wn1 + 2 * wn2) / 6.0; b3 = (2 * w0 - 3 * wn1 + wn2); c3 = (w0 - 2 * wn1 + wn2) / 2.0;
    p[0] = w0 + df[0] * (a3 + b3 * x + c3 * x * x - w0); px[0] = df[0] * (b3 + 2.0 * c3 * x) / h;
    a3 = (5 * w0 - wn1 + 2 * wp1) / 6.0; b3 = (-w0 + wp1); c3 = (-2 * w0 + wn1 + wp1) / 2.0;
    p[1] = w0 + df[1] * (a3 + b3 * x + c3 * x * x - w0); px[1] = df[1] * (b3 + 2.0 * c3 * x) / h;
    a3 = (2 * w0 + 5 * wp1 - wp2) / 6.0; b3 = (-w0 + wp1); c3 = (w0 - 2 * wp1 + wp2) / 2.0;
    p[2] = w0 + df[2] * (a3 + b3 * x + c3 * x * x - w0); px[2] = df[2] * (b3 + 2.0 * c3 * x) / h;
    double a5, b5, c5, d5, e5;
    a5 = (47 * w0 - 13 * wn1 + 2 * wn2 + 27 * wp1 - 3 * wp2) / 60.0;
    b5 = (-15 * w0 + wn1 + 15 * wp1 - wp2) / 12.0;
    c5 = (-8 * w0 + 6 * wn1 - wn2 + 2 * wp1 + wp2) / 8.0;
    d5 = (3 * w0 - wn1 - 3 * wp1 + wp2) / 6.0;
    e5 = (6 * w0 - 4 * wn1 + wn2 - 4 * wp1 + wp2) / 24.0;
    p[3] = w0 + df[3] * (a5 + b5 * x + c5 * x * x + d5 * x * x * x + e5 * x * x * x * x - w0);
    px[3] = df[3] * (b5 + 2.0 * c5 * x + 3.0 * d5 * x * x + 4.0 * e5 * x * x * x) / h;
    double a7, b7, c7, d7, e7, f7, g7;
    a7 = (319 * w0 - 101 * wn1 + 25 * wn2 - 3 * wn3 + 214 * wp1 - 38 * wp2 + 4 * wp3) / 420.0;
    b7 = (-245 * w0 + 25 * wn1 - 2 * wn2 + 245 * wp1 - 25 * wp2 + 2 * wp3) / 180.0;
    c7 = (-230 * w0 + 210 * wn1 - 57 * wn2 + 7 * wn3 + 15 * wp1 + 63 * wp2 - 8 * wp3) / 240.0;
    d7 = (28 * w0 - 11 * wn1 + wn2 - 28 * wp1 + 11 * wp2 - wp3) / 36.0;
    e7 = (46 * w0 - 39 * wn1 + 15 * wn2 - 2 * wn3 - 24 * wp1 + 3 * wp2 + wp3) / 144.0;
    f7 = (-10 * w0 + 5 * wn1 - wn2 + 10 * wp1 - 5 * wp2 + wp3) / 120.0;
    g7 = (-20 * w0 + 15 * wn1 - 6 * wn2 + wn3 + 15 * wp1 - 6 * wp2 + wp3) / 720.0;
    p[4] = w0 + df[4] * (a7 + b7 * x + c7 * x * x + d7 * x * x * x + e7 * x * x * x * x + f7 * x * x * x * x * x + g7 * x * x * x * x * x * x - w0);
    px[4] = df[4] * (b7 + 2.0 * c7 * x + 3.0 * d7 * x * x + 4.0 * e7 * x * x * x + 5.0 * f7 * x * x * x * x + 6.0 * g7 * x * x * x * x * x) / h;
    double a9, b9, c9, d9, e9, f9, g9, h9, i9;
    a9 = (1879 * w0 - 641 * wn1 + 199 * wn2 - 41 * wn3 + 4 * wn4 + 1375 * wp1 - 305 * wp2 + 55 * wp3 - 5 * wp4) / 2520.0;
    b9 = (-7175 * w0 + 889 * wn1 - 119 * wn2 + 9 * wn3 + 7175 * wp1 - 889 * wp2 + 119 * wp3 - 9 * wp4) / 5040.0;
    c9 = (-27895 * w0 + 28679 * wn1 - 9835 * wn2 + 2081 * wn3 - 205 * wn4 - 2065 * wp1 + 11459 * wp2 - 2455 * wp3 + 236 * wp4) / 30240.0;
    d9 = (1365 * w0 - 587 * wn1 + 89 * wn2 - 7 * wn3 - 1365 * wp1 + 587 * wp2 - 89 * wp3 + 7 * wp4) / 1440.0;
    e9 = (1174 * w0 - 1160 * wn1 + 556 * wn2 - 128 * wn3 + 13 * wn4 - 464 * wp1 - 68 * wp2 + 88 * wp3 - 11 * wp4) / 3456.0;
    f9 = (-75 * w0 + 41 * wn1 - 11 * wn2 + wn3 + 75 * wp1 - 41 * wp2 + 11 * wp3 - wp4) / 480.0;
    g9 = (-380 * w0 + 334 * wn1 - 170 * wn2 + 46 * wn3 - 5 * wn4 + 250 * wp1 - 86 * wp2 + 10 * wp3 + wp4) / 8640.0;
    h9 = (35 * w0 - 21 * wn1 + 7 * wn2 - wn3 - 35 * wp1 + 21 * wp2 - 7 * wp3 + wp4) / 5040.0;
    i9 = (70 * w0 - 56 * wn1 + 28 * wn2 - 8 * wn3 + wn4 - 56 * wp1 + 28 * wp2 - 8 * wp3 + wp4) / 40320.0;
    p[5] = w0 + df[5] * (a9 + b9 * x + c9 * x * x + d9 * x * x * x + e9 * x * x * x * x + f9 * x * x * x * x * x
                         + g9 * x * x * x * x * x * x + h9 * x * x * x * x * x * x * x + i9 * x * x * x * x * x * x * x * x - w0);
    px[5] = df[5] * (b9 + 2.0 * c9 * x + 3.0 * d9 * x * x + 4.0 * e9 * x * x * x + 5.0 * f9 * x * x * x * x
                     + 6.0 * g9 * x * x * x * x * x + 7.0 * h9 * x * x * x * x * x * x + 8.0 * i9 * x * x * x * x * x * x * x) / h;
}

// ----------------------------------------------------------------------------------------
// Non-DF WENO5-AO (the 1D step-0 scheme and the 3D scheme).
// ----------------------------------------------------------------------------------------
// full 5th-order indicator of the big stencil (src/reconstruction.cpp:184-188, :2423-2427)
inline double beta5_big(double wn2, double wn1, double w0, double wp1, double wp2) {
    return (1.0 / 5040.0) * (231153.0 * w0 * w0 + 104963.0 * wn1 * wn1 + 6908.0 * wn2 * wn2 -
                             38947.0 * wn2 * wp1 + 104963.0 * wp1 * wp1 +
                             wn1 * (-51001.0 * wn2 + 179098.0 * wp1 - 38947.0 * wp2) -
                             3.0 * w0 * (99692.0 * wn1 - 22641.0 * wn2 + 99692.0 * wp1 - 22641.0 * wp2) +
                             8209.0 * wn2 * wp2 - 51001.0 * wp1 * wp2 + 6908.0 * wp2 * wp2);
}

// Nonlinear weights of the non-DF WENO5-AO kernels for each wenotype (the reference's
// WENOtype global, src/reconstruction.cpp:7): WENO_Z alpha_k = d_k (1 + (tau / (beta_k + eps))^2),
// WENO_JS alpha_k = d_k / (eps + beta_k)^2, WENO_LINEAR the linear weights (:176-216).
enum { WENO_Z = 0, WENO_JS = 1, WENO_LINEAR = 2 };
inline void weno5_nonlinear(int wtype, const double* d, const double* beta, double tau, double eps, double* ww) {
    if (wtype == WENO_LINEAR) {
        for (int k = 0; k < 4; ++k) ww[k] = d[k];
        return;
    }
    double alpha[4], sum = 0.0;
    for (int k = 0; k < 4; ++k) {
        if (wtype == WENO_JS) {
            alpha[k] = d[k] / ((eps + beta[k]) * (eps + beta[k]));
        } else {
            double gd = tau / (beta[k] + eps);
            alpha[k] = d[k] * (1 + gd * gd);
        }
        sum += alpha[k];
    }
    for (int k = 0; k < 4; ++k) ww[k] = alpha[k] / sum;
}

// non-DF WENO5-AO (epsilon 1e-10, full 5th-order indicator), :161-360
inline void weno5_plain(int side, const double* s, double h, double& var, double& der, int wtype = WENO_Z) {
    const double dhi = 0.85, dlo = 0.85, eps = 1e-10;
    const double wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
    double d[4] = {(1.0 - dhi) * (1.0 - dlo) / 2.0, (1.0 - dhi) * dlo, (1.0 - dhi) * (1.0 - dlo) / 2.0, dhi};
    double beta[4];
    beta3(s, 2, beta);
    beta[3] = beta5_big(wn2, wn1, w0, wp1, wp2);
    double tau = 1.0 / 3.0 * (std::abs(beta[3] - beta[0]) + std::abs(beta[3] - beta[1]) + std::abs(beta[3] - beta[2]));
    double ww[4], fw[4], p[4], px[4];
    weno5_nonlinear(wtype, d, beta, tau, eps, ww);
    if (side == 0) {
        p[0] = -1.0 / 6.0 * wn2 + 5.0 / 6.0 * wn1 + 1.0 / 3.0 * w0;
        p[1] = 1.0 / 3.0 * wn1 + 5.0 / 6.0 * w0 - 1.0 / 6.0 * wp1;
        p[2] = 11.0 / 6.0 * w0 - 7.0 / 6.0 * wp1 + 1.0 / 3.0 * wp2;
        p[3] = (1.0 / 60.0) * (47.0 * w0 + 27.0 * wn1 - 3.0 * wn2 - 13.0 * wp1 + 2.0 * wp2);
        px[0] = (w0 - wn1) / h;
        px[1] = (w0 - wn1) / h;
        px[2] = -((2.0 * w0 - 3.0 * wp1 + wp2) / h);
        px[3] = (15.0 * w0 - 15.0 * wn1 + wn2 - wp1) / (12.0 * h);
    } else {
        p[0] = 1.0 / 3.0 * wn2 - 7.0 / 6.0 * wn1 + 11.0 / 6.0 * w0;
        p[1] = -1.0 / 6.0 * wn1 + 5.0 / 6.0 * w0 + 1.0 / 3.0 * wp1;
        p[2] = 1.0 / 3.0 * w0 + 5.0 / 6.0 * wp1 - 1.0 / 6.0 * wp2;
        p[3] = (1.0 / 60.0) * (47.0 * w0 - 13.0 * wn1 + 2.0 * wn2 + 27.0 * wp1 - 3.0 * wp2);
        px[0] = (2.0 * w0 - 3.0 * wn1 + wn2) / h;
        px[1] = (-w0 + wp1) / h;
        px[2] = (-w0 + wp1) / h;
        px[3] = (-15.0 * w0 + wn1 + 15.0 * wp1 - wp2) / (12.0 * h);
    }
    fw[3] = ww[3] / d[3];
    for (int k = 0; k < 3; ++k) fw[k] = ww[k] - ww[3] / d[3] * d[k];
    var = 0.0;
    der = 0.0;
    for (int k = 0; k < 4; ++k) {
        var += fw[k] * p[k];
        der += fw[k] * px[k];
    }
}

// Non-DF WENO5-AO at the two Gauss-Legendre points -h/(2 sqrt 3) (g[0]) and +h/(2 sqrt 3)
// (g[1]) of the centre cell, with first derivatives when want_der (weno_5th_ao_2gauss,
// src/reconstruction.cpp:2393-2551: epsilon 1e-6; Z-type or Jiang-Shu weights).  Under
// wenotype = linear the reference leaves alpha and sum_alpha unset (:2446-2468 have no linear
// branch), so its result is undefined; this restatement takes the linear weights there.
inline void weno5_2gauss(const double* s, double h, bool want_der, double* g, double* gx, int wtype = WENO_Z) {
    const double dhi = 0.85, dlo = 0.85, eps = 1e-6;
    const double wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
    double d[4] = {(1 - dhi) * (1 - dlo) * 0.5, (1 - dhi) * dlo, (1 - dhi) * (1 - dlo) * 0.5, dhi};
    double beta[4];
    beta3(s, 2, beta);
    beta[3] = beta5_big(wn2, wn1, w0, wp1, wp2);
    double tau = 1.0 / 3.0 * (std::abs(beta[3] - beta[0]) + std::abs(beta[3] - beta[1]) + std::abs(beta[3] - beta[2]));
    double ww[4], fw[4], p[4], px[4];
    weno5_nonlinear(wtype, d, beta, tau, eps, ww);
    fw[3] = ww[3] / d[3];
    for (int k = 0; k < 3; ++k) fw[k] = ww[k] - ww[3] / d[3] * d[k];
    const double sqrt3 = 1.732050807568877294;
    p[0] = w0 - (sqrt3 * w0) / 4 + (4 * wn1 - wn2) / (4 * sqrt3);
    p[1] = w0 + (wn1 - wp1) / (4 * sqrt3);
    p[2] = (1.0 / 12.0) * (3 * (4 + sqrt3) * w0 + sqrt3 * (-4 * wp1 + wp2));
    p[3] = (4314 * w0 + (4 + 500 * sqrt3) * wn1 - wn2 - 70 * sqrt3 * wn2 +
            4 * wp1 - 500 * sqrt3 * wp1 - wp2 + 70 * sqrt3 * wp2) / 4320;
    g[0] = 0;
    for (int k = 0; k < 4; ++k) g[0] += fw[k] * p[k];
    if (want_der) {
        px[0] = -((-9 + sqrt3) * w0 - 2 * (-6 + sqrt3) * wn1 + (-3 + sqrt3) * wn2) / (6 * h);
        px[1] = -(-2 * sqrt3 * w0 + (3 + sqrt3) * wn1 + (-3 + sqrt3) * wp1) / (6 * h);
        px[2] = -((9 + sqrt3) * w0 - 2 * (6 + sqrt3) * wp1 + (3 + sqrt3) * wp2) / (6 * h);
        px[3] = (48 * sqrt3 * w0 - 72 * wn1 - 26 * sqrt3 * wn1 + 9 * wn2 +
                 2 * sqrt3 * wn2 + 72 * wp1 - 26 * sqrt3 * wp1 - 9 * wp2 + 2 * sqrt3 * wp2) / (108 * h);
        gx[0] = 0;
        for (int k = 0; k < 4; ++k) gx[0] += fw[k] * px[k];
    }
    p[0] = (1.0 / 12.0) * (3 * (4 + sqrt3) * w0 + sqrt3 * (-4 * wn1 + wn2));
    p[1] = w0 + (-wn1 + wp1) / (4 * sqrt3);
    p[2] = w0 - (sqrt3 * w0) / 4 + (4 * wp1 - wp2) / (4 * sqrt3);
    p[3] = (4314 * w0 + (4 - 500 * sqrt3) * wn1 - wn2 + 70 * sqrt3 * wn2 +
            4 * wp1 + 500 * sqrt3 * wp1 - wp2 - 70 * sqrt3 * wp2) / 4320;
    g[1] = 0;
    for (int k = 0; k < 4; ++k) g[1] += fw[k] * p[k];
    if (want_der) {
        px[0] = ((9 + sqrt3) * w0 - 2 * (6 + sqrt3) * wn1 + (3 + sqrt3) * wn2) / (6 * h);
        px[1] = (-2 * sqrt3 * w0 + (-3 + sqrt3) * wn1 + (3 + sqrt3) * wp1) / (6 * h);
        px[2] = ((-9 + sqrt3) * w0 - 2 * (-6 + sqrt3) * wp1 + (-3 + sqrt3) * wp2) / (6 * h);
        px[3] = -((48 * sqrt3 * w0 + 72 * wn1 - 26 * sqrt3 * wn1 - 9 * wn2 +
                   2 * sqrt3 * wn2 - 72 * wp1 - 26 * sqrt3 * wp1 + 9 * wp2 + 2 * sqrt3 * wp2) / (108 * h));
        gx[1] = 0;
        for (int k = 0; k < 4; ++k) gx[1] += fw[k] * px[k];
    }
}

}  // namespace oracle_weno
