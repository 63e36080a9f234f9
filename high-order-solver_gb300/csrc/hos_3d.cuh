// hos_3d.cuh -- device code of the 3D step: WENO5-AO (non-DF) face values, the two
// tangential sweeps to the 2 x 2 Gauss points of every face, GKS3D at each point, the S2O4
// update and the CFL reduction (the reference's CubicTube loop, src/3Dproblem.cpp:125-157).
//
// Data layout in HBM (FP64 state, SoA): W[v][cell], cell = (i*ny + j)*nz + k over the block
// with ghosts, the reference's cell order (k fastest).  Every face direction works on its own
// local grid (normal a, first tangential b, second tangential c) in the face's frame:
//   x faces (a, b, c) = (i, j, k),  y faces (j, nx-1-i, k),  z faces (k, j, nx-1-i),
// so that both tangential sweeps run forward in local indices, as the reference's line and
// point loops run along y/-x/y and z/z/-x (src/reconstruction.cpp:3927-3960, :4145-4163),
// and the frame rotations are Ydirection / Zdirection (src/basic_function.cpp:1208-1224).
// Per-direction buffers are laid out with the local axis that is the global k axis fastest
// (c for x and y faces, a for z faces) so that neighbouring threads touch neighbouring cells.
//
// Per stage and direction: face3 (one thread per cell: its two face values, normal WENO5-AO,
// order reduction per cell) -> FV; line3 (one thread per face position: the sweep along b to
// two lines) -> LV; point3 (one thread per line of a face: the sweep along c to two points,
// then GKS3D at both; the two lines of a face sum in a lane pair) -> FS (f, derf summed over
// the four Gauss points with weight 1/4).  Then one update over the cells.
#pragma once
#include <cuda_runtime.h>

#include "hos_weno.cuh"

namespace hos {
namespace d3 {

struct Ctl3 {
    double dt, t;
    unsigned long long cfl_bits;  // running min of CFL candidates (positive doubles as bits)
    unsigned int status, active;  // status bit 0: negative density/pressure or NaN; WAIT_TIMEOUT_BIT:
                                  // a tensor-core MMA of the gate ran past its wait limit
    int step, pad;
    double tbeg;
};

struct Geo3 {
    int nx, ny, nz, g, nodex, nodey, nodez;
    double dx, dy, dz, rc, cfl, gamma, K, c1, c2, mu;
    double idx, idy, idz;   // 1 / dx, 1 / dy, 1 / dz (host)
    double prandtl_coef;    // 1 / Pr - 1 with the Prandtl fix, else 0
    int tau_type, characteristic;
    int bc[6];
    int p_slot;   // FP64: the reference's GKS3D convention, pressure where lambda belongs
    // FP32 copies of gamma, K, c1, c2, mu, prandtl_coef, narrowed on the host (narrow_params3)
    float fgamma, fK, fc1, fc2, fmu, fprc;
};

// index space of one per-direction array: extents (NA, NB, NC), k-aligned axis fastest
struct Lay {
    int NA, NB, NC;
    int afast;
    __host__ __device__ size_t n() const { return (size_t)NA * NB * NC; }
    __device__ __forceinline__ size_t idx(int a, int b, int c) const {
        return afast ? ((size_t)c * NB + b) * NA + a : ((size_t)a * NB + b) * NC + c;
    }
    __device__ __forceinline__ void decode(size_t t, int& a, int& b, int& c) const {
        if (afast) {
            a = (int)(t % NA);
            t /= NA;
            b = (int)(t % NB);
            c = (int)(t / NB);
        } else {
            c = (int)(t % NC);
            t /= NC;
            b = (int)(t % NB);
            a = (int)(t / NB);
        }
    }
};

// one face direction: interior extents of the local grid and spacings
struct Dir3 {
    int dir;
    int n0, n1, n2;
    double hn, h1, h2;
    double ihn, ih1, ih2;   // their inverses, computed on the host (no FP64 division per thread)
    float fihn, fih1, fih2; // and their FP32 copies
    Lay fv;   // face values: faces 0..n0, b in [-2, n1+2), c in [-2, n2+2)
    Lay cel;  // face3 thread space: cells -1..n0 of the normal, fv's b and c
    Lay lv;   // line values: faces 0..n0, b interior, c in [-2, n2+2)
    Lay fs;   // fluxes: faces 0..n0, b and c interior
};

// a launch parameter in the compute type: the FP32 kernels take the copy narrowed on the host (a
// conversion from FP64 runs on GB300's narrow FP64 pipe, once per thread and use otherwise)
template <class T>
__device__ __forceinline__ T par(double d, float f) {
    if constexpr (sizeof(T) == 4) return f;
    else return d;
}
inline void narrow_params3(Geo3& g) {
    g.fgamma = (float)g.gamma;
    g.fK = (float)g.K;
    g.fc1 = (float)g.c1;
    g.fc2 = (float)g.c2;
    g.fmu = (float)g.mu;
    g.fprc = (float)g.prandtl_coef;
}

// global cell of local absolute (A, B, C) (ghosts included)
__device__ __forceinline__ size_t cell_of(const Geo3& g, int dir, int A, int B, int C) {
    int i, j, k;
    if (dir == 0) { i = A; j = B; k = C; }
    else if (dir == 1) { i = g.nx - 1 - B; j = A; k = C; }
    else { i = g.nx - 1 - C; j = B; k = A; }
    return ((size_t)i * g.ny + j) * g.nz + k;
}

// ---- conversions (src/basic_function.cpp:819-857, 994-1095) --------------------------------
template <class T>
__device__ __forceinline__ void prim5(T* pr, const T* w, T gamma) {  // (rho, u, v, w, p)
    const T ir = T(1) / w[0];
    pr[0] = w[0];
    pr[1] = w[1] * ir;
    pr[2] = w[2] * ir;
    pr[3] = w[3] * ir;
    pr[4] = (gamma - T(1)) * (w[4] - T(0.5) * (w[1] * pr[1] + w[2] * pr[2] + w[3] * pr[3]));
}
template <class T>
__device__ __forceinline__ T lambda5(const T* w, T K) {  // (K+3) rho / (4 (rho E - rho |u|^2/2))
    const T ir = T(1) / w[0];
    return (K + T(3)) * T(0.25) * w[0] / (w[4] - T(0.5) * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]) * ir);
}
template <class T>
__device__ __forceinline__ bool reduce5(const T* w, T K) {  // Check_Order_Reduce_by_Lambda_3D
    const T lam = lambda5(w, K);
    return !(lam > T(0));
}
template <class T, class S>
__device__ __forceinline__ void rotate_in(int dir, T* o, const S* wv) {
    o[0] = (T)wv[0];
    o[4] = (T)wv[4];
    if (dir == 0) { o[1] = (T)wv[1]; o[2] = (T)wv[2]; o[3] = (T)wv[3]; }
    else if (dir == 1) { o[1] = (T)wv[2]; o[2] = -(T)wv[1]; o[3] = (T)wv[3]; }
    else { o[1] = (T)wv[3]; o[2] = (T)wv[2]; o[3] = -(T)wv[1]; }
}

// characteristic projection about a primitive base (Char_base_3D / Char_to_convar_3D) with
// the structural zeros of the eigenvector matrices dropped
template <class T>
struct Char5 {
    T u, v, w, c, H, alfa, k2, R;  // k2 = |u|^2 / 2, R = c / (gamma - 1), H = k2 + c R
    __device__ __forceinline__ void init(const T* pr, T gamma) {
        const T gm1 = gamma - T(1);
        u = pr[1];
        v = pr[2];
        w = pr[3];
        c = sqrt(gamma * pr[4] / pr[0]);
        k2 = T(0.5) * (u * u + v * v + w * w);
        alfa = gm1 / (T(2) * c * c);
        R = c / gm1;
        H = k2 + c * R;
    }
    // rows of the left eigenvector matrix: alfa [H + R(u-c), -(u+R), -v, -w, 1],
    // alfa [4 c R - 2H, 2u, 2v, 2w, -2], [-v, 0, 1, 0, 0], [-w, 0, 0, 1, 0],
    // alfa [H - R(u+c), R - u, -v, -w, 1]
    __device__ __forceinline__ void to_char(T* ch, const T* q) const {
        const T m = u * q[1] + v * q[2] + w * q[3];
        ch[0] = alfa * ((H + R * (u - c)) * q[0] - R * q[1] - m + q[4]);
        ch[1] = alfa * T(2) * ((T(2) * R * c - H) * q[0] + m - q[4]);
        ch[2] = q[2] - v * q[0];
        ch[3] = q[3] - w * q[0];
        ch[4] = alfa * ((H - R * (u + c)) * q[0] + R * q[1] - m + q[4]);
    }
    // columns of the right eigenvector matrix: (1, u-c, v, w, H-uc), (1, u, v, w, k2),
    // (0, 0, 1, 0, v), (0, 0, 0, 1, w), (1, u+c, v, w, H+uc)
    __device__ __forceinline__ void from_char(T* q, const T* ch) const {
        const T s = ch[0] + ch[1] + ch[4];
        q[0] = s;
        q[1] = u * s + c * (ch[4] - ch[0]);
        q[2] = v * s + ch[2];
        q[3] = w * s + ch[3];
        q[4] = H * (ch[0] + ch[4]) + u * c * (ch[4] - ch[0]) + k2 * ch[1] + v * ch[2] + w * ch[3];
    }
};

// non-DF WENO5-AO (weights5, weno5_face, weno5_2g): hos_weno.cuh

// ---- GKS3D (src/flux_function.cpp:813-1103) ------------------------------------------------
// Moments of one Maxwellian: whole-space <u^i> (u), one half-space (h: u>0 for the left
// state, u<0 for the right), <v^j>, <w^k>, <xi^2>, <xi^4> (MMDF3d_left/_right/MMDF3d).
template <class T>
struct Mom3 {
    T u[7], h[7], v[6], w[6], x1, x2;
};
template <class T>
__device__ __forceinline__ T erfcT(T x) { return erfc(x); }
// FP32: the fitted form of ferfc (hos_f32x2.cuh), without the library's conversion instructions
template <>
__device__ __forceinline__ float erfcT<float>(float x) { return ferfc(x); }
template <>
__device__ __forceinline__ F2 erfcT<F2>(F2 x) { return ferfc(x); }
template <class T>
__device__ __forceinline__ T expT(T x) { return exp(x); }
template <>
__device__ __forceinline__ float expT<float>(float x) { return __expf(x); }
template <>
__device__ __forceinline__ F2 expT<F2>(F2 x) { return fexp(x); }

template <class T>
__device__ __forceinline__ void mom_whole(Mom3<T>& m, T u, T v, T w, T lambda, T K) {
    const T ol = T(1) / lambda, hl = T(0.5) * ol;
    m.u[0] = T(1);
    m.u[1] = u;
    m.v[0] = T(1);
    m.v[1] = v;
    m.w[0] = T(1);
    m.w[1] = w;
#pragma unroll
    for (int i = 2; i <= 6; ++i) m.u[i] = u * m.u[i - 1] + T(i - 1) * hl * m.u[i - 2];
#pragma unroll
    for (int i = 2; i <= 5; ++i) {
        m.v[i] = v * m.v[i - 1] + T(i - 1) * hl * m.v[i - 2];
        m.w[i] = w * m.w[i - 1] + T(i - 1) * hl * m.w[i - 2];
    }
    m.x1 = T(0.5) * K * ol;
    m.x2 = T(0.25) * (K * K + T(2) * K) * ol * ol;
}
// sgn = +1: u > 0 half space (left state); -1: u < 0 (right state)
template <class T>
__device__ __forceinline__ void mom_half(Mom3<T>& m, T u, T lambda, T sgn) {
    const T hl = T(0.5) / lambda;
    const T a = T(0.5) * erfcT<T>(-sgn * sqrt(lambda) * u);
    const T b = T(0.5) * expT<T>(-lambda * u * u) / sqrt(T(3.14159265358979323846) * lambda);
    m.h[0] = a;
    m.h[1] = u * a + sgn * b;
#pragma unroll
    for (int i = 2; i <= 6; ++i) m.h[i] = u * m.h[i - 1] + T(i - 1) * hl * m.h[i - 2];
}
// <u^i v^j w^k xi^2q> over the whole space (H = false) or the stored half space (H = true)
// (the paired FP32 type leaves out the unit factors u[0] = v[0] = w[0] = 1: a paired multiply is
// not folded away; the scalar types keep the products as written)
template <class T, bool H>
__device__ __forceinline__ T M(const Mom3<T>& m, int i, int j, int k, int q) {
    if constexpr (std::is_same<T, F2>::value) {
        const bool unit_u = !H && i == 0;
        const T& ui = H ? m.h[i] : m.u[i];
        T r;
        if (j == 0 && k == 0) r = unit_u ? T(1.0f) : ui;
        else if (j == 0) r = unit_u ? m.w[k] : T(ui * m.w[k]);
        else if (k == 0) r = unit_u ? m.v[j] : T(ui * m.v[j]);
        else r = unit_u ? T(m.v[j] * m.w[k]) : T(ui * m.v[j] * m.w[k]);
        if (q == 0) return r;
        const T& x = q == 1 ? m.x1 : m.x2;
        return unit_u && j == 0 && k == 0 ? x : T(r * x);
    } else {
        const T r = (H ? m.h[i] : m.u[i]) * m.v[j] * m.w[k];
        return q == 0 ? r : q == 1 ? r * m.x1 : r * m.x2;
    }
}
// <a psi u^NU v^NV w^NW> (GL_/GR_/G_address, include/basic_function.h:222-358)
template <class T, bool H, int NU, int NV, int NW>
__device__ __forceinline__ void gaddr(const Mom3<T>& m, const T* a, T* psi) {
#define MM(i, j, k, q) M<T, H>(m, NU + (i), NV + (j), NW + (k), (q))
    psi[0] = a[0] * MM(0, 0, 0, 0) + a[1] * MM(1, 0, 0, 0) + a[2] * MM(0, 1, 0, 0) + a[3] * MM(0, 0, 1, 0)
             + a[4] * T(0.5) * (MM(2, 0, 0, 0) + MM(0, 2, 0, 0) + MM(0, 0, 2, 0) + MM(0, 0, 0, 1));
    psi[1] = a[0] * MM(1, 0, 0, 0) + a[1] * MM(2, 0, 0, 0) + a[2] * MM(1, 1, 0, 0) + a[3] * MM(1, 0, 1, 0)
             + a[4] * T(0.5) * (MM(3, 0, 0, 0) + MM(1, 2, 0, 0) + MM(1, 0, 2, 0) + MM(1, 0, 0, 1));
    psi[2] = a[0] * MM(0, 1, 0, 0) + a[1] * MM(1, 1, 0, 0) + a[2] * MM(0, 2, 0, 0) + a[3] * MM(0, 1, 1, 0)
             + a[4] * T(0.5) * (MM(2, 1, 0, 0) + MM(0, 3, 0, 0) + MM(0, 1, 2, 0) + MM(0, 1, 0, 1));
    psi[3] = a[0] * MM(0, 0, 1, 0) + a[1] * MM(1, 0, 1, 0) + a[2] * MM(0, 1, 1, 0) + a[3] * MM(0, 0, 2, 0)
             + a[4] * T(0.5) * (MM(2, 0, 1, 0) + MM(0, 2, 1, 0) + MM(0, 0, 3, 0) + MM(0, 0, 1, 1));
    psi[4] = T(0.5) * (a[0] * (MM(2, 0, 0, 0) + MM(0, 2, 0, 0) + MM(0, 0, 2, 0) + MM(0, 0, 0, 1)) +
                       a[1] * (MM(3, 0, 0, 0) + MM(1, 2, 0, 0) + MM(1, 0, 2, 0) + MM(1, 0, 0, 1)) +
                       a[2] * (MM(2, 1, 0, 0) + MM(0, 3, 0, 0) + MM(0, 1, 2, 0) + MM(0, 1, 0, 1)) +
                       a[3] * (MM(2, 0, 1, 0) + MM(0, 2, 1, 0) + MM(0, 0, 3, 0) + MM(0, 0, 1, 1)) +
                       a[4] * T(0.5) * (MM(4, 0, 0, 0) + MM(0, 4, 0, 0) + MM(0, 0, 4, 0) + MM(0, 0, 0, 2) +
                                        T(2) * (MM(2, 2, 0, 0) + MM(2, 0, 2, 0) + MM(2, 0, 0, 1) + MM(0, 2, 2, 0) +
                                                MM(0, 2, 0, 1) + MM(0, 0, 2, 1))));
#undef MM
}
// <psi u^NU> of the Maxwellian itself (a = (1, 0, 0, 0, 0))
template <class T, bool H, int NU>
__device__ __forceinline__ void gunit(const Mom3<T>& m, T* psi) {
    psi[0] = M<T, H>(m, NU, 0, 0, 0);
    psi[1] = M<T, H>(m, NU + 1, 0, 0, 0);
    psi[2] = M<T, H>(m, NU, 1, 0, 0);
    psi[3] = M<T, H>(m, NU, 0, 1, 0);
    psi[4] = T(0.5) * (M<T, H>(m, NU + 2, 0, 0, 0) + M<T, H>(m, NU, 2, 0, 0) + M<T, H>(m, NU, 0, 2, 0)
                       + M<T, H>(m, NU, 0, 0, 1));
}
// microslope from a conserved-variable slope (A 3D, src/basic_function.cpp:585-601);
// pr = (rho, u, v, w, lambda)
template <class T>
__device__ __forceinline__ void micro3(T* a, const T* der, const T* pr, T K) {
    const T ir = T(1) / pr[0], ol = T(1) / pr[4];
    const T u = pr[1], v = pr[2], w = pr[3], lam = pr[4];
    const T q2 = u * u + v * v + w * w + T(0.5) * (K + T(3)) * ol;
    const T A = (T(2) * der[4] - q2 * der[0]) * ir;
    const T B = (der[1] - u * der[0]) * ir;
    const T C = (der[2] - v * der[0]) * ir;
    const T D = (der[3] - w * der[0]) * ir;
    a[4] = T(4) * lam * lam / (K + T(3)) * (A - T(2) * (u * B + v * C + w * D));
    a[3] = T(2) * lam * D - w * a[4];
    a[2] = T(2) * lam * C - v * a[4];
    a[1] = T(2) * lam * B - u * a[4];
    a[0] = der[0] * ir - u * a[1] - v * a[2] - w * a[3] - T(0.5) * a[4] * q2;
}
template <class T>
__device__ __forceinline__ void ulambda5(T* pr, const T* w, T K) {
    const T ir = T(1) / w[0];
    pr[0] = w[0];
    pr[1] = w[1] * ir;
    pr[2] = w[2] * ir;
    pr[3] = w[3] * ir;
    pr[4] = (K + T(3)) * T(0.25) * w[0] / (w[4] - T(0.5) * w[0] * (pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]));
}
// the six time-integration coefficients of the 2nd-order GKS flux over [0, dt]
template <class T>
__device__ __forceinline__ void tcoef(T* t, T tau, T tn, T dt) {
    const T eta = expT<T>(-dt / tn);
    t[0] = tn * (T(1) - eta);
    t[1] = tn * (eta * (dt + tn) - tn) + tau * tn * (eta - T(1));
    t[2] = tau * tn * (eta - T(1));
    t[3] = tn * eta + dt - tn;
    t[4] = tn * (tn - eta * (dt + tn) - tau * (eta - T(1))) - dt * tau;
    t[5] = T(0.5) * dt * dt - tau * tn * (eta - T(1)) - tau * dt;
}
template <class T>
__device__ __forceinline__ T tau_num3(const Geo3& g, T dl, T dr, T ll, T lr, T d0, T l0, T dt) {
    const T C = par<T>(g.c2, g.fc2) * fabsT(dl / ll - dr / lr) / fabsT(dl / ll + dr / lr);
    if (g.tau_type == 0) {
        if (g.c1 <= 0 && g.c2 <= 0) return T(0);
        return par<T>(g.c1, g.fc1) * dt + dt * C;
    }
    T tn = C * dt;
    if (tn != tn) tn = T(0);
    return g.mu > 0 ? tn + T(2) * par<T>(g.mu, g.fmu) * l0 / d0 : T(0);
}

// one side's contribution to the flux: rho t0 <u g> + rho t1 <u a.psi (u, v, w)> +
// rho t2 <u A psi>, for the two time levels (coefficients ta, tb)
// The three moment sets of one side: g = <u psi>, s1 = <u a.psi (u, v, w)>, s2 = <u A psi>.
template <class T>
__device__ __forceinline__ void side_terms(const Mom3<T>& m, const T* pr, const T (*al)[5], T K, T* g, T* s1, T* s2) {
    T tmp[5];
    gunit<T, true, 1>(m, g);
    gaddr<T, true, 2, 0, 0>(m, al[0], s1);
    gaddr<T, true, 1, 1, 0>(m, al[1], tmp);
#pragma unroll
    for (int v = 0; v < 5; ++v) s1[v] += tmp[v];
    gaddr<T, true, 1, 0, 1>(m, al[2], tmp);
#pragma unroll
    for (int v = 0; v < 5; ++v) s1[v] += tmp[v];
    // time derivative from the compatibility condition, with whole-space moments
    T der[5];
    gaddr<T, false, 1, 0, 0>(m, al[0], der);
    gaddr<T, false, 0, 1, 0>(m, al[1], tmp);
#pragma unroll
    for (int v = 0; v < 5; ++v) der[v] += tmp[v];
    gaddr<T, false, 0, 0, 1>(m, al[2], tmp);
#pragma unroll
    for (int v = 0; v < 5; ++v) der[v] = -pr[0] * (der[v] + tmp[v]);
    T A[5];
    micro3<T>(A, der, pr, K);
    gaddr<T, true, 1, 0, 0>(m, A, s2);
}
template <class T>
__device__ __forceinline__ void side_flux(const Mom3<T>& m, const T* pr, const T (*al)[5], T K, const T* ta,
                                          const T* tb, T* Fa, T* Fb) {
    T g[5], s1[5], s2[5];
    side_terms<T>(m, pr, al, K, g, s1, s2);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        Fa[v] += pr[0] * (ta[0] * g[v] + ta[1] * s1[v] + ta[2] * s2[v]);
        Fb[v] += pr[0] * (tb[0] * g[v] + tb[1] * s1[v] + tb[2] * s2[v]);
    }
}

// Collision-state primitives p0 and the time-integration coefficients of both time levels (ta:
// dt, tb: dt / 2) from the sides' densities and lambdas; returns the physical collision time.
template <class T>
__device__ __forceinline__ T gks3_coef(const T* c0, T pl0, T pr0, T pl4, T pr4, T dt, const Geo3& g, T K, bool p_slot,
                                       T* p0, T* ta, T* tb) {
    if (p_slot) prim5<T>(p0, c0, T(g.gamma));
    else ulambda5<T>(p0, c0, K);
    const T tau = (g.tau_type != 0 && g.mu > 0) ? T(2) * par<T>(g.mu, g.fmu) * p0[4] / p0[0] : T(0);
    const T dt2 = T(0.5) * dt;
    tcoef<T>(ta, tau, tau_num3<T>(g, pl0, pr0, pl4, pr4, p0[0], p0[4], dt), dt);
    tcoef<T>(tb, tau, tau_num3<T>(g, pl0, pr0, pl4, pr4, p0[0], p0[4], dt2), dt2);
    return tau;
}

// The equilibrium part about the centre state p0 (slopes d0 of the collision state) added to the
// sides' time-integrated fluxes Fa (dt) and Fb (dt / 2); f, df: the S2O4 pair.
template <class T>
__device__ __forceinline__ void gks3_centre(const T* p0, const T (*d0)[5], T tau, const T* ta, const T* tb, T dt,
                                            const Geo3& g, T K, T* Fa, T* Fb, T* f, T* df) {
    const T dt2 = T(0.5) * dt;
    Mom3<T> m0;
    mom_whole<T>(m0, p0[1], p0[2], p0[3], p0[4], K);
    T g0u[5], a0[5], s4[5], der[5], tmp[5], tmp2[5];
    gunit<T, false, 1>(m0, g0u);
    micro3<T>(a0, d0[0], p0, K);
    gaddr<T, false, 2, 0, 0>(m0, a0, s4);
    gaddr<T, false, 1, 0, 0>(m0, a0, der);
    T a0xuu[5];   // the x-slope part alone, for the Prandtl fix
#pragma unroll
    for (int v = 0; v < 5; ++v) a0xuu[v] = s4[v];
    micro3<T>(a0, d0[1], p0, K);
    gaddr<T, false, 1, 1, 0>(m0, a0, tmp);
    gaddr<T, false, 0, 1, 0>(m0, a0, tmp2);
#pragma unroll
    for (int v = 0; v < 5; ++v) { s4[v] += tmp[v]; der[v] += tmp2[v]; }
    micro3<T>(a0, d0[2], p0, K);
    gaddr<T, false, 1, 0, 1>(m0, a0, tmp);
    gaddr<T, false, 0, 0, 1>(m0, a0, tmp2);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        s4[v] += tmp[v];
        der[v] = -p0[0] * (der[v] + tmp2[v]);
    }
    micro3<T>(a0, der, p0, K);
    gaddr<T, false, 1, 0, 0>(m0, a0, tmp);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        Fa[v] += p0[0] * (ta[3] * g0u[v] + ta[4] * s4[v] + ta[5] * tmp[v]);
        Fb[v] += p0[0] * (tb[3] * g0u[v] + tb[4] * s4[v] + tb[5] * tmp[v]);
    }
    if (g.prandtl_coef != 0.0) {
        // Prandtl-number correction of the heat flux: GKS2D's (src/flux_function.cpp:630-636,
        // 678-684; the reference's GKS3D has none) with the third velocity component
        const T prc = par<T>(g.prandtl_coef, g.fprc);
        const T qs = a0xuu[4] + tmp[4] - p0[1] * (a0xuu[1] + tmp[1]) - p0[2] * (a0xuu[2] + tmp[2]) -
                     p0[3] * (a0xuu[3] + tmp[3]);
        Fa[4] += prc * (qs * (-p0[0] * tau * dt));
        Fb[4] += prc * (qs * (-p0[0] * tau * dt2));
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        f[v] = T(4) * Fb[v] - Fa[v];
        df[v] = T(4) * (Fa[v] - T(2) * Fb[v]);
    }
}

// GKS3D at one Gauss point, face frame: S2O4 pair f = 4 F(dt/2) - F(dt), derf = 4 (F(dt) - 2 F(dt/2)).
// L/R: value (c) and slopes along normal, t1, t2 (d[3]) of the left and right states.
template <class T>
__device__ void gks3(const T* Lc, const T (*Ld)[5], const T* Rc, const T (*Rd)[5], T dt, const Geo3& g, T* f,
                     T* df) {
    const T K = par<T>(g.K, g.fK);
    T pl[5], pr[5];
    // the reference's GKS3D hands Convar_to_primvar_3D's pressure to every lambda slot
    // (src/flux_function.cpp:831-836, 914); only the FP64 kernels carry that convention
    const bool p_slot = sizeof(T) == 8 && g.p_slot;
    if (p_slot) {
        prim5<T>(pl, Lc, T(g.gamma));
        prim5<T>(pr, Rc, T(g.gamma));
    } else {
        ulambda5<T>(pl, Lc, K);
        ulambda5<T>(pr, Rc, K);
    }
    Mom3<T> ml, mr;
    mom_whole<T>(ml, pl[1], pl[2], pl[3], pl[4], K);
    mom_half<T>(ml, pl[1], pl[4], T(1));
    mom_whole<T>(mr, pr[1], pr[2], pr[3], pr[4], K);
    mom_half<T>(mr, pr[1], pr[4], T(-1));
    // all-collision centre state and its slopes
    T c0[5];
    c0[0] = pl[0] * ml.h[0] + pr[0] * mr.h[0];
    c0[1] = pl[0] * ml.h[1] + pr[0] * mr.h[1];
    c0[2] = pl[0] * ml.v[1] * ml.h[0] + pr[0] * mr.v[1] * mr.h[0];
    c0[3] = pl[0] * ml.w[1] * ml.h[0] + pr[0] * mr.w[1] * mr.h[0];
    c0[4] = T(0.5) * pl[0] * (ml.h[2] + ml.h[0] * (ml.v[2] + ml.w[2] + ml.x1))
            + T(0.5) * pr[0] * (mr.h[2] + mr.h[0] * (mr.v[2] + mr.w[2] + mr.x1));
    T al[3][5], ar[3][5], d0[3][5];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        micro3<T>(al[d], Ld[d], pl, K);
        micro3<T>(ar[d], Rd[d], pr, K);
        T a0l[5], a0r[5];
        gaddr<T, true, 0, 0, 0>(ml, al[d], a0l);
        gaddr<T, true, 0, 0, 0>(mr, ar[d], a0r);
#pragma unroll
        for (int v = 0; v < 5; ++v) d0[d][v] = pl[0] * a0l[v] + pr[0] * a0r[v];
    }
    T p0[5], ta[6], tb[6];
    const T tau = gks3_coef<T>(c0, pl[0], pr[0], pl[4], pr[4], dt, g, K, p_slot, p0, ta, tb);
    T Fa[5] = {T(0), T(0), T(0), T(0), T(0)}, Fb[5] = {T(0), T(0), T(0), T(0), T(0)};
    side_flux<T>(ml, pl, al, K, ta, tb, Fa, Fb);
    side_flux<T>(mr, pr, ar, K, ta, tb, Fa, Fb);
    gks3_centre<T>(p0, d0, tau, ta, tb, dt, g, K, Fa, Fb, f, df);
}

// FP32 GKS3D with the two sides in the two lanes of the paired FP32 type (lane x the left state
// and the u > 0 half space of its Maxwellian, lane y the right state and its u < 0 half space):
// the side moments, micro-slopes, the collision state and its slopes and the sides' flux
// contributions are formed on both lanes at once and summed across them; the time coefficients
// and the centre part are scalar (gks3_coef, gks3_centre).  Euler or Navier-Stokes collision
// time, the lambda convention (the reference's pressure slot is FP64 only).
__device__ __forceinline__ void gks3_lr(const float* Lc, const float (*Ld)[5], const float* Rc, const float (*Rd)[5],
                                        float dt, const Geo3& g, float* f, float* df) {
    const float K = g.fK;
    const F2 Kp(K);
    F2 w[5], ps[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) w[v] = F2(Lc[v], Rc[v]);
    ulambda5<F2>(ps, w, Kp);
    Mom3<F2> m;
    mom_whole<F2>(m, ps[1], ps[2], ps[3], ps[4], Kp);
    mom_half<F2>(m, ps[1], ps[4], F2(1.0f, -1.0f));
    const F2 r = ps[0];
    float c0[5];
    c0[0] = hsum(r * m.h[0]);
    c0[1] = hsum(r * m.h[1]);
    c0[2] = hsum(r * m.v[1] * m.h[0]);
    c0[3] = hsum(r * m.w[1] * m.h[0]);
    c0[4] = hsum(F2(0.5f) * r * (m.h[2] + m.h[0] * (m.v[2] + m.w[2] + m.x1)));
    F2 a[3][5];
    float d0[3][5];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        F2 sl[5], a0[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) sl[v] = F2(Ld[d][v], Rd[d][v]);
        micro3<F2>(a[d], sl, ps, Kp);
        gaddr<F2, true, 0, 0, 0>(m, a[d], a0);
#pragma unroll
        for (int v = 0; v < 5; ++v) d0[d][v] = hsum(r * a0[v]);
    }
    // the sides' moment sets before the time coefficients: the moments and micro-slopes need not
    // stay live across the scalar part
    F2 gs[5], s1[5], s2[5];
    side_terms<F2>(m, ps, a, Kp, gs, s1, s2);
    float p0[5], ta[6], tb[6];
    const float tau = gks3_coef<float>(c0, r.v.x, r.v.y, ps[4].v.x, ps[4].v.y, dt, g, K, false, p0, ta, tb);
    float Fa[5], Fb[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        Fa[v] = hsum(r * (F2(ta[0]) * gs[v] + F2(ta[1]) * s1[v] + F2(ta[2]) * s2[v]));
        Fb[v] = hsum(r * (F2(tb[0]) * gs[v] + F2(tb[1]) * s1[v] + F2(tb[2]) * s2[v]));
    }
    gks3_centre<float>(p0, d0, tau, ta, tb, dt, g, K, Fa, Fb, f, df);
}


// ---- learned gate (FP32 path): linear reconstructions and their check --------------------
// Per cell one flag byte, bit a set when the gate predicts the WENO5-AO weights of the cell's
// stencil along global axis a (0 x, 1 y, 2 z) to stay near the linear weights.  Flagged
// reconstructions take the big-stencil polynomial alone in conservative variables (the linear
// weights select it, and a linear reconstruction commutes with the characteristic projection);
// a result that fails the check below takes the full WENO5-AO path.
struct Gate3 {
    const unsigned char* flags;    // null: no gate
    unsigned long long* fallback;  // linear results the check rejected
};
// global axis of a direction's normal (k 0), first (1) and second (2) tangential sweep
__host__ __device__ constexpr int axis3(int dir, int k) {
    return k == 0 ? dir : k == 1 ? (dir == 1 ? 0 : 1) : (dir == 2 ? 0 : 2);
}
// value and slope of the big-stencil polynomial at the left (side 0) or right face
template <class T>
__device__ __forceinline__ void lin5_face(int side, const T* s, T ih, T& var, T& der) {
    const T wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
    if (side == 0) {
        var = T(1.0 / 60.0) * (T(47) * w0 + T(27) * wn1 - T(3) * wn2 - T(13) * wp1 + T(2) * wp2);
        der = (T(15) * w0 - T(15) * wn1 + wn2 - wp1) * (T(1.0 / 12.0) * ih);
    } else {
        var = T(1.0 / 60.0) * (T(47) * w0 - T(13) * wn1 + T(2) * wn2 + T(27) * wp1 - T(3) * wp2);
        der = (T(-15) * w0 + wn1 + T(15) * wp1 - wp2) * (T(1.0 / 12.0) * ih);
    }
}
// the big-stencil polynomial at the two Gauss points (and its slope when DER)
template <class T, bool DER>
__device__ __forceinline__ void lin5_2g(const T* s, T ih, T* g, T* gx) {
    const T wn2 = s[0], wn1 = s[1], w0 = s[2], wp1 = s[3], wp2 = s[4];
    const T r3 = T(1.732050807568877294);
    g[0] = (T(4314) * w0 + (T(4) + T(500) * r3) * wn1 - wn2 - T(70) * r3 * wn2 + T(4) * wp1 - T(500) * r3 * wp1 - wp2
            + T(70) * r3 * wp2) * T(1.0 / 4320.0);
    g[1] = (T(4314) * w0 + (T(4) - T(500) * r3) * wn1 - wn2 + T(70) * r3 * wn2 + T(4) * wp1 + T(500) * r3 * wp1 - wp2
            - T(70) * r3 * wp2) * T(1.0 / 4320.0);
    if (DER) {
        const T i108h = ih * T(1.0 / 108.0);
        gx[0] = (T(48) * r3 * w0 - T(72) * wn1 - T(26) * r3 * wn1 + T(9) * wn2 + T(2) * r3 * wn2 + T(72) * wp1
                 - T(26) * r3 * wp1 - T(9) * wp2 + T(2) * r3 * wp2) * i108h;
        gx[1] = -(T(48) * r3 * w0 + T(72) * wn1 - T(26) * r3 * wn1 - T(9) * wn2 + T(2) * r3 * wn2 - T(72) * wp1
                  - T(26) * r3 * wp1 + T(9) * wp2 + T(2) * r3 * wp2) * i108h;
    }
}
// a linear result is kept when it has a positive temperature and its density and total energy
// lie within the three central stencil states' range widened by a tenth of that range
template <class T>
__device__ __forceinline__ bool lin5_ok(const T* q, const T* wm, const T* w0, const T* wp, T K) {
    if (reduce5<T>(q, K)) return false;
#pragma unroll
    for (int v = 0; v < 5; v += 4) {
        const T lo = fminT(fminT(wm[v], w0[v]), wp[v]), hi = fmaxT(fmaxT(wm[v], w0[v]), wp[v]);
        const T m = T(0.1) * (hi - lo) + T(1e-6) * fabsT(w0[v]);
        if (!(q[v] >= lo - m && q[v] <= hi + m)) return false;
    }
    return true;
}

// ---- kernels ---------------------------------------------------------------------------
constexpr int FACE3_THREADS = 128;
constexpr int LINE3_THREADS = 128;
constexpr int POINT3_THREADS = 128;

// Face values: one thread per local cell (normal index -1..n0, tangential halo 2); the cell's
// value at its left face (the right-hand state of face a) and at its right face (the
// left-hand state of face a+1), WENO5_AO (src/reconstruction.cpp:3803-3925).  The two values
// fall back to the cell average with zero slope when either has a non-positive lambda.
// FV planes: q 0..4 left-hand value, 5..9 its normal slope, 10..14 right-hand value, 15..19.
// W: the state in the compute type -- the FP64 state, or for T = float the FP32 mirror the
// stage's mirror3 pass writes (converted once per cell instead of once per stencil use)
template <class T, bool GATED = false>
__global__ void __launch_bounds__(FACE3_THREADS) face3_kernel(const T* __restrict__ W, T* __restrict__ FV,
                                                              Geo3 g, Dir3 d, const Ctl3* ctl, Gate3 gt) {
    if (!ctl->active) return;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.cel.n()) return;
    int a0, b0, c0;
    d.cel.decode(t, a0, b0, c0);
    const int ac = a0 - 1, G = g.g;
    const size_t plane = (size_t)g.nx * g.ny * g.nz;
    const T gamma = par<T>(g.gamma, g.fgamma), K = par<T>(g.K, g.fK), ih = par<T>(d.ihn, d.fihn);
    T st[5][5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
        const size_t cc = cell_of(g, d.dir, ac - 2 + m + G, b0 - 2 + G, c0 - 2 + G);
        T wv[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) wv[v] = W[v * plane + cc];
        rotate_in<T>(d.dir, st[m], wv);
    }
    T pr[3][5];
#pragma unroll
    for (int m = 0; m < 3; ++m) prim5<T>(pr[m], st[1 + m], gamma);
    T oc[2][5], od[2][5];
    bool lin = false;
    if constexpr (GATED) {
        const size_t cc = cell_of(g, d.dir, ac + G, b0 - 2 + G, c0 - 2 + G);
        if ((gt.flags[cc] >> axis3(d.dir, 0)) & 1) {
#pragma unroll
            for (int side = 0; side < 2; ++side)
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    const T s5[5] = {st[0][v], st[1][v], st[2][v], st[3][v], st[4][v]};
                    lin5_face<T>(side, s5, ih, oc[side][v], od[side][v]);
                }
            lin = lin5_ok<T>(oc[0], st[1], st[2], st[3], K) && lin5_ok<T>(oc[1], st[1], st[2], st[3], K);
            if (!lin) atomicAdd(gt.fallback, 1ull);
        }
    }
#pragma unroll
    for (int side = 0; side < 2 && !lin; ++side) {
        T s5[5][5];
        Char5<T> ch;
        if (g.characteristic) {
            T base[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) base[v] = T(0.5) * (pr[side == 0 ? 0 : 2][v] + pr[1][v]);
            ch.init(base, gamma);
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                T q[5];
                ch.to_char(q, st[m]);
#pragma unroll
                for (int v = 0; v < 5; ++v) s5[v][m] = q[v];
            }
        } else {
#pragma unroll
            for (int m = 0; m < 5; ++m)
#pragma unroll
                for (int v = 0; v < 5; ++v) s5[v][m] = st[m][v];
        }
        T var[5], der[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) weno5_face<T>(side, s5[v], ih, var[v], der[v]);
        if (g.characteristic) {
            ch.from_char(oc[side], var);
            ch.from_char(od[side], der);
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) { oc[side][v] = var[v]; od[side][v] = der[v]; }
        }
    }
    if (reduce5<T>(oc[0], K) || reduce5<T>(oc[1], K)) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            oc[0][v] = oc[1][v] = st[2][v];
            od[0][v] = od[1][v] = T(0);
        }
    }
    const size_t nfv = d.fv.n();
    if (ac >= 0) {
        const size_t f = d.fv.idx(ac, b0, c0);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            FV[(10 + v) * nfv + f] = oc[0][v];
            FV[(15 + v) * nfv + f] = od[0][v];
        }
    }
    if (ac + 1 <= d.n0) {
        const size_t f = d.fv.idx(ac + 1, b0, c0);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            FV[v * nfv + f] = oc[1][v];
            FV[(5 + v) * nfv + f] = od[1][v];
        }
    }
}

// One side of a tangential sweep: five states along the sweep (centre m = 2) of NQ
// quantities (q 0: values, whose sweep also gives the slope along the sweep; q >= 1: carried
// slopes) -> the two Gauss points: out[ig][q] for q < NQ, and out[ig][NQ] the new slope.
// Characteristic variables about the centre state's primitives (WENO5_AO_for_line_value,
// :3963-4108; WENO5_AO_for_point_value, :4165-4360).
template <class T, int NQ>
__device__ __forceinline__ void sweep_side(const T (*st)[NQ][5], T ih, const Geo3& g, T (*out)[NQ + 1][5]) {
    const T gamma = par<T>(g.gamma, g.fgamma);
    Char5<T> ch;
    if (g.characteristic) {
        T base[5];
        prim5<T>(base, st[2][0], gamma);
        ch.init(base, gamma);
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        T s5[5][5];
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            if (g.characteristic) {
                T x[5];
                ch.to_char(x, st[m][q]);
#pragma unroll
                for (int v = 0; v < 5; ++v) s5[v][m] = x[v];
            } else {
#pragma unroll
                for (int v = 0; v < 5; ++v) s5[v][m] = st[m][q][v];
            }
        }
        T gv[2][5], gx[2][5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            T a[2], b[2];
            if (q == 0) weno5_2g<T, true>(s5[v], ih, a, b);
            else weno5_2g<T, false>(s5[v], ih, a, b);
            gv[0][v] = a[0];
            gv[1][v] = a[1];
            gx[0][v] = b[0];
            gx[1][v] = b[1];
        }
#pragma unroll
        for (int ig = 0; ig < 2; ++ig) {
            if (g.characteristic) {
                ch.from_char(out[ig][q], gv[ig]);
                if (q == 0) ch.from_char(out[ig][NQ], gx[ig]);
            } else {
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    out[ig][q][v] = gv[ig][v];
                    if (q == 0) out[ig][NQ][v] = gx[ig][v];
                }
            }
        }
    }
}

// Lines: one thread per face position (faces 0..n0, b interior, c in the halo); the sweep
// along b of the face values of both sides to the two Gauss lines, with the order reduction
// of the position (any non-positive lambda: both lines take the face values, zero slope).
// LV planes [ig][side][value 5 | normal slope 5 | t1 slope 5].
template <class T, bool GATED = false>
__global__ void __launch_bounds__(LINE3_THREADS) line3_kernel(const T* __restrict__ FV, T* __restrict__ LV, Geo3 g,
                                                              Dir3 d, const Ctl3* ctl, Gate3 gt) {
    if (!ctl->active) return;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.lv.n()) return;
    int a, b, c;
    d.lv.decode(t, a, b, c);
    const size_t nfv = d.fv.n(), nlv = d.lv.n();
    const T ih = par<T>(d.ih1, d.fih1), K = par<T>(g.K, g.fK);
    bool reduce = false;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        T st[5][2][5];
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            const size_t f = d.fv.idx(a, b + m, c);
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                st[m][0][v] = FV[(side * 10 + v) * nfv + f];
                st[m][1][v] = FV[(side * 10 + 5 + v) * nfv + f];
            }
        }
        T out[2][3][5];
        bool lin = false;
        if constexpr (GATED) {
            // the side's cell, smooth along this sweep's axis: the big-stencil polynomial
            const size_t cc = cell_of(g, d.dir, a - 1 + side + g.g, b + g.g, c - 2 + g.g);
            if ((gt.flags[cc] >> axis3(d.dir, 1)) & 1) {
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    const T s0[5] = {st[0][0][v], st[1][0][v], st[2][0][v], st[3][0][v], st[4][0][v]};
                    const T s1[5] = {st[0][1][v], st[1][1][v], st[2][1][v], st[3][1][v], st[4][1][v]};
                    T gv[2], gx[2], gd[2];
                    lin5_2g<T, true>(s0, ih, gv, gx);
                    lin5_2g<T, false>(s1, ih, gd, gd);
#pragma unroll
                    for (int ig = 0; ig < 2; ++ig) {
                        out[ig][0][v] = gv[ig];
                        out[ig][2][v] = gx[ig];
                        out[ig][1][v] = gd[ig];
                    }
                }
                lin = lin5_ok<T>(out[0][0], st[1][0], st[2][0], st[3][0], K) &&
                      lin5_ok<T>(out[1][0], st[1][0], st[2][0], st[3][0], K);
                if (!lin) atomicAdd(gt.fallback, 1ull);
            }
        }
        if (!lin) sweep_side<T, 2>(st, ih, g, out);
#pragma unroll
        for (int ig = 0; ig < 2; ++ig) {
            reduce = reduce || reduce5<T>(out[ig][0], K);
#pragma unroll
            for (int q = 0; q < 3; ++q)
#pragma unroll
                for (int v = 0; v < 5; ++v) LV[(((ig * 2 + side) * 3 + q) * 5 + v) * nlv + t] = out[ig][q][v];
        }
    }
    if (reduce) {  // rare: overwrite with the face values
        const size_t f = d.fv.idx(a, b + 2, c);
        for (int side = 0; side < 2; ++side)
            for (int ig = 0; ig < 2; ++ig)
                for (int v = 0; v < 5; ++v) {
                    LV[(((ig * 2 + side) * 3 + 0) * 5 + v) * nlv + t] = FV[(side * 10 + v) * nfv + f];
                    LV[(((ig * 2 + side) * 3 + 1) * 5 + v) * nlv + t] = FV[(side * 10 + 5 + v) * nfv + f];
                    LV[(((ig * 2 + side) * 3 + 2) * 5 + v) * nlv + t] = T(0);
                }
    }
}

// Points and fluxes: one thread per Gauss line of an interior face (the two lines of a face
// in a lane pair).  The sweep along c of the line values of both sides to the line's two
// Gauss points (order reduction per line), GKS3D at both points, the face's (f, derf) summed
// over its four points with weight 1/4, and the S2O4 stage combination in FP64 (Update_gauss,
// src/time_advance.cpp:862-940; S2O4_3D :732-741): FS[0][v][face] receives the stage's
// combined flux, 1/2 f0 + 1/8 derf0 at stage 0 and (f0 + 1/6 derf0) + (0 f1 + 1/3 derf1) at
// stage 1, whose first part stage 0 leaves in FS[1][v][face].  Face frame.  T = float runs
// three 128-thread CTAs per SM (168 registers).
template <class T, bool GATED = false>
__global__ void __launch_bounds__(POINT3_THREADS, sizeof(T) == 4 ? 3 : 1) point3_kernel(const T* __restrict__ LV, double* __restrict__ FS,
                                                                Geo3 g, Dir3 d, const Ctl3* ctl, int stage, Gate3 gt) {
    if (!ctl->active) return;
    // point states [ip][side][value | normal | t1 | t2 slope][5]: FP64 in registers, FP32 in
    // shared memory (one column per thread), which leaves the paired GKS its registers
    __shared__ float pt_sm[sizeof(T) == 4 ? 80 : 1][POINT3_THREADS];
    T pt_reg[sizeof(T) == 4 ? 1 : 2][2][4][5];
    auto PT = [&](int ip, int side, int q, int v) -> T& {
        if constexpr (sizeof(T) == 4) return pt_sm[((ip * 2 + side) * 4 + q) * 5 + v][threadIdx.x];
        else return pt_reg[ip][side][q][v];
    };
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nfs = d.fs.n(), nlv = d.lv.n();
    const bool valid = t < 2 * nfs;
    const int ig = (int)(t & 1);
    const size_t face = t >> 1;
    T acc[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) acc[q] = T(0);
    int a = 0, b = 0, c = 0;
    if (valid) {
        d.fs.decode(face, a, b, c);
        const T ih = par<T>(d.ih2, d.fih2), K = par<T>(g.K, g.fK), dt = T(ctl->dt);
        bool reduce = false;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            T st[5][3][5];
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                const size_t l = d.lv.idx(a, b, c + m);
#pragma unroll
                for (int q = 0; q < 3; ++q)
#pragma unroll
                    for (int v = 0; v < 5; ++v) st[m][q][v] = LV[(((ig * 2 + side) * 3 + q) * 5 + v) * nlv + l];
            }
            T out[2][4][5];
            bool lin = false;
            if constexpr (GATED) {
                const size_t cc = cell_of(g, d.dir, a - 1 + side + g.g, b + g.g, c + g.g);
                if ((gt.flags[cc] >> axis3(d.dir, 2)) & 1) {
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        T sv[5], gv[2], gx[2];
#pragma unroll
                        for (int m = 0; m < 5; ++m) sv[m] = st[m][0][v];
                        lin5_2g<T, true>(sv, ih, gv, gx);
#pragma unroll
                        for (int ig = 0; ig < 2; ++ig) { out[ig][0][v] = gv[ig]; out[ig][3][v] = gx[ig]; }
#pragma unroll
                        for (int q = 1; q < 3; ++q) {
#pragma unroll
                            for (int m = 0; m < 5; ++m) sv[m] = st[m][q][v];
                            lin5_2g<T, false>(sv, ih, gv, gx);
                            out[0][q][v] = gv[0];
                            out[1][q][v] = gv[1];
                        }
                    }
                    lin = lin5_ok<T>(out[0][0], st[1][0], st[2][0], st[3][0], K) &&
                          lin5_ok<T>(out[1][0], st[1][0], st[2][0], st[3][0], K);
                    if (!lin) atomicAdd(gt.fallback, 1ull);
                }
            }
            if (!lin) sweep_side<T, 3>(st, ih, g, out);
#pragma unroll
            for (int ip = 0; ip < 2; ++ip) {
                reduce = reduce || reduce5<T>(out[ip][0], K);
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int v = 0; v < 5; ++v) PT(ip, side, q, v) = out[ip][q][v];
            }
        }
        if (reduce) {  // rare: both points take the line values with zero slope along c
            const size_t l = d.lv.idx(a, b, c + 2);
            for (int side = 0; side < 2; ++side)
                for (int ip = 0; ip < 2; ++ip) {
                    for (int q = 0; q < 3; ++q)
                        for (int v = 0; v < 5; ++v) PT(ip, side, q, v) = LV[(((ig * 2 + side) * 3 + q) * 5 + v) * nlv + l];
                    for (int v = 0; v < 5; ++v) PT(ip, side, 3, v) = T(0);
                }
        }
#pragma unroll 1
        for (int ip = 0; ip < 2; ++ip) {
            T f[5], df[5];
            if constexpr (sizeof(T) == 4) {
                float Lp[4][5], Rp[4][5];
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        Lp[q][v] = PT(ip, 0, q, v);
                        Rp[q][v] = PT(ip, 1, q, v);
                    }
                gks3_lr(Lp[0], &Lp[1], Rp[0], &Rp[1], dt, g, f, df);
            } else {
                gks3<T>(pt_reg[ip][0][0], &pt_reg[ip][0][1], pt_reg[ip][1][0], &pt_reg[ip][1][1], dt, g, f, df);
            }
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                acc[v] += T(0.25) * f[v];
                acc[5 + v] += T(0.25) * df[v];
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 10; ++q) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], 1);
    if (valid && ig == 0) {
        const size_t f = d.fs.idx(a, b, c);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            if constexpr (sizeof(T) == 4) {
                // FP32: widened on the integer pipes, one FP64 operation per result (the FP64
                // pipe also runs conversions): X0 = 0.5 F + D / 8 (D / 8 exact), P0 = F + D / 6,
                // X1 = P0 + D / 3
                const float fq = float(acc[v]), dq = float(acc[5 + v]);
                if (stage == 0) {
                    const double fv = f32_to_f64(fq);
                    FS[v * nfs + f] = fma(0.5, fv, f32_to_f64(0.125f * dq));
                    FS[(5 + v) * nfs + f] = fma(1.0 / 6.0, f32_to_f64(dq), fv);
                } else {
                    FS[v * nfs + f] = fma(1.0 / 3.0, f32_to_f64(dq), FS[(5 + v) * nfs + f]);
                }
            } else {
                const double fv = (double)acc[v], dv = (double)acc[5 + v];
                if (stage == 0) {
                    FS[v * nfs + f] = 0.0 + (0.5 * fv + (1.0 / 8.0) * dv);
                    FS[(5 + v) * nfs + f] = 0.0 + (1.0 * fv + (1.0 / 6.0) * dv);
                } else {
                    FS[v * nfs + f] = FS[(5 + v) * nfs + f] + (0.0 * fv + (1.0 / 3.0) * dv);
                }
            }
        }
    }
}

}  // namespace d3
}  // namespace hos
