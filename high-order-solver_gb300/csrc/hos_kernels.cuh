// hos_kernels.cuh -- CUDA kernels of one S2O4 step on a uniform 2D block (sm_103a).
//
// Data layout in HBM (all FP64 regardless of the compute type T):
//   W[4][nx*ny]        conserved variables, SoA planes, cell (i, j) at i*ny + j (the
//                      reference's Fluid2d order, include/fluid_mesh.h:125-160), ghosts included
//   Wold[4][nx*ny]     state at the start of the step (CopyFluid_new_to_old)
//   AX, AY[nx*ny]      DF indicators alpha_x, alpha_y per cell (ghost entries stay 0)
//   FX[4][nfx], FP[4][nfx], FAX[nfx]   x-face stage flux, stage-0 partial, face alpha
//   FY[4][nfy], ...                     same for y-faces; faces indexed over the interior:
//                      x-face (I, J), I in [0, nodex], J in [0, nodey): I*nodey + J
//                      y-face (I, J), I in [0, nodex), J in [0, nodey]: I*(nodey+1) + J
//   ctl                dt, t, CFL accumulator (bits of a positive double), status word
//   W32[6][nx*P]       FP32 solvers: FP32 mirror of W0..W3, alpha_x, alpha_y, rows padded to
//                      the pitch P = mirror_pitch(ny) (hos_tma.cuh); the FP32 face kernels
//                      stage their tiles from it with TMA tile loads
//
// One stage = bc_fill -> face_kernel<x> -> face_kernel<y> -> update_kernel.  The face
// kernel fuses, for a tile of faces, the normal line reconstruction (staged in shared
// memory), the tangential Gauss-point reconstruction (shared memory), the GKS flux per
// Gauss point and the Gauss-weighted stage combination, so reconstructed interface states
// never travel to HBM.
#pragma once
#include <cstdint>
#include <type_traits>
#include "hos_gks.cuh"
#include "hos_tma.cuh"

namespace hos {

struct StepCtl {
    double dt;           // time step of the current step
    double t;            // simulation time at the end of the current step
    unsigned long long cfl_bits;  // running min of CFL candidates (positive doubles as bits)
    unsigned int status; // bit 0: negative density/pressure or NaN (reference would exit);
                         // WAIT_TIMEOUT_BIT: a TMA tile load or a tensor-core MMA did not
                         // complete within its wait limit
    unsigned int active; // 0 once t >= tstop: the step's kernels return without work
    double tbeg;         // simulation time at the start of the current step (Block2d::t)
};

struct Geometry {
    int nx, ny, g, nodex, nodey;
    double dx, dy, cfl;
    double gamma, K, c1, c2;
    int characteristic;
    int integrator = 0;   // HOS_INT_*: S2O4, S1O1, S1O2, RK2, RK3, RK4
    int flux = 0;         // HOS_FLUX_*: GKS2D, LF2D
    int first_order = 0;  // 1: first-order reconstruction (First_order_normal / _tangent)
    // 1: the non-DF WENO5-AO scheme (WENO5_AO_normal / WENO5_AO_tangent, is_using_df_factor
    // false): the DF indicators are neither read nor updated; wenotype picks its weights
    int plain = 0;
    int wenotype = 0;
    int source = 0;       // 1: Update_with_source (gravity along +y; S2O4 stage 0 alone updates)
    // Navier-Stokes collision time (tau_type 1): Mu, Nu; Prandtl fix factor 1/Pr - 1 (0: off)
    int tau_type = 0;
    double mu = -1.0, nu = -1.0, prandtl_coef = 0.0;
    double prandtl = 1.0;   // Pr of LF2D's viscous term (NS_by_central_difference_prim_2D)
    // learned gate: the a-posteriori check widens the three central cells' range by this
    // fraction of it (density and total energy of a linear reconstruction)
    float gate_slack = 0.1f;
    int stages = 2;
    // 1 (the single-problem FP32 solvers): under plain S2O4 the face kernels store the stage-
    // combined fluxes per unit cell width -- the FP32 quadrature sums times the inverse normal
    // spacing, in FP32 -- and the update (update_kernel_scaled) sums them without FP64 products
    int scaled_flux = 0;
    // 1 / dx, 1 / dy, set on the host by set_spacing(): a double division costs the FP64 pipe
    // about ten instructions per thread
    double idx = 0.0, idy = 0.0;
    __host__ void set_spacing(double dx_, double dy_) {
        dx = dx_;
        dy = dy_;
        idx = 1.0 / dx_;
        idy = 1.0 / dy_;
    }
};

// Stages per step and Block2d::timecoefficient[s][k][f or derf] of each time-marching method
// (S1O1_2D ... RK4_2D, src/time_advance.cpp:197-247).  RK3 combines states instead
// (Update_with_gauss_RK3, :476-532): its flux weights per stage are 1, 1/4, 2/3.
__host__ __device__ constexpr int integrator_stages(int integrator) {
    return integrator == 1 || integrator == 2 ? 1 : integrator == 4 ? 3 : integrator == 5 ? 4 : 2;
}
__device__ __forceinline__ double time_coefficient(int integrator, int s, int k, int j) {
    switch (integrator) {
        case 0:   // S2O4
            if (s == 0) return k == 0 ? (j == 0 ? 0.5 : 1.0 / 8.0) : 0.0;
            return k == 0 ? (j == 0 ? 1.0 : 1.0 / 6.0) : (j == 0 ? 0.0 : 1.0 / 3.0);
        case 1:   // S1O1
            return s == 0 && k == 0 && j == 0 ? 1.0 : 0.0;
        case 2:   // S1O2
            return s == 0 && k == 0 ? (j == 0 ? 1.0 : 0.5) : 0.0;
        case 3:   // RK2
            if (j) return 0.0;
            return s == 0 ? (k == 0 ? 1.0 : 0.0) : 0.5;
        case 4:   // RK3: flux weight of the stage itself
            if (j || k != s) return 0.0;
            return s == 0 ? 1.0 : s == 1 ? 0.25 : 2.0 / 3.0;
        default:  // RK4
            if (j) return 0.0;
            if (s < 3) return k == s ? (s == 2 ? 1.0 : 0.5) : 0.0;
            return k == 0 || k == 3 ? 1.0 / 6.0 : 1.0 / 3.0;
    }
}

// ------------------------------------------------------------------------------------------
// ghost-cell fill: a single gather equal to the reference's sequential left, right, down, up
// sweeps (src/boundary_condition.cpp:66-186, 244-258, 367-442): every ghost value comes from
// an interior cell (or an inflow state) with the x-side rule applied first, then the y-side.
// ------------------------------------------------------------------------------------------
struct BcSpec {
    int kind[4];          // left, right, down, up
    double inflow[4][4];  // conserved inflow state per side
    // wedge boundaries: x of the wall start, x of the top shock trace at t = 0 and its speed,
    // cell-centre x of cell i = left + (i + 0.5 - ghost) dx, post/pre-shock conserved states
    double wx0, wthr0, wspeed, left, dx;
    double wpost[4], wpre[4];
    double wall[4][2];    // no-slip walls (HOS_BC_NOSLIP): wall velocity per side
};

__device__ __forceinline__ int bc_map(int idx, int n_tot, int g, int node, int kind, bool low) {
    if (kind == 0) return low ? g : n_tot - g - 1;                       // free: nearest interior
    if (kind == 1) return low ? idx + node : idx - node;                 // periodic
    return low ? 2 * g - 1 - idx : 2 * n_tot - 2 * g - 1 - idx;          // reflective / no-slip
}

// arguments of the cell update kernel (defined in hos_solver.cu)
struct UpdateArgs {
    double* W;
    double* Wold;
    double* AX;
    double* AY;
    const double* FXx;  // x-face stage flux [4][nfx]
    const double* FXy;  // y-face stage flux [4][nfy]
    const double* FAx;
    const double* FAy;
    StepCtl* ctl;
    int stage;
    float* W32;   // FP32 solvers: mirror of W (planes 0-3) and of alpha_x | alpha_y (planes
    float* A32;   // 4-5, A32 = W32 + 4 * nx * P), pitch P = mirror_pitch(ny); may be null
};

// step kernels defined in hos_solver.cu
__global__ void bc_fill_kernel(double* __restrict__ W, Geometry geo, BcSpec bc, const StepCtl* ctl, int skip_inactive,
                               float* W32 = nullptr);
__global__ void __launch_bounds__(256) update_kernel(UpdateArgs a, Geometry geo);

// ------------------------------------------------------------------------------------------
// face kernel
// ------------------------------------------------------------------------------------------
struct FaceArgs {
    const double* W;
    const double* AN;   // DF alpha of the normal direction (alpha_x for x-faces)
    const double* AT;   // DF alpha of the tangential direction
    double* FX;         // stage flux combination [4][nf]
    double* FP;         // stage-0 partial kept for stage 1 [4][nf]
    double* FA;         // face DF indicator [nf]
    const StepCtl* ctl;
    int stage;
    // learned gate (FP32 path only): per-cell flags, bit 0 x-smooth, bit 1 y-smooth, bits 2 / 3
    // x / y audited and found not smooth; counter of linear results the a-posteriori check
    // rejected
    const unsigned char* gate;
    unsigned long long* fallback;
    // time-marching methods other than S2O4: Gauss-integrated flux and its time derivative of
    // every earlier stage [stage][4][nf]
    double* FS;
    double* DS;
    // FP32 solvers: FP32 mirrors of the state and of the DF indicators (pitch mirror_pitch(ny)),
    // read by the FP32 tiles instead of converting the FP64 arrays (null: convert)
    const float* W32;
    const float* AN32;
    const float* AT32;
    // gated: counters of the linear reconstructions in audited not-smooth cell-directions, tried
    // and accepted by the a-posteriori check (null: not counted)
    unsigned long long* fn_check = nullptr;
};

// A tile is TN faces along the normal by TT along the tangent, handled by one CTA of 256
// threads: 128 faces (one thread per face side in the tangential phase) or 256 faces (two).
constexpr int FACE_THREADS = 256;
template <int TN_, int TT_> struct TileShape {
    static constexpr int N = TN_, T = TT_;
    static_assert((2 * TN_ * TT_) % FACE_THREADS == 0, "a tile has 128 or 256 faces");
};
using DefaultTile = TileShape<8, 16>;
constexpr int TILE_N = DefaultTile::N;    // default tile: 8 faces along the normal
constexpr int TILE_T = DefaultTile::T;    // by 16 along the tangent

template <int ORDER> struct GaussCount { static constexpr int GP = ORDER == 5 ? 2 : ORDER == 7 ? 3 : 4; };

template <class T, int ORDER, class TS = DefaultTile>
struct FaceSmem {
    static constexpr int TILE_N = TS::N, TILE_T = TS::T;
    static constexpr int r = ORDER / 2;
    static constexpr int GP = GaussCount<ORDER>::GP;
    static constexpr int TL = TILE_T + 2 * r;                      // line states along t
    // line states: for face row fn, entry pair qp (values 0-3, normal slopes 4-7, two per pair),
    // tangential cell tl and side: [fn][qp][tl][side][2], so that the tangential pass, whose
    // consecutive threads take consecutive (tl, side), reads consecutive pairs
    static constexpr int LINES = TILE_N * TL * 2 * 8;
    static constexpr int GSTATES = TILE_N * TILE_T * 2 * GP * 12;  // [face][side][gp][12]
    static constexpr int FLUX = TILE_N * TILE_T * GP * 9;          // [face][gp][f4 d4 alpha]
    static constexpr int UNION = LINES > FLUX ? LINES : FLUX;
    // phase-1 input tile: cells n in [g+N0-1-r, g+N0+TILE_N-1+r], t as the line states
    static constexpr int TN = TILE_N + 1 + 2 * r;
    static constexpr int WTILE = 5 * TN * TL;                      // W[4] + normal alpha, aliases GSTATES
    static constexpr int ATILE = (TILE_N + 1) * TL;                // tangential alpha of the face cells
    static_assert(WTILE <= GSTATES, "input tile must fit the Gauss-state region");
    static constexpr int GFLAGS = ((TILE_N + 1) * TL + (int)sizeof(T) - 1) / (int)sizeof(T);  // gate flag bytes
    static constexpr size_t bytes = sizeof(T) * (size_t)(UNION + GSTATES + ATILE);
    static constexpr size_t gated_bytes = bytes + sizeof(T) * (size_t)GFLAGS;
};

// TMA box of one FP32 face tile in the pitched mirror: x runs along j, y along i, z over the
// six planes.  x faces: rows are the TN normal cells, x covers the TL tangential cells; y faces:
// rows are the TL tangential cells, x covers the TN normal cells.  The x origin is rounded
// down to 4 floats (a TMA box must start on a 16-byte boundary), so x takes up to 3 more
// cells, rounded up to a multiple of 4.  The box is staged in the line-state region, which is
// free until phase 1 writes it.
template <int ORDER, int DIR, class TS = DefaultTile>
struct TmaBox {
    using S = FaceSmem<float, ORDER, TS>;
    static constexpr int X = ((DIR == 0 ? S::TL : S::TN) + 3 + 3) / 4 * 4;
    static constexpr int Y = DIR == 0 ? S::TN : S::TL;
    static constexpr int Z = MIRROR_PLANES;
    static constexpr unsigned bytes = 4u * X * Y * Z;
    static_assert(X * Y * Z <= S::UNION, "the staged box must fit the line-state region");
    static_assert(X <= 256 && Y <= 256, "TMA box extents are at most 256");
};

// Gauss weights of gausspoint 2 / 3 / 4 (SetGuassPoint, src/fluid_mesh.cpp:20-44)
template <int GP>
__device__ __forceinline__ double gauss_weight(int ig) {
    if (GP == 2) return 0.5;
    if (GP == 3) return ig == 0 ? 4.0 / 9.0 : 0.5 - 0.5 * (4.0 / 9.0);
    return ig < 2 ? 1.0 / 12.0 : 5.0 / 12.0;
}

// DF indicator contribution of one Gauss point (Calculate_alpha_k, src/reconstruction.cpp:1463-1476);
// y-face states are rotated back (XchangetoY) so the two Mach terms add in the reference order.
template <class T, int DIR>
__device__ __forceinline__ T alpha_k(const T* wl, const T* wr, T gamma) {
    T pl[4], pr[4];
    to_prim(pl, wl, gamma);
    to_prim(pr, wr, gamma);
    const T cl = sqrt(gamma * pl[3] / pl[0]);
    const T cr = sqrt(gamma * pr[3] / pr[0]);
    const T dn = pl[1] / cl - pr[1] / cr;
    const T dtg = pl[2] / cl - pr[2] / cr;
    T A = fabsT(pl[3] - pr[3]) / pl[3] + fabsT(pl[3] - pr[3]) / pr[3];
    if (DIR == 0) A = A + dn * dn + dtg * dtg;
    else A = A + dtg * dtg + dn * dn;
    return A;
}

// A-posteriori check of a linear (gated) reconstruction: density and total energy of each
// reconstructed state stay within the range of the three central stencil entries widened by
// slack times that range (a tenth unless set), and the state keeps a positive temperature.
template <class T, class A, class B, class C>
__device__ __forceinline__ bool linear_ok(const T* q, const A& wm, const B& w0, const C& wp, T K, T slack = T(0.1)) {
    if (needs_order_reduction(q, K)) return false;
#pragma unroll
    for (int v = 0; v < 4; v += 3) {
        const T lo = fminT(fminT(wm[v], w0[v]), wp[v]), hi = fmaxT(fmaxT(wm[v], w0[v]), wp[v]);
        const T m = slack * (hi - lo) + T(1e-6) * fabsT(w0[v]);
        if (!(q[v] >= lo - m && q[v] <= hi + m)) return false;
    }
    return true;
}

// One entry (line cell, side) of the line states: element q (0-3 values, 4-7 normal slopes) at
// base[(q / 2) * stride + q % 2]
template <class T>
struct LineRef {
    const T* base;
    int stride;
    __device__ __forceinline__ T operator[](int q) const { return base[(q >> 1) * stride + (q & 1)]; }
    __device__ __forceinline__ const T* pair(int qp) const { return base + qp * stride; }
};

// One tile of faces: N0, T0 are the first face indices along the normal and the tangent.
// GATED (FP32 only): cells the learned gate marks smooth reconstruct with the full-stencil
// polynomial alone; see hos_gate.cuh.
// PLAIN (ORDER 5 only): the non-DF WENO5-AO of the drivers' default slots (WENO5_AO,
// src/reconstruction.cpp:1589-1699, and WENO5_AO_tangential, :2244-2391) in place of the DF
// variant, with the wenotype weights of geo.wenotype.
// TMA (FP32 with the pitched mirror): phase 0 stages the tile from the mirror with one TMA
// tile load (tmap: the mirror's tensor map with this tile shape's box).
template <class T, int ORDER, int DIR, class TS, bool GATED = false, bool NS = false, bool TMA = false,
          bool PLAIN = false>
__device__ __forceinline__ void face_tile(const FaceArgs& a, const Geometry& geo, const int N0, const int T0,
                                          unsigned char* smem_raw, const CUtensorMap* tmap = nullptr) {
    static_assert(!TMA || sizeof(T) == 4, "TMA staging reads the FP32 mirror");
    static_assert(!PLAIN || (ORDER == 5 && !GATED), "the non-DF scheme is WENO5-AO, without the gate");
    using S = FaceSmem<T, ORDER, TS>;
    constexpr int TILE_N = TS::N, TILE_T = TS::T;
    constexpr int r = S::r, N = ORDER, GP = S::GP, TL = S::TL;
    constexpr int NW = AO<ORDER>::N;
    T* lines = reinterpret_cast<T*>(smem_raw);           // phase 1-2
    T* flux = lines;                                     // phase 3-4 (aliases lines)
    T* gst = lines + S::UNION;                           // phase 2-3
    T* wtile = gst;                                      // phase 0-1 (aliases gst)
    T* antile = gst + 4 * S::TN * TL;                    // phase 0-1
    T* attile = gst + S::GSTATES;                        // phase 0-2
    unsigned char* gfl = reinterpret_cast<unsigned char*>(attile + S::ATILE);  // phase 0-2 (GATED)

    const int nx = geo.nx, ny = geo.ny, g = geo.g;
    const int nodeN = DIR == 0 ? geo.nodex : geo.nodey;  // faces along normal: nodeN + 1
    const int nodeT = DIR == 0 ? geo.nodey : geo.nodex;  // faces along tangent: nodeT
    const size_t plane = (size_t)nx * ny;
    const int tid = threadIdx.x;
    if (!a.ctl->active) return;
    __shared__ unsigned rejected;   // GATED: linear results the check rejected in this tile
    // GATED: linear reconstructions in cell-directions the gate's audit found not smooth, tried
    // and accepted by the check
    __shared__ unsigned fn_seen[2];
    if constexpr (GATED)
        if (tid == 0) {
            rejected = 0;
            fn_seen[0] = fn_seen[1] = 0;
        }
    // FP32: the launch's FP64 parameters narrowed once per tile (a conversion from FP64 runs on
    // GB300's narrow FP64 pipe; per thread they would cost as much as the stage combination)
    __shared__ float fpar[7];
    if constexpr (sizeof(T) == 4) {
        if (tid == 0) {
            fpar[0] = float(DIR == 0 ? geo.idx : geo.idy);
            fpar[1] = float(DIR == 0 ? geo.idy : geo.idx);
            fpar[2] = float(geo.gamma);
            fpar[3] = float(geo.K);
            fpar[4] = float(a.ctl->dt);
            fpar[5] = float(geo.c1);
            fpar[6] = float(geo.c2);
        }
    }
    auto cidx = [&](int n, int t) -> size_t {
        return DIR == 0 ? (size_t)n * ny + t : (size_t)t * ny + n;
    };

    // ---------------- phase 0: stage the tile's cells once, converted to T ----------------
    // cells n in [g+N0-1-r, g+N0+TILE_N-1+r] (the normal stencils), t in [g+T0-r, g+T0+TILE_T+r);
    // y-face states are rotated into the x-face frame here (YchangetoX: (u, v) -> (v, -u)).
    if constexpr (TMA) {
        // one TMA tile load of W0..W3, alpha_x, alpha_y with the stencil halo into the line-state
        // region, then the same rotation / split into the tile arrays from shared memory
        using B = TmaBox<ORDER, DIR, TS>;
        constexpr int PZ = B::X * B::Y;   // floats per staged plane
        __shared__ __align__(8) uint64_t tma_bar;
        float* stg = reinterpret_cast<float*>(smem_raw);
        const int x0 = DIR == 0 ? g + T0 - r : g + N0 - 1 - r;   // j of the first staged cell
        const int y0 = DIR == 0 ? g + N0 - 1 - r : g + T0 - r;   // i of the first staged row
        const int xa = x0 & ~3, off = x0 - xa;                    // 16-byte aligned box origin
        const bool aligned = (smem_u32(stg) & 127u) == 0;
        if (tid == 0 && aligned) {
            mbar_init(&tma_bar, 1);
            mbar_expect_tx(&tma_bar, B::bytes);
            tma_load_3d(stg, tmap, xa, y0, 0, &tma_bar);
        }
        const int nmax = DIR == 0 ? nx : ny, tmax = DIR == 0 ? ny : nx;
        // GATED: the face cells' gate flags, loaded before the wait so that their latency overlaps
        // the tile load's; consecutive threads take consecutive cells of a row (coalesced)
        constexpr int NGF = (TILE_N + 1) * TL, GFL_PER = (NGF + FACE_THREADS - 1) / FACE_THREADS;
        unsigned char gpre[GATED ? GFL_PER : 1];
        if constexpr (GATED) {
#pragma unroll
            for (int k = 0; k < GFL_PER; ++k) {
                const int c = tid + k * FACE_THREADS;
                const int fnn = DIR == 0 ? c / TL : c % (TILE_N + 1), tl = DIR == 0 ? c % TL : c / (TILE_N + 1);
                const int n = g + N0 - 1 + fnn, t = g + T0 - r + tl;
                gpre[k] = c < NGF && n < nmax && t < tmax ? a.gate[cidx(n, t)] : (unsigned char)0;
            }
        }
        __syncthreads();   // the barrier is initialised before any thread polls it
        const bool ok = __syncthreads_and(aligned && mbar_wait(&tma_bar, 0));
        if (!ok) {
            // record the failure, let a load still in flight land, and leave the tile
            if (tid == 0) atomicOr(const_cast<unsigned*>(&a.ctl->status), WAIT_TIMEOUT_BIT);
            if (aligned) mbar_wait(&tma_bar, 0);
            return;
        }
        if constexpr (GATED) {
#pragma unroll
            for (int k = 0; k < GFL_PER; ++k) {
                const int c = tid + k * FACE_THREADS;
                const int fnn = DIR == 0 ? c / TL : c % (TILE_N + 1), tl = DIR == 0 ? c % TL : c / (TILE_N + 1);
                if (c < NGF) gfl[fnn * TL + tl] = gpre[k];
            }
        }
        for (int c = tid; c < S::TN * TL; c += FACE_THREADS) {
            const int nn = c / TL, tl = c % TL;
            const int n = g + N0 - 1 - r + nn, t = g + T0 - r + tl;
            if (n >= nmax || t >= tmax) continue;
            const float* q = stg + (DIR == 0 ? nn * B::X + off + tl : tl * B::X + off + nn);
            T* d = wtile + (nn * TL + tl) * 4;
            if (DIR == 0) { d[0] = q[0]; d[1] = q[PZ]; d[2] = q[2 * PZ]; d[3] = q[3 * PZ]; }
            else { d[0] = q[0]; d[1] = q[2 * PZ]; d[2] = -q[PZ]; d[3] = q[3 * PZ]; }
            antile[nn * TL + tl] = q[(DIR == 0 ? 4 : 5) * PZ];
            if (nn >= r && nn <= r + TILE_N) attile[(nn - r) * TL + tl] = q[(DIR == 0 ? 5 : 4) * PZ];
        }
    } else {
        const int nmax = DIR == 0 ? nx : ny, tmax = DIR == 0 ? ny : nx;
        const size_t pitch = (size_t)mirror_pitch(ny), plane32 = (size_t)nx * pitch;
        for (int c = tid; c < S::TN * TL; c += FACE_THREADS) {
            // x faces: t (= j) runs fastest; y faces: n (= j) runs fastest -- coalesced rows
            const int nn = DIR == 0 ? c / TL : c % S::TN;
            const int tl = DIR == 0 ? c % TL : c / S::TN;
            const int n = g + N0 - 1 - r + nn, t = g + T0 - r + tl;
            if (n >= nmax || t >= tmax) continue;
            const size_t ci = cidx(n, t);
            T w0, w1, w2, w3, an, at;
            bool mirrored = false;
            if constexpr (sizeof(T) == 4) {
                if (a.W32) {
                    const size_t cm = DIR == 0 ? (size_t)n * pitch + t : (size_t)t * pitch + n;
                    w0 = a.W32[cm]; w1 = a.W32[plane32 + cm]; w2 = a.W32[2 * plane32 + cm]; w3 = a.W32[3 * plane32 + cm];
                    an = a.AN32[cm];
                    at = a.AT32[cm];
                    mirrored = true;
                }
            }
            if (!mirrored) {
                w0 = T(a.W[ci]); w1 = T(a.W[plane + ci]); w2 = T(a.W[2 * plane + ci]); w3 = T(a.W[3 * plane + ci]);
                an = T(a.AN[ci]);
                at = T(a.AT[ci]);
            }
            T* d = wtile + (nn * TL + tl) * 4;
            if (DIR == 0) { d[0] = w0; d[1] = w1; d[2] = w2; d[3] = w3; }
            else { d[0] = w0; d[1] = w2; d[2] = -w1; d[3] = w3; }
            antile[nn * TL + tl] = an;
            if (nn >= r && nn <= r + TILE_N) {
                attile[(nn - r) * TL + tl] = at;
                if constexpr (GATED) gfl[(nn - r) * TL + tl] = a.gate[ci];
            }
        }
    }
    __syncthreads();   // also publishes fpar
    const T hN = sizeof(T) == 4 ? T(fpar[0]) : T(DIR == 0 ? geo.idx : geo.idy);   // inverse normal spacing
    const T hT = sizeof(T) == 4 ? T(fpar[1]) : T(DIR == 0 ? geo.idy : geo.idx);   // inverse face length
    const T gamma = sizeof(T) == 4 ? T(fpar[2]) : T(geo.gamma);
    const T K = sizeof(T) == 4 ? T(fpar[3]) : T(geo.K);

    // ---------------- phase 1: normal reconstruction of the tile's cells ----------------
    // cells n in [g+N0-1, g+N0+TILE_N), t in [g+T0-r, g+T0+TILE_T+r)
    for (int c = tid; c < (TILE_N + 1) * TL; c += FACE_THREADS) {
        const int nl = c / TL, tl = c % TL;
        const int n = g + N0 - 1 + nl;
        const int t = g + T0 - r + tl;
        const int tmax = DIR == 0 ? ny : nx;
        if (n > g + nodeN || t >= tmax) continue;
        T st[N][4], al[N];
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const T* q = wtile + ((nl + k) * TL + tl) * 4;
#pragma unroll
            for (int v = 0; v < 4; ++v) st[k][v] = q[v];
            al[k] = antile[(nl + k) * TL + tl];
        }
        T outv[2][8];
        bool lin = false;
        if (geo.first_order) {
            // First_order_normal (src/reconstruction.cpp:1537-1560): the cell average in the
            // face frame, zero slope, on both faces
#pragma unroll
            for (int side = 0; side < 2; ++side)
#pragma unroll
                for (int v = 0; v < 4; ++v) { outv[side][v] = st[r][v]; outv[side][4 + v] = T(0.0); }
            lin = true;
        }
        if constexpr (GATED) if (!lin && ((gfl[nl * TL + tl] >> DIR) & 1)) {
            // predicted smooth: the linear weights select the full-stencil polynomial, and a
            // linear reconstruction commutes with the characteristic projection; two variables
            // per paired FP32 operation
            using C = lin::Normal<ORDER>;
            const T dfl = df_full<T, ORDER>(al);
            const F2 dft(dfl), dfi(dfl * hN);
#pragma unroll
            for (int vp = 0; vp < 2; ++vp) {
                F2 s2[N];
#pragma unroll
                for (int k = 0; k < N; ++k) s2[k] = F2(st[k][2 * vp], st[k][2 * vp + 1]);
#pragma unroll
                for (int side = 0; side < 2; ++side) {
                    const F2 val = lin_value<F2, N, C>(side, s2, dft);
                    const F2 der = lin_slope<F2, N, C>(side, s2, dfi);
                    outv[side][2 * vp] = val.v.x;
                    outv[side][2 * vp + 1] = val.v.y;
                    outv[side][4 + 2 * vp] = der.v.x;
                    outv[side][5 + 2 * vp] = der.v.y;
                }
            }
            const T slack = T(geo.gate_slack);
            lin = linear_ok<T>(outv[0], st[r - 1], st[r], st[r + 1], K, slack) &&
                  linear_ok<T>(outv[1], st[r - 1], st[r], st[r + 1], K, slack);
            if (!lin) atomicAdd(&rejected, 1u);
            if ((gfl[nl * TL + tl] >> (2 + DIR)) & 1) {
                atomicAdd(&fn_seen[0], 1u);
                if (lin) atomicAdd(&fn_seen[1], 1u);
            }
        }
        // the DF factors and the characteristic bases' primitives, only for cells that take the
        // WENO-AO path
        T df[NW];
        if (!lin) {
            if constexpr (PLAIN) {
#pragma unroll
                for (int k = 0; k < NW; ++k) df[k] = T(1.0);
            } else {
                df_factors<T, ORDER>(al, df);
            }
        }
        T pn1[4], p0[4], pp1[4];
        if (!lin && geo.characteristic) {
            to_prim(pn1, st[r - 1], gamma);
            to_prim(p0, st[r], gamma);
            to_prim(pp1, st[r + 1], gamma);
        }
#pragma unroll
        for (int side = 0; side < 2 && !lin; ++side) {
            CharBase<T> cb;
            T ch[N][4];
            if (geo.characteristic) {
                T base[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) base[v] = T(0.5) * ((side == 0 ? pn1[v] : pp1[v]) + p0[v]);
                cb.init(base, gamma);
#pragma unroll
                for (int k = 0; k < N; ++k) cb.to_char(ch[k], st[k]);
            } else {
#pragma unroll
                for (int k = 0; k < N; ++k)
#pragma unroll
                    for (int v = 0; v < 4; ++v) ch[k][v] = st[k][v];
            }
            T var[4], der[4];
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                T s[N];
#pragma unroll
                for (int k = 0; k < N; ++k) s[k] = ch[k][v];
                if constexpr (PLAIN) {
                    // weno_5th_ao_left / _right (:161-360): epsilon 1e-10, full 5th-order indicator
                    weno5_face<T>(side, s, hN, var[v], der[v], geo.wenotype);
                } else {
                    T fw[NW], p[NW], px[NW];
                    ao_weights<T, ORDER>(s, fw);
                    if (side == 0) normal_face<T, ORDER, 0>(s, df, hN, p, px);
                    else normal_face<T, ORDER, 1>(s, df, hN, p, px);
                    T x = T(0.0), y = T(0.0);
#pragma unroll
                    for (int k = 0; k < NW; ++k) { x += fw[k] * p[k]; y += fw[k] * px[k]; }
                    var[v] = x;
                    der[v] = y;
                }
            }
            if (geo.characteristic) {
                cb.from_char(outv[side], var);
                cb.from_char(outv[side] + 4, der);
            } else {
#pragma unroll
                for (int v = 0; v < 4; ++v) { outv[side][v] = var[v]; outv[side][4 + v] = der[v]; }
            }
        }
        // positivity fallback couples the two faces of the cell (src/reconstruction.cpp:1843-1858);
        // a linear reconstruction the check accepted has passed it, and a first-order one is the
        // fallback's own result
        if (!lin && (needs_order_reduction(outv[1], K) || needs_order_reduction(outv[0], K))) {
#pragma unroll
            for (int side = 0; side < 2; ++side)
#pragma unroll
                for (int v = 0; v < 4; ++v) { outv[side][v] = st[r][v]; outv[side][4 + v] = T(0.0); }
        }
        // left-face value -> right side of face n; right-face value -> left side of face n+1
        const int fl = n - (g + N0);
        if (fl >= 0 && fl < TILE_N) {
            T* d = lines + ((fl * 4 * TL + tl) * 2 + 1) * 2;
#pragma unroll
            for (int q = 0; q < 8; ++q) d[(q >> 1) * 4 * TL + (q & 1)] = outv[0][q];
        }
        if (fl + 1 >= 0 && fl + 1 < TILE_N) {
            T* d = lines + (((fl + 1) * 4 * TL + tl) * 2 + 0) * 2;
#pragma unroll
            for (int q = 0; q < 8; ++q) d[(q >> 1) * 4 * TL + (q & 1)] = outv[1][q];
        }
    }
    __syncthreads();

    // ---------------- phase 2: tangential reconstruction, one (face, side) per thread and pass ----------------
#pragma unroll 1
    for (int item = tid; item < 2 * TILE_N * TILE_T; item += FACE_THREADS) {
        const int side = item & 1;
        const int fidx = item >> 1;                // face within the tile
        const int fn = fidx / TILE_T, ft = fidx % TILE_T;
        const int facen = N0 + fn, facet = T0 + ft;
        if (facen <= nodeN && facet < nodeT) {
            constexpr int sgn = DIR == 0 ? 1 : -1;  // y-face tangents run toward -x
            const int tc = ft + r;                  // centre line index in the tile
            T al[N];
#pragma unroll
            for (int k = 0; k < N; ++k) al[k] = attile[(fn + side) * TL + tc + sgn * (k - r)];
            auto line = [&](int k, int sd) -> LineRef<T> {
                return LineRef<T>{lines + ((fn * 4 * TL + (tc + sgn * (k - r))) * 2 + sd) * 2, 4 * TL};
            };
            const LineRef<T> w0 = line(r, side);
            T res[GP][12];
            bool lin = false;
            if (geo.first_order) {
                // First_order_tangent (:2214-2231): every Gauss point takes the line value and
                // its normal slope, zero tangential slope
#pragma unroll
                for (int ig = 0; ig < GP; ++ig)
#pragma unroll
                    for (int v = 0; v < 4; ++v) {
                        res[ig][v] = w0[v];
                        res[ig][4 + v] = w0[4 + v];
                        res[ig][8 + v] = T(0.0);
                    }
                lin = true;
            }
            if constexpr (GATED) if (!lin && ((gfl[(fn + side) * TL + tc] >> (1 - DIR)) & 1)) {
                // the side cell is smooth along the tangent: full-stencil polynomial at the
                // Gauss points, in conservative variables; two line entries per paired FP32
                // operation (values and normal slopes; tangential slopes of the values)
                using C = lin::Tangent<ORDER>;
                const T dfl = df_full<T, ORDER>(al);
                const F2 dft(dfl), dfi(dfl * hT);
#pragma unroll
                for (int vp = 0; vp < 4; ++vp) {
                    F2 s2[N];
#pragma unroll
                    for (int k = 0; k < N; ++k) s2[k] = F2(*reinterpret_cast<const float2*>(line(k, side).pair(vp)));
#pragma unroll
                    for (int ig = 0; ig < GP; ++ig) {
                        const F2 val = lin_value<F2, N, C>(ig, s2, dft);
                        res[ig][2 * vp] = val.v.x;
                        res[ig][2 * vp + 1] = val.v.y;
                        if (vp < 2) {
                            const F2 der = lin_slope<F2, N, C>(ig, s2, dfi);
                            res[ig][8 + 2 * vp] = der.v.x;
                            res[ig][9 + 2 * vp] = der.v.y;
                        }
                    }
                }
                lin = true;
#pragma unroll
                for (int ig = 0; ig < GP; ++ig)
                    lin = lin && linear_ok<T>(res[ig], line(r - 1, side), w0, line(r + 1, side), K, T(geo.gate_slack));
                if (!lin) atomicAdd(&rejected, 1u);
                if ((gfl[(fn + side) * TL + tc] >> (3 - DIR)) & 1) {
                    atomicAdd(&fn_seen[0], 1u);
                    if (lin) atomicAdd(&fn_seen[1], 1u);
                }
            }
            // the DF factors, only for faces that take the WENO-AO path
            T df[NW];
            if (!lin) {
                if constexpr (PLAIN) {
#pragma unroll
                    for (int k = 0; k < NW; ++k) df[k] = T(1.0);
                } else {
                    df_factors<T, ORDER>(al, df);
                }
            }
            if (lin) {
            } else if (geo.characteristic) {
                T base[4], w0c[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) w0c[v] = w0[v];
                to_prim(base, w0c, gamma);
                CharBase<T> cb;
                cb.init(base, gamma);
                T ch[N][4];
#pragma unroll
                for (int k = 0; k < N; ++k) {
                    T w[4];
#pragma unroll
                    for (int v = 0; v < 4; ++v) w[v] = line(k, side)[v];
                    cb.to_char(ch[k], w);
                }
                if (ORDER == 9 && side == 1) {
                    // the reference's right side keeps the left side's projection of the two
                    // outermost entries (src/reconstruction.cpp:3318-3327)
                    const LineRef<T> l0 = line(r, 0);
                    T b0[4], lw[4];
#pragma unroll
                    for (int v = 0; v < 4; ++v) lw[v] = l0[v];
                    to_prim(b0, lw, gamma);
                    CharBase<T> cl;
                    cl.init(b0, gamma);
                    T w[4];
#pragma unroll
                    for (int v = 0; v < 4; ++v) w[v] = line(0, 0)[v];
                    cl.to_char(ch[0], w);
#pragma unroll
                    for (int v = 0; v < 4; ++v) w[v] = line(N - 1, 0)[v];
                    cl.to_char(ch[N - 1], w);
                }
                T gv[GP][4], gd[GP][4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    T s[N], fw[NW];
#pragma unroll
                    for (int k = 0; k < N; ++k) s[k] = ch[k][v];
                    if constexpr (PLAIN) {
                        // weno_5th_ao_2gauss (:2393-2551): epsilon 1e-6, full 5th-order indicator
                        T g2[2], gx2[2];
                        weno5_2g<T, true>(s, hT, g2, gx2, geo.wenotype);
#pragma unroll
                        for (int ig = 0; ig < GP; ++ig) { gv[ig][v] = g2[ig]; gd[ig][v] = gx2[ig]; }
                        continue;
                    }
                    ao_weights<T, ORDER>(s, fw);
#pragma unroll
                    for (int ig = 0; ig < GP; ++ig) {
                        T p[NW], px[NW];
                        tangent_point<T, ORDER>(ig, s, df, hT, p, px);
                        T x = T(0.0), y = T(0.0);
#pragma unroll
                        for (int k = 0; k < NW; ++k) { x += fw[k] * p[k]; y += fw[k] * px[k]; }
                        gv[ig][v] = x;
                        gd[ig][v] = y;
                    }
                }
#pragma unroll
                for (int ig = 0; ig < GP; ++ig) {
                    cb.from_char(res[ig], gv[ig]);
                    cb.from_char(res[ig] + 8, gd[ig]);
                }
            } else {
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    T s[N], fw[NW];
#pragma unroll
                    for (int k = 0; k < N; ++k) s[k] = line(k, side)[v];
                    if constexpr (PLAIN) {
                        T g2[2], gx2[2];
                        weno5_2g<T, true>(s, hT, g2, gx2, geo.wenotype);
#pragma unroll
                        for (int ig = 0; ig < GP; ++ig) { res[ig][v] = g2[ig]; res[ig][8 + v] = gx2[ig]; }
                        continue;
                    }
                    ao_weights<T, ORDER>(s, fw);
#pragma unroll
                    for (int ig = 0; ig < GP; ++ig) {
                        T p[NW], px[NW];
                        tangent_point<T, ORDER>(ig, s, df, hT, p, px);
                        T x = T(0.0), y = T(0.0);
#pragma unroll
                        for (int k = 0; k < NW; ++k) { x += fw[k] * p[k]; y += fw[k] * px[k]; }
                        res[ig][v] = x;
                        res[ig][8 + v] = y;
                    }
                }
            }
            // normal slope, reconstructed in conservative variables
#pragma unroll
            for (int v = 0; v < 4 && !lin; ++v) {
                T s[N], fw[NW];
#pragma unroll
                for (int k = 0; k < N; ++k) s[k] = line(k, side)[4 + v];
                if constexpr (PLAIN) {
                    T g2[2], gx2[2];
                    weno5_2g<T, false>(s, hT, g2, gx2, geo.wenotype);
#pragma unroll
                    for (int ig = 0; ig < GP; ++ig) res[ig][4 + v] = g2[ig];
                    continue;
                }
                ao_weights<T, ORDER>(s, fw);
#pragma unroll
                for (int ig = 0; ig < GP; ++ig) {
                    T p[NW], px[NW];
                    tangent_point<T, ORDER>(ig, s, df, hT, p, px);
                    T x = T(0.0);
#pragma unroll
                    for (int k = 0; k < NW; ++k) x += fw[k] * p[k];
                    res[ig][4 + v] = x;
                }
            }
            // positivity fallback per Gauss point (src/reconstruction.cpp:2764-2791); not for a
            // linear or first-order result (checked, or the fallback's own values)
#pragma unroll
            for (int ig = 0; ig < GP; ++ig) {
                if (!lin && needs_order_reduction(res[ig], K)) {
#pragma unroll
                    for (int v = 0; v < 4; ++v) {
                        res[ig][v] = w0[v];
                        res[ig][4 + v] = w0[4 + v];
                        res[ig][8 + v] = T(0.0);
                    }
                }
                T* d = gst + ((fidx * 2 + side) * GP + ig) * 12;
#pragma unroll
                for (int q = 0; q < 12; ++q) d[q] = res[ig][q];
            }
        }
    }
    __syncthreads();

    if constexpr (GATED)
        if (tid == 0) {
            if (rejected) atomicAdd(a.fallback, (unsigned long long)rejected);
            if (fn_seen[0] && a.fn_check) {
                atomicAdd(a.fn_check, (unsigned long long)fn_seen[0]);
                atomicAdd(a.fn_check + 1, (unsigned long long)fn_seen[1]);
            }
        }

    // ---------------- phase 3: GKS flux, one (face, Gauss point) per thread ----------------
    const T dt = sizeof(T) == 4 ? T(fpar[4]) : T(a.ctl->dt);
    for (int item = tid; item < TILE_N * TILE_T * GP; item += FACE_THREADS) {
        const int fidx = item / GP, ig = item % GP;
        const int fn = fidx / TILE_T, ft = fidx % TILE_T;
        if (N0 + fn > nodeN || T0 + ft >= nodeT) continue;
        GState<T> L, R;
        const T* sl = gst + ((fidx * 2 + 0) * GP + ig) * 12;
        const T* sr = gst + ((fidx * 2 + 1) * GP + ig) * 12;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            L.w[v] = sl[v]; L.dx[v] = sl[4 + v]; L.dy[v] = sl[8 + v];
            R.w[v] = sr[v]; R.dx[v] = sr[4 + v]; R.dy[v] = sr[8 + v];
        }
        T f[4], d[4];
        float alk = 0.0f;   // FP32 GKS: the DF indicator contribution from its lanes
        bool alk_set = false;
        if (geo.flux == 1) {
            lf_point<T>(L.w, R.w, dt, gamma, f);
            // the Navier-Stokes instantiation adds LF2D's viscous term
            if constexpr (NS) lf_viscous<T>(L, R, dt, K, T(geo.mu), T(geo.nu), T(geo.prandtl), f);
#pragma unroll
            for (int v = 0; v < 4; ++v) d[v] = T(0.0);
        } else {
            // the Navier-Stokes form is a separate instantiation: the Euler kernels carry none
            // of its code
            if constexpr (NS)
                gks_point_ns<T>(L, R, dt, K, NsParam<T>{T(geo.c2), T(geo.mu), T(geo.nu), T(geo.prandtl_coef)}, f, d);
            else if constexpr (std::is_same<T, float>::value) {
                // FP32: the left and right states share the paired FP32 lanes, and the DF
                // indicator's contribution comes from the same lanes
                gks_point_lr(L, R, dt, K, fpar[5], fpar[6], f, d, gamma, DIR, &alk);
                alk_set = true;
            } else {
                gks_point<T>(L, R, dt, K, T(geo.c1), T(geo.c2), f, d);
            }
            if (geo.integrator == 1) {   // S1O1 takes the dt integral F0 = f + d / 2 alone
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    f[v] = f[v] + T(0.5) * d[v];
                    d[v] = T(0.0);
                }
            }
        }
        T* o = flux + (fidx * GP + ig) * 9;
#pragma unroll
        for (int v = 0; v < 4; ++v) { o[v] = f[v]; o[4 + v] = d[v]; }
        o[8] = alk_set ? alk : alpha_k<T, DIR>(L.w, R.w, gamma);
    }
    __syncthreads();

    // ---------------- phase 4: Gauss quadrature, S2O4 stage combination, face DF indicator ----------------
    // the FP64 stage combination and the face's global reads and writes, from its Gauss-quadrature
    // sums of f and f_t (in the compute type) and of the DF contributions.  stg: the S2O4 stage
    // as a compile-time constant (std::integral_constant) where the FP32 kernels run plain S2O4,
    // -1 where the stage and the time marching are read at run time.  With the stage fixed, the
    // other stage's FP64 operations are not compiled in: the compiler if-converts short uniform
    // branches, and an FP64 operation predicated off in every lane still takes its FP64-pipe slot.
    auto finish = [&](auto stg, int fn, int ft, const T* Fq, const T* Dq, T asum) {
        constexpr int SG = decltype(stg)::value;
        const int facen = N0 + fn, facet = T0 + ft;
        const size_t nf = DIR == 0 ? (size_t)(geo.nodex + 1) * geo.nodey : (size_t)geo.nodex * (geo.nodey + 1);
        const size_t fi = DIR == 0 ? (size_t)facen * geo.nodey + facet : (size_t)facet * (geo.nodey + 1) + facen;
        double X[4], P[4];
        const bool s2o4 = SG >= 0 || geo.integrator == 0;
        const bool st0 = SG >= 0 ? SG == 0 : a.stage == 0;
        // FP32 kernels, plain S2O4: the FP64 pipe bounds this phase, so the conversions run on
        // the integer pipes (f32_to_f64, exact) and each result takes one FP64 operation:
        // X0 = 0.5 F + D / 8 (D / 8 exact in FP32), P0 = F + D / 6, X1 = P0 + D / 3
        const bool fast64 = SG >= 0 || (sizeof(T) == 4 && s2o4 && !geo.source);
        const float sc = geo.scaled_flux ? float(hN) : 1.0f;
#pragma unroll
        for (int v = 0; v < 4 && fast64; ++v) {
            const float fq = float(Fq[v]) * sc, dq = float(Dq[v]) * sc;
            if (st0) {
                const double F = f32_to_f64(fq);
                X[v] = fma(0.5, F, f32_to_f64(0.125f * dq));
                P[v] = fma(1.0 / 6.0, f32_to_f64(dq), F);
            } else {
                X[v] = fma(1.0 / 3.0, f32_to_f64(dq), a.FP[v * nf + fi]);
                P[v] = 0.0;
            }
        }
#pragma unroll
        for (int v = 0; v < 4 && !fast64; ++v) {
            const double F = double(Fq[v]), D = double(Dq[v]);
            if (s2o4) {
                if (geo.source) {
                    // Update_with_source: the Gauss-weighted f of the stage itself
                    X[v] = F;
                    P[v] = 0.0;
                } else if (st0) {
                    X[v] = 0.5 * F + (1.0 / 8.0) * D;
                    P[v] = 1.0 * F + (1.0 / 6.0) * D;
                } else {
                    X[v] = (1.0 / 3.0) * D;
                    P[v] = 0.0;
                }
            } else {
                // X_s = sum over stages k <= s of c[s][k] (F_k, D_k) (Update, :378-428)
                const int sg = a.stage;
                double x = time_coefficient(geo.integrator, sg, sg, 0) * F +
                           time_coefficient(geo.integrator, sg, sg, 1) * D;
                for (int k = 0; k < sg; ++k)
                    x += time_coefficient(geo.integrator, sg, k, 0) * a.FS[((size_t)k * 4 + v) * nf + fi] +
                         time_coefficient(geo.integrator, sg, k, 1) * a.DS[((size_t)k * 4 + v) * nf + fi];
                X[v] = x;
                if (sg + 1 < geo.stages) {
                    a.FS[((size_t)sg * 4 + v) * nf + fi] = F;
                    a.DS[((size_t)sg * 4 + v) * nf + fi] = D;
                }
                P[v] = 0.0;
            }
        }
        // mean over Gauss points, zeroed below 2 (Calculate_alpha, :1497-1516)
        // FP64 divides as the reference does; the FP32 path takes the mean in FP32 (an
        // indicator, not part of the FP64 stage combination) instead of a double division
        if constexpr (sizeof(T) == 8) {
            const double as = double(asum);
            const double am = GP == 2 ? 0.5 * as : GP == 3 ? as / 3.0 : 0.25 * as;
            a.FA[fi] = am < 2.0 ? 0.0 : am;
        } else {
            const float am = float(GP == 2 ? T(0.5) * asum : GP == 3 ? asum * T(1.0 / 3.0) : T(0.25) * asum);
            a.FA[fi] = am < 2.0f ? 0.0 : f32_to_f64(am);
        }
        if (s2o4 && !st0 && !geo.source && !fast64) {
#pragma unroll
            for (int v = 0; v < 4; ++v) X[v] = a.FP[v * nf + fi] + X[v];
        }
        // y-face local (normal, tangential) momentum -> global (Local_to_Global, :1226-1233)
        double Xg[4] = {X[0], X[1], X[2], X[3]};
        if (DIR == 1) { Xg[1] = -X[2]; Xg[2] = X[1]; }
#pragma unroll
        for (int v = 0; v < 4; ++v) a.FX[v * nf + fi] = Xg[v];
        if (s2o4 && st0) {
#pragma unroll
            for (int v = 0; v < 4; ++v) a.FP[v * nf + fi] = P[v];
        }
    };
    auto phase4 = [&](auto stg) {
        // y faces lie along n in memory (fi = t (nodey + 1) + n) while the tile's threads run along t:
        // their sums are staged in the Gauss-state region (free after phase 3), [9][TILE_T][TILE_N + 1]
        // (the padding keeps both passes free of bank conflicts), and the combination runs with
        // consecutive threads on consecutive faces of memory, so its global accesses coalesce
        constexpr int SP = TILE_N + 1;
        T* qst = gst;
#pragma unroll 1
        for (int fidx = tid; fidx < TILE_N * TILE_T; fidx += FACE_THREADS) {
            const int fn = fidx / TILE_T, ft = fidx % TILE_T;
            if (N0 + fn > nodeN || T0 + ft >= nodeT) continue;
            // Gauss quadrature of f and f_t over the face in the compute type; the S2O4 stage
            // combination of the two time-integral moments is FP64
            T Fq[4], Dq[4], asum = T(0.0);
#pragma unroll
            for (int v = 0; v < 4; ++v) { Fq[v] = T(0.0); Dq[v] = T(0.0); }
#pragma unroll
            for (int ig = 0; ig < GP; ++ig) {
                const T* o = flux + (fidx * GP + ig) * 9;
                const T gw = T(gauss_weight<GP>(ig));
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    Fq[v] += gw * o[v];
                    Dq[v] += gw * o[4 + v];
                }
                asum += o[8];
            }
            if constexpr (DIR == 0) {
                finish(stg, fn, ft, Fq, Dq, asum);
            } else {
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    qst[(v * TILE_T + ft) * SP + fn] = Fq[v];
                    qst[((4 + v) * TILE_T + ft) * SP + fn] = Dq[v];
                }
                qst[(8 * TILE_T + ft) * SP + fn] = asum;
            }
        }
        if constexpr (DIR == 1) {
            static_assert(9 * TILE_T * (TILE_N + 1) <= S::GSTATES, "the staged sums must fit the Gauss-state region");
            __syncthreads();
#pragma unroll 1
            for (int fc = tid; fc < TILE_N * TILE_T; fc += FACE_THREADS) {
                const int fn = fc % TILE_N, ft = fc / TILE_N;
                if (N0 + fn > nodeN || T0 + ft >= nodeT) continue;
                T Fq[4], Dq[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    Fq[v] = qst[(v * TILE_T + ft) * SP + fn];
                    Dq[v] = qst[((4 + v) * TILE_T + ft) * SP + fn];
                }
                finish(stg, fn, ft, Fq, Dq, qst[(8 * TILE_T + ft) * SP + fn]);
            }
        }
    };
    // FP32 kernels, plain S2O4: phase 4 compiled once per stage (finish's stg)
    if constexpr (sizeof(T) == 4) {
        if (geo.integrator == 0 && !geo.source) {
            if (a.stage == 0)
                phase4(std::integral_constant<int, 0>{});
            else
                phase4(std::integral_constant<int, 1>{});
            return;
        }
    }
    phase4(std::integral_constant<int, -1>{});
}

// Tile of the single-problem face kernels: 16 x 16 faces for WENO5/7 (256 faces: every thread
// has the same number of (face, Gauss point) flux items; at WENO7 103 KB of shared memory in
// FP32, two CTAs per SM, and 206 KB in FP64, one), 8 x 16 for WENO9 (its four Gauss points would
// need 137 KB in FP32 at 16 x 16).
template <int ORDER>
using KernelTile = typename std::conditional<ORDER == 9, TileShape<8, 16>, TileShape<16, 16>>::type;
template <int ORDER>
using TmaTile = KernelTile<ORDER>;

template <class T, int ORDER, int DIR, bool GATED = false, bool NS = false, bool PLAIN = false>
__global__ void __launch_bounds__(FACE_THREADS, sizeof(T) == 4 ? 2 : 1) face_kernel(FaceArgs a, Geometry geo) {
    using TS = KernelTile<ORDER>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    face_tile<T, ORDER, DIR, TS, GATED, NS, false, PLAIN>(a, geo, blockIdx.y * TS::N, blockIdx.x * TS::T, smem_raw);
}

// FP32 face kernel of the solvers with the pitched FP32 mirror: the tile is staged by one TMA
// tile load (tmap: the mirror's tensor map, box TmaBox<ORDER, DIR, TmaTile<ORDER>>)
template <int ORDER, int DIR, bool GATED = false, bool NS = false, bool PLAIN = false>
__global__ void __launch_bounds__(FACE_THREADS, 2)
    face_kernel_tma(FaceArgs a, Geometry geo, const __grid_constant__ CUtensorMap tmap) {
    using TS = TmaTile<ORDER>;
    extern __shared__ __align__(128) unsigned char smem_tma[];
    face_tile<float, ORDER, DIR, TS, GATED, NS, true, PLAIN>(a, geo, blockIdx.y * TS::N, blockIdx.x * TS::T, smem_tma,
                                                            &tmap);
}

}  // namespace hos
