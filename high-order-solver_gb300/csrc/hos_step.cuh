// hos_step.cuh -- per-element device functions of the step kernels other than the face
// kernel: ghost-cell gather, cell update with the CFL / blow-up reduction, step prologue.
// Shared by the single-problem kernels (hos_solver.cu) and the batched kernels (hos_batch.cu).
#pragma once
#include "../../include/hos_gb300.h"
#include "hos_kernels.cuh"

namespace hos {

// ghost cell number e of the block (left/right strips first, then bottom/top strips)
__device__ __forceinline__ void bc_fill_one(double* __restrict__ W, const Geometry& geo, const BcSpec& bc,
                                            const StepCtl* ctl, long long e, float* __restrict__ W32 = nullptr) {
    const int nx = geo.nx, ny = geo.ny, g = geo.g;
    const long long nlr = 2LL * g * ny, ndu = 2LL * g * geo.nodex;
    if (e >= nlr + ndu) return;
    int i, j;
    if (e < nlr) {
        int il = (int)(e / ny);
        j = (int)(e % ny);
        i = il < g ? il : nx - 2 * g + il;
    } else {
        long long e2 = e - nlr;
        int jl = (int)(e2 / geo.nodex);
        i = g + (int)(e2 % geo.nodex);
        j = jl < g ? jl : ny - 2 * g + jl;
    }
    const size_t plane = (size_t)nx * ny;
    // the FP32 mirror of the state (FP32 solvers, pitch mirror_pitch(ny)) takes the same ghost
    // values, rounded
    const size_t pitch = (size_t)mirror_pitch(ny), plane32 = (size_t)nx * pitch;
    auto put = [&](int v, double x) {
        W[v * plane + (size_t)i * ny + j] = x;
        if (W32) W32[v * plane32 + (size_t)i * pitch + j] = (float)x;
    };
    double out[4];
    int si = i, sj = j;
    bool flipu = false, flipv = false;
    int wallx = -1, wally = -1;   // no-slip side applied on the x / y axis
    const bool yg = j < g || j >= ny - g;
    const bool xg = i < g || i >= nx - g;
    if (yg) {
        const int side = j < g ? 2 : 3;
        const int kind = bc.kind[side];
        if (kind == 3) {
            for (int v = 0; v < 4; ++v) put(v, bc.inflow[side][v]);
            return;
        }
        if (kind == 4 || kind == 5) {
            // wedge boundaries act on i >= ghost only; the left ghost columns keep the
            // left-side (inflow) value (src/2Dproblem.cpp:1045-1092)
            if (i >= g) {
                const double x = bc.left + (i + 0.5 - g) * bc.dx;
                const double* st = nullptr;
                if (kind == 5) {
                    const double tb = ctl ? ctl->tbeg : 0.0;
                    st = x < bc.wthr0 + bc.wspeed * tb ? bc.wpost : bc.wpre;
                } else if (x < bc.wx0) {
                    st = bc.wpost;
                }
                if (st) {
                    for (int v = 0; v < 4; ++v) put(v, st[v]);
                    return;
                }
                sj = 2 * g - 1 - j;  // reflecting wall
                flipv = true;
            }
        } else {
            sj = bc_map(j, ny, g, geo.nodey, kind, side == 2);
            flipv = kind == 2;
            if (kind == HOS_BC_NOSLIP) wally = side;
        }
    }
    if (xg) {
        const int side = i < g ? 0 : 1;
        const int kind = bc.kind[side];
        if (kind == 3) {
            for (int v = 0; v < 4; ++v) out[v] = bc.inflow[side][v];
            if (flipv) out[2] = -out[2];
            for (int v = 0; v < 4; ++v) put(v, out[v]);
            return;
        }
        si = bc_map(i, nx, g, geo.nodex, kind, side == 0);
        flipu = kind == 2;
        if (kind == HOS_BC_NOSLIP) wallx = side;
    }
    const size_t src = (size_t)si * ny + sj;
    for (int v = 0; v < 4; ++v) out[v] = W[v * plane + src];
    // the x sides' rule first, then the y sides' (the drivers fill left, right, down, up);
    // no-slip: 2 rho u_wall - rho u for both components (noslip_adiabatic_boundary_*,
    // src/boundary_condition.cpp:290-365)
    if (flipu) out[1] = -out[1];
    if (wallx >= 0) {
        out[1] = 2 * out[0] * bc.wall[wallx][0] - out[1];
        out[2] = 2 * out[0] * bc.wall[wallx][1] - out[2];
    }
    if (flipv) out[2] = -out[2];
    if (wally >= 0) {
        out[1] = 2 * out[0] * bc.wall[wally][0] - out[1];
        out[2] = 2 * out[0] * bc.wall[wally][1] - out[2];
    }
    for (int v = 0; v < 4; ++v) put(v, out[v]);
}


__device__ __forceinline__ void atomic_min_pos(unsigned long long* addr, double v) {
    // positive doubles order like their bit patterns
    atomicMin(addr, (unsigned long long)__double_as_longlong(v));
}

// the stage whose update produces the next step's CFL candidates
__host__ __device__ __forceinline__ int cfl_stage(const Geometry& geo) { return geo.stages >= 2 ? geo.stages - 2 : 0; }

// a cell's signal speed |u| + c for the CFL reduction; one that is not finite gives no candidate
// in Dtx (its dt is not > 0), as 0 does in cfl_of_speed (dt = inf)
__device__ __forceinline__ double signal_speed(double tmp) { return tmp <= 1.7976931348623157e308 ? tmp : 0.0; }

// update of interior cell idx; returns its signal speed |u| + c for the CFL (at cfl_stage; 0 when
// it is not finite, -1 for no candidate) and its blow-up bit.  Dtx's candidate CFL dx / (|u| + c)
// falls monotonically with the speed, so the block converts its largest speed once
// (cfl_of_speed) and gets the same minimum.
// SCALED: the fluxes are stored per unit cell width (Geometry::scaled_flux; plain S2O4 only).
// PLAIN: plain S2O4 without the source term (the scaled update, the batches), so the RK3 and
// source forms are not compiled in.  KIND: the tail the update runs, when the launch
// knows it -- 1 the stage that gives the CFL candidates (primitives, blow-up test, signal speed),
// 0 a stage without candidates of a solver with the FP32 mirror (the division-free positivity
// test), -1 decided per launch from a.stage.  The compiler if-converts short uniform branches, and
// predicated-off FP64 instructions still take the FP64 pipe that bounds this kernel, so the
// forms a launch does not run are left out at compile time.
template <bool SCALED = false, int KIND = -1, bool PLAIN = SCALED>
__device__ __forceinline__ void update_one(const UpdateArgs& a, const Geometry& geo, int idx, double& spd,
                                           unsigned int& bad) {
    const int nodex = geo.nodex, nodey = geo.nodey, g = geo.g, ny = geo.ny;
    spd = -1.0;
    bad = 0;
    if (idx < nodex * nodey) {
        const int I = idx / nodey, J = idx % nodey;
        const size_t plane = (size_t)geo.nx * ny;
        const size_t c = (size_t)(I + g) * ny + (J + g);
        // the cell in the FP32 mirror (FP32 solvers): pitch mirror_pitch(ny)
        const size_t pitch = (size_t)mirror_pitch(ny), plane32 = (size_t)geo.nx * pitch;
        const size_t cm = (size_t)(I + g) * pitch + (J + g);
        const size_t nfx = (size_t)(nodex + 1) * nodey, nfy = (size_t)nodex * (nodey + 1);
        const size_t fl = (size_t)I * nodey + J, fr = fl + nodey;
        const size_t fd = (size_t)I * (nodey + 1) + J, fu = fd + 1;
        // the FP64 pipe is the update's bound: the flux balance
        // (dx (F_down - F_up) + dy (F_left - F_right)) / (dx dy) is taken as two differences
        // scaled by 1 / dy and 1 / dx (precomputed), not as four products and a division
        const bool src = !PLAIN && geo.source, rk3 = !PLAIN && geo.integrator == 4;
        double w[4], w0[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            // the state the stage started from: needed at stage 0 (snapshot, and the CFL of
            // one-stage methods) and by RK3's state combination
            const bool need_cur = a.stage == 0 || rk3 || src;
            const double cur = need_cur ? a.W[v * plane + c] : 0.0;
            double old;
            if (a.stage == 0) {
                old = cur;
                a.Wold[v * plane + c] = old;
            } else {
                old = a.Wold[v * plane + c];
            }
            w0[v] = cur;
            double rate;
            if constexpr (SCALED)
                rate = (a.FXy[v * nfy + fd] - a.FXy[v * nfy + fu]) + (a.FXx[v * nfx + fl] - a.FXx[v * nfx + fr]);
            else
                rate = (a.FXy[v * nfy + fd] - a.FXy[v * nfy + fu]) * geo.idy +
                       (a.FXx[v * nfx + fl] - a.FXx[v * nfx + fr]) * geo.idx;
            if (src) {
                // Update_with_source under S2O4 (src/time_advance.cpp:534-704): stage 0 takes
                // W_old + dt (L + S), S = (0, 0, rho, rho v) of the stage's state; stage 1
                // leaves the state
                if (a.stage == 0) {
                    // the stage's state: w0[0] and w0[2] hold rho and rho v read before this
                    // loop wrote the new values
                    const double S = v == 2 ? w0[0] : v == 3 ? w0[2] : 0.0;
                    w[v] = old + (rate + a.ctl->dt * S);
                } else {
                    w[v] = cur;
                }
            } else if (rk3 && a.stage == 1)        // RK3 (Update_with_gauss_RK3, :511-526)
                w[v] = 0.75 * old + 0.25 * cur + rate;
            else if (rk3 && a.stage == 2)
                w[v] = 1.0 / 3.0 * old + 2.0 / 3.0 * cur + rate;
            else
                w[v] = old + rate;
            a.W[v * plane + c] = w[v];
            // the mirror's rounding on the integer pipes (f64_to_f32: the same values as float())
            if (a.W32) a.W32[v * plane32 + cm] = f64_to_f32(w[v]);
        }
        const int jend = nodex < nodey ? nodex : nodey;
        // Update_alpha runs only under is_using_df_factor (src/2Dproblem.cpp:154)
        if (J < jend && !geo.plain) {
            const double ax = a.FAx[fl] + a.FAx[fr], ay = a.FAy[fd] + a.FAy[fu];
            a.AX[c] = ax;
            a.AY[c] = ay;
            if (a.A32) {
                a.A32[cm] = f64_to_f32(ax);
                a.A32[plane32 + cm] = f64_to_f32(ay);
            }
        }
        if (KIND == 0 || (KIND < 0 && a.W32 && a.stage != cfl_stage(geo))) {
            // FP32 solvers, a stage without CFL candidates: Convar_to_Primvar's sign tests without
            // its division (the FP64 pipe bounds this kernel): rho > 0 and
            // 2 rho (rho E) - |rho u|^2 >= 0, which a NaN fails
            const double e = 2.0 * w[0] * w[3] - (w[1] * w[1] + w[2] * w[2]);
            if (!(w[0] > 0.0) || !(e >= 0.0)) bad = 1;
            return;
        }
        const double ir = 1.0 / w[0];
        double pr[4];
        pr[0] = w[0];
        pr[1] = w[1] * ir;
        pr[2] = w[2] * ir;
        pr[3] = (geo.gamma - 1.0) * (w[3] - 0.5 * (w[1] * pr[1] + w[2] * pr[2]));
        if (!(pr[0] >= 0.0) || !(pr[3] >= 0.0)) bad = 1;   // negative or NaN
        if (KIND == 1 || (KIND < 0 && a.stage == cfl_stage(geo))) {
            // the reference's Get_CFL reads the primitives converted at the start of the last
            // stage: the new state of stage stages - 2, or the step's starting state for
            // one-stage methods
            double ir2 = ir;
            if (!PLAIN && geo.stages == 1) {
                ir2 = 1.0 / w0[0];
                pr[0] = w0[0];
                pr[1] = w0[1] * ir2;
                pr[2] = w0[2] * ir2;
                pr[3] = (geo.gamma - 1.0) * (w0[3] - 0.5 * (w0[1] * pr[1] + w0[2] * pr[2]));
            }
            // Dtx's speed (src/time_advance.cpp:295)
            const double tmp = sqrt(pr[1] * pr[1] + pr[2] * pr[2]) + sqrt(geo.gamma * pr[3] * ir2);
            spd = signal_speed(tmp);
        }
    }
}

// Dtx (src/time_advance.cpp:264-305) for the largest signal speed of a set of cells: the update
// takes one reciprocal for both directions, the upload of a state the reference's CFL dx / tmp
// (REF); the viscous cap (:300-303) is the same for every cell.  A negative speed: no cell of the
// set produced a candidate.
template <bool REF = false>
__device__ __forceinline__ double cfl_of_speed(const Geometry& geo, double smax) {
    double cand = 1e300;
    if (!(smax >= 0.0)) return cand;
    double qx, qy;
    if constexpr (REF) {
        qx = geo.cfl * geo.dx / smax;
        qy = geo.cfl * geo.dy / smax;
    } else {
        const double it = geo.cfl / smax;
        qx = geo.dx * it;
        qy = geo.dy * it;
    }
    if (qx > 0) cand = qx;
    if (qy > 0 && qy < cand) cand = qy;
    if (geo.tau_type == 1 && geo.mu > 0) {
        const double cx = 0.25 * geo.cfl * geo.dx * geo.dx / geo.mu;
        const double cy = 0.25 * geo.cfl * geo.dy * geo.dy / geo.mu;
        if (cx < cand) cand = cx;
        if (cy < cand) cand = cy;
    }
    return cand;
}

// block reduction of the cells' signal speeds (update_one) and status bits into one problem's
// control word: the largest speed, converted to the block's CFL candidate by one thread.  A
// speed is -1 (no candidate), +0 or a positive finite double, and over these values the bit
// patterns read as signed 64-bit integers order as the doubles do, so the maximum is taken on
// the integer pipes (the update's bound is the FP64 pipe).
template <bool REF = false>
__device__ __forceinline__ void reduce_block_speed(double spd, unsigned int bad, StepCtl* ctl, bool do_cfl,
                                                   const Geometry& geo) {
    long long sk = __double_as_longlong(spd);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long other = __shfl_xor_sync(0xffffffffu, sk, o);
        sk = other > sk ? other : sk;
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    __shared__ long long sc[8];
    __shared__ unsigned int sb[8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sc[wid] = sk; sb[wid] = bad; }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long mk = sc[0];
        unsigned int b = sb[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { mk = sc[k] > mk ? sc[k] : mk; b |= sb[k]; }
        const double m = __longlong_as_double(mk);
        const double cand = cfl_of_speed<REF>(geo, m);
        if (do_cfl && cand < 1e300) atomic_min_pos(&ctl->cfl_bits, cand);
        if (b) atomicOr(&ctl->status, 1u);
    }
}

// step prologue: dt from the CFL accumulator (seeded with dx, as Get_CFL seeds with the
// first cell's dx), clipped to the stop time (src/time_advance.cpp:285-289); the
// accumulator is re-seeded for the candidates this step's stage 0 produces.
__device__ __forceinline__ void begin_step_one(StepCtl* ctl, double tstop, double seed) {
    double dt = __longlong_as_double((long long)ctl->cfl_bits);
    const double t = ctl->t;
    // the driver loop runs while t < tstop; steps queued past it do nothing.  A problem whose
    // state went bad (status bit 0; the reference exits there) or whose step lost a tile to a
    // TMA load that never completed takes no further steps.
    const bool go = t < tstop && !(ctl->status & (1u | WAIT_TIMEOUT_BIT));
    ctl->active = go ? 1u : 0u;
    ctl->tbeg = t;
    if (!go) return;
    if (t + dt > tstop) dt = tstop - t + 1e-16;
    ctl->dt = dt;
    ctl->t = t + dt;
    ctl->cfl_bits = (unsigned long long)__double_as_longlong(seed);
}


}  // namespace hos
