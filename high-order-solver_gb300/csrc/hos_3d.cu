// hos_3d.cu -- the 3D step on the GPU and its C ABI (hos3d_* in include/hos_gb300.h):
// boundaries, the S2O4 update with the CFL reduction, the step prologue, and the host side.
// The reconstruction and flux kernels are in hos_3d.cuh (instantiated in hos_3d_k64.cu and
// hos_3d_k32.cu).
//
// One stage = bc3 -> for x, y, z faces: face3 -> line3 -> point3 (GKS3D) -> update3.
// One step adds begin3 (CopyFluid_new_to_old is the stage-0 snapshot inside update3).
// As in the reference's 3D loop: the CFL reads the primitives converted at the start of the
// last stage (the state after stage 0; the initial primitives at step 0), seeded with
// R_c = min(dx, dy, dz), capped by the viscous limit for Navier-Stokes, clipped to
// tstop - t + 1e-16 (src/time_advance.cpp:793-848).
#include <cstring>
#include <new>
#include <string>

#include "../../include/hos_gb300.h"
#include "hos_3d_gate.cuh"
#include "hos_3d_launch.h"

namespace hos {
namespace d3 {

// per-axis source of ghost index x: free (nearest interior layer), periodic, reflecting.
// Applying the three axes' maps at once gives the cells the reference's six side functions
// leave, called x, then y, then z over the whole block (src/boundary_condition.cpp:445-570).
__device__ __forceinline__ int bc_src3(int x, int n, int g, int kind, bool low, bool& flip) {
    flip = false;
    if (kind == HOS_BC_PERIODIC) return low ? x + (n - 2 * g) : x - (n - 2 * g);
    if (kind == HOS_BC_REFLECT) {
        flip = true;
        return low ? 2 * g - 1 - x : 2 * (n - g) - 1 - x;
    }
    return low ? g : n - g - 1;
}

__global__ void __launch_bounds__(256) bc3_kernel(double* __restrict__ W, Geo3 g, const Ctl3* ctl) {
    if (ctl && !ctl->active) return;
    const size_t plane = (size_t)g.nx * g.ny * g.nz;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= plane) return;
    const int k = (int)(t % g.nz), j = (int)((t / g.nz) % g.ny), i = (int)(t / ((size_t)g.nz * g.ny));
    const int x[3] = {i, j, k}, n[3] = {g.nx, g.ny, g.nz};
    int src[3];
    bool flip[3], ghost = false;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        flip[ax] = false;
        src[ax] = x[ax];
        if (x[ax] < g.g || x[ax] >= n[ax] - g.g) {
            const bool low = x[ax] < g.g;
            src[ax] = bc_src3(x[ax], n[ax], g.g, g.bc[2 * ax + (low ? 0 : 1)], low, flip[ax]);
            ghost = true;
        }
    }
    if (!ghost) return;
    const size_t s = ((size_t)src[0] * g.ny + src[1]) * g.nz + src[2];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        double q = W[v * plane + s];
        if (v >= 1 && v <= 3 && flip[v - 1]) q = -q;
        W[v * plane + t] = q;
    }
}

// with_cfl false: the state check alone (stage 1 takes no candidates; the square roots and
// divisions of the candidate are the FP64 pipe's largest cost in the update)
__device__ __forceinline__ double cfl_candidate3(const double* w, const Geo3& g, unsigned& bad, bool is_prim,
                                                 bool with_cfl = true) {
    double pr[5];
    if (is_prim) {
        for (int v = 0; v < 5; ++v) pr[v] = w[v];
    } else {
        const double ir = 1.0 / w[0];
        pr[0] = w[0];
        pr[1] = w[1] * ir;
        pr[2] = w[2] * ir;
        pr[3] = w[3] * ir;
        pr[4] = (g.gamma - 1.0) * (w[4] - 0.5 * (w[1] * pr[1] + w[2] * pr[2] + w[3] * pr[3]));
    }
    bad = (pr[0] < 0 || pr[4] < 0 || isnan(pr[0]) || isnan(pr[4])) ? 1u : 0u;
    if (!with_cfl) return 1e300;
    // Dtx_3d (src/time_advance.cpp:826-848)
    const double tmp = sqrt(pr[1] * pr[1] + pr[2] * pr[2] + pr[3] * pr[3]) + sqrt(g.gamma * pr[4] / pr[0]);
    double q = g.cfl * g.rc / tmp;
    if (g.tau_type != 0 && g.mu > 0) {
        const double cap = 0.33 * g.cfl * g.rc * g.rc * pr[0] / g.mu;
        if (cap < q) q = cap;
    }
    return q > 0 ? q : 1e300;
}

__device__ __forceinline__ void reduce3(double cand, unsigned bad, Ctl3* ctl, bool do_cfl) {
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

// the stage-combined flux of one face (written by the point kernel)
__device__ __forceinline__ void load_flux3(const double* FS, size_t nf, size_t f, double* out) {
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v] = FS[v * nf + f];
}

// FP32 solvers, once per stage after the ghost fill: the FP32 mirror of the whole state
// (ghosts included) that the FP32 face kernels read, and -- with the gate on -- each cell's FP32
// (density, pressure) pair for the gate's features.  GB300's FP64 pipe converts at 1/64 of the
// FP32 rate: converting once per cell here replaces the 25 conversions per cell and direction
// the face kernel would make.
__global__ void __launch_bounds__(256) mirror3_kernel(const double* __restrict__ W, float* __restrict__ W32,
                                                      float2* __restrict__ rp, size_t plane, float gamma,
                                                      const Ctl3* ctl) {
    if (!ctl->active) return;
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= plane) return;
    float w[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        w[v] = (float)W[v * plane + c];
        W32[v * plane + c] = w[v];
    }
    if (rp) rp[c] = make_float2(w[0], (gamma - 1.0f) * (w[4] - 0.5f * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]) / w[0]));
}

// W = W_old + sum over the six faces; y and z face fluxes turned back to the global frame
// (src/time_advance.cpp:942-997).  Stage 0 takes the snapshot W_old and produces the next
// step's CFL candidates from its new state; every stage flags a bad state.
__global__ void __launch_bounds__(256) update3_kernel(double* __restrict__ W, double* __restrict__ Wold,
                                                      const double* __restrict__ FX, const double* __restrict__ FY,
                                                      const double* __restrict__ FZ, Ctl3* ctl, Geo3 g, Lay lx,
                                                      Lay ly, Lay lz, int stage) {
    if (!ctl->active) return;
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t ncell = (size_t)g.nodex * g.nodey * g.nodez;
    double cand = 1e300;
    unsigned bad = 0;
    if (t < ncell) {
        const int K = (int)(t % g.nodez), J = (int)((t / g.nodez) % g.nodey), I = (int)(t / ((size_t)g.nodez * g.nodey));
        const size_t plane = (size_t)g.nx * g.ny * g.nz;
        const size_t c = ((size_t)(I + g.g) * g.ny + (J + g.g)) * g.nz + (K + g.g);
        double xl[5], xr[5], yl[5], yr[5], zl[5], zr[5];
        const int Ib = g.nodex - 1 - I;
        load_flux3(FX, lx.n(), lx.idx(I, J, K), xl);
        load_flux3(FX, lx.n(), lx.idx(I + 1, J, K), xr);
        load_flux3(FY, ly.n(), ly.idx(J, Ib, K), yl);
        load_flux3(FY, ly.n(), ly.idx(J + 1, Ib, K), yr);
        load_flux3(FZ, lz.n(), lz.idx(K, J, Ib), zl);
        load_flux3(FZ, lz.n(), lz.idx(K + 1, J, Ib), zr);
        const double idx_ = g.idx, idy = g.idy, idz = g.idz;
        // global-frame flux differences: y faces (u, v) = (-v', u'), z faces (u, w) = (-w', u')
        double tot[5];
        tot[0] = idz * (zl[0] - zr[0]) + idy * (yl[0] - yr[0]) + idx_ * (xl[0] - xr[0]);
        tot[1] = idz * (zr[3] - zl[3]) + idy * (yr[2] - yl[2]) + idx_ * (xl[1] - xr[1]);
        tot[2] = idz * (zl[2] - zr[2]) + idy * (yl[1] - yr[1]) + idx_ * (xl[2] - xr[2]);
        tot[3] = idz * (zl[1] - zr[1]) + idy * (yl[3] - yr[3]) + idx_ * (xl[3] - xr[3]);
        tot[4] = idz * (zl[4] - zr[4]) + idy * (yl[4] - yr[4]) + idx_ * (xl[4] - xr[4]);
        double w[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            double old;
            if (stage == 0) {
                old = W[v * plane + c];
                Wold[v * plane + c] = old;
            } else {
                old = Wold[v * plane + c];
            }
            w[v] = old + tot[v];
            W[v * plane + c] = w[v];
        }
        const double q = cfl_candidate3(w, g, bad, false, stage == 0);
        if (stage == 0) cand = q;
    }
    reduce3(cand, bad, ctl, stage == 0);
}

// CFL candidates of the initial state (the primitives the first Get_CFL reads)
__global__ void __launch_bounds__(256) cfl3_init_kernel(const double* __restrict__ Q, Ctl3* ctl, Geo3 g, int is_prim) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t ncell = (size_t)g.nodex * g.nodey * g.nodez;
    double cand = 1e300;
    unsigned bad = 0;
    if (t < ncell) {
        const int K = (int)(t % g.nodez), J = (int)((t / g.nodez) % g.nodey), I = (int)(t / ((size_t)g.nodez * g.nodey));
        const size_t plane = (size_t)g.nx * g.ny * g.nz;
        const size_t c = ((size_t)(I + g.g) * g.ny + (J + g.g)) * g.nz + (K + g.g);
        double w[5];
        for (int v = 0; v < 5; ++v) w[v] = Q[v * plane + c];
        cand = cfl_candidate3(w, g, bad, is_prim != 0);
    }
    reduce3(cand, bad, ctl, true);
}

__global__ void begin3_kernel(Ctl3* ctl, double tstop, double seed, int first) {
    if (!first) ctl->step += ctl->active ? 1 : 0;
    const double t = ctl->t;
    const bool go = t < tstop && !(ctl->status & (1u | WAIT_TIMEOUT_BIT));
    ctl->active = go ? 1u : 0u;
    ctl->tbeg = t;
    double dt = __longlong_as_double((long long)ctl->cfl_bits);
    if (!go) return;
    ctl->cfl_bits = (unsigned long long)__double_as_longlong(seed);
    if (t + dt > tstop) dt = tstop - t + 1e-16;
    ctl->dt = dt;
    ctl->t = t + dt;
}

// AoS [ncell][5] <-> SoA [5][ncell]; to_prim converts the state to (rho, u, v, w, p)
__global__ void __launch_bounds__(256) aos_to_soa3(const double* __restrict__ in, double* __restrict__ out, size_t n) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    for (int v = 0; v < 5; ++v) out[v * n + t] = in[5 * t + v];
}
__global__ void __launch_bounds__(256) soa_to_aos3(const double* __restrict__ in, double* __restrict__ out, size_t n,
                                                   double gamma, int to_prim) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double w[5];
    for (int v = 0; v < 5; ++v) w[v] = in[v * n + t];
    if (to_prim) {
        const double r = w[0];
        w[1] = w[1] / r;
        w[2] = w[2] / r;
        w[3] = w[3] / r;
        w[4] = (gamma - 1.0) * (w[4] - 0.5 * r * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]));
    }
    for (int v = 0; v < 5; ++v) out[5 * t + v] = w[v];
}

thread_local std::string g_err3;
int fail3(int code, const std::string& m) {
    g_err3 = m;
    return code;
}

}  // namespace d3
}  // namespace hos

using namespace hos;
using namespace hos::d3;

struct hos_solver3d {
    hos_params3d p;
    int precision = 0;
    Geo3 geo;
    Dir3 dirs[3];
    cudaStream_t stream = nullptr;
    double *W = nullptr, *Wold = nullptr, *stage_buf = nullptr;
    float* W32 = nullptr;   // FP32 solvers: the FP32 mirror of W, refreshed once per stage
    double* FS[3] = {nullptr, nullptr, nullptr};
    void *FV = nullptr, *LV = nullptr;
    Ctl3* ctl = nullptr;
    bool first = true;
    size_t ncell = 0;
    // learned gate (FP32): flags per cell, counters, the network's inference copy
    bool gated = false;
    unsigned char* gflags = nullptr;
    float2* grp = nullptr;
    Stats3* gstats = nullptr;
    __nv_bfloat16* gw = nullptr;
    float* gb = nullptr;
    float gthreshold = 0.0f;
    unsigned gaudit_mask = 0, gseed = 1;
};

namespace {

void free3(hos_solver3d* s) {
    double* b[] = {s->W, s->Wold, s->stage_buf, s->FS[0], s->FS[1], s->FS[2]};
    for (double* x : b)
        if (x) cudaFree(x);
    if (s->FV) cudaFree(s->FV);
    if (s->LV) cudaFree(s->LV);
    void* gbufs[] = {s->gflags, s->grp, s->gstats, s->gw, s->gb, s->W32};
    for (void* x : gbufs)
        if (x) cudaFree(x);
    if (s->ctl) cudaFree(s->ctl);
    if (s->stream) cudaStreamDestroy(s->stream);
}

Dir3 make_dir(const Geo3& g, int dir) {
    Dir3 d{};
    d.dir = dir;
    if (dir == 0) { d.n0 = g.nodex; d.n1 = g.nodey; d.n2 = g.nodez; d.hn = g.dx; d.h1 = g.dy; d.h2 = g.dz; }
    else if (dir == 1) { d.n0 = g.nodey; d.n1 = g.nodex; d.n2 = g.nodez; d.hn = g.dy; d.h1 = g.dx; d.h2 = g.dz; }
    else { d.n0 = g.nodez; d.n1 = g.nodey; d.n2 = g.nodex; d.hn = g.dz; d.h1 = g.dy; d.h2 = g.dx; }
    d.ihn = 1.0 / d.hn;
    d.ih1 = 1.0 / d.h1;
    d.ih2 = 1.0 / d.h2;
    d.fihn = (float)d.ihn;
    d.fih1 = (float)d.ih1;
    d.fih2 = (float)d.ih2;
    const int af = dir == 2 ? 1 : 0;
    d.fv = Lay{d.n0 + 1, d.n1 + 4, d.n2 + 4, af};
    d.cel = Lay{d.n0 + 2, d.n1 + 4, d.n2 + 4, af};
    d.lv = Lay{d.n0 + 1, d.n1, d.n2 + 4, af};
    d.fs = Lay{d.n0 + 1, d.n1, d.n2, af};
    return d;
}

cudaError_t flux_dir(hos_solver3d* s, int dir, int stage, cudaEvent_t* ev) {
    const Dir3& d = s->dirs[dir];
    const Gate3 gt{s->gated ? s->gflags : nullptr, s->gated ? &s->gstats->fallback : nullptr};
    if (s->precision == HOS_FP32)
        return launch_flux3<float>(s->W32, (float*)s->FV, (float*)s->LV, s->FS[dir], s->geo, d, s->ctl, stage, s->stream,
                                   ev, gt);
    return launch_flux3<double>(s->W, (double*)s->FV, (double*)s->LV, s->FS[dir], s->geo, d, s->ctl, stage, s->stream, ev,
                                gt);
}

GateRun3 gate_run(hos_solver3d* s, const gate::Net& net) {
    GateRun3 r{};
    r.W = s->W;
    r.rp = s->grp;
    r.g = s->geo;
    r.net = net;
    r.ctl = s->ctl;
    return r;
}

unsigned blocks(size_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

int enqueue_begin3(hos_solver3d* s, double tstop, cudaEvent_t ev) {
    begin3_kernel<<<1, 1, 0, s->stream>>>(s->ctl, tstop, s->geo.rc, s->first ? 1 : 0);
    s->first = false;
    if (ev) cudaEventRecord(ev, s->stream);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HOS_OK : fail3(HOS_E_CUDA, std::string("begin3: ") + cudaGetErrorString(e));
}

// ev (may be null): 12 events, after the boundaries, after the gate (recorded without a launch
// when the solver has no gate), after face/line/point of x, then of y, then of z, and after the
// update
int enqueue_stage3(hos_solver3d* s, int stage, cudaEvent_t* ev) {
    const Geo3& g = s->geo;
    bc3_kernel<<<blocks((size_t)g.nx * g.ny * g.nz, 256), 256, 0, s->stream>>>(s->W, g, s->ctl);
    if (s->W32) {
        const size_t plane = (size_t)g.nx * g.ny * g.nz;
        mirror3_kernel<<<blocks(plane, 256), 256, 0, s->stream>>>(s->W, s->W32, s->gated ? s->grp : nullptr, plane,
                                                                  (float)g.gamma, s->ctl);
    }
    if (ev) cudaEventRecord(ev[0], s->stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && s->gated) {
        GateRun3 r = gate_run(s, gate::Net{s->gw, s->gw + gate::NH * gate::NF, s->gw + gate::NH * gate::NF + gate::NH * gate::NH,
                                           s->gb, s->gb + gate::NH, s->gb + 2 * gate::NH});
        r.flags = s->gflags;
        r.stats = s->gstats;
        r.threshold = s->gthreshold;
        r.audit_mask = s->gaudit_mask;
        r.seed = s->gseed++;
        e = launch_gate3(r, s->stream, /*rp_ready=*/true);   // mirror3 wrote the (density, pressure) pairs
    }
    if (ev) cudaEventRecord(ev[1], s->stream);
    for (int dir = 0; dir < 3 && e == cudaSuccess; ++dir) {
        e = flux_dir(s, dir, stage, ev ? ev + 2 + 3 * dir : nullptr);
    }
    if (e != cudaSuccess) return fail3(HOS_E_CUDA, std::string("flux3: ") + cudaGetErrorString(e));
    const size_t nc = (size_t)g.nodex * g.nodey * g.nodez;
    update3_kernel<<<blocks(nc, 256), 256, 0, s->stream>>>(s->W, s->Wold, s->FS[0], s->FS[1], s->FS[2], s->ctl, g,
                                                           s->dirs[0].fs, s->dirs[1].fs, s->dirs[2].fs, stage);
    if (ev) cudaEventRecord(ev[11], s->stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail3(HOS_E_CUDA, std::string("update3: ") + cudaGetErrorString(e));
    return HOS_OK;
}

int enqueue_step3(hos_solver3d* s, double tstop) {
    int st = enqueue_begin3(s, tstop, nullptr);
    for (int stage = 0; stage < 2 && !st; ++stage) st = enqueue_stage3(s, stage, nullptr);
    return st;
}

int check_bc3(const int* bc) {
    for (int k = 0; k < 6; ++k)
        if (bc[k] < 0 || bc[k] > 2) return fail3(HOS_E_CONFIG, "3D boundaries: free, periodic or reflective");
    for (int a = 0; a < 3; ++a)
        if ((bc[2 * a] == HOS_BC_PERIODIC) != (bc[2 * a + 1] == HOS_BC_PERIODIC))
            return fail3(HOS_E_CONFIG, "periodic boundaries must be paired");
    return HOS_OK;
}

int read_ctl(hos_solver3d* s, Ctl3& c) {
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&c, s->ctl, sizeof c, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? HOS_OK : fail3(HOS_E_CUDA, std::string("control read: ") + cudaGetErrorString(e));
}

}  // namespace

extern "C" {

const char* hos3d_last_error(void) { return g_err3.c_str(); }

int hos3d_create(const hos_params3d* params, int precision, hos_solver3d** out) {
    if (!params || !out) return fail3(HOS_E_ARG, "null argument");
    const hos_params3d& p = *params;
    if (p.ghost < 3 || p.ghost > 8) return fail3(HOS_E_CONFIG, "ghost must be 3..8 (WENO5 with a tangential halo of 2)");
    if (p.nodex < p.ghost || p.nodey < p.ghost || p.nodez < p.ghost) return fail3(HOS_E_CONFIG, "nodes must be >= ghost");
    if (int st = check_bc3(p.bc)) return st;
    if (p.tau_type != 0 && p.tau_type != 1) return fail3(HOS_E_CONFIG, "tau_type must be 0 (Euler) or 1 (NS)");
    if (p.prandtl_fix && !(p.prandtl > 0)) return fail3(HOS_E_CONFIG, "the Prandtl fix needs prandtl > 0");
    if (precision != HOS_FP64 && precision != HOS_FP32) return fail3(HOS_E_CONFIG, "bad precision");
    if (p.gks3d_pressure_slot && (precision != HOS_FP64 || p.prandtl_fix))
        return fail3(HOS_E_CONFIG, "the reference's GKS3D pressure convention runs in FP64 without the Prandtl fix");
    hos_solver3d* s = new (std::nothrow) hos_solver3d();
    if (!s) return fail3(HOS_E_NOMEM, "host allocation");
    s->p = p;
    s->precision = precision;
    Geo3& g = s->geo;
    g.g = p.ghost;
    g.nodex = p.nodex;
    g.nodey = p.nodey;
    g.nodez = p.nodez;
    g.nx = p.nodex + 2 * p.ghost;
    g.ny = p.nodey + 2 * p.ghost;
    g.nz = p.nodez + 2 * p.ghost;
    g.dx = (p.right - p.left) / p.nodex;
    g.dy = (p.up - p.down) / p.nodey;
    g.dz = (p.front - p.back) / p.nodez;
    g.prandtl_coef = p.prandtl_fix ? 1.0 / p.prandtl - 1.0 : 0.0;
    g.p_slot = p.gks3d_pressure_slot ? 1 : 0;
    g.idx = 1.0 / g.dx;
    g.idy = 1.0 / g.dy;
    g.idz = 1.0 / g.dz;
    g.rc = g.dx;
    if (g.dy < g.rc) g.rc = g.dy;
    if (g.dz < g.rc) g.rc = g.dz;
    g.cfl = p.cfl;
    g.gamma = p.gamma;
    g.K = p.K;
    g.c1 = p.c1_euler;
    g.c2 = p.c2_euler;
    g.mu = p.mu;
    g.tau_type = p.tau_type;
    g.characteristic = p.characteristic ? 1 : 0;
    for (int k = 0; k < 6; ++k) g.bc[k] = p.bc[k];
    narrow_params3(g);
    for (int d = 0; d < 3; ++d) s->dirs[d] = make_dir(g, d);
    s->ncell = (size_t)g.nx * g.ny * g.nz;
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return fail3(HOS_E_CUDA, std::string("stream: ") + cudaGetErrorString(e));
    }
    const size_t tsz = precision == HOS_FP32 ? sizeof(float) : sizeof(double);
    size_t nfv = 0, nlv = 0;
    for (int d = 0; d < 3; ++d) {
        if (s->dirs[d].fv.n() > nfv) nfv = s->dirs[d].fv.n();
        if (s->dirs[d].lv.n() > nlv) nlv = s->dirs[d].lv.n();
    }
    struct { void** q; size_t bytes; } al[] = {
        {(void**)&s->W, 5 * s->ncell * sizeof(double)},
        {(void**)&s->Wold, 5 * s->ncell * sizeof(double)},
        {(void**)&s->stage_buf, 5 * s->ncell * sizeof(double)},
        {(void**)&s->FS[0], 10 * s->dirs[0].fs.n() * sizeof(double)},
        {(void**)&s->FS[1], 10 * s->dirs[1].fs.n() * sizeof(double)},
        {(void**)&s->FS[2], 10 * s->dirs[2].fs.n() * sizeof(double)},
        {&s->FV, 20 * nfv * tsz},
        {&s->LV, 60 * nlv * tsz},
        {(void**)&s->ctl, sizeof(Ctl3)},
        {(void**)&s->W32, precision == HOS_FP32 ? 5 * s->ncell * sizeof(float) : 0}};
    for (auto& a : al) {
        if (a.bytes == 0) continue;
        if ((e = cudaMalloc(a.q, a.bytes)) != cudaSuccess) {
            free3(s);
            delete s;
            return fail3(HOS_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        cudaMemsetAsync(*a.q, 0, a.bytes, s->stream);
    }
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) {
        free3(s);
        delete s;
        return fail3(HOS_E_CUDA, std::string("create: ") + cudaGetErrorString(e));
    }
    *out = s;
    return HOS_OK;
}

int hos3d_destroy(hos_solver3d* s) {
    if (!s) return HOS_OK;
    cudaStreamSynchronize(s->stream);
    free3(s);
    delete s;
    return HOS_OK;
}

int hos3d_set_state(hos_solver3d* s, const double* convar, const double* primvar) {
    if (!s || !convar) return fail3(HOS_E_ARG, "null argument");
    const size_t n = s->ncell, bytes = 5 * n * sizeof(double);
    // host AoS -> device staging -> SoA state (and primitives into W_old, free until stage 0)
    cudaError_t e = cudaMemcpyAsync(s->stage_buf, convar, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
        aos_to_soa3<<<blocks(n, 256), 256, 0, s->stream>>>(s->stage_buf, s->W, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && primvar) {
        e = cudaMemcpyAsync(s->stage_buf, primvar, bytes, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) {
            aos_to_soa3<<<blocks(n, 256), 256, 0, s->stream>>>(s->stage_buf, s->Wold, n);
            e = cudaGetLastError();
        }
    }
    Ctl3 c{};
    const double seed = s->geo.rc;
    std::memcpy(&c.cfl_bits, &seed, sizeof seed);
    c.active = 1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->ctl, &c, sizeof c, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
        const size_t nc = (size_t)s->geo.nodex * s->geo.nodey * s->geo.nodez;
        cfl3_init_kernel<<<blocks(nc, 256), 256, 0, s->stream>>>(primvar ? s->Wold : s->W, s->ctl, s->geo, primvar ? 1 : 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail3(HOS_E_CUDA, std::string("set_state: ") + cudaGetErrorString(e));
    s->first = true;
    Ctl3 back;
    if (int st = read_ctl(s, back)) return st;
    if (back.status & 1u) return fail3(HOS_E_BLOWUP, "initial state has negative density/pressure or NaN");
    return HOS_OK;
}

int hos3d_get_state(hos_solver3d* s, double* convar, double* primvar) {
    if (!s) return fail3(HOS_E_ARG, "null solver");
    const size_t n = s->ncell, bytes = 5 * n * sizeof(double);
    cudaError_t e = cudaSuccess;
    double* outs[2] = {convar, primvar};
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        if (!outs[k]) continue;
        soa_to_aos3<<<blocks(n, 256), 256, 0, s->stream>>>(s->W, s->stage_buf, n, s->geo.gamma, k);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(outs[k], s->stage_buf, bytes, cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    }
    return e == cudaSuccess ? HOS_OK : fail3(HOS_E_CUDA, std::string("get_state: ") + cudaGetErrorString(e));
}

int hos3d_step(hos_solver3d* s, double tstop) {
    if (!s) return fail3(HOS_E_ARG, "null solver");
    return enqueue_step3(s, tstop);
}

int hos3d_advance(hos_solver3d* s, int nsteps, double tstop) {
    if (!s) return fail3(HOS_E_ARG, "null solver");
    for (int k = 0; k < nsteps; ++k)
        if (int st = enqueue_step3(s, tstop)) return st;
    return HOS_OK;
}

int hos3d_begin_step(hos_solver3d* s, double tstop) {
    if (!s) return fail3(HOS_E_ARG, "null solver");
    return enqueue_begin3(s, tstop, nullptr);
}

int hos3d_stage(hos_solver3d* s, int stage) {
    if (!s) return fail3(HOS_E_ARG, "null solver");
    if (stage != 0 && stage != 1) return fail3(HOS_E_ARG, "stage must be 0 or 1");
    return enqueue_stage3(s, stage, nullptr);
}

int hos3d_sync(hos_solver3d* s, double* t, double* dt) {
    if (!s) return fail3(HOS_E_ARG, "null solver");
    Ctl3 c;
    if (int st = read_ctl(s, c)) return st;
    if (t) *t = c.t;
    if (dt) *dt = c.dt;
    if (c.status & 1u) return fail3(HOS_E_BLOWUP, "negative density/pressure or NaN in the state");
    if (c.status & WAIT_TIMEOUT_BIT)
        return fail3(HOS_E_TIMEOUT, "a tensor-core MMA of the gate did not complete within its wait limit");
    return HOS_OK;
}

int hos3d_set_time(hos_solver3d* s, double t) {
    if (!s) return fail3(HOS_E_ARG, "null solver");
    Ctl3 c;
    if (int st = read_ctl(s, c)) return st;
    c.t = t;
    cudaError_t e = cudaMemcpy(s->ctl, &c, sizeof c, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? HOS_OK : fail3(HOS_E_CUDA, std::string("set_time: ") + cudaGetErrorString(e));
}

int hos3d_stream(hos_solver3d* s, void** stream) {
    if (!s || !stream) return fail3(HOS_E_ARG, "null argument");
    *stream = (void*)s->stream;
    return HOS_OK;
}

int hos3d_profile_step(hos_solver3d* s, double tstop, float* ms, int n) {
    if (!s || !ms || n < 25) return fail3(HOS_E_ARG, "need 25 timings");
    cudaEvent_t ev[26];
    for (auto& x : ev) cudaEventCreate(&x);
    cudaEventRecord(ev[0], s->stream);
    int st = enqueue_begin3(s, tstop, ev[1]);
    for (int stage = 0; stage < 2 && !st; ++stage) st = enqueue_stage3(s, stage, ev + 2 + 12 * stage);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (!st && e == cudaSuccess)
        for (int k = 0; k < 25; ++k) cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]);
    for (auto& x : ev) cudaEventDestroy(x);
    if (st) return st;
    return e == cudaSuccess ? HOS_OK : fail3(HOS_E_CUDA, std::string("profile: ") + cudaGetErrorString(e));
}

int hos3d_set_gate(hos_solver3d* s, const hos_gate* g, float threshold, int audit_log2) {
    using namespace gate;
    if (!s) return fail3(HOS_E_ARG, "null solver");
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return fail3(HOS_E_CUDA, std::string("set_gate: ") + cudaGetErrorString(e));
    if (!g) {
        s->gated = false;
        return HOS_OK;
    }
    if (s->precision != HOS_FP32) return fail3(HOS_E_CONFIG, "the learned gate runs on the FP32-bulk path");
    if (audit_log2 < 0 || audit_log2 > 31) return fail3(HOS_E_ARG, "audit_log2 must be 0..31");
    if (!s->grp && (e = cudaMalloc(&s->grp, s->ncell * sizeof(float2))) != cudaSuccess)
        return fail3(HOS_E_NOMEM, std::string("gate buffers: ") + cudaGetErrorString(e));
    if (!s->gflags) {
        if ((e = cudaMalloc(&s->gflags, s->ncell)) == cudaSuccess && (e = cudaMalloc(&s->gstats, sizeof(Stats3))) == cudaSuccess &&
            (e = cudaMalloc(&s->gw, NET_BF16 * sizeof(__nv_bfloat16))) == cudaSuccess)
            e = cudaMalloc(&s->gb, NET_F32 * sizeof(float));
        if (e == cudaSuccess) e = cudaMemset(s->gstats, 0, sizeof(Stats3));
        if (e != cudaSuccess) return fail3(HOS_E_NOMEM, std::string("gate buffers: ") + cudaGetErrorString(e));
    }
    // the solver keeps its own copy of the network, which can go on training
    if ((e = cudaStreamSynchronize(g->stream)) == cudaSuccess &&
        (e = cudaMemcpy(s->gw, g->wbf, NET_BF16 * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice)) == cudaSuccess)
        e = cudaMemcpy(s->gb, g->bias, NET_F32 * sizeof(float), cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) return fail3(HOS_E_CUDA, std::string("set_gate copy: ") + cudaGetErrorString(e));
    s->gthreshold = threshold;
    s->gaudit_mask = audit_log2 == 31 ? 0xffffffffu : (1u << audit_log2) - 1u;
    s->gated = true;
    return HOS_OK;
}

int hos3d_gate_stats(hos_solver3d* s, unsigned long long* stats, int reset) {
    if (!s || !stats) return fail3(HOS_E_ARG, "null argument");
    if (!s->gstats) {
        std::memset(stats, 0, 10 * sizeof(unsigned long long));
        return HOS_OK;
    }
    Stats3 st;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&st, s->gstats, sizeof st, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && reset) e = cudaMemset(s->gstats, 0, sizeof st);
    if (e != cudaSuccess) return fail3(HOS_E_CUDA, std::string("gate_stats: ") + cudaGetErrorString(e));
    const unsigned long long v[10] = {st.cells[0], st.cells[1], st.cells[2], st.smooth[0], st.smooth[1], st.smooth[2],
                                      st.audited, st.false_neg, st.fallback, 0};
    std::memcpy(stats, v, sizeof v);
    return HOS_OK;
}

int hos_gate_collect3d(hos_gate* g, hos_solver3d* s, int sample_log2) {
    using namespace gate;
    if (!g || !s || sample_log2 < 0 || sample_log2 > 31) return fail3(HOS_E_ARG, "bad argument");
    if (!g->samples) return fail3(HOS_E_CONFIG, "the gate was created without sample capacity");
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && !s->grp) e = cudaMalloc(&s->grp, s->ncell * sizeof(float2));
    if (e != cudaSuccess) return fail3(HOS_E_NOMEM, std::string("gate collect: ") + cudaGetErrorString(e));
    const Geo3& geo = s->geo;
    bc3_kernel<<<blocks((size_t)geo.nx * geo.ny * geo.nz, 256), 256, 0, s->stream>>>(s->W, geo, nullptr);
    GateRun3 r = gate_run(s, g->net());
    r.ctl = nullptr;
    r.seed = g->collect_seed++;
    r.samples = g->samples;
    r.capacity = g->capacity;
    r.sample_count = &g->stats->samples;
    r.sample_mask = sample_log2 == 31 ? 0xffffffffu : (1u << sample_log2) - 1u;
    e = cudaStreamSynchronize(g->stream);   // the network's copy is current
    if (e == cudaSuccess) e = launch_gate3(r, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? HOS_OK : fail3(HOS_E_CUDA, std::string("gate collect: ") + cudaGetErrorString(e));
}

}  // extern "C"
