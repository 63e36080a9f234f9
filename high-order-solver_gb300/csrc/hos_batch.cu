// hos_batch.cu -- many independent 2D problems of uneven sizes advanced together: one launch
// per phase for the whole batch (persistent face kernels striding over a table of tiles of
// every problem), each problem with its own dt, stop time and boundaries, the step
// capturable as one CUDA graph, and the face-tile shape picked by timing the candidates on
// the batch itself.
//
// The reference has no batch mode: each of its problem drivers advances one Block2d
// (src/2Dproblem.cpp:108-159).  Per problem, the batched step performs exactly the operations
// of the single-problem step (hos_solver.cu): WENO5 and WENO9 results agree bit for bit;
// in the WENO7 instantiation nvcc contracts a few multiply-adds differently, so WENO7 agrees
// to rounding (relative 2e-16 in FP64 per step).
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "hos_batch.cuh"
#include "hos_gate.cuh"

namespace hos {

// kernels defined in hos_solver.cu
__global__ void aos_to_soa_kernel(const double* __restrict__ aos, double* __restrict__ soa, size_t n);
__global__ void soa_to_aos_kernel(const double* __restrict__ soa, double* __restrict__ aos, size_t n);
__global__ void __launch_bounds__(256) cfl_from_prim_kernel(const double* __restrict__ prim, Geometry geo, StepCtl* ctl);
__global__ void prim_of_state_kernel(const double* __restrict__ W, double* __restrict__ P, size_t n, double gamma);
__global__ void mirror_state_kernel(const double* __restrict__ W, const double* __restrict__ AX,
                                    const double* __restrict__ AY, float* __restrict__ W32, float* __restrict__ A32,
                                    int nx, int ny);
void fill_wedge(BcSpec& bc, const hos_params2d& p, double dx);

namespace batch {

__global__ void bc_batch_kernel(const Prob* __restrict__ probs) {
    const Prob* pr = probs + blockIdx.y;
    if (!pr->ctl->active) return;
    const Geometry geo = pr->geo;
    const long long n = 2LL * geo.g * geo.ny + 2LL * geo.g * geo.nodex;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        bc_fill_one(pr->W, geo, pr->bc, pr->ctl, e, pr->W32);
}

// every problem of a batch runs plain S2O4 (hos_batch2d_create): one instantiation per stage kind
// (update_one's KIND: 1 at stage 0, which gives the CFL candidates; 0 at stage 1 of an FP32
// batch, whose problems all have the FP32 mirror; -1, the generic form, at stage 1 of an FP64 batch)
template <int KIND>
__global__ void __launch_bounds__(256) update_batch_kernel(const Prob* __restrict__ probs, int stage) {
    const Prob* pr = probs + blockIdx.y;
    if (!pr->ctl->active) return;
    const Geometry geo = pr->geo;
    float* A32 = pr->W32 ? pr->W32 + 4 * (size_t)geo.nx * mirror_pitch(geo.ny) : nullptr;
    UpdateArgs a{pr->W, pr->Wold, pr->AX, pr->AY, pr->FXx, pr->FXy, pr->FAx, pr->FAy, pr->ctl, stage, pr->W32, A32};
    const int n = geo.nodex * geo.nodey;
    // the largest speed on the bit patterns (-1, +0 and positive speeds order as signed integers)
    long long smax = __double_as_longlong(-1.0);
    unsigned int bad = 0;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        double c;
        unsigned int b;
        update_one<false, KIND, (KIND >= 0)>(a, geo, base + threadIdx.x, c, b);
        const long long ck = __double_as_longlong(c);
        smax = ck > smax ? ck : smax;
        bad |= b;
    }
    reduce_block_speed(__longlong_as_double(smax), bad, pr->ctl, stage == cfl_stage(geo), geo);
}

// step prologue for every problem (one block); *counter is the batch step index
__global__ void begin_batch_kernel(const Prob* __restrict__ probs, int count, int* counter) {
    const int step = *counter;
    for (int p = threadIdx.x; p < count; p += blockDim.x) {
        const Prob* pr = probs + p;
        begin_step_one(pr->ctl, pr->tstop, pr->geo.dx);
        if (pr->ctl->active) *pr->last_step = step;
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter = step + 1;
}


// learned gate over all problems: one block per 16 x 16 tile of a problem's cells
struct GateTile { int p, i0, j0, pad; };

template <int ORDER>
__global__ void __launch_bounds__(gate::GATE_THREADS) gate_batch_kernel(const Prob* __restrict__ probs,
                                                                        const GateTile* __restrict__ tiles, int ntiles,
                                                                        gate::Net net, gate::Stats* stats, float threshold,
                                                                        unsigned audit_mask, unsigned seed) {
    __shared__ gate::MlpTc mlp;   // the network on the tcgen05 tensor cores, set up once per block
    if (blockIdx.x >= ntiles) return;
    gate::mlp_tc_setup(mlp, net);
    unsigned phase = 0;
    bool broken = false;
    for (int k = blockIdx.x; k < ntiles; k += gridDim.x) {
        const GateTile t = tiles[k];
        const Prob* pr = probs + t.p;
        gate::GateArgs a{pr->W, pr->AX, pr->AY, pr->gflags, stats, threshold, audit_mask, seed,
                         nullptr, 0, 0xffffffffu, pr->ctl, pr->W32};
        gate::gate_tile<ORDER>(a, pr->geo, t.i0, t.j0, (unsigned)k, mlp, phase, broken);
    }
    gate::mlp_tc_teardown(mlp, phase, broken);
}

thread_local std::string g_errb;
int failb(int code, const std::string& m) {
    g_errb = m;
    return code;
}

}  // namespace batch
}  // namespace hos

using namespace hos;
using namespace hos::batch;

struct hos_batch2d {
    int count = 0, order = 5, precision = 0;
    std::vector<hos_params2d> params;
    std::vector<Prob> host_probs;
    Prob* probs = nullptr;
    double* arena = nullptr;
    float* arena32 = nullptr;   // FP32 batches: every problem's FP32 mirror
    StepCtl* ctls = nullptr;
    int* last_step = nullptr;
    int* counter = nullptr;
    TileRef* tiles[2] = {nullptr, nullptr};
    int ntiles[2][kShapes] = {{0}};
    TileRef* tiles_by_shape[2][kShapes] = {{nullptr}};
    int shape[2] = {0, 0};
    int bps[2][kShapes] = {{1}};
    int sms = 1;
    double* staging = nullptr;
    size_t staging_cells = 0;
    long long cells = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    // learned gate (FP32 batches)
    int gated = 0;
    unsigned char* gflags = nullptr;
    gate::Stats* gstats = nullptr;
    __nv_bfloat16* gw = nullptr;
    float* gb = nullptr;
    GateTile* gtiles = nullptr;
    int ngtiles = 0;
    float gthreshold = 0.0f;
    unsigned gaudit_mask = 0;
    unsigned gseed = 0;
};

namespace {

void freeb(hos_batch2d* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (int d = 0; d < 2; ++d)
        for (int k = 0; k < kShapes; ++k)
            if (b->tiles_by_shape[d][k]) cudaFree(b->tiles_by_shape[d][k]);
    void* ptrs[] = {b->probs, b->arena, b->arena32, b->ctls, b->last_step, b->counter, b->staging,
                    b->gflags, b->gstats, b->gw, b->gb, b->gtiles};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
}

cudaError_t launch_faces(hos_batch2d* b, int dir, int stage) {
    const int sh = b->shape[dir];
    const int nt = b->ntiles[dir][sh];
    const int grid = std::max(1, std::min(nt, b->sms * std::max(1, b->bps[dir][sh])));
    const TileRef* t = b->tiles_by_shape[dir][sh];
    const int prec = b->gated ? 2 : b->precision;
    unsigned long long* fb = b->gated ? &b->gstats->fallback : nullptr;
    if (b->order == 5) return launch_batch_faces5(prec, sh, dir, b->probs, t, nt, stage, grid, b->stream, fb);
    if (b->order == 7) return launch_batch_faces7(prec, sh, dir, b->probs, t, nt, stage, grid, b->stream, fb);
    return launch_batch_faces9(prec, sh, dir, b->probs, t, nt, stage, grid, b->stream, fb);
}

int enqueue_batch_step(hos_batch2d* b) {
    cudaError_t e;
    begin_batch_kernel<<<1, 256, 0, b->stream>>>(b->probs, b->count, b->counter);
    int maxg = 0, maxc = 0;
    for (const auto& p : b->host_probs) {
        maxg = std::max(maxg, (int)((2LL * p.geo.g * (p.geo.ny + p.geo.nodex) + 255) / 256));
        maxc = std::max(maxc, (p.geo.nodex * p.geo.nodey + 255) / 256);
    }
    for (int stage = 0; stage < 2; ++stage) {
        bc_batch_kernel<<<dim3(std::min(maxg, 64), b->count), 256, 0, b->stream>>>(b->probs);
        if (b->gated) {
            const int grid = std::min(b->ngtiles, b->sms * 8);
            const gate::Net net{b->gw, b->gw + gate::NH * gate::NF, b->gw + gate::NH * gate::NF + gate::NH * gate::NH,
                                b->gb, b->gb + gate::NH, b->gb + 2 * gate::NH};
            const unsigned seed = b->gseed++;
            if (b->order == 5)
                gate_batch_kernel<5><<<grid, gate::GATE_THREADS, 0, b->stream>>>(b->probs, b->gtiles, b->ngtiles, net, b->gstats,
                                                                                 b->gthreshold, b->gaudit_mask, seed);
            else if (b->order == 7)
                gate_batch_kernel<7><<<grid, gate::GATE_THREADS, 0, b->stream>>>(b->probs, b->gtiles, b->ngtiles, net, b->gstats,
                                                                                 b->gthreshold, b->gaudit_mask, seed);
            else
                gate_batch_kernel<9><<<grid, gate::GATE_THREADS, 0, b->stream>>>(b->probs, b->gtiles, b->ngtiles, net, b->gstats,
                                                                                 b->gthreshold, b->gaudit_mask, seed);
        }
        if ((e = launch_faces(b, 0, stage)) != cudaSuccess) return failb(HOS_E_CUDA, std::string("face x: ") + cudaGetErrorString(e));
        if ((e = launch_faces(b, 1, stage)) != cudaSuccess) return failb(HOS_E_CUDA, std::string("face y: ") + cudaGetErrorString(e));
        const dim3 ugrid(std::min(maxc, 256), b->count);
        if (stage == 0)
            update_batch_kernel<1><<<ugrid, 256, 0, b->stream>>>(b->probs, stage);
        else if (b->arena32)
            update_batch_kernel<0><<<ugrid, 256, 0, b->stream>>>(b->probs, stage);
        else
            update_batch_kernel<-1><<<ugrid, 256, 0, b->stream>>>(b->probs, stage);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return failb(HOS_E_CUDA, std::string("batch step: ") + cudaGetErrorString(e));
    return HOS_OK;
}

}  // namespace

extern "C" {

const char* hos_batch2d_last_error(void) { return g_errb.c_str(); }

int hos_batch2d_create(const hos_params2d* params, const double* tstop, int count, int precision, hos_batch2d** out) {
    if (!params || !tstop || !out || count <= 0) return failb(HOS_E_ARG, "bad argument");
    const int order = params[0].order;
    for (int k = 0; k < count; ++k) {
        const hos_params2d& p = params[k];
        if (p.order != order) return failb(HOS_E_CONFIG, "all problems of a batch share the WENO-AO order");
        if (p.gausspoint != (order == 5 ? 2 : order == 7 ? 3 : 4) || !p.use_df || p.ghost < order / 2 + 1 ||
            p.nodex < p.ghost || p.nodey < p.ghost)
            return failb(HOS_E_CONFIG, "problem " + std::to_string(k) + ": bad order/gausspoint/ghost/size");
        for (int s = 0; s < 4; ++s)
            if (p.bc[s] < 0 || p.bc[s] > 5) return failb(HOS_E_CONFIG, "bad boundary kind");
        if (p.integrator != HOS_INT_S2O4 || p.flux != HOS_FLUX_GKS || p.tau_type != HOS_TAU_EULER)
            return failb(HOS_E_CONFIG, "batches run S2O4 with the Euler GKS flux");
        if (p.bc[0] >= 4 || p.bc[1] >= 4 || p.bc[2] == HOS_BC_WEDGE_TOP || p.bc[3] == HOS_BC_WEDGE_BOTTOM ||
            ((p.bc[2] >= 4 || p.bc[3] >= 4) && p.bc[0] != HOS_BC_INFLOW))
            return failb(HOS_E_CONFIG, "bad wedge boundary placement");
        if ((p.bc[0] == HOS_BC_PERIODIC) != (p.bc[1] == HOS_BC_PERIODIC) ||
            (p.bc[2] == HOS_BC_PERIODIC) != (p.bc[3] == HOS_BC_PERIODIC))
            return failb(HOS_E_CONFIG, "periodic boundaries must be paired");
    }
    if (precision != HOS_FP64 && precision != HOS_FP32) return failb(HOS_E_CONFIG, "bad precision");
    hos_batch2d* b = new (std::nothrow) hos_batch2d();
    if (!b) return failb(HOS_E_NOMEM, "host allocation");
    b->count = count;
    b->order = order;
    b->precision = precision;
    b->params.assign(params, params + count);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        freeb(b);
        delete b;
        return failb(HOS_E_CUDA, std::string("device: ") + cudaGetErrorString(e));
    }
    // one arena for every problem's buffers
    size_t total = 0, maxcells = 0, total32 = 0;
    std::vector<size_t> off(count), off32(count);
    for (int k = 0; k < count; ++k) {
        const hos_params2d& p = params[k];
        const size_t nc = (size_t)(p.nodex + 2 * p.ghost) * (p.nodey + 2 * p.ghost);
        const size_t nfx = (size_t)(p.nodex + 1) * p.nodey, nfy = (size_t)p.nodex * (p.nodey + 1);
        off[k] = total;
        total += 10 * nc + 9 * nfx + 9 * nfy;
        off32[k] = total32;
        total32 += (size_t)MIRROR_PLANES * (p.nodex + 2 * p.ghost) * mirror_pitch(p.nodey + 2 * p.ghost);
        maxcells = std::max(maxcells, nc);
        b->cells += (long long)p.nodex * p.nodey;
    }
    b->staging_cells = maxcells;
    auto alloc = [&](void** q, size_t bytes) {
        if (e != cudaSuccess) return;
        e = cudaMalloc(q, bytes);
        if (e == cudaSuccess) e = cudaMemset(*q, 0, bytes);
    };
    alloc((void**)&b->arena, total * sizeof(double));
    if (precision == HOS_FP32) alloc((void**)&b->arena32, total32 * sizeof(float));
    alloc((void**)&b->staging, 8 * maxcells * sizeof(double));
    alloc((void**)&b->ctls, count * sizeof(StepCtl));
    alloc((void**)&b->last_step, count * sizeof(int));
    alloc((void**)&b->counter, sizeof(int));
    alloc((void**)&b->probs, count * sizeof(Prob));
    if (e != cudaSuccess) {
        freeb(b);
        delete b;
        return failb(HOS_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b->host_probs.resize(count);
    std::vector<TileRef> tl[2][kShapes];
    for (int k = 0; k < count; ++k) {
        const hos_params2d& p = params[k];
        Prob& pr = b->host_probs[k];
        Geometry& geo = pr.geo;
        geo.g = p.ghost;
        geo.nodex = p.nodex;
        geo.nodey = p.nodey;
        geo.nx = p.nodex + 2 * p.ghost;
        geo.ny = p.nodey + 2 * p.ghost;
        geo.set_spacing((p.right - p.left) / p.nodex, (p.up - p.down) / p.nodey);
        geo.cfl = p.cfl;
        geo.gamma = p.gamma;
        geo.K = p.K;
        geo.c1 = p.c1_euler;
        geo.c2 = p.c2_euler;
        geo.characteristic = p.characteristic ? 1 : 0;
        for (int s = 0; s < 4; ++s) {
            pr.bc.kind[s] = p.bc[s];
            const double* q = p.bc_prim[s];
            pr.bc.inflow[s][0] = q[0];
            pr.bc.inflow[s][1] = q[0] * q[1];
            pr.bc.inflow[s][2] = q[0] * q[2];
            pr.bc.inflow[s][3] = q[0] * (q[3] / q[0] / (p.gamma - 1) + 0.5 * (q[1] * q[1] + q[2] * q[2]));
        }
        fill_wedge(pr.bc, p, geo.dx);
        const size_t nc = (size_t)geo.nx * geo.ny;
        const size_t nfx = (size_t)(p.nodex + 1) * p.nodey, nfy = (size_t)p.nodex * (p.nodey + 1);
        double* q = b->arena + off[k];
        pr.W = q; q += 4 * nc;
        pr.Wold = q; q += 4 * nc;
        pr.AX = q; q += nc;
        pr.AY = q; q += nc;
        pr.FXx = q; q += 4 * nfx;
        pr.FPx = q; q += 4 * nfx;
        pr.FAx = q; q += nfx;
        pr.FXy = q; q += 4 * nfy;
        pr.FPy = q; q += 4 * nfy;
        pr.FAy = q;
        pr.W32 = b->arena32 ? b->arena32 + off32[k] : nullptr;
        pr.ctl = b->ctls + k;
        pr.tstop = tstop[k];
        pr.last_step = b->last_step + k;
        for (int sh = 0; sh < kShapes; ++sh)
            for (int dir = 0; dir < 2; ++dir) {
                const int nN = (dir == 0 ? p.nodex : p.nodey) + 1, nT = dir == 0 ? p.nodey : p.nodex;
                for (int n0 = 0; n0 < nN; n0 += kShapeN[sh])
                    for (int t0 = 0; t0 < nT; t0 += kShapeT[sh]) tl[dir][sh].push_back(TileRef{k, n0, t0, 0});
            }
    }
    e = cudaMemcpy(b->probs, b->host_probs.data(), count * sizeof(Prob), cudaMemcpyHostToDevice);
    for (int dir = 0; dir < 2 && e == cudaSuccess; ++dir)
        for (int sh = 0; sh < kShapes && e == cudaSuccess; ++sh) {
            b->ntiles[dir][sh] = (int)tl[dir][sh].size();
            e = cudaMalloc(&b->tiles_by_shape[dir][sh], tl[dir][sh].size() * sizeof(TileRef));
            if (e == cudaSuccess)
                e = cudaMemcpy(b->tiles_by_shape[dir][sh], tl[dir][sh].data(), tl[dir][sh].size() * sizeof(TileRef),
                               cudaMemcpyHostToDevice);
        }
    if (e == cudaSuccess) {
        for (int dir = 0; dir < 2 && e == cudaSuccess; ++dir)
            e = order == 5 ? configure_batch5(precision, dir, b->bps[dir])
              : order == 7 ? configure_batch7(precision, dir, b->bps[dir])
                           : configure_batch9(precision, dir, b->bps[dir]);
    }
    if (e != cudaSuccess) {
        freeb(b);
        delete b;
        return failb(HOS_E_CUDA, std::string("batch setup: ") + cudaGetErrorString(e));
    }
    *out = b;
    return HOS_OK;
}

int hos_batch2d_destroy(hos_batch2d* b) {
    if (!b) return HOS_OK;
    cudaStreamSynchronize(b->stream);
    freeb(b);
    delete b;
    return HOS_OK;
}

int hos_batch2d_set_state(hos_batch2d* b, int k, const double* convar, const double* primvar) {
    if (!b || !convar || k < 0 || k >= b->count) return failb(HOS_E_ARG, "bad argument");
    const Prob& pr = b->host_probs[k];
    const size_t n = (size_t)pr.geo.nx * pr.geo.ny;
    double* stage = b->staging;
    double* prim = b->staging + 4 * b->staging_cells;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    cudaError_t e = cudaMemcpyAsync(stage, convar, 4 * n * sizeof(double), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) {
        aos_to_soa_kernel<<<blocks, 256, 0, b->stream>>>(stage, pr.W, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && primvar) {
        e = cudaMemcpyAsync(stage, primvar, 4 * n * sizeof(double), cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess) aos_to_soa_kernel<<<blocks, 256, 0, b->stream>>>(stage, prim, n);
    } else if (e == cudaSuccess) {
        prim_of_state_kernel<<<blocks, 256, 0, b->stream>>>(pr.W, prim, n, pr.geo.gamma);
    }
    StepCtl c{};
    double seed = pr.geo.dx;
    std::memcpy(&c.cfl_bits, &seed, sizeof seed);
    c.active = 1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(pr.ctl, &c, sizeof c, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) {
        cfl_from_prim_kernel<<<(pr.geo.nodex * pr.geo.nodey + 255) / 256, 256, 0, b->stream>>>(prim, pr.geo, pr.ctl);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(pr.AX, 0, n * sizeof(double), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(pr.AY, 0, n * sizeof(double), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(pr.last_step, 0xff, sizeof(int), b->stream);
    if (e == cudaSuccess && pr.W32) {
        const size_t n32 = (size_t)pr.geo.nx * mirror_pitch(pr.geo.ny);
        mirror_state_kernel<<<std::min(blocks, 4096u), 256, 0, b->stream>>>(pr.W, pr.AX, pr.AY, pr.W32, pr.W32 + 4 * n32,
                                                                             pr.geo.nx, pr.geo.ny);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return failb(HOS_E_CUDA, std::string("set_state: ") + cudaGetErrorString(e));
    StepCtl back;
    cudaMemcpy(&back, pr.ctl, sizeof back, cudaMemcpyDeviceToHost);
    if (back.status & 1u) return failb(HOS_E_BLOWUP, "problem " + std::to_string(k) + ": bad initial state");
    return HOS_OK;
}

int hos_batch2d_get_state(hos_batch2d* b, int k, double* convar, double* alpha_x, double* alpha_y) {
    if (!b || k < 0 || k >= b->count) return failb(HOS_E_ARG, "bad argument");
    const Prob& pr = b->host_probs[k];
    const size_t n = (size_t)pr.geo.nx * pr.geo.ny;
    cudaError_t e = cudaSuccess;
    if (convar) {
        soa_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, b->stream>>>(pr.W, b->staging, n);
        e = cudaMemcpyAsync(convar, b->staging, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    }
    if (e == cudaSuccess && alpha_x) e = cudaMemcpyAsync(alpha_x, pr.AX, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess && alpha_y) e = cudaMemcpyAsync(alpha_y, pr.AY, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    return e == cudaSuccess ? HOS_OK : failb(HOS_E_CUDA, std::string("get_state: ") + cudaGetErrorString(e));
}

// Times every tile shape on the batch's current state (face kernels only: they read the state
// and write per-face buffers that every stage rewrites) and keeps the fastest per direction.
int hos_batch2d_autotune(hos_batch2d* b, int reps, int* chosen, double* ms) {
    if (!b) return failb(HOS_E_ARG, "null batch");
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    // a valid dt in every control word for the trial launches, restored afterwards
    std::vector<StepCtl> saved(b->count);
    std::vector<int> saved_last(b->count);
    int saved_counter = 0;
    cudaError_t e = cudaMemcpy(saved.data(), b->ctls, b->count * sizeof(StepCtl), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(saved_last.data(), b->last_step, b->count * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&saved_counter, b->counter, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return failb(HOS_E_CUDA, "autotune save");
    begin_batch_kernel<<<1, 256, 0, b->stream>>>(b->probs, b->count, b->counter);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    reps = std::max(1, reps);
    for (int dir = 0; dir < 2; ++dir) {
        double best = 1e300;
        int best_sh = 0;
        for (int sh = 0; sh < kShapes; ++sh) {
            if (b->bps[dir][sh] <= 0) {
                if (ms) ms[dir * kShapes + sh] = -1.0;
                continue;
            }
            b->shape[dir] = sh;
            launch_faces(b, dir, 0);  // warm-up
            cudaEventRecord(e0, b->stream);
            for (int r = 0; r < reps; ++r) launch_faces(b, dir, 0);
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            if (ms) ms[dir * kShapes + sh] = t / reps;
            if (t < best) {
                best = t;
                best_sh = sh;
            }
        }
        b->shape[dir] = best_sh;
        if (chosen) chosen[dir] = best_sh;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) e = cudaMemcpy(b->ctls, saved.data(), b->count * sizeof(StepCtl), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->last_step, saved_last.data(), b->count * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->counter, &saved_counter, sizeof(int), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? HOS_OK : failb(HOS_E_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
}

int hos_batch2d_advance(hos_batch2d* b, int nsteps, int use_graph) {
    if (!b || nsteps < 0) return failb(HOS_E_ARG, "bad argument");
    cudaError_t e;
    if (use_graph) {
        if (!b->graph) {
            cudaGraph_t g;
            if ((e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                return failb(HOS_E_CUDA, "begin capture");
            int st = enqueue_batch_step(b);
            e = cudaStreamEndCapture(b->stream, &g);
            if (st) return st;
            if (e != cudaSuccess) return failb(HOS_E_CUDA, "end capture");
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return failb(HOS_E_CUDA, "graph instantiate");
        }
        for (int k = 0; k < nsteps; ++k)
            if ((e = cudaGraphLaunch(b->graph, b->stream)) != cudaSuccess) return failb(HOS_E_CUDA, "graph launch");
        return HOS_OK;
    }
    for (int k = 0; k < nsteps; ++k) {
        int st = enqueue_batch_step(b);
        if (st) return st;
    }
    return HOS_OK;
}

int hos_batch2d_status(hos_batch2d* b, int* active, double* t, int* last_step, int* failed) {
    if (!b) return failb(HOS_E_ARG, "null batch");
    cudaError_t e = cudaStreamSynchronize(b->stream);
    std::vector<StepCtl> c(b->count);
    if (e == cudaSuccess) e = cudaMemcpy(c.data(), b->ctls, b->count * sizeof(StepCtl), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && last_step) e = cudaMemcpy(last_step, b->last_step, b->count * sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return failb(HOS_E_CUDA, std::string("status: ") + cudaGetErrorString(e));
    int act = 0, bad = 0;
    for (int k = 0; k < b->count; ++k) {
        const int f = (int)(c[k].status & 1u);
        if (t) t[k] = c[k].t;
        if (failed) failed[k] = f;
        act += (c[k].t < b->host_probs[k].tstop && !f) ? 1 : 0;
        bad += f;
    }
    if (active) *active = act;
    if (!bad) return HOS_OK;
    // with per-problem flags the caller sees which problems failed; the others are intact
    return failed ? HOS_OK : failb(HOS_E_BLOWUP, std::to_string(bad) + " problem(s) of the batch blew up");
}

int hos_batch2d_set_reconstruction(hos_batch2d* b, int mode) {
    if (!b) return failb(HOS_E_ARG, "null batch");
    if (mode != HOS_RECON_WENO && mode != HOS_RECON_FIRST_ORDER) return failb(HOS_E_ARG, "bad reconstruction mode");
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return failb(HOS_E_CUDA, "set_reconstruction");
    for (auto& pr : b->host_probs) pr.geo.first_order = mode;
    // the face tiles read each problem's geometry from the table when they run, so a captured
    // step picks the change up without being captured again
    e = cudaMemcpy(b->probs, b->host_probs.data(), b->count * sizeof(Prob), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return failb(HOS_E_CUDA, "problem table");
    return HOS_OK;
}

int hos_batch2d_set_gate(hos_batch2d* b, const hos_gate* g, float threshold, int audit_log2) {
    using namespace gate;
    if (!b) return failb(HOS_E_ARG, "null batch");
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return failb(HOS_E_CUDA, "set_gate");
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (!g) {
        b->gated = 0;
        return HOS_OK;
    }
    if (b->precision != HOS_FP32) return failb(HOS_E_CONFIG, "the learned gate runs on the FP32-bulk path");
    if (audit_log2 < 0 || audit_log2 > 31) return failb(HOS_E_ARG, "audit_log2 must be 0..31");
    if (!b->gflags) {
        size_t total = 0;
        std::vector<GateTile> gt;
        for (int k = 0; k < b->count; ++k) {
            const Geometry& geo = b->host_probs[k].geo;
            total += (size_t)geo.nx * geo.ny;
            for (int i0 = 0; i0 < geo.nx; i0 += GATE_TILE)
                for (int j0 = 0; j0 < geo.ny; j0 += GATE_TILE) gt.push_back(GateTile{k, i0, j0, 0});
        }
        if ((e = cudaMalloc(&b->gflags, total)) == cudaSuccess && (e = cudaMemset(b->gflags, 0, total)) == cudaSuccess &&
            (e = cudaMalloc(&b->gstats, sizeof(Stats))) == cudaSuccess && (e = cudaMemset(b->gstats, 0, sizeof(Stats))) == cudaSuccess &&
            (e = cudaMalloc(&b->gw, NET_BF16 * sizeof(__nv_bfloat16))) == cudaSuccess &&
            (e = cudaMalloc(&b->gb, NET_F32 * sizeof(float))) == cudaSuccess &&
            (e = cudaMalloc(&b->gtiles, gt.size() * sizeof(GateTile))) == cudaSuccess)
            e = cudaMemcpy(b->gtiles, gt.data(), gt.size() * sizeof(GateTile), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return failb(HOS_E_NOMEM, std::string("gate buffers: ") + cudaGetErrorString(e));
        b->ngtiles = (int)gt.size();
        size_t off = 0;
        for (int k = 0; k < b->count; ++k) {
            const Geometry& geo = b->host_probs[k].geo;
            b->host_probs[k].gflags = b->gflags + off;
            off += (size_t)geo.nx * geo.ny;
        }
        e = cudaMemcpy(b->probs, b->host_probs.data(), b->count * sizeof(Prob), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return failb(HOS_E_CUDA, "problem table");
    }
    if ((e = cudaStreamSynchronize(g->stream)) == cudaSuccess &&
        (e = cudaMemcpy(b->gw, g->wbf, NET_BF16 * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice)) == cudaSuccess)
        e = cudaMemcpy(b->gb, g->bias, NET_F32 * sizeof(float), cudaMemcpyDeviceToDevice);
    for (int dir = 0; dir < 2 && e == cudaSuccess; ++dir) {
        int bps[kShapes] = {0, 0, 0};
        e = b->order == 5 ? configure_batch5(2, dir, bps) : b->order == 7 ? configure_batch7(2, dir, bps)
                                                                          : configure_batch9(2, dir, bps);
    }
    if (e != cudaSuccess) return failb(HOS_E_CUDA, std::string("set_gate: ") + cudaGetErrorString(e));
    b->gthreshold = threshold;
    b->gaudit_mask = audit_log2 == 31 ? 0xffffffffu : (1u << audit_log2) - 1u;
    b->gated = 1;
    return HOS_OK;
}

int hos_batch2d_gate_stats(hos_batch2d* b, unsigned long long* stats, int reset) {
    if (!b || !stats) return failb(HOS_E_ARG, "null argument");
    if (!b->gstats) {
        std::memset(stats, 0, 8 * sizeof(unsigned long long));
        return HOS_OK;
    }
    gate::Stats st;
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&st, b->gstats, sizeof st, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && reset) e = cudaMemset(b->gstats, 0, sizeof st);
    if (e != cudaSuccess) return failb(HOS_E_CUDA, "gate_stats");
    const unsigned long long v[8] = {st.cells[0], st.cells[1], st.smooth[0], st.smooth[1], st.audited, st.false_neg,
                                     st.fallback, st.samples};
    std::memcpy(stats, v, sizeof v);
    return HOS_OK;
}

long long hos_batch2d_cells(const hos_batch2d* b) { return b ? b->cells : 0; }
void* hos_batch2d_stream(hos_batch2d* b) { return b ? (void*)b->stream : nullptr; }

}  // extern "C"
