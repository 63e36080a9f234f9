// hos_solver.cu -- step kernels other than the face kernels, the C++ host solver and the
// C ABI declared in include/hos_gb300.h.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "../../include/hos_gb300.h"
#include "hos_gate.cuh"
#include "hos_launch.h"
#include "hos_step.cuh"

namespace hos {

// ghost fill; inside a step (skip_inactive) a finished problem does nothing.  ctl supplies the
// step's start time for the time-dependent wedge boundary.
__global__ void bc_fill_kernel(double* __restrict__ W, Geometry geo, BcSpec bc, const StepCtl* ctl, int skip_inactive,
                               float* W32) {
    if (skip_inactive && !ctl->active) return;
    bc_fill_one(W, geo, bc, ctl, blockIdx.x * (long long)blockDim.x + threadIdx.x, W32);
}

// FP32 mirrors of the whole state and of the DF indicators (after an upload), rows at the
// mirror's pitch
__global__ void mirror_state_kernel(const double* __restrict__ W, const double* __restrict__ AX,
                                    const double* __restrict__ AY, float* __restrict__ W32, float* __restrict__ A32,
                                    int nx, int ny) {
    const size_t n = (size_t)nx * ny, pitch = (size_t)mirror_pitch(ny), n32 = (size_t)nx * pitch;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t cm = (c / ny) * pitch + c % ny;
#pragma unroll
        for (int v = 0; v < 4; ++v) W32[v * n32 + cm] = (float)W[v * n + c];
        A32[cm] = (float)AX[c];
        A32[n32 + cm] = (float)AY[c];
    }
}

// ------------------------------------------------------------------------------------------
// update: W = Wold + (sum of face fluxes x length) / area over the interior cells
// (Update_with_gauss, src/time_advance.cpp:431-474), the DF indicators of the cell
// (Update_alpha, src/reconstruction.cpp:1523-1534) and, at stage 0, the CFL candidates of the
// new state for the next step (Get_CFL / Dtx, src/time_advance.cpp:264-305: the reference
// reads primitive variables refreshed at the start of the last stage).
// ------------------------------------------------------------------------------------------


__global__ void __launch_bounds__(256) update_kernel(UpdateArgs a, Geometry geo) {
    if (!a.ctl->active) return;
    double spd;
    unsigned int bad;
    update_one(a, geo, blockIdx.x * blockDim.x + threadIdx.x, spd, bad);
    reduce_block_speed(spd, bad, a.ctl, a.stage == cfl_stage(geo), geo);
}
// the same for fluxes stored per unit cell width (Geometry::scaled_flux, plain S2O4, the FP32
// mirror present), one instantiation per stage kind (update_one's KIND: 1 at stage 0, which
// gives the CFL candidates, 0 at stage 1)
template <int KIND>
__global__ void __launch_bounds__(256) update_kernel_scaled(UpdateArgs a, Geometry geo) {
    if (!a.ctl->active) return;
    double spd;
    unsigned int bad;
    update_one<true, KIND>(a, geo, blockIdx.x * blockDim.x + threadIdx.x, spd, bad);
    reduce_block_speed(spd, bad, a.ctl, KIND == 1, geo);
}

// CFL candidates from a primitive state (the initial data's primvar at step 0)
__global__ void __launch_bounds__(256) cfl_from_prim_kernel(const double* __restrict__ prim, Geometry geo, StepCtl* ctl) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    double spd = -1.0;
    unsigned int bad = 0;
    if (idx < geo.nodex * geo.nodey) {
        const int I = idx / geo.nodey, J = idx % geo.nodey;
        const size_t plane = (size_t)geo.nx * geo.ny;
        const size_t c = (size_t)(I + geo.g) * geo.ny + (J + geo.g);
        const double rho = prim[c], u = prim[plane + c], v = prim[2 * plane + c], p = prim[3 * plane + c];
        spd = signal_speed(sqrt(u * u + v * v) + sqrt(geo.gamma * p / rho));
        if (rho < 0 || p < 0 || isnan(rho) || isnan(p)) bad = 1;
    }
    reduce_block_speed<true>(spd, bad, ctl, true, geo);
}

__global__ void begin_step_kernel(StepCtl* ctl, double tstop, double seed) { begin_step_one(ctl, tstop, seed); }

// AoS [cells][4] <-> SoA [4][cells] transposes for the host-facing entry points
__global__ void aos_to_soa_kernel(const double* __restrict__ aos, double* __restrict__ soa, size_t n) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= n) return;
    for (int v = 0; v < 4; ++v) soa[v * n + c] = aos[4 * c + v];
}
// SoA -> AoS staged through shared memory, so that each warp writes 256 contiguous bytes: the
// destination may be pinned host memory written over the host link, where a warp's strided
// 8-byte stores would each move a partial line.  blockDim.x == 256.
__global__ void __launch_bounds__(256) soa_to_aos_kernel(const double* __restrict__ soa, double* __restrict__ aos,
                                                         size_t n) {
    __shared__ double t[4][256];
    const size_t c0 = (size_t)blockIdx.x * 256;
    const int tid = threadIdx.x;
    if (c0 + tid < n)
        for (int v = 0; v < 4; ++v) t[v][tid] = soa[v * n + c0 + tid];
    __syncthreads();
    const int m = (int)(n - c0 < 256 ? n - c0 : 256) * 4;
    for (int k = tid; k < m; k += 256) aos[4 * c0 + k] = t[k & 3][k >> 2];
}
// The host-facing upload in one pass over the cells (hos2d_set_state): the staged AoS conserved
// state into the SoA planes, the DF indicators zeroed, the FP32 mirror (if any) written, and for
// interior cells the CFL candidates of the primitives -- the staged AoS primvar if given, else
// the state's own (Convar_to_primvar_2D) -- with the same arithmetic as cfl_from_prim_kernel.
__global__ void __launch_bounds__(256) upload_state_kernel(const double* __restrict__ aos,
                                                           const double* __restrict__ prim_aos, double* __restrict__ W,
                                                           double* __restrict__ AX, double* __restrict__ AY,
                                                           float* __restrict__ W32, Geometry geo, StepCtl* ctl) {
    const size_t n = (size_t)geo.nx * geo.ny;
    const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    double spd = -1.0;
    unsigned int bad = 0;
    if (c < n) {
        double w[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            w[v] = aos[4 * c + v];
            W[v * n + c] = w[v];
        }
        AX[c] = 0.0;
        AY[c] = 0.0;
        const int i = (int)(c / geo.ny), j = (int)(c % geo.ny);
        if (W32) {
            const size_t pitch = (size_t)mirror_pitch(geo.ny), plane32 = (size_t)geo.nx * pitch;
            const size_t cm = (size_t)i * pitch + j;
#pragma unroll
            for (int v = 0; v < 4; ++v) W32[v * plane32 + cm] = (float)w[v];
            W32[4 * plane32 + cm] = 0.0f;
            W32[5 * plane32 + cm] = 0.0f;
        }
        if (i >= geo.g && i < geo.g + geo.nodex && j >= geo.g && j < geo.g + geo.nodey) {
            double p[4];
            if (prim_aos) {
#pragma unroll
                for (int v = 0; v < 4; ++v) p[v] = prim_aos[4 * c + v];
            } else {
                to_prim<double>(p, w, geo.gamma);
            }
            const double rho = p[0], u = p[1], v = p[2], pr = p[3];
            spd = signal_speed(sqrt(u * u + v * v) + sqrt(geo.gamma * pr / rho));
            if (rho < 0 || pr < 0 || isnan(rho) || isnan(pr)) bad = 1;
        }
    }
    reduce_block_speed<true>(spd, bad, ctl, true, geo);
}

// primitive variables of a conserved state (Convar_to_primvar_2D, src/basic_function.cpp:811-817)
__global__ void prim_of_state_kernel(const double* __restrict__ W, double* __restrict__ P, size_t n, double gamma) {
    size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (c >= n) return;
    double w[4], p[4];
    for (int v = 0; v < 4; ++v) w[v] = W[v * n + c];
    to_prim<double>(p, w, gamma);
    for (int v = 0; v < 4; ++v) P[v * n + c] = p[v];
}

// The gate's flags of the step's first stage for a later stage: a cell keeps its x (y) bit only
// when its neighbours along x (y) have it too.  Within a stage a front moves by at most a
// quarter cell (CFL 0.5, half a step), so it cannot enter a stencil that a flagged neighbour's
// stencil, one cell further out, did not already see.
__global__ void __launch_bounds__(256) dilate_flags_kernel(const unsigned char* __restrict__ f0,
                                                           unsigned char* __restrict__ f1, int nx, int ny,
                                                           const StepCtl* ctl) {
    if (!ctl->active) return;
    const size_t n = (size_t)nx * ny;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c / ny), j = (int)(c % ny);
        unsigned x = f0[c] & 1u, y = f0[c] & 2u;
        if (x) x = i > 0 && i + 1 < nx ? f0[c - ny] & f0[c + ny] & 1u : 0u;
        if (y) y = j > 0 && j + 1 < ny ? f0[c - 1] & f0[c + 1] & 2u : 0u;
        f1[c] = (unsigned char)(x | y);
    }
}

// one block waits on an mbarrier that expects one arrival and receives none: the bounded wait
// must give up and report (hos_wait_limit_selftest)
__global__ void wait_limit_selftest_kernel(unsigned* out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const bool done = mbar_wait(&bar, 0);
    if (threadIdx.x == 0) *out = done ? 1u : 2u;
}

// f32_to_f64 over an array (hos_convert_selftest)
__global__ void convert_selftest_kernel(const float* __restrict__ x, double* __restrict__ y, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = f32_to_f64(x[i]);
}

static thread_local std::string g_last_error;

// conserved wedge states and geometry (Primvar_to_convar_2D on the primitive states)
void fill_wedge(BcSpec& bc, const hos_params2d& p, double dx) {
    auto con = [&](const double* q, double* w) {
        w[0] = q[0];
        w[1] = q[0] * q[1];
        w[2] = q[0] * q[2];
        w[3] = q[0] * (q[3] / q[0] / (p.gamma - 1) + 0.5 * (q[1] * q[1] + q[2] * q[2]));
    };
    con(p.wedge_post, bc.wpost);
    con(p.wedge_pre, bc.wpre);
    bc.wx0 = p.wedge_x0;
    bc.wthr0 = p.wedge_x0 + (p.up - p.down) / sqrt(3.0);
    bc.wspeed = p.wedge_top_speed;
    bc.left = p.left;
    bc.dx = dx;
}

static int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
// The device address of a pinned host buffer (cudaHostAlloc, cudaMallocHost, cudaHostRegister:
// under unified addressing every pinned allocation is mapped), else nullptr.  The host-facing
// transfers read and write such buffers from their kernels over the host link, which moves the
// data at the copy engine's rate and leaves out the staging pass on the device.
static const void* mapped_host(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

static int cuda_fail(cudaError_t e, const char* where) {
    return fail(HOS_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Tensor maps of the FP32 mirror (base: nx rows of ny cells at pitch mirror_pitch(ny), six
// planes) with the x-face and the y-face tile boxes of the given WENO order's TMA face tile and
// the gate tile's box.  The encoder is
// the driver's cuTensorMapEncodeTiled, fetched through the runtime so that the library does not
// link libcuda.  Cells past ny in a row read as zero (the out-of-bounds fill).
static int encode_mirror_maps(CUtensorMap* maps, float* base, int nx, int ny, int order) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return fail(HOS_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    int bx[3], by[3];
    switch (order) {
        case 5: bx[0] = TmaBox<5, 0, TmaTile<5>>::X; by[0] = TmaBox<5, 0, TmaTile<5>>::Y;
                 bx[1] = TmaBox<5, 1, TmaTile<5>>::X; by[1] = TmaBox<5, 1, TmaTile<5>>::Y;
                 bx[2] = gate::GateBox<5>::X; by[2] = gate::GateBox<5>::Y; break;
        case 7: bx[0] = TmaBox<7, 0, TmaTile<7>>::X; by[0] = TmaBox<7, 0, TmaTile<7>>::Y;
                 bx[1] = TmaBox<7, 1, TmaTile<7>>::X; by[1] = TmaBox<7, 1, TmaTile<7>>::Y;
                 bx[2] = gate::GateBox<7>::X; by[2] = gate::GateBox<7>::Y; break;
        default: bx[0] = TmaBox<9, 0, TmaTile<9>>::X; by[0] = TmaBox<9, 0, TmaTile<9>>::Y;
                 bx[1] = TmaBox<9, 1, TmaTile<9>>::X; by[1] = TmaBox<9, 1, TmaTile<9>>::Y;
                 bx[2] = gate::GateBox<9>::X; by[2] = gate::GateBox<9>::Y; break;
    }
    const cuuint64_t pitch = (cuuint64_t)mirror_pitch(ny);
    const cuuint64_t dims[3] = {(cuuint64_t)ny, (cuuint64_t)nx, (cuuint64_t)MIRROR_PLANES};
    const cuuint64_t strides[2] = {pitch * sizeof(float), pitch * (cuuint64_t)nx * sizeof(float)};
    const cuuint32_t es[3] = {1, 1, 1};
    for (int d = 0; d < 3; ++d) {
        const cuuint32_t box[3] = {(cuuint32_t)bx[d], (cuuint32_t)by[d], (cuuint32_t)MIRROR_PLANES};
        CUresult r = encode(&maps[d], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(HOS_E_CUDA, "cuTensorMapEncodeTiled failed on the FP32 mirror (code " +
                                                       std::to_string((int)r) + ")");
    }
    return HOS_OK;
}

}  // namespace hos

using namespace hos;

struct hos_solver2d {
    hos_params2d p;
    int precision = 0;
    Geometry geo;
    BcSpec bc;
    size_t ncell = 0, nfx = 0, nfy = 0;
    cudaStream_t stream = nullptr;
    int device = 0;
    // device buffers
    double* W = nullptr;
    double* Wold = nullptr;
    double* AX = nullptr;
    double* AY = nullptr;
    double* FXx = nullptr;
    double* FPx = nullptr;
    double* FAx = nullptr;
    double* FXy = nullptr;
    double* FPy = nullptr;
    double* FAy = nullptr;
    double* scratch = nullptr;  // 8 * ncell doubles: AoS staging + primitive planes
    float* W32 = nullptr;       // FP32 solvers: mirror of W [4][nx*P] ...
    float* A32 = nullptr;       // ... and of alpha_x | alpha_y [2][nx*P] (inside the W32 allocation)
    CUtensorMap tmap[3];        // FP32 solvers: the mirror's tensor maps with the x- / y-face boxes
                                // and the gate tile's box
    double* stagex = nullptr;   // methods other than S2O4: per-stage F and D of x faces [2][4][4][nfx]
    double* stagey = nullptr;   // ... and of y faces
    StepCtl* ctl = nullptr;
    StepCtl* hctl = nullptr;    // pinned host copy: control-word uploads and read-backs on the stream
    // captured step
    cudaGraphExec_t graph = nullptr;
    double graph_tstop = 0.0;
    // learned gate (FP32 path): per-cell flags, counters, the network's inference copy
    int gated = 0;
    unsigned char* gflags = nullptr;
    // the network runs at stage 0 only; later stages take its flags dilated by one cell along
    // each flag's axis (gflags2)
    int greuse = 0;
    unsigned char* gflags2 = nullptr;
    gate::Stats* gstats = nullptr;
    __nv_bfloat16* gw = nullptr;
    float* gb = nullptr;
    float gthreshold = 0.0f;
    unsigned gaudit_mask = 0;
    unsigned gseed = 0;
    gate::Net gnet() const {
        using namespace gate;
        return Net{gw, gw + NH * NF, gw + NH * NF + NH * NH, gb, gb + NH, gb + 2 * NH};
    }
};

namespace {

int check_boundaries(const hos_params2d& p) {
    auto wedge = [](int k) { return k == HOS_BC_WEDGE_BOTTOM || k == HOS_BC_WEDGE_TOP; };
    for (int k = 0; k < 4; ++k)
        if (p.bc[k] < 0 || p.bc[k] > HOS_BC_NOSLIP) return fail(HOS_E_CONFIG, "bad boundary kind");
    if (wedge(p.bc[0]) || wedge(p.bc[1]) || (p.bc[2] == HOS_BC_WEDGE_TOP) || (p.bc[3] == HOS_BC_WEDGE_BOTTOM))
        return fail(HOS_E_CONFIG, "wedge boundaries: HOS_BC_WEDGE_BOTTOM on the bottom, HOS_BC_WEDGE_TOP on the top");
    if ((wedge(p.bc[2]) || wedge(p.bc[3])) && p.bc[0] != HOS_BC_INFLOW)
        return fail(HOS_E_CONFIG, "wedge boundaries need an inflow left boundary");
    if ((p.bc[0] == HOS_BC_PERIODIC) != (p.bc[1] == HOS_BC_PERIODIC) ||
        (p.bc[2] == HOS_BC_PERIODIC) != (p.bc[3] == HOS_BC_PERIODIC))
        return fail(HOS_E_CONFIG, "periodic boundaries must be paired");
    return HOS_OK;
}

void fill_boundaries(BcSpec& bc, const hos_params2d& p, double dx) {
    for (int k = 0; k < 4; ++k) {
        bc.kind[k] = p.bc[k];
        const double* q = p.bc_prim[k];  // Primvar_to_convar_2D (src/basic_function.cpp:851-857)
        bc.inflow[k][0] = q[0];
        bc.inflow[k][1] = q[0] * q[1];
        bc.inflow[k][2] = q[0] * q[2];
        bc.inflow[k][3] = q[0] * (q[3] / q[0] / (p.gamma - 1) + 0.5 * (q[1] * q[1] + q[2] * q[2]));
        bc.wall[k][0] = q[1];   // no-slip wall velocity (bcvalue.primvar[1..2])
        bc.wall[k][1] = q[2];
    }
    fill_wedge(bc, p, dx);
}

void free_all(hos_solver2d* s) {
    double* bufs[] = {s->W, s->Wold, s->AX, s->AY, s->FXx, s->FPx, s->FAx, s->FXy, s->FPy, s->FAy, s->scratch,
                      s->stagex, s->stagey};
    for (double* b : bufs)
        if (b) cudaFree(b);
    if (s->ctl) cudaFree(s->ctl);
    if (s->hctl) cudaFreeHost(s->hctl);
    void* gbufs[] = {s->gflags, s->gflags2, s->gstats, s->gw, s->gb, s->W32};
    for (void* b : gbufs)
        if (b) cudaFree(b);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->stream) cudaStreamDestroy(s->stream);
}

// ev (optional): 5 events, after the boundary fill, the gate (recorded with no launch when the
// solver has no gate), the x faces, the y faces and the update
int enqueue_stage(hos_solver2d* s, int stage, cudaEvent_t* ev = nullptr) {
    cudaError_t e;
    const Geometry& geo = s->geo;
    auto mark = [&](int k) {
        if (ev) cudaEventRecord(ev[k], s->stream);
    };
    {
        const long long n = 2LL * geo.g * geo.ny + 2LL * geo.g * geo.nodex;
        bc_fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(s->W, geo, s->bc, s->ctl, 1, s->W32);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "bc_fill");
        mark(0);
    }
    FaceArgs ax{s->W, s->AX, s->AY, s->FXx, s->FPx, s->FAx, s->ctl, stage};
    FaceArgs ay{s->W, s->AY, s->AX, s->FXy, s->FPy, s->FAy, s->ctl, stage};
    if (s->W32) {
        ax.W32 = ay.W32 = s->W32;
        ax.AN32 = ay.AT32 = s->A32;
        ax.AT32 = ay.AN32 = s->A32 + s->ncell;
    }
    if (s->stagex) {
        ax.FS = s->stagex;
        ax.DS = s->stagex + 16 * s->nfx;
        ay.FS = s->stagey;
        ay.DS = s->stagey + 16 * s->nfy;
    }
    if (s->gated && (stage == 0 || !s->greuse)) {
        // per-cell smoothness flags of this stage's state (ghosts filled) for both directions
        gate::GateArgs ga{s->W, s->AX, s->AY, s->gflags, s->gstats, s->gthreshold, s->gaudit_mask, s->gseed++,
                          nullptr, 0, 0xffffffffu, s->ctl, s->W32};
        if ((e = gate::launch_gate(s->p.order, ga, s->gnet(), geo, s->stream, s->W32 ? &s->tmap[2] : nullptr)) !=
            cudaSuccess)
            return cuda_fail(e, "gate");
        ax.gate = ay.gate = s->gflags;
        ax.fallback = ay.fallback = &s->gstats->fallback;
        ax.fn_check = ay.fn_check = &s->gstats->fn_linear;
    } else if (s->gated) {
        const size_t n = s->ncell;
        dilate_flags_kernel<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s->stream>>>(
            s->gflags, s->gflags2, geo.nx, geo.ny, s->ctl);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "dilate_flags");
        ax.gate = ay.gate = s->gflags2;
        ax.fallback = ay.fallback = &s->gstats->fallback;
    }
    mark(1);
    // x faces then y faces, back to back on the stream (events after each when profiling)
    const int prec = geo.tau_type == HOS_TAU_NS ? (s->precision == HOS_FP64 ? 3 : 4) : s->gated ? 2 : s->precision;
    // FP32 solvers stage their tiles from the mirror with TMA tile loads
    const CUtensorMap* tm = s->W32 ? s->tmap : nullptr;
    e = launch_faces(s->p.order, prec, ax, ay, geo, s->stream, ev ? ev + 2 : nullptr, tm);
    if (e != cudaSuccess) return cuda_fail(e, "face_kernel");
    UpdateArgs ua{s->W, s->Wold, s->AX, s->AY, s->FXx, s->FXy, s->FAx, s->FAy, s->ctl, stage, s->W32, s->A32};
    const int n = geo.nodex * geo.nodey;
    if (geo.scaled_flux && geo.integrator == HOS_INT_S2O4 && !geo.source) {   // FP32 solvers: W32 set
        if (stage == cfl_stage(geo))
            update_kernel_scaled<1><<<(n + 255) / 256, 256, 0, s->stream>>>(ua, geo);
        else
            update_kernel_scaled<0><<<(n + 255) / 256, 256, 0, s->stream>>>(ua, geo);
    } else
        update_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(ua, geo);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "update");
    mark(4);
    return HOS_OK;
}

int enqueue_begin(hos_solver2d* s, double tstop) {
    begin_step_kernel<<<1, 1, 0, s->stream>>>(s->ctl, tstop, s->geo.dx);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HOS_OK : cuda_fail(e, "begin_step");
}

int enqueue_step(hos_solver2d* s, double tstop) {
    int st = enqueue_begin(s, tstop);
    if (st) return st;
    for (int k = 0; k < s->geo.stages; ++k)
        if ((st = enqueue_stage(s, k)) != HOS_OK) return st;
    return HOS_OK;
}

cudaError_t refresh_mirror(hos_solver2d* s) {
    if (!s->W32) return cudaSuccess;
    mirror_state_kernel<<<(unsigned)std::min<size_t>((s->ncell + 255) / 256, 4096), 256, 0, s->stream>>>(
        s->W, s->AX, s->AY, s->W32, s->A32, s->geo.nx, s->geo.ny);
    return cudaGetLastError();
}

int reset_ctl_and_cfl(hos_solver2d* s, const double* dprim_soa) {
    StepCtl c{};
    c.dt = 0.0;
    c.t = 0.0;
    double seed = s->geo.dx;
    std::memcpy(&c.cfl_bits, &seed, sizeof seed);
    c.status = 0;
    c.active = 1;
    cudaError_t e = cudaMemcpyAsync(s->ctl, &c, sizeof c, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "ctl upload");
    const int n = s->geo.nodex * s->geo.nodey;
    cfl_from_prim_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(dprim_soa, s->geo, s->ctl);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "cfl_from_prim");
    if ((e = cudaMemsetAsync(s->AX, 0, s->ncell * sizeof(double), s->stream)) != cudaSuccess) return cuda_fail(e, "memset");
    if ((e = cudaMemsetAsync(s->AY, 0, s->ncell * sizeof(double), s->stream)) != cudaSuccess) return cuda_fail(e, "memset");
    if ((e = refresh_mirror(s)) != cudaSuccess) return cuda_fail(e, "mirror");
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cuda_fail(e, "set_state");
    StepCtl back;
    if ((e = cudaMemcpy(&back, s->ctl, sizeof back, cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_fail(e, "ctl read");
    if (back.status & 1u) return fail(HOS_E_BLOWUP, "initial state has negative density/pressure or NaN");
    return HOS_OK;
}

}  // namespace

extern "C" {

const char* hos_last_error(void) { return g_last_error.c_str(); }

int hos_wait_limit_selftest(void) {
    unsigned* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(unsigned));
    if (e != cudaSuccess) return cuda_fail(e, "selftest alloc");
    unsigned h = 0;
    if ((e = cudaMemset(d, 0, sizeof(unsigned))) == cudaSuccess) {
        wait_limit_selftest_kernel<<<1, 32>>>(d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "selftest");
    if (h == 2u) return fail(HOS_E_TIMEOUT, "the wait gave up at its limit (expected)");
    return h == 1u ? fail(HOS_OK, "the wait completed: the barrier was not expected to") : fail(HOS_E_CUDA, "no result");
}

int hos_convert_selftest(const float* x, double* y, size_t n) {
    if ((!x || !y) && n) return fail(HOS_E_ARG, "null argument");
    if (n == 0) return HOS_OK;
    float* dx = nullptr;
    double* dy = nullptr;
    cudaError_t e = cudaMalloc(&dx, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dy, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        convert_selftest_kernel<<<(unsigned)((n + 255) / 256), 256>>>(dx, dy, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(y, dy, n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    return e == cudaSuccess ? HOS_OK : cuda_fail(e, "convert selftest");
}

int hos2d_create(const hos_params2d* params, int precision, hos_solver2d** out) {
    if (!params || !out) return fail(HOS_E_ARG, "null argument");
    const hos_params2d& p = *params;
    if (!(p.order == 5 || p.order == 7 || p.order == 9)) return fail(HOS_E_CONFIG, "order must be 5, 7 or 9");
    const int need_gp = p.order == 5 ? 2 : p.order == 7 ? 3 : 4;
    if (p.gausspoint != need_gp) return fail(HOS_E_CONFIG, "gausspoint must be 2/3/4 for order 5/7/9");
    // use_df = 0: the drivers' default WENO5_AO_normal / WENO5_AO_tangent, which exist for
    // WENO5 only (and write the Gauss points only with gausspoint = 2, :2264, :2279)
    if (!p.use_df && p.order != 5)
        return fail(HOS_E_CONFIG, "without the DF factor (use_df = 0) the reconstruction is WENO5-AO: order must be 5");
    if (!p.use_df && (p.wenotype < HOS_WENO_Z || p.wenotype > HOS_WENO_LINEAR))
        return fail(HOS_E_CONFIG, "wenotype must be HOS_WENO_Z, HOS_WENO_JS or HOS_WENO_LINEAR");
    if (p.ghost < p.order / 2 + 1) return fail(HOS_E_CONFIG, "ghost must be >= order/2 + 1");
    if (p.nodex < p.ghost || p.nodey < p.ghost) return fail(HOS_E_CONFIG, "nodex and nodey must be >= ghost");
    if (precision != HOS_FP64 && precision != HOS_FP32) return fail(HOS_E_CONFIG, "precision must be HOS_FP64 or HOS_FP32");
    if (int st = check_boundaries(p)) return st;
    if (p.integrator < HOS_INT_S2O4 || p.integrator > HOS_INT_RK4) return fail(HOS_E_CONFIG, "bad time-marching method");
    if (p.flux != HOS_FLUX_GKS && p.flux != HOS_FLUX_LF) return fail(HOS_E_CONFIG, "bad flux");
    if (p.tau_type != HOS_TAU_EULER && p.tau_type != HOS_TAU_NS) return fail(HOS_E_CONFIG, "bad tau_type");
    if (p.prandtl_fix && !(p.prandtl > 0)) return fail(HOS_E_CONFIG, "the Prandtl fix needs prandtl > 0");
    if (p.tau_type == HOS_TAU_NS && p.flux == HOS_FLUX_LF && !(p.prandtl > 0))
        return fail(HOS_E_CONFIG, "LF2D's viscous term divides by the Prandtl number: prandtl must be > 0");
    hos_solver2d* s = new (std::nothrow) hos_solver2d();
    if (!s) return fail(HOS_E_NOMEM, "host allocation");
    s->p = p;
    s->precision = precision;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) { delete s; return cuda_fail(e, "cudaGetDevice"); }
    Geometry& geo = s->geo;
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
    geo.plain = p.use_df ? 0 : 1;
    geo.wenotype = p.use_df ? 0 : p.wenotype;
    geo.integrator = p.integrator;
    geo.flux = p.flux;
    geo.stages = integrator_stages(p.integrator);
    geo.tau_type = p.tau_type;
    geo.mu = p.mu;
    geo.nu = p.nu;
    geo.prandtl_coef = p.tau_type == HOS_TAU_NS && p.prandtl_fix ? 1.0 / p.prandtl - 1.0 : 0.0;
    geo.prandtl = p.prandtl;
    geo.scaled_flux = precision == HOS_FP32 ? 1 : 0;
    fill_boundaries(s->bc, p, geo.dx);
    s->ncell = (size_t)geo.nx * geo.ny;
    s->nfx = (size_t)(geo.nodex + 1) * geo.nodey;
    s->nfy = (size_t)geo.nodex * (geo.nodey + 1);
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete s;
        return cuda_fail(e, "stream");
    }
    struct { double** p; size_t n; } allocs[] = {
        {&s->W, 4 * s->ncell}, {&s->Wold, 4 * s->ncell}, {&s->AX, s->ncell}, {&s->AY, s->ncell},
        {&s->FXx, 4 * s->nfx}, {&s->FPx, 4 * s->nfx}, {&s->FAx, s->nfx},
        {&s->FXy, 4 * s->nfy}, {&s->FPy, 4 * s->nfy}, {&s->FAy, s->nfy}, {&s->scratch, 8 * s->ncell},
        {&s->stagex, p.integrator ? 32 * s->nfx : 0}, {&s->stagey, p.integrator ? 32 * s->nfy : 0}};
    for (auto& a : allocs) {
        if (a.n == 0) continue;
        if ((e = cudaMalloc(a.p, a.n * sizeof(double))) != cudaSuccess) {
            free_all(s);
            delete s;
            return fail(HOS_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        cudaMemset(*a.p, 0, a.n * sizeof(double));
    }
    if ((e = cudaMalloc(&s->ctl, sizeof(StepCtl))) != cudaSuccess ||
        (e = cudaMallocHost(&s->hctl, sizeof(StepCtl))) != cudaSuccess) {
        free_all(s);
        delete s;
        return fail(HOS_E_NOMEM, "ctl allocation");
    }
    if (precision == HOS_FP32) {
        const size_t n32 = (size_t)s->geo.nx * mirror_pitch(s->geo.ny);
        if ((e = cudaMalloc(&s->W32, MIRROR_PLANES * n32 * sizeof(float))) != cudaSuccess ||
            (e = cudaMemset(s->W32, 0, MIRROR_PLANES * n32 * sizeof(float))) != cudaSuccess) {
            free_all(s);
            delete s;
            return fail(HOS_E_NOMEM, "cudaMalloc FP32 mirror");
        }
        s->A32 = s->W32 + 4 * n32;
        const int st = encode_mirror_maps(s->tmap, s->W32, s->geo.nx, s->geo.ny, p.order);
        if (st != HOS_OK) {
            free_all(s);
            delete s;
            return st;
        }
    }
    cudaMemset(s->ctl, 0, sizeof(StepCtl));
    const int variant = p.tau_type == HOS_TAU_NS ? (precision == HOS_FP64 ? 3 : 4) : precision;
    e = configure_faces(s->geo, p.order, variant);
    if (e != cudaSuccess) {
        free_all(s);
        delete s;
        return cuda_fail(e, "configure face kernels");
    }
    *out = s;
    return HOS_OK;
}

int hos2d_destroy(hos_solver2d* s) {
    if (!s) return HOS_OK;
    cudaStreamSynchronize(s->stream);
    free_all(s);
    delete s;
    return HOS_OK;
}

int hos2d_dims(const hos_solver2d* s, int* nx, int* ny) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    if (nx) *nx = s->geo.nx;
    if (ny) *ny = s->geo.ny;
    return HOS_OK;
}

int hos2d_set_state(hos_solver2d* s, const double* convar, const double* primvar) {
    if (!s || !convar) return fail(HOS_E_ARG, "null argument");
    const size_t n = s->ncell;
    // one pass (upload_state_kernel) for the transposition, the DF indicators, the FP32 mirror
    // and the first CFL candidates; it reads pinned host buffers over the host link, other
    // buffers from a device staging copy (AoS [n][4] of convar, then of primvar)
    const double* src = static_cast<const double*>(mapped_host(convar));
    const double* src_prim = primvar ? static_cast<const double*>(mapped_host(primvar)) : nullptr;
    cudaError_t e = cudaSuccess;
    if (!src) {
        double* stage = s->scratch;
        if ((e = cudaMemcpyAsync(stage, convar, 4 * n * sizeof(double), cudaMemcpyHostToDevice, s->stream)) != cudaSuccess)
            return cuda_fail(e, "upload convar");
        src = stage;
    }
    if (primvar && !src_prim) {
        double* stage_prim = s->scratch + 4 * n;
        if ((e = cudaMemcpyAsync(stage_prim, primvar, 4 * n * sizeof(double), cudaMemcpyHostToDevice, s->stream)) !=
            cudaSuccess)
            return cuda_fail(e, "upload primvar");
        src_prim = stage_prim;
    }
    // the control word reset from the pinned host copy, read back into it after the pass: one
    // synchronisation
    StepCtl c{};
    double seed = s->geo.dx;
    std::memcpy(&c.cfl_bits, &seed, sizeof seed);
    c.active = 1;
    *s->hctl = c;
    if ((e = cudaMemcpyAsync(s->ctl, s->hctl, sizeof c, cudaMemcpyHostToDevice, s->stream)) != cudaSuccess)
        return cuda_fail(e, "ctl upload");
    upload_state_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(src, src_prim, s->W, s->AX, s->AY, s->W32,
                                                                             s->geo, s->ctl);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "set_state");
    if ((e = cudaMemcpyAsync(s->hctl, s->ctl, sizeof c, cudaMemcpyDeviceToHost, s->stream)) != cudaSuccess)
        return cuda_fail(e, "ctl read");
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cuda_fail(e, "set_state");
    if (s->hctl->status & 1u) return fail(HOS_E_BLOWUP, "initial state has negative density/pressure or NaN");
    return HOS_OK;
}

int hos2d_set_state_device(hos_solver2d* s, const double* d_convar_soa, const double* d_primvar_soa) {
    if (!s || !d_convar_soa) return fail(HOS_E_ARG, "null argument");
    const size_t n = s->ncell;
    double* prim = s->scratch + 4 * n;
    cudaError_t e = cudaMemcpyAsync(s->W, d_convar_soa, 4 * n * sizeof(double), cudaMemcpyDeviceToDevice, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "copy convar");
    if (d_primvar_soa) {
        e = cudaMemcpyAsync(prim, d_primvar_soa, 4 * n * sizeof(double), cudaMemcpyDeviceToDevice, s->stream);
    } else {
        prim_of_state_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(s->W, prim, n, s->geo.gamma);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return cuda_fail(e, "copy primvar");
    return reset_ctl_and_cfl(s, prim);
}

int hos2d_set_alpha(hos_solver2d* s, const double* alpha_x, const double* alpha_y) {
    if (!s || !alpha_x || !alpha_y) return fail(HOS_E_ARG, "null argument");
    cudaError_t e = cudaMemcpyAsync(s->AX, alpha_x, s->ncell * sizeof(double), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->AY, alpha_y, s->ncell * sizeof(double), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = refresh_mirror(s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? HOS_OK : cuda_fail(e, "set_alpha");
}

int hos2d_get_state(hos_solver2d* s, double* convar, double* primvar, double* alpha_x, double* alpha_y) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    const size_t n = s->ncell;
    double* stage = s->scratch;
    double* prim = s->scratch + 4 * n;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    cudaError_t e;
    // pinned host buffers are written by the transposition itself over the host link; other
    // buffers through a device staging copy
    if (convar) {
        double* dst = static_cast<double*>(const_cast<void*>(mapped_host(convar)));
        soa_to_aos_kernel<<<blocks, 256, 0, s->stream>>>(s->W, dst ? dst : stage, n);
        if (!dst && (e = cudaMemcpyAsync(convar, stage, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, s->stream)) !=
                        cudaSuccess)
            return cuda_fail(e, "download convar");
        if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cuda_fail(e, "download convar");
    }
    if (primvar) {
        double* dst = static_cast<double*>(const_cast<void*>(mapped_host(primvar)));
        prim_of_state_kernel<<<blocks, 256, 0, s->stream>>>(s->W, prim, n, s->geo.gamma);
        soa_to_aos_kernel<<<blocks, 256, 0, s->stream>>>(prim, dst ? dst : stage, n);
        if (!dst && (e = cudaMemcpyAsync(primvar, stage, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, s->stream)) !=
                        cudaSuccess)
            return cuda_fail(e, "download primvar");
        if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cuda_fail(e, "download primvar");
    }
    if (alpha_x && (e = cudaMemcpyAsync(alpha_x, s->AX, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream)) != cudaSuccess)
        return cuda_fail(e, "download alpha_x");
    if (alpha_y && (e = cudaMemcpyAsync(alpha_y, s->AY, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream)) != cudaSuccess)
        return cuda_fail(e, "download alpha_y");
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cuda_fail(e, "get_state");
    return HOS_OK;
}

int hos2d_set_boundary(hos_solver2d* s, const int* bc, const double* bc_prim) {
    if (!s || !bc) return fail(HOS_E_ARG, "null argument");
    hos_params2d p = s->p;
    for (int k = 0; k < 4; ++k) {
        p.bc[k] = bc[k];
        if (bc_prim)
            for (int v = 0; v < 4; ++v) p.bc_prim[k][v] = bc_prim[4 * k + v];
    }
    if (int st = check_boundaries(p)) return st;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "set_boundary");
    s->p = p;
    fill_boundaries(s->bc, p, s->geo.dx);
    if (s->graph) {  // the captured step holds the old boundary description
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    return HOS_OK;
}

int hos2d_set_reconstruction(hos_solver2d* s, int mode) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    if (mode != HOS_RECON_WENO && mode != HOS_RECON_FIRST_ORDER) return fail(HOS_E_ARG, "bad reconstruction mode");
    if (s->geo.first_order == mode) return HOS_OK;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "set_reconstruction");
    s->geo.first_order = mode;
    if (s->graph) {  // the captured step holds the old geometry
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    return HOS_OK;
}

int hos2d_set_source(hos_solver2d* s, int on) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    if (on && s->geo.integrator != HOS_INT_S2O4) return fail(HOS_E_CONFIG, "the source update is provided with S2O4");
    const int mode = on ? 1 : 0;
    if (s->geo.source == mode) return HOS_OK;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "set_source");
    s->geo.source = mode;
    if (s->graph) {  // the captured step holds the old geometry
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    return HOS_OK;
}

int hos2d_set_time(hos_solver2d* s, double t) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    StepCtl c;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&c, s->ctl, sizeof c, cudaMemcpyDeviceToHost);
    c.t = t;
    if (e == cudaSuccess) e = cudaMemcpy(s->ctl, &c, sizeof c, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? HOS_OK : cuda_fail(e, "set_time");
}

int hos2d_set_gate_check(hos_solver2d* s, double slack) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    if (!(slack >= 0.0 && slack <= 10.0)) return fail(HOS_E_ARG, "slack must be in [0, 10]");
    if (s->geo.gate_slack == (float)slack) return HOS_OK;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "set_gate_check");
    s->geo.gate_slack = (float)slack;
    if (s->graph) {  // the captured step holds the old geometry
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    return HOS_OK;
}

int hos2d_set_gate(hos_solver2d* s, const hos_gate* g, float threshold, int audit_log2) {
    using namespace gate;
    if (!s) return fail(HOS_E_ARG, "null solver");
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "set_gate");
    if (s->graph) {  // the captured step has the old launch sequence
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    if (!g) {
        s->gated = 0;
        return HOS_OK;
    }
    if (s->precision != HOS_FP32) return fail(HOS_E_CONFIG, "the learned gate runs on the FP32-bulk path");
    if (s->geo.tau_type == HOS_TAU_NS) return fail(HOS_E_CONFIG, "the learned gate runs with the Euler collision time");
    if (s->geo.plain) return fail(HOS_E_CONFIG, "the learned gate runs with the DF variants (use_df = 1)");
    if (audit_log2 < 0 || audit_log2 > 31) return fail(HOS_E_ARG, "audit_log2 must be 0..31");
    if (!s->gflags) {
        if ((e = cudaMalloc(&s->gflags, s->ncell)) == cudaSuccess && (e = cudaMalloc(&s->gstats, sizeof(Stats))) == cudaSuccess &&
            (e = cudaMalloc(&s->gw, NET_BF16 * sizeof(__nv_bfloat16))) == cudaSuccess)
            e = cudaMalloc(&s->gb, NET_F32 * sizeof(float));
        if (e == cudaSuccess) e = cudaMemset(s->gstats, 0, sizeof(Stats));
        if (e != cudaSuccess) return fail(HOS_E_NOMEM, std::string("gate buffers: ") + cudaGetErrorString(e));
    }
    // the solver keeps its own copy, so the network can go on training
    if ((e = cudaStreamSynchronize(g->stream)) == cudaSuccess &&
        (e = cudaMemcpy(s->gw, g->wbf, NET_BF16 * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice)) == cudaSuccess)
        e = cudaMemcpy(s->gb, g->bias, NET_F32 * sizeof(float), cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "set_gate copy");
    switch (s->p.order) {
        case 5: e = configure_faces5(2); break;
        case 7: e = configure_faces7(2); break;
        default: e = configure_faces9(2); break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "configure gated face kernels");
    s->gthreshold = threshold;
    s->gaudit_mask = audit_log2 == 31 ? 0xffffffffu : (1u << audit_log2) - 1u;
    s->gated = 1;
    return HOS_OK;
}

int hos2d_set_gate_reuse(hos_solver2d* s, int reuse) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "set_gate_reuse");
    if (reuse && !s->gflags2 && (e = cudaMalloc(&s->gflags2, s->ncell)) != cudaSuccess)
        return fail(HOS_E_NOMEM, std::string("gate flags: ") + cudaGetErrorString(e));
    if (s->graph && (reuse != 0) != (s->greuse != 0)) {  // the captured step has the old launch sequence
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    s->greuse = reuse ? 1 : 0;
    return HOS_OK;
}

int hos2d_gate_stats(hos_solver2d* s, unsigned long long* stats, int reset) {
    if (!s || !stats) return fail(HOS_E_ARG, "null argument");
    if (!s->gstats) {
        std::memset(stats, 0, 8 * sizeof(unsigned long long));
        return HOS_OK;
    }
    gate::Stats st;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&st, s->gstats, sizeof st, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && reset) e = cudaMemset(s->gstats, 0, sizeof st);
    if (e != cudaSuccess) return cuda_fail(e, "gate_stats");
    const unsigned long long v[8] = {st.cells[0], st.cells[1], st.smooth[0], st.smooth[1], st.audited, st.false_neg,
                                     st.fallback, st.samples};
    std::memcpy(stats, v, sizeof v);
    return HOS_OK;
}

int hos2d_gate_audit_check(hos_solver2d* s, unsigned long long* out) {
    if (!s || !out) return fail(HOS_E_ARG, "null argument");
    out[0] = out[1] = 0;
    if (!s->gstats) return HOS_OK;
    gate::Stats st;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&st, s->gstats, sizeof st, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "gate_audit_check");
    out[0] = st.fn_linear;
    out[1] = st.fn_linear_accepted;
    return HOS_OK;
}

int hos_gate_collect(hos_gate* g, hos_solver2d* s, int sample_log2) {
    using namespace gate;
    if (!g || !s || sample_log2 < 0 || sample_log2 > 31) return fail(HOS_E_ARG, "bad argument");
    if (!g->samples) return fail(HOS_E_CONFIG, "the gate was created without sample capacity");
    const Geometry& geo = s->geo;
    const long long n = 2LL * geo.g * geo.ny + 2LL * geo.g * geo.nodex;
    bc_fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(s->W, geo, s->bc, s->ctl, 0, s->W32);
    GateArgs ga{s->W, s->AX, s->AY, nullptr, g->stats, 0.0f, 0xffffffffu, g->collect_seed++, g->samples, g->capacity,
                sample_log2 == 31 ? 0xffffffffu : (1u << sample_log2) - 1u, nullptr};
    cudaError_t e = cudaStreamSynchronize(g->stream);   // the network's copy is current
    if (e == cudaSuccess) e = launch_gate(s->p.order, ga, g->net(), geo, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    return e == cudaSuccess ? HOS_OK : cuda_fail(e, "gate collect");
}

int hos2d_begin_step(hos_solver2d* s, double tstop) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    return enqueue_begin(s, tstop);
}

int hos2d_boundary(hos_solver2d* s) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    const Geometry& geo = s->geo;
    const long long n = 2LL * geo.g * geo.ny + 2LL * geo.g * geo.nodex;
    bc_fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(s->W, geo, s->bc, s->ctl, 0, s->W32);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HOS_OK : cuda_fail(e, "bc_fill");
}

int hos2d_stage(hos_solver2d* s, int stage) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    if (stage < 0 || stage >= s->geo.stages) return fail(HOS_E_ARG, "stage out of range for the time-marching method");
    return enqueue_stage(s, stage);
}

int hos2d_step(hos_solver2d* s, double tstop) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    return enqueue_step(s, tstop);
}

int hos2d_advance(hos_solver2d* s, int nsteps, double tstop, int use_graph) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    if (nsteps < 0) return fail(HOS_E_ARG, "nsteps < 0");
    cudaError_t e;
    if (use_graph) {
        if (!s->graph || s->graph_tstop != tstop) {
            if (s->graph) {
                cudaGraphExecDestroy(s->graph);
                s->graph = nullptr;
            }
            cudaGraph_t g;
            if ((e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                return cuda_fail(e, "begin capture");
            int st = enqueue_step(s, tstop);
            e = cudaStreamEndCapture(s->stream, &g);
            if (st) return st;
            if (e != cudaSuccess) return cuda_fail(e, "end capture");
            e = cudaGraphInstantiate(&s->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
            s->graph_tstop = tstop;
        }
        for (int k = 0; k < nsteps; ++k)
            if ((e = cudaGraphLaunch(s->graph, s->stream)) != cudaSuccess) return cuda_fail(e, "graph launch");
        return HOS_OK;
    }
    for (int k = 0; k < nsteps; ++k) {
        int st = enqueue_step(s, tstop);
        if (st) return st;
    }
    return HOS_OK;
}

int hos2d_sync(hos_solver2d* s, double* t, double* dt) {
    if (!s) return fail(HOS_E_ARG, "null solver");
    cudaError_t e = cudaMemcpyAsync(s->hctl, s->ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "ctl read");
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return cuda_fail(e, "sync");
    const StepCtl c = *s->hctl;
    if (t) *t = c.t;
    if (dt) *dt = c.dt;
    if (c.status & 1u) return fail(HOS_E_BLOWUP, "negative density/pressure or NaN in the state");
    if (c.status & WAIT_TIMEOUT_BIT) return fail(HOS_E_TIMEOUT, "a TMA tile load or tensor-core MMA did not complete within its wait limit");
    return HOS_OK;
}

int hos2d_profile_step(hos_solver2d* s, double tstop, double* ms) {
    if (!s || !ms) return fail(HOS_E_ARG, "null argument");
    if (s->geo.stages != 2) return fail(HOS_E_CONFIG, "per-kernel profiling covers two-stage methods");
    cudaEvent_t ev[12];
    for (auto& x : ev) cudaEventCreate(&x);
    cudaEventRecord(ev[0], s->stream);
    int st = enqueue_begin(s, tstop);
    if (!st) {
        cudaEventRecord(ev[1], s->stream);
        st = enqueue_stage(s, 0, ev + 2);
    }
    if (!st) st = enqueue_stage(s, 1, ev + 7);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (!st && e == cudaSuccess) {
        float f;
        for (int k = 0; k < 11; ++k) {
            cudaEventElapsedTime(&f, ev[k], ev[k + 1]);
            ms[k] = f;
        }
    }
    for (auto& x : ev) cudaEventDestroy(x);
    if (st) return st;
    return e == cudaSuccess ? HOS_OK : cuda_fail(e, "profile_step");
}

int hos2d_launches_per_step(const hos_solver2d* s) {
    // begin_step + per stage (bc, [gate,] x faces, y faces, update)
    return 1 + (s ? s->geo.stages : 2) * (4 + (s && s->gated ? 1 : 0));
}

void* hos2d_stream(hos_solver2d* s) { return s ? (void*)s->stream : nullptr; }

}  // extern "C"
