// hos_static.cu -- hos2d_step_static: one S2O4 step that allocates no device memory.
//
// Some callers of this step cannot allocate device memory once they are running: host
// codes that reserve their whole HBM budget in a pool at start-up and forbid cudaMalloc /
// cudaFree afterwards (both can synchronise the device and can fail mid-run), or that run
// under a fixed per-process memory quota on a shared GPU.  hos2d_create allocates the
// state and the face-flux buffers, so those callers use this entry point instead: the
// caller owns the state (conserved variables and DF indicators), and the step's scratch
// (step-start state, face fluxes, face DF indicators, step control word) lives in one
// file-scope static device array of fixed size, held by every GPU that loads the library
// until the process exits.
//
// Limits: nodex, nodey <= HOS_STATIC_MAX_NODE (256) and ghost <= HOS_STATIC_MAX_GHOST (5),
// i.e. about 11.7 MB of scratch.  Larger problems are rejected with HOS_E_CONFIG, and so are
// settings the step does not run: time marching other than S2O4, the LF flux, the non-DF
// scheme, and the wedge and no-slip boundaries.  Both collision times (Euler, Navier-Stokes
// with the Prandtl fix) are run as hos2d_create runs them.  Each call waits for its stream
// to finish before returning (it reads the step's status word back).
// The first call on a device looks up the array's device address (cudaGetSymbolAddress)
// and enables the face kernels' shared-memory size for that device; make that first call
// before any stream capture.  Every call shares the one array and it keeps the last call's
// contents, so calls that overlap on the GPU (other streams, other host threads) race.
#include <cstring>
#include <string>

#include "../../include/hos_gb300.h"
#include "hos_launch.h"

namespace hos {
namespace {

constexpr int kMaxNode = HOS_STATIC_MAX_NODE;
constexpr int kMaxGhost = HOS_STATIC_MAX_GHOST;
constexpr size_t kMaxCells = (size_t)(kMaxNode + 2 * kMaxGhost) * (kMaxNode + 2 * kMaxGhost);
constexpr size_t kMaxFaces = (size_t)(kMaxNode + 1) * kMaxNode;   // per direction
constexpr size_t kCtlDoubles = (sizeof(StepCtl) + sizeof(double) - 1) / sizeof(double);
// layout: Wold[4][cells] | x: FX[4][f] FP[4][f] FA[f] | y: same | StepCtl
constexpr size_t kScratchDoubles = 4 * kMaxCells + 2 * 9 * kMaxFaces + kCtlDoubles;

static __device__ __align__(256) double g_step_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
// Per-device set-up state.  These host globals are written without a lock: two host threads
// making a device's first call at the same time both look up the same address and set the
// same bits, so the race is benign; calls themselves must be serialised per device anyway.
double* g_scratch_ptr[kMaxDevices] = {nullptr};
unsigned g_configured[kMaxDevices] = {0};   // bit (order/2 - 2) * 5 + face-kernel variant

thread_local std::string g_err;

int fail_static(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

__global__ void static_ctl_kernel(StepCtl* ctl, double dt, double seed) {
    ctl->dt = dt;
    ctl->t = dt;
    ctl->cfl_bits = (unsigned long long)__double_as_longlong(seed);
    ctl->status = 0u;
    ctl->active = 1u;
}

}  // namespace
}  // namespace hos

using namespace hos;

extern "C" const char* hos_static_last_error(void) { return g_err.c_str(); }

extern "C" int hos2d_step_static(const hos_params2d* params, int precision, double* d_W, double* d_alpha_x,
                                 double* d_alpha_y, double dt, void* stream) {
    if (!params || !d_W || !d_alpha_x || !d_alpha_y) return fail_static(HOS_E_ARG, "null argument");
    const hos_params2d& p = *params;
    if (!(p.order == 5 || p.order == 7 || p.order == 9)) return fail_static(HOS_E_CONFIG, "order must be 5, 7 or 9");
    if (p.gausspoint != (p.order == 5 ? 2 : p.order == 7 ? 3 : 4))
        return fail_static(HOS_E_CONFIG, "gausspoint must be 2/3/4 for order 5/7/9");
    if (!p.use_df) return fail_static(HOS_E_CONFIG, "use_df must be 1");
    if (p.integrator != HOS_INT_S2O4 || p.flux != HOS_FLUX_GKS)
        return fail_static(HOS_E_CONFIG, "the allocation-free step runs S2O4 with the GKS flux");
    if (p.tau_type != HOS_TAU_EULER && p.tau_type != HOS_TAU_NS) return fail_static(HOS_E_CONFIG, "bad tau_type");
    if (p.tau_type == HOS_TAU_NS && p.prandtl_fix && !(p.prandtl > 0))
        return fail_static(HOS_E_CONFIG, "the Prandtl fix needs prandtl > 0");
    if (p.ghost < p.order / 2 + 1) return fail_static(HOS_E_CONFIG, "ghost must be >= order/2 + 1");
    if (p.nodex < p.ghost || p.nodey < p.ghost) return fail_static(HOS_E_CONFIG, "nodex and nodey must be >= ghost");
    if (p.nodex > kMaxNode || p.nodey > kMaxNode || p.ghost > kMaxGhost)
        return fail_static(HOS_E_CONFIG, "hos2d_step_static: problem exceeds the static scratch limit (nodex, nodey <= " +
                                             std::to_string(kMaxNode) + ", ghost <= " + std::to_string(kMaxGhost) +
                                             "); use hos2d_create for larger problems");
    if (precision != HOS_FP64 && precision != HOS_FP32) return fail_static(HOS_E_CONFIG, "bad precision");
    for (int k = 0; k < 4; ++k)
        if (p.bc[k] < 0 || p.bc[k] > 3)
            return fail_static(HOS_E_CONFIG, "the allocation-free step takes free, periodic, reflective and inflow "
                                             "boundaries (HOS_BC_FREE .. HOS_BC_INFLOW)");
    if ((p.bc[0] == HOS_BC_PERIODIC) != (p.bc[1] == HOS_BC_PERIODIC) ||
        (p.bc[2] == HOS_BC_PERIODIC) != (p.bc[3] == HOS_BC_PERIODIC))
        return fail_static(HOS_E_CONFIG, "periodic boundaries must be paired");
    if (!(dt > 0.0)) return fail_static(HOS_E_ARG, "dt must be positive");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_static(HOS_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail_static(HOS_E_CUDA, "device index out of range");
    // set-up, once per device, with that device current
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_step_scratch);
        if (e != cudaSuccess) return fail_static(HOS_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<double*>(ptr);
    }
    // face-kernel variant: 0 / 1 FP64 / FP32 with the Euler collision time, 3 / 4 with the
    // Navier-Stokes one
    const int variant = p.tau_type == HOS_TAU_NS ? (precision == HOS_FP64 ? 3 : 4) : precision;
    const unsigned bit = 1u << ((p.order / 2 - 2) * 5 + variant);
    if (!(g_configured[dev] & bit)) {
        e = p.order == 5 ? configure_faces5(variant) : p.order == 7 ? configure_faces7(variant) : configure_faces9(variant);
        if (e != cudaSuccess) return fail_static(HOS_E_CUDA, std::string("configure face kernels: ") + cudaGetErrorString(e));
        g_configured[dev] |= bit;
    }

    Geometry geo;
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
    geo.tau_type = p.tau_type;
    geo.mu = p.mu;
    geo.nu = p.nu;
    geo.prandtl_coef = p.tau_type == HOS_TAU_NS && p.prandtl_fix ? 1.0 / p.prandtl - 1.0 : 0.0;
    BcSpec bc;
    for (int k = 0; k < 4; ++k) {
        bc.kind[k] = p.bc[k];
        const double* q = p.bc_prim[k];
        bc.inflow[k][0] = q[0];
        bc.inflow[k][1] = q[0] * q[1];
        bc.inflow[k][2] = q[0] * q[2];
        bc.inflow[k][3] = q[0] * (q[3] / q[0] / (p.gamma - 1) + 0.5 * (q[1] * q[1] + q[2] * q[2]));
    }
    double* base = g_scratch_ptr[dev];
    double* Wold = base;
    double* fx = base + 4 * kMaxCells;
    double* FXx = fx;
    double* FPx = fx + 4 * kMaxFaces;
    double* FAx = fx + 8 * kMaxFaces;
    double* fy = fx + 9 * kMaxFaces;
    double* FXy = fy;
    double* FPy = fy + 4 * kMaxFaces;
    double* FAy = fy + 8 * kMaxFaces;
    StepCtl* ctl = reinterpret_cast<StepCtl*>(fy + 9 * kMaxFaces);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // the control word must start from a known state every call: dt, status 0, active
    static_ctl_kernel<<<1, 1, 0, s>>>(ctl, dt, geo.dx);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_static(HOS_E_CUDA, std::string("ctl: ") + cudaGetErrorString(e));
    for (int stage = 0; stage < 2; ++stage) {
        const long long nb = 2LL * geo.g * geo.ny + 2LL * geo.g * geo.nodex;
        bc_fill_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(d_W, geo, bc, ctl, 1);
        FaceArgs ax{d_W, d_alpha_x, d_alpha_y, FXx, FPx, FAx, ctl, stage};
        FaceArgs ay{d_W, d_alpha_y, d_alpha_x, FXy, FPy, FAy, ctl, stage};
        e = p.order == 5 ? launch_faces5(variant, ax, ay, geo, s)
          : p.order == 7 ? launch_faces7(variant, ax, ay, geo, s)
                         : launch_faces9(variant, ax, ay, geo, s);
        if (e != cudaSuccess) return fail_static(HOS_E_CUDA, std::string("face kernels: ") + cudaGetErrorString(e));
        UpdateArgs ua{d_W, Wold, d_alpha_x, d_alpha_y, FXx, FXy, FAx, FAy, ctl, stage};
        const int n = geo.nodex * geo.nodey;
        update_kernel<<<(n + 255) / 256, 256, 0, s>>>(ua, geo);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail_static(HOS_E_CUDA, std::string("update: ") + cudaGetErrorString(e));
    }
    unsigned int status = 0;
    e = cudaMemcpyAsync(&status, &ctl->status, sizeof status, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail_static(HOS_E_CUDA, std::string("step: ") + cudaGetErrorString(e));
    if (status & 1u) return fail_static(HOS_E_BLOWUP, "negative density/pressure or NaN in the state");
    return HOS_OK;
}
