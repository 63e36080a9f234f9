// hos_batch.cuh -- device side of the batched 2D step: problem descriptors, the tile table,
// the persistent face kernel over the tiles of every problem, and the batched boundary,
// update and step-prologue kernels (bodies shared with the single-problem step).
#pragma once
#include "../../include/hos_gb300.h"
#include "hos_launch.h"
#include "hos_step.cuh"

namespace hos {
namespace batch {

struct Prob {
    Geometry geo;
    BcSpec bc;
    double *W, *Wold, *AX, *AY, *FXx, *FPx, *FAx, *FXy, *FPy, *FAy;
    StepCtl* ctl;
    double tstop;
    int* last_step;   // batch step index of this problem's last active step
    unsigned char* gflags;   // learned-gate flags of this problem's cells (gated batches)
    // FP32 batches: FP32 mirror of W0..W3, alpha_x, alpha_y (pitch mirror_pitch(ny)), written by
    // the boundary and update kernels and read by the FP32 face and gate tiles (null: FP64)
    float* W32;
};

struct TileRef { int p, n0, t0, pad; };

// candidate tile shapes (faces along normal x tangent): 128 faces, or 256 for 16 x 16 (every
// thread then has the same number of flux items; WENO5 only)
using Shape0 = TileShape<8, 16>;
using Shape1 = TileShape<16, 16>;
using Shape2 = TileShape<16, 8>;
constexpr int kShapes = 3;
const int kShapeN[kShapes] = {8, 16, 16};
const int kShapeT[kShapes] = {16, 16, 8};

// FP32 tiles fit two CTAs per SM in 128 registers; FP64 tiles need more registers than that
template <class T, int ORDER, int DIR, class TS, bool GATED = false>
__global__ void __launch_bounds__(FACE_THREADS, sizeof(T) == 4 ? 2 : 1) face_batch_kernel(const Prob* __restrict__ probs,
                                                                  const TileRef* __restrict__ tiles, int ntiles,
                                                                  int stage, unsigned long long* fallback) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    for (int k = blockIdx.x; k < ntiles; k += gridDim.x) {
        const TileRef tr = tiles[k];
        const Prob* pr = probs + tr.p;
        const Geometry geo = pr->geo;
        FaceArgs a{};   // members not set below (per-stage buffers) stay null
        a.W = pr->W;
        a.AN = DIR == 0 ? pr->AX : pr->AY;
        a.AT = DIR == 0 ? pr->AY : pr->AX;
        a.FX = DIR == 0 ? pr->FXx : pr->FXy;
        a.FP = DIR == 0 ? pr->FPx : pr->FPy;
        a.FA = DIR == 0 ? pr->FAx : pr->FAy;
        a.ctl = pr->ctl;
        a.stage = stage;
        a.gate = pr->gflags;
        a.fallback = fallback;
        if (pr->W32) {
            const size_t plane32 = (size_t)geo.nx * mirror_pitch(geo.ny);
            a.W32 = pr->W32;
            a.AN32 = pr->W32 + (DIR == 0 ? 4 : 5) * plane32;
            a.AT32 = pr->W32 + (DIR == 0 ? 5 : 4) * plane32;
        }
        face_tile<T, ORDER, DIR, TS, GATED>(a, geo, tr.n0, tr.t0, smem_raw);
        __syncthreads();  // the next tile reuses the shared memory
    }
}

// launch / configure the face kernels of one order (defined per order in hos_batch{5,7,9}.cu);
// orders 7 and 9 provide the default tile shape only; prec 0 FP64, 1 FP32, 2 gated FP32
cudaError_t launch_batch_faces5(int prec, int shape, int dir, const Prob* probs, const TileRef* tiles, int ntiles, int stage, int grid, cudaStream_t s, unsigned long long* fallback);
cudaError_t launch_batch_faces7(int prec, int shape, int dir, const Prob* probs, const TileRef* tiles, int ntiles, int stage, int grid, cudaStream_t s, unsigned long long* fallback);
cudaError_t launch_batch_faces9(int prec, int shape, int dir, const Prob* probs, const TileRef* tiles, int ntiles, int stage, int grid, cudaStream_t s, unsigned long long* fallback);
cudaError_t configure_batch5(int prec, int dir, int* bps);
cudaError_t configure_batch7(int prec, int dir, int* bps);
cudaError_t configure_batch9(int prec, int dir, int* bps);

}  // namespace batch
}  // namespace hos
