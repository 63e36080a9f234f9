// hos_batch5.cu -- batched WENO5-AO-DF face kernels (3 tile shapes: 8 x 16, 16 x 16, 16 x 8; FP64, FP32
// and gated FP32).
#include "hos_batch.cuh"

namespace hos {
namespace batch {

template <class T, int DIR, bool GATED>
static cudaError_t launch_t(int shape, const Prob* probs, const TileRef* tiles, int ntiles, int stage, int grid,
                            cudaStream_t s, unsigned long long* fallback) {
    switch (shape) {
        case 0: {
            using S = FaceSmem<T, 5, Shape0>;
            face_batch_kernel<T, 5, DIR, Shape0, GATED><<<grid, FACE_THREADS, GATED ? S::gated_bytes : S::bytes, s>>>(
                probs, tiles, ntiles, stage, fallback);
            break;
        }
        case 1: {
            using S = FaceSmem<T, 5, Shape1>;
            face_batch_kernel<T, 5, DIR, Shape1, GATED><<<grid, FACE_THREADS, GATED ? S::gated_bytes : S::bytes, s>>>(
                probs, tiles, ntiles, stage, fallback);
            break;
        }
        case 2: {
            using S = FaceSmem<T, 5, Shape2>;
            face_batch_kernel<T, 5, DIR, Shape2, GATED><<<grid, FACE_THREADS, GATED ? S::gated_bytes : S::bytes, s>>>(
                probs, tiles, ntiles, stage, fallback);
            break;
        }
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <class T, int DIR, class TS, bool GATED>
static cudaError_t configure_one(int* blocks_per_sm) {
    auto k = face_batch_kernel<T, 5, DIR, TS, GATED>;
    using S = FaceSmem<T, 5, TS>;
    const int bytes = (int)(GATED ? S::gated_bytes : S::bytes);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, FACE_THREADS, bytes);
    return e;
}

template <class T, int DIR, bool GATED>
static cudaError_t configure_t(int* bps) {
    cudaError_t e;
    if ((e = configure_one<T, DIR, Shape0, GATED>(&bps[0])) != cudaSuccess) return e;
    if ((e = configure_one<T, DIR, Shape1, GATED>(&bps[1])) != cudaSuccess) return e;
    if ((e = configure_one<T, DIR, Shape2, GATED>(&bps[2])) != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t launch_batch_faces5(int prec, int shape, int dir, const Prob* probs, const TileRef* tiles, int ntiles, int stage,
                                 int grid, cudaStream_t s, unsigned long long* fallback) {
    if (prec == 0) return dir == 0 ? launch_t<double, 0, false>(shape, probs, tiles, ntiles, stage, grid, s, fallback)
                                   : launch_t<double, 1, false>(shape, probs, tiles, ntiles, stage, grid, s, fallback);
    if (prec == 1) return dir == 0 ? launch_t<float, 0, false>(shape, probs, tiles, ntiles, stage, grid, s, fallback)
                                   : launch_t<float, 1, false>(shape, probs, tiles, ntiles, stage, grid, s, fallback);
    return dir == 0 ? launch_t<float, 0, true>(shape, probs, tiles, ntiles, stage, grid, s, fallback)
                    : launch_t<float, 1, true>(shape, probs, tiles, ntiles, stage, grid, s, fallback);
}

cudaError_t configure_batch5(int prec, int dir, int* bps) {
    if (prec == 0) return dir == 0 ? configure_t<double, 0, false>(bps) : configure_t<double, 1, false>(bps);
    if (prec == 1) return dir == 0 ? configure_t<float, 0, false>(bps) : configure_t<float, 1, false>(bps);
    return dir == 0 ? configure_t<float, 0, true>(bps) : configure_t<float, 1, true>(bps);
}

}  // namespace batch
}  // namespace hos
