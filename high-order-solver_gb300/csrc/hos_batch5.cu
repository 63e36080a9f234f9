// hos_batch5.cu -- batched WENO5-AO-DF face kernels (3 tile shapes, FP64 and FP32 compute).
#include "hos_batch.cuh"

namespace hos {
namespace batch {

template <class T, int DIR>
static cudaError_t launch_t(int shape, const Prob* probs, const TileRef* tiles, int ntiles, int stage, int grid,
                            cudaStream_t s) {
    switch (shape) {
        case 0:
            face_batch_kernel<T, 5, DIR, Shape0><<<grid, FACE_THREADS, FaceSmem<T, 5, Shape0>::bytes, s>>>(probs, tiles, ntiles, stage);
            break;
        case 1:
            face_batch_kernel<T, 5, DIR, Shape1><<<grid, FACE_THREADS, FaceSmem<T, 5, Shape1>::bytes, s>>>(probs, tiles, ntiles, stage);
            break;
        case 2:
            face_batch_kernel<T, 5, DIR, Shape2><<<grid, FACE_THREADS, FaceSmem<T, 5, Shape2>::bytes, s>>>(probs, tiles, ntiles, stage);
            break;
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <class T, int DIR, class TS>
static cudaError_t configure_one(int* blocks_per_sm) {
    auto k = face_batch_kernel<T, 5, DIR, TS>;
    const int bytes = (int)FaceSmem<T, 5, TS>::bytes;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, FACE_THREADS, bytes);
    return e;
}

template <class T, int DIR>
static cudaError_t configure_t(int* bps) {
    cudaError_t e;
    if ((e = configure_one<T, DIR, Shape0>(&bps[0])) != cudaSuccess) return e;
    if ((e = configure_one<T, DIR, Shape1>(&bps[1])) != cudaSuccess) return e;
    if ((e = configure_one<T, DIR, Shape2>(&bps[2])) != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t launch_batch_faces5(int prec, int shape, int dir, const Prob* probs, const TileRef* tiles, int ntiles, int stage,
                                 int grid, cudaStream_t s) {
    if (prec == 0) return dir == 0 ? launch_t<double, 0>(shape, probs, tiles, ntiles, stage, grid, s)
                                   : launch_t<double, 1>(shape, probs, tiles, ntiles, stage, grid, s);
    return dir == 0 ? launch_t<float, 0>(shape, probs, tiles, ntiles, stage, grid, s)
                    : launch_t<float, 1>(shape, probs, tiles, ntiles, stage, grid, s);
}

cudaError_t configure_batch5(int prec, int dir, int* bps) {
    if (prec == 0) return dir == 0 ? configure_t<double, 0>(bps) : configure_t<double, 1>(bps);
    return dir == 0 ? configure_t<float, 0>(bps) : configure_t<float, 1>(bps);
}

}  // namespace batch
}  // namespace hos
