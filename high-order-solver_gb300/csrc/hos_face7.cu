// hos_face7.cu -- WENO7-AO-DF face kernels (x and y faces; FP64, FP32 and gated FP32 compute).
#include "hos_launch.h"

namespace hos {

template <class T, int DIR, bool GATED, bool NS = false>
static cudaError_t launch_one(const FaceArgs& a, const Geometry& geo, cudaStream_t s) {
    using S = FaceSmem<T, 7>;
    const int nodeN = DIR == 0 ? geo.nodex : geo.nodey;
    const int nodeT = DIR == 0 ? geo.nodey : geo.nodex;
    dim3 grid((nodeT + TILE_T - 1) / TILE_T, (nodeN + 1 + TILE_N - 1) / TILE_N);
    face_kernel<T, 7, DIR, GATED, NS><<<grid, FACE_THREADS, GATED ? S::gated_bytes : S::bytes, s>>>(a, geo);
    return cudaGetLastError();
}

// dynamic shared memory above 48 KB must be enabled per kernel on the current device; the
// carveout asks for the largest shared-memory share of L1 so several tiles can be resident
template <class T, int DIR, bool GATED, bool NS = false>
static cudaError_t configure_one() {
    using S = FaceSmem<T, 7>;
    auto k = face_kernel<T, 7, DIR, GATED, NS>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(GATED ? S::gated_bytes : S::bytes));
    return e;
}

// precision: 0 FP64, 1 FP32, 2 FP32 with the learned gate, 3 FP64 and 4 FP32 with the
// Navier-Stokes collision time
cudaError_t configure_faces7(int precision) {
    cudaError_t e;
    if (precision == 3) {
        if ((e = configure_one<double, 0, false, true>()) != cudaSuccess) return e;
        return configure_one<double, 1, false, true>();
    }
    if (precision == 4) {
        if ((e = configure_one<float, 0, false, true>()) != cudaSuccess) return e;
        return configure_one<float, 1, false, true>();
    }
    if (precision == 0) {
        if ((e = configure_one<double, 0, false>()) != cudaSuccess) return e;
        return configure_one<double, 1, false>();
    }
    if (precision == 1) {
        if ((e = configure_one<float, 0, false>()) != cudaSuccess) return e;
        return configure_one<float, 1, false>();
    }
    if ((e = configure_one<float, 0, true>()) != cudaSuccess) return e;
    return configure_one<float, 1, true>();
}

// ev (optional): ev[0] recorded after the x-face launch, ev[1] after the y-face launch
cudaError_t launch_faces7(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                           cudaEvent_t* ev) {
    cudaError_t e;
    if (precision == 3) {
        if ((e = launch_one<double, 0, false, true>(ax, geo, s)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[0], s);
        if ((e = launch_one<double, 1, false, true>(ay, geo, s)) != cudaSuccess) return e;
    } else if (precision == 4) {
        if ((e = launch_one<float, 0, false, true>(ax, geo, s)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[0], s);
        if ((e = launch_one<float, 1, false, true>(ay, geo, s)) != cudaSuccess) return e;
    } else if (precision == 0) {
        if ((e = launch_one<double, 0, false>(ax, geo, s)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[0], s);
        if ((e = launch_one<double, 1, false>(ay, geo, s)) != cudaSuccess) return e;
    } else if (precision == 1) {
        if ((e = launch_one<float, 0, false>(ax, geo, s)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[0], s);
        if ((e = launch_one<float, 1, false>(ay, geo, s)) != cudaSuccess) return e;
    } else {
        if ((e = launch_one<float, 0, true>(ax, geo, s)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[0], s);
        if ((e = launch_one<float, 1, true>(ay, geo, s)) != cudaSuccess) return e;
    }
    if (ev) cudaEventRecord(ev[1], s);
    return cudaSuccess;
}

}  // namespace hos
