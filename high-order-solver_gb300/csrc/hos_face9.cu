// hos_face9.cu -- WENO9-AO-DF face kernels (x and y faces, FP64 and FP32 compute).
#include "hos_launch.h"

namespace hos {

template <class T, int DIR>
static cudaError_t launch_one(const FaceArgs& a, const Geometry& geo, cudaStream_t s) {
    using S = FaceSmem<T, 9>;
    const int nodeN = DIR == 0 ? geo.nodex : geo.nodey;
    const int nodeT = DIR == 0 ? geo.nodey : geo.nodex;
    dim3 grid((nodeT + TILE_T - 1) / TILE_T, (nodeN + 1 + TILE_N - 1) / TILE_N);
    face_kernel<T, 9, DIR><<<grid, FACE_THREADS, S::bytes, s>>>(a, geo);
    return cudaGetLastError();
}

// dynamic shared memory above 48 KB must be enabled per kernel on the current device; the
// carveout asks for the largest shared-memory share of L1 so several tiles can be resident
template <class T, int DIR>
static cudaError_t carveout() {
    return cudaFuncSetAttribute(face_kernel<T, 9, DIR>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared);
}

cudaError_t configure_faces9(int precision) {
    cudaError_t e;
    if (precision == 0) {
        if ((e = carveout<double, 0>()) != cudaSuccess || (e = carveout<double, 1>()) != cudaSuccess) return e;
        if ((e = cudaFuncSetAttribute(face_kernel<double, 9, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)FaceSmem<double, 9>::bytes)) != cudaSuccess) return e;
        return cudaFuncSetAttribute(face_kernel<double, 9, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)FaceSmem<double, 9>::bytes);
    }
    if ((e = carveout<float, 0>()) != cudaSuccess || (e = carveout<float, 1>()) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(face_kernel<float, 9, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)FaceSmem<float, 9>::bytes)) != cudaSuccess) return e;
    return cudaFuncSetAttribute(face_kernel<float, 9, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)FaceSmem<float, 9>::bytes);
}

// ev (optional): ev[0] recorded after the x-face launch, ev[1] after the y-face launch
cudaError_t launch_faces9(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                           cudaEvent_t* ev) {
    cudaError_t e;
    if (precision == 0) {
        if ((e = launch_one<double, 0>(ax, geo, s)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[0], s);
        if ((e = launch_one<double, 1>(ay, geo, s)) != cudaSuccess) return e;
    } else {
        if ((e = launch_one<float, 0>(ax, geo, s)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[0], s);
        if ((e = launch_one<float, 1>(ay, geo, s)) != cudaSuccess) return e;
    }
    if (ev) cudaEventRecord(ev[1], s);
    return cudaSuccess;
}

}  // namespace hos
