// hos_launch.h -- host-side launchers of the templated face kernels (one translation unit
// per WENO-AO order so the three orders compile in parallel).
#pragma once
#include <cuda_runtime.h>
#include "hos_kernels.cuh"

namespace hos {
// precision: 0 = FP64 compute, 1 = FP32 compute (state and accumulation stay FP64),
// 2 = FP32 compute with the learned gate (FaceArgs::gate set), 3 / 4 = FP64 / FP32 with the
// Navier-Stokes collision time.  tm: the FP32 mirror's tensor maps (x- and y-face boxes); with
// them the FP32 kernels stage their tiles by TMA tile loads from the mirror.
cudaError_t configure_faces5(int precision);
cudaError_t configure_faces7(int precision);
cudaError_t configure_faces9(int precision);
cudaError_t launch_faces5(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                           cudaEvent_t* ev = nullptr, const CUtensorMap* tm = nullptr);
cudaError_t launch_faces7(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                           cudaEvent_t* ev = nullptr, const CUtensorMap* tm = nullptr);
cudaError_t launch_faces9(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                           cudaEvent_t* ev = nullptr, const CUtensorMap* tm = nullptr);
// the non-DF WENO5-AO kernels (Geometry::plain; precisions 0, 1, 3, 4)
cudaError_t configure_faces5p(int precision);
cudaError_t launch_faces5p(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                            cudaEvent_t* ev = nullptr, const CUtensorMap* tm = nullptr);
// the face kernels of geo's order and scheme
inline cudaError_t configure_faces(const Geometry& geo, int order, int precision) {
    if (geo.plain) return configure_faces5p(precision);
    return order == 5 ? configure_faces5(precision) : order == 7 ? configure_faces7(precision) : configure_faces9(precision);
}
inline cudaError_t launch_faces(int order, int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo,
                                cudaStream_t s, cudaEvent_t* ev = nullptr, const CUtensorMap* tm = nullptr) {
    if (geo.plain) return launch_faces5p(precision, ax, ay, geo, s, ev, tm);
    return order == 5 ? launch_faces5(precision, ax, ay, geo, s, ev, tm)
         : order == 7 ? launch_faces7(precision, ax, ay, geo, s, ev, tm)
                      : launch_faces9(precision, ax, ay, geo, s, ev, tm);
}
}  // namespace hos
