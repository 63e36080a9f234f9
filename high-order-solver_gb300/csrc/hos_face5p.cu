// hos_face5p.cu -- non-DF WENO5-AO face kernels: the reconstruction the reference's 2D drivers
// install first (WENO5_AO_normal / WENO5_AO_tangent, src/reconstruction.cpp:1562-1699,
// 2233-2551), used while is_using_df_factor is false; FP64 and FP32 compute, Euler and
// Navier-Stokes collision times.
#include "hos_face_impl.cuh"

namespace hos {

cudaError_t configure_faces5p(int precision) { return FaceLaunch<5, true>::configure(precision); }

cudaError_t launch_faces5p(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                            cudaEvent_t* ev, const CUtensorMap* tm) {
    return FaceLaunch<5, true>::launch(precision, ax, ay, geo, s, ev, tm);
}

}  // namespace hos
