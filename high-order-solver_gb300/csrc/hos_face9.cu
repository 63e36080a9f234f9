// hos_face9.cu -- WENO9-AO-DF face kernels (x and y faces; FP64, FP32 and gated FP32 compute;
// FP32 with TMA tile staging for the solvers that keep the FP32 mirror).
#include "hos_face_impl.cuh"

namespace hos {

cudaError_t configure_faces9(int precision) { return FaceLaunch<9>::configure(precision); }

// ev (optional): ev[0] recorded after the x-face launch, ev[1] after the y-face launch;
// tm (optional, FP32 precisions): the FP32 mirror's tensor maps with the x- and y-face boxes
cudaError_t launch_faces9(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                           cudaEvent_t* ev, const CUtensorMap* tm) {
    return FaceLaunch<9>::launch(precision, ax, ay, geo, s, ev, tm);
}

}  // namespace hos
