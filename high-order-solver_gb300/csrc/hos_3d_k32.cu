// hos_3d_k32.cu -- the 3D face / line / point+GKS kernels with float bulk arithmetic.
#include "hos_3d_launch.h"

namespace hos {
namespace d3 {

namespace {
template <bool GATED>
cudaError_t flux3_f32(const float* W, float* FV, float* LV, double* FS, const Geo3& g, const Dir3& d, const Ctl3* ctl,
                      int stage, cudaStream_t s, cudaEvent_t* ev, Gate3 gt) {
    const size_t nc = d.cel.n(), nl = d.lv.n(), np = 2 * d.fs.n();
    face3_kernel<float, GATED><<<(unsigned)((nc + FACE3_THREADS - 1) / FACE3_THREADS), FACE3_THREADS, 0, s>>>(W, FV, g, d, ctl,
                                                                                                         gt);
    if (ev) cudaEventRecord(ev[0], s);
    line3_kernel<float, GATED><<<(unsigned)((nl + LINE3_THREADS - 1) / LINE3_THREADS), LINE3_THREADS, 0, s>>>(FV, LV, g, d,
                                                                                                         ctl, gt);
    if (ev) cudaEventRecord(ev[1], s);
    point3_kernel<float, GATED><<<(unsigned)((np + POINT3_THREADS - 1) / POINT3_THREADS), POINT3_THREADS, 0, s>>>(
        LV, FS, g, d, ctl, stage, gt);
    if (ev) cudaEventRecord(ev[2], s);
    return cudaGetLastError();
}
}  // namespace

template <>
cudaError_t launch_flux3<float>(const float* W, float* FV, float* LV, double* FS, const Geo3& g, const Dir3& d,
                                const Ctl3* ctl, int stage, cudaStream_t s, cudaEvent_t* ev, Gate3 gt) {
    return gt.flags ? flux3_f32<true>(W, FV, LV, FS, g, d, ctl, stage, s, ev, gt)
                    : flux3_f32<false>(W, FV, LV, FS, g, d, ctl, stage, s, ev, gt);
}

}  // namespace d3
}  // namespace hos
