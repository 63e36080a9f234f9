// hos_3d_launch.h -- the per-direction flux launches of the 3D step, instantiated for FP64
// (hos_3d_k64.cu) and FP32 (hos_3d_k32.cu) bulk arithmetic in their own translation units.
#pragma once
#include <cuda_runtime.h>

#include "hos_3d.cuh"

namespace hos {
namespace d3 {

// face3 -> line3 -> point3 for one direction; W: the state in the compute type (FP64 state or
// the FP32 mirror); ev (may be null) receives an event after each; gt.flags non-null (FP32
// only) runs the gated kernels
template <class T>
cudaError_t launch_flux3(const T* W, T* FV, T* LV, double* FS, const Geo3& g, const Dir3& d, const Ctl3* ctl,
                         int stage, cudaStream_t s, cudaEvent_t* ev, Gate3 gt);

}  // namespace d3
}  // namespace hos
