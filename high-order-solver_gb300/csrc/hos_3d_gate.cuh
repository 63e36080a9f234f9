// hos_3d_gate.cuh -- the learned smoothness gate on the 3D FP32-bulk path.
//
// The network, its training and its sample format are those of the 2D gate (hos_gate.cuh):
// a 16 -> 32 -> 32 -> 1 BF16 MLP, evaluated on the tcgen05 tensor cores by the 2D gate's routine.  Its inputs for one cell and one
// global axis are the normalised smoothness indicators of the cell's WENO5-AO stencil along
// that axis (the three small-stencil betas, the big-stencil beta padded to 6, and tau) for
// density and for pressure; there is no discontinuity-feedback indicator in 3D (inputs 14
// and 15 are zero).  The label is whether the nonlinear weights of every characteristic
// variable on both faces stay within GATE_EPS of the linear ones.  Flags (bit a for axis a)
// feed the gated face / line / point kernels of hos_3d.cuh.
#pragma once
#include "hos_3d.cuh"
#include "hos_gate.cuh"

namespace hos {
namespace d3 {

// counters of the 3D gate: cells gated and predicted smooth per axis, audits, false negatives
// among them, linear results rejected by the kernels' check
struct Stats3 {
    unsigned long long cells[3];
    unsigned long long smooth[3];
    unsigned long long audited;
    unsigned long long false_neg;
    unsigned long long fallback;
};

struct GateRun3 {
    const double* W;
    float2* rp;                       // scratch, one (density, pressure) pair per cell
    Geo3 g;
    gate::Net net;
    unsigned char* flags;             // null: collect samples only
    Stats3* stats;
    float threshold;                  // logit above which a cell is predicted smooth
    unsigned audit_mask;              // audit the predicted-smooth cells of warps whose hash & mask == 0
    unsigned seed;
    float* samples;                   // collect mode: [capacity][gate::NS] records
    unsigned long long capacity;
    unsigned long long* sample_count; // the network's sample counter
    unsigned sample_mask;             // collect cells whose hash & mask == 0
    const Ctl3* ctl;                  // inactive solver: no work (may be null)
};

// rp_ready: r.rp already holds this stage's (density, pressure) pairs (the FP32 solver's
// mirror pass writes them); otherwise they are computed first
cudaError_t launch_gate3(const GateRun3& r, cudaStream_t s, bool rp_ready = false);

}  // namespace d3
}  // namespace hos
