// hos_3d_gate.cu -- the 3D gate kernel: features, the MLP on the tensor cores, flags,
// training samples and audits (see hos_3d_gate.cuh).
#include "hos_3d_gate.cuh"

namespace hos {
namespace d3 {
namespace {

constexpr int GATE3_THREADS = 256;

// normalised indicators of one 5-cell stencil: beta_0..2 and the big stencil's beta, padded to
// 6, then tau, over (sum beta + tau + 1e-10 c^2) with c the centre value
__device__ __forceinline__ void indicator5(const float* s, float* f) {
    float b[4];
    beta3<float>(s, b);
    // about the centre value: the indicator depends on differences only (see weights5)
    b[3] = beta5_big<float>(s[0] - s[2], s[1] - s[2], 0.0f, s[3] - s[2], s[4] - s[2]);
    const float tau = (1.0f / 3.0f) * (fabsf(b[3] - b[0]) + fabsf(b[3] - b[1]) + fabsf(b[3] - b[2]));
    const float inv = 1.0f / (b[0] + b[1] + b[2] + b[3] + tau + 1e-10f * s[2] * s[2] + 1e-30f);
#pragma unroll
    for (int k = 0; k < 4; ++k) f[k] = b[k] * inv;
    f[4] = f[5] = 0.0f;
    f[6] = tau * inv;
}

// largest distance of the nonlinear WENO5-AO weights from the linear ones over both faces and
// the five characteristic variables of cell c along axis ax, in face3's variables, with the
// regularisation epsilon 1e-6 of the 2D gate's label
__device__ float weight_distance3(const double* __restrict__ W, const Geo3& g, size_t c, size_t stride, int ax) {
    const size_t plane = (size_t)g.nx * g.ny * g.nz;
    const float gamma = g.fgamma;
    float st[5][5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
        const size_t q = c + (size_t)(m - 2) * stride;   // m - 2 < 0 wraps; q stays in range
        double wv[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) wv[v] = W[v * plane + q];
        rotate_in<float>(ax, st[m], wv);
    }
    float pr[3][5];
#pragma unroll
    for (int m = 0; m < 3; ++m) prim5<float>(pr[m], st[1 + m], gamma);
    const float d[4] = {0.5f * 0.15f * 0.15f, 0.15f * 0.85f, 0.5f * 0.15f * 0.15f, 0.85f};
    float dmax = 0.0f;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        float base[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) base[v] = 0.5f * (pr[side == 0 ? 0 : 2][v] + pr[1][v]);
        Char5<float> ch;
        ch.init(base, gamma);
        float s5[5][5];
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            float q[5];
            if (g.characteristic) ch.to_char(q, st[m]);
            else for (int v = 0; v < 5; ++v) q[v] = st[m][v];
#pragma unroll
            for (int v = 0; v < 5; ++v) s5[v][m] = q[v];
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            float b[4];
            beta3<float>(s5[v], b);
            const float* q5 = s5[v];
            b[3] = beta5_big<float>(q5[0] - q5[2], q5[1] - q5[2], 0.0f, q5[3] - q5[2], q5[4] - q5[2]);
            const float tau = (1.0f / 3.0f) * (fabsf(b[3] - b[0]) + fabsf(b[3] - b[1]) + fabsf(b[3] - b[2]));
            float al[4], sum = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                // label epsilon 1e-6 (the 2D gate's and the tangential sweeps'): variations far
                // below the state's own size do not count as structure
                const float q = tau / (b[k] + 1e-6f);
                al[k] = d[k] * (1.0f + q * q);
                sum += al[k];
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) dmax = fmaxf(dmax, fabsf(al[k] / sum - d[k]));
        }
    }
    return dmax;
}

// density and pressure of every cell, ghosts included, in FP32: the FP64 state is read and
// converted once per cell rather than once per stencil use
__global__ void __launch_bounds__(256) density_pressure3(GateRun3 r) {
    if (r.ctl && !r.ctl->active) return;
    const size_t plane = (size_t)r.g.nx * r.g.ny * r.g.nz;
    const size_t c = (size_t)blockIdx.x * 256 + threadIdx.x;
    if (c >= plane) return;
    const double rho = r.W[c], mx = r.W[plane + c], my = r.W[2 * plane + c], mz = r.W[3 * plane + c], e = r.W[4 * plane + c];
    r.rp[c] = make_float2(float(rho), float((r.g.gamma - 1.0) * (e - 0.5 * (mx * mx + my * my + mz * mz) / rho)));
}

// One thread per cell, three rows of the network per cell (one per axis): the block's 768
// rows go through the tcgen05 routine of the 2D gate in two 512-row passes (axes x and y,
// then z with an empty second half).
__global__ void __launch_bounds__(GATE3_THREADS, 3) gate3_kernel(GateRun3 r) {
    using namespace gate;
    static_assert(GATE3_THREADS == TC_THREADS, "two network rows per thread and pass");
    __shared__ MlpTc mlp;
    __shared__ unsigned counts[6];   // cells x, y, z; smooth x, y, z of the block
    if (r.ctl && !r.ctl->active) return;   // uniform over the grid
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid < 6) counts[tid] = 0;
    mlp_tc_setup(mlp, r.net);   // synchronises the block
    unsigned phase = 0;
    bool broken = false;
    const Geo3& g = r.g;
    const size_t plane = (size_t)g.nx * g.ny * g.nz;
    const size_t c = (size_t)blockIdx.x * GATE3_THREADS + tid;
    const bool in = c < plane;
    const int k = in ? (int)(c % g.nz) : 0, j = in ? (int)((c / g.nz) % g.ny) : 0;
    const int i = in ? (int)(c / ((size_t)g.nz * g.ny)) : 0;
    auto stride_of = [&](int ax) {
        return ax == 0 ? (size_t)g.ny * g.nz : ax == 1 ? (size_t)g.nz : (size_t)1;
    };
    auto fits_of = [&](int ax) {
        const int pos = ax == 0 ? i : ax == 1 ? j : k, n = ax == 0 ? g.nx : ax == 1 ? g.ny : g.nz;
        return in && pos >= 2 && pos < n - 2;
    };
    // features of this cell along axis ax (zero where the stencil leaves the array)
    auto features = [&](int ax, float* f) {
#pragma unroll
        for (int q = 0; q < NF; ++q) f[q] = 0.0f;
        if (fits_of(ax)) {
            const size_t stride = stride_of(ax);
            float rs[5], ps[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                const float2 v = r.rp[c + (size_t)(m - 2) * stride];
                rs[m] = v.x;
                ps[m] = v.y;
            }
            indicator5(rs, f);
            indicator5(ps, f + 7);
        }
    };
    float z[3];
    {
        float f[NF];
        features(0, f);
        mlp_tc_put(mlp, 0, f);
        features(1, f);
        mlp_tc_put(mlp, 1, f);
        mlp_tc_eval(mlp, z, phase, broken);
        features(2, f);
        mlp_tc_put(mlp, 0, f);
#pragma unroll
        for (int q = 0; q < NF; ++q) f[q] = 0.0f;
        mlp_tc_put(mlp, 1, f);
        float zz[2];
        mlp_tc_eval(mlp, zz, phase, broken);
        z[2] = zz[0];
    }
    unsigned char flag = 0;
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        const size_t stride = stride_of(ax);
        const bool fits = fits_of(ax);
        const bool smooth = fits && z[ax] > r.threshold;
        const unsigned h = mix_hash((unsigned)c * 3u + (unsigned)ax + r.seed * 0x9e3779b9u);
        if (r.samples && fits && (h & r.sample_mask) == 0) {
            const float d = weight_distance3(r.W, g, c, stride, ax);
            const unsigned long long slot = atomicAdd(r.sample_count, 1ull);
            if (slot < r.capacity) {
                float f[NF];
                features(ax, f);
                float* o = r.samples + slot * NS;
#pragma unroll
                for (int q = 0; q < NF; ++q) o[q] = f[q];
                o[NF] = d <= GATE_EPS ? 1.0f : 0.0f;
                o[NF + 1] = d;
                o[NF + 2] = float(c);
                o[NF + 3] = float(ax);
            }
        }
        if (r.flags) {
            // audits are drawn per warp: an audited warp re-checks all its predicted-smooth cells
            const unsigned wid = blockIdx.x * (GATE3_THREADS / 32) + warp;
            const unsigned hw = mix_hash(wid * 3u + (unsigned)ax + r.seed * 0x85ebca6bu);
            if (smooth && (hw & r.audit_mask) == 0) {
                const float d = weight_distance3(r.W, g, c, stride, ax);
                atomicAdd(&r.stats->audited, 1ull);
                if (d > GATE_EPS) atomicAdd(&r.stats->false_neg, 1ull);
            }
            const unsigned fm = __ballot_sync(0xffffffffu, fits), sm = __ballot_sync(0xffffffffu, smooth);
            if (lane == 0) {
                atomicAdd(&counts[ax], (unsigned)__popc(fm));
                atomicAdd(&counts[3 + ax], (unsigned)__popc(sm));
            }
        }
        flag |= smooth ? (unsigned char)(1u << ax) : (unsigned char)0;
    }
    if (r.flags) {
        if (in) r.flags[c] = flag;
        __syncthreads();
        if (tid < 3) atomicAdd(&r.stats->cells[tid], (unsigned long long)counts[tid]);
        else if (tid < 6) atomicAdd(&r.stats->smooth[tid - 3], (unsigned long long)counts[tid]);
    }
    // a tensor-core wait past its limit: the block's cells got no smooth flags (full WENO-AO,
    // still correct); the solver's status records it and its next step does not start
    if (broken && tid == 0 && r.ctl) atomicOr(const_cast<unsigned*>(&r.ctl->status), WAIT_TIMEOUT_BIT);
    mlp_tc_teardown(mlp, phase, broken);
}

}  // namespace

cudaError_t launch_gate3(const GateRun3& r, cudaStream_t s, bool rp_ready) {
    const size_t plane = (size_t)r.g.nx * r.g.ny * r.g.nz;
    if (!rp_ready) density_pressure3<<<(unsigned)((plane + 255) / 256), 256, 0, s>>>(r);
    gate3_kernel<<<(unsigned)((plane + GATE3_THREADS - 1) / GATE3_THREADS), GATE3_THREADS, 0, s>>>(r);
    return cudaGetLastError();
}

}  // namespace d3
}  // namespace hos
