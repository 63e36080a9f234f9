// hos_gate.cuh -- the learned smoothness gate of the FP32-bulk path.
//
// A 16 -> 32 -> 32 -> 1 MLP (ReLU, BF16 weights and activations, FP32 accumulation on the
// tensor cores through mma.sync m16n8k16) reads, for one cell and one direction, the
// normalised WENO-AO smoothness indicators of the cell's normal stencil in density and
// pressure (7 per variable: the candidate-stencil betas padded to 6, and tau) and the cell's
// discontinuity-feedback indicator, and predicts whether the nonlinear WENO-AO weights of all
// four characteristic variables on both faces of the cell stay within GATE_EPS of the linear
// weights.  Where it says so, the face kernel reconstructs with the full-stencil polynomial
// alone (no characteristic projection, no weights); everything else, and every linear result
// that fails the positivity / oscillation check, takes the full WENO-AO path.
//
// The reference has no such gate; its full WENO-AO reconstruction (src/reconstruction.cpp)
// stays the judge: labels, audits and the deviation tests compare against it.
#pragma once
#include <cuda_bf16.h>

#include "hos_kernels.cuh"
#include "hos_umma.cuh"

namespace hos {
namespace gate {

constexpr int NF = 16;   // inputs
constexpr int NH = 32;   // hidden width
// parameter vector (floats): W1[NH][NF], b1[NH], W2[NH][NH], b2[NH], w3[NH], b3 -- weights
// stored output-major (W[out][in]) so that an mma B fragment pair is one 32-bit load
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + NH * NF;
constexpr int OFF_W2 = OFF_B1 + NH;
constexpr int OFF_B2 = OFF_W2 + NH * NH;
constexpr int OFF_W3 = OFF_B2 + NH;
constexpr int OFF_B3 = OFF_W3 + NH;
constexpr int NPARAM = OFF_B3 + 1;
constexpr float GATE_EPS = 0.02f;   // label: max_k |omega_k - d_k| <= GATE_EPS
constexpr int NS = NF + 4;          // sample record: features, label, distance, cell, direction

// inference copy of the network: BF16 weights (w3 padded to 8 output rows) and FP32 biases
struct Net {
    const __nv_bfloat16* w1;   // [NH][NF]
    const __nv_bfloat16* w2;   // [NH][NH]
    const __nv_bfloat16* w3;   // [8][NH], rows 1..7 zero
    const float* b1;
    const float* b2;
    const float* b3;
};
constexpr size_t NET_BF16 = NH * NF + NH * NH + 8 * NH;   // bf16 elements of the inference copy
constexpr size_t NET_F32 = NH + NH + 1;                  // fp32 elements (biases)

struct Stats {
    unsigned long long cells[2];      // cells gated per direction
    unsigned long long smooth[2];     // predicted smooth per direction
    unsigned long long audited;       // predicted-smooth cells re-checked with full weights
    unsigned long long false_neg;     // of those, weights farther than GATE_EPS from linear
    unsigned long long samples;       // training samples written
    unsigned long long fallback;      // linear results rejected by the a-posteriori check
    // linear reconstructions in cell-directions an audit found not smooth (flag bits 2 + d):
    // tried, and accepted by the a-posteriori check
    unsigned long long fn_linear, fn_linear_accepted;
};

// ---------------- features ----------------

// Normalised indicators of one stencil: betas / (sum beta + tau + 1e-10 c^2), padded to 6, then
// tau.  The floor keeps variations below 1e-5 of the value (FP32 rounding of the primitives
// included) from looking like structure.
// T = float, or F2 for two stencils at once (the gate kernels: a cell's x and y stencils).
template <int ORDER, class T = float>
__device__ __forceinline__ void indicator_features(const T* s, T* f) {
    constexpr int NW = AO<ORDER>::N;
    T beta[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) beta[k] = T(0.0f);
    const T tau = ao_betas<T, ORDER>(s, beta);
    T sum = tau;
#pragma unroll
    for (int k = 0; k < NW; ++k) sum = sum + beta[k];
    const T c = s[ORDER / 2];
    const T inv = T(1.0f) / (sum + T(1e-10f) * c * c + T(1e-30f));
#pragma unroll
    for (int k = 0; k < 6; ++k) f[k] = k < NW ? T(beta[k] * inv) : T(0.0f);
    f[6] = tau * inv;
}

// True label quantity of cell c along DIR: the largest distance of the nonlinear weights from
// the linear ones over both faces and the four (characteristic) variables, computed as the
// face kernel's normal reconstruction would (src/reconstruction.cpp:1861-2028 for WENO7).
template <int ORDER, int DIR>
__device__ __forceinline__ float weight_distance(const double* __restrict__ W, size_t plane, size_t c,
                                                 long long stride, float gamma, int characteristic) {
    constexpr int N = ORDER, r = ORDER / 2;
    float st[N][4];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const size_t q = (size_t)((long long)c + (k - r) * stride);
        const float w0 = float(W[q]), w1 = float(W[plane + q]), w2 = float(W[2 * plane + q]), w3 = float(W[3 * plane + q]);
        st[k][0] = w0;
        st[k][1] = DIR == 0 ? w1 : w2;   // y stencils in the rotated frame (YchangetoX)
        st[k][2] = DIR == 0 ? w2 : -w1;
        st[k][3] = w3;
    }
    float pn1[4], p0[4], pp1[4];
    to_prim(pn1, st[r - 1], gamma);
    to_prim(p0, st[r], gamma);
    to_prim(pp1, st[r + 1], gamma);
    float dmax = 0.0f;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        float ch[N][4];
        if (characteristic) {
            float base[4];
#pragma unroll
            for (int v = 0; v < 4; ++v) base[v] = 0.5f * ((side == 0 ? pn1[v] : pp1[v]) + p0[v]);
            CharBase<float> cb;
            cb.init(base, gamma);
#pragma unroll
            for (int k = 0; k < N; ++k) cb.to_char(ch[k], st[k]);
        } else {
#pragma unroll
            for (int k = 0; k < N; ++k)
#pragma unroll
                for (int v = 0; v < 4; ++v) ch[k][v] = st[k][v];
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            float s[N];
#pragma unroll
            for (int k = 0; k < N; ++k) s[k] = ch[k][v];
            dmax = fmaxf(dmax, ao_weight_distance<float, ORDER>(s));
        }
    }
    return dmax;
}

// ---------------- the MLP on the tensor cores ----------------

__device__ __forceinline__ void mma_bf16_16816(float* c, const unsigned* a, unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&v);
}

__device__ __forceinline__ unsigned ld_pair(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

// One warp evaluates 16 rows: x points at the rows' BF16 features ([16][NF], row stride NF);
// hidden activations (after ReLU, rounded to BF16 as the next layer reads them) go to h1/h2
// ([16][NH] FP32, may be null) and the output logits to z[16].
__device__ __forceinline__ void mlp16(const Net& net, const __nv_bfloat16* x, float* h1, float* h2, float* z) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    unsigned a[4];
    a[0] = ld_pair(x + g * NF + 2 * t);
    a[1] = ld_pair(x + (g + 8) * NF + 2 * t);
    a[2] = ld_pair(x + g * NF + 2 * t + 8);
    a[3] = ld_pair(x + (g + 8) * NF + 2 * t + 8);
    float c1[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const int n = nt * 8 + 2 * t;
        c1[nt][0] = net.b1[n];
        c1[nt][1] = net.b1[n + 1];
        c1[nt][2] = net.b1[n];
        c1[nt][3] = net.b1[n + 1];
        const __nv_bfloat16* wr = net.w1 + (nt * 8 + g) * NF;
        mma_bf16_16816(c1[nt], a, ld_pair(wr + 2 * t), ld_pair(wr + 2 * t + 8));
#pragma unroll
        for (int q = 0; q < 4; ++q) c1[nt][q] = __bfloat162float(__float2bfloat16_rn(fmaxf(c1[nt][q], 0.0f)));
        if (h1) {
            h1[g * NH + n] = c1[nt][0];
            h1[g * NH + n + 1] = c1[nt][1];
            h1[(g + 8) * NH + n] = c1[nt][2];
            h1[(g + 8) * NH + n + 1] = c1[nt][3];
        }
    }
    float c2[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const int n = nt * 8 + 2 * t;
        c2[nt][0] = net.b2[n];
        c2[nt][1] = net.b2[n + 1];
        c2[nt][2] = net.b2[n];
        c2[nt][3] = net.b2[n + 1];
    }
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        // accumulator fragments of layer 1 are the A fragments of layer 2
        unsigned a2[4] = {pack_bf16(c1[2 * ks][0], c1[2 * ks][1]), pack_bf16(c1[2 * ks][2], c1[2 * ks][3]),
                          pack_bf16(c1[2 * ks + 1][0], c1[2 * ks + 1][1]),
                          pack_bf16(c1[2 * ks + 1][2], c1[2 * ks + 1][3])};
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const __nv_bfloat16* wr = net.w2 + (nt * 8 + g) * NH + ks * 16;
            mma_bf16_16816(c2[nt], a2, ld_pair(wr + 2 * t), ld_pair(wr + 2 * t + 8));
        }
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const int n = nt * 8 + 2 * t;
#pragma unroll
        for (int q = 0; q < 4; ++q) c2[nt][q] = __bfloat162float(__float2bfloat16_rn(fmaxf(c2[nt][q], 0.0f)));
        if (h2) {
            h2[g * NH + n] = c2[nt][0];
            h2[g * NH + n + 1] = c2[nt][1];
            h2[(g + 8) * NH + n] = c2[nt][2];
            h2[(g + 8) * NH + n + 1] = c2[nt][3];
        }
    }
    float c3[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
        unsigned a3[4] = {pack_bf16(c2[2 * ks][0], c2[2 * ks][1]), pack_bf16(c2[2 * ks][2], c2[2 * ks][3]),
                          pack_bf16(c2[2 * ks + 1][0], c2[2 * ks + 1][1]),
                          pack_bf16(c2[2 * ks + 1][2], c2[2 * ks + 1][3])};
        const __nv_bfloat16* wr = net.w3 + g * NH + ks * 16;
        mma_bf16_16816(c3, a3, ld_pair(wr + 2 * t), ld_pair(wr + 2 * t + 8));
    }
    if (t == 0) {   // output column 0
        z[g] = c3[0] + net.b3[0];
        z[g + 8] = c3[2] + net.b3[0];
    }
}

// ---------------- the MLP on the 5th-generation tensor cores (tcgen05) ----------------
// The gate kernels evaluate the network for 512 rows per CTA, two per thread (row t and row
// 256 + t: a cell's x and y stencils): layer 1 is four 128 x 32 x 16 MMAs, layer 2 four
// 128 x 32 x 32 MMAs (two K steps each), issued by one thread over BF16 operands in shared
// memory with FP32 accumulators in 128 tensor-memory columns (columns 32 m .. 32 m + 31 hold
// rows 128 m .. 128 m + 127).  Bias, ReLU and the BF16 rounding of the activations run on the
// CUDA cores between the layers, as does the 32-wide output layer.  Rounding points are those
// of mlp16 above (BF16 inputs, weights and activations, FP32 accumulation).
constexpr int TC_THREADS = 256;
constexpr int TC_ROWS = 2 * TC_THREADS;
constexpr int TC_MTILES = TC_ROWS / 128;
constexpr uint32_t TC_COLS = TC_MTILES * NH;

struct MlpTc {
    // features (K = 16, 16 KB) until the layer-1 MMAs have read them, then the layer-1
    // activations (K = 32, 32 KB) over the same bytes
    alignas(128) unsigned char act[TC_ROWS * NH * 2];
    alignas(128) unsigned char b1[NH * NF * 2];        // W1 [out][in], K-major canonical layout
    alignas(128) unsigned char b2[NH * NH * 2];        // W2 [out][in]
    float bias1[NH], bias2[NH], w3[NH];
    float b3;
    uint64_t bar;        // tcgen05.commit arrives here once the issued MMAs complete
    uint32_t tmem;       // base address of the CTA's tensor-memory columns
};

// Per-CTA set-up, by all TC_THREADS threads: weights into the operand layouts, the barrier,
// the tensor memory.  An allocation that finds the SM's 512 columns taken waits for resident
// CTAs to release theirs; they never wait on this one.
__device__ __forceinline__ void mlp_tc_setup(MlpTc& s, const Net& net) {
    const int tid = threadIdx.x;
    for (int e = tid; e < NH * NF; e += blockDim.x)
        *reinterpret_cast<__nv_bfloat16*>(s.b1 + umma::kmajor_offset<NF>(e / NF, e % NF)) = net.w1[e];
    for (int e = tid; e < NH * NH; e += blockDim.x)
        *reinterpret_cast<__nv_bfloat16*>(s.b2 + umma::kmajor_offset<NH>(e / NH, e % NH)) = net.w2[e];
    if (tid < NH) {
        s.bias1[tid] = net.b1[tid];
        s.bias2[tid] = net.b2[tid];
        s.w3[tid] = __bfloat162float(net.w3[tid]);
    }
    if (tid == 0) {
        s.b3 = net.b3[0];
        mbar_init(&s.bar, 1);
    }
    if (tid < 32) umma::tmem_alloc(&s.tmem, TC_COLS);
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
}

// Per-CTA tear-down, by all threads: after a wait that ran past its limit, the MMAs still in
// flight get one more bounded wait before their columns are released.
__device__ __forceinline__ void mlp_tc_teardown(MlpTc& s, unsigned phase, bool broken) {
    if (broken) mbar_wait(&s.bar, phase);
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) {
        umma::fence_after_sync();
        umma::tmem_dealloc(s.tmem, TC_COLS);
    }
}

// Row h * 256 + t of the network's input (x: its NF features), written by thread t.
__device__ __forceinline__ void mlp_tc_put(MlpTc& s, int h, const float* x) {
    const int row = h * TC_THREADS + threadIdx.x;
    *reinterpret_cast<uint4*>(s.act + umma::kmajor_offset<NF>(row, 0)) =
        make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]), pack_bf16(x[6], x[7]));
    *reinterpret_cast<uint4*>(s.act + umma::kmajor_offset<NF>(row, 8)) =
        make_uint4(pack_bf16(x[8], x[9]), pack_bf16(x[10], x[11]), pack_bf16(x[12], x[13]), pack_bf16(x[14], x[15]));
}

// Logits z[0], z[1] of this thread's rows t and 256 + t, whose features every thread has put
// (mlp_tc_put); called by all 256 threads of the CTA.  phase: parity of the barrier's next
// phase, the same in every thread.  A wait past its limit sets broken (uniformly): the network
// is then not evaluated any more (-inf: not smooth) and the caller records the timeout.
__device__ __forceinline__ void mlp_tc_eval(MlpTc& s, float* z, unsigned& phase, bool& broken) {
    const int tid = threadIdx.x, warp = tid >> 5;
    z[0] = z[1] = -INFINITY;
    if (broken) return;
    umma::fence_smem_to_async();
    __syncthreads();
    constexpr uint32_t ID = umma::idesc_bf16_f32<128, NH>();
    constexpr uint32_t LBO = umma::KMAJOR_LBO, SBO1 = umma::kmajor_sbo<NF>(), SBO2 = umma::kmajor_sbo<NH>();
    const uint32_t tm = s.tmem;
    if (tid == 0) {
        umma::fence_after_sync();
#pragma unroll
        for (int mt = 0; mt < TC_MTILES; ++mt)
            umma::mma_bf16(tm + mt * NH, umma::smem_desc(s.act + mt * 128 * NF * 2, LBO, SBO1),
                           umma::smem_desc(s.b1, LBO, SBO1), ID, 0);
        umma::commit(&s.bar);
    }
    if (!__syncthreads_and(mbar_wait(&s.bar, phase))) {
        broken = true;
        return;
    }
    phase ^= 1u;
    umma::fence_after_sync();
    // row h * 256 + t sits in M tile 2 h + warp / 4, tensor-memory lane 32 (warp % 4) + lane
    const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
    float d[NH];
    // every layer-1 MMA has read the features: the activations overwrite them
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        umma::ld_32cols(tm + lanes + (uint32_t)(2 * h + (warp >> 2)) * NH, d);
#pragma unroll
        for (int q = 0; q < NH / 8; ++q) {
            float a[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] = fmaxf(d[8 * q + k] + s.bias1[8 * q + k], 0.0f);
            *reinterpret_cast<uint4*>(s.act + umma::kmajor_offset<NH>(h * TC_THREADS + tid, 8 * q)) =
                make_uint4(pack_bf16(a[0], a[1]), pack_bf16(a[2], a[3]), pack_bf16(a[4], a[5]), pack_bf16(a[6], a[7]));
        }
    }
    umma::fence_before_sync();
    umma::fence_smem_to_async();
    __syncthreads();
    if (tid == 0) {
        umma::fence_after_sync();
#pragma unroll
        for (int mt = 0; mt < TC_MTILES; ++mt)
#pragma unroll
            for (int ks = 0; ks < NH / 16; ++ks)
                umma::mma_bf16(tm + mt * NH, umma::smem_desc(s.act + mt * 128 * NH * 2 + ks * 2 * LBO, LBO, SBO2),
                               umma::smem_desc(s.b2 + ks * 2 * LBO, LBO, SBO2), ID, (uint32_t)ks);
        umma::commit(&s.bar);
    }
    if (!__syncthreads_and(mbar_wait(&s.bar, phase))) {
        broken = true;
        return;
    }
    phase ^= 1u;
    umma::fence_after_sync();
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        umma::ld_32cols(tm + lanes + (uint32_t)(2 * h + (warp >> 2)) * NH, d);
        float o = s.b3;
#pragma unroll
        for (int k = 0; k < NH; ++k)
            o += __bfloat162float(__float2bfloat16_rn(fmaxf(d[k] + s.bias2[k], 0.0f))) * s.w3[k];
        z[h] = o;
    }
    umma::fence_before_sync();
}

__device__ __forceinline__ unsigned mix_hash(unsigned x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

struct GateArgs {
    const double* W;
    const double* AX;
    const double* AY;
    unsigned char* flags;      // [nx*ny]: bit 0 x-smooth, bit 1 y-smooth (null in collect mode)
    Stats* stats;
    float threshold;           // logit above which a cell is predicted smooth
    unsigned audit_mask;       // audit predicted-smooth cells whose hash & mask == 0
    unsigned seed;
    float* samples;            // collect mode: [capacity][NS] features, label, distance, cell, dir
    unsigned long long capacity;
    unsigned sample_mask;      // collect cells whose hash & mask == 0
    const StepCtl* ctl;        // inactive problems skip (may be null)
    const float* W32 = nullptr;   // FP32 mirror of W (FP32 solvers; null: convert W)
};

constexpr int GATE_THREADS = 256;
constexpr int GATE_TILE = 16;   // 16 x 16 cells per block, one thread per cell

// One block per 16 x 16 tile of cells, one thread per cell, both directions.  The tile and
// its stencil halo are converted once to FP32 density and pressure in shared memory; the
// features are read from there.  Stencils that leave the array get no flag (the face kernel
// then reconstructs that cell with full WENO-AO).  The network runs on the tcgen05 tensor
// cores for the tile's 256 cells per direction (mlp: set up by the kernel, see mlp_tc_rows).
// One 16 x 16 tile with first cell (i0, j0); tile_id numbers the tile for the audit draw.
static_assert(GATE_TILE * GATE_TILE == TC_THREADS && GATE_THREADS == TC_THREADS, "two network rows per thread");

// TMA box of a gate tile in the FP32 mirror (x along j, y along i, the six planes): the tile
// and its stencil halo, the x origin rounded down to 16 bytes.  It is staged in the network's
// operand region, which is free until the features are written.
template <int ORDER>
struct GateBox {
    static constexpr int H = GATE_TILE + 2 * (ORDER / 2);
    static constexpr int X = (H + 3 + 3) / 4 * 4, Y = H, Z = MIRROR_PLANES;
    static constexpr unsigned bytes = 4u * X * Y * Z;
    static_assert(bytes <= sizeof(MlpTc::act), "the staged box must fit the operand region");
};

// tmap (TMA): the mirror's tensor map with the GateBox<ORDER> box; the tile is then staged by
// one TMA tile load instead of per-cell loads of the mirror
// iter: tiles this block handled before (TMA: the load barrier is initialised on the first and
// its phase parity follows the count).
template <int ORDER, bool TMA = false>
__device__ __forceinline__ void gate_tile(const GateArgs& a, const Geometry& geo, int i0, int j0, unsigned tile_id,
                                          MlpTc& mlp, unsigned& phase, bool& broken,
                                          const CUtensorMap* tmap = nullptr, int iter = 0) {
    constexpr int r = ORDER / 2, H = GATE_TILE + 2 * r;
    __shared__ float srho[H][H + 1], sp[H][H + 1];
    __shared__ float salpha[2][GATE_TILE * GATE_TILE];   // TMA: the tile cells' alpha_x, alpha_y
    __shared__ unsigned counts[4];           // cells x, cells y, smooth x, smooth y of the block
    if (a.ctl && !a.ctl->active) return;   // uniform over the block
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid < 4) counts[tid] = 0;
    const size_t plane = (size_t)geo.nx * geo.ny;
    const float gamma = float(geo.gamma);
    if constexpr (TMA) {
        using B = GateBox<ORDER>;
        constexpr int PZ = B::X * B::Y;
        __shared__ __align__(8) uint64_t gbar;
        float* stg = reinterpret_cast<float*>(mlp.act);
        const int x0 = j0 - r, y0 = i0 - r, xa = x0 & ~3, off = x0 - xa;   // negative origins read zeros
        const unsigned par = (unsigned)iter & 1u;
        // after a load that did not complete (broken, uniform over the block) the barrier's phase
        // is unknown: no further loads are issued, and the network is skipped for the rest
        if (!broken) {
            if (tid == 0) {
                if (iter == 0) mbar_init(&gbar, 1);
                mbar_expect_tx(&gbar, B::bytes);
                tma_load_3d(stg, tmap, xa, y0, 0, &gbar);
            }
            __syncthreads();
            if (!__syncthreads_and(mbar_wait(&gbar, par))) {
                // the load did not complete: let a late one land, and flag no cell of the kernel
                // smooth (the network is skipped; the caller records the timeout)
                mbar_wait(&gbar, par);
                broken = true;
            }
        }
        for (int e = tid; e < H * H; e += GATE_THREADS) {
            const int hi = e / H, hj = e % H;
            const int gi = i0 - r + hi, gj = j0 - r + hj;
            float rho = 0.0f, pr = 0.0f;
            if (gi >= 0 && gi < geo.nx && gj >= 0 && gj < geo.ny) {
                const float* q = stg + hi * B::X + off + hj;
                float w[4] = {q[0], q[PZ], q[2 * PZ], q[3 * PZ]}, pv[4];
                to_prim(pv, w, gamma);
                rho = pv[0];
                pr = pv[3];
            }
            srho[hi][hj] = rho;
            sp[hi][hj] = pr;
            if (hi >= r && hi < r + GATE_TILE && hj >= r && hj < r + GATE_TILE) {
                const int t = (hi - r) * GATE_TILE + (hj - r);
                salpha[0][t] = stg[4 * PZ + hi * B::X + off + hj];
                salpha[1][t] = stg[5 * PZ + hi * B::X + off + hj];
            }
        }
    } else
    for (int e = tid; e < H * H; e += GATE_THREADS) {
        const int hi = e / H, hj = e % H;               // j fastest: coalesced rows
        const int gi = i0 - r + hi, gj = j0 - r + hj;
        float rho = 0.0f, pr = 0.0f;
        if (gi >= 0 && gi < geo.nx && gj >= 0 && gj < geo.ny) {
            const size_t q = (size_t)gi * geo.ny + gj;
            float w[4];
            if (a.W32) {
                // the FP32 mirror's rows are padded to mirror_pitch(ny)
                const size_t p32 = (size_t)mirror_pitch(geo.ny), pl32 = (size_t)geo.nx * p32;
                const size_t qm = (size_t)gi * p32 + gj;
                w[0] = a.W32[qm]; w[1] = a.W32[pl32 + qm]; w[2] = a.W32[2 * pl32 + qm]; w[3] = a.W32[3 * pl32 + qm];
            } else {
                w[0] = float(a.W[q]); w[1] = float(a.W[plane + q]); w[2] = float(a.W[2 * plane + q]); w[3] = float(a.W[3 * plane + q]);
            }
            float pv[4];
            to_prim(pv, w, gamma);
            rho = pv[0];
            pr = pv[3];
        }
        srho[hi][hj] = rho;
        sp[hi][hj] = pr;
    }
    __syncthreads();
    const int ti = tid / GATE_TILE, tj = tid % GATE_TILE;
    const int i = i0 + ti, j = j0 + tj;
    const bool in = i < geo.nx && j < geo.ny;
    const size_t c = in ? (size_t)i * geo.ny + j : 0;
    unsigned char flag = 0;
    // features of this cell along dir (zero where the stencil leaves the array)
    auto features = [&](int dir, float* f) {
        const int pos = dir == 0 ? i : j, n = dir == 0 ? geo.nx : geo.ny;
        const bool fits = in && pos >= r && pos < n - r;
        if (fits) {
            float rs[ORDER], ps[ORDER];
#pragma unroll
            for (int k = 0; k < ORDER; ++k) {
                const int hi = dir == 0 ? ti + k : ti + r, hj = dir == 0 ? tj + r : tj + k;
                rs[k] = srho[hi][hj];
                ps[k] = sp[hi][hj];
            }
            indicator_features<ORDER>(rs, f);
            indicator_features<ORDER>(ps, f + 7);
            float al;
            if constexpr (TMA) al = salpha[dir][tid];   // the mirror's FP32 copy of alpha
            else al = float(dir == 0 ? a.AX[c] : a.AY[c]);
            f[14] = al / (1.0f + al);
            f[15] = 0.0f;
        } else {
#pragma unroll
            for (int k = 0; k < NF; ++k) f[k] = 0.0f;
        }
    };
    // both directions' features into the network's input, then one pass over the tile's 512
    // rows; the x and y stencils of the cell run in the two lanes of the paired FP32 type.
    // Sampled cells (collect mode) compute their features again afterwards, one direction at a
    // time.
    {
        const bool fx = in && i >= r && i < geo.nx - r, fy = in && j >= r && j < geo.ny - r;
        F2 rs[ORDER], ps[ORDER], f2[NF];
#pragma unroll
        for (int k = 0; k < ORDER; ++k) {
            rs[k] = F2(srho[ti + k][tj + r], srho[ti + r][tj + k]);
            ps[k] = F2(sp[ti + k][tj + r], sp[ti + r][tj + k]);
        }
        indicator_features<ORDER, F2>(rs, f2);
        indicator_features<ORDER, F2>(ps, f2 + 7);
        float ax, ay;
        if constexpr (TMA) {
            ax = salpha[0][tid];   // the mirror's FP32 copy of alpha
            ay = salpha[1][tid];
        } else {
            ax = in ? float(a.AX[c]) : 0.0f;
            ay = in ? float(a.AY[c]) : 0.0f;
        }
        f2[14] = F2(ax / (1.0f + ax), ay / (1.0f + ay));
        f2[15] = F2(0.0f);
        float f[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) f[k] = fx ? f2[k].v.x : 0.0f;
        mlp_tc_put(mlp, 0, f);
#pragma unroll
        for (int k = 0; k < NF; ++k) f[k] = fy ? f2[k].v.y : 0.0f;
        mlp_tc_put(mlp, 1, f);
    }
    float zd[2];
    mlp_tc_eval(mlp, zd, phase, broken);
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const int pos = dir == 0 ? i : j, n = dir == 0 ? geo.nx : geo.ny;
        const bool fits = in && pos >= r && pos < n - r;
        const long long stride = dir == 0 ? geo.ny : 1;
        const bool smooth = fits && zd[dir] > a.threshold;
        const unsigned h = mix_hash((unsigned)c * 2u + (unsigned)dir + a.seed * 0x9e3779b9u);
        if (a.samples && fits && (h & a.sample_mask) == 0) {
            const float d = dir == 0 ? weight_distance<ORDER, 0>(a.W, plane, c, stride, gamma, geo.characteristic)
                                     : weight_distance<ORDER, 1>(a.W, plane, c, stride, gamma, geo.characteristic);
            const unsigned long long slot = atomicAdd(&a.stats->samples, 1ull);
            if (slot < a.capacity) {
                float f[NF];
                features(dir, f);
                float* o = a.samples + slot * NS;
#pragma unroll
                for (int k = 0; k < NF; ++k) o[k] = f[k];
                o[NF] = d <= GATE_EPS ? 1.0f : 0.0f;
                o[NF + 1] = d;
                o[NF + 2] = float(c);
                o[NF + 3] = float(dir);
            }
        }
        if (a.flags) {
            // audits are drawn per warp, so an audited warp re-checks all its predicted-smooth
            // cells together instead of stalling 31 lanes behind one
            const unsigned wid = tile_id * (GATE_THREADS / 32) + warp;
            const unsigned hw = mix_hash(wid * 2u + (unsigned)dir + a.seed * 0x85ebca6bu);
            if (smooth && (hw & a.audit_mask) == 0) {
                const float d = dir == 0 ? weight_distance<ORDER, 0>(a.W, plane, c, stride, gamma, geo.characteristic)
                                         : weight_distance<ORDER, 1>(a.W, plane, c, stride, gamma, geo.characteristic);
                atomicAdd(&a.stats->audited, 1ull);
                if (d > GATE_EPS) {
                    atomicAdd(&a.stats->false_neg, 1ull);
                    flag |= (unsigned char)(4u << dir);   // the face kernels count what the check does with it
                }
            }
            const unsigned fits_mask = __ballot_sync(0xffffffffu, fits);
            const unsigned smooth_mask = __ballot_sync(0xffffffffu, smooth);
            if (lane == 0) {
                atomicAdd(&counts[dir], (unsigned)__popc(fits_mask));
                atomicAdd(&counts[2 + dir], (unsigned)__popc(smooth_mask));
            }
        }
        flag |= smooth ? (unsigned char)(1u << dir) : (unsigned char)0;
        __syncwarp();
    }
    if (a.flags && in) a.flags[c] = flag;
    if (a.flags) {
        // one global update per block and counter
        __syncthreads();
        if (tid < 2) atomicAdd(&a.stats->cells[tid], (unsigned long long)counts[tid]);
        else if (tid < 4) atomicAdd(&a.stats->smooth[tid - 2], (unsigned long long)counts[tid]);
    }
    // a tensor-core wait past its limit: the tile got no smooth flags (full WENO-AO, still
    // correct); the problem's status records it and its next step does not start
    if (broken && tid == 0 && a.ctl) atomicOr(const_cast<unsigned*>(&a.ctl->status), WAIT_TIMEOUT_BIT);
    __syncthreads();   // the shared arrays are reused by the block's next tile
}

// Persistent blocks (a grid of resident blocks) walk the 16 x 16 tiles, so the network's
// set-up (weights into the operand layouts, tensor memory, barrier) happens once per block.  The
// kernel is latency bound (the tile loads, the two MMA round trips): WENO5/7 tiles fit three
// blocks per SM in registers, WENO9 two.  ntx: tiles along j; ntiles: all tiles.
template <int ORDER>
__global__ void __launch_bounds__(GATE_THREADS, ORDER == 9 ? 2 : 3)
    gate_kernel(GateArgs a, Net net, Geometry geo, int ntx, int ntiles) {
    __shared__ MlpTc mlp;
    if (a.ctl && !a.ctl->active) return;   // uniform: nothing allocated yet
    mlp_tc_setup(mlp, net);
    unsigned phase = 0;
    bool broken = false;
    for (int k = blockIdx.x; k < ntiles; k += gridDim.x)
        gate_tile<ORDER>(a, geo, (k / ntx) * GATE_TILE, (k % ntx) * GATE_TILE, (unsigned)k, mlp, phase, broken);
    mlp_tc_teardown(mlp, phase, broken);
}

// the FP32 solvers' gate: each tile staged from the FP32 mirror by one TMA tile load
template <int ORDER>
__global__ void __launch_bounds__(GATE_THREADS, ORDER == 9 ? 2 : 3)
    gate_kernel_tma(GateArgs a, Net net, Geometry geo, int ntx, int ntiles, const __grid_constant__ CUtensorMap tmap) {
    __shared__ MlpTc mlp;
    if (a.ctl && !a.ctl->active) return;   // uniform: nothing allocated yet
    mlp_tc_setup(mlp, net);
    unsigned phase = 0;
    bool broken = false;
    for (int k = blockIdx.x, it = 0; k < ntiles; k += gridDim.x, ++it)
        gate_tile<ORDER, true>(a, geo, (k / ntx) * GATE_TILE, (k % ntx) * GATE_TILE, (unsigned)k, mlp, phase, broken,
                               &tmap, it);
    mlp_tc_teardown(mlp, phase, broken);
}

}  // namespace gate
}  // namespace hos

// ---------------- host side (hos_gate.cu) ----------------
namespace hos {
namespace gate {
// tm (may be null): the FP32 mirror's tensor map with the GateBox<order> box; with it the
// tiles are staged by TMA
cudaError_t launch_gate(int order, const GateArgs& a, const Net& net, const Geometry& geo, cudaStream_t s,
                        const CUtensorMap* tm = nullptr);
}  // namespace gate
}  // namespace hos

// the network object behind the C ABI's hos_gate handle
struct hos_gate {
    float* params = nullptr;          // [NPARAM] FP32 master parameters
    float* m = nullptr;               // Adam moments
    float* v = nullptr;
    float* grad = nullptr;
    __nv_bfloat16* wbf = nullptr;     // inference copy: w1 | w2 | w3 (NET_BF16)
    float* bias = nullptr;            // b1 | b2 | b3 (NET_F32)
    float* samples = nullptr;         // [capacity][NS]
    unsigned long long capacity = 0;
    hos::gate::Stats* stats = nullptr;
    double* loss = nullptr;
    int step = 0;
    unsigned collect_seed = 1;
    cudaStream_t stream = nullptr;
    hos::gate::Net net() const {
        using namespace hos::gate;
        return Net{wbf, wbf + NH * NF, wbf + NH * NF + NH * NH, bias, bias + NH, bias + 2 * NH};
    }
};
