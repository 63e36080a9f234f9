// hos_gate.cu -- the learned gate's network object: creation, parameters, training on the
// GPU (forward on the tensor cores, backward and Adam on the FP32 cores) and the per-stage
// gate launch.  The solver couples it to a problem in hos_solver.cu (hos2d_set_gate,
// hos_gate_collect).  The reference has no counterpart.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/hos_gb300.h"
#include "hos_gate.cuh"

namespace hos {
namespace gate {

// ---------------- training ----------------

constexpr int TRAIN_ROWS = 64;    // samples per block (4 warps x 16); 2 threads per sample

struct TrainArgs {
    const float* samples;        // [n][NF + 2]
    unsigned long long n;
    unsigned long long first;    // batch start in the permuted order
    unsigned long long stride;   // permutation: index = (first + k) * stride mod n, stride coprime to n
    int batch;
    float w_pos, w_neg;          // class weights of smooth (1) and non-smooth (0) samples
    float* grad;                 // [NPARAM] accumulated (atomic) gradient of the mean loss
    double* loss;                // accumulated loss (may be null)
    float* logits;               // forward-only: [n] outputs (may be null)
};

// Logits of samples [first, first + n) through the inference network on the tcgen05 tensor
// cores (the gate kernels' routine), 512 samples per block of 256 threads; status bit 0: a
// wait ran past its limit.
__global__ void __launch_bounds__(TC_THREADS) forward_tc_kernel(const float* samples, unsigned long long first,
                                                                int n, Net net, float* logits, unsigned* status) {
    __shared__ MlpTc mlp;
    mlp_tc_setup(mlp, net);
    unsigned phase = 0;
    bool broken = false;
    float f[2][NF], z[2];
    long long b[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        b[h] = (long long)blockIdx.x * TC_ROWS + h * TC_THREADS + threadIdx.x;
#pragma unroll
        for (int k = 0; k < NF; ++k) f[h][k] = b[h] < n ? samples[(first + (unsigned long long)b[h]) * NS + k] : 0.0f;
    }
    mlp_tc_put(mlp, 0, f[0]);
    mlp_tc_put(mlp, 1, f[1]);
    mlp_tc_eval(mlp, z, phase, broken);
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (b[h] < n) logits[b[h]] = z[h];
    if (broken && threadIdx.x == 0) atomicOr(status, 1u);
    mlp_tc_teardown(mlp, phase, broken);
}

// Forward on the tensor cores (mma.sync, keeping the hidden activations for the backward
// pass), backward on the FP32 cores; each block
// adds its share of the weighted binary cross-entropy gradient to a.grad.
__global__ void __launch_bounds__(TRAIN_ROWS * 2) train_grad_kernel(TrainArgs a, Net net, const float* params) {
    __shared__ __align__(16) __nv_bfloat16 xs[TRAIN_ROWS * NF];
    __shared__ float h1[TRAIN_ROWS][NH], h2[TRAIN_ROWS][NH], z[TRAIN_ROWS], dz[TRAIN_ROWS];
    __shared__ float d2[TRAIN_ROWS][NH + 1], d1[TRAIN_ROWS][NH + 1];
    __shared__ float wq[NPARAM];   // BF16-rounded weights as the forward pass used them
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long row0 = (long long)blockIdx.x * TRAIN_ROWS;
    for (int k = tid; k < NPARAM; k += blockDim.x) {
        const bool is_w = k < OFF_B1 || (k >= OFF_W2 && k < OFF_B2) || (k >= OFF_W3 && k < OFF_B3);
        wq[k] = is_w ? __bfloat162float(__float2bfloat16_rn(params[k])) : params[k];
    }
    float y_row = 0.0f;
    bool valid = false;
    if (tid < TRAIN_ROWS) {
        const long long b = row0 + tid;
        valid = b < a.batch;
        const float* s = nullptr;
        if (valid) {
            const unsigned long long idx = ((a.first + (unsigned long long)b) % a.n) * a.stride % a.n;
            s = a.samples + idx * NS;
            y_row = s[NF];
        }
#pragma unroll
        for (int k = 0; k < NF; ++k) xs[tid * NF + k] = __float2bfloat16_rn(valid ? s[k] : 0.0f);
    }
    __syncthreads();
    if (warp < TRAIN_ROWS / 16)
        mlp16(net, xs + warp * 16 * NF, &h1[warp * 16][0], &h2[warp * 16][0], z + warp * 16);
    __syncthreads();
    const float inv_b = 1.0f / float(a.batch);
    if (tid < TRAIN_ROWS) {
        float g = 0.0f;
        if (valid) {
            const float zz = z[tid];
            const float p = 1.0f / (1.0f + __expf(-zz));
            g = (y_row > 0.5f ? a.w_pos * (p - 1.0f) : a.w_neg * p) * inv_b;
            if (a.loss) {
                // softplus form of the cross-entropy
                const float sp = fmaxf(zz, 0.0f) + log1pf(__expf(-fabsf(zz)));
                const float l = y_row > 0.5f ? a.w_pos * (sp - zz) : a.w_neg * sp;
                atomicAdd(a.loss, double(l * inv_b));
            }
            if (a.logits) a.logits[row0 + tid] = zz;
        }
        dz[tid] = g;
    }
    __syncthreads();
    // dH2 = dz w3 * relu'(h2); dH1 = (dH2 W2) * relu'(h1)
    for (int e = tid; e < TRAIN_ROWS * NH; e += blockDim.x) {
        const int rr = e / NH, j = e % NH;
        d2[rr][j] = h2[rr][j] > 0.0f ? dz[rr] * wq[OFF_W3 + j] : 0.0f;
    }
    __syncthreads();
    for (int e = tid; e < TRAIN_ROWS * NH; e += blockDim.x) {
        const int rr = e / NH, i = e % NH;
        float s = 0.0f;
        if (h1[rr][i] > 0.0f)
#pragma unroll 8
            for (int j = 0; j < NH; ++j) s += d2[rr][j] * wq[OFF_W2 + j * NH + i];
        d1[rr][i] = s;
    }
    __syncthreads();
    // weight gradients summed over the block's rows
    for (int k = tid; k < NPARAM; k += blockDim.x) {
        float s = 0.0f;
        if (k < OFF_B1) {
            const int o = k / NF, in_ = k % NF;
            for (int rr = 0; rr < TRAIN_ROWS; ++rr) s += d1[rr][o] * __bfloat162float(xs[rr * NF + in_]);
        } else if (k < OFF_W2) {
            const int o = k - OFF_B1;
            for (int rr = 0; rr < TRAIN_ROWS; ++rr) s += d1[rr][o];
        } else if (k < OFF_B2) {
            const int o = (k - OFF_W2) / NH, in_ = (k - OFF_W2) % NH;
            for (int rr = 0; rr < TRAIN_ROWS; ++rr) s += d2[rr][o] * h1[rr][in_];
        } else if (k < OFF_W3) {
            const int o = k - OFF_B2;
            for (int rr = 0; rr < TRAIN_ROWS; ++rr) s += d2[rr][o];
        } else if (k < OFF_B3) {
            const int in_ = k - OFF_W3;
            for (int rr = 0; rr < TRAIN_ROWS; ++rr) s += dz[rr] * h2[rr][in_];
        } else {
            for (int rr = 0; rr < TRAIN_ROWS; ++rr) s += dz[rr];
        }
        if (s != 0.0f) atomicAdd(a.grad + k, s);
    }
}

// Adam step on the FP32 master parameters; refreshes the BF16 inference copy.
__global__ void adam_kernel(float* params, float* m, float* v, float* grad, int step, float lr, float b1, float b2,
                            float eps, __nv_bfloat16* w1, __nv_bfloat16* w2, __nv_bfloat16* w3, float* bias) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NPARAM) return;
    if (step > 0) {
        const float g = grad[k];
        const float mk = b1 * m[k] + (1.0f - b1) * g;
        const float vk = b2 * v[k] + (1.0f - b2) * g * g;
        m[k] = mk;
        v[k] = vk;
        const float mh = mk / (1.0f - powf(b1, float(step)));
        const float vh = vk / (1.0f - powf(b2, float(step)));
        params[k] -= lr * mh / (sqrtf(vh) + eps);
        grad[k] = 0.0f;
    }
    const float p = params[k];
    if (k < OFF_B1) w1[k] = __float2bfloat16_rn(p);
    else if (k < OFF_W2) bias[k - OFF_B1] = p;
    else if (k < OFF_B2) w2[k - OFF_W2] = __float2bfloat16_rn(p);
    else if (k < OFF_W3) bias[NH + k - OFF_B2] = p;
    else if (k < OFF_B3) w3[k - OFF_W3] = __float2bfloat16_rn(p);
    else bias[2 * NH] = p;
}


cudaError_t launch_gate(int order, const GateArgs& a, const Net& net, const Geometry& geo, cudaStream_t s,
                        const CUtensorMap* tm) {
    // the resident blocks of the current device (blocks per SM: the kernels' launch bounds)
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int ntx = (geo.ny + GATE_TILE - 1) / GATE_TILE, ntiles = ntx * ((geo.nx + GATE_TILE - 1) / GATE_TILE);
    const int grid = std::min(ntiles, sms * (order == 9 ? 2 : 3));
    if (tm) {
        if (order == 5) gate_kernel_tma<5><<<grid, GATE_THREADS, 0, s>>>(a, net, geo, ntx, ntiles, *tm);
        else if (order == 7) gate_kernel_tma<7><<<grid, GATE_THREADS, 0, s>>>(a, net, geo, ntx, ntiles, *tm);
        else gate_kernel_tma<9><<<grid, GATE_THREADS, 0, s>>>(a, net, geo, ntx, ntiles, *tm);
        return cudaGetLastError();
    }
    if (order == 5) gate_kernel<5><<<grid, GATE_THREADS, 0, s>>>(a, net, geo, ntx, ntiles);
    else if (order == 7) gate_kernel<7><<<grid, GATE_THREADS, 0, s>>>(a, net, geo, ntx, ntiles);
    else gate_kernel<9><<<grid, GATE_THREADS, 0, s>>>(a, net, geo, ntx, ntiles);
    return cudaGetLastError();
}

}  // namespace gate
}  // namespace hos

using namespace hos::gate;

namespace {

thread_local std::string g_gerr;
int gfail(int code, const std::string& m) {
    g_gerr = m;
    return code;
}
int gcuda(cudaError_t e, const char* what) { return gfail(HOS_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e)); }

void free_gate(hos_gate* g) {
    void* p[] = {g->params, g->wbf, g->bias, g->samples, g->stats, g->loss};
    for (void* q : p)
        if (q) cudaFree(q);
    if (g->stream) cudaStreamDestroy(g->stream);
}

// refresh the BF16/bias inference copy from the master parameters (Adam with step 0)
cudaError_t refresh(hos_gate* g) {
    adam_kernel<<<(NPARAM + 255) / 256, 256, 0, g->stream>>>(g->params, g->m, g->v, g->grad, 0, 0.f, 0.f, 0.f, 0.f,
                                                             g->wbf, g->wbf + NH * NF, g->wbf + NH * NF + NH * NH, g->bias);
    return cudaGetLastError();
}

unsigned long long coprime_stride(unsigned long long n, unsigned long long x) {
    if (n <= 1) return 1;
    unsigned long long s = (x % (n - 1)) + 1;
    auto gcd = [](unsigned long long a, unsigned long long b) {
        while (b) {
            unsigned long long t = a % b;
            a = b;
            b = t;
        }
        return a;
    };
    while (gcd(s, n) != 1) s = s % (n - 1) + 1;
    return s;
}

}  // namespace

extern "C" {

const char* hos_gate_last_error(void) { return g_gerr.c_str(); }

int hos_gate_create(unsigned long long sample_capacity, unsigned seed, hos_gate** out) {
    if (!out) return gfail(HOS_E_ARG, "null argument");
    hos_gate* g = new (std::nothrow) hos_gate();
    if (!g) return gfail(HOS_E_NOMEM, "host allocation");
    g->capacity = sample_capacity;
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&g->params, 4 * NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->wbf, NET_BF16 * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&g->bias, NET_F32 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->stats, sizeof(Stats));
    if (e == cudaSuccess) e = cudaMalloc(&g->loss, sizeof(double));
    if (e == cudaSuccess && sample_capacity) e = cudaMalloc(&g->samples, sample_capacity * NS * sizeof(float));
    if (e != cudaSuccess) {
        free_gate(g);
        delete g;
        return gfail(HOS_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    g->m = g->params + NPARAM;
    g->v = g->params + 2 * NPARAM;
    g->grad = g->params + 3 * NPARAM;
    // He-uniform weights from a seeded LCG, zero biases, zero Adam state
    std::vector<float> h(4 * NPARAM, 0.0f);
    unsigned long long st = 0x9e3779b97f4a7c15ull ^ seed;
    auto uni = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return float((st >> 40) & 0xffffff) / float(1 << 24);
    };
    auto fill = [&](int off, int count, int fan_in) {
        const float lim = std::sqrt(6.0f / float(fan_in));
        for (int k = 0; k < count; ++k) h[off + k] = (2.0f * uni() - 1.0f) * lim;
    };
    fill(OFF_W1, NH * NF, 14);
    fill(OFF_W2, NH * NH, NH);
    fill(OFF_W3, NH, NH);
    e = cudaMemcpy(g->params, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(g->wbf, 0, NET_BF16 * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMemset(g->stats, 0, sizeof(Stats));
    if (e == cudaSuccess) e = refresh(g);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) {
        free_gate(g);
        delete g;
        return gcuda(e, "gate init");
    }
    *out = g;
    return HOS_OK;
}

int hos_gate_destroy(hos_gate* g) {
    if (!g) return HOS_OK;
    cudaStreamSynchronize(g->stream);
    free_gate(g);
    delete g;
    return HOS_OK;
}

int hos_gate_get_params(hos_gate* g, float* params) {
    if (!g || !params) return gfail(HOS_E_ARG, "null argument");
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaMemcpy(params, g->params, NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? HOS_OK : gcuda(e, "get_params");
}

int hos_gate_set_params(hos_gate* g, const float* params) {
    if (!g || !params) return gfail(HOS_E_ARG, "null argument");
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaMemcpy(g->params, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(g->m, 0, 3 * NPARAM * sizeof(float));
    if (e == cudaSuccess) e = refresh(g);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    g->step = 0;
    return e == cudaSuccess ? HOS_OK : gcuda(e, "set_params");
}

int hos_gate_sample_count(hos_gate* g, unsigned long long* n) {
    if (!g || !n) return gfail(HOS_E_ARG, "null argument");
    Stats st;
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&st, g->stats, sizeof st, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return gcuda(e, "sample_count");
    *n = st.samples < g->capacity ? st.samples : g->capacity;
    return HOS_OK;
}

int hos_gate_get_samples(hos_gate* g, float* out, unsigned long long n) {
    if (!g || !out || n > g->capacity) return gfail(HOS_E_ARG, "bad argument");
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaMemcpy(out, g->samples, n * NS * sizeof(float), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? HOS_OK : gcuda(e, "get_samples");
}

int hos_gate_set_samples(hos_gate* g, const float* in, unsigned long long n) {
    if (!g || !in || n > g->capacity) return gfail(HOS_E_ARG, "bad argument");
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaMemcpy(g->samples, in, n * NS * sizeof(float), cudaMemcpyHostToDevice);
    Stats st{};
    st.samples = n;
    if (e == cudaSuccess) e = cudaMemcpy(g->stats, &st, sizeof st, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? HOS_OK : gcuda(e, "set_samples");
}

int hos_gate_clear_samples(hos_gate* g) {
    if (!g) return gfail(HOS_E_ARG, "null argument");
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaMemset(g->stats, 0, sizeof(Stats));
    return e == cudaSuccess ? HOS_OK : gcuda(e, "clear_samples");
}

// Gradient of the weighted mean cross-entropy over samples [first, first + n) (no update).
int hos_gate_gradient(hos_gate* g, unsigned long long first, int n, float w_pos, float w_neg, float* grad,
                      double* loss) {
    unsigned long long have = 0;
    if (int st = hos_gate_sample_count(g, &have)) return st;
    if (!grad || n <= 0 || first + (unsigned long long)n > have) return gfail(HOS_E_ARG, "bad sample range");
    cudaError_t e = cudaMemset(g->grad, 0, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(g->loss, 0, sizeof(double));
    TrainArgs a{g->samples, have, first, 1, n, w_pos, w_neg, g->grad, g->loss, nullptr};
    if (e == cudaSuccess) {
        train_grad_kernel<<<(n + TRAIN_ROWS - 1) / TRAIN_ROWS, TRAIN_ROWS * 2, 0, g->stream>>>(a, g->net(), g->params);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaMemcpy(grad, g->grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && loss) e = cudaMemcpy(loss, g->loss, sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(g->grad, 0, NPARAM * sizeof(float));
    return e == cudaSuccess ? HOS_OK : gcuda(e, "gradient");
}

// Logits of samples [first, first + n) through the inference network.
int hos_gate_forward(hos_gate* g, unsigned long long first, int n, float* logits) {
    unsigned long long have = 0;
    if (int st = hos_gate_sample_count(g, &have)) return st;
    if (!logits || n <= 0 || first + (unsigned long long)n > have) return gfail(HOS_E_ARG, "bad sample range");
    float* d = nullptr;
    cudaError_t e = cudaMalloc(&d, (size_t)n * sizeof(float));
    float* scratch = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&scratch, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(scratch, 0, NPARAM * sizeof(float));
    unsigned* status = reinterpret_cast<unsigned*>(scratch);
    if (e == cudaSuccess) {
        forward_tc_kernel<<<(n + TC_ROWS - 1) / TC_ROWS, TC_THREADS, 0, g->stream>>>(g->samples, first, n, g->net(),
                                                                                     d, status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaMemcpy(logits, d, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    unsigned st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, status, sizeof st, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (scratch) cudaFree(scratch);
    if (e != cudaSuccess) return gcuda(e, "forward");
    return st ? gfail(HOS_E_TIMEOUT, "a tensor-core MMA did not complete within its wait limit") : HOS_OK;
}

// Adam on mini-batches drawn from the collected samples (a fresh coprime-stride permutation
// per pass over the data); mean_loss receives the loss of the final mini-batch.
int hos_gate_train(hos_gate* g, int steps, int batch, float lr, float w_pos, float w_neg, unsigned seed,
                   double* mean_loss) {
    unsigned long long have = 0;
    if (int st = hos_gate_sample_count(g, &have)) return st;
    if (have < 2 || steps <= 0 || batch <= 0) return gfail(HOS_E_ARG, "no samples or bad step/batch count");
    if ((unsigned long long)batch > have) batch = (int)have;
    unsigned long long rng = 0x2545f4914f6cdd1dull ^ seed;
    auto next = [&]() {
        rng ^= rng << 13;
        rng ^= rng >> 7;
        rng ^= rng << 17;
        return rng;
    };
    unsigned long long stride = coprime_stride(have, next()), first = next() % have;
    cudaError_t e = cudaMemset(g->grad, 0, NPARAM * sizeof(float));
    for (int k = 0; k < steps && e == cudaSuccess; ++k) {
        if (first + (unsigned long long)batch > have) {   // next pass over the data
            stride = coprime_stride(have, next());
            first = 0;
        }
        const bool last = k == steps - 1;
        if (last) e = cudaMemsetAsync(g->loss, 0, sizeof(double), g->stream);
        TrainArgs a{g->samples, have, first, stride, batch, w_pos, w_neg, g->grad, last ? g->loss : nullptr, nullptr};
        train_grad_kernel<<<(batch + TRAIN_ROWS - 1) / TRAIN_ROWS, TRAIN_ROWS * 2, 0, g->stream>>>(a, g->net(), g->params);
        adam_kernel<<<(NPARAM + 255) / 256, 256, 0, g->stream>>>(g->params, g->m, g->v, g->grad, ++g->step, lr, 0.9f,
                                                                 0.999f, 1e-8f, g->wbf, g->wbf + NH * NF,
                                                                 g->wbf + NH * NF + NH * NH, g->bias);
        e = cudaGetLastError();
        first += (unsigned long long)batch;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess && mean_loss) e = cudaMemcpy(mean_loss, g->loss, sizeof(double), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? HOS_OK : gcuda(e, "train");
}

}  // extern "C"
