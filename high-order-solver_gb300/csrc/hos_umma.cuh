// hos_umma.cuh -- 5th-generation tensor-core primitives (sm_100 family, here sm_103a):
// tensor-memory allocation, shared-memory matrix and instruction descriptors, tcgen05.mma of
// kind::f16 issued by one thread, its completion through tcgen05.commit on an mbarrier, and
// tcgen05.ld of the FP32 accumulators back into registers.
//
// Operand layout used here: no swizzle, K-major canonical layout -- the matrix is cut into
// core matrices of 8 rows x 16 bytes (8 BF16 along K), each stored as 128 contiguous bytes;
// core matrices adjacent along K are LBO bytes apart, those adjacent along M (or N) SBO bytes
// apart.  kmajor_offset() gives the byte offset of element (row, k) with LBO = 128 and
// SBO = K * 2 * 8 (the K core matrices of one 8-row group stored together).
#pragma once
#include <cstdint>

#include "hos_tma.cuh"

namespace hos {
namespace umma {

template <int K>
__host__ __device__ constexpr int kmajor_offset(int row, int k) {
    return (row >> 3) * (K * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}
template <int K>
__host__ __device__ constexpr uint32_t kmajor_sbo() { return K * 16; }
constexpr uint32_t KMAJOR_LBO = 128;

// shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), descriptor version 1
// (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(const void* p, uint32_t lbo, uint32_t sbo) {
    const uint32_t a = smem_u32(p);
    return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16 with FP32 accumulation, A and B BF16, both K-major:
// bits 4-5 D format (1 = F32), 7-9 A format (1 = BF16), 10-12 B format (1 = BF16),
// 15 / 16 A / B major (0 = K), 17-22 N >> 3, 24-28 M >> 4
template <int M, int N>
__host__ __device__ constexpr uint32_t idesc_bf16_f32() {
    static_assert(M == 64 || M == 128, "cta_group::1 tiles are 64 or 128 rows");
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "N: multiple of 16 in [16, 256]");
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// one warp allocates ncols (a power of two >= 32) columns of tensor memory; the address is
// written to shared memory.  The permit is released at once so other CTAs on the SM allocate.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy writes to shared memory become visible to the tensor core's (async) proxy
__device__ __forceinline__ void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, one thread issues; accumulate = 0 overwrites D
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// the mbarrier receives one arrival when every MMA this thread issued before has completed
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive 32-bit columns of this thread's tensor-memory lane (warp w reads lanes
// 32 (w % 4) .. 32 (w % 4) + 31; taddr carries that lane base in bits 16-31)
__device__ __forceinline__ void ld_32cols(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

}  // namespace umma
}  // namespace hos
