// hos_tma.cuh -- TMA tile loads (cp.async.bulk.tensor) into shared memory, completed on an
// mbarrier, with bounded waits; and the FP32 state mirror's pitched layout that the tensor maps
// describe.
//
// The FP32 solvers keep an FP32 mirror of the FP64 state for their face and gate kernels:
// planes W0..W3, alpha_x, alpha_y of nx rows, each row ny cells padded to a pitch of
// mirror_pitch(ny) floats (a multiple of 8, so every row starts on a 32-byte boundary, as a
// tensor map's strides must be multiples of 16 bytes).  One 3D tensor map (x = j along the
// row, y = i, z = plane) covers all six planes, so one TMA instruction stages a tile's
// conserved variables and both DF indicators with its stencil halo.
#pragma once
#include <cuda.h>
#include <cstdint>

namespace hos {

constexpr int MIRROR_PLANES = 6;
__host__ __device__ __forceinline__ int mirror_pitch(int ny) { return (ny + 7) & ~7; }

// waits on an mbarrier give up after this many polls, each suspending the thread for at most
// TMA_WAIT_HINT_NS (about a second in all); a TMA load or tensor-core MMA that never completes
// then raises WAIT_TIMEOUT_BIT in the step's status word instead of hanging the kernel
constexpr unsigned TMA_WAIT_POLLS = 1u << 20;
constexpr unsigned TMA_WAIT_HINT_NS = 1000;
constexpr unsigned WAIT_TIMEOUT_BIT = 4u;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// true once the barrier's phase `parity` completed; false after TMA_WAIT_POLLS polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const uint32_t a = smem_u32(bar);
    for (unsigned k = 0; k < TMA_WAIT_POLLS; ++k) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(TMA_WAIT_HINT_NS)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 3D tiled load of the box at (x, y, z) of the tensor map into shared memory (dense, x
// fastest), completing `bytes` of transactions on the barrier.  x * element size must be a
// multiple of 16 bytes; the destination 128-byte aligned.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace hos
