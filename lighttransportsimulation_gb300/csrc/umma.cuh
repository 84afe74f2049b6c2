// 5th-generation tensor core (tcgen05) helpers for sm_103a, in inline PTX: shared-memory matrix
// descriptors, the BF16 MMA with FP32 accumulation in tensor memory (TMEM), commit to an
// mbarrier, bounded mbarrier waits, TMEM allocation and loads, and the fences between them.
//
// Operand layout used everywhere here ("RC" layout): a row-major R x C bf16 matrix is stored as
// 8 x 8 core matrices; core matrix (i, j) (rows 8i..8i+7, columns 8j..8j+7) occupies 128
// contiguous bytes at ((i * C/8) + j) * 128, row r of it at +16 r.  The same buffer serves as
//   * a K-major operand when its rows are M (or N) and its columns K:
//       leading byte offset (K direction) 128, stride byte offset (M/N direction) 16 C;
//   * an MN-major operand when its rows are K and its columns M (or N):
//       stride byte offset (M/N direction) 128, leading byte offset (K direction) 16 C;
// so activations, their gradients and the weights are each stored once and read as either
// operand of the forward, input-gradient and weight-gradient products.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dev_common.cuh"

namespace lts {
namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, c) of an R x C matrix in RC layout.
__host__ __device__ __forceinline__ uint32_t rc_offset(uint32_t r, uint32_t c, uint32_t C) {
    return ((r >> 3) * (C >> 3) + (c >> 3)) * 128u + (r & 7u) * 16u + (c & 7u) * 2u;
}

// Shared-memory matrix descriptor (no swizzle): start address, leading and stride byte offsets
// (each >> 4), the fixed 0b001 field at bits 46-48, base offset 0.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D; a_mn / b_mn: MN-major operand.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D (TMEM) = A * B (+ D when acc); issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)acc));
}

// Arrives on the mbarrier once every MMA this thread issued before has completed.
__device__ __forceinline__ void umma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Poll limit of mbar_wait: kSpinLimit, unless a test shrinks it (lts_set_option
// "debug_spin_limit") to see a wait run out.
__device__ int g_mbar_spin_limit = kSpinLimit;

// Waits for phase `parity` of the mbarrier to complete, at most g_mbar_spin_limit polls; on
// timeout sets DEV_ERR_MMA_TIMEOUT and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t* err) {
    const uint32_t a = smem_u32(mbar);
    const int limit = g_mbar_spin_limit;
    for (int i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    atomicOr(err, DEV_ERR_MMA_TIMEOUT);
    return false;
}

// TMEM allocation by one whole warp; the column address lands in *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Makes this thread's generic-proxy shared-memory writes visible to the tensor cores.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32w .. 32w + 31).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

}  // namespace
}  // namespace lts
