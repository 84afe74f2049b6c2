// Radiance-cache MLP kernels on the 5th-generation tensor cores (tcgen05, BF16 operands in shared
// memory, FP32 accumulators in tensor memory), and a product check of the operand layouts.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dev_common.cuh"
#include "mlp.cuh"
#include "umma.cuh"

namespace lts {
namespace {

constexpr int kProbeSmem = 96 * 1024;

__global__ __launch_bounds__(128) void k_umma_probe(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                    float* __restrict__ D, int mode, int swap, uint32_t* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;
    unsigned char* sB = smem + 32 * 1024;
    uint64_t* mbar = (uint64_t*)(smem + 64 * 1024);
    uint32_t* tslot = (uint32_t*)(smem + 64 * 1024 + 64);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // operand shapes (rows x columns of the stored RC matrices) and the product's M, N, K
    const int ar = 128, ac = mode == 2 ? 96 : 64;
    const int br = mode == 2 ? 128 : 64, bc = mode == 0 ? 64 : (mode == 1 ? 96 : 64);
    const int N = mode == 1 ? 96 : 64, K = mode == 2 ? 128 : 64;
    for (int e = tid; e < ar * ac; e += 128) {
        const int r = e / ac, c = e % ac;
        *(uint16_t*)(sA + rc_offset(r, c, ac)) = A[e];
    }
    for (int e = tid; e < br * bc; e += 128) {
        const int r = e / bc, c = e % bc;
        *(uint16_t*)(sB + rc_offset(r, c, bc)) = B[e];
    }
    if (tid == 0) mbar_init(mbar, 1);
    if (warp == 0) tmem_alloc(tslot, 128);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    if (tid == 0) {
        const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
        const uint32_t idesc = umma_idesc_bf16(128, N, mode == 2, mode != 0);
        for (int s = 0; s < K / 16; ++s) {
            uint64_t da, db;
            if (mode == 2) {  // MN-major A: K rows of 16 ac bytes
                const uint32_t lbo = swap ? 128u : 16u * ac, sbo = swap ? 16u * ac : 128u;
                da = umma_desc(a0 + s * 2 * 16 * ac, lbo, sbo);
            } else {
                da = umma_desc(a0 + s * 256, 128, 16 * ac);
            }
            if (mode == 0) {
                db = umma_desc(b0 + s * 256, 128, 16 * bc);
            } else {
                const uint32_t lbo = swap ? 128u : 16u * bc, sbo = swap ? 16u * bc : 128u;
                db = umma_desc(b0 + s * 2 * 16 * bc, lbo, sbo);
            }
            umma_bf16(tmem, da, db, idesc, s > 0);
        }
        umma_commit(mbar);
    }
    const bool ok = mbar_wait(mbar, 0, err);
    tc_fence_after();
    if (ok) {
        const int row = 32 * warp + lane;
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + c0, v);
            for (int k = 0; k < 16; ++k) D[row * N + c0 + k] = v[k];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tmem, 128);
}

}  // namespace

#define TRY(call)                                                                       \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
    } while (0)

std::string umma_probe(int mode, int swap, const uint16_t* a, const uint16_t* b, float* d, uint32_t* d_err,
                       cudaStream_t s) {
    if (mode < 0 || mode > 2) return "umma_probe: mode must be 0, 1 or 2";
    const size_t na = 128 * (mode == 2 ? 96 : 64), nb = mode == 2 ? 128 * 64 : 64 * (mode == 1 ? 96 : 64);
    const size_t nd = 128 * (mode == 1 ? 96 : 64);
    void *da = nullptr, *db = nullptr, *dd = nullptr;
    std::string e;
    auto fail = [&](const std::string& m) {
        dev_free(da);
        dev_free(db);
        dev_free(dd);
        return m;
    };
    if (dev_alloc(&da, 2 * na) != cudaSuccess || dev_alloc(&db, 2 * nb) != cudaSuccess ||
        dev_alloc(&dd, 4 * nd) != cudaSuccess)
        return fail("umma_probe: allocation failed");
    cudaError_t c = cudaMemcpyAsync(da, a, 2 * na, cudaMemcpyHostToDevice, s);
    if (c == cudaSuccess) c = cudaMemcpyAsync(db, b, 2 * nb, cudaMemcpyHostToDevice, s);
    if (c == cudaSuccess) c = cudaFuncSetAttribute(k_umma_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, kProbeSmem);
    if (c != cudaSuccess) return fail(std::string("umma_probe: ") + cudaGetErrorString(c));
    k_umma_probe<<<1, 128, kProbeSmem, s>>>((const uint16_t*)da, (const uint16_t*)db, (float*)dd, mode, swap, d_err);
    c = cudaGetLastError();
    if (c == cudaSuccess) c = cudaMemcpyAsync(d, dd, 4 * nd, cudaMemcpyDeviceToHost, s);
    if (c == cudaSuccess) c = cudaStreamSynchronize(s);
    if (c != cudaSuccess) return fail(std::string("umma_probe: ") + cudaGetErrorString(c));
    return fail("");
}

}  // namespace lts
