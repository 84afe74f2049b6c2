// Radiance-cache MLP kernels on the 5th-generation tensor cores (tcgen05, BF16 operands in shared
// memory, FP32 accumulators in tensor memory), and a product check of the operand layouts.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "dev_common.cuh"
#include "mlp.cuh"
#include "umma.cuh"

#include <cuda_bf16.h>
#include <cmath>

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


// ------------------------------------------------------------------ the radiance-cache MLP
// Shared memory (bytes).  Weights in RC layout: W0 64x96, W1..W4 64x64, W5 16x64; the input
// tile X (128 x 96), hidden activations H1..H5 (128 x 64 each),
// the output-gradient tile Gz (128 x 16) and one hidden-gradient tile Ga (128 x 64).  MN-major
// reads of a 64- or 96-column buffer with M = 128 run past its end into the next buffer; those
// product rows are never used.
__host__ __device__ constexpr uint32_t kSW(int L) { return L == 0 ? 0u : 12288u + 8192u * (uint32_t)(L - 1); }
constexpr uint32_t kSX = 47104;
constexpr uint32_t kSH = kSX + 24576;
constexpr uint32_t kSGz = kSH + 5 * 16384;
constexpr uint32_t kSGa = kSGz + 4096;
constexpr uint32_t kTrainBar = kSGa + 16384;
constexpr uint32_t kTrainSmem = kTrainBar + 64;
// Inference keeps kFwdGroups tiles in flight per CTA (one CTA per SM), one warpgroup of 128
// threads per tile, sharing the weights: each tile has one 24 KB operand buffer at
// fwd_buf(g) -- its features X (128 x 96), then each hidden layer's activations (128 x 64),
// written over the buffer once the layer's products have completed -- an mbarrier and 64 TMEM
// columns.
#ifndef LTS_MLP_FWD_GROUPS
#define LTS_MLP_FWD_GROUPS 6
#endif
constexpr int kFwdGroups = LTS_MLP_FWD_GROUPS;
constexpr uint32_t kFwdTileBytes = 24576;
__host__ __device__ constexpr uint32_t fwd_buf(int g) { return kSX + kFwdTileBytes * (uint32_t)g; }
constexpr uint32_t kFwdBar = kSX + kFwdTileBytes * kFwdGroups;  // kFwdGroups mbarriers, then the TMEM slot
constexpr uint32_t kFwdSmem = kFwdBar + 8 * kFwdGroups + 16;
constexpr uint32_t kFwdCols = 64 * kFwdGroups <= 128 ? 128 : (64 * kFwdGroups <= 256 ? 256 : 512);
static_assert(64 * kFwdGroups <= 512 && kFwdSmem <= 232448, "inference tiles exceed TMEM or shared memory");
// TMEM columns: 0..63 the working product; dW_k^T accumulators (training) at kDwCol(k)
__host__ __device__ constexpr uint32_t kDwCol(int L) { return 64u * (uint32_t)(L + 1); }

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// Row `row` of an R x C RC-layout buffer, C a multiple of 8: store / load n = C values.
__device__ __forceinline__ void rc_store_row(unsigned char* buf, int row, int C, const float* v) {
    for (int j = 0; j < C / 8; ++j) {
        const uint4 q = make_uint4(pack_bf16x2(v[8 * j], v[8 * j + 1]), pack_bf16x2(v[8 * j + 2], v[8 * j + 3]),
                                   pack_bf16x2(v[8 * j + 4], v[8 * j + 5]), pack_bf16x2(v[8 * j + 6], v[8 * j + 7]));
        *(uint4*)(buf + rc_offset(row, 8 * j, C)) = q;
    }
}
__device__ __forceinline__ void rc_load_row(const unsigned char* buf, int row, int C, float* v) {
    for (int j = 0; j < C / 8; ++j) {
        const uint4 q = *(const uint4*)(buf + rc_offset(row, 8 * j, C));
        v[8 * j] = bf16_lo(q.x); v[8 * j + 1] = bf16_hi(q.x);
        v[8 * j + 2] = bf16_lo(q.y); v[8 * j + 3] = bf16_hi(q.y);
        v[8 * j + 4] = bf16_lo(q.z); v[8 * j + 5] = bf16_hi(q.z);
        v[8 * j + 6] = bf16_lo(q.w); v[8 * j + 7] = bf16_hi(q.w);
    }
}

// Weights (global, bf16 row-major [out][in]) into their RC slots.
__device__ void load_weights(unsigned char* smem, const uint16_t* __restrict__ w16) {
    for (int L = 0; L < kMlpLayers; ++L) {
        const int R = mlp_out(L), C = mlp_in(L);
        const uint4* src = (const uint4*)(w16 + mlp_offset(L));
        for (int e = threadIdx.x; e < R * C / 8; e += blockDim.x) {
            const int r = e / (C / 8), j = e % (C / 8);
            *(uint4*)(smem + kSW(L) + rc_offset(r, 8 * j, C)) = __ldg(src + e);
        }
    }
}

// All threads: makes the shared-memory operands written so far visible to the tensor cores.
__device__ __forceinline__ void publish_smem() {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

// Issue (thread 0) D[128 x N] = A[128 x K] . W^T with A (row-major activations, K-major) at a_off
// (a_cols columns) and W [N x K] (K-major) at w_off.
__device__ __forceinline__ void issue_fwd(uint32_t tmem_d, uint32_t sbase, uint32_t a_off, int a_cols, uint32_t w_off,
                                          int N, int K) {
    const uint32_t idesc = umma_idesc_bf16(128, N, false, false);
    for (int s = 0; s < K / 16; ++s)
        umma_bf16(tmem_d, umma_desc(sbase + a_off + s * 256, 128, 16 * a_cols),
                  umma_desc(sbase + w_off + s * 256, 128, 16 * K), idesc, s > 0);
}

// 64 columns of this thread's TMEM lane starting at column c0.
__device__ __forceinline__ void tmem_row64(uint32_t tmem, int c0, float* v) {
    const uint32_t lane_base = (uint32_t)(32 * (threadIdx.x >> 5)) << 16;
#pragma unroll
    for (int q = 0; q < 4; ++q) tmem_ld16(tmem + lane_base + c0 + 16 * q, v + 16 * q);
}

// Forward pass of one 128-row training tile whose features are already in X; leaves the hidden
// activations H1..H5 in their slots (the backward pass reads them) and returns z (16 values).
__device__ bool mlp_forward_tile(unsigned char* smem, uint32_t tmem, uint64_t* mbar, uint32_t& phase, uint32_t* err,
                                 float* z) {
    const uint32_t sbase = smem_u32(smem);
    const int row = threadIdx.x;
    float v[64];
    for (int L = 0; L < kMlpLayers; ++L) {
        const uint32_t a_off = L == 0 ? kSX : kSH + (L - 1) * 16384;
        const int K = mlp_in(L), N = mlp_out(L);
        if (threadIdx.x == 0) {
            issue_fwd(tmem, sbase, a_off, K, kSW(L), N, K);
            umma_commit(mbar);
        }
        if (!__syncthreads_and(mbar_wait(mbar, phase, err))) return false;  // every thread agrees
        phase ^= 1u;
        tc_fence_after();
        if (L < kMlpLayers - 1) {
            tmem_row64(tmem, 0, v);
#pragma unroll
            for (int k = 0; k < 64; ++k) v[k] = fmaxf(v[k], 0.0f);
            rc_store_row(smem + kSH + L * 16384, row, 64, v);
            publish_smem();
        } else {
            tmem_ld16(tmem + ((uint32_t)(32 * (threadIdx.x >> 5)) << 16), z);
        }
    }
    return true;
}

__device__ __forceinline__ void load_feature_row(unsigned char* smem, const uint16_t* __restrict__ feat, long grow,
                                                 bool valid) {
    const uint4* src = (const uint4*)(feat + grow * kMlpIn);
    for (int j = 0; j < kMlpIn / 8; ++j) {
        const uint4 q = valid ? __ldg(src + j) : make_uint4(0, 0, 0, 0);
        *(uint4*)(smem + kSX + rc_offset(threadIdx.x, 8 * j, kMlpIn)) = q;
    }
}

// Named barrier over the 128 threads of warpgroup `id - 1` (barrier 0 is __syncthreads).
__device__ __forceinline__ void wg_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ bool wg_sync_and(int id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.and.pred q, %2, 128, p;\nselp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id)
        : "memory");
    return r != 0;
}
// The warpgroup's shared-memory operands written so far, visible to the tensor cores.
__device__ __forceinline__ void wg_publish(int id) {
    fence_async_smem();
    tc_fence_before();
    wg_sync(id);
    tc_fence_after();
}

// Inference: out[r * stride + c] = exp(z_c), c < 3, for the feature rows r = rows[i] (rows null:
// r = i), i < n.  Persistent CTAs of kFwdGroups warpgroups; warpgroup g runs tiles
// blockIdx.x * kFwdGroups + g, + gridDim.x * kFwdGroups, ..., one row per thread, and
// synchronises with named barrier 1 + g only, so the tiles of a CTA overlap each other's
// epilogues and waits.
__global__ __launch_bounds__(128 * kFwdGroups) void k_mlp_forward(const uint16_t* __restrict__ w16,
                                                                 const uint16_t* __restrict__ feat,
                                                                 const int32_t* __restrict__ rows, int n,
                                                                 const uint32_t* d_n, float* __restrict__ out,
                                                                 int stride, uint32_t* err) {
    if (d_n) n = min(n, (int)*d_n);  // a count produced on the device (at most n)
    extern __shared__ __align__(1024) unsigned char smem[];
    const int g = threadIdx.x >> 7, row = threadIdx.x & 127, bar_id = 1 + g;
    uint64_t* mbar = (uint64_t*)(smem + kFwdBar) + g;
    uint32_t* tslot = (uint32_t*)(smem + kFwdBar + 8 * kFwdGroups);
    load_weights(smem, w16);
    if (row == 0) mbar_init(mbar, 1);
    if ((threadIdx.x >> 5) == 0) tmem_alloc(tslot, kFwdCols);
    publish_smem();
    const uint32_t tmem = *tslot + 64u * (uint32_t)g;
    const uint32_t lane_base = (uint32_t)(32 * ((threadIdx.x >> 5) & 3)) << 16;  // warp w: lanes 32 (w % 4) ..
    const uint32_t sbase = smem_u32(smem), buf = fwd_buf(g);
    uint32_t phase = 0;
    const int ntiles = (n + 127) / 128;
    for (int tile = blockIdx.x * kFwdGroups + g; tile < ntiles; tile += gridDim.x * kFwdGroups) {
        const long i = (long)tile * 128 + row;
        const bool valid = i < n;
        const long r = valid ? (rows ? (long)__ldg(rows + i) : i) : 0;
        const uint4* src = (const uint4*)(feat + r * kMlpIn);
        for (int j = 0; j < kMlpIn / 8; ++j) {
            const uint4 q = valid ? __ldg(src + j) : make_uint4(0, 0, 0, 0);
            *(uint4*)(smem + buf + rc_offset(row, 8 * j, kMlpIn)) = q;
        }
        wg_publish(bar_id);
        bool ok = true;
        for (int L = 0; L < kMlpLayers; ++L) {
            const int K = mlp_in(L), N = mlp_out(L);
            if (row == 0) {
                issue_fwd(tmem, sbase, buf, K, kSW(L), N, K);
                umma_commit(mbar);
            }
            ok = wg_sync_and(bar_id, mbar_wait(mbar, phase, err));  // every thread of the warpgroup agrees
            phase ^= 1u;
            tc_fence_after();
            if (!ok) break;
            if (L < kMlpLayers - 1) {
                float v[64];
#pragma unroll
                for (int q = 0; q < 4; ++q) tmem_ld16(tmem + lane_base + 16 * q, v + 16 * q);
#pragma unroll
                for (int k = 0; k < 64; ++k) v[k] = fmaxf(v[k], 0.0f);
                rc_store_row(smem + buf, row, 64, v);  // the layer's products have read the buffer
                wg_publish(bar_id);
            } else {
                float z[16];
                tmem_ld16(tmem + lane_base, z);
                if (valid)
                    for (int c = 0; c < kMlpOut; ++c) out[r * stride + c] = expf(z[c]);
            }
        }
        if (!ok) break;
        tc_fence_before();
        wg_sync(bar_id);  // every row read the output before the next tile's products
        tc_fence_after();
    }
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tmem_free(*tslot, kFwdCols);
}

// Training: gradient of mean over samples and channels of (pred - t)^2 / (pred^2 + 0.01)
// (relative L2; the denominator is not differentiated) for every weight, accumulated per CTA in
// TMEM (dW_k^T = H_k^T G_k) and added to grad[] once per CTA.
__global__ __launch_bounds__(128) void k_mlp_train(const uint16_t* __restrict__ w16, const uint16_t* __restrict__ feat,
                                                   const float* __restrict__ target, int n, float* __restrict__ grad,
                                                   float* __restrict__ loss, uint32_t* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* mbar = (uint64_t*)(smem + kTrainBar);
    uint32_t* tslot = (uint32_t*)(smem + kTrainBar + 16);
    const uint32_t sbase = smem_u32(smem);
    load_weights(smem, w16);
    if (threadIdx.x == 0) mbar_init(mbar, 1);
    if ((threadIdx.x >> 5) == 0) tmem_alloc(tslot, 512);
    publish_smem();
    const uint32_t tmem = *tslot;
    const uint32_t lane_base = (uint32_t)(32 * (threadIdx.x >> 5)) << 16;
    uint32_t phase = 0;
    bool first = true, ok = true;
    float loss_acc = 0.0f;
    const float inv_count = 1.0f / (3.0f * (float)n);
    const int ntiles = (n + 127) / 128;
    const int row = threadIdx.x;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const long grow = (long)tile * 128 + row;
        const bool valid = grow < n;
        load_feature_row(smem, feat, grow, valid);
        publish_smem();
        float z[16];
        if (!(ok = mlp_forward_tile(smem, tmem, mbar, phase, err, z))) break;
        // output gradient
        float g[64];
#pragma unroll
        for (int c = 0; c < 16; ++c) g[c] = 0.0f;
        if (valid) {
            for (int c = 0; c < kMlpOut; ++c) {
                const float pred = expf(z[c]), t = target[grow * 3 + c];
                const float d = pred - t, den = pred * pred + 0.01f;
                loss_acc += d * d / den;
                g[c] = 2.0f * d / den * pred * inv_count;  // d/dz through exp
            }
        }
        rc_store_row(smem + kSGz, row, 16, g);
        publish_smem();
        // layer 5: G_h5 = Gz . W5 ; dW5^T += H5^T . Gz
        if (threadIdx.x == 0) {
            umma_bf16(tmem, umma_desc(sbase + kSGz, 128, 16 * 16), umma_desc(sbase + kSW(5), 16 * 64, 128),
                      umma_idesc_bf16(128, 64, false, true), false);
            const uint32_t h5 = kSH + 4 * 16384;
            for (int s = 0; s < 8; ++s)
                umma_bf16(tmem + kDwCol(5), umma_desc(sbase + h5 + s * 2 * 16 * 64, 16 * 64, 128),
                          umma_desc(sbase + kSGz + s * 2 * 16 * 16, 16 * 16, 128), umma_idesc_bf16(128, 16, true, true),
                          !(first && s == 0));
            umma_commit(mbar);
        }
        for (int L = 4; L >= 0; --L) {
            // D holds G_h(L+1) for the activations feeding W_(L+1); mask with H(L+1) > 0
            if (!(ok = __syncthreads_and(mbar_wait(mbar, phase, err)))) break;
            phase ^= 1u;
            tc_fence_after();
            tmem_row64(tmem, 0, g);
            float h[64];
            rc_load_row(smem + kSH + L * 16384, row, 64, h);  // H(L+1)
#pragma unroll
            for (int k = 0; k < 64; ++k) g[k] = h[k] > 0.0f ? g[k] : 0.0f;
            rc_store_row(smem + kSGa, row, 64, g);
            publish_smem();
            if (threadIdx.x == 0) {
                const uint32_t a_in = L == 0 ? kSX : kSH + (L - 1) * 16384;  // input of W_L
                const int cin = mlp_in(L);
                if (L > 0) {  // G_h(L) = Ga . W_L (W_L [64 out x 64 in] as MN-major B)
                    for (int s = 0; s < 4; ++s)
                        umma_bf16(tmem, umma_desc(sbase + kSGa + s * 256, 128, 16 * 64),
                                  umma_desc(sbase + kSW(L) + s * 2 * 16 * cin, 16 * cin, 128),
                                  umma_idesc_bf16(128, cin, false, true), s > 0);
                }
                for (int s = 0; s < 8; ++s)  // dW_L^T += A_in^T . Ga
                    umma_bf16(tmem + kDwCol(L), umma_desc(sbase + a_in + s * 2 * 16 * cin, 16 * cin, 128),
                              umma_desc(sbase + kSGa + s * 2 * 16 * 64, 16 * 64, 128),
                              umma_idesc_bf16(128, 64, true, true), !(first && s == 0));
                umma_commit(mbar);
            }
            if (L == 0) {
                if (!(ok = __syncthreads_and(mbar_wait(mbar, phase, err)))) break;
                phase ^= 1u;
                tc_fence_after();
            }
        }
        first = false;
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    // flush the accumulated weight gradients (rows = input features, columns = outputs)
    if (!first && ok) {
        for (int L = 0; L < kMlpLayers; ++L) {
            const int in = mlp_in(L), nout = L == 5 ? kMlpOut : 64;
            float v[64];
            if (L == 5)
                tmem_ld16(tmem + lane_base + kDwCol(5), v);
            else
                tmem_row64(tmem, kDwCol(L), v);
            if (row < in)
                for (int o = 0; o < nout; ++o) atomicAdd(grad + mlp_offset(L) + o * in + row, v[o]);
        }
    }
    float tot = loss_acc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(~0u, tot, o);
    if ((threadIdx.x & 31) == 0 && tot != 0.0f) atomicAdd(loss, tot / (3.0f * (float)n));
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tmem_free(tmem, 512);
}

// One Adam step, then the inference copy: an exponential moving average of the weights with
// decay `ema` (0: the weights themselves), kept in FP32 and BF16.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       uint16_t* __restrict__ w16, float* __restrict__ e32, uint16_t* __restrict__ e16, int n, float lr,
                       float b1, float b2, float c1, float c2, float eps, float ema) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    w16[i] = __bfloat16_as_ushort(__float2bfloat16_rn(wi));
    const float ei = ema > 0.0f ? ema * e32[i] + (1.0f - ema) * wi : wi;
    e32[i] = ei;
    e16[i] = __bfloat16_as_ushort(__float2bfloat16_rn(ei));
    g[i] = 0.0f;
}

__global__ void k_to_bf16(const float* __restrict__ w, uint16_t* __restrict__ w16, float* __restrict__ e32,
                          uint16_t* __restrict__ e16, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint16_t b = __bfloat16_as_ushort(__float2bfloat16_rn(w[i]));
    w16[i] = b;
    e32[i] = w[i];
    e16[i] = b;
}

// Check of the bounded mbarrier wait itself: an mbarrier expecting one arrival that never comes.
__global__ void k_debug_mbar_timeout(uint32_t* err) {
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x == 0) mbar_init(&mbar, 1);
    __syncthreads();
    (void)mbar_wait(&mbar, 0, err);
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


Mlp::~Mlp() {
    dev_free(w32_);
    dev_free(grad_);
    dev_free(m_);
    dev_free(v_);
    dev_free(w16_);
    dev_free(e32_);
    dev_free(e16_);
    dev_free(loss_);
}

std::string Mlp::init(uint32_t seed, cudaStream_t s) {
    if (!w32_) {
        TRY(dev_alloc((void**)&w32_, 4 * kMlpParams));
        TRY(dev_alloc((void**)&grad_, 4 * kMlpParams));
        TRY(dev_alloc((void**)&m_, 4 * kMlpParams));
        TRY(dev_alloc((void**)&v_, 4 * kMlpParams));
        TRY(dev_alloc((void**)&w16_, 2 * kMlpParams));
        TRY(dev_alloc((void**)&e32_, 4 * kMlpParams));
        TRY(dev_alloc((void**)&e16_, 2 * kMlpParams));
        TRY(dev_alloc((void**)&loss_, 4));
        int dev = 0, sms = 0;
        TRY(cudaGetDevice(&dev));
        TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        TRY(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem));
        TRY(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem));
        blocks_train_ = sms;
        blocks_fwd_ = sms;  // one CTA of kFwdGroups tiles per SM
    }
    // He-uniform weights, xorshift32 stream from the seed; W5 rows 3..15 zero
    std::vector<float> w(kMlpParams, 0.0f);
    uint32_t x = seed ? seed : 0x9e3779b9u;
    for (int L = 0; L < kMlpLayers; ++L) {
        const int in = mlp_in(L), out = L == 5 ? kMlpOut : mlp_out(L);
        const float a = std::sqrt(6.0f / in) * (L == 5 ? 0.1f : 1.0f);
        for (int o = 0; o < out; ++o)
            for (int i = 0; i < in; ++i) {
                x ^= x << 13;
                x ^= x >> 17;
                x ^= x << 5;
                w[mlp_offset(L) + o * in + i] = a * (2.0f * ((x >> 8) * (1.0f / 16777216.0f)) - 1.0f);
            }
    }
    steps = 0;
    return set_params(w.data(), s);
}

std::string Mlp::sync_bf16(cudaStream_t s) {
    k_to_bf16<<<(kMlpParams + 255) / 256, 256, 0, s>>>(w32_, w16_, e32_, e16_, kMlpParams);
    TRY(cudaGetLastError());
    return "";
}

std::string Mlp::set_params(const float* host, cudaStream_t s) {
    if (!w32_) return "MLP not initialised";
    TRY(cudaMemcpyAsync(w32_, host, 4 * kMlpParams, cudaMemcpyHostToDevice, s));
    TRY(cudaMemsetAsync(grad_, 0, 4 * kMlpParams, s));
    TRY(cudaMemsetAsync(m_, 0, 4 * kMlpParams, s));
    TRY(cudaMemsetAsync(v_, 0, 4 * kMlpParams, s));
    steps = 0;
    const std::string e = sync_bf16(s);
    if (!e.empty()) return e;
    TRY(cudaStreamSynchronize(s));
    return "";
}

std::string Mlp::get_params(float* host, cudaStream_t s) {
    if (!w32_) return "MLP not initialised";
    TRY(cudaMemcpyAsync(host, w32_, 4 * kMlpParams, cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    return "";
}

std::string Mlp::get_grad(float* host, cudaStream_t s) {
    if (!w32_) return "MLP not initialised";
    TRY(cudaMemcpyAsync(host, grad_, 4 * kMlpParams, cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    return "";
}

std::string Mlp::forward(const uint16_t* d_feat, int n, float* d_out, uint32_t* d_err, cudaStream_t s,
                         const int32_t* d_rows, int out_stride, const uint32_t* d_n) {
    if (!w32_) return "MLP not initialised";
    if (n <= 0) return "";
    const int tiles = (n + 127) / 128;
    const int groups = (tiles + kFwdGroups - 1) / kFwdGroups;
    k_mlp_forward<<<std::min(groups, blocks_fwd_), 128 * kFwdGroups, kFwdSmem, s>>>(e16_, d_feat, d_rows, n, d_n, d_out,
                                                                                   out_stride, d_err);
    TRY(cudaGetLastError());
    return "";
}

std::string Mlp::train_step(const uint16_t* d_feat, const float* d_target, int n, float lr, float* d_loss,
                            uint32_t* d_err, cudaStream_t s) {
    if (!w32_) return "MLP not initialised";
    if (n <= 0) return "";
    TRY(cudaMemsetAsync(grad_, 0, 4 * kMlpParams, s));
    TRY(cudaMemsetAsync(d_loss, 0, 4, s));
    const int tiles = (n + 127) / 128;
    k_mlp_train<<<std::min(tiles, blocks_train_), 128, kTrainSmem, s>>>(w16_, d_feat, d_target, n, grad_, d_loss, d_err);
    TRY(cudaGetLastError());
    return lr > 0 ? adam(lr, s) : std::string();
}

std::string Mlp::adam(float lr, cudaStream_t s) {
    if (!w32_) return "MLP not initialised";
    ++steps;
    const float b1 = 0.9f, b2 = 0.99f;
    const float c1 = 1.0f - std::pow(b1, (float)steps), c2 = 1.0f - std::pow(b2, (float)steps);
    k_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(w32_, grad_, m_, v_, w16_, e32_, e16_, kMlpParams, lr, b1, b2, c1,
                                                     c2, 1e-8f, ema);
    TRY(cudaGetLastError());
    return "";
}

std::string mlp_set_spin_limit(int limit) {
    const int v = limit > 0 ? limit : kSpinLimit;
    TRY(cudaMemcpyToSymbol(g_mbar_spin_limit, &v, sizeof v));
    return "";
}

std::string mlp_debug_mbar_timeout(uint32_t* d_err, cudaStream_t s) {
    k_debug_mbar_timeout<<<1, 32, 0, s>>>(d_err);
    TRY(cudaGetLastError());
    TRY(cudaStreamSynchronize(s));
    return "";
}

}  // namespace lts
