// PLOC render BVH (see ploc.cuh): per iteration one nearest-neighbour pass over a window of
// kPlocRadius clusters on either side (staged in shared memory), one prefix sum of the
// (kept, merged) flags, and one pass that writes the merged pairs' nodes and compacts the
// surviving clusters in order.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <utility>

#include "dev_common.cuh"
#include "ploc.cuh"

namespace lts {
namespace {

constexpr int kPlocBlock = 256;   // nearest-neighbour tile
constexpr int kScanBlock = 1024;  // prefix-sum block

inline int grid_of(long items, int per_block) { return (int)((items + per_block - 1) / per_block); }

// Clusters of the leaves: lo = (min xyz, id bits ~l), hi = (max xyz, 0).
__global__ void k_ploc_init(const float4* __restrict__ leaf_v, int n, float4* __restrict__ lo, float4* __restrict__ hi) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n) return;
    const float4 a = leaf_v[3 * (size_t)l], b = leaf_v[3 * (size_t)l + 1], c = leaf_v[3 * (size_t)l + 2];
    lo[l] = make_float4(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z),
                        __int_as_float(~l));
    hi[l] = make_float4(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z), 0.f);
}

__device__ __forceinline__ float union_half_area(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    const float dx = fmaxf(ahi.x, bhi.x) - fminf(alo.x, blo.x);
    const float dy = fmaxf(ahi.y, bhi.y) - fminf(alo.y, blo.y);
    const float dz = fmaxf(ahi.z, bhi.z) - fminf(alo.z, blo.z);
    return dx * dy + dy * dz + dz * dx;
}

// nn[i]: the cluster within kPlocRadius of i whose union with i has the smallest surface area.
// Pairs are ordered by (cost, lower index, higher index), which for one i means the smaller j
// among equal costs; the globally smallest pair is then mutual, so every iteration merges.
__global__ __launch_bounds__(kPlocBlock) void k_ploc_nn(const float4* __restrict__ lo, const float4* __restrict__ hi,
                                                        int nk, int32_t* __restrict__ nn) {
    __shared__ float4 s_lo[kPlocBlock + 2 * kPlocRadius], s_hi[kPlocBlock + 2 * kPlocRadius];
    const int base = blockIdx.x * kPlocBlock - kPlocRadius;
    for (int k = threadIdx.x; k < kPlocBlock + 2 * kPlocRadius; k += kPlocBlock) {
        const int c = base + k;
        if (c >= 0 && c < nk) {
            s_lo[k] = lo[c];
            s_hi[k] = hi[c];
        }
    }
    __syncthreads();
    const int i = blockIdx.x * kPlocBlock + threadIdx.x;
    if (i >= nk) return;
    const float4 ilo = s_lo[i - base], ihi = s_hi[i - base];
    float best = INFINITY;
    int bj = -1;
    const int j0 = max(0, i - kPlocRadius), j1 = min(nk - 1, i + kPlocRadius);
    for (int j = j0; j <= j1; ++j) {
        if (j == i) continue;
        const float c = union_half_area(ilo, ihi, s_lo[j - base], s_hi[j - base]);
        if (c < best || bj < 0) {
            best = c;
            bj = j;
        }
    }
    nn[i] = bj;
}

// Inclusive scan of int2 over a block of kScanBlock threads (s_warp: kScanBlock / 32 entries).
__device__ __forceinline__ int2 block_scan2(int2 v, int2* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(~0u, v.x, o), y = __shfl_up_sync(~0u, v.y, o);
        if (lane >= o) {
            v.x += x;
            v.y += y;
        }
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        int2 w = lane < kScanBlock / 32 ? s_warp[lane] : make_int2(0, 0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int x = __shfl_up_sync(~0u, w.x, o), y = __shfl_up_sync(~0u, w.y, o);
            if (lane >= o) {
                w.x += x;
                w.y += y;
            }
        }
        if (lane < kScanBlock / 32) s_warp[lane] = w;
    }
    __syncthreads();
    if (warp > 0) {
        const int2 p = s_warp[warp - 1];
        v.x += p.x;
        v.y += p.y;
    }
    __syncthreads();
    return v;
}

// Per cluster: kept (not the upper index of a merged pair) and merged (the lower index of a
// mutual pair); exclusive counts within the block, block totals.
__global__ __launch_bounds__(kScanBlock) void k_ploc_scan(const int32_t* __restrict__ nn, int nk, int2* __restrict__ excl,
                                                          int2* __restrict__ block_sums) {
    __shared__ int2 s_warp[kScanBlock / 32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    int2 f = make_int2(0, 0);
    if (i < nk) {
        const int j = nn[i];
        const bool mutual = nn[j] == i;
        f.x = (mutual && i > j) ? 0 : 1;
        f.y = (mutual && i < j) ? 1 : 0;
    }
    const int2 inc = block_scan2(f, s_warp);
    if (i < nk) excl[i] = make_int2(inc.x - f.x, inc.y - f.y);
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = inc;
}

// Exclusive prefix of the nb block totals, in place; totals[0..1] = all kept, all merged.
__global__ __launch_bounds__(kScanBlock) void k_ploc_block_prefix(int2* __restrict__ sums, int nb, int32_t* totals) {
    __shared__ int2 s_warp[kScanBlock / 32];
    __shared__ int2 s_carry;
    if (threadIdx.x == 0) s_carry = make_int2(0, 0);
    __syncthreads();
    for (int base = 0; base < nb; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int2 v = i < nb ? sums[i] : make_int2(0, 0);
        const int2 inc = block_scan2(v, s_warp);
        const int2 carry = s_carry;
        if (i < nb) sums[i] = make_int2(carry.x + inc.x - v.x, carry.y + inc.y - v.y);
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) s_carry = make_int2(carry.x + inc.x, carry.y + inc.y);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        totals[0] = s_carry.x;
        totals[1] = s_carry.y;
    }
}

// Merged pairs write their node (index node_base - their rank among this iteration's merges);
// kept clusters move to their rank among the kept ones.
__global__ __launch_bounds__(kScanBlock) void k_ploc_apply(const float4* __restrict__ lo, const float4* __restrict__ hi,
                                                           const int32_t* __restrict__ nn, const int2* __restrict__ excl,
                                                           const int2* __restrict__ block_pref, int nk, int node_base,
                                                           float4* __restrict__ lo_out, float4* __restrict__ hi_out,
                                                           BvhNode* __restrict__ nodes, float* __restrict__ sah,
                                                           int node_cap, uint32_t* err) {
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i >= nk) return;
    const int j = nn[i];
    const bool mutual = nn[j] == i;
    if (mutual && i > j) return;  // merged into the pair's lower index
    const int2 e = excl[i], b = block_pref[blockIdx.x];
    const int pos = e.x + b.x;
    const float4 ilo = lo[i], ihi = hi[i];
    if (!mutual) {
        lo_out[pos] = ilo;
        hi_out[pos] = ihi;
        return;
    }
    const int node = node_base - (e.y + b.y);
    if ((unsigned)node >= (unsigned)node_cap) {
        atomicOr(err, DEV_ERR_CAPACITY);
        return;
    }
    const float4 jlo = lo[j], jhi = hi[j];
    float4* P = reinterpret_cast<float4*>(nodes + node);
    P[0] = make_float4(ilo.x, ilo.y, ilo.z, ihi.x);
    P[1] = make_float4(ihi.y, ihi.z, jlo.x, jlo.y);
    P[2] = make_float4(jlo.z, jhi.x, jhi.y, jhi.z);
    const int ci = __float_as_int(ilo.w), cj = __float_as_int(jlo.w);
    const int count = (ci < 0 ? 1 : nodes[ci].d.z) + (cj < 0 ? 1 : nodes[cj].d.z);
    const float4 ulo = make_float4(fminf(ilo.x, jlo.x), fminf(ilo.y, jlo.y), fminf(ilo.z, jlo.z), __int_as_float(node));
    const float4 uhi = make_float4(fmaxf(ihi.x, jhi.x), fmaxf(ihi.y, jhi.y), fmaxf(ihi.z, jhi.z), 0.f);
    lo_out[pos] = ulo;
    hi_out[pos] = uhi;
    // SAH collapse costs of the new node from its children's (formed in earlier iterations)
    float cl[8], cr[8];
    for (int k = 0; k < 8; ++k) {
        cl[k] = ci < 0 ? kSahTri * union_half_area(ilo, ihi, ilo, ihi) : sah[8 * (size_t)ci + k];
        cr[k] = cj < 0 ? kSahTri * union_half_area(jlo, jhi, jlo, jhi) : sah[8 * (size_t)cj + k];
    }
    float dist[9];  // dist[i]: best split of i slots between the two children
    for (int i = 2; i <= 8; ++i) {
        float b = INFINITY;
        for (int k = 1; k < i; ++k) b = fminf(b, cl[k - 1] + cr[i - k - 1]);
        dist[i] = b;
    }
    // C(node, 1): its own wide node, or one leaf slot of all its triangles
    const float area = union_half_area(ulo, uhi, ulo, uhi);
    const float c_node = kSahNode * area + dist[8];
    const float c_leaf = count <= kWideLeafMax ? kSahTri * area * (float)count : INFINITY;
    const bool leaf_slot = c_leaf < c_node;
    float c = leaf_slot ? c_leaf : c_node;
    reinterpret_cast<int4*>(P)[3] = make_int4(ci, cj, count, leaf_slot ? 1 : 0);
    float* out_c = sah + 8 * (size_t)node;
    out_c[0] = c;
    for (int i = 2; i <= 8; ++i) {
        c = fminf(c, dist[i]);
        out_c[i - 1] = c;
    }
}

}  // namespace

#define TRY(call)                                                                       \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
    } while (0)

void PlocBvh::release() {
    void* ptrs[] = {nodes, sah, lo_a_, hi_a_, lo_b_, hi_b_, nn_, excl_, block_sums_, counters_};
    for (void* p : ptrs)
        if (p) dev_free(p);
    nodes = nullptr;
    sah = nullptr;
    lo_a_ = hi_a_ = lo_b_ = hi_b_ = nullptr;
    nn_ = nullptr;
    excl_ = block_sums_ = nullptr;
    counters_ = nullptr;
    cap_ = 0;
}

PlocBvh::~PlocBvh() {
    release();
    if (counters_host_) cudaFreeHost(counters_host_);
}

std::string PlocBvh::build(const float4* leaf_v, int nl, cudaStream_t s, uint32_t* d_err) {
    n = nl;
    iterations = 0;
    if (n < 2) return "PLOC needs at least two primitives";
    if (cap_ < n) {
        release();
        const size_t N = (size_t)n;
        TRY(dev_alloc((void**)&nodes, sizeof(BvhNode) * (N - 1)));
        TRY(dev_alloc((void**)&sah, 32 * (N - 1)));
        TRY(dev_alloc((void**)&lo_a_, 16 * N));
        TRY(dev_alloc((void**)&hi_a_, 16 * N));
        TRY(dev_alloc((void**)&lo_b_, 16 * N));
        TRY(dev_alloc((void**)&hi_b_, 16 * N));
        TRY(dev_alloc((void**)&nn_, 4 * N));
        TRY(dev_alloc((void**)&excl_, 8 * N));
        TRY(dev_alloc((void**)&block_sums_, 8 * (size_t)grid_of(n, kScanBlock)));
        TRY(dev_alloc((void**)&counters_, 16));
        cap_ = n;
    }
    if (!counters_host_) TRY(cudaMallocHost((void**)&counters_host_, 16));
    cudaEvent_t e0, e1;
    TRY(cudaEventCreate(&e0));
    TRY(cudaEventCreate(&e1));
    TRY(cudaEventRecord(e0, s));
    k_ploc_init<<<grid_of(n, 256), 256, 0, s>>>(leaf_v, n, lo_a_, hi_a_);
    float4 *lo = lo_a_, *hi = hi_a_, *lo2 = lo_b_, *hi2 = hi_b_;
    int nk = n, node_base = n - 2;
    while (nk > 1) {
        if (++iterations > 1 << 20) return "PLOC did not terminate";
        const int nb = grid_of(nk, kScanBlock);
        k_ploc_nn<<<grid_of(nk, kPlocBlock), kPlocBlock, 0, s>>>(lo, hi, nk, nn_);
        k_ploc_scan<<<nb, kScanBlock, 0, s>>>(nn_, nk, excl_, block_sums_);
        k_ploc_block_prefix<<<1, kScanBlock, 0, s>>>(block_sums_, nb, counters_);
        k_ploc_apply<<<nb, kScanBlock, 0, s>>>(lo, hi, nn_, excl_, block_sums_, nk, node_base, lo2, hi2, nodes, sah,
                                               n - 1, d_err);
        TRY(cudaGetLastError());
        TRY(cudaMemcpyAsync(counters_host_, counters_, 8, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        const int kept = counters_host_[0], merged = counters_host_[1];
        if (merged < 1 || kept != nk - merged) return "PLOC clustering made no progress";
        nk = kept;
        node_base -= merged;
        std::swap(lo, lo2);
        std::swap(hi, hi2);
    }
    TRY(cudaEventRecord(e1, s));
    TRY(cudaEventSynchronize(e1));
    TRY(cudaEventElapsedTime(&build_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (node_base != -1) return "PLOC node count mismatch";
    uint32_t flags = 0;
    TRY(cudaMemcpy(&flags, d_err, 4, cudaMemcpyDeviceToHost));
    if (flags & DEV_ERR_CAPACITY) return "PLOC overflowed its node capacity";
    return "";
}

}  // namespace lts
