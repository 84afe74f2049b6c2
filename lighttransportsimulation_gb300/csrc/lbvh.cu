// LBVH build kernels (sm_103a).  Stages and the reference code each one restates:
//   1 k_scene_bounds   per-triangle AABB + scene AABB            BVH.cuh:92-97, Triangle.cuh:48-53,
//                                                                 Geometry.cuh:647-655
//   2 k_morton         centroid -> 30-bit Morton code + ids, and the 4x256 radix histograms
//                                                                 BVH.cuh:101-116,134-137, Bound.cuh:169-175
//   3 k_digit_prefix + 4 x k_onesweep   stable LSD radix sort of (code, id), 8-bit digits,
//                      decoupled look-back (replaces thrust::stable_sort_by_key, BVH.cuh:140-146)
//   4 k_tree           Karras topology and bottom-up AABBs in one climb
//                                                                 BVH.cuh:173-262
// Output layout: one 64-byte node per interior node carrying both child boxes (see lbvh.cuh).
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/lts_capi.h"

#include "dev_common.cuh"
#include "lbvh.cuh"

namespace lts {
namespace {

constexpr int kBlock = 256;
constexpr uint32_t kFlagAgg = 1u << 30, kFlagPrefix = 2u << 30, kCountMask = (1u << 30) - 1;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Stage a block's run of `count` triangles (9 floats each) into shared memory with 16-byte
// loads when the run start is 16-byte aligned, scalar loads otherwise.
// Poll limit of the waits on another block's flag: kSpinLimit, unless a test shrinks it
// (lts_set_option "debug_spin_limit") to see a wait run out.
__device__ int g_spin_limit = kSpinLimit;

// One poll of a bounded wait: counts it and backs off, or, past the limit, sets
// DEV_ERR_LOOKBACK_TIMEOUT and returns false so that the caller gives up.
__device__ __forceinline__ bool spin_or_give_up(int& spins, uint32_t* err) {
    if (++spins > g_spin_limit) {
        atomicOr(err, DEV_ERR_LOOKBACK_TIMEOUT);
        return false;
    }
    __nanosleep(32);
    return true;
}

// Check of the bounded wait itself: one thread waits on a flag word that nothing sets.
__global__ void k_debug_wait_flag(const uint32_t* flag, uint32_t* err) {
    int spins = 0;
    while (ld_relaxed(flag) == 0u)
        if (!spin_or_give_up(spins, err)) return;
}

__device__ __forceinline__ void stage_tris(const float* __restrict__ tri, long first, int count, float* s) {
    const long f0 = first * 9;
    const int nf = count * 9;
    const float* src = tri + f0;
    if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
        const int n4 = nf >> 2;
        const float4* s4 = reinterpret_cast<const float4*>(src);
        for (int i = threadIdx.x; i < n4; i += blockDim.x) reinterpret_cast<float4*>(s)[i] = __ldg(s4 + i);
        for (int i = (n4 << 2) + threadIdx.x; i < nf; i += blockDim.x) s[i] = __ldg(src + i);
    } else {
        for (int i = threadIdx.x; i < nf; i += blockDim.x) s[i] = __ldg(src + i);
    }
}

__device__ __forceinline__ void tri_bounds(const float* t, float mn[3], float mx[3]) {
    // Triangle::worldBound: bUnion(Bounds3f(p0, p1), p2)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mn[k] = fminf(fminf(t[k], t[3 + k]), t[6 + k]);
        mx[k] = fmaxf(fmaxf(t[k], t[3 + k]), t[6 + k]);
    }
}

// Box of triangle `prim` gathered from an array of n triangles (9 floats each).  With a 16-byte
// aligned array, the 48-byte aligned window [floor16(36 prim), +48) always holds the triangle and
// lies inside the array for prim <= n - 2, so three 16-byte loads replace nine 4-byte ones (a third
// of the L1 wavefronts of a random gather); the last triangle and unaligned arrays load floats.
__device__ __forceinline__ void gather_tri_bounds(const float* __restrict__ tri, int n, bool aligned16, int prim,
                                                  float mn[3], float mx[3]) {
    float t[9];
    if (aligned16 && prim <= n - 2) {
        const long f = 9L * prim;
        const float4* w = reinterpret_cast<const float4*>(tri + (f & ~3L));
        const float4 w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2);
        const float v[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
        const int sh = (int)(f & 3L);
#pragma unroll
        for (int k = 0; k < 9; ++k) t[k] = sh == 0 ? v[k] : sh == 1 ? v[k + 1] : sh == 2 ? v[k + 2] : v[k + 3];
    } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) t[k] = __ldg(tri + 9L * prim + k);
    }
    tri_bounds(t, mn, mx);
}

// ------------------------------------------------------------------ 1. scene bounds
__global__ __launch_bounds__(kBlock) void k_scene_bounds(const float* __restrict__ tri, int n,
                                                         uint32_t* __restrict__ gb) {
    __shared__ float s_tri[kBlock * 9];
    uint32_t kmn[3] = {~0u, ~0u, ~0u}, kmx[3] = {0u, 0u, 0u};
    for (long first = (long)blockIdx.x * kBlock; first < n; first += (long)gridDim.x * kBlock) {
        const int cnt = (int)min((long)kBlock, n - first);
        __syncthreads();
        stage_tris(tri, first, cnt, s_tri);
        __syncthreads();
        if (threadIdx.x < cnt) {
            float mn[3], mx[3];
            tri_bounds(s_tri + 9 * threadIdx.x, mn, mx);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                kmn[k] = min(kmn[k], float_key(mn[k]));
                kmx[k] = max(kmx[k], float_key(mx[k]));
            }
        }
    }
    // warp, then block reduction: one atomic per block and bound (same-address atomics serialise)
    __shared__ uint32_t s_red[kBlock / 32][6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            kmn[k] = min(kmn[k], __shfl_xor_sync(0xffffffffu, kmn[k], o));
            kmx[k] = max(kmx[k], __shfl_xor_sync(0xffffffffu, kmx[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            s_red[threadIdx.x >> 5][k] = kmn[k];
            s_red[threadIdx.x >> 5][3 + k] = kmx[k];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        uint32_t v = s_red[0][threadIdx.x];
        for (int w = 1; w < kBlock / 32; ++w)
            v = threadIdx.x < 3 ? min(v, s_red[w][threadIdx.x]) : max(v, s_red[w][threadIdx.x]);
        if (threadIdx.x < 3) atomicMin(gb + threadIdx.x, v);
        else atomicMax(gb + threadIdx.x, v);
    }
}

// ------------------------------------------------------------------ 2. Morton codes + histograms
__device__ __forceinline__ uint32_t left_shift3(uint32_t x) {
    // BVH.cuh:101-109
    if (x == (1u << 10)) --x;
    x = (x | (x << 16)) & 0b00000011000000000000000011111111u;
    x = (x | (x << 8)) & 0b00000011000000001111000000001111u;
    x = (x | (x << 4)) & 0b00000011000011000011000011000011u;
    x = (x | (x << 2)) & 0b00001001001001001001001001001001u;
    return x;
}

__global__ __launch_bounds__(kBlock) void k_morton(const float* __restrict__ tri, int n, const uint32_t* __restrict__ gb,
                                                   int code_limit, uint32_t* __restrict__ codes,
                                                   int32_t* __restrict__ ids, uint32_t* __restrict__ hist) {
    __shared__ float s_tri[kBlock * 9];
    __shared__ uint32_t s_hist[4 * 256];
    for (int i = threadIdx.x; i < 4 * 256; i += kBlock) s_hist[i] = 0;
    float gmn[3], gmx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        gmn[k] = key_float(gb[k]);
        gmx[k] = key_float(gb[3 + k]);
    }
    for (long first = (long)blockIdx.x * kBlock; first < n; first += (long)gridDim.x * kBlock) {
        const int cnt = (int)min((long)kBlock, n - first);
        __syncthreads();
        stage_tris(tri, first, cnt, s_tri);
        __syncthreads();
        if (threadIdx.x < cnt) {
            const long i = first + threadIdx.x;
            uint32_t code = 0;
            int32_t id = 0;
            if (code_limit < 0 || i < code_limit) {
                float mn[3], mx[3];
                tri_bounds(s_tri + 9 * threadIdx.x, mn, mx);
                uint32_t q[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float c = mn[k] * 0.5f + mx[k] * 0.5f;        // BVH.cuh:95
                    float o = c - gmn[k];                                // Bound.cuh:169-175
                    if (gmx[k] > gmn[k]) o = __fdiv_rn(o, gmx[k] - gmn[k]);
                    const float s = __fmul_rn((float)(1 << 10), o);     // * mortonScale (BVH.cuh:136)
                    q[k] = (uint32_t)s;                                  // float -> uint32_t truncation
                }
                code = left_shift3(q[0]) | (left_shift3(q[1]) << 1) | (left_shift3(q[2]) << 2);
                id = (int32_t)i;
            }
            codes[i] = code;
            if (ids) ids[i] = id;  // null: every id is its position, generated by the first sort pass
#pragma unroll
            for (int p = 0; p < 4; ++p) atomicAdd(&s_hist[p * 256 + ((code >> (8 * p)) & 255u)], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += kBlock)
        if (s_hist[i]) atomicAdd(hist + i, s_hist[i]);
}

// ------------------------------------------------------------------ 3. radix sort
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t wsum = 0;
    for (int w = 0; w < warp; ++w) wsum += s_warp[w];
    __syncthreads();
    return wsum + x - v;
}

__global__ void k_digit_prefix(const uint32_t* __restrict__ hist, uint32_t* __restrict__ prefix) {
    __shared__ uint32_t s_warp[8];
    const uint32_t v = hist[blockIdx.x * 256 + threadIdx.x];
    prefix[blockIdx.x * 256 + threadIdx.x] = block_excl_scan256(v, s_warp);
}

#ifndef LTS_SORT_MIN_BLOCKS
#define LTS_SORT_MIN_BLOCKS 4  // resident sort tiles per SM the register budget is cut for
#endif
#ifndef LTS_SORT_LOOKBACK
#define LTS_SORT_LOOKBACK 4  // predecessor tiles read per look-back round trip
#endif
constexpr int kLookback = LTS_SORT_LOOKBACK;
#ifndef LTS_SORT_BALLOT_MATCH
#define LTS_SORT_BALLOT_MATCH 1  // 0: __match_any_sync
#endif
// Lanes of the warp whose valid key has the same 8-bit digit d (only valid lanes: `valid`).  One
// ballot per digit bit: a lane keeps the lanes that agree with it on every bit.  MATCH.ANY is
// issued on the slow ADU pipe; the ballots are not.
__device__ __forceinline__ uint32_t digit_peers(uint32_t d, bool valid) {
#if LTS_SORT_BALLOT_MATCH
    uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const bool bit = (d >> b) & 1u;
        const uint32_t m = __ballot_sync(0xffffffffu, bit);
        peers &= bit ? m : ~m;
    }
    return valid ? peers : (1u << (threadIdx.x & 31));  // an invalid lane ranks alone (unused)
#else
    return __match_any_sync(0xffffffffu, valid ? d : 256u);
#endif
}

// vin null: every value is its key's position (the identity ids of the first pass).
__global__ __launch_bounds__(kSortThreads, LTS_SORT_MIN_BLOCKS) void k_onesweep(const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin,
                                                           uint32_t* __restrict__ kout, int32_t* __restrict__ vout,
                                                           int n, int shift, const uint32_t* __restrict__ gprefix,
                                                           uint32_t* __restrict__ status, uint32_t* __restrict__ tile_counter,
                                                           uint32_t* __restrict__ err) {
    __shared__ uint32_t s_keys[kSortTile];
    __shared__ int32_t s_vals[kSortTile];
    __shared__ uint32_t s_whist[kSortThreads / 32][256];
    __shared__ uint32_t s_tile_start[256];
    __shared__ uint32_t s_dst[256];
    __shared__ uint32_t s_warp[8];
    __shared__ int s_tile;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(tile_counter, 1u);
    for (int i = threadIdx.x; i < (kSortThreads / 32) * 256; i += kSortThreads) (&s_whist[0][0])[i] = 0;
    __syncthreads();
    const int tile = s_tile;
    const long base = (long)tile * kSortTile;
    const long wbase = base + (long)warp * 32 * kSortItems;

    uint32_t key[kSortItems];
    int32_t val[kSortItems];
    uint32_t rank[kSortItems];
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const long idx = wbase + i * 32 + lane;
        if (idx < n) {
            key[i] = __ldg(kin + idx);
            val[i] = vin ? __ldg(vin + idx) : (int32_t)idx;
        } else {
            key[i] = 0;
            val[i] = 0;
        }
    }
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const long idx = wbase + i * 32 + lane;
        const bool valid = idx < n;
        const uint32_t d = (key[i] >> shift) & 255u;
        const uint32_t peers = digit_peers(d, valid);
        const int leader = __ffs(peers) - 1;
        uint32_t b = 0;
        if (valid && lane == leader) {
            b = s_whist[warp][d];
            s_whist[warp][d] = b + __popc(peers);
        }
        b = __shfl_sync(0xffffffffu, b, leader);
        rank[i] = b + __popc(peers & lt);
    }
    __syncthreads();
    const uint32_t dig = threadIdx.x;
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) {
        const uint32_t c = s_whist[w][dig];
        s_whist[w][dig] = tot;
        tot += c;
    }
    uint32_t* st = status + (size_t)tile * 256;
    st_relaxed(st + dig, (tile == 0 ? kFlagPrefix : kFlagAgg) | tot);
    const uint32_t start = block_excl_scan256(tot, s_warp);
    s_tile_start[dig] = start;
    uint32_t excl = 0;
    if (tile > 0) {
        // look back kLookback predecessors per round trip (each status word carries its flag and
        // count together), consumed newest first until an inclusive prefix; a predecessor that
        // has published nothing yet is re-read (bounded wait)
        int k = tile - 1, spins = 0;
        while (k >= 0) {
            uint32_t v[kLookback];
#pragma unroll
            for (int j = 0; j < kLookback; ++j)
                v[j] = k - j >= 0 ? ld_relaxed(status + (size_t)(k - j) * 256 + dig) : kFlagPrefix;
            int used = kLookback;
            bool done = false;
#pragma unroll
            for (int j = 0; j < kLookback; ++j) {
                if (done || used < kLookback) continue;
                const uint32_t f = v[j] & ~kCountMask;
                if (f == 0) {
                    used = j;
                } else {
                    excl += v[j] & kCountMask;
                    done = f == kFlagPrefix;
                }
            }
            if (done) break;
            k -= used;
            if (used < kLookback && !spin_or_give_up(spins, err)) break;
        }
        st_relaxed(st + dig, kFlagPrefix | (excl + tot));
    }
    s_dst[dig] = gprefix[dig] + excl;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const long idx = wbase + i * 32 + lane;
        if (idx < n) {
            const uint32_t d = (key[i] >> shift) & 255u;
            const uint32_t pos = s_tile_start[d] + s_whist[warp][d] + rank[i];
            s_keys[pos] = key[i];
            s_vals[pos] = val[i];
        }
    }
    __syncthreads();
    const int tile_n = (int)min((long)kSortTile, n - base);
    for (int j = threadIdx.x; j < tile_n; j += kSortThreads) {
        const uint32_t k = s_keys[j];
        const uint32_t d = (k >> shift) & 255u;
        const uint32_t dst = s_dst[d] + (uint32_t)j - s_tile_start[d];
        kout[dst] = k;
        vout[dst] = s_vals[j];
    }
}

// ------------------------------------------------------------------ 4+5. tree: topology and refit
// delta (BVH.cuh:173-190): common-prefix length of the Morton codes at sorted positions a and b;
// for equal codes 40 + the common prefix of the positions; -1 when b lies outside [0, n).
__device__ __forceinline__ int delta_codes(uint32_t ca, uint32_t cb, int a, int b) {
    uint32_t x = ca ^ cb;
    int extra = 0;
    if (x == 0) {
        extra = 40;
        x = (uint32_t)(a ^ b);
    }
    return __clz((int)x) + extra;
}
__device__ __forceinline__ int delta(const uint32_t* __restrict__ c, int n, int a, int b) {
    if (b < 0 || b >= n) return -1;
    return delta_codes(__ldg(c + a), __ldg(c + b), a, b);
}

// The reference builds the tree in two passes: every interior node i finds its leaf range and
// split by binary searches over delta (BVH.cuh:192-236), then every leaf climbs to the root
// through parent links, the second child to arrive forming the union (BVH.cuh:238-262).  The
// result is the binary radix tree of the sorted codes: node [lo, hi] with split g has children
// [lo, g] and [g+1, hi]; an interior child sits at index g when it is a left child (its last
// position) and at g+1 when it is a right child (its first position); the root, [0, n-1], at 0.
// The same tree is built here in ONE bottom-up pass (the agglomerative order of Apetrei, "Fast
// and Simple Agglomerative LBVH Construction", 2014, with the indices above): node [L, R] is the
// left child of a parent split at R when delta(R, R+1) > delta(L-1, L) and the right child of a
// parent split at L-1 otherwise (the two deltas differ for distinct augmented keys), which also
// gives the node's own index (R or L).  Each thread climbs from one leaf; the two children of a
// parent meet at the parent's split g, the first to arrive stops, the second forms the union,
// writes the parent's whole 64-byte record (both child boxes, children, range) and climbs on:
//  * a block of kTreeBlock threads owns kTreeBlock consecutive leaves; when g and g+1 both lie in
//    the block the children meet in a shared-memory slot of g (box, child reference, far range
//    end; a block-scope fence and a shared arrival bitmask), without barriers;
//  * otherwise they meet in device memory, in a second kernel (k_tree_top), so that no block of
//    k_tree waits on another: k_tree lists such a child (its reference; its record is written),
//    and also a child left alone in a shared slot after the block's climbs (its sibling reaches
//    into another block).  k_tree_top climbs from every listed child: both children of a parent
//    swap the build's epoch into the arrival word of g with acq_rel order, and the second reads
//    its sibling back -- the sibling's node record, or its triangle for a leaf.  Only the
//    ~log2(n / kTreeBlock) ancestors of each block edge meet there.
constexpr int kTreeBlock = 512;
#ifndef LTS_TREE_MIN_BLOCKS
#define LTS_TREE_MIN_BLOCKS 4  // resident blocks per SM the register budget is cut for
#endif

__device__ __forceinline__ void put_node(BvhNode* __restrict__ nodes, int idx, const float* cb, int lref, int rref, int lo,
                                         int hi) {
    float4* P = reinterpret_cast<float4*>(nodes + idx);
    P[0] = make_float4(cb[0], cb[1], cb[2], cb[3]);
    P[1] = make_float4(cb[4], cb[5], cb[6], cb[7]);
    P[2] = make_float4(cb[8], cb[9], cb[10], cb[11]);
    reinterpret_cast<int4*>(P)[3] = make_int4(lref, rref, lo, hi);
}
__device__ __forceinline__ void put_root(float* __restrict__ root_bounds, const float* mn, const float* mx) {
    for (int k = 0; k < 3; ++k) {
        root_bounds[k] = mn[k];
        root_bounds[3 + k] = mx[k];
    }
}

// Children (own box / ref, sibling box / ref) of the parent in left-right order, and the union.
__device__ __forceinline__ void pair_up(bool left, float* mn, float* mx, const float* smn, const float* smx, float* cb) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        cb[k] = left ? mn[k] : smn[k];
        cb[3 + k] = left ? mx[k] : smx[k];
        cb[6 + k] = left ? smn[k] : mn[k];
        cb[9 + k] = left ? smx[k] : mx[k];
        mn[k] = fminf(cb[k], cb[6 + k]);  // bUnion(left, right)
        mx[k] = fmaxf(cb[3 + k], cb[9 + k]);
    }
}

// Arrival word of a split: the build's epoch (kEpochBits) above a leaf flag and the far range end
// of the child that arrived (its first leaf for a left child, its last for a right child), so
// that the second arrival learns its sibling's shape from the exchange itself.
constexpr int kEpochBits = 7;
constexpr uint32_t kEpochMax = (1u << kEpochBits) - 1u;
constexpr uint32_t kArrivalLeaf = 1u << 24, kArrivalEnd = kArrivalLeaf - 1u;
static_assert(32 - kEpochBits == 25, "epoch above the leaf flag and a 24-bit position");

// The climb through device memory from node [L, R] (reference ref, box mn/mx, its record already
// written), the `left` child of the parent split at g.
__device__ void climb_global(const float* __restrict__ tri, int n, int mode, const int32_t* __restrict__ ids,
                             const uint32_t* __restrict__ codes, BvhNode* __restrict__ nodes,
                             uint32_t* __restrict__ arrivals, uint32_t epoch, float* __restrict__ root_bounds, int L,
                             int R, int ref, int g, bool left, float* mn, float* mx) {
    for (;;) {
        cuda::atomic_ref<uint32_t, cuda::thread_scope_device> arrival(arrivals[g]);
        const uint32_t mine = (epoch << 25) | (L == R ? kArrivalLeaf : 0u) | (uint32_t)(left ? L : R);
        const uint32_t other = arrival.exchange(mine, cuda::memory_order_acq_rel);
        if ((other >> 25) != epoch) return;  // first arrival stops
        const int sp = left ? g + 1 : g;     // the sibling's position next to the split
        const int send = (int)(other & kArrivalEnd);
        if (left) R = send;
        else L = send;
        const bool root = (L == 0 && R == n - 1);
        // the parent's side, read alongside the sibling's box
        const bool pleft = !root && delta(codes, n, R, R + 1) > delta(codes, n, L, L - 1);
        float smn[3], smx[3];
        int sref;
        if (other & kArrivalLeaf) {
            const int prim = (mode == BVH_MODE_REFERENCE) ? sp : __ldg(ids + sp);
            float t[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) t[k] = __ldg(tri + 9L * prim + k);
            tri_bounds(t, smn, smx);
            sref = ~sp;
        } else {
            const float4 a = __ldcg(&nodes[sp].a), b = __ldcg(&nodes[sp].b), c = __ldcg(&nodes[sp].c);
            smn[0] = fminf(a.x, b.z); smn[1] = fminf(a.y, b.w); smn[2] = fminf(a.z, c.x);
            smx[0] = fmaxf(a.w, c.y); smx[1] = fmaxf(b.x, c.z); smx[2] = fmaxf(b.y, c.w);
            sref = sp;
        }
        float cb[12];
        pair_up(left, mn, mx, smn, smx, cb);
        const int lref = left ? ref : sref, rref = left ? sref : ref;
        if (root) {
            put_node(nodes, 0, cb, lref, rref, L, R);
            put_root(root_bounds, mn, mx);
            return;
        }
        left = pleft;
        ref = left ? R : L;
        put_node(nodes, ref, cb, lref, rref, L, R);
        g = left ? R : L - 1;
    }
}

__global__ __launch_bounds__(kTreeBlock, LTS_TREE_MIN_BLOCKS) void k_tree(const float* __restrict__ tri, int n, int mode,
                                                     const int32_t* __restrict__ ids, const uint32_t* __restrict__ codes,
                                                     BvhNode* __restrict__ nodes, int32_t* __restrict__ pending,
                                                     uint32_t* __restrict__ pending_count, int32_t* __restrict__ leaf_prim,
                                                     float* __restrict__ root_bounds) {
    // Slot g - b0 of a split g inside the block holds what its parent's record needs: both child
    // boxes, both child references, the parent's range [far end of the left child, far end of the
    // right child] and, once both children arrived, the parent's node index.  The climbs touch
    // only shared memory (so the block-scope fences wait on nothing in flight to device memory);
    // the records go out after the block's barrier, one 64-byte line per thread.
    //   s_slot[slot][2 side + 0] = (min.x, min.y, min.z, max.x)      side 0: left child, 1: right
    //   s_slot[slot][2 side + 1] = (max.y, max.z, reference, far end)
    //   s_slot[slot][4]          = (parent index, arrival bits: 1 left, 2 right, -, -)
    // Five 16-byte words per slot put eight consecutive slots in distinct bank groups.
    // Children that meet across blocks are listed in shared memory first and appended to the
    // device list with one atomic per block (a same-address atomic per child serialises): the
    // climbs list at most two (the one node ending at the block's last leaf whose parent lies
    // beyond, and the one starting at its first), the lone slots at most one each.
    __shared__ uint32_t s_code[kTreeBlock + 2];      // codes of positions b0-1 .. b0+kTreeBlock
    __shared__ float4 s_slot[kTreeBlock][5];
    constexpr uint32_t kPendCap = kTreeBlock + 2;
    __shared__ int32_t s_pend[kPendCap];
    __shared__ uint32_t s_npend, s_pbase;
    auto push = [&](int32_t r) {  // past the bound above (never, by the count) straight to the device list
        const uint32_t i = atomicAdd(&s_npend, 1u);
        if (i < kPendCap) s_pend[i] = r;
        else pending[atomicAdd(pending_count, 1u)] = r;
    };
    const int b0 = blockIdx.x * kTreeBlock, b1 = min(b0 + kTreeBlock, n) - 1;
    for (int k = threadIdx.x; k < kTreeBlock + 2; k += kTreeBlock) {
        const int pos = b0 - 1 + k;
        s_code[k] = (pos >= 0 && pos < n) ? __ldg(codes + pos) : 0u;
    }
    s_slot[threadIdx.x][4] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (threadIdx.x == 0) s_npend = 0u;
    __syncthreads();
    auto sdelta = [&](int a, int b) -> int {  // delta of positions within [b0-1, b1+1]
        if (b < 0 || b >= n) return -1;
        return delta_codes(s_code[a - b0 + 1], s_code[b - b0 + 1], a, b);
    };
    auto have_of = [&](int slot) -> uint32_t* { return reinterpret_cast<uint32_t*>(&s_slot[slot][4]) + 1; };

    const int l = b0 + threadIdx.x;
    int prim = 0;
    if (l <= b1) {
        prim = (mode == BVH_MODE_REFERENCE) ? l : __ldg(ids + l);
        float mn[3], mx[3];
        gather_tri_bounds(tri, n, (reinterpret_cast<uintptr_t>(tri) & 15u) == 0, prim, mn, mx);
        if (n == 1) {
            put_root(root_bounds, mn, mx);
        } else {
            int L = l, R = l, ref = ~l;
            bool left = sdelta(l, l + 1) > sdelta(l, l - 1);
            int g = left ? l : l - 1;
            // block-local climb
            for (;;) {
                if (g < b0 || g + 1 > b1) {  // the parent reaches into another block
                    push(ref);
                    break;
                }
                const int side = left ? 0 : 1, slot = g - b0;
                s_slot[slot][2 * side] = make_float4(mn[0], mn[1], mn[2], mx[0]);
                s_slot[slot][2 * side + 1] = make_float4(mx[1], mx[2], __int_as_float(ref), __int_as_float(left ? L : R));
                __threadfence_block();
                if (!(atomicOr(have_of(slot), 1u << side) & (2u >> side))) break;  // first arrival stops
                __threadfence_block();
                const float4 e0 = s_slot[slot][2 * (side ^ 1)], e1 = s_slot[slot][2 * (side ^ 1) + 1];
                const float smn[3] = {e0.x, e0.y, e0.z}, smx[3] = {e0.w, e1.x, e1.y};
#pragma unroll
                for (int k = 0; k < 3; ++k) {  // bUnion(left, right), operands in that order
                    mn[k] = left ? fminf(mn[k], smn[k]) : fminf(smn[k], mn[k]);
                    mx[k] = left ? fmaxf(mx[k], smx[k]) : fmaxf(smx[k], mx[k]);
                }
                if (left) R = __float_as_int(e1.w);
                else L = __float_as_int(e1.w);
                int* idx = reinterpret_cast<int*>(&s_slot[slot][4]);
                if (L == 0 && R == n - 1) {
                    *idx = 0;
                    put_root(root_bounds, mn, mx);
                    break;
                }
                left = sdelta(R, R + 1) > sdelta(L, L - 1);
                ref = left ? R : L;
                *idx = ref;
                g = left ? R : L - 1;
            }
        }
    }
    __syncthreads();
    if (l <= b1) leaf_prim[l] = prim;
    const int slot = threadIdx.x;
    if (b0 + slot + 1 <= b1) {
        const float4 w = s_slot[slot][4];
        const uint32_t have = __float_as_uint(w.y);
        if (have == 3u) {  // the record of the parent formed here
            const float4 a0 = s_slot[slot][0], a1 = s_slot[slot][1], c0 = s_slot[slot][2], c1 = s_slot[slot][3];
            float4* P = reinterpret_cast<float4*>(nodes + __float_as_int(w.x));
            P[0] = a0;
            P[1] = make_float4(a1.x, a1.y, c0.x, c0.y);
            P[2] = make_float4(c0.z, c0.w, c1.x, c1.y);
            reinterpret_cast<int4*>(P)[3] = make_int4(__float_as_int(a1.z), __float_as_int(c1.z), __float_as_int(a1.w),
                                                      __float_as_int(c1.w));  // (left ref, right ref, lo, hi)
        } else if (have != 0u) {  // a child alone: its sibling reaches into another block
            push(__float_as_int(s_slot[slot][have == 1u ? 1 : 3].z));
        }
    }
    __syncthreads();
    const uint32_t np = min(s_npend, kPendCap);
    if (np == 0u) return;
    if (threadIdx.x == 0) s_pbase = atomicAdd(pending_count, np);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < np; i += kTreeBlock) pending[s_pbase + i] = s_pend[i];
}

// Climbs from every child k_tree listed (at most 2n - 2 of them), grid-stride.
__global__ __launch_bounds__(kBlock) void k_tree_top(const float* __restrict__ tri, int n, int mode,
                                                     const int32_t* __restrict__ ids, const uint32_t* __restrict__ codes,
                                                     BvhNode* __restrict__ nodes, uint32_t* __restrict__ arrivals,
                                                     uint32_t epoch, const int32_t* __restrict__ pending,
                                                     const uint32_t* __restrict__ pending_count,
                                                     float* __restrict__ root_bounds) {
    const int count = (int)*pending_count;
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < count; i += gridDim.x * kBlock) {
        const int ref = pending[i];
        int L, R;
        float mn[3], mx[3];
        if (ref < 0) {  // leaf ~ref
            L = R = ~ref;
            const int prim = (mode == BVH_MODE_REFERENCE) ? L : __ldg(ids + L);
            float t[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) t[k] = __ldg(tri + 9L * prim + k);
            tri_bounds(t, mn, mx);
        } else {        // interior node: its record holds both child boxes and its range
            const float4 a = __ldcg(&nodes[ref].a), b = __ldcg(&nodes[ref].b), c = __ldcg(&nodes[ref].c);
            const int4 d = __ldcg(&nodes[ref].d);
            mn[0] = fminf(a.x, b.z); mn[1] = fminf(a.y, b.w); mn[2] = fminf(a.z, c.x);
            mx[0] = fmaxf(a.w, c.y); mx[1] = fmaxf(b.x, c.z); mx[2] = fmaxf(b.y, c.w);
            L = d.z;
            R = d.w;
        }
        const bool left = delta(codes, n, R, R + 1) > delta(codes, n, L, L - 1);
        climb_global(tri, n, mode, ids, codes, nodes, arrivals, epoch, root_bounds, L, R, ref, left ? R : L - 1, left,
                     mn, mx);
    }
}

inline int grid_for(long items, int per_block) { return (int)((items + per_block - 1) / per_block); }
#ifndef LTS_TREE_TOP_BLOCKS_PER_SM
#define LTS_TREE_TOP_BLOCKS_PER_SM 32
#endif
// k_tree_top's grid: close to one listed child per thread (the list holds at most 2n - 2;
// each climb is a chain of dependent device-memory round trips, so a thread should start its
// climbs at once rather than one after another), capped at LTS_TREE_TOP_BLOCKS_PER_SM per SM.
inline int tree_top_grid(long n, int sms) {
    return (int)std::max<long>(1, std::min<long>(grid_for(2 * n, kBlock), (long)sms * LTS_TREE_TOP_BLOCKS_PER_SM));
}

}  // namespace

#define LTS_TRY(call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
    } while (0)

Lbvh::~Lbvh() {
    void* ptrs[] = {nodes, root_bounds, leaf_prim, codes, ids, codes_alt_, hist_, status_, counters_, gbounds_, flags_};
    for (void* p : ptrs)
        if (p) dev_free(p);
    for (auto& e : ev_)
        if (e) cudaEventDestroy(e);
}

std::string Lbvh::reserve(int nn) {
    if (!ev_[0])
        for (auto& e : ev_) LTS_TRY(cudaEventCreate(&e));
    if (nn <= cap_) return "";
    void* ptrs[] = {nodes, root_bounds, leaf_prim, codes, ids, codes_alt_, hist_, status_, counters_, gbounds_, flags_};
    for (void* p : ptrs)
        if (p) dev_free(p);
    const size_t N = (size_t)nn, tiles = (N + kSortTile - 1) / kSortTile;
    bytes_ = 0;
    auto al = [&](void** p, size_t b) -> cudaError_t {
        bytes_ += b;
        return dev_alloc(p, b);
    };
    LTS_TRY(al((void**)&nodes, sizeof(BvhNode) * (N > 1 ? N - 1 : 1)));
    LTS_TRY(al((void**)&root_bounds, 6 * sizeof(float)));
    LTS_TRY(al((void**)&leaf_prim, 4 * N));
    LTS_TRY(al((void**)&codes, 4 * N));
    LTS_TRY(al((void**)&ids, 4 * N));
    // the sort's ping-pong keys and ids, one allocation: after the sort it holds the tree's list
    // of up to 2n - 2 children that meet across blocks
    LTS_TRY(al((void**)&codes_alt_, 8 * N));
    ids_alt_ = reinterpret_cast<int32_t*>(codes_alt_ + N);
    LTS_TRY(al((void**)&hist_, 4 * 2 * 4 * 256));  // histograms then prefixes
    LTS_TRY(al((void**)&status_, 4 * 4 * 256 * tiles));
    LTS_TRY(al((void**)&counters_, 4 * 8));
    LTS_TRY(al((void**)&gbounds_, 4 * 6));
    LTS_TRY(al((void**)&flags_, 4 * (N > 1 ? N - 1 : 1)));
    clear_arrivals_ = true;  // arrival words of fresh memory are zeroed before the first build
    cap_ = nn;
    return "";
}

std::string Lbvh::build(const float* d_tri, int nn, int md, int code_limit, cudaStream_t s, uint32_t* d_error) {
    if (nn < 1) return "LBVH needs at least one primitive";
    if (nn > (1 << 24)) return "LBVH is limited to 2^24 primitives (the reference's float index arithmetic)";
    std::string e = reserve(nn);
    if (!e.empty()) return e;
    n = nn;
    mode = md;
    launches = 0;
    ++serial;
    const size_t N = (size_t)nn, tiles = (N + kSortTile - 1) / kSortTile;
    int dev = 0, sms = 0;
    LTS_TRY(cudaGetDevice(&dev));
    LTS_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int stream_grid = std::min(grid_for((long)N, kBlock), sms * 8);

    LTS_TRY(cudaEventRecord(ev_[0], s));
    LTS_TRY(cudaMemsetAsync(gbounds_, 0xff, 12, s));
    LTS_TRY(cudaMemsetAsync(gbounds_ + 3, 0x00, 12, s));
    k_scene_bounds<<<stream_grid, kBlock, 0, s>>>(d_tri, nn, gbounds_);
    ++launches;
    LTS_TRY(cudaEventRecord(ev_[1], s));
    LTS_TRY(cudaMemsetAsync(hist_, 0, 4 * 4 * 256, s));
    const bool identity = code_limit < 0 || code_limit >= nn;  // every id is its position
    k_morton<<<stream_grid, kBlock, 0, s>>>(d_tri, nn, gbounds_, code_limit, codes, identity ? nullptr : ids, hist_);
    ++launches;
    LTS_TRY(cudaEventRecord(ev_[2], s));
    LTS_TRY(cudaMemsetAsync(status_, 0, 4 * 4 * 256 * tiles, s));
    LTS_TRY(cudaMemsetAsync(counters_, 0, 4 * 8, s));
    k_digit_prefix<<<4, 256, 0, s>>>(hist_, hist_ + 4 * 256);
    ++launches;
    uint32_t* kin = codes;
    int32_t* vin = ids;
    uint32_t* kout = codes_alt_;
    int32_t* vout = ids_alt_;
    for (int p = 0; p < 4; ++p) {
        k_onesweep<<<(int)tiles, kSortThreads, 0, s>>>(kin, (p == 0 && identity) ? nullptr : vin, kout, vout, nn, 8 * p,
                                                        hist_ + 4 * 256 + 256 * p, status_ + (size_t)p * 256 * tiles,
                                                        counters_ + p, d_error);
        ++launches;
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    LTS_TRY(cudaEventRecord(ev_[3], s));
    // the arrival words keep the epoch of the build that last touched them, so a new epoch per
    // build replaces clearing them; they are cleared only when fresh or when the epoch wraps
    if (++epoch_ > kEpochMax) {
        clear_arrivals_ = true;
        epoch_ = 1u;
    }
    if (clear_arrivals_) {  // every word of the allocation: a later, larger build reads past n - 1
        LTS_TRY(cudaMemsetAsync(flags_, 0, 4 * (size_t)(cap_ > 1 ? cap_ - 1 : 1), s));
        clear_arrivals_ = false;
    }
    LTS_TRY(cudaEventRecord(ev_[4], s));  // topology and refit run as one kernel, timed as the refit stage
    int32_t* pending = reinterpret_cast<int32_t*>(codes_alt_);
    k_tree<<<grid_for((long)N, kTreeBlock), kTreeBlock, 0, s>>>(d_tri, nn, md, ids, codes, nodes, pending, counters_ + 4,
                                                                leaf_prim, root_bounds);
    ++launches;
    if (nn > 1) {
        k_tree_top<<<tree_top_grid(nn, sms), kBlock, 0, s>>>(d_tri, nn, md, ids, codes, nodes, flags_, epoch_, pending,
                                                             counters_ + 4, root_bounds);
        ++launches;
    }
    LTS_TRY(cudaEventRecord(ev_[5], s));
    LTS_TRY(cudaGetLastError());
    return "";
}

std::string lbvh_set_spin_limit(int limit) {
    const int v = limit > 0 ? limit : kSpinLimit;
    LTS_TRY(cudaMemcpyToSymbol(g_spin_limit, &v, sizeof v));
    return "";
}

std::string lbvh_debug_wait_flag(uint32_t* d_err, cudaStream_t s) {
    uint32_t* flag = nullptr;
    LTS_TRY(dev_alloc((void**)&flag, 4));
    cudaError_t e = cudaMemsetAsync(flag, 0, 4, s);
    if (e == cudaSuccess) {
        k_debug_wait_flag<<<1, 1, 0, s>>>(flag, d_err);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dev_free(flag);
    return e == cudaSuccess ? std::string() : std::string("debug wait: ") + cudaGetErrorString(e);
}

void Lbvh::stage_ms(float out[5]) const {
    for (int i = 0; i < 5; ++i) {
        out[i] = 0.f;
        if (ev_[i] && ev_[i + 1]) {
            cudaEventSynchronize(ev_[i + 1]);
            cudaEventElapsedTime(&out[i], ev_[i], ev_[i + 1]);
        }
    }
}

}  // namespace lts

// ---------------------------------------------------------------------------------------------
// Allocation-free LBVH build.
//
// Some callers cannot allocate device memory at all: code running inside a host allocator or
// memory-pool callback, real-time render loops that forbid cudaMalloc/cudaFree (both can
// synchronise the whole device), and plugins whose host application owns every device
// allocation.  This variant keeps all of the build's scratch (the sort's ping-pong buffers and
// look-back table, histograms, the tree's arrival words, the scene box and an error word) in
// one file-scope device array of fixed size, so a call allocates nothing; the caller supplies the
// triangles and every output buffer.
//
// Limits and sharing: at most kNoAllocMaxPrims primitives (about 3.3 MiB of device memory that
// every GPU which loads the library keeps until process exit).  All calls share the one array and
// it keeps the previous call's contents, so everything that must start at zero is cleared at the
// start of each call, and two calls that overlap on the GPU (different streams, or different host
// threads) race on it.  The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (which may load the module), so that first call should be made before any
// stream capture begins.  The address is kept for the life of the process: after
// cudaDeviceReset on a device, its next call would use a stale address, so a program that resets
// a device does not call this entry point on it again.  Every call blocks until its work on the
// given stream has finished (it reads the kernels' error word back before returning).
// ---------------------------------------------------------------------------------------------
namespace lts {
namespace {

constexpr int kNoAllocMaxPrims = 1 << 18;
constexpr size_t kNoAllocTiles = (kNoAllocMaxPrims + kSortTile - 1) / kSortTile;
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffCodes = 0;
constexpr size_t kOffIds = kOffCodes + align256(4ull * kNoAllocMaxPrims);
constexpr size_t kOffHist = kOffIds + align256(4ull * kNoAllocMaxPrims);
static_assert(kOffIds == kOffCodes + 4ull * kNoAllocMaxPrims, "the tree's list of 2n ints spans both sort buffers");
constexpr size_t kOffStatus = kOffHist + align256(4ull * 2 * 4 * 256);
constexpr size_t kOffCounters = kOffStatus + align256(4ull * 4 * 256 * kNoAllocTiles);
constexpr size_t kOffBounds = kOffCounters + 256;
constexpr size_t kOffError = kOffBounds + 256;
constexpr size_t kOffFlags = kOffError + 256;
constexpr size_t kNoAllocBytes = kOffFlags + align256(4ull * kNoAllocMaxPrims);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

}  // namespace

int lbvh_noalloc_limit() { return kNoAllocMaxPrims; }

}  // namespace lts





namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_addr[256] = {nullptr};
}  // namespace

extern "C" int lts_bvh_build_noalloc(const float* d_tri, int32_t n, int32_t mode, int32_t code_limit,
                                     uint32_t* d_codes, int32_t* d_ids, void* d_nodes, int32_t* d_leaf_prim,
                                     float* d_root_bounds, void* stream) {
    using namespace lts;
    if (!d_tri || !d_codes || !d_ids || !d_leaf_prim || !d_root_bounds || n < 1) return LTS_ERR_ARG;
    if (n > kNoAllocMaxPrims) return LTS_ERR_ARG;
    if (n > 1 && !d_nodes) return LTS_ERR_ARG;
    if (mode != BVH_MODE_REFERENCE && mode != BVH_MODE_SORTED) return LTS_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return LTS_ERR_CUDA;
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return LTS_ERR_CUDA;
            g_noalloc_addr[dev] = p;
        }
        base = static_cast<unsigned char*>(g_noalloc_addr[dev]);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* codes_alt = reinterpret_cast<uint32_t*>(base + kOffCodes);
    int32_t* ids_alt = reinterpret_cast<int32_t*>(base + kOffIds);
    uint32_t* hist = reinterpret_cast<uint32_t*>(base + kOffHist);
    uint32_t* status = reinterpret_cast<uint32_t*>(base + kOffStatus);
    uint32_t* counters = reinterpret_cast<uint32_t*>(base + kOffCounters);
    uint32_t* gbounds = reinterpret_cast<uint32_t*>(base + kOffBounds);
    uint32_t* err = reinterpret_cast<uint32_t*>(base + kOffError);
    uint32_t* flags = reinterpret_cast<uint32_t*>(base + kOffFlags);
    BvhNode* nodes = static_cast<BvhNode*>(d_nodes);
    const size_t N = (size_t)n, tiles = (N + kSortTile - 1) / kSortTile;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return LTS_ERR_CUDA;
    const int stream_grid = std::min(grid_for((long)N, kBlock), sms * 8);
    // clear everything the kernels expect to start zeroed (or all-ones)
    if (cudaMemsetAsync(err, 0, 4, s) != cudaSuccess || cudaMemsetAsync(gbounds, 0xff, 12, s) != cudaSuccess ||
        cudaMemsetAsync(gbounds + 3, 0x00, 12, s) != cudaSuccess ||
        cudaMemsetAsync(hist, 0, 4 * 4 * 256, s) != cudaSuccess ||
        cudaMemsetAsync(status, 0, 4 * 4 * 256 * tiles, s) != cudaSuccess ||
        cudaMemsetAsync(counters, 0, 4 * 8, s) != cudaSuccess)
        return LTS_ERR_CUDA;
    k_scene_bounds<<<stream_grid, kBlock, 0, s>>>(d_tri, n, gbounds);
    const bool identity = code_limit < 0 || code_limit >= n;  // every id is its position
    k_morton<<<stream_grid, kBlock, 0, s>>>(d_tri, n, gbounds, code_limit, d_codes, identity ? nullptr : d_ids, hist);
    k_digit_prefix<<<4, 256, 0, s>>>(hist, hist + 4 * 256);
    uint32_t* kin = d_codes;
    int32_t* vin = d_ids;
    uint32_t* kout = codes_alt;
    int32_t* vout = ids_alt;
    for (int p = 0; p < 4; ++p) {
        k_onesweep<<<(int)tiles, kSortThreads, 0, s>>>(kin, (p == 0 && identity) ? nullptr : vin, kout, vout, n, 8 * p,
                                                        hist + 4 * 256 + 256 * p, status + (size_t)p * 256 * tiles,
                                                        counters + p, err);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    if (n > 1 && cudaMemsetAsync(flags, 0, 4 * (N - 1), s) != cudaSuccess) return LTS_ERR_CUDA;  // arrival words, epoch 1
    int32_t* pending = reinterpret_cast<int32_t*>(codes_alt);  // codes_alt and ids_alt: 2n ints
    k_tree<<<grid_for((long)N, kTreeBlock), kTreeBlock, 0, s>>>(d_tri, n, mode, d_ids, d_codes, nodes, pending,
                                                                counters + 4, d_leaf_prim, d_root_bounds);
    if (n > 1)
        k_tree_top<<<tree_top_grid(n, sms), kBlock, 0, s>>>(d_tri, n, mode, d_ids, d_codes, nodes, flags, 1u, pending,
                                                            counters + 4, d_root_bounds);
    if (cudaGetLastError() != cudaSuccess) return LTS_ERR_CUDA;
    uint32_t h_err = 0;
    if (cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) return LTS_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return LTS_ERR_CUDA;
    return h_err ? LTS_ERR_DEVICE : LTS_OK;
}
