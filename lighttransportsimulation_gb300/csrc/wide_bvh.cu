// Collapse of a binary BVH (the LBVH, or the PLOC tree with its SAH cost table) into the 8-wide
// compressed BVH (see wide_bvh.cuh), one kernel launch per level of the wide tree.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "dev_common.cuh"
#include "ploc.cuh"
#include "wide_bvh.cuh"

namespace lts {
namespace {

struct Child {
    float lo[3], hi[3];
    int ref;     // >= 0 interior binary node, < 0 leaf ~l
    int ntri;    // 0: an interior child (a wide node of its own); 1..3: a leaf slot of these leaves
    int leaf[3];
};

__device__ __forceinline__ void set_ref(Child& c, int ref) {
    c.ref = ref;
    c.ntri = ref < 0 ? 1 : 0;
    c.leaf[0] = ~ref;
}

__device__ __forceinline__ void split_node(const BvhNode& nd, Child& l, Child& r) {
    l.lo[0] = nd.a.x; l.lo[1] = nd.a.y; l.lo[2] = nd.a.z;
    l.hi[0] = nd.a.w; l.hi[1] = nd.b.x; l.hi[2] = nd.b.y;
    r.lo[0] = nd.b.z; r.lo[1] = nd.b.w; r.lo[2] = nd.c.x;
    r.hi[0] = nd.c.y; r.hi[1] = nd.c.z; r.hi[2] = nd.c.w;
    set_ref(l, nd.d.x);
    set_ref(r, nd.d.y);
}

// Turns interior child c (a subtree of at most kWideLeafMax triangles) into one leaf slot of all
// its leaves; false if it has more.
__device__ __forceinline__ bool gather_leaf_slot(const BvhNode* __restrict__ bn, Child& c) {
    int st[kWideLeafMax];
    int ns = 0;
    st[ns++] = c.ref;
    c.ntri = 0;
    while (ns > 0) {
        const int4 d = __ldg(&bn[st[--ns]].d);
        const int xs[2] = {d.x, d.y};
        for (int h = 0; h < 2; ++h) {
            const int x = xs[h];
            if (x < 0) {
                if (c.ntri >= kWideLeafMax) return false;
                c.leaf[c.ntri++] = ~x;
            } else {
                if (ns >= kWideLeafMax) return false;
                st[ns++] = x;
            }
        }
    }
    return true;
}

__device__ __forceinline__ float half_area(const Child& c) {
    const float dx = c.hi[0] - c.lo[0], dy = c.hi[1] - c.lo[1], dz = c.hi[2] - c.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// Smallest exponent e (scale 2^e) with 255 * 2^e >= ext, at least -126 (normal scales only).
__device__ int axis_exponent(float ext) {
    if (!(ext > 0.0f)) return -126;
    int e2;
    frexpf(ext, &e2);  // ext <= 2^e2
    int e = e2 - 8;
    if (__fmul_rn(255.0f, ldexpf(1.0f, e)) < ext) ++e;
    return max(e, -126);
}

// SAH collapse costs of a child: its row of the cost table (interior), or kSahTri x its half
// area for every slot count (a leaf: one triangle).
__device__ __forceinline__ void child_costs(const Child& c, const float* __restrict__ sah, float out[8]) {
    if (c.ref < 0) {
        const float v = kSahTri * half_area(c);
        for (int k = 0; k < 8; ++k) out[k] = v;
    } else {
        const float4 a = __ldg(reinterpret_cast<const float4*>(sah + 8 * (size_t)c.ref));
        const float4 b = __ldg(reinterpret_cast<const float4*>(sah + 8 * (size_t)c.ref) + 1);
        out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w;
        out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
    }
}

// Slots given to the left child when i >= 2 slots are split between l and r: the k in 1..i-1
// with the smallest C(l, k) + C(r, i - k) (the smallest k among equal costs).
__device__ __forceinline__ int best_split(const Child& l, const Child& r, int i, const float* __restrict__ sah) {
    float cl[8], cr[8];
    child_costs(l, sah, cl);
    child_costs(r, sah, cr);
    int bk = 1;
    float bc = INFINITY;
    for (int k = 1; k < i; ++k) {
        const float c = cl[k - 1] + cr[i - k - 1];
        if (c < bc) {
            bc = c;
            bk = k;
        }
    }
    return bk;
}

// One item: interior binary node it.x becomes wide node it.y.
//   kSah false: children are gathered by repeatedly opening the interior child of largest
//     surface area until there are eight or only leaves remain.
//   kSah true: the SAH-optimal choice of the cost table (Ylitie, Karras and Laine, HPG 2017):
//     the node's two binary children share its eight slots at the best split; a subtree given
//     i slots takes the fewest slots i' <= i of equal cost C(n, i') = C(n, i), and with i' = 1
//     becomes one interior child (a wide node of its own), else splits i' between its children
//     the same way.  Every subtree is given at least one slot and the shares sum to at most
//     eight, so at most eight children result (and the pending list never holds more than eight).
//     A one-slot subtree whose cheapest form is a leaf slot (BvhNode d.w) becomes one leaf slot
//     of its up to kWideLeafMax triangles.
// Slots are assigned greedily so that slot s (bit 0: +x, bit 1: +y, bit 2: +z) holds the child
// whose centroid lies furthest towards that octant of the node.
template <bool kSah>
__global__ __launch_bounds__(128) void k_collapse(const BvhNode* __restrict__ bn, const float* __restrict__ sah,
                                                  const float4* __restrict__ leaf_v, const int2* __restrict__ in,
                                                  int nin, int2* __restrict__ out, uint32_t* counters,
                                                  WideNode* __restrict__ wn, float4* __restrict__ wtri, int cap_nodes,
                                                  int cap_tris, uint32_t* err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nin) return;
    const int2 it = in[t];
    Child ch[8];
    int cnt = 0;
    if constexpr (kSah) {
        Child pend[8];
        int budget[8];
        int np = 0;
        Child l, r;
        split_node(bn[it.x], l, r);
        int k = best_split(l, r, 8, sah);
        pend[0] = r;
        budget[0] = 8 - k;
        pend[1] = l;
        budget[1] = k;
        np = 2;
        while (np > 0) {
            --np;
            const Child c = pend[np];
            int i = budget[np];
            if (c.ref >= 0 && i > 1) {
                float cc[8];
                child_costs(c, sah, cc);
                while (i > 1 && cc[i - 2] == cc[i - 1]) --i;
            }
            if (c.ref < 0 || i == 1) {
                if (cnt >= 8) {  // unreachable: the shares never exceed eight slots
                    atomicOr(err, DEV_ERR_CAPACITY);
                    return;
                }
                ch[cnt] = c;
                if (c.ref >= 0 && __ldg(&bn[c.ref].d.w) && !gather_leaf_slot(bn, ch[cnt])) {
                    atomicOr(err, DEV_ERR_CAPACITY);  // unreachable: d.w is set for small subtrees only
                    return;
                }
                ++cnt;
                continue;
            }
            if (np + 2 > 8) {  // unreachable: every pending share is at least one slot
                atomicOr(err, DEV_ERR_CAPACITY);
                return;
            }
            split_node(bn[c.ref], l, r);
            k = best_split(l, r, i, sah);
            pend[np] = r;
            budget[np] = i - k;
            pend[np + 1] = l;
            budget[np + 1] = k;
            np += 2;
        }
    } else {
        cnt = 2;
        split_node(bn[it.x], ch[0], ch[1]);
        while (cnt < 8) {
            int best = -1;
            float ba = -1.0f;
            for (int k = 0; k < cnt; ++k)
                if (ch[k].ref >= 0) {
                    const float a = half_area(ch[k]);
                    if (a > ba) {
                        ba = a;
                        best = k;
                    }
                }
            if (best < 0) break;
            const BvhNode nd = bn[ch[best].ref];
            split_node(nd, ch[best], ch[cnt]);
            ++cnt;
        }
    }
    float nlo[3], nhi[3];
    for (int a = 0; a < 3; ++a) {
        nlo[a] = ch[0].lo[a];
        nhi[a] = ch[0].hi[a];
        for (int k = 1; k < cnt; ++k) {
            nlo[a] = fminf(nlo[a], ch[k].lo[a]);
            nhi[a] = fmaxf(nhi[a], ch[k].hi[a]);
        }
    }
    // octant slots
    int slot_child[8];
    for (int s = 0; s < 8; ++s) slot_child[s] = -1;
    uint32_t used = 0, placed = 0;
    for (int round = 0; round < cnt; ++round) {
        float bc = INFINITY;
        int bk = -1, bs = -1;
        for (int k = 0; k < cnt; ++k) {
            if ((placed >> k) & 1u) continue;
            float d[3];
            for (int a = 0; a < 3; ++a) d[a] = (ch[k].lo[a] + ch[k].hi[a]) - (nlo[a] + nhi[a]);
            for (int s = 0; s < 8; ++s) {
                if ((used >> s) & 1u) continue;
                const float c = -((s & 1 ? d[0] : -d[0]) + (s & 2 ? d[1] : -d[1]) + (s & 4 ? d[2] : -d[2]));
                if (c < bc) {
                    bc = c;
                    bk = k;
                    bs = s;
                }
            }
        }
        slot_child[bs] = bk;
        used |= 1u << bs;
        placed |= 1u << bk;
    }
    uint32_t imask = 0, omask = 0, layout = 0;
    int ni = 0, nl = 0;
    for (int s = 0; s < 8; ++s) {
        const int k = slot_child[s];
        if (k < 0) continue;
        omask |= 1u << s;
        if (ch[k].ntri == 0) {
            imask |= 1u << s;
            ++ni;
        } else {
            layout |= ((1u << ch[k].ntri) - 1u) << (3 * s);
            nl += ch[k].ntri;
        }
    }
    const uint32_t child_base = ni ? atomicAdd(counters + 0, (uint32_t)ni) : 0u;
    const uint32_t tri_base = nl ? atomicAdd(counters + 1, (uint32_t)nl) : 0u;
    if (child_base + ni > (uint32_t)cap_nodes || tri_base + nl > (uint32_t)cap_tris) {
        atomicOr(err, DEV_ERR_CAPACITY);
        return;
    }
    // quantisation per axis; qlo rounds down, qhi up, each checked against the decoded plane
    uint32_t ebyte[3];
    unsigned long long qlo[3] = {0, 0, 0}, qhi[3] = {0, 0, 0};
    for (int a = 0; a < 3; ++a) {
        const float p = nlo[a];
        int e = axis_exponent(__fsub_ru(nhi[a], p));
        bool ok = false;
        for (int attempt = 0; attempt < 4 && !ok; ++attempt, ++e) {
            const float scale = ldexpf(1.0f, e);
            ok = true;
            qlo[a] = qhi[a] = 0;
            for (int s = 0; s < 8 && ok; ++s) {
                const int k = slot_child[s];
                if (k < 0) continue;
                const float lo = ch[k].lo[a], hi = ch[k].hi[a];
                const float fl = fminf(floorf(__fdiv_rd(__fsub_rd(lo, p), scale)), 255.0f);
                uint32_t ql = fl > 0.0f ? (uint32_t)fl : 0u;
                while (ql > 0 && wide_plane(p, ql, scale) > lo) --ql;
                const float fh = ceilf(__fdiv_ru(__fsub_ru(hi, p), scale));
                if (!(fh <= 255.0f)) {
                    ok = false;
                    break;
                }
                uint32_t qh = fh > 0.0f ? (uint32_t)fh : 0u;
                while (wide_plane(p, qh, scale) < hi) {
                    if (++qh > 255u) {
                        ok = false;
                        break;
                    }
                }
                if (!ok) break;
                qlo[a] |= (unsigned long long)ql << (8 * s);
                qhi[a] |= (unsigned long long)qh << (8 * s);
            }
            if (ok) ebyte[a] = (uint32_t)(e + 127);
        }
        if (!ok) {
            atomicOr(err, DEV_ERR_CAPACITY);
            return;
        }
    }
    WideNode w;
    w.h = make_float4(nlo[0], nlo[1], nlo[2], __uint_as_float(ebyte[0] | ebyte[1] << 8 | ebyte[2] << 16 | imask << 24));
    w.m = make_uint4(child_base, tri_base, omask, layout);
    w.q0 = make_uint4((uint32_t)qlo[0], (uint32_t)(qlo[0] >> 32), (uint32_t)qlo[1], (uint32_t)(qlo[1] >> 32));
    w.q1 = make_uint4((uint32_t)qlo[2], (uint32_t)(qlo[2] >> 32), (uint32_t)qhi[0], (uint32_t)(qhi[0] >> 32));
    w.q2 = make_uint4((uint32_t)qhi[1], (uint32_t)(qhi[1] >> 32), (uint32_t)qhi[2], (uint32_t)(qhi[2] >> 32));
    wn[it.y] = w;
    int ri = 0, rl = 0;
    for (int s = 0; s < 8; ++s) {
        const int k = slot_child[s];
        if (k < 0) continue;
        if (ch[k].ntri == 0) {
            const uint32_t pos = atomicAdd(counters + 2, 1u);
            out[pos] = make_int2(ch[k].ref, (int)child_base + ri);
            ++ri;
        } else {
            for (int j = 0; j < ch[k].ntri; ++j) {
                const int l = ch[k].leaf[j];
                float4* dst = wtri + 3 * ((size_t)tri_base + rl);
                dst[0] = __ldg(leaf_v + 3 * (size_t)l);
                dst[1] = __ldg(leaf_v + 3 * (size_t)l + 1);
                dst[2] = __ldg(leaf_v + 3 * (size_t)l + 2);
                ++rl;
            }
        }
    }
}

}  // namespace

#define TRY(call)                                                                       \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
    } while (0)

void WideBvh::release() {
    dev_free(nodes);
    dev_free(tris);
    dev_free(items_a_);
    dev_free(items_b_);
    dev_free(counters_);
    nodes = nullptr;
    tris = nullptr;
    items_a_ = items_b_ = nullptr;
    counters_ = nullptr;
    cap_ = 0;
}

WideBvh::~WideBvh() {
    release();
    if (counters_host_) cudaFreeHost(counters_host_);
}

std::string WideBvh::build(const Lbvh& bvh, const float4* leaf_v, cudaStream_t s, uint32_t* d_err) {
    return build(bvh.nodes, nullptr, bvh.n, bvh.serial, leaf_v, s, d_err);
}

std::string WideBvh::build(const BvhNode* bnodes, const float* sah, int nleaves, uint64_t key, const float4* leaf_v,
                           cudaStream_t s, uint32_t* d_err) {
    n = nleaves;
    count = levels = 0;
    serial = 0;
    if (n < 2) return "wide BVH needs at least two primitives";
    if (cap_ < n) {
        release();
        TRY(dev_alloc((void**)&nodes, sizeof(WideNode) * (size_t)(n - 1)));
        TRY(dev_alloc((void**)&tris, 3 * sizeof(float4) * (size_t)n));
        TRY(dev_alloc((void**)&items_a_, sizeof(int2) * (size_t)n));
        TRY(dev_alloc((void**)&items_b_, sizeof(int2) * (size_t)n));
        TRY(dev_alloc((void**)&counters_, 64));
        cap_ = n;
    }
    if (!counters_host_) TRY(cudaMallocHost((void**)&counters_host_, 64));
    cudaEvent_t e0, e1;
    TRY(cudaEventCreate(&e0));
    TRY(cudaEventCreate(&e1));
    // counters: [0] wide nodes allocated (the root), [1] triangles placed, [2] next-level items;
    // words 4, 5: the root item (binary node 0 -> wide node 0)
    counters_host_[0] = 1;
    counters_host_[1] = counters_host_[2] = counters_host_[3] = 0;
    counters_host_[4] = counters_host_[5] = 0;
    TRY(cudaEventRecord(e0, s));
    // zeroed nodes have no occupied slot: a node the collapse could not write is empty, never garbage
    TRY(cudaMemsetAsync(nodes, 0, sizeof(WideNode) * (size_t)(n - 1), s));
    TRY(cudaMemcpyAsync(counters_, counters_host_, 16, cudaMemcpyHostToDevice, s));
    TRY(cudaMemcpyAsync(items_a_, counters_host_ + 4, 8, cudaMemcpyHostToDevice, s));
    TRY(cudaStreamSynchronize(s));
    int2 *in = items_a_, *out = items_b_;
    int nin = 1;
    while (nin > 0) {
        TRY(cudaMemsetAsync(counters_ + 2, 0, 4, s));
        if (sah)
            k_collapse<true><<<(nin + 127) / 128, 128, 0, s>>>(bnodes, sah, leaf_v, in, nin, out, counters_, nodes,
                                                               tris, n - 1, n, d_err);
        else
            k_collapse<false><<<(nin + 127) / 128, 128, 0, s>>>(bnodes, sah, leaf_v, in, nin, out, counters_, nodes,
                                                                tris, n - 1, n, d_err);
        TRY(cudaGetLastError());
        TRY(cudaMemcpyAsync(counters_host_, counters_, 16, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        nin = (int)counters_host_[2];
        std::swap(in, out);
        ++levels;
        if (levels > 4096) return "wide BVH collapse did not terminate";
    }
    TRY(cudaEventRecord(e1, s));
    TRY(cudaEventSynchronize(e1));
    TRY(cudaEventElapsedTime(&build_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    count = (int)counters_host_[0];
    uint32_t flags = 0;
    TRY(cudaMemcpy(&flags, d_err, 4, cudaMemcpyDeviceToHost));
    if (flags & DEV_ERR_CAPACITY) return "wide BVH collapse overflowed its node or triangle capacity";
    if ((int)counters_host_[1] != n) return "wide BVH collapse lost triangles";
    serial = key;
    return "";
}

}  // namespace lts
