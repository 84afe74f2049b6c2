// Render BVH by parallel locally-ordered clustering (PLOC: Meister and Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction", TVCG 2018).
//
// The reference renders through its Karras LBVH (acceleration/BVH.cuh:173-262), whose splits
// follow Morton-code bits, not surface area.  Any BVH over the same triangles finds the same
// closest hits, so the renderer may traverse a better one: starting from the LBVH's leaves (in
// Morton order), every cluster finds the neighbour within kPlocRadius positions whose union has
// the smallest surface area; mutual nearest neighbours merge into a new node; the survivors are
// compacted in order; repeat until one cluster is left.  The binary LBVH itself is still built
// (bit-exact, it supplies the Morton order and is what the reference's interfaces return).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "lbvh.cuh"

namespace lts {

#ifndef LTS_PLOC_RADIUS
#define LTS_PLOC_RADIUS 8  // neighbours searched on either side of a cluster (8, 16, 32, 64 measured)
#endif
constexpr int kPlocRadius = LTS_PLOC_RADIUS;
#ifndef LTS_SAH_TRI
#define LTS_SAH_TRI 0.5f  // SAH cost of a triangle test relative to a wide-node visit (0.2 .. 1.0 measured)
#endif
constexpr float kSahNode = 1.0f, kSahTri = LTS_SAH_TRI;
#ifndef LTS_WIDE_LEAF_MAX
#define LTS_WIDE_LEAF_MAX 3  // triangles one leaf slot of an 8-wide node may hold (1, 2, 3 measured)
#endif
constexpr int kWideLeafMax = LTS_WIDE_LEAF_MAX;
static_assert(kWideLeafMax >= 1 && kWideLeafMax <= 3, "a leaf slot holds one to three triangles");

class PlocBvh {
   public:
    PlocBvh() = default;
    ~PlocBvh();
    PlocBvh(const PlocBvh&) = delete;
    PlocBvh& operator=(const PlocBvh&) = delete;

    // Binary BVH over the n >= 2 leaves of leaf_v (3 float4 per leaf: the triangle of leaf l)
    // in BvhNode form (nodes[0] the root; child >= 0 an interior node, < 0 leaf ~l; d.z the
    // subtree's triangle count, d.w 1 when the subtree's smallest one-slot cost C(k, 1) is a leaf
    // slot holding all its triangles, else 0).
    // Synchronises on s once per clustering iteration.
    std::string build(const float4* leaf_v, int n, cudaStream_t s, uint32_t* d_err);

    BvhNode* nodes = nullptr;  // [n - 1]
    // [n - 1][8]: sah[8 k + i - 1] = C(k, i), the smallest SAH cost of covering node k's subtree
    // with at most i children of an 8-wide node (Ylitie, Karras and Laine, HPG 2017: node cost
    // kSahNode, triangle cost kSahTri, leaf slots of up to kWideLeafMax triangles), filled as the
    // nodes are formed
    float* sah = nullptr;
    int n = 0, iterations = 0;
    float build_ms = 0;

   private:
    void release();
    int cap_ = 0;
    float4 *lo_a_ = nullptr, *hi_a_ = nullptr, *lo_b_ = nullptr, *hi_b_ = nullptr;  // clusters (w of lo: id)
    int32_t* nn_ = nullptr;      // nearest neighbour of each cluster
    int2* excl_ = nullptr;       // per cluster: exclusive (kept, merged) counts within its block
    int2* block_sums_ = nullptr; // per block: (kept, merged), then their exclusive prefix
    int32_t* counters_ = nullptr;       // device: total kept, total merged
    int32_t* counters_host_ = nullptr;  // pinned
};

}  // namespace lts
