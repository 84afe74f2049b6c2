// 8-wide compressed BVH for traversal (sm_103a), collapsed from a binary BVH over the LBVH's
// leaves.
//
// The reference traverses its binary LBVH (acceleration/BVH.cuh:331-398).  The binary tree is
// still built exactly as the reference builds it (lbvh.cu); for rendering, it or a PLOC tree
// clustered from its Morton order (ploc.cu) is collapsed into nodes of up to eight children --
// interior nodes, or leaf slots of one to three triangles -- with child boxes quantised to 8 bits
// per plane relative to the node's origin and a power-of-two scale per axis (the compressed wide
// BVH of Ylitie, Karras and Laine, HPG 2017, in a layout of our own).  Decoded boxes always
// contain the exact child boxes, and every triangle sits in exactly one leaf slot, so traversal
// finds the same closest hit as the binary traversal.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "lbvh.cuh"

namespace lts {

// 80 bytes = five 16-byte loads.
//   h.xyz  origin p (the node box's minimum corner)
//   h.w    bits: e_x | e_y << 8 | e_z << 16 | imask << 24, e = biased exponent of the axis scale
//          2^(e-127); imask bit s set: slot s is an interior child
//   m.x    index of the first interior child (interior children are stored in slot order)
//   m.y    index of the first leaf triangle (the leaf children's triangles, in slot order)
//   m.z    omask: bit s set: slot s is occupied
//   m.w    leaf layout: bits 3s .. 3s+2 hold 1, 3 or 7 for a leaf slot s of 1, 2 or 3 triangles
//          (0 for interior and empty slots), so triangle m.y + k is the k-th set bit of m.w
//   q0     qlo_x[8] (x, y words), qlo_y[8] (z, w words); q1 = qlo_z[8], qhi_x[8];
//   q2     qhi_y[8], qhi_z[8]; byte s of each 8-byte group belongs to slot s
struct alignas(16) WideNode {
    float4 h;
    uint4 m;
    uint4 q0, q1, q2;
};
static_assert(sizeof(WideNode) == 80, "wide node is five 16-byte words");

// Decoded plane: p + q * scale, rounded once per operation, identically in build and traversal.
__device__ __forceinline__ float wide_plane(float p, uint32_t q, float scale) {
    return __fadd_rn(p, __fmul_rn(__uint2float_rn(q), scale));
}
__device__ __forceinline__ float wide_scale(uint32_t ebyte) { return __int_as_float((int)(ebyte << 23)); }

class WideBvh {
   public:
    WideBvh() = default;
    ~WideBvh();
    WideBvh(const WideBvh&) = delete;
    WideBvh& operator=(const WideBvh&) = delete;

    // Collapses `bvh` (n >= 2 leaves) whose leaf l holds triangle leaf_v[3l .. 3l+2] (w of the
    // first vertex = primitive id).  Synchronises on s once per tree level.
    std::string build(const Lbvh& bvh, const float4* leaf_v, cudaStream_t s, uint32_t* d_err);
    // The same from any binary BVH over the n leaves of leaf_v (BvhNode form, root 0), cached
    // under `key`; with `sah` (the tree's collapse cost table, PlocBvh::sah) the children of each
    // wide node are the SAH-optimal choice, without it the greedy largest-area opening.
    std::string build(const BvhNode* bnodes, const float* sah, int nleaves, uint64_t key, const float4* leaf_v,
                      cudaStream_t s, uint32_t* d_err);

    WideNode* nodes = nullptr;  // [count]; the root is node 0
    float4* tris = nullptr;     // [3 n] triangles in wide-leaf order
    int count = 0, levels = 0, n = 0;
    uint64_t serial = 0;        // key of the binary tree this was collapsed from
    float build_ms = 0;

   private:
    void release();
    int cap_ = 0;
    int2 *items_a_ = nullptr, *items_b_ = nullptr;
    uint32_t* counters_ = nullptr;
    uint32_t* counters_host_ = nullptr;
};

}  // namespace lts
