// Karras 2012 LBVH build on sm_103a: the reference's CreateBVHTree (acceleration/BVH.cuh:411-452)
// as five stream-ordered stages over structure-of-arrays buffers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace lts {

// One interior node with both child boxes, 64 bytes = four 16-byte loads in traversal.
// Child encoding: >= 0 interior node index, < 0 leaf ~l (l = position in Morton order).
struct alignas(16) BvhNode {
    float4 a;  // left  min.xyz, left  max.x
    float4 b;  // left  max.yz,  right min.xy
    float4 c;  // right min.z,   right max.xyz
    int4 d;    // left child, right child, first and last leaf (Morton position) of the node's range
};

enum { BVH_MODE_REFERENCE = 0, BVH_MODE_SORTED = 1 };

class Lbvh {
   public:
    Lbvh() = default;
    ~Lbvh();
    Lbvh(const Lbvh&) = delete;
    Lbvh& operator=(const Lbvh&) = delete;

    // Enqueue a build over n triangles (9 floats each, device pointer) on stream s.
    // mode: BVH_MODE_*; code_limit: primitives >= code_limit keep code 0 / id 0 (reference
    // Morton launch extent), < 0 for none.  stage events are recorded when timing is on.
    // Returns "" or an error message (allocation failure).
    std::string build(const float* d_tri, int n, int mode, int code_limit, cudaStream_t s, uint32_t* d_error);

    // Elapsed device milliseconds of the 5 stages of the last build (synchronises on events);
    // topology and refit run as one kernel, reported as the refit stage (topology ~0).
    void stage_ms(float out[5]) const;

    int n = 0;
    int mode = BVH_MODE_SORTED;
    // Outputs (device).
    BvhNode* nodes = nullptr;        // [n-1] (n >= 2)
    float* root_bounds = nullptr;    // [6]
    int32_t* leaf_prim = nullptr;    // [n] primitive held by leaf l
    uint32_t* codes = nullptr;       // [n] sorted Morton codes
    int32_t* ids = nullptr;          // [n] sorted primitive ids
    int launches = 0;
    uint64_t serial = 0;  // incremented by every build; consumers cache derived data by it
    size_t bytes_allocated() const { return bytes_; }

   private:
    std::string reserve(int n);
    int cap_ = 0;
    size_t bytes_ = 0;
    uint32_t *codes_alt_ = nullptr, *hist_ = nullptr, *status_ = nullptr, *counters_ = nullptr,
             *gbounds_ = nullptr, *flags_ = nullptr;
    int32_t* ids_alt_ = nullptr;  // second half of codes_alt_'s allocation
    uint32_t epoch_ = 0;            // tree-build epoch written into the arrival words (flags_)
    bool clear_arrivals_ = false;   // flags_ is fresh memory and must be zeroed once
    cudaEvent_t ev_[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
};

// Radix-sort tile geometry (exposed for the byte model and tests).
constexpr int kSortThreads = 256;
#ifndef LTS_SORT_ITEMS
#define LTS_SORT_ITEMS 15  // keys per thread of one sort tile
#endif
constexpr int kSortItems = LTS_SORT_ITEMS;
constexpr int kSortTile = kSortThreads * kSortItems;

// Bounded waits on another block's flag (the sort's look-back): set the poll limit (<= 0: the
// default kSpinLimit); run one such wait on a flag that nothing sets, so that it runs out and
// sets DEV_ERR_LOOKBACK_TIMEOUT in *d_err (synchronises the stream).
std::string lbvh_set_spin_limit(int limit);
std::string lbvh_debug_wait_flag(uint32_t* d_err, cudaStream_t s);

}  // namespace lts
