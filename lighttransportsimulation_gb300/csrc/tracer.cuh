// Path tracer (sm_103a): the reference's PathTracingIntegrator over SoA scene tables.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/lts_capi.h"
#include "host_scene.hpp"
#include "lbvh.cuh"
#include "wide_bvh.cuh"
#include "ploc.cuh"

namespace lts {

struct DevTex {
    int32_t kind;
    float v[4];
};
struct DevMat {
    int32_t kind;
    float extra, on_a, on_b;
    DevTex tex[2];
    int32_t shade_class;  // 1..15: materials with the same BSDF and texture kinds share a class
};
constexpr int kShadeClasses = 16;  // class 0: rays that left the scene
struct DevLight {
    int32_t kind, prim;
    float L[3], p[3], radius, area;
};

// One image texture's pyramid (the fixed mode of Mipmap, materials/textures/Mipmap.cuh:34-73):
// level l holds w[l] x h[l] linear-RGB texels from img_texels + off[l] on, in 4 x 4 blocks
// (BlockedArray, core/MemoryHelper.cuh:36-100, with the in-block row v & 3): texel (u, v) is
// 16 (bw (v >> 2) + (u >> 2)) + 4 (v & 3) + (u & 3) with bw = ceil(w / 4).
constexpr int kImageLevels = 16;
struct DevImage {
    int32_t levels, wrap;  // wrap: 0 repeat, 1 black, 2 clamp
    float lod;             // levels - 1 + log2(0.01), the lookup's level coordinate
    int32_t pad;
    int32_t off[kImageLevels], w[kImageLevels], h[kImageLevels];
};

// Everything a render kernel reads, passed by value.
// One instance of the two-level render BVH (a mesh entry of the loader's `instances` record):
// world position = object position * scale + t.  96 bytes, six 16-byte loads.
struct alignas(16) DevInstance {
    float4 xf;        // t.xyz, 1 / scale
    float4 wlo, whi;  // world-space box of the instance's triangles (w unused)
    float4 olo, ohi;  // object-space box of the prototype's triangles (w unused)
    int4 ref;         // root node of the prototype's tree, the entry's first primitive (scene
                      // order), the shade class of its material, 0
};
constexpr int kMaxInstances = 32;

struct SceneView {
    int32_t ntri, nlight, width, height;
    const float4* __restrict__ leaf_v;   // [3 ntri] triangle of leaf l: p0 (w = prim id bits), p1, p2
    const float4* __restrict__ prim_v;   // [3 ntri] scene order
    // [8 ntri] shading record of each scene triangle, one 128-byte line (what a hit reads):
    //   [0] p0.xyz uv0.x  [1] p1.xyz uv0.y  [2] p2.xyz uv1.x
    //   [3] n0.xyz uv1.y  [4] n1.xyz uv2.x  [5] n2.xyz uv2.y
    //   [6] int bits: has vertex normals, mesh (= material) index, area-light index (-1: none), 0
    //   [7] unused
    // uvs are the mesh's, or (0,0) (1,0) (1,1) when it has none (Triangle.cu:137-143); normals
    // are zero when the mesh has none.
    const float4* __restrict__ prim_rec;
    const DevMat* __restrict__ mats;
    const DevLight* __restrict__ lights;
    const float* __restrict__ light_func;
    const float* __restrict__ light_cdf;
    float light_func_int;
    const BvhNode* __restrict__ nodes;
    const float* __restrict__ root_bounds;
    const WideNode* __restrict__ wnodes;  // 8-wide compressed BVH (null: traverse the binary tree)
    const float4* __restrict__ wtris;     // [3 ntri] triangles in wide-leaf order
    int32_t wcount;                       // wide nodes
    int32_t wtri_count;                   // triangles in wtris
    int32_t watertight;                   // 1: watertight triangle tests (fixed mode), 0: the reference's
    const DevInstance* __restrict__ inst;  // two-level render BVH: the instances (null, 0: none)
    int32_t ninst;
    const float4* __restrict__ img_texels;  // image-texture pyramids (DevImage)
    const DevImage* __restrict__ images;
    const float* __restrict__ filter;    // 16 x 16 Gaussian table
    float cam[23];
};

struct RenderParams {
    int32_t spp, max_bounce, rr_start;
    uint32_t seed;
    int32_t x0, y0, x1, y1;
    float spp_scale;                 // quake_rsqrt(spp) for ray differentials
    double* __restrict__ film;       // [W*H*4] compensated sums resolved in FP64
    float* __restrict__ sample_L;    // [crop * spp * 3] (record mode)
    uint64_t* __restrict__ sample_sig;
    unsigned long long* __restrict__ counters;  // [0] rays issued
    uint32_t* __restrict__ err;
    float* __restrict__ trace;       // record mode: 16-float event records of one sample
    long trace_sample;               // crop sample index traced (-1: none)
};

// One slice of a batched wavefront render: samples s_first .. s_first + nsc - 1 per pixel of a
// view's crop.  Batch sample index w in [base, base + nsc * npix) maps to sample
// s_first + (w - base) / npix of crop pixel (w - base) % npix in row-major order (sample-major;
// the finished samples are stored in this order; generation visits the pixels in tiles).  Plain
// data shared by the host and the kernels.
constexpr int kMaxViews = 256;  // view slices per wavefront batch
struct WfView {
    float cam[12];                 // origin, right, up, lower-left corner (HostScene::cam[0..11])
    int32_t W, H, x0, y0, x1, y1;  // film size and crop
    int32_t spp, s_first, nsc;     // the view's samples per pixel; the slice's first sample and count
    uint32_t seed;
    float spp_scale;               // quake_rsqrt(spp) for ray differentials
    int32_t pad;
    int64_t base, npix, film_off;  // first batch sample index; crop pixels; first film pixel
};

// The procedural textures' tables (host copies): the 512-entry Perlin permutation and the
// 10 x 3 marble colours; each translation unit with device textures uploads its own.
void texture_tables(unsigned char perm512[512], const float** marble30);

// The float renderer's transcendentals (cos, sin, acos, log2): 1 = evaluated in double and
// rounded once (option "libm_double"), 0 = CUDA's float functions.
std::string set_libm_double(int on);

// Known-answer check of single float device functions (lts_debug_kat): n records of 16 floats.
std::string kat_launch(int fn, const float* d_in, int n, float* d_out, cudaStream_t s);

// FP64 oracle renderer (render64.cu): the megakernel integrator in double on the binary LBVH.
std::string render64_launch(const SceneView& sv, const RenderParams& rp, int nleaf, bool record, cudaStream_t s);

class Tracer {
   public:
    Tracer() = default;
    ~Tracer();
    Tracer(const Tracer&) = delete;
    Tracer& operator=(const Tracer&) = delete;

    std::string upload_scene(const HostScene& sc, cudaStream_t s);
    // Forgets the uploaded scene after a failed upload: the scene tables are freed and the view
    // is emptied, so nothing can read a half-written or freed table.
    void drop_scene();
    size_t last_upload_bytes = 0;  // host-to-device bytes of the last upload_scene
    // The uploaded scene's triangles as 9 floats each, scene order (the LBVH build's input).
    std::string triangle_soup(float* d_soup, cudaStream_t s) const;
    std::string render(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, lts_render_out* out,
                       cudaStream_t s, uint32_t* d_err);
    std::string render_async(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, cudaStream_t s,
                             uint32_t* d_err);
    std::string film_get(const HostScene& sc, float* rgb, double* sums, cudaStream_t s);
    std::string autotune_views(const HostScene& sc, const Lbvh& bvh, const lts_view* views, int n,
                               const lts_render_desc& d, lts_autotune_result* res, cudaStream_t s, uint32_t* d_err);
    // Batched views (lts_render_views): every view's full frame through the wavefront loop.
    std::string render_views(const HostScene& sc, const Lbvh& bvh, const lts_view* views, int n,
                             const lts_render_desc& d, float* const* films, lts_render_out* out, cudaStream_t s,
                             uint32_t* d_err);

    double last_ms = 0, last_paths = 0, last_rays = 0, last_node_visits = 0, last_tri_tests = 0;
    // Path-pool capacity of the wavefront integrator (0: automatic, see auto_pool).
    long wf_pool = 0;
    // Traversal structure: 8 = the collapsed 8-wide compressed BVH, 2 = the binary LBVH.
    int bvh_width = 8;
    // Triangle test: 0 = the reference's epsilon-shrunk Moller-Trumbore (parity), 1 = watertight.
    int watertight = 0;
    // Binary tree the 8-wide BVH is collapsed from, and how: 1 = PLOC over the LBVH's Morton
    // order, SAH-optimal collapse; 2 = the PLOC tree, greedy collapse; 0 = the LBVH itself, greedy.
    int render_bvh = 1;
    float last_render_bvh_ms = 0;  // PLOC + collapse of the last rebuild
    // Scenes with instanced meshes: 1 = the two-level 8-wide BVH (one tree per prototype under
    // a top level), 0 = one flat tree over every triangle.  Needs bvh_width 8 and render_bvh != 0.
    int two_level = 1;
    // Bidirectional integrator: -1 all strategies MIS-weighted, else only s = v / 100, t = v % 100.
    int bdpt_strategy = -1;
    bool last_two_level = false;  // the last render traversed the two-level BVH
    // Radiance cache (wavefront integrator): on/off, the MLP it queries and trains (owned by the
    // context), the share of paths traced in full (per mille), training records per render, Adam
    // steps per render and learning rate; statistics of the last render.
    int cache_mode = 0;
    class Mlp* mlp = nullptr;
    int cache_unbiased_permille = 30, cache_train_cap = 65536, cache_train_steps = 8;
    float cache_lr = 1e-3f;
    double last_cache_queries = 0, last_cache_bias = 0;
    int last_train_samples = 0, last_train_eligible = 0;
    float last_train_loss = 0, last_train_ms = 0;
    // Keep the film's sums across renders (progressive rendering) instead of clearing them.
    bool film_accumulate = false;
    bool last_wide = false;  // the last render traversed the wide BVH
    // Wavefront iterations as CUDA graphs launched in groups (1), or launched one by one with
    // host-sized grids and per-stage timing (0).
    int wf_graph = 1;
    // Persistent trace blocks per SM (0: as many as stay resident).
    int trace_blocks_per_sm = 0;
    // Finished-sample buffer capacity of the wavefront film gather, in samples (0: 2^27).
    long wf_sample_cap = 0;
    int last_iterations = 0;
    // Parity debugging: the record-mode render writes the events of this crop sample index.
    long trace_sample_ = -1;
    float* trace_ = nullptr;
    int last_launches = 0;
    // Wavefront: device time per stage (generate, trace, finalize, shade, compact, film gather)
    // summed over the loop's iterations, and rays / node visits / triangle tests per traversal kind
    // (path rays, shadow rays, MIS rays).  Zero for the megakernel.
    double last_stage_ms[6] = {0, 0, 0, 0, 0, 0};
    double last_kind_work[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};

    // Batch ray queries (lts_intersect): rays as n x {o.xyz, tmax, d.xyz, 0} on the device; any = 0
    // closest hit -> prim (-1: none) and t; any = 1 -> prim 1 (occluded) or 0.
    std::string intersect(const Lbvh& bvh, const float4* d_rays, int n, int any, int32_t* d_prim, float* d_t,
                          cudaStream_t s, uint32_t* d_err);

    // n image-texture lookups (Mipmap::lookUp) of image `idx` at d_st[2n] into d_rgb[3n].
    std::string image_lookup(int idx, const float* d_st, int n, float* d_rgb, cudaStream_t s);

    // Device bytes of the render BVH's nodes and triangles last used (two-level or flat).
    size_t render_bvh_bytes = 0;

   private:
    std::string traversal_view(const Lbvh& bvh, cudaStream_t s, uint32_t* d_err, SceneView* sv);
    // Two-level render BVH of a scene with instanced meshes: upload_scene keeps the instances,
    // the prototypes' object-space triangles and the ids of the other triangles; build_instanced
    // builds an LBVH + PLOC + 8-wide tree over those other triangles (the top-level tree, root 0,
    // leaf triangles carrying their scene-order ids) and one over each prototype (leaf triangles
    // carrying their index in the prototype), and concatenates them with rebased indices.
    struct InstHost {
        int32_t mesh, proto, prim_first, ntri, cls;
        float t[3], s;
    };
    std::string capture_instances(const HostScene& sc, const std::vector<DevMat>& mats, cudaStream_t s);
    std::string build_instanced(uint64_t key, cudaStream_t s, uint32_t* d_err);
    void release_instanced();
    std::vector<InstHost> inst_host_;
    std::vector<size_t> proto_off_;  // first triangle of each prototype in proto_soup_d_
    std::vector<int> proto_n_;
    std::vector<float> proto_box_;   // per prototype: object-space lo.xyz, hi.xyz
    float world_box_[6] = {0, 0, 0, 0, 0, 0};  // the non-instanced triangles' bounds
    float* proto_soup_d_ = nullptr;  // the prototypes' object-space triangles, 9 floats each
    int32_t* world_ids_d_ = nullptr; // scene-order ids of the non-instanced triangles
    int world_n_ = 0;
    float* isoup_ = nullptr;         // one tree's input triangles (9 floats each)
    float4* ileaf_ = nullptr;        // one tree's leaf-ordered triangles
    size_t isoup_cap_ = 0, ileaf_cap_ = 0;
    Lbvh ilbvh_;
    PlocBvh iploc_;
    WideBvh iwide_;
    WideNode* inodes_ = nullptr;     // the concatenated trees: top level first (root 0)
    float4* itris_ = nullptr;
    DevInstance* dinst_ = nullptr;
    float* iroot_ = nullptr;         // bounds of the whole two-level scene
    size_t inodes_cap_ = 0, itris_cap_ = 0;
    int icount_ = 0, itri_n_ = 0, ilevels_ = 0;
    // shade classes of the loaded scene: used, lobe mask and textured (the shade kernel variant)
    bool shade_used_[kShadeClasses] = {false};
    int shade_lm_[kShadeClasses] = {0};
    bool bdpt_matte_only_ = false;  // every material Lambertian / Oren-Nayar with constant textures
    bool shade_tex_[kShadeClasses] = {false};
    unsigned shade_grid_ = 0;  // resident blocks of the shade kernel on this device
    // side streams and fork / join events: the classes' shade launches run concurrently (as
    // parallel branches of the captured iteration graph)
    cudaStream_t shade_streams_[kShadeClasses] = {nullptr};
    cudaEvent_t shade_fork_ = nullptr, shade_join_[kShadeClasses] = {nullptr};
    double* splat_ = nullptr;  // bidirectional integrator: light-to-camera splats, RGB per pixel
    size_t splat_cap_ = 0;
    long splat_spp_ = 0;       // samples per pixel the splats hold
    uint64_t ikey_ = 0;              // key of the scene upload and render-tree choice built from
    uint64_t upload_serial_ = 0;
    int two_level_ok_ = 0;
    std::string prepare(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, cudaStream_t s,
                        uint32_t* d_err, RenderParams* rp, SceneView* sv, long* crop_samples);
    void free_all();
    std::string render_wavefront(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, cudaStream_t s,
                                 uint32_t* d_err, const RenderParams& rp, const SceneView& sv, long total);
    std::string run_wavefront(const std::vector<std::vector<WfView>>& batches, const Lbvh& bvh, cudaStream_t s,
                              uint32_t* d_err, const RenderParams& rp, const SceneView& sv);
    void* wf_bufs_[48] = {nullptr};
    // Device bytes per pool slot: the path state and lists, and the radiance cache's features,
    // prediction, query list and training-record links.
    static constexpr size_t kPoolSlotBytes = 392, kCacheSlotBytes = 248;
    long auto_pool(bool cache) const;
    long wf_cache_cap_ = 0, wf_train_cap_ = 0;
    // eligible training vertices per path of the last cached render (-1: none yet) and the
    // path count of the current one (the training-record coin's rate)
    double cache_eligible_rate_ = -1, cache_render_paths_ = 0;
    std::string train_cache(uint32_t* d_counts, uint16_t* tr_feat, float* tr_target, uint32_t tr_cap, cudaStream_t s,
                            uint32_t* d_err);
    long wf_cap_ = 0, wf_fs_cap_ = 0;
    uint32_t* wf_counts_host_ = nullptr;
    void* wf_ctl_host_ = nullptr;  // pinned mirror of the wavefront control block
    cudaEvent_t wf_ev_[7] = {nullptr};
    unsigned wf_trace_blocks_[3] = {0, 0, 0};  // resident blocks of k_wf_trace: wide, binary, two-level
    unsigned wf_sms_ = 0;  // resident blocks of k_wf_trace (wide, binary) on this device
    SceneView view_{};
    WideBvh wide_;
    PlocBvh ploc_;
    static constexpr int kSceneBufs = 17;
    void* bufs_[kSceneBufs] = {nullptr};   // scene tables, kept across scene loads while big enough
    size_t bufcap_[kSceneBufs] = {0};
    float4* leaf_v_ = nullptr;
    int leaf_n_ = 0;
    uint64_t leaf_serial_ = 0;  // Lbvh::serial the leaf_v_ copy was gathered for
    double* film_ = nullptr;
    double* views_film_ = nullptr;
    size_t views_film_cap_ = 0;
    size_t film_cap_ = 0;
    float* rec_L_ = nullptr;
    uint64_t* rec_sig_ = nullptr;
    size_t rec_cap_ = 0;
    unsigned long long* counters_ = nullptr;
    float* rgb_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
};

}  // namespace lts
