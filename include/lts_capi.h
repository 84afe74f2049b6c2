/*
 * lts_capi.h -- C-ABI of the GB300 (sm_103a) renderer for the hot path of
 * tierChampion/LightTransportSimulation: the Karras LBVH build and the unidirectional path
 * tracer.  Plain pointers and sizes only; every call returns an int status (LTS_OK == 0) and
 * never exits the process.  One host thread per context; calls are synchronous on the
 * context's own CUDA stream unless the name ends in _async.  The context owns all device
 * memory it allocates; the caller owns every host buffer it passes.
 *
 * Each entry point names the reference code it replaces (paths inside the reference tree).
 */
#ifndef LTS_CAPI_H
#define LTS_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define LTS_OK 0
#define LTS_ERR_ARG 1         /* bad argument / size                                   */
#define LTS_ERR_IO 2          /* file missing or unreadable                            */
#define LTS_ERR_PARSE 3       /* malformed app.params / .scene / .subject / .bin       */
#define LTS_ERR_CUDA 4        /* CUDA runtime error (message in lts_last_error)        */
#define LTS_ERR_OOM 5         /* an allocation failed or exceeded LTS_MAX_DEVICE_MB    */
#define LTS_ERR_UNSUPPORTED 6 /* input uses a feature outside this renderer's scope    */
#define LTS_ERR_STATE 7       /* call order (e.g. render before load)                  */
#define LTS_ERR_DEVICE 8      /* a kernel reported an error flag (queue overflow, wait limit) */

typedef struct lts_ctx lts_ctx;

/* Replaces the process-wide setup of LightTransportSimulation.cu:23-61 (no exit on error).
 * device == -1 makes a host-only context: files can be parsed and the scene queried, every
 * call that needs the GPU returns LTS_ERR_STATE.  There is no CPU rendering fallback. */
int lts_create(lts_ctx** out, int device);
void lts_destroy(lts_ctx* ctx);
/* Last error message of this context ("" if none).  Replaces gpuAssert's stderr print +
 * exit (core/ErrorHelper.cuh:26-32). */
const char* lts_last_error(const lts_ctx* ctx);
/* The cudaStream_t every call of this context is issued on (as void*). */
void* lts_stream(lts_ctx* ctx);

/* ---------------------------------------------------------------- inputs */
typedef struct {
    int32_t width, height, spp, max_bounce, rr_start, format;
    char output[256]; /* token + ".pfm" (format 1) or ".hdr" (format 0, PPM content) */
    char scene[256];
    char subject[256];
} lts_app_params;

/* Parses app.params: `W H spp bounces rrStart format output scene subject`.
 * Replaces readApplicationParameters (core/FileIO.cuh:234-257). */
int lts_read_app_params(const char* path, lts_app_params* out);

/* Converts mesh_name + ".obj" to mesh_name + ".bin" (the loader's binary mesh layout).
 * Replaces parseMeshFile + binMeshWrite (core/FileIO.cuh:20-45, 73-164): whitespace tokens,
 * "v"/"vn" three floats, "vt" two, "f" three "p/uv/n" corners (uv index 0 until a "vt" has been
 * read).  LTS_ERR_IO when a file cannot be opened or written, LTS_ERR_PARSE on input the
 * reference's reader has no defined result for. */
int lts_obj_to_bin(const char* mesh_name);

/* Loads `root + scene + ".scene"` and optionally `root + subject + ".subject"` with their
 * meshes (`name.bin`, else `name.obj`, converted and also written to `name.bin` as the
 * reference's parseMesh does, core/FileIO.cuh:213-232), transforms subject meshes, builds the camera for a width x height film and
 * the light table, and uploads SoA tables to the device.  subject may be NULL or "".
 * Replaces parseScene (core/SceneLoader.cuh:195-360) and the init kernels of
 * core/SceneLoader_kernels.cu:8-111.  Image textures ('i') load PNG and baseline JPEG files in
 * the fixed mode of lts_scene_get_image; other image formats, interlaced PNGs and progressive
 * JPEGs give LTS_ERR_UNSUPPORTED. */
int lts_load_scene(lts_ctx* ctx, const char* root, const char* scene, const char* subject,
                   int32_t width, int32_t height);

typedef struct {
    int32_t triangles, meshes, subject_meshes, materials, lights, area_light_meshes, has_infinite;
    int32_t width, height;
    int32_t max_mesh_triangles; /* largest mesh: bounds the reference's Morton launch */
    int32_t instances, prototypes; /* the `instances` record: instanced mesh entries, their files */
    int32_t images;                /* image textures */
} lts_scene_info;
int lts_scene_info_get(lts_ctx* ctx, lts_scene_info* out);

/* World-space vertex positions of every primitive in scene order (9 floats per triangle),
 * the camera as 23 floats {o, right, up, llc, u, v, w (3 each), lensRadius, focalDist}
 * (rendering/Camera.cu:9-43), and the light power distribution func[lights], cdf[lights+1]
 * (intergrators/IntegratorHelper.cuh:147-162, sampling/Sampling.cuh:123-144). */
int lts_scene_get_triangles(lts_ctx* ctx, float* out_p9);
int lts_scene_get_camera(lts_ctx* ctx, float* out23);
int lts_scene_get_light_distribution(lts_ctx* ctx, float* func, float* cdf);

/* Image textures of the loaded scene, in the reference's image order (subject images first):
 * the fixed mode of ImageTexture / Mipmap (materials/textures/ImageTexture.cuh:13-28,
 * Mipmap.cuh:34-73, Mipmap_kernel.cu:39-73), whose reference storage is undefined (its
 * BlockedArray shares rows and writes past its allocation, core/MemoryHelper.cuh:86-100).  PNG
 * and baseline JPEG files, decoded to the 8-bit values the reference's stb_image gives;
 * texel = (c / 255)^2.2 in float, rows
 * flipped so v = 0 is the bottom row; floor(log2(max(w, h))) levels (at least one), level l the
 * 2 x 2 box mean of level l - 1 with black outside.  wh_levels[3] receives the level's width,
 * height and the image's level count; rgb (NULL or 3 w h floats) its texels, row-major. */
int lts_scene_get_image(lts_ctx* ctx, int32_t image, int32_t level, int32_t* wh_levels, float* rgb);
/* n lookups of one image texture on the device (Mipmap::lookUp at the reference's fixed width
 * 0.01, Mipmap.cuh:61-72, trilinear between the two levels around log2 of the width):
 * st[2n] texture coordinates in, rgb[3n] out; host buffers. */
int lts_debug_image_lookup(lts_ctx* ctx, int32_t image, const float* st, int32_t n, float* rgb);

/* ---------------------------------------------------------------- LBVH */
/* LTS_BVH_REFERENCE: the reference's build exactly (acceleration/BVH.cuh:77-452): Morton
 *   codes only for primitives below code_limit (SceneLoader.cuh:324-339 launches
 *   ceil(maxMeshTris/16)*16 threads; the rest keep code 0 / id 0 from zeroed memory), and
 *   leaf l holds primitive l, not the sorted primitive (BVH.cuh:242,315,383).
 * LTS_BVH_SORTED: the textbook LBVH: every primitive coded, leaf l holds sorted primitive
 *   ids[l].  Same Morton arithmetic, stable order and Karras topology. */
#define LTS_BVH_REFERENCE 0
#define LTS_BVH_SORTED 1

/* Host buffers to receive the build; any pointer may be NULL.  N primitives, 2N-1 nodes in
 * the reference's flattened order (interior 0..N-2, leaves N-1..2N-2, BVH.cuh:311-329). */
typedef struct {
    uint32_t* sorted_codes; /* [N]   */
    int32_t* sorted_ids;    /* [N]   */
    int32_t* node_key;      /* [2N-1] -1 for interior nodes, leaf index l for leaves */
    int32_t* node_left;     /* [2N-1] child node index, -1 for leaves */
    int32_t* node_right;    /* [2N-1] */
    float* node_bounds;     /* [6(2N-1)] pMin xyz, pMax xyz */
} lts_bvh_dump;

/* Builds the LBVH of the loaded scene.  Replaces CreateBVHTree (BVH.cuh:411-452) with the
 * Morton pass (BVH_kernels.cu:8-15) and the bounds of sceneInitKernel
 * (SceneLoader_kernels.cu:87, BVH.cuh:92-97). */
int lts_bvh_build(lts_ctx* ctx, int32_t mode, lts_bvh_dump* dump);

/* Same build over a host triangle soup (9 floats per triangle, n >= 1); code_limit < 0
 * means "all primitives".  The BVH is kept in the context for lts_bvh_dump_get. */
int lts_bvh_build_triangles(lts_ctx* ctx, const float* tri_p9, int32_t n, int32_t mode, int32_t code_limit,
                            lts_bvh_dump* dump);

/* Device-resident variant for benchmarks: d_tri_p9 is a device pointer (9 floats per
 * triangle, 4-byte aligned).  Enqueued on the context stream; returns without waiting. */
int lts_bvh_build_device_async(lts_ctx* ctx, const float* d_tri_p9, int32_t n, int32_t mode,
                               int32_t code_limit);
/* Copies the last build to host buffers (synchronises the stream). */
int lts_bvh_dump_get(lts_ctx* ctx, lts_bvh_dump* dump);

/* No counterpart in the reference.  The same LBVH build for callers that may not allocate
 * device memory (memory-pool or allocator callbacks, real-time loops that forbid cudaMalloc,
 * plugins whose host owns every allocation): no context, no cudaMalloc/cudaFree, all scratch in
 * one fixed file-scope device array of about 3.3 MiB that each GPU loading the library keeps
 * until exit.  n <= LTS_NOALLOC_MAX_PRIMITIVES, else LTS_ERR_ARG.  The caller passes device
 * buffers: d_tri_p9 [9n floats], outputs d_sorted_codes [n], d_sorted_ids [n], d_nodes
 * [(n-1) x 64 bytes: left box, right box, children (>= 0 interior, < 0 leaf ~l), first and last
 * leaf of the node's range], d_leaf_prim
 * [n], d_root_bounds [6].  Runs on `stream` (a cudaStream_t, NULL for the default stream) and
 * blocks until that work has finished: it copies the kernels' error word to the host and
 * synchronises the stream before returning.  The first call on a device looks up the array's
 * address (may load the module): make it before any stream capture.  The address is kept for
 * the process's life, so after cudaDeviceReset of a device this entry point is not called on it
 * again.  Calls share the array, so calls that overlap on the GPU race. */
#define LTS_NOALLOC_MAX_PRIMITIVES 262144
int lts_bvh_build_noalloc(const float* d_tri_p9, int32_t n, int32_t mode, int32_t code_limit,
                          uint32_t* d_sorted_codes, int32_t* d_sorted_ids, void* d_nodes, int32_t* d_leaf_prim,
                          float* d_root_bounds, void* stream);

/* ---------------------------------------------------------------- rendering */
#define LTS_INTEGRATOR_MEGAKERNEL 0 /* one thread per pixel, all spp and bounces        */
#define LTS_INTEGRATOR_WAVEFRONT 1  /* generate / extend / shade / shadow / film queues  */
#define LTS_INTEGRATOR_FP64 2       /* the megakernel in double: FP64 oracle renders      */
/* Bidirectional path tracing (the reference's disabled BidirectionalPathIntegrator,
 * intergrators/BidirectionalPathIntegrator.cuh:285-660, built as PBRT v3 states the algorithm):
 * every connection of a camera and a light subpath, MIS-weighted; light-to-camera connections are
 * splatted and added at lts_film_get.  Area and point lights only (LTS_ERR_UNSUPPORTED with an
 * infinite light), max_bounce <= 8, no record mode, no Russian roulette. */
#define LTS_INTEGRATOR_BDPT 3

typedef struct {
    int32_t spp, max_bounce, rr_start;
    uint32_t seed;
    int32_t integrator; /* LTS_INTEGRATOR_* */
    /* Pixel crop [x0,x1) x [y0,y1) of the loaded film; x1 = y1 = 0 means the whole film. */
    int32_t x0, y0, x1, y1;
    /* Non-zero: record per-(pixel, sample) radiance and event hash for parity checks. */
    int32_t record_samples;
    int32_t bvh_mode; /* LTS_BVH_* used for traversal (results agree up to exact-t ties) */
} lts_render_desc;

typedef struct {
    float* film_rgb;      /* [W*H*3] resolved film (Camera::getRender: rgb/w, clamp >= 0,
                             Y flipped), or NULL */
    double* film_sums;    /* [W*H*4] FP64 resolve of the compensated sums {r,g,b,w}, or NULL */
    float* sample_L;      /* [crop pixels * spp * 3], requires record_samples, or NULL */
    uint64_t* sample_sig; /* [crop pixels * spp] FNV-1a hash of each sample's events, or NULL */
    double render_ms;     /* device time of the render kernels (CUDA events) */
    double rays;          /* ray queries issued (extension + shadow + MIS) */
    double node_visits;   /* BVH interior nodes fetched (64 bytes each) */
    double tri_tests;     /* ray-triangle tests (48 bytes of triangle data each) */
} lts_render_out;

/* Renders the loaded scene.  Replaces PathTracingKernel / PathTracingIntegrator::evaluate
 * (intergrators/IntegratorKernels.cu:17-23, PathTracingIntegrator.cuh:26-109) and the film
 * (rendering/Camera.cu:192-218,256-289).  Builds the LBVH first if none matches bvh_mode. */
int lts_render(lts_ctx* ctx, const lts_render_desc* desc, lts_render_out* out);

/* Enqueues one render of the whole film on the context stream without copying anything back
 * (film stays on the device); used for device-time benchmarks. */
int lts_render_async(lts_ctx* ctx, const lts_render_desc* desc);
/* Copies the film of the last render (synchronises). */
int lts_film_get(lts_ctx* ctx, float* film_rgb, double* film_sums);

/* Writes a film as the reference does: format 0 -> PPM P3 with gamma 1/2.2, format 1 -> PFM
 * (little-endian, scale -1).  Replaces writeToPPM / writeToPFM (core/ImageO.cuh:16-78). */
int lts_write_image(const char* path, const float* rgb, int32_t width, int32_t height, int32_t format);

/* Parity debugging (no counterpart in the reference): the next record-mode lts_render also
 * writes the intermediate values of one sample -- crop sample index k = (row * crop width +
 * column) * spp + sample, -1 to stop -- as up to 64 records of 16 floats (record[0] = event tag:
 * 1 hit, 2 material, 3 light sample, 4 MIS BSDF sample, 5 path BSDF sample, 6 final radiance). */
int lts_debug_trace_sample(lts_ctx* ctx, int64_t crop_sample_index);
int lts_debug_trace_get(lts_ctx* ctx, float* out_64x16);

/* Batched views (no counterpart in the reference: it renders the one camera of its scene file).
 * Camera records like the scene file's (from, at, up, vertical field of view in degrees, focus
 * distance), each with its own film size, samples per pixel and seed.  lts_render_views renders
 * all of them in batched wavefront launches that share the scene, its BVH and (when on) the
 * radiance cache: small views fill the GPU together.  desc gives max_bounce, rr_start and
 * bvh_mode (its integrator must be LTS_INTEGRATOR_WAVEFRONT; spp, seed and crop are ignored).
 * films_rgb[v] (host, width*height*3 floats) receives view v's resolved image like lts_render's
 * film_rgb; out (may be NULL) gets the total device time and ray counts. */
typedef struct {
    float from[3], at[3], up[3];
    float vfov, focus;
    int32_t width, height, spp;
    uint32_t seed;
} lts_view;
int lts_render_views(lts_ctx* ctx, const lts_view* views, int32_t n, const lts_render_desc* desc,
                     float* const* films_rgb, lts_render_out* out);

/* Autotuner (no counterpart in the reference): renders the views at 1/8 of their spp under each
 * candidate shape of the wavefront -- path-pool capacity 2^18 .. 2^26 below the tuning render's
 * path count, or the automatic pool (queue size), persistent trace blocks per SM 2 / 4 / all
 * resident (block shape), graph or kernel-by-kernel iterations -- one knob at a time from the
 * current settings, keeps the fastest and leaves it set on the context (the options
 * wavefront_pool, trace_blocks_per_sm, wavefront_graph).  pool_log2 0: the automatic pool. */
typedef struct {
    int32_t pool_log2, trace_blocks_per_sm, graph;
    double ms_default, ms_best; /* device ms of one tuning render before and after */
} lts_autotune_result;
int lts_autotune_views(lts_ctx* ctx, const lts_view* views, int32_t n, const lts_render_desc* desc,
                       lts_autotune_result* result);

/* Tuning knobs of the renderer (no counterpart in the reference).  Keys:
 *   "radiance_cache"          1: wavefront paths end at the first rough vertex (roughness > 0.3)
 *                             after their first rough vertex, with the MLP's radiance there
 *                             (specular vertices in between are traced); a share of paths is
 *                             traced in full, supervises the MLP (one record per path at that
 *                             vertex) and measures its bias; after each render the MLP takes Adam
 *                             steps on the records.  Needs lts_mlp_init.
 *   "radiance_cache_unbiased_permille" share of full paths (default 30 = 3 %)
 *   "radiance_cache_train_samples"     training records per render (default 65536)
 *   "radiance_cache_train_steps"       Adam steps per render (default 8)
 *   "radiance_cache_lr_micro"          learning rate in 1e-6 (default 1000 = 1e-3)
 *   "radiance_cache_ema_permille"      the cache's queries use an exponential moving average of the
 *                             weights with this decay per Adam step (per mille; 0: the weights)
 *   "film_accumulate"         1: renders add to the film's sums instead of clearing them
 *   "trace_blocks_per_sm"     persistent trace blocks per SM (0, default: all that stay resident)
 *   "wavefront_graph"         1 (default): each wavefront iteration runs as a captured CUDA graph,
 *                             launched in groups with one host check per group; 0: kernel by
 *                             kernel with host-sized grids and per-stage timing (lts_metrics)
 *   "bvh_width"               traversal structure: 8 (default) the 8-wide compressed BVH collapsed
 *                             from a binary tree, 2 the binary LBVH itself; all give the same hits
 *   "render_bvh"              binary tree the 8-wide BVH is collapsed from: 1 (default) a
 *                             surface-area tree clustered (PLOC) from the LBVH's Morton order,
 *                             collapsed by the SAH-optimal choice of children; 2 the same tree
 *                             collapsed greedily (largest child opened first); 0 the LBVH itself,
 *                             collapsed greedily
 *   "bdpt_strategy"           bidirectional integrator: 10000 (default) every strategy with its MIS
 *                             weight; 100 s + t renders the one strategy of s light and t camera
 *                             vertices unweighted (a debugging view: each strategy alone estimates
 *                             the paths it can sample)
 *   "two_level_bvh"           scenes with an `instances` record: 1 (default) one 8-wide tree per
 *                             instanced mesh file (prototype) under a top-level tree over the
 *                             other triangles, each instance entered with its ray moved to object
 *                             space; 0 one flat tree over every triangle.  Needs bvh_width 8 and
 *                             render_bvh 1 or 2; the closest hits are the same up to rounding
 *   "wavefront_pool"          path-state pool capacity in paths (0: automatic -- every path of
 *                             a batch at once, up to 2^26 slots and a quarter of the free
 *                             device memory, ~400 B per slot, ~650 B with the radiance cache)
 *   "wavefront_sample_chunk"  finished-sample buffer capacity in samples (0: automatic, 2^27);
 *                             samples per pixel are rendered in chunks that fit it
 *   "watertight"              0 (default): the reference's triangle tests (Moller-Trumbore with
 *                             barycentrics shrunk by 1e-4, Triangle.cu:50-128), 1: the watertight
 *                             test of Woop, Benthin and Wald (2013), which lets no ray through a
 *                             shared edge or vertex of a closed mesh (the fixed mode; renders differ
 *                             from the reference's near edges)
 *   "libm_double"             1: the float integrator's cos, sin, acos and log2 are evaluated in
 *                             double and rounded once to float (the correctly rounded values, as
 *                             the reference's host build gets them from glibc); 0 (default): CUDA's
 *                             float functions.  Process-wide; accepted before any scene is loaded
 *   "debug_spin_limit"        poll limit of every bounded wait of the kernels (the sort's
 *                             look-back on a predecessor tile, the tensor-core mbarrier waits);
 *                             0 restores the default (2^22 polls, over a second).  A test lowers
 *                             it to see a wait run out; accepted before any scene is loaded
 * Unknown keys and negative values return LTS_ERR_ARG. */
int lts_set_option(lts_ctx* ctx, const char* key, int64_t value);

/* Batch ray queries against the loaded scene, through the renderer's traversal and triangle
 * tests (the "watertight" option selects the test).  Each ray is one Scene::intersect (any = 0:
 * closest hit, acceleration/Scene.cuh:26-29) or Scene::simpleIntersect (any = 1: a hit before
 * tMax, Scene.cuh:30-32).  rays: n x 8 floats {ox, oy, oz, tMax, dx, dy, dz, 0} (host).  Out
 * (host): prim[n] the hit primitive in scene order (-1: none) or, for any = 1, 1 / 0; t[n] the hit
 * distance (INFINITY for none; t may be NULL).  Uses the render BVH of the last render, else
 * builds a sorted-leaf LBVH of the scene. */
int lts_intersect(lts_ctx* ctx, const float* rays, int32_t n, int32_t any, int32_t* prim, float* t);

/* Known-answer check of single device functions (no counterpart in the reference: it runs the
 * renderer's float device code on the GPU for values a test compares with the reference's own
 * functions).  n records of 16 floats in `in` (host), 16 floats out per record in `out` (host);
 * unused slots are zero.  Function fn and its record layout (inputs -> outputs):
 *   LTS_KAT_QUAKE_RSQRT        x -> quakeIIIFastInvSqrt(x)                   (Geometry.cuh:15-29)
 *   LTS_KAT_FRESNEL_DIELECTRIC cos, etaI, etaT -> F                          (BxDF.cuh:16-37)
 *   LTS_KAT_FRESNEL_CONDUCTOR  cos, etaT rgb, k rgb -> F rgb (etaI = 1)      (BxDF.cuh:44-67)
 *   LTS_KAT_TR_D               wh xyz, alphaX, alphaY -> D(wh)               (Microfacet.cuh:157-165)
 *   LTS_KAT_TR_LAMBDA          w xyz, alphaX, alphaY -> Lambda(w)            (Microfacet.cuh:130-137)
 *   LTS_KAT_TR_G1              w xyz, alphaX, alphaY -> G1(w)                (Microfacet.cuh:167-169)
 *   LTS_KAT_TR_G               wo xyz, wi xyz, alphaX, alphaY -> G(wo, wi)   (Microfacet.cuh:171-173)
 *   LTS_KAT_TR_SAMPLE11        cosTheta, u1, u2 -> slopeX, slopeY            (Microfacet.cuh:53-96)
 *   LTS_KAT_TR_SAMPLE_WH       wo xyz, alphaX, alphaY, u1, u2 -> wh xyz      (Microfacet.cuh:175-185)
 *   LTS_KAT_TR_PDF             wo xyz, wh xyz, alphaX, alphaY -> Pdf(wo, wh) (Microfacet.cuh:187-189)
 *   LTS_KAT_MF_F               wo xyz, wi xyz, alpha, R rgb, eta rgb, k rgb -> f rgb
 *                              (MicrofacetReflection::f with FresnelConductor(1, eta, k), Microfacet.cuh:200-209)
 *   LTS_KAT_MF_PDF             wo xyz, wi xyz, alpha -> Pdf(wo, wi)          (Microfacet.cuh:224-228)
 *   LTS_KAT_MF_SAMPLE          wo xyz, alpha, u1, u2, R rgb, eta rgb, k rgb -> wi xyz, f rgb, pdf
 *                              (MicrofacetReflection::sampleF, Microfacet.cuh:211-222)
 *   LTS_KAT_PERLIN             x, y, z -> perlinNoise                        (Procedural.cuh:130-155)
 *   LTS_KAT_FBM                p xyz, dpdx xyz, dpdy xyz, omega, maxOctaves -> fbm (Procedural.cuh:161-179)
 *   LTS_KAT_TURBULENCE         same inputs -> turbulence                     (Procedural.cuh:181-205)
 *   LTS_KAT_OFFSET_ORIGIN      p xyz, pError xyz, n xyz, w xyz -> origin xyz (Geometry.cuh:782-797)
 * The BSDF-level functions are evaluated in the shading frame (identity transform). */
#define LTS_KAT_QUAKE_RSQRT 0
#define LTS_KAT_FRESNEL_DIELECTRIC 1
#define LTS_KAT_FRESNEL_CONDUCTOR 2
#define LTS_KAT_TR_D 3
#define LTS_KAT_TR_LAMBDA 4
#define LTS_KAT_TR_G1 5
#define LTS_KAT_TR_G 6
#define LTS_KAT_TR_SAMPLE11 7
#define LTS_KAT_TR_SAMPLE_WH 8
#define LTS_KAT_TR_PDF 9
#define LTS_KAT_MF_F 10
#define LTS_KAT_MF_PDF 11
#define LTS_KAT_MF_SAMPLE 12
#define LTS_KAT_PERLIN 13
#define LTS_KAT_FBM 14
#define LTS_KAT_TURBULENCE 15
#define LTS_KAT_OFFSET_ORIGIN 16
#define LTS_KAT_COUNT 17
int lts_debug_kat(lts_ctx* ctx, int32_t fn, const float* in, int32_t n, float* out);

/* Check of the bounded waits (no counterpart in the reference; the reference has no bounded
 * wait).  Runs one wait that nothing ends: which 0 polls a flag word as the sort's look-back
 * does, which 1 waits on an mbarrier phase as the tensor-core kernels do.  The wait gives up
 * after the poll limit, the kernel sets its error flag and returns, and the call returns
 * LTS_ERR_DEVICE with the flag in lts_last_error; the context stays usable. */
int lts_debug_wait_timeout(lts_ctx* ctx, int32_t which);

/* Tensor-core layout check (no counterpart in the reference): one 5th-generation tensor-core
 * product of bf16 operands with FP32 accumulation, in one of the three operand arrangements the
 * radiance-cache MLP uses.  mode 0: a 128x64, b 64x64, d = a b^T (128x64); mode 1: a 128x64,
 * b 64x96, d = a b (128x96); mode 2: a 128x96, b 128x64, d = a^T b (rows 0..95 of a 128x64 d).
 * a, b: host arrays of bf16 bit patterns, row-major; d: host FP32. */
int lts_debug_umma_probe(lts_ctx* ctx, int32_t mode, int32_t swap, const uint16_t* a, const uint16_t* b, float* d);

/* ---------------------------------------------------------------- radiance-cache MLP
 * No counterpart in the reference.  A 96 -> 5 x 64 (ReLU) -> 3 (exp) network without biases,
 * BF16 weights and activations on the tensor cores, FP32 master weights and Adam state, trained
 * with the relative L2 loss mean((pred - target)^2 / (pred^2 + 0.01)).  Parameters: FP32, the
 * row-major [out][in] matrices W0 (64x96), W1..W4 (64x64), W5 (16x64, rows 3..15 unused)
 * concatenated (LTS_MLP_PARAMS values).  Features: n x 96 bf16 bit patterns per sample. */
#define LTS_MLP_PARAMS 23552
#define LTS_MLP_FEATURES 96
int lts_mlp_init(lts_ctx* ctx, uint32_t seed);
int lts_mlp_set_params(lts_ctx* ctx, const float* params);
int lts_mlp_get_params(lts_ctx* ctx, float* params);
int lts_mlp_forward(lts_ctx* ctx, const uint16_t* features, int32_t n, float* out_rgb);
/* Gradient of the loss over the n samples; *loss receives the loss; grad (may be NULL) the
 * gradient before the update; then one Adam step (beta1 0.9, beta2 0.99, eps 1e-8) when lr > 0. */
int lts_mlp_train_step(lts_ctx* ctx, const uint16_t* features, const float* targets, int32_t n, float lr,
                       float* loss, float* grad);
/* Device-pointer variants, enqueued on the context's stream (lts_stream) without synchronising:
 * the inference and training passes the renderer runs on its own buffers, for callers whose
 * features already live on the device.  d_loss: one device float (may be NULL for none). */
int lts_mlp_forward_device_async(lts_ctx* ctx, const uint16_t* d_features, int32_t n, float* d_out_rgb);
int lts_mlp_train_step_device_async(lts_ctx* ctx, const uint16_t* d_features, const float* d_targets, int32_t n,
                                    float lr, float* d_loss);

/* ---------------------------------------------------------------- metrics */
typedef struct {
    double bvh_build_ms;  /* device time of the last LBVH build */
    double bvh_stage_ms[5]; /* bounds, morton, sort, topology, refit */
    double render_ms;
    double paths, rays;
    int64_t device_bytes; /* bytes currently allocated by the context */
    int32_t kernel_launches; /* kernels launched by the last build + render */
    int32_t render_launches; /* kernels launched by the last render alone */
    int32_t render_iterations; /* wavefront: stage-loop iterations of the last render (1 for the megakernel) */
    /* wavefront: device ms per stage (generate, trace, finalize, shade, compact, film gather) of
     * the last render, and per traversal kind (path rays, shadow rays, MIS rays) its rays, node
     * visits and triangle tests (filled by a synchronous lts_render); zero for the megakernel */
    double render_stage_ms[6];
    double kind_rays[3], kind_node_visits[3], kind_tri_tests[3];
    /* radiance cache (wavefront with the option radiance_cache = 1): queries answered by the
     * network, training records taken from the unbiased paths, the last Adam step's loss, the
     * relative bias of the cache's mean against those records before the update, and the time of
     * the bias check and training after the render */
    double cache_queries;
    int32_t cache_train_samples;
    double cache_train_loss, cache_bias, cache_train_ms;
    /* last lts_load_scene: host milliseconds parsing the files, and uploading the tables and
     * expanding them on the device (until the stream is idle) */
    double scene_parse_ms, scene_upload_ms;
    /* device milliseconds of the last render-BVH rebuild (clustering + 8-wide collapse) */
    double render_bvh_ms;
    /* host-to-device bytes copied by the last lts_load_scene (the scene's tables) */
    int64_t scene_upload_bytes;
    /* device bytes of the nodes, triangles and instance table the last render or ray query
     * traversed, and 1 when that was the two-level BVH of a scene with instanced meshes */
    int64_t render_bvh_bytes;
    int32_t render_two_level;
} lts_metrics;
int lts_get_metrics(lts_ctx* ctx, lts_metrics* out);

#ifdef __cplusplus
}
#endif
#endif
