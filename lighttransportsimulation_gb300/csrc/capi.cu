// C-ABI of include/lts_capi.h: context, inputs, LBVH build and rendering orchestration.
// Host code only; kernels live in lbvh.cu and tracer.cu.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/lts_capi.h"
#include "dev_common.cuh"
#include "host_scene.hpp"
#include "lbvh.cuh"
#include "mlp.cuh"
#include "tracer.cuh"

namespace lts {

static std::atomic<long long> g_bytes{0};
static std::mutex g_mu;
static std::unordered_map<void*, size_t> g_sizes;

static long long cap_bytes() {
    static long long cap = [] {
        const char* e = getenv("LTS_MAX_DEVICE_MB");
        return e ? (long long)atoll(e) * 1024 * 1024 : -1LL;
    }();
    return cap;
}

cudaError_t dev_alloc(void** p, size_t bytes) {
    *p = nullptr;
    const long long cap = cap_bytes();
    if (cap >= 0 && g_bytes.load() + (long long)bytes > cap) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e == cudaSuccess) {
        g_bytes += (long long)bytes;
        std::lock_guard<std::mutex> lk(g_mu);
        g_sizes[*p] = bytes;
    }
    return e;
}

void dev_free(void* p) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_sizes.find(p);
        if (it != g_sizes.end()) {
            g_bytes -= (long long)it->second;
            g_sizes.erase(it);
        }
    }
    cudaFree(p);
}

size_t dev_bytes_in_use() { return (size_t)g_bytes.load(); }

}  // namespace lts

using namespace lts;

struct lts_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    uint32_t* d_error = nullptr;

    HostScene scene;
    // The scene before the current one: the next load parses into it (its tables keep their
    // capacity, so a reload of a same-sized scene allocates nothing) and then swaps it in, so a
    // load that fails leaves `scene` as it was.
    HostScene spare_scene;
    bool loaded = false;
    float* d_tri = nullptr;  // scene triangle soup, 9 floats per triangle (scene order)
    size_t d_tri_cap = 0;
    std::unique_ptr<Lbvh> bvh;
    std::unique_ptr<Mlp> mlp;
    int bvh_mode = -1;        // mode of the BVH currently held (-1: none)
    bool bvh_is_scene = false;
    std::unique_ptr<Tracer> tracer;
    lts_metrics metrics{};
};

namespace {

int fail(lts_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}
int cuda_fail(lts_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? LTS_ERR_OOM : LTS_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                       \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

int check_device_error(lts_ctx* ctx) {
    uint32_t h = 0;
    CK(cudaMemcpyAsync(&h, ctx->d_error, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (h) {
        CK(cudaMemsetAsync(ctx->d_error, 0, 4, ctx->stream));
        char hex[16];
        snprintf(hex, sizeof hex, "0x%x", h);
        return fail(ctx, LTS_ERR_DEVICE, std::string("a kernel reported device error flags ") + hex);
    }
    return LTS_OK;
}

int ensure_tri_buffer(lts_ctx* ctx, size_t floats) {
    if (floats * 4 <= ctx->d_tri_cap) return LTS_OK;
    dev_free(ctx->d_tri);
    ctx->d_tri = nullptr;
    ctx->d_tri_cap = 0;
    CK(dev_alloc((void**)&ctx->d_tri, floats * 4));
    ctx->d_tri_cap = floats * 4;
    return LTS_OK;
}

int do_build(lts_ctx* ctx, const float* d_tri, int n, int mode, int code_limit) {
    if (mode != LTS_BVH_REFERENCE && mode != LTS_BVH_SORTED) return fail(ctx, LTS_ERR_ARG, "unknown BVH mode");
    if (!ctx->bvh) ctx->bvh.reset(new Lbvh());
    std::string e = ctx->bvh->build(d_tri, n, mode, code_limit, ctx->stream, ctx->d_error);
    if (!e.empty()) {
        ctx->bvh_mode = -1;
        return fail(ctx, e.find("memory") != std::string::npos ? LTS_ERR_OOM : LTS_ERR_CUDA, e);
    }
    ctx->bvh_mode = mode;
    return LTS_OK;
}

int dump_bvh(lts_ctx* ctx, lts_bvh_dump* d) {
    if (!ctx->bvh || ctx->bvh_mode < 0) return fail(ctx, LTS_ERR_STATE, "no BVH has been built");
    int rc = check_device_error(ctx);
    if (rc) return rc;
    Lbvh& b = *ctx->bvh;
    float st[5];
    b.stage_ms(st);
    ctx->metrics.bvh_build_ms = 0;
    for (int i = 0; i < 5; ++i) {
        ctx->metrics.bvh_stage_ms[i] = st[i];
        ctx->metrics.bvh_build_ms += st[i];
    }
    if (!d) return LTS_OK;
    const int n = b.n, nodes = 2 * n - 1;
    if (d->sorted_codes) CK(cudaMemcpy(d->sorted_codes, b.codes, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    if (d->sorted_ids) CK(cudaMemcpy(d->sorted_ids, b.ids, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    if (!d->node_key && !d->node_left && !d->node_right && !d->node_bounds) return LTS_OK;
    std::vector<BvhNode> h((size_t)(n > 1 ? n - 1 : 0));
    if (n > 1) CK(cudaMemcpy(h.data(), b.nodes, sizeof(BvhNode) * (n - 1), cudaMemcpyDeviceToHost));
    float root[6];
    CK(cudaMemcpy(root, b.root_bounds, 24, cudaMemcpyDeviceToHost));
    // Reference flattened order: interior 0..n-2, leaves n-1..2n-2 (BVH.cuh:311-329).
    std::vector<int32_t> key(nodes, -1), left(nodes, -1), right(nodes, -1);
    std::vector<float> bnd((size_t)nodes * 6, 0.f);
    for (int l = 0; l < n; ++l) key[n - 1 + l] = l;
    auto flat = [n](int c) { return c < 0 ? (n - 1) + ~c : c; };
    memcpy(&bnd[0], root, 24);
    if (n == 1) memcpy(&bnd[0], root, 24);
    for (int i = 0; i < n - 1; ++i) {
        const float* f = reinterpret_cast<const float*>(&h[i]);
        const int lc = flat(h[i].d.x), rc = flat(h[i].d.y);
        left[i] = lc;
        right[i] = rc;
        memcpy(&bnd[(size_t)lc * 6], f, 24);
        memcpy(&bnd[(size_t)rc * 6], f + 6, 24);
    }
    if (d->node_key) memcpy(d->node_key, key.data(), 4 * (size_t)nodes);
    if (d->node_left) memcpy(d->node_left, left.data(), 4 * (size_t)nodes);
    if (d->node_right) memcpy(d->node_right, right.data(), 4 * (size_t)nodes);
    if (d->node_bounds) memcpy(d->node_bounds, bnd.data(), 24 * (size_t)nodes);
    return LTS_OK;
}

void copy_str(char* dst, const std::string& s) {
    strncpy(dst, s.c_str(), 255);
    dst[255] = 0;
}

}  // namespace

extern "C" {

int lts_create(lts_ctx** out, int device) {
    if (!out) return LTS_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<lts_ctx> c(new lts_ctx());
    c->device = device;
    lts_ctx* ctx = c.get();
    if (device == -1) {  // host-only context: parsing and scene queries, no device work
        *out = c.release();
        return LTS_OK;
    }
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return LTS_ERR_CUDA;  // no device: the renderer has no CPU fallback
    if (device < 0 || device >= count) return LTS_ERR_ARG;
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(dev_alloc((void**)&c->d_error, 4));
    CK(cudaMemset(c->d_error, 0, 4));
    *out = c.release();
    return LTS_OK;
}

void lts_destroy(lts_ctx* ctx) {
    if (!ctx) return;
    if (ctx->device == -1) {
        delete ctx;
        return;
    }
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->tracer.reset();
    ctx->bvh.reset();
    dev_free(ctx->d_tri);
    dev_free(ctx->d_error);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* lts_last_error(const lts_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }
void* lts_stream(lts_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int lts_read_app_params(const char* path, lts_app_params* out) {
    if (!path || !out) return LTS_ERR_ARG;
    AppParams p;
    int code = LTS_OK;
    read_app_params(path, &p, &code);
    if (code) return code;
    out->width = p.width;
    out->height = p.height;
    out->spp = p.spp;
    out->max_bounce = p.max_bounce;
    out->rr_start = p.rr_start;
    out->format = p.format;
    copy_str(out->output, p.output);
    copy_str(out->scene, p.scene);
    copy_str(out->subject, p.subject);
    return LTS_OK;
}

int lts_obj_to_bin(const char* mesh_name) {
    if (!mesh_name) return LTS_ERR_ARG;
    int code = LTS_OK;
    obj_to_bin(mesh_name, &code);
    return code;
}

int lts_load_scene(lts_ctx* ctx, const char* root, const char* scene, const char* subject, int32_t width,
                   int32_t height) {
    if (!ctx || !root || !scene) return fail(ctx, LTS_ERR_ARG, "null argument");
    int code = LTS_OK;
    const auto t0 = std::chrono::steady_clock::now();
    std::string msg = load_scene(root, scene, subject ? subject : "", width, height, &ctx->spare_scene, &code);
    if (code) return fail(ctx, code, msg);
    const auto t1 = std::chrono::steady_clock::now();
    ctx->metrics.scene_parse_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    ctx->metrics.scene_upload_ms = 0;
    ctx->metrics.scene_upload_bytes = 0;
    std::swap(ctx->scene, ctx->spare_scene);
    ctx->loaded = true;
    ctx->bvh_mode = -1;
    ctx->bvh_is_scene = false;
    if (ctx->device == -1) return LTS_OK;
    CK(cudaSetDevice(ctx->device));
    if (!ctx->tracer) ctx->tracer.reset(new Tracer());
    // From here on the host scene is the new one: if its upload fails part way, the device copy
    // is incomplete (and buffers of the previous scene may already be freed), so the context
    // holds no usable scene until the next load succeeds.
    auto upload_failed = [ctx](int code, const std::string& msg) {
        ctx->loaded = false;
        ctx->tracer->drop_scene();
        return fail(ctx, code, msg);
    };
    std::string e = ctx->tracer->upload_scene(ctx->scene, ctx->stream);
    if (!e.empty()) return upload_failed(e.find("memory") != std::string::npos ? LTS_ERR_OOM : LTS_ERR_CUDA, e);
    // the LBVH input (9 floats per triangle), expanded on the device from the uploaded tables
    int rc = ensure_tri_buffer(ctx, 9 * (size_t)ctx->scene.triangles());
    if (rc) return upload_failed(rc, ctx->err);
    e = ctx->tracer->triangle_soup(ctx->d_tri, ctx->stream);
    if (!e.empty()) return upload_failed(LTS_ERR_CUDA, e);
    const cudaError_t se = cudaStreamSynchronize(ctx->stream);
    if (se != cudaSuccess) return upload_failed(LTS_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(se));
    ctx->metrics.scene_upload_bytes = (int64_t)ctx->tracer->last_upload_bytes;
    ctx->metrics.scene_upload_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
    return LTS_OK;
}

int lts_scene_info_get(lts_ctx* ctx, lts_scene_info* out) {
    if (!ctx || !out) return fail(ctx, LTS_ERR_ARG, "null argument");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    const HostScene& s = ctx->scene;
    out->triangles = s.triangles();
    out->meshes = (int32_t)s.mesh_tri_count.size();
    out->subject_meshes = s.subject_meshes;
    out->materials = (int32_t)s.materials.size();
    out->lights = (int32_t)s.lights.size();
    out->area_light_meshes = s.area_light_meshes;
    out->has_infinite = s.has_infinite ? 1 : 0;
    out->width = s.width;
    out->height = s.height;
    out->max_mesh_triangles = s.max_mesh_triangles();
    out->instances = (int32_t)s.instances.size();
    out->prototypes = (int32_t)s.proto_soup.size();
    out->images = (int32_t)s.images.size();
    return LTS_OK;
}

int lts_scene_get_triangles(lts_ctx* ctx, float* out) {
    if (!ctx || !out) return fail(ctx, LTS_ERR_ARG, "null argument");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    std::vector<float> soup;
    ctx->scene.triangle_soup(soup);
    memcpy(out, soup.data(), soup.size() * 4);
    return LTS_OK;
}

int lts_scene_get_camera(lts_ctx* ctx, float* out23) {
    if (!ctx || !out23) return fail(ctx, LTS_ERR_ARG, "null argument");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    memcpy(out23, ctx->scene.cam, sizeof ctx->scene.cam);
    return LTS_OK;
}

int lts_scene_get_light_distribution(lts_ctx* ctx, float* func, float* cdf) {
    if (!ctx) return LTS_ERR_ARG;
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    if (func) memcpy(func, ctx->scene.light_func.data(), 4 * ctx->scene.light_func.size());
    if (cdf) memcpy(cdf, ctx->scene.light_cdf.data(), 4 * ctx->scene.light_cdf.size());
    return LTS_OK;
}

int lts_bvh_build(lts_ctx* ctx, int32_t mode, lts_bvh_dump* dump) {
    if (!ctx) return LTS_ERR_ARG;
    if (ctx->device == -1) return fail(ctx, LTS_ERR_STATE, "host-only context (device -1) cannot run kernels");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    CK(cudaSetDevice(ctx->device));
    const int n = ctx->scene.triangles();
    // The reference's Morton launch covers ceil(maxMeshTris/16)*16 primitives
    // (SceneLoader.cuh:323-339, BVH_kernels.cu:10-12).
    const int limit = mode == LTS_BVH_REFERENCE ? ((ctx->scene.max_mesh_triangles() + 15) / 16) * 16 : -1;
    int rc = do_build(ctx, ctx->d_tri, n, mode, limit);
    if (rc) return rc;
    ctx->bvh_is_scene = true;
    return dump_bvh(ctx, dump);
}

int lts_bvh_build_triangles(lts_ctx* ctx, const float* tri, int32_t n, int32_t mode, int32_t code_limit,
                            lts_bvh_dump* dump) {
    if (!ctx || !tri || n < 1) return fail(ctx, LTS_ERR_ARG, "bad triangle input");
    if (ctx->device == -1) return fail(ctx, LTS_ERR_STATE, "host-only context (device -1) cannot run kernels");
    CK(cudaSetDevice(ctx->device));
    float* d = nullptr;
    CK(dev_alloc((void**)&d, 36 * (size_t)n));
    cudaError_t e = cudaMemcpyAsync(d, tri, 36 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        dev_free(d);
        return cuda_fail(ctx, e, "copy triangles");
    }
    int rc = do_build(ctx, d, n, mode, code_limit);
    if (rc == LTS_OK) rc = dump_bvh(ctx, dump);
    cudaStreamSynchronize(ctx->stream);
    dev_free(d);
    ctx->bvh_is_scene = false;
    return rc;
}

int lts_bvh_build_device_async(lts_ctx* ctx, const float* d_tri, int32_t n, int32_t mode, int32_t code_limit) {
    if (!ctx || !d_tri || n < 1) return fail(ctx, LTS_ERR_ARG, "bad triangle input");
    if (ctx->device == -1) return fail(ctx, LTS_ERR_STATE, "host-only context (device -1) cannot run kernels");
    ctx->bvh_is_scene = false;
    return do_build(ctx, d_tri, n, mode, code_limit);
}

int lts_bvh_dump_get(lts_ctx* ctx, lts_bvh_dump* dump) {
    if (!ctx) return LTS_ERR_ARG;
    return dump_bvh(ctx, dump);
}

int lts_render(lts_ctx* ctx, const lts_render_desc* desc, lts_render_out* out) {
    if (!ctx || !desc) return fail(ctx, LTS_ERR_ARG, "null argument");
    if (ctx->device == -1) return fail(ctx, LTS_ERR_STATE, "host-only context (device -1) cannot run kernels");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    CK(cudaSetDevice(ctx->device));
    const int mode = desc->bvh_mode == LTS_BVH_REFERENCE ? LTS_BVH_REFERENCE : LTS_BVH_SORTED;
    if (!(ctx->bvh_is_scene && ctx->bvh_mode == mode)) {
        int rc = lts_bvh_build(ctx, mode, nullptr);
        if (rc) return rc;
    }
    std::string e = ctx->tracer->render(ctx->scene, *ctx->bvh, *desc, out, ctx->stream, ctx->d_error);
    if (!e.empty()) return fail(ctx, e.find("argument") != std::string::npos ? LTS_ERR_ARG : LTS_ERR_CUDA, e);
    int rc = check_device_error(ctx);
    if (rc) return rc;
    ctx->metrics.render_ms = ctx->tracer->last_ms;
    ctx->metrics.paths = ctx->tracer->last_paths;
    ctx->metrics.rays = ctx->tracer->last_rays;
    return LTS_OK;
}

int lts_render_views(lts_ctx* ctx, const lts_view* views, int32_t n, const lts_render_desc* desc,
                     float* const* films_rgb, lts_render_out* out) {
    if (!ctx || !desc || !views || !films_rgb || n <= 0) return fail(ctx, LTS_ERR_ARG, "null argument");
    if (ctx->device == -1) return fail(ctx, LTS_ERR_STATE, "host-only context (device -1) cannot run kernels");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    CK(cudaSetDevice(ctx->device));
    const int mode = desc->bvh_mode == LTS_BVH_REFERENCE ? LTS_BVH_REFERENCE : LTS_BVH_SORTED;
    if (!(ctx->bvh_is_scene && ctx->bvh_mode == mode)) {
        int rc = lts_bvh_build(ctx, mode, nullptr);
        if (rc) return rc;
    }
    std::string e = ctx->tracer->render_views(ctx->scene, *ctx->bvh, views, n, *desc, films_rgb, out, ctx->stream,
                                              ctx->d_error);
    if (!e.empty()) return fail(ctx, e.find("argument") != std::string::npos ? LTS_ERR_ARG : LTS_ERR_CUDA, e);
    int rc = check_device_error(ctx);
    if (rc) return rc;
    ctx->metrics.render_ms = ctx->tracer->last_ms;
    ctx->metrics.paths = ctx->tracer->last_paths;
    ctx->metrics.rays = ctx->tracer->last_rays;
    return LTS_OK;
}

int lts_autotune_views(lts_ctx* ctx, const lts_view* views, int32_t n, const lts_render_desc* desc,
                       lts_autotune_result* result) {
    if (!ctx || !desc || !views || n <= 0) return fail(ctx, LTS_ERR_ARG, "null argument");
    if (ctx->device == -1) return fail(ctx, LTS_ERR_STATE, "host-only context (device -1) cannot run kernels");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    CK(cudaSetDevice(ctx->device));
    const int mode = desc->bvh_mode == LTS_BVH_REFERENCE ? LTS_BVH_REFERENCE : LTS_BVH_SORTED;
    if (!(ctx->bvh_is_scene && ctx->bvh_mode == mode)) {
        int rc = lts_bvh_build(ctx, mode, nullptr);
        if (rc) return rc;
    }
    std::string e = ctx->tracer->autotune_views(ctx->scene, *ctx->bvh, views, n, *desc, result, ctx->stream,
                                                ctx->d_error);
    if (!e.empty()) return fail(ctx, e.find("argument") != std::string::npos ? LTS_ERR_ARG : LTS_ERR_CUDA, e);
    return check_device_error(ctx);
}

int lts_render_async(lts_ctx* ctx, const lts_render_desc* desc) {
    if (!ctx || !desc) return fail(ctx, LTS_ERR_ARG, "null argument");
    if (ctx->device == -1) return fail(ctx, LTS_ERR_STATE, "host-only context (device -1) cannot run kernels");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    const int mode = desc->bvh_mode == LTS_BVH_REFERENCE ? LTS_BVH_REFERENCE : LTS_BVH_SORTED;
    if (!(ctx->bvh_is_scene && ctx->bvh_mode == mode)) {
        int rc = lts_bvh_build(ctx, mode, nullptr);
        if (rc) return rc;
    }
    std::string e = ctx->tracer->render_async(ctx->scene, *ctx->bvh, *desc, ctx->stream, ctx->d_error);
    if (!e.empty()) return fail(ctx, LTS_ERR_ARG, e);
    return LTS_OK;
}

int lts_film_get(lts_ctx* ctx, float* film_rgb, double* film_sums) {
    if (!ctx) return LTS_ERR_ARG;
    if (!ctx->tracer) return fail(ctx, LTS_ERR_STATE, "nothing rendered");
    int rc = check_device_error(ctx);
    if (rc) return rc;
    std::string e = ctx->tracer->film_get(ctx->scene, film_rgb, film_sums, ctx->stream);
    if (!e.empty()) return fail(ctx, LTS_ERR_CUDA, e);
    return LTS_OK;
}

int lts_write_image(const char* path, const float* rgb, int32_t w, int32_t h, int32_t format) {
    if (!path || !rgb || w < 1 || h < 1) return LTS_ERR_ARG;
    if (format == 1) {  // ImageO.cuh:16-50
        FILE* f = fopen(path, "wb");
        if (!f) return LTS_ERR_IO;
        fprintf(f, "PF\n%d %d\n%f\n", w, h, -1.0f);
        const size_t cnt = 3 * (size_t)w * h;
        const bool ok = fwrite(rgb, sizeof(float), cnt, f) == cnt;
        fclose(f);
        return ok ? LTS_OK : LTS_ERR_IO;
    }
    FILE* f = fopen(path, "w");  // ImageO.cuh:52-78
    if (!f) return LTS_ERR_IO;
    fprintf(f, "P3\n%d %d\n%d\n", w, h, 255);
    for (long i = 0; i < (long)w * h; ++i) {
        int c[3];
        for (int k = 0; k < 3; ++k) {
            float x = rgb[3 * i + k];
            x = (x < 0) ? 0 : ((x > 1) ? 1 : x);
            c[k] = int(powf(x, 1 / 2.2f) * 255 + 0.5);
        }
        fprintf(f, "%d %d %d ", c[0], c[1], c[2]);
    }
    fclose(f);
    return LTS_OK;
}

int lts_debug_umma_probe(lts_ctx* ctx, int32_t mode, int32_t swap, const uint16_t* a, const uint16_t* b, float* d) {
    if (!ctx || !a || !b || !d) return LTS_ERR_ARG;
    if (ctx->device < 0) return fail(ctx, LTS_ERR_STATE, "host-only context");
    const std::string e = umma_probe(mode, swap, a, b, d, ctx->d_error, ctx->stream);
    if (!e.empty()) return fail(ctx, LTS_ERR_ARG, e);
    return check_device_error(ctx);
}

namespace {
int mlp_ready(lts_ctx* ctx) {
    if (!ctx) return LTS_ERR_ARG;
    if (ctx->device < 0) return fail(ctx, LTS_ERR_STATE, "host-only context");
    if (!ctx->mlp || !ctx->mlp->ready()) return fail(ctx, LTS_ERR_STATE, "MLP not initialised (lts_mlp_init)");
    return LTS_OK;
}
}  // namespace

int lts_mlp_init(lts_ctx* ctx, uint32_t seed) {
    if (!ctx) return LTS_ERR_ARG;
    if (ctx->device < 0) return fail(ctx, LTS_ERR_STATE, "host-only context");
    if (!ctx->mlp) ctx->mlp.reset(new Mlp());
    const std::string e = ctx->mlp->init(seed, ctx->stream);
    return e.empty() ? LTS_OK : fail(ctx, LTS_ERR_DEVICE, e);
}

int lts_mlp_set_params(lts_ctx* ctx, const float* params) {
    if (int r = mlp_ready(ctx)) return r;
    if (!params) return LTS_ERR_ARG;
    const std::string e = ctx->mlp->set_params(params, ctx->stream);
    return e.empty() ? LTS_OK : fail(ctx, LTS_ERR_DEVICE, e);
}

int lts_mlp_get_params(lts_ctx* ctx, float* params) {
    if (int r = mlp_ready(ctx)) return r;
    if (!params) return LTS_ERR_ARG;
    const std::string e = ctx->mlp->get_params(params, ctx->stream);
    return e.empty() ? LTS_OK : fail(ctx, LTS_ERR_DEVICE, e);
}

int lts_mlp_forward(lts_ctx* ctx, const uint16_t* features, int32_t n, float* out_rgb) {
    if (int r = mlp_ready(ctx)) return r;
    if (!features || !out_rgb || n < 0) return LTS_ERR_ARG;
    if (n == 0) return LTS_OK;
    void *df = nullptr, *dout = nullptr;
    int rc = LTS_OK;
    if (dev_alloc(&df, 2 * (size_t)n * kMlpIn) != cudaSuccess || dev_alloc(&dout, 12 * (size_t)n) != cudaSuccess) {
        rc = fail(ctx, LTS_ERR_DEVICE, "MLP buffers: allocation failed");
    } else {
        std::string e;
        cudaError_t c = cudaMemcpyAsync(df, features, 2 * (size_t)n * kMlpIn, cudaMemcpyHostToDevice, ctx->stream);
        if (c == cudaSuccess) e = ctx->mlp->forward((const uint16_t*)df, n, (float*)dout, ctx->d_error, ctx->stream);
        if (c == cudaSuccess && e.empty())
            c = cudaMemcpyAsync(out_rgb, dout, 12 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
        if (c != cudaSuccess) e = cudaGetErrorString(c);
        rc = e.empty() ? check_device_error(ctx) : fail(ctx, LTS_ERR_DEVICE, e);
    }
    dev_free(df);
    dev_free(dout);
    return rc;
}

int lts_mlp_train_step(lts_ctx* ctx, const uint16_t* features, const float* targets, int32_t n, float lr,
                       float* loss, float* grad) {
    if (int r = mlp_ready(ctx)) return r;
    if (!features || !targets || n <= 0) return LTS_ERR_ARG;
    void *df = nullptr, *dt = nullptr, *dl = nullptr;
    int rc = LTS_OK;
    if (dev_alloc(&df, 2 * (size_t)n * kMlpIn) != cudaSuccess || dev_alloc(&dt, 12 * (size_t)n) != cudaSuccess ||
        dev_alloc(&dl, 4) != cudaSuccess) {
        rc = fail(ctx, LTS_ERR_DEVICE, "MLP buffers: allocation failed");
    } else {
        std::string e;
        cudaError_t c = cudaMemcpyAsync(df, features, 2 * (size_t)n * kMlpIn, cudaMemcpyHostToDevice, ctx->stream);
        if (c == cudaSuccess) c = cudaMemcpyAsync(dt, targets, 12 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
        if (c == cudaSuccess)
            e = ctx->mlp->train_step((const uint16_t*)df, (const float*)dt, n, 0.0f, (float*)dl, ctx->d_error,
                                     ctx->stream);
        if (c == cudaSuccess && e.empty() && grad) e = ctx->mlp->get_grad(grad, ctx->stream);
        if (c == cudaSuccess && e.empty() && loss) c = cudaMemcpyAsync(loss, dl, 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (c == cudaSuccess && e.empty() && lr > 0) e = ctx->mlp->adam(lr, ctx->stream);
        if (c == cudaSuccess && e.empty()) c = cudaStreamSynchronize(ctx->stream);
        if (c != cudaSuccess) e = cudaGetErrorString(c);
        rc = e.empty() ? check_device_error(ctx) : fail(ctx, LTS_ERR_DEVICE, e);
    }
    dev_free(df);
    dev_free(dt);
    dev_free(dl);
    return rc;
}

int lts_mlp_forward_device_async(lts_ctx* ctx, const uint16_t* d_features, int32_t n, float* d_out_rgb) {
    if (int r = mlp_ready(ctx)) return r;
    if (!d_features || !d_out_rgb || n < 0) return LTS_ERR_ARG;
    if (n == 0) return LTS_OK;
    const std::string e = ctx->mlp->forward(d_features, n, d_out_rgb, ctx->d_error, ctx->stream);
    return e.empty() ? LTS_OK : fail(ctx, LTS_ERR_DEVICE, e);
}

int lts_mlp_train_step_device_async(lts_ctx* ctx, const uint16_t* d_features, const float* d_targets, int32_t n,
                                    float lr, float* d_loss) {
    if (int r = mlp_ready(ctx)) return r;
    if (!d_features || !d_targets || n <= 0) return LTS_ERR_ARG;
    float* dl = d_loss ? d_loss : ctx->mlp->scratch_loss();
    const std::string e = ctx->mlp->train_step(d_features, d_targets, n, lr, dl, ctx->d_error, ctx->stream);
    return e.empty() ? LTS_OK : fail(ctx, LTS_ERR_DEVICE, e);
}

int lts_set_option(lts_ctx* ctx, const char* key, int64_t value) {
    if (!ctx || !key) return LTS_ERR_ARG;
    if (value < 0) return fail(ctx, LTS_ERR_ARG, "option value must be >= 0");
    if (!strcmp(key, "libm_double")) {
        if (ctx->device < 0) return fail(ctx, LTS_ERR_STATE, "host-only context");
        if (value > 1) return fail(ctx, LTS_ERR_ARG, "libm_double must be 0 or 1");
        CK(cudaSetDevice(ctx->device));
        const std::string e = set_libm_double((int)value);
        return e.empty() ? LTS_OK : fail(ctx, LTS_ERR_CUDA, e);
    }
    if (!strcmp(key, "debug_spin_limit")) {
        if (ctx->device < 0) return fail(ctx, LTS_ERR_STATE, "host-only context");
        if (value > (1 << 30)) return fail(ctx, LTS_ERR_ARG, "debug_spin_limit too large");
        CK(cudaSetDevice(ctx->device));
        std::string e = lbvh_set_spin_limit((int)value);
        if (e.empty()) e = mlp_set_spin_limit((int)value);
        return e.empty() ? LTS_OK : fail(ctx, LTS_ERR_CUDA, e);
    }
    if (!ctx->tracer) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    if (!strcmp(key, "wavefront_pool")) {
        if (value >= (1ll << 30)) return fail(ctx, LTS_ERR_ARG, "wavefront_pool too large");
        ctx->tracer->wf_pool = (long)value;
    } else if (!strcmp(key, "radiance_cache")) {
        if (value && (!ctx->mlp || !ctx->mlp->ready()))
            return fail(ctx, LTS_ERR_STATE, "radiance_cache needs an initialised MLP (lts_mlp_init)");
        ctx->tracer->cache_mode = value ? 1 : 0;
        ctx->tracer->mlp = ctx->mlp.get();
    } else if (!strcmp(key, "radiance_cache_unbiased_permille")) {
        if (value > 1000) return fail(ctx, LTS_ERR_ARG, "radiance_cache_unbiased_permille must be <= 1000");
        ctx->tracer->cache_unbiased_permille = (int)value;
    } else if (!strcmp(key, "radiance_cache_train_samples")) {
        if (value > (1 << 22)) return fail(ctx, LTS_ERR_ARG, "radiance_cache_train_samples too large");
        ctx->tracer->cache_train_cap = (int)value;
    } else if (!strcmp(key, "radiance_cache_train_steps")) {
        if (value < 1 || value > 64) return fail(ctx, LTS_ERR_ARG, "radiance_cache_train_steps must be 1..64");
        ctx->tracer->cache_train_steps = (int)value;
    } else if (!strcmp(key, "radiance_cache_lr_micro")) {
        ctx->tracer->cache_lr = (float)value * 1e-6f;
    } else if (!strcmp(key, "trace_blocks_per_sm")) {
        if (value > 64) return fail(ctx, LTS_ERR_ARG, "trace_blocks_per_sm must be 0..64");
        ctx->tracer->trace_blocks_per_sm = (int)value;
    } else if (!strcmp(key, "wavefront_graph")) {
        ctx->tracer->wf_graph = value ? 1 : 0;
    } else if (!strcmp(key, "film_accumulate")) {
        ctx->tracer->film_accumulate = value != 0;
    } else if (!strcmp(key, "bvh_width")) {
        if (value != 2 && value != 8) return fail(ctx, LTS_ERR_ARG, "bvh_width must be 2 or 8");
        ctx->tracer->bvh_width = (int)value;
    } else if (!strcmp(key, "render_bvh")) {
        if (value < 0 || value > 2) return fail(ctx, LTS_ERR_ARG, "render_bvh must be 0, 1 or 2");
        ctx->tracer->render_bvh = (int)value;
    } else if (!strcmp(key, "bdpt_strategy")) {
        if (value > 10000) return fail(ctx, LTS_ERR_ARG, "bdpt_strategy must be 0..9999, or 10000 for all");
        ctx->tracer->bdpt_strategy = value == 10000 ? -1 : (int)value;
    } else if (!strcmp(key, "two_level_bvh")) {
        if (value > 1) return fail(ctx, LTS_ERR_ARG, "two_level_bvh must be 0 or 1");
        ctx->tracer->two_level = (int)value;
    } else if (!strcmp(key, "radiance_cache_ema_permille")) {
        if (value > 999) return fail(ctx, LTS_ERR_ARG, "radiance_cache_ema_permille must be 0..999");
        if (!ctx->mlp) return fail(ctx, LTS_ERR_STATE, "no radiance-cache network (lts_mlp_init)");
        ctx->mlp->ema = (float)value / 1000.0f;
    } else if (!strcmp(key, "watertight")) {
        if (value > 1) return fail(ctx, LTS_ERR_ARG, "watertight must be 0 or 1");
        ctx->tracer->watertight = (int)value;
    } else if (!strcmp(key, "wavefront_sample_chunk")) {
        ctx->tracer->wf_sample_cap = (long)value;
    } else {
        return fail(ctx, LTS_ERR_ARG, std::string("unknown option ") + key);
    }
    return LTS_OK;
}

int lts_intersect(lts_ctx* ctx, const float* rays, int32_t n, int32_t any, int32_t* prim, float* t) {
    if (!ctx || n < 0 || (n > 0 && (!rays || !prim)) || (any != 0 && any != 1) || n > (1 << 28))
        return fail(ctx, LTS_ERR_ARG, "bad ray query");
    if (ctx->device == -1) return fail(ctx, LTS_ERR_STATE, "host-only context (device -1) cannot run kernels");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    CK(cudaSetDevice(ctx->device));
    if (!(ctx->bvh_is_scene && ctx->bvh_mode >= 0)) {  // the last render's BVH, else a sorted-leaf one
        const int rc = lts_bvh_build(ctx, LTS_BVH_SORTED, nullptr);
        if (rc) return rc;
    }
    if (n == 0) return LTS_OK;
    unsigned char* d = nullptr;
    CK(dev_alloc((void**)&d, 32 * (size_t)n + 8 * (size_t)n));
    float4* d_rays = reinterpret_cast<float4*>(d);
    int32_t* d_prim = reinterpret_cast<int32_t*>(d + 32 * (size_t)n);
    float* d_t = reinterpret_cast<float*>(d + 36 * (size_t)n);
    cudaError_t e = cudaMemcpyAsync(d_rays, rays, 32 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
    std::string msg = e == cudaSuccess ? ctx->tracer->intersect(*ctx->bvh, d_rays, n, any, d_prim, d_t, ctx->stream,
                                                                 ctx->d_error)
                                       : "";
    if (e == cudaSuccess && msg.empty())
        e = cudaMemcpyAsync(prim, d_prim, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && msg.empty() && t)
        e = cudaMemcpyAsync(t, d_t, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && msg.empty()) e = cudaStreamSynchronize(ctx->stream);
    dev_free(d);
    if (!msg.empty()) return fail(ctx, LTS_ERR_CUDA, msg);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "ray query");
    return check_device_error(ctx);
}

int lts_debug_kat(lts_ctx* ctx, int32_t fn, const float* in, int32_t n, float* out) {
    if (!ctx) return LTS_ERR_ARG;
    if (fn < 0 || fn >= LTS_KAT_COUNT || n < 0 || (n > 0 && (!in || !out)) || n > (1 << 24))
        return fail(ctx, LTS_ERR_ARG, "bad known-answer request");
    if (ctx->device < 0) return fail(ctx, LTS_ERR_STATE, "host-only context");
    if (n == 0) return LTS_OK;
    CK(cudaSetDevice(ctx->device));
    float* d = nullptr;
    CK(dev_alloc((void**)&d, 2 * 64 * (size_t)n));
    cudaError_t e = cudaMemcpyAsync(d, in, 64 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
    std::string msg = e == cudaSuccess ? kat_launch(fn, d, n, d + 16 * (size_t)n, ctx->stream) : "";
    if (e == cudaSuccess && msg.empty())
        e = cudaMemcpyAsync(out, d + 16 * (size_t)n, 64 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && msg.empty()) e = cudaStreamSynchronize(ctx->stream);
    dev_free(d);
    if (!msg.empty()) return fail(ctx, LTS_ERR_CUDA, msg);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "known-answer check");
    return LTS_OK;
}

int lts_scene_get_image(lts_ctx* ctx, int32_t image, int32_t level, int32_t* wh_levels, float* rgb) {
    if (!ctx || !wh_levels) return fail(ctx, LTS_ERR_ARG, "null argument");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    const std::vector<HostImage>& ims = ctx->scene.images;
    if (image < 0 || image >= (int32_t)ims.size()) return fail(ctx, LTS_ERR_ARG, "image index out of range");
    const HostImage& im = ims[(size_t)image];
    if (level < 0 || level >= im.levels) return fail(ctx, LTS_ERR_ARG, "level out of range");
    wh_levels[0] = im.w[(size_t)level];
    wh_levels[1] = im.h[(size_t)level];
    wh_levels[2] = im.levels;
    if (rgb) memcpy(rgb, im.rgb[(size_t)level].data(), im.rgb[(size_t)level].size() * sizeof(float));
    return LTS_OK;
}

int lts_debug_image_lookup(lts_ctx* ctx, int32_t image, const float* st, int32_t n, float* rgb) {
    if (!ctx) return LTS_ERR_ARG;
    if (n < 0 || (n > 0 && (!st || !rgb)) || n > (1 << 24)) return fail(ctx, LTS_ERR_ARG, "bad lookup request");
    if (ctx->device < 0) return fail(ctx, LTS_ERR_STATE, "host-only context");
    if (!ctx->loaded) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    if (image < 0 || image >= (int32_t)ctx->scene.images.size()) return fail(ctx, LTS_ERR_ARG, "image index out of range");
    if (n == 0) return LTS_OK;
    CK(cudaSetDevice(ctx->device));
    float* d = nullptr;
    CK(dev_alloc((void**)&d, 20 * (size_t)n));
    cudaError_t e = cudaMemcpyAsync(d, st, 8 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
    std::string msg = e == cudaSuccess ? ctx->tracer->image_lookup(image, d, n, d + 2 * (size_t)n, ctx->stream) : "";
    if (e == cudaSuccess && msg.empty())
        e = cudaMemcpyAsync(rgb, d + 2 * (size_t)n, 12 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && msg.empty()) e = cudaStreamSynchronize(ctx->stream);
    dev_free(d);
    if (!msg.empty()) return fail(ctx, LTS_ERR_CUDA, msg);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "image lookup");
    return LTS_OK;
}

int lts_debug_wait_timeout(lts_ctx* ctx, int32_t which) {
    if (!ctx) return LTS_ERR_ARG;
    if (which < 0 || which > 1) return fail(ctx, LTS_ERR_ARG, "which must be 0 or 1");
    if (ctx->device < 0) return fail(ctx, LTS_ERR_STATE, "host-only context");
    CK(cudaSetDevice(ctx->device));
    const std::string e = which == 0 ? lbvh_debug_wait_flag(ctx->d_error, ctx->stream)
                                     : mlp_debug_mbar_timeout(ctx->d_error, ctx->stream);
    if (!e.empty()) return fail(ctx, LTS_ERR_CUDA, e);
    return check_device_error(ctx);
}

int lts_debug_trace_sample(lts_ctx* ctx, int64_t k) {
    if (!ctx) return LTS_ERR_ARG;
    if (!ctx->tracer) return fail(ctx, LTS_ERR_STATE, "no scene loaded");
    ctx->tracer->trace_sample_ = (long)k;
    return LTS_OK;
}

int lts_debug_trace_get(lts_ctx* ctx, float* out) {
    if (!ctx || !out) return LTS_ERR_ARG;
    if (!ctx->tracer || !ctx->tracer->trace_) return fail(ctx, LTS_ERR_STATE, "no trace recorded");
    CK(cudaMemcpy(out, ctx->tracer->trace_, 64 * 16 * 4, cudaMemcpyDeviceToHost));
    return LTS_OK;
}

int lts_get_metrics(lts_ctx* ctx, lts_metrics* out) {
    if (!ctx || !out) return LTS_ERR_ARG;
    *out = ctx->metrics;
    out->device_bytes = (int64_t)dev_bytes_in_use();
    out->kernel_launches = (ctx->bvh ? ctx->bvh->launches : 0) + (ctx->tracer ? ctx->tracer->last_launches : 0);
    out->render_launches = ctx->tracer ? ctx->tracer->last_launches : 0;
    out->render_iterations = ctx->tracer ? ctx->tracer->last_iterations : 0;
    for (int k = 0; k < 6; ++k) out->render_stage_ms[k] = ctx->tracer ? ctx->tracer->last_stage_ms[k] : 0.0;
    out->cache_queries = ctx->tracer ? ctx->tracer->last_cache_queries : 0.0;
    out->cache_train_samples = ctx->tracer ? ctx->tracer->last_train_samples : 0;
    out->cache_train_loss = ctx->tracer ? ctx->tracer->last_train_loss : 0.0;
    out->cache_bias = ctx->tracer ? ctx->tracer->last_cache_bias : 0.0;
    out->cache_train_ms = ctx->tracer ? ctx->tracer->last_train_ms : 0.0;
    out->render_bvh_ms = ctx->tracer ? ctx->tracer->last_render_bvh_ms : 0.0;
    out->scene_upload_bytes = ctx->metrics.scene_upload_bytes;
    out->render_bvh_bytes = ctx->tracer ? (int64_t)ctx->tracer->render_bvh_bytes : 0;
    out->render_two_level = ctx->tracer && ctx->tracer->last_two_level ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
        out->kind_rays[k] = ctx->tracer ? ctx->tracer->last_kind_work[3 * k] : 0.0;
        out->kind_node_visits[k] = ctx->tracer ? ctx->tracer->last_kind_work[3 * k + 1] : 0.0;
        out->kind_tri_tests[k] = ctx->tracer ? ctx->tracer->last_kind_work[3 * k + 2] : 0.0;
    }
    return LTS_OK;
}

}  // extern "C"
