// Path-tracing megakernel (sm_103a): one thread per pixel, all samples and bounces, as the
// reference's PathTracingKernel (intergrators/IntegratorKernels.cu:17-23) runs
// PathTracingIntegrator::evaluate (intergrators/PathTracingIntegrator.cuh:26-109).
//
// Differences in mechanism, not in arithmetic:
//  - scene tables are SoA arrays and materials/lights are `switch`-dispatched records, so the
//    per-bounce device `new`/`free` of BSDFs and BxDFs (materials/Material.cuh:41-52) is gone;
//  - traversal reads 64-byte two-child nodes and triangles in leaf order, visits the nearer
//    child first and keeps its node stack in shared memory; the closest hit is the same as the
//    reference's left-first visit (edges are excluded by the epsilon test, so exact-t ties
//    between neighbouring triangles cannot occur);
//  - the closest-hit SurfaceInteraction is built once from the winning triangle rather than on
//    every closer hit (it is a pure function of the ray and the triangle);
//  - the film accumulates each pixel's own 2x2 splat footprint in compensated FP32 (Kahan) in
//    shared memory and flushes it once per pixel to FP64 sums; the rare wider splats go straight
//    to FP64 atomics.  The resolve divides in FP64.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "dev_common.cuh"
#include "dev_math.cuh"
#include "tracer.cuh"
#include "tracer_dev.cuh"
#include "mlp.cuh"

namespace lts {
namespace {

}  // namespace
}  // namespace lts

#include "megakernel.cuh"
#include "bdpt.cuh"

namespace lts {
namespace {

// Camera::getRender (Camera.cu:256-289): divide by the filter weight (in FP64 here), clamp at 0,
// flip rows.
// The filter weight that camera samples at unit density put on pixel x in expectation, along one
// axis: samples lie in (0, n] and reach pixels with |x - pf| <= 1, at weight table(|x - pf - 0.5|)
// (the footprint and lookup of Camera::addSample); the Gaussian table is a product of one factor
// per axis, g(ix) = table[ix] / sqrt(table[0]).  Steps of 1/16 keep every lookup constant.
__device__ __forceinline__ double film_weight_1d(const float* __restrict__ table, int x, int n) {
    const double g0 = sqrt((double)table[0]);
    double e = 0;
    for (int k = 0; k < 32; ++k) {
        const double d = -1.0 + (k + 0.5) / 16.0, pf = x + d;
        if (pf <= 0 || pf > n) continue;
        const int ix = min((int)floor(fabs(-d - 0.5) * 16), 15);
        e += (double)table[ix] / g0 / 16.0;
    }
    return e;
}

__global__ void k_resolve(const double* __restrict__ film, float* __restrict__ rgb, int W, int H,
                          const double* __restrict__ splat, double splat_scale, const float* __restrict__ table) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * H) return;
    const int i = idx % W, jj = idx / W;
    const int src = (H - 1 - jj) * W + i;
    const double w = film[4 * src + 3];
    // the bidirectional integrator's splats, per sample per pixel, over the expected filter weight
    const double sw = splat ? splat_scale / (film_weight_1d(table, i, W) * film_weight_1d(table, H - 1 - jj, H)) : 0.0;
    for (int c = 0; c < 3; ++c) {
        double v = film[4 * src + c] / w;
        if (splat) v += splat[3 * src + c] * sw;
        rgb[3 * idx + c] = fmaxf(0.0f, (float)v);
    }
}

// Scene-order triangles as 3 float4 (w = 0) from the vertex pool and the corner indices.
__global__ void k_expand_tris(const float* __restrict__ p, const int32_t* __restrict__ tri_p, int nt,
                              float4* __restrict__ prim_v) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    for (int c = 0; c < 3; ++c) {
        const int vi = tri_p[3 * t + c];
        prim_v[3 * (size_t)t + c] = make_float4(p[3 * vi], p[3 * vi + 1], p[3 * vi + 2], 0.f);
    }
}
// The same triangles as 9 floats each (the LBVH build's input).
__global__ void k_soup_from_tris(const float4* __restrict__ prim_v, int nt, float* __restrict__ soup) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    for (int c = 0; c < 3; ++c) {
        const float4 q = prim_v[3 * (size_t)t + c];
        soup[9 * (size_t)t + 3 * c] = q.x;
        soup[9 * (size_t)t + 3 * c + 1] = q.y;
        soup[9 * (size_t)t + 3 * c + 2] = q.z;
    }
}

// Shading record of each scene triangle (layout: SceneView::prim_rec) from the loader's
// per-corner indices (-1 for none): positions, uvs or the defaults (0,0) (1,0) (1,1)
// (Triangle.cu:137-143), vertex normals or zeros, and (has normals, mesh, area light, 0).
__global__ void k_build_prim_rec(const float4* __restrict__ prim_v, const int32_t* __restrict__ tri_n,
                                 const int32_t* __restrict__ tri_uv, const int32_t* __restrict__ tri_mesh,
                                 const float* __restrict__ normals, const float* __restrict__ uvs,
                                 const int32_t* __restrict__ prim_light, int nt, float4* __restrict__ rec) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int n3[3] = {tri_n[3 * t], tri_n[3 * t + 1], tri_n[3 * t + 2]};
    const int u3[3] = {tri_uv[3 * t], tri_uv[3 * t + 1], tri_uv[3 * t + 2]};
    float uv[6] = {0.f, 0.f, 1.f, 0.f, 1.f, 1.f};
    if (u3[0] >= 0) {
        for (int c = 0; c < 3; ++c) {
            uv[2 * c] = uvs[2 * u3[c]];
            uv[2 * c + 1] = uvs[2 * u3[c] + 1];
        }
    }
    float4* r = rec + 8 * (size_t)t;
    for (int c = 0; c < 3; ++c) {
        const float4 q = prim_v[3 * (size_t)t + c];
        r[c] = make_float4(q.x, q.y, q.z, uv[c]);
        r[3 + c] = n3[0] >= 0 ? make_float4(normals[3 * n3[c]], normals[3 * n3[c] + 1], normals[3 * n3[c] + 2], uv[3 + c])
                              : make_float4(0.f, 0.f, 0.f, uv[3 + c]);
    }
    reinterpret_cast<int4*>(r)[6] = make_int4(n3[0] >= 0 ? 1 : 0, tri_mesh[t], prim_light[t], 0);
    r[7] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Leaf-ordered triangles: w of the first vertex = primitive id, w of the second = the shade
// class of its material (what a closest hit records, see hit_prim / hit_class).  With `ids` the
// tree was built over the scene triangles ids[0 .. n-1] and leaf_prim indexes that list.
__global__ void k_gather_leaves(const float4* __restrict__ prim_v, const float4* __restrict__ prim_rec,
                                const DevMat* __restrict__ mats, const int32_t* __restrict__ leaf_prim, int n,
                                float4* __restrict__ leaf_v, const int32_t* __restrict__ ids = nullptr) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n) return;
    const int p = ids ? __ldg(ids + __ldg(leaf_prim + l)) : __ldg(leaf_prim + l);
    float4 a = __ldg(prim_v + 3 * p), b = __ldg(prim_v + 3 * p + 1);
    a.w = __int_as_float(p);
    const int mesh = __float_as_int(__ldg(prim_rec + 8 * (size_t)p + 6).y);
    b.w = __int_as_float(__ldg(&mats[mesh].shade_class));
    leaf_v[3 * l] = a;
    leaf_v[3 * l + 1] = b;
    leaf_v[3 * l + 2] = __ldg(prim_v + 3 * p + 2);
}

// The scene triangles ids[0 .. n-1] as 9 floats each (the top-level tree's LBVH input).
__global__ void k_soup_subset(const float4* __restrict__ prim_v, const int32_t* __restrict__ ids, int n,
                              float* __restrict__ soup) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int p = __ldg(ids + t);
    for (int c = 0; c < 3; ++c) {
        const float4 q = __ldg(prim_v + 3 * (size_t)p + c);
        soup[9 * (size_t)t + 3 * c] = q.x;
        soup[9 * (size_t)t + 3 * c + 1] = q.y;
        soup[9 * (size_t)t + 3 * c + 2] = q.z;
    }
}
// Leaf-ordered triangles of a prototype's tree from its object-space soup: w of the first vertex
// = the triangle's index in the prototype (the instance adds its first primitive and its class).
__global__ void k_gather_soup_leaves(const float* __restrict__ soup, const int32_t* __restrict__ leaf_prim, int n,
                                     float4* __restrict__ leaf_v) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n) return;
    const int p = __ldg(leaf_prim + l);
    const float* q = soup + 9 * (size_t)p;
    leaf_v[3 * (size_t)l] = make_float4(q[0], q[1], q[2], __int_as_float(p));
    leaf_v[3 * (size_t)l + 1] = make_float4(q[3], q[4], q[5], 0.f);
    leaf_v[3 * (size_t)l + 2] = make_float4(q[6], q[7], q[8], 0.f);
}
// One tree's wide nodes into the concatenated array: child and triangle indices rebased.
__global__ void k_rebase_wide(const WideNode* __restrict__ src, int count, uint32_t node_base, uint32_t tri_base,
                              WideNode* __restrict__ dst) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    WideNode w = src[k];
    w.m.x += node_base;
    w.m.y += tri_base;
    dst[k] = w;
}

// Image-texture lookups at given texture coordinates (lts_debug_image_lookup).
__global__ void k_image_lookup(const SceneView sv, int idx, const float* __restrict__ st, int n,
                               float* __restrict__ rgb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Spec c = img_lookup(sv, idx, st[2 * i], st[2 * i + 1]);
    rgb[3 * i] = c.r;
    rgb[3 * i + 1] = c.g;
    rgb[3 * i + 2] = c.b;
}

// Known-answer check: one float device function per record (LTS_KAT_* layouts of lts_capi.h).
__global__ void k_debug_kat(int fn, const float* __restrict__ in, int n, float* __restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    float a[16], o[16];
    for (int k = 0; k < 16; ++k) {
        a[k] = in[16 * (size_t)r + k];
        o[k] = 0.0f;
    }
    const V3 v0 = v3(a[0], a[1], a[2]), v3_ = v3(a[3], a[4], a[5]);
    switch (fn) {
        case LTS_KAT_QUAKE_RSQRT: o[0] = rsqrt_q3(a[0]); break;
        case LTS_KAT_FRESNEL_DIELECTRIC: o[0] = fresnel_dielectric(a[0], a[1], a[2]); break;
        case LTS_KAT_FRESNEL_CONDUCTOR: {
            const Spec F = fresnel_conductor(a[0], Spec{a[1], a[2], a[3]}, Spec{a[4], a[5], a[6]});
            o[0] = F.r, o[1] = F.g, o[2] = F.b;
            break;
        }
        case LTS_KAT_TR_D: o[0] = tr_d(v0, a[3], a[4]); break;
        case LTS_KAT_TR_LAMBDA: o[0] = tr_lambda(v0, a[3], a[4]); break;
        case LTS_KAT_TR_G1: o[0] = tr_g1(v0, a[3], a[4]); break;
        case LTS_KAT_TR_G: o[0] = tr_g(v0, v3_, a[6], a[7]); break;
        case LTS_KAT_TR_SAMPLE11: {
            real sx, sy;
            tr_sample11(a[0], a[1], a[2], sx, sy);
            o[0] = sx, o[1] = sy;
            break;
        }
        case LTS_KAT_TR_SAMPLE_WH: {
            const V3 wh = tr_sample_wh(v0, a[3], a[4], a[5], a[6]);
            o[0] = wh.x, o[1] = wh.y, o[2] = wh.z;
            break;
        }
        case LTS_KAT_TR_PDF: o[0] = tr_pdf(v0, v3_, a[6], a[7]); break;
        case LTS_KAT_MF_F:
        case LTS_KAT_MF_PDF:
        case LTS_KAT_MF_SAMPLE: {
            // the conductor lobe of MetalMaterial in its shading frame (identity transform)
            Bsdf f;
            f.lobe = LOBE_MICROFACET;
            f.type = BSDF_REFLECTION | BSDF_GLOSSY;
            f.ns = f.ng = v3(0, 0, 1);
            f.ss = v3(1, 0, 0);
            f.ts = v3(0, 1, 0);
            f.eta = 1;
            if (fn == LTS_KAT_MF_SAMPLE) {
                f.alpha = a[3];
                f.R = Spec{a[6], a[7], a[8]};
                f.eta3 = Spec{a[9], a[10], a[11]};
                f.k = Spec{a[12], a[13], a[14]};
                V3 wi = v3(0, 0, 0);
                real pdf = 0;
                uint32_t st = 0;
                const Spec v = bsdf_sample(f, v0, wi, F2{a[4], a[5]}, pdf, BSDF_ALL, st, nullptr);
                o[0] = wi.x, o[1] = wi.y, o[2] = wi.z, o[3] = v.r, o[4] = v.g, o[5] = v.b, o[6] = pdf;
            } else if (fn == LTS_KAT_MF_F) {
                f.alpha = a[6];
                f.R = Spec{a[7], a[8], a[9]};
                f.eta3 = Spec{a[10], a[11], a[12]};
                f.k = Spec{a[13], a[14], a[15]};
                const Spec v = lobe_f(f, v0, v3_);
                o[0] = v.r, o[1] = v.g, o[2] = v.b;
            } else {
                f.alpha = a[6];
                o[0] = lobe_pdf(f, v0, v3_, nullptr);
            }
            break;
        }
        case LTS_KAT_PERLIN: o[0] = perlin(a[0], a[1], a[2]); break;
        case LTS_KAT_FBM:
        case LTS_KAT_TURBULENCE: {
            const V3 dx = v3_, dy = v3(a[6], a[7], a[8]);
            o[0] = fn == LTS_KAT_FBM ? fbm(v0, dx, dy, a[9], (int)a[10], nullptr)
                                     : turbulence(v0, dx, dy, a[9], (int)a[10], nullptr);
            break;
        }
        case LTS_KAT_OFFSET_ORIGIN: {
            const V3 po = offset_origin(v0, v3_, v3(a[6], a[7], a[8]), v3(a[9], a[10], a[11]));
            o[0] = po.x, o[1] = po.y, o[2] = po.z;
            break;
        }
        default: break;
    }
    for (int k = 0; k < 16; ++k) out[16 * (size_t)r + k] = o[k];
}

// Batch ray queries: Scene::intersect (closest hit) or Scene::simpleIntersect (any hit within
// tMax), one ray per thread, through the renderer's own traversal and triangle tests.
template <bool ANY>
__global__ __launch_bounds__(kThreads) void k_intersect(const SceneView sv, int nleaf, const float4* __restrict__ rays,
                                                        int n, int32_t* __restrict__ prim, float* __restrict__ tout,
                                                        uint32_t* err) {
    __shared__ uint32_t s_stack[kStack * kThreads];
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const float4 a = rays[2 * (size_t)i], b = rays[2 * (size_t)i + 1];
    const TraceRay r = make_trace_ray(v3(a.x, a.y, a.z), v3(b.x, b.y, b.z));
    real tmax = a.w, bu = 0, bv = 0, binv = 0;
    Work wk{0u, 0u};
    const int h = sv.ninst ? traverse<ANY, true>(sv, nleaf, r, tmax, bu, bv, binv, s_stack + threadIdx.x, err, wk)
                           : traverse<ANY>(sv, nleaf, r, tmax, bu, bv, binv, s_stack + threadIdx.x, err, wk);
    if (!ANY && h >= 0) hit_exact(sv, h, r.o, r.d, tmax, bu, bv, binv);
    prim[i] = ANY ? (h > 0 ? 1 : 0) : h;
    if (tout) tout[i] = (!ANY && h >= 0) ? (float)tmax : INFINITY;
}

}  // namespace
}  // namespace lts

#include "wavefront.cuh"

namespace lts {
namespace {

static_assert(kWfBlock == kThreads, "wavefront stages share the traversal stack layout");

#define TRY(call)                                                                       \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
    } while (0)

// A device buffer of at least `bytes` in `slot` (capacity `cap`): kept when big enough, so that
// loading another scene of the same size allocates nothing.
std::string reserve_buf(void*& slot, size_t& cap, size_t bytes) {
    bytes = std::max<size_t>(bytes, 16);
    if (slot && cap >= bytes) return "";
    if (slot) dev_free(slot);
    slot = nullptr;
    cap = 0;
    TRY(dev_alloc(&slot, bytes));
    cap = bytes;
    return "";
}
template <class T, class A>
std::string upload(void*& slot, size_t& cap, const std::vector<T, A>& v, cudaStream_t s, size_t* bytes) {
    const std::string e = reserve_buf(slot, cap, sizeof(T) * v.size());
    if (!e.empty()) return e;
    if (!v.empty()) TRY(cudaMemcpyAsync(slot, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    *bytes += sizeof(T) * v.size();
    return "";
}

float quake_host(float f) { return quake_rsqrt(f); }

// The procedural textures' tables in this translation unit's device copies (once per process).
std::string ensure_texture_tables() {
    static bool consts = false;
    if (!consts) {
        unsigned char p2[512];
        const float* mc = nullptr;
        texture_tables(p2, &mc);
        TRY(cudaMemcpyToSymbol(c_perm, p2, 512));
        TRY(cudaMemcpyToSymbol(c_marble, mc, 30 * sizeof(float)));
        consts = true;
    }
    return "";
}

}  // namespace

std::string set_libm_double(int on) {
    const int v = on ? 1 : 0;
    TRY(cudaMemcpyToSymbol(c_libm_double, &v, sizeof v));
    return "";
}

std::string kat_launch(int fn, const float* d_in, int n, float* d_out, cudaStream_t s) {
    const std::string e = ensure_texture_tables();
    if (!e.empty()) return e;
    if (n > 0) k_debug_kat<<<(n + 127) / 128, 128, 0, s>>>(fn, d_in, n, d_out);
    TRY(cudaGetLastError());
    return "";
}

void Tracer::release_instanced() {
    for (void* p : {(void*)proto_soup_d_, (void*)world_ids_d_, (void*)isoup_, (void*)ileaf_, (void*)inodes_,
                    (void*)itris_, (void*)dinst_, (void*)iroot_})
        dev_free(p);
    proto_soup_d_ = nullptr;
    world_ids_d_ = nullptr;
    isoup_ = nullptr;
    ileaf_ = nullptr;
    inodes_ = nullptr;
    itris_ = nullptr;
    dinst_ = nullptr;
    iroot_ = nullptr;
    isoup_cap_ = ileaf_cap_ = inodes_cap_ = itris_cap_ = 0;
    inst_host_.clear();
    proto_off_.clear();
    proto_n_.clear();
    proto_box_.clear();
    world_n_ = 0;
    icount_ = itri_n_ = ilevels_ = 0;
    ikey_ = 0;
    two_level_ok_ = 0;
}

void Tracer::free_all() {
    release_instanced();
    for (int k = 0; k < kSceneBufs; ++k) {
        if (bufs_[k]) dev_free(bufs_[k]);
        bufs_[k] = nullptr;
        bufcap_[k] = 0;
    }
    dev_free(leaf_v_);
    leaf_v_ = nullptr;
    dev_free(film_);
    film_ = nullptr;
    dev_free(rec_L_);
    rec_L_ = nullptr;
    dev_free(rec_sig_);
    rec_sig_ = nullptr;
    dev_free(counters_);
    counters_ = nullptr;
    dev_free(rgb_);
    rgb_ = nullptr;
    dev_free(splat_);
    splat_ = nullptr;
    splat_cap_ = 0;
    splat_spp_ = 0;
    dev_free(trace_);
    trace_ = nullptr;
    dev_free(views_film_);
    views_film_ = nullptr;
    views_film_cap_ = 0;
    for (void*& p : wf_bufs_) {
        if (p) dev_free(p);
        p = nullptr;
    }
    wf_cap_ = wf_fs_cap_ = 0;
    wf_cache_cap_ = wf_train_cap_ = 0;
    film_cap_ = rec_cap_ = 0;
    leaf_serial_ = 0;
}

// Improved-Perlin permutation (Perlin 2002), and the marble colour table with one repeated
// final row, so t == 1 (sinf == 1) reads a defined entry (Procedural.cuh:286-300).
static const unsigned char kPerlinPerm[256] = {
        151, 160, 137, 91,  90,  15,  131, 13,  201, 95,  96,  53,  194, 233, 7,   225, 140, 36,  103, 30,  69,  142,
        8,   99,  37,  240, 21,  10,  23,  190, 6,   148, 247, 120, 234, 75,  0,   26,  197, 62,  94,  252, 219, 203,
        117, 35,  11,  32,  57,  177, 33,  88,  237, 149, 56,  87,  174, 20,  125, 136, 171, 168, 68,  175, 74,  165,
        71,  134, 139, 48,  27,  166, 77,  146, 158, 231, 83,  111, 229, 122, 60,  211, 133, 230, 220, 105, 92,  41,
        55,  46,  245, 40,  244, 102, 143, 54,  65,  25,  63,  161, 1,   216, 80,  73,  209, 76,  132, 187, 208, 89,
        18,  169, 200, 196, 135, 130, 116, 188, 159, 86,  164, 100, 109, 198, 173, 186, 3,   64,  52,  217, 226, 250,
        124, 123, 5,   202, 38,  147, 118, 126, 255, 82,  85,  212, 207, 206, 59,  227, 47,  16,  58,  17,  182, 189,
        28,  42,  223, 183, 170, 213, 119, 248, 152, 2,   44,  154, 163, 70,  221, 153, 101, 155, 167, 43,  172, 9,
        129, 22,  39,  253, 19,  98,  108, 110, 79,  113, 224, 232, 178, 185, 112, 104, 218, 246, 97,  228, 251, 34,
        242, 193, 238, 210, 144, 12,  191, 179, 162, 241, 81,  51,  145, 235, 249, 14,  239, 107, 49,  192, 214, 31,
        181, 199, 106, 157, 184, 84,  204, 176, 115, 121, 50,  45,  127, 4,   150, 254, 138, 236, 205, 93,  222, 114,
        67,  29,  24,  72,  243, 141, 128, 195, 78,  66,  215, 61,  156, 180};
static const float kMarble[10][3] = {{.58f, .58f, .6f}, {.58f, .58f, .6f}, {.58f, .58f, .6f}, {.5f, .5f, .5f},
                             {.6f, .59f, .58f}, {.58f, .58f, .6f}, {.58f, .58f, .6f}, {.2f, .2f, .33f},
                             {.58f, .58f, .6f}, {.58f, .58f, .6f}};

void texture_tables(unsigned char perm512[512], const float** marble30) {
    for (int k = 0; k < 512; ++k) perm512[k] = kPerlinPerm[k & 255];
    *marble30 = &kMarble[0][0];
}

Tracer::~Tracer() {
    free_all();
    if (wf_counts_host_) cudaFreeHost(wf_counts_host_);
    if (wf_ctl_host_) cudaFreeHost(wf_ctl_host_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    for (cudaEvent_t e : wf_ev_)
        if (e) cudaEventDestroy(e);
    for (int k = 0; k < kShadeClasses; ++k) {
        if (shade_streams_[k]) cudaStreamDestroy(shade_streams_[k]);
        if (shade_join_[k]) cudaEventDestroy(shade_join_[k]);
    }
    if (shade_fork_) cudaEventDestroy(shade_fork_);
}

void Tracer::drop_scene() {
    release_instanced();
    for (int k = 0; k < kSceneBufs; ++k) {
        if (bufs_[k]) dev_free(bufs_[k]);
        bufs_[k] = nullptr;
        bufcap_[k] = 0;
    }
    dev_free(leaf_v_);
    leaf_v_ = nullptr;
    leaf_n_ = 0;
    leaf_serial_ = 0;
    view_ = SceneView{};
}

std::string Tracer::upload_scene(const HostScene& sc, cudaStream_t s) {
    // buffers stay allocated (each is re-sized where it is used); the leaf-ordered triangle copy
    // belongs to the previous scene's BVH.  The view is rebuilt below: until then it names no
    // table, since a failed upload can leave any of them freed or half written.
    leaf_serial_ = 0;
    last_upload_bytes = 0;
    view_ = SceneView{};
    {
        const std::string te = ensure_texture_tables();
        if (!te.empty()) return te;
    }
    if (!ev0_) {
        TRY(cudaEventCreate(&ev0_));
        TRY(cudaEventCreate(&ev1_));
    }
    const int nt = sc.triangles();
    std::vector<DevMat> mats(sc.materials.size());
    std::vector<int> class_keys;  // shade classes: distinct (kind, Oren-Nayar, texture kinds) in order of appearance
    for (size_t m = 0; m < mats.size(); ++m) {
        const HostMaterial& h = sc.materials[m];
        mats[m].kind = h.kind;
        mats[m].extra = h.extra;
        mats[m].on_a = h.on_a;
        mats[m].on_b = h.on_b;
        for (int k = 0; k < 2; ++k) {
            mats[m].tex[k].kind = h.tex[k].kind;
            for (int q = 0; q < 4; ++q) mats[m].tex[k].v[q] = h.tex[k].v[q];
        }
        const int key = ((h.kind * 2 + (h.extra != 0.0f ? 1 : 0)) * 8 + h.tex[0].kind) * 8 + h.tex[1].kind;
        int c = -1;
        for (size_t u = 0; u < class_keys.size(); ++u)
            if (class_keys[u] == key) c = (int)u;
        if (c < 0) {
            c = (int)class_keys.size();
            class_keys.push_back(key);
        }
        mats[m].shade_class = 1 + c % (kShadeClasses - 1);
    }
    // each class's shade kernel variant: the lobes its materials can have, and whether any of
    // their textures is procedural or an image (classes alias past 15 material kinds)
    for (int c = 0; c < kShadeClasses; ++c) {
        shade_used_[c] = c == 0;
        shade_lm_[c] = 0;
        shade_tex_[c] = false;
    }
    bdpt_matte_only_ = true;
    for (size_t m = 0; m < mats.size(); ++m) {
        const HostMaterial& h = sc.materials[m];
        const int c = mats[m].shade_class;
        shade_used_[c] = true;
        const int lm = h.kind == 1 ? LM_MATTE : h.kind == 2 ? LM_GLASS : h.kind == 3 ? LM_MIRROR : h.kind == 4 ? LM_METAL : 0;
        shade_lm_[c] |= lm;
        const bool tex = h.tex[0].kind != TEX_CONSTANT || (h.kind == 2 && h.tex[1].kind != TEX_CONSTANT);
        shade_tex_[c] = shade_tex_[c] || tex;
        if ((lm & ~LM_MATTE) || tex) bdpt_matte_only_ = false;
    }
    std::vector<DevLight> lights(sc.lights.size());
    for (size_t l = 0; l < lights.size(); ++l) {
        const HostLight& h = sc.lights[l];
        lights[l].kind = h.kind;
        lights[l].prim = h.prim;
        for (int c = 0; c < 3; ++c) {
            lights[l].L[c] = h.L[c];
            lights[l].p[c] = h.p[c];
        }
        lights[l].radius = h.radius;
        lights[l].area = h.area;
    }
    std::vector<float> filt(sc.filter, sc.filter + 256);
    // vertex pools and per-corner indices go up as loaded; the per-triangle positions and the
    // shading records are expanded on the device
    std::string e;
    if (!(e = upload(bufs_[12], bufcap_[12], sc.p, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[13], bufcap_[13], sc.tri_p, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[2], bufcap_[2], sc.tri_n, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[3], bufcap_[3], sc.tri_uv, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[4], bufcap_[4], sc.n, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[5], bufcap_[5], sc.uv, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[11], bufcap_[11], sc.prim_light, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[14], bufcap_[14], sc.tri_mesh, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[6], bufcap_[6], mats, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[7], bufcap_[7], lights, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[8], bufcap_[8], sc.light_func, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[9], bufcap_[9], sc.light_cdf, s, &last_upload_bytes)).empty()) return e;
    if (!(e = upload(bufs_[10], bufcap_[10], filt, s, &last_upload_bytes)).empty()) return e;
    {  // image-texture pyramids in 4 x 4 texel blocks
        std::vector<DevImage> di(sc.images.size());
        size_t total = 0;
        for (size_t i = 0; i < sc.images.size(); ++i) {
            const HostImage& h = sc.images[i];
            if (h.levels > kImageLevels) return "bad argument: image too large";
            DevImage& d = di[i];
            memset(&d, 0, sizeof d);
            d.levels = h.levels;
            d.wrap = h.wrap;
            d.lod = h.lod;
            for (int l = 0; l < h.levels; ++l) {
                d.off[l] = (int32_t)total;
                d.w[l] = h.w[l];
                d.h[l] = h.h[l];
                total += 16 * (size_t)((h.w[l] + 3) / 4) * (size_t)((h.h[l] + 3) / 4);
            }
            if (total > (size_t)INT32_MAX) return "bad argument: images too large";
        }
        std::vector<float4> tex(total, make_float4(0.f, 0.f, 0.f, 0.f));
        for (size_t i = 0; i < sc.images.size(); ++i) {
            const HostImage& h = sc.images[i];
            for (int l = 0; l < h.levels; ++l) {
                const int w = h.w[l], bw = (w + 3) / 4;
                const float* src = h.rgb[l].data();
                for (int v = 0; v < h.h[l]; ++v)
                    for (int u = 0; u < w; ++u) {
                        const float* q = src + 3 * ((size_t)v * w + u);
                        tex[(size_t)di[i].off[l] + 16 * ((size_t)(v >> 2) * bw + (u >> 2)) + 4 * (v & 3) + (u & 3)] =
                                make_float4(q[0], q[1], q[2], 0.f);
                    }
            }
        }
        if (!(e = upload(bufs_[15], bufcap_[15], tex, s, &last_upload_bytes)).empty()) return e;
        if (!(e = upload(bufs_[16], bufcap_[16], di, s, &last_upload_bytes)).empty()) return e;
    }
    if (!(e = reserve_buf(bufs_[0], bufcap_[0], 48 * (size_t)nt)).empty()) return e;
    if (!(e = reserve_buf(bufs_[1], bufcap_[1], 128 * (size_t)nt)).empty()) return e;
    if (nt > 0) {
        k_expand_tris<<<(nt + 255) / 256, 256, 0, s>>>((const float*)bufs_[12], (const int32_t*)bufs_[13], nt,
                                                       (float4*)bufs_[0]);
        k_build_prim_rec<<<(nt + 255) / 256, 256, 0, s>>>(
            (const float4*)bufs_[0], (const int32_t*)bufs_[2], (const int32_t*)bufs_[3], (const int32_t*)bufs_[14],
            (const float*)bufs_[4], (const float*)bufs_[5], (const int32_t*)bufs_[11], nt, (float4*)bufs_[1]);
    }
    TRY(cudaGetLastError());
    if (!counters_) TRY(dev_alloc((void**)&counters_, 128));
    view_ = SceneView{};
    view_.ntri = nt;
    view_.nlight = (int)lights.size();
    view_.width = sc.width;
    view_.height = sc.height;
    view_.prim_v = (const float4*)bufs_[0];
    view_.prim_rec = (const float4*)bufs_[1];
    view_.mats = (const DevMat*)bufs_[6];
    view_.lights = (const DevLight*)bufs_[7];
    view_.light_func = (const float*)bufs_[8];
    view_.light_cdf = (const float*)bufs_[9];
    view_.light_func_int = sc.light_func_int;
    view_.filter = (const float*)bufs_[10];
    view_.img_texels = (const float4*)bufs_[15];
    view_.images = (const DevImage*)bufs_[16];
    memcpy(view_.cam, sc.cam, sizeof sc.cam);
    return capture_instances(sc, mats, s);
}

// The two-level BVH's inputs: each instance's placement, first primitive and shade class, the
// prototypes' object-space triangles and boxes, and the ids and bounds of the triangles of the
// other meshes.  The trees are built on first use (build_instanced).
std::string Tracer::capture_instances(const HostScene& sc, const std::vector<DevMat>& mats, cudaStream_t s) {
    release_instanced();
    ++upload_serial_;
    if (sc.instances.empty()) return "";
    static_assert(kMaxInstances == kMaxSceneInstances, "instance limits of the loader and the traversal agree");
    if (sc.instances.size() > (size_t)kMaxInstances) return "bad argument: too many instances";
    const int nt = sc.triangles();
    std::vector<char> instanced(sc.mesh_first_tri.size(), 0);
    for (const HostInstance& h : sc.instances) {
        InstHost ih;
        ih.mesh = h.mesh;
        ih.proto = h.proto;
        ih.prim_first = sc.mesh_first_tri[h.mesh];
        ih.ntri = sc.mesh_tri_count[h.mesh];
        ih.cls = mats[h.mesh].shade_class;
        for (int c = 0; c < 3; ++c) ih.t[c] = h.t[c];
        ih.s = h.s;
        if (ih.ntri * 9 != (int)sc.proto_soup[h.proto].size()) return "bad argument: instance and prototype differ";
        inst_host_.push_back(ih);
        instanced[h.mesh] = 1;
    }
    std::vector<float> all;
    for (const std::vector<float>& soup : sc.proto_soup) {
        proto_off_.push_back(all.size() / 9);
        proto_n_.push_back((int)(soup.size() / 9));
        float b[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        for (size_t k = 0; k < soup.size(); ++k) {
            b[k % 3] = std::min(b[k % 3], soup[k]);
            b[3 + k % 3] = std::max(b[3 + k % 3], soup[k]);
        }
        proto_box_.insert(proto_box_.end(), b, b + 6);
        all.insert(all.end(), soup.begin(), soup.end());
    }
    std::vector<int32_t> ids;
    for (float& v : world_box_) v = 0;
    float* wb = world_box_;
    wb[0] = wb[1] = wb[2] = INFINITY;
    wb[3] = wb[4] = wb[5] = -INFINITY;
    for (int t = 0; t < nt; ++t) {
        if (instanced[sc.tri_mesh[t]]) continue;
        ids.push_back(t);
        for (int c = 0; c < 3; ++c)
            for (int a = 0; a < 3; ++a) {
                const float v = sc.p[3 * (size_t)sc.tri_p[3 * (size_t)t + c] + a];
                wb[a] = std::min(wb[a], v);
                wb[3 + a] = std::max(wb[3 + a], v);
            }
    }
    world_n_ = (int)ids.size();
    two_level_ok_ = world_n_ >= 2;
    for (int n : proto_n_) two_level_ok_ = two_level_ok_ && n >= 2;
    if (!two_level_ok_) return "";  // rendered through the flat tree
    void* p = nullptr;
    size_t cap = 0;
    std::string e = upload(p, cap, all, s, &last_upload_bytes);
    proto_soup_d_ = (float*)p;
    if (!e.empty()) return e;
    p = nullptr;
    cap = 0;
    e = upload(p, cap, ids, s, &last_upload_bytes);
    world_ids_d_ = (int32_t*)p;
    return e;
}

std::string Tracer::build_instanced(uint64_t key, cudaStream_t s, uint32_t* d_err) {
    ikey_ = 0;
    const int np = (int)proto_n_.size(), ni = (int)inst_host_.size();
    size_t tot_tris = (size_t)world_n_, tot_nodes = (size_t)world_n_ - 1, max_n = (size_t)world_n_;
    for (int n : proto_n_) {
        tot_tris += (size_t)n;
        tot_nodes += (size_t)n - 1;
        max_n = std::max(max_n, (size_t)n);
    }
    std::string e;
    void* p;
    p = isoup_;
    if (!(e = reserve_buf(p, isoup_cap_, 36 * max_n)).empty()) return e;
    isoup_ = (float*)p;
    p = ileaf_;
    if (!(e = reserve_buf(p, ileaf_cap_, 48 * max_n)).empty()) return e;
    ileaf_ = (float4*)p;
    p = inodes_;
    if (!(e = reserve_buf(p, inodes_cap_, sizeof(WideNode) * tot_nodes)).empty()) return e;
    inodes_ = (WideNode*)p;
    p = itris_;
    if (!(e = reserve_buf(p, itris_cap_, 48 * tot_tris)).empty()) return e;
    itris_ = (float4*)p;
    if (!dinst_) TRY(dev_alloc((void**)&dinst_, sizeof(DevInstance) * kMaxInstances));
    if (!iroot_) TRY(dev_alloc((void**)&iroot_, 6 * sizeof(float)));
    const auto t0 = std::chrono::steady_clock::now();
    uint32_t node_base = 0, tri_base = 0;
    int levels = 0;
    std::vector<int> roots((size_t)np, 0);
    for (int tree = -1; tree < np; ++tree) {  // the top level, then one tree per prototype
        const int n = tree < 0 ? world_n_ : proto_n_[tree];
        const float* soup = tree < 0 ? isoup_ : proto_soup_d_ + 9 * proto_off_[tree];
        if (tree < 0) k_soup_subset<<<(n + 255) / 256, 256, 0, s>>>(view_.prim_v, world_ids_d_, n, isoup_);
        if (!(e = ilbvh_.build(soup, n, BVH_MODE_SORTED, -1, s, d_err)).empty()) return e;
        if (tree < 0)
            k_gather_leaves<<<(n + 255) / 256, 256, 0, s>>>(view_.prim_v, view_.prim_rec, view_.mats,
                                                            ilbvh_.leaf_prim, n, ileaf_, world_ids_d_);
        else
            k_gather_soup_leaves<<<(n + 255) / 256, 256, 0, s>>>(soup, ilbvh_.leaf_prim, n, ileaf_);
        TRY(cudaGetLastError());
        if (!(e = iploc_.build(ileaf_, n, s, d_err)).empty()) return e;
        if (!(e = iwide_.build(iploc_.nodes, render_bvh == 1 ? iploc_.sah : nullptr, n, key, ileaf_, s, d_err)).empty())
            return e;
        if ((size_t)node_base + iwide_.count > tot_nodes) return "two-level BVH: node count out of range";
        k_rebase_wide<<<(iwide_.count + 127) / 128, 128, 0, s>>>(iwide_.nodes, iwide_.count, node_base, tri_base,
                                                                inodes_ + node_base);
        TRY(cudaGetLastError());
        TRY(cudaMemcpyAsync(itris_ + 3 * (size_t)tri_base, iwide_.tris, 48 * (size_t)n, cudaMemcpyDeviceToDevice, s));
        if (tree >= 0) roots[tree] = (int)node_base;
        node_base += (uint32_t)iwide_.count;
        tri_base += (uint32_t)n;
        levels = std::max(levels, iwide_.levels);
    }
    // the instance table; world boxes padded by 1e-5 of their largest coordinate, so that they
    // hold every point the object-space tests can hit after the ray's transform has rounded
    std::vector<DevInstance> di((size_t)ni);
    float root[6];
    for (int a = 0; a < 6; ++a) root[a] = world_box_[a];
    for (int i = 0; i < ni; ++i) {
        const InstHost& h = inst_host_[i];
        const float* b = &proto_box_[6 * (size_t)h.proto];
        float lo[3], hi[3], m = 0;
        for (int a = 0; a < 3; ++a) {
            lo[a] = b[a] * h.s + h.t[a];
            hi[a] = b[3 + a] * h.s + h.t[a];
            m = std::max(m, std::max(std::fabs(lo[a]), std::fabs(hi[a])));
        }
        const float pad = 1e-5f * m + 1e-30f;
        for (int a = 0; a < 3; ++a) {
            lo[a] -= pad;
            hi[a] += pad;
            root[a] = std::min(root[a], lo[a]);
            root[3 + a] = std::max(root[3 + a], hi[a]);
        }
        DevInstance& d = di[i];
        d.xf = make_float4(h.t[0], h.t[1], h.t[2], 1.0f / h.s);
        d.wlo = make_float4(lo[0], lo[1], lo[2], 0.f);
        d.whi = make_float4(hi[0], hi[1], hi[2], 0.f);
        d.olo = make_float4(b[0], b[1], b[2], 0.f);
        d.ohi = make_float4(b[3], b[4], b[5], 0.f);
        d.ref = make_int4(roots[h.proto], h.prim_first, h.cls, 0);
    }
    TRY(cudaMemcpyAsync(dinst_, di.data(), sizeof(DevInstance) * (size_t)ni, cudaMemcpyHostToDevice, s));
    TRY(cudaMemcpyAsync(iroot_, root, sizeof root, cudaMemcpyHostToDevice, s));
    TRY(cudaStreamSynchronize(s));
    last_render_bvh_ms = (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    icount_ = (int)node_base;
    itri_n_ = (int)tri_base;
    ilevels_ = levels;
    ikey_ = key;
    return "";
}

std::string Tracer::image_lookup(int idx, const float* d_st, int n, float* d_rgb, cudaStream_t s) {
    if (!view_.images) return "no scene on the device";
    if (n > 0) k_image_lookup<<<(n + 127) / 128, 128, 0, s>>>(view_, idx, d_st, n, d_rgb);
    TRY(cudaGetLastError());
    return "";
}

std::string Tracer::triangle_soup(float* d_soup, cudaStream_t s) const {
    if (view_.ntri > 0)
        k_soup_from_tris<<<(view_.ntri + 255) / 256, 256, 0, s>>>(view_.prim_v, view_.ntri, d_soup);
    TRY(cudaGetLastError());
    return "";
}

// The scene view with the traversal structures of `bvh`: the leaf-ordered triangles and, with
// bvh_width 8, the 8-wide compressed BVH collapsed from the binary tree (both kept while the
// tree is unchanged); the wide tree is used when its depth fits the traversal stack.
std::string Tracer::traversal_view(const Lbvh& bvh, cudaStream_t s, uint32_t* d_err, SceneView* sv) {
    // leaf-ordered triangles for traversal
    if (leaf_serial_ != bvh.serial || leaf_n_ != bvh.n) {
        dev_free(leaf_v_);
        leaf_v_ = nullptr;
        TRY(dev_alloc((void**)&leaf_v_, sizeof(float4) * 3 * (size_t)bvh.n));
        k_gather_leaves<<<(bvh.n + 255) / 256, 256, 0, s>>>(view_.prim_v, view_.prim_rec, view_.mats, bvh.leaf_prim,
                                                            bvh.n, leaf_v_);
        leaf_serial_ = bvh.serial;
        leaf_n_ = bvh.n;
    }
    // 8-wide compressed BVH collapsed from the binary tree (kept while the tree is unchanged); it
    // is used when the wide tree's depth fits the traversal stack.  Scenes with instanced meshes
    // use the two-level tree instead (built once per scene upload and render-tree choice).
    bool use_wide = bvh_width == 8 && bvh.n >= 2;
    bool use_inst = false;
    if (use_wide && render_bvh != 0 && two_level && two_level_ok_) {
        const uint64_t ikey = 4 * upload_serial_ + (uint64_t)render_bvh;
        if (ikey_ != ikey) {
            const std::string e = build_instanced(ikey, s, d_err);
            if (!e.empty()) return e;
        }
        use_inst = ilevels_ - 1 <= kStack / 2;
    }
    const uint64_t wide_key = 4 * bvh.serial + (uint64_t)render_bvh;  // the binary tree and collapse it came from
    if (use_wide && !use_inst && wide_.serial != wide_key) {
        std::string e;
        if (render_bvh) {
            e = ploc_.build(leaf_v_, bvh.n, s, d_err);
            if (e.empty())
                e = wide_.build(ploc_.nodes, render_bvh == 1 ? ploc_.sah : nullptr, bvh.n, wide_key, leaf_v_, s,
                                d_err);
            last_render_bvh_ms = ploc_.build_ms + wide_.build_ms;
        } else {
            e = wide_.build(bvh.nodes, nullptr, bvh.n, wide_key, leaf_v_, s, d_err);
            last_render_bvh_ms = wide_.build_ms;
        }
        if (!e.empty()) return e;
    }
    if (use_wide && !use_inst && wide_.levels - 1 > kStack / 2) use_wide = false;
    *sv = view_;
    sv->leaf_v = leaf_v_;
    sv->nodes = bvh.nodes;
    sv->root_bounds = use_inst ? iroot_ : bvh.root_bounds;
    sv->wnodes = use_inst ? inodes_ : (use_wide ? wide_.nodes : nullptr);
    sv->wtris = use_inst ? itris_ : (use_wide ? wide_.tris : nullptr);
    sv->wcount = use_inst ? icount_ : (use_wide ? wide_.count : 0);
    sv->wtri_count = use_inst ? itri_n_ : (use_wide ? bvh.n : 0);
    sv->inst = use_inst ? dinst_ : nullptr;
    sv->ninst = use_inst ? (int32_t)inst_host_.size() : 0;
    sv->watertight = watertight;
    last_wide = use_wide;
    last_two_level = use_inst;
    render_bvh_bytes = use_inst ? sizeof(WideNode) * (size_t)icount_ + 48 * (size_t)itri_n_ +
                                          sizeof(DevInstance) * inst_host_.size()
                                : use_wide ? sizeof(WideNode) * (size_t)wide_.count + 48 * (size_t)bvh.n
                                           : sizeof(BvhNode) * (size_t)(bvh.n - 1) + 48 * (size_t)bvh.n;
    return "";
}

std::string Tracer::intersect(const Lbvh& bvh, const float4* d_rays, int n, int any, int32_t* d_prim, float* d_t,
                              cudaStream_t s, uint32_t* d_err) {
    if (bvh.n != view_.ntri) return "bad argument: BVH does not match the scene";
    SceneView sv;
    const std::string e = traversal_view(bvh, s, d_err, &sv);
    if (!e.empty()) return e;
    if (n <= 0) return "";
    const unsigned grid = (unsigned)((n + kThreads - 1) / kThreads);
    if (any)
        k_intersect<true><<<grid, kThreads, 0, s>>>(sv, bvh.n, d_rays, n, d_prim, d_t, d_err);
    else
        k_intersect<false><<<grid, kThreads, 0, s>>>(sv, bvh.n, d_rays, n, d_prim, d_t, d_err);
    TRY(cudaGetLastError());
    return "";
}

std::string Tracer::prepare(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, cudaStream_t s,
                            uint32_t* d_err, RenderParams* rp, SceneView* sv, long* crop_samples) {
    if (d.spp < 1 || d.max_bounce < 0) return "bad argument: spp must be >= 1 and max_bounce >= 0";
    if (d.integrator != LTS_INTEGRATOR_MEGAKERNEL && d.integrator != LTS_INTEGRATOR_WAVEFRONT &&
        d.integrator != LTS_INTEGRATOR_FP64 && d.integrator != LTS_INTEGRATOR_BDPT)
        return "bad argument: unknown integrator";
    if (d.integrator == LTS_INTEGRATOR_BDPT) {
        if (d.record_samples) return "bad argument: the bidirectional integrator has no record mode";
        if (d.max_bounce > kBdptMaxBounce) return "bad argument: the bidirectional integrator takes max_bounce <= 8";
        if (sc.lights.empty()) return "bad argument: the bidirectional integrator needs a light";
        for (const HostLight& l : sc.lights)
            if (l.kind == LIGHT_INFINITE) return "unsupported: the bidirectional integrator takes area and point lights";
    }
    if (d.integrator == LTS_INTEGRATOR_WAVEFRONT && d.max_bounce < 1)
        return "bad argument: the wavefront integrator needs max_bounce >= 1";
    int x0 = d.x0, y0 = d.y0, x1 = d.x1, y1 = d.y1;
    if (x1 == 0 && y1 == 0) {
        x0 = y0 = 0;
        x1 = sc.width;
        y1 = sc.height;
    }
    if (x0 < 0 || y0 < 0 || x1 > sc.width || y1 > sc.height || x0 >= x1 || y0 >= y1) return "bad argument: crop";
    if (bvh.n != sc.triangles()) return "bad argument: BVH does not match the scene";
    std::string te = traversal_view(bvh, s, d_err, sv);
    if (!te.empty()) return te;
    const size_t film_bytes = 32 * (size_t)sc.width * sc.height;
    if (film_cap_ < film_bytes) {
        dev_free(film_);
        film_ = nullptr;
        dev_free(rgb_);
        rgb_ = nullptr;
        TRY(dev_alloc((void**)&film_, film_bytes));
        TRY(dev_alloc((void**)&rgb_, 12 * (size_t)sc.width * sc.height));
        film_cap_ = film_bytes;
    }
    if (!film_accumulate) TRY(cudaMemsetAsync(film_, 0, film_bytes, s));
    // light-to-camera splats of the bidirectional integrator, scaled by 1 / (samples so far)
    if (!film_accumulate) splat_spp_ = 0;
    if (d.integrator == LTS_INTEGRATOR_BDPT) {
        const size_t sb = 24 * (size_t)sc.width * sc.height;
        if (splat_cap_ < sb) {
            dev_free(splat_);
            splat_ = nullptr;
            TRY(dev_alloc((void**)&splat_, sb));
            splat_cap_ = sb;
            TRY(cudaMemsetAsync(splat_, 0, sb, s));
        }
        if (splat_spp_ == 0) TRY(cudaMemsetAsync(splat_, 0, sb, s));
        splat_spp_ += d.spp;
    } else if (splat_spp_ > 0 && !film_accumulate) {
        splat_spp_ = 0;
    }
    TRY(cudaMemsetAsync(counters_, 0, 128, s));
    const long ns = (long)(x1 - x0) * (y1 - y0) * d.spp;
    *crop_samples = ns;
    if (d.record_samples) {
        if (rec_cap_ < (size_t)ns) {
            dev_free(rec_L_);
            dev_free(rec_sig_);
            rec_L_ = nullptr;
            rec_sig_ = nullptr;
            TRY(dev_alloc((void**)&rec_L_, 12 * (size_t)ns));
            TRY(dev_alloc((void**)&rec_sig_, 8 * (size_t)ns));
            rec_cap_ = (size_t)ns;
        }
    }
    *rp = RenderParams{};
    rp->spp = d.spp;
    rp->max_bounce = d.max_bounce;
    rp->rr_start = d.rr_start;
    rp->seed = d.seed;
    rp->x0 = x0;
    rp->y0 = y0;
    rp->x1 = x1;
    rp->y1 = y1;
    rp->spp_scale = quake_host((float)d.spp);
    rp->film = film_;
    rp->sample_L = d.record_samples ? rec_L_ : nullptr;
    rp->sample_sig = d.record_samples ? rec_sig_ : nullptr;
    rp->counters = counters_;
    rp->err = d_err;
    rp->trace = nullptr;
    rp->trace_sample = -1;
    if (d.record_samples && trace_sample_ >= 0) {
        if (!trace_) TRY(dev_alloc((void**)&trace_, 64 * 16 * 4));
        TRY(cudaMemsetAsync(trace_, 0, 64 * 16 * 4, s));
        rp->trace = trace_;
        rp->trace_sample = trace_sample_;
    }
    return "";
}

std::string Tracer::render_async(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, cudaStream_t s,
                                 uint32_t* d_err) {
    RenderParams rp;
    SceneView sv;
    long ns = 0;
    std::string e = prepare(sc, bvh, d, s, d_err, &rp, &sv, &ns);
    if (!e.empty()) return e;
    last_paths = (double)ns;
    if (d.integrator == LTS_INTEGRATOR_WAVEFRONT) return render_wavefront(sc, bvh, d, s, d_err, rp, sv, ns);
    const dim3 block(kBX, kBY);
    const dim3 grid((rp.x1 - rp.x0 + kBX - 1) / kBX, (rp.y1 - rp.y0 + kBY - 1) / kBY);
    TRY(cudaEventRecord(ev0_, s));
    if (d.integrator == LTS_INTEGRATOR_FP64) {
        e = render64_launch(sv, rp, bvh.n, d.record_samples != 0, s);
        if (!e.empty()) return e;
    } else if (d.integrator == LTS_INTEGRATOR_BDPT) {
        // one thread per pixel and sample slice: enough blocks for every SM to hold its resident
        // ones about four times over (a small film alone would leave most SMs idle)
        int dev = 0, sms = 0;
        TRY(cudaGetDevice(&dev));
        TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const long want = 4L * LTS_BDPT_MIN_BLOCKS * sms, have = (long)grid.x * grid.y;
        const dim3 gridz(grid.x, grid.y, (unsigned)std::max(1L, std::min<long>(rp.spp, (want + have - 1) / have)));
        // compiled for the lobes the scene has: Lambertian / Oren-Nayar alone, or every lobe
        if (bdpt_matte_only_) k_bdpt<LM_MATTE, false><<<gridz, block, 0, s>>>(sv, rp, bvh.n, splat_, bdpt_strategy);
        else k_bdpt<LM_ALL, true><<<gridz, block, 0, s>>>(sv, rp, bvh.n, splat_, bdpt_strategy);
    } else if (d.record_samples) {
        k_pathtrace<true><<<grid, block, 0, s>>>(sv, rp, bvh.n);
    } else {
        k_pathtrace<false><<<grid, block, 0, s>>>(sv, rp, bvh.n);
    }
    TRY(cudaEventRecord(ev1_, s));
    TRY(cudaGetLastError());
    last_launches = 1;
    last_iterations = 1;
    for (double& x : last_stage_ms) x = 0;
    last_paths = (double)ns;
    return "";
}

std::string Tracer::render_wavefront(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, cudaStream_t s,
                                     uint32_t* d_err, const RenderParams& rp, const SceneView& sv, long total) {
    (void)sc;
    (void)total;
    // Samples per pixel are rendered in chunks whose finished samples fit the sample buffer; the
    // path pool drains at the end of each chunk and the chunk is gathered into the film.  Each
    // chunk is a batch of one view slice.
    const long npix = (long)(rp.x1 - rp.x0) * (rp.y1 - rp.y0);
    const long cap = wf_sample_cap > 0 ? wf_sample_cap : (1l << 27);
    const int chunk = (int)std::max<long>(1, std::min<long>(d.spp, cap / npix));
    if (npix * chunk >= (1l << 31)) return "wavefront: crop too large for one sample chunk";
    std::vector<std::vector<WfView>> batches;
    for (int s0 = 0; s0 < d.spp; s0 += chunk) {
        WfView v{};
        for (int k = 0; k < 12; ++k) v.cam[k] = sv.cam[k];
        v.W = sv.width;
        v.H = sv.height;
        v.x0 = rp.x0; v.y0 = rp.y0; v.x1 = rp.x1; v.y1 = rp.y1;
        v.spp = d.spp;
        v.s_first = s0;
        v.nsc = std::min(chunk, d.spp - s0);
        v.seed = rp.seed;
        v.spp_scale = rp.spp_scale;
        v.base = 0;
        v.npix = npix;
        v.film_off = 0;
        batches.push_back({v});
    }
    return run_wavefront(batches, bvh, s, d_err, rp, sv);
}

// Automatic path-pool capacity: large enough to hold a whole batch's paths (then every path of
// an iteration is at the same bounce, and a render takes about max_bounce + 1 full iterations
// instead of many partly drained ones: 2^21 slots gave 355 Mpaths/s on the 1024x1024x64 spp
// render, 2^24 398, all 2^26 paths 421), up to kPoolMax slots and a quarter of the device memory
// that is free or already held by the pool.
long Tracer::auto_pool(bool cache) const {
    constexpr long kPoolMax = 1l << 26, kPoolMin = 1l << 21;
    const size_t per_slot = kPoolSlotBytes + (cache ? kCacheSlotBytes : 0);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return kPoolMin;
    }
    const size_t avail = free_b + (size_t)wf_cap_ * kPoolSlotBytes + (size_t)wf_cache_cap_ * kCacheSlotBytes;
    long cap = kPoolMax;
    while (cap > kPoolMin && (size_t)cap * per_slot > avail / 4) cap >>= 1;
    return cap;
}

// The wavefront loop over batches of view slices (see WfView): per batch, the path pool runs
// until it drains, then every slice is gathered into its view's film.
// The shade launch of one class: the kernel variant compiled for its lobes and textures
// (record mode, the parity runs, uses the general one).
static std::string launch_shade(bool record, int cls, int lm, bool tex, unsigned grid, const SceneView& sv,
                                const RenderParams& rp, const WfState& st, int pool, cudaStream_t s) {
    if (record) {
        k_wf_shade<true, LM_ALL, true><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
    } else if (cls == 0) {
        k_wf_shade<false, 0, false><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
    } else if (lm == LM_MATTE) {
        if (tex) k_wf_shade<false, LM_MATTE, true><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
        else k_wf_shade<false, LM_MATTE, false><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
    } else if (lm == LM_GLASS) {
        if (tex) k_wf_shade<false, LM_GLASS, true><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
        else k_wf_shade<false, LM_GLASS, false><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
    } else if (lm == LM_MIRROR) {
        if (tex) k_wf_shade<false, LM_MIRROR, true><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
        else k_wf_shade<false, LM_MIRROR, false><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
    } else if (lm == LM_METAL) {
        if (tex) k_wf_shade<false, LM_METAL, true><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
        else k_wf_shade<false, LM_METAL, false><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
    } else {
        k_wf_shade<false, LM_ALL, true><<<grid, kWfBlock, 0, s>>>(sv, rp, st, pool, cls);
    }
    TRY(cudaGetLastError());
    return "";
}

std::string Tracer::run_wavefront(const std::vector<std::vector<WfView>>& batches, const Lbvh& bvh, cudaStream_t s,
                                  uint32_t* d_err, const RenderParams& rp, const SceneView& sv) {
    (void)d_err;
    long batch_max = 1;
    for (const auto& bt : batches) {
        long t = 0;
        for (const WfView& v : bt) t += v.npix * v.nsc;
        batch_max = std::max(batch_max, t);
        if (bt.size() > (size_t)kMaxViews) return "wavefront: too many views in one batch";
    }
    if (batch_max >= (1l << 31)) return "wavefront: batch too large";
    const long chunk_total = batch_max;
    const bool cache = cache_mode != 0 && mlp != nullptr && mlp->ready();
    const long P = std::max<long>(1, std::min<long>(chunk_total, wf_pool > 0 ? wf_pool : auto_pool(cache)));
    WfState st{};
    if (wf_cap_ < P) {
        for (int k : {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26,
                      27, 28, 29, 30, 31, 32, 35, 45}) {
            if (wf_bufs_[k]) dev_free(wf_bufs_[k]);
            wf_bufs_[k] = nullptr;
        }
        wf_cap_ = 0;
        const size_t n = (size_t)P;
        const size_t sizes[] = {4 * n, 4 * n, 4 * n, 4 * n, 4 * n, 4 * n,                       // pix smp draw flags pend vis
                                16 * n, 16 * n, 16 * n, 16 * n, 8 * n, 8 * n, 4 * n, 16 * n,  // ro rd beta L pf sig hprim huvi
                                16 * n, 16 * n, 16 * n, 16 * n, 16 * n, 16 * n, 16 * n, 16 * n, 16 * n,  // sh_* mis_* ld nee
                                8 * n, 8 * n, 4 * n, 4 * n, 4 * n, 4 * n, 4 * n, 4 * n, 256,  // ev mis_hit queues counts
                                4 * n};                                                           // wid
        for (size_t k = 0; k < sizeof sizes / sizeof sizes[0]; ++k) TRY(dev_alloc(&wf_bufs_[k], sizes[k]));
        TRY(dev_alloc(&wf_bufs_[35], 4 * (size_t)kShadeClasses * n));  // class-grouped shade lists
        TRY(dev_alloc(&wf_bufs_[45], 4 * n));                             // view slice of each path
        wf_cap_ = P;
    }
    if (wf_fs_cap_ < chunk_total) {
        dev_free(wf_bufs_[33]);
        dev_free(wf_bufs_[34]);
        wf_bufs_[33] = wf_bufs_[34] = nullptr;
        wf_fs_cap_ = 0;
        TRY(dev_alloc(&wf_bufs_[33], 16 * (size_t)chunk_total));
        TRY(dev_alloc(&wf_bufs_[34], 4 * (size_t)chunk_total));
        wf_fs_cap_ = chunk_total;
    }
    if (!wf_counts_host_) TRY(cudaMallocHost((void**)&wf_counts_host_, 64));
    void** b = wf_bufs_;
    st.pix = (int32_t*)b[0]; st.smp = (int32_t*)b[1]; st.draw = (uint32_t*)b[2]; st.flags = (uint32_t*)b[3];
    st.pend = (uint32_t*)b[4]; st.vis = (uint32_t*)b[5];
    st.ro = (float4*)b[6]; st.rd = (float4*)b[7]; st.beta = (float4*)b[8]; st.L = (float4*)b[9];
    st.pf = (float2*)b[10]; st.sig = (uint64_t*)b[11]; st.hprim = (int32_t*)b[12]; st.huvi = (float4*)b[13];
    st.sh_o = (float4*)b[14]; st.sh_d = (float4*)b[15]; st.sh_c = (float4*)b[16];
    st.mis_o = (float4*)b[17]; st.mis_d = (float4*)b[18]; st.mis_fv = (float4*)b[19]; st.mis_x = (float4*)b[20];
    st.ld_mis = (float4*)b[21]; st.nee_beta = (float4*)b[22];
    st.ev_mis = (uint64_t*)b[23]; st.ev_main = (uint64_t*)b[24]; st.mis_hit = (int32_t*)b[25];
    st.q_a = (int32_t*)b[26]; st.q_b = (int32_t*)b[27]; st.q_shadow = (int32_t*)b[28]; st.q_mis = (int32_t*)b[29];
    st.q_free = (int32_t*)b[30]; st.counts = (uint32_t*)b[31]; st.wid = (int32_t*)b[32];
    st.fs_L = (float4*)b[33]; st.fs_y = (float*)b[34];
    st.q_cls = (int32_t*)b[35];
    st.view = (int32_t*)b[45];
    if (!wf_bufs_[46]) TRY(dev_alloc(&wf_bufs_[46], sizeof(WfView) * kMaxViews));
    st.views = (const WfView*)b[46];
    // radiance cache buffers (allocated on first use with the cache on)
    st.cache = cache ? 1 : 0;
    st.unb_permille = (uint32_t)std::max(0, std::min(1000, cache_unbiased_permille));
    st.tr_cap = (uint32_t)std::max(0, cache_train_cap);
    {
        // acceptance rate of the training-record coin: the previous render's eligible vertices
        // per path (before any render: every unbiased path), scaled so that ~90 % of tr_cap fills
        long paths = 0;
        for (const auto& bt : batches)
            for (const WfView& v : bt) paths += v.npix * v.nsc;
        cache_render_paths_ = (double)paths;
        const double rate = cache_eligible_rate_ >= 0 ? cache_eligible_rate_ : st.unb_permille / 1000.0;
        const double expect = rate * (double)paths, keep = 0.9 * (double)st.tr_cap;
        st.tr_accept = expect <= keep ? 0xFFFFFFFFu : (uint32_t)std::min(4294967295.0, 4294967296.0 * keep / expect);
    }
    st.bounds = bvh.root_bounds;  // the cache's position features: the scene's bounds in every BVH mode
    if (cache) {
        if (wf_cache_cap_ < P || wf_train_cap_ < (long)st.tr_cap) {
            for (int k = 36; k < 45; ++k) {
                dev_free(wf_bufs_[k]);
                wf_bufs_[k] = nullptr;
            }
            wf_cache_cap_ = wf_train_cap_ = 0;
            const size_t n = (size_t)P, m = std::max<size_t>(1, st.tr_cap);
            const size_t sz[7] = {2 * 96 * n, 16 * n, 4 * n, 16 * n, 16 * n, 4 * n, 2 * 96 * m};
            for (int k = 0; k < 7; ++k) TRY(dev_alloc(&wf_bufs_[36 + k], sz[k]));
            TRY(dev_alloc(&wf_bufs_[43], 12 * m + 16));  // targets, then the loss word
            TRY(dev_alloc(&wf_bufs_[44], 12 * m));       // the cache's predictions for the records
            wf_cache_cap_ = P;
            wf_train_cap_ = (long)st.tr_cap;
        }
        st.feat = (uint16_t*)b[36]; st.cache_L = (float4*)b[37]; st.q_cache = (int32_t*)b[38];
        st.tr_beta = (float4*)b[39]; st.tr_L0 = (float4*)b[40]; st.tr_idx = (int32_t*)b[41];
        st.tr_feat = (uint16_t*)b[42]; st.tr_target = (float*)b[43];
    }
    last_cache_queries = 0;
    last_train_samples = 0;
    if (rp.sample_sig) {
        TRY(cudaMemsetAsync(st.ev_mis, 0, 8 * (size_t)P, s));
        TRY(cudaMemsetAsync(st.ev_main, 0, 8 * (size_t)P, s));
    }
    auto blocks = [](long n) { return (unsigned)((n + kWfBlock - 1) / kWfBlock); };
    TRY(cudaEventRecord(ev0_, s));
    TRY(cudaMemsetAsync(st.counts, 0, 128, s));
    k_wf_init_free<<<blocks(P), kWfBlock, 0, s>>>(st.q_free, st.pix, st.counts, (int)P);  // every slot free
    TRY(cudaMemsetAsync(st.counts + 32, 0, 8, s));  // training records and eligible vertices of this render
    const bool rec = rp.sample_sig != nullptr;
    const bool wide = sv.wnodes != nullptr;
    int iters = 0, launches = 1;
    for (cudaEvent_t& e : wf_ev_)
        if (!e) TRY(cudaEventCreate(&e));
    for (double& x : last_stage_ms) x = 0;
    // persistent trace grid: every SM filled with as many blocks as stay resident
    if (wf_trace_blocks_[0] == 0) {
        int dev = 0, sms = 0, per_w = 0, per_b = 0, per_i = 0;
        TRY(cudaGetDevice(&dev));
        TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_w, k_wf_trace<true>, kWfBlock, 0));
        TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_b, k_wf_trace<false>, kWfBlock, 0));
        TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_i, k_wf_trace<true, true>, kWfBlock, 0));
        wf_trace_blocks_[0] = (unsigned)std::max(1, per_w * sms);
        wf_trace_blocks_[1] = (unsigned)std::max(1, per_b * sms);
        wf_trace_blocks_[2] = (unsigned)std::max(1, per_i * sms);
        wf_sms_ = (unsigned)sms;
        int per_s = 0;
        TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_s, k_wf_shade<false, LM_ALL, true>, kWfBlock, 0));
        shade_grid_ = (unsigned)std::max(1, per_s * sms * 2);
        for (int k = 0; k < kShadeClasses; ++k) {
            TRY(cudaStreamCreateWithFlags(&shade_streams_[k], cudaStreamNonBlocking));
            TRY(cudaEventCreateWithFlags(&shade_join_[k], cudaEventDisableTiming));
        }
        TRY(cudaEventCreateWithFlags(&shade_fork_, cudaEventDisableTiming));
    }
    const bool two_level = wide && sv.ninst > 0;
    unsigned tb = wf_trace_blocks_[two_level ? 2 : (wide ? 0 : 1)];
    if (trace_blocks_per_sm > 0) tb = std::min(tb, (unsigned)trace_blocks_per_sm * wf_sms_);
    const unsigned cgrid = (unsigned)((P + kCompactTile - 1) / kCompactTile);
    const dim3 gblock(32, 4);
    // control block (device) and its host mirror
    if (!wf_bufs_[47]) TRY(dev_alloc(&wf_bufs_[47], sizeof(WfCtl)));
    WfCtl* d_ctl = (WfCtl*)wf_bufs_[47];
    if (!wf_ctl_host_) TRY(cudaMallocHost((void**)&wf_ctl_host_, sizeof(WfCtl)));
    WfCtl* h_ctl = (WfCtl*)wf_ctl_host_;
    // graph mode: one iteration captured twice (path-ray list in q_a or in q_b), launched in groups
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    auto free_graphs = [&]() {
        for (cudaGraphExec_t& g : gexec)
            if (g) cudaGraphExecDestroy(g);
    };
    auto launch_iteration = [&](int32_t* q_ext, int32_t* q_fin, bool full, uint32_t take, uint32_t n_ext,
                                uint32_t n_fin, uint32_t nray, uint32_t n_query) -> std::string {
        // full: grids for the largest lists (graph mode); else sized to the host's counts
        k_wf_control<<<1, 32, 0, s>>>(st, d_ctl);
        if (!full) TRY(cudaEventRecord(wf_ev_[0], s));
        if (full || take) k_wf_generate<<<full ? blocks(P) : blocks(take), kWfBlock, 0, s>>>(sv, rp, st, q_ext, d_ctl);
        if (!full) TRY(cudaEventRecord(wf_ev_[1], s));
        if (full || nray) {
            const unsigned g = full ? tb : std::min(blocks(nray), tb);
            if (two_level) k_wf_trace<true, true><<<g, kWfBlock, 0, s>>>(sv, rp, st, q_ext, d_ctl, st.counts + 8, bvh.n);
            else if (wide) k_wf_trace<true><<<g, kWfBlock, 0, s>>>(sv, rp, st, q_ext, d_ctl, st.counts + 8, bvh.n);
            else k_wf_trace<false><<<g, kWfBlock, 0, s>>>(sv, rp, st, q_ext, d_ctl, st.counts + 8, bvh.n);
        }
        if (st.cache && (full || n_query)) {  // the previous shade's cache queries, before finalize adds them
            const std::string me = mlp->forward(st.feat, full ? (int)P : (int)n_query, (float*)st.cache_L, rp.err, s,
                                                st.q_cache, 4, &d_ctl->n_query);
            if (!me.empty()) return me;
        }
        if (!full) TRY(cudaEventRecord(wf_ev_[2], s));
        if (full || n_fin) {
            const unsigned g = full ? blocks(P) : blocks(n_fin);
            if (rec) k_wf_finalize<true><<<g, kWfBlock, 0, s>>>(sv, rp, st, q_fin, d_ctl);
            else k_wf_finalize<false><<<g, kWfBlock, 0, s>>>(sv, rp, st, q_fin, d_ctl);
        }
        if (!full) TRY(cudaEventRecord(wf_ev_[3], s));
        if (full || n_ext) {
            const unsigned g = full ? blocks(P) : blocks(n_ext);
            k_wf_classify<<<g, kWfBlock, 0, s>>>(sv, st, q_ext, d_ctl, (int)P);
            const unsigned gs = std::min(g, shade_grid_);
            TRY(cudaEventRecord(shade_fork_, s));
            int nb = 0;
            for (int c = 0; c < kShadeClasses; ++c) {
                if (!shade_used_[c]) continue;
                cudaStream_t cs = shade_streams_[nb];
                TRY(cudaStreamWaitEvent(cs, shade_fork_, 0));
                const std::string le = launch_shade(rec, c, shade_lm_[c], shade_tex_[c], gs, sv, rp, st, (int)P, cs);
                if (!le.empty()) return le;
                TRY(cudaEventRecord(shade_join_[nb], cs));
                ++nb;
            }
            for (int k = 0; k < nb; ++k) TRY(cudaStreamWaitEvent(s, shade_join_[k], 0));
        }
        if (!full) TRY(cudaEventRecord(wf_ev_[4], s));
        k_wf_compact<<<cgrid, kCompactThreads, 0, s>>>(st, q_fin, (int)P);
        if (!full) TRY(cudaEventRecord(wf_ev_[5], s));
        TRY(cudaGetLastError());
        return "";
    };
    const bool graph = wf_graph != 0;
    if (graph) {
        for (int k = 0; k < 2; ++k) {
            cudaGraph_t g = nullptr;
            TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            const std::string ce = launch_iteration(k ? st.q_b : st.q_a, k ? st.q_a : st.q_b, true, 0, 0, 0, 0, 0);
            cudaGraph_t gg = nullptr;
            const cudaError_t ee = cudaStreamEndCapture(s, &gg);
            g = gg;
            if (!ce.empty() || ee != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                free_graphs();
                return ce.empty() ? std::string("graph capture: ") + cudaGetErrorString(ee) : ce;
            }
            const cudaError_t ie = cudaGraphInstantiate(&gexec[k], g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) {
                free_graphs();
                return std::string("graph instantiate: ") + cudaGetErrorString(ie);
            }
        }
    }
    for (const auto& batch : batches) {
        std::vector<WfView> vv = batch;
        long ctot = 0;
        for (WfView& v : vv) {
            v.base = ctot;
            ctot += v.npix * v.nsc;
        }
        TRY(cudaMemcpyAsync(wf_bufs_[46], vv.data(), sizeof(WfView) * vv.size(), cudaMemcpyHostToDevice, s));
        WfCtl c0{};
        c0.ctot = ctot;
        c0.nviews = (uint32_t)vv.size();
        *h_ctl = c0;
        TRY(cudaMemcpyAsync(d_ctl, h_ctl, sizeof(WfCtl), cudaMemcpyHostToDevice, s));
        uint32_t nfree = (uint32_t)P;
        if (graph) {
            int par = 0, group = 4;
            for (;;) {
                for (int k = 0; k < group; ++k, par ^= 1) TRY(cudaGraphLaunch(gexec[par], s));
                launches += group * (st.cache ? 8 : 7);
                TRY(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(WfCtl), cudaMemcpyDeviceToHost, s));
                TRY(cudaStreamSynchronize(s));
                if (!h_ctl->active) break;
                if (h_ctl->iters > 1000000) {
                    free_graphs();
                    return "wavefront did not converge";
                }
                group = std::min(group * 2, 16);
            }
            iters += (int)h_ctl->iters;
            last_cache_queries += (double)h_ctl->queries;
            nfree = h_ctl->nfree;
        } else {
            long generated = 0;
            uint32_t n_cont = 0, n_fin = 0, n_sh = 0, n_mis = 0, n_query = 0;
            int32_t *q_ext = st.q_a, *q_fin = st.q_b;
            for (;; ++iters) {
                const uint32_t take = (uint32_t)std::min<long>(nfree, ctot - generated);
                const uint32_t n_ext = n_cont + take;
                if (n_ext == 0 && n_fin == 0) break;
                if (iters > 1000000) return "wavefront did not converge";
                const std::string ie = launch_iteration(q_ext, q_fin, false, take, n_ext, n_fin, n_ext + n_sh + n_mis,
                                                        n_query);
                if (!ie.empty()) return ie;
                launches += 7 + (n_query ? 1 : 0);
                last_cache_queries += n_query;
                TRY(cudaMemcpyAsync(wf_counts_host_, st.counts, 64, cudaMemcpyDeviceToHost, s));
                TRY(cudaStreamSynchronize(s));
                for (int k = 0; k < 5; ++k) {
                    float ms = 0;
                    TRY(cudaEventElapsedTime(&ms, wf_ev_[k], wf_ev_[k + 1]));
                    last_stage_ms[k] += ms;
                }
                generated += take;
                n_fin = n_ext;
                n_cont = wf_counts_host_[0];
                n_sh = wf_counts_host_[2];
                n_mis = wf_counts_host_[3];
                nfree = wf_counts_host_[4];
                n_query = wf_counts_host_[12];
                std::swap(q_ext, q_fin);
            }
            // the last compaction left the counts of an empty pool; the control block follows them
        }
        if (nfree != (uint32_t)P) {
            free_graphs();
            return "wavefront: path pool did not drain";
        }
        TRY(cudaEventRecord(wf_ev_[0], s));
        for (const WfView& v : vv) {
            const dim3 ggrid((unsigned)((std::min(v.x1 + 2, v.W) - v.x0 + 31) / 32),
                             (unsigned)((std::min(v.y1 + 2, v.H) - v.y0 + 3) / 4));
            k_film_gather<<<ggrid, gblock, 0, s>>>(sv, rp.film, v, st.fs_L, st.fs_y);
            ++launches;
        }
        TRY(cudaEventRecord(wf_ev_[6], s));
        TRY(cudaGetLastError());
        TRY(cudaEventSynchronize(wf_ev_[6]));
        float ms = 0;
        TRY(cudaEventElapsedTime(&ms, wf_ev_[0], wf_ev_[6]));
        last_stage_ms[5] += ms;
    }
    free_graphs();
    if (cache) {  // train the cache on this render's unbiased suffixes
        const std::string te = train_cache(st.counts, st.tr_feat, st.tr_target, st.tr_cap, s, rp.err);
        if (!te.empty()) return te;
        launches += 1 + cache_train_steps;
    }
    TRY(cudaEventRecord(ev1_, s));
    last_launches = launches;
    last_iterations = iters;
    return "";
}

// After a render with the radiance cache: the cache's bias on this render's training records
// (its prediction against the unbiased suffix radiance), then `cache_train_steps` Adam steps over
// the records in equal mini-batches.
std::string Tracer::train_cache(uint32_t* d_counts, uint16_t* tr_feat, float* tr_target, uint32_t tr_cap,
                                cudaStream_t s, uint32_t* d_err) {
    uint32_t cnt[2] = {0, 0};  // records taken, eligible vertices
    TRY(cudaMemcpyAsync(cnt, d_counts + 32, 8, cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    if (cache_render_paths_ > 0) cache_eligible_rate_ = cnt[1] / cache_render_paths_;
    last_train_eligible = (int)cnt[1];
    const int n = (int)std::min<uint32_t>(cnt[0], tr_cap);
    last_train_samples = n;
    if (n <= 0) return "";
    cudaEvent_t a, b;
    TRY(cudaEventCreate(&a));
    TRY(cudaEventCreate(&b));
    TRY(cudaEventRecord(a, s));
    // bias of the cache before this frame's update, on the same vertices
    float* pred = (float*)wf_bufs_[44];
    std::string e = mlp->forward(tr_feat, n, pred, d_err, s);
    if (!e.empty()) return e;
    std::vector<float> hp(3 * (size_t)n), ht(3 * (size_t)n);
    TRY(cudaMemcpyAsync(hp.data(), pred, 12 * (size_t)n, cudaMemcpyDeviceToHost, s));
    TRY(cudaMemcpyAsync(ht.data(), tr_target, 12 * (size_t)n, cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    double num = 0, den = 0;
    for (size_t k = 0; k < hp.size(); ++k) {
        num += (double)hp[k] - (double)ht[k];
        den += (double)ht[k];
    }
    last_cache_bias = den != 0 ? num / den : 0.0;  // relative bias of the mean
    float* d_loss = tr_target + 3 * (size_t)tr_cap;
    const int steps = std::max(1, cache_train_steps);
    const int nb = std::max(1, n / steps);
    for (int k = 0; k < steps && k * nb < n; ++k) {
        const int cnt = std::min(nb, n - k * nb);
        e = mlp->train_step(tr_feat + (size_t)k * nb * 96, tr_target + 3 * (size_t)k * nb, cnt, cache_lr, d_loss, d_err,
                            s);
        if (!e.empty()) return e;
    }
    TRY(cudaEventRecord(b, s));
    TRY(cudaMemcpyAsync(&last_train_loss, d_loss, 4, cudaMemcpyDeviceToHost, s));
    TRY(cudaEventSynchronize(b));
    float ms = 0;
    TRY(cudaEventElapsedTime(&ms, a, b));
    last_train_ms = ms;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return "";
}

std::string Tracer::render(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, lts_render_out* out,
                           cudaStream_t s, uint32_t* d_err) {
    std::string e = render_async(sc, bvh, d, s, d_err);
    if (!e.empty()) return e;
    TRY(cudaStreamSynchronize(s));
    float ms = 0;
    TRY(cudaEventElapsedTime(&ms, ev0_, ev1_));
    last_ms = ms;
    unsigned long long cnt[12] = {0};
    TRY(cudaMemcpy(cnt, counters_, sizeof cnt, cudaMemcpyDeviceToHost));
    for (int k = 0; k < 9; ++k) last_kind_work[k] = (double)cnt[3 + k];
    last_rays = (double)cnt[0];
    last_node_visits = (double)cnt[1];
    last_tri_tests = (double)cnt[2];
    const double rays = (double)cnt[0];
    if (out) {
        out->render_ms = ms;
        out->rays = rays;
        out->node_visits = last_node_visits;
        out->tri_tests = last_tri_tests;
        if (out->film_rgb || out->film_sums) {
            e = film_get(sc, out->film_rgb, out->film_sums, s);
            if (!e.empty()) return e;
        }
        if (d.record_samples) {
            const size_t ns = (size_t)last_paths;
            if (out->sample_L) TRY(cudaMemcpy(out->sample_L, rec_L_, 12 * ns, cudaMemcpyDeviceToHost));
            if (out->sample_sig) TRY(cudaMemcpy(out->sample_sig, rec_sig_, 8 * ns, cudaMemcpyDeviceToHost));
        }
    }
    return "";
}

std::string Tracer::film_get(const HostScene& sc, float* rgb, double* sums, cudaStream_t s) {
    if (!film_) return "nothing rendered";
    const int W = sc.width, H = sc.height;
    if (rgb) {
        k_resolve<<<(W * H + 255) / 256, 256, 0, s>>>(film_, rgb_, W, H, splat_spp_ > 0 ? splat_ : nullptr,
                                                      splat_spp_ > 0 ? 1.0 / splat_spp_ : 0.0, view_.filter);
        TRY(cudaGetLastError());
        TRY(cudaMemcpyAsync(rgb, rgb_, 12 * (size_t)W * H, cudaMemcpyDeviceToHost, s));
    }
    if (sums) TRY(cudaMemcpyAsync(sums, film_, 32 * (size_t)W * H, cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    return "";
}


std::string Tracer::render_views(const HostScene& sc, const Lbvh& bvh, const lts_view* views, int n,
                                 const lts_render_desc& d, float* const* films, lts_render_out* out, cudaStream_t s,
                                 uint32_t* d_err) {
    if (n <= 0 || !views || !films) return "bad argument: no views";
    if (d.integrator != LTS_INTEGRATOR_WAVEFRONT) return "bad argument: batched views need the wavefront integrator";
    lts_render_desc d0 = d;  // scene-wide set-up (BVH views, counters) through the one-view path
    d0.spp = 1;
    d0.x0 = d0.y0 = d0.x1 = d0.y1 = 0;
    d0.record_samples = 0;
    RenderParams rp;
    SceneView sv;
    long ns = 0;
    std::string e = prepare(sc, bvh, d0, s, d_err, &rp, &sv, &ns);
    if (!e.empty()) return e;
    // the views' films, one after another
    std::vector<WfView> slices;
    long pixels = 0, paths = 0, max_pix = 0;
    const long cap = wf_sample_cap > 0 ? wf_sample_cap : (1l << 27);
    for (int v = 0; v < n; ++v) {
        const lts_view& lv = views[v];
        if (lv.width < 2 || lv.height < 2 || lv.spp < 1) return "bad argument: view size or spp";
        const long npix = (long)lv.width * lv.height;
        if (npix > cap) return "bad argument: view larger than the sample buffer";
        WfView w{};
        const float cf[11] = {lv.from[0], lv.from[1], lv.from[2], lv.at[0], lv.at[1], lv.at[2],
                              lv.up[0],   lv.up[1],   lv.up[2],   lv.vfov,  lv.focus};
        float cam[23];
        build_camera(cf, lv.width, lv.height, cam);
        for (int k = 0; k < 12; ++k) w.cam[k] = cam[k];
        w.W = lv.width;
        w.H = lv.height;
        w.x0 = w.y0 = 0;
        w.x1 = lv.width;
        w.y1 = lv.height;
        w.spp = lv.spp;
        w.seed = lv.seed;
        w.spp_scale = quake_host((float)lv.spp);
        w.npix = npix;
        w.film_off = pixels;
        const int chunk = (int)std::max<long>(1, std::min<long>(lv.spp, cap / npix));
        for (int s0 = 0; s0 < lv.spp; s0 += chunk) {
            w.s_first = s0;
            w.nsc = std::min(chunk, lv.spp - s0);
            slices.push_back(w);
        }
        pixels += npix;
        paths += npix * lv.spp;
        max_pix = std::max(max_pix, npix);
    }
    // greedy batches of whole slices within the sample buffer
    std::vector<std::vector<WfView>> batches(1);
    long acc = 0;
    for (const WfView& w : slices) {
        const long t = w.npix * w.nsc;
        if (!batches.back().empty() && (acc + t > cap || (int)batches.back().size() >= kMaxViews)) {
            batches.emplace_back();
            acc = 0;
        }
        batches.back().push_back(w);
        acc += t;
    }
    if ((size_t)pixels * 32 > views_film_cap_) {
        dev_free(views_film_);
        views_film_ = nullptr;
        views_film_cap_ = 0;
        TRY(dev_alloc((void**)&views_film_, (size_t)pixels * 32));
        views_film_cap_ = (size_t)pixels * 32;
    }
    if (!film_accumulate) TRY(cudaMemsetAsync(views_film_, 0, (size_t)pixels * 32, s));
    rp.film = views_film_;
    last_paths = (double)paths;
    e = run_wavefront(batches, bvh, s, d_err, rp, sv);
    if (!e.empty()) return e;
    TRY(cudaStreamSynchronize(s));
    float ms = 0;
    TRY(cudaEventElapsedTime(&ms, ev0_, ev1_));
    last_ms = ms;
    unsigned long long cnt[12] = {0};
    TRY(cudaMemcpy(cnt, counters_, sizeof cnt, cudaMemcpyDeviceToHost));
    for (int k = 0; k < 9; ++k) last_kind_work[k] = (double)cnt[3 + k];
    last_rays = (double)cnt[0];
    last_node_visits = (double)cnt[1];
    last_tri_tests = (double)cnt[2];
    // resolve each view
    float* rgb = nullptr;
    TRY(dev_alloc((void**)&rgb, 12 * (size_t)max_pix));
    long off = 0;
    for (int v = 0; v < n; ++v) {
        const int W = views[v].width, H = views[v].height;
        k_resolve<<<(W * H + 255) / 256, 256, 0, s>>>(views_film_ + 4 * off, rgb, W, H, nullptr, 0.0, nullptr);
        cudaError_t c = cudaGetLastError();
        if (c == cudaSuccess && films[v]) c = cudaMemcpyAsync(films[v], rgb, 12 * (size_t)W * H, cudaMemcpyDeviceToHost, s);
        if (c == cudaSuccess) c = cudaStreamSynchronize(s);
        if (c != cudaSuccess) {
            dev_free(rgb);
            return std::string("resolve views: ") + cudaGetErrorString(c);
        }
        off += (long)W * H;
    }
    dev_free(rgb);
    if (out) {
        out->render_ms = ms;
        out->rays = last_rays;
        out->node_visits = last_node_visits;
        out->tri_tests = last_tri_tests;
    }
    return "";
}


// Autotuner: renders the views at reduced spp under each candidate of the wavefront's runtime
// shape -- path-pool capacity (queue size), persistent trace blocks per SM, graph or
// kernel-by-kernel iterations -- one knob at a time from the defaults, keeps the fastest and leaves
// it set.
std::string Tracer::autotune_views(const HostScene& sc, const Lbvh& bvh, const lts_view* views, int n,
                                   const lts_render_desc& d, lts_autotune_result* res, cudaStream_t s,
                                   uint32_t* d_err) {
    std::vector<lts_view> tv(views, views + n);
    long max_pix = 0;
    for (lts_view& v : tv) {
        v.spp = std::max(1, v.spp / 8);
        max_pix = std::max(max_pix, (long)v.width * v.height);
    }
    std::vector<float> scratch(3 * (size_t)max_pix);
    std::vector<float*> films(n, scratch.data());  // every view resolves into the same host buffer
    const bool accum = film_accumulate;
    film_accumulate = false;
    auto trial = [&](double* ms) -> std::string {
        double best = 1e30;
        for (int rep = 0; rep < 2; ++rep) {  // first run may allocate; keep the faster of two
            const std::string e = render_views(sc, bvh, tv.data(), n, d, films.data(), nullptr, s, d_err);
            if (!e.empty()) return e;
            best = std::min(best, (double)last_ms);
        }
        *ms = best;
        return "";
    };
    long pool = wf_pool;  // 0: automatic
    int bps = trace_blocks_per_sm, graph = wf_graph;
    double t0 = 0;
    std::string e = trial(&t0);
    if (!e.empty()) return e;
    double best = t0;
    long paths = 0;  // of one tuning render; larger pools hold them all, as the automatic one does
    for (const lts_view& v : tv) paths += (long)v.width * v.height * v.spp;
    for (int lg = 18; lg <= 26 && (1l << lg) < paths; ++lg) {
        wf_pool = 1l << lg;
        double t;
        if (!(e = trial(&t)).empty()) return e;
        if (t < best) {
            best = t;
            pool = wf_pool;
        }
    }
    wf_pool = pool;
    for (int b : {2, 4, 0}) {  // 0: as many as stay resident
        trace_blocks_per_sm = b;
        double t;
        if (!(e = trial(&t)).empty()) return e;
        if (t < best) {
            best = t;
            bps = b;
        }
    }
    trace_blocks_per_sm = bps;
    wf_graph = 1 - graph;
    {
        double t;
        if (!(e = trial(&t)).empty()) return e;
        if (t < best) {
            best = t;
            graph = wf_graph;
        }
    }
    wf_graph = graph;
    film_accumulate = accum;
    if (res) {
        int lg = 0;
        while (pool > 0 && (1l << lg) < pool) ++lg;
        res->pool_log2 = lg;
        res->trace_blocks_per_sm = bps;
        res->graph = graph;
        res->ms_default = t0;
        res->ms_best = best;
    }
    return "";
}

}  // namespace lts
