/*
 * Test infrastructure only (oracle).  Unity translation unit that compiles the reference's
 * own sources -- tierChampion/LightTransportSimulation src/*.cu, read in place -- as a host
 * program, plus a small driver that dumps what the parity fixtures need:
 *
 *   lts_ref bvh    ROOT SCENE SUBJECT OUT W H
 *       parseScene (core/SceneLoader.cuh:195-360) -> sorted Morton codes and ids
 *       (BVH.cuh:140-146), the flattened traversal tree (BVH.cuh:311-329: key, children,
 *       AABB of all 2N-1 nodes), world-space triangle vertices in primitive order, the camera
 *       (rendering/Camera.cu:9-43) and the light power distribution
 *       (intergrators/IntegratorHelper.cuh:147-162).
 *   lts_ref image IN W H FORMAT OUT
 *       writeToPPM (FORMAT 0) / writeToPFM (FORMAT 1) (core/ImageO.cuh:16-78), the writers of
 *       Camera::sendRenderToImageFile (rendering/Camera.cu:250-253), on W x H x 3 raw floats.
 *   lts_ref render ROOT SCENE SUBJECT OUT W H SPP MAXB RR SEED X0 Y0 X1 Y1 THREADS FILM
 *       PathTracingIntegrator::evaluate (PathTracingIntegrator.cuh:26-109) over the pixel
 *       crop [X0,X1)x[Y0,Y1) -> per-(pixel, sample) radiance L and a 64-bit FNV-1a hash of the
 *       sample's events (extension hit primitive per bounce, shadow-ray visibility, MIS-ray
 *       hit primitive, texture branch decisions, BSDF grazing tests), the render wall time, and (FILM=1) the resolved film of
 *       Camera::getRender (Camera.cu:256-289).
 *   lts_ref imread FILE OUT / lts_ref jpgwrite RAW W H COMP QUALITY OUT
 *       the reference's image reader loadImageFile_s (core/ImageI.cuh:11-34, stb_image) on a
 *       PNG or JPEG file; stb_image_write's JPEG writer (test inputs).
 *   lts_ref kat FN IN OUT
 *       the reference's own single functions (Trowbridge-Reitz distribution and sampling,
 *       MicrofacetReflection, Fresnel terms, Perlin noise, fbm, turbulence, offsetRayOrigin,
 *       quakeIIIFastInvSqrt) on raw input records: the known-answer vectors of
 *       tests/golden/kat_reference.npz (record layouts: LTS_KAT_* in include/lts_capi.h).
 *
 * Build: oracle/ref/build_ref.sh (g++ -E | instrument.pl | g++).  Output: oracle/_ref/lts_ref.
 */
#include <cassert>
#include <charconv>
#include <chrono>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <string_view>

#define private public
#define protected public
#define class struct
#include "core/SceneLoader_kernels.cu"
#include "acceleration/BVH_kernels.cu"
#include "shapes/Triangle.cu"
#include "geometry/Interaction.cu"
#include "lights/Light.cu"
#include "lights/VisibilityTester.cu"
#include "rendering/Camera.cu"
#include "intergrators/IntegratorKernels.cu"
#include "materials/textures/Mipmap_kernel.cu"
#undef class
#undef private
#undef protected

using namespace lts;

/* ------------------------------------------------------------------ LTSD container */
struct LtsdWriter {
    FILE* f;
    explicit LtsdWriter(const char* path) {
        f = fopen(path, "wb");
        if (!f) {
            fprintf(stderr, "cannot open %s\n", path);
            exit(3);
        }
        fwrite("LTSD", 1, 4, f);
    }
    void put(const char* name, char dtype, const void* data, uint64_t count, size_t elem) {
        uint32_t nl = (uint32_t)strlen(name);
        fwrite(&nl, 4, 1, f);
        fwrite(name, 1, nl, f);
        fwrite(&dtype, 1, 1, f);
        fwrite(&count, 8, 1, f);
        if (count) fwrite(data, elem, count, f);
    }
    ~LtsdWriter() { fclose(f); }
};

/* ------------------------------------------------------------------ recording hooks */
static const Primitive* g_prim_base = nullptr;
static int g_crop_x0, g_crop_y0, g_crop_w, g_crop_h, g_spp, g_width;
static std::vector<float> g_L;
static std::vector<uint64_t> g_sig;
static thread_local uint64_t t_hash;

static inline void fnv_mix(uint64_t v) {
    for (int i = 0; i < 8; ++i) {
        t_hash ^= (v >> (8 * i)) & 0xffu;
        t_hash *= 0x100000001b3ull;
    }
}
static inline int64_t prim_index(const void* p) {
    return p ? (int64_t)((const Primitive*)p - g_prim_base) : -1;
}

void lts_hook_begin_sample(int id, int s) {
    (void)id;
    lts_ref_cur_sample = (uint32_t)s;
    t_hash = 0xcbf29ce484222325ull;
}
void lts_hook_hit(const void* prim) { fnv_mix(0x100000000ull + (uint64_t)(prim_index(prim) + 1)); }
void lts_hook_branch(unsigned long long v) { fnv_mix(v); }
bool lts_hook_bool(unsigned long long tag, bool v) {
    fnv_mix(tag + (v ? 1u : 0u));
    return v;
}
void lts_hook_mis(const void* prim) { fnv_mix(0x200000000ull + (uint64_t)(prim_index(prim) + 1)); }
bool lts_hook_vis(bool unoccluded) {
    fnv_mix(0x300000000ull + (unoccluded ? 1u : 0u));
    return unoccluded;
}
void lts_hook_sample(int id, int s, float r, float g, float b) {
    const int i = id % g_width, j = id / g_width;
    const int ci = i - g_crop_x0, cj = j - g_crop_y0;
    if (ci < 0 || cj < 0 || ci >= g_crop_w || cj >= g_crop_h) return;
    const size_t k = ((size_t)cj * g_crop_w + ci) * g_spp + s;
    g_L[3 * k + 0] = r;
    g_L[3 * k + 1] = g;
    g_L[3 * k + 2] = b;
    g_sig[k] = t_hash;
}

/* ------------------------------------------------------------------ driver */
static Scene* load(const std::string& root, const std::string& scene, const std::string& subject, int w, int h,
                   Camera** cam) {
    Filter* f = new GaussianFilter(Vector2f(1.0f, 1.0f), 1.0f); /* LightTransportSimulation.cu:64 */
    Scene* s = parseScene(cam, f, 0.f, w, h, root, scene, subject == "-" ? "" : subject);
    delete f;
    return s;
}

static Distribution1D* light_distribution(Scene* scene) {
    Distribution1D* d = (Distribution1D*)calloc(1, sizeof(Distribution1D));
    lts_launch(lightDistributionKernel, dim3(1), dim3(1))(d, (const Scene*)scene);
    return d;
}

static int cmd_bvh(int argc, char** argv) {
    if (argc < 8) return 2;
    const std::string root = argv[2], scene = argv[3], subject = argv[4];
    const char* out = argv[5];
    const int w = atoi(argv[6]), h = atoi(argv[7]);
    Camera* cam = nullptr;
    Scene* sc = load(root, scene, subject, w, h, &cam);
    BVH* bvh = sc->traversalTree;
    const int nodes = bvh->count, n = (nodes + 1) / 2;
    std::vector<int32_t> key(nodes), left(nodes), right(nodes);
    std::vector<float> bounds((size_t)nodes * 6);
    for (int i = 0; i < nodes; ++i) {
        const LBVHTraversalNode& t = bvh->tree[i];
        key[i] = t.key;
        left[i] = t.left ? (int32_t)(t.left - bvh->tree) : -1;
        right[i] = t.right ? (int32_t)(t.right - bvh->tree) : -1;
        const float b[6] = {t.bounds.pMin.x, t.bounds.pMin.y, t.bounds.pMin.z,
                            t.bounds.pMax.x, t.bounds.pMax.y, t.bounds.pMax.z};
        memcpy(&bounds[(size_t)i * 6], b, sizeof b);
    }
    std::vector<float> tri((size_t)n * 9);
    for (int i = 0; i < n; ++i) {
        const Triangle* t = bvh->primitives[i].tri;
        for (int c = 0; c < 3; ++c) {
            const Point3f& p = t->mesh->p[t->vertices[3 * c]];
            tri[(size_t)i * 9 + 3 * c + 0] = p.x;
            tri[(size_t)i * 9 + 3 * c + 1] = p.y;
            tri[(size_t)i * 9 + 3 * c + 2] = p.z;
        }
    }
    const float camv[23] = {cam->o.x, cam->o.y, cam->o.z, cam->right.x, cam->right.y, cam->right.z,
                            cam->up.x, cam->up.y, cam->up.z, cam->llc.x, cam->llc.y, cam->llc.z,
                            cam->u.x, cam->u.y, cam->u.z, cam->v.x, cam->v.y, cam->v.z,
                            cam->w.x, cam->w.y, cam->w.z, cam->lensRadius, cam->focalDist};
    Distribution1D* d = light_distribution(sc);
    std::vector<float> func(d->size > 0 ? d->func : nullptr, d->size > 0 ? d->func + d->size : nullptr);
    std::vector<float> cdf(d->cdf, d->cdf + d->size + 1);
    const int32_t lc = sc->lightCount;
    std::vector<int32_t> lflags(lc);
    for (int l = 0; l < lc; ++l) lflags[l] = sc->lights[l] ? sc->lights[l]->flag : -1;
    std::vector<float> filt(bvh->count > 0 ? 256 : 0);
    memcpy(filt.data(), cam->d_table, 256 * sizeof(float));

    LtsdWriter wr(out);
    wr.put("sorted_codes", 'u', lts_ref_sorted_codes.data(), lts_ref_sorted_codes.size(), 4);
    wr.put("sorted_ids", 'i', lts_ref_sorted_ids.data(), lts_ref_sorted_ids.size(), 4);
    wr.put("node_key", 'i', key.data(), nodes, 4);
    wr.put("node_left", 'i', left.data(), nodes, 4);
    wr.put("node_right", 'i', right.data(), nodes, 4);
    wr.put("node_bounds", 'f', bounds.data(), bounds.size(), 4);
    wr.put("tri_p", 'f', tri.data(), tri.size(), 4);
    wr.put("camera", 'f', camv, 23, 4);
    wr.put("light_flags", 'i', lflags.data(), lflags.size(), 4);
    wr.put("light_func", 'f', func.data(), func.size(), 4);
    wr.put("light_cdf", 'f', cdf.data(), cdf.size(), 4);
    wr.put("filter_table", 'f', filt.data(), filt.size(), 4);
    return 0;
}

static int cmd_render(int argc, char** argv) {
    if (argc < 18) return 2;
    const std::string root = argv[2], scene = argv[3], subject = argv[4];
    const char* out = argv[5];
    const int w = atoi(argv[6]), h = atoi(argv[7]), spp = atoi(argv[8]), maxb = atoi(argv[9]),
              rr = atoi(argv[10]);
    const unsigned seed = (unsigned)strtoul(argv[11], nullptr, 10);
    const int x0 = atoi(argv[12]), y0 = atoi(argv[13]), x1 = atoi(argv[14]), y1 = atoi(argv[15]);
    const int threads = atoi(argv[16]), want_film = atoi(argv[17]);
    if (threads > 0) omp_set_num_threads(threads);

    Camera* cam = nullptr;
    Scene* sc = load(root, scene, subject, w, h, &cam);
    g_prim_base = sc->traversalTree->primitives;
    Distribution1D* dist = light_distribution(sc);

    /* LightTransportSimulation.cu:95-100 */
    Sampler h_samp(spp, w * h);
    Sampler* d_samp = passToDevice(&h_samp);
    PathTracingIntegrator h_int(maxb, rr, cam, d_samp, sc);
    PathTracingIntegrator* d_int = passToDevice(&h_int);

    g_crop_x0 = x0;
    g_crop_y0 = y0;
    g_crop_w = x1 - x0;
    g_crop_h = y1 - y0;
    g_spp = spp;
    g_width = w;
    const size_t ns = (size_t)g_crop_w * g_crop_h * spp;
    g_L.assign(3 * ns, 0.f);
    g_sig.assign(ns, 0);

    const long npix = (long)g_crop_w * g_crop_h;
    auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel for schedule(dynamic, 16)
    for (long p = 0; p < npix; ++p) {
        const int i = x0 + (int)(p % g_crop_w), j = y0 + (int)(p / g_crop_w);
        d_int->evaluate(i, j, *dist, (int)seed);
    }
    auto t1 = std::chrono::steady_clock::now();
    const double secs = std::chrono::duration<double>(t1 - t0).count();
    const int32_t nthreads = omp_get_max_threads();

    LtsdWriter wr(out);
    wr.put("L", 'f', g_L.data(), g_L.size(), 4);
    wr.put("sig", 'q', g_sig.data(), g_sig.size(), 8);
    wr.put("time_s", 'd', &secs, 1, 8);
    wr.put("threads", 'i', &nthreads, 1, 4);
    if (want_film) {
        std::vector<float> rgb((size_t)w * h * 3);
        cam->getRender(rgb.data(), 0.0f);
        wr.put("film", 'f', rgb.data(), rgb.size(), 4);
    }
    return 0;
}

static int cmd_image(int argc, char** argv) {
    if (argc < 7) return 2;
    const int w = atoi(argv[3]), h = atoi(argv[4]), format = atoi(argv[5]);
    std::vector<float> rgb((size_t)w * h * 3);
    FILE* f = fopen(argv[2], "rb");
    if (!f || fread(rgb.data(), sizeof(float), rgb.size(), f) != rgb.size()) return 3;
    fclose(f);
    const bool ok = format == 0 ? writeToPPM(argv[6], rgb.data(), w, h) : writeToPFM(argv[6], rgb.data(), w, h);
    return ok ? 0 : 3;
}

/* lts_ref imread FILE OUT: the reference's image reader, loadImageFile_s (core/ImageI.cuh:11-34:
 * stbi_loadf with three channels, rows flipped) -> OUT: int32 width, int32 height, then
 * width*height*3 float32 texels.  An unreadable image ends the program with status 1, as the
 * reference does. */
static int cmd_imread(int argc, char** argv) {
    if (argc < 4) return 2;
    int w = 0, h = 0;
    Spectrum* img = loadImageFile_s(argv[2], &w, &h);
    FILE* g = fopen(argv[3], "wb");
    if (!g) return 3;
    const int32_t dims[2] = {w, h};
    bool ok = fwrite(dims, 4, 2, g) == 2;
    for (long i = 0; ok && i < (long)w * h; ++i) {
        const float t[3] = {img[i].r, img[i].g, img[i].b};
        ok = fwrite(t, 4, 3, g) == 3;
    }
    fclose(g);
    delete[] img;
    return ok ? 0 : 3;
}

/* lts_ref jpgwrite RAW W H COMP QUALITY OUT: stbi_write_jpg of the vendored stb_image_write
 * (extern/stb_image_write.h) on W x H x COMP raw bytes (test inputs for the JPEG decoder). */
static int cmd_jpgwrite(int argc, char** argv) {
    if (argc < 8) return 2;
    const int w = atoi(argv[3]), h = atoi(argv[4]), comp = atoi(argv[5]), quality = atoi(argv[6]);
    std::vector<unsigned char> px((size_t)w * h * comp);
    FILE* f = fopen(argv[2], "rb");
    if (!f || fread(px.data(), 1, px.size(), f) != px.size()) return 3;
    fclose(f);
    return stbi_write_jpg(argv[7], w, h, comp, px.data(), quality) ? 0 : 3;
}

/* ------------------------------------------------------------------ known-answer vectors
 * lts_ref kat FN IN OUT: IN holds n records of 16 raw float32 inputs; OUT receives 16 floats per
 * record, the reference's own function FN (LTS_KAT_* and record layouts of include/lts_capi.h)
 * evaluated on each. */
#include "../../include/lts_capi.h"

static int cmd_kat(int argc, char** argv) {
    if (argc < 5) return 2;
    const int fn = atoi(argv[2]);
    FILE* f = fopen(argv[3], "rb");
    if (!f) return 3;
    std::vector<float> in;
    float buf[16];
    while (fread(buf, 4, 16, f) == 16) in.insert(in.end(), buf, buf + 16);
    fclose(f);
    const size_t n = in.size() / 16;
    std::vector<float> out(16 * n, 0.0f);
    for (size_t r = 0; r < n; ++r) {
        const float* a = &in[16 * r];
        float* o = &out[16 * r];
        const Vector3f v0(a[0], a[1], a[2]), v3(a[3], a[4], a[5]);
        switch (fn) {
            case LTS_KAT_QUAKE_RSQRT: o[0] = quakeIIIFastInvSqrt(a[0]); break;
            case LTS_KAT_FRESNEL_DIELECTRIC: o[0] = fresnelReflectionDielectric(a[0], a[1], a[2]); break;
            case LTS_KAT_FRESNEL_CONDUCTOR: {
                const Spectrum s = fresnelReflectionConductor(a[0], Spectrum(1.0f), Spectrum(a[1], a[2], a[3]),
                                                              Spectrum(a[4], a[5], a[6]));
                o[0] = s.r, o[1] = s.g, o[2] = s.b;
                break;
            }
            case LTS_KAT_TR_D: o[0] = TrowbridgeReitzMicrofacetDistribution(a[3], a[4]).d(v0); break;
            case LTS_KAT_TR_LAMBDA: o[0] = TrowbridgeReitzMicrofacetDistribution(a[3], a[4]).lambda(v0); break;
            case LTS_KAT_TR_G1: o[0] = TrowbridgeReitzMicrofacetDistribution(a[3], a[4]).g1(v0); break;
            case LTS_KAT_TR_G: o[0] = TrowbridgeReitzMicrofacetDistribution(a[6], a[7]).g(v0, v3); break;
            case LTS_KAT_TR_SAMPLE11: TrowbridgeReitzSample11(a[0], a[1], a[2], &o[0], &o[1]); break;
            case LTS_KAT_TR_SAMPLE_WH: {
                const Vector3f wh = TrowbridgeReitzMicrofacetDistribution(a[3], a[4]).sampleWH(v0, Point2f(a[5], a[6]));
                o[0] = wh.x, o[1] = wh.y, o[2] = wh.z;
                break;
            }
            case LTS_KAT_TR_PDF: o[0] = TrowbridgeReitzMicrofacetDistribution(a[6], a[7]).Pdf(v0, v3); break;
            case LTS_KAT_MF_F:
            case LTS_KAT_MF_PDF: {
                Fresnel* fr = fn == LTS_KAT_MF_F ? new FresnelConductor(Spectrum(1.0f), Spectrum(a[10], a[11], a[12]),
                                                                        Spectrum(a[13], a[14], a[15]))
                                                 : new FresnelConductor(Spectrum(1.0f), Spectrum(1.0f), Spectrum(1.0f));
                const Spectrum R = fn == LTS_KAT_MF_F ? Spectrum(a[7], a[8], a[9]) : Spectrum(1.0f);
                const MicrofacetReflection mr(R, a[6], a[6], fr);
                if (fn == LTS_KAT_MF_F) {
                    const Spectrum s = mr.f(v0, v3);
                    o[0] = s.r, o[1] = s.g, o[2] = s.b;
                } else {
                    o[0] = mr.Pdf(v0, v3);
                }
                delete fr;
                break;
            }
            case LTS_KAT_MF_SAMPLE: {
                Fresnel* fr = new FresnelConductor(Spectrum(1.0f), Spectrum(a[9], a[10], a[11]),
                                                   Spectrum(a[12], a[13], a[14]));
                const MicrofacetReflection mr(Spectrum(a[6], a[7], a[8]), a[3], a[3], fr);
                Vector3f wi(0.0f, 0.0f, 0.0f);
                float pdf = 0.0f;
                Point2f u(a[4], a[5]);
                const Spectrum s = mr.sampleF(v0, &wi, u, &pdf);
                o[0] = wi.x, o[1] = wi.y, o[2] = wi.z, o[3] = s.r, o[4] = s.g, o[5] = s.b, o[6] = pdf;
                delete fr;
                break;
            }
            case LTS_KAT_PERLIN: o[0] = perlinNoise(a[0], a[1], a[2]); break;
            case LTS_KAT_FBM:
            case LTS_KAT_TURBULENCE: {
                const Point3f p(a[0], a[1], a[2]);
                const Vector3f dx(a[3], a[4], a[5]), dy(a[6], a[7], a[8]);
                o[0] = fn == LTS_KAT_FBM ? fbm(p, dx, dy, a[9], (int)a[10]) : turbulence(p, dx, dy, a[9], (int)a[10]);
                break;
            }
            case LTS_KAT_OFFSET_ORIGIN: {
                const Point3f po = offsetRayOrigin(Point3f(a[0], a[1], a[2]), v3, Normal3f(a[6], a[7], a[8]),
                                                   Vector3f(a[9], a[10], a[11]));
                o[0] = po.x, o[1] = po.y, o[2] = po.z;
                break;
            }
            default: return 2;
        }
    }
    FILE* g = fopen(argv[4], "wb");
    if (!g) return 3;
    const bool ok = fwrite(out.data(), 4, out.size(), g) == out.size();
    fclose(g);
    return ok ? 0 : 3;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: lts_ref bvh|render|image|imread|jpgwrite|kat ...\n");
        return 2;
    }
    std::cout.setstate(std::ios_base::failbit); /* silence the loader's banners */
    const std::string c = argv[1];
    int rc = 2;
    if (c == "bvh") rc = cmd_bvh(argc, argv);
    if (c == "render") rc = cmd_render(argc, argv);
    if (c == "image") rc = cmd_image(argc, argv);
    if (c == "kat") rc = cmd_kat(argc, argv);
    if (c == "imread") rc = cmd_imread(argc, argv);
    if (c == "jpgwrite") rc = cmd_jpgwrite(argc, argv);
    if (rc == 2) fprintf(stderr, "bad arguments\n");
    return rc;
}
