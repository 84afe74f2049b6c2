// Bidirectional path tracing (sm_103a megakernel): one thread per pixel, every sample builds a
// camera subpath and a light subpath and combines every connection strategy (s light vertices,
// t camera vertices) with multiple-importance weights -- the algorithm of Veach's thesis as PBRT
// v3 states it (ch. 16.3: random walks with forward / reverse area densities, ConnectBDPT,
// MISWeight's ratio chain).
//
// The reference ships this integrator disabled and unfinished (intergrators/
// BidirectionalPathIntegrator.cuh:285-660, LightTransportSimulation.cu:116-121): its light walk
// starts on top of the light vertex (`randomWalk(..., path, id)` overwrites path[0]), its
// strategy loops stop one vertex short (`t < nCamera`, `s < nLight`), and its camera importance
// (Camera.cu:88-186) divides by the raster's pixel count instead of the image plane's area.  Here
// the published algorithm is built over this renderer's own pieces -- the traversal, make_si,
// the materials' BSDFs, the area and point lights -- so that it estimates the same image as the
// path tracer: tests compare the two films.
//
// The reference's dielectric is not reciprocal (its "reflection" continues straight through the
// surface with the Fresnel term of the arriving side, Specular.cuh:112), so paths through glass
// are weighted differently when traced from the light: where glass shapes the image (a caustic)
// this estimator and the path tracer's differ.
//
// Scope: area and point lights (the reference's infinite light has no consistent emission
// density: its sampleLi draws a hemisphere about +y with a latitude-longitude pdf about +z, so a
// scene with one is refused).  The camera is the reference's pinhole (lens radius 0): importance
// We = 1 / (A cos^4), direction density 1 / (A cos^3) with A the film's area on the plane at unit
// distance.  Subpaths have no Russian roulette (MIS needs the plain densities); camera subpaths
// carry up to max_bounce + 2 vertices, light subpaths up to max_bounce + 1.  Connections to the
// camera (t = 1) land anywhere on the film and are splatted, unfiltered, into a separate buffer
// scaled by 1 / spp at resolve.
#pragma once

#include "tracer_dev.cuh"

namespace lts {
namespace {

constexpr int kBdptMaxBounce = 8;  // longest path the kernel's vertex arrays hold

enum : int { BV_CAMERA = 0, BV_LIGHT = 1, BV_SURFACE = 2 };

struct BVert {
    int type;        // BV_*
    int delta;       // surface vertex that sampled a specular lobe (0 for light and camera vertices)
    int light;       // light vertices and emitting surfaces: light index, else -1
    V3 p, n, perr;   // position, geometric normal (zero: not on a surface), position error bound
    V3 wo;           // surface: direction toward the vertex it was reached from
    Spec beta;       // throughput up to and including this vertex
    real pdf_fwd, pdf_rev;  // area densities of sampling this vertex from either direction
    Bsdf f;          // surface: its scattering functions
};

// Camera model (rendering/Camera.cu:9-43, lens radius 0): origin, screen corner and edge vectors
// at the focal distance, viewing direction -w.
struct BCam {
    V3 o, right, up, llc, w;
    real focal, area;  // film area on the plane at unit distance
    int W, H;
};
__device__ __forceinline__ BCam bdpt_camera(const SceneView& sv) {
    BCam c;
    const float* m = sv.cam;
    c.o = v3(m[0], m[1], m[2]);
    c.right = v3(m[3], m[4], m[5]);
    c.up = v3(m[6], m[7], m[8]);
    c.llc = v3(m[9], m[10], m[11]);
    c.w = v3(m[18], m[19], m[20]);
    c.focal = m[22];
    c.W = sv.width;
    c.H = sv.height;
    // rays go through llc + right * px / (W - 1) + up * py / (H - 1) for px in [0, W), py in [0, H)
    const real sx = xsqrt(len2(c.right)) * ((real)c.W / (real)(c.W - 1));
    const real sy = xsqrt(len2(c.up)) * ((real)c.H / (real)(c.H - 1));
    c.area = sx * sy / (c.focal * c.focal);
    return c;
}
// The film position of direction d from the camera (false: behind the camera or off the film),
// and cos(theta) to the viewing axis.
__device__ __forceinline__ bool bdpt_raster(const BCam& c, V3 d, real& px, real& py, real& cos_t) {
    cos_t = -dot(d, c.w);
    if (cos_t <= 0) return false;
    const V3 s = c.o + d * (c.focal / cos_t) - c.llc;
    px = dot(s, c.right) / len2(c.right) * (real)(c.W - 1);
    py = dot(s, c.up) / len2(c.up) * (real)(c.H - 1);
    return px >= 0 && px < (real)c.W && py >= 0 && py < (real)c.H;
}
__device__ __forceinline__ real bdpt_we(const BCam& c, real cos_t) {
    const real c2 = cos_t * cos_t;
    return 1 / (c.area * c2 * c2);
}
__device__ __forceinline__ real bdpt_pdf_dir(const BCam& c, real cos_t) { return 1 / (c.area * cos_t * cos_t * cos_t); }

// Light choice with the power distribution (Distribution1D, sampling/Sampling.cuh:104-198) over
// every light -- without the reference's findInterval clamp that never picks the last light.
__device__ __forceinline__ int bdpt_pick_light(const SceneView& sv, real u, real& pdf) {
    const int n = sv.nlight;
    int first = 0, len = n + 1;
    while (len > 0) {
        const int half = len >> 1, middle = first + half;
        if (__ldg(sv.light_cdf + middle) <= u) {
            first = middle + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    const int i = max(0, min(first - 1, n - 1));
    pdf = __ldg(sv.light_func + i) / (sv.light_func_int * n);
    return i;
}
__device__ __forceinline__ real bdpt_light_pdf(const SceneView& sv, int i) {
    return __ldg(sv.light_func + i) / (sv.light_func_int * sv.nlight);
}

__device__ __forceinline__ bool bv_on_surface(const BVert& v) { return v.n.x != 0 || v.n.y != 0 || v.n.z != 0; }
__device__ __forceinline__ bool bv_delta_light(const SceneView& sv, const BVert& v) {
    return v.type == BV_LIGHT && sv.lights[v.light].kind == 2;  // a point light's position
}
__device__ __forceinline__ bool bv_is_light(const BVert& v) {
    return v.type == BV_LIGHT || (v.type == BV_SURFACE && v.light >= 0);
}
__device__ __forceinline__ bool bv_connectible(const BVert& v) {
    if (v.type != BV_SURFACE) return true;
    return v.f.lobe != LOBE_NONE && (v.f.type & (BSDF_DIFFUSE | BSDF_GLOSSY)) != 0;
}
// Vertex::ConvertDensity: a solid-angle density at `from` toward `to` in area measure at `to`.
__device__ __forceinline__ real bv_convert(real pdf, const BVert& from, const BVert& to) {
    const V3 d = to.p - from.p;
    const real l2 = len2(d);
    if (l2 == 0) return 0;
    const real inv = 1 / l2;
    if (bv_on_surface(to)) pdf *= absdot(to.n, d * xsqrt(inv));
    return pdf * inv;
}
// PBRT's CorrectShadingNormal for importance transport (the reference's correctShadingNormal,
// BidirectionalPathIntegrator.cuh:11-22).
__device__ __forceinline__ real bdpt_shading_fix(const Bsdf& f, V3 wo, V3 wi) {
    const real den = absdot(wo, f.ng) * absdot(wi, f.ns);
    if (den == 0) return 0;
    return absdot(wo, f.ns) * absdot(wi, f.ng) / den;
}
// Vertex::f: scattering at surface vertex v toward `next`.  LM (and TEX below): the lobes (and
// textures) the scene's materials can have -- the kernel is compiled for them only, as the
// wavefront's shade kernels are.
template <int LM>
__device__ __forceinline__ Spec bv_f(const BVert& v, const BVert& next, bool importance) {
    const V3 wi = normalize(next.p - v.p);
    Spec c = bsdf_f<LM>(v.f, v.wo, wi, BSDF_ALL, nullptr);
    if (importance) c = c * bdpt_shading_fix(v.f, v.wo, wi);
    return c;
}
// Emitted radiance of light vertex or emitting surface v toward w (DiffuseAreaLight::L: one-sided
// along the surface normal; a point light's intensity is reached only by connections).
__device__ __forceinline__ Spec bv_le(const SceneView& sv, const BVert& v, V3 w) {
    if (v.light < 0) return spec(0.0f);
    const DevLight& L = sv.lights[v.light];
    if (L.kind != 0) return spec(0.0f);
    return dot(v.n, w) > 0 ? Spec{L.L[0], L.L[1], L.L[2]} : spec(0.0f);
}
// Vertex::PdfLight: density (area measure at `to`) of light vertex v emitting toward `to`.
__device__ __forceinline__ real bv_pdf_light(const SceneView& sv, const BVert& v, const BVert& to) {
    const V3 d = to.p - v.p;
    const real l2 = len2(d);
    if (l2 == 0) return 0;
    const V3 w = d * xsqrt(1 / l2);
    const DevLight& L = sv.lights[v.light];
    real pdf = L.kind == 0 ? xmax(0.0f, dot(v.n, w)) * LTS_INV_PI_F : (real)(0.25 * LTS_INV_PI_F);
    pdf /= l2;
    if (bv_on_surface(to)) pdf *= absdot(to.n, w);
    return pdf;
}
// Vertex::PdfLightOrigin: light choice times the position density (0 for a point light's delta).
__device__ __forceinline__ real bv_pdf_light_origin(const SceneView& sv, const BVert& v) {
    const DevLight& L = sv.lights[v.light];
    return L.kind == 0 ? bdpt_light_pdf(sv, v.light) / L.area : 0.0f;
}
// Vertex::Pdf: density (area measure at `next`) of sampling `next` from v, which was reached from
// `prev` (null for an endpoint).
template <int LM>
__device__ __forceinline__ real bv_pdf(const SceneView& sv, const BCam& cam, const BVert& v, const BVert* prev,
                                       const BVert& next) {
    if (v.type == BV_LIGHT) return bv_pdf_light(sv, v, next);
    const V3 d = next.p - v.p;
    if (len2(d) == 0) return 0;
    const V3 wn = normalize(d);
    real pdf;
    if (v.type == BV_CAMERA) {
        real px, py, cos_t;
        if (!bdpt_raster(cam, wn, px, py, cos_t)) return 0;
        pdf = bdpt_pdf_dir(cam, cos_t);
    } else {
        if (!prev) return 0;
        const V3 wp = normalize(prev->p - v.p);
        pdf = bsdf_pdf<LM>(v.f, wp, wn, BSDF_ALL, nullptr);
    }
    return bv_convert(pdf, v, next);
}

// VisibilityTester::unoccluded between two vertices (offset origins as spawnRayTo).
__device__ __forceinline__ bool bdpt_visible(const SceneView& sv, int nleaf, const BVert& a, const BVert& b,
                                             uint32_t* stack, uint32_t* err, Work& wk) {
    const V3 org = offset_origin(a.p, a.perr, a.n, b.p - a.p);
    const V3 tgt = offset_origin(b.p, b.perr, b.n, org - b.p);
    return !scene_occluded(sv, nleaf, org, tgt - org, 1 - kShadowEps, stack, err, wk);
}

// RandomWalk: extends `path` (path[0] is the walk's start, already filled) by up to max_depth
// surface vertices; returns the vertices added.
template <int LM, bool TEX>
__device__ int bdpt_walk(const SceneView& sv, int nleaf, BVert* path, V3 ro, V3 rd, Spec beta, real pdf_fwd,
                         int max_depth, bool importance, Rng& rng, bool diff0, V3 rxo, V3 rxd, V3 ryd,
                         uint32_t* stack, uint32_t* err, Work& wk, unsigned long long& rays) {
    int bounces = 0;
    real pdf_rev = 0;
    while (bounces < max_depth) {
        SI si;
        ++rays;
        if (!scene_intersect(sv, nleaf, ro, rd, INFINITY, si, stack, err, wk)) break;
        if (is_black(beta)) break;
        BVert& v = path[bounces + 1];
        BVert& prev = path[bounces];
        if (diff0 && bounces == 0) {  // camera-ray differentials for the first hit's textures
            const V3 n = si.n;
            const real d = -dot(n, si.p);
            const real tx = (-dot(n, rxo) - d) / dot(n, rxd);
            const real ty = (-dot(n, rxo) - d) / dot(n, ryd);
            si.dpdx = (rxo + rxd * tx) - si.p;
            si.dpdy = (rxo + ryd * ty) - si.p;
        } else {
            si.dpdx = v3(0, 0, 0);
            si.dpdy = v3(0, 0, 0);
        }
        v.type = BV_SURFACE;
        v.delta = 0;
        v.light = si.light;
        v.p = si.p;
        v.n = si.n;
        v.perr = si.perr;
        v.wo = -rd;
        v.beta = beta;
        v.pdf_rev = 0;
        v.pdf_fwd = bv_convert(pdf_fwd, prev, v);
        if (!make_bsdf<LM, TEX>(sv, si, v.f, nullptr)) v.f.lobe = LOBE_NONE;
        ++bounces;
        if (bounces >= max_depth || v.f.lobe == LOBE_NONE) break;
        V3 wi;
        uint32_t stype = 0;
        real pdf = 0;
        const Spec fv = bsdf_sample<LM>(v.f, v.wo, wi, rng_2d(rng), pdf, BSDF_ALL, stype, nullptr);
        if (is_black(fv) || pdf == 0) break;
        beta = beta * (fv * absdot(wi, v.f.ns) / pdf);
        pdf_fwd = pdf;
        pdf_rev = bsdf_pdf<LM>(v.f, wi, v.wo, BSDF_ALL, nullptr);
        if (stype & BSDF_SPECULAR) {
            v.delta = 1;
            pdf_fwd = pdf_rev = 0;
        }
        if (importance) {
            beta = beta * bdpt_shading_fix(v.f, v.wo, wi);
            // specular transmission scales radiance by (eta_i / eta_t)^2 (the BSDF applies it);
            // importance is not scaled (PBRT's TransportMode), so light paths undo it
            if (v.f.lobe == LOBE_FRESNEL_SPECULAR && (stype & BSDF_TRANSMISSION)) {
                const bool entering = dot(v.wo, v.f.ns) > 0;
                const real ei = entering ? 1.0f : v.f.eta, et = entering ? v.f.eta : 1.0f;
                beta = beta * ((et * et) / (ei * ei));
            }
        }
        prev.pdf_rev = bv_convert(pdf_rev, v, prev);
        ro = offset_origin(si.p, si.perr, si.n, wi);
        rd = wi;
    }
    return bounces;
}

// MISWeight: the balance heuristic over every strategy that could have made the same path, from
// the ratio chain of forward and reverse densities; the connection endpoints' densities (and the
// resampled endpoint of s = 1 or t = 1) replace the stored ones for the evaluation.
template <int LM>
__device__ real bdpt_mis(const SceneView& sv, const BCam& cam, const BVert* lp, const BVert* cp, const BVert& sampled,
                         int s, int t) {
    if (s + t == 2) return 1;
    const BVert* qs = s > 0 ? (s == 1 ? &sampled : &lp[s - 1]) : nullptr;
    const BVert* pt = t > 0 ? (t == 1 ? &sampled : &cp[t - 1]) : nullptr;
    const BVert* qsm = s > 1 ? &lp[s - 2] : nullptr;
    const BVert* ptm = t > 1 ? &cp[t - 2] : nullptr;
    // overridden reverse densities of the four vertices around the connection
    real pt_rev = 0, ptm_rev = 0, qs_rev = 0, qsm_rev = 0;
    if (pt) {
        if (s > 0) pt_rev = bv_pdf<LM>(sv, cam, *qs, qsm, *pt);
        else pt_rev = bv_pdf_light_origin(sv, *pt);  // pt is an emitting surface
    }
    if (ptm) {
        if (s > 0) ptm_rev = bv_pdf<LM>(sv, cam, *pt, qs, *ptm);
        else {  // PdfLight of the emitting surface pt toward ptm
            BVert lv = *pt;
            lv.type = BV_LIGHT;
            ptm_rev = bv_pdf_light(sv, lv, *ptm);
        }
    }
    if (qs) qs_rev = bv_pdf<LM>(sv, cam, *pt, ptm, *qs);
    if (qsm) qsm_rev = bv_pdf<LM>(sv, cam, *qs, pt, *qsm);
    auto remap0 = [](real f) -> real { return f != 0 ? f : 1; };
    real sum = 0, ri = 1;
    for (int i = t - 1; i > 0; --i) {
        const BVert& v = i == t - 1 ? *pt : cp[i];
        const real rev = i == t - 1 ? pt_rev : (i == t - 2 ? ptm_rev : cp[i].pdf_rev);
        ri *= remap0(rev) / remap0(v.pdf_fwd);
        const bool d_i = i == t - 1 ? false : cp[i].delta != 0;
        const bool d_im = (i - 1 == t - 1) ? false : cp[i - 1].delta != 0;
        if (!d_i && !d_im) sum += ri;
    }
    ri = 1;
    for (int i = s - 1; i >= 0; --i) {
        const BVert& v = i == s - 1 ? *qs : lp[i];
        const real rev = i == s - 1 ? qs_rev : (i == s - 2 ? qsm_rev : lp[i].pdf_rev);
        ri *= remap0(rev) / remap0(v.pdf_fwd);
        const bool d_i = i == s - 1 ? false : lp[i].delta != 0;
        const bool d_light = i > 0 ? lp[i - 1].delta != 0 : bv_delta_light(sv, s == 1 ? sampled : lp[0]);
        if (!d_i && !d_light) sum += ri;
    }
    return 1 / (1 + sum);
}

// Film writes: a camera sample through the reference's Gaussian filter (Camera::addSample), with
// its footprint and table lookup; a light-to-camera splat through the same footprint and weights,
// without a weight sum: the resolve divides it by the weight the camera samples of spp per pixel
// put on that pixel in expectation (film_weight_1d), so that both parts estimate the same filtered
// image, borders included.
__device__ __forceinline__ void bdpt_add_sample(const SceneView& sv, const RenderParams& rp, real pfx, real pfy, Spec L) {
    const int W = sv.width, H = sv.height;
    const int px0 = max((int)xceil(pfx - 1.0f), 0), py0 = max((int)xceil(pfy - 1.0f), 0);
    const int px1 = min((int)xfloor(pfx + 1.0f) + 1, W), py1 = min((int)xfloor(pfy + 1.0f) + 1, H);
    for (int y = py0; y < py1; ++y)
        for (int x = px0; x < px1; ++x) {
            const real fdx = xabs((x - pfx - 0.5f) * 1.0f * 16);
            const real fdy = xabs((y - pfy - 0.5f) * 1.0f * 16);
            const int ix = min((int)xfloor(fdx), 15), iy = min((int)xfloor(fdy), 15);
            const real wgt = __ldg(sv.filter + iy * 16 + ix);
            double* fp = rp.film + 4 * ((size_t)y * W + x);
            atomicAdd(fp + 0, (double)(L.r * wgt));
            atomicAdd(fp + 1, (double)(L.g * wgt));
            atomicAdd(fp + 2, (double)(L.b * wgt));
            atomicAdd(fp + 3, (double)wgt);
        }
}

// only >= 0: the single strategy s = only / 100, t = only % 100, unweighted (each strategy alone
// estimates its own paths; a debugging view of the estimator, as PBRT's visualizeStrategies).
__device__ __forceinline__ void bdpt_add_splat(const SceneView& sv, real rx, real ry, Spec L, double* splat) {
    const int W = sv.width, H = sv.height;
    const int px0 = max((int)xceil(rx - 1.0f), 0), py0 = max((int)xceil(ry - 1.0f), 0);
    const int px1 = min((int)xfloor(rx + 1.0f) + 1, W), py1 = min((int)xfloor(ry + 1.0f) + 1, H);
    for (int y = py0; y < py1; ++y)
        for (int x = px0; x < px1; ++x) {
            const real fdx = xabs((x - rx - 0.5f) * 1.0f * 16);
            const real fdy = xabs((y - ry - 0.5f) * 1.0f * 16);
            const int ix = min((int)xfloor(fdx), 15), iy = min((int)xfloor(fdy), 15);
            const real wgt = __ldg(sv.filter + iy * 16 + ix);
            double* sp = splat + 3 * ((size_t)y * W + x);
            atomicAdd(sp + 0, (double)(L.r * wgt));
            atomicAdd(sp + 1, (double)(L.g * wgt));
            atomicAdd(sp + 2, (double)(L.b * wgt));
        }
}

#ifndef LTS_BDPT_MIN_BLOCKS
// Resident blocks per SM the register budget is cut for: the kernel is bound by latency, and more
// warps pay even with spills (Msamples/s on the bench's box: 2 blocks 5.44, 3 (168 registers, no
// spills) 5.84, 4 6.27, 5 6.60, 6 7.14, 8 (64 registers) 8.19; the traversal stacks' shared
// memory allows 9).
#define LTS_BDPT_MIN_BLOCKS 8
#endif
template <int LM, bool TEX>
__global__ __launch_bounds__(kThreads, LTS_BDPT_MIN_BLOCKS) void k_bdpt(const SceneView sv, const RenderParams rp, int nleaf,
                                                      double* __restrict__ splat, int only) {
    __shared__ uint32_t s_stack[kStack * kThreads];
    const int tid = threadIdx.y * kBX + threadIdx.x;
    uint32_t* stack = s_stack + tid;
    const int i = rp.x0 + blockIdx.x * kBX + threadIdx.x;
    const int j = rp.y0 + blockIdx.y * kBY + threadIdx.y;
    if (i >= rp.x1 || j >= rp.y1) return;
    const BCam cam = bdpt_camera(sv);
    const int W = sv.width, H = sv.height;
    const real rx = (real)(W - 1), ry = (real)(H - 1);
    Rng rng;
    rng.key = rp.seed + wang_hash((uint32_t)(j * W + i));
    unsigned long long rays = 0;
    Work wk{0u, 0u};
    const int maxb = min(rp.max_bounce, kBdptMaxBounce);
    BVert cp[kBdptMaxBounce + 2], lp[kBdptMaxBounce + 1];
    // the pixel's samples are split over gridDim.z slices of the grid (sample s_ix draws the same
    // numbers whatever the split; the film and splat sums are atomic)
    for (int s_ix = (int)blockIdx.z; s_ix < rp.spp; s_ix += (int)gridDim.z) {
        rng.sample = (uint32_t)s_ix;
        rng.draw = 0;
        // camera subpath (GenerateCameraSubpath): the path tracer's primary ray and differentials
        const F2 fs = rng_2d(rng);
        (void)rng_2d(rng);
        const real pfx = (real)(i + fs.x), pfy = (real)(j + fs.y);
        const V3 rd = normalize(cam.llc + cam.right * (pfx / rx) + cam.up * (pfy / ry) - cam.o);
        const V3 dx0 = normalize(cam.llc + cam.right * ((pfx + 1) / rx) + cam.up * (pfy / ry) - cam.o);
        const V3 dy0 = normalize(cam.llc + cam.right * (pfx / rx) + cam.up * ((pfy + 1) / ry) - cam.o);
        const V3 rxd = rd + (dx0 - rd) * rp.spp_scale, ryd = rd + (dy0 - rd) * rp.spp_scale;
        BVert& c0 = cp[0];
        c0.type = BV_CAMERA;
        c0.delta = 0;
        c0.light = -1;
        c0.p = cam.o;
        c0.n = v3(0, 0, 0);
        c0.perr = v3(0, 0, 0);
        c0.beta = spec(1.0f);
        c0.pdf_fwd = c0.pdf_rev = 0;
        c0.f.lobe = LOBE_NONE;
        real cpx, cpy, cos_t;
        bdpt_raster(cam, rd, cpx, cpy, cos_t);
        const int n_cam = 1 + bdpt_walk<LM, TEX>(sv, nleaf, cp, cam.o, rd, spec(1.0f), bdpt_pdf_dir(cam, cos_t), maxb + 1,
                                        false, rng, true, cam.o, rxd, ryd, stack, rp.err, wk, rays);
        // light subpath (GenerateLightSubpath)
        int n_light = 0;
        {
            real lpick;
            const int li = bdpt_pick_light(sv, rng_1d(rng), lpick);
            const F2 u1 = rng_2d(rng), u2 = rng_2d(rng);
            const DevLight& L = sv.lights[li];
            BVert& l0 = lp[0];
            l0.type = BV_LIGHT;
            l0.light = li;
            l0.pdf_rev = 0;
            l0.f.lobe = LOBE_NONE;
            V3 dir, nl;
            real pdf_pos = 0, pdf_dir = 0;
            Spec Le = spec(0.0f);
            if (L.kind == 0) {  // point on the triangle (Triangle::sample), cosine-weighted direction
                // weights of p0, p1, p2 as Triangle::sample draws them (Triangle.cu:232-259); the
                // emitting side is the surface normal make_si gives a hit there
                const real su = xsqrt(u1.x);
                const real w0 = 1 - su, w1 = u1.y * su, w2 = 1 - w0 - w1;
                V3 p0, p1, p2;
                prim_tri(sv, L.prim, p0, p1, p2);
                SI ls;
                make_si(sv, L.prim, v3(0, 0, 1), w1, w2, 1.0f, ls);
                nl = ls.n;
                l0.p = p0 * w0 + p1 * w1 + p2 * w2;
                l0.perr = (vabs(p0 * w0) + vabs(p1 * w1) + vabs(p2 * w2)) * gamma_n(6);
                l0.n = nl;
                l0.delta = 0;
                const real r = xsqrt(u2.x), th = mul_dc(u2.y, LTS_2PI);
                const real lx = r * xcos(th), ly = r * xsin(th), lz = xsqrt(xmax(0.0f, 1 - lx * lx - ly * ly));
                V3 a, b;
                coordinate_system(nl, a, b);
                dir = normalize(a * lx + b * ly + nl * lz);
                pdf_pos = 1 / L.area;
                pdf_dir = lz * LTS_INV_PI_F;
                Le = Spec{L.L[0], L.L[1], L.L[2]};
            } else {  // point light: uniform sphere of directions
                const real z = 1 - 2 * u1.x, r = xsqrt(xmax(0.0f, 1 - z * z)), ph = mul_dc(u1.y, LTS_2PI);
                dir = v3(r * xcos(ph), r * xsin(ph), z);
                nl = dir;
                l0.p = v3(L.p[0], L.p[1], L.p[2]);
                l0.perr = v3(0, 0, 0);
                l0.n = v3(0, 0, 0);
                l0.delta = 0;
                pdf_pos = 1;
                pdf_dir = (real)(0.25 * LTS_INV_PI_F);
                Le = Spec{L.L[0], L.L[1], L.L[2]};
            }
            if (pdf_pos > 0 && pdf_dir > 0 && !is_black(Le)) {
                l0.beta = Le;
                l0.pdf_fwd = pdf_pos * lpick;
                const Spec beta = Le * (absdot(nl, dir) / (lpick * pdf_pos * pdf_dir));
                const V3 org = offset_origin(l0.p, l0.perr, l0.n, dir);
                n_light = 1 + bdpt_walk<LM, TEX>(sv, nleaf, lp, org, dir, beta, pdf_dir, maxb, true, rng, false, org, dir, dir,
                                        stack, rp.err, wk, rays);
            }
        }
        // every strategy
        Spec L = spec(0.0f);
        for (int t = 1; t <= n_cam; ++t) {
            for (int s = 0; s <= n_light; ++s) {
                const int depth = t + s - 2;
                if ((s == 1 && t == 1) || depth < 0 || depth > maxb) continue;
                if (only >= 0 && (s != only / 100 || t != only % 100)) continue;
                Spec c = spec(0.0f);
                BVert sampled;
                sampled.type = BV_CAMERA;
                sampled.delta = 0;
                sampled.light = -1;
                bool splat_it = false;
                real spx = 0, spy = 0;
                if (t > 1 && s != 0 && cp[t - 1].type == BV_LIGHT) continue;
                if (s == 0) {  // the camera path's end is on a light
                    const BVert& pt = cp[t - 1];
                    if (bv_is_light(pt)) c = bv_le(sv, pt, normalize(cp[t - 2].p - pt.p)) * pt.beta;
                } else if (t == 1) {  // connect the light path's end to the camera
                    const BVert& qs = lp[s - 1];
                    if (bv_connectible(qs)) {
                        const V3 d = cam.o - qs.p;
                        const real l2 = len2(d);
                        const V3 wi = d * xsqrt(1 / l2);
                        real cos_c;
                        if (l2 > 0 && bdpt_raster(cam, -wi, spx, spy, cos_c)) {
                            const real pdf = l2 / cos_c;  // solid angle at qs (lens area 1)
                            sampled.type = BV_CAMERA;
                            sampled.p = cam.o;
                            sampled.n = v3(0, 0, 0);
                            sampled.perr = v3(0, 0, 0);
                            sampled.beta = spec(bdpt_we(cam, cos_c) / pdf);
                            sampled.pdf_fwd = sampled.pdf_rev = 0;
                            sampled.f.lobe = LOBE_NONE;
                            // qs is a surface vertex: s >= 2 whenever t = 1
                            c = qs.beta * bv_f<LM>(qs, sampled, true) * sampled.beta * absdot(wi, qs.f.ns);
                            if (!is_black(c)) {
                                ++rays;
                                if (!bdpt_visible(sv, nleaf, qs, sampled, stack, rp.err, wk)) c = spec(0.0f);
                            }
                            splat_it = true;
                        }
                    }
                } else if (s == 1) {  // connect the camera path's end to a sampled light point
                    const BVert& pt = cp[t - 1];
                    if (bv_connectible(pt)) {
                        real lpick;
                        const int li = bdpt_pick_light(sv, rng_1d(rng), lpick);
                        const F2 ul = rng_2d(rng);
                        const DevLight& Lt = sv.lights[li];
                        SI psi;
                        psi.p = pt.p;
                        psi.perr = pt.perr;
                        psi.n = pt.n;
                        LightSample ls;
                        const bool delta = sample_li(sv, Lt, psi, ul, ls);
                        if (ls.pdf > 0 && !is_black(ls.Li)) {
                            sampled.type = BV_LIGHT;
                            sampled.light = li;
                            sampled.delta = 0;
                            sampled.p = ls.p1;
                            sampled.n = delta ? v3(0, 0, 0) : ls.n1;
                            sampled.perr = ls.perr1;
                            sampled.beta = ls.Li / (ls.pdf * lpick);
                            sampled.pdf_rev = 0;
                            sampled.f.lobe = LOBE_NONE;
                            sampled.pdf_fwd = bv_pdf_light_origin(sv, sampled);
                            c = pt.beta * bv_f<LM>(pt, sampled, false) * sampled.beta;
                            c = c * absdot(ls.wi, pt.f.ns);
                            if (!is_black(c)) {
                                ++rays;
                                if (!bdpt_visible(sv, nleaf, pt, sampled, stack, rp.err, wk)) c = spec(0.0f);
                            }
                        }
                    }
                } else {  // connect two surface vertices (s >= 2, t >= 2)
                    const BVert& qs = lp[s - 1];
                    const BVert& pt = cp[t - 1];
                    if (bv_connectible(qs) && bv_connectible(pt)) {
                        c = qs.beta * bv_f<LM>(qs, pt, true) * bv_f<LM>(pt, qs, false) * pt.beta;
                        if (!is_black(c)) {  // generalized geometry term G with visibility
                            V3 d = qs.p - pt.p;
                            real g = 1 / len2(d);
                            d = d * xsqrt(g);
                            g *= absdot(qs.f.ns, d) * absdot(pt.f.ns, d);
                            ++rays;
                            c = bdpt_visible(sv, nleaf, qs, pt, stack, rp.err, wk) ? c * g : spec(0.0f);
                        }
                    }
                }
                if (is_black(c)) continue;
                if (only < 0) c = c * bdpt_mis<LM>(sv, cam, lp, cp, sampled, s, t);
                if (splat_it) {
                    bdpt_add_splat(sv, spx, spy, c, splat);
                } else {
                    L = L + c;
                }
            }
        }
        bdpt_add_sample(sv, rp, pfx, pfy, L);
    }
    const unsigned mask = __activemask();
    const unsigned tot = __reduce_add_sync(mask, (unsigned)rays);
    const unsigned lane = (unsigned)tid & 31u;
    if ((mask & ((1u << lane) - 1u)) == 0u && rp.counters) atomicAdd(rp.counters, (unsigned long long)tot);
}

}  // namespace
}  // namespace lts
