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
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "dev_common.cuh"
#include "dev_math.cuh"
#include "tracer.cuh"

namespace lts {
namespace {

// Float forms of the reference's double-precision comparisons:
//   u > 1.0 - SHADOW_EPSILON  <=>  u >= kOneMinusEpsUp   (Triangle.cu:116,122)
//   u > 1.0 + SHADOW_EPSILON  <=>  u >= kOnePlusEpsUp    (Triangle.cu:72,78)
//   x > 1e-4                  <=>  x >= 0.0001f          (models/Microfacet.cuh:32)
//   cosT > .9999              <=>  cosT >= kOneMinusEpsUp (models/Microfacet.cuh:56)
#define kShadowEps 0.0001f
#define kOneMinusEpsUp __int_as_float(0x3f7ff973)
#define kOnePlusEpsUp __int_as_float(0x3f800347)
#define kSlabScale (1.0f + 2.0f * gamma_n(3))

constexpr int kStack = 40;
constexpr int kBX = 16, kBY = 8, kThreads = kBX * kBY;

enum BxdfType : uint32_t {
    BSDF_REFLECTION = 1u,
    BSDF_TRANSMISSION = 2u,
    BSDF_DIFFUSE = 4u,
    BSDF_GLOSSY = 8u,
    BSDF_SPECULAR = 16u,
    BSDF_ALL = 31u
};
enum LobeKind : int { LOBE_NONE = 0, LOBE_LAMBERT, LOBE_OREN_NAYAR, LOBE_FRESNEL_SPECULAR, LOBE_SPECULAR_REFL, LOBE_MICROFACET };

// ------------------------------------------------------------------ sampler (project Philox)
struct Rng {
    uint32_t key, sample, draw;
    uint32_t w0, w1, w2, w3;
};
__device__ __forceinline__ void philox_block(Rng& r) {
    uint32_t c0 = r.draw >> 2, c1 = r.sample, c2 = 0u, c3 = 0u, k0 = r.key, k1 = 0x4c54530au;
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    r.w0 = c0;
    r.w1 = c1;
    r.w2 = c2;
    r.w3 = c3;
}
__device__ __forceinline__ uint32_t wang_hash(uint32_t a) {
    a = (a ^ 61u) ^ (a >> 16);
    a = a + (a << 3);
    a = a ^ (a >> 4);
    a = a * 0x27d4eb2du;
    a = a ^ (a >> 15);
    return a;
}
__device__ __forceinline__ float rng_1d(Rng& r) {
    if ((r.draw & 3u) == 0u) philox_block(r);
    const uint32_t x = r.w0;
    r.w0 = r.w1;
    r.w1 = r.w2;
    r.w2 = r.w3;
    ++r.draw;
    return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f);
}
struct F2 {
    float x, y;
};
// Sampler::uniformSample (Sampler.cuh:70-73) as the reference's host build evaluates it:
// the constructor arguments are evaluated right to left, so x receives the second draw.
__device__ __forceinline__ F2 rng_2d(Rng& r) {
    const float a = rng_1d(r);
    const float b = rng_1d(r);
    return F2{b, a};
}

// ------------------------------------------------------------------ event hash (record mode)
__device__ __forceinline__ void fnv_mix(uint64_t& h, uint64_t v) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        h ^= (v >> (8 * i)) & 0xffull;
        h *= 0x100000001b3ull;
    }
}

// ------------------------------------------------------------------ single-sample trace (record mode)
struct Tracer16 {
    float* out;
    int n;
    __device__ void put(float tag, float a = 0, float b = 0, float c = 0, float d = 0, float e = 0, float f = 0,
                        float g = 0, float h = 0, float i = 0, float j = 0, float k = 0, float l = 0, float m = 0,
                        float o = 0, float p = 0) {
        if (!out || n >= 64) return;
        float* r = out + 16 * n++;
        r[0] = tag; r[1] = a; r[2] = b; r[3] = c; r[4] = d; r[5] = e; r[6] = f; r[7] = g; r[8] = h;
        r[9] = i; r[10] = j; r[11] = k; r[12] = l; r[13] = m; r[14] = o; r[15] = p;
    }
};

// ------------------------------------------------------------------ geometry fetch
__device__ __forceinline__ V3 f4v(float4 a) { return v3(a.x, a.y, a.z); }
__device__ __forceinline__ void prim_tri(const SceneView& sv, int prim, V3& p0, V3& p1, V3& p2) {
    p0 = f4v(__ldg(sv.prim_v + 3 * prim));
    p1 = f4v(__ldg(sv.prim_v + 3 * prim + 1));
    p2 = f4v(__ldg(sv.prim_v + 3 * prim + 2));
}
__device__ __forceinline__ V3 normal_at(const SceneView& sv, int idx) {
    return v3(__ldg(sv.normals + 3 * idx), __ldg(sv.normals + 3 * idx + 1), __ldg(sv.normals + 3 * idx + 2));
}

// ------------------------------------------------------------------ triangle tests
// Triangle::intersect test part (shapes/Triangle.cu:94-128).
__device__ __forceinline__ bool tri_test(V3 p0, V3 p1, V3 p2, V3 o, V3 d, float tmax, float& t_out, float& u_out,
                                         float& v_out, float& inv_out) {
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const V3 pv = cross(d, e2);
    const float det = dot(e1, pv);
    if (det == 0) return false;
    const float inv = __frcp_rn(det);  // == (float)(1.0 / (double)det)
    const V3 tv = o - p0;
    const float u = inv * dot(tv, pv);
    if (u < kShadowEps || u >= kOneMinusEpsUp) return false;
    const V3 qv = cross(tv, e1);
    const float v = inv * dot(d, qv);
    if (v < kShadowEps || u + v >= kOneMinusEpsUp) return false;
    const float t = inv * dot(e2, qv);
    if (!(t > 0 && t < tmax)) return false;
    t_out = t;
    u_out = u;
    v_out = v;
    inv_out = inv;
    return true;
}
// Triangle::simpleIntersect (shapes/Triangle.cu:50-84): swapped edges, grown bound.
__device__ __forceinline__ bool tri_test_shadow(V3 p0, V3 p1, V3 p2, V3 o, V3 d, float tmax) {
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const V3 pv = cross(d, e1);
    const float det = dot(e2, pv);
    if (det == 0) return false;
    const float inv = __frcp_rn(det);
    const V3 tv = o - p0;
    const float u = inv * dot(tv, pv);
    if (u < kShadowEps || u >= kOnePlusEpsUp) return false;
    const V3 qv = cross(tv, e2);
    const float v = inv * dot(d, qv);
    if (v < kShadowEps || u + v >= kOnePlusEpsUp) return false;
    const float t = inv * dot(e1, qv);
    return t > 0 && t < tmax;
}

// ------------------------------------------------------------------ surface interaction
struct SI {
    V3 p, perr, wo, n;  // Interaction
    V3 dpdu, dpdv;      // geometric partials
    V3 sn, sdpdu;       // shading normal and tangent
    V3 dpdx, dpdy;      // computeDifferentials
    int prim;
};

__device__ __forceinline__ void coordinate_system(V3 v1, V3& v2, V3& v3o) {
    // Geometry.cuh:250-258
    if (fabsf(v1.x) > fabsf(v1.y))
        v2 = v3(-v1.z, 0, v1.x) * rsqrt_q3(v1.x * v1.x + v1.z * v1.z);
    else
        v2 = v3(0, v1.z, -v1.y) * rsqrt_q3(v1.y * v1.y + v1.z * v1.z);
    v3o = cross(v1, v2);
}

// Builds the SurfaceInteraction of a hit (Triangle.cu:128-199 and the SurfaceInteraction
// constructor, geometry/Interaction.cuh:85-116).
__device__ void make_si(const SceneView& sv, int prim, V3 p0, V3 p1, V3 p2, V3 d, float u, float v, float inv,
                        SI& si) {
    const float w = 1 - u - v;
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const int4 uvi = __ldg(sv.prim_uv + prim);
    float uv0x = 0, uv0y = 0, uv1x = 1, uv1y = 0, uv2x = 1, uv2y = 1;
    if (uvi.x >= 0) {
        uv0x = __ldg(sv.uvs + 2 * uvi.x); uv0y = __ldg(sv.uvs + 2 * uvi.x + 1);
        uv1x = __ldg(sv.uvs + 2 * uvi.y); uv1y = __ldg(sv.uvs + 2 * uvi.y + 1);
        uv2x = __ldg(sv.uvs + 2 * uvi.z); uv2y = __ldg(sv.uvs + 2 * uvi.z + 1);
    }
    const float d02x = uv0x - uv2x, d02y = uv0y - uv2y, d12x = uv1x - uv2x, d12y = uv1y - uv2y;
    const V3 dp02 = p0 - p2, dp12 = p1 - p2;
    const float determinant = d02x * d12y - d02y * d12x;
    V3 dpdu, dpdv;
    if (determinant == 0) {
        coordinate_system(normalize(cross(e2, e1)), dpdu, dpdv);
    } else {
        // the reference scales by the ray's invDet, not the uv determinant (Triangle.cu:148-149)
        dpdu = (dp02 * d12y - dp12 * d02y) * inv;
        dpdv = (dp02 * -d12x + dp12 * d02x) * inv;
    }
    const float xs = fabsf(w * p0.x) + fabsf(u * p1.x) + fabsf(v * p2.x);
    const float ys = fabsf(w * p0.y) + fabsf(u * p1.y) + fabsf(v * p2.y);
    const float zs = fabsf(w * p0.z) + fabsf(u * p1.z) + fabsf(v * p2.z);
    si.perr = v3(xs, ys, zs) * gamma_n(7);
    si.p = p0 * w + p1 * u + p2 * v;
    si.wo = -d;
    si.dpdu = dpdu;
    si.dpdv = dpdv;
    si.n = normalize(cross(dpdu, dpdv));
    si.sn = si.n;
    si.sdpdu = dpdu;
    si.prim = prim;
    const int4 ni = __ldg(sv.prim_n + prim);
    if (ni.x >= 0) {
        const V3 n0 = normal_at(sv, ni.x), n1 = normal_at(sv, ni.y), n2 = normal_at(sv, ni.z);
        const V3 ns = normalize(n0 * w + n1 * u + n2 * v);
        V3 ss = si.dpdu;
        V3 ts = cross(ns, ss);
        if (len2(ts) > 0.0f) {
            ts = normalize(ts);
            ss = cross(ts, ns);
        } else {
            coordinate_system(ns, ss, ts);
        }
        si.sn = normalize(cross(ss, ts));         // setShaddingGeometry
        si.n = face_towards(si.n, si.sn);
        si.sdpdu = ss;
        si.n = face_towards(si.n, si.sn);         // Triangle.cu:196
    }
}

// ------------------------------------------------------------------ BVH traversal
struct TraceRay {
    V3 o, d, inv;
    int neg[3];
};
__device__ __forceinline__ TraceRay make_trace_ray(V3 o, V3 d) {
    TraceRay r;
    r.o = o;
    r.d = d;
    r.inv = v3(__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z));
    r.neg[0] = r.inv.x < 0;
    r.neg[1] = r.inv.y < 0;
    r.neg[2] = r.inv.z < 0;
    return r;
}
// Bounds3::simpleIntersect (geometry/Bound.cuh:199-227), returning the entry distance.
__device__ __forceinline__ bool slab(const TraceRay& r, float tmax_ray, float mnx, float mny, float mnz, float mxx,
                                     float mxy, float mxz, float& tentry) {
    float tMin = ((r.neg[0] ? mxx : mnx) - r.o.x) * r.inv.x;
    float tMax = ((r.neg[0] ? mnx : mxx) - r.o.x) * r.inv.x;
    const float tyMin = ((r.neg[1] ? mxy : mny) - r.o.y) * r.inv.y;
    float tyMax = ((r.neg[1] ? mny : mxy) - r.o.y) * r.inv.y;
    tMax *= kSlabScale;
    tyMax *= kSlabScale;
    if (tMin > tyMax || tyMin > tMax) return false;
    if (tyMin > tMin) tMin = tyMin;
    if (tyMax < tMax) tMax = tyMax;
    const float tzMin = ((r.neg[2] ? mxz : mnz) - r.o.z) * r.inv.z;
    float tzMax = ((r.neg[2] ? mnz : mxz) - r.o.z) * r.inv.z;
    tzMax *= kSlabScale;
    if (tMin > tzMax || tzMin > tMax) return false;
    if (tzMin > tMin) tMin = tzMin;
    if (tzMax < tMax) tMax = tzMax;
    tentry = tMin;
    return (tMin < tmax_ray) && (tMax > 0);
}

template <bool ANY>
__device__ __forceinline__ bool leaf_test(const SceneView& sv, int leaf, const TraceRay& r, float& tmax, int& best,
                                          float& bu, float& bv, float& binv) {
    const float4 a = __ldg(sv.leaf_v + 3 * leaf), b = __ldg(sv.leaf_v + 3 * leaf + 1), c = __ldg(sv.leaf_v + 3 * leaf + 2);
    if (ANY) return tri_test_shadow(f4v(a), f4v(b), f4v(c), r.o, r.d, tmax);
    float t, u, v, inv;
    if (tri_test(f4v(a), f4v(b), f4v(c), r.o, r.d, tmax, t, u, v, inv)) {
        tmax = t;
        best = __float_as_int(a.w);
        bu = u;
        bv = v;
        binv = inv;
    }
    return false;
}

// BVH::intersect / simpleIntersect (acceleration/BVH.cuh:331-398).  Returns the hit primitive
// (closest) or 1/-1 (any), -1 for a miss.  `stack` is this thread's column of the shared stack.
struct Work {
    uint32_t nodes, tris;
};

template <bool ANY>
__device__ int traverse(const SceneView& sv, int nleaf, const TraceRay& r, float& tmax, float& bu, float& bv,
                        float& binv, uint32_t* stack, uint32_t* err, Work& wk) {
    int best = -1;
    float te;
    const float* rb = sv.root_bounds;
    if (!slab(r, tmax, __ldg(rb), __ldg(rb + 1), __ldg(rb + 2), __ldg(rb + 3), __ldg(rb + 4), __ldg(rb + 5), te))
        return -1;
    if (nleaf == 1) {
        ++wk.tris;
        if (leaf_test<ANY>(sv, 0, r, tmax, best, bu, bv, binv)) return 1;
        return ANY ? -1 : best;
    }
    int node = 0, sp = 0;
    for (;;) {
        const BvhNode* nd = sv.nodes + node;
        const float4 a = __ldg(&nd->a), b = __ldg(&nd->b), c = __ldg(&nd->c);
        const int4 lr = __ldg(&nd->d);
        ++wk.nodes;
        float tl, tr;
        bool hl = slab(r, tmax, a.x, a.y, a.z, a.w, b.x, b.y, tl);
        bool hr = slab(r, tmax, b.z, b.w, c.x, c.y, c.z, c.w, tr);
        if (hl && lr.x < 0) {
            ++wk.tris;
            if (leaf_test<ANY>(sv, ~lr.x, r, tmax, best, bu, bv, binv)) return 1;
            hl = false;
        }
        if (hr && lr.y < 0) {
            ++wk.tris;
            if (leaf_test<ANY>(sv, ~lr.y, r, tmax, best, bu, bv, binv)) return 1;
            hr = false;
        }
        if (hl && hr) {
            const bool left_first = tl <= tr;
            if (sp >= kStack) {
                atomicOr(err, DEV_ERR_STACK_OVERFLOW);
                return ANY ? -1 : best;
            }
            stack[(sp++) * kThreads] = left_first ? lr.y : lr.x;
            node = left_first ? lr.x : lr.y;
        } else if (hl) {
            node = lr.x;
        } else if (hr) {
            node = lr.y;
        } else {
            if (sp == 0) break;
            node = stack[(--sp) * kThreads];
        }
    }
    return ANY ? -1 : best;
}

struct Hit {
    bool found;
    SI si;
};

__device__ __forceinline__ bool scene_intersect(const SceneView& sv, int nleaf, V3 o, V3 d, float tmax, SI& si,
                                                uint32_t* stack, uint32_t* err, Work& wk) {
    const TraceRay r = make_trace_ray(o, d);
    float bu = 0, bv = 0, binv = 0;
    const int prim = traverse<false>(sv, nleaf, r, tmax, bu, bv, binv, stack, err, wk);
    if (prim < 0) return false;
    V3 p0, p1, p2;
    prim_tri(sv, prim, p0, p1, p2);
    make_si(sv, prim, p0, p1, p2, d, bu, bv, binv, si);
    return true;
}
__device__ __forceinline__ bool scene_occluded(const SceneView& sv, int nleaf, V3 o, V3 d, float tmax, uint32_t* stack,
                                               uint32_t* err, Work& wk) {
    const TraceRay r = make_trace_ray(o, d);
    float bu, bv, binv;
    return traverse<true>(sv, nleaf, r, tmax, bu, bv, binv, stack, err, wk) > 0;
}

// ------------------------------------------------------------------ rays from interactions
// offsetRayOrigin (Geometry.cuh:782-797)
__device__ __forceinline__ V3 offset_origin(V3 p, V3 perr, V3 n, V3 w) {
    const float dd = dot(vabs(n), perr);
    V3 off = n * dd;
    if (dot(w, n) < 0) off = -off;
    V3 po = p + off;
    if (off.x > 0) po.x = next_float_up(po.x); else if (off.x < 0) po.x = next_float_down(po.x);
    if (off.y > 0) po.y = next_float_up(po.y); else if (off.y < 0) po.y = next_float_down(po.y);
    if (off.z > 0) po.z = next_float_up(po.z); else if (off.z < 0) po.z = next_float_down(po.z);
    return po;
}

// ------------------------------------------------------------------ textures
__constant__ unsigned char c_perm[512];
__constant__ float c_marble[10][3];

__device__ __forceinline__ float noise_weight(float t) {
    const float t3 = t * t * t, t4 = t3 * t;
    return 6 * t4 * t - 15 * t4 + 10 * t3;
}
__device__ __forceinline__ float lerpf(float t, float a, float b) { return (1 - t) * a + t * b; }
__device__ __forceinline__ float grad(int x, int y, int z, float dx, float dy, float dz) {
    int h = c_perm[c_perm[c_perm[x] + y] + z];
    h &= 15;
    const float u = h < 8 || h == 12 || h == 13 ? dx : dy;
    const float v = h < 4 || h == 12 || h == 13 ? dy : dz;
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}
// textures/Procedural.cuh:130-155 (improved Perlin noise)
__device__ float perlin(float x, float y, float z) {
    int ix = (int)floorf(x), iy = (int)floorf(y), iz = (int)floorf(z);
    const float dx = x - ix, dy = y - iy, dz = z - iz;
    ix &= 255;
    iy &= 255;
    iz &= 255;
    const float w000 = grad(ix, iy, iz, dx, dy, dz);
    const float w100 = grad(ix + 1, iy, iz, dx - 1, dy, dz);
    const float w010 = grad(ix, iy + 1, iz, dx, dy - 1, dz);
    const float w001 = grad(ix, iy, iz + 1, dx, dy, dz - 1);
    const float w110 = grad(ix + 1, iy + 1, iz, dx - 1, dy - 1, dz);
    const float w011 = grad(ix, iy + 1, iz + 1, dx, dy - 1, dz - 1);
    const float w101 = grad(ix + 1, iy, iz + 1, dx - 1, dy, dz - 1);
    const float w111 = grad(ix + 1, iy + 1, iz + 1, dx - 1, dy - 1, dz - 1);
    const float wx = noise_weight(dx), wy = noise_weight(dy), wz = noise_weight(dz);
    const float x00 = lerpf(wx, w000, w100), x10 = lerpf(wx, w010, w110);
    const float x01 = lerpf(wx, w001, w101), x11 = lerpf(wx, w011, w111);
    const float y0 = lerpf(wy, x00, x10), y1 = lerpf(wy, x01, x11);
    return lerpf(wz, y0, y1);
}
__device__ __forceinline__ float smooth_step(float mn, float mx, float val) {
    const float v = clampf((val - mn) / (mx - mn), 0, 1);
    return v * v * (-2 * v + 3);
}
__device__ __forceinline__ float octaves_of(V3 dpdx, V3 dpdy, int max_oct) {
    const float l2 = fmaxf(len2(dpdx), len2(dpdy));
    return clampf(-1 - 0.5f * log2f(l2), 0, (float)max_oct);
}
// Procedural.cuh:161-179
__device__ float fbm(V3 p, V3 dpdx, V3 dpdy, float omega, int max_oct, uint64_t* sig) {
    const float n = octaves_of(dpdx, dpdy, max_oct);
    const int ni = (int)floorf(n);
    if (sig) fnv_mix(*sig, 0x400000000ull + (unsigned)ni);
    float sum = 0, lambda = 1, o = 1;
    for (int i = 0; i < ni; ++i) {
        sum += o * perlin(p.x * lambda, p.y * lambda, p.z * lambda);
        lambda *= 1.99f;
        o *= omega;
    }
    const float np = n - ni;
    sum += o * smooth_step(0.3f, 0.7f, np) * perlin(p.x * lambda, p.y * lambda, p.z * lambda);
    return sum;
}
// Procedural.cuh:181-205
__device__ float turbulence(V3 p, V3 dpdx, V3 dpdy, float omega, int max_oct, uint64_t* sig) {
    const float n = octaves_of(dpdx, dpdy, max_oct);
    const int ni = (int)floorf(n);
    if (sig) fnv_mix(*sig, 0x400000000ull + (unsigned)ni);
    float sum = 0, lambda = 1, o = 1;
    for (int i = 0; i < ni; ++i) {
        sum += o * fabsf(perlin(p.x * lambda, p.y * lambda, p.z * lambda));
        lambda *= 1.99f;
        o *= omega;
    }
    const float np = n - ni;
    sum += o * lerpf(smooth_step(0.3f, 0.7f, np), 0.2f, fabsf(perlin(p.x * lambda, p.y * lambda, p.z * lambda)));
    for (int i = ni; i < max_oct; ++i) {
        sum += o * 0.2f;
        o *= omega;
    }
    return sum;
}

__device__ Spec eval_texture(const DevTex& t, const SI& si, uint64_t* sig) {
    switch (t.kind) {
        case 1:  // FBmTexture (Procedural.cuh:207-225)
            return spec(fbm(si.p, si.dpdx, si.dpdy, t.v[1], (int)t.v[0], sig));
        case 2:  // WrinkledTexture (Procedural.cuh:227-245)
            return spec(turbulence(si.p, si.dpdx, si.dpdy, t.v[1], (int)t.v[0], sig));
        case 3: {  // MarbleTexture (Procedural.cuh:267-311)
            const float scale = t.v[2], var = t.v[3];
            const V3 p = si.p * scale;
            const float marble = p.y + var * fbm(p, si.dpdx * scale, si.dpdy * scale, t.v[1], (int)t.v[0], sig);
            float tt = 0.5f + 0.5f * sinf(marble);
            const int first = (int)floorf(tt * 6.0f);
            if (sig) fnv_mix(*sig, 0x500000000ull + (unsigned)first);
            tt = (tt * 6.0f - first);
            Spec c[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) c[k] = Spec{c_marble[first + k][0], c_marble[first + k][1], c_marble[first + k][2]};
            Spec s0 = c[0] * (1.0f - tt) + c[1] * tt;
            Spec s1 = c[1] * (1.0f - tt) + c[2] * tt;
            const Spec s2 = c[2] * (1.0f - tt) + c[3] * tt;
            s0 = s0 * (1.0f - tt) + s1 * tt;
            s1 = s1 * (1.0f - tt) + s2 * tt;
            return (s0 * (1.0f - tt) + s1 * tt) * 1.5f;
        }
        case 4: {  // WindyTexture (Procedural.cuh:247-265)
            const float wind = fbm(si.p * 0.1f, si.dpdx * 0.1f, si.dpdy * 0.1f, 0.5f, 3, sig);
            const float wave = fbm(si.p, si.dpdx, si.dpdy, 0.5f, 6, sig);
            return spec(fabsf(wind) * wave);
        }
        default:
            return Spec{t.v[0], t.v[1], t.v[2]};
    }
}

// ------------------------------------------------------------------ BxDFs
__device__ __forceinline__ float cos2t(V3 w) { return w.z * w.z; }
__device__ __forceinline__ float sin2t(V3 w) { return fmaxf(1 - cos2t(w), 0.0f); }
__device__ __forceinline__ float sint(V3 w) { return sqrtf(sin2t(w)); }
__device__ __forceinline__ float tant(V3 w) { return sint(w) / w.z; }
__device__ __forceinline__ float tan2t(V3 w) { return sin2t(w) / cos2t(w); }
// cosPhi/sinPhi compare the function sinTheta (not its value) with 0, so they never take the
// sin == 0 branch (models/BxDF.cuh:144-153).
__device__ __forceinline__ float cosphi(V3 w) { return clampf(w.x / sint(w), -1, 1); }
__device__ __forceinline__ float sinphi(V3 w) { return clampf(w.y / sint(w), -1, 1); }
__device__ __forceinline__ bool same_hemi(V3 a, V3 b, uint64_t* sig) {  // sameHemisphere, recorded
    const bool v = a.z * b.z > 0;
    if (sig) fnv_mix(*sig, 0x700000000ull + (v ? 1u : 0u));
    return v;
}

// models/BxDF.cuh:16-37 with the swapped clamp bounds of line 17.
__device__ float fresnel_dielectric(float cos_i, float eta_i, float eta_t) {
    cos_i = clampf(cos_i, 1, -1);
    const bool entering = cos_i > 0.0f;
    if (!entering) {
        const float tmp = eta_i;
        eta_i = eta_t;
        eta_t = tmp;
        cos_i = fabsf(cos_i);
    }
    const float sin_i = sqrtf(fmaxf(0.0f, 1 - cos_i * cos_i));
    const float sin_t = eta_i / eta_t * sin_i;
    if (sin_t >= 1) return 1;
    const float cos_t = sqrtf(fmaxf(0.0f, 1 - sin_t * sin_t));
    const float rpar = ((eta_t * cos_i) - (eta_i * cos_t)) / ((eta_t * cos_i) + (eta_i * cos_t));
    const float rperp = ((eta_i * cos_i) - (eta_t * cos_t)) / ((eta_i * cos_i) + (eta_t * cos_t));
    return (rpar * rpar + rperp * rperp) / 2;
}
// models/BxDF.cuh:44-67 (etaI = 1)
__device__ Spec fresnel_conductor(float cos_i, Spec eta_t, Spec k) {
    cos_i = clampf(cos_i, -1, 1);
    const Spec eta = eta_t / 1.0f, etak = k / 1.0f;
    const float c2 = cos_i * cos_i, s2 = 1.0f - c2;
    const Spec eta2 = eta * eta, etak2 = etak * etak;
    const Spec t0 = eta2 - etak2 - spec(s2);
    const Spec a2b2 = ssqrt(t0 * t0 + eta2 * 4.0f * etak2);
    const Spec t1 = a2b2 + spec(c2);
    const Spec a = ssqrt((a2b2 + t0) * 0.5f);
    const Spec t2 = a * (2.0f * cos_i);
    const Spec rs = (t1 - t2) / (t1 + t2);
    const Spec t3 = a2b2 * c2 + spec(s2 * s2);
    const Spec t4 = t2 * s2;
    const Spec rp = rs * (t3 - t4) / (t3 + t4);
    return (rp + rs) * 0.5f;
}
// models/BxDF.cuh:156-166
__device__ __forceinline__ bool refract(V3 wi, V3 n, float eta, V3& wt) {
    const float ci = dot(n, wi);
    const float s2i = fmaxf(0.0f, 1.0f - ci * ci);
    const float s2t = eta * eta * s2i;
    if (s2t >= 1) return false;
    const float ct = sqrtf(1 - s2t);
    wt = -wi * eta + n * (eta * ci - ct);
    return true;
}

// Trowbridge-Reitz (models/Microfacet.cuh:53-181)
__device__ float tr_lambda(V3 w, float ax, float ay) {
    const float at = fabsf(tant(w));
    if (isinf(at)) return 0.0f;
    const float cp = cosphi(w), sp = sinphi(w);
    const float alpha = sqrtf(cp * cp * ax * ax + sp * sp * ay * ay);
    const float a2t2 = (alpha * at) * (alpha * at);
    return (-1 + sqrtf(1.0f + a2t2)) / 2;
}
__device__ float tr_d(V3 wh, float ax, float ay) {
    const float t2 = tan2t(wh);
    if (isinf(t2)) return 0;
    const float c4 = cos2t(wh) * cos2t(wh);
    const float cp = cosphi(wh), sp = sinphi(wh);
    const float e = (cp * cp / (ax * ax) + sp * sp / (ay * ay)) * t2;
    return 1 / (3.14159265358979f * ax * ay * c4 * (1 + e) * (1 + e));
}
__device__ __forceinline__ float tr_g1(V3 w, float ax, float ay) { return 1 / (1 + tr_lambda(w, ax, ay)); }
__device__ __forceinline__ float tr_g(V3 wo, V3 wi, float ax, float ay) {
    return 1 / (1 + tr_lambda(wo, ax, ay) + tr_lambda(wi, ax, ay));
}
__device__ void tr_sample11(float cosT, float U1, float U2, float& sx, float& sy) {
    if (cosT >= kOneMinusEpsUp) {
        const float r = sqrtf(U1 / (1 - U1));
        const float phi = mul_dc(U2, LTS_2PI_HI, LTS_2PI_LO);
        sx = r * cosf(phi);
        sy = r * sinf(phi);
        return;
    }
    const float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
    const float tanT = sinT / cosT;
    const float a = 1 / tanT;
    const float G1 = 2 / (1 + sqrtf(1.f + 1.f / (a * a)));
    const float A = 2 * U1 / G1 - 1;
    float tmp = 1.f / (A * A - 1.f);
    if (tmp > 1e10f) tmp = 1e10f;
    const float B = tanT;
    const float D = sqrtf(fmaxf(float(B * B * tmp * tmp - (A * A - B * B) * tmp), 0.0f));
    const float s1 = B * tmp - D, s2 = B * tmp + D;
    sx = (A < 0 || s2 > 1.f / tanT) ? s1 : s2;
    float S;
    if (U2 > 0.5f) {
        S = 1.f;
        U2 = 2.f * (U2 - .5f);
    } else {
        S = -1.f;
        U2 = 2.f * (.5f - U2);
    }
    const float z = (U2 * (U2 * (U2 * 0.27385f - 0.73369f) + 0.46341f)) /
                    (U2 * (U2 * (U2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
    sy = S * z * sqrtf(1.f + sx * sx);
}
__device__ V3 tr_sample(V3 wi, float ax, float ay, float U1, float U2) {
    const V3 ws = normalize(v3(ax * wi.x, ay * wi.y, wi.z));
    float sx, sy;
    tr_sample11(ws.z, U1, U2, sx, sy);
    const float tmp = cosphi(ws) * sx - sinphi(ws) * sy;
    sy = sinphi(ws) * sx + cosphi(ws) * sy;
    sx = tmp;
    sx = ax * sx;
    sy = ay * sy;
    return normalize(v3(-sx, -sy, 1.f));
}

struct Bsdf {
    int lobe;           // LobeKind; at most one lobe for every reachable material
    uint32_t type;      // BxDF type bits of the lobe
    V3 ns, ng, ss, ts;
    Spec R, T, k, eta3;
    float eta, a, b, alpha;
};

__device__ __forceinline__ V3 to_local(const Bsdf& f, V3 v) { return v3(dot(v, f.ss), dot(v, f.ts), dot(v, f.ns)); }
__device__ __forceinline__ V3 to_world(const Bsdf& f, V3 v) {
    return v3(f.ss.x * v.x + f.ts.x * v.y + f.ns.x * v.z, f.ss.y * v.x + f.ts.y * v.y + f.ns.y * v.z,
              f.ss.z * v.x + f.ts.z * v.y + f.ns.z * v.z);
}
__device__ __forceinline__ bool matches(uint32_t type, uint32_t flags) { return (type & flags) == type; }

// BxDF::f
__device__ Spec lobe_f(const Bsdf& f, V3 wo, V3 wi) {
    switch (f.lobe) {
        case LOBE_LAMBERT: return f.R * LTS_1_PI_HI;
        case LOBE_OREN_NAYAR: {  // Microfacet.cuh:27-50
            const float so = sint(wo), si_ = sint(wi);
            float maxcos = 0.0f;
            if (si_ >= 0.0001f && so >= 0.0001f) {
                const float spo = sinphi(wo), cpo = cosphi(wo), spi = sinphi(wi), cpi = cosphi(wi);
                const float dcos = cpi * cpo + spi * spo;
                maxcos = fmaxf(0.0f, dcos);
            }
            float sin_a, tan_b;
            if (fabsf(wi.z) > fabsf(wo.z)) {
                sin_a = so;
                tan_b = si_ / fabsf(wi.z);
            } else {
                sin_a = si_;
                tan_b = so / fabsf(wo.z);
            }
            return f.R * LTS_1_PI_HI * (f.a + f.b * maxcos * sin_a * tan_b);
        }
        case LOBE_MICROFACET: {  // Microfacet.cuh:200-209
            const float co = fabsf(wo.z), ci = fabsf(wi.z);
            V3 wh = wi + wo;
            if (ci == 0 || co == 0) return spec(0.0f);
            if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return spec(0.0f);
            wh = normalize(wh);
            const Spec F = fresnel_conductor(fabsf(dot(wi, wh)), f.eta3, f.k);
            return f.R * tr_d(wh, f.alpha, f.alpha) * tr_g(wo, wi, f.alpha, f.alpha) * F / (4 * ci * co);
        }
        default: return spec(0.0f);  // specular lobes
    }
}
// BxDF::Pdf
__device__ float lobe_pdf(const Bsdf& f, V3 wo, V3 wi, uint64_t* sig) {
    switch (f.lobe) {
        case LOBE_LAMBERT:
        case LOBE_OREN_NAYAR:
            return same_hemi(wo, wi, sig) ? mul_dc(fabsf(wi.z), LTS_1_PI_HI, LTS_1_PI_LO) : 0.0f;
        case LOBE_MICROFACET: {
            if (!same_hemi(wo, wi, sig)) return 0;
            const V3 wh = normalize(wo + wi);
            const float pd = tr_d(wh, f.alpha, f.alpha) * tr_g1(wo, f.alpha, f.alpha) * absdot(wo, wh) / fabsf(wo.z);
            return pd / (4 * dot(wo, wh));
        }
        default: return 0.0f;
    }
}
// BSDF::f (materials/BSDF.cuh:192-204)
__device__ Spec bsdf_f(const Bsdf& f, V3 woW, V3 wiW, uint32_t flags, uint64_t* sig) {
    const bool reflect = dot(wiW, f.ng) * dot(woW, f.ng) > 0;
    if (sig) fnv_mix(*sig, 0x600000000ull + (reflect ? 1u : 0u));
    if (f.lobe == LOBE_NONE || !matches(f.type, flags)) return spec(0.0f);
    const V3 wi = to_local(f, wiW), wo = to_local(f, woW);
    if ((reflect && (f.type & BSDF_REFLECTION)) || (!reflect && (f.type & BSDF_TRANSMISSION)))
        return spec(0.0f) + lobe_f(f, wo, wi);
    return spec(0.0f);
}
// BSDF::Pdf (BSDF.cuh:261-276)
__device__ float bsdf_pdf(const Bsdf& f, V3 woW, V3 wiW, uint32_t flags, uint64_t* sig) {
    if (f.lobe == LOBE_NONE) return 0.0f;
    const V3 wo = to_local(f, woW), wi = to_local(f, wiW);
    if (wo.z == 0) return 0.0f;
    if (!matches(f.type, flags)) return 0.0f;
    const float pdf = 0.0f + lobe_pdf(f, wo, wi, sig);
    return pdf / 1;
}
// BSDF::sampleF with a single matching lobe (BSDF.cuh:206-259) and the lobes' sampleF.
__device__ Spec bsdf_sample(const Bsdf& f, V3 woW, V3& wiW, F2 u, float& pdf, uint32_t flags, uint32_t& sampled,
                            uint64_t* sig) {
    if (f.lobe == LOBE_NONE || !matches(f.type, flags)) {
        pdf = 0;
        return spec(0.0f);
    }
    // comp = min((int)floorf(u.x * 1), 0) = 0; the remapped sample is u itself
    const V3 wo = to_local(f, woW);
    V3 wi = v3(0, 0, 0);
    pdf = 0;
    sampled = f.type;
    Spec val = spec(0.0f);
    switch (f.lobe) {
        case LOBE_LAMBERT:
        case LOBE_OREN_NAYAR: {  // BxDF::sampleF (BxDF.cuh:196-204)
            const float r = sqrtf(u.x);
            const float th = mul_dc(u.y, LTS_2PI_HI, LTS_2PI_LO);
            const float dx = r * cosf(th), dy = r * sinf(th);
            wi = v3(dx, dy, sqrtf(fmaxf(0.0f, 1 - dx * dx - dy * dy)));
            if (wo.z < 0) wi.z *= -1;
            pdf = lobe_pdf(f, wo, wi, sig);
            val = lobe_f(f, wo, wi);
            break;
        }
        case LOBE_SPECULAR_REFL: {  // Specular.cuh:30-39, FresnelNoOp
            wi = v3(-wo.x, -wo.y, wo.z);
            pdf = 1.0f;
            val = (spec(1.0f) * f.R) / fabsf(wi.z);
            break;
        }
        case LOBE_FRESNEL_SPECULAR: {  // Specular.cuh:107-135
            const float F = fresnel_dielectric(wo.z, 1.0f, f.eta);
            if (u.x < F) {
                wi = v3(-wo.x, -wo.y, -wo.z);  // the reference's "reflection" keeps going straight
                sampled = BSDF_SPECULAR | BSDF_REFLECTION;
                pdf = F;
                val = (f.R * F) / fabsf(wi.z);
            } else {
                const bool entering = wo.z > 0;
                const float ei = entering ? 1.0f : f.eta, et = entering ? f.eta : 1.0f;
                const V3 n = face_towards(v3(0, 0, 1), wo);
                if (!refract(wo, n, ei / et, wi)) {
                    pdf = 0;
                    return spec(0.0f);
                }
                Spec ft = f.T * (1 - F);
                ft = ft * ((ei * ei) / (et * et));
                sampled = BSDF_SPECULAR | BSDF_TRANSMISSION;
                pdf = 1.0f - F;
                val = ft / fabsf(wi.z);
            }
            break;
        }
        case LOBE_MICROFACET: {  // Microfacet.cuh:211-222
            if (wo.z == 0) return spec(0.0f);
            const bool flip = wo.z < 0;
            V3 wh = tr_sample(flip ? -wo : wo, f.alpha, f.alpha, u.x, u.y);
            if (flip) wh = -wh;
            if (dot(wo, wh) < 0) return spec(0.0f);
            wi = -wo + wh * (2 * dot(wo, wh));
            if (!same_hemi(wo, wi, sig)) return spec(0.0f);
            const float pd = tr_d(wh, f.alpha, f.alpha) * tr_g1(wo, f.alpha, f.alpha) * absdot(wo, wh) / fabsf(wo.z);
            pdf = pd / (4 * dot(wo, wh));
            val = lobe_f(f, wo, wi);
            break;
        }
    }
    if (pdf == 0) return spec(0.0f);
    wiW = to_world(f, wi);
    return val;
}

// Material::computeScatteringFunctions (materials/Material.cuh:31-130) into a Bsdf record.
// Returns false when the primitive has no material (the reference's skipped 'M' entries).
__device__ bool make_bsdf(const SceneView& sv, const SI& si, Bsdf& f, uint64_t* sig) {
    const int mesh = __ldg(&sv.prim_n[si.prim].w);
    const DevMat& m = sv.mats[mesh];
    if (m.kind == 0) return false;
    f.ns = si.sn;
    f.ng = si.n;
    f.ss = normalize(si.sdpdu);
    f.ts = cross(f.ns, f.ss);
    f.lobe = LOBE_NONE;
    f.type = 0;
    f.eta = 1;
    switch (m.kind) {
        case 1: {  // Matte
            const Spec kd = eval_texture(m.tex[0], si, sig);
            if (!is_black(kd)) {
                f.R = kd;
                if (m.extra == 0) {
                    f.lobe = LOBE_LAMBERT;
                } else {
                    f.lobe = LOBE_OREN_NAYAR;
                    f.a = m.on_a;
                    f.b = m.on_b;
                }
                f.type = BSDF_REFLECTION | BSDF_DIFFUSE;
            }
            break;
        }
        case 2: {  // Glass
            f.eta = m.extra;
            const Spec r = eval_texture(m.tex[0], si, sig), t = eval_texture(m.tex[1], si, sig);
            if (is_black(r) && is_black(t)) break;
            f.R = r;
            f.T = t;
            f.lobe = LOBE_FRESNEL_SPECULAR;
            f.type = BSDF_REFLECTION | BSDF_TRANSMISSION | BSDF_SPECULAR;
            break;
        }
        case 3: {  // Mirror
            const Spec r = eval_texture(m.tex[0], si, sig);
            if (is_black(r)) break;
            f.R = r;
            f.lobe = LOBE_SPECULAR_REFL;
            f.type = BSDF_REFLECTION | BSDF_SPECULAR;
            break;
        }
        case 4: {  // Metal (alpha given directly)
            f.k = eval_texture(m.tex[0], si, sig);
            f.eta3 = Spec{m.tex[1].v[0], m.tex[1].v[1], m.tex[1].v[2]};
            f.R = spec(1.0f);
            f.alpha = m.extra;
            f.lobe = LOBE_MICROFACET;
            f.type = BSDF_REFLECTION | BSDF_GLOSSY;
            break;
        }
    }
    return true;
}

// ------------------------------------------------------------------ lights
struct LightSample {
    Spec Li;
    V3 wi;
    float pdf;
    V3 p1, perr1, n1;  // visibility target interaction
};
__device__ __forceinline__ float sph_pdf_infinite(V3 w) {
    // uniformSampleHemispherePDF() / (2 * M_PI * M_PI * sinf(sphericalTheta(w)))
    const float s = sinf(acosf(clampf(w.z, -1.0f, 1.0f)));
    return 0.159154937f / (19.7392088f * s);
}

// Triangle::Pdf(it, wi) (shapes/Triangle.cu:211-225): re-intersects the light triangle.
__device__ float area_pdf(const SceneView& sv, const DevLight& L, V3 p, V3 perr, V3 n, V3 wi) {
    const V3 o = offset_origin(p, perr, n, wi);
    V3 p0, p1, p2;
    prim_tri(sv, L.prim, p0, p1, p2);
    float t, u, v, inv;
    if (!tri_test(p0, p1, p2, o, wi, INFINITY, t, u, v, inv)) return 0;
    SI is;
    make_si(sv, L.prim, p0, p1, p2, wi, u, v, inv, is);
    const V3 dpt = p - is.p;
    return len2(dpt) / (absdot(is.n, -wi) * L.area);
}

__device__ bool sample_li(const SceneView& sv, const DevLight& L, const SI& si, F2 u, LightSample& ls) {
    ls.Li = spec(0.0f);
    ls.pdf = 0;
    ls.perr1 = v3(0, 0, 0);
    ls.n1 = v3(0, 0, 0);
    if (L.kind == 0) {  // AreaLight::sampleLi (Light.cu:28-37) + Triangle::sample (Triangle.cu:232-259)
        const float su = sqrtf(u.x);
        const float b0 = 1 - su, b1 = u.y * su;
        V3 p0, p1, p2;
        prim_tri(sv, L.prim, p0, p1, p2);
        const float b2 = 1 - b0 - b1;
        const V3 ps = p0 * b0 + p1 * b1 + p2 * b2;
        V3 ns;
        const int4 ni = __ldg(sv.prim_n + L.prim);
        if (ni.x >= 0)
            ns = normalize(normal_at(sv, ni.x) * b0 + normal_at(sv, ni.y) * b1 + normal_at(sv, ni.z) * b2);
        else
            ns = normalize(cross(p1 - p0, p2 - p0));
        const V3 pabs = vabs(p0 * b0) + vabs(p1 * b1) + vabs(p2 * b2);
        ls.perr1 = pabs * gamma_n(6);
        ls.p1 = ps;
        ls.n1 = ns;
        ls.wi = normalize(ps - si.p);
        ls.pdf = area_pdf(sv, L, si.p, si.perr, si.n, ls.wi);
        ls.Li = dot(ns, -ls.wi) > 0.f ? Spec{L.L[0], L.L[1], L.L[2]} : spec(0.0f);
        return false;
    }
    if (L.kind == 1) {  // InfiniteLight::sampleLi (Light.cu:68-90)
        const float z = u.x;
        const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
        const float phi = mul_dc(u.y, LTS_2PI_HI, LTS_2PI_LO);
        const V3 w0 = v3(r * cosf(phi), r * sinf(phi), z);
        const V3 ref = v3(0, 1, 0);
        V3 a, b;
        coordinate_system(ref, a, b);
        const V3 w = a * w0.x + b * w0.y + ref * w0.z;
        const V3 pl = v3(L.p[0], L.p[1], L.p[2]) + w * L.radius;
        ls.wi = normalize(pl - si.p);
        ls.pdf = sph_pdf_infinite(ls.wi);
        ls.p1 = pl;
        ls.Li = Spec{L.L[0], L.L[1], L.L[2]};
        return false;
    }
    // PointLight::sampleLi (Light.cu:8-17)
    const V3 pl = v3(L.p[0], L.p[1], L.p[2]);
    ls.wi = normalize(pl - si.p);
    ls.pdf = 1.0f;
    ls.p1 = pl;
    ls.Li = Spec{L.L[0], L.L[1], L.L[2]} / len2(pl - si.p);
    return true;  // delta light
}

// ------------------------------------------------------------------ film
struct FilmAcc {
    float* s;  // shared: [16][kThreads] sums (2x2 pixels x rgbw), then [16][kThreads] compensations
};
__device__ __forceinline__ void kahan_add(float* sum, float* c, float v) {
    const float y = v - *c;
    const float t = *sum + y;
    *c = (t - *sum) - y;
    *sum = t;
}

// ------------------------------------------------------------------ the kernel
template <bool RECORD>
__global__ __launch_bounds__(kThreads) void k_pathtrace(const SceneView sv, const RenderParams rp, int nleaf) {
    __shared__ uint32_t s_stack[kStack * kThreads];
    __shared__ float s_film[32 * kThreads];
    const int tid = threadIdx.y * kBX + threadIdx.x;
    uint32_t* stack = s_stack + tid;
    float* acc = s_film + tid;
    const int i = rp.x0 + blockIdx.x * kBX + threadIdx.x;
    const int j = rp.y0 + blockIdx.y * kBY + threadIdx.y;
    if (i >= rp.x1 || j >= rp.y1) return;
    const int W = sv.width, H = sv.height;
    const int id = j * W + i;
    unsigned long long rays = 0;
    Work wk{0u, 0u};
#pragma unroll
    for (int k = 0; k < 32; ++k) acc[k * kThreads] = 0.0f;

    const float* cam = sv.cam;
    const V3 co = v3(cam[0], cam[1], cam[2]), cright = v3(cam[3], cam[4], cam[5]), cup = v3(cam[6], cam[7], cam[8]),
             cllc = v3(cam[9], cam[10], cam[11]);
    const float rx = (float)(W - 1), ry = (float)(H - 1);

    Rng rng;
    rng.key = rp.seed + wang_hash((uint32_t)id);

    for (int s = 0; s < rp.spp; ++s) {
        rng.sample = (uint32_t)s;
        rng.draw = 0;
        uint64_t sig = 0xcbf29ce484222325ull;
        Tracer16 tr{nullptr, 0};
        if (RECORD && rp.trace &&
            ((long)((j - rp.y0) * (rp.x1 - rp.x0) + (i - rp.x0)) * rp.spp + s) == rp.trace_sample)
            tr.out = rp.trace;
        // 3. camera ray (PathTracingIntegrator.cuh:40-46, Camera.cu:51-81); aperture is 0, so the
        // lens sample moves nothing, but it is drawn.
        const F2 fs = rng_2d(rng);
        (void)rng_2d(rng);
        const float pfx = (float)(i + fs.x), pfy = (float)(j + fs.y);
        V3 ro = co;
        V3 rd = normalize(cllc + cright * (pfx / rx) + cup * (pfy / ry) - co);
        // differentials scaled by rsqrt(spp) (Ray.cuh:35-40); origins equal o exactly
        const V3 dx0 = normalize(cllc + cright * ((pfx + 1) / rx) + cup * (pfy / ry) - co);
        const V3 dy0 = normalize(cllc + cright * (pfx / rx) + cup * ((pfy + 1) / ry) - co);
        V3 rxd = rd + (dx0 - rd) * rp.spp_scale, ryd = rd + (dy0 - rd) * rp.spp_scale;
        bool has_diff = true;

        Spec L = spec(0.0f), beta = spec(1.0f);
        bool specular = false;
        for (int bounce = 0; bounce < rp.max_bounce; ++bounce) {
            SI si;
            ++rays;
            const bool hit = scene_intersect(sv, nleaf, ro, rd, INFINITY, si, stack, rp.err, wk);
            if (RECORD) fnv_mix(sig, 0x100000000ull + (uint64_t)((hit ? si.prim : -1) + 1));
            if (RECORD) tr.put(1, hit, hit ? si.prim : -1, si.p.x, si.p.y, si.p.z, si.n.x, si.n.y, si.n.z, si.sn.x, si.sn.y,
                               si.sn.z, beta.r, beta.g, beta.b, L.r);
            if (bounce == 0 || specular) {
                if (hit) {
                    const int li = __ldg(sv.prim_light + si.prim);
                    if (li >= 0) {
                        const DevLight& Lt = sv.lights[li];
                        const Spec le = dot(si.n, -rd) > 0.f ? Spec{Lt.L[0], Lt.L[1], Lt.L[2]} : spec(0.0f);
                        L = L + beta * le;
                    } else {
                        L = L + beta * spec(0.0f);
                    }
                } else {
                    for (int l = 0; l < sv.nlight; ++l) {
                        const DevLight& Lt = sv.lights[l];
                        L = L + beta * (Lt.kind == 1 ? Spec{Lt.L[0], Lt.L[1], Lt.L[2]} : spec(0.0f));
                    }
                }
            }
            if (!hit) break;
            // 7. scattering functions: differentials (Interaction.cuh:118-160) then material
            if (has_diff) {
                const V3 n = si.n;
                const float d = -dot(n, si.p);
                const float tx = (-dot(n, ro) - d) / dot(n, rxd);
                const float ty = (-dot(n, ro) - d) / dot(n, ryd);
                si.dpdx = (ro + rxd * tx) - si.p;
                si.dpdy = (ro + ryd * ty) - si.p;
            } else {
                si.dpdx = v3(0, 0, 0);
                si.dpdy = v3(0, 0, 0);
            }
            Bsdf f;
            if (!make_bsdf(sv, si, f, RECORD ? &sig : nullptr)) break;
            if (RECORD) tr.put(2, f.lobe, f.R.r, f.R.g, f.R.b, f.ss.x, f.ss.y, f.ss.z, f.ts.x, f.ts.y, f.ts.z, si.dpdx.x,
                               si.dpdx.y, si.dpdx.z);
            // 7a. direct lighting: uniformSampleOneLight + estimateDirect (IntegratorHelper.cuh:51-149)
            if (sv.nlight > 0) {
                const float ul = rng_1d(rng);
                int off = 0;
                {  // Distribution1D::findInterval with the reference's clamp to size - 2
                    const int size = sv.nlight;
                    if (size != 1) {
                        int first = 0, len = size;
                        while (len > 0) {
                            const int half = len >> 1, middle = first + half;
                            if (__ldg(sv.light_cdf + middle) <= ul) {
                                first = middle + 1;
                                len -= half + 1;
                            } else {
                                len = half;
                            }
                        }
                        off = (int)clampf((float)(first - 1), 0.0f, (float)(size - 2));
                    }
                }
                const float lpdf_sel = __ldg(sv.light_func + off) / (sv.light_func_int * sv.nlight);
                const F2 ulight = rng_2d(rng);
                const F2 uscat = rng_2d(rng);
                const DevLight& Lt = sv.lights[off];
                const uint32_t flags = specular ? BSDF_ALL : (BSDF_ALL & ~BSDF_SPECULAR);
                Spec Ld = spec(0.0f);
                LightSample ls;
                const bool delta = sample_li(sv, Lt, si, ulight, ls);
                if (ls.pdf > 0 && !is_black(ls.Li)) {
                    const Spec fv = bsdf_f(f, si.wo, ls.wi, flags, RECORD ? &sig : nullptr) * absdot(ls.wi, si.sn);
                    const float spdf = bsdf_pdf(f, si.wo, ls.wi, flags, RECORD ? &sig : nullptr);
                    if (!is_black(fv)) {
                        // VisibilityTester::unoccluded -> spawnRayTo(Interaction) (Interaction.cuh:47-51)
                        const V3 org = offset_origin(si.p, si.perr, si.n, ls.p1 - si.p);
                        const V3 tgt = offset_origin(ls.p1, ls.perr1, ls.n1, org - ls.p1);
                        ++rays;
                        const bool occ = scene_occluded(sv, nleaf, org, tgt - org, 1 - kShadowEps, stack, rp.err, wk);
                        if (RECORD) tr.put(3, off, lpdf_sel, ls.pdf, ls.Li.r, ls.wi.x, ls.wi.y, ls.wi.z, fv.r, fv.g, fv.b, spdf, occ);
                        if (RECORD) fnv_mix(sig, 0x300000000ull + (occ ? 0u : 1u));
                        Spec Li = ls.Li;
                        if (occ) Li = spec(0.0f);
                        if (!is_black(Li)) {
                            if (delta) {
                                Ld = Ld + fv * Li / ls.pdf;
                            } else {
                                const float fp = 1 * ls.pdf, gp = 1 * spdf;
                                const float wgt = (fp * fp) / (fp * fp + gp * gp);
                                Ld = Ld + fv * Li * wgt / ls.pdf;
                            }
                        }
                    }
                }
                if (!delta) {
                    V3 wi = ls.wi;
                    float spdf = 0;
                    uint32_t stype = 0;
                    Spec fv = bsdf_sample(f, si.wo, wi, uscat, spdf, flags, stype, RECORD ? &sig : nullptr);
                    fv = fv * absdot(wi, si.sn);
                    const bool sampled_spec = (stype & BSDF_SPECULAR) != 0;
                    if (!is_black(fv) && spdf > 0) {
                        float wgt = 1;
                        bool done = false;
                        if (!sampled_spec) {
                            float lp;
                            if (Lt.kind == 0) lp = area_pdf(sv, Lt, si.p, si.perr, si.n, wi);
                            else if (Lt.kind == 1) lp = sph_pdf_infinite(wi);
                            else lp = 0.0f;
                            if (lp == 0) done = true;
                            else {
                                const float fp = 1 * spdf, gp = 1 * lp;
                                wgt = (fp * fp) / (fp * fp + gp * gp);
                            }
                        }
                        if (!done) {
                            SI lit;
                            const V3 org = offset_origin(si.p, si.perr, si.n, wi);
                            ++rays;
                            const bool found = scene_intersect(sv, nleaf, org, wi, INFINITY, lit, stack, rp.err, wk);
                            if (RECORD) fnv_mix(sig, 0x200000000ull + (uint64_t)((found ? lit.prim : -1) + 1));
                            Spec Li = spec(0.0f);
                            if (found) {
                                if (__ldg(sv.prim_light + lit.prim) == off && Lt.kind == 0)
                                    Li = dot(lit.n, -wi) > 0.f ? Spec{Lt.L[0], Lt.L[1], Lt.L[2]} : spec(0.0f);
                            } else {
                                Li = Lt.kind == 1 ? Spec{Lt.L[0], Lt.L[1], Lt.L[2]} : spec(0.0f);
                            }
                            if (!is_black(Li)) Ld = Ld + fv * Li * spec(1.0f) * wgt / spdf;
                            if (RECORD) tr.put(4, spdf, fv.r, fv.g, fv.b, wgt, found, Li.r, Ld.r, Ld.g, Ld.b, wi.x, wi.y, wi.z);
                        }
                    }
                }
                L = L + beta * (Ld / lpdf_sel);
            }
            // 7b. BSDF sample (PathTracingIntegrator.cuh:80-91)
            V3 wi = v3(0, 0, 0);
            float pdf = 0;
            uint32_t stype = 0;
            const F2 ub = rng_2d(rng);
            const Spec fv = bsdf_sample(f, si.wo, wi, ub, pdf, BSDF_ALL, stype, RECORD ? &sig : nullptr);
            if (is_black(fv) || pdf == 0) break;
            specular = (stype & BSDF_SPECULAR) != 0;
            beta = beta * (fv * absdot(wi, si.sn) / pdf);
            if (RECORD) tr.put(5, wi.x, wi.y, wi.z, pdf, fv.r, fv.g, fv.b, beta.r, beta.g, beta.b, L.r, L.g, L.b);
            // 8. new ray: spawnRay, no differentials
            ro = offset_origin(si.p, si.perr, si.n, wi);
            rd = wi;
            has_diff = false;
            // 9. Russian roulette
            if (bounce >= rp.rr_start) {
                const float q = fmaxf(0.05f, 1 - lum(beta));
                if (rng_1d(rng) < q) break;
                beta = beta / (1 - q);
            }
        }
        // 10. film (Camera::addSample, Camera.cu:192-218)
        {
            const int px0 = max((int)ceilf(pfx - 1.0f), 0), py0 = max((int)ceilf(pfy - 1.0f), 0);
            const int px1 = min((int)floorf(pfx + 1.0f) + 1, W), py1 = min((int)floorf(pfy + 1.0f) + 1, H);
            for (int y = py0; y < py1; ++y) {
                for (int x = px0; x < px1; ++x) {
                    const float fdx = fabsf((x - pfx - 0.5f) * 1.0f * 16);
                    const float fdy = fabsf((y - pfy - 0.5f) * 1.0f * 16);
                    const int ix = min((int)floorf(fdx), 15), iy = min((int)floorf(fdy), 15);
                    const float wgt = __ldg(sv.filter + iy * 16 + ix);
                    const Spec c = L * wgt;
                    const int ox = x - i, oy = y - j;
                    if (ox >= 0 && ox <= 1 && oy >= 0 && oy <= 1) {
                        const int base = (oy * 2 + ox) * 4;
                        kahan_add(acc + (base + 0) * kThreads, acc + (16 + base + 0) * kThreads, c.r);
                        kahan_add(acc + (base + 1) * kThreads, acc + (16 + base + 1) * kThreads, c.g);
                        kahan_add(acc + (base + 2) * kThreads, acc + (16 + base + 2) * kThreads, c.b);
                        kahan_add(acc + (base + 3) * kThreads, acc + (16 + base + 3) * kThreads, wgt);
                    } else {
                        double* fp = rp.film + 4 * ((size_t)y * W + x);
                        atomicAdd(fp + 0, (double)c.r);
                        atomicAdd(fp + 1, (double)c.g);
                        atomicAdd(fp + 2, (double)c.b);
                        atomicAdd(fp + 3, (double)wgt);
                    }
                }
            }
        }
        if (RECORD) tr.put(6, L.r, L.g, L.b);
        if (RECORD) {
            const size_t k = ((size_t)(j - rp.y0) * (rp.x1 - rp.x0) + (i - rp.x0)) * rp.spp + s;
            rp.sample_L[3 * k + 0] = L.r;
            rp.sample_L[3 * k + 1] = L.g;
            rp.sample_L[3 * k + 2] = L.b;
            rp.sample_sig[k] = sig;
        }
    }
    // flush the 2x2 core accumulators (sum minus compensation) to the FP64 film
    for (int oy = 0; oy < 2; ++oy)
        for (int ox = 0; ox < 2; ++ox) {
            const int x = i + ox, y = j + oy;
            if (x >= W || y >= H) continue;
            double* fp = rp.film + 4 * ((size_t)y * W + x);
            const int base = (oy * 2 + ox) * 4;
            for (int c = 0; c < 4; ++c) {
                const float sum = acc[(base + c) * kThreads], cmp = acc[(16 + base + c) * kThreads];
                if (sum != 0.0f || cmp != 0.0f) atomicAdd(fp + c, (double)sum - (double)cmp);
            }
        }
    // ray counter: one atomic per warp (lanes outside the crop have already returned)
    const unsigned mask = __activemask();
    const unsigned tot = __reduce_add_sync(mask, (unsigned)rays);
    const unsigned tn = __reduce_add_sync(mask, wk.nodes), tt = __reduce_add_sync(mask, wk.tris);
    const unsigned lane = (unsigned)tid & 31u;
    if ((mask & ((1u << lane) - 1u)) == 0u && rp.counters) {
        atomicAdd(rp.counters, (unsigned long long)tot);
        atomicAdd(rp.counters + 1, (unsigned long long)tn);
        atomicAdd(rp.counters + 2, (unsigned long long)tt);
    }
}

// Camera::getRender (Camera.cu:256-289): divide by the filter weight (in FP64 here), clamp at 0,
// flip rows.
__global__ void k_resolve(const double* __restrict__ film, float* __restrict__ rgb, int W, int H) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * H) return;
    const int i = idx % W, jj = idx / W;
    const int src = (H - 1 - jj) * W + i;
    const double w = film[4 * src + 3];
    for (int c = 0; c < 3; ++c) {
        const double v = film[4 * src + c] / w;
        rgb[3 * idx + c] = fmaxf(0.0f, (float)v);
    }
}

__global__ void k_gather_leaves(const float4* __restrict__ prim_v, const int32_t* __restrict__ leaf_prim, int n,
                                float4* __restrict__ leaf_v) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n) return;
    const int p = __ldg(leaf_prim + l);
    float4 a = __ldg(prim_v + 3 * p);
    a.w = __int_as_float(p);
    leaf_v[3 * l] = a;
    leaf_v[3 * l + 1] = __ldg(prim_v + 3 * p + 1);
    leaf_v[3 * l + 2] = __ldg(prim_v + 3 * p + 2);
}

#define TRY(call)                                                                       \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return std::string(#call ": ") + cudaGetErrorString(e_); \
    } while (0)

template <class T>
std::string upload(void*& slot, const std::vector<T>& v, cudaStream_t s) {
    if (slot) dev_free(slot);
    slot = nullptr;
    const size_t b = std::max<size_t>(sizeof(T) * v.size(), 16);
    TRY(dev_alloc(&slot, b));
    if (!v.empty()) TRY(cudaMemcpyAsync(slot, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    return "";
}

float quake_host(float f) { return quake_rsqrt(f); }

}  // namespace

void Tracer::free_all() {
    for (void*& p : bufs_) {
        if (p) dev_free(p);
        p = nullptr;
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
    dev_free(trace_);
    trace_ = nullptr;
    film_cap_ = rec_cap_ = 0;
    leaf_serial_ = 0;
}

Tracer::~Tracer() {
    free_all();
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
}

std::string Tracer::upload_scene(const HostScene& sc, cudaStream_t s) {
    free_all();
    static bool consts = false;
    if (!consts) {
        // improved-Perlin permutation (Perlin 2002) and the marble colour table with one repeated
        // final row, so t == 1 (sinf == 1) reads a defined entry (Procedural.cuh:286-300)
        static const unsigned char p[256] = {
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
        unsigned char p2[512];
        for (int k = 0; k < 512; ++k) p2[k] = p[k & 255];
        TRY(cudaMemcpyToSymbol(c_perm, p2, 512));
        const float mc[10][3] = {{.58f, .58f, .6f}, {.58f, .58f, .6f}, {.58f, .58f, .6f}, {.5f, .5f, .5f},
                                 {.6f, .59f, .58f}, {.58f, .58f, .6f}, {.58f, .58f, .6f}, {.2f, .2f, .33f},
                                 {.58f, .58f, .6f}, {.58f, .58f, .6f}};
        TRY(cudaMemcpyToSymbol(c_marble, mc, sizeof mc));
        consts = true;
    }
    if (!ev0_) {
        TRY(cudaEventCreate(&ev0_));
        TRY(cudaEventCreate(&ev1_));
    }
    const int nt = sc.triangles();
    std::vector<float4> pv(3 * (size_t)nt);
    std::vector<int4> pn((size_t)nt), puv((size_t)nt);
    for (int t = 0; t < nt; ++t) {
        for (int c = 0; c < 3; ++c) {
            const int vi = sc.tri_p[3 * t + c];
            pv[3 * (size_t)t + c] = make_float4(sc.p[3 * vi], sc.p[3 * vi + 1], sc.p[3 * vi + 2], 0.f);
        }
        pn[t] = make_int4(sc.tri_n[3 * t], sc.tri_n[3 * t + 1], sc.tri_n[3 * t + 2], sc.tri_mesh[t]);
        puv[t] = make_int4(sc.tri_uv[3 * t], sc.tri_uv[3 * t + 1], sc.tri_uv[3 * t + 2], 0);
    }
    std::vector<DevMat> mats(sc.materials.size());
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
    std::string e;
    if (!(e = upload(bufs_[0], pv, s)).empty()) return e;
    if (!(e = upload(bufs_[1], pn, s)).empty()) return e;
    if (!(e = upload(bufs_[2], puv, s)).empty()) return e;
    if (!(e = upload(bufs_[3], sc.n, s)).empty()) return e;
    if (!(e = upload(bufs_[4], sc.uv, s)).empty()) return e;
    if (!(e = upload(bufs_[5], sc.prim_light, s)).empty()) return e;
    if (!(e = upload(bufs_[6], mats, s)).empty()) return e;
    if (!(e = upload(bufs_[7], lights, s)).empty()) return e;
    if (!(e = upload(bufs_[8], sc.light_func, s)).empty()) return e;
    if (!(e = upload(bufs_[9], sc.light_cdf, s)).empty()) return e;
    if (!(e = upload(bufs_[10], filt, s)).empty()) return e;
    TRY(dev_alloc((void**)&counters_, 64));
    view_ = SceneView{};
    view_.ntri = nt;
    view_.nlight = (int)lights.size();
    view_.width = sc.width;
    view_.height = sc.height;
    view_.prim_v = (const float4*)bufs_[0];
    view_.prim_n = (const int4*)bufs_[1];
    view_.prim_uv = (const int4*)bufs_[2];
    view_.normals = (const float*)bufs_[3];
    view_.uvs = (const float*)bufs_[4];
    view_.prim_light = (const int32_t*)bufs_[5];
    view_.mats = (const DevMat*)bufs_[6];
    view_.lights = (const DevLight*)bufs_[7];
    view_.light_func = (const float*)bufs_[8];
    view_.light_cdf = (const float*)bufs_[9];
    view_.light_func_int = sc.light_func_int;
    view_.filter = (const float*)bufs_[10];
    memcpy(view_.cam, sc.cam, sizeof sc.cam);
    return "";
}

std::string Tracer::prepare(const HostScene& sc, const Lbvh& bvh, const lts_render_desc& d, cudaStream_t s,
                            uint32_t* d_err, RenderParams* rp, SceneView* sv, long* crop_samples) {
    if (d.spp < 1 || d.max_bounce < 0) return "bad argument: spp must be >= 1 and max_bounce >= 0";
    if (d.integrator != LTS_INTEGRATOR_MEGAKERNEL) return "bad argument: only the megakernel integrator is built";
    int x0 = d.x0, y0 = d.y0, x1 = d.x1, y1 = d.y1;
    if (x1 == 0 && y1 == 0) {
        x0 = y0 = 0;
        x1 = sc.width;
        y1 = sc.height;
    }
    if (x0 < 0 || y0 < 0 || x1 > sc.width || y1 > sc.height || x0 >= x1 || y0 >= y1) return "bad argument: crop";
    if (bvh.n != sc.triangles()) return "bad argument: BVH does not match the scene";
    // leaf-ordered triangles for traversal
    if (leaf_serial_ != bvh.serial || leaf_n_ != bvh.n) {
        dev_free(leaf_v_);
        leaf_v_ = nullptr;
        TRY(dev_alloc((void**)&leaf_v_, sizeof(float4) * 3 * (size_t)bvh.n));
        k_gather_leaves<<<(bvh.n + 255) / 256, 256, 0, s>>>(view_.prim_v, bvh.leaf_prim, bvh.n, leaf_v_);
        leaf_serial_ = bvh.serial;
        leaf_n_ = bvh.n;
    }
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
    TRY(cudaMemsetAsync(film_, 0, film_bytes, s));
    TRY(cudaMemsetAsync(counters_, 0, 64, s));
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
    *sv = view_;
    sv->leaf_v = leaf_v_;
    sv->nodes = bvh.nodes;
    sv->root_bounds = bvh.root_bounds;
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
    const dim3 block(kBX, kBY);
    const dim3 grid((rp.x1 - rp.x0 + kBX - 1) / kBX, (rp.y1 - rp.y0 + kBY - 1) / kBY);
    TRY(cudaEventRecord(ev0_, s));
    if (d.record_samples)
        k_pathtrace<true><<<grid, block, 0, s>>>(sv, rp, bvh.n);
    else
        k_pathtrace<false><<<grid, block, 0, s>>>(sv, rp, bvh.n);
    TRY(cudaEventRecord(ev1_, s));
    TRY(cudaGetLastError());
    last_launches = 1;
    last_paths = (double)ns;
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
    unsigned long long cnt[3] = {0, 0, 0};
    TRY(cudaMemcpy(cnt, counters_, 24, cudaMemcpyDeviceToHost));
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
        k_resolve<<<(W * H + 255) / 256, 256, 0, s>>>(film_, rgb_, W, H);
        TRY(cudaGetLastError());
        TRY(cudaMemcpyAsync(rgb, rgb_, 12 * (size_t)W * H, cudaMemcpyDeviceToHost, s));
    }
    if (sums) TRY(cudaMemcpyAsync(sums, film_, 32 * (size_t)W * H, cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    return "";
}

}  // namespace lts
