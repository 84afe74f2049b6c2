// Device functions shared by the megakernel (tracer.cu) and the wavefront stages
// (wavefront.cu): sampler, triangle tests, SurfaceInteraction, BVH traversal, textures, BxDFs,
// materials and light sampling -- each restating the reference function it cites.
#pragma once

#include <cuda_runtime.h>

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
// (the FP64 build compares in double: the next double above 1 -+ 1e-4)
#if LTS_FP64
#define kShadowEps 1e-4
#define kOneMinusEpsUp __longlong_as_double(__double_as_longlong(1.0 - 1e-4) + 1)
#define kOnePlusEpsUp __longlong_as_double(__double_as_longlong(1.0 + 1e-4) + 1)
#define kSlabScale (1.0 + 2.0 * gamma_n(3))
#else
#define kShadowEps 0.0001f
#define kOneMinusEpsUp __int_as_float(0x3f7ff973)
#define kOnePlusEpsUp __int_as_float(0x3f800347)
#define kSlabScale (1.0f + 2.0f * gamma_n(3))
#endif

// Per-thread traversal stack in shared memory, in 32-bit words (binary: one node per word; wide:
// one node group per two words).
constexpr int kStack = 48;
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
// Lobe masks (bit k: LobeKind k may occur): the BSDF functions take one as a template argument so
// that a kernel specialised to one material kind compiles only its lobes (LM_ALL: every lobe).
constexpr int LM_MATTE = (1 << LOBE_LAMBERT) | (1 << LOBE_OREN_NAYAR), LM_GLASS = 1 << LOBE_FRESNEL_SPECULAR,
              LM_MIRROR = 1 << LOBE_SPECULAR_REFL, LM_METAL = 1 << LOBE_MICROFACET,
              LM_ALL = LM_MATTE | LM_GLASS | LM_MIRROR | LM_METAL;
#define LTS_HAS_LOBE(LM, L) ((((LM) >> (L)) & 1) != 0)

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

// Event recording for the parity hash: h != nullptr mixes events into the sample's hash at once;
// h == nullptr captures the (single) event for a stage that must mix it later, in the
// reference's order (the wavefront records shadow and MIS results in later kernels).
struct EvSink {
    uint64_t* h;
    uint64_t cap;
    __device__ __forceinline__ void put(uint64_t v) {
        if (h) fnv_mix(*h, v);
        else cap = v;
    }
};

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
// The shading-record word of a triangle: (has vertex normals, mesh, area-light index, 0).
__device__ __forceinline__ int4 prim_word(const SceneView& sv, int prim) {
    return __ldg(reinterpret_cast<const int4*>(sv.prim_rec) + 8 * (size_t)prim + 6);
}

// ------------------------------------------------------------------ triangle tests
// Triangle::intersect test part (shapes/Triangle.cu:94-128).
// EXACT: the reference's arithmetic (its double-rounded cross products, unfused dot products);
// else the traversal's faster form: Kahan cross products and FMA dot products, a few ulps from
// the reference's values -- it only ranks the candidates, and the winner's values are recomputed
// exactly (make_si's `ro`).
__device__ __forceinline__ real dot_fma(V3 a, V3 b) { return xfma(a.z, b.z, xfma(a.y, b.y, a.x * b.x)); }
template <bool EXACT = true>
__device__ __forceinline__ bool tri_test(V3 p0, V3 p1, V3 p2, V3 o, V3 d, real tmax, real& t_out, real& u_out,
                                         real& v_out, real& inv_out) {
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const V3 pv = EXACT ? cross(d, e2) : cross_fast(d, e2);
    const real det = EXACT ? dot(e1, pv) : dot_fma(e1, pv);
    if (det == 0) return false;
    const real inv = xrcp(det);  // == (real)(1.0 / (double)det)
    const V3 tv = o - p0;
    const real u = inv * (EXACT ? dot(tv, pv) : dot_fma(tv, pv));
    if (u < kShadowEps || u >= kOneMinusEpsUp) return false;
    const V3 qv = EXACT ? cross(tv, e1) : cross_fast(tv, e1);
    const real v = inv * (EXACT ? dot(d, qv) : dot_fma(d, qv));
    if (v < kShadowEps || u + v >= kOneMinusEpsUp) return false;
    const real t = inv * (EXACT ? dot(e2, qv) : dot_fma(e2, qv));
    if (!(t > 0 && t < tmax)) return false;
    t_out = t;
    u_out = u;
    v_out = v;
    inv_out = inv;
    return true;
}
// Triangle::simpleIntersect (shapes/Triangle.cu:50-84): swapped edges, grown bound.
template <bool EXACT = true>
__device__ __forceinline__ bool tri_test_shadow(V3 p0, V3 p1, V3 p2, V3 o, V3 d, real tmax) {
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const V3 pv = EXACT ? cross(d, e1) : cross_fast(d, e1);
    const real det = EXACT ? dot(e2, pv) : dot_fma(e2, pv);
    if (det == 0) return false;
    const real inv = xrcp(det);
    const V3 tv = o - p0;
    const real u = inv * (EXACT ? dot(tv, pv) : dot_fma(tv, pv));
    if (u < kShadowEps || u >= kOnePlusEpsUp) return false;
    const V3 qv = EXACT ? cross(tv, e2) : cross_fast(tv, e2);
    const real v = inv * (EXACT ? dot(d, qv) : dot_fma(d, qv));
    if (v < kShadowEps || u + v >= kOnePlusEpsUp) return false;
    const real t = inv * (EXACT ? dot(e1, qv) : dot_fma(e1, qv));
    return t > 0 && t < tmax;
}

// Unfused products and differences (no FMA contraction): the watertight test below needs each
// 2D edge function to come out exactly negated when the two triangles sharing the edge evaluate
// it with their vertices in the other order.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ real vcomp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// ------------------------------------------------------------------ surface interaction
struct SI {
    V3 p, perr, wo, n;  // Interaction
    V3 dpdu, dpdv;      // geometric partials
    V3 sn, sdpdu;       // shading normal and tangent
    V3 dpdx, dpdy;      // computeDifferentials
    real tu, tv;        // surface uv at the hit (uvHit, Triangle.cu:160)
    int prim;
    int mesh, light;    // material index, area-light index (-1: none) of the primitive
};

// Cross products of the interaction's frames (make_si's normals and tangents, coordinate_system,
// make_bsdf): the faster form by default -- within 1.5 ulp, with every per-sample parity case
// inside its bound, 4 % more throughput on the stress scene -- or the reference's rounding
// (LTS_SI_CROSS=1: the stress scene's bit-exact share 0.76 instead of 0.70).  The hit's
// barycentrics always use the reference's rounding (make_si's `ro`).
#ifndef LTS_SI_CROSS
#define LTS_SI_CROSS 0
#endif
__device__ __forceinline__ V3 cross_si(V3 a, V3 b) { return LTS_SI_CROSS ? cross(a, b) : cross_fast(a, b); }

__device__ __forceinline__ void coordinate_system(V3 v1, V3& v2, V3& v3o) {
    // Geometry.cuh:250-258
    if (xabs(v1.x) > xabs(v1.y))
        v2 = v3(-v1.z, 0, v1.x) * rsqrt_q3(v1.x * v1.x + v1.z * v1.z);
    else
        v2 = v3(0, v1.z, -v1.y) * rsqrt_q3(v1.y * v1.y + v1.z * v1.z);
    v3o = cross_si(v1, v2);
}

// Builds the SurfaceInteraction of a hit (Triangle.cu:128-199 and the SurfaceInteraction
// constructor, geometry/Interaction.cuh:85-116).
// Triangle::intersect's SurfaceInteraction (shapes/Triangle.cu:130-203) from the triangle's
// shading record: positions, uvs (or the defaults) and vertex normals in one 128-byte line.
// With the ray's origin `ro` (closest hits found by the traversal, whose triangle tests use the
// faster cross products), the triangle test is repeated on the record's positions with the
// reference's rounding first, so that the interaction is built from the reference's barycentrics
// and 1 / det (a hit the exact test rejects, within rounding of an edge, keeps the traversal's
// values; the watertight test's values are its own).
__device__ void make_si(const SceneView& sv, int prim, V3 d, real u, real v, real inv, SI& si,
                        const V3* ro = nullptr) {
    const float4* rec = sv.prim_rec + 8 * (size_t)prim;
    const float4 r0 = __ldg(rec), r1 = __ldg(rec + 1), r2 = __ldg(rec + 2);
    const float4 r3 = __ldg(rec + 3), r4 = __ldg(rec + 4), r5 = __ldg(rec + 5);
    const int4 word = __ldg(reinterpret_cast<const int4*>(rec) + 6);
    const V3 p0 = v3(r0.x, r0.y, r0.z), p1 = v3(r1.x, r1.y, r1.z), p2 = v3(r2.x, r2.y, r2.z);
#if !LTS_FP64
    if (ro && !sv.watertight) {
        real t2, u2, v2, inv2;
        if (tri_test<true>(p0, p1, p2, *ro, d, INFINITY, t2, u2, v2, inv2)) {
            u = u2;
            v = v2;
            inv = inv2;
        }
    }
#endif
    const real w = 1 - u - v;
    const V3 e1 = p1 - p0, e2 = p2 - p0;
    const real uv0x = r0.w, uv0y = r1.w, uv1x = r2.w, uv1y = r3.w, uv2x = r4.w, uv2y = r5.w;
    const real d02x = uv0x - uv2x, d02y = uv0y - uv2y, d12x = uv1x - uv2x, d12y = uv1y - uv2y;
    const V3 dp02 = p0 - p2, dp12 = p1 - p2;
    const real determinant = d02x * d12y - d02y * d12x;
    V3 dpdu, dpdv;
    if (determinant == 0) {
        coordinate_system(normalize(cross_si(e2, e1)), dpdu, dpdv);
    } else {
        // the reference scales by the ray's invDet, not the uv determinant (Triangle.cu:148-149)
        dpdu = (dp02 * d12y - dp12 * d02y) * inv;
        dpdv = (dp02 * -d12x + dp12 * d02x) * inv;
    }
    const real xs = xabs(w * p0.x) + xabs(u * p1.x) + xabs(v * p2.x);
    const real ys = xabs(w * p0.y) + xabs(u * p1.y) + xabs(v * p2.y);
    const real zs = xabs(w * p0.z) + xabs(u * p1.z) + xabs(v * p2.z);
    si.perr = v3(xs, ys, zs) * gamma_n(7);
    si.p = p0 * w + p1 * u + p2 * v;
    si.tu = uv0x * w + uv1x * u + uv2x * v;
    si.tv = uv0y * w + uv1y * u + uv2y * v;
    si.wo = -d;
    si.dpdu = dpdu;
    si.dpdv = dpdv;
    si.n = normalize(cross_si(dpdu, dpdv));
    si.sn = si.n;
    si.sdpdu = dpdu;
    si.prim = prim;
    si.mesh = word.y;
    si.light = word.z;
    if (word.x) {
        const V3 n0 = v3(r3.x, r3.y, r3.z), n1 = v3(r4.x, r4.y, r4.z), n2 = v3(r5.x, r5.y, r5.z);
        const V3 ns = normalize(n0 * w + n1 * u + n2 * v);
        V3 ss = si.dpdu;
        V3 ts = cross_si(ns, ss);
        if (len2(ts) > 0.0f) {
            ts = normalize(ts);
            ss = cross_si(ts, ns);
        } else {
            coordinate_system(ns, ss, ts);
        }
        si.sn = normalize(cross_si(ss, ts));         // setShaddingGeometry
        si.n = face_towards(si.n, si.sn);
        si.sdpdu = ss;
        si.n = face_towards(si.n, si.sn);         // Triangle.cu:196
    }
}

// ------------------------------------------------------------------ BVH traversal
struct TraceRay {
    V3 o, d, inv;
    // direction sign per axis (from inv: -0 gives -inf), derived where used rather than held in
    // three more registers through the traversal loop
    __device__ __forceinline__ bool neg(int a) const { return (a == 0 ? inv.x : (a == 1 ? inv.y : inv.z)) < 0; }
};
__device__ __forceinline__ TraceRay make_trace_ray(V3 o, V3 d) {
    TraceRay r;
    r.o = o;
    r.d = d;
    r.inv = v3(xdiv(1.0f, d.x), xdiv(1.0f, d.y), xdiv(1.0f, d.z));
    return r;
}
// Bounds3::simpleIntersect (geometry/Bound.cuh:199-227), returning the entry distance.
__device__ __forceinline__ bool slab(const TraceRay& r, real tmax_ray, real mnx, real mny, real mnz, real mxx,
                                     real mxy, real mxz, real& tentry) {
    real tMin = ((r.neg(0) ? mxx : mnx) - r.o.x) * r.inv.x;
    real tMax = ((r.neg(0) ? mnx : mxx) - r.o.x) * r.inv.x;
    const real tyMin = ((r.neg(1) ? mxy : mny) - r.o.y) * r.inv.y;
    real tyMax = ((r.neg(1) ? mny : mxy) - r.o.y) * r.inv.y;
    tMax *= kSlabScale;
    tyMax *= kSlabScale;
    if (tMin > tyMax || tyMin > tMax) return false;
    if (tyMin > tMin) tMin = tyMin;
    if (tyMax < tMax) tMax = tyMax;
    const real tzMin = ((r.neg(2) ? mxz : mnz) - r.o.z) * r.inv.z;
    real tzMax = ((r.neg(2) ? mnz : mxz) - r.o.z) * r.inv.z;
    tzMax *= kSlabScale;
    if (tMin > tzMax || tzMin > tMax) return false;
    if (tzMin > tMin) tMin = tzMin;
    if (tzMax < tMax) tMax = tzMax;
    tentry = tMin;
    return (tMin < tmax_ray) && (tMax > 0);
}

// A closest hit as the traversal records it: the primitive id (below 2^24, the LBVH's limit) with
// the shade class of its material (1 .. 15) in bits 24 .. 27, both read from the leaf triangle
// (w of its first and second vertex), so the wavefront can group hits by class without reading
// the shading record; -1: no hit.
constexpr int kHitPrimBits = 24;
constexpr int kHitPrimMask = (1 << kHitPrimBits) - 1;
__device__ __forceinline__ int hit_prim(int best) { return best < 0 ? best : (best & kHitPrimMask); }
__device__ __forceinline__ int hit_class(int best) { return best < 0 ? 0 : (best >> kHitPrimBits); }

// Watertight ray/triangle test (the fixed mode of the reference's epsilon-shrunk Moller-Trumbore
// test, whose barycentric margin of 1e-4 lets rays through shared edges): Woop, Benthin and Wald,
// "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013.  The ray's dominant axis becomes z
// (x and y swapped when it points down that axis, to keep the winding), the vertices are sheared
// into ray space, and the signs of the three 2D edge functions decide inside or outside, with an
// edge function that rounds to zero recomputed in double (exact products).  A ray through a
// shared edge or vertex of a closed mesh hits one of its triangles.  t in (0, tmax) is tested
// before the division, on T and det.  u, v: the weights of p1 and p2, as tri_test returns them.
__device__ __forceinline__ bool tri_test_wt(V3 p0, V3 p1, V3 p2, const TraceRay& r, real tmax, real& t_out,
                                            real& u_out, real& v_out) {
    const real ax = xabs(r.d.x), ay = xabs(r.d.y), az = xabs(r.d.z);
    const int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
    if (vcomp(r.d, kz) < 0) {
        const int tmp = kx;
        kx = ky;
        ky = tmp;
    }
    const real rz = vcomp(r.inv, kz);
    const real sx = vcomp(r.d, kx) * rz, sy = vcomp(r.d, ky) * rz;
    const V3 A = p0 - r.o, B = p1 - r.o, C = p2 - r.o;
    const real Az0 = vcomp(A, kz), Bz0 = vcomp(B, kz), Cz0 = vcomp(C, kz);
    const real Ax = vcomp(A, kx) - sx * Az0, Ay = vcomp(A, ky) - sy * Az0;
    const real Bx = vcomp(B, kx) - sx * Bz0, By = vcomp(B, ky) - sy * Bz0;
    const real Cx = vcomp(C, kx) - sx * Cz0, Cy = vcomp(C, ky) - sy * Cz0;
    real U = sub_rn(mul_rn(Cx, By), mul_rn(Cy, Bx));
    real V = sub_rn(mul_rn(Ax, Cy), mul_rn(Ay, Cx));
    real W = sub_rn(mul_rn(Bx, Ay), mul_rn(By, Ax));
    if (U == 0 || V == 0 || W == 0) {
        U = (real)sub_rn(mul_rn((double)Cx, (double)By), mul_rn((double)Cy, (double)Bx));
        V = (real)sub_rn(mul_rn((double)Ax, (double)Cy), mul_rn((double)Ay, (double)Cx));
        W = (real)sub_rn(mul_rn((double)Bx, (double)Ay), mul_rn((double)By, (double)Ax));
    }
    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
    const real det = U + V + W;
    if (det == 0) return false;
    const real T = U * (rz * Az0) + V * (rz * Bz0) + W * (rz * Cz0);
    if (det > 0 ? (T <= 0 || T >= tmax * det) : (T >= 0 || T <= tmax * det)) return false;
    const real rcp = 1 / det;
    t_out = T * rcp;
    u_out = V * rcp;
    v_out = W * rcp;
    return true;
}
// The Moller-Trumbore 1 / det that make_si scales dpdu and dpdv by (the reference's quirk, kept
// in the watertight mode so that only the hit test differs).
__device__ __forceinline__ real mt_inv_det(V3 p0, V3 p1, V3 p2, V3 d) { return xrcp(dot(p1 - p0, cross(d, p2 - p0))); }

// The closest hit's barycentrics, 1 / det and distance with the reference's arithmetic: the
// traversal found triangle `prim` with the faster cross products; its test is repeated once with
// the exact ones (diff_prod), so the surface interaction is built from the reference's values.
// A hit the exact test rejects (within rounding of an edge) keeps the traversal's values.  The
// watertight test's values are its own.
__device__ __forceinline__ void hit_exact(const SceneView& sv, int prim, V3 o, V3 d, real& t, real& u, real& v,
                                          real& inv) {
#if !LTS_FP64
    if (sv.watertight) return;
    const float4* q = sv.prim_v + 3 * (size_t)prim;
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
    real t2, u2, v2, inv2;
    if (tri_test<true>(v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), o, d, INFINITY, t2, u2, v2, inv2)) {
        t = t2;
        u = u2;
        v = v2;
        inv = inv2;
    }
#endif
}

// The hit word of a leaf triangle: its primitive id and shade class from the triangle (top-level
// tree), or, inside instance `ii` of a two-level BVH, the instance's first primitive plus the
// triangle's index in its prototype and the instance's class; then 1 / det (make_si's dpdu scale)
// goes from object to world space (det scales with scale^3).
__device__ __forceinline__ int hit_word(float4 a, float4 b, const bool inst, int ii, const DevInstance* insts,
                                        real& binv) {
    if (inst && ii >= 0) {
        const int4 ref = __ldg(&insts[ii].ref);
        const real is = __ldg(&insts[ii].xf.w);
        binv = binv * (is * is * is);
        return (ref.y + __float_as_int(a.w)) | (ref.z << kHitPrimBits);
    }
    return __float_as_int(a.w) | (__float_as_int(b.w) << kHitPrimBits);
}

__device__ __forceinline__ bool leaf_test(const bool any, const float4* __restrict__ tv, int leaf, const TraceRay& r,
                                          real& tmax, int& best, real& bu, real& bv, real& binv, const bool wt,
                                          const bool inst = false, int ii = -1, const DevInstance* insts = nullptr) {
    const float4 a = __ldg(tv + 3 * leaf), b = __ldg(tv + 3 * leaf + 1), c = __ldg(tv + 3 * leaf + 2);
    real t, u, v, inv;
    if (wt) {
        if (!tri_test_wt(f4v(a), f4v(b), f4v(c), r, tmax, t, u, v)) return false;
        if (any) return true;
        tmax = t;
        bu = u;
        bv = v;
        binv = mt_inv_det(f4v(a), f4v(b), f4v(c), r.d);
        best = hit_word(a, b, inst, ii, insts, binv);
        return false;
    }
    if (any) return tri_test_shadow<false>(f4v(a), f4v(b), f4v(c), r.o, r.d, tmax);
    if (tri_test<false>(f4v(a), f4v(b), f4v(c), r.o, r.d, tmax, t, u, v, inv)) {
        tmax = t;
        bu = u;
        bv = v;
        binv = inv;
        best = hit_word(a, b, inst, ii, insts, binv);
    }
    return false;
}

// Traversal work counters of one thread (node visits, triangle tests).
struct Work {
    uint32_t nodes, tris;
};

// BVH traversal as a state machine: trav_begin sets a ray up, each trav_step opens one node, so a
// thread can run one ray to completion (traverse) or a persistent warp can interleave steps with
// fetching new rays for lanes whose ray has finished (the wavefront trace kernels).
//
// Binary LBVH (BVH::intersect / simpleIntersect, acceleration/BVH.cuh:331-398): both child
// boxes per node, nearer child first, the other on the stack (one word per entry).
// 8-wide compressed BVH: the same box test on the decoded (conservative) child boxes; children
// are visited in the order slot ^ octant(ray direction), nearest octant first; a node's leaf
// triangles are tested when it is opened; the stack holds (first child, remaining hit slots |
// imask << 8) groups, two words per entry.  `stack` is the thread's column of a shared-memory
// stack with row stride kThreads.
struct Trav {
    TraceRay r;
    real tmax, bu, bv, binv;
    int best;  // closest: primitive (-1 none); any: 1 on a hit
    int node, sp;
    uint32_t gbase, gbits;
    uint32_t lbits, lbase;  // split steps: the last node's pending triangles (bit k: triangle lbase + k)
    // two-level BVH: the instance being traversed (-1: the top-level tree, whose ray is the world
    // ray) and the instances whose world boxes the ray enters, still to visit
    int inst;
    uint32_t imask;
};

// Returns true when the ray needs traversal steps; false when it is already resolved (missed
// the scene bounds, or a one-triangle scene).  any: any hit (shadow rays), else closest hit.
__device__ __forceinline__ bool trav_begin(const bool any, Trav& t, const SceneView& sv, int nleaf, V3 o, V3 d,
                                           real tmax, Work& wk, const bool inst = false) {
    t.r = make_trace_ray(o, d);
    t.tmax = tmax;
    t.bu = t.bv = t.binv = 0.f;
    t.best = -1;
    t.node = 0;
    t.sp = 0;
    t.gbase = 0;
    t.gbits = 0;
    t.lbits = 0;
    t.lbase = 0;
    t.inst = -1;
    t.imask = 0;
    real te;
    const float* rb = sv.root_bounds;
    if (!slab(t.r, t.tmax, __ldg(rb), __ldg(rb + 1), __ldg(rb + 2), __ldg(rb + 3), __ldg(rb + 4), __ldg(rb + 5), te))
        return false;
    if (inst) {  // the instances whose world boxes the ray enters
        for (int i = 0; i < sv.ninst; ++i) {
            const float4 lo = __ldg(&sv.inst[i].wlo), hi = __ldg(&sv.inst[i].whi);
            if (slab(t.r, t.tmax, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, te)) t.imask |= 1u << i;
        }
    }
    if (nleaf == 1) {
        ++wk.tris;
        if (leaf_test(any, sv.leaf_v, 0, t.r, t.tmax, t.best, t.bu, t.bv, t.binv, sv.watertight != 0)) t.best = 1;
        return false;
    }
    return true;
}

#if !LTS_FP64  // the wide BVH is traversed in float only; the FP64 build uses the binary LBVH
// Child-box test of a wide node in FMA form.  Per node and axis: A = scale * inv,
// B = (p - o) * inv, so a plane's distance is q * A + B; both end planes are moved outwards by
// E = 16 * 2^-24 * |inv| * (|p| + |o| + 255 scale), which bounds the rounding of this form and of
// the reference's ((p + q scale) - o) * inv alike, so the interval contains the one the
// reference's box test computes for the decoded box; the far planes then get the reference's
// (1 + 2 gamma(3)) factor.  Needs finite inv (see trav_step_wide).
struct WideAxis {
    real A, Bn, Af, Bf;
    uint32_t near_lo, near_hi, far_lo, far_hi;  // the 8 near / far plane bytes of the axis
};
__device__ __forceinline__ WideAxis wide_axis(real p, real o, real inv, uint32_t ebyte, bool neg, uint32_t lo0,
                                              uint32_t lo1, uint32_t hi0, uint32_t hi1) {
    WideAxis a;
    const real sc = wide_scale(ebyte);
    const real A = sc * inv;
    const real B = (p - o) * inv;
    const real E = (16.0f * 5.9604645e-8f) * xabs(inv) * (xabs(p) + xabs(o) + 255.0f * sc);
    a.A = A;
    a.Bn = B - E;
    a.Af = A * kSlabScale;
    a.Bf = (B + E) * kSlabScale;
    a.near_lo = neg ? hi0 : lo0;
    a.near_hi = neg ? hi1 : lo1;
    a.far_lo = neg ? lo0 : hi0;
    a.far_hi = neg ? lo1 : hi1;
    return a;
}
__device__ __forceinline__ real wide_byte(uint32_t lo, uint32_t hi, int s) {
    // (a byte permute under the exponent of 2^23 and a subtraction measured 2.5 % slower)
    return __uint2float_rn(((s < 4 ? lo : hi) >> ((s & 3) * 8)) & 0xffu);
}
// Three-input min / max (one instruction on sm_100 and later: PTX ISA 8.8).
__device__ __forceinline__ float fmax3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
// Bit s of an 8-bit child mask to bit s ^ oct (the ray's octant order).
__device__ __forceinline__ uint32_t octant_order(uint32_t m, uint32_t oct) {
    if (oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (oct & 4u) m = ((m & 0x0fu) << 4) | ((m >> 4) & 0x0fu);
    return m;
}

// The triangles of a node's hit leaf slots `leaves`, given its leaf layout u (WideNode m.w):
// bit k set = triangle m.y + k.  A slot's group of u is 1, 3 or 7, so shifting it to the count
// of triangles in the slots before it gives the slot's triangles.
__device__ __forceinline__ uint32_t leaf_tri_bits(uint32_t leaves, uint32_t u) {
    uint32_t tb = 0;
    while (leaves) {
        const int s = __ffs(leaves) - 1;
        leaves &= leaves - 1u;
        tb |= ((u >> (3 * s)) & 7u) << __popc(u & ((1u << (3 * s)) - 1u));
    }
    return tb;
}

// One node; returns true when the traversal has finished.
__device__ __forceinline__ bool trav_step_wide(const bool any, Trav& t, const SceneView& sv, uint32_t* stack,
                                               uint32_t* err, Work& wk, const bool inst = false) {
    if ((unsigned)t.node >= (unsigned)sv.wcount) {
        atomicOr(err, DEV_ERR_BAD_INDEX);
        return true;
    }
    const uint32_t oct = (t.r.neg(0) ? 1u : 0u) | (t.r.neg(1) ? 2u : 0u) | (t.r.neg(2) ? 4u : 0u);
    const WideNode* nd = sv.wnodes + t.node;
    const float4 h = __ldg(&nd->h);
    const uint4 m = __ldg(&nd->m), q0 = __ldg(&nd->q0), q1 = __ldg(&nd->q1), q2 = __ldg(&nd->q2);
    ++wk.nodes;
    const uint32_t hb = __float_as_uint(h.w);
    const uint32_t imask = hb >> 24, omask = m.z;
    uint32_t hits = 0, leaves = 0;
    if (isfinite(t.r.inv.x) && isfinite(t.r.inv.y) && isfinite(t.r.inv.z)) {
        const WideAxis ax = wide_axis(h.x, t.r.o.x, t.r.inv.x, hb & 0xffu, t.r.neg(0), q0.x, q0.y, q1.z, q1.w);
        const WideAxis ay = wide_axis(h.y, t.r.o.y, t.r.inv.y, (hb >> 8) & 0xffu, t.r.neg(1), q0.z, q0.w, q2.x, q2.y);
        const WideAxis az = wide_axis(h.z, t.r.o.z, t.r.inv.z, (hb >> 16) & 0xffu, t.r.neg(2), q1.x, q1.y, q2.z, q2.w);
        // every slot is tested (a warp runs a slot's test whenever any of its nodes has that
        // slot) and the empty ones are masked off after; the interval is clipped to [0, tmax]
        // and tested once, which also enters the boxes touching t = 0 or t = tmax exactly (a
        // superset of the boxes the reference's test enters: the closest hit is unchanged)
        uint32_t hit8 = 0;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const real tnx = xfma(wide_byte(ax.near_lo, ax.near_hi, s), ax.A, ax.Bn);
            const real tny = xfma(wide_byte(ay.near_lo, ay.near_hi, s), ay.A, ay.Bn);
            const real tnz = xfma(wide_byte(az.near_lo, az.near_hi, s), az.A, az.Bn);
            const real tfx = xfma(wide_byte(ax.far_lo, ax.far_hi, s), ax.Af, ax.Bf);
            const real tfy = xfma(wide_byte(ay.far_lo, ay.far_hi, s), ay.Af, ay.Bf);
            const real tfz = xfma(wide_byte(az.far_lo, az.far_hi, s), az.Af, az.Bf);
            const real tn = fmax3f(tnx, tny, fmaxf(tnz, 0.0f)), tf = fmin3f(tfx, tfy, fminf(tfz, t.tmax));
            hit8 |= (tn <= tf ? 1u : 0u) << s;
        }
        hit8 &= omask;
        leaves = hit8 & ~imask;
        hits = octant_order(hit8 & imask, oct);
    } else {  // an axis-parallel ray: the reference's slab test on the decoded planes
        const real sx = wide_scale(hb & 0xffu), sy = wide_scale((hb >> 8) & 0xffu), sz = wide_scale((hb >> 16) & 0xffu);
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            if (!((omask >> s) & 1u)) continue;
            const int sh = (s & 3) * 8;
            const uint32_t lx = ((s < 4 ? q0.x : q0.y) >> sh) & 0xffu, ly = ((s < 4 ? q0.z : q0.w) >> sh) & 0xffu;
            const uint32_t lz = ((s < 4 ? q1.x : q1.y) >> sh) & 0xffu, hx = ((s < 4 ? q1.z : q1.w) >> sh) & 0xffu;
            const uint32_t hy = ((s < 4 ? q2.x : q2.y) >> sh) & 0xffu, hz = ((s < 4 ? q2.z : q2.w) >> sh) & 0xffu;
            real te;
            if (slab(t.r, t.tmax, wide_plane(h.x, lx, sx), wide_plane(h.y, ly, sy), wide_plane(h.z, lz, sz),
                     wide_plane(h.x, hx, sx), wide_plane(h.y, hy, sy), wide_plane(h.z, hz, sz), te)) {
                if ((imask >> s) & 1u) hits |= 1u << ((uint32_t)s ^ oct);
                else leaves |= 1u << s;
            }
        }
    }
    uint32_t tb = leaves ? leaf_tri_bits(leaves, m.w) : 0u;
    while (tb) {
        const int tri = (int)m.y + __ffs(tb) - 1;
        tb &= tb - 1u;
        if ((unsigned)tri >= (unsigned)sv.wtri_count) {
            atomicOr(err, DEV_ERR_BAD_INDEX);
            return true;
        }
        ++wk.tris;
        if (leaf_test(any, sv.wtris, tri, t.r, t.tmax, t.best, t.bu, t.bv, t.binv, sv.watertight != 0, inst, t.inst,
                      sv.inst)) {
            t.best = 1;
            return true;
        }
    }
    if (hits) {
        if (t.gbits & 0xffu) {
            if (2 * t.sp + 1 >= kStack) {
                atomicOr(err, DEV_ERR_STACK_OVERFLOW);
                return true;
            }
            stack[(2 * t.sp) * kThreads] = t.gbase;
            stack[(2 * t.sp + 1) * kThreads] = t.gbits;
            ++t.sp;
        }
        t.gbase = m.x;
        t.gbits = hits | (imask << 8);
    }
    if (!(t.gbits & 0xffu)) {
        if (t.sp == 0) return true;
        --t.sp;
        t.gbase = stack[(2 * t.sp) * kThreads];
        t.gbits = stack[(2 * t.sp + 1) * kThreads];
    }
    const uint32_t p = (uint32_t)__ffs(t.gbits & 0xffu) - 1u;
    t.gbits &= ~(1u << p);
    const uint32_t s = p ^ oct;
    t.node = (int)t.gbase + __popc((t.gbits >> 8) & ((1u << s) - 1u));
    return false;
}

// The same node visit split in two (the wavefront trace kernel): wide_node_step tests the child
// boxes and leaves the node's hit leaves pending in t.lbits instead of testing them; then
// wide_leaf_step tests them one triangle per call before the next node step.  Per ray the order
// of box and triangle tests is trav_step_wide's, so the hits are the same; a warp can run the
// triangle tests of all its lanes together instead of inside divergent node steps.  Both
// return true when the traversal has finished.
__device__ __forceinline__ bool wide_node_step(const bool any, Trav& t, const SceneView& sv, uint32_t* stack,
                                               uint32_t* err, Work& wk, const bool inst = false) {
    if ((unsigned)t.node >= (unsigned)sv.wcount) {
        atomicOr(err, DEV_ERR_BAD_INDEX);
        return true;
    }
    const uint32_t oct = (t.r.neg(0) ? 1u : 0u) | (t.r.neg(1) ? 2u : 0u) | (t.r.neg(2) ? 4u : 0u);
    const WideNode* nd = sv.wnodes + t.node;
    const float4 h = __ldg(&nd->h);
    const uint4 m = __ldg(&nd->m), q0 = __ldg(&nd->q0), q1 = __ldg(&nd->q1), q2 = __ldg(&nd->q2);
    ++wk.nodes;
    const uint32_t hb = __float_as_uint(h.w);
    const uint32_t imask = hb >> 24, omask = m.z;
    uint32_t hits = 0, leaves = 0;
    if (isfinite(t.r.inv.x) && isfinite(t.r.inv.y) && isfinite(t.r.inv.z)) {
        const WideAxis ax = wide_axis(h.x, t.r.o.x, t.r.inv.x, hb & 0xffu, t.r.neg(0), q0.x, q0.y, q1.z, q1.w);
        const WideAxis ay = wide_axis(h.y, t.r.o.y, t.r.inv.y, (hb >> 8) & 0xffu, t.r.neg(1), q0.z, q0.w, q2.x, q2.y);
        const WideAxis az = wide_axis(h.z, t.r.o.z, t.r.inv.z, (hb >> 16) & 0xffu, t.r.neg(2), q1.x, q1.y, q2.z, q2.w);
        // every slot is tested (a warp runs a slot's test whenever any of its nodes has that
        // slot) and the empty ones are masked off after; the interval is clipped to [0, tmax]
        // and tested once, which also enters the boxes touching t = 0 or t = tmax exactly (a
        // superset of the boxes the reference's test enters: the closest hit is unchanged)
        uint32_t hit8 = 0;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const real tnx = xfma(wide_byte(ax.near_lo, ax.near_hi, s), ax.A, ax.Bn);
            const real tny = xfma(wide_byte(ay.near_lo, ay.near_hi, s), ay.A, ay.Bn);
            const real tnz = xfma(wide_byte(az.near_lo, az.near_hi, s), az.A, az.Bn);
            const real tfx = xfma(wide_byte(ax.far_lo, ax.far_hi, s), ax.Af, ax.Bf);
            const real tfy = xfma(wide_byte(ay.far_lo, ay.far_hi, s), ay.Af, ay.Bf);
            const real tfz = xfma(wide_byte(az.far_lo, az.far_hi, s), az.Af, az.Bf);
            const real tn = fmax3f(tnx, tny, fmaxf(tnz, 0.0f)), tf = fmin3f(tfx, tfy, fminf(tfz, t.tmax));
            hit8 |= (tn <= tf ? 1u : 0u) << s;
        }
        hit8 &= omask;
        leaves = hit8 & ~imask;
        hits = octant_order(hit8 & imask, oct);
    } else {  // an axis-parallel ray: the reference's slab test on the decoded planes
        const real sx = wide_scale(hb & 0xffu), sy = wide_scale((hb >> 8) & 0xffu), sz = wide_scale((hb >> 16) & 0xffu);
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            if (!((omask >> s) & 1u)) continue;
            const int sh = (s & 3) * 8;
            const uint32_t lx = ((s < 4 ? q0.x : q0.y) >> sh) & 0xffu, ly = ((s < 4 ? q0.z : q0.w) >> sh) & 0xffu;
            const uint32_t lz = ((s < 4 ? q1.x : q1.y) >> sh) & 0xffu, hx = ((s < 4 ? q1.z : q1.w) >> sh) & 0xffu;
            const uint32_t hy = ((s < 4 ? q2.x : q2.y) >> sh) & 0xffu, hz = ((s < 4 ? q2.z : q2.w) >> sh) & 0xffu;
            real te;
            if (slab(t.r, t.tmax, wide_plane(h.x, lx, sx), wide_plane(h.y, ly, sy), wide_plane(h.z, lz, sz),
                     wide_plane(h.x, hx, sx), wide_plane(h.y, hy, sy), wide_plane(h.z, hz, sz), te)) {
                if ((imask >> s) & 1u) hits |= 1u << ((uint32_t)s ^ oct);
                else leaves |= 1u << s;
            }
        }
    }
    if (leaves) {
        t.lbits = leaf_tri_bits(leaves, m.w);
        t.lbase = m.y;
    }
    if (hits) {
        if (t.gbits & 0xffu) {
            if (2 * t.sp + 1 >= kStack) {
                atomicOr(err, DEV_ERR_STACK_OVERFLOW);
                return true;
            }
            stack[(2 * t.sp) * kThreads] = t.gbase;
            stack[(2 * t.sp + 1) * kThreads] = t.gbits;
            ++t.sp;
        }
        t.gbase = m.x;
        t.gbits = hits | (imask << 8);
    }
    if (!(t.gbits & 0xffu)) {
        if (t.sp == 0) {  // no node left: done unless leaves are pending
            t.node = -1;
            return t.lbits == 0u;
        }
        --t.sp;
        t.gbase = stack[(2 * t.sp) * kThreads];
        t.gbits = stack[(2 * t.sp + 1) * kThreads];
    }
    const uint32_t p = (uint32_t)__ffs(t.gbits & 0xffu) - 1u;
    t.gbits &= ~(1u << p);
    const uint32_t s = p ^ oct;
    t.node = (int)t.gbase + __popc((t.gbits >> 8) & ((1u << s) - 1u));
    return false;
}


__device__ __forceinline__ bool wide_leaf_step(const bool any, Trav& t, const SceneView& sv, uint32_t* err, Work& wk,
                                               const bool inst = false) {
    const int tri = (int)t.lbase + __ffs(t.lbits) - 1;
    t.lbits &= t.lbits - 1u;
    if ((unsigned)tri >= (unsigned)sv.wtri_count) {
        atomicOr(err, DEV_ERR_BAD_INDEX);
        return true;
    }
    ++wk.tris;
    if (leaf_test(any, sv.wtris, tri, t.r, t.tmax, t.best, t.bu, t.bv, t.binv, sv.watertight != 0, inst, t.inst,
                  sv.inst)) {
        t.best = 1;
        return true;
    }
    return t.lbits == 0u && t.node < 0;
}

#endif  // !LTS_FP64

__device__ __forceinline__ bool trav_step_binary(const bool any, Trav& t, const SceneView& sv, uint32_t* stack,
                                                 uint32_t* err, Work& wk) {
    const BvhNode* nd = sv.nodes + t.node;
    const float4 a = __ldg(&nd->a), b = __ldg(&nd->b), c = __ldg(&nd->c);
    const int4 lr = __ldg(&nd->d);
    ++wk.nodes;
    real tl, tr;
    bool hl = slab(t.r, t.tmax, a.x, a.y, a.z, a.w, b.x, b.y, tl);
    bool hr = slab(t.r, t.tmax, b.z, b.w, c.x, c.y, c.z, c.w, tr);
    if (hl && lr.x < 0) {
        ++wk.tris;
        if (leaf_test(any, sv.leaf_v, ~lr.x, t.r, t.tmax, t.best, t.bu, t.bv, t.binv, sv.watertight != 0)) {
            t.best = 1;
            return true;
        }
        hl = false;
    }
    if (hr && lr.y < 0) {
        ++wk.tris;
        if (leaf_test(any, sv.leaf_v, ~lr.y, t.r, t.tmax, t.best, t.bu, t.bv, t.binv, sv.watertight != 0)) {
            t.best = 1;
            return true;
        }
        hr = false;
    }
    if (hl && hr) {
        const bool left_first = tl <= tr;
        if (t.sp >= kStack) {  // one word per entry
            atomicOr(err, DEV_ERR_STACK_OVERFLOW);
            return true;
        }
        stack[(t.sp++) * kThreads] = left_first ? lr.y : lr.x;
        t.node = left_first ? lr.x : lr.y;
    } else if (hl) {
        t.node = lr.x;
    } else if (hr) {
        t.node = lr.y;
    } else {
        if (t.sp == 0) return true;
        t.node = stack[(--t.sp) * kThreads];
    }
    return false;
}

__device__ __forceinline__ bool trav_step(const bool any, Trav& t, const SceneView& sv, uint32_t* stack, uint32_t* err,
                                          Work& wk, const bool inst = false) {
#if LTS_FP64
    return trav_step_binary(any, t, sv, stack, err, wk);
#else
    return sv.wnodes ? trav_step_wide(any, t, sv, stack, err, wk, inst) : trav_step_binary(any, t, sv, stack, err, wk);
#endif
}

#if !LTS_FP64
// Two-level BVH: when the traversal of the top-level tree or of an instance has finished, starts
// the next instance whose world box the ray entered (its object-space ray o' = (o - t) / scale,
// d' = d / scale keeps the ray parameter, so tmax carries over), skipping instances whose
// prototype box lies beyond the closest hit so far.  Returns false when none is left (or an
// any-hit query has its hit).
__device__ __forceinline__ bool inst_next(const bool any, Trav& t, const SceneView& sv, V3 wo, V3 wd) {
    if (any && t.best == 1) return false;
    while (t.imask) {
        const int i = __ffs(t.imask) - 1;
        t.imask &= t.imask - 1u;
        const DevInstance* I = sv.inst + i;
        const float4 xf = __ldg(&I->xf), lo = __ldg(&I->olo), hi = __ldg(&I->ohi);
        const int4 ref = __ldg(&I->ref);
        t.r = make_trace_ray(v3((wo.x - xf.x) * xf.w, (wo.y - xf.y) * xf.w, (wo.z - xf.z) * xf.w),
                             v3(wd.x * xf.w, wd.y * xf.w, wd.z * xf.w));
        real te;
        if (!slab(t.r, t.tmax, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, te)) continue;
        t.inst = i;
        t.node = ref.x;
        t.sp = 0;
        t.gbase = 0;
        t.gbits = 0;
        t.lbits = 0;
        return true;
    }
    return false;
}
#endif

// Whole traversal: the hit primitive (closest) or 1 / -1 (any), -1 for a miss.
template <bool ANY, bool INST = false>
__device__ int traverse(const SceneView& sv, int nleaf, const TraceRay& r, real& tmax, real& bu, real& bv,
                        real& binv, uint32_t* stack, uint32_t* err, Work& wk) {
    Trav t;
    if (trav_begin(ANY, t, sv, nleaf, r.o, r.d, tmax, wk, INST)) {
        for (;;) {
            while (!trav_step(ANY, t, sv, stack, err, wk, INST)) {
            }
#if !LTS_FP64
            if (INST && inst_next(ANY, t, sv, r.o, r.d)) continue;
#endif
            break;
        }
    }
    tmax = t.tmax;
    bu = t.bu;
    bv = t.bv;
    binv = t.binv;
    return ANY ? (t.best == 1 ? 1 : -1) : hit_prim(t.best);
}

struct Hit {
    bool found;
    SI si;
};

__device__ __forceinline__ bool scene_intersect(const SceneView& sv, int nleaf, V3 o, V3 d, real tmax, SI& si,
                                                uint32_t* stack, uint32_t* err, Work& wk) {
    const TraceRay r = make_trace_ray(o, d);
    real bu = 0, bv = 0, binv = 0;
#if !LTS_FP64
    // one traversal loop for both BVH forms (without instances the instance mask stays empty), so
    // the megakernel inlines a single copy
    const int prim = traverse<false, true>(sv, nleaf, r, tmax, bu, bv, binv, stack, err, wk);
#else
    const int prim = traverse<false>(sv, nleaf, r, tmax, bu, bv, binv, stack, err, wk);
#endif
    if (prim < 0) return false;
    make_si(sv, prim, d, bu, bv, binv, si, &o);
    return true;
}
__device__ __forceinline__ bool scene_occluded(const SceneView& sv, int nleaf, V3 o, V3 d, real tmax, uint32_t* stack,
                                               uint32_t* err, Work& wk) {
    const TraceRay r = make_trace_ray(o, d);
    real bu, bv, binv;
#if !LTS_FP64
    return traverse<true, true>(sv, nleaf, r, tmax, bu, bv, binv, stack, err, wk) > 0;
#else
    return traverse<true>(sv, nleaf, r, tmax, bu, bv, binv, stack, err, wk) > 0;
#endif
}

// ------------------------------------------------------------------ rays from interactions
// offsetRayOrigin (Geometry.cuh:782-797)
__device__ __forceinline__ V3 offset_origin(V3 p, V3 perr, V3 n, V3 w) {
    const real dd = dot(vabs(n), perr);
    V3 off = n * dd;
    if (dot(w, n) < 0) off = -off;
    V3 po = p + off;
    if (off.x > 0) po.x = next_float_up(po.x); else if (off.x < 0) po.x = next_float_down(po.x);
    if (off.y > 0) po.y = next_float_up(po.y); else if (off.y < 0) po.y = next_float_down(po.y);
    if (off.z > 0) po.z = next_float_up(po.z); else if (off.z < 0) po.z = next_float_down(po.z);
    return po;
}

// ------------------------------------------------------------------ textures
// Perlin permutation and marble colour tables in device memory, read through L1: the lanes of a
// warp index them at different places, which the constant cache would serve one address at a
// time (a 512-byte table spans four L1 lines).
__device__ unsigned char c_perm[512];
__device__ float c_marble[10][3];

__device__ __forceinline__ real noise_weight(real t) {
    const real t3 = t * t * t, t4 = t3 * t;
    return 6 * t4 * t - 15 * t4 + 10 * t3;
}
__device__ __forceinline__ real lerpf(real t, real a, real b) { return (1 - t) * a + t * b; }
__device__ __forceinline__ real grad(int x, int y, int z, real dx, real dy, real dz) {
    int h = __ldg(c_perm + __ldg(c_perm + __ldg(c_perm + x) + y) + z);
    h &= 15;
    const real u = h < 8 || h == 12 || h == 13 ? dx : dy;
    const real v = h < 4 || h == 12 || h == 13 ? dy : dz;
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}
// textures/Procedural.cuh:130-155 (improved Perlin noise)
__device__ real perlin(real x, real y, real z) {
    int ix = (int)xfloor(x), iy = (int)xfloor(y), iz = (int)xfloor(z);
    const real dx = x - ix, dy = y - iy, dz = z - iz;
    ix &= 255;
    iy &= 255;
    iz &= 255;
    const real w000 = grad(ix, iy, iz, dx, dy, dz);
    const real w100 = grad(ix + 1, iy, iz, dx - 1, dy, dz);
    const real w010 = grad(ix, iy + 1, iz, dx, dy - 1, dz);
    const real w001 = grad(ix, iy, iz + 1, dx, dy, dz - 1);
    const real w110 = grad(ix + 1, iy + 1, iz, dx - 1, dy - 1, dz);
    const real w011 = grad(ix, iy + 1, iz + 1, dx, dy - 1, dz - 1);
    const real w101 = grad(ix + 1, iy, iz + 1, dx - 1, dy, dz - 1);
    const real w111 = grad(ix + 1, iy + 1, iz + 1, dx - 1, dy - 1, dz - 1);
    const real wx = noise_weight(dx), wy = noise_weight(dy), wz = noise_weight(dz);
    const real x00 = lerpf(wx, w000, w100), x10 = lerpf(wx, w010, w110);
    const real x01 = lerpf(wx, w001, w101), x11 = lerpf(wx, w011, w111);
    const real y0 = lerpf(wy, x00, x10), y1 = lerpf(wy, x01, x11);
    return lerpf(wz, y0, y1);
}
__device__ __forceinline__ real smooth_step(real mn, real mx, real val) {
    const real v = clampf((val - mn) / (mx - mn), 0, 1);
    return v * v * (-2 * v + 3);
}
__device__ __forceinline__ real octaves_of(V3 dpdx, V3 dpdy, int max_oct) {
    const real l2 = xmax(len2(dpdx), len2(dpdy));
    return clampf(-1 - 0.5f * xlog2(l2), 0, (real)max_oct);
}
// Procedural.cuh:161-179
__device__ real fbm(V3 p, V3 dpdx, V3 dpdy, real omega, int max_oct, EvSink* sig) {
    const real n = octaves_of(dpdx, dpdy, max_oct);
    const int ni = (int)xfloor(n);
    if (sig) sig->put(0x400000000ull + (unsigned)ni);
    real sum = 0, lambda = 1, o = 1;
    for (int i = 0; i < ni; ++i) {
        sum += o * perlin(p.x * lambda, p.y * lambda, p.z * lambda);
        lambda *= 1.99f;
        o *= omega;
    }
    const real np = n - ni;
    sum += o * smooth_step(0.3f, 0.7f, np) * perlin(p.x * lambda, p.y * lambda, p.z * lambda);
    return sum;
}
// Procedural.cuh:181-205
__device__ real turbulence(V3 p, V3 dpdx, V3 dpdy, real omega, int max_oct, EvSink* sig) {
    const real n = octaves_of(dpdx, dpdy, max_oct);
    const int ni = (int)xfloor(n);
    if (sig) sig->put(0x400000000ull + (unsigned)ni);
    real sum = 0, lambda = 1, o = 1;
    for (int i = 0; i < ni; ++i) {
        sum += o * xabs(perlin(p.x * lambda, p.y * lambda, p.z * lambda));
        lambda *= 1.99f;
        o *= omega;
    }
    const real np = n - ni;
    sum += o * lerpf(smooth_step(0.3f, 0.7f, np), 0.2f, xabs(perlin(p.x * lambda, p.y * lambda, p.z * lambda)));
    for (int i = ni; i < max_oct; ++i) {
        sum += o * 0.2f;
        o *= omega;
    }
    return sum;
}

// Image textures, the fixed mode of ImageTexture::evaluate (ImageTexture.cuh:24-28) over its
// Mipmap (Mipmap.cuh:14-73) in the reference's operation order.  Fixed: the repeat mode wraps
// negative coordinates into the level (the reference's fmodf leaves them negative and reads
// before the level's storage), and a level coordinate past the coarsest level reads texel (0, 0)
// of that level (the reference reads texel (levels - 1, 0) of level 0).
__device__ __forceinline__ Spec img_texel(const SceneView& sv, const DevImage* im, int l, int s, int t) {
    const int w = __ldg(&im->w[l]), h = __ldg(&im->h[l]), wrap = __ldg(&im->wrap);
    if (wrap == 0) {
        s %= w;
        if (s < 0) s += w;
        t %= h;
        if (t < 0) t += h;
    } else if (wrap == 2) {
        s = s < 0 ? 0 : (s > w - 1 ? w - 1 : s);
        t = t < 0 ? 0 : (t > h - 1 ? h - 1 : t);
    } else if (s < 0 || s >= w || t < 0 || t >= h) {
        return spec(0.0f);
    }
    const float4 q = __ldg(sv.img_texels + __ldg(&im->off[l]) + 16 * ((t >> 2) * ((w + 3) >> 2) + (s >> 2)) +
                           4 * (t & 3) + (s & 3));
    return Spec{q.x, q.y, q.z};
}
// Mipmap::triangle: bilinear over level l (clamped to the pyramid).
__device__ __forceinline__ Spec img_bilerp(const SceneView& sv, const DevImage* im, int l, real st0, real st1) {
    const int levels = __ldg(&im->levels);
    l = l < 0 ? 0 : (l > levels - 1 ? levels - 1 : l);
    const real s = st0 * (real)__ldg(&im->w[l]) - 0.5f, t = st1 * (real)__ldg(&im->h[l]) - 0.5f;
    const int s0 = (int)xfloor(s), t0 = (int)xfloor(t);
    const real ds = s - (real)s0, dt = t - (real)t0;
    return img_texel(sv, im, l, s0, t0) * ((1 - ds) * (1 - dt)) + img_texel(sv, im, l, s0, t0 + 1) * ((1 - ds) * dt) +
           img_texel(sv, im, l, s0 + 1, t0) * (ds * (1 - dt)) + img_texel(sv, im, l, s0 + 1, t0 + 1) * (ds * dt);
}
// Mipmap::lookUp at the fixed width 0.01 (EVALUATION_WIDTH), whose level coordinate the loader
// computes once per image.
__device__ __noinline__ Spec img_lookup(const SceneView& sv, int idx, real st0, real st1) {
    const DevImage* im = sv.images + idx;
    const real lod = __ldg(&im->lod);
    const int levels = __ldg(&im->levels);
    if (lod < 0) return img_bilerp(sv, im, 0, st0, st1);
    if (lod >= (real)(levels - 1)) return img_texel(sv, im, levels - 1, 0, 0);
    const int il = (int)xfloor(lod);
    const real delta = lod - (real)il;
    return img_bilerp(sv, im, il, st0, st1) * (1 - delta) + img_bilerp(sv, im, il + 1, st0, st1) * delta;
}

// TEX false: the material's textures are constants (a kernel specialised to such materials
// compiles none of the procedural or image textures).
template <bool TEX = true>
__device__ Spec eval_texture(const SceneView& sv, const DevTex& t, const SI& si, EvSink* sig) {
    if (!TEX) return Spec{t.v[0], t.v[1], t.v[2]};
    switch (t.kind) {
        case 5:  // ImageTexture with UVMapping2D(1, 1, 0, 0) (SceneLoader.cuh:375): st = uv
            return img_lookup(sv, (int)t.v[0], si.tu, si.tv);
        case 1:  // FBmTexture (Procedural.cuh:207-225)
            return spec(fbm(si.p, si.dpdx, si.dpdy, t.v[1], (int)t.v[0], sig));
        case 2:  // WrinkledTexture (Procedural.cuh:227-245)
            return spec(turbulence(si.p, si.dpdx, si.dpdy, t.v[1], (int)t.v[0], sig));
        case 3: {  // MarbleTexture (Procedural.cuh:267-311)
            const real scale = t.v[2], var = t.v[3];
            const V3 p = si.p * scale;
            const real marble = p.y + var * fbm(p, si.dpdx * scale, si.dpdy * scale, t.v[1], (int)t.v[0], sig);
            real tt = 0.5f + 0.5f * xsin(marble);
            const int first = (int)xfloor(tt * 6.0f);
            if (sig) sig->put(0x500000000ull + (unsigned)first);
            tt = (tt * 6.0f - first);
            Spec c[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                c[k] = Spec{__ldg(&c_marble[first + k][0]), __ldg(&c_marble[first + k][1]), __ldg(&c_marble[first + k][2])};
            Spec s0 = c[0] * (1.0f - tt) + c[1] * tt;
            Spec s1 = c[1] * (1.0f - tt) + c[2] * tt;
            const Spec s2 = c[2] * (1.0f - tt) + c[3] * tt;
            s0 = s0 * (1.0f - tt) + s1 * tt;
            s1 = s1 * (1.0f - tt) + s2 * tt;
            return (s0 * (1.0f - tt) + s1 * tt) * 1.5f;
        }
        case 4: {  // WindyTexture (Procedural.cuh:247-265)
            const real wind = fbm(si.p * 0.1f, si.dpdx * 0.1f, si.dpdy * 0.1f, 0.5f, 3, sig);
            const real wave = fbm(si.p, si.dpdx, si.dpdy, 0.5f, 6, sig);
            return spec(xabs(wind) * wave);
        }
        default:
            return Spec{t.v[0], t.v[1], t.v[2]};
    }
}

// ------------------------------------------------------------------ BxDFs
__device__ __forceinline__ real cos2t(V3 w) { return w.z * w.z; }
__device__ __forceinline__ real sin2t(V3 w) { return xmax(1 - cos2t(w), 0.0f); }
__device__ __forceinline__ real sint(V3 w) { return xsqrt(sin2t(w)); }
__device__ __forceinline__ real tant(V3 w) { return sint(w) / w.z; }
__device__ __forceinline__ real tan2t(V3 w) { return sin2t(w) / cos2t(w); }
// cosPhi/sinPhi compare the function sinTheta (not its value) with 0, so they never take the
// sin == 0 branch (models/BxDF.cuh:144-153).
__device__ __forceinline__ real cosphi(V3 w) { return clampf(w.x / sint(w), -1, 1); }
__device__ __forceinline__ real sinphi(V3 w) { return clampf(w.y / sint(w), -1, 1); }
__device__ __forceinline__ bool same_hemi(V3 a, V3 b, EvSink* sig) {  // sameHemisphere, recorded
    const bool v = a.z * b.z > 0;
    if (sig) sig->put(0x700000000ull + (v ? 1u : 0u));
    return v;
}

// models/BxDF.cuh:16-37 with the swapped clamp bounds of line 17.
__device__ real fresnel_dielectric(real cos_i, real eta_i, real eta_t) {
    cos_i = clampf(cos_i, 1, -1);
    const bool entering = cos_i > 0.0f;
    if (!entering) {
        const real tmp = eta_i;
        eta_i = eta_t;
        eta_t = tmp;
        cos_i = xabs(cos_i);
    }
    const real sin_i = xsqrt(xmax(0.0f, 1 - cos_i * cos_i));
    const real sin_t = eta_i / eta_t * sin_i;
    if (sin_t >= 1) return 1;
    const real cos_t = xsqrt(xmax(0.0f, 1 - sin_t * sin_t));
    const real rpar = ((eta_t * cos_i) - (eta_i * cos_t)) / ((eta_t * cos_i) + (eta_i * cos_t));
    const real rperp = ((eta_i * cos_i) - (eta_t * cos_t)) / ((eta_i * cos_i) + (eta_t * cos_t));
    return (rpar * rpar + rperp * rperp) / 2;
}
// models/BxDF.cuh:44-67 (etaI = 1)
__device__ Spec fresnel_conductor(real cos_i, Spec eta_t, Spec k) {
    cos_i = clampf(cos_i, -1, 1);
    const Spec eta = eta_t / 1.0f, etak = k / 1.0f;
    const real c2 = cos_i * cos_i, s2 = 1.0f - c2;
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
__device__ __forceinline__ bool refract(V3 wi, V3 n, real eta, V3& wt) {
    const real ci = dot(n, wi);
    const real s2i = xmax(0.0f, 1.0f - ci * ci);
    const real s2t = eta * eta * s2i;
    if (s2t >= 1) return false;
    const real ct = xsqrt(1 - s2t);
    wt = -wi * eta + n * (eta * ci - ct);
    return true;
}

// Trowbridge-Reitz (models/Microfacet.cuh:53-181)
__device__ real tr_lambda(V3 w, real ax, real ay) {
    const real at = xabs(tant(w));
    if (isinf(at)) return 0.0f;
    const real cp = cosphi(w), sp = sinphi(w);
    const real alpha = xsqrt(cp * cp * ax * ax + sp * sp * ay * ay);
    const real a2t2 = (alpha * at) * (alpha * at);
    return (-1 + xsqrt(1.0f + a2t2)) / 2;
}
__device__ real tr_d(V3 wh, real ax, real ay) {
    const real t2 = tan2t(wh);
    if (isinf(t2)) return 0;
    const real c4 = cos2t(wh) * cos2t(wh);
    const real cp = cosphi(wh), sp = sinphi(wh);
    const real e = (cp * cp / (ax * ax) + sp * sp / (ay * ay)) * t2;
    return 1 / (3.14159265358979f * ax * ay * c4 * (1 + e) * (1 + e));
}
__device__ __forceinline__ real tr_g1(V3 w, real ax, real ay) { return 1 / (1 + tr_lambda(w, ax, ay)); }
__device__ __forceinline__ real tr_g(V3 wo, V3 wi, real ax, real ay) {
    return 1 / (1 + tr_lambda(wo, ax, ay) + tr_lambda(wi, ax, ay));
}
__device__ void tr_sample11(real cosT, real U1, real U2, real& sx, real& sy) {
    if (cosT >= kOneMinusEpsUp) {
        const real r = xsqrt(U1 / (1 - U1));
        const real phi = mul_dc(U2, LTS_2PI);
#if !LTS_FP64
        if (c_libm_double) {  // the reference calls cos / sin in double here and multiplies in double
            sx = (float)((double)r * cos((double)phi));
            sy = (float)((double)r * sin((double)phi));
            return;
        }
#endif
        sx = r * xcos(phi);
        sy = r * xsin(phi);
        return;
    }
    const real sinT = xsqrt(xmax(0.0f, 1.0f - cosT * cosT));
    const real tanT = sinT / cosT;
    const real a = 1 / tanT;
    const real G1 = 2 / (1 + xsqrt(1.f + 1.f / (a * a)));
    const real A = 2 * U1 / G1 - 1;
    real tmp = 1.f / (A * A - 1.f);
    if (tmp > 1e10f) tmp = 1e10f;
    const real B = tanT;
    const real D = xsqrt(xmax(real(B * B * tmp * tmp - (A * A - B * B) * tmp), 0.0f));
    const real s1 = B * tmp - D, s2 = B * tmp + D;
    sx = (A < 0 || s2 > 1.f / tanT) ? s1 : s2;
    real S;
    if (U2 > 0.5f) {
        S = 1.f;
        U2 = 2.f * (U2 - .5f);
    } else {
        S = -1.f;
        U2 = 2.f * (.5f - U2);
    }
    const real z = (U2 * (U2 * (U2 * 0.27385f - 0.73369f) + 0.46341f)) /
                    (U2 * (U2 * (U2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
    sy = S * z * xsqrt(1.f + sx * sx);
}
__device__ V3 tr_sample(V3 wi, real ax, real ay, real U1, real U2) {
    const V3 ws = normalize(v3(ax * wi.x, ay * wi.y, wi.z));
    real sx, sy;
    tr_sample11(ws.z, U1, U2, sx, sy);
    const real tmp = cosphi(ws) * sx - sinphi(ws) * sy;
    sy = sinphi(ws) * sx + cosphi(ws) * sy;
    sx = tmp;
    sx = ax * sx;
    sy = ay * sy;
    return normalize(v3(-sx, -sy, 1.f));
}

// TrowbridgeReitzMicrofacetDistribution::sampleWH and ::Pdf (Microfacet.cuh:175-189)
__device__ __forceinline__ V3 tr_sample_wh(V3 wo, real ax, real ay, real U1, real U2) {
    const bool flip = wo.z < 0;
    V3 wh = tr_sample(flip ? -wo : wo, ax, ay, U1, U2);
    if (flip) wh = -wh;
    return wh;
}
__device__ __forceinline__ real tr_pdf(V3 wo, V3 wh, real ax, real ay) {
    return tr_d(wh, ax, ay) * tr_g1(wo, ax, ay) * absdot(wo, wh) / xabs(wo.z);
}

struct Bsdf {
    int lobe;           // LobeKind; at most one lobe for every reachable material
    uint32_t type;      // BxDF type bits of the lobe
    V3 ns, ng, ss, ts;
    Spec R, T, k, eta3;
    real eta, a, b, alpha;
};

__device__ __forceinline__ V3 to_local(const Bsdf& f, V3 v) { return v3(dot(v, f.ss), dot(v, f.ts), dot(v, f.ns)); }
__device__ __forceinline__ V3 to_world(const Bsdf& f, V3 v) {
    return v3(f.ss.x * v.x + f.ts.x * v.y + f.ns.x * v.z, f.ss.y * v.x + f.ts.y * v.y + f.ns.y * v.z,
              f.ss.z * v.x + f.ts.z * v.y + f.ns.z * v.z);
}
__device__ __forceinline__ bool matches(uint32_t type, uint32_t flags) { return (type & flags) == type; }

// BxDF::f
template <int LM = LM_ALL>
__device__ Spec lobe_f(const Bsdf& f, V3 wo, V3 wi) {
    switch (f.lobe) {
        case LOBE_LAMBERT:
            if (!LTS_HAS_LOBE(LM, LOBE_LAMBERT)) return spec(0.0f);
            return f.R * LTS_INV_PI_F;
        case LOBE_OREN_NAYAR: {  // Microfacet.cuh:27-50
            if (!LTS_HAS_LOBE(LM, LOBE_OREN_NAYAR)) return spec(0.0f);
            const real so = sint(wo), si_ = sint(wi);
            real maxcos = 0.0f;
            if (si_ >= 0.0001f && so >= 0.0001f) {
                const real spo = sinphi(wo), cpo = cosphi(wo), spi = sinphi(wi), cpi = cosphi(wi);
                const real dcos = cpi * cpo + spi * spo;
                maxcos = xmax(0.0f, dcos);
            }
            real sin_a, tan_b;
            if (xabs(wi.z) > xabs(wo.z)) {
                sin_a = so;
                tan_b = si_ / xabs(wi.z);
            } else {
                sin_a = si_;
                tan_b = so / xabs(wo.z);
            }
            return f.R * LTS_INV_PI_F * (f.a + f.b * maxcos * sin_a * tan_b);
        }
        case LOBE_MICROFACET: {  // Microfacet.cuh:200-209
            if (!LTS_HAS_LOBE(LM, LOBE_MICROFACET)) return spec(0.0f);
            const real co = xabs(wo.z), ci = xabs(wi.z);
            V3 wh = wi + wo;
            if (ci == 0 || co == 0) return spec(0.0f);
            if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return spec(0.0f);
            wh = normalize(wh);
            const Spec F = fresnel_conductor(xabs(dot(wi, wh)), f.eta3, f.k);
            return f.R * tr_d(wh, f.alpha, f.alpha) * tr_g(wo, wi, f.alpha, f.alpha) * F / (4 * ci * co);
        }
        default: return spec(0.0f);  // specular lobes
    }
}
// BxDF::Pdf
template <int LM = LM_ALL>
__device__ real lobe_pdf(const Bsdf& f, V3 wo, V3 wi, EvSink* sig) {
    switch (f.lobe) {
        case LOBE_LAMBERT:
        case LOBE_OREN_NAYAR:
            if (!(LM & LM_MATTE)) return 0.0f;
            return same_hemi(wo, wi, sig) ? mul_dc(xabs(wi.z), LTS_1_PI) : 0.0f;
        case LOBE_MICROFACET: {
            if (!LTS_HAS_LOBE(LM, LOBE_MICROFACET)) return 0.0f;
            if (!same_hemi(wo, wi, sig)) return 0;
            const V3 wh = normalize(wo + wi);
            return tr_pdf(wo, wh, f.alpha, f.alpha) / (4 * dot(wo, wh));
        }
        default: return 0.0f;
    }
}
// BSDF::f (materials/BSDF.cuh:192-204)
template <int LM = LM_ALL>
__device__ Spec bsdf_f(const Bsdf& f, V3 woW, V3 wiW, uint32_t flags, EvSink* sig) {
    const bool reflect = dot(wiW, f.ng) * dot(woW, f.ng) > 0;
    if (sig) sig->put(0x600000000ull + (reflect ? 1u : 0u));
    if (f.lobe == LOBE_NONE || !matches(f.type, flags)) return spec(0.0f);
    const V3 wi = to_local(f, wiW), wo = to_local(f, woW);
    if ((reflect && (f.type & BSDF_REFLECTION)) || (!reflect && (f.type & BSDF_TRANSMISSION)))
        return spec(0.0f) + lobe_f<LM>(f, wo, wi);
    return spec(0.0f);
}
// BSDF::Pdf (BSDF.cuh:261-276)
template <int LM = LM_ALL>
__device__ real bsdf_pdf(const Bsdf& f, V3 woW, V3 wiW, uint32_t flags, EvSink* sig) {
    if (f.lobe == LOBE_NONE) return 0.0f;
    const V3 wo = to_local(f, woW), wi = to_local(f, wiW);
    if (wo.z == 0) return 0.0f;
    if (!matches(f.type, flags)) return 0.0f;
    const real pdf = 0.0f + lobe_pdf<LM>(f, wo, wi, sig);
    return pdf / 1;
}
// BSDF::sampleF with a single matching lobe (BSDF.cuh:206-259) and the lobes' sampleF.
template <int LM = LM_ALL>
__device__ Spec bsdf_sample(const Bsdf& f, V3 woW, V3& wiW, F2 u, real& pdf, uint32_t flags, uint32_t& sampled,
                            EvSink* sig) {
    if (f.lobe == LOBE_NONE || !matches(f.type, flags)) {
        pdf = 0;
        return spec(0.0f);
    }
    // comp = min((int)xfloor(u.x * 1), 0) = 0; the remapped sample is u itself
    const V3 wo = to_local(f, woW);
    V3 wi = v3(0, 0, 0);
    pdf = 0;
    sampled = f.type;
    Spec val = spec(0.0f);
    switch (f.lobe) {
        case LOBE_LAMBERT:
        case LOBE_OREN_NAYAR: {  // BxDF::sampleF (BxDF.cuh:196-204)
            if (!(LM & LM_MATTE)) break;
            const real r = xsqrt(u.x);
            const real th = mul_dc(u.y, LTS_2PI);
            const real dx = r * xcos(th), dy = r * xsin(th);
            wi = v3(dx, dy, xsqrt(xmax(0.0f, 1 - dx * dx - dy * dy)));
            if (wo.z < 0) wi.z *= -1;
            pdf = lobe_pdf<LM>(f, wo, wi, sig);
            val = lobe_f<LM>(f, wo, wi);
            break;
        }
        case LOBE_SPECULAR_REFL: {  // Specular.cuh:30-39, FresnelNoOp
            if (!LTS_HAS_LOBE(LM, LOBE_SPECULAR_REFL)) break;
            wi = v3(-wo.x, -wo.y, wo.z);
            pdf = 1.0f;
            val = (spec(1.0f) * f.R) / xabs(wi.z);
            break;
        }
        case LOBE_FRESNEL_SPECULAR: {  // Specular.cuh:107-135
            if (!LTS_HAS_LOBE(LM, LOBE_FRESNEL_SPECULAR)) break;
            const real F = fresnel_dielectric(wo.z, 1.0f, f.eta);
            if (u.x < F) {
                wi = v3(-wo.x, -wo.y, -wo.z);  // the reference's "reflection" keeps going straight
                sampled = BSDF_SPECULAR | BSDF_REFLECTION;
                pdf = F;
                val = (f.R * F) / xabs(wi.z);
            } else {
                const bool entering = wo.z > 0;
                const real ei = entering ? 1.0f : f.eta, et = entering ? f.eta : 1.0f;
                const V3 n = face_towards(v3(0, 0, 1), wo);
                if (!refract(wo, n, ei / et, wi)) {
                    pdf = 0;
                    return spec(0.0f);
                }
                Spec ft = f.T * (1 - F);
                ft = ft * ((ei * ei) / (et * et));
                sampled = BSDF_SPECULAR | BSDF_TRANSMISSION;
                pdf = 1.0f - F;
                val = ft / xabs(wi.z);
            }
            break;
        }
        case LOBE_MICROFACET: {  // Microfacet.cuh:211-222
            if (!LTS_HAS_LOBE(LM, LOBE_MICROFACET)) break;
            if (wo.z == 0) return spec(0.0f);
            const V3 wh = tr_sample_wh(wo, f.alpha, f.alpha, u.x, u.y);
            if (dot(wo, wh) < 0) return spec(0.0f);
            wi = -wo + wh * (2 * dot(wo, wh));
            if (!same_hemi(wo, wi, sig)) return spec(0.0f);
            pdf = tr_pdf(wo, wh, f.alpha, f.alpha) / (4 * dot(wo, wh));
            val = lobe_f<LM>(f, wo, wi);
            break;
        }
    }
    if (pdf == 0) return spec(0.0f);
    wiW = to_world(f, wi);
    return val;
}

// Material::computeScatteringFunctions (materials/Material.cuh:31-130) into a Bsdf record.
// Returns false when the primitive has no material (the reference's skipped 'M' entries).
template <int LM = LM_ALL, bool TEX = true>
__device__ bool make_bsdf(const SceneView& sv, const SI& si, Bsdf& f, EvSink* sig) {
    const int mesh = si.mesh;
    const DevMat& m = sv.mats[mesh];
    if (m.kind == 0) return false;
    f.ns = si.sn;
    f.ng = si.n;
    f.ss = normalize(si.sdpdu);
    f.ts = cross_si(f.ns, f.ss);
    f.lobe = LOBE_NONE;
    f.type = 0;
    f.eta = 1;
    switch (m.kind) {
        case 1: {  // Matte
            if (!(LM & LM_MATTE)) break;
            const Spec kd = eval_texture<TEX>(sv, m.tex[0], si, sig);
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
            if (!(LM & LM_GLASS)) break;
            f.eta = m.extra;
            const Spec r = eval_texture<TEX>(sv, m.tex[0], si, sig), t = eval_texture<TEX>(sv, m.tex[1], si, sig);
            if (is_black(r) && is_black(t)) break;
            f.R = r;
            f.T = t;
            f.lobe = LOBE_FRESNEL_SPECULAR;
            f.type = BSDF_REFLECTION | BSDF_TRANSMISSION | BSDF_SPECULAR;
            break;
        }
        case 3: {  // Mirror
            if (!(LM & LM_MIRROR)) break;
            const Spec r = eval_texture<TEX>(sv, m.tex[0], si, sig);
            if (is_black(r)) break;
            f.R = r;
            f.lobe = LOBE_SPECULAR_REFL;
            f.type = BSDF_REFLECTION | BSDF_SPECULAR;
            break;
        }
        case 4: {  // Metal (alpha given directly)
            if (!(LM & LM_METAL)) break;
            f.k = eval_texture<TEX>(sv, m.tex[0], si, sig);
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
    real pdf;
    V3 p1, perr1, n1;  // visibility target interaction
};
__device__ __forceinline__ real sph_pdf_infinite(V3 w) {
    // uniformSampleHemispherePDF() / (2 * M_PI * M_PI * xsin(sphericalTheta(w)))
    const real s = xsin(xacos(clampf(w.z, -1.0f, 1.0f)));
    return 0.159154937f / (19.7392088f * s);
}

// Triangle::Pdf(it, wi) (shapes/Triangle.cu:211-225): re-intersects the light triangle.
__device__ real area_pdf(const SceneView& sv, const DevLight& L, V3 p, V3 perr, V3 n, V3 wi) {
    const V3 o = offset_origin(p, perr, n, wi);
    V3 p0, p1, p2;
    prim_tri(sv, L.prim, p0, p1, p2);
    real t, u, v, inv;
    if (sv.watertight) {
        if (!tri_test_wt(p0, p1, p2, make_trace_ray(o, wi), INFINITY, t, u, v)) return 0;
        inv = mt_inv_det(p0, p1, p2, wi);
    } else if (!tri_test(p0, p1, p2, o, wi, INFINITY, t, u, v, inv)) {
        return 0;
    }
    SI is;
    make_si(sv, L.prim, wi, u, v, inv, is);
    const V3 dpt = p - is.p;
    return len2(dpt) / (absdot(is.n, -wi) * L.area);
}

__device__ bool sample_li(const SceneView& sv, const DevLight& L, const SI& si, F2 u, LightSample& ls) {
    ls.Li = spec(0.0f);
    ls.pdf = 0;
    ls.perr1 = v3(0, 0, 0);
    ls.n1 = v3(0, 0, 0);
    if (L.kind == 0) {  // AreaLight::sampleLi (Light.cu:28-37) + Triangle::sample (Triangle.cu:232-259)
        const real su = xsqrt(u.x);
        const real b0 = 1 - su, b1 = u.y * su;
        V3 p0, p1, p2;
        prim_tri(sv, L.prim, p0, p1, p2);
        const real b2 = 1 - b0 - b1;
        const V3 ps = p0 * b0 + p1 * b1 + p2 * b2;
        V3 ns;
        if (prim_word(sv, L.prim).x) {
            const float4* rec = sv.prim_rec + 8 * (size_t)L.prim;
            const float4 n0 = __ldg(rec + 3), n1 = __ldg(rec + 4), n2 = __ldg(rec + 5);
            ns = normalize(v3(n0.x, n0.y, n0.z) * b0 + v3(n1.x, n1.y, n1.z) * b1 + v3(n2.x, n2.y, n2.z) * b2);
        } else
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
        const real z = u.x;
        const real r = xsqrt(xmax(0.0f, 1.0f - z * z));
        const real phi = mul_dc(u.y, LTS_2PI);
        const V3 w0 = v3(r * xcos(phi), r * xsin(phi), z);
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

}  // namespace
}  // namespace lts
