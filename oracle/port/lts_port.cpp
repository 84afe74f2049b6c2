/*
 * Test infrastructure only (oracle).  CPU restatement of the reference's hot path --
 * tierChampion/LightTransportSimulation's Karras LBVH build and PathTracingIntegrator -- in plain
 * scalar C++, compiled with g++ -O2 -fopenmp -ffp-contract=off so that every float and double
 * expression rounds as the reference's own host build does.  It is pinned to the reference
 * (oracle/_ref/lts_ref, tests/golden/*) and used where the reference build cannot go: on the GPU
 * box, as the parity oracle at arbitrary sizes and as the timed CPU baseline.
 *
 * Scene input comes from the renderer's host loader (lighttransportsimulation_gb300/csrc/
 * host_scene.cpp), itself pinned bit-exactly to the reference's parseScene.
 *
 * CLI (same dump format as oracle/ref/ref_unity.cpp):
 *   lts_port bvh    ROOT SCENE SUBJECT OUT W H [MODE]
 *   lts_port render ROOT SCENE SUBJECT OUT W H SPP MAXB RR SEED X0 Y0 X1 Y1 THREADS FILM [MODE]
 *   lts_port kat    FN IN OUT   (single functions on raw records, layouts of include/lts_capi.h)
 * MODE 0 (default) is the reference's LBVH (leaf l holds primitive l, Morton codes only below the
 * reference's launch extent), MODE 1 the textbook LBVH (leaf l holds sorted primitive ids[l]).
 */
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/lts_capi.h"
#include "../../lighttransportsimulation_gb300/csrc/host_scene.hpp"
#include "lts_rng.h"

namespace port {

using lts::HostScene;

// <math.h>'s M_PI and M_1_PI are doubles on Linux (the reference's float fallbacks in
// core/GeneralHelper.cuh:8-14 are not taken).
static const double kPi = 3.14159265358979323846;
static const double k1Pi = 0.31830988618379067154;
static const float kShadowEps = 0.0001f;  // ErrorHelper.cuh:39-41

struct V {
    float x, y, z;
};
static inline V mk(float x, float y, float z) { return V{x, y, z}; }
static inline V operator+(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V operator-(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V operator-(V a) { return mk(-a.x, -a.y, -a.z); }
static inline V operator*(V a, float f) { return mk(f * a.x, f * a.y, f * a.z); }  // Vector3::operator*(U f)
static inline float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float absdot(V a, V b) { return fabsf(dot(a, b)); }
static inline float len2(V a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline V vabs(V a) { return mk(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
static inline float comp(V a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
static inline V face(V n, V v) { return dot(n, v) < 0.0f ? -n : n; }
// Geometry.cuh:76-83
static inline V cross(V a, V b) {
    const double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
    return mk((float)((ay * bz) - (az * by)), (float)((az * bx) - (ax * bz)), (float)((ax * by) - (ay * bx)));
}
static inline float rsq(float f) { return lts::quake_rsqrt(f); }
static inline V normalize(V v) { return v * rsq(len2(v)); }
static inline float clampf(float f, float lo, float hi) { return (f < lo) ? lo : ((f > hi) ? hi : f); }
static inline float mach_eps() { return 0.5f * 1.19209290e-07F; }
static inline float gammaf(int n) { return (n * mach_eps()) / (1 - n * mach_eps()); }

struct S {  // Spectrum
    float r, g, b;
};
static inline S sp(float v) { return S{v, v, v}; }
static inline S operator+(S a, S b) { return S{a.r + b.r, a.g + b.g, a.b + b.b}; }
static inline S operator-(S a, S b) { return S{a.r - b.r, a.g - b.g, a.b - b.b}; }
static inline S operator*(S a, S b) { return S{a.r * b.r, a.g * b.g, a.b * b.b}; }
static inline S operator*(S a, float v) { return S{a.r * v, a.g * v, a.b * v}; }
static inline S operator/(S a, float v) { return S{a.r / v, a.g / v, a.b / v}; }
static inline S operator/(S a, S b) { return S{a.r / b.r, a.g / b.g, a.b / b.b}; }
static inline bool black(S s) { return s.r == 0.0f && s.g == 0.0f && s.b == 0.0f; }
static inline float lum(S s) { return 0.212671f * s.r + 0.715160f * s.g + 0.072169f * s.b; }
static inline S ssqrt(S s) { return S{sqrtf(s.r), sqrtf(s.g), sqrtf(s.b)}; }

// ErrorHelper.cuh:55-75
static inline float next_up(float f) {
    if (std::isinf(f) && f > 0.0f) return f;
    if (f == -0.0f) f = 0.0f;
    uint32_t u;
    memcpy(&u, &f, 4);
    if (f >= 0) ++u;
    else --u;
    memcpy(&f, &u, 4);
    return f;
}
static inline float next_down(float f) {
    if (std::isinf(f) && f > 0.0f) return f;
    if (f == -0.0f) f = 0.0f;
    uint32_t u;
    memcpy(&u, &f, 4);
    if (f >= 0) --u;
    else ++u;
    memcpy(&f, &u, 4);
    return f;
}
// Geometry.cuh:782-797
static V offset_origin(V p, V perr, V n, V w) {
    const float d = dot(vabs(n), perr);
    V off = n * d;
    if (dot(w, n) < 0) off = -off;
    V po = p + off;
    float* c[3] = {&po.x, &po.y, &po.z};
    for (int i = 0; i < 3; ++i) {
        if (comp(off, i) > 0) *c[i] = next_up(*c[i]);
        else if (comp(off, i) < 0) *c[i] = next_down(*c[i]);
    }
    return po;
}
// Geometry.cuh:250-258
static void coord_system(V v1, V* v2, V* v3) {
    if (fabsf(v1.x) > fabsf(v1.y)) *v2 = mk(-v1.z, 0, v1.x) * rsq(v1.x * v1.x + v1.z * v1.z);
    else *v2 = mk(0, v1.z, -v1.y) * rsq(v1.y * v1.y + v1.z * v1.z);
    *v3 = cross(v1, *v2);
}

/* ---------------------------------------------------------------- sampler */
struct Rng {
    uint32_t key, sample, draw;
};
static inline float r1(Rng& r) { return lts_rng_uniform(r.key, r.sample, r.draw++); }
struct P2 {
    float x, y;
};
// Sampler::uniformSample as the reference's host build evaluates it (arguments right to left).
static inline P2 r2(Rng& r) {
    const float a = r1(r);
    const float b = r1(r);
    return P2{b, a};
}

/* ---------------------------------------------------------------- LBVH (BVH.cuh) */
struct Node {
    int key = -1, left = -1, right = -1;
    float b[6];
};
struct Bvh {
    int n = 0;
    std::vector<uint32_t> codes;  // sorted
    std::vector<int> ids;         // sorted
    std::vector<Node> nodes;      // 2n-1 flattened (interior 0..n-2, leaves n-1..2n-2)
    std::vector<int> leaf_prim;
};

static uint32_t shift3(uint32_t x) {  // BVH.cuh:101-109
    if (x == (1u << 10)) --x;
    x = (x | (x << 16)) & 0b00000011000000000000000011111111u;
    x = (x | (x << 8)) & 0b00000011000000001111000000001111u;
    x = (x | (x << 4)) & 0b00000011000011000011000011000011u;
    x = (x | (x << 2)) & 0b00001001001001001001001001001001u;
    return x;
}
static int clz32(uint32_t x) { return x == 0 ? 32 : __builtin_clz(x); }
static int delta(const std::vector<uint32_t>& c, int i1, int i2) {  // BVH.cuh:173-190
    const int n = (int)c.size();
    if (i1 < 0 || i1 >= n || i2 < 0 || i2 >= n) return -1;
    uint32_t x = c[i1] ^ c[i2];
    int tot = 0;
    if (x == 0) {
        tot += 40;
        x = (uint32_t)(i1 ^ i2);
    }
    return clz32(x) + tot;
}

static void tri_box(const std::vector<float>& soup, int p, float b[6]) {  // Triangle.cuh:48-53
    const float* t = &soup[9 * (size_t)p];
    for (int k = 0; k < 3; ++k) {
        b[k] = fminf(fminf(t[k], t[3 + k]), t[6 + k]);
        b[3 + k] = fmaxf(fmaxf(t[k], t[3 + k]), t[6 + k]);
    }
}

static Bvh build_bvh(const std::vector<float>& soup, int mode, int code_limit) {
    Bvh B;
    const int n = (int)(soup.size() / 9);
    B.n = n;
    std::vector<float> box(6 * (size_t)n);
    float gb[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < n; ++i) {  // BVHPrimitiveInfo::addPrimitive, BVH.cuh:92-97
        tri_box(soup, i, &box[6 * (size_t)i]);
        for (int k = 0; k < 3; ++k) {
            gb[k] = fminf(gb[k], box[6 * (size_t)i + k]);
            gb[3 + k] = fmaxf(gb[3 + k], box[6 * (size_t)i + 3 + k]);
        }
    }
    std::vector<uint32_t> codes(n, 0);
    std::vector<int> ids(n, 0);
    for (int i = 0; i < n; ++i) {  // convertInfoToMorton, BVH.cuh:134-137
        if (code_limit >= 0 && i >= code_limit) continue;
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            const float c = box[6 * (size_t)i + k] * 0.5f + box[6 * (size_t)i + 3 + k] * 0.5f;
            float o = c - gb[k];
            if (gb[3 + k] > gb[k]) o /= gb[3 + k] - gb[k];
            q[k] = (uint32_t)(1024 * o);
        }
        codes[i] = shift3(q[0]) | (shift3(q[1]) << 1) | (shift3(q[2]) << 2);
        ids[i] = i;
    }
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return codes[a] < codes[b]; });
    B.codes.resize(n);
    B.ids.resize(n);
    for (int i = 0; i < n; ++i) {
        B.codes[i] = codes[order[i]];
        B.ids[i] = ids[order[i]];
    }
    B.nodes.assign(2 * (size_t)n - 1, Node());
    B.leaf_prim.resize(n);
    for (int l = 0; l < n; ++l) {
        B.nodes[n - 1 + l].key = l;
        B.leaf_prim[l] = mode == 0 ? l : B.ids[l];
        memcpy(B.nodes[n - 1 + l].b, &box[6 * (size_t)B.leaf_prim[l]], 24);
    }
    std::vector<int> parent(2 * (size_t)n - 1, -1);
    for (int i = 0; i < n - 1; ++i) {  // treeBuilding, BVH.cuh:192-236
        int d = delta(B.codes, i, i + 1) - delta(B.codes, i, i - 1);
        d = d > 0 ? 1 : -1;
        const int dmin = delta(B.codes, i, i - d);
        long lmax = 128;
        while (delta(B.codes, i, (int)(i + lmax * d)) > dmin) lmax *= 4;
        long l = 0;
        for (long t = lmax / 2; t >= 1; t /= 2)
            if (delta(B.codes, i, (int)(i + (l + t) * d)) > dmin) l += t;
        const int j = (int)(i + l * d);
        const int dnode = delta(B.codes, i, j);
        int s = 0;
        for (int t = (int)ceilf(l / 2.0f); t >= 1; t = t == 1 ? 0 : (int)ceilf(t / 2.0f))
            if (delta(B.codes, i, i + (s + t) * d) > dnode) s += t;
        const int gamma = (int)(i + s * d + fminf(d, 0));
        const int lc = fminf(i, j) == gamma ? n - 1 + gamma : gamma;
        const int rc = fmaxf(i, j) == gamma + 1 ? n - 1 + gamma + 1 : gamma + 1;
        B.nodes[i].left = lc;
        B.nodes[i].right = rc;
        parent[lc] = i;
        parent[rc] = i;
    }
    // addBoundsToNode (BVH.cuh:238-262) climbs with a visited flag; the result is the union of
    // children in any order, so a post-order walk gives the same bits.
    if (n > 1) {
        std::vector<int> st;
        std::vector<char> done(2 * (size_t)n - 1, 0);
        st.push_back(0);
        while (!st.empty()) {
            const int v = st.back();
            Node& N = B.nodes[v];
            if (N.left < 0 || done[v]) {
                st.pop_back();
                continue;
            }
            const bool lready = B.nodes[N.left].left < 0 || done[N.left];
            const bool rready = B.nodes[N.right].left < 0 || done[N.right];
            if (lready && rready) {
                const float* a = B.nodes[N.left].b;
                const float* c = B.nodes[N.right].b;
                for (int k = 0; k < 3; ++k) {
                    N.b[k] = fminf(a[k], c[k]);
                    N.b[3 + k] = fmaxf(a[3 + k], c[3 + k]);
                }
                done[v] = 1;
                st.pop_back();
            } else {
                if (!rready) st.push_back(N.right);
                if (!lready) st.push_back(N.left);
            }
        }
    }
    return B;
}

/* ---------------------------------------------------------------- scene view */
struct Scene {
    const HostScene* h;
    std::vector<float> soup;  // 9 floats per triangle
    Bvh bvh;
    V p(int prim, int c) const {
        const float* t = &soup[9 * (size_t)prim + 3 * c];
        return mk(t[0], t[1], t[2]);
    }
    bool has_n(int prim) const { return h->tri_n[3 * (size_t)prim] >= 0; }
    V n(int prim, int c) const {
        const int i = h->tri_n[3 * (size_t)prim + c];
        return mk(h->n[3 * (size_t)i], h->n[3 * (size_t)i + 1], h->n[3 * (size_t)i + 2]);
    }
};

/* ---------------------------------------------------------------- triangles (Triangle.cu) */
struct SI {
    V p, perr, wo, n;
    V dpdu, dpdv, sn, sdpdu;
    V dpdx, dpdy;
    float tu = 0, tv = 0;  // uvHit (Triangle.cu:160)
    int prim = -1;
};

// Triangle::intersect (Triangle.cu:94-203); `ray_tmax` is the ray's tMax.
static bool tri_intersect(const Scene& sc, int prim, V o, V d, float ray_tmax, float* thit, SI* si) {
    const V p0 = sc.p(prim, 0), p1 = sc.p(prim, 1), p2 = sc.p(prim, 2);
    const V e1 = p1 - p0, e2 = p2 - p0;
    const V pv = cross(d, e2);
    const float det = dot(e1, pv);
    if (det == 0) return false;
    const float inv = 1.0 / det;
    const V tv = o - p0;
    const float u = inv * dot(tv, pv);
    if (u < kShadowEps || u > 1.0 - kShadowEps) return false;
    const V qv = cross(tv, e1);
    const float v = inv * dot(d, qv);
    if (v < kShadowEps || u + v > 1.0 - kShadowEps) return false;
    const float t = inv * dot(e2, qv);
    if (!(t > 0 && t < ray_tmax)) return false;
    const float w = 1 - u - v;
    float uv0x = 0, uv0y = 0, uv1x = 1, uv1y = 0, uv2x = 1, uv2y = 1;
    const int* ui = &sc.h->tri_uv[3 * (size_t)prim];
    if (ui[0] >= 0) {
        uv0x = sc.h->uv[2 * ui[0]]; uv0y = sc.h->uv[2 * ui[0] + 1];
        uv1x = sc.h->uv[2 * ui[1]]; uv1y = sc.h->uv[2 * ui[1] + 1];
        uv2x = sc.h->uv[2 * ui[2]]; uv2y = sc.h->uv[2 * ui[2] + 1];
    }
    const float d02x = uv0x - uv2x, d02y = uv0y - uv2y, d12x = uv1x - uv2x, d12y = uv1y - uv2y;
    const V dp02 = p0 - p2, dp12 = p1 - p2;
    const float determinant = d02x * d12y - d02y * d12x;
    V dpdu, dpdv;
    if (determinant == 0) {
        coord_system(normalize(cross(e2, e1)), &dpdu, &dpdv);
    } else {
        dpdu = (dp02 * d12y - dp12 * d02y) * inv;
        dpdv = (dp02 * -d12x + dp12 * d02x) * inv;
    }
    const float xs = fabsf(w * p0.x) + fabsf(u * p1.x) + fabsf(v * p2.x);
    const float ys = fabsf(w * p0.y) + fabsf(u * p1.y) + fabsf(v * p2.y);
    const float zs = fabsf(w * p0.z) + fabsf(u * p1.z) + fabsf(v * p2.z);
    si->perr = mk(xs, ys, zs) * gammaf(7);
    si->p = p0 * w + p1 * u + p2 * v;
    si->tu = uv0x * w + uv1x * u + uv2x * v;
    si->tv = uv0y * w + uv1y * u + uv2y * v;
    si->wo = -d;
    si->dpdu = dpdu;
    si->dpdv = dpdv;
    si->n = normalize(cross(dpdu, dpdv));
    si->sn = si->n;
    si->sdpdu = dpdu;
    si->prim = prim;
    if (sc.has_n(prim)) {
        const V ns = normalize(sc.n(prim, 0) * w + sc.n(prim, 1) * u + sc.n(prim, 2) * v);
        V ss = si->dpdu;
        V ts = cross(ns, ss);
        if (len2(ts) > 0.0f) {
            ts = normalize(ts);
            ss = cross(ts, ns);
        } else {
            coord_system(ns, &ss, &ts);
        }
        si->sn = normalize(cross(ss, ts));
        si->n = face(si->n, si->sn);
        si->sdpdu = ss;
        si->n = face(si->n, si->sn);
    }
    *thit = t;
    return true;
}

// Triangle::simpleIntersect (Triangle.cu:50-84)
static bool tri_shadow(const Scene& sc, int prim, V o, V d, float tmax) {
    const V p0 = sc.p(prim, 0), p1 = sc.p(prim, 1), p2 = sc.p(prim, 2);
    const V e1 = p1 - p0, e2 = p2 - p0;
    const V pv = cross(d, e1);
    const float det = dot(e2, pv);
    if (det == 0) return false;
    const float inv = 1.0 / det;
    const V tv = o - p0;
    const float u = inv * dot(tv, pv);
    if (u < kShadowEps || u > 1.0 + kShadowEps) return false;
    const V qv = cross(tv, e2);
    const float v = inv * dot(d, qv);
    if (v < kShadowEps || u + v > 1.0 + kShadowEps) return false;
    const float t = inv * dot(e1, qv);
    return t > 0 && t < tmax;
}

// Bounds3::simpleIntersect (Bound.cuh:199-227)
static bool slab(const float* b, V o, V inv, const int neg[3], float ray_tmax) {
    const float s = 1 + 2 * gammaf(3);
    float tMin = (b[3 * neg[0] + 0] - o.x) * inv.x;
    float tMax = (b[3 * (1 - neg[0]) + 0] - o.x) * inv.x;
    const float tyMin = (b[3 * neg[1] + 1] - o.y) * inv.y;
    float tyMax = (b[3 * (1 - neg[1]) + 1] - o.y) * inv.y;
    tMax *= s;
    tyMax *= s;
    if (tMin > tyMax || tyMin > tMax) return false;
    if (tyMin > tMin) tMin = tyMin;
    if (tyMax < tMax) tMax = tyMax;
    const float tzMin = (b[3 * neg[2] + 2] - o.z) * inv.z;
    float tzMax = (b[3 * (1 - neg[2]) + 2] - o.z) * inv.z;
    tzMax *= s;
    if (tMin > tzMax || tzMin > tMax) return false;
    if (tzMin > tMin) tMin = tzMin;
    if (tzMax < tMax) tMax = tzMax;
    return (tMin < ray_tmax) && (tMax > 0);
}

// BVH::intersect / simpleIntersect (BVH.cuh:331-398): left-first stack traversal.
static bool bvh_trace(const Scene& sc, V o, V d, float& tmax, SI* si, bool any) {
    const Bvh& B = sc.bvh;
    const V inv = mk(1 / d.x, 1 / d.y, 1 / d.z);
    const int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
    int stack[128];
    int sp = 0;
    int cur = 0;
    stack[sp++] = -1;
    bool hit = false;
    do {
        const Node& N = B.nodes[cur];
        if (slab(N.b, o, inv, neg, tmax)) {
            if (N.left < 0) {
                const int prim = B.leaf_prim[N.key];
                if (any) {
                    if (tri_shadow(sc, prim, o, d, tmax)) return true;
                } else {
                    float t;
                    SI tmp;
                    if (tri_intersect(sc, prim, o, d, tmax, &t, &tmp)) {
                        tmax = t;
                        *si = tmp;
                        hit = true;
                    }
                }
            } else {
                if (sp + 2 > 128) {
                    fprintf(stderr, "lts_port: traversal stack overflow\n");
                    abort();
                }
                stack[sp++] = N.right;
                stack[sp++] = N.left;
            }
        }
        cur = stack[--sp];
    } while (cur != -1);
    return hit;
}

/* ---------------------------------------------------------------- textures (Procedural.cuh) */
static const unsigned char kPerm[256] = {
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
static inline int perm(int i) { return kPerm[i & 255]; }
static float nweight(float t) {
    const float t3 = t * t * t, t4 = t3 * t;
    return 6 * t4 * t - 15 * t4 + 10 * t3;
}
static float lerpf(float t, float a, float b) { return (1 - t) * a + t * b; }
static float grad(int x, int y, int z, float dx, float dy, float dz) {
    int h = perm(perm(perm(x) + y) + z);
    h &= 15;
    const float u = h < 8 || h == 12 || h == 13 ? dx : dy;
    const float v = h < 4 || h == 12 || h == 13 ? dy : dz;
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}
static float perlin(float x, float y, float z) {
    int ix = (int)floorf(x), iy = (int)floorf(y), iz = (int)floorf(z);
    const float dx = x - ix, dy = y - iy, dz = z - iz;
    ix &= 255;
    iy &= 255;
    iz &= 255;
    const float w000 = grad(ix, iy, iz, dx, dy, dz), w100 = grad(ix + 1, iy, iz, dx - 1, dy, dz);
    const float w010 = grad(ix, iy + 1, iz, dx, dy - 1, dz), w001 = grad(ix, iy, iz + 1, dx, dy, dz - 1);
    const float w110 = grad(ix + 1, iy + 1, iz, dx - 1, dy - 1, dz), w011 = grad(ix, iy + 1, iz + 1, dx, dy - 1, dz - 1);
    const float w101 = grad(ix + 1, iy, iz + 1, dx - 1, dy, dz - 1);
    const float w111 = grad(ix + 1, iy + 1, iz + 1, dx - 1, dy - 1, dz - 1);
    const float wx = nweight(dx), wy = nweight(dy), wz = nweight(dz);
    const float x00 = lerpf(wx, w000, w100), x10 = lerpf(wx, w010, w110), x01 = lerpf(wx, w001, w101),
                x11 = lerpf(wx, w011, w111);
    return lerpf(wz, lerpf(wy, x00, x10), lerpf(wy, x01, x11));
}
static float smooth(float mn, float mx, float v) {
    const float t = clampf((v - mn) / (mx - mn), 0, 1);
    return t * t * (-2 * t + 3);
}
static void fnv(uint64_t& h, uint64_t v);
static float fbm(V p, V dx, V dy, float omega, int maxo, uint64_t* sig) {
    const float l2 = fmaxf(len2(dx), len2(dy));
    const float n = clampf(-1 - 0.5f * log2f(l2), 0, maxo);
    const int ni = (int)floorf(n);
    if (sig) fnv(*sig, 0x400000000ull + (unsigned)ni);
    float sum = 0, lam = 1, o = 1;
    for (int i = 0; i < ni; ++i) {
        sum += o * perlin(p.x * lam, p.y * lam, p.z * lam);
        lam *= 1.99f;
        o *= omega;
    }
    const float np = n - ni;
    sum += o * smooth(0.3f, 0.7f, np) * perlin(p.x * lam, p.y * lam, p.z * lam);
    return sum;
}
static float turbulence(V p, V dx, V dy, float omega, int maxo, uint64_t* sig) {
    const float l2 = fmaxf(len2(dx), len2(dy));
    const float n = clampf(-1 - 0.5f * log2f(l2), 0, maxo);
    const int ni = (int)floorf(n);
    if (sig) fnv(*sig, 0x400000000ull + (unsigned)ni);
    float sum = 0, lam = 1, o = 1;
    for (int i = 0; i < ni; ++i) {
        sum += o * fabsf(perlin(p.x * lam, p.y * lam, p.z * lam));
        lam *= 1.99f;
        o *= omega;
    }
    const float np = n - ni;
    sum += o * lerpf(smooth(0.3f, 0.7f, np), 0.2f, fabsf(perlin(p.x * lam, p.y * lam, p.z * lam)));
    for (int i = ni; i < maxo; ++i) {
        sum += o * 0.2f;
        o *= omega;
    }
    return sum;
}
static const float kMarble[10][3] = {{.58f, .58f, .6f}, {.58f, .58f, .6f}, {.58f, .58f, .6f}, {.5f, .5f, .5f},
                                     {.6f, .59f, .58f}, {.58f, .58f, .6f}, {.58f, .58f, .6f}, {.2f, .2f, .33f},
                                     {.58f, .58f, .6f}, {.58f, .58f, .6f}};
// Image textures in the fixed mode (texel / Mipmap::triangle / Mipmap::lookUp, Mipmap.cuh:14-73,
// with the repeat wrap taken into the level and the coarsest-level read fixed), over the loader's
// row-major pyramid.
static S img_texel(const lts::HostImage& im, int l, int s, int t) {
    const int w = im.w[l], h = im.h[l];
    if (im.wrap == 0) {
        s %= w;
        if (s < 0) s += w;
        t %= h;
        if (t < 0) t += h;
    } else if (im.wrap == 2) {
        s = s < 0 ? 0 : (s > w - 1 ? w - 1 : s);
        t = t < 0 ? 0 : (t > h - 1 ? h - 1 : t);
    } else if (s < 0 || s >= w || t < 0 || t >= h) {
        return S{0, 0, 0};
    }
    const float* q = &im.rgb[l][3 * ((size_t)t * w + s)];
    return S{q[0], q[1], q[2]};
}
static S img_bilerp(const lts::HostImage& im, int l, float st0, float st1) {
    l = l < 0 ? 0 : (l > im.levels - 1 ? im.levels - 1 : l);
    const float s = st0 * (float)im.w[l] - 0.5f, t = st1 * (float)im.h[l] - 0.5f;
    const int s0 = (int)floorf(s), t0 = (int)floorf(t);
    const float ds = s - (float)s0, dt = t - (float)t0;
    return img_texel(im, l, s0, t0) * ((1 - ds) * (1 - dt)) + img_texel(im, l, s0, t0 + 1) * ((1 - ds) * dt) +
           img_texel(im, l, s0 + 1, t0) * (ds * (1 - dt)) + img_texel(im, l, s0 + 1, t0 + 1) * (ds * dt);
}
static S img_lookup(const lts::HostImage& im, float st0, float st1) {
    if (im.lod < 0) return img_bilerp(im, 0, st0, st1);
    if (im.lod >= (float)(im.levels - 1)) return img_texel(im, im.levels - 1, 0, 0);
    const int il = (int)floorf(im.lod);
    const float delta = im.lod - (float)il;
    return img_bilerp(im, il, st0, st1) * (1 - delta) + img_bilerp(im, il + 1, st0, st1) * delta;
}

static S texture(const Scene& sc, const lts::HostTexture& t, const SI& si, uint64_t* sig) {
    switch (t.kind) {
        case lts::TEX_IMAGE: return img_lookup(sc.h->images[(size_t)t.v[0]], si.tu, si.tv);
        case lts::TEX_FBM: return sp(fbm(si.p, si.dpdx, si.dpdy, t.v[1], (int)t.v[0], sig));
        case lts::TEX_WRINKLED: return sp(turbulence(si.p, si.dpdx, si.dpdy, t.v[1], (int)t.v[0], sig));
        case lts::TEX_MARBLE: {
            const float scale = t.v[2], var = t.v[3];
            const V p = si.p * scale;
            const float marble = p.y + var * fbm(p, si.dpdx * scale, si.dpdy * scale, t.v[1], (int)t.v[0], sig);
            float tt = 0.5f + 0.5f * sinf(marble);
            const int first = (int)floorf(tt * (float)6);
            if (sig) fnv(*sig, 0x500000000ull + (unsigned)first);
            tt = (tt * (float)6 - first);
            S c[4];
            for (int k = 0; k < 4; ++k) c[k] = S{kMarble[first + k][0], kMarble[first + k][1], kMarble[first + k][2]};
            S s0 = c[0] * (1.0f - tt) + c[1] * tt, s1 = c[1] * (1.0f - tt) + c[2] * tt;
            const S s2 = c[2] * (1.0f - tt) + c[3] * tt;
            s0 = s0 * (1.0f - tt) + s1 * tt;
            s1 = s1 * (1.0f - tt) + s2 * tt;
            return (s0 * (1.0f - tt) + s1 * tt) * 1.5f;
        }
        case lts::TEX_WINDY: {
            const float wind = fbm(si.p * 0.1f, si.dpdx * 0.1f, si.dpdy * 0.1f, 0.5f, 3, sig);
            const float wave = fbm(si.p, si.dpdx, si.dpdy, 0.5f, 6, sig);
            return sp(fabsf(wind) * wave);
        }
        default: return S{t.v[0], t.v[1], t.v[2]};
    }
}

/* ---------------------------------------------------------------- BxDFs */
enum : uint32_t { REFL = 1, TRANS = 2, DIFF = 4, GLOSSY = 8, SPEC = 16, ALL = 31 };
enum Lobe { NONE, LAMBERT, OREN, FSPEC, SREFL, MICRO };
struct Bsdf {
    Lobe lobe = NONE;
    uint32_t type = 0;
    V ns, ng, ss, ts;
    S R{0, 0, 0}, T{0, 0, 0}, k{0, 0, 0}, eta3{0, 0, 0};
    float eta = 1, A = 0, B = 0, alpha = 0;
};
static inline float sin2t(V w) { return fmaxf(1 - w.z * w.z, 0.0f); }
static inline float sint(V w) { return sqrtf(sin2t(w)); }
static inline float cosphi(V w) { return clampf(w.x / sint(w), -1, 1); }  // BxDF.cuh:144-147
static inline float sinphi(V w) { return clampf(w.y / sint(w), -1, 1); }
static inline bool same(V a, V b) { return a.z * b.z > 0; }

static float fr_dielectric(float ci, float ei, float et) {  // BxDF.cuh:16-37
    ci = clampf(ci, 1, -1);
    const bool entering = ci > 0.0f;
    if (!entering) {
        std::swap(ei, et);
        ci = fabsf(ci);
    }
    const float si = sqrtf(fmaxf(0.0f, 1 - ci * ci));
    const float st = ei / et * si;
    if (st >= 1) return 1;
    const float ct = sqrtf(fmaxf(0.0f, 1 - st * st));
    const float rpar = ((et * ci) - (ei * ct)) / ((et * ci) + (ei * ct));
    const float rperp = ((ei * ci) - (et * ct)) / ((ei * ci) + (et * ct));
    return (rpar * rpar + rperp * rperp) / 2;
}
static S fr_conductor(float ci, S eta_i, S eta_t, S k) {  // BxDF.cuh:44-67
    ci = clampf(ci, -1, 1);
    const S eta = eta_t / eta_i, etak = k / eta_i;
    const float c2 = ci * ci, s2 = 1.0f - c2;
    const S eta2 = eta * eta, etak2 = etak * etak;
    const S t0 = eta2 - etak2 - sp(s2);
    const S a2b2 = ssqrt(t0 * t0 + eta2 * 4 * etak2);
    const S t1 = a2b2 + sp(c2);
    const S a = ssqrt((a2b2 + t0) * 0.5f);
    const S t2 = a * (2.0f * ci);
    const S rs = (t1 - t2) / (t1 + t2);
    const S t3 = a2b2 * c2 + sp(s2 * s2);
    const S t4 = t2 * s2;
    const S rp = rs * (t3 - t4) / (t3 + t4);
    return (rp + rs) * 0.5f;
}
static bool refract(V wi, V n, float eta, V* wt) {
    const float ci = dot(n, wi);
    const float s2i = fmaxf(0.0f, 1.0f - ci * ci);
    const float s2t = eta * eta * s2i;
    if (s2t >= 1) return false;
    const float ct = sqrtf(1 - s2t);
    *wt = -wi * eta + n * (eta * ci - ct);
    return true;
}
// Trowbridge-Reitz (Microfacet.cuh:53-181)
static float tr_lambda(V w, float ax, float ay) {
    const float at = fabsf(sint(w) / w.z);
    if (std::isinf(at)) return 0.0f;
    const float alpha = sqrtf(cosphi(w) * cosphi(w) * ax * ax + sinphi(w) * sinphi(w) * ay * ay);
    const float a2t2 = (alpha * at) * (alpha * at);
    return (-1 + sqrtf(1.0f + a2t2)) / 2;
}
static float tr_d(V wh, float ax, float ay) {
    const float t2 = sin2t(wh) / (wh.z * wh.z);
    if (std::isinf(t2)) return 0;
    const float c4 = (wh.z * wh.z) * (wh.z * wh.z);
    const float e = (cosphi(wh) * cosphi(wh) / (ax * ax) + sinphi(wh) * sinphi(wh) / (ay * ay)) * t2;
    return 1 / (kPi * ax * ay * c4 * (1 + e) * (1 + e));
}
static float tr_g1(V w, float a) { return 1 / (1 + tr_lambda(w, a, a)); }
static float tr_g(V wo, V wi, float a) { return 1 / (1 + tr_lambda(wo, a, a) + tr_lambda(wi, a, a)); }
static void tr_sample11(float cosT, float U1, float U2, float* sx, float* sy) {
    if (cosT > .9999) {
        const float r = sqrtf(U1 / (1 - U1));
        const float phi = 6.28318530718 * U2;
        *sx = r * cos(phi);
        *sy = r * sin(phi);
        return;
    }
    const float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
    const float tanT = sinT / cosT;
    const float a = 1 / tanT;
    const float G1 = 2 / (1 + sqrtf(1.f + 1.f / (a * a)));
    const float A = 2 * U1 / G1 - 1;
    float tmp = 1.f / (A * A - 1.f);
    if (tmp > 1e10) tmp = 1e10;
    const float B = tanT;
    const float D = sqrtf(fmaxf(float(B * B * tmp * tmp - (A * A - B * B) * tmp), 0.0f));
    const float s1 = B * tmp - D, s2 = B * tmp + D;
    *sx = (A < 0 || s2 > 1.f / tanT) ? s1 : s2;
    float S_;
    if (U2 > 0.5f) {
        S_ = 1.f;
        U2 = 2.f * (U2 - .5f);
    } else {
        S_ = -1.f;
        U2 = 2.f * (.5f - U2);
    }
    const float z = (U2 * (U2 * (U2 * 0.27385f - 0.73369f) + 0.46341f)) /
                    (U2 * (U2 * (U2 * 0.093073f + 0.309420f) - 1.000000f) + 0.597999f);
    *sy = S_ * z * sqrtf(1.f + *sx * *sx);
}
static V tr_sample(V wi, float ax, float ay, float U1, float U2) {
    const V ws = normalize(mk(ax * wi.x, ay * wi.y, wi.z));
    float sx, sy;
    tr_sample11(ws.z, U1, U2, &sx, &sy);
    const float tmp = cosphi(ws) * sx - sinphi(ws) * sy;
    sy = sinphi(ws) * sx + cosphi(ws) * sy;
    sx = tmp;
    sx = ax * sx;
    sy = ay * sy;
    return normalize(mk(-sx, -sy, 1.));
}

static V to_local(const Bsdf& f, V v) { return mk(dot(v, f.ss), dot(v, f.ts), dot(v, f.ns)); }
static V to_world(const Bsdf& f, V v) {
    return mk(f.ss.x * v.x + f.ts.x * v.y + f.ns.x * v.z, f.ss.y * v.x + f.ts.y * v.y + f.ns.y * v.z,
              f.ss.z * v.x + f.ts.z * v.y + f.ns.z * v.z);
}
static bool match(uint32_t type, uint32_t flags) { return (type & flags) == type; }
static inline bool same_h(V a, V b, uint64_t* sig) {  // sameHemisphere, recorded
    const bool v = same(a, b);
    if (sig) fnv(*sig, 0x700000000ull + (v ? 1u : 0u));
    return v;
}
static float default_pdf(V wo, V wi, uint64_t* sig) { return same_h(wo, wi, sig) ? fabsf(wi.z) * k1Pi : 0; }  // BxDF.cuh:192-194

static S lobe_f(const Bsdf& f, V wo, V wi) {
    switch (f.lobe) {
        case LAMBERT: return f.R * (float)k1Pi;
        case OREN: {
            const float so = sint(wo), si_ = sint(wi);
            float maxcos = 0.0f;
            if (si_ > 1e-4 && so > 1e-4) {
                const float spo = sinphi(wo), cpo = cosphi(wo), spi = sinphi(wi), cpi = cosphi(wi);
                maxcos = fmaxf(0.0f, cpi * cpo + spi * spo);
            }
            float sa, tb;
            if (fabsf(wi.z) > fabsf(wo.z)) {
                sa = so;
                tb = si_ / fabsf(wi.z);
            } else {
                sa = si_;
                tb = so / fabsf(wo.z);
            }
            return f.R * (float)k1Pi * (f.A + f.B * maxcos * sa * tb);
        }
        case MICRO: {
            const float co = fabsf(wo.z), ci = fabsf(wi.z);
            V wh = wi + wo;
            if (ci == 0 || co == 0) return sp(0.0f);
            if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return sp(0.0f);
            wh = normalize(wh);
            const S F = fr_conductor(fabsf(dot(wi, wh)), sp(1.0f), f.eta3, f.k);
            return f.R * tr_d(wh, f.alpha, f.alpha) * tr_g(wo, wi, f.alpha) * F / (4 * ci * co);
        }
        default: return sp(0.0f);
    }
}
static float lobe_pdf(const Bsdf& f, V wo, V wi, uint64_t* sig) {
    switch (f.lobe) {
        case LAMBERT:
        case OREN: return default_pdf(wo, wi, sig);
        case MICRO: {
            if (!same_h(wo, wi, sig)) return 0;
            const V wh = normalize(wo + wi);
            return tr_d(wh, f.alpha, f.alpha) * tr_g1(wo, f.alpha) * absdot(wo, wh) / fabsf(wo.z) / (4 * dot(wo, wh));
        }
        default: return 0.0f;
    }
}
static S bsdf_f(const Bsdf& f, V woW, V wiW, uint32_t flags, uint64_t* sig) {  // BSDF.cuh:192-204
    S r = sp(0.0f);
    const V wi = to_local(f, wiW), wo = to_local(f, woW);
    const bool reflect = dot(wiW, f.ng) * dot(woW, f.ng) > 0;
    if (sig) fnv(*sig, 0x600000000ull + (reflect ? 1u : 0u));
    if (f.lobe == NONE) return r;
    if (match(f.type, flags) && ((reflect && (f.type & REFL)) || (!reflect && (f.type & TRANS)))) r = r + lobe_f(f, wo, wi);
    return r;
}
static float bsdf_pdf(const Bsdf& f, V woW, V wiW, uint32_t flags, uint64_t* sig) {  // BSDF.cuh:261-276
    if (f.lobe == NONE) return 0.0f;
    const V wo = to_local(f, woW), wi = to_local(f, wiW);
    if (wo.z == 0) return 0.0f;
    float pdf = 0.0f;
    int m = 0;
    if (match(f.type, flags)) {
        ++m;
        pdf = pdf + lobe_pdf(f, wo, wi, sig);
    }
    return m > 0 ? pdf / m : 0.0f;
}
static S bsdf_sample(const Bsdf& f, V woW, V* wiW, P2 u, float* pdf, uint32_t flags, uint32_t* stype,
                     uint64_t* sig) {
    if (f.lobe == NONE || !match(f.type, flags)) {  // matchingComps == 0
        *pdf = 0;
        return sp(0.0f);
    }
    const int comp = (int)fminf((int)floorf(u.x * 1), 1 - 1);
    const P2 rem{u.x * 1 - comp, u.y};
    const V wo = to_local(f, woW);
    V wi = mk(0, 0, 0);
    *pdf = 0;
    *stype = f.type;
    S val = sp(0.0f);
    switch (f.lobe) {
        case LAMBERT:
        case OREN: {  // BxDF::sampleF + cosineSampleHemisphere (Sampling.cuh:53-77)
            const float r = sqrtf(rem.x);
            const float th = 2 * kPi * rem.y;
            const float dx = r * cosf(th), dy = r * sinf(th);
            wi = mk(dx, dy, sqrtf(fmaxf(0.0f, 1 - dx * dx - dy * dy)));
            if (wo.z < 0) wi.z *= -1;
            *pdf = default_pdf(wo, wi, sig);
            val = lobe_f(f, wo, wi);
            break;
        }
        case SREFL: {  // Specular.cuh:30-39
            wi = mk(-wo.x, -wo.y, wo.z);
            *pdf = 1.0f;
            val = sp(1.0f) * f.R / fabsf(wi.z);
            break;
        }
        case FSPEC: {  // Specular.cuh:107-135
            const float F = fr_dielectric(wo.z, 1.0f, f.eta);
            if (rem.x < F) {
                wi = mk(-wo.x, -wo.y, -wo.z);
                *stype = SPEC | REFL;
                *pdf = F;
                val = f.R * F / fabsf(wi.z);
            } else {
                const bool entering = wo.z > 0;
                const float ei = entering ? 1.0f : f.eta, et = entering ? f.eta : 1.0f;
                if (!refract(wo, face(mk(0, 0, 1), wo), ei / et, &wi)) return sp(0.0f);
                S ft = f.T * (1 - F);
                ft = ft * ((ei * ei) / (et * et));
                *stype = SPEC | TRANS;
                *pdf = 1.0f - F;
                val = ft / fabsf(wi.z);
            }
            break;
        }
        case MICRO: {  // Microfacet.cuh:211-222
            if (wo.z == 0) return sp(0.0f);
            const bool flip = wo.z < 0;
            V wh = tr_sample(flip ? -wo : wo, f.alpha, f.alpha, rem.x, rem.y);
            if (flip) wh = -wh;
            if (dot(wo, wh) < 0) return sp(0.0f);
            wi = -wo + wh * (2 * dot(wo, wh));
            if (!same_h(wo, wi, sig)) return sp(0.0f);
            *pdf = tr_d(wh, f.alpha, f.alpha) * tr_g1(wo, f.alpha) * absdot(wo, wh) / fabsf(wo.z) / (4 * dot(wo, wh));
            val = lobe_f(f, wo, wi);
            break;
        }
        default: break;
    }
    if (*pdf == 0) return sp(0.0f);
    *wiW = to_world(f, wi);
    return val;
}

static bool make_bsdf(const Scene& sc, const SI& si, Bsdf* f, uint64_t* sig) {  // Material.cuh:31-130
    const int mesh = sc.h->tri_mesh[si.prim];
    const lts::HostMaterial& m = sc.h->materials[mesh];
    if (m.kind == lts::MAT_NONE) return false;
    f->ns = si.sn;
    f->ng = si.n;
    f->ss = normalize(si.sdpdu);
    f->ts = cross(f->ns, f->ss);
    switch (m.kind) {
        case lts::MAT_MATTE: {
            const S kd = texture(sc, m.tex[0], si, sig);
            if (!black(kd)) {
                f->R = kd;
                f->lobe = m.extra == 0 ? LAMBERT : OREN;
                f->A = m.on_a;
                f->B = m.on_b;
                f->type = REFL | DIFF;
            }
            break;
        }
        case lts::MAT_GLASS: {
            f->eta = m.extra;
            const S r = texture(sc, m.tex[0], si, sig), t = texture(sc, m.tex[1], si, sig);
            if (black(r) && black(t)) break;
            f->R = r;
            f->T = t;
            f->lobe = FSPEC;
            f->type = REFL | TRANS | SPEC;
            break;
        }
        case lts::MAT_MIRROR: {
            const S r = texture(sc, m.tex[0], si, sig);
            if (black(r)) break;
            f->R = r;
            f->lobe = SREFL;
            f->type = REFL | SPEC;
            break;
        }
        case lts::MAT_METAL: {
            f->k = texture(sc, m.tex[0], si, sig);
            f->eta3 = S{m.tex[1].v[0], m.tex[1].v[1], m.tex[1].v[2]};
            f->R = sp(1.0f);
            f->alpha = m.extra;
            f->lobe = MICRO;
            f->type = REFL | GLOSSY;
            break;
        }
        default: break;
    }
    return true;
}

/* ---------------------------------------------------------------- lights (Light.cu) */
static float area_pdf(const Scene& sc, const lts::HostLight& L, const SI& it, V wi) {  // Triangle.cu:211-225
    const V o = offset_origin(it.p, it.perr, it.n, wi);
    float t;
    SI is;
    if (!tri_intersect(sc, L.prim, o, wi, INFINITY, &t, &is)) return 0;
    return len2(it.p - is.p) / (absdot(is.n, -wi) * L.area);
}
static float inf_pdf(V w) {  // Light.cuh:159-164
    const float sinTheta = sinf(acosf(clampf(w.z, -1.0f, 1.0f)));
    const float hemi = 0.5f * k1Pi;
    return hemi / (2 * kPi * kPi * sinTheta);
}
struct LSample {
    S Li;
    V wi, p1, perr1, n1;
    float pdf;
    bool delta;
};
static void sample_li(const Scene& sc, const lts::HostLight& L, const SI& it, P2 u, LSample* s) {
    s->perr1 = mk(0, 0, 0);
    s->n1 = mk(0, 0, 0);
    s->delta = false;
    if (L.kind == lts::LIGHT_AREA) {
        const float t = sqrtf(u.x);
        const float b0 = 1 - t, b1 = u.y * t;
        const V p0 = sc.p(L.prim, 0), p1 = sc.p(L.prim, 1), p2 = sc.p(L.prim, 2);
        const V ps = p0 * b0 + p1 * b1 + p2 * (1 - b0 - b1);
        V n;
        if (sc.has_n(L.prim))
            n = normalize(sc.n(L.prim, 0) * b0 + sc.n(L.prim, 1) * b1 + sc.n(L.prim, 2) * (1 - b0 - b1));
        else
            n = normalize(cross(p1 - p0, p2 - p0));
        const V pa = vabs(p0 * b0) + vabs(p1 * b1) + vabs(p2 * (1 - b0 - b1));
        s->perr1 = pa * gammaf(6);
        s->p1 = ps;
        s->n1 = n;
        s->wi = normalize(ps - it.p);
        s->pdf = area_pdf(sc, L, it, s->wi);
        s->Li = dot(n, -s->wi) > 0.f ? S{L.L[0], L.L[1], L.L[2]} : sp(0.0f);
    } else if (L.kind == lts::LIGHT_INFINITE) {
        const float z = u.x;
        const float r = sqrtf(fmaxf(0, 1.0f - z * z));
        const float phi = 2 * kPi * u.y;
        const V w0 = mk(r * cosf(phi), r * sinf(phi), z);
        const V ref = mk(0, 1, 0);
        V v1, v2;
        coord_system(ref, &v1, &v2);
        const V w = v1 * w0.x + v2 * w0.y + ref * w0.z;
        const V pl = mk(L.p[0], L.p[1], L.p[2]) + w * L.radius;
        s->wi = normalize(pl - it.p);
        s->pdf = inf_pdf(s->wi);
        s->p1 = pl;
        s->Li = S{L.L[0], L.L[1], L.L[2]};
    } else {
        const V pl = mk(L.p[0], L.p[1], L.p[2]);
        s->wi = normalize(pl - it.p);
        s->pdf = 1.0f;
        s->p1 = pl;
        s->Li = S{L.L[0], L.L[1], L.L[2]} / len2(pl - it.p);
        s->delta = true;
    }
}

/* ---------------------------------------------------------------- integrator */
struct Params {
    int W, H, spp, maxb, rr;
    uint32_t seed;
};
struct Film {
    std::vector<float> rgb, w;
};
static void fnv(uint64_t& h, uint64_t v) {
    for (int i = 0; i < 8; ++i) {
        h ^= (v >> (8 * i)) & 0xffu;
        h *= 0x100000001b3ull;
    }
}

// Parity debugging: the intermediate values of one crop sample (LTS_PORT_TRACE=k), as 16-float
// records with the renderer's tags (1 hit, 2 material, 3 light sample, 4 MIS, 5 BSDF sample, 6 L).
static long g_trace_k = -1;
static std::vector<float> g_trace;
struct Tr {
    bool on = false;
    void put(float tag, std::initializer_list<float> v) {
        if (!on || g_trace.size() >= 64 * 16) return;
        float r[16] = {0};
        r[0] = tag;
        int i = 1;
        for (float x : v)
            if (i < 16) r[i++] = x;
        g_trace.insert(g_trace.end(), r, r + 16);
    }
};

// PathTracingIntegrator::evaluate (PathTracingIntegrator.cuh:26-109) for one pixel.
static void evaluate(const Scene& sc, const Params& pr, int i, int j, float* outL, uint64_t* outsig, Film* film,
                     long crop_index) {
    const HostScene& h = *sc.h;
    const float* cm = h.cam;
    const V o = mk(cm[0], cm[1], cm[2]), right = mk(cm[3], cm[4], cm[5]), up = mk(cm[6], cm[7], cm[8]),
            llc = mk(cm[9], cm[10], cm[11]);
    const int id = j * pr.W + i;
    Rng rng{lts_rng_key(pr.seed, (uint32_t)id), 0, 0};
    const int nl = (int)h.lights.size();
    for (int s = 0; s < pr.spp; ++s) {
        rng.sample = (uint32_t)s;
        rng.draw = 0;
        uint64_t sig = 0xcbf29ce484222325ull;
        Tr tr;
        tr.on = g_trace_k >= 0 && crop_index * pr.spp + s == g_trace_k;
        const P2 fs = r2(rng);
        (void)r2(rng);  // lens sample (aperture 0)
        const float pfx = (float)(i + fs.x), pfy = (float)(j + fs.y);
        const float rx = (float)(pr.W - 1), ry = (float)(pr.H - 1);
        V ro = o;
        V rd = normalize(llc + right * (pfx / rx) + up * (pfy / ry) - o);
        const V dx0 = normalize(llc + right * ((pfx + 1) / rx) + up * (pfy / ry) - o);
        const V dy0 = normalize(llc + right * (pfx / rx) + up * ((pfy + 1) / ry) - o);
        const float sc_spp = rsq((float)pr.spp);
        const V rxd = rd + (dx0 - rd) * sc_spp, ryd = rd + (dy0 - rd) * sc_spp;
        bool diff = true;
        S L = sp(0.0f), beta = sp(1.0f);
        bool specular = false;
        for (int bounce = 0; bounce < pr.maxb; ++bounce) {
            SI si;
            float tmax = INFINITY;
            const bool hit = bvh_trace(sc, ro, rd, tmax, &si, false);
            fnv(sig, 0x100000000ull + (uint64_t)((hit ? si.prim : -1) + 1));
            tr.put(1, {(float)hit, (float)(hit ? si.prim : -1), si.p.x, si.p.y, si.p.z, si.n.x, si.n.y, si.n.z, si.sn.x,
                       si.sn.y, si.sn.z, beta.r, beta.g, beta.b, L.r});
            if (bounce == 0 || specular) {
                if (hit) {
                    const int li = h.prim_light[si.prim];
                    const S le = (li >= 0 && dot(si.n, -rd) > 0.f) ? S{h.lights[li].L[0], h.lights[li].L[1], h.lights[li].L[2]}
                                                                   : sp(0.0f);
                    L = L + beta * le;
                } else {
                    for (int l = 0; l < nl; ++l) {
                        const lts::HostLight& Lt = h.lights[l];
                        L = L + beta * (Lt.kind == lts::LIGHT_INFINITE ? S{Lt.L[0], Lt.L[1], Lt.L[2]} : sp(0.0f));
                    }
                }
            }
            if (!hit) break;
            if (diff) {  // Interaction.cuh:118-160
                const float d = -dot(si.n, si.p);
                const float tx = (-dot(si.n, ro) - d) / dot(si.n, rxd);
                const float ty = (-dot(si.n, ro) - d) / dot(si.n, ryd);
                si.dpdx = (ro + rxd * tx) - si.p;
                si.dpdy = (ro + ryd * ty) - si.p;
            } else {
                si.dpdx = si.dpdy = mk(0, 0, 0);
            }
            Bsdf f;
            if (!make_bsdf(sc, si, &f, &sig)) break;
            tr.put(2, {(float)f.lobe, f.R.r, f.R.g, f.R.b, f.ss.x, f.ss.y, f.ss.z, f.ts.x, f.ts.y, f.ts.z, si.dpdx.x,
                       si.dpdx.y, si.dpdx.z});
            if (nl > 0) {  // uniformSampleOneLight + estimateDirect (IntegratorHelper.cuh:51-149)
                const float ul = r1(rng);
                int off = 0;
                if (nl != 1) {
                    int first = 0, len = nl;
                    while (len > 0) {
                        const int half = len >> 1, middle = first + half;
                        if (h.light_cdf[middle] <= ul) {
                            first = middle + 1;
                            len -= half + 1;
                        } else {
                            len = half;
                        }
                    }
                    off = (int)clampf(first - 1, 0, nl - 2);
                }
                const float lpdf = h.light_func[off] / (h.light_func_int * nl);
                const P2 ulight = r2(rng);
                const P2 uscat = r2(rng);
                const lts::HostLight& Lt = h.lights[off];
                const uint32_t flags = specular ? ALL : (ALL & ~SPEC);
                S Ld = sp(0.0f);
                LSample ls;
                sample_li(sc, Lt, si, ulight, &ls);
                if (ls.pdf > 0 && !black(ls.Li)) {
                    const S fv = bsdf_f(f, si.wo, ls.wi, flags, &sig) * absdot(ls.wi, si.sn);
                    const float spdf = bsdf_pdf(f, si.wo, ls.wi, flags, &sig);
                    if (!black(fv)) {
                        const V org = offset_origin(si.p, si.perr, si.n, ls.p1 - si.p);
                        const V tgt = offset_origin(ls.p1, ls.perr1, ls.n1, org - ls.p1);
                        float tm = 1 - kShadowEps;
                        const bool occ = bvh_trace(sc, org, tgt - org, tm, nullptr, true);
                        fnv(sig, 0x300000000ull + (occ ? 0u : 1u));
                        tr.put(3, {(float)off, lpdf, ls.pdf, ls.Li.r, ls.wi.x, ls.wi.y, ls.wi.z, fv.r, fv.g, fv.b, spdf,
                                   (float)occ});
                        S Li = ls.Li;
                        if (occ) Li = sp(0.0f);
                        if (!black(Li)) {
                            if (ls.delta) {
                                Ld = Ld + fv * Li / ls.pdf;
                            } else {
                                const float fp = 1 * ls.pdf, gp = 1 * spdf;
                                const float w = (fp * fp) / (fp * fp + gp * gp);
                                Ld = Ld + fv * Li * w / ls.pdf;
                            }
                        }
                    }
                }
                if (!ls.delta) {
                    V wi = ls.wi;
                    float spdf = 0;
                    uint32_t st = 0;
                    S fv = bsdf_sample(f, si.wo, &wi, uscat, &spdf, flags, &st, &sig);
                    fv = fv * absdot(wi, si.sn);
                    const bool sspec = (st & SPEC) != 0;
                    if (!black(fv) && spdf > 0) {
                        float w = 1;
                        bool done = false;
                        if (!sspec) {
                            float lp = 0;
                            if (Lt.kind == lts::LIGHT_AREA) lp = area_pdf(sc, Lt, si, wi);
                            else if (Lt.kind == lts::LIGHT_INFINITE) lp = inf_pdf(wi);
                            if (lp == 0) done = true;
                            else {
                                const float fp = 1 * spdf, gp = 1 * lp;
                                w = (fp * fp) / (fp * fp + gp * gp);
                            }
                        }
                        if (!done) {
                            SI lit;
                            const V org = offset_origin(si.p, si.perr, si.n, wi);
                            float tm = INFINITY;
                            const bool found = bvh_trace(sc, org, wi, tm, &lit, false);
                            fnv(sig, 0x200000000ull + (uint64_t)((found ? lit.prim : -1) + 1));
                            S Li = sp(0.0f);
                            if (found) {
                                if (h.prim_light[lit.prim] == off && Lt.kind == lts::LIGHT_AREA)
                                    Li = dot(lit.n, -wi) > 0.f ? S{Lt.L[0], Lt.L[1], Lt.L[2]} : sp(0.0f);
                            } else {
                                Li = Lt.kind == lts::LIGHT_INFINITE ? S{Lt.L[0], Lt.L[1], Lt.L[2]} : sp(0.0f);
                            }
                            if (!black(Li)) Ld = Ld + fv * Li * sp(1.0f) * w / spdf;
                            tr.put(4, {spdf, fv.r, fv.g, fv.b, w, (float)found, Li.r, Ld.r, Ld.g, Ld.b, wi.x, wi.y, wi.z});
                        }
                    }
                }
                L = L + beta * (Ld / lpdf);
            }
            V wi = mk(0, 0, 0);
            float pdf = 0;
            uint32_t st = 0;
            const P2 ub = r2(rng);
            const S fv = bsdf_sample(f, si.wo, &wi, ub, &pdf, ALL, &st, &sig);
            if (black(fv) || pdf == 0) break;
            specular = (st & SPEC) != 0;
            beta = beta * (fv * absdot(wi, si.sn) / pdf);
            tr.put(5, {wi.x, wi.y, wi.z, pdf, fv.r, fv.g, fv.b, beta.r, beta.g, beta.b, L.r, L.g, L.b});
            ro = offset_origin(si.p, si.perr, si.n, wi);
            rd = wi;
            diff = false;
            if (bounce >= pr.rr) {
                const float q = fmaxf(0.05f, 1 - lum(beta));
                if (r1(rng) < q) break;
                beta = beta / (1 - q);
            }
        }
        tr.put(6, {L.r, L.g, L.b});
        outL[3 * s + 0] = L.r;
        outL[3 * s + 1] = L.g;
        outL[3 * s + 2] = L.b;
        outsig[s] = sig;
        if (film) {  // Camera::addSample (Camera.cu:192-218), single-threaded use only
            const int px0 = std::max((int)ceilf(pfx - 1.0f), 0), py0 = std::max((int)ceilf(pfy - 1.0f), 0);
            const int px1 = std::min((int)floorf(pfx + 1.0f) + 1, pr.W), py1 = std::min((int)floorf(pfy + 1.0f) + 1, pr.H);
            for (int y = py0; y < py1; ++y)
                for (int x = px0; x < px1; ++x) {
                    const float dx = fabsf((x - pfx - 0.5f) * 1.0f * 16), dy = fabsf((y - pfy - 0.5f) * 1.0f * 16);
                    const int ix = (int)fminf((int)floorf(dx), 15), iy = (int)fminf((int)floorf(dy), 15);
                    const float wgt = h.filter[iy * 16 + ix];
                    const size_t px = (size_t)y * pr.W + x;
                    film->rgb[3 * px + 0] += L.r * wgt;
                    film->rgb[3 * px + 1] += L.g * wgt;
                    film->rgb[3 * px + 2] += L.b * wgt;
                    film->w[px] += wgt;
                }
        }
    }
}

/* ---------------------------------------------------------------- LTSD writer + CLI */
struct Writer {
    FILE* f;
    explicit Writer(const char* p) : f(fopen(p, "wb")) {
        if (!f) {
            fprintf(stderr, "cannot open %s\n", p);
            exit(3);
        }
        fwrite("LTSD", 1, 4, f);
    }
    void put(const char* name, char dt, const void* d, uint64_t n, size_t el) {
        const uint32_t nl = (uint32_t)strlen(name);
        fwrite(&nl, 4, 1, f);
        fwrite(name, 1, nl, f);
        fwrite(&dt, 1, 1, f);
        fwrite(&n, 8, 1, f);
        if (n) fwrite(d, el, n, f);
    }
    ~Writer() { fclose(f); }
};

static int load(const char* root, const char* scene, const char* subject, int w, int h, HostScene* hs) {
    int code = 0;
    std::string msg = lts::load_scene(root, scene, strcmp(subject, "-") ? subject : "", w, h, hs, &code);
    if (code) fprintf(stderr, "lts_port: %s\n", msg.c_str());
    return code;
}

static Scene make_scene(const HostScene* hs, int mode) {
    Scene sc;
    sc.h = hs;
    hs->triangle_soup(sc.soup);
    const int limit = mode == 0 ? ((hs->max_mesh_triangles() + 15) / 16) * 16 : -1;
    sc.bvh = build_bvh(sc.soup, mode, limit);
    return sc;
}

static void dump_bvh(Writer& wr, const Bvh& B) {
    const int nodes = 2 * B.n - 1;
    std::vector<int32_t> key(nodes), l(nodes), r(nodes);
    std::vector<float> b((size_t)nodes * 6);
    for (int i = 0; i < nodes; ++i) {
        key[i] = B.nodes[i].key;
        l[i] = B.nodes[i].left;
        r[i] = B.nodes[i].right;
        memcpy(&b[6 * (size_t)i], B.nodes[i].b, 24);
    }
    wr.put("sorted_codes", 'u', B.codes.data(), B.n, 4);
    wr.put("sorted_ids", 'i', B.ids.data(), B.n, 4);
    wr.put("node_key", 'i', key.data(), nodes, 4);
    wr.put("node_left", 'i', l.data(), nodes, 4);
    wr.put("node_right", 'i', r.data(), nodes, 4);
    wr.put("node_bounds", 'f', b.data(), b.size(), 4);
}

/* ---------------------------------------------------------------- known-answer vectors
 * kat FN IN OUT: the port's own function FN (LTS_KAT_* record layouts of include/lts_capi.h) on
 * n records of 16 raw float32 inputs, 16 floats out per record.  The distribution's G1, G and
 * Pdf are the port's isotropic forms: their records carry alphaX == alphaY. */
static int kat(int fn, const char* in_path, const char* out_path) {
    FILE* f = fopen(in_path, "rb");
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
        const V v0 = mk(a[0], a[1], a[2]), v3 = mk(a[3], a[4], a[5]);
        Bsdf b;
        b.lobe = MICRO;
        b.type = REFL | GLOSSY;
        b.ns = b.ng = mk(0, 0, 1);
        b.ss = mk(1, 0, 0);
        b.ts = mk(0, 1, 0);
        switch (fn) {
            case LTS_KAT_QUAKE_RSQRT: o[0] = rsq(a[0]); break;
            case LTS_KAT_FRESNEL_DIELECTRIC: o[0] = fr_dielectric(a[0], a[1], a[2]); break;
            case LTS_KAT_FRESNEL_CONDUCTOR: {
                const S F = fr_conductor(a[0], sp(1.0f), S{a[1], a[2], a[3]}, S{a[4], a[5], a[6]});
                o[0] = F.r, o[1] = F.g, o[2] = F.b;
                break;
            }
            case LTS_KAT_TR_D: o[0] = tr_d(v0, a[3], a[4]); break;
            case LTS_KAT_TR_LAMBDA: o[0] = tr_lambda(v0, a[3], a[4]); break;
            case LTS_KAT_TR_G1: o[0] = tr_g1(v0, a[3]); break;
            case LTS_KAT_TR_G: o[0] = tr_g(v0, v3, a[6]); break;
            case LTS_KAT_TR_SAMPLE11: tr_sample11(a[0], a[1], a[2], &o[0], &o[1]); break;
            case LTS_KAT_TR_SAMPLE_WH: {
                const bool flip = v0.z < 0;
                V wh = tr_sample(flip ? -v0 : v0, a[3], a[4], a[5], a[6]);
                if (flip) wh = -wh;
                o[0] = wh.x, o[1] = wh.y, o[2] = wh.z;
                break;
            }
            case LTS_KAT_TR_PDF: o[0] = tr_d(v3, a[6], a[6]) * tr_g1(v0, a[6]) * absdot(v0, v3) / fabsf(v0.z); break;
            case LTS_KAT_MF_F: {
                b.alpha = a[6];
                b.R = S{a[7], a[8], a[9]};
                b.eta3 = S{a[10], a[11], a[12]};
                b.k = S{a[13], a[14], a[15]};
                const S v = lobe_f(b, v0, v3);
                o[0] = v.r, o[1] = v.g, o[2] = v.b;
                break;
            }
            case LTS_KAT_MF_PDF:
                b.alpha = a[6];
                o[0] = lobe_pdf(b, v0, v3, nullptr);
                break;
            case LTS_KAT_MF_SAMPLE: {
                b.alpha = a[3];
                b.R = S{a[6], a[7], a[8]};
                b.eta3 = S{a[9], a[10], a[11]};
                b.k = S{a[12], a[13], a[14]};
                V wi = mk(0, 0, 0);
                float pdf = 0;
                uint32_t st = 0;
                const S v = bsdf_sample(b, v0, &wi, P2{a[4], a[5]}, &pdf, ALL, &st, nullptr);
                o[0] = wi.x, o[1] = wi.y, o[2] = wi.z, o[3] = v.r, o[4] = v.g, o[5] = v.b, o[6] = pdf;
                break;
            }
            case LTS_KAT_PERLIN: o[0] = perlin(a[0], a[1], a[2]); break;
            case LTS_KAT_FBM: o[0] = fbm(v0, v3, mk(a[6], a[7], a[8]), a[9], (int)a[10], nullptr); break;
            case LTS_KAT_TURBULENCE: o[0] = turbulence(v0, v3, mk(a[6], a[7], a[8]), a[9], (int)a[10], nullptr); break;
            case LTS_KAT_OFFSET_ORIGIN: {
                const V po = offset_origin(v0, v3, mk(a[6], a[7], a[8]), mk(a[9], a[10], a[11]));
                o[0] = po.x, o[1] = po.y, o[2] = po.z;
                break;
            }
            default: return 2;
        }
    }
    FILE* g = fopen(out_path, "wb");
    if (!g) return 3;
    const bool ok = fwrite(out.data(), 4, out.size(), g) == out.size();
    fclose(g);
    return ok ? 0 : 3;
}

}  // namespace port

int main(int argc, char** argv) {
    using namespace port;
    if (argc < 2) return 2;
    const std::string cmd = argv[1];
    if (cmd == "bvh" && argc >= 8) {
        HostScene hs;
        if (load(argv[2], argv[3], argv[4], atoi(argv[6]), atoi(argv[7]), &hs)) return 1;
        const int mode = argc > 8 ? atoi(argv[8]) : 0;
        Scene sc = make_scene(&hs, mode);
        Writer wr(argv[5]);
        dump_bvh(wr, sc.bvh);
        return 0;
    }
    if (cmd == "kat" && argc >= 5) return kat(atoi(argv[2]), argv[3], argv[4]);
    if (cmd == "bvhsoup" && argc >= 5) {  // bvhsoup IN(float32 x 9N raw) OUT MODE [CODE_LIMIT]
        FILE* f = fopen(argv[2], "rb");
        if (!f) return 3;
        std::vector<float> soup;
        float buf[4096];
        size_t k;
        while ((k = fread(buf, 4, 4096, f)) > 0) soup.insert(soup.end(), buf, buf + k);
        fclose(f);
        const int mode = atoi(argv[4]);
        const int limit = argc > 5 ? atoi(argv[5]) : -1;
        Bvh B = build_bvh(soup, mode, limit);
        Writer wr(argv[3]);
        dump_bvh(wr, B);
        return 0;
    }
    if (cmd == "render" && argc >= 18) {
        Params pr{atoi(argv[6]), atoi(argv[7]), atoi(argv[8]), atoi(argv[9]), atoi(argv[10]),
                  (uint32_t)strtoul(argv[11], nullptr, 10)};
        const int x0 = atoi(argv[12]), y0 = atoi(argv[13]), x1 = atoi(argv[14]), y1 = atoi(argv[15]);
        const int threads = atoi(argv[16]), want_film = atoi(argv[17]);
        const int mode = argc > 18 ? atoi(argv[18]) : 0;
        HostScene hs;
        if (load(argv[2], argv[3], argv[4], pr.W, pr.H, &hs)) return 1;
        Scene sc = make_scene(&hs, mode);
        if (threads > 0) omp_set_num_threads(threads);
        if (const char* t = getenv("LTS_PORT_TRACE")) g_trace_k = atol(t);
        const int cw = x1 - x0, ch = y1 - y0;
        std::vector<float> L((size_t)cw * ch * pr.spp * 3);
        std::vector<uint64_t> sig((size_t)cw * ch * pr.spp);
        Film film;
        if (want_film) {
            film.rgb.assign((size_t)pr.W * pr.H * 3, 0.f);
            film.w.assign((size_t)pr.W * pr.H, 0.f);
        }
        const long np = (long)cw * ch;
        auto t0 = std::chrono::steady_clock::now();
        if (want_film) {  // the film accumulation is sequential, in pixel order
            for (long p = 0; p < np; ++p)
                evaluate(sc, pr, x0 + (int)(p % cw), y0 + (int)(p / cw), &L[3 * p * pr.spp], &sig[p * pr.spp], &film, p);
        } else {
#pragma omp parallel for schedule(dynamic, 16)
            for (long p = 0; p < np; ++p)
                evaluate(sc, pr, x0 + (int)(p % cw), y0 + (int)(p / cw), &L[3 * p * pr.spp], &sig[p * pr.spp], nullptr, p);
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        const int32_t nth = want_film ? 1 : omp_get_max_threads();
        Writer wr(argv[5]);
        wr.put("L", 'f', L.data(), L.size(), 4);
        wr.put("sig", 'q', sig.data(), sig.size(), 8);
        wr.put("time_s", 'd', &secs, 1, 8);
        wr.put("threads", 'i', &nth, 1, 4);
        if (g_trace_k >= 0) wr.put("trace", 'f', g_trace.data(), g_trace.size(), 4);
        if (want_film) {  // Camera::getRender (Camera.cu:256-289)
            std::vector<float> rgb((size_t)pr.W * pr.H * 3);
            for (int jj = 0; jj < pr.H; ++jj)
                for (int ii = 0; ii < pr.W; ++ii) {
                    const size_t src = (size_t)(pr.H - 1 - jj) * pr.W + ii, dst = (size_t)jj * pr.W + ii;
                    const float inv = 1 / film.w[src];
                    for (int c = 0; c < 3; ++c) rgb[3 * dst + c] = fmaxf(0.0f, film.rgb[3 * src + c] * inv);
                }
            wr.put("film", 'f', rgb.data(), rgb.size(), 4);
        }
        return 0;
    }
    fprintf(stderr, "usage: lts_port bvh|bvhsoup|render ...\n");
    return 2;
}
