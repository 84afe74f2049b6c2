// Wavefront path tracer (sm_103a): the same integrator as k_pathtrace, split into stage kernels
// over a pool of path states, so each stage runs with its own (small) register budget and all
// lanes of a warp execute the same stage.  One iteration of the host loop runs
//
//   generate  start new (pixel, sample) paths in free slots: film + lens draws, camera ray
//   trace     one persistent launch over three ray lists: this iteration's path rays (closest
//             hit), and the previous shade's NEE shadow rays (any hit) and MIS BSDF rays
//             (closest hit, light radiance where they land)
//   finalize  for the paths shaded in the previous iteration: their bounce's direct light in the
//             reference's order (Ld = light part + MIS part, L += beta * Ld / lightPdf) and the
//             deferred parity events; a finished path stores its sample (radiance, film
//             position) and frees its slot
//   shade     this iteration's hits: emission, SurfaceInteraction, material, light sample (NEE)
//             + MIS BSDF sample, path BSDF sample, throughput, Russian roulette
//   compact   one pass over the slots builds the next iteration's lists in slot order (path
//             rays, shadow rays, MIS rays, free slots), so every stage reads and writes the
//             structure-of-arrays path state in near-contiguous runs
//   gather    after a chunk of samples per pixel has finished: one thread per film pixel sums the
//             filter-weighted samples of its 3x3 source pixels in a fixed order (compensated FP32,
//             then added to the FP64 film), so the film has no atomics and is reproducible
//
// The sampler is keyed per (pixel, sample) with a draw counter kept in the path state, so a path
// produces exactly the draws of the megakernel (PathTracingIntegrator.cuh:41-99) in any order of
// execution.  Included by tracer.cu (one translation unit shares the constant tables).
#pragma once

namespace lts {
namespace {

enum : uint32_t { WF_VIS = 1u, WF_MIS = 2u, WF_NEE = 4u, WF_DONE = 8u, WF_CACHE = 16u };
// path flags (low byte; the bounce count sits above bit 8)
// FL_RECORDED: the path holds a training record; FL_OFFERED: its one chance of a record (at its
// first vertex after a rough one) has been taken, whether or not the coin accepted it.
enum : uint32_t { FL_SPECULAR = 1u, FL_ROUGH = 2u, FL_UNBIASED = 4u, FL_RECORDED = 8u, FL_OFFERED = 16u };
constexpr int kWfBlock = 128;
constexpr uint64_t kSigBasis = 0xcbf29ce484222325ull;

struct WfState {
    int32_t *pix, *smp, *wid;  // pixel (within its view's film), sample, the sample's batch index
                               // in row-major pixel order (where finalize stores it)
    int32_t* view;             // slice of the batch the path belongs to
    const WfView* views;       // the batch's slices (count in WfCtl::nviews)
    uint32_t *draw, *flags, *pend, *vis;
    float4 *ro, *rd, *beta, *L;
    float2* pf;
    uint64_t* sig;
    int32_t* hprim;
    float4* huvi;
    float4 *sh_o, *sh_d, *sh_c;
    float4 *mis_o, *mis_d, *mis_fv, *mis_x, *ld_mis;
    float4* nee_beta;
    uint64_t *ev_mis, *ev_main;
    int32_t* mis_hit;
    int32_t *q_a, *q_b, *q_shadow, *q_mis, *q_free;
    uint32_t* counts;  // written by compact: [0] next path rays, [2] shadow, [3] mis, [4] free;
                       // [8] trace fetch counter; [16 + c] paths of shade class c (classify)
    int32_t* q_cls;    // [kShadeClasses][pool] this iteration's paths grouped by shade class
    float4* fs_L;      // finished samples of the chunk: radiance rgb, film x (chunk index order)
    float* fs_y;       // film y
    // radiance cache (cache == 0: off, pointers unused)
    int cache;
    uint32_t unb_permille;  // share of paths traced in full (unbiased), per mille
    uint32_t tr_cap;        // training records per render
    // Records are a uniform random subset of the render's eligible vertices (every unbiased
    // path's first vertex after a rough one, count in counts[33]): a vertex is kept when a hash
    // of its path is <= tr_accept, a rate set from the previous render's eligible count so that
    // the records rarely reach tr_cap (first come, first served would keep only the vertices of
    // the earliest bounces and of the first shade classes).
    uint32_t tr_accept;
    const float* bounds;    // scene bounds: position features are normalised to the unit cube
    uint16_t* feat;         // [pool][96] features of the vertex a path queries
    float4* cache_L;        // [pool] the cache's radiance for that vertex
    int32_t* q_cache;       // this iteration's queries (count in counts[12])
    float4 *tr_beta, *tr_L0;  // an unbiased path's throughput and radiance at its recorded vertex
    int32_t* tr_idx;        // its training record
    uint16_t* tr_feat;      // [tr_cap][96] training features (count in counts[32])
    float* tr_target;       // [tr_cap][3] training targets
};

// Per-iteration bookkeeping on the device (so an iteration can run as a CUDA graph): k_wf_control
// turns the previous compaction's counts into this iteration's list sizes and new samples.
struct WfCtl {
    uint32_t take, n_cont, n_ext, n_fin, n_sh, n_mis, n_query, nfree, active, iters, nviews, pad;
    long long gen0, generated, ctot;
    unsigned long long queries;  // cache queries answered in the batch
};

// Radiance-cache features of a shading point (the layout oracle/mlp_np.py's encode states):
// 12-frequency sin/cos of the position in the unit cube of the scene bounds, the direction
// towards the previous vertex, the shading normal, roughness, diffuse and specular albedo, 1.
__device__ __forceinline__ float bsdf_roughness(const Bsdf& f) {
    return (f.lobe == LOBE_LAMBERT || f.lobe == LOBE_OREN_NAYAR) ? 1.0f : (f.lobe == LOBE_MICROFACET ? f.alpha : 0.0f);
}
// A vertex is rough for the radiance cache above this roughness: the cache is trained and queried
// at rough vertices only, whose outgoing radiance varies slowly with direction.
constexpr float kCacheRough = 0.3f;
__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}
// The 96 features as bf16, written four at a time (8-byte words) as they are computed, so no
// 96-entry array has to live in registers or local memory: sin of the 36 position angles at
// 0..35, their cos at 36..71, then the 14 scalars at 72..85, zeros to 95.
__device__ void write_features(const WfState& st, const SI& si, const Bsdf& f, uint16_t* out) {
    uint2* o = reinterpret_cast<uint2*>(out);
    const float pc[3] = {si.p.x, si.p.y, si.p.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float lo = __ldg(st.bounds + a), ext = __ldg(st.bounds + 3 + a) - lo;
        const float u = ext > 0.0f ? (pc[a] - lo) / ext : 0.5f;
        float fr = 3.14159265358979f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {  // frequencies 4c .. 4c + 3 of axis a
            float sn[4], cs[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                sincosf(u * fr, &sn[q], &cs[q]);
                fr *= 2.0f;
            }
            const int m = a * 12 + 4 * c;
            o[m / 4] = make_uint2(bf16x2(sn[0], sn[1]), bf16x2(sn[2], sn[3]));
            o[9 + m / 4] = make_uint2(bf16x2(cs[0], cs[1]), bf16x2(cs[2], cs[3]));
        }
    }
    const float rough = bsdf_roughness(f);
    const bool diffuse = f.lobe == LOBE_LAMBERT || f.lobe == LOBE_OREN_NAYAR;
    const Spec ks = f.lobe == LOBE_MICROFACET ? spec(1.0f) : f.R;
    const Spec kd = diffuse ? f.R : spec(0.0f), kss = diffuse ? spec(0.0f) : ks;
    o[18] = make_uint2(bf16x2(si.wo.x, si.wo.y), bf16x2(si.wo.z, si.sn.x));
    o[19] = make_uint2(bf16x2(si.sn.y, si.sn.z), bf16x2(rough, kd.r));
    o[20] = make_uint2(bf16x2(kd.g, kd.b), bf16x2(kss.r, kss.g));
    o[21] = make_uint2(bf16x2(kss.b, 1.0f), 0u);
    o[22] = make_uint2(0u, 0u);
    o[23] = make_uint2(0u, 0u);
}

// Resume a (pixel, sample) stream at draw `draw` (regenerates the current Philox block).
__device__ __forceinline__ void rng_resume(Rng& r) {
    const uint32_t k = r.draw & 3u;
    if (k == 0u) return;
    const uint32_t d = r.draw;
    r.draw = d & ~3u;
    philox_block(r);
    r.draw = d;
    for (uint32_t q = 0; q < k; ++q) {
        r.w0 = r.w1;
        r.w1 = r.w2;
        r.w2 = r.w3;
    }
}

__device__ __forceinline__ void camera_ray(const WfView& vw, float pfx, float pfy, V3& rd, V3& rxd, V3& ryd) {
    const float* cam = vw.cam;
    const float spp_scale = vw.spp_scale;
    const V3 co = v3(cam[0], cam[1], cam[2]), cright = v3(cam[3], cam[4], cam[5]), cup = v3(cam[6], cam[7], cam[8]),
             cllc = v3(cam[9], cam[10], cam[11]);
    const float rx = (float)(vw.W - 1), ry = (float)(vw.H - 1);
    rd = normalize(cllc + cright * (pfx / rx) + cup * (pfy / ry) - co);
    const V3 dx0 = normalize(cllc + cright * ((pfx + 1) / rx) + cup * (pfy / ry) - co);
    const V3 dy0 = normalize(cllc + cright * (pfx / rx) + cup * ((pfy + 1) / ry) - co);
    rxd = rd + (dx0 - rd) * spp_scale;
    ryd = rd + (dy0 - rd) * spp_scale;
}

// Order in which a slice's samples of one sample index visit the crop's pixels: 8 x 4 tiles
// (one warp each) left to right in bands of four rows, so the rays a warp traces start from a
// compact patch of the image instead of a 32 x 1 strip (partial tiles at the right and bottom
// edges are row-major).  Position k in 0 .. cw * ch - 1 -> crop pixel (ci, cj).
#ifndef LTS_PIXEL_TILES
#define LTS_PIXEL_TILES 1  // 0: row-major pixel order
#endif
constexpr int kTileW = 8, kTileH = 4;
__device__ __forceinline__ void tile_pixel(long k, int cw, int ch, int& ci, int& cj) {
    if (!LTS_PIXEL_TILES) {
        ci = (int)(k % cw);
        cj = (int)(k / cw);
        return;
    }
    const long band_px = (long)kTileH * cw;
    const int band = (int)(k / band_px);
    const int rows = min(kTileH, ch - band * kTileH);
    const int o = (int)(k - band * band_px);
    const int full = cw / kTileW, tile_px = kTileW * rows;
    if (o < full * tile_px) {
        const int tx = o / tile_px, r = o - tx * tile_px;
        ci = tx * kTileW + r % kTileW;
        cj = band * kTileH + r / kTileW;
    } else {  // the narrower last tile of the band
        const int rem = cw - full * kTileW, r = o - full * tile_px;
        ci = full * kTileW + r % rem;
        cj = band * kTileH + r / rem;
    }
}

// generate: starts batch samples gen0 .. gen0 + take - 1 in the first `take` free slots,
// appending them to the path-ray list after its `n_cont` continuing paths.
__global__ __launch_bounds__(kWfBlock) void k_wf_generate(const SceneView sv, const RenderParams rp, WfState st,
                                                          int32_t* q_ext, const WfCtl* __restrict__ ctl) {
    const long t = (long)blockIdx.x * kWfBlock + threadIdx.x;
    if (t >= (long)ctl->take) return;
    const long w = ctl->gen0 + t;
    const uint32_t n_cont = ctl->n_cont;
    const int nviews = (int)ctl->nviews;
    const int slot = st.q_free[t];
    int v = 0;
    while (v + 1 < nviews && st.views[v + 1].base <= w) ++v;
    const WfView& vw = st.views[v];
    const long local = w - vw.base;
    const int cw = vw.x1 - vw.x0;
    const int s = vw.s_first + (int)(local / vw.npix);
    const long pc = local % vw.npix;
    int ci, cj;
    tile_pixel(pc, cw, vw.y1 - vw.y0, ci, cj);
    const int i = vw.x0 + ci, j = vw.y0 + cj;
    const int id = j * vw.W + i;
    Rng rng;
    rng.key = vw.seed + wang_hash((uint32_t)id);
    rng.sample = (uint32_t)s;
    rng.draw = 0;
    const F2 fs = rng_2d(rng);
    (void)rng_2d(rng);
    const float pfx = (float)(i + fs.x), pfy = (float)(j + fs.y);
    V3 rd, rxd, ryd;
    camera_ray(vw, pfx, pfy, rd, rxd, ryd);
    st.view[slot] = v;
    st.pix[slot] = id;
    st.smp[slot] = s;
    st.wid[slot] = (int32_t)(w - pc + (long)cj * cw + ci);  // the sample's place in row-major order
    st.draw[slot] = rng.draw;
    st.flags[slot] =
        (st.cache && wang_hash((uint32_t)id ^ ((uint32_t)s * 0x9E3779B9u) ^ (vw.seed * 0x85EBCA6Bu)) % 1000u < st.unb_permille)
            ? FL_UNBIASED : 0u;
    st.pend[slot] = 0u;
    st.pf[slot] = make_float2(pfx, pfy);
    st.ro[slot] = make_float4(vw.cam[0], vw.cam[1], vw.cam[2], 0.f);
    st.rd[slot] = make_float4(rd.x, rd.y, rd.z, 0.f);
    st.beta[slot] = make_float4(1.f, 1.f, 1.f, 0.f);
    st.L[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
    st.sig[slot] = kSigBasis;
    q_ext[n_cont + t] = slot;
}

// Work counters (RenderParams::counters): [0..2] all rays (rays, node visits, triangle tests),
// then the same three per traversal kind (0 extend, 1 shadow, 2 MIS) at [3 + 3 * kind].
enum : int { TR_EXTEND = 0, TR_SHADOW = 1, TR_MIS = 2 };


// The ray of path slot p for each traversal kind.
__device__ __forceinline__ bool wf_ray_begin(int kind, Trav& t, const SceneView& sv, const WfState& st, int p,
                                             int nleaf, Work& wk, const bool inst = false) {
    if (kind == TR_EXTEND) {  // path ray, closest hit (BVH::intersect, BVH.cuh:365-398)
        const float4 o = st.ro[p], d = st.rd[p];
        return trav_begin(false, t, sv, nleaf, v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), INFINITY, wk, inst);
    } else if (kind == TR_SHADOW) {  // VisibilityTester::unoccluded (VisibilityTester.cu:9-12), any hit
        const float4 o = st.sh_o[p], d = st.sh_d[p];
        return trav_begin(true, t, sv, nleaf, v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), d.w, wk, inst);
    } else {  // MIS BSDF ray, closest hit
        const float4 o = st.mis_o[p], d = st.mis_d[p];
        return trav_begin(false, t, sv, nleaf, v3(o.x, o.y, o.z), v3(d.x, d.y, d.z), INFINITY, wk, inst);
    }
}
// Two-level BVH: the world ray of a ray in flight, re-read from the path state (the traversal
// holds the current instance's object-space ray) to enter the next instance.
__device__ __forceinline__ bool wf_ray_next_instance(int kind, Trav& t, const SceneView& sv, const WfState& st,
                                                     int p) {
    const float4 o = kind == TR_EXTEND ? st.ro[p] : (kind == TR_SHADOW ? st.sh_o[p] : st.mis_o[p]);
    const float4 d = kind == TR_EXTEND ? st.rd[p] : (kind == TR_SHADOW ? st.sh_d[p] : st.mis_d[p]);
    return inst_next(kind == TR_SHADOW, t, sv, v3(o.x, o.y, o.z), v3(d.x, d.y, d.z));
}

// Results of a finished traversal.  MIS: radiance of the sampled light where the BSDF ray lands
// (IntegratorHelper.cuh:225-243).
__device__ __forceinline__ void wf_ray_end(int kind, const Trav& t, const SceneView& sv, WfState& st, int p) {
    if (kind == TR_EXTEND) {
        st.hprim[p] = t.best;  // with its shade class (hit_prim / hit_class)
        st.huvi[p] = make_float4(t.bu, t.bv, t.binv, t.tmax);
    } else if (kind == TR_SHADOW) {
        st.vis[p] = t.best == 1 ? 0u : 1u;
    } else {
        // Landing on the sampled area light needs the surface at the hit (its normal faces the
        // ray?): that evaluation is left to finalize (ld_mis.w = 2, xyz = barycentrics and inv),
        // which has the registers for it; here only the light index of the hit is read.
        const float4 x = st.mis_x[p];
        const int off = __float_as_int(x.y);
        const DevLight& Lt = sv.lights[off];
        const int hp = hit_prim(t.best);
        const bool found = hp >= 0;
        if (found) {
            const bool on_light = prim_word(sv, hp).z == off && Lt.kind == 0;
            st.ld_mis[p] = on_light ? make_float4(t.bu, t.bv, t.binv, 2.f) : make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            const float4 fv = st.mis_fv[p];
            const Spec Li = Lt.kind == 1 ? Spec{Lt.L[0], Lt.L[1], Lt.L[2]} : spec(0.0f);
            Spec c = spec(0.0f);
            const bool add = !is_black(Li);
            if (add) c = Spec{fv.x, fv.y, fv.z} * Li * spec(1.0f) * fv.w / x.x;
            st.ld_mis[p] = make_float4(c.r, c.g, c.b, add ? 1.f : 0.f);
        }
        st.mis_hit[p] = found ? hp + 1 : 0;
    }
}

// Lanes left idle before a warp fetches new rays (while the lists last).
#ifndef LTS_REFILL_IDLE
#define LTS_REFILL_IDLE 12 // idle lanes of a warp that trigger fetching new rays
#endif
constexpr int kRefillIdle = LTS_REFILL_IDLE;
#ifndef LTS_LEAF_BIAS
#define LTS_LEAF_BIAS 1  // leaf steps when lanes with pending leaves x 4 >= lanes due a node x this
#endif
constexpr int kLeafBias = LTS_LEAF_BIAS;
// Resident blocks per SM the trace kernel is compiled for (caps its registers): 8 blocks = 32
// warps at 64 registers without spills; the kernel waits on node and triangle loads, and the
// extra warps hide them (stress scene: trace 420 ms per render at 8, 444 at 7, 484 at 6; 9 and
// 10 spill).
#ifndef LTS_TRACE_MIN_BLOCKS
#define LTS_TRACE_MIN_BLOCKS 8
#endif
constexpr int kTraceMinBlocks = LTS_TRACE_MIN_BLOCKS;

// Persistent traversal of the three ray lists as one index space [path rays | shadow rays | MIS
// rays]: each warp keeps up to 32 rays in flight; when at least kRefillIdle lanes have finished,
// the warp claims that many entries with one atomic and starts them, so lanes do not idle while
// the warp's longest ray finishes (dynamic ray fetch, Aila and Laine, HPG 2009), and the short
// shadow and MIS lists share the launch's tail with the path rays.  Launched with whole warps;
// `fetch` is zeroed before the launch.  WIDE: the 8-wide compressed BVH, else the binary LBVH.
template <bool WIDE, bool INST = false>
__global__ __launch_bounds__(kWfBlock, kTraceMinBlocks) void k_wf_trace(const SceneView sv, const RenderParams rp, WfState st,
                                                       const int32_t* __restrict__ q_ext,
                                                       const WfCtl* __restrict__ ctl, uint32_t* fetch, int nleaf) {
    __shared__ uint32_t s_stack[kStack * kWfBlock];
    // the block's finished rays, node visits and triangle tests per traversal kind (kept out of
    // the registers of the traversal loop)
    __shared__ uint32_t s_work[9];
    uint32_t* stack = s_stack + threadIdx.x;
    if (threadIdx.x < 9) s_work[threadIdx.x] = 0u;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    Trav t;
    int p = -1, kind = 0;
    bool active = false, exhausted = false;
    Work cur{0u, 0u};  // work of the ray in flight, credited to its kind when it finishes
    auto credit = [&]() {
        uint32_t* w = s_work + 3 * kind;
        atomicAdd(w, 1u);
        atomicAdd(w + 1, cur.nodes);
        atomicAdd(w + 2, cur.tris);
        cur.nodes = cur.tris = 0u;
    };
    for (;;) {
        const unsigned idle = __ballot_sync(~0u, !active);
        if (!exhausted && __popc(idle) >= kRefillIdle) {
            // the list sizes, read at each refill rather than held through the traversal
            const uint32_t e1 = __ldg(&ctl->n_ext), e2 = e1 + __ldg(&ctl->n_sh), n = e2 + __ldg(&ctl->n_mis);
            const int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(idle));
            base = __shfl_sync(~0u, base, leader);
            if (base + (uint32_t)__popc(idle) >= n) exhausted = true;
            if (!active) {
                const uint32_t idx = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (idx < n) {
                    kind = idx < e1 ? TR_EXTEND : (idx < e2 ? TR_SHADOW : TR_MIS);
                    p = kind == TR_EXTEND ? q_ext[idx] : (kind == TR_SHADOW ? st.q_shadow[idx - e1] : st.q_mis[idx - e2]);
                    active = wf_ray_begin(kind, t, sv, st, p, nleaf, cur, INST);
                    if (INST && !active && t.imask) active = wf_ray_next_instance(kind, t, sv, st, p);
                    if (!active) {
                        wf_ray_end(kind, t, sv, st, p);
                        credit();
                    }
                }
            }
        }
        if (__ballot_sync(~0u, active) == 0u) {
            if (exhausted) break;
            continue;
        }
        for (;;) {
            bool fin = false;
            if (WIDE) {
                // lanes with pending leaf triangles and lanes due a node visit: the warp runs
                // whichever step more of its lanes wait for
                const bool has_leaf = active && t.lbits != 0u;
                const bool want_node = active && !has_leaf;
                const unsigned lm = __ballot_sync(~0u, has_leaf), nm = __ballot_sync(~0u, want_node);
                const bool leaf_mode = lm != 0u && __popc(lm) * 4 >= __popc(nm) * kLeafBias;
                if (leaf_mode ? has_leaf : want_node) {
                    const bool any = kind == TR_SHADOW;
                    fin = leaf_mode ? wide_leaf_step(any, t, sv, rp.err, cur, INST)
                                    : wide_node_step(any, t, sv, stack, rp.err, cur, INST);
                    if (INST && fin && wf_ray_next_instance(kind, t, sv, st, p)) fin = false;
                }
            } else if (active) {
                fin = trav_step_binary(kind == TR_SHADOW, t, sv, stack, rp.err, cur);
            }
            if (fin) {
                wf_ray_end(kind, t, sv, st, p);
                credit();
                active = false;
            }
            const unsigned act = __ballot_sync(~0u, active);
            if (act == 0u || (!exhausted && 32 - __popc(act) >= kRefillIdle)) break;
        }
    }
    __syncthreads();
    if (threadIdx.x < 9 && rp.counters) {
        const uint32_t v = s_work[threadIdx.x];
        if (v) {
            atomicAdd(rp.counters + 3 + threadIdx.x, (unsigned long long)v);  // per kind
            atomicAdd(rp.counters + threadIdx.x % 3, (unsigned long long)v);  // all rays
        }
    }
}

// shade: one bounce of PathTracingIntegrator::evaluate up to the next ray.
// classify: groups this iteration's paths by the shade class of what they hit (0: left the
// scene), so that shade runs warps over one material kind at a time.
__global__ __launch_bounds__(kWfBlock) void k_wf_classify(const SceneView sv, WfState st, const int32_t* __restrict__ q,
                                                          const WfCtl* __restrict__ ctl, int pool) {
    const int t = blockIdx.x * kWfBlock + threadIdx.x;
    if (t >= (int)ctl->n_ext) return;
    const int p = q[t];
    const int c = hit_class(st.hprim[p]);  // 0: left the scene
    const unsigned grp = __match_any_sync(__activemask(), c);
    const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(st.counts + 16 + c, (uint32_t)__popc(grp));
    base = __shfl_sync(grp, base, leader);
    st.q_cls[(size_t)c * pool + base + __popc(grp & ((1u << lane) - 1u))] = p;
}

// Resident blocks per SM the shade kernel is compiled for (caps its registers).
#ifndef LTS_SHADE_MIN_BLOCKS
#define LTS_SHADE_MIN_BLOCKS 5  // 6 and 4 measured 2 % and 5 % slower on the stress scene
#endif
// One path's bounce; LM / TEX: the lobes and textures its material can have (shade_variant).
template <bool RECORD, int LM, bool TEX>
__device__ __forceinline__ void shade_one(const SceneView& sv, const RenderParams& rp, WfState& st, int p) {
    const uint32_t flags = st.flags[p];
    const int bounce = (int)(flags >> 8);
    bool specular = (flags & 1u) != 0;
    const float4 o4 = st.ro[p], d4 = st.rd[p];
    const V3 ro = v3(o4.x, o4.y, o4.z), rd = v3(d4.x, d4.y, d4.z);
    const float4 b4 = st.beta[p], l4 = st.L[p];
    Spec beta{b4.x, b4.y, b4.z}, L{l4.x, l4.y, l4.z};
    uint64_t sig = RECORD ? st.sig[p] : 0ull;
    EvSink evs{&sig, 0};
    const int prim = hit_prim(st.hprim[p]);
    const bool hit = prim >= 0;
    uint32_t pend = 0;
    if (RECORD) fnv_mix(sig, 0x100000000ull + (uint64_t)(prim + 1));
    SI si;
    if (hit) {
        const float4 h = st.huvi[p];
        make_si(sv, prim, rd, h.x, h.y, h.z, si, &ro);
    }
    if (bounce == 0 || specular) {
        if (hit) {
            const int li = si.light;
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
    Rng rng;
    const WfView& vw = st.views[st.view[p]];
    rng.key = vw.seed + wang_hash((uint32_t)st.pix[p]);
    rng.sample = (uint32_t)st.smp[p];
    rng.draw = st.draw[p];
    rng_resume(rng);
    bool done = !hit;
    Bsdf f;
    if (!done) {
        if (bounce == 0) {  // camera-ray differentials (Interaction.cuh:118-160)
            const float2 pf = st.pf[p];
            V3 rd0, rxd, ryd;
            camera_ray(vw, pf.x, pf.y, rd0, rxd, ryd);
            const V3 n = si.n;
            const float dd = -dot(n, si.p);
            const float tx = (-dot(n, ro) - dd) / dot(n, rxd);
            const float ty = (-dot(n, ro) - dd) / dot(n, ryd);
            si.dpdx = (ro + rxd * tx) - si.p;
            si.dpdy = (ro + ryd * ty) - si.p;
        } else {
            si.dpdx = v3(0, 0, 0);
            si.dpdy = v3(0, 0, 0);
        }
        if (!make_bsdf<LM, TEX>(sv, si, f, RECORD ? &evs : nullptr)) done = true;
    }
    bool recorded = (flags & FL_RECORDED) != 0, rough_seen = (flags & FL_ROUGH) != 0;
    bool offered = (flags & FL_OFFERED) != 0;
    if (st.cache && !done && rough_seen && bsdf_roughness(f) > kCacheRough) {
        // the first rough vertex after a rough one: cached paths end here with the cache's
        // radiance, unbiased paths are offered one training record here and go on.  Specular and
        // near-specular vertices in between are traced through (their outgoing radiance is
        // too directional for the network: a caustic seen on a diffuse floor through a glass
        // sphere would be lost)
        if (!(flags & FL_UNBIASED)) {
            write_features(st, si, f, st.feat + (size_t)p * 96);
            st.q_cache[atomicAdd(&st.counts[12], 1u)] = p;
            pend |= WF_CACHE;
            done = true;
        } else if (!offered) {
            offered = true;
            atomicAdd(&st.counts[33], 1u);
            const uint32_t coin = wang_hash((uint32_t)st.pix[p] * 0x9E3779B9u ^ (uint32_t)st.smp[p] * 0x85EBCA6Bu ^
                                            vw.seed * 0xC2B2AE35u ^ 0x27D4EB2Fu);
            const uint32_t r = coin <= st.tr_accept ? atomicAdd(&st.counts[32], 1u) : 0xFFFFFFFFu;
            if (r < st.tr_cap) {
                write_features(st, si, f, st.tr_feat + (size_t)r * 96);
                st.tr_idx[p] = (int32_t)r;
                st.tr_beta[p] = make_float4(beta.r, beta.g, beta.b, 0.f);
                st.tr_L0[p] = make_float4(L.r, L.g, L.b, 0.f);
                recorded = true;
            }
        }
    }
    if (!done && bsdf_roughness(f) > kCacheRough) rough_seen = true;
    uint64_t ev_mis = 0, ev_main = 0;
    if (!done) {
        if (sv.nlight > 0) {
            pend |= WF_NEE;
            const float ul = rng_1d(rng);
            int off = 0;
            {
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
            st.nee_beta[p] = make_float4(beta.r, beta.g, beta.b, lpdf_sel);
            const F2 ulight = rng_2d(rng);
            const F2 uscat = rng_2d(rng);
            const DevLight& Lt = sv.lights[off];
            const uint32_t fl = specular ? BSDF_ALL : (BSDF_ALL & ~BSDF_SPECULAR);
            LightSample ls;
            const bool delta = sample_li(sv, Lt, si, ulight, ls);
            if (ls.pdf > 0 && !is_black(ls.Li)) {
                const Spec fv = bsdf_f<LM>(f, si.wo, ls.wi, fl, RECORD ? &evs : nullptr) * absdot(ls.wi, si.sn);
                const float spdf = bsdf_pdf<LM>(f, si.wo, ls.wi, fl, RECORD ? &evs : nullptr);
                if (!is_black(fv)) {
                    const V3 org = offset_origin(si.p, si.perr, si.n, ls.p1 - si.p);
                    const V3 tgt = offset_origin(ls.p1, ls.perr1, ls.n1, org - ls.p1);
                    Spec c;
                    if (delta) {
                        c = fv * ls.Li / ls.pdf;
                    } else {
                        const float fp = 1 * ls.pdf, gp = 1 * spdf;
                        const float wgt = (fp * fp) / (fp * fp + gp * gp);
                        c = fv * ls.Li * wgt / ls.pdf;
                    }
                    const V3 dir = tgt - org;
                    st.sh_o[p] = make_float4(org.x, org.y, org.z, 0.f);
                    st.sh_d[p] = make_float4(dir.x, dir.y, dir.z, 1 - kShadowEps);
                    st.sh_c[p] = make_float4(c.r, c.g, c.b, is_black(ls.Li) ? 0.f : 1.f);
                    pend |= WF_VIS;
                }
            }
            if (!delta) {
                V3 wi = ls.wi;
                float spdf = 0;
                uint32_t stype = 0;
                EvSink cap{nullptr, 0};
                Spec fv = bsdf_sample<LM>(f, si.wo, wi, uscat, spdf, fl, stype, RECORD ? &cap : nullptr);
                ev_mis = cap.cap;
                fv = fv * absdot(wi, si.sn);
                const bool sampled_spec = (stype & BSDF_SPECULAR) != 0;
                if (!is_black(fv) && spdf > 0) {
                    float wgt = 1;
                    bool skip = false;
                    if (!sampled_spec) {
                        float lp;
                        if (Lt.kind == 0) lp = area_pdf(sv, Lt, si.p, si.perr, si.n, wi);
                        else if (Lt.kind == 1) lp = sph_pdf_infinite(wi);
                        else lp = 0.0f;
                        if (lp == 0) skip = true;
                        else {
                            const float fp = 1 * spdf, gp = 1 * lp;
                            wgt = (fp * fp) / (fp * fp + gp * gp);
                        }
                    }
                    if (!skip) {
                        const V3 org = offset_origin(si.p, si.perr, si.n, wi);
                        st.mis_o[p] = make_float4(org.x, org.y, org.z, 0.f);
                        st.mis_d[p] = make_float4(wi.x, wi.y, wi.z, 0.f);
                        st.mis_fv[p] = make_float4(fv.r, fv.g, fv.b, wgt);
                        st.mis_x[p] = make_float4(spdf, __int_as_float(off), 0.f, 0.f);
                        pend |= WF_MIS;
                    }
                }
            }
        }
        // path BSDF sample, throughput, spawn, Russian roulette (PathTracingIntegrator.cuh:80-103)
        V3 wi = v3(0, 0, 0);
        float pdf = 0;
        uint32_t stype = 0;
        const F2 ub = rng_2d(rng);
        EvSink cap{nullptr, 0};
        const Spec fv = bsdf_sample<LM>(f, si.wo, wi, ub, pdf, BSDF_ALL, stype, RECORD ? &cap : nullptr);
        ev_main = cap.cap;
        if (is_black(fv) || pdf == 0) {
            done = true;
        } else {
            specular = (stype & BSDF_SPECULAR) != 0;
            beta = beta * (fv * absdot(wi, si.sn) / pdf);
            const V3 no = offset_origin(si.p, si.perr, si.n, wi);
            st.ro[p] = make_float4(no.x, no.y, no.z, 0.f);
            st.rd[p] = make_float4(wi.x, wi.y, wi.z, 0.f);
            if (bounce >= rp.rr_start) {
                const float qq = fmaxf(0.05f, 1 - lum(beta));
                if (rng_1d(rng) < qq) done = true;
                else beta = beta / (1 - qq);
            }
            if (bounce + 1 >= rp.max_bounce) done = true;
        }
    }
    st.pend[p] = pend | (done ? WF_DONE : 0u);
    st.draw[p] = rng.draw;
    st.flags[p] = ((uint32_t)(bounce + 1) << 8) | (specular ? FL_SPECULAR : 0u) | (rough_seen ? FL_ROUGH : 0u) |
                  (flags & FL_UNBIASED) | (recorded ? FL_RECORDED : 0u) | (offered ? FL_OFFERED : 0u);
    st.beta[p] = make_float4(beta.r, beta.g, beta.b, 0.f);
    st.L[p] = make_float4(L.r, L.g, L.b, 0.f);
    if (RECORD) {
        st.sig[p] = sig;
        st.ev_mis[p] = ev_mis;
        st.ev_main[p] = ev_main;
    }
}

// shade over one class's list (k_wf_classify), grid-stride: one launch per shade class present in
// the scene, each compiled for its material kind (fewer registers, no spills, a smaller kernel).
template <bool RECORD, int LM, bool TEX>
__global__ __launch_bounds__(kWfBlock, LTS_SHADE_MIN_BLOCKS) void k_wf_shade(const SceneView sv, const RenderParams rp,
                                                                              WfState st, int pool, int cls) {
    const uint32_t n = st.counts[16 + cls];
    const int32_t* __restrict__ q = st.q_cls + (size_t)cls * pool;
    for (uint32_t i = blockIdx.x * kWfBlock + threadIdx.x; i < n; i += gridDim.x * kWfBlock)
        shade_one<RECORD, LM, TEX>(sv, rp, st, q[i]);
}


// finalize: direct light of the bounce, deferred parity events; a finished path stores its
// sample and frees its slot (pix = -1).
template <bool RECORD>
__global__ __launch_bounds__(kWfBlock) void k_wf_finalize(const SceneView sv, const RenderParams rp, WfState st,
                                                          const int32_t* __restrict__ q, const WfCtl* __restrict__ ctl) {
    const int t = blockIdx.x * kWfBlock + threadIdx.x;
    if (t >= (int)ctl->n_fin) return;
    const int p = q[t];
    const uint32_t pend = st.pend[p];
    float4 l4 = st.L[p];
    Spec L{l4.x, l4.y, l4.z};
    uint64_t sig = RECORD ? st.sig[p] : 0ull;
    if (pend & WF_NEE) {
        Spec Ld = spec(0.0f);
        if (pend & WF_VIS) {
            const uint32_t vis = st.vis[p];
            if (RECORD) fnv_mix(sig, 0x300000000ull + vis);
            const float4 c = st.sh_c[p];
            if (vis && c.w != 0.f) Ld = Ld + Spec{c.x, c.y, c.z};
        }
        if (RECORD && st.ev_mis[p]) fnv_mix(sig, st.ev_mis[p]);
        if (pend & WF_MIS) {
            if (RECORD) fnv_mix(sig, 0x200000000ull + (uint64_t)st.mis_hit[p]);
            float4 c = st.ld_mis[p];
            if (c.w == 2.f) {  // the BSDF ray landed on the sampled area light (IntegratorHelper.cuh:225-243)
                const float4 d = st.mis_d[p], fv = st.mis_fv[p], x = st.mis_x[p], mo = st.mis_o[p];
                const V3 wi = v3(d.x, d.y, d.z);
                const DevLight& Lt = sv.lights[__float_as_int(x.y)];
                SI lit;
                const V3 mro = v3(mo.x, mo.y, mo.z);
                make_si(sv, st.mis_hit[p] - 1, wi, c.x, c.y, c.z, lit, &mro);
                const Spec Li = dot(lit.n, -wi) > 0.f ? Spec{Lt.L[0], Lt.L[1], Lt.L[2]} : spec(0.0f);
                Spec cs = spec(0.0f);
                const bool add = !is_black(Li);
                if (add) cs = Spec{fv.x, fv.y, fv.z} * Li * spec(1.0f) * fv.w / x.x;
                c = make_float4(cs.r, cs.g, cs.b, add ? 1.f : 0.f);
            }
            if (c.w != 0.f) Ld = Ld + Spec{c.x, c.y, c.z};
        }
        const float4 nb = st.nee_beta[p];
        L = L + Spec{nb.x, nb.y, nb.z} * (Ld / nb.w);
    }
    if (pend & WF_CACHE) {  // the path ends in the cache: beta * cached radiance of the vertex
        const float4 c = st.cache_L[p], b = st.beta[p];
        L = L + Spec{b.x, b.y, b.z} * Spec{c.x, c.y, c.z};
    }
    if (RECORD && st.ev_main[p]) fnv_mix(sig, st.ev_main[p]);
    if (RECORD) {
        st.sig[p] = sig;
        st.ev_mis[p] = 0;
        st.ev_main[p] = 0;
    }
    if (!(pend & WF_DONE)) {
        st.L[p] = make_float4(L.r, L.g, L.b, 0.f);
        return;
    }
    if (st.cache && (st.flags[p] & FL_RECORDED)) {  // training target: radiance after the vertex / beta there
        const int r = st.tr_idx[p];
        const float4 tb = st.tr_beta[p], l0 = st.tr_L0[p];
        float* tg = st.tr_target + 3 * (size_t)r;
        tg[0] = tb.x > 0.f ? (L.r - l0.x) / tb.x : 0.f;
        tg[1] = tb.y > 0.f ? (L.g - l0.y) / tb.y : 0.f;
        tg[2] = tb.z > 0.f ? (L.b - l0.z) / tb.z : 0.f;
    }
    // Camera::addSample (Camera.cu:192-218): the sample reaches film pixels [ceil(pf - 1),
    // floor(pf + 1)] per axis.  With pf in [i, i + 1] that is i .. i + 2, gathered later, plus
    // the column i - 1 (row j - 1) when pf rounds to exactly i (j), added here.
    const float2 pf = st.pf[p];
    const int id = st.pix[p];
    const WfView& vw = st.views[st.view[p]];
    const int W = vw.W, H = vw.H;
    const int i = id % W, j = id / W;
    double* const film = rp.film + 4 * (size_t)vw.film_off;
    const int px0 = max((int)ceilf(pf.x - 1.0f), 0), py0 = max((int)ceilf(pf.y - 1.0f), 0);
    if (px0 < i || py0 < j) {
        const int px1 = min((int)floorf(pf.x + 1.0f) + 1, W), py1 = min((int)floorf(pf.y + 1.0f) + 1, H);
        for (int y = py0; y < py1; ++y)
            for (int x = px0; x < px1; ++x) {
                if (x >= i && y >= j) continue;
                const float fdx = fabsf((x - pf.x - 0.5f) * 1.0f * 16);
                const float fdy = fabsf((y - pf.y - 0.5f) * 1.0f * 16);
                const int ix = min((int)floorf(fdx), 15), iy = min((int)floorf(fdy), 15);
                const float wgt = __ldg(sv.filter + iy * 16 + ix);
                const Spec c = L * wgt;
                double* fp = film + 4 * ((size_t)y * W + x);
                atomicAdd(fp + 0, (double)c.r);
                atomicAdd(fp + 1, (double)c.g);
                atomicAdd(fp + 2, (double)c.b);
                atomicAdd(fp + 3, (double)wgt);
            }
    }
    const int w = st.wid[p];
    st.fs_L[w] = make_float4(L.r, L.g, L.b, pf.x);
    st.fs_y[w] = pf.y;
    if (RECORD) {
        const size_t k = ((size_t)(j - vw.y0) * (vw.x1 - vw.x0) + (i - vw.x0)) * vw.spp + st.smp[p];
        rp.sample_L[3 * k + 0] = L.r;
        rp.sample_L[3 * k + 1] = L.g;
        rp.sample_L[3 * k + 2] = L.b;
        rp.sample_sig[k] = sig;
    }
    st.pix[p] = -1;
}

// Every slot starts free (pix = -1, in the free list in slot order); the counts read as after a
// compaction of an empty pool (counts zeroed by the host first).
__global__ void k_wf_init_free(int32_t* q_free, int32_t* pix, uint32_t* counts, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        q_free[t] = t;
        pix[t] = -1;
    }
    if (t == 0) counts[4] = (uint32_t)n;
}

// control: one iteration's sizes from the previous compaction (path rays continuing, shadow and
// MIS rays, free slots, cache queries) and the batch's remaining samples; then clears the
// per-iteration counters (words 0..31).  `active` is 0 once nothing is left to do, and every
// kernel of such an iteration finds empty lists.
__global__ void k_wf_control(WfState st, WfCtl* ctl) {
    __shared__ uint32_t c[16];
    if (threadIdx.x < 16) c[threadIdx.x] = st.counts[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
        WfCtl x = *ctl;
        x.n_fin = x.n_ext;  // paths shaded in the previous iteration
        x.n_cont = c[0];
        x.n_sh = c[2];
        x.n_mis = c[3];
        x.nfree = c[4];
        x.n_query = c[12];
        const long long rem = x.ctot - x.generated;
        x.take = (uint32_t)min((long long)x.nfree, rem);
        x.n_ext = x.n_cont + x.take;
        x.gen0 = x.generated;
        x.generated += x.take;
        x.active = (x.n_ext | x.n_fin | x.n_sh | x.n_mis | x.n_query) ? 1u : 0u;
        x.queries += x.n_query;
        if (x.active) ++x.iters;
        *ctl = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) st.counts[threadIdx.x] = 0u;
}

// compact: one pass over the pool after shade.  Every live slot (pix >= 0) was shaded in this
// iteration, so its pend flags say which lists it joins: path rays (not finished), shadow rays
// (WF_VIS), MIS rays (WF_MIS); a slot with pix < 0 is free.  Each block scans its tile of
// kCompactTile slots and reserves its runs with one atomic per list, so every list is in slot
// order within a tile.
constexpr int kCompactThreads = 256, kCompactItems = 4, kCompactTile = kCompactThreads * kCompactItems;
__global__ __launch_bounds__(kCompactThreads) void k_wf_compact(WfState st, int32_t* __restrict__ q_ext_next, int P) {
    __shared__ uint32_t s_warp[4][kCompactThreads / 32];
    __shared__ uint32_t s_base[4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int first = blockIdx.x * kCompactTile + tid * kCompactItems;
    uint32_t flags[kCompactItems];
    uint32_t cnt[4] = {0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < kCompactItems; ++k) {
        const int slot = first + k;
        uint32_t f = 0;
        if (slot < P) {
            if (st.pix[slot] >= 0) {
                const uint32_t pend = st.pend[slot];
                f = ((pend & WF_DONE) ? 0u : 1u) | ((pend & WF_VIS) ? 2u : 0u) | ((pend & WF_MIS) ? 4u : 0u);
            } else {
                f = 8u;
            }
        }
        flags[k] = f;
#pragma unroll
        for (int l = 0; l < 4; ++l) cnt[l] += (f >> l) & 1u;
    }
    // exclusive scan of the four counts over the block (warp shuffles, then the warps' totals)
    uint32_t incl[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        uint32_t v = cnt[l];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(~0u, v, o);
            if (lane >= o) v += u;
        }
        incl[l] = v;
        if (lane == 31) s_warp[l][warp] = v;
    }
    __syncthreads();
    if (tid < 4) {
        uint32_t tot = 0;
        for (int w = 0; w < kCompactThreads / 32; ++w) {
            const uint32_t v = s_warp[tid][w];
            s_warp[tid][w] = tot;
            tot += v;
        }
        uint32_t* c = st.counts + (tid == 0 ? 0 : tid + 1);  // [0] path rays, [2] shadow, [3] mis, [4] free
        s_base[tid] = tot ? atomicAdd(c, tot) : 0u;
    }
    __syncthreads();
    int32_t* dst[4] = {q_ext_next, st.q_shadow, st.q_mis, st.q_free};
    uint32_t pos[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) pos[l] = s_base[l] + s_warp[l][warp] + incl[l] - cnt[l];
#pragma unroll
    for (int k = 0; k < kCompactItems; ++k) {
        const uint32_t f = flags[k];
#pragma unroll
        for (int l = 0; l < 4; ++l)
            if ((f >> l) & 1u) dst[l][pos[l]++] = first + k;
    }
}

// Film gather: thread (x, y) over the crop's film footprint [x0, x1 + 2) x [y0, y1 + 2) sums, in
// the fixed order (source row, source column, sample), every finished sample of the chunk whose
// filter footprint covers it from source pixels x - 2 .. x (y - 2 .. y): the pixels i .. i + 2
// that k_wf_finalize left to this kernel.  Kahan-compensated FP32 per channel, then one
// non-atomic FP64 add per channel (each film pixel has exactly one thread).
__global__ __launch_bounds__(128) void k_film_gather(const SceneView sv, double* __restrict__ film_all, const WfView vw,
                                                     const float4* __restrict__ fs_L, const float* __restrict__ fs_y) {
    __shared__ float s_filter[256];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int k = tid; k < 256; k += blockDim.x * blockDim.y) s_filter[k] = sv.filter[k];
    __syncthreads();
    const int W = vw.W, H = vw.H;
    const int x = vw.x0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int y = vw.y0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (x >= min(vw.x1 + 2, W) || y >= min(vw.y1 + 2, H)) return;
    const int cw = vw.x1 - vw.x0;
    const long npix = vw.npix;
    const int nsc = vw.nsc;
    fs_L += vw.base;
    fs_y += vw.base;
    float sum[4] = {0, 0, 0, 0}, cmp[4] = {0, 0, 0, 0};
    const int j0 = max(y - 2, vw.y0), j1 = min(y, vw.y1 - 1);
    const int i0 = max(x - 2, vw.x0), i1 = min(x, vw.x1 - 1);
    for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            const long pc = (long)(j - vw.y0) * cw + (i - vw.x0);
            for (int s = 0; s < nsc; ++s) {
                const long k = (long)s * npix + pc;
                const float4 v = __ldg(fs_L + k);
                const float fy = __ldg(fs_y + k);
                const int px1 = min((int)floorf(v.w + 1.0f) + 1, W), py1 = min((int)floorf(fy + 1.0f) + 1, H);
                if (x >= px1 || y >= py1) continue;
                const float fdx = fabsf((x - v.w - 0.5f) * 1.0f * 16);
                const float fdy = fabsf((y - fy - 0.5f) * 1.0f * 16);
                const int ix = min((int)floorf(fdx), 15), iy = min((int)floorf(fdy), 15);
                const float wgt = s_filter[iy * 16 + ix];
                const float c[4] = {v.x * wgt, v.y * wgt, v.z * wgt, wgt};
#pragma unroll
                for (int q = 0; q < 4; ++q) {  // Kahan compensation
                    const float yv = __fsub_rn(c[q], cmp[q]);
                    const float tv = __fadd_rn(sum[q], yv);
                    cmp[q] = __fsub_rn(__fsub_rn(tv, sum[q]), yv);
                    sum[q] = tv;
                }
            }
        }
    if (sum[3] == 0.f && cmp[3] == 0.f) return;
    double* fp = film_all + 4 * ((size_t)vw.film_off + (size_t)y * W + x);
#pragma unroll
    for (int q = 0; q < 4; ++q) fp[q] += (double)sum[q] - (double)cmp[q];
}

}  // namespace
}  // namespace lts
