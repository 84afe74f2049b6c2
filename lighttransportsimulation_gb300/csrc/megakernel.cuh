// Path-tracing megakernel: one thread per pixel, all samples and bounces, as the reference's
// PathTracingKernel (intergrators/IntegratorKernels.cu:17-23) runs
// PathTracingIntegrator::evaluate (intergrators/PathTracingIntegrator.cuh:26-109).  Compiled in
// `real` = real by tracer.cu (the megakernel integrator) and in `real` = double by render64.cu
// (the FP64 oracle renderer).
#pragma once

#include "tracer_dev.cuh"

namespace lts {
namespace {

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
// Resident blocks per SM the register budget is cut for.
#ifndef LTS_MEGA_MIN_BLOCKS
#define LTS_MEGA_MIN_BLOCKS 1
#endif
template <bool RECORD>
__global__ __launch_bounds__(kThreads, LTS_MEGA_MIN_BLOCKS) void k_pathtrace(const SceneView sv, const RenderParams rp, int nleaf) {
    __shared__ uint32_t s_stack[kStack * kThreads];
    const int tid = threadIdx.y * kBX + threadIdx.x;
    uint32_t* stack = s_stack + tid;
#if !LTS_FP64
    __shared__ float s_film[32 * kThreads];
    float* acc = s_film + tid;
#else  // the FP64 build sums its 2x2 core pixels in double (no compensation needed)
    __shared__ double s_film64[16 * kThreads];
    double* acc64 = s_film64 + tid;
#endif
    const int i = rp.x0 + blockIdx.x * kBX + threadIdx.x;
    const int j = rp.y0 + blockIdx.y * kBY + threadIdx.y;
    if (i >= rp.x1 || j >= rp.y1) return;
    const int W = sv.width, H = sv.height;
    const int id = j * W + i;
    unsigned long long rays = 0;
    Work wk{0u, 0u};
#if !LTS_FP64
#pragma unroll
    for (int k = 0; k < 32; ++k) acc[k * kThreads] = 0.0f;
#else
#pragma unroll
    for (int k = 0; k < 16; ++k) acc64[k * kThreads] = 0.0;
#endif

    const float* cam = sv.cam;
    const V3 co = v3(cam[0], cam[1], cam[2]), cright = v3(cam[3], cam[4], cam[5]), cup = v3(cam[6], cam[7], cam[8]),
             cllc = v3(cam[9], cam[10], cam[11]);
    const real rx = (real)(W - 1), ry = (real)(H - 1);

    Rng rng;
    rng.key = rp.seed + wang_hash((uint32_t)id);

    // samples of the pixel: all of them when gridDim.z is 1 (the float renderer); the FP64 oracle
    // launch splits them over z so that a small crop still fills the GPU (every sample has its own
    // counter-based stream, so the split changes no value)
    for (int s = (int)blockIdx.z; s < rp.spp; s += (int)gridDim.z) {
        rng.sample = (uint32_t)s;
        rng.draw = 0;
        uint64_t sig = 0xcbf29ce484222325ull;
        EvSink evs{&sig, 0};
        Tracer16 tr{nullptr, 0};
        if (RECORD && rp.trace &&
            ((long)((j - rp.y0) * (rp.x1 - rp.x0) + (i - rp.x0)) * rp.spp + s) == rp.trace_sample)
            tr.out = rp.trace;
        // 3. camera ray (PathTracingIntegrator.cuh:40-46, Camera.cu:51-81); aperture is 0, so the
        // lens sample moves nothing, but it is drawn.
        const F2 fs = rng_2d(rng);
        (void)rng_2d(rng);
        const real pfx = (real)(i + fs.x), pfy = (real)(j + fs.y);
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
            if (!hit) break;
            // 7. scattering functions: differentials (Interaction.cuh:118-160) then material
            if (has_diff) {
                const V3 n = si.n;
                const real d = -dot(n, si.p);
                const real tx = (-dot(n, ro) - d) / dot(n, rxd);
                const real ty = (-dot(n, ro) - d) / dot(n, ryd);
                si.dpdx = (ro + rxd * tx) - si.p;
                si.dpdy = (ro + ryd * ty) - si.p;
            } else {
                si.dpdx = v3(0, 0, 0);
                si.dpdy = v3(0, 0, 0);
            }
            Bsdf f;
            if (!make_bsdf(sv, si, f, RECORD ? &evs : nullptr)) break;
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
                        off = (int)clampf((real)(first - 1), 0.0f, (real)(size - 2));
                    }
                }
                const real lpdf_sel = __ldg(sv.light_func + off) / (sv.light_func_int * sv.nlight);
                const F2 ulight = rng_2d(rng);
                const F2 uscat = rng_2d(rng);
                const DevLight& Lt = sv.lights[off];
                const uint32_t flags = specular ? BSDF_ALL : (BSDF_ALL & ~BSDF_SPECULAR);
                Spec Ld = spec(0.0f);
                LightSample ls;
                const bool delta = sample_li(sv, Lt, si, ulight, ls);
                if (ls.pdf > 0 && !is_black(ls.Li)) {
                    const Spec fv = bsdf_f(f, si.wo, ls.wi, flags, RECORD ? &evs : nullptr) * absdot(ls.wi, si.sn);
                    const real spdf = bsdf_pdf(f, si.wo, ls.wi, flags, RECORD ? &evs : nullptr);
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
                                const real fp = 1 * ls.pdf, gp = 1 * spdf;
                                const real wgt = (fp * fp) / (fp * fp + gp * gp);
                                Ld = Ld + fv * Li * wgt / ls.pdf;
                            }
                        }
                    }
                }
                if (!delta) {
                    V3 wi = ls.wi;
                    real spdf = 0;
                    uint32_t stype = 0;
                    Spec fv = bsdf_sample(f, si.wo, wi, uscat, spdf, flags, stype, RECORD ? &evs : nullptr);
                    fv = fv * absdot(wi, si.sn);
                    const bool sampled_spec = (stype & BSDF_SPECULAR) != 0;
                    if (!is_black(fv) && spdf > 0) {
                        real wgt = 1;
                        bool done = false;
                        if (!sampled_spec) {
                            real lp;
                            if (Lt.kind == 0) lp = area_pdf(sv, Lt, si.p, si.perr, si.n, wi);
                            else if (Lt.kind == 1) lp = sph_pdf_infinite(wi);
                            else lp = 0.0f;
                            if (lp == 0) done = true;
                            else {
                                const real fp = 1 * spdf, gp = 1 * lp;
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
                                if (lit.light == off && Lt.kind == 0)
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
            real pdf = 0;
            uint32_t stype = 0;
            const F2 ub = rng_2d(rng);
            const Spec fv = bsdf_sample(f, si.wo, wi, ub, pdf, BSDF_ALL, stype, RECORD ? &evs : nullptr);
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
                const real q = xmax(0.05f, 1 - lum(beta));
                if (rng_1d(rng) < q) break;
                beta = beta / (1 - q);
            }
        }
        // 10. film (Camera::addSample, Camera.cu:192-218)
        {
            const int px0 = max((int)xceil(pfx - 1.0f), 0), py0 = max((int)xceil(pfy - 1.0f), 0);
            const int px1 = min((int)xfloor(pfx + 1.0f) + 1, W), py1 = min((int)xfloor(pfy + 1.0f) + 1, H);
            for (int y = py0; y < py1; ++y) {
                for (int x = px0; x < px1; ++x) {
                    const real fdx = xabs((x - pfx - 0.5f) * 1.0f * 16);
                    const real fdy = xabs((y - pfy - 0.5f) * 1.0f * 16);
                    const int ix = min((int)xfloor(fdx), 15), iy = min((int)xfloor(fdy), 15);
                    const real wgt = __ldg(sv.filter + iy * 16 + ix);
                    const Spec c = L * wgt;
                    const int ox = x - i, oy = y - j;
                    if (ox >= 0 && ox <= 1 && oy >= 0 && oy <= 1) {
                        const int base = (oy * 2 + ox) * 4;
#if !LTS_FP64
                        kahan_add(acc + (base + 0) * kThreads, acc + (16 + base + 0) * kThreads, c.r);
                        kahan_add(acc + (base + 1) * kThreads, acc + (16 + base + 1) * kThreads, c.g);
                        kahan_add(acc + (base + 2) * kThreads, acc + (16 + base + 2) * kThreads, c.b);
                        kahan_add(acc + (base + 3) * kThreads, acc + (16 + base + 3) * kThreads, wgt);
#else
                        acc64[(base + 0) * kThreads] += (double)c.r;
                        acc64[(base + 1) * kThreads] += (double)c.g;
                        acc64[(base + 2) * kThreads] += (double)c.b;
                        acc64[(base + 3) * kThreads] += (double)wgt;
#endif
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
    // flush the 2x2 core accumulators (float: sum minus compensation) to the FP64 film
    for (int oy = 0; oy < 2; ++oy)
        for (int ox = 0; ox < 2; ++ox) {
            const int x = i + ox, y = j + oy;
            if (x >= W || y >= H) continue;
            double* fp = rp.film + 4 * ((size_t)y * W + x);
            const int base = (oy * 2 + ox) * 4;
            for (int c = 0; c < 4; ++c) {
#if !LTS_FP64
                const float sum = acc[(base + c) * kThreads], cmp = acc[(16 + base + c) * kThreads];
                if (sum != 0.0f || cmp != 0.0f) atomicAdd(fp + c, (double)sum - (double)cmp);
#else
                const double sum = acc64[(base + c) * kThreads];
                if (sum != 0.0) atomicAdd(fp + c, sum);
#endif
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

}  // namespace
}  // namespace lts
