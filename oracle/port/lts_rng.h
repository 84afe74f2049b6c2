/*
 * Test infrastructure (oracle): CPU statement of the project's per-pixel sampler.
 *
 * The reference draws from cuRAND XORWOW, seeded per pixel with `seed + wangHash(id)`
 * (sampling/Sampler.cuh:39-42, core/GeneralHelper.cuh:141-148) and read with
 * curand_uniform, whose range is (0, 1].  cuRAND's generator is NVIDIA's code and is not
 * restated here.  Both the GPU renderer and this oracle instead use one project-owned
 * counter-based generator, Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
 * numbers: as easy as 1, 2, 3", SC'11), written from the paper:
 *
 *   key      = { seed + wangHash(pixel), 0x4c54530a }
 *   counter  = { draw / 4, sample, 0, 0 }           (one sub-stream per (pixel, sample))
 *   word     = philox4x32_10(counter, key)[draw % 4]
 *   uniform  = ((word >> 8) + 1) * 2^-24            in (0, 1], like curand_uniform
 *
 * The draw ORDER within a sample is the reference's (PathTracingIntegrator.cuh:41-99):
 * film(2), lens(2); per bounce: light select(1), light(2), scatter(2) when the scene has
 * lights, BSDF(2), Russian roulette(1) from the roulette bounce on.
 */
#ifndef LTS_ORACLE_RNG_H
#define LTS_ORACLE_RNG_H

#include <stdint.h>

#define LTS_RNG_KEY1 0x4c54530au

static inline uint32_t lts_wang_hash(uint32_t a) {
    /* GeneralHelper.cuh:141-148 */
    a = (a ^ 61u) ^ (a >> 16);
    a = a + (a << 3);
    a = a ^ (a >> 4);
    a = a * 0x27d4eb2du;
    a = a ^ (a >> 15);
    return a;
}

static inline void lts_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

static inline uint32_t lts_rng_key(uint32_t seed, uint32_t pixel) { return seed + lts_wang_hash(pixel); }

static inline float lts_rng_word_to_uniform(uint32_t w) {
    return (float)((w >> 8) + 1u) * (1.0f / 16777216.0f);
}

static inline float lts_rng_uniform(uint32_t key0, uint32_t sample, uint32_t draw) {
    const uint32_t ctr[4] = {draw >> 2, sample, 0u, 0u};
    const uint32_t key[2] = {key0, LTS_RNG_KEY1};
    uint32_t out[4];
    lts_philox4x32_10(ctr, key, out);
    return lts_rng_word_to_uniform(out[draw & 3u]);
}

#endif
