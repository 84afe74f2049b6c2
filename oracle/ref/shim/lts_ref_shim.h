/*
 * Test infrastructure only: nothing in the product links or calls this file.
 *
 * Host shim that lets the reference's CUDA C++ (tierChampion/LightTransportSimulation,
 * src/) compile unmodified as host C++ with g++ + OpenMP.  It is force-included ahead of
 * every reference header by oracle/ref/build_ref.sh, together with empty stand-ins for
 * <cuda_runtime.h>, <curand_kernel.h> and <thrust/*.h> from oracle/ref/shim/include/.
 *
 * What it supplies:
 *   - __host__/__device__/__global__ defined away; dim3, blockIdx/threadIdx as thread_local;
 *   - lts_launch(kernel, grid, block)(args...): the build script rewrites every
 *     `k<<<g,b>>>(args)` launch of the preprocessed reference into this call, which runs the
 *     blocks under `#pragma omp parallel for schedule(dynamic,1)` and the threads of one
 *     block sequentially (no reference kernel uses __syncthreads or shared memory);
 *   - cudaMalloc/Memcpy/Free on host memory (allocations are padded by 64 KiB and zeroed,
 *     because SceneLoader.cuh:297,321 under-allocate the material and light pointer tables;
 *     cudaFree leaks on purpose so the harness can still read freed tables);
 *   - atomics via GCC __atomic builtins, __clz, __float_as_int/uint;
 *   - thrust::stable_sort_by_key via std::stable_sort over an index permutation (same stable
 *     order as the reference's BVH.cuh:140-146), recording its output for the dump;
 *   - curand_init/curand_uniform mapped onto the project's counter-based sampler
 *     (Philox-4x32-10, oracle/port/lts_rng.h), keyed per pixel by `seed + wangHash(id)`
 *     exactly as Sampler.cuh:39-42 keys cuRAND, with one sub-stream per (pixel, sample).
 */
#pragma once

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits.h>
#include <numeric>
#include <string>
#include <vector>
#include <omp.h>

#include "../../port/lts_rng.h"

using std::isinf;
using std::isnan;

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __constant__

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned xx = 1, unsigned yy = 1, unsigned zz = 1) : x(xx), y(yy), z(zz) {}
};
typedef dim3 uint3;

inline thread_local dim3 blockIdx(0, 0, 0);
inline thread_local dim3 threadIdx(0, 0, 0);
inline thread_local dim3 blockDim(1, 1, 1);
inline thread_local dim3 gridDim(1, 1, 1);

template <class K>
struct lts_launcher {
    K k;
    dim3 g, b;
    template <class... A>
    void operator()(A... a) const {
        const long nb = (long)g.x * g.y * g.z;
        const dim3 gg = g, bb = b;
        const K kk = k;
#pragma omp parallel for schedule(dynamic, 1)
        for (long bi = 0; bi < nb; ++bi) {
            gridDim = gg;
            blockDim = bb;
            blockIdx = dim3((unsigned)(bi % gg.x), (unsigned)((bi / gg.x) % gg.y),
                            (unsigned)(bi / ((long)gg.x * gg.y)));
            for (unsigned tz = 0; tz < bb.z; ++tz)
                for (unsigned ty = 0; ty < bb.y; ++ty)
                    for (unsigned tx = 0; tx < bb.x; ++tx) {
                        threadIdx = dim3(tx, ty, tz);
                        kk(a...);
                    }
        }
    }
};
template <class K>
inline lts_launcher<K> lts_launch(K k, dim3 g, dim3 b) {
    return lts_launcher<K>{k, g, b};
}

/* ---- CUDA runtime on host memory ---- */
typedef int cudaError_t;
typedef int cudaError;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3
};
enum cudaLimit { cudaLimitStackSize = 0, cudaLimitMallocHeapSize = 2 };
static const size_t LTS_SHIM_PAD = 64 * 1024;
inline cudaError_t cudaMalloc(void** p, size_t n) {
    *p = calloc(n + LTS_SHIM_PAD, 1);
    return *p ? 0 : 2;
}
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t n) {
    return cudaMalloc((void**)p, n);
}
inline cudaError_t cudaFree(void*) { return 0; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    if (n) memcpy(d, s, n);
    return 0;
}
inline cudaError_t cudaDeviceSynchronize() { return 0; }
inline cudaError_t cudaPeekAtLastError() { return 0; }
inline cudaError_t cudaGetLastError() { return 0; }
inline const char* cudaGetErrorString(cudaError_t) { return "host shim"; }
inline cudaError_t cudaRuntimeGetVersion(int* v) { *v = 0; return 0; }
inline cudaError_t cudaDeviceSetLimit(cudaLimit, size_t) { return 0; }

/* ---- atomics ---- */
inline float atomicAdd(float* a, float v) {
    uint32_t* ui = (uint32_t*)a;
    uint32_t old = __atomic_load_n(ui, __ATOMIC_SEQ_CST), nw;
    do {
        float f;
        memcpy(&f, &old, 4);
        f += v;
        memcpy(&nw, &f, 4);
    } while (!__atomic_compare_exchange_n(ui, &old, nw, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST));
    float r;
    memcpy(&r, &old, 4);
    return r;
}
inline int atomicAdd(int* a, int v) { return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST); }
inline unsigned atomicAdd(unsigned* a, unsigned v) { return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST); }
inline int atomicCAS(int* a, int cmp, int val) {
    __atomic_compare_exchange_n(a, &cmp, val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return cmp;
}
template <class T>
inline T lts_atomic_minmax(T* a, T v, bool is_min) {
    T old = __atomic_load_n(a, __ATOMIC_SEQ_CST);
    while (is_min ? (v < old) : (v > old)) {
        if (__atomic_compare_exchange_n(a, &old, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) break;
    }
    return old;
}
inline int atomicMin(int* a, int v) { return lts_atomic_minmax(a, v, true); }
inline int atomicMax(int* a, int v) { return lts_atomic_minmax(a, v, false); }
inline unsigned atomicMin(unsigned* a, unsigned v) { return lts_atomic_minmax(a, v, true); }
inline unsigned atomicMax(unsigned* a, unsigned v) { return lts_atomic_minmax(a, v, false); }

inline int __float_as_int(float f) { int i; memcpy(&i, &f, 4); return i; }
inline unsigned __float_as_uint(float f) { unsigned i; memcpy(&i, &f, 4); return i; }
inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz((unsigned)x); }

/* ---- Windows-only helpers the reference names ---- */
#define _aligned_free free
inline char* _fullpath(char* buf, const char* path, size_t) { return realpath(path, buf); }

/* ---- thrust stand-in: stable key sort, recorded for the dump ---- */
inline std::vector<uint32_t> lts_ref_sorted_codes;
inline std::vector<int> lts_ref_sorted_ids;
namespace thrust {
template <class T>
struct device_ptr {
    T* p;
    device_ptr operator+(long n) const { return device_ptr{p + n}; }
    long operator-(const device_ptr& o) const { return (long)(p - o.p); }
};
template <class T>
inline device_ptr<T> device_pointer_cast(T* p) { return device_ptr<T>{p}; }
template <class K, class V>
inline void stable_sort_by_key(device_ptr<K> kb, device_ptr<K> ke, device_ptr<V> vb) {
    const long n = ke - kb;
    std::vector<long> idx(n);
    std::iota(idx.begin(), idx.end(), 0L);
    std::stable_sort(idx.begin(), idx.end(), [&](long a, long b) { return kb.p[a] < kb.p[b]; });
    std::vector<K> ks(n);
    std::vector<V> vs(n);
    for (long i = 0; i < n; ++i) {
        ks[i] = kb.p[idx[i]];
        vs[i] = vb.p[idx[i]];
    }
    for (long i = 0; i < n; ++i) {
        kb.p[i] = ks[i];
        vb.p[i] = vs[i];
    }
    lts_ref_sorted_codes.assign(ks.begin(), ks.end());
    lts_ref_sorted_ids.assign(vs.begin(), vs.end());
}
}  // namespace thrust

/* ---- cuRAND stand-in on the project sampler ---- */
inline thread_local uint32_t lts_ref_cur_sample = 0;
struct curandState_t {
    uint32_t key;
    uint32_t sample;
    uint32_t draw;
};
typedef curandState_t curandState;
inline void curand_init(unsigned long long seed, unsigned long long, unsigned long long, curandState_t* s) {
    s->key = (uint32_t)seed;
    s->sample = lts_ref_cur_sample;
    s->draw = 0;
}
inline float curand_uniform(curandState_t* s) {
    if (s->sample != lts_ref_cur_sample) {
        s->sample = lts_ref_cur_sample;
        s->draw = 0;
    }
    return lts_rng_uniform(s->key, s->sample, s->draw++);
}

/* ---- per-sample recording hooks (called from lines the build script instruments) ---- */
void lts_hook_begin_sample(int id, int s);
void lts_hook_hit(const void* prim);
void lts_hook_mis(const void* prim);
bool lts_hook_vis(bool unoccluded);
void lts_hook_sample(int id, int s, float r, float g, float b);
void lts_hook_branch(unsigned long long v);
bool lts_hook_bool(unsigned long long tag, bool v);
