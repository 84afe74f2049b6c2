// Shared device helpers for the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace lts {

// Monotone u32 key of a float: key(a) < key(b) iff a < b, with -0 ordered before +0.
__host__ __device__ inline uint32_t float_key(float f) {
    uint32_t b;
#ifdef __CUDA_ARCH__
    b = __float_as_uint(f);
#else
    memcpy(&b, &f, 4);
#endif
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__host__ __device__ inline float key_float(uint32_t k) {
    uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
#ifdef __CUDA_ARCH__
    f = __uint_as_float(b);
#else
    memcpy(&f, &b, 4);
#endif
    return f;
}

// Device-side error word shared by all kernels of a context: a kernel that gives up a bounded
// wait (or meets an impossible state) ORs a code in and returns; the host reads it after the
// stream synchronises and reports LTS_ERR_DEVICE.
enum DeviceError : uint32_t {
    DEV_ERR_LOOKBACK_TIMEOUT = 1u,
    DEV_ERR_STACK_OVERFLOW = 2u,
    DEV_ERR_QUEUE_OVERFLOW = 4u,
    DEV_ERR_BAD_INDEX = 8u,
    DEV_ERR_CAPACITY = 16u,
    DEV_ERR_MMA_TIMEOUT = 32u,
};

// Upper bound of spin iterations of any wait on another block's flag.  A tile's predecessor
// publishes within microseconds; 1<<22 polls with nanosleep back-off is well over a second.
constexpr int kSpinLimit = 1 << 22;

// Every device allocation of the library goes through these: they keep the byte count of the
// context metrics and honour LTS_MAX_DEVICE_MB (a cap used to inject out-of-memory failures).
cudaError_t dev_alloc(void** p, size_t bytes);
void dev_free(void* p);
size_t dev_bytes_in_use();

}  // namespace lts
