// Device vector math with the reference's evaluation order (geometry/Vector.cuh, Point.cuh,
// Normal.cuh, Geometry.cuh, rendering/Spectrum.cuh).  Sums associate left to right as the
// reference's operators do; FMA contraction is left to the compiler.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lts {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(V3 a, float f) { return v3(f * a.x, f * a.y, f * a.z); }
__device__ __forceinline__ V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float absdot(V3 a, V3 b) { return fabsf(dot(a, b)); }
__device__ __forceinline__ float len2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ V3 vabs(V3 a) { return v3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__device__ __forceinline__ float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ V3 face_towards(V3 n, V3 v) { return dot(n, v) < 0.0f ? -n : n; }

// a*b - c*d with Kahan's FMA algorithm: within 1.5 ulp, and in nearly every case the correctly
// rounded result -- which is what the reference's double-precision cross product rounds to
// (Geometry.cuh:76-83: exact double products, one double subtraction, one float rounding).
__device__ __forceinline__ float diff_prod(float a, float b, float c, float d) {
    const float w = c * d;
    const float e = fmaf(-c, d, w);
    const float f = fmaf(a, b, -w);
    return f + e;
}
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(diff_prod(a.y, b.z, a.z, b.y), diff_prod(a.z, b.x, a.x, b.z), diff_prod(a.x, b.y, a.y, b.x));
}

// Geometry.cuh:15-29, 32-bit integer read (the Windows build the reference targets).
__device__ __forceinline__ float rsqrt_q3(float f) {
    const float x2 = f * 0.5f;
    float y = f;
    int i = __float_as_int(y);
    i = 0x5f3759df - (i >> 1);
    y = __int_as_float(i);
    y = y * (1.5f - (x2 * y * y));
    y = y * (1.5f - (x2 * y * y));
    return y;
}
__device__ __forceinline__ V3 normalize(V3 v) { return v * rsqrt_q3(len2(v)); }

// x * C for a double constant C = hi + lo, rounded once to float: the value the reference
// gets from `float * M_PI`-style double expressions converted back to float.
__device__ __forceinline__ float mul_dc(float x, float hi, float lo) {
    const float p = x * hi;
    const float e = fmaf(x, hi, -p);
    return p + fmaf(x, lo, e);
}
// 2*M_PI and M_1_PI split into float hi + lo parts.
#define LTS_2PI_HI 6.28318548202514648438f
#define LTS_2PI_LO (-1.7484555314695172e-07f)
#define LTS_1_PI_HI 0.31830987334251403809f
#define LTS_1_PI_LO 1.2841276486597053e-08f

// core/ErrorHelper.cuh:55-85
__device__ __forceinline__ float next_float_up(float f) {
    if (isinf(f) && f > 0.0f) return f;
    if (f == -0.0f) f = 0.0f;
    uint32_t ui = __float_as_uint(f);
    if (f >= 0) ++ui;
    else --ui;
    return __uint_as_float(ui);
}
__device__ __forceinline__ float next_float_down(float f) {
    if (isinf(f) && f > 0.0f) return f;
    if (f == -0.0f) f = 0.0f;
    uint32_t ui = __float_as_uint(f);
    if (f >= 0) --ui;
    else ++ui;
    return __uint_as_float(ui);
}
__host__ __device__ constexpr float machine_eps() { return 0.5f * 1.19209290e-07F; }
__host__ __device__ constexpr float gamma_n(int n) { return (n * machine_eps()) / (1 - n * machine_eps()); }

__device__ __forceinline__ float clampf(float f, float lo, float hi) { return (f < lo) ? lo : ((f > hi) ? hi : f); }

// Spectrum (rendering/Spectrum.cuh)
struct Spec {
    float r, g, b;
};
__device__ __forceinline__ Spec spec(float v) { return Spec{v, v, v}; }
__device__ __forceinline__ Spec operator+(Spec a, Spec b) { return Spec{a.r + b.r, a.g + b.g, a.b + b.b}; }
__device__ __forceinline__ Spec operator-(Spec a, Spec b) { return Spec{a.r - b.r, a.g - b.g, a.b - b.b}; }
__device__ __forceinline__ Spec operator*(Spec a, Spec b) { return Spec{a.r * b.r, a.g * b.g, a.b * b.b}; }
__device__ __forceinline__ Spec operator*(Spec a, float v) { return Spec{a.r * v, a.g * v, a.b * v}; }
__device__ __forceinline__ Spec operator/(Spec a, float v) { return Spec{a.r / v, a.g / v, a.b / v}; }
__device__ __forceinline__ Spec operator/(Spec a, Spec b) { return Spec{a.r / b.r, a.g / b.g, a.b / b.b}; }
__device__ __forceinline__ bool is_black(Spec s) { return s.r == 0.0f && s.g == 0.0f && s.b == 0.0f; }
__device__ __forceinline__ float lum(Spec s) { return 0.212671f * s.r + 0.715160f * s.g + 0.072169f * s.b; }
__device__ __forceinline__ Spec ssqrt(Spec s) { return Spec{sqrtf(s.r), sqrtf(s.g), sqrtf(s.b)}; }

}  // namespace lts
