// Device vector math with the reference's evaluation order (geometry/Vector.cuh, Point.cuh,
// Normal.cuh, Geometry.cuh, rendering/Spectrum.cuh).  Sums associate left to right as the
// reference's operators do; FMA contraction is left to the compiler.
//
// The integrator's arithmetic type is `real`: float for the renderer, double for the FP64
// oracle renderer (render64.cu defines LTS_REAL as double before including the integrator).
// The float build keeps the reference's float-specific forms (Quake rsqrt, float thresholds of
// its double comparisons, double constants rounded once to float); the double build evaluates
// the same expressions in double with exact square roots and the double comparisons themselves.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#ifndef LTS_REAL
#define LTS_REAL float
#define LTS_FP64 0
#else
#define LTS_FP64 1
#endif

namespace lts {
namespace {

typedef LTS_REAL real;

// math on `real` (the float build calls the float functions by name)
#if LTS_FP64
__device__ __forceinline__ real xabs(real a) { return fabs(a); }
__device__ __forceinline__ real xsqrt(real a) { return sqrt(a); }
__device__ __forceinline__ real xmin(real a, real b) { return fmin(a, b); }
__device__ __forceinline__ real xmax(real a, real b) { return fmax(a, b); }
__device__ __forceinline__ real xfloor(real a) { return floor(a); }
__device__ __forceinline__ real xceil(real a) { return ceil(a); }
__device__ __forceinline__ real xcos(real a) { return cos(a); }
__device__ __forceinline__ real xsin(real a) { return sin(a); }
__device__ __forceinline__ real xacos(real a) { return acos(a); }
__device__ __forceinline__ real xlog2(real a) { return log2(a); }
__device__ __forceinline__ real xfma(real a, real b, real c) { return fma(a, b, c); }
__device__ __forceinline__ real xrcp(real a) { return 1.0 / a; }
__device__ __forceinline__ real xdiv(real a, real b) { return a / b; }
#else
__device__ __forceinline__ real xabs(real a) { return fabsf(a); }
__device__ __forceinline__ real xsqrt(real a) { return sqrtf(a); }
__device__ __forceinline__ real xmin(real a, real b) { return fminf(a, b); }
__device__ __forceinline__ real xmax(real a, real b) { return fmaxf(a, b); }
__device__ __forceinline__ real xfloor(real a) { return floorf(a); }
__device__ __forceinline__ real xceil(real a) { return ceilf(a); }
// The four transcendentals of the float path.  c_libm_double = 1 (option "libm_double")
// evaluates them in double and rounds once to float -- the correctly rounded result except when
// the double result lies within its own last bit of a float rounding boundary -- which is what
// the reference's host build gets from glibc (or from the double functions it calls on float
// arguments); 0 (default) uses CUDA's float functions.  The flag is uniform over a launch.
__constant__ int c_libm_double;
__device__ __forceinline__ real xcos(real a) { return c_libm_double ? (float)cos((double)a) : cosf(a); }
__device__ __forceinline__ real xsin(real a) { return c_libm_double ? (float)sin((double)a) : sinf(a); }
__device__ __forceinline__ real xacos(real a) { return c_libm_double ? (float)acos((double)a) : acosf(a); }
__device__ __forceinline__ real xlog2(real a) { return c_libm_double ? (float)log2((double)a) : log2f(a); }
__device__ __forceinline__ real xfma(real a, real b, real c) { return fmaf(a, b, c); }
__device__ __forceinline__ real xrcp(real a) { return __frcp_rn(a); }     // == (float)(1.0 / (double)a)
__device__ __forceinline__ real xdiv(real a, real b) { return __fdiv_rn(a, b); }
#endif

struct V3 {
    real x, y, z;
};
__device__ __forceinline__ V3 v3(real x, real y, real z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(V3 a, real f) { return v3(f * a.x, f * a.y, f * a.z); }
__device__ __forceinline__ V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ real dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ real absdot(V3 a, V3 b) { return xabs(dot(a, b)); }
__device__ __forceinline__ real len2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ V3 vabs(V3 a) { return v3(xabs(a.x), xabs(a.y), xabs(a.z)); }
__device__ __forceinline__ real comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ V3 face_towards(V3 n, V3 v) { return dot(n, v) < 0 ? -n : n; }

// a*b - c*d as the reference's cross product rounds it (Geometry.cuh:76-83: exact products in
// double, one double subtraction, one rounding to float), which is the correctly rounded value
// except when the double subtraction lands within 2^-53 of a float midpoint.  In float: both
// products split exactly into value + error (FMA), the difference of the values exactly into
// s + t (TwoSum, Knuth), and s + (t + (e1 - e2)) rounded once more; the inner sum is below half
// an ulp of s, so the result is the correctly rounded one unless the exact value lies within
// ~2^-24 ulp of a midpoint (none in 60,000 random and cancelling cases against exact rational
// arithmetic).  13 operations.
__device__ __forceinline__ real diff_prod(real a, real b, real c, real d) {
#if LTS_FP64
    return a * b - c * d;
#else
    const real p1 = a * b, e1 = xfma(a, b, -p1);
    const real p2 = c * d, e2 = xfma(c, d, -p2);
    const real s = p1 - p2;
    const real bb = s - p1;
    const real t = (p1 - (s - bb)) + (-p2 - bb);
    return s + (t + (e1 - e2));
#endif
}
// The same within 1.5 ulp in 4 operations (Kahan: w = cd; (ab - w) + (w - cd)), misrounding about
// 15 % of random cases: the traversal's triangle tests use it, and the winning triangle's values
// are recomputed with diff_prod (hit_exact).
__device__ __forceinline__ real diff_prod_fast(real a, real b, real c, real d) {
    const real w = c * d;
    const real e = xfma(-c, d, w);
    const real f = xfma(a, b, -w);
    return f + e;
}
__device__ __forceinline__ V3 cross_fast(V3 a, V3 b) {
    return v3(diff_prod_fast(a.y, b.z, a.z, b.y), diff_prod_fast(a.z, b.x, a.x, b.z), diff_prod_fast(a.x, b.y, a.y, b.x));
}
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(diff_prod(a.y, b.z, a.z, b.y), diff_prod(a.z, b.x, a.x, b.z), diff_prod(a.x, b.y, a.y, b.x));
}

#if LTS_FP64
__device__ __forceinline__ real rsqrt_q3(real f) { return 1.0 / sqrt(f); }
// x * C for the double constant C
__device__ __forceinline__ real mul_dc(real x, double c) { return x * c; }
#define LTS_2PI (2.0 * 3.14159265358979323846)
#define LTS_1_PI (1.0 / 3.14159265358979323846)
#define LTS_INV_PI_F (1.0 / 3.14159265358979323846)
#else
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
// x * C for a double constant C = hi + lo, rounded once to float: the value the reference
// gets from `float * M_PI`-style double expressions converted back to float.
struct DConst {
    float hi, lo;
};
__device__ __forceinline__ float mul_dc(float x, DConst c) {
    const float p = x * c.hi;
    const float e = fmaf(x, c.hi, -p);
    return p + fmaf(x, c.lo, e);
}
// 2*M_PI and M_1_PI split into float hi + lo parts.
#define LTS_2PI (DConst{6.28318548202514648438f, -1.7484555314695172e-07f})
#define LTS_1_PI (DConst{0.31830987334251403809f, 1.2841276486597053e-08f})
// a float constant 1/pi (the reference's InvPi)
#define LTS_INV_PI_F 0.31830987334251403809f
#endif
__device__ __forceinline__ V3 normalize(V3 v) { return v * rsqrt_q3(len2(v)); }

// core/ErrorHelper.cuh:55-85
#if LTS_FP64
__device__ __forceinline__ real next_float_up(real f) {
    if (isinf(f) && f > 0) return f;
    if (f == -0.0) f = 0.0;
    long long ui = __double_as_longlong(f);
    if (f >= 0) ++ui;
    else --ui;
    return __longlong_as_double(ui);
}
__device__ __forceinline__ real next_float_down(real f) {
    if (isinf(f) && f > 0) return f;
    if (f == -0.0) f = 0.0;
    long long ui = __double_as_longlong(f);
    if (f >= 0) --ui;
    else ++ui;
    return __longlong_as_double(ui);
}
__host__ __device__ constexpr double machine_eps() { return 0.5 * 2.220446049250313e-16; }
__host__ __device__ constexpr double gamma_n(int n) { return (n * machine_eps()) / (1 - n * machine_eps()); }
#else
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
#endif

__device__ __forceinline__ real clampf(real f, real lo, real hi) { return (f < lo) ? lo : ((f > hi) ? hi : f); }

// Spectrum (rendering/Spectrum.cuh)
struct Spec {
    real r, g, b;
};
__device__ __forceinline__ Spec spec(real v) { return Spec{v, v, v}; }
__device__ __forceinline__ Spec operator+(Spec a, Spec b) { return Spec{a.r + b.r, a.g + b.g, a.b + b.b}; }
__device__ __forceinline__ Spec operator-(Spec a, Spec b) { return Spec{a.r - b.r, a.g - b.g, a.b - b.b}; }
__device__ __forceinline__ Spec operator*(Spec a, Spec b) { return Spec{a.r * b.r, a.g * b.g, a.b * b.b}; }
__device__ __forceinline__ Spec operator*(Spec a, real v) { return Spec{a.r * v, a.g * v, a.b * v}; }
__device__ __forceinline__ Spec operator/(Spec a, real v) { return Spec{a.r / v, a.g / v, a.b / v}; }
__device__ __forceinline__ Spec operator/(Spec a, Spec b) { return Spec{a.r / b.r, a.g / b.g, a.b / b.b}; }
__device__ __forceinline__ bool is_black(Spec s) { return s.r == 0 && s.g == 0 && s.b == 0; }
__device__ __forceinline__ real lum(Spec s) { return 0.212671f * s.r + 0.715160f * s.g + 0.072169f * s.b; }
__device__ __forceinline__ Spec ssqrt(Spec s) { return Spec{xsqrt(s.r), xsqrt(s.g), xsqrt(s.b)}; }

}  // namespace
}  // namespace lts
