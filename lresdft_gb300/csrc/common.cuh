// Shared device helpers for the LRes window solve (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

namespace lres {

// ---------------------------------------------------------------------------
// element traits: real double (inertia / Cholesky), complex double, complex float
// ---------------------------------------------------------------------------
template <class T> struct El;

template <> struct El<double> {
    using R = double;
    static constexpr bool complex = false;
    __device__ __forceinline__ static double zero() { return 0.0; }
    __device__ __forceinline__ static double from(double x) { return x; }
    __device__ __forceinline__ static double mul(double a, double b) { return a * b; }
    __device__ __forceinline__ static double fma(double a, double b, double c) { return ::fma(a, b, c); }
    __device__ __forceinline__ static double fms(double a, double b, double c) { return ::fma(-a, b, c); }   // c - a*b
    __device__ __forceinline__ static double sub(double a, double b) { return a - b; }
    __device__ __forceinline__ static double add(double a, double b) { return a + b; }
    __device__ __forceinline__ static double inv(double a) { return 1.0 / a; }
    __device__ __forceinline__ static double scale(double a, double s) { return a * s; }
    __device__ __forceinline__ static double re(double a) { return a; }
    __device__ __forceinline__ static double mag2(double a) { return a * a; }
    __device__ __forceinline__ static double shift_minus(double z, double b, double c) { return ::fma(z, b, -c); } // z*b - c
    __device__ __forceinline__ static double csqrt(double a) { return sqrt(fabs(a)); }   // unused for real pivots
};

template <> struct El<double2> {
    using R = double;
    static constexpr bool complex = true;
    __device__ __forceinline__ static double2 zero() { return make_double2(0.0, 0.0); }
    __device__ __forceinline__ static double2 from(double x) { return make_double2(x, 0.0); }
    __device__ __forceinline__ static double2 mul(double2 a, double2 b) {
        return make_double2(::fma(a.x, b.x, -a.y * b.y), ::fma(a.x, b.y, a.y * b.x));
    }
    __device__ __forceinline__ static double2 fma(double2 a, double2 b, double2 c) {   // c + a*b
        c.x = ::fma(a.x, b.x, c.x); c.x = ::fma(-a.y, b.y, c.x);
        c.y = ::fma(a.x, b.y, c.y); c.y = ::fma(a.y, b.x, c.y);
        return c;
    }
    __device__ __forceinline__ static double2 fms(double2 a, double2 b, double2 c) {   // c - a*b
        c.x = ::fma(-a.x, b.x, c.x); c.x = ::fma(a.y, b.y, c.x);
        c.y = ::fma(-a.x, b.y, c.y); c.y = ::fma(-a.y, b.x, c.y);
        return c;
    }
    __device__ __forceinline__ static double2 sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
    __device__ __forceinline__ static double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
    __device__ __forceinline__ static double2 inv(double2 a) {
        // 1/a with one rescaling to keep |a|^2 in range
        double s = fmax(fabs(a.x), fabs(a.y));
        double ax = a.x / s, ay = a.y / s;
        double d = ax * ax + ay * ay;
        return make_double2(ax / (d * s), -ay / (d * s));
    }
    __device__ __forceinline__ static double2 scale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
    __device__ __forceinline__ static double re(double2 a) { return a.x; }
    __device__ __forceinline__ static double mag2(double2 a) { return a.x * a.x + a.y * a.y; }
    __device__ __forceinline__ static double2 shift_minus(double2 z, double b, double c) {
        return make_double2(::fma(z.x, b, -c), z.y * b);
    }
    // principal square root: sqrt(z) = (sqrt((|z|+x)/2), sign(y) sqrt((|z|-x)/2))
    __device__ __forceinline__ static double2 csqrt(double2 a) {
        const double r = hypot(a.x, a.y);
        double re = sqrt(0.5 * (r + fabs(a.x)));
        double im = (re > 0.0) ? 0.5 * a.y / re : 0.0;
        if (a.x < 0.0) {
            const double t = re;
            re = fabs(im);
            im = copysign(t, a.y);
        }
        return make_double2(re, im);
    }
};

template <> struct El<float2> {
    using R = float;
    static constexpr bool complex = true;
    __device__ __forceinline__ static float2 zero() { return make_float2(0.f, 0.f); }
    __device__ __forceinline__ static float2 from(float x) { return make_float2(x, 0.f); }
    __device__ __forceinline__ static float2 mul(float2 a, float2 b) {
        return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
    }
    __device__ __forceinline__ static float2 fma(float2 a, float2 b, float2 c) {
        c.x = fmaf(a.x, b.x, c.x); c.x = fmaf(-a.y, b.y, c.x);
        c.y = fmaf(a.x, b.y, c.y); c.y = fmaf(a.y, b.x, c.y);
        return c;
    }
    __device__ __forceinline__ static float2 fms(float2 a, float2 b, float2 c) {
        c.x = fmaf(-a.x, b.x, c.x); c.x = fmaf(a.y, b.y, c.x);
        c.y = fmaf(-a.x, b.y, c.y); c.y = fmaf(-a.y, b.x, c.y);
        return c;
    }
    __device__ __forceinline__ static float2 sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
    __device__ __forceinline__ static float2 add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
    __device__ __forceinline__ static float2 inv(float2 a) {
        float s = fmaxf(fabsf(a.x), fabsf(a.y));
        float ax = a.x / s, ay = a.y / s;
        float d = ax * ax + ay * ay;
        return make_float2(ax / (d * s), -ay / (d * s));
    }
    __device__ __forceinline__ static float2 scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
    __device__ __forceinline__ static float re(float2 a) { return a.x; }
    __device__ __forceinline__ static float mag2(float2 a) { return a.x * a.x + a.y * a.y; }
    __device__ __forceinline__ static float2 shift_minus(float2 z, float b, float c) {
        return make_float2(fmaf(z.x, b, -c), z.y * b);
    }
    __device__ __forceinline__ static float2 csqrt(float2 a) {
        const float r = hypotf(a.x, a.y);
        float re = sqrtf(0.5f * (r + fabsf(a.x)));
        float im = (re > 0.f) ? 0.5f * a.y / re : 0.f;
        if (a.x < 0.f) {
            const float t = re;
            re = fabsf(im);
            im = copysignf(t, a.y);
        }
        return make_float2(re, im);
    }
};

// status bits reported by the window kernels (OR-ed into one device word)
enum : int {
    ST_ZERO_PIVOT = 1,      // a pivot was zero or not finite
    ST_BAD_SHAPE = 2,       // a work item exceeded the launch's size limits
    ST_TIMEOUT = 4,         // a bounded wait on a tensor-core completion barrier ran out
};

}  // namespace lres

#define LRES_CUDA_TRY(expr)                                                          \
    do {                                                                             \
        cudaError_t _e = (expr);                                                     \
        if (_e != cudaSuccess) {                                                     \
            ::lres_set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr,             \
                             cudaGetErrorString(_e));                                \
            return LRES_ECUDA;                                                       \
        }                                                                            \
    } while (0)

extern "C" void lres_set_error(const char* fmt, ...);
