// ss_common.cuh -- shared types and device helpers of the sm_103a Krylov path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace ssg {

// ---------------------------------------------------------------- scalars
// Complex-symmetric systems use unconjugated bilinear products
// (dot_no_conj, include/SparseSolv/MatSolverBase.hpp:121-122), so only the
// field operations and the modulus are needed.
struct cplx {
    double x, y;
};
struct cplxf {
    float x, y;
};

// Products rounded on their own (no fused multiply-add), so that a sum of two
// products such as a.x*b.x - a.y*b.y gives the same bits in every kernel: with
// contraction the compiler may fuse either product, and picks differently in
// differently shaped loops. This is also the rounding of a CPU without FMA.
__host__ __device__ __forceinline__ double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ __forceinline__ float mul_rn(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

__host__ __device__ __forceinline__ cplx operator+(cplx a, cplx b) { return {a.x + b.x, a.y + b.y}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a, cplx b) { return {a.x - b.x, a.y - b.y}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a) { return {-a.x, -a.y}; }
__host__ __device__ __forceinline__ cplx operator*(cplx a, cplx b) {
    return {mul_rn(a.x, b.x) - mul_rn(a.y, b.y), mul_rn(a.x, b.y) + mul_rn(a.y, b.x)};
}
__host__ __device__ __forceinline__ cplx operator*(double s, cplx a) { return {s * a.x, s * a.y}; }
// Smith's algorithm (R. L. Smith, CACM 5(8), 1962) for robust complex division
__host__ __device__ __forceinline__ cplx operator/(cplx a, cplx b) {
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, d = b.x + b.y * r;
        return {(a.x + a.y * r) / d, (a.y - a.x * r) / d};
    } else {
        const double r = b.x / b.y, d = b.y + b.x * r;
        return {(a.x * r + a.y) / d, (a.y * r - a.x) / d};
    }
}
__host__ __device__ __forceinline__ cplxf operator+(cplxf a, cplxf b) { return {a.x + b.x, a.y + b.y}; }
__host__ __device__ __forceinline__ cplxf operator-(cplxf a, cplxf b) { return {a.x - b.x, a.y - b.y}; }
__host__ __device__ __forceinline__ cplxf operator-(cplxf a) { return {-a.x, -a.y}; }
__host__ __device__ __forceinline__ cplxf operator*(cplxf a, cplxf b) {
    return {mul_rn(a.x, b.x) - mul_rn(a.y, b.y), mul_rn(a.x, b.y) + mul_rn(a.y, b.x)};
}
__host__ __device__ __forceinline__ cplxf operator/(cplxf a, cplxf b) {
    if (fabsf(b.x) >= fabsf(b.y)) {
        const float r = b.y / b.x, d = b.x + b.y * r;
        return {(a.x + a.y * r) / d, (a.y - a.x * r) / d};
    } else {
        const float r = b.x / b.y, d = b.y + b.x * r;
        return {(a.x * r + a.y) / d, (a.y * r - a.x) / d};
    }
}

// acc + a * b for the hot multiply-add loops (SpMV, triangular sweeps), with
// the products fused into the sums in one fixed pattern. Complex: four fused
// multiply-adds, real part a.x*b.x then -a.y*b.y, imaginary part a.x*b.y then
// a.y*b.x -- half the FP64 operations of the separately rounded product plus
// two additions, and the same bits in every kernel that uses it.
__host__ __device__ __forceinline__ double madd(double acc, double a, double b) { return fma(a, b, acc); }
__host__ __device__ __forceinline__ float madd(float acc, float a, float b) { return fmaf(a, b, acc); }
__host__ __device__ __forceinline__ cplx madd(cplx acc, cplx a, cplx b) {
    return {fma(-a.y, b.y, fma(a.x, b.x, acc.x)), fma(a.y, b.x, fma(a.x, b.y, acc.y))};
}
// FP32 complex (the inner solves of mixed precision) keeps the separately rounded
// product: with the fused pattern the inner IC-MRTR on the 60^3 eddy-current
// system needed 1,213 instead of 768 iterations (FP32 pipes are not the bound)
__host__ __device__ __forceinline__ cplxf madd(cplxf acc, cplxf a, cplxf b) { return acc + a * b; }

template <typename T>
struct Sc;

template <>
struct Sc<double> {
    using real = double;
    static constexpr bool is_complex = false;
    __host__ __device__ static double zero() { return 0.0; }
    __host__ __device__ static double one() { return 1.0; }
    __host__ __device__ static double from(double r) { return r; }
    __host__ __device__ static double abs2(double a) { return a * a; }
    __host__ __device__ static double absv(double a) { return fabs(a); }
    __host__ __device__ static double re(double a) { return a; }
    __device__ static double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
    __device__ static double shfl(double v, int l) { return __shfl_sync(0xffffffffu, v, l); }
};
template <>
struct Sc<cplx> {
    using real = double;
    static constexpr bool is_complex = true;
    __host__ __device__ static cplx zero() { return {0.0, 0.0}; }
    __host__ __device__ static cplx one() { return {1.0, 0.0}; }
    __host__ __device__ static cplx from(double r) { return {r, 0.0}; }
    __host__ __device__ static double abs2(cplx a) { return a.x * a.x + a.y * a.y; }
    __host__ __device__ static double absv(cplx a) { return hypot(a.x, a.y); }
    __host__ __device__ static double re(cplx a) { return a.x; }
    __device__ static cplx shfl_xor(cplx v, int m) {
        return {__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m)};
    }
    __device__ static cplx shfl(cplx v, int l) {
        return {__shfl_sync(0xffffffffu, v.x, l), __shfl_sync(0xffffffffu, v.y, l)};
    }
};
template <>
struct Sc<float> {
    using real = float;
    static constexpr bool is_complex = false;
    __host__ __device__ static float zero() { return 0.0f; }
    __host__ __device__ static float one() { return 1.0f; }
    __host__ __device__ static float from(double r) { return (float)r; }
    __host__ __device__ static float abs2(float a) { return a * a; }
    __host__ __device__ static float absv(float a) { return fabsf(a); }
    __host__ __device__ static float re(float a) { return a; }
    __device__ static float shfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
    __device__ static float shfl(float v, int l) { return __shfl_sync(0xffffffffu, v, l); }
};
template <>
struct Sc<cplxf> {
    using real = float;
    static constexpr bool is_complex = true;
    __host__ __device__ static cplxf zero() { return {0.0f, 0.0f}; }
    __host__ __device__ static cplxf one() { return {1.0f, 0.0f}; }
    __host__ __device__ static cplxf from(double r) { return {(float)r, 0.0f}; }
    __host__ __device__ static float abs2(cplxf a) { return a.x * a.x + a.y * a.y; }
    __host__ __device__ static float absv(cplxf a) { return hypotf(a.x, a.y); }
    __host__ __device__ static float re(cplxf a) { return a.x; }
    __device__ static cplxf shfl_xor(cplxf v, int m) {
        return {__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m)};
    }
    __device__ static cplxf shfl(cplxf v, int l) {
        return {__shfl_sync(0xffffffffu, v.x, l), __shfl_sync(0xffffffffu, v.y, l)};
    }
};

// conversions between working precisions
__host__ __device__ __forceinline__ float to_lo(double v) { return (float)v; }
__host__ __device__ __forceinline__ cplxf to_lo(cplx v) { return {(float)v.x, (float)v.y}; }
__host__ __device__ __forceinline__ double to_hi(float v) { return (double)v; }
__host__ __device__ __forceinline__ cplx to_hi(cplxf v) { return {(double)v.x, (double)v.y}; }
template <typename T>
struct Lo;
template <>
struct Lo<double> {
    using type = float;
};
template <>
struct Lo<cplx> {
    using type = cplxf;
};

// ---------------------------------------------------------------- sentinels
// Sync-free sweeps publish each solved entry by overwriting a sentinel NaN
// (all bits set) with its value: a 4- or 8-byte aligned store is single-copy
// atomic, so the value is its own ready flag. Computed NaNs are canonicalised
// to a quiet NaN with a different payload so they can never look unsolved.
constexpr unsigned long long SENT64 = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned int SENT32 = 0xFFFFFFFFu;

__device__ __forceinline__ double ld_vol(const double *p) { return *(const volatile double *)p; }
__device__ __forceinline__ float ld_vol(const float *p) { return *(const volatile float *)p; }
__device__ __forceinline__ bool is_sent(double v) { return (unsigned long long)__double_as_longlong(v) == SENT64; }
__device__ __forceinline__ bool is_sent(float v) { return __float_as_uint(v) == SENT32; }
__device__ __forceinline__ double unsent(double v) { return is_sent(v) ? __longlong_as_double(0x7FF8000000000001ll) : v; }
__device__ __forceinline__ float unsent(float v) { return is_sent(v) ? __uint_as_float(0x7FC00001u) : v; }

__device__ __forceinline__ void st_vol(double *p, double v) { *(volatile double *)p = v; }
__device__ __forceinline__ void st_vol(float *p, float v) { *(volatile float *)p = v; }

// ---------------------------------------------------------------- status
// Device-side error word shared by the kernels of one handle.
enum : int {
    ERR_NONE = 0,
    ERR_TIMEOUT = 1,   // a bounded spin gave up
    ERR_NO_DIAG = 2,   // a row of the lower triangle lacks its diagonal
    ERR_ROW_TOO_LONG = 3,  // a factor row exceeds the per-warp register budget
    ERR_PATTERN = 4,   // a caller-given row has a column out of range or columns not ascending
};

// Spin bound: a wait gives up after this many nanoseconds of %globaltimer.
// The int after an error word holds the owner's limit in microseconds
// (SSG_TUNE_SPIN_LIMIT_US); zero, as in freshly cleared scratch, means the
// default of 4 s.
constexpr unsigned long long SPIN_LIMIT_NS = 4000000000ull;  // 4 s
__device__ __forceinline__ unsigned long long spin_limit_ns(const int *err) {
    const int us = ((const volatile int *)err)[1];
    return us > 0 ? 1000ull * (unsigned long long)us : SPIN_LIMIT_NS;
}

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// xor-shuffle within a group of G lanes using only the group's own lanes:
// groups of one warp may wait on each other (a row of one group depending on
// a row of another), so a full-warp mask could tie them together
__device__ __forceinline__ unsigned group_mask(int G) {
    return G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
}
__device__ __forceinline__ double gshfl_xor(double v, int m, unsigned mask) { return __shfl_xor_sync(mask, v, m); }
__device__ __forceinline__ float gshfl_xor(float v, int m, unsigned mask) { return __shfl_xor_sync(mask, v, m); }
__device__ __forceinline__ cplx gshfl_xor(cplx v, int m, unsigned mask) {
    return {__shfl_xor_sync(mask, v.x, m), __shfl_xor_sync(mask, v.y, m)};
}
__device__ __forceinline__ cplxf gshfl_xor(cplxf v, int m, unsigned mask) {
    return {__shfl_xor_sync(mask, v.x, m), __shfl_xor_sync(mask, v.y, m)};
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v = v + Sc<T>::shfl_xor(v, m);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace ssg
