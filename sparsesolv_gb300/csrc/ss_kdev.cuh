// ss_kdev.cuh -- device helpers shared by the single-system and the batched
// Krylov kernels: KState scalars as T, and the per-iteration decision.
#pragma once

#include "ss_krylov.cuh"

namespace ssg {

// the FP64 type of the Krylov scalars for vectors of type T
template <typename T>
struct Wide {
    using type = T;
};
template <>
struct Wide<float> {
    using type = double;
};
template <>
struct Wide<cplxf> {
    using type = cplx;
};

// scalars of KState as T
template <typename T>
__device__ __forceinline__ T getS(const double *a);
template <>
__device__ __forceinline__ double getS<double>(const double *a) { return a[0]; }
template <>
__device__ __forceinline__ cplx getS<cplx>(const double *a) { return {a[0], a[1]}; }
template <>
__device__ __forceinline__ float getS<float>(const double *a) { return (float)a[0]; }
template <>
__device__ __forceinline__ cplxf getS<cplxf>(const double *a) { return {(float)a[0], (float)a[1]}; }
template <typename T>
__device__ __forceinline__ void putS(double *a, T v);
template <>
__device__ __forceinline__ void putS<double>(double *a, double v) { a[0] = v; a[1] = 0.0; }
template <>
__device__ __forceinline__ void putS<cplx>(double *a, cplx v) { a[0] = v.x; a[1] = v.y; }
template <>
__device__ __forceinline__ void putS<float>(double *a, float v) { a[0] = v; a[1] = 0.0; }
template <>
__device__ __forceinline__ void putS<cplxf>(double *a, cplxf v) { a[0] = v.x; a[1] = v.y; }
template <typename T>
__device__ __forceinline__ void acc_parts(double *acc, T v);
template <>
__device__ __forceinline__ void acc_parts<double>(double *acc, double v) { acc[0] += v; }
template <>
__device__ __forceinline__ void acc_parts<cplx>(double *acc, cplx v) { acc[0] += v.x; acc[1] += v.y; }
template <>
__device__ __forceinline__ void acc_parts<float>(double *acc, float v) { acc[0] += (double)v; }
template <>
__device__ __forceinline__ void acc_parts<cplxf>(double *acc, cplxf v) { acc[0] += (double)v.x; acc[1] += (double)v.y; }
template <typename T>
constexpr int nparts() { return Sc<T>::is_complex ? 2 : 1; }

// convergence test, best tracking and divergence judge of one iteration
// (src/MatSolverICCG.cpp:267-305; identical in the MRTR loops)
__device__ __forceinline__ void decide(KState *st, double pure, double *log) {
    const double normR = pure / st->normalizer;
    const int it = st->it + 1;
    st->it = it;
    st->last_norm = pure;
    if (st->log_enabled) log[it] = normR;
    st->improved = 0;
    if (normR < st->conv_cri || pure < st->abs_conv_cri) {
        st->status = ST_CONVERGED;
        st->active = 0;
        return;
    }
    if (normR < st->best) {
        st->best = normR;
        st->improved = 1;
    }
    if (st->diverge_type == 1) {
        if (normR < st->best * st->bad_div_val) st->bad_counter = 0;
        if (normR >= st->best * st->bad_div_val) st->bad_counter++;
        if (st->bad_counter >= st->bad_div_count_thres) {
            st->status = ST_DIVERGED;
            st->active = 0;
            return;
        }
    }
    if (st->stall_limit > 0) {
        if (normR < 0.99 * st->stall_best) {
            st->stall_best = normR;
            st->stall = 0;
        } else if (++st->stall >= st->stall_limit) {
            st->status = ST_MAXIT;
            st->active = 0;
            return;
        }
    }
    if (it >= st->max_ite) {
        st->status = ST_MAXIT;
        st->active = 0;
    }
}

}  // namespace ssg
