// ss_spmv_vec.cu -- CSR SpMV and the fused vector / reduction kernels of the
// Krylov iterations, with the scalar recurrences evaluated on the device.
//
// SpMV restates Eigen's row-major sparse * dense product used at
// src/MatSolverICCG.cpp:259 and src/MatSolverMRTR_ICver.cpp:272: y_i is the
// sum over the stored entries of row i. G lanes share a row (G from the mean
// row length), consecutive groups take consecutive rows, so a warp streams a
// contiguous stretch of the value and column arrays.
#include <algorithm>
#include <vector>

#include "ss_internal.cuh"
#include "ss_krylov.cuh"
#include "ss_kdev.cuh"

namespace ssg {

constexpr int RED_T = 256;
constexpr int RED_MAXGRID = 2048;

int red_grid(int n) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const int want = div_up(n, RED_T * 4);
    const int cap = sms * 4 < RED_MAXGRID ? sms * 4 : RED_MAXGRID;
    return want < 1 ? 1 : (want < cap ? want : cap);
}

__host__ __device__ static unsigned *part_counter(double *part) { return (unsigned *)(part + RED_MAXGRID * 8); }

// Block-reduce K doubles, then the last block to arrive reduces all partials
// (fixed order) and returns true in every thread of that block with tot[] set.
template <int K>
__device__ bool grid_reduce(double (&v)[K], double *part, unsigned *counter, double (&tot)[K]) {
    __shared__ double sh[K][RED_T / 32];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double w = warp_sum_d(v[k]);
        if (lane == 0) sh[k][wid] = w;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double w = lane < RED_T / 32 ? sh[k][lane] : 0.0;
            w = warp_sum_d(w);
            if (lane == 0) part[blockIdx.x * K + k] = w;
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double a[K];
#pragma unroll
    for (int k = 0; k < K; ++k) a[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += RED_T)
#pragma unroll
        for (int k = 0; k < K; ++k) a[k] += __ldcg(part + b * K + k);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double w = warp_sum_d(a[k]);
        if (lane == 0) sh[k][wid] = w;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double w = lane < RED_T / 32 ? sh[k][lane] : 0.0;
            w = warp_sum_d(w);
            if (lane == 0) sh[k][0] = w;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) tot[k] = sh[k][0];
    if (threadIdx.x == 0) *counter = 0;
    return true;
}

// ---------------------------------------------------------------- SpMV
template <typename T, int G, bool DOT>
__global__ void __launch_bounds__(RED_T) k_spmv(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                                const T *__restrict__ val, const T *__restrict__ x, T *__restrict__ y,
                                                KState *st, double *part) {
    if (st && !st->active) return;
    constexpr int RPB = RED_T / G;
    const int g = threadIdx.x / G, gl = threadIdx.x % G;
    double acc2[2] = {0.0, 0.0};
    for (int row0 = blockIdx.x * RPB; row0 < n; row0 += gridDim.x * RPB) {
        const int row = row0 + g;
        T acc = Sc<T>::zero();
        if (row < n) {
            const int a = rp[row], e = rp[row + 1];
            for (int k = a + gl; k < e; k += G) acc = madd(acc, val[k], x[ci[k]]);
        }
#pragma unroll
        for (int m = G / 2; m >= 1; m >>= 1) acc = acc + Sc<T>::shfl_xor(acc, m);
        if (row < n && gl == 0) {
            y[row] = acc;
            if (DOT) acc_parts<T>(acc2, x[row] * acc);
        }
    }
    if (DOT) {
        double v[2] = {acc2[0], acc2[1]}, tot[2];
        if (grid_reduce<2>(v, part, &st->red_count, tot)) {
            if (threadIdx.x == 0) {
                T temp2;
                if (Sc<T>::is_complex) temp2 = getS<T>(tot);
                else temp2 = getS<T>(tot);
                st->dots[0] = tot[0];
                st->dots[1] = tot[1];
                putS<T>(st->alpha, getS<T>(st->rur0) / temp2);
            }
        }
    }
}

// Lanes a row from the row-length distribution: the length at which half of the
// nonzeros lie in rows of that length or shorter (the rows that carry the work),
// divided by about 8 real (16 complex) entries a lane. GB300 issues few FP64
// operations per clock, and every lane pays the butterfly adds and the padding of
// its last step, while fewer lanes read the values and columns less coalesced;
// measured on the 33-entry rows of the voxel systems: 2 lanes 191 us, 4 lanes
// 173 us, 8 lanes 233 us, 16 lanes 411 us (80^3, real); 2 lanes 173 us, 4 lanes
// 195 us, 8 lanes 240 us (60^3, complex).
int spmv_group(double rowlen, bool cplx) {
    const double lanes = rowlen / (cplx ? 16.0 : 8.0);
    int g = 2;
    while (g < 32 && 1.5 * g < lanes) g *= 2;
    return g;
}

// the nonzero-weighted median row length of a CSR pattern (host row pointers)
double spmv_rowlen(int n, const int *rp) {
    if (n <= 0 || rp[n] <= 0) return 0.0;
    int mx = 0;
    for (int i = 0; i < n; ++i) mx = std::max(mx, rp[i + 1] - rp[i]);
    std::vector<long long> w((size_t)mx + 1, 0);
    for (int i = 0; i < n; ++i) w[rp[i + 1] - rp[i]] += rp[i + 1] - rp[i];
    long long acc = 0;
    for (int len = 0; len <= mx; ++len)
        if ((acc += w[len]) * 2 >= (long long)rp[n]) return (double)len;
    return (double)mx;
}

template <typename T, int G>
static void spmv_launch_g(int n, const int *rp, const int *ci, const T *val, const T *x, T *y, KState *st,
                          bool dot_alpha, double *part, cudaStream_t s) {
    const int rows_per_block = RED_T / G;
    int grid = div_up(n, rows_per_block);
    if (dot_alpha) {
        const int cap = red_grid(n) * 8;  // bounded partial count for the fused reduction
        grid = grid < cap ? grid : cap;
        if (grid > RED_MAXGRID) grid = RED_MAXGRID;
        k_spmv<T, G, true><<<grid, RED_T, 0, s>>>(n, rp, ci, val, x, y, st, part);
    } else {
        const int cap = 65535 * 16;
        grid = grid < cap ? grid : cap;
        k_spmv<T, G, false><<<grid, RED_T, 0, s>>>(n, rp, ci, val, x, y, st, part);
    }
    SSG_LAUNCHED();
}

template <typename T>
void k_spmv_launch(int n, int group, const int *rp, const int *ci, const T *val, const T *x, T *y, KState *st,
                   bool dot_alpha, double *part, cudaStream_t s) {
    if (n == 0) return;
    switch (group) {
        case 2: spmv_launch_g<T, 2>(n, rp, ci, val, x, y, st, dot_alpha, part, s); break;
        case 4: spmv_launch_g<T, 4>(n, rp, ci, val, x, y, st, dot_alpha, part, s); break;
        case 16: spmv_launch_g<T, 16>(n, rp, ci, val, x, y, st, dot_alpha, part, s); break;
        case 32: spmv_launch_g<T, 32>(n, rp, ci, val, x, y, st, dot_alpha, part, s); break;
        default: spmv_launch_g<T, 8>(n, rp, ci, val, x, y, st, dot_alpha, part, s); break;
    }
}

// ---------------------------------------------------------------- ICCG steps
template <typename T>
__global__ void __launch_bounds__(RED_T) k_iccg_update(int n, KState *st, T *x, T *r, const T *p, const T *ap,
                                                       double *part, double *log) {
    if (!st->active) return;
    const T alpha = getS<T>(st->alpha);
    double acc[1] = {0.0}, tot[1];
    for (int i = blockIdx.x * RED_T + threadIdx.x; i < n; i += gridDim.x * RED_T) {
        x[i] = x[i] + alpha * p[i];
        const T ri = r[i] - alpha * ap[i];
        r[i] = ri;
        acc[0] += Sc<T>::abs2(ri);
    }
    if (grid_reduce<1>(acc, part, &st->red_count, tot) && threadIdx.x == 0) decide(st, sqrt(tot[0]), log);
}

template <typename T>
__global__ void __launch_bounds__(RED_T) k_iccg_beta(int n, KState *st, const T *r, const T *z, double *part) {
    if (!st->active) return;
    double acc[2] = {0.0, 0.0}, tot[2];
    for (int i = blockIdx.x * RED_T + threadIdx.x; i < n; i += gridDim.x * RED_T) acc_parts<T>(acc, r[i] * z[i]);
    if (grid_reduce<2>(acc, part, &st->red_count, tot) && threadIdx.x == 0) {
        const T rur1 = getS<T>(tot);
        const T beta = rur1 / getS<T>(st->rur0);
        putS<T>(st->beta, beta);
        putS<T>(st->rur0, rur1);
    }
}

template <typename T>
__global__ void k_iccg_p(int n, const KState *st, T *p, const T *z) {
    if (!st->active) return;
    const T beta = getS<T>(st->beta);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = p[i] * beta + z[i];
}

// ---------------------------------------------------------------- MRTR steps
template <typename T>
__global__ void __launch_bounds__(RED_T) k_mrtr_dots(int n, KState *st, const T *a, const T *b, const T *c,
                                                     const T *y, double *part) {
    if (!st->active) return;
    double acc[6] = {0, 0, 0, 0, 0, 0}, tot[6];
    for (int i = blockIdx.x * RED_T + threadIdx.x; i < n; i += gridDim.x * RED_T) {
        const T ai = a[i];
        acc_parts<T>(acc + 0, ai * b[i]);
        acc_parts<T>(acc + 2, c[i] * ai);
        acc_parts<T>(acc + 4, ai * y[i]);
    }
    if (grid_reduce<6>(acc, part, &st->red_count, tot) && threadIdx.x == 0) {
        const T wr = getS<T>(tot + 0), vw = getS<T>(tot + 2), wy = getS<T>(tot + 4);
        for (int k = 0; k < 6; ++k) st->dots[k] = tot[k];
        T zeta, eta, nu = getS<T>(st->nu), zeta_old = getS<T>(st->zeta_old);
        if (st->it == 0) {
            zeta = wr / vw;
            zeta_old = zeta;
            eta = Sc<T>::zero();
        } else {
            const T temp0 = Sc<T>::one() / (nu * vw - wy * wy);
            zeta = nu * wr * temp0;
            eta = (-1.0 * wy) * wr * temp0;
        }
        nu = zeta * wr;
        const T ptemp = eta * zeta_old / zeta;
        zeta_old = zeta;
        putS<T>(st->zeta, zeta);
        putS<T>(st->eta, eta);
        putS<T>(st->nu, nu);
        putS<T>(st->ptemp, ptemp);
        putS<T>(st->zeta_old, zeta_old);
    }
}

template <typename T, bool QUIRK>
__global__ void __launch_bounds__(RED_T) k_mrtr_update(int n, KState *st, T *p, const T *u, T *x, T *y, const T *v,
                                                       T *r, double *part, double *log) {
    if (!st->active) return;
    const T zeta = getS<T>(st->zeta), eta = getS<T>(st->eta), pt = getS<T>(st->ptemp);
    double acc[1] = {0.0}, tot[1];
    for (int i = blockIdx.x * RED_T + threadIdx.x; i < n; i += gridDim.x * RED_T) {
        const T ui = u[i];
        // the reference's IC-MRTR sets p = u; p += t p, i.e. p = (1 + t) u
        const T pi = QUIRK ? (ui + pt * ui) : (p[i] * pt + ui);
        p[i] = pi;
        x[i] = x[i] + zeta * pi;
        const T yi = y[i] * eta + zeta * v[i];
        y[i] = yi;
        const T ri = r[i] - yi;
        r[i] = ri;
        acc[0] += Sc<T>::abs2(ri);
    }
    if (grid_reduce<1>(acc, part, &st->red_count, tot) && threadIdx.x == 0) decide(st, sqrt(tot[0]), log);
}

template <typename T>
__global__ void k_mrtr_zu(int n, const KState *st, T *z, const T *w, T *u) {
    if (!st->active) return;
    const T zeta = getS<T>(st->zeta), eta = getS<T>(st->eta);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const T zi = z[i] * eta + zeta * w[i];
        z[i] = zi;
        u[i] = u[i] - zi;
    }
}

template <typename T>
__global__ void k_copy_if_improved(int n, const KState *st, const T *x, T *best) {
    if (!st->improved) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) best[i] = x[i];
}

// ---------------------------------------------------------------- plain helpers
template <typename T>
__global__ void k_vec_sub(int n, const T *a, const T *b, T *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = a[i] - b[i];
}
template <typename T>
__global__ void k_vec_neg(int n, const T *a, T *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = -1.0 * a[i];
}
template <typename T>
__global__ void k_vec_mul(int n, T *x, const T *d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = x[i] * d[i];
}
template <typename T>
__global__ void k_vec_div(int n, T *x, const T *d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = x[i] / d[i];
}
template <typename T>
__global__ void __launch_bounds__(RED_T) k_norm2(int n, const T *a, double *out, double *part) {
    double acc[1] = {0.0}, tot[1];
    for (int i = blockIdx.x * RED_T + threadIdx.x; i < n; i += gridDim.x * RED_T) acc[0] += Sc<T>::abs2(a[i]);
    if (grid_reduce<1>(acc, part, part_counter(part), tot) && threadIdx.x == 0) *out = sqrt(tot[0]);
}
template <typename T>
__global__ void __launch_bounds__(RED_T) k_dot_into(int n, const T *a, const T *b, double *out2, double *part) {
    double acc[2] = {0.0, 0.0}, tot[2];
    for (int i = blockIdx.x * RED_T + threadIdx.x; i < n; i += gridDim.x * RED_T) acc_parts<T>(acc, a[i] * b[i]);
    if (grid_reduce<2>(acc, part, part_counter(part), tot) && threadIdx.x == 0) {
        out2[0] = tot[0];
        out2[1] = tot[1];
    }
}
template <typename T>
__global__ void k_fill_sentinel(T *p, size_t words, const KState *st) {
    if (st && !st->active) return;
    unsigned long long *q = (unsigned long long *)p;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        q[i] = SENT64;
}

static int ew_grid(int n) {
    const int g = div_up(n, 256);
    return g < 4096 ? (g < 1 ? 1 : g) : 4096;
}

template <typename T>
void iccg_update(int n, KState *st, T *x, T *r, const T *p, const T *ap, double *part, double *log, cudaStream_t s) {
    k_iccg_update<T><<<red_grid(n), RED_T, 0, s>>>(n, st, x, r, p, ap, part, log);
    SSG_LAUNCHED();
}
template <typename T>
void iccg_beta(int n, KState *st, const T *r, const T *z, double *part, cudaStream_t s) {
    k_iccg_beta<T><<<red_grid(n), RED_T, 0, s>>>(n, st, r, z, part);
    SSG_LAUNCHED();
}
template <typename T>
void iccg_p(int n, KState *st, T *p, const T *z, cudaStream_t s) {
    k_iccg_p<T><<<ew_grid(n), 256, 0, s>>>(n, st, p, z);
    SSG_LAUNCHED();
}
template <typename T>
void mrtr_dots(int n, KState *st, const T *a, const T *b, const T *c, const T *y, double *part, cudaStream_t s) {
    k_mrtr_dots<T><<<red_grid(n), RED_T, 0, s>>>(n, st, a, b, c, y, part);
    SSG_LAUNCHED();
}
template <typename T>
void mrtr_update(int n, KState *st, T *p, const T *u, T *x, T *y, const T *v, T *r, double *part, double *log,
                 bool ic_quirk, cudaStream_t s) {
    if (ic_quirk)
        k_mrtr_update<T, true><<<red_grid(n), RED_T, 0, s>>>(n, st, p, u, x, y, v, r, part, log);
    else
        k_mrtr_update<T, false><<<red_grid(n), RED_T, 0, s>>>(n, st, p, u, x, y, v, r, part, log);
    SSG_LAUNCHED();
}
template <typename T>
void mrtr_zu(int n, KState *st, T *z, const T *w, T *u, cudaStream_t s) {
    k_mrtr_zu<T><<<ew_grid(n), 256, 0, s>>>(n, st, z, w, u);
    SSG_LAUNCHED();
}
template <typename T>
void copy_if_improved(int n, const KState *st, const T *x, T *best, cudaStream_t s) {
    k_copy_if_improved<T><<<ew_grid(n), 256, 0, s>>>(n, st, x, best);
    SSG_LAUNCHED();
}
template <typename T>
void vec_sub(int n, const T *a, const T *b, T *out, cudaStream_t s) {
    if (!n) return;
    k_vec_sub<T><<<ew_grid(n), 256, 0, s>>>(n, a, b, out);
    SSG_LAUNCHED();
}
template <typename T>
void vec_neg(int n, const T *a, T *out, cudaStream_t s) {
    if (!n) return;
    k_vec_neg<T><<<ew_grid(n), 256, 0, s>>>(n, a, out);
    SSG_LAUNCHED();
}
template <typename T>
void vec_mul(int n, T *x, const T *d, cudaStream_t s) {
    if (!n) return;
    k_vec_mul<T><<<ew_grid(n), 256, 0, s>>>(n, x, d);
    SSG_LAUNCHED();
}
template <typename T>
void vec_div(int n, T *x, const T *d, cudaStream_t s) {
    if (!n) return;
    k_vec_div<T><<<ew_grid(n), 256, 0, s>>>(n, x, d);
    SSG_LAUNCHED();
}
template <typename T>
void norm2(int n, const T *a, double *out, double *part, cudaStream_t s) {
    k_norm2<T><<<red_grid(n), RED_T, 0, s>>>(n, a, out, part);
    SSG_LAUNCHED();
}
template <typename T>
void dot_into(int n, const T *a, const T *b, double *out2, double *part, cudaStream_t s) {
    k_dot_into<T><<<red_grid(n), RED_T, 0, s>>>(n, a, b, out2, part);
    SSG_LAUNCHED();
}
template <typename T>
void fill_sentinel_st(T *p, int n, const KState *st, cudaStream_t s) {
    const size_t words = (size_t)n * sizeof(T) / 8;
    if (!words) return;
    k_fill_sentinel<T><<<ew_grid((int)(words < (1u << 30) ? words : (1u << 30))), 256, 0, s>>>(p, words, st);
    SSG_LAUNCHED();
}
template <typename T>
void spmv(int n, int group, const int *rp, const int *ci, const T *val, const T *x, T *y, cudaStream_t s) {
    k_spmv_launch<T>(n, group, rp, ci, val, x, y, nullptr, false, nullptr, s);
}

#define SSG_INST(T)                                                                                              \
    template void k_spmv_launch<T>(int, int, const int *, const int *, const T *, const T *, T *, KState *,    \
                                   bool, double *, cudaStream_t);                                                \
    template void spmv<T>(int, int, const int *, const int *, const T *, const T *, T *, cudaStream_t);         \
    template void iccg_update<T>(int, KState *, T *, T *, const T *, const T *, double *, double *,             \
                                 cudaStream_t);                                                                  \
    template void iccg_beta<T>(int, KState *, const T *, const T *, double *, cudaStream_t);                    \
    template void iccg_p<T>(int, KState *, T *, const T *, cudaStream_t);                                       \
    template void mrtr_dots<T>(int, KState *, const T *, const T *, const T *, const T *, double *,             \
                               cudaStream_t);                                                                    \
    template void mrtr_update<T>(int, KState *, T *, const T *, T *, T *, const T *, T *, double *, double *,   \
                                 bool, cudaStream_t);                                                            \
    template void mrtr_zu<T>(int, KState *, T *, const T *, T *, cudaStream_t);                                 \
    template void copy_if_improved<T>(int, const KState *, const T *, T *, cudaStream_t);                       \
    template void vec_sub<T>(int, const T *, const T *, T *, cudaStream_t);                                    \
    template void vec_neg<T>(int, const T *, T *, cudaStream_t);                                                \
    template void vec_mul<T>(int, T *, const T *, cudaStream_t);                                                \
    template void vec_div<T>(int, T *, const T *, cudaStream_t);                                                \
    template void norm2<T>(int, const T *, double *, double *, cudaStream_t);                                   \
    template void dot_into<T>(int, const T *, const T *, double *, double *, cudaStream_t);                     \
    template void fill_sentinel_st<T>(T *, int, const KState *, cudaStream_t);
SSG_INST(double)
SSG_INST(cplx)
#undef SSG_INST

size_t part_bytes() { return sizeof(double) * RED_MAXGRID * 8 + 64; }

}  // namespace ssg
