/*
 * sparsesolv_oracle.c -- CPU oracle for the SparseSolv Krylov hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * algorithms (shifted IC(0), ICCG/ICCOCG, IC-MRTR, Eisenstat SGS-MRTR, the
 * diagonal scaling and the alpha search), used by the tests as the checker and
 * by bench.py as the timed CPU baseline. Nothing in the product links or calls
 * it. Parity of this restatement is pinned against the reference itself: the
 * recipe in oracle/Makefile compiles the reference's own sources into
 * oracle/_ref/ and tests/test_oracle_vs_reference.py compares the two on the
 * same systems; tests/golden/ holds residual logs and solutions the reference
 * produced, made by tests/golden/make_golden.py.
 *
 * Also here: the host recomputation of the integer work the GPU does
 * (lower/upper patterns, transpose, level sets and level permutation).
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fPIC -shared (no FMA contraction,
 * so x86-64 and aarch64 builds round identically).
 */
#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* host threads the row-parallel SpMV uses (1 without OpenMP) */
int or_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* threads of the row-parallel SpMV for the following solves (no effect without OpenMP) */
void or_set_threads(int k) {
#ifdef _OPENMP
    if (k > 0) omp_set_num_threads(k);
#else
    (void)k;
#endif
}

/* wall time of the last or_solve call: [0] set-up before the iterations (scaling,
 * lower triangle, IC factor, transpose), [1] the iterations, [2] the whole call */
static double or_timing[3];
static double or_now(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}
void or_last_timings(double *out) {
    for (int k = 0; k < 3; ++k) out[k] = or_timing[k];
}

typedef struct {
    int n;
    int *rp;  /* n+1 */
    int *ci;  /* nnz */
    int *src; /* entry k of this matrix comes from entry src[k] of its source (or NULL) */
} or_csr;

/* solver settings: MatSolverBase.hpp:58-90 (defaults MatSolverBase.cpp:32-47),
 * MatSolverICCG.hpp:40 (alpha), MatSolverMRTR.hpp:40-43 (alpha, precondition type) */
typedef struct {
    int is_init;
    int is_diag_scale;
    int is_save_best;
    int is_save_residual_log;
    int diverge_judge_type;
    double bad_div_val;
    int bad_div_count_thres;
    int conv_normalize_type;
    double conv_normalize_const;
    double accel_factor;
    int precondition_type;
    int mrtr_reference_quirks;
} or_opts;

void or_free(or_csr *M) {
    free(M->rp);
    free(M->ci);
    free(M->src);
    M->rp = M->ci = M->src = NULL;
}

/* setNormalizer, src/MatSolverBase.cpp:72-87 */
static double or_normalizer(const or_opts *o, double normB, double pure_normR) {
    if (o->conv_normalize_type == 0) return normB;
    if (o->conv_normalize_type == 1) return pure_normR;
    if (o->conv_normalize_type == 2) return o->conv_normalize_const;
    return normB;
}

/* entries with col <= row (keep_lower) or col >= row, explicit zeros kept:
 * SprsTrans::MatLower / MatUpper, src/SprsTrans.cpp:372-394 */
static int or_triangle(const or_csr *A, or_csr *T, int keep_lower) {
    const int n = A->n;
    T->n = n;
    T->rp = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    int cnt = 0;
    for (int i = 0; i < n; ++i)
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k)
            if (keep_lower ? A->ci[k] <= i : A->ci[k] >= i) ++cnt;
    T->ci = (int *)malloc(sizeof(int) * (size_t)(cnt + 1));
    T->src = (int *)malloc(sizeof(int) * (size_t)(cnt + 1));
    if (!T->rp || !T->ci || !T->src) { or_free(T); return -1; }
    cnt = 0;
    for (int i = 0; i < n; ++i) {
        T->rp[i] = cnt;
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k)
            if (keep_lower ? A->ci[k] <= i : A->ci[k] >= i) {
                T->ci[cnt] = A->ci[k];
                T->src[cnt] = k;
                ++cnt;
            }
    }
    T->rp[n] = cnt;
    return 0;
}

int or_lower(const or_csr *A, or_csr *L) { return or_triangle(A, L, 1); }
int or_upper(const or_csr *A, or_csr *U) { return or_triangle(A, U, 0); }

/* CSR transpose with sorted columns: SprsTrans::trans, src/SprsTrans.cpp:312-319 */
int or_transpose(const or_csr *A, or_csr *T) {
    const int n = A->n;
    const int nnz = A->rp[n];
    T->n = n;
    T->rp = (int *)calloc((size_t)(n + 1), sizeof(int));
    T->ci = (int *)malloc(sizeof(int) * (size_t)(nnz + 1));
    T->src = (int *)malloc(sizeof(int) * (size_t)(nnz + 1));
    int *fill = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    if (!T->rp || !T->ci || !T->src || !fill) { or_free(T); free(fill); return -1; }
    for (int k = 0; k < nnz; ++k) T->rp[A->ci[k] + 1]++;
    for (int i = 0; i < n; ++i) T->rp[i + 1] += T->rp[i];
    memcpy(fill, T->rp, sizeof(int) * (size_t)(n + 1));
    for (int i = 0; i < n; ++i)
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k) {
            const int pos = fill[A->ci[k]]++;
            T->ci[pos] = i;
            T->src[pos] = k;
        }
    free(fill);
    return 0;
}

/* out[k] = in[M->src[k]] for elements of size sz */
void or_gather_values(const or_csr *M, const void *in, size_t sz, void *out) {
    const int nnz = M->rp[M->n];
    for (int k = 0; k < nnz; ++k)
        memcpy((char *)out + (size_t)k * sz, (const char *)in + (size_t)M->src[k] * sz, sz);
}
#define or_permute_values or_gather_values

/* ---------------------------------------------------------------------- */
/* level schedule (host recomputation of the GPU's integer work)           */
/* ---------------------------------------------------------------------- */

/*
 * Level of row i in the forward (lower = 1) or backward (lower = 0) sweep:
 *   forward : level(i) = 1 + max{level(j) : j < i, a_ij stored}, 0 if none
 *   backward: level(i) = 1 + max{level(j) : j > i, a_ij stored}, 0 if none
 * perm lists rows by (level, row id); lptr[l] is the first position of level l.
 * Returns the number of levels, or -1.
 */
int or_levels(int n, const int *rp, const int *ci, int lower, int *level, int *perm, int *lptr) {
    int nlev = 0;
    if (lower) {
        for (int i = 0; i < n; ++i) {
            int l = 0;
            for (int k = rp[i]; k < rp[i + 1]; ++k)
                if (ci[k] < i && level[ci[k]] + 1 > l) l = level[ci[k]] + 1;
            level[i] = l;
            if (l + 1 > nlev) nlev = l + 1;
        }
    } else {
        for (int i = n; i-- > 0;) {
            int l = 0;
            for (int k = rp[i]; k < rp[i + 1]; ++k)
                if (ci[k] > i && level[ci[k]] + 1 > l) l = level[ci[k]] + 1;
            level[i] = l;
            if (l + 1 > nlev) nlev = l + 1;
        }
    }
    if (lptr) {
        memset(lptr, 0, sizeof(int) * (size_t)(nlev + 1));
        for (int i = 0; i < n; ++i) lptr[level[i] + 1]++;
        for (int l = 0; l < nlev; ++l) lptr[l + 1] += lptr[l];
        if (perm) {
            int *fill = (int *)malloc(sizeof(int) * (size_t)(nlev + 1));
            if (!fill) return -1;
            memcpy(fill, lptr, sizeof(int) * (size_t)(nlev + 1));
            for (int i = 0; i < n; ++i) perm[fill[level[i]]++] = i;
            free(fill);
        }
    }
    return nlev;
}

/* lower/upper pattern with source map, exported for pattern tests */
int or_triangle_pattern(int n, const int *rp, const int *ci, int keep_lower, int *trp, int *tci, int *tsrc) {
    or_csr A = {n, (int *)rp, (int *)ci, NULL}, T;
    if (or_triangle(&A, &T, keep_lower)) return -1;
    memcpy(trp, T.rp, sizeof(int) * (size_t)(n + 1));
    memcpy(tci, T.ci, sizeof(int) * (size_t)T.rp[n]);
    if (tsrc) memcpy(tsrc, T.src, sizeof(int) * (size_t)T.rp[n]);
    or_free(&T);
    return 0;
}

int or_transpose_pattern(int n, const int *rp, const int *ci, int *trp, int *tci, int *tsrc) {
    or_csr A = {n, (int *)rp, (int *)ci, NULL}, T;
    if (or_transpose(&A, &T)) return -1;
    memcpy(trp, T.rp, sizeof(int) * (size_t)(n + 1));
    memcpy(tci, T.ci, sizeof(int) * (size_t)T.rp[n]);
    if (tsrc) memcpy(tsrc, T.src, sizeof(int) * (size_t)T.rp[n]);
    or_free(&T);
    return 0;
}

/* ---------------------------------------------------------------------- */
/* the two scalar instantiations                                            */
/* ---------------------------------------------------------------------- */
#define T double
#define SFX _d
#define TABS(x) fabs(x)
#define TABS2(x) ((x) * (x))
#define TPOS(x) ((x) > 0)
#define IS_COMPLEX 0
#include "oracle_impl.h"
#undef T
#undef SFX
#undef TABS
#undef TABS2
#undef TPOS
#undef IS_COMPLEX

#define T double _Complex
#define SFX _z
#define TABS(x) cabs(x)
#define TABS2(x) (creal(x) * creal(x) + cimag(x) * cimag(x))
#define TPOS(x) (creal(x) > 0)
#define IS_COMPLEX 1
#include "oracle_impl.h"
