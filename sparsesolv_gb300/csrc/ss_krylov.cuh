// ss_krylov.cuh -- device-resident Krylov state.
//
// The scalar recurrences, the convergence test, the divergence judge and the
// best-residual tracking of the reference's solve_main loops
// (src/MatSolverICCG.cpp:257-318, src/MatSolverMRTR_ICver.cpp:270-360,
// src/MatSolverMRTR_SGSver.cpp:182-269) run on the GPU in FP64, in the last
// block of the fused reduction kernels. Every kernel of an iteration first
// reads `active` and returns when the solve has ended, so the host can queue
// (or replay as a CUDA graph) whole chunks of iterations and only look at the
// state between chunks.
#pragma once

#include "ss_common.cuh"

namespace ssg {

enum : int { ST_RUNNING = 0, ST_CONVERGED = 1, ST_MAXIT = 2, ST_DIVERGED = 3 };

enum : int { KM_ICCG = 0, KM_MRTR_IC = 1, KM_MRTR_SGS = 2 };

struct KState {
    // control
    int active;
    int status;
    int it;           // completed iterations
    int max_ite;
    int bad_counter;
    int improved;     // this iteration lowered the best residual (save-best copy pending)
    int diverge_type;
    int bad_div_count_thres;
    int log_enabled;
    int quirks;       // reproduce the reference's IC-MRTR p update
    unsigned int red_count;  // last-block ticket of the fused reductions
    int log_len;             // batched solves: residual-log entries, -1 for it + 1
    double conv_cri, abs_conv_cri, normalizer, best, bad_div_val;
    double last_norm;        // |r| of the latest iteration
    // scalars; complex values use [0] = re, [1] = im
    double rur0[2], alpha[2], beta[2];
    double zeta[2], zeta_old[2], eta[2], nu[2], ptemp[2];
    double dots[8];          // latest fused dot products (for the host's diagnostics)
    // inner solves of the mixed-precision refinement: end when the residual has not
    // fallen below 0.99 x its best for stall_limit iterations (0: rule off)
    int stall_limit, stall;
    double stall_best;
};

}  // namespace ssg

namespace ssg {

// ---------------------------------------------------------------- launchers (ss_spmv_vec.cu)
// Reductions are deterministic: fixed grid per size, block partials summed in
// a fixed order by the last block to arrive.
struct RedBuf {
    double *part;      // grid * 8 doubles
    double *scalar;    // one result slot (host-visible through a copy)
};

int red_grid(int n);

// y = A x ; with st: skipped when the solve is inactive; with dot_alpha: also
// alpha = rur0 / (x . y) into st (ICCG)
template <typename T>
void k_spmv_launch(int n, int group, const int *rp, const int *ci, const T *val, const T *x, T *y, KState *st,
                   bool dot_alpha, double *part, cudaStream_t s);
int spmv_group(double rowlen, bool cplx);  // lanes a row from the nonzero-weighted median row length
double spmv_rowlen(int n, const int *host_row_ptr);  // that length
// ICCG: x += alpha p, r -= alpha Ap, |r| -> convergence decision
template <typename T>
void iccg_update(int n, KState *st, T *x, T *r, const T *p, const T *ap, double *part, double *log, cudaStream_t s);
// ICCG: rur1 = r . z; beta = rur1 / rur0; rur0 = rur1
template <typename T>
void iccg_beta(int n, KState *st, const T *r, const T *z, double *part, cudaStream_t s);
// ICCG: p = beta p + z
template <typename T>
void iccg_p(int n, KState *st, T *p, const T *z, cudaStream_t s);
// MRTR: d0 = a.b, d1 = c.a, d2 = a.y -> zeta, eta, nu, p-factor
template <typename T>
void mrtr_dots(int n, KState *st, const T *a, const T *b, const T *c, const T *y, double *part, cudaStream_t s);
// MRTR: p update, x += zeta p, y = eta y + zeta v, r -= y, |r| -> decision.
// ic_quirk selects the reference's IC-MRTR p = (1 + t) u.
template <typename T>
void mrtr_update(int n, KState *st, T *p, const T *u, T *x, T *y, const T *v, T *r, double *part, double *log,
                 bool ic_quirk, cudaStream_t s);
// IC-MRTR: z = eta z + zeta w ; u -= z
template <typename T>
void mrtr_zu(int n, KState *st, T *z, const T *w, T *u, cudaStream_t s);
// save-best copy when the last decision improved the best residual
template <typename T>
void copy_if_improved(int n, const KState *st, const T *x, T *best, cudaStream_t s);

// plain vector helpers (no state)
template <typename T>
void vec_sub(int n, const T *a, const T *b, T *out, cudaStream_t s);      // out = a - b
template <typename T>
void vec_neg(int n, const T *a, T *out, cudaStream_t s);                  // out = -1 * a
template <typename T>
void vec_mul(int n, T *x, const T *d, cudaStream_t s);                    // x *= d
template <typename T>
void vec_div(int n, T *x, const T *d, cudaStream_t s);                    // x /= d
template <typename T>
void norm2(int n, const T *a, double *out, double *part, cudaStream_t s); // out = |a|
template <typename T>
void dot_into(int n, const T *a, const T *b, double *out2, double *part, cudaStream_t s);  // out2 = a.b (2 doubles)
template <typename T>
void fill_sentinel_st(T *p, int n, const KState *st, cudaStream_t s);
struct SweepCfg;
template <typename T>
void sweep_st(const struct Tri &tri, const T *val, int mode, const T *rhs, const T *aux, const T *D, T *out, T *out2,
              int *d_ticket, int *d_err, const KState *st, cudaStream_t s, const SweepCfg &cfg, const T *dinv);

}  // namespace ssg
