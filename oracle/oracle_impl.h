/*
 * oracle_impl.h -- type-generic body of the CPU oracle (TEST INFRASTRUCTURE).
 *
 * Included twice by sparsesolv_oracle.c, once with T = double and once with
 * T = double _Complex. Each function restates one reference function, cited
 * by file:line inside the SparseSolv project. Arithmetic is written in the
 * reference's operand order so that, compiled without FMA contraction, the
 * results track the reference to rounding (its Eigen reductions are
 * vectorised, so sums of dots and norms differ in the last bits).
 *
 * Required macros: T (scalar), SFX (name suffix), TABS(x) (modulus),
 * TABS2(x) (squared modulus), TPOS(x) (positivity test used by the alpha
 * search), IS_COMPLEX (0/1).
 */
#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* y = A x, row by row in stored order (Eigen sparse*dense, row-major;
 * 000_thirdparty/Eigen/src/SparseCore/SparseDenseProduct.h:48-56, whose rows
 * are split over OpenMP threads; each row's sum is the same either way). */
static void FN(spmv)(const or_csr *A, const T *restrict v, const T *x, T *y) {
#pragma omp parallel for schedule(static) if (A->n > 20000)
    for (int i = 0; i < A->n; ++i) {
        T s = 0;
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k) s += v[k] * x[A->ci[k]];
        y[i] = s;
    }
}

static T FN(dotnc)(int n, const T *a, const T *b) {
    T s = 0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

static double FN(nrm2)(int n, const T *a) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += TABS2(a[i]);
    return sqrt(s);
}

/*
 * Shifted IC(0) in root-free form on the lower triangle L (pattern of
 * lower(A), diagonal last in every row); overwrites vl, writes D = 1/pivot.
 * src/SprsPreconditioner.cpp:43-111. Returns -2 when a row has no diagonal
 * (the reference prints and calls exit(1), :91-94).
 */
static int FN(ic_decomp_sub)(const or_csr *L, T *vl, T *D, double accela) {
    const int n = L->n;
    const int *rp = L->rp, *ci = L->ci;
    for (int i = 0; i < n; ++i) D[i] = 0;
    for (int i = 0; i < n; ++i) {
        T s;
        for (int jj = rp[i]; jj < rp[i + 1]; ++jj) {
            const int j = ci[jj];
            if (j >= i) break;
            s = vl[jj];
            for (int kk = rp[i]; kk < rp[i + 1]; ++kk) {
                if (ci[kk] <= j - 1) {
                    for (int ll = rp[j]; ll < rp[j + 1]; ++ll) {
                        if (ci[ll] == ci[kk]) {
                            s -= vl[kk] * vl[ll] * D[ci[ll]];
                            break;
                        } else if (ci[kk] < ci[ll]) {
                            break;
                        }
                    }
                } else {
                    break;
                }
            }
            vl[jj] = s;
        }
        const int last = rp[i + 1] - 1;
        if (last < rp[i] || ci[last] != i) return -2;
        s = vl[last] * accela;
        for (int kk = rp[i]; kk < last; ++kk) {
            if (ci[kk] <= i - 1) s -= vl[kk] * vl[kk] * D[ci[kk]];
            else break;
        }
        vl[last] = s;
        if (TABS(s) < 1.0e-12) D[i] = 1.0 / (DBL_EPSILON);
        else D[i] = 1.0 / s;
    }
    return 0;
}

/* IC_decomp = MatLower + IC_decomp_sub (src/SprsPreconditioner.cpp:133-142).
 * Fills L (allocated here) and D[n]. */
static int FN(ic_decomp)(const or_csr *A, const T *va, double accela, or_csr *L, T **vl, T *D) {
    if (or_lower(A, L) != 0) return -1;
    *vl = (T *)malloc(sizeof(T) * (size_t)(L->rp[L->n] + 1));
    if (!*vl) return -1;
    or_gather_values(L, va, sizeof(T), *vl);
    return FN(ic_decomp_sub)(L, *vl, D, accela);
}

/*
 * Forward then backward substitution with L D L^T, D = diag(1/L_ii):
 * MatSolverBase::IC_frbc_process, src/MatSolverBase.cpp:177-231.
 * Lt is trans(L) (diagonal first in each row).
 */
static void FN(ic_frbc)(const or_csr *L, const T *vl, const or_csr *Lt, const T *vlt,
                        const T *D, const T *r, T *out, T *tmp) {
    const int n = L->n;
    for (int i = 0; i < n; ++i) {
        T s = r[i];
        const int c_size = L->rp[i + 1] - 1;
        for (int jj = L->rp[i]; jj < c_size; ++jj) s -= vl[jj] * tmp[L->ci[jj]];
        tmp[i] = s / vl[c_size];
    }
    for (int i = n; i-- > 0;) {
        T s = 0;
        for (int j = Lt->rp[i] + 1; j < Lt->rp[i + 1]; ++j) s -= vlt[j] * out[Lt->ci[j]];
        s *= D[i];
        out[i] = s + tmp[i];
    }
}

/* plain forward substitution with the diagonal last: fr_process, src/MatSolverBase.cpp:243-278 */
static void FN(fr)(const or_csr *L, const T *vl, const T *r, T *v) {
    for (int i = 0; i < L->n; ++i) {
        T s = r[i];
        const int c_size = L->rp[i + 1] - 1;
        for (int jj = L->rp[i]; jj < c_size; ++jj) s -= vl[jj] * v[L->ci[jj]];
        v[i] = s / vl[c_size];
    }
}

/* plain backward substitution with the diagonal first: bc_process, src/MatSolverBase.cpp:291-327 */
static void FN(bc)(const or_csr *U, const T *vu, const T *r, T *v) {
    for (int i = U->n; i-- > 0;) {
        T s = r[i];
        for (int j = U->rp[i] + 1; j < U->rp[i + 1]; ++j) s -= vu[j] * v[U->ci[j]];
        v[i] = s / vu[U->rp[i]];
    }
}

/*
 * Diagonal scaling d_i = 1/sqrt(|a_ii|) (1/eps when tiny), b~ = D b:
 * SprsPreconditioner::DiagScaling, src/SprsPreconditioner.cpp:150-231.
 * The complex version takes sqrt(std::norm(a_ii)) = |a_ii| (:214-215).
 */
static void FN(diag_scaling)(const or_csr *A, const T *va, const T *b, T *d, T *bs) {
    for (int i = 0; i < A->n; ++i) {
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k) {
            if (A->ci[k] == i) {
#if IS_COMPLEX
                const double t1 = TABS2(va[k]);
#else
                const double t1 = fabs(va[k]);
#endif
                const double t1b = sqrt(t1);
                const double t2 = (t1b < 1.0e-12) ? 1.0 / (DBL_EPSILON) : 1.0 / t1b;
                d[i] = t2;
                bs[i] = b[i] * (T)t2;
                break;
            }
        }
    }
}

/* D A D: MatSolverBase::makeDiagMatTrans, src/MatSolverBase.cpp:99-141 */
static void FN(dad)(const or_csr *A, const T *va, const T *d, T *out) {
    for (int i = 0; i < A->n; ++i) {
        const T di = d[i];
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k) out[k] = va[k] * (di * d[A->ci[k]]);
    }
}

/* alpha search: MatSolverBase::auto_accel_determine, src/MatSolverBase.cpp:344-391 */
static int FN(auto_accel)(const or_csr *A, const T *va, double accel_ini, or_csr *L, T **vl, T *D, double *used) {
    double a = fabs(accel_ini);
    if (a < 0.9 || a > 1.8) a = 1;
    for (int t = 0; t < 80; ++t) {
        int rc = FN(ic_decomp)(A, va, a, L, vl, D);
        if (rc) return rc;
        int ok = 1;
        for (int i = 0; i < A->n; ++i) ok &= TPOS(D[i]);
        if (ok) { *used = a; return 0; }
        or_free(L);
        free(*vl);
        *vl = NULL;
        a += 0.01;
    }
    *used = 1.8;
    return FN(ic_decomp)(A, va, 1.8, L, vl, D);
}

/* ---------------------------------------------------------------------- */
/* Krylov drivers                                                          */
/* ---------------------------------------------------------------------- */

typedef struct {
    const or_opts *o;
    double *log;
    int log_cap;
    int log_len;
} FN(logger);

static void FN(log_push)(FN(logger) *lg, double v) {
    if (!lg->o->is_save_residual_log) return;
    if (lg->log_len < lg->log_cap) lg->log[lg->log_len] = v;
    lg->log_len++;
}

/* convergence set-up shared by all solve_main variants (e.g.
 * src/MatSolverICCG.cpp:212-237). Returns 1 when the solve ends early. */
static int FN(conv_setup)(const or_opts *o, FN(logger) *lg, double normB, double pure_normR,
                          double conv_cri, double *abs_conv_cri, double *normalizer) {
    const double rhs_eps = 1.0e-30;
    if (normB <= rhs_eps && pure_normR <= 1.0e-20) {
        if (o->is_save_residual_log) { lg->log_len = 0; FN(log_push)(lg, 0.0); }
        return 1;
    }
    *abs_conv_cri = (normB * conv_cri * 0.9 < 1.0e-20 ? 1.0e-20 : normB * conv_cri * 0.9);
    const double first_normR = pure_normR / normB;
    if (first_normR < conv_cri * 0.5 || pure_normR < *abs_conv_cri * 0.5) return 1;
    *normalizer = or_normalizer(o, normB, pure_normR);
    FN(log_push)(lg, pure_normR / *normalizer);
    return 0;
}

/* divergence judge and best tracking (e.g. src/MatSolverICCG.cpp:283-305).
 * Returns 1 when the solve must stop as diverged. */
static int FN(track)(const or_opts *o, double normR, double *best, int *bad, const T *x, T *best_x, int n) {
    if (normR < *best) {
        *best = normR;
        if (o->is_save_best) memcpy(best_x, x, sizeof(T) * (size_t)n);
    }
    if (o->diverge_judge_type == 1) {
        if (normR < *best * o->bad_div_val) *bad = 0;
        if (normR >= *best * o->bad_div_val) (*bad)++;
        if (*bad >= o->bad_div_count_thres) return 1;
    }
    return 0;
}

/*
 * Shifted ICCG / ICCOCG body: MatSolverICCG::solve_main,
 * src/MatSolverICCG.cpp:178-328 (real), :477-626 (complex).
 */
static int FN(iccg_main)(const or_opts *o, FN(logger) *lg, const or_csr *A, const T *va,
                         const or_csr *L, const T *vl, const or_csr *Lt, const T *vlt, const T *D,
                         double normB, double conv_cri, int max_ite, const T *b, T *x, int *iters) {
    const int n = A->n;
    T *p = (T *)calloc((size_t)n, sizeof(T)), *r = (T *)malloc(sizeof(T) * (size_t)n);
    T *z = (T *)malloc(sizeof(T) * (size_t)n), *ap = (T *)malloc(sizeof(T) * (size_t)n);
    T *tmp = (T *)malloc(sizeof(T) * (size_t)n);
    T *best_x = o->is_save_best ? (T *)calloc((size_t)n, sizeof(T)) : NULL;
    int is_conv = 0;
    *iters = 0;
    if (o->is_init) memset(x, 0, sizeof(T) * (size_t)n);
    lg->log_len = 0;
    double best = 1.0e+6;
    memcpy(r, b, sizeof(T) * (size_t)n);
    if (!o->is_init) {
        FN(spmv)(A, va, x, ap);
        for (int i = 0; i < n; ++i) r[i] -= ap[i];
    }
    const double pure_normR = FN(nrm2)(n, r);
    double abs_conv_cri = 0.0, normalizer = 1.0;
    if (FN(conv_setup)(o, lg, normB, pure_normR, conv_cri, &abs_conv_cri, &normalizer)) {
        is_conv = 1;
        goto done;
    }
    FN(ic_frbc)(L, vl, Lt, vlt, D, r, p, tmp);
    memcpy(z, p, sizeof(T) * (size_t)n);
    T rur0 = FN(dotnc)(n, r, z);
    int bad = 0;
    for (int it = 0; it < max_ite; ++it) {
        FN(spmv)(A, va, p, ap);
        const T temp2 = FN(dotnc)(n, p, ap);
        const T alpha = rur0 / temp2;
        for (int i = 0; i < n; ++i) x[i] += alpha * p[i];
        for (int i = 0; i < n; ++i) r[i] -= alpha * ap[i];
        const double pure_norm = FN(nrm2)(n, r);
        const double normR = pure_norm / normalizer;
        FN(log_push)(lg, normR);
        *iters = it + 1;
        if (normR < conv_cri || pure_norm < abs_conv_cri) { is_conv = 1; break; }
        if (FN(track)(o, normR, &best, &bad, x, best_x, n)) { is_conv = 0; break; }
        FN(ic_frbc)(L, vl, Lt, vlt, D, r, z, tmp);
        const T rur1 = FN(dotnc)(n, r, z);
        const T beta = rur1 / rur0;
        rur0 = rur1;
        for (int i = 0; i < n; ++i) { p[i] *= beta; p[i] += z[i]; }
    }
    if (!is_conv && o->is_save_best) memcpy(x, best_x, sizeof(T) * (size_t)n);
done:
    free(p); free(r); free(z); free(ap); free(tmp); free(best_x);
    return is_conv;
}

/*
 * IC-preconditioned MRTR body: MatSolverMRTR::solve_main,
 * src/MatSolverMRTR_ICver.cpp:183-373 (real), :529-722 (complex).
 * With o->mrtr_reference_quirks = 1 the reference's p update p = (1+t) u
 * (:303-304, :651-652) and its warm start r0 = b (:213-216) are reproduced;
 * with 0, p = u + t p_old and r0 = b - A x0. Neither changes the residual
 * recurrence for a zero initial guess.
 */
static int FN(mrtr_ic_main)(const or_opts *o, FN(logger) *lg, const or_csr *A, const T *va,
                            const or_csr *L, const T *vl, const or_csr *Lt, const T *vlt, const T *D,
                            double normB, double conv_cri, int max_ite, const T *b, T *results, int *iters) {
    const int n = A->n;
    T *p = (T *)calloc((size_t)n, sizeof(T)), *r = (T *)malloc(sizeof(T) * (size_t)n);
    T *u = (T *)malloc(sizeof(T) * (size_t)n), *X = (T *)calloc((size_t)n, sizeof(T));
    T *y = (T *)malloc(sizeof(T) * (size_t)n), *z = (T *)malloc(sizeof(T) * (size_t)n);
    T *v = (T *)malloc(sizeof(T) * (size_t)n), *w = (T *)malloc(sizeof(T) * (size_t)n);
    T *tmp = (T *)malloc(sizeof(T) * (size_t)n);
    T *best_x = o->is_save_best ? (T *)calloc((size_t)n, sizeof(T)) : NULL;
    int is_conv = 0;
    *iters = 0;
    if (o->is_init) memset(results, 0, sizeof(T) * (size_t)n);
    else memcpy(X, results, sizeof(T) * (size_t)n);
    lg->log_len = 0;
    double best = 1.0e+6;
    memcpy(r, b, sizeof(T) * (size_t)n);
    if (o->mrtr_reference_quirks ? o->is_init : !o->is_init) {
        FN(spmv)(A, va, results, v);
        for (int i = 0; i < n; ++i) r[i] -= v[i];
    }
    const double pure_normR = FN(nrm2)(n, r);
    double abs_conv_cri = 0.0, normalizer = 1.0;
    if (FN(conv_setup)(o, lg, normB, pure_normR, conv_cri, &abs_conv_cri, &normalizer)) {
        is_conv = 1;
        goto done_early;
    }
    FN(ic_frbc)(L, vl, Lt, vlt, D, r, u, tmp);
    for (int i = 0; i < n; ++i) y[i] = -1.0 * r[i];
    FN(ic_frbc)(L, vl, Lt, vlt, D, y, z, tmp);
    T zeta = 1.0, zeta_old = 1.0, eta = 0.0, nu = 1.0;
    int bad = 0;
    for (int it = 0; it < max_ite; ++it) {
        FN(spmv)(A, va, u, v);
        FN(ic_frbc)(L, vl, Lt, vlt, D, v, w, tmp);
        const T w_r = FN(dotnc)(n, w, r);
        const T v_w = FN(dotnc)(n, v, w);
        if (it == 0) {
            zeta = w_r / v_w;
            zeta_old = zeta;
            eta = 0.0;
        } else {
            const T w_y = FN(dotnc)(n, w, y);
            const T temp0 = 1.0 / (nu * v_w - w_y * w_y);
            zeta = nu * w_r * temp0;
            eta = -1.0 * w_y * w_r * temp0;
        }
        nu = zeta * w_r;
        const T temp = eta * zeta_old / zeta;
        if (o->mrtr_reference_quirks) {
            for (int i = 0; i < n; ++i) { p[i] = u[i]; p[i] += temp * p[i]; }
        } else {
            for (int i = 0; i < n; ++i) { p[i] *= temp; p[i] += u[i]; }
        }
        zeta_old = zeta;
        for (int i = 0; i < n; ++i) X[i] += zeta * p[i];
        for (int i = 0; i < n; ++i) { y[i] *= eta; y[i] += zeta * v[i]; }
        for (int i = 0; i < n; ++i) r[i] -= y[i];
        const double norm_r = FN(nrm2)(n, r);
        const double normR = norm_r / normalizer;
        FN(log_push)(lg, normR);
        *iters = it + 1;
        if (normR < conv_cri || norm_r < abs_conv_cri) { is_conv = 1; break; }
        if (FN(track)(o, normR, &best, &bad, X, best_x, n)) { is_conv = 0; break; }
        for (int i = 0; i < n; ++i) { z[i] *= eta; z[i] += zeta * w[i]; }
        for (int i = 0; i < n; ++i) u[i] -= z[i];
    }
    memcpy(results, X, sizeof(T) * (size_t)n);
    if (!is_conv && o->is_save_best) memcpy(results, best_x, sizeof(T) * (size_t)n);
done_early:
    free(p); free(r); free(u); free(X); free(y); free(z); free(v); free(w); free(tmp); free(best_x);
    return is_conv;
}

/*
 * Eisenstat SGS-MRTR body on the scaled system: MatSolverMRTR::solve_SGS_MRTR_main,
 * src/MatSolverMRTR_SGSver.cpp:81-282 (real), :340-539 (complex).
 * C = lower(DAD) with the diagonal, U = upper(DAD) with the diagonal.
 */
static int FN(sgs_mrtr_main)(const or_opts *o, FN(logger) *lg, const or_csr *A, const T *va,
                             const or_csr *Lc, const T *vl, const or_csr *Uc, const T *vu,
                             double normB, double conv_cri, int max_ite, const T *b, T *results, int *iters) {
    const int n = A->n;
    T *p = (T *)calloc((size_t)n, sizeof(T)), *rd = (T *)malloc(sizeof(T) * (size_t)n);
    T *u = (T *)malloc(sizeof(T) * (size_t)n), *X = (T *)calloc((size_t)n, sizeof(T));
    T *y = (T *)malloc(sizeof(T) * (size_t)n), *ard = (T *)malloc(sizeof(T) * (size_t)n);
    T *tmp = (T *)malloc(sizeof(T) * (size_t)n);
    T *best_x = o->is_save_best ? (T *)calloc((size_t)n, sizeof(T)) : NULL;
    int is_conv = 0;
    *iters = 0;
    if (o->is_init) memset(results, 0, sizeof(T) * (size_t)n);
    else memcpy(X, results, sizeof(T) * (size_t)n);
    lg->log_len = 0;
    double best = 1.0e+6;
    memcpy(rd, b, sizeof(T) * (size_t)n);
    if (o->mrtr_reference_quirks ? o->is_init : !o->is_init) {
        FN(spmv)(A, va, results, u);
        for (int i = 0; i < n; ++i) rd[i] -= u[i];
    }
    memcpy(tmp, rd, sizeof(T) * (size_t)n);
    FN(fr)(Lc, vl, tmp, rd);
    const double pure_normR = FN(nrm2)(n, rd);
    double abs_conv_cri = 0.0, normalizer = 1.0;
    if (FN(conv_setup)(o, lg, normB, pure_normR, conv_cri, &abs_conv_cri, &normalizer)) {
        is_conv = 1;
        goto done_early;
    }
    for (int i = 0; i < n; ++i) y[i] = -1.0 * rd[i];
    T zeta = 1.0, zeta_old = 1.0, eta = 0.0, nu = 1.0;
    int bad = 0;
    for (int it = 0; it < max_ite; ++it) {
        FN(bc)(Uc, vu, rd, u);
        for (int i = 0; i < n; ++i) tmp[i] = rd[i] - u[i];
        FN(fr)(Lc, vl, tmp, ard);
        for (int i = 0; i < n; ++i) ard[i] += u[i];
        const T Ar_r = FN(dotnc)(n, ard, rd);
        const T Ar_Ar = FN(dotnc)(n, ard, ard);
        if (it == 0) {
            zeta = Ar_r / Ar_Ar;
            zeta_old = zeta;
            eta = 0.0;
        } else {
            const T Ar_y = FN(dotnc)(n, ard, y);
            const T temp = 1.0 / (nu * Ar_Ar - Ar_y * Ar_y);
            zeta = nu * Ar_r * temp;
            eta = -1.0 * Ar_y * Ar_r * temp;
        }
        nu = zeta * Ar_r;
        const T temp2 = eta * zeta_old / zeta;
        for (int i = 0; i < n; ++i) { p[i] *= temp2; p[i] += u[i]; }
        zeta_old = zeta;
        for (int i = 0; i < n; ++i) X[i] += zeta * p[i];
        for (int i = 0; i < n; ++i) { y[i] *= eta; y[i] += zeta * ard[i]; }
        for (int i = 0; i < n; ++i) rd[i] -= y[i];
        const double norm_r = FN(nrm2)(n, rd);
        const double normR = norm_r / normalizer;
        FN(log_push)(lg, normR);
        *iters = it + 1;
        if (normR < conv_cri || norm_r < abs_conv_cri) { is_conv = 1; break; }
        if (FN(track)(o, normR, &best, &bad, X, best_x, n)) { is_conv = 0; break; }
    }
    memcpy(results, X, sizeof(T) * (size_t)n);
    if (!is_conv && o->is_save_best) memcpy(results, best_x, sizeof(T) * (size_t)n);
done_early:
    free(p); free(rd); free(u); free(X); free(y); free(ard); free(tmp); free(best_x);
    return is_conv;
}

/* ---------------------------------------------------------------------- */
/* public entry: one solve() call of MatSolverICCG or MatSolverMRTR        */
/* ---------------------------------------------------------------------- */

/*
 * method: 0 = ICCG (MatSolverICCG::solve, src/MatSolverICCG.cpp:99-168, :401-467)
 *         1 = MRTR (MatSolverMRTR::solve, src/MatSolverMRTR_ICver.cpp:99-173, :446-519;
 *             o->precondition_type 1 dispatches to SGS, :102-104)
 * normB < 0 means "compute sqrt(sum b_i^2)" as the pointer overloads do
 * (src/MatSolverICCG.cpp:44-58).
 * Returns 1 converged, 0 not converged, < 0 error.
 */
int FN(or_solve)(const or_opts *o, int method, int n, const int *rp, const int *ci, const T *va,
                 const T *b, double normB, double conv_cri, int max_ite, T *x,
                 double *log, int log_cap, int *log_len, int *iters) {
    const double t_start = or_now();
    double t_iter = t_start;
    or_csr A = {n, (int *)rp, (int *)ci};
    FN(logger) lg = {o, log, log_cap, 0};
    int rc = 0;
    *iters = 0;
    if (normB < 0.0) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += TABS2(b[i]);
        normB = sqrt(s);
    }
    const int sgs = (method == 1 && o->precondition_type == 1);
    const int scale = sgs || o->is_diag_scale;
    T *d = NULL, *bs = NULL, *vs = NULL;
    const T *vA = va, *bb = b;
    if (scale) {
        d = (T *)malloc(sizeof(T) * (size_t)n);
        bs = (T *)malloc(sizeof(T) * (size_t)n);
        vs = (T *)malloc(sizeof(T) * (size_t)(rp[n] + 1));
        FN(diag_scaling)(&A, va, b, d, bs);
        FN(dad)(&A, va, d, vs);
        vA = vs;
        bb = bs;
        normB = FN(nrm2)(n, bs);
        if (!o->is_init)
            for (int i = 0; i < n; ++i) x[i] /= d[i];
    }
    if (sgs) {
        or_csr Lc, Uc;
        if (or_lower(&A, &Lc) || or_upper(&A, &Uc)) { rc = -1; goto out; }
        T *vl = (T *)malloc(sizeof(T) * (size_t)(Lc.rp[n] + 1));
        T *vu = (T *)malloc(sizeof(T) * (size_t)(Uc.rp[n] + 1));
        or_gather_values(&Lc, vA, sizeof(T), vl);
        or_gather_values(&Uc, vA, sizeof(T), vu);
        t_iter = or_now();
        rc = FN(sgs_mrtr_main)(o, &lg, &A, vA, &Lc, vl, &Uc, vu, normB, conv_cri, max_ite, bb, x, iters);
        or_free(&Lc); or_free(&Uc); free(vl); free(vu);
    } else {
        or_csr L, Lt;
        T *vl = NULL, *vlt = NULL;
        T *D = (T *)malloc(sizeof(T) * (size_t)n);
        double used = o->accel_factor;
        if (o->accel_factor < 0.0) rc = FN(auto_accel)(&A, vA, o->accel_factor, &L, &vl, D, &used);
        else rc = FN(ic_decomp)(&A, vA, o->accel_factor, &L, &vl, D);
        if (rc) { free(D); free(vl); goto out; }
        if (or_transpose(&L, &Lt)) { rc = -1; free(D); free(vl); goto out; }
        vlt = (T *)malloc(sizeof(T) * (size_t)(Lt.rp[n] + 1));
        or_permute_values(&Lt, vl, sizeof(T), vlt);
        t_iter = or_now();
        if (method == 0)
            rc = FN(iccg_main)(o, &lg, &A, vA, &L, vl, &Lt, vlt, D, normB, conv_cri, max_ite, bb, x, iters);
        else
            rc = FN(mrtr_ic_main)(o, &lg, &A, vA, &L, vl, &Lt, vlt, D, normB, conv_cri, max_ite, bb, x, iters);
        or_free(&L); or_free(&Lt); free(vl); free(vlt); free(D);
    }
    if (scale)
        for (int i = 0; i < n; ++i) x[i] *= d[i];
out:
    free(d); free(bs); free(vs);
    *log_len = lg.log_len;
    {
        const double t_end = or_now();
        or_timing[0] = t_iter - t_start;
        or_timing[1] = t_end - t_iter;
        or_timing[2] = t_end - t_start;
    }
    return rc;
}

/* IC factor alone (for factor parity tests): L values in the lower(A) pattern and D */
int FN(or_ic_factor)(int n, const int *rp, const int *ci, const T *va, double accela,
                     int *lrp, int *lci, T *lval, T *D) {
    or_csr A = {n, (int *)rp, (int *)ci}, L;
    T *vl = NULL;
    int rc = FN(ic_decomp)(&A, va, accela, &L, &vl, D);
    if (rc == 0 || rc == -2) {
        memcpy(lrp, L.rp, sizeof(int) * (size_t)(n + 1));
        memcpy(lci, L.ci, sizeof(int) * (size_t)L.rp[n]);
        memcpy(lval, vl, sizeof(T) * (size_t)L.rp[n]);
        or_free(&L);
    }
    free(vl);
    return rc;
}

/* z = (L D L^T)^{-1} r given a factor (for trisolve parity tests) */
int FN(or_ic_apply)(int n, const int *lrp, const int *lci, const T *lval, const T *D, const T *r, T *z) {
    or_csr L = {n, (int *)lrp, (int *)lci}, Lt;
    if (or_transpose(&L, &Lt)) return -1;
    T *vlt = (T *)malloc(sizeof(T) * (size_t)(Lt.rp[n] + 1));
    T *tmp = (T *)malloc(sizeof(T) * (size_t)n);
    or_permute_values(&Lt, lval, sizeof(T), vlt);
    FN(ic_frbc)(&L, lval, &Lt, vlt, D, r, z, tmp);
    or_free(&Lt); free(vlt); free(tmp);
    return 0;
}

void FN(or_spmv)(int n, const int *rp, const int *ci, const T *va, const T *x, T *y) {
    or_csr A = {n, (int *)rp, (int *)ci};
    FN(spmv)(&A, va, x, y);
}

#undef FN
#undef CAT
#undef CAT_
