/*
 * ref_shim.cpp -- C entry points over the reference's own solver classes
 * (TEST INFRASTRUCTURE ONLY).
 *
 * Compiled together with the reference's sources (src/*.cpp of SparseSolv,
 * vendored Eigen headers) by oracle/Makefile into oracle/_ref/. The tests use
 * it to pin the C restatement in sparsesolv_oracle.c and to produce the golden
 * fixtures; bench.py may time it as the CPU baseline where it exists. It calls
 * only the reference's public API: SparseMat, MatSolverICCG, MatSolverMRTR
 * (include/SparseSolv/*.hpp) and SprsPreconditioner::IC_decomp.
 */
#include <SparseSolv/MatSolverICCG.hpp>
#include <SparseSolv/MatSolverMRTR.hpp>
#include <complex>
#include <vector>

using namespace JPMRspace::SparseSolv;
using JPMRspace::dcomplex;

namespace {
template <typename T>
SparseMatTMPL<T> make_mat(int n, const int *rp, const int *ci, const T *va) {
    std::vector<Eigen::Triplet<T>> trip;
    trip.reserve((size_t)rp[n]);
    for (int i = 0; i < n; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) trip.emplace_back(i, ci[k], va[k]);
    Eigen::SparseMatrix<T, Eigen::RowMajor> M(n, n);
    M.setFromTriplets(trip.begin(), trip.end());
    return SparseMatTMPL<T>(std::move(M));
}

struct Settings {
    int is_init, is_diag_scale, is_save_best, is_save_residual_log, diverge_judge_type;
    double bad_div_val;
    int bad_div_count_thres, conv_normalize_type;
    double conv_normalize_const, accel_factor;
    int precondition_type;
};

void apply(MatSolverBase &s, const Settings &o) {
    s.setInitSolution(o.is_init != 0);
    s.setDiagScale(o.is_diag_scale != 0);
    s.setSaveBest(o.is_save_best != 0);
    s.setSaveLog(o.is_save_residual_log != 0);
    s.setDirvegeType(o.diverge_judge_type);
    s.setBadDivVal(o.bad_div_val);
    s.setBadDivCount(o.bad_div_count_thres);
    s.setConvNormalizeType(o.conv_normalize_type);
    s.setConvNormalizeConst(o.conv_normalize_const);
}

template <typename T>
int solve_any(const Settings *o, int method, int n, const int *rp, const int *ci, const T *va, const T *b,
              double normB, double conv, int maxit, T *x, double *log, int log_cap, int *log_len) {
    SparseMatTMPL<T> A = make_mat<T>(n, rp, ci, va);
    bool ok;
    std::vector<double> lg;
    if (method == 0) {
        MatSolverICCG s;
        apply(s, *o);
        s.setAccelFactor(o->accel_factor);
        ok = normB < 0 ? s.solve(conv, maxit, A, b, x) : s.solve(conv, maxit, normB, A, b, x);
        s.getResidualLog(lg);
    } else {
        MatSolverMRTR s;
        apply(s, *o);
        s.setAccelFactor(o->accel_factor);
        s.setPreconditionType(o->precondition_type);
        ok = normB < 0 ? s.solve(conv, maxit, A, b, x) : s.solve(conv, maxit, normB, A, b, x);
        s.getResidualLog(lg);
    }
    *log_len = (int)lg.size();
    for (int i = 0; i < (int)lg.size() && i < log_cap; ++i) log[i] = lg[i];
    return ok ? 1 : 0;
}

template <typename T>
int factor_any(int n, const int *rp, const int *ci, const T *va, double accela, int *lrp, int *lci, T *lval, T *D) {
    SparseMatTMPL<T> A = make_mat<T>(n, rp, ci, va);
    SparseMatTMPL<T> L = SprsPreconditioner::IC_decomp(A, D, accela);
    std::vector<slv_int> s, e;
    L.getCols(s, e);
    const slv_int *c = L.getColPtr();
    const T *v = L.getValuePtr();
    int pos = 0;
    for (int i = 0; i < n; ++i) {
        lrp[i] = pos;
        for (int k = s[i]; k < e[i]; ++k, ++pos) {
            lci[pos] = c[k];
            lval[pos] = v[k];
        }
    }
    lrp[n] = pos;
    return 0;
}
}  // namespace

// SparseMatTMPL's COO constructor (src/SparseMat.cpp:80-104): CSR out; returns
// the stored entry count, or its negative when cap is too small
template <typename T>
int coo_any(int nnz, const int *rows, const int *cols, const T *vals, int *nrows, int *ncols, int *rp, int *ci,
            T *va, int cap) {
    std::vector<slv_int> r(rows, rows + nnz), c(cols, cols + nnz);
    std::vector<T> v(vals, vals + nnz);
    SparseMatTMPL<T> M(nnz, r, c, v);
    auto &E = M.mat();
    E.makeCompressed();
    *nrows = (int)E.rows();
    *ncols = (int)E.cols();
    const int nz = (int)E.nonZeros();
    if (nz > cap) return -nz;
    for (int i = 0; i <= *nrows; ++i) rp[i] = E.outerIndexPtr()[i];
    for (int k = 0; k < nz; ++k) {
        ci[k] = E.innerIndexPtr()[k];
        va[k] = E.valuePtr()[k];
    }
    return nz;
}

extern "C" {
int ref_coo_to_csr_d(int nnz, const int *rows, const int *cols, const double *vals, int *nrows, int *ncols, int *rp,
                     int *ci, double *va, int cap) {
    return coo_any<double>(nnz, rows, cols, vals, nrows, ncols, rp, ci, va, cap);
}
int ref_coo_to_csr_z(int nnz, const int *rows, const int *cols, const dcomplex *vals, int *nrows, int *ncols, int *rp,
                     int *ci, dcomplex *va, int cap) {
    return coo_any<dcomplex>(nnz, rows, cols, vals, nrows, ncols, rp, ci, va, cap);
}
int ref_solve_d(const Settings *o, int method, int n, const int *rp, const int *ci, const double *va,
                const double *b, double normB, double conv, int maxit, double *x, double *log, int log_cap,
                int *log_len) {
    return solve_any<double>(o, method, n, rp, ci, va, b, normB, conv, maxit, x, log, log_cap, log_len);
}
int ref_solve_z(const Settings *o, int method, int n, const int *rp, const int *ci, const dcomplex *va,
                const dcomplex *b, double normB, double conv, int maxit, dcomplex *x, double *log, int log_cap,
                int *log_len) {
    return solve_any<dcomplex>(o, method, n, rp, ci, va, b, normB, conv, maxit, x, log, log_cap, log_len);
}
int ref_ic_factor_d(int n, const int *rp, const int *ci, const double *va, double accela, int *lrp, int *lci,
                    double *lval, double *D) {
    return factor_any<double>(n, rp, ci, va, accela, lrp, lci, lval, D);
}
int ref_ic_factor_z(int n, const int *rp, const int *ci, const dcomplex *va, double accela, int *lrp, int *lci,
                    dcomplex *lval, dcomplex *D) {
    return factor_any<dcomplex>(n, rp, ci, va, accela, lrp, lci, lval, D);
}
}
