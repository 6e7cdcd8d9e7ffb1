/*
 * MatSolverBase.hpp -- drop-in for the reference's solver base class
 * (include/SparseSolv/MatSolverBase.hpp:42-152 of SparseSolv), implemented
 * over the C ABI of libsparsesolv_gb300 (include/sparsesolv_gb300.h).
 *
 * Same setters, defaults and solve() overloads. Differences a caller can see:
 *  - the solve runs on the GPU (device 0 unless setDevice is called first);
 *  - a row without its diagonal throws std::runtime_error instead of exit(1);
 *  - the Eigen-vector overloads are templates over any vector type with
 *    data() and size() (Eigen::VectorXd/VectorXcd, std::vector, ...);
 *  - additions: getIterations(), getTimings(), getAccelUsed(), getOptions(),
 *    setDevice(), setPrecision(), setReferenceQuirks().
 */
#ifndef SPARSESOLV_GB300_MATSOLVERBASE_HPP
#define SPARSESOLV_GB300_MATSOLVERBASE_HPP

#include <cmath>
#include <iostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../sparsesolv_gb300.h"
#include "SparseMat.hpp"

namespace JPMRspace {
namespace SparseSolv {

namespace detail {
template <class V, class = void>
struct is_vec : std::false_type {};
template <class V>
struct is_vec<V, std::void_t<decltype(std::declval<V &>().data()), decltype(std::declval<V &>().size())>>
    : std::true_type {};
}  // namespace detail

class MatSolverBase {
   public:
    MatSolverBase() { ssg_default_options(&opt); }
    virtual ~MatSolverBase() {
        if (h) ssg_destroy(h);
    }
    MatSolverBase(const MatSolverBase &) = delete;
    MatSolverBase &operator=(const MatSolverBase &) = delete;

    void setInitSolution(bool bl) { opt.is_init = bl ? 1 : 0; }
    void setDiagScale(bool bl) { opt.is_diag_scale = bl ? 1 : 0; }
    void setSaveBest(bool bl) { opt.is_save_best = bl ? 1 : 0; }
    void setSaveLog(bool bl) { opt.is_save_residual_log = bl ? 1 : 0; }
    void getResidualLog(std::vector<double> &log) {
        log.clear();
        if (!h) return;
        int len = 0;
        ssg_get_residual_log(h, nullptr, 0, &len);
        log.resize(len);
        ssg_get_residual_log(h, log.data(), len, &len);
    }
    void setDirvegeType(int x) { opt.diverge_judge_type = x; }
    void setBadDivVal(double x) { opt.bad_div_val = x; }
    void setBadDivCount(int x) { opt.bad_div_count_thres = x; }
    void setConvNormalizeType(int x) { opt.conv_normalize_type = x; }
    void setConvNormalizeConst(double x) { opt.conv_normalize_const = x; }

    /* additions */
    void setDevice(int d) { device = d; }
    void setPrecision(int mode) { opt.precision = mode; }
    void setReferenceQuirks(bool bl) { opt.mrtr_reference_quirks = bl ? 1 : 0; }
    int getIterations() const {
        int it = 0;
        if (h) ssg_get_iters(h, &it);
        return it;
    }
    std::vector<double> getTimings() const {
        std::vector<double> t(2, 0.0);
        if (h) ssg_get_timings(h, t.data(), 2);
        return t;
    }
    /* the settings the next solve passes to the library (accel_factor and
     * precondition_type as the derived solver sets them) */
    ssg_options getOptions() const {
        ssg_options o = opt;
        o.accel_factor = accel();
        o.precondition_type = ptype();
        return o;
    }
    double getAccelUsed() const {
        double a = 0.0;
        if (h) ssg_get_accel_used(h, &a);
        return a;
    }

    /* the eight overloads of the reference (MatSolverBase.hpp:142-150) */
    bool solve(const double conv_cri, const int max_ite, const SparseMat &A, const double *b, double *x) {
        return run(conv_cri, max_ite, -1.0, A, b, x, SSG_REAL);
    }
    bool solve(const double conv_cri, const int max_ite, const double normB, const SparseMat &A, const double *b,
               double *x) {
        return run(conv_cri, max_ite, normB, A, b, x, SSG_REAL);
    }
    bool solve(const double conv_cri, const int max_ite, const SparseMatC &A, const dcomplex *b, dcomplex *x) {
        return run(conv_cri, max_ite, -1.0, A, (const double *)b, (double *)x, SSG_COMPLEX);
    }
    bool solve(const double conv_cri, const int max_ite, const double normB, const SparseMatC &A, const dcomplex *b,
               dcomplex *x) {
        return run(conv_cri, max_ite, normB, A, (const double *)b, (double *)x, SSG_COMPLEX);
    }
    template <class V, class = std::enable_if_t<detail::is_vec<V>::value>>
    bool solve(const double conv_cri, const int max_ite, const SparseMat &A, const V &b, V &x) {
        check_size(A.getSize(), b.size(), x.size());
        return solve(conv_cri, max_ite, A, (const double *)b.data(), (double *)x.data());
    }
    template <class V, class = std::enable_if_t<detail::is_vec<V>::value>>
    bool solve(const double conv_cri, const int max_ite, const double normB, const SparseMat &A, const V &b, V &x) {
        check_size(A.getSize(), b.size(), x.size());
        return solve(conv_cri, max_ite, normB, A, (const double *)b.data(), (double *)x.data());
    }
    template <class V, class = std::enable_if_t<detail::is_vec<V>::value>>
    bool solve(const double conv_cri, const int max_ite, const SparseMatC &A, const V &b, V &x) {
        check_size(A.getSize(), b.size(), x.size());
        return solve(conv_cri, max_ite, A, (const dcomplex *)b.data(), (dcomplex *)x.data());
    }
    template <class V, class = std::enable_if_t<detail::is_vec<V>::value>>
    bool solve(const double conv_cri, const int max_ite, const double normB, const SparseMatC &A, const V &b, V &x) {
        check_size(A.getSize(), b.size(), x.size());
        return solve(conv_cri, max_ite, normB, A, (const dcomplex *)b.data(), (dcomplex *)x.data());
    }

   protected:
    virtual int method() const = 0;
    ssg_options opt{};

   private:
    static void check_size(long n, long nb, long nx) {
        if (nb != n || nx != n) throw std::invalid_argument("SparseSolv: vector size does not match the matrix");
    }
    template <typename DType>
    bool run(double conv_cri, int max_ite, double normB, const SparseMatTMPL<DType> &A, const double *b, double *x,
             int vtype) {
        if (!h) {
            const int rc = ssg_create(&h, device);
            if (rc != SSG_OK) throw std::runtime_error("sparsesolv_gb300: no CUDA device / handle");
        }
        if (cached != (const void *)&A || cached_ver != A.version() || cached_type != vtype) {
            const int rc = ssg_set_matrix(h, A.getSize(), A.nonZeros(), A.rowPtr(), A.getColPtr(),
                                          (const double *)A.getValuePtr(), vtype);
            if (rc != SSG_OK) throw std::runtime_error(std::string("sparsesolv_gb300: ") + ssg_last_error(h));
            cached = &A;
            cached_ver = A.version();
            cached_type = vtype;
        }
        opt.accel_factor = accel();
        opt.precondition_type = ptype();
        ssg_set_options(h, &opt);
        const int rc = ssg_solve(h, method(), conv_cri, max_ite, normB, b, x);
        if (rc == SSG_ERR_NO_DIAGONAL) throw std::runtime_error("there is not diagonal element!");
        if (rc < 0) throw std::runtime_error(std::string("sparsesolv_gb300: ") + ssg_last_error(h));
        if (rc != SSG_OK) std::cout << "not Convergence!!! " << std::endl;
        return rc == SSG_OK;
    }
    virtual double accel() const = 0;
    virtual int ptype() const { return 0; }
    ssg_handle h = nullptr;
    int device = 0;
    const void *cached = nullptr;
    uint64_t cached_ver = ~0ull;
    int cached_type = -1;
};

}  // namespace SparseSolv
}  // namespace JPMRspace

#endif
