/*
 * SparseMat.hpp -- drop-in for SparseMatTMPL / SparseMat / SparseMatC
 * (include/SparseSolv/SparseMat.hpp:49-136 of SparseSolv).
 *
 * Storage is row-major CSR with sorted columns and summed duplicates, the
 * layout of Eigen::SparseMatrix<T, RowMajor> after setFromTriplets
 * (src/SparseMat.cpp:54-122). Eigen is not a dependency: without it the
 * matrix is read through rowPtr()/getColPtr()/getValuePtr(). Every mutation
 * takes a new version() from one process-wide counter, so two matrices never
 * share a version (a matrix built where a freed one lived is not mistaken for
 * it); the solvers use it to decide when the device copy and its factor must
 * be refreshed.
 *
 * Always available, as in the reference: the builder, COO and CSR
 * constructors, build, getSize, getTrueSize, getMaxCol, getCols, getColPtr,
 * getValuePtr, resetMat, add (coefficient +=, inserting a missing entry),
 * compressed, isInclude, getTargetRowVal, getTargetColVal, prune, printMat,
 * print and readMat (src/SparseMat.cpp:188-409).
 *
 * With Eigen included before this header (<Eigen/Sparse>, or define
 * SPARSESOLV_WITH_EIGEN to have it included here): the constructors from an
 * Eigen::SparseMatrix<T, RowMajor> and from std::vector<Eigen::Triplet<T>>,
 * setMatrix, and mat(). mat() returns an Eigen::Map of the CSR arrays
 * (Eigen::Map<Eigen::SparseMatrix<T, RowMajor, int>>) rather than a reference
 * to a stored Eigen matrix: it serves every expression the reference builds on
 * mat() (products, sums, transpose, triangularView, cast, coeff, nonZeros) and
 * writes to existing coefficients; a structural change goes through add(),
 * prune() or setMatrix(). The non-const mat() bumps version().
 */
#ifndef SPARSESOLV_GB300_SPARSEMAT_HPP
#define SPARSESOLV_GB300_SPARSEMAT_HPP

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <fstream>
#include <limits>
#include <numeric>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "SparseBuilder.hpp"

#if defined(SPARSESOLV_WITH_EIGEN) && !defined(EIGEN_SPARSECORE_MODULE_H)
#include <Eigen/Sparse>
#endif
#include <cmath>
#include <iostream>

namespace JPMRspace {
namespace SparseSolv {

template <typename DType>
class SparseMatTMPL {
   public:
    SparseMatTMPL() : rp(1, 0) {}
    SparseMatTMPL(SparseBuilderTMPL<DType> &builder, bool to_square = false) { build(builder, to_square); }
    /* COO constructor: size = largest index + 1, duplicates summed (src/SparseMat.cpp:80-104) */
    SparseMatTMPL(slv_int n_nonZero, const std::vector<slv_int> &rows, const std::vector<slv_int> &cols,
                  const std::vector<DType> &vals) {
        if (n_nonZero < 0 || (size_t)n_nonZero > rows.size() || (size_t)n_nonZero > cols.size() ||
            (size_t)n_nonZero > vals.size())
            throw std::invalid_argument("SparseMat: n_nonzero exceeds the rows/cols/vals given");
        std::vector<typename SparseBuilderTMPL<DType>::Triplet> t;
        t.reserve(n_nonZero);
        slv_int mr = 0, mc = 0;
        for (slv_int i = 0; i < n_nonZero; ++i) {
            t.push_back({rows[i], cols[i], vals[i]});
            mr = std::max(mr, rows[i]);
            mc = std::max(mc, cols[i]);
        }
        from_triplets(t, mr + 1, mc + 1);
    }
    /* CSR constructor (addition): sorted, duplicate-free rows */
    SparseMatTMPL(slv_int n, const slv_int *row_ptr, const slv_int *col, const DType *val)
        : rp(row_ptr, row_ptr + n + 1), ci(col, col + row_ptr[n]), va(val, val + row_ptr[n]), nrows(n), ncols(n) {}

    void build(SparseBuilderTMPL<DType> &builder, bool to_square = false) {
        std::vector<typename SparseBuilderTMPL<DType>::Triplet> t;
        const slv_int size = builder.getSize();
        const slv_int max_retu = builder.build(t, to_square);
        from_triplets(t, size, max_retu);
    }

    slv_int getSize() const {
        if (nrows > (int64_t)std::numeric_limits<slv_int>::max())
            throw std::overflow_error("SparseMat size exceeds slv_int range");
        return (slv_int)nrows;
    }
    int64_t getTrueSize() const { return nrows; }
    slv_int getMaxCol() const { return ci.empty() ? 0 : *std::max_element(ci.begin(), ci.end()); }
    void getCols(slv_int *start, slv_int *end) const {
        for (int64_t i = 0; i < nrows; ++i) {
            start[i] = rp[i];
            end[i] = rp[i + 1];
        }
    }
    void getCols(std::vector<slv_int> &start, std::vector<slv_int> &end) const {
        start.resize(nrows);
        end.resize(nrows);
        getCols(start.data(), end.data());
    }
    const slv_int *rowPtr() const { return rp.data(); }
    slv_int *getColPtr() { return ci.data(); }
    const slv_int *getColPtr() const { return ci.data(); }
    DType *getValuePtr() {
        ver = next_version();  // the caller may write through it
        return va.data();
    }
    const DType *getValuePtr() const { return va.data(); }
    slv_int nonZeros() const { return (slv_int)ci.size(); }
    void resetMat() {
        std::fill(va.begin(), va.end(), DType{});
        ver = next_version();
    }
    uint64_t version() const { return ver; }
    int64_t getNumCols() const { return ncols; }  // (addition) column count

    /* coefficient += val, inserting the entry when the pattern lacks it (Eigen coeffRef) */
    void add(slv_int gyo, slv_int retu, DType val) {
        if (gyo < 0 || gyo >= nrows || retu < 0 || retu >= ncols)
            throw std::out_of_range("SparseMat::add: (row, column) outside the matrix");
        auto b = ci.begin() + rp[gyo], e = ci.begin() + rp[gyo + 1];
        auto it = std::lower_bound(b, e, retu);
        const size_t k = (size_t)(it - ci.begin());
        if (it != e && *it == retu) {
            va[k] += val;
        } else {
            ci.insert(it, retu);
            va.insert(va.begin() + k, DType{} + val);
            for (int64_t i = gyo + 1; i <= nrows; ++i) ++rp[i];
        }
        ver = next_version();
    }
    /* the storage is always compressed (Eigen makeCompressed is a no-op here) */
    void compressed() {}

    /* does row gyo hold column target_r? result_retu = its offset within the row (0 if not) */
    bool isInclude(slv_int gyo, slv_int target_r, slv_int &result_retu) const {
        if (gyo >= 0 && gyo < nrows)
            for (slv_int k = rp[gyo]; k < rp[gyo + 1]; ++k)
                if (ci[k] == target_r) {
                    result_retu = k - rp[gyo];
                    return true;
                }
        result_retu = 0;
        return false;
    }
    /* rows and values of the entries in column target, in row order */
    void getTargetRowVal(slv_int target, std::vector<slv_int> &row_pos, std::vector<DType> &row_val) const {
        row_pos.clear();
        row_val.clear();
        for (int64_t i = 0; i < nrows; ++i)
            for (slv_int k = rp[i]; k < rp[i + 1]; ++k)
                if (ci[k] == target) {
                    row_pos.push_back((slv_int)i);
                    row_val.push_back(va[k]);
                }
    }
    /* columns and values of the entries of row target */
    void getTargetColVal(slv_int target, std::vector<slv_int> &col_pos, std::vector<DType> &col_val) const {
        if (target < 0 || target >= nrows) throw std::out_of_range("SparseMat::getTargetColVal: row outside the matrix");
        col_pos.assign(ci.begin() + rp[target], ci.begin() + rp[target + 1]);
        col_val.assign(va.begin() + rp[target], va.begin() + rp[target + 1]);
    }
    /* drop the entries with |v| <= |thres| * 1e-12 (Eigen's pruned(thres) with its default
     * double precision 1e-12, src/SparseMat.cpp:288-291) */
    void prune(double thres) {
        const double cut = std::abs(thres) * 1e-12;
        slv_int w = 0;
        std::vector<slv_int> nrp(rp.size(), 0);
        for (int64_t i = 0; i < nrows; ++i) {
            for (slv_int k = rp[i]; k < rp[i + 1]; ++k)
                if (std::abs(va[k]) > cut) {
                    ci[w] = ci[k];
                    va[w] = va[k];
                    ++w;
                }
            nrp[i + 1] = w;
        }
        rp.swap(nrp);
        ci.resize(w);
        va.resize(w);
        ver = next_version();
    }
    /* the matrix as rows of dense text (with Eigen present: Eigen's own printout) */
    void print() const {
#if defined(EIGEN_SPARSECORE_MODULE_H)
        std::cout << Eigen::SparseMatrix<DType, Eigen::RowMajor>(mat()) << std::endl;
#else
        for (int64_t i = 0; i < nrows; ++i) {
            slv_int k = rp[i];
            for (int64_t j = 0; j < ncols; ++j) {
                const DType v = (k < rp[i + 1] && ci[k] == j) ? va[k++] : DType{};
                std::cout << v << (j + 1 < ncols ? " " : "");
            }
            std::cout << "\n";
        }
        std::cout << std::endl;
#endif
    }
    /* read the printMat format (src/SparseMat.cpp:353-409): the row count, the entries per
     * row, the columns of each row (-1 for an empty row), then the values row by row; the
     * column count is the largest column + 1 */
    void readMat(const std::string &filename) {
        std::ifstream fp(filename);
        if (!fp) throw std::runtime_error("SparseMat::readMat: cannot open " + filename);
        std::string w1, w2, w3;
        slv_int size = 0;
        fp >> w1 >> w2 >> w3 >> size;
        if (!fp || size < 0) throw std::runtime_error("SparseMat::readMat: bad header in " + filename);
        std::vector<slv_int> cnt(size);
        for (auto &c : cnt) fp >> c;
        fp >> w1 >> w2;
        std::vector<std::vector<slv_int>> cols(size);
        for (slv_int i = 0; i < size; ++i) {
            if (cnt[i] == 0) {
                slv_int skip;
                fp >> skip;
            } else {
                cols[i].resize(cnt[i]);
                for (auto &c : cols[i]) fp >> c;
            }
        }
        fp >> w1 >> w2 >> w3;
        SparseBuilderTMPL<DType> builder(size);
        for (slv_int i = 0; i < size; ++i)
            for (slv_int j = 0; j < cnt[i]; ++j) {
                DType v;
                fp >> v;
                builder.add(i, cols[i][j], v);
            }
        if (!fp) throw std::runtime_error("SparseMat::readMat: truncated file " + filename);
        std::vector<typename SparseBuilderTMPL<DType>::Triplet> t;
        const slv_int max_retu = builder.build(t, false);
        from_triplets(t, size, max_retu);
    }

#if defined(EIGEN_SPARSECORE_MODULE_H)
    using EigenMat = Eigen::SparseMatrix<DType, Eigen::RowMajor, slv_int>;
    /* from an Eigen row-major matrix (copied into CSR) */
    explicit SparseMatTMPL(const EigenMat &M) { setMatrix(EigenMat(M)); }
    /* from Eigen triplets: rows = largest row + 1, columns = largest column + 1, duplicates
     * summed (src/SparseMat.cpp:54-70) */
    explicit SparseMatTMPL(const std::vector<Eigen::Triplet<DType>> &sparse_data) {
        std::vector<typename SparseBuilderTMPL<DType>::Triplet> t;
        t.reserve(sparse_data.size());
        slv_int mr = 0, mc = 0;
        for (const auto &e : sparse_data) {
            t.push_back({(slv_int)e.row(), (slv_int)e.col(), e.value()});
            mr = std::max(mr, (slv_int)e.row());
            mc = std::max(mc, (slv_int)e.col());
        }
        from_triplets(t, mr + 1, mc + 1);
    }
    void setMatrix(EigenMat &&M) {
        M.makeCompressed();
        nrows = M.rows();
        ncols = M.cols();
        rp.assign(M.outerIndexPtr(), M.outerIndexPtr() + nrows + 1);
        ci.assign(M.innerIndexPtr(), M.innerIndexPtr() + M.nonZeros());
        va.assign(M.valuePtr(), M.valuePtr() + M.nonZeros());
        for (int64_t i = 0; i < nrows; ++i) {  // Eigen keeps inner indices sorted; make sure
            std::vector<std::pair<slv_int, DType>> row;
            for (slv_int k = rp[i]; k < rp[i + 1]; ++k) row.emplace_back(ci[k], va[k]);
            if (std::is_sorted(row.begin(), row.end(), [](const auto &a, const auto &b) { return a.first < b.first; }))
                continue;
            std::stable_sort(row.begin(), row.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
            for (slv_int k = rp[i]; k < rp[i + 1]; ++k) std::tie(ci[k], va[k]) = row[k - rp[i]];
        }
        ver = next_version();
    }
    /* the CSR arrays as an Eigen sparse matrix (a map: no copy) */
    Eigen::Map<EigenMat> mat() {
        ver = next_version();  // the caller may write coefficients through it
        return Eigen::Map<EigenMat>((typename EigenMat::Index)nrows, (typename EigenMat::Index)ncols,
                                    (typename EigenMat::Index)ci.size(), rp.data(), ci.data(), va.data());
    }
    Eigen::Map<const EigenMat> mat() const {
        return Eigen::Map<const EigenMat>((typename EigenMat::Index)nrows, (typename EigenMat::Index)ncols,
                                          (typename EigenMat::Index)ci.size(), rp.data(), ci.data(), va.data());
    }
#endif
    void printMat(const std::string &str = "Mat.csv") const {
        std::ofstream fp(str);
        fp << "Column size : " << nrows << "\n";
        for (int64_t i = 0; i < nrows; ++i) fp << rp[i + 1] - rp[i] << "\n";
        fp << "Column : \n";
        for (int64_t i = 0; i < nrows; ++i) {
            if (rp[i + 1] == rp[i]) fp << "-1";
            for (slv_int k = rp[i]; k < rp[i + 1]; ++k) fp << ci[k] << " ";
            fp << "\n";
        }
        fp << "Mat value : \n";
        fp << std::scientific;
        for (int64_t i = 0; i < nrows; ++i) {
            for (slv_int k = rp[i]; k < rp[i + 1]; ++k) fp << va[k] << " ";
            fp << "\n";
        }
    }

   private:
    void from_triplets(std::vector<typename SparseBuilderTMPL<DType>::Triplet> &t, int64_t nr, int64_t nc) {
        for (const auto &e : t)
            if (e.row < 0 || e.col < 0 || e.row >= nr || e.col >= nc)
                throw std::out_of_range("SparseMat: negative or out-of-range index");
        std::stable_sort(t.begin(), t.end(), [](const auto &a, const auto &b) {
            return a.row != b.row ? a.row < b.row : a.col < b.col;
        });
        nrows = nr;
        ncols = nc;
        rp.assign(nr + 1, 0);
        ci.clear();
        va.clear();
        for (size_t k = 0; k < t.size(); ++k) {
            if (!ci.empty() && k > 0 && t[k].row == t[k - 1].row && t[k].col == t[k - 1].col) {
                va.back() += t[k].val;
                continue;
            }
            ci.push_back(t[k].col);
            va.push_back(t[k].val);
            rp[t[k].row + 1]++;
        }
        std::partial_sum(rp.begin(), rp.end(), rp.begin());
        ver = next_version();
    }
    std::vector<slv_int> rp, ci;
    std::vector<DType> va;
    int64_t nrows = 0, ncols = 0;
    uint64_t ver = next_version();
    static uint64_t next_version() {
        static std::atomic<uint64_t> counter{0};
        return ++counter;
    }
};

using SparseMat = SparseMatTMPL<double>;
using SparseMatC = SparseMatTMPL<dcomplex>;

}  // namespace SparseSolv
}  // namespace JPMRspace

#endif
