/*
 * SparseMat.hpp -- drop-in for SparseMatTMPL / SparseMat / SparseMatC
 * (include/SparseSolv/SparseMat.hpp:49-136 of SparseSolv).
 *
 * Storage is row-major CSR with sorted columns and summed duplicates, the
 * layout of Eigen::SparseMatrix<T, RowMajor> after setFromTriplets
 * (src/SparseMat.cpp:54-122). Eigen itself is not a dependency here: the
 * reference's mat() accessor is replaced by rowPtr()/getColPtr()/
 * getValuePtr(); getCols, getSize, getMaxCol, resetMat and printMat keep
 * their meaning. Every mutation bumps version(), which the solvers use to
 * decide when the device copy and its factor must be refreshed.
 */
#ifndef SPARSESOLV_GB300_SPARSEMAT_HPP
#define SPARSESOLV_GB300_SPARSEMAT_HPP

#include <algorithm>
#include <cstdint>
#include <fstream>
#include <limits>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "SparseBuilder.hpp"

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
        ++ver;  // the caller may write through it
        return va.data();
    }
    const DType *getValuePtr() const { return va.data(); }
    slv_int nonZeros() const { return (slv_int)ci.size(); }
    void resetMat() {
        std::fill(va.begin(), va.end(), DType{});
        ++ver;
    }
    uint64_t version() const { return ver; }
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
        ++ver;
    }
    std::vector<slv_int> rp, ci;
    std::vector<DType> va;
    int64_t nrows = 0, ncols = 0;
    uint64_t ver = 0;
};

using SparseMat = SparseMatTMPL<double>;
using SparseMatC = SparseMatTMPL<dcomplex>;

}  // namespace SparseSolv
}  // namespace JPMRspace

#endif
