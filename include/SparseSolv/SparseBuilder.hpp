/*
 * SparseBuilder.hpp -- drop-in for SparseBuilderTMPL / SparseBuilder /
 * SparseBuilderC (include/SparseSolv/SparseBuilder.hpp:53-121 of SparseSolv):
 * a row-wise map accumulator. add() is +=; build() emits triplets sorted by
 * (row, column), empties the builder, and with to_square pads (n-1, n-1)
 * with a zero when the largest column is below the row count
 * (src/SparseBuilder.cpp:107-141).
 */
#ifndef SPARSESOLV_GB300_BUILDER_HPP
#define SPARSESOLV_GB300_BUILDER_HPP

#include <map>
#include <stdexcept>
#include <tuple>
#include <vector>

#include "SparseTypeDefine.hpp"

namespace JPMRspace {
namespace SparseSolv {

template <typename DType>
class SparseBuilderTMPL {
   public:
    struct Triplet {
        slv_int row, col;
        DType val;
    };
    SparseBuilderTMPL() = default;
    explicit SparseBuilderTMPL(slv_int size0) { initialize(size0); }
    slv_int getSize() const { return size; }
    void initialize(slv_int ss) {
        size = ss;
        initialize();
    }
    void initialize() { tempMat.assign(size, std::map<slv_int, DType>()); }
    void reInitialize(slv_int new_size) { initialize(new_size); }
    void resetMat() {
        for (auto &row : tempMat)
            for (auto &kv : row) kv.second = DType{};
    }
    void add(slv_int gyo, slv_int retu, DType val) {
        if (gyo < 0 || gyo >= size) throw std::out_of_range("SparseBuilder::add: row out of range");
        tempMat[gyo][retu] += val;
    }
    /* emits (row, col, val) in row-major order and empties the builder; returns max column + 1 */
    slv_int build(std::vector<Triplet> &list, bool to_square) {
        slv_int max_retu = 0;
        list.clear();
        for (slv_int i = 0; i < size; ++i) {
            for (const auto &kv : tempMat[i]) {
                list.push_back(Triplet{i, kv.first, kv.second});
                if (kv.first > max_retu) max_retu = kv.first;
            }
            std::map<slv_int, DType>().swap(tempMat[i]);
        }
        ++max_retu;
        if (to_square && max_retu < size) {
            list.push_back(Triplet{size - 1, size - 1, DType{}});
            max_retu = size;
        }
        return max_retu;
    }

   private:
    slv_int size = 0;
    std::vector<std::map<slv_int, DType>> tempMat;
};

using SparseBuilder = SparseBuilderTMPL<double>;
using SparseBuilderC = SparseBuilderTMPL<dcomplex>;

}  // namespace SparseSolv
}  // namespace JPMRspace

#endif
