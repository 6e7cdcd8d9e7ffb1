// Exercises the SparseMat drop-in (include/SparseSolv/SparseMat.hpp) without a GPU:
// add, compressed, isInclude, getTargetRowVal/ColVal, prune, printMat -> readMat,
// and, when compiled with -DWITH_EIGEN against an Eigen checkout, the Eigen
// triplet and matrix constructors, setMatrix and mat(). Prints one line per
// check ("name value ..."); tests/test_sparsemat_api.py compares them with
// scipy on the same matrix.
#ifdef WITH_EIGEN
#include <Eigen/Sparse>
#endif
#include <complex>
#include <cstdio>
#include <string>
#include <vector>

#include "SparseSolv/SparseMat.hpp"

using namespace JPMRspace;
using namespace JPMRspace::SparseSolv;

template <typename M>
static void dump(const char *name, const M &A) {
    std::printf("%s %d %d", name, (int)A.getSize(), (int)A.nonZeros());
    for (int i = 0; i <= A.getSize(); ++i) std::printf(" %d", A.rowPtr()[i]);
    for (int k = 0; k < A.nonZeros(); ++k) std::printf(" %d", A.getColPtr()[k]);
    std::printf("\n");
}

static void dump_vals(const char *name, const SparseMat &A) {
    std::printf("%s", name);
    for (int k = 0; k < A.nonZeros(); ++k) std::printf(" %.17g", A.getValuePtr()[k]);
    std::printf("\n");
}

int main(int argc, char **argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    // 5 x 5: duplicates summed, (4, 4) missing until add() inserts it
    SparseMat A(9, {0, 0, 1, 1, 2, 3, 4, 0, 2}, {0, 1, 1, 3, 2, 3, 0, 0, 4},
                {4.0, -1.0, 3.0, 0.5, 2.0, 1e-20, 7.0, 1.0, 1.5});
    dump("coo", A);
    dump_vals("coo_val", A);
    const uint64_t v0 = A.version();
    A.add(4, 4, 6.0);  // inserted
    A.add(1, 1, 0.25);  // existing
    A.add(4, 2, -2.0);  // inserted before (4, 4)
    A.compressed();
    std::printf("add_version %d\n", A.version() > v0 ? 1 : 0);
    dump("add", A);
    dump_vals("add_val", A);
    slv_int pos = -1;
    const bool in1 = A.isInclude(1, 3, pos);
    std::printf("isInclude13 %d %d\n", in1 ? 1 : 0, pos);
    const bool in2 = A.isInclude(2, 0, pos);
    std::printf("isInclude20 %d %d\n", in2 ? 1 : 0, pos);
    std::vector<slv_int> idx;
    std::vector<double> val;
    A.getTargetRowVal(0, idx, val);  // entries of column 0
    std::printf("col0");
    for (size_t k = 0; k < idx.size(); ++k) std::printf(" %d %.17g", idx[k], val[k]);
    std::printf("\n");
    A.getTargetColVal(4, idx, val);  // entries of row 4
    std::printf("row4");
    for (size_t k = 0; k < idx.size(); ++k) std::printf(" %d %.17g", idx[k], val[k]);
    std::printf("\n");
    // printMat -> readMat round trip, real and complex
    A.printMat(dir + "/A.csv");
    SparseMat B;
    B.readMat(dir + "/A.csv");
    dump("read", B);
    dump_vals("read_val", B);
    SparseMatC C(3, {0, 1, 2}, {0, 2, 1}, {dcomplex(1.5, -2.0), dcomplex(0.0, 3.0), dcomplex(-4.0, 0.25)});
    C.printMat(dir + "/C.csv");
    SparseMatC D;
    D.readMat(dir + "/C.csv");
    dump("readc", D);
    std::printf("readc_val");
    for (int k = 0; k < D.nonZeros(); ++k) std::printf(" %.17g %.17g", D.getValuePtr()[k].real(), D.getValuePtr()[k].imag());
    std::printf("\n");
    // prune(1.0): entries with |v| <= 1e-12 go (the 1e-20 one)
    A.prune(1.0);
    dump("prune", A);
#ifdef WITH_EIGEN
    // triplets: rows = largest row + 1, columns = largest column + 1, duplicates summed
    std::vector<Eigen::Triplet<double>> t{{0, 0, 4.0}, {1, 1, 3.0}, {0, 1, -1.0}, {1, 0, -1.0},
                                          {0, 0, 1.0}, {2, 2, 5.0}, {2, 1, 0.5}};
    SparseMat E(t);
    dump("trip", E);
    dump_vals("trip_val", E);
    Eigen::VectorXd x(3);
    x << 1.0, -2.0, 0.5;
    Eigen::VectorXd y = E.mat() * x;
    std::printf("matvec %.17g %.17g %.17g\n", y[0], y[1], y[2]);
    Eigen::SparseMatrix<double, Eigen::RowMajor> Lo = E.mat().triangularView<Eigen::Lower>();
    Eigen::SparseMatrix<double, Eigen::RowMajor> Tr = E.mat().transpose();
    std::printf("lower_nnz %d transpose01 %.17g\n", (int)Lo.nonZeros(), Tr.coeff(0, 1));
    const uint64_t ve = E.version();
    E.mat().coeffRef(2, 2) = 9.0;  // write through the map
    std::printf("write %.17g version %d\n", E.getValuePtr()[E.nonZeros() - 1], E.version() > ve ? 1 : 0);
    Eigen::SparseMatrix<double, Eigen::RowMajor> M(2, 4);
    M.insert(1, 3) = 2.0;
    M.insert(0, 2) = -1.0;
    M.insert(1, 0) = 8.0;
    SparseMat F(M);
    dump("eigen", F);
    dump_vals("eigen_val", F);
    std::printf("eigen_cols %d\n", (int)F.getNumCols());
    SparseMat G;
    G.setMatrix(std::move(M));
    dump("setmatrix", G);
    const SparseMat &Gc = G;
    std::printf("const_mat %d %d %d\n", (int)Gc.mat().rows(), (int)Gc.mat().cols(), (int)Gc.mat().nonZeros());
#endif
    return 0;
}
