// Uses the C++ drop-in headers exactly as the reference's example driver uses
// the reference (examples/VoxelFEM/main.cpp:143-161 of SparseSolv): build a
// matrix with SparseBuilder, solve with MatSolverICCG and MatSolverMRTR, read
// the residual log. Matrix and right-hand side come from a CSR file written by
// the test (n, nnz, row_ptr, col, val, b as raw binary).
#include <SparseSolv/MatSolverICCG.hpp>
#include <SparseSolv/MatSolverMRTR.hpp>

#include <cmath>
#include <cstdio>
#include <fstream>
#include <vector>

using namespace JPMRspace::SparseSolv;

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    std::ifstream f(argv[1], std::ios::binary);
    int n = 0, nnz = 0;
    f.read((char *)&n, 4);
    f.read((char *)&nnz, 4);
    std::vector<int> rp(n + 1), ci(nnz);
    std::vector<double> va(nnz), b(n);
    f.read((char *)rp.data(), 4 * (n + 1));
    f.read((char *)ci.data(), 4 * nnz);
    f.read((char *)va.data(), 8 * nnz);
    f.read((char *)b.data(), 8 * n);
    SparseBuilder builder(n);
    for (int i = 0; i < n; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) builder.add(i, ci[k], va[k]);
    SparseMat A(builder);
    std::vector<double> x(n, 0.0);
    MatSolverICCG iccg;
    iccg.setSaveLog(true);
    iccg.setAccelFactor(1.1);
    const bool ok1 = iccg.solve(1.0e-8, 10000, A, b.data(), x.data());
    std::vector<double> log;
    iccg.getResidualLog(log);
    std::vector<double> x2(n, 0.0);
    MatSolverMRTR mrtr;  // default: Eisenstat SGS
    mrtr.setSaveLog(true);
    const bool ok2 = mrtr.solve(1.0e-8, 10000, A, b, x2);
    std::vector<double> log2;
    mrtr.getResidualLog(log2);
    std::printf("%d %d %d %d %.17g %.17g\n", ok1 ? 1 : 0, (int)log.size() - 1, ok2 ? 1 : 0, (int)log2.size() - 1,
                x[n / 2], x2[n / 2]);
    return (ok1 && ok2) ? 0 : 1;
}
