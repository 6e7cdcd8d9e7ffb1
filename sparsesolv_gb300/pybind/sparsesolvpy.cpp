// sparsesolvpy.cpp -- the compiled Python module SparseSolvPy: pybind11 bindings of
// the C++ drop-in classes of include/SparseSolv/ (builders, matrices, ICCG and MRTR
// solvers), which in turn run on the GPU through the C ABI of libsparsesolv_gb300.
//
// Same classes, method names, argument names and defaults as the reference's module
// (pybind/pybind.cpp:16-139 of SparseSolv):
//   SparseBuilder(size)   getSize, initialize, reInitialize, add, resetMat
//   SparseBuilderC(size)  get_size (sic), initialize, reInitialize, add, resetMat
//   SparseMat / SparseMatC  (), (builder, to_square=True), (n_nonzero, rows, cols, vals);
//                         getSize, getMaxCol, print_mat(filename="Mat.csv")
//   MatSolverBase         setInitSolution, setDiagScale, setSaveBest, setSaveLog,
//                         setDirvegeType (sic), setBadDivVal, setBadDivCount,
//                         setConvNormalizeType, setConvNormalizeConst, getResidualLog
//   MatSolverICCG         setAccelFactor, solve_real, solve_complex
//   MatSolverMRTR         setAccelFactor, setPreconditionType, solve_real, solve_complex
// solve_real / solve_complex(conv_cri, max_ite, A, b, x0) return (converged, x) with x a
// new array (x0 is the initial guess after setInitSolution(False)), as the reference's
// lambdas do with their by-value Eigen x0.
//
// Additions: builders' addMany(rows, cols, vals); matrices' shape, row_ptr, col, val,
// from_csr, add, isInclude, getTargetRowVal, getTargetColVal, prune, readMat, print;
// solvers' getIterations, getTimings, getAccelUsed, options, setDevice, setPrecision,
// setReferenceQuirks. Solves release the GIL.
#include <pybind11/complex.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <complex>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "SparseSolv/MatSolverICCG.hpp"
#include "SparseSolv/MatSolverMRTR.hpp"
#include "SparseSolv/SparseBuilder.hpp"
#include "SparseSolv/SparseMat.hpp"

namespace py = pybind11;
using namespace JPMRspace;
using namespace JPMRspace::SparseSolv;

namespace {

template <typename T>
using carr = py::array_t<T, py::array::c_style | py::array::forcecast>;

template <typename T>
py::array_t<T> to_numpy(const T *p, size_t n) {
    py::array_t<T> a(n);
    if (n) std::memcpy(a.mutable_data(), p, sizeof(T) * n);
    return a;
}

template <typename DType>
void bind_builder(py::module_ &m, const char *name, const char *size_name) {
    using B = SparseBuilderTMPL<DType>;
    py::class_<B>(m, name)
        .def(py::init<slv_int>(), py::arg("size"))
        .def(size_name, &B::getSize)
        .def("initialize", py::overload_cast<slv_int>(&B::initialize), py::arg("size"))
        .def("reInitialize", &B::reInitialize, py::arg("size"))
        .def("add", &B::add, py::arg("row"), py::arg("col"), py::arg("val"))
        .def("resetMat", &B::resetMat)
        .def(
            "addMany",
            [](B &b, carr<slv_int> rows, carr<slv_int> cols, carr<DType> vals) {
                const size_t n = (size_t)rows.size();
                if ((size_t)cols.size() != n || (size_t)vals.size() != n)
                    throw std::invalid_argument("addMany: rows, cols and vals differ in length");
                const slv_int *r = rows.data(), *c = cols.data();
                const DType *v = vals.data();
                for (size_t k = 0; k < n; ++k) b.add(r[k], c[k], v[k]);
            },
            py::arg("rows"), py::arg("cols"), py::arg("vals"),
            "(addition) add() over arrays of entries, in order");
}

template <typename DType>
void bind_mat(py::module_ &m, const char *name) {
    using M = SparseMatTMPL<DType>;
    py::class_<M>(m, name)
        .def(py::init<>())
        .def(py::init<SparseBuilderTMPL<DType> &, bool>(), py::arg("builder"), py::arg("to_square") = true)
        .def(py::init<slv_int, const std::vector<slv_int> &, const std::vector<slv_int> &,
                      const std::vector<DType> &>(),
             py::arg("n_nonzero"), py::arg("rows"), py::arg("cols"), py::arg("vals"))
        .def("getSize", &M::getSize)
        .def("getMaxCol", &M::getMaxCol)
        .def("print_mat", &M::printMat, py::arg("filename") = "Mat.csv")
        // additions
        .def_static(
            "from_csr",
            [](carr<slv_int> row_ptr, carr<slv_int> col, carr<DType> val) {
                const slv_int n = (slv_int)row_ptr.size() - 1;
                if (n < 0) throw std::invalid_argument("from_csr: empty row_ptr");
                const slv_int *rp = row_ptr.data();
                if (rp[0] != 0 || (size_t)rp[n] != (size_t)col.size() || col.size() != val.size())
                    throw std::invalid_argument("from_csr: row_ptr does not match col/val");
                for (slv_int i = 0; i < n; ++i)
                    if (rp[i + 1] < rp[i]) throw std::invalid_argument("from_csr: row_ptr decreases");
                const slv_int *ci = col.data();
                for (slv_int i = 0; i < n; ++i)
                    for (slv_int k = rp[i]; k < rp[i + 1]; ++k)
                        if (ci[k] < 0 || ci[k] >= n || (k > rp[i] && ci[k] <= ci[k - 1]))
                            throw std::invalid_argument("from_csr: columns must be ascending, unique and in range");
                return M(n, rp, ci, val.data());
            },
            py::arg("row_ptr"), py::arg("col"), py::arg("val"),
            "(addition) a square matrix from sorted, duplicate-free CSR arrays")
        .def_property_readonly("shape", [](const M &a) { return py::make_tuple(a.getTrueSize(), a.getNumCols()); })
        .def_property_readonly("row_ptr", [](const M &a) { return to_numpy(a.rowPtr(), (size_t)a.getTrueSize() + 1); })
        .def_property_readonly("col", [](const M &a) { return to_numpy(a.getColPtr(), (size_t)a.nonZeros()); })
        .def_property_readonly("val", [](const M &a) { return to_numpy(a.getValuePtr(), (size_t)a.nonZeros()); })
        .def("nonZeros", &M::nonZeros)
        .def("add", &M::add, py::arg("row"), py::arg("col"), py::arg("val"))
        .def("compressed", &M::compressed)
        .def(
            "isInclude",
            [](const M &a, slv_int row, slv_int col) {
                slv_int pos = 0;
                const bool in = a.isInclude(row, col, pos);
                return py::make_tuple(in, pos);
            },
            py::arg("row"), py::arg("col"))
        .def(
            "getTargetRowVal",
            [](const M &a, slv_int target) {
                std::vector<slv_int> pos;
                std::vector<DType> val;
                a.getTargetRowVal(target, pos, val);
                return py::make_tuple(pos, val);
            },
            py::arg("target"))
        .def(
            "getTargetColVal",
            [](const M &a, slv_int target) {
                std::vector<slv_int> pos;
                std::vector<DType> val;
                a.getTargetColVal(target, pos, val);
                return py::make_tuple(pos, val);
            },
            py::arg("target"))
        .def("prune", &M::prune, py::arg("thres"))
        .def("readMat", &M::readMat, py::arg("filename"))
        .def("print", &M::print);
}

template <class S, class M, typename DType>
py::tuple solve_one(S &self, double conv_cri, int max_ite, const M &A, carr<DType> b, carr<DType> x0) {
    const size_t n = (size_t)A.getSize();
    if ((size_t)b.size() != n || (size_t)x0.size() != n)
        throw std::invalid_argument("SparseSolvPy: vector size does not match the matrix");
    py::array_t<DType> x(n);
    if (n) std::memcpy(x.mutable_data(), x0.data(), sizeof(DType) * n);
    const DType *bp = b.data();
    DType *xp = x.mutable_data();
    bool ok;
    {
        py::gil_scoped_release unlocked;
        ok = self.solve(conv_cri, max_ite, A, bp, xp);
    }
    return py::make_tuple(ok, x);
}

template <class S, class Cls>
void bind_solve(Cls &c) {
    c.def("setAccelFactor", &S::setAccelFactor)
        .def(
            "solve_real",
            [](S &self, double conv_cri, int max_ite, const SparseMat &A, carr<double> b, carr<double> x0) {
                return solve_one<S, SparseMat, double>(self, conv_cri, max_ite, A, b, x0);
            },
            py::arg("conv_cri"), py::arg("max_ite"), py::arg("A"), py::arg("b"), py::arg("x0"))
        .def(
            "solve_complex",
            [](S &self, double conv_cri, int max_ite, const SparseMatC &A, carr<dcomplex> b, carr<dcomplex> x0) {
                return solve_one<S, SparseMatC, dcomplex>(self, conv_cri, max_ite, A, b, x0);
            },
            py::arg("conv_cri"), py::arg("max_ite"), py::arg("A"), py::arg("b"), py::arg("x0"));
}

py::dict options_dict(const MatSolverBase &s) {
    const ssg_options o = s.getOptions();
    py::dict d;
    d["is_init"] = o.is_init;
    d["is_diag_scale"] = o.is_diag_scale;
    d["is_save_best"] = o.is_save_best;
    d["is_save_residual_log"] = o.is_save_residual_log;
    d["diverge_judge_type"] = o.diverge_judge_type;
    d["bad_div_val"] = o.bad_div_val;
    d["bad_div_count_thres"] = o.bad_div_count_thres;
    d["conv_normalize_type"] = o.conv_normalize_type;
    d["conv_normalize_const"] = o.conv_normalize_const;
    d["accel_factor"] = o.accel_factor;
    d["precondition_type"] = o.precondition_type;
    d["precision"] = o.precision;
    d["mrtr_reference_quirks"] = o.mrtr_reference_quirks;
    return d;
}

}  // namespace

PYBIND11_MODULE(SparseSolvPy, m) {
    m.doc() = "SparseSolv bindings: GB300 (sm_103a) shifted ICCG / ICCOCG / MRTR through libsparsesolv_gb300";

    bind_builder<double>(m, "SparseBuilder", "getSize");
    bind_builder<dcomplex>(m, "SparseBuilderC", "get_size");
    bind_mat<double>(m, "SparseMat");
    bind_mat<dcomplex>(m, "SparseMatC");

    py::class_<MatSolverBase>(m, "MatSolverBase")
        .def("setInitSolution", &MatSolverBase::setInitSolution)
        .def("setDiagScale", &MatSolverBase::setDiagScale)
        .def("setSaveBest", &MatSolverBase::setSaveBest)
        .def("setSaveLog", &MatSolverBase::setSaveLog)
        .def("setDirvegeType", &MatSolverBase::setDirvegeType)
        .def("setBadDivVal", &MatSolverBase::setBadDivVal)
        .def("setBadDivCount", &MatSolverBase::setBadDivCount)
        .def("setConvNormalizeType", &MatSolverBase::setConvNormalizeType)
        .def("setConvNormalizeConst", &MatSolverBase::setConvNormalizeConst)
        .def("getResidualLog",
             [](MatSolverBase &self) {
                 std::vector<double> log;
                 self.getResidualLog(log);
                 return log;
             })
        // additions
        .def("setDevice", &MatSolverBase::setDevice, py::arg("device"))
        .def("setPrecision", &MatSolverBase::setPrecision, py::arg("mode"),
             "0 = FP64 throughout (default), 1 = FP32 inner loop with FP64 refinement")
        .def("setReferenceQuirks", &MatSolverBase::setReferenceQuirks, py::arg("bl"),
             "reproduce the reference's IC-MRTR p update and MRTR warm start")
        .def("getIterations", &MatSolverBase::getIterations)
        .def("getTimings",
             [](const MatSolverBase &self) {
                 const std::vector<double> t = self.getTimings();
                 return py::make_tuple(t[0], t[1]);
             },
             "(setup + factor ms, iterations ms) of the last solve")
        .def("getAccelUsed", &MatSolverBase::getAccelUsed)
        .def_property_readonly("options", &options_dict, "the settings the next solve uses");

    py::class_<MatSolverICCG, MatSolverBase> iccg(m, "MatSolverICCG");
    iccg.def(py::init<>());
    bind_solve<MatSolverICCG>(iccg);

    py::class_<MatSolverMRTR, MatSolverBase> mrtr(m, "MatSolverMRTR");
    mrtr.def(py::init<>()).def("setPreconditionType", &MatSolverMRTR::setPreconditionType);
    bind_solve<MatSolverMRTR>(mrtr);
}
