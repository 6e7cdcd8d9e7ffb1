/*
 * SparseTypeDefine.hpp -- drop-in for the reference header of the same name
 * (include/SparseSolv/SparseTypeDefine.hpp:24-41 of SparseSolv): the
 * JPMRspace::SparseSolv namespace, slv_int and dcomplex.
 */
#ifndef SPARSESOLV_GB300_TYPEDEFINE_HPP
#define SPARSESOLV_GB300_TYPEDEFINE_HPP

#include <complex>

namespace JPMRspace {
using dcomplex = std::complex<double>;
namespace SparseSolv {
using slv_int = int;
}  // namespace SparseSolv
}  // namespace JPMRspace

#endif
