/*
 * MatSolverMRTR.hpp -- drop-in for MatSolverMRTR (include/SparseSolv/
 * MatSolverMRTR.hpp:36-88 of SparseSolv): precondition type 0 = shifted IC
 * (src/MatSolverMRTR_ICver.cpp), 1 = Eisenstat SGS (default,
 * src/MatSolverMRTR_SGSver.cpp). The reference's file names
 * MatSolverMRTR_ICver / _SGSver are not classes; the aliases below name the
 * two variants for callers that want them spelled out.
 */
#ifndef SPARSESOLV_GB300_MATSOLVERMRTR_HPP
#define SPARSESOLV_GB300_MATSOLVERMRTR_HPP

#include "MatSolverBase.hpp"

namespace JPMRspace {
namespace SparseSolv {

class MatSolverMRTR : public MatSolverBase {
   public:
    MatSolverMRTR() = default;
    ~MatSolverMRTR() override = default;
    void setAccelFactor(double accel_factor0) { accel_factor = accel_factor0; }
    void setPreconditionType(int precondition_type0) { precondition_type = precondition_type0; }

   protected:
    int method() const override { return SSG_METHOD_MRTR; }
    double accel() const override { return accel_factor; }
    int ptype() const override { return precondition_type; }

   private:
    double accel_factor = 1.05;
    int precondition_type = 1;
};

/* MRTR with the shifted IC preconditioner */
class MatSolverMRTR_ICver : public MatSolverMRTR {
   public:
    MatSolverMRTR_ICver() { setPreconditionType(0); }
};
/* MRTR with the Eisenstat SGS preconditioner */
class MatSolverMRTR_SGSver : public MatSolverMRTR {
   public:
    MatSolverMRTR_SGSver() { setPreconditionType(1); }
};

}  // namespace SparseSolv
}  // namespace JPMRspace

#endif
