/*
 * MatSolverICCG.hpp -- drop-in for MatSolverICCG (shifted ICCG / ICCOCG,
 * include/SparseSolv/MatSolverICCG.hpp:36-76 of SparseSolv; default
 * acceleration factor 1.05, negative = automatic search).
 */
#ifndef SPARSESOLV_GB300_MATSOLVERICCG_HPP
#define SPARSESOLV_GB300_MATSOLVERICCG_HPP

#include "MatSolverBase.hpp"

namespace JPMRspace {
namespace SparseSolv {

class MatSolverICCG : public MatSolverBase {
   public:
    MatSolverICCG() = default;
    ~MatSolverICCG() override = default;
    void setAccelFactor(double accel_factor0) { accel_factor = accel_factor0; }

   protected:
    int method() const override { return SSG_METHOD_ICCG; }
    double accel() const override { return accel_factor; }

   private:
    double accel_factor = 1.05;
};

}  // namespace SparseSolv
}  // namespace JPMRspace

#endif
