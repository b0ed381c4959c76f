// ref_basis_harness.cpp -- exposes the reference's own 1-D basis functions
// (src/basis_functions.h, compiled unmodified from the Karamelo source tree)
// through a C ABI, so that the oracle's restatement can be pinned against
// them.  Test infrastructure: built by oracle/Makefile into oracle/_ref/.
#include <cmath>
#include "basis_functions.h"

extern "C" double ref_basis(int basis, int kind, double r, int ntype, double icellsize) {
  using namespace BasisFunction;
  switch (basis) {
    case 0: return kind ? derivative_linear(r, ntype, icellsize) : linear(r, ntype);
    case 1: return kind ? derivative_cubic_spline(r, ntype, icellsize) : cubic_spline(r, ntype);
    case 2: return kind ? derivative_bernstein_quadratic(r, ntype, icellsize) : bernstein_quadratic(r, ntype);
    default: return kind ? derivative_quadratic_spline(r, ntype, icellsize) : quadratic_spline(r, ntype);
  }
}
