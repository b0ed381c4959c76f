// Instantiates the step kernels for 3-D, cubic B-spline basis.
#include "kmpm_step_impl.cuh"
namespace kmpm { void get_step_kernels_3_1(StepKernels &k) { fill_step_kernels<3, 1>(k); } }
