// Instantiates the step kernels for 2-D, cubic B-spline basis.
#include "kmpm_step_impl.cuh"
namespace kmpm { void get_step_kernels_2_1(StepKernels &k) { fill_step_kernels<2, 1>(k); } }
