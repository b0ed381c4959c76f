// Instantiates the step kernels for 2-D, quadratic B-spline basis.
#include "kmpm_step_impl.cuh"
namespace kmpm { void get_step_kernels_2_3(StepKernels &k) { fill_step_kernels<2, 3>(k); } }
