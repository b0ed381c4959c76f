// Instantiates the step kernels for 3-D, quadratic B-spline basis.
#include "kmpm_step_impl.cuh"
namespace kmpm { void get_step_kernels_3_3(StepKernels &k) { fill_step_kernels<3, 3>(k); } }
