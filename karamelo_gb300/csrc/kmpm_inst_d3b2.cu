// Instantiates the step kernels for 3-D, Bernstein-quadratic basis.
#include "kmpm_step_impl.cuh"
namespace kmpm { void get_step_kernels_3_2(StepKernels &k) { fill_step_kernels<3, 2>(k); } }
