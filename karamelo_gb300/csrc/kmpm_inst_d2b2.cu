// Instantiates the step kernels for 2-D, Bernstein-quadratic basis.
#include "kmpm_step_impl.cuh"
namespace kmpm { void get_step_kernels_2_2(StepKernels &k) { fill_step_kernels<2, 2>(k); } }
