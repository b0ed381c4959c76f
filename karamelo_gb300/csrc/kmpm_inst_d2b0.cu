// Instantiates the step kernels for 2-D, linear basis.
#include "kmpm_step_impl.cuh"
namespace kmpm { void get_step_kernels_2_0(StepKernels &k) { fill_step_kernels<2, 0>(k); } }
