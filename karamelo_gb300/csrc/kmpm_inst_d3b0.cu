// Instantiates the step kernels for 3-D, linear basis.
#include "kmpm_step_impl.cuh"
namespace kmpm { void get_step_kernels_3_0(StepKernels &k) { fill_step_kernels<3, 0>(k); } }
