// Instantiates the step kernels for 2-D, all bases.
#include "kmpm_step_impl.cuh"
namespace kmpm {
void get_step_kernels_2_0(StepKernels &k) { fill_step_kernels<2, 0>(k); }
void get_step_kernels_2_1(StepKernels &k) { fill_step_kernels<2, 1>(k); }
void get_step_kernels_2_2(StepKernels &k) { fill_step_kernels<2, 2>(k); }
void get_step_kernels_2_3(StepKernels &k) { fill_step_kernels<2, 3>(k); }
}
