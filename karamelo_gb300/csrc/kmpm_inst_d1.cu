// Instantiates the step kernels for 1-D, all bases.
#include "kmpm_step_impl.cuh"
namespace kmpm {
void get_step_kernels_1_0(StepKernels &k) { fill_step_kernels<1, 0>(k); }
void get_step_kernels_1_1(StepKernels &k) { fill_step_kernels<1, 1>(k); }
void get_step_kernels_1_2(StepKernels &k) { fill_step_kernels<1, 2>(k); }
void get_step_kernels_1_3(StepKernels &k) { fill_step_kernels<1, 3>(k); }
}
