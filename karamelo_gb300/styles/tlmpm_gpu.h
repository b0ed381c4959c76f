/* tlmpm_gpu.h -- Karamelo method style `tlmpm/gpu`: TLMPM whose time steps
 * run on the GPU through libkmpm.so (include/kmpm.h).
 *
 * Registered with MethodStyle (the style_method.h registry,
 * src/update.cpp:119-124).  setup() runs TLMPM::setup (basis, flags) and then
 * hands the run loop to SchemeGPU (scheme_gpu.h) in place of the CPU scheme,
 * so a script only changes `method(tlmpm, ...)` to `method(tlmpm/gpu, ...)`.
 * The per-phase entry points of Method are not used by SchemeGPU; reaching
 * one means a CPU scheme was installed after this method (a later scheme()
 * command), which stops the run with an error. */
#ifdef METHOD_CLASS

MethodStyle(tlmpm/gpu, TLMPMGPU)

#else

#ifndef KMPM_STYLE_TLMPM_GPU_H
#define KMPM_STYLE_TLMPM_GPU_H

#include "tlmpm.h"

class TLMPMGPU : public TLMPM {
 public:
  TLMPMGPU(class MPM *mpm) : TLMPM(mpm) {}
  void setup(vector<string> args) override;
  void compute_grid_weight_functions_and_gradients() override;
};

#endif
#endif
