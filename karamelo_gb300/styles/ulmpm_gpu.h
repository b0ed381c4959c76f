/* ulmpm_gpu.h -- Karamelo method style `ulmpm/gpu`: ULMPM whose time steps
 * run on the GPU through libkmpm.so (include/kmpm.h).  Same design as
 * tlmpm_gpu.h over ULMPM. */
#ifdef METHOD_CLASS

MethodStyle(ulmpm/gpu, ULMPMGPU)

#else

#ifndef KMPM_STYLE_ULMPM_GPU_H
#define KMPM_STYLE_ULMPM_GPU_H

#include "ulmpm.h"

class ULMPMGPU : public ULMPM {
 public:
  ULMPMGPU(class MPM *mpm) : ULMPM(mpm) {}
  void setup(vector<string> args) override;
  void compute_grid_weight_functions_and_gradients() override;
};

#endif
#endif
