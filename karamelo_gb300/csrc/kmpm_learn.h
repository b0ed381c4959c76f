// Host/device interface of the learned return map kernels (kmpm_learn.cu,
// kmpm_mlp.cu).
#pragma once
#include <cstdint>

#include "../../include/kmpm.h"

namespace kmpm {

enum LearnMode : int { MODE_PLAIN = 0, MODE_LOG = 1, MODE_SUR = 2 };

struct LearnArgs {
  const unsigned char *blob;       // network image (kmpm_mlp.cuh layout)
  float tol;                       // residual tolerance, relative to the flow stress
  unsigned long long *stats;       // plastic, served by the network, outside envelope, residual miss
  float *log;                      // [log_cap x 22] logged pairs
  unsigned long long *log_count;
  long long log_cap;
  unsigned long long log_seed;
  uint32_t log_thresh;             // a plastic particle-step is logged when its hash < log_thresh
  int nblk;                        // 256-particle blocks of the particle layout
};

struct LearnKernels {
  void *log, *sur, *label, *queue;
  int sur_smem;
};
void get_learn_kernels(LearnKernels &k);
int mlp_nin();
int mlp_nout();
int mlp_blob_bytes();
int mlp_device_blob(kmpm_mlp *m, const unsigned char **blob);

}  // namespace kmpm
