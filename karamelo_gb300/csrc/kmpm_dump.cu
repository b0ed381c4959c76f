// Particle downloads for dumps, on the device: one solid's field gathered into
// the caller's particle order and converted to FP64 (the download before
// Output::write, src/output.cpp:128-200, and the fields DumpParticle writes,
// src/dump_particle.cpp:52-161), so a dump is one kernel and one copy.
#include "../../include/kmpm.h"
#include "kmpm_kernels.cuh"

namespace kmpm {

struct DumpArgs {
  int ri, solid, base, field, TL, rotate;
  double T_ref;
  double *out;
};

__global__ void k_dump(PartArgs a, DumpArgs d) {
  const RangeDev rd = a.ranges[d.ri];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= rd.count) return;
  const int p = rd.start + q;
  const float *P = *a.Pp;
  const size_t ps = a.ps;
  if (__float_as_int(P[PF_SID * ps + p]) != d.solid) return;
  const size_t i = (size_t)(__float_as_int(P[PF_ORIG * ps + p]) - d.base);
  auto f = [&](int fld) { return (double)P[fld * ps + p]; };
  double *o = d.out;
  const int sm[9] = {0, 3, 4, 3, 1, 5, 4, 5, 2};  // symmetric 6 -> 3x3 row-major
  switch (d.field) {
    case KMPM_P_X:
      for (int k = 0; k < 3; k++) o[3 * i + k] = f(PF_X0 + k) + (d.TL ? f(PF_X + k) : f(PF_XN + k));
      break;
    case KMPM_P_X0:
      for (int k = 0; k < 3; k++) o[3 * i + k] = f(PF_X0 + k);
      break;
    case KMPM_P_V:
      for (int k = 0; k < 3; k++) o[3 * i + k] = f(PF_V + k);
      break;
    case KMPM_P_SIGMA:
      for (int k = 0; k < 9; k++) o[9 * i + k] = f(PF_SIG + sm[k]);
      break;
    case KMPM_P_STRAIN_EL:
      for (int k = 0; k < 9; k++) o[9 * i + k] = f(PF_STRAIN + sm[k]);
      break;
    case KMPM_P_SIGMA_ROT:
    case KMPM_P_SIGMA_ROT6: {
      // the six components s11 s22 s33 s12 s13 s23 the reference dump writes
      // (src/dump_particle.cpp:116-121), or the full 3x3
      const bool six = d.field == KMPM_P_SIGMA_ROT6;
      const int up[6] = {0, 4, 8, 1, 2, 5};
      if (!d.rotate) {
        if (six)
          for (int k = 0; k < 6; k++) o[6 * i + k] = f(PF_SIG + k);
        else
          for (int k = 0; k < 9; k++) o[9 * i + k] = f(PF_SIG + sm[k]);
        break;
      }
      // R of F = R U by the stress kernel's FP32 polar iteration, and R sigma
      // R^T in FP32 as the stress kernel forms its PK1 operand: sigma, F and R
      // are FP32 state, and FP64 runs at 1/60 of the FP32 rate here
      float Ff[9], R[9], Sm[9], RS[9], RSR[9];
      for (int k = 0; k < 9; k++) Ff[k] = P[(PF_H + k) * ps + p] + (k % 4 == 0 ? 1.f : 0.f);
      if (!polar_rotation(Ff, R))  // det F <= 0: the step has raised its error; the stress goes out unrotated
        for (int k = 0; k < 9; k++) R[k] = (k % 4 == 0) ? 1.f : 0.f;
      for (int k = 0; k < 9; k++) Sm[k] = P[(PF_SIG + sm[k]) * ps + p];
      matmul3(R, Sm, RS);
      matmulT3(RS, R, RSR);
      if (six)
        for (int k = 0; k < 6; k++) o[6 * i + k] = (double)RSR[up[k]];
      else
        for (int k = 0; k < 9; k++) o[9 * i + k] = (double)RSR[k];
      break;
    }
    case KMPM_P_F:
      for (int k = 0; k < 9; k++) o[9 * i + k] = f(PF_H + k) + (k % 4 == 0 ? 1.0 : 0.0);
      break;
    case KMPM_P_VOL0PK1:
      for (int k = 0; k < 9; k++) o[9 * i + k] = d.TL ? f(PF_PK + k) : 0.0;
      break;
    case KMPM_P_J:
    case KMPM_P_VOL: {
      double H[9];
      for (int k = 0; k < 9; k++) H[k] = f(PF_H + k);
      const double jm1 = (H[0] + H[4] + H[8]) +
                         (H[0] * H[4] - H[1] * H[3] + H[0] * H[8] - H[2] * H[6] + H[4] * H[8] - H[5] * H[7]) +
                         (H[0] * (H[4] * H[8] - H[5] * H[7]) - H[1] * (H[3] * H[8] - H[5] * H[6]) +
                          H[2] * (H[3] * H[7] - H[4] * H[6]));
      o[i] = d.field == KMPM_P_J ? 1.0 + jm1 : (1.0 + jm1) * f(PF_VOL0);
      break;
    }
    case KMPM_P_EPS_P: o[i] = f(PF_EPSP); break;
    case KMPM_P_EPSDOT_P: o[i] = f(PF_EPSDOT); break;
    case KMPM_P_DAMAGE: o[i] = f(PF_DMG); break;
    case KMPM_P_DAMAGE_INIT: o[i] = f(PF_DMGI); break;
    case KMPM_P_T: o[i] = d.T_ref + f(PF_T); break;
    case KMPM_P_MASS: o[i] = f(PF_MASS); break;
  }
}

// Uploads for a restart (Solid::read_restart, src/solid.cpp:2894-2957): the
// inverse of k_dump, one field of one solid from caller order into its slots.
// Positions go in as the displacement from the stored x0, formed in FP64, so
// a download followed by an upload is exact.
struct LoadArgs {
  int ri, solid, base, field, TL;
  double T_ref;
  const double *in;
};

__global__ void k_load(PartArgs a, LoadArgs d) {
  const RangeDev rd = a.ranges[d.ri];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= rd.count) return;
  const int p = rd.start + q;
  float *P = *a.Pp;
  const size_t ps = a.ps;
  if (__float_as_int(P[PF_SID * ps + p]) != d.solid) return;
  const size_t i = (size_t)(__float_as_int(P[PF_ORIG * ps + p]) - d.base);
  const double *in = d.in;
  auto put = [&](int fld, double v) { P[fld * ps + p] = (float)v; };
  // upper triangle of a row-major 3x3 into the symmetric order xx yy zz xy xz yz
  const int up[6] = {0, 4, 8, 1, 2, 5};
  bool ul_pk = false;
  switch (d.field) {
    case KMPM_P_X:
      for (int k = 0; k < 3; k++) {
        const double u = in[3 * i + k] - (double)P[(PF_X0 + k) * ps + p];
        put(PF_X + k, u);
        if (!d.TL) put(PF_XN + k, u);
      }
      break;
    case KMPM_P_V:
      for (int k = 0; k < 3; k++) put(PF_V + k, in[3 * i + k]);
      break;
    case KMPM_P_SIGMA:
      for (int k = 0; k < 6; k++) put(PF_SIG + k, in[9 * i + up[k]]);
      ul_pk = !d.TL;
      break;
    case KMPM_P_STRAIN_EL:
      for (int k = 0; k < 6; k++) put(PF_STRAIN + k, in[9 * i + up[k]]);
      break;
    case KMPM_P_F:
      for (int k = 0; k < 9; k++) put(PF_H + k, in[9 * i + k] - (k % 4 == 0 ? 1.0 : 0.0));
      ul_pk = !d.TL;
      break;
    case KMPM_P_VOL0PK1:
      for (int k = 0; k < 9; k++) put(PF_PK + k, in[9 * i + k]);
      break;
    case KMPM_P_EPS_P: put(PF_EPSP, in[i]); break;
    case KMPM_P_EPSDOT_P: put(PF_EPSDOT, in[i]); break;
    case KMPM_P_DAMAGE: put(PF_DMG, in[i]); break;
    case KMPM_P_DAMAGE_INIT: put(PF_DMGI, in[i]); break;
    case KMPM_P_T: put(PF_T, in[i] - d.T_ref); break;
  }
  if (ul_pk) {
    // ULMPM scatters vol sigma with vol = J vol0, as the stress kernel stores it
    float H[9];
    for (int k = 0; k < 9; k++) H[k] = P[(PF_H + k) * ps + p];
    const float vol = (1.f + jm1_of_H(H)) * P[PF_VOL0 * ps + p];
    for (int k = 0; k < 6; k++) P[(PF_PK + k) * ps + p] = vol * P[(PF_SIG + k) * ps + p];
  }
}

void launch_load(const PartArgs &a, int ri, int count, int solid, int base, int field, int TL, double T_ref,
                 const double *in, cudaStream_t st) {
  LoadArgs d{ri, solid, base, field, TL, T_ref, in};
  if (count > 0) k_load<<<(count + 255) / 256, 256, 0, st>>>(a, d);
}

int dump_width(int field) {
  switch (field) {
    case KMPM_P_X: case KMPM_P_X0: case KMPM_P_V: return 3;
    case KMPM_P_SIGMA: case KMPM_P_SIGMA_ROT: case KMPM_P_F: case KMPM_P_STRAIN_EL: case KMPM_P_VOL0PK1: return 9;
    case KMPM_P_SIGMA_ROT6: return 6;
    case KMPM_P_EPS_P: case KMPM_P_EPSDOT_P: case KMPM_P_DAMAGE: case KMPM_P_DAMAGE_INIT: case KMPM_P_T:
    case KMPM_P_J: case KMPM_P_VOL: case KMPM_P_MASS: return 1;
    default: return 0;
  }
}

void launch_dump(const PartArgs &a, int ri, int count, int solid, int base, int field, int TL, int rotate,
                 double T_ref, double *out, cudaStream_t st) {
  DumpArgs d{ri, solid, base, field, TL, rotate, T_ref, out};
  if (count > 0) k_dump<<<(count + 255) / 256, 256, 0, st>>>(a, d);
}

}  // namespace kmpm
