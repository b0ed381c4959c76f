// Contact fixes between two solids (sm_103a): the particle-pair forces of
// FixContactMinPenetration::initial_integrate
// (src/fix_contact_min_penetration.cpp:83-235) and FixContactHertz::initial_integrate
// (src/fix_contact_hertz.cpp:82-197), added to the external force vector mbp
// that the force scatter then spreads to the nodes.
//
// The reference tests every pair of the two solids.  Here a pair can only
// interact when every coordinate difference is below the larger cellsize
// (the reference's first screen), so the members are binned on a hashed cell
// list with that cell size (spatial hash of M. Teschner et al., "Optimized
// Spatial Hashing for Collision Detection of Deformable Objects", VMV 2003)
// and each member visits the 3^dim cells around its own.  Every member sums
// its own pairs in a fixed order (neighbour cells in lexicographic order,
// members of a cell in sorted member order): no atomics, the same result on
// every run.  Both members of a pair evaluate the same expression on the
// same operands, so the two forces are exactly opposite.
#include "../../include/kmpm.h"
#include "kmpm_kernels.cuh"

namespace kmpm {

__device__ __forceinline__ unsigned cell_hash(int x, int y, int z, int nb) {
  return (((unsigned)x * 73856093u) ^ ((unsigned)y * 19349663u) ^ ((unsigned)z * 83492791u)) & (unsigned)(nb - 1);
}

// member i -> particle slot and tag (0 solid1, 1 solid2, -1 neither)
__device__ __forceinline__ int member_slot(const ContactDev &c, const float *P, size_t ps, int i, int &tag) {
  if (c.ul) {
    const int p = c.start1 + i;
    const int sid = __float_as_int(P[PF_SID * ps + p]);
    tag = sid == c.sid1 ? 0 : (sid == c.sid2 ? 1 : -1);
    return p;
  }
  tag = i < c.n1 ? 0 : 1;
  return i < c.n1 ? c.start1 + i : c.start2 + (i - c.n1);
}

// current position, radius Rp (half the cube / square root of the current
// volume J vol0), velocity and mass of every member; its cell and bucket
__global__ void k_contact_prep(PartArgs a, ContactDev c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.nmem || run_finished(a.scalars)) return;
  const float *P = *a.Pp;
  const size_t ps = a.ps;
  int tag;
  const int p = member_slot(c, P, ps, i, tag);
  c.vals[i] = i;
  if (tag < 0) {
    c.keys[i] = c.nb;  // sorts after every bucket, never visited
    c.rc[i] = make_int4(0, 0, 0, -1);
    return;
  }
  float x[3], H[9];
#pragma unroll
  for (int d = 0; d < 3; d++) x[d] = P[(PF_X0 + d) * ps + p] + P[(PF_X + d) * ps + p];
#pragma unroll
  for (int k = 0; k < 9; k++) H[k] = P[(PF_H + k) * ps + p];
  const float vol = (1.f + jm1_of_H(H)) * P[PF_VOL0 * ps + p];
  // Rp = 0.5 vol^(1/3) (3-D; the Hertz fix writes pow(vol, 0.333333333), which
  // differs from the cube root by less than FP32 resolution) or 0.5 vol^(1/2)
  // (the 2-D min-penetration fix takes vol / x_r in axisymmetric runs,
  // src/fix_contact_min_penetration.cpp:119-125)
  const float Rp = c.dim == 3 ? 0.5f * cbrtf(vol)
                              : 0.5f * sqrtf((c.axisym && c.kind == KMPM_CONTACT_MIN_PENETRATION) ? vol / x[0] : vol);
  int cell[3] = {0, 0, 0};
  for (int d = 0; d < c.dim; d++) cell[d] = (int)floorf((x[d] - c.boxlo[d]) * c.inv_cmax);
  c.ra[i] = make_float4(x[0], x[1], x[2], Rp);
  c.rb[i] = make_float4(P[PF_V * ps + p], P[(PF_V + 1) * ps + p], P[(PF_V + 2) * ps + p], P[PF_MASS * ps + p]);
  c.rc[i] = make_int4(cell[0], cell[1], cell[2], tag);
  c.keys[i] = (int)cell_hash(cell[0], cell[1], cell[2], c.nb);
}

// first / one-past-last sorted position of every bucket (arrays zeroed before)
__global__ void k_bucket_ranges(ContactDev c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.nmem) return;
  const int k = c.keys[i];
  if (k >= c.nb) return;
  if (i == 0 || c.keys[i - 1] != k) c.bstart[k] = i;
  if (i + 1 == c.nmem || c.keys[i + 1] != k) c.bend[k] = i + 1;
}

// The force of one pair in the reference's convention (dx = x2 - x1; the
// min-penetration fix adds f to solid1 and subtracts it from solid2, the Hertz
// fix the reverse) and the frictional heat g = ffric |vt| dt.  Returns false
// for a pair the reference screens out.
__device__ __forceinline__ bool pair_force(const ContactDev &c, float dt, const float4 &xa, const float4 &va,
                                           const float4 &xb, const float4 &vb, float f[3], float &g) {
  const float dx[3] = {xb.x - xa.x, xb.y - xa.y, xb.z - xa.z};
  // first screen: every coordinate difference below the larger cellsize (the
  // 2-D min-penetration fix screens x and y; z differences are 0 in 2-D runs)
  const int ns = (c.dim == 2 && c.kind == KMPM_CONTACT_MIN_PENETRATION) ? 2 : 3;
  for (int d = 0; d < ns; d++)
    if (!(dx[d] < c.cmax && dx[d] > -c.cmax)) return false;
  const float Rp = xa.w + xb.w;
  // the reference's second screen |dx_d| < Rp follows from r < Rp
  const float r = sqrtf(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
  if (!(r < Rp)) return false;
  g = 0.f;
  if (c.kind == KMPM_CONTACT_HERTZ) {
    const float pen = Rp - r;
    const float fmag = c.hcoef * c.estar * sqrtf(xa.w * xb.w / (xa.w + xb.w) * pen * pen * pen);
#pragma unroll
    for (int d = 0; d < 3; d++) f[d] = fmag * dx[d] / r;
    return true;
  }
  const float ir = 1.f / r;
  const float fmag = va.w * vb.w / ((va.w + vb.w) * dt * dt) * (1.f - Rp * ir);
#pragma unroll
  for (int d = 0; d < 3; d++) f[d] = fmag * dx[d];
  if (c.mu != 0.f) {
    const float dv[3] = {vb.x - va.x, vb.y - va.y, vb.z - va.z};
    const float dvn = (dv[0] * dx[0] + dv[1] * dx[1] + dv[2] * dx[2]) * ir * ir;
    float vt[3];
#pragma unroll
    for (int d = 0; d < 3; d++) vt[d] = dv[d] - dvn * dx[d];
    const float vtn = sqrtf(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
    if (vtn != 0.f) {
      const float ffric = c.mu * fmag * r;
#pragma unroll
      for (int d = 0; d < 3; d++) f[d] -= ffric * (vt[d] / vtn);
      g = ffric * vtn * dt;
    }
  }
  return true;
}

// every member sums its pairs into mbp (and gamma); solid1 members also sum
// the pair forces for the fix's total
__global__ void __launch_bounds__(256) k_contact_force(PartArgs a, ContactDev c) {
  __shared__ double red[3][256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (run_finished(a.scalars)) return;
  float tot[3] = {0.f, 0.f, 0.f};
  if (i < c.nmem) {
    const int4 own = c.rc[i];
    if (own.w >= 0) {
      const float dt = (float)a.scalars[0].dt;
      const float4 xo = c.ra[i], vo = c.rb[i];
      const int other = 1 - own.w;
      // the sign of this member's share: min-penetration +f on solid1, Hertz -f
      const float sgn = (own.w == 0) == (c.kind == KMPM_CONTACT_MIN_PENETRATION) ? 1.f : -1.f;
      float acc[3] = {0.f, 0.f, 0.f}, gam = 0.f;
      const int rz = c.dim == 3 ? 1 : 0, ry = c.dim >= 2 ? 1 : 0;
      for (int ox = -1; ox <= 1; ox++)
        for (int oy = -ry; oy <= ry; oy++)
          for (int oz = -rz; oz <= rz; oz++) {
            const int cx = own.x + ox, cy = own.y + oy, cz = own.z + oz;
            const int b = (int)cell_hash(cx, cy, cz, c.nb);
            const int e = c.bend[b];
            for (int j = c.bstart[b]; j < e; j++) {
              const int m = c.vals[j];
              const int4 oc = c.rc[m];
              // other solid, and this very cell (buckets can hold several cells)
              if (oc.w != other || oc.x != cx || oc.y != cy || oc.z != cz) continue;
              const float4 xm = c.ra[m], vm = c.rb[m];
              float f[3], g;
              const bool hit = own.w == 0 ? pair_force(c, dt, xo, vo, xm, vm, f, g)
                                          : pair_force(c, dt, xm, vm, xo, vo, f, g);
              if (!hit) continue;
#pragma unroll
              for (int d = 0; d < 3; d++) acc[d] = fmaf(sgn, f[d], acc[d]);
              if (own.w == 0)
#pragma unroll
                for (int d = 0; d < 3; d++) tot[d] += f[d];
              gam += g;
            }
          }
      const float *P = *a.Pp;
      const size_t ps = a.ps;
      int tag;
      const int p = member_slot(c, P, ps, i, tag);
#pragma unroll
      for (int d = 0; d < 3; d++) c.mbp[d * ps + p] += acc[d];
      if (c.thermal && gam != 0.f) {
        // frictional heat: alpha / (1 - alpha) in 2-D; the 3-D fix gives both
        // solids the share alpha (src/fix_contact_min_penetration.cpp:145-150, 207-212)
        const float share = c.dim == 2 ? (own.w == 0 ? c.alpha : 1.f - c.alpha) : c.alpha;
        const float invcp = own.w == 0 ? c.invcp1 : c.invcp2;
        float *Pw = *a.Pp;
        Pw[PF_GAMMA * ps + p] += share * P[PF_VOL0 * ps + p] * invcp * gam;
      }
    }
  }
  for (int d = 0; d < 3; d++) red[d][threadIdx.x] = (double)tot[d];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int d = 0; d < 3; d++) red[d][threadIdx.x] += red[d][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int d = 0; d < 3; d++) c.blk[3 * blockIdx.x + d] = red[d][0];
}

// the fix's total force: block partials summed in a fixed order
__global__ void k_contact_sum(ContactDev c, int nblk, const StepScalars *sc) {
  __shared__ double red[3][256];
  if (run_finished(sc)) return;
  double s[3] = {0, 0, 0};
  for (int b = threadIdx.x; b < nblk; b += blockDim.x)
    for (int d = 0; d < 3; d++) s[d] += c.blk[3 * b + d];
  for (int d = 0; d < 3; d++) red[d][threadIdx.x] = s[d];
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k)
      for (int d = 0; d < 3; d++) red[d][threadIdx.x] += red[d][threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int d = 0; d < 3; d++) c.ftot[d] = red[d][0];
}

int launch_contact(const PartArgs &a, const ContactDev &c, RadixTemp &rt, cudaStream_t st) {
  if (c.nmem <= 0 || c.dim < 2) return 0;
  const int nblk = (c.nmem + 255) / 256;
  int nl = 0;
  k_contact_prep<<<nblk, 256, 0, st>>>(a, c);
  nl++;
  radix_sort(c.keys, c.vals, c.nmem, c.key_bits, rt, st);
  nl += 3 * ((c.key_bits + 7) / 8);
  cudaMemsetAsync(c.bstart, 0, sizeof(int) * c.nb, st);
  cudaMemsetAsync(c.bend, 0, sizeof(int) * c.nb, st);
  k_bucket_ranges<<<nblk, 256, 0, st>>>(c);
  k_contact_force<<<nblk, 256, 0, st>>>(a, c);
  k_contact_sum<<<1, 256, 0, st>>>(c, nblk, a.scalars);
  nl += 3;
  return nl;
}

}  // namespace kmpm
