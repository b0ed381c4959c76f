// kmpm_misc.cu -- time-step control, binning and reductions.
//
//   cell keys + stable radix sort + permutation: the per-step neighbour
//     search of ULMPM (src/ulmpm.cpp:88-337) becomes a binning of particles by
//     cell (tile-major order), deterministic because the sort is stable;
//   dt: adjust_dt (src/tlmpm.cpp:489-514, src/ulmpm.cpp:525-551) and
//     update_time (src/update.cpp:201-206);
//   energy: FixKineticEnergy / ComputeStrainEnergy reductions.
#include "kmpm_kernels.cuh"

namespace kmpm {

// ------------------------------------------------------------------ keys
// key = global tile * cells_per_tile + cell within tile, from the FP32
// position the kernels use (TL: x0, UL: x0 + the moved displacement PF_XN)
__global__ void k_cell_keys(PartArgs a, int *keys, int use_x0, int pad_last) {
  if (a.scalars != nullptr && run_finished(a.scalars)) return;
  const int ri = a.blk_range[blockIdx.x];
  const RangeDev rd = a.ranges[ri];
  const int p = rd.start + (blockIdx.x - rd.blk0) * 256 + threadIdx.x;
  const GridDev &g = a.grids[rd.grid];  // by reference: a copy lands on the stack
  const int T0 = a.tile_t[0], T1 = a.tile_t[1], T2 = a.tile_t[2];
  if (p >= rd.start + rd.count) {
    // padding slot: the last key of its grid, so that a stable sort of all
    // slots keeps every range's particles first and its padding last
    if (pad_last)
      keys[p] = (g.tile_off + g.ntile[0] * g.ntile[1] * g.ntile[2]) * (T0 * T1 * T2) - 1;
    return;
  }
  const float *P = *a.Pp;
  float x[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int d = 0; d < 3; d++)
    if (d < a.dim) x[d] = P[(PF_X0 + d) * a.ps + p] + (use_x0 ? 0.f : P[(PF_XN + d) * a.ps + p]);
  keys[p] = cell_key(g, T0, T1, T2, x, a.dim);
}

void launch_cell_keys(const PartArgs &a, int nblk, int *keys, int use_x0, cudaStream_t st, int pad_last) {
  k_cell_keys<<<nblk, 256, 0, st>>>(a, keys, use_x0, pad_last);
}

// Solid::populate's state into the buffer (src/solid.cpp:2284-2310): x0,
// the displacement x - x0 (formed in FP64, so FP32 keeps it to its own
// precision), v, mass, vol0, the caller index, the solid id and T - T_ref
__global__ void k_stage_solid(StageArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const size_t n = (size_t)a.n, ps = a.ps, p = (size_t)a.slot0 + i;
  const double *x0 = a.in, *x = a.in + 3 * n, *v = a.in + 6 * n, *m = a.in + 9 * n, *vol0 = a.in + 10 * n;
  float *P = a.P;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double xd = x0[3 * i + d];
    const float u = (float)(x[3 * i + d] - xd);
    P[(PF_X0 + d) * ps + p] = (float)xd;
    P[(PF_X + d) * ps + p] = u;
    if (a.ul) P[(PF_XN + d) * ps + p] = u;
    P[(PF_V + d) * ps + p] = (float)v[3 * i + d];
  }
  P[PF_MASS * ps + p] = (float)m[i];
  P[PF_VOL0 * ps + p] = (float)vol0[i];
  P[PF_ORIG * ps + p] = __int_as_float(a.orig0 + i);
  P[PF_SID * ps + p] = __int_as_float(a.sid);
  if (a.thermal) P[PF_T * ps + p] = a.T;
}
void launch_stage_solid(const StageArgs &a, cudaStream_t st) {
  if (a.n > 0) k_stage_solid<<<(a.n + 255) / 256, 256, 0, st>>>(a);
}

__global__ void k_publish_err(const ErrState *d, ErrState *h) { *h = *d; }
void launch_publish_err(const ErrState *d, ErrState *h_mapped, cudaStream_t st) {
  k_publish_err<<<1, 1, 0, st>>>(d, h_mapped);
}

// first / last particle of every cell and tile in sorted keys (arrays zeroed before)
__global__ void k_cell_ranges(const int *keys, int start, int n, int ncpt, int *cs, int *ce, int *ts, int *te) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = keys[i];
  const int kp = i > 0 ? keys[i - 1] : -1;
  const int kn = i + 1 < n ? keys[i + 1] : -1;
  if (k != kp) cs[k] = start + i;
  if (k != kn) ce[k] = start + i + 1;
  const int t = k / ncpt;
  if (i == 0 || kp / ncpt != t) ts[t] = start + i;
  if (i + 1 == n || kn / ncpt != t) te[t] = start + i + 1;
}

void launch_cell_ranges(const int *sorted_keys, int start, int n, int ncpt, int *cs, int *ce, int *ts, int *te,
                        cudaStream_t st) {
  if (n > 0) k_cell_ranges<<<(n + 255) / 256, 256, 0, st>>>(sorted_keys, start, n, ncpt, cs, ce, ts, te);
}

// ------------------------------------------------------------------ radix sort
// Stable least-significant-digit radix sort, 8 bits per pass.  Each block
// owns a chunk of 2048 consecutive items; a pass is (1) per-block digit
// histograms, (2) a scan of every digit's row over the blocks, (3) a scatter
// in which items are ranked inside the chunk in index order (warp match +
// per-warp prefix), so equal keys keep their order and the result does not
// depend on scheduling.
constexpr int RS_CHUNK = 2048;

__global__ void k_rs_hist(const int *keys, int n, int shift, int *hist, int nblk) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_CHUNK;
  for (int i = threadIdx.x; i < RS_CHUNK; i += 256) {
    const int idx = base + i;
    if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255], 1);
  }
  __syncthreads();
  hist[threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

__device__ __forceinline__ int block_excl_scan256(int v, int *tmp, int &total) {
  // Hillis-Steele inclusive scan over 256 threads, returns exclusive prefix
  tmp[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < 256; off <<= 1) {
    int x = threadIdx.x >= off ? tmp[threadIdx.x - off] : 0;
    __syncthreads();
    tmp[threadIdx.x] += x;
    __syncthreads();
  }
  total = tmp[255];
  const int incl = tmp[threadIdx.x];
  __syncthreads();
  return incl - v;
}

__global__ void k_rs_rowscan(int *hist, int nblk, int *tot) {
  __shared__ int tmp[256];
  int *row = hist + (size_t)blockIdx.x * nblk;
  int running = 0;
  for (int c0 = 0; c0 < nblk; c0 += 256) {
    const int i = c0 + threadIdx.x;
    const int v = i < nblk ? row[i] : 0;
    int total;
    const int ex = block_excl_scan256(v, tmp, total);
    if (i < nblk) row[i] = running + ex;
    running += total;
  }
  if (threadIdx.x == 0) tot[blockIdx.x] = running;
}

__global__ void k_rs_scatter(const int *kin, const int *vin, int *kout, int *vout, int n, int shift,
                             const int *hist, int nblk, const int *tot) {
  __shared__ int tmp[256];
  __shared__ int s_base[256];
  __shared__ int s_wc[8][256];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  int total;
  const int ex = block_excl_scan256(tot[t], tmp, total);
  s_base[t] = ex + hist[t * nblk + blockIdx.x];
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int sub = 0; sub < RS_CHUNK / 256; sub++) {
    const int idx = blockIdx.x * RS_CHUNK + sub * 256 + t;
    const bool valid = idx < n;
    const int key = valid ? kin[idx] : 0;
    const int dig = valid ? ((key >> shift) & 255) : 256 + lane;
#pragma unroll
    for (int w = 0; w < 8; w++) s_wc[w][t] = 0;
    __syncthreads();
    const unsigned peers = __match_any_sync(0xffffffffu, dig);
    const int rank = __popc(peers & lt_mask);
    if (valid && (__ffs(peers) - 1) == lane) s_wc[warp][dig] = __popc(peers);
    __syncthreads();
    int run = s_base[t];
#pragma unroll
    for (int w = 0; w < 8; w++) {
      const int c = s_wc[w][t];
      s_wc[w][t] = run;
      run += c;
    }
    s_base[t] = run;
    __syncthreads();
    if (valid) {
      const int pos = s_wc[warp][dig] + rank;
      kout[pos] = key;
      vout[pos] = vin[idx];
    }
    __syncthreads();
  }
}

void radix_sort(int *keys, int *vals, int n, int key_bits, RadixTemp &tmp, cudaStream_t st) {
  if (n <= 0) return;
  const int nblk = (n + RS_CHUNK - 1) / RS_CHUNK;
  int *ka = keys, *va = vals, *kb = tmp.k1, *vb = tmp.v1;
  int passes = (key_bits + 7) / 8;
  if (passes < 1) passes = 1;
  for (int ps = 0; ps < passes; ps++) {
    const int shift = 8 * ps;
    k_rs_hist<<<nblk, 256, 0, st>>>(ka, n, shift, tmp.hist, nblk);
    k_rs_rowscan<<<256, 256, 0, st>>>(tmp.hist, nblk, tmp.tot);
    k_rs_scatter<<<nblk, 256, 0, st>>>(ka, va, kb, vb, n, shift, tmp.hist, nblk, tmp.tot);
    int *t1 = ka; ka = kb; kb = t1;
    int *t2 = va; va = vb; vb = t2;
  }
  if (ka != keys) {  // odd number of passes: result lives in the temp buffers
    cudaMemcpyAsync(keys, ka, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(vals, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
  }
}

__global__ void k_iota(int *v, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}
void launch_iota(int *v, int n, cudaStream_t st) {
  if (n > 0) k_iota<<<(n + 255) / 256, 256, 0, st>>>(v, n);
}

// dst[f][start+i] = src[srcf][start+perm[i]] for the listed fields; fields are
// packed as (dst_field << 8) | src_field
struct FieldList { int f[64]; };
__global__ void k_permute(float *const *src_pp, float *const *dst_pp, size_t ps, const int *perm, int start, int n,
                          FieldList fl, int nf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *src = *src_pp;
  float *dst = *dst_pp;
  const int j = start + perm[i];
  // eight independent loads in flight before their stores: the gather is
  // latency-bound with one
  constexpr int B = 8;
  for (int k0 = 0; k0 < nf; k0 += B) {
    float v[B];
#pragma unroll
    for (int b = 0; b < B; b++)
      if (k0 + b < nf) v[b] = __ldg(src + (size_t)(fl.f[k0 + b] & 255) * ps + j);
#pragma unroll
    for (int b = 0; b < B; b++)
      if (k0 + b < nf) dst[(size_t)(fl.f[k0 + b] >> 8) * ps + start + i] = v[b];
  }
}
void launch_permute(float *const *src_pp, float *const *dst_pp, size_t ps, const int *perm, int start, int n,
                    const int *fields, int nfields, cudaStream_t st) {
  FieldList fl;
  for (int k = 0; k < nfields && k < 64; k++) fl.f[k] = fields[k];
  if (n > 0) k_permute<<<(n + 255) / 256, 256, 0, st>>>(src_pp, dst_pp, ps, perm, start, n, fl, nfields);
}

// swap the two particle-buffer pointers kept on the device
__global__ void k_swap_ptrs(float **pp) {
  float *t = pp[0];
  pp[0] = pp[1];
  pp[1] = t;
}
void launch_swap_ptrs(float **pp, cudaStream_t st) { k_swap_ptrs<<<1, 1, 0, st>>>(pp); }

// ------------------------------------------------------------------ dt
__device__ __forceinline__ void raise_error_m(ErrState *e, int code, int p, long long step) {
  if (atomicCAS(&e->code, 0, code) == 0) {
    e->particle = p;
    e->step = step;
  }
}

// per range: dtCFL = cellsize * min_h_ratio / max_p_wave_speed (src/solid.cpp:1430)
template <int BS>
__global__ void __launch_bounds__(BS) k_dt_range(DtArgs a) {
  static_assert(BS % 32 == 0 && BS <= 1024, "whole warps");
  __shared__ float rc[BS / 32], rh[BS / 32];
  if (run_finished(a.scalars)) return;
  const RangeDev rd = a.ranges[blockIdx.x];
  float c = 0.f, h = 1.f;
  // eight independent loads of each kind in flight per thread (max / min are
  // order-free), then the block's maximum and minimum by warp shuffles
  const int end = rd.blk0 + rd.nblk;
  int b = rd.blk0 + threadIdx.x;
  for (; b + 7 * BS < end; b += 8 * BS) {
    float cv[8], hv[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      cv[k] = a.blk_c[b + k * BS];
      hv[k] = a.blk_h[b + k * BS];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      c = fmaxf(c, cv[k]);
      h = fminf(h, hv[k]);
    }
  }
  for (; b < end; b += BS) {
    c = fmaxf(c, a.blk_c[b]);
    h = fminf(h, a.blk_h[b]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    c = fmaxf(c, __shfl_xor_sync(0xffffffffu, c, o));
    h = fminf(h, __shfl_xor_sync(0xffffffffu, h, o));
  }
  if ((threadIdx.x & 31) == 0) {
    rc[threadIdx.x >> 5] = c;
    rh[threadIdx.x >> 5] = h;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 1; w < BS / 32; w++) {
      rc[0] = fmaxf(rc[0], rc[w]);
      rh[0] = fminf(rh[0], rh[w]);
    }
    // TLMPM: a minimum at or above the range's bound may come from a particle
    // that reported the bound; k_h_exact then recomputes it (HRange)
    bool need = false;
    if (a.hr) {
      HRange &q = a.hr[blockIdx.x];
      need = !(rh[0] < q.bound);
      q.need = need;
      q.cmax = rc[0];
      q.hmin = need ? 1.f : rh[0];
      if (need) a.hflags[atomicAdd(a.nhflag, 1)] = blockIdx.x;
    }
    if (!need) {
      const GridDev g = a.grids[rd.grid];
      const double dtcfl = (double)g.cellsize * (double)rh[0] / (double)rc[0];
      a.solid_dtcfl[blockIdx.x] = dtcfl;
      if (rh[0] == 0.f || dtcfl == 0.0 || isnan(dtcfl))
        raise_error_m(a.err, ERR_DTCFL, -1, a.scalars[a.indep ? blockIdx.x : 0].ntimestep);
    }
  }
}

// The exact h ratio of the ranges k_dt_range flagged: min(1, |Re lambda(F)|)
// over every particle with damage below 1, as the stress kernel evaluates it,
// by a grid-stride loop and an order-free minimum (non-negative floats order
// as their bits).  With no range flagged every block returns at once.
__global__ void __launch_bounds__(256) k_h_exact(DtArgs a) {
  if (run_finished(a.scalars)) return;
  const int nf = *a.nhflag;
  if (nf == 0) return;
  const float *P = *a.Pp;
  const size_t ps = a.ps;
  for (int f = 0; f < nf; f++) {
    const int r = a.hflags[f];
    const RangeDev rd = a.ranges[r];
    float m = 1.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rd.count; i += gridDim.x * blockDim.x) {
      const int p = rd.start + i;
      if (!(P[PF_DMG * ps + p] < 1.f)) continue;
      float H[9];
#pragma unroll
      for (int k = 0; k < 9; k++) H[k] = P[(PF_H + k) * ps + p];
      m = fminf(m, fminf(1.f, min_abs_eig_real(H)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMin(reinterpret_cast<int *>(&a.hr[r].hmin), __float_as_int(m));
  }
}

// update_time, then adjust_dt; in independent mode every range keeps its own clock
__global__ void k_dt_final(DtArgs a) {
  if (run_finished(a.scalars)) return;
  if (a.hr) {
    // the ranges k_h_exact recomputed; every range's bound for the next step
    for (int r = threadIdx.x; r < a.nranges; r += blockDim.x) {
      HRange &q = a.hr[r];
      if (q.need) {
        const double dtcfl = (double)a.grids[a.ranges[r].grid].cellsize * (double)q.hmin / (double)q.cmax;
        a.solid_dtcfl[r] = dtcfl;
        if (q.hmin == 0.f || dtcfl == 0.0 || isnan(dtcfl))
          raise_error_m(a.err, ERR_DTCFL, -1, a.scalars[a.indep ? r : 0].ntimestep);
        q.need = 0;
      }
      q.bound = fminf(1.f, 1.001f * q.hmin);
    }
    __syncthreads();
    if (threadIdx.x == 0) *a.nhflag = 0;
  }
  if (a.indep) {
    for (int r = threadIdx.x; r < a.nranges; r += blockDim.x) {
      StepScalars &s = a.scalars[r];
      s.time += s.dt;
      s.dtCFL = a.solid_dtcfl[r];
      if (!a.dt_constant) s.dt = a.solid_dtcfl[r] * a.dt_factor;
    }
    return;
  }
  if (threadIdx.x == 0) {
    double m = 1.0e22;
    for (int r = 0; r < a.nranges; r++) m = fmin(m, a.solid_dtcfl[r]);
    StepScalars &s = a.scalars[0];
    s.time += s.dt;
    s.dtCFL = m;
    if (!a.dt_constant) s.dt = m * a.dt_factor;
  }
}

// the step counter advances at the start of a step (Update::update_timestep)
__global__ void k_step_begin(StepScalars *s, int n) {
  if (run_finished(s)) return;
  for (int r = threadIdx.x; r < n; r += blockDim.x) s[r].ntimestep++;
}

void launch_dt(const DtArgs &a, cudaStream_t st) {
  // wide CTAs for few large ranges, narrow ones for many small ranges
  if (a.max_nblk > 4096) k_dt_range<1024><<<a.nranges, 1024, 0, st>>>(a);
  else k_dt_range<256><<<a.nranges, 256, 0, st>>>(a);
  if (a.hr) k_h_exact<<<a.exact_blocks, 256, 0, st>>>(a);
  k_dt_final<<<1, 256, 0, st>>>(a);
}

void launch_step_begin(StepScalars *s, int n, cudaStream_t st) { k_step_begin<<<1, 256, 0, st>>>(s, n); }

// FixVelocityNodes' values at this step's time and one dt earlier
// (src/fix_velocity_nodes.cpp:130-271): time and dt do not change between
// the start of a step and its time update, so once per step serves every
// masked node
__global__ void k_fix_values(FixDev *fixes, int nfix, const GridDev *grids, const StepScalars *scalars, int indep) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nfix) return;
  FixDev &f = fixes[k];
  const StepScalars &sc = scalars[indep ? grids[f.grid].solid0 : 0];
  const double t = sc.time, tp = sc.time - sc.dt;
  for (int d = 0; d < 3; d++) {
    f.now[d] = f.c[d][0] + f.c[d][1] * t + f.c[d][2] * exp(f.c[d][3] * t);
    f.prev[d] = f.c[d][0] + f.c[d][1] * tp + f.c[d][2] * exp(f.c[d][3] * tp);
  }
}
void launch_fix_values(FixDev *fixes, int nfix, const GridDev *grids, const StepScalars *scalars, int indep,
                       cudaStream_t st) {
  if (nfix > 0) k_fix_values<<<(nfix + 127) / 128, 128, 0, st>>>(fixes, nfix, grids, scalars, indep);
}

// ------------------------------------------------------------------ energy
// 1/2 m |v|^2 and 1/2 vol sigma:strain_el in FP64 block partials, then a
// fixed-order sum (deterministic)
__global__ void k_energy_part(PartArgs a, double *blk) {
  __shared__ double rk[256], rs[256];
  const int ri = a.blk_range[blockIdx.x];
  const RangeDev rd = a.ranges[ri];
  const int p = rd.start + (blockIdx.x - rd.blk0) * 256 + threadIdx.x;
  double ek = 0, es = 0;
  if (p < rd.start + rd.count) {
    const size_t ps = a.ps;
    const float *P = *a.Pp;
    double v2 = 0;
    for (int d = 0; d < 3; d++) {
      const double v = P[(PF_V + d) * ps + p];
      v2 += v * v;
    }
    ek = 0.5 * P[PF_MASS * ps + p] * v2;
    if (a.track_strain) {
      float H[9];
      for (int k = 0; k < 9; k++) H[k] = P[(PF_H + k) * ps + p];
      const double vol = (1.0 + (double)jm1_of_H(H)) * P[PF_VOL0 * ps + p];
      double e = 0;
      for (int k = 0; k < 6; k++)
        e += (k < 3 ? 1.0 : 2.0) * (double)P[(PF_SIG + k) * ps + p] * (double)P[(PF_STRAIN + k) * ps + p];
      es = 0.5 * vol * e;
    }
  }
  rk[threadIdx.x] = ek;
  rs[threadIdx.x] = es;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rk[threadIdx.x] += rk[threadIdx.x + s];
      rs[threadIdx.x] += rs[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    blk[2 * blockIdx.x] = rk[0];
    blk[2 * blockIdx.x + 1] = rs[0];
  }
}

__global__ void k_energy_final(const double *blk, int nblk, double *out) {
  __shared__ double rk[256], rs[256];
  double ek = 0, es = 0;
  for (int b = threadIdx.x; b < nblk; b += 256) {
    ek += blk[2 * b];
    es += blk[2 * b + 1];
  }
  rk[threadIdx.x] = ek;
  rs[threadIdx.x] = es;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      rk[threadIdx.x] += rk[threadIdx.x + s];
      rs[threadIdx.x] += rs[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = rk[0];
    out[1] = rs[0];
  }
}

void launch_energy(const PartArgs &a, int nblk, double *blk, double *out, cudaStream_t st) {
  k_energy_part<<<nblk, 256, 0, st>>>(a, blk);
  k_energy_final<<<1, 256, 0, st>>>(blk, nblk, out);
}

// ------------------------------------------------------------------ kernel table
void get_step_kernels_1_0(StepKernels &k);
void get_step_kernels_1_1(StepKernels &k);
void get_step_kernels_1_2(StepKernels &k);
void get_step_kernels_2_0(StepKernels &k);
void get_step_kernels_2_1(StepKernels &k);
void get_step_kernels_2_2(StepKernels &k);
void get_step_kernels_3_0(StepKernels &k);
void get_step_kernels_3_1(StepKernels &k);
void get_step_kernels_3_2(StepKernels &k);
void get_step_kernels_1_3(StepKernels &k);
void get_step_kernels_2_3(StepKernels &k);
void get_step_kernels_3_3(StepKernels &k);

void get_step_kernels(int dim, int basis, StepKernels &k) {
  typedef void (*F)(StepKernels &);
  static const F tab[3][4] = {
      {get_step_kernels_1_0, get_step_kernels_1_1, get_step_kernels_1_2, get_step_kernels_1_3},
      {get_step_kernels_2_0, get_step_kernels_2_1, get_step_kernels_2_2, get_step_kernels_2_3},
      {get_step_kernels_3_0, get_step_kernels_3_1, get_step_kernels_3_2, get_step_kernels_3_3}};
  tab[dim - 1][basis](k);
}

int p2g_smem_bytes(int dim, int basis, int mode, bool thermal) {
  const int S = stencil_width(basis), SC = stencil_sc(basis);
  int t[3];
  tile_dims(dim, basis, t);
  const int L = t[0] / 8;
  const int WY = dim >= 2 ? (t[1] - 1) * SC + S : 1, WZ = dim == 3 ? (t[2] - 1) * SC + S : 1;
  const int NF = ((L - 1) * SC + S) * WY * WZ;
  const int Q = p2g_nq(mode, thermal), QINP = (p2g_nin(mode, thermal) + 3) & ~3;
  const int slab = (Q * NF + 3) & ~3;
  // affine modes also stage the per-slot offsets (x_node - x_p) / h; the
  // row scatter (k_p2g_row) pads each of its dim * S basis rows by one float2
  return 4 * 8 * (slab + 32 * QINP + 32 * dim * S * (p2g_apic(mode) ? 3 : 2) + dim * S * 2);
}

}  // namespace kmpm
