// G2P stress kernels of the learned return map.
//
//   MODE_LOG  the plain FP32 update of k_g2p2 that also logs, for a hashed
//             subset of the plastic particle-steps, the pair
//             (15 network inputs, 7 return-map outputs) to a device buffer
//   MODE_SUR  the same update with the Johnson-Cook radial return
//             (src/strength_jc.cpp:100-184) replaced on plastic steps by the
//             tensor-core MLP (kmpm_mlp.cuh), falling back to the closed form
//             where the inputs leave the training envelope or the network's
//             answer (its stress correction kept along the trial deviator)
//             misses the yield-function or flow-rule residual tolerance
//
//   queue     the network over the plastic steps that the plain stress
//             kernel (k_g2p2 with QUEUE, linear EOS + Johnson-Cook) queued
//             after its closed-form update: where the network's answer
//             passes the same tests it replaces that update
//
// All cover TLMPM with materials of type eos-strength whose strength is
// Johnson-Cook (the host checks this), FP32, no nodal temperature field.
// Everything else is the arithmetic of k_g2p2: rate of deformation,
// deformation gradient, polar decomposition, EOS, damage, plastic-work heat,
// PK1 operand and the dtCFL partials (src/solid.cpp:798-858, 1155-1438).
#include "kmpm_mlp.cuh"
#include "kmpm_step_impl.cuh"
#include "kmpm_learn.h"

namespace kmpm {

// the 15 network inputs of one particle-step
__device__ __forceinline__ void learn_features(const Sym<float> &D, float dt, const Sym<float> &sig, float epsp,
                                               float T, float epsdot, float epsdot0, float (&x)[mlp::NIN]) {
#pragma unroll
  for (int k = 0; k < 6; k++) x[k] = dt * D.a[k];
#pragma unroll
  for (int k = 0; k < 6; k++) x[6 + k] = sig.a[k];
  x[12] = epsp;
  x[13] = T;
  x[14] = log1pf(epsdot / epsdot0);
}

__device__ __forceinline__ bool log_selected(unsigned long long key, uint32_t thresh) {
  key += 0x9E3779B97F4A7C15ull;
  key = (key ^ (key >> 30)) * 0xBF58476D1CE4E5B9ull;
  key = (key ^ (key >> 27)) * 0x94D049BB133111EBull;
  key ^= key >> 31;
  return (uint32_t)(key >> 32) < thresh;
}

template <int DIM, int BASIS, int MODE>
__global__ void __launch_bounds__(MODE == MODE_SUR ? 512 : 256, MODE == MODE_SUR ? 1 : 2) k_g2p2_learn(PartArgs a, LearnArgs l) {
  constexpr int NT = MODE == MODE_SUR ? 512 : 256, NSUB = NT / 256, NTILE = NT / 128;
  extern __shared__ __align__(1024) unsigned char lsmem[];
  if (run_finished(a.scalars)) return;
  mlp::TileCtx tcx;
  bool wready = false;
  if (MODE == MODE_SUR) mlp::tile_begin<NTILE>(tcx, lsmem, l.blob);
  const int sub = threadIdx.x >> 8, tid = threadIdx.x & 255;
  const int vb = blockIdx.x * NSUB + sub;
  int p = -1;
  RangeDev rd;
  if (vb < l.nblk) {
    rd = a.ranges[a.blk_range[vb]];
    p = rd.start + (vb - rd.blk0) * 256 + tid;
    if (p >= rd.start + rd.count) p = -1;
  }
  float my_c = 0.f, my_h = 1.f;
  float *P = *a.Pp;
  const size_t ps = a.ps;
  // state carried across the network evaluation
  float H[9], cofF[9], R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  float J = 1.f, dmg = 0.f, vol0 = 0.f, rho = 0.f, dt = 0.f, cellsize = 0.f;
  float T = 0.f, epsp = 0.f, epsdot = 0.f, pH = 0.f, ys = 0.f, Gd = 0.f, J2tr = 0.f;
  Sym<float> D, sig, str;
  long long step = 0;
  int mi = 0;
  bool plastic = false, hasT = false;
  float feat[mlp::NIN];
  if (p >= 0) {
    const GridDev g = a.grids[rd.grid];
    cellsize = g.cellsize;
    mi = rd.mat >= 0 ? rd.mat : a.solid_mat[__float_as_int(P[PF_SID * ps + p])];
    const MatDev &m = a.mats[mi];
    const StepScalars &sc = a.scalars[a.indep ? a.blk_range[vb] : 0];
    dt = (float)sc.dt;
    step = sc.ntimestep;
    float xp[3];
#pragma unroll
    for (int d = 0; d < 3; d++) xp[d] = P[(PF_X0 + d) * ps + p];
    PAxes<DIM, BASIS> ax;
    ax.eval(g, xp);
    constexpr int S = Stencil<BASIS>::S;
    constexpr int SY = DIM >= 2 ? S : 1, SZ = DIM == 3 ? S : 1;
    float G[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int cx[S], cy[SY], cz[SZ];
#pragma unroll
    for (int k = 0; k < S; k++) cx[k] = min(max(ax.ax[0].i0 + k, 0), g.n[0] - 1);
#pragma unroll
    for (int k = 0; k < SY; k++) cy[k] = min(max(ax.ax[1].i0 + k, 0), g.n[1] - 1);
#pragma unroll
    for (int k = 0; k < SZ; k++) cz[k] = min(max(ax.ax[2].i0 + k, 0), g.n[2] - 1);
    const float4 *__restrict__ NV = (a.use_vu ? a.nodeB : a.nodeA) + NODE_STRIDE * g.node_off;
    // the gather of k_g2p2 (sum factorisation over the z slots)
#pragma unroll
    for (int i = 0; i < S; i++) {
      const float sx = ax.ax[0].s[i], dsx = ax.ax[0].ds[i];
#pragma unroll
      for (int j = 0; j < SY; j++) {
        const float sy = ax.ax[1].s[j], dsy = ax.ax[1].ds[j];
        const int row = (cx[i] * g.n[1] + cy[j]) * g.n[2];
        float A[3] = {0.f, 0.f, 0.f}, B[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < SZ; k++) {
          const float sz = ax.ax[2].s[k], dsz = ax.ax[2].ds[k];
          const float4 V = __ldg(NV + NODE_STRIDE * (row + cz[k]));
          const float vn[3] = {V.x, V.y, V.z};
#pragma unroll
          for (int r = 0; r < DIM; r++) {
            A[r] += sz * vn[r];
            if (DIM == 3) B[r] += dsz * vn[r];
          }
        }
        const float sxy = sx * sy, gx = dsx * sy, gy = sx * dsy;
#pragma unroll
        for (int r = 0; r < DIM; r++) {
          G[3 * r] += gx * A[r];
          if (DIM >= 2) G[3 * r + 1] += gy * A[r];
          if (DIM == 3) G[3 * r + 2] += sxy * B[r];
        }
      }
    }
    // F += dt Fdot, kept as H = F - I
#pragma unroll
    for (int k = 0; k < 9; k++) H[k] = P[(PF_H + k) * ps + p] + dt * G[k];
#pragma unroll
    for (int k = 0; k < 9; k++) P[(PF_H + k) * ps + p] = H[k];
    float F[9];
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = H[k] + ((k % 4 == 0) ? 1.f : 0.f);
    const float Jm1 = jm1_of_H(H);
    J = 1.f + Jm1;
    cof3(F, cofF);
    dmg = P[PF_DMG * ps + p];
    if (J <= 0.f && dmg < 1.f) raise_error(a.err, ERR_J, p, step);
    vol0 = P[PF_VOL0 * ps + p];
    rho = m.f_rho0 / J;
    if (!polar_rotation(F, R)) {
      if (dmg < 1.f) raise_error(a.err, ERR_POLDEC, p, step);
    }
    {
      float L[9], RtL[9], Dm[9], Ls[9];
      matmulT3(G, cofF, L);
      const float iJ = 1.f / J;
#pragma unroll
      for (int k = 0; k < 9; k++) L[k] *= iJ;
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) Ls[3 * r + c] = 0.5f * (L[3 * r + c] + L[3 * c + r]);
      matTmul3(R, Ls, RtL);
      matmul3(RtL, R, Dm);
      D.a[0] = Dm[0]; D.a[1] = Dm[4]; D.a[2] = Dm[8];
      D.a[3] = 0.5f * (Dm[1] + Dm[3]); D.a[4] = 0.5f * (Dm[2] + Dm[6]); D.a[5] = 0.5f * (Dm[5] + Dm[7]);
    }
#pragma unroll
    for (int k = 0; k < 6; k++) sig.a[k] = P[(PF_SIG + k) * ps + p];
    hasT = m.f_cp != 0.f;
    T = hasT ? a.T_ref + P[PF_T * ps + p] : 0.f;
    epsp = P[PF_EPSP * ps + p];
    epsdot = P[PF_EPSDOT * ps + p];
    pH = eos_pressure<float>(m, J, Jm1, rho, dmg, D.tr(), g.cellsize, T);
    if (hasT) pH += m.f_temp_p[3] * (m.f_temp_p[4] - T);
    // trial state of the radial return (src/strength_jc.cpp:150-170)
    const float *sp = m.f_str_p;
    if (dmg >= 1.f) {
#pragma unroll
      for (int k = 0; k < 6; k++) str.a[k] = 0.f;
    } else {
      ys = jc_flow_stress<float>(sp, epsp, epsdot, T);
      Gd = sp[0];
      if (dmg > 0.f) { Gd *= 1.f - dmg; ys *= 1.f - dmg; }
      const float f = dt * 2.f * Gd;
#pragma unroll
      for (int k = 0; k < 6; k++) str.a[k] = sig.a[k] + f * D.a[k];
      str.dev();
      J2tr = (float)KMPM_SQRT_3_OVER_2 * str.norm();
      plastic = !(J2tr < ys);
    }
    learn_features(D, dt, sig, epsp, T, epsdot, sp[4], feat);
  } else {
#pragma unroll
    for (int k = 0; k < mlp::NIN; k++) feat[k] = 0.f;
  }

  // ---- return map: closed form, or the network on plastic steps
  Sym<float> sdev = str;
  float dep = 0.f;
  bool use_net = false;
  if (MODE == MODE_SUR) {
    const bool cand = plastic && dmg == 0.f;
    const bool inside = mlp::tile_put_features(tcx, feat, cand);
    const bool any = __syncthreads_or(cand);
    float y[mlp::NOUT];
    if (any) {
      mlp::tile_weights_ready(tcx, wready);
      if (!mlp::tile_forward<NTILE>(tcx, y)) {
        if (threadIdx.x == 0) raise_error(a.err, ERR_TIMEOUT, -1, step);
      } else if (cand && inside) {
        // J2 flow returns along the trial deviator, so the predicted
        // correction is kept through its component along s_trial:
        // s_new = (1 + a) s_trial, a = <ds, s_trial> / <s_trial, s_trial>
        float dsn = 0.f, ss = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) {
          const float wk = k < 3 ? 1.f : 2.f;
          dsn += wk * y[k] * str.a[k];
          ss += wk * str.a[k] * str.a[k];
        }
        const float f1 = 1.f + dsn / ss;
        Sym<float> sn;
#pragma unroll
        for (int k = 0; k < 6; k++) sn.a[k] = f1 * str.a[k];
        const float J2n = J2tr * fabsf(f1);
        const float depn = y[6];
        // residuals relative to the flow stress: the yield function at the new
        // state and the flow rule (stress drop = 3 G dep)
        const float iys = 1.f / ys;
        const float r_yield = fabsf(J2n - ys) * iys;
        const float r_flow = fabsf(J2tr - J2n - 3.f * Gd * depn) * iys;
        if (depn >= 0.f && f1 > 0.f && r_yield <= l.tol && r_flow <= l.tol) {
          use_net = true;
          sdev = sn;
          dep = depn;
        }
      }
    }
    // particle-step counters: plastic, served by the network, outside the
    // envelope, residual above the tolerance
    const unsigned b_pl = __ballot_sync(0xffffffffu, cand), b_net = __ballot_sync(0xffffffffu, use_net),
                   b_out = __ballot_sync(0xffffffffu, cand && !inside),
                   b_res = __ballot_sync(0xffffffffu, cand && inside && !use_net);
    if ((threadIdx.x & 31) == 0 && b_pl) {
      atomicAdd(&l.stats[0], (unsigned long long)__popc(b_pl));
      atomicAdd(&l.stats[1], (unsigned long long)__popc(b_net));
      atomicAdd(&l.stats[2], (unsigned long long)__popc(b_out));
      atomicAdd(&l.stats[3], (unsigned long long)__popc(b_res));
    }
  }
  if (p >= 0 && plastic && !use_net) {  // closed-form radial return
    dep = (J2tr - ys) / (3.f * Gd);
    const float sc = ys / J2tr;
#pragma unroll
    for (int k = 0; k < 6; k++) sdev.a[k] = str.a[k] * sc;
  }
  if (MODE == MODE_LOG && p >= 0 && plastic && dmg == 0.f &&
      log_selected(((unsigned long long)step << 32) ^ (unsigned long long)(unsigned)p ^ l.log_seed, l.log_thresh)) {
    const unsigned long long slot = atomicAdd(l.log_count, 1ull);
    if (slot < (unsigned long long)l.log_cap) {
      float *row = l.log + slot * (mlp::NIN + mlp::NOUT);
#pragma unroll
      for (int k = 0; k < mlp::NIN; k++) row[k] = feat[k];
#pragma unroll
      for (int k = 0; k < 6; k++) row[mlp::NIN + k] = sdev.a[k] - str.a[k];
      row[mlp::NIN + 6] = dep;
    }
  }

  if (p >= 0) {
    const MatDev &m = a.mats[mi];
    epsp += dep;
    const float tav = 1000.f * cellsize / m.f_signal_velocity;
    epsdot -= epsdot * dt / tav;
    epsdot += dep / tav;
    epsdot = fmaxf(0.f, epsdot);
    if (m.damage >= 0) {
      float dinit = P[PF_DMGI * ps + p];
      float Tdm = a.thermal ? a.T_ref + P[PF_T * ps + p] : 0.f;
      damage_update<float>(m, dinit, dmg, pH, sdev, epsdot, dep, Tdm);
      P[PF_DMGI * ps + p] = dinit;
      P[PF_DMG * ps + p] = dmg;
    }
    if (hasT) {
      const float flow = (float)KMPM_SQRT_3_OVER_2 * sdev.norm();
      float gam = T < m.f_temp_p[5] ? m.f_temp_p[0] * flow * epsdot : 0.f;
      gam *= vol0 * m.f_invcp;
      P[PF_GAMMA * ps + p] = gam;
    }
    P[PF_EPSP * ps + p] = epsp;
    P[PF_EPSDOT * ps + p] = epsdot;
    const float pf = (dmg == 0.f || pH >= 0.f) ? pH : pH * (1.f - dmg);
#pragma unroll
    for (int k = 0; k < 6; k++) sig.a[k] = sdev.a[k];
    sig.a[0] -= pf; sig.a[1] -= pf; sig.a[2] -= pf;
    if (a.track_strain) {
      float tre = 0.f;
#pragma unroll
      for (int k = 0; k < 3; k++) tre += P[(PF_STRAIN + k) * ps + p];
      const float tr3 = (dt * D.tr() + tre) / 3.f;
      const float iG = dmg > 1e-10f ? 1.f / (m.f_G * (1.f - dmg)) : 1.f / m.f_G;
#pragma unroll
      for (int k = 0; k < 6; k++) P[(PF_STRAIN + k) * ps + p] = sdev.a[k] * iG + (k < 3 ? tr3 : 0.f);
    }
#pragma unroll
    for (int k = 0; k < 6; k++) P[(PF_SIG + k) * ps + p] = sig.a[k];
    {
      float Sm[9] = {sig.a[0], sig.a[3], sig.a[4], sig.a[3], sig.a[1], sig.a[5], sig.a[4], sig.a[5], sig.a[2]};
      float RS[9], RSR[9], PK1[9];
      matmul3(R, Sm, RS);
      matmulT3(RS, R, RSR);
      matmul3(RSR, cofF, PK1);
#pragma unroll
      for (int k = 0; k < 9; k++) P[(PF_PK + k) * ps + p] = PK1[k] * vol0;
    }
    if (dmg < 1.f) {
      const float vx = P[PF_V * ps + p], vy = P[(PF_V + 1) * ps + p], vz = P[(PF_V + 2) * ps + p];
      const float c = sqrtf(m.f_c2 / rho) + fmaxf(fmaxf(fabsf(vx), fabsf(vy)), fabsf(vz));
      if (isnan(c)) raise_error(a.err, ERR_NAN, p, step);
      my_c = c;
      my_h = fminf(1.f, min_abs_eig_real(H));
    }
  }
  // per 256-particle block: max wave speed, min h ratio (order-free)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    my_c = fmaxf(my_c, __shfl_xor_sync(0xffffffffu, my_c, o));
    my_h = fminf(my_h, __shfl_xor_sync(0xffffffffu, my_h, o));
  }
  __shared__ float red_c[NT / 32], red_h[NT / 32];
  if ((threadIdx.x & 31) == 0) {
    red_c[threadIdx.x >> 5] = my_c;
    red_h[threadIdx.x >> 5] = my_h;
  }
  __syncthreads();
  if (tid == 0 && vb < l.nblk) {
    float c = 0.f, h = 1.f;
#pragma unroll
    for (int w = 0; w < 8; w++) {
      c = fmaxf(c, red_c[sub * 8 + w]);
      h = fminf(h, red_h[sub * 8 + w]);
    }
    a.blk_c[vb] = c;
    a.blk_h[vb] = h;
  }
  if (MODE == MODE_SUR) {
    mlp::tile_weights_ready(tcx, wready);
    mlp::tile_end<NTILE>(tcx);
  }
}

// The network over the queue of plastic particle-steps.  The plain kernel
// has already written the closed-form update of every queued step; where the
// network's answer passes the residual tests of k_g2p2_learn (MODE_SUR), this
// kernel writes the update again from that answer: eps_p, its rate, sigma,
// strain_el and the PK1 operand (the material has linear EOS + Johnson-Cook,
// no damage and no temperature, so nothing else depends on the return).
// One 512-thread CTA per SM walks the queue in 512-row chunks (four 128-row
// M-tiles per forward pass).
__global__ void __launch_bounds__(512, 1) k_learn_queue(PartArgs a, LearnArgs l) {
  extern __shared__ __align__(1024) unsigned char lsmem[];
  if (run_finished(a.scalars)) return;
  mlp::TileCtx tcx;
  bool wready = false;
  mlp::tile_begin<4>(tcx, lsmem, l.blob);
  mlp::tile_weights_ready(tcx, wready);
  const long long cap = a.lq_cap;
  const int n = (int)min((long long)*a.lq_count, cap);
  const int nch = (n + 511) / 512;
  float *P = *a.Pp;
  const size_t ps = a.ps;
  const float *q = a.lq_f;
  for (int ch = blockIdx.x; ch < nch && tcx.ok; ch += gridDim.x) {
    const long long j = (long long)ch * 512 + threadIdx.x;
    const bool valid = j < n;
    int p = 0, mi = 0;
    float dt = 0.f, epsp = 0.f, epsdot = 0.f;
    Sym<float> D, sig;
    float feat[mlp::NIN];
    if (valid) {
      p = a.lq_i[LQ_P * cap + j];
      mi = a.lq_i[LQ_MAT * cap + j];
      dt = q[LQ_DT * cap + j];
#pragma unroll
      for (int k = 0; k < 6; k++) {
        D.a[k] = q[(LQ_D + k) * cap + j];
        sig.a[k] = q[(LQ_SIG + k) * cap + j];
      }
      epsp = q[LQ_EPSP * cap + j];
      epsdot = q[LQ_EPSDOT * cap + j];
      learn_features(D, dt, sig, epsp, 0.f, epsdot, a.mats[mi].f_str_p[4], feat);
    } else {
#pragma unroll
      for (int k = 0; k < mlp::NIN; k++) feat[k] = 0.f;
    }
    const bool inside = mlp::tile_put_features(tcx, feat, valid);
    float y[mlp::NOUT];
    if (!mlp::tile_forward<4>(tcx, y)) {
      if (threadIdx.x == 0) raise_error(a.err, ERR_TIMEOUT, -1, a.scalars[0].ntimestep);
      break;
    }
    bool use_net = false;
    if (valid && inside) {
      const MatDev &m = a.mats[mi];
      const float *sp = m.f_str_p;
      // the trial state and flow stress of the closed form (dmg = 0, T = 0)
      const float ys = jc_flow_stress<float>(sp, epsp, epsdot, 0.f);
      const float Gd = sp[0], f = dt * 2.f * Gd;
      Sym<float> str;
#pragma unroll
      for (int k = 0; k < 6; k++) str.a[k] = sig.a[k] + f * D.a[k];
      str.dev();
      const float J2tr = (float)KMPM_SQRT_3_OVER_2 * str.norm();
      float dsn = 0.f, ss = 0.f;
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const float wk = k < 3 ? 1.f : 2.f;
        dsn += wk * y[k] * str.a[k];
        ss += wk * str.a[k] * str.a[k];
      }
      const float f1 = 1.f + dsn / ss;
      const float J2n = J2tr * fabsf(f1);
      const float dep = y[6];
      const float iys = 1.f / ys;
      const float r_yield = fabsf(J2n - ys) * iys;
      const float r_flow = fabsf(J2tr - J2n - 3.f * Gd * dep) * iys;
      if (dep >= 0.f && f1 > 0.f && r_yield <= l.tol && r_flow <= l.tol) {
        use_net = true;
        Sym<float> sdev;
#pragma unroll
        for (int k = 0; k < 6; k++) sdev.a[k] = f1 * str.a[k];
        // the tail of k_g2p2's eos-strength update with this return
        const float tav = q[LQ_TAV * cap + j];
        float ed = epsdot;
        ed -= ed * dt / tav;
        ed += dep / tav;
        ed = fmaxf(0.f, ed);
        P[PF_EPSP * ps + p] = epsp + dep;
        P[PF_EPSDOT * ps + p] = ed;
        const float pf = q[LQ_PH * cap + j];
        if (a.track_strain) {
          const float tr3 = (dt * D.tr() + q[LQ_TRE * cap + j]) / 3.f;
          const float iG = 1.f / m.f_G;
#pragma unroll
          for (int k = 0; k < 6; k++) P[(PF_STRAIN + k) * ps + p] = sdev.a[k] * iG + (k < 3 ? tr3 : 0.f);
        }
        Sym<float> sn = sdev;
        sn.a[0] -= pf; sn.a[1] -= pf; sn.a[2] -= pf;
#pragma unroll
        for (int k = 0; k < 6; k++) P[(PF_SIG + k) * ps + p] = sn.a[k];
        float R[9], cofF[9];
#pragma unroll
        for (int k = 0; k < 9; k++) {
          R[k] = q[(LQ_R + k) * cap + j];
          cofF[k] = q[(LQ_COF + k) * cap + j];
        }
        float Sm[9] = {sn.a[0], sn.a[3], sn.a[4], sn.a[3], sn.a[1], sn.a[5], sn.a[4], sn.a[5], sn.a[2]};
        float RS[9], RSR[9], PK1[9];
        matmul3(R, Sm, RS);
        matmulT3(RS, R, RSR);
        matmul3(RSR, cofF, PK1);
        const float vol0 = P[PF_VOL0 * ps + p];
#pragma unroll
        for (int k = 0; k < 9; k++) P[(PF_PK + k) * ps + p] = PK1[k] * vol0;
      }
    }
    const unsigned b_net = __ballot_sync(0xffffffffu, use_net), b_out = __ballot_sync(0xffffffffu, valid && !inside),
                   b_res = __ballot_sync(0xffffffffu, valid && inside && !use_net);
    if ((threadIdx.x & 31) == 0 && (b_net | b_out | b_res)) {
      atomicAdd(&a.lq_stats[1], (unsigned long long)__popc(b_net));
      atomicAdd(&a.lq_stats[2], (unsigned long long)__popc(b_out));
      atomicAdd(&a.lq_stats[3], (unsigned long long)__popc(b_res));
    }
  }
  mlp::tile_end<4>(tcx);
}

// Closed-form return map of material `mat` on logged inputs (labels for the
// training set): Y = (s_new - s_trial (6), dep, plastic flag).
__global__ void k_jc_label(const MatDev *mats, int mat, const float *__restrict__ X, long long n, float *__restrict__ Y) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const MatDev &m = mats[mat];
  const float *x = X + i * mlp::NIN;
  const float *sp = m.f_str_p;
  const float epsdot = sp[4] * expm1f(x[14]);
  const float ys = jc_flow_stress<float>(sp, x[12], epsdot, x[13]);
  Sym<float> str;
#pragma unroll
  for (int k = 0; k < 6; k++) str.a[k] = x[6 + k] + 2.f * sp[0] * x[k];
  str.dev();
  const float J2 = (float)KMPM_SQRT_3_OVER_2 * str.norm();
  float *y = Y + i * (mlp::NOUT + 1);
  const bool pl = !(J2 < ys);
  const float sc = pl ? ys / J2 : 1.f;
#pragma unroll
  for (int k = 0; k < 6; k++) y[k] = str.a[k] * sc - str.a[k];
  y[6] = pl ? (J2 - ys) / (3.f * sp[0]) : 0.f;
  y[7] = pl ? 1.f : 0.f;
}

int mlp_nin() { return mlp::NIN; }
int mlp_nout() { return mlp::NOUT; }
int mlp_blob_bytes() { return mlp::BLOB_BYTES; }

void get_learn_kernels(LearnKernels &k) {
  k.log = (void *)k_g2p2_learn<3, 1, MODE_LOG>;
  k.sur = (void *)k_g2p2_learn<3, 1, MODE_SUR>;
  k.label = (void *)k_jc_label;
  k.queue = (void *)k_learn_queue;
  k.sur_smem = mlp::Smem<4>::BYTES;
}

}  // namespace kmpm
