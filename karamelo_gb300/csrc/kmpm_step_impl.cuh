// kmpm_step_impl.cuh -- the time-step kernels (sm_103a), instantiated per
// (dimension, basis) in kmpm_inst_*.cu.
//
//   k_p2g      deterministic cell-binned scatter (Solid::compute_*_nodes,
//              src/solid.cpp:317-522; MUSL re-map src/tlmpm.cpp:440-452)
//   k_grid     nodal sums -> v = p/m, body force, v_update, velocity fixes
//              (Grid::update_grid_velocities src/grid.cpp:448-466, fixes
//              src/fix_body_force.cpp:106-179, src/fix_velocity_nodes.cpp:130-271)
//   k_g2p1     grid_to_points + advance_particles (src/solid.cpp:576-635, 786-790)
//   k_g2p2     rate of deformation + F + stress + dtCFL partials
//              (src/solid.cpp:798-936, 1155-1438)
//   k_dt_*     adjust_dt / update_time (src/tlmpm.cpp:489-514, src/update.cpp:201-206)
#pragma once
#include "kmpm_kernels.cuh"

namespace kmpm {

// ============================================================== P2G (scatter)
// One CTA per non-empty tile of T^DIM cells, 8 warps.  Cells are processed in
// colour rounds (cell index mod C in every axis); the stencils of the cells of
// one round are disjoint, so each round adds into the shared footprint
// accumulator without conflicts, in a fixed order.  Inside a cell, a warp's
// lanes own the cell's stencil nodes (2 per lane) and loop over the cell's
// particles in sorted order, accumulating in registers.  The footprint is then
// written to the tile's slice of the partial buffer.
template <int DIM, int BASIS, int MODE, bool THERMAL>
__global__ void __launch_bounds__(256) k_p2g(P2GArgs a) {
  using TS = TileShape<DIM, BASIS>;
  constexpr int T = TS::T, S = TS::S, W = TS::W, NS = TS::NS, NW = TS::NW;
  constexpr int C = Stencil<BASIS>::C, SC = Stencil<BASIS>::SC, LO = Stencil<BASIS>::LO;
  constexpr int Q = p2g_nq(MODE, THERMAL);
  constexpr int QIN = p2g_nin(MODE, THERMAL);
  constexpr int TPC = T / C;  // cells per colour per axis
  constexpr int NCOL = DIM == 3 ? C * C * C : (DIM == 2 ? C * C : C);
  constexpr int NCPC = DIM == 3 ? TPC * TPC * TPC : (DIM == 2 ? TPC * TPC : TPC);
  constexpr int NSL = (NS + 31) / 32;  // stencil nodes per lane

  constexpr int QNW = (Q * NW + 3) & ~3;  // keeps the float2 staging 16-byte aligned
  extern __shared__ __align__(16) float smem[];
  float *acc = smem;                              // Q * NW
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *wbase = smem + QNW + warp * (32 * (DIM + QIN) + 32 * DIM * S * 2);
  float *spos = wbase;                            // 32 * DIM
  float *spay = spos + 32 * DIM;                  // 32 * QIN
  float2 *sbas = reinterpret_cast<float2 *>(spay + 32 * QIN);  // 32 * DIM * S

  const int2 td = a.tiles[blockIdx.x];
  const GridDev g = a.grids[td.x];
  const int tlin = td.y;
  int tc[3];
  tc[2] = DIM == 3 ? tlin % g.ntile[2] : 0;
  tc[1] = DIM >= 2 ? (DIM == 3 ? (tlin / g.ntile[2]) % g.ntile[1] : tlin % g.ntile[1]) : 0;
  tc[0] = DIM == 3 ? tlin / (g.ntile[1] * g.ntile[2]) : (DIM == 2 ? tlin / g.ntile[1] : tlin);
  const int tile_global = g.tile_off + tlin;
  const float h = g.cellsize / SC, ih = g.inv_cellsize;
  const float *P = *a.Pp;
  if (a.tile_end[tile_global] == a.tile_start[tile_global] || run_finished(a.scalars)) return;

  for (int k = threadIdx.x; k < Q * NW; k += blockDim.x) acc[k] = 0.f;
  __syncthreads();

  // stencil slots of this lane
  int soff[NSL][3];
#pragma unroll
  for (int u = 0; u < NSL; u++) {
    int sidx = lane + 32 * u;
    if (DIM == 3) { soff[u][0] = sidx / (S * S); soff[u][1] = (sidx / S) % S; soff[u][2] = sidx % S; }
    else if (DIM == 2) { soff[u][0] = sidx / S; soff[u][1] = sidx % S; soff[u][2] = 0; }
    else { soff[u][0] = sidx; soff[u][1] = 0; soff[u][2] = 0; }
  }

  for (int col = 0; col < NCOL; col++) {
    int cc[3];
    if (DIM == 3) { cc[0] = col / (C * C); cc[1] = (col / C) % C; cc[2] = col % C; }
    else if (DIM == 2) { cc[0] = col / C; cc[1] = col % C; cc[2] = 0; }
    else { cc[0] = col; cc[1] = 0; cc[2] = 0; }
    for (int kc = warp; kc < NCPC; kc += 8) {
      int lc[3];
      if (DIM == 3) { lc[0] = cc[0] + C * (kc / (TPC * TPC)); lc[1] = cc[1] + C * ((kc / TPC) % TPC); lc[2] = cc[2] + C * (kc % TPC); }
      else if (DIM == 2) { lc[0] = cc[0] + C * (kc / TPC); lc[1] = cc[1] + C * (kc % TPC); lc[2] = 0; }
      else { lc[0] = cc[0] + C * kc; lc[1] = 0; lc[2] = 0; }
      const int lcell = DIM == 3 ? (lc[0] * T + lc[1]) * T + lc[2] : (DIM == 2 ? lc[0] * T + lc[1] : lc[0]);
      const int cell_id = tile_global * TS::NCELL + lcell;
      const int cstart = a.cell_start[cell_id];
      const int ccount = a.cell_end[cell_id] - cstart;
      if (ccount == 0) continue;
      // base node index of the stencil along each axis
      int i0[3];
#pragma unroll
      for (int d = 0; d < 3; d++) i0[d] = (d < DIM) ? (tc[d] * T + lc[d]) * SC - LO : 0;

      float accr[NSL][Q];
#pragma unroll
      for (int u = 0; u < NSL; u++)
#pragma unroll
        for (int q = 0; q < Q; q++) accr[u][q] = 0.f;

      for (int c0 = 0; c0 < ccount; c0 += 32) {
        const int cnt = min(32, ccount - c0);
        // ---- stage positions and payload (lane = particle)
        if (lane < cnt) {
          const int p = cstart + c0 + lane;
#pragma unroll
          for (int d = 0; d < DIM; d++)
            spos[lane * DIM + d] = P[(PF_X0 + d) * a.ps + p] + (a.pos_field == PF_X ? P[(PF_X + d) * a.ps + p] : 0.f);
          float pay[QIN];
          p2g_payload<MODE, THERMAL>(a, P, p, pay);
#pragma unroll
          for (int q = 0; q < QIN; q++) spay[lane * QIN + q] = pay[q];
        }
        __syncwarp();
        // ---- per (particle, axis, slot) basis values
        for (int it = lane; it < cnt * DIM * S; it += 32) {
          const int j = it / (DIM * S), d = (it / S) % DIM, k = it % S;
          const int i = i0[d] + k;
          float s = 0.f, ds = 0.f;
          if (i >= 0 && i < g.n[d]) {
            const float xn = g.lo[d] + (float)i * h;
            const float r = (spos[j * DIM + d] - xn) * ih;
            basis<BASIS>(r, node_type<BASIS>(i, g.ng[d]), ih, s, ds);
          }
          sbas[it] = make_float2(s, ds);
        }
        __syncwarp();
        // ---- accumulate (lane = stencil node)
        for (int j = 0; j < cnt; j++) {
          const float *pay = spay + j * QIN;
          const float2 *bj = sbas + j * DIM * S;
#pragma unroll
          for (int u = 0; u < NSL; u++) {
            if (lane + 32 * u >= NS) continue;
            float2 bx = bj[soff[u][0]];
            float2 by = DIM >= 2 ? bj[S + soff[u][1]] : make_float2(1.f, 0.f);
            float2 bz = DIM == 3 ? bj[2 * S + soff[u][2]] : make_float2(1.f, 0.f);
            float wxy = bx.x * by.x;
            float w = wxy * bz.x;
            // the reference keeps a particle-node pair only when every 1-D
            // value is non-zero (src/tlmpm.cpp:263, src/ulmpm.cpp:259-272); the
            // cubic spline at ntype 1 has a zero value but a non-zero slope
            if (w == 0.f) continue;
            float gw[3] = {bx.y * by.x * bz.x, bx.x * by.y * bz.x, wxy * bz.y};
            p2g_accumulate<MODE, THERMAL, Q>(accr[u], pay, w, gw);
          }
        }
        __syncwarp();
      }
      // ---- flush into the footprint (no conflicts within a colour round)
#pragma unroll
      for (int u = 0; u < NSL; u++) {
        if (lane + 32 * u >= NS) continue;
        int fl[3];
#pragma unroll
        for (int d = 0; d < 3; d++) fl[d] = (d < DIM) ? lc[d] * SC + soff[u][d] : 0;
        const int fi = DIM == 3 ? (fl[0] * W + fl[1]) * W + fl[2] : (DIM == 2 ? fl[0] * W + fl[1] : fl[0]);
#pragma unroll
        for (int q = 0; q < Q; q++) acc[q * NW + fi] += accr[u][q];
      }
    }
    __syncthreads();
  }
  // ---- write the footprint
  float *out = a.partial + (size_t)tile_global * a.pstride_tile;
  for (int k = threadIdx.x; k < Q * NW; k += blockDim.x) out[k] = acc[k];
}

// ============================================================== grid
// Sum of the tile partials covering one node, in a fixed tile order.
template <int DIM, int BASIS, int Q>
__device__ __forceinline__ void gather_partials(const GridArgs &a, const GridDev &g, int li, const int *ix, double *sum) {
  using TS = TileShape<DIM, BASIS>;
  constexpr int T = TS::T, W = TS::W, NW = TS::NW, SC = Stencil<BASIS>::SC, LO = Stencil<BASIS>::LO;
  constexpr int TN = T * SC;  // nodes per tile step
  int tlo[3], thi[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (d < DIM) {
      // tile t covers nodes [t*TN - LO, t*TN - LO + W - 1]
      int hi = (ix[d] + LO) / TN;
      int lo_num = ix[d] + LO - W + 1;
      int lo = lo_num <= 0 ? 0 : (lo_num + TN - 1) / TN;
      tlo[d] = max(lo, 0);
      thi[d] = min(hi, g.ntile[d] - 1);
    } else {
      tlo[d] = thi[d] = 0;
    }
  }
#pragma unroll
  for (int q = 0; q < Q; q++) sum[q] = 0.0;
  for (int tx = tlo[0]; tx <= thi[0]; tx++)
    for (int ty = tlo[1]; ty <= thi[1]; ty++)
      for (int tz = tlo[2]; tz <= thi[2]; tz++) {
        const int tl = DIM == 3 ? (tx * g.ntile[1] + ty) * g.ntile[2] + tz : (DIM == 2 ? tx * g.ntile[1] + ty : tx);
        const int tg = g.tile_off + tl;
        if (a.tile_end[tg] == a.tile_start[tg]) continue;
        int fl[3] = {ix[0] - (tx * TN - LO), DIM >= 2 ? ix[1] - (ty * TN - LO) : 0, DIM == 3 ? ix[2] - (tz * TN - LO) : 0};
        const int fi = DIM == 3 ? (fl[0] * W + fl[1]) * W + fl[2] : (DIM == 2 ? fl[0] * W + fl[1] : fl[0]);
        const float *src = a.partial + (size_t)tg * a.pstride_tile;
#pragma unroll
        for (int q = 0; q < Q; q++) sum[q] += (double)src[q * NW + fi];
      }
  (void)li;
}

__device__ __forceinline__ double fix_value(const FixDev &f, int d, double t) {
  return f.c[d][0] + f.c[d][1] * t + f.c[d][2] * exp(f.c[d][3] * t);
}

// MODE_GRID_MASS: nodal mass only (TL once).  MODE_GRID_UPDATE: after the
// first scatter.  MODE_GRID_VEL: after the MUSL re-map (or USL: positions only).
template <int DIM, int BASIS, int GMODE, bool TL, bool THERMAL>
__global__ void __launch_bounds__(256) k_grid(GridArgs a) {
  if (run_finished(a.scalars)) return;
  const int gi = a.blk_grid[blockIdx.x];
  const GridDev g = a.grids[gi];
  const int li = (blockIdx.x - a.grid_blk0[gi]) * 256 + threadIdx.x;
  const int nn = g.n[0] * g.n[1] * g.n[2];
  if (li >= nn) return;
  int ix[3];
  ix[2] = li % g.n[2];
  ix[1] = (li / g.n[2]) % g.n[1];
  ix[0] = li / (g.n[1] * g.n[2]);
  const int node = g.node_off + li;
  const StepScalars &sc = a.scalars[a.indep ? g.solid0 : 0];
  const double dt = sc.dt, time = sc.time;

  if (GMODE == GM_MASS) {
    double s[1];
    gather_partials<DIM, BASIS, 1>(a, g, li, ix, s);
    float4 A = a.nodeA[node];
    A.w = (float)s[0];
    a.nodeA[node] = A;
    return;
  }
  if (GMODE == GM_UPDATE) {
    // quantities: TL [p3 f3 (+mT Qext Qint)]; UL [m p3 f3 (+...)]
    constexpr int Q = TL ? (THERMAL ? 9 : 6) : (THERMAL ? 10 : 7);
    double s[Q];
    gather_partials<DIM, BASIS, Q>(a, g, li, ix, s);
    const int o = TL ? 0 : 1;
    float4 A = a.nodeA[node];
    double m = TL ? (double)A.w : s[0];
    double v[3], f[3], mb[3] = {0, 0, 0}, vu[3];
    // Solid::compute_velocity_nodes: v = p/m only where m > 0 (src/solid.cpp:357)
    for (int d = 0; d < 3; d++) {
      v[d] = m > 0 ? s[o + d] / m : 0.0;
      f[d] = s[o + 3 + d];
    }
    // body force on nodes with mass (src/fix_body_force.cpp:122-136)
    for (int k = a.fix_start[gi]; k < a.fix_start[gi] + a.fix_count[gi]; k++) {
      const FixDev &fx = a.fixes[k];
      if (fx.kind != 1 || !fx.mask[li] || !(m > 0)) continue;
      for (int d = 0; d < 3; d++)
        if (fx.set[d]) mb[d] += fx.c[d][0] * m;
    }
    // Grid::update_grid_velocities (src/grid.cpp:448-466)
    for (int d = 0; d < 3; d++) vu[d] = m != 0 ? v[d] + dt * (f[d] + mb[d]) / m : v[d];
    double T = 0, Tu = 0;
    if (THERMAL) {
      T = m > 0 ? s[o + 6] / m : 0.0;
      Tu = m != 0 ? T + dt * (s[o + 8] + s[o + 7]) / m : T;  // src/grid.cpp:1354-1361
    }
    // FixVelocityNodes::post_update_grid_state (src/fix_velocity_nodes.cpp:130-225)
    for (int k = a.fix_start[gi]; k < a.fix_start[gi] + a.fix_count[gi]; k++) {
      const FixDev &fx = a.fixes[k];
      if (fx.kind != 0 || !fx.mask[li]) continue;
      for (int d = 0; d < 3; d++)
        if (fx.set[d]) { vu[d] = fix_value(fx, d, time); v[d] = fix_value(fx, d, time - dt); }
    }
    a.nodeA[node] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)m);
    a.nodeB[node] = make_float4((float)vu[0], (float)vu[1], (float)vu[2], (float)Tu);
    if (THERMAL) a.nodeT[node] = (float)T;
    return;
  }
  // GM_VEL: MUSL velocities_to_grid (+ BCs on v) and TL grid positions
  float4 A = a.nodeA[node];
  double v[3] = {A.x, A.y, A.z};
  if (a.remap) {
    constexpr int Q = THERMAL ? 4 : 3;
    double s[Q];
    gather_partials<DIM, BASIS, Q>(a, g, li, ix, s);
    double m = A.w;
    for (int d = 0; d < 3; d++) v[d] = m > 0 ? s[d] / m : 0.0;
    if (THERMAL) a.nodeT[node] = (float)(m > 0 ? s[3] / m : 0.0);
    // FixVelocityNodes::post_velocities_to_grid (src/fix_velocity_nodes.cpp:227-271)
    for (int k = a.fix_start[gi]; k < a.fix_start[gi] + a.fix_count[gi]; k++) {
      const FixDev &fx = a.fixes[k];
      if (fx.kind != 0 || !fx.mask[li]) continue;
      for (int d = 0; d < 3; d++)
        if (fx.set[d]) v[d] = fix_value(fx, d, time);
    }
    a.nodeA[node] = make_float4((float)v[0], (float)v[1], (float)v[2], A.w);
  }
  if (TL) {  // Grid::update_grid_positions (src/grid.cpp:468-474): x += dt v
    float4 X = a.nodeX[node];
    X.x += (float)(dt * v[0]);
    X.y += (float)(dt * v[1]);
    X.z += (float)(dt * v[2]);
    a.nodeX[node] = X;
  }
}


// ============================================================== G2P
template <int DIM, int BASIS> struct PAxes {
  Axis<BASIS> ax[3];
  __device__ __forceinline__ void eval(const GridDev &g, const float *xp) {
    const float h = g.cellsize / Stencil<BASIS>::SC;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      if (d < DIM) ax[d].eval(xp[d], g.lo[d], g.inv_cellsize, h, g.n[d], g.ng[d]);
      else ax[d].unit();
    }
  }
};

__device__ __forceinline__ void raise_error(ErrState *e, int code, int p, long long step) {
  if (atomicCAS(&e->code, 0, code) == 0) {
    e->particle = p;
    e->step = step;
  }
}

// Particle index of this thread within its 256-particle range block, or -1.
__device__ __forceinline__ int range_particle(const PartArgs &a, RangeDev &rd) {
  const int ri = a.blk_range[blockIdx.x];
  rd = a.ranges[ri];
  const int p = rd.start + (blockIdx.x - rd.blk0) * 256 + threadIdx.x;
  return p < rd.start + rd.count ? p : -1;
}

// grid_to_points + advance_particles (src/solid.cpp:576-635, 786-790)
template <int DIM, int BASIS, bool TL, bool THERMAL>
__global__ void __launch_bounds__(256) k_g2p1(PartArgs a) {
  if (run_finished(a.scalars)) return;
  RangeDev rd;
  const int p = range_particle(a, rd);
  if (p < 0) return;
  float *P = *a.Pp;
  const GridDev g = a.grids[rd.grid];
  const StepScalars &sc = a.scalars[a.indep ? a.blk_range[blockIdx.x] : 0];
  const float dt = (float)sc.dt;
  const size_t ps = a.ps;
  float xp[3], up[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    up[d] = P[(PF_X + d) * ps + p];
    xp[d] = P[(PF_X0 + d) * ps + p] + (TL ? 0.f : up[d]);
  }
  PAxes<DIM, BASIS> ax;
  ax.eval(g, xp);
  constexpr int S = Stencil<BASIS>::S;
  constexpr int SY = DIM >= 2 ? S : 1, SZ = DIM == 3 ? S : 1;
  float vu[3] = {0, 0, 0}, dv[3] = {0, 0, 0}, Tp = 0.f;
  for (int i = 0; i < S; i++) {
    const float sx = ax.ax[0].s[i];
    if (sx == 0.f) continue;
    for (int j = 0; j < SY; j++) {
      const float sxy = sx * ax.ax[1].s[j];
      if (sxy == 0.f) continue;
#pragma unroll
      for (int k = 0; k < SZ; k++) {
        const float w = sxy * ax.ax[2].s[k];
        if (w == 0.f) continue;
        const int node = g.node_off + ((ax.ax[0].i0 + i) * g.n[1] + (ax.ax[1].i0 + j)) * g.n[2] + ax.ax[2].i0 + k;
        const float4 A = a.nodeA[node];
        const float4 B = a.nodeB[node];
        vu[0] += w * B.x; vu[1] += w * B.y; vu[2] += w * B.z;
        dv[0] += w * (B.x - A.x); dv[1] += w * (B.y - A.y); dv[2] += w * (B.z - A.z);
        if (THERMAL) Tp += w * B.w;
      }
    }
  }
  const float alpha = a.pic_flip;
  float xn[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    // x += dt * v_update.  Positions are kept as the displacement u = x - x0
    // (FP32 rounding then scales with the displacement, not with |x|).  UL
    // writes the moved displacement to PF_XN: this step's weights keep PF_X.
    if (TL) P[(PF_X + d) * ps + p] = up[d] + dt * vu[d];
    else {
      const float un = up[d] + dt * vu[d];
      P[(PF_XN + d) * ps + p] = un;
      xn[d] = P[(PF_X0 + d) * ps + p] + un;
    }
    const float v = P[(PF_V + d) * ps + p];
    // v = (1-alpha) v_update + alpha (v + dt a), with dt a = sum w (v_update - v)
    P[(PF_V + d) * ps + p] = (1.f - alpha) * vu[d] + alpha * (v + dv[d]);
  }
  if (THERMAL) P[PF_T * ps + p] = Tp;
  if (!TL) {
    if (!(xn[0] >= a.boxlo[0] && xn[0] <= a.boxhi[0] && xn[1] >= a.boxlo[1] && xn[1] <= a.boxhi[1] &&
          xn[2] >= a.boxlo[2] && xn[2] <= a.boxhi[2]))
      raise_error(a.err, ERR_LEFT, p, sc.ntimestep);
  }
}

// rate of deformation + deformation gradient + stress + wave speed
// (src/solid.cpp:798-936, 1155-1438)
template <int DIM, int BASIS, bool TL, bool THERMAL, int PREC>
__global__ void __launch_bounds__(256) k_g2p2(PartArgs a) {
  __shared__ float red_c[256], red_h[256];
  if (run_finished(a.scalars)) return;
  RangeDev rd;
  const int p = range_particle(a, rd);
  float my_c = 0.f, my_h = 1.f;
  if (p >= 0) {
    float *P = *a.Pp;
    const size_t ps = a.ps;
    const GridDev g = a.grids[rd.grid];
    const int mi = rd.mat >= 0 ? rd.mat : a.solid_mat[__float_as_int(P[PF_SID * ps + p])];
    const MatDev &m = a.mats[mi];
    const StepScalars &sc = a.scalars[a.indep ? a.blk_range[blockIdx.x] : 0];
    const float dt = (float)sc.dt;
    float xp[3];
#pragma unroll
    for (int d = 0; d < 3; d++) xp[d] = P[(PF_X0 + d) * ps + p] + (TL ? 0.f : P[(PF_X + d) * ps + p]);
    PAxes<DIM, BASIS> ax;
    ax.eval(g, xp);
    constexpr int S = Stencil<BASIS>::S;
    constexpr int SY = DIM >= 2 ? S : 1, SZ = DIM == 3 ? S : 1;
    float G[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float qg[3] = {0, 0, 0};
    for (int i = 0; i < S; i++) {
      const float sx = ax.ax[0].s[i], dsx = ax.ax[0].ds[i];
      if (sx == 0.f) continue;
      for (int j = 0; j < SY; j++) {
        const float sy = ax.ax[1].s[j], dsy = ax.ax[1].ds[j];
        if (sx * sy == 0.f) continue;
#pragma unroll
        for (int k = 0; k < SZ; k++) {
          const float sz = ax.ax[2].s[k], dsz = ax.ax[2].ds[k];
          if (sx * sy * sz == 0.f) continue;
          const float gw[3] = {dsx * sy * sz, sx * dsy * sz, sx * sy * dsz};
          const int node = g.node_off + ((ax.ax[0].i0 + i) * g.n[1] + (ax.ax[1].i0 + j)) * g.n[2] + ax.ax[2].i0 + k;
          const float4 V = a.use_vu ? a.nodeB[node] : a.nodeA[node];
          const float vn[3] = {V.x, V.y, V.z};
#pragma unroll
          for (int r = 0; r < DIM; r++)
#pragma unroll
            for (int c = 0; c < DIM; c++) G[3 * r + c] += vn[r] * gw[c];
          if (THERMAL) {
            const float Tn = a.use_vu ? V.w : a.nodeT[node];
#pragma unroll
            for (int c = 0; c < 3; c++) qg[c] -= gw[c] * Tn;
          }
        }
      }
    }
    // ---- deformation gradient (src/solid.cpp:1155-1244), stored as H = F - I
    float H[9];
#pragma unroll
    for (int k = 0; k < 9; k++) H[k] = P[(PF_H + k) * ps + p];
    if (TL) {
#pragma unroll
      for (int k = 0; k < 9; k++) H[k] += dt * G[k];  // F += dt Fdot
    } else {
      float LH[9];  // F = (I + dt L) F  ->  H += dt (L + L H)
      matmul3(G, H, LH);
#pragma unroll
      for (int k = 0; k < 9; k++) H[k] += dt * (G[k] + LH[k]);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) P[(PF_H + k) * ps + p] = H[k];
    float F[9];
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = H[k] + ((k % 4 == 0) ? 1.f : 0.f);
    float J, Jm1, cofF[9];
    if (PREC == 1) {
      double Fd[9], Hd[9], cd[9];
#pragma unroll
      for (int k = 0; k < 9; k++) { Hd[k] = H[k]; Fd[k] = (double)H[k] + ((k % 4 == 0) ? 1.0 : 0.0); }
      double jm1 = (Hd[0] + Hd[4] + Hd[8]) +
                   (Hd[0] * Hd[4] - Hd[1] * Hd[3] + Hd[0] * Hd[8] - Hd[2] * Hd[6] + Hd[4] * Hd[8] - Hd[5] * Hd[7]) +
                   det3d(Hd);
      cof3d(Fd, cd);
#pragma unroll
      for (int k = 0; k < 9; k++) cofF[k] = (float)cd[k];
      Jm1 = (float)jm1;
      J = (float)(1.0 + jm1);
    } else {
      Jm1 = jm1_of_H(H);
      J = 1.f + Jm1;
      cof3(F, cofF);
    }
    float dmg = P[PF_DMG * ps + p];
    if (J <= 0.f && dmg < 1.f) raise_error(a.err, ERR_J, p, sc.ntimestep);
    const float vol0 = P[PF_VOL0 * ps + p];
    const float rho = (float)m.rho0 / J;
    float R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    Sym<float> D;
#pragma unroll
    for (int k = 0; k < 6; k++) D.a[k] = 0.f;
    const bool nh = m.type == 1;
    if (!nh) {
      if (TL) {
        if (!polar_rotation(F, R)) {
          if (dmg < 1.f) raise_error(a.err, ERR_POLDEC, p, sc.ntimestep);
        }
        // L = Fdot F^-1 = Fdot cof(F)^T / J ; D = R^T sym(L) R
        float L[9], RtL[9], Dm[9];
        matmulT3(G, cofF, L);
        const float iJ = 1.f / J;
#pragma unroll
        for (int k = 0; k < 9; k++) L[k] *= iJ;
        float Ls[9];
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
          for (int c = 0; c < 3; c++) Ls[3 * r + c] = 0.5f * (L[3 * r + c] + L[3 * c + r]);
        matTmul3(R, Ls, RtL);
        matmul3(RtL, R, Dm);
        D.a[0] = Dm[0]; D.a[1] = Dm[4]; D.a[2] = Dm[8];
        D.a[3] = 0.5f * (Dm[1] + Dm[3]); D.a[4] = 0.5f * (Dm[2] + Dm[6]); D.a[5] = 0.5f * (Dm[5] + Dm[7]);
      } else {
        D.a[0] = G[0]; D.a[1] = G[4]; D.a[2] = G[8];
        D.a[3] = 0.5f * (G[1] + G[3]); D.a[4] = 0.5f * (G[2] + G[6]); D.a[5] = 0.5f * (G[5] + G[7]);
      }
    }
    // ---- stress (src/solid.cpp:1246-1374)
    Sym<float> sig;
#pragma unroll
    for (int k = 0; k < 6; k++) sig.a[k] = P[(PF_SIG + k) * ps + p];
    float PK1[9];
    bool have_pk1 = false;
    if (m.type == 0) {  // LINEAR
      const float G2 = 2.f * (float)m.G, lam = (float)m.lambda;
      const float trinc = dt * D.tr();
#pragma unroll
      for (int k = 0; k < 6; k++) sig.a[k] += G2 * dt * D.a[k];
      sig.a[0] += lam * trinc; sig.a[1] += lam * trinc; sig.a[2] += lam * trinc;
      if (a.track_strain)
#pragma unroll
        for (int k = 0; k < 6; k++) P[(PF_STRAIN + k) * ps + p] += dt * D.a[k];
    } else if (nh) {  // NEO_HOOKEAN
      const float iJ = 1.f / J;
      float FiT[9];
#pragma unroll
      for (int k = 0; k < 9; k++) FiT[k] = cofF[k] * iJ;
      const float Gm = (float)m.G, lam = (float)m.lambda;
      const float lnJ = log1pf(Jm1);
#pragma unroll
      for (int k = 0; k < 9; k++) PK1[k] = Gm * (F[k] - FiT[k]) + lam * lnJ * FiT[k];
      have_pk1 = true;
      float FPt[9];
      matmulT3(F, PK1, FPt);  // F PK1^T
      sig.a[0] = iJ * FPt[0]; sig.a[1] = iJ * FPt[4]; sig.a[2] = iJ * FPt[8];
      sig.a[3] = iJ * FPt[1]; sig.a[4] = iJ * FPt[2]; sig.a[5] = iJ * FPt[5];
      if (a.track_strain) {
        float FtF[9];
        matTmul3(F, F, FtF);
        P[(PF_STRAIN + 0) * ps + p] = 0.5f * (FtF[0] - 1.f);
        P[(PF_STRAIN + 1) * ps + p] = 0.5f * (FtF[4] - 1.f);
        P[(PF_STRAIN + 2) * ps + p] = 0.5f * (FtF[8] - 1.f);
        P[(PF_STRAIN + 3) * ps + p] = 0.5f * FtF[1];
        P[(PF_STRAIN + 4) * ps + p] = 0.5f * FtF[2];
        P[(PF_STRAIN + 5) * ps + p] = 0.5f * FtF[5];
      }
    } else {  // EOS + strength (+ damage + temperature)
      const bool hasT = m.cp != 0.0;
      float T = hasT ? P[PF_T * ps + p] : 0.f;
      float epsp = P[PF_EPSP * ps + p], epsdot = P[PF_EPSDOT * ps + p];
      float dinit = m.damage >= 0 ? P[PF_DMGI * ps + p] : 0.f;
      float pH, dep;
      Sym<float> sdev;
      if (PREC == 1) {
        Sym<double> sg, Dd;
#pragma unroll
        for (int k = 0; k < 6; k++) { sg.a[k] = sig.a[k]; Dd.a[k] = D.a[k]; }
        double depd = 0;
        double Jd = 1.0 + (double)Jm1;
        double pHd = eos_pressure<double>(m, Jd, (double)Jm1, m.rho0 / Jd, dmg, Dd.tr(), g.cellsize, T);
        if (hasT) pHd += m.temp_p[3] * (m.temp_p[4] - (double)T);
        Sym<double> sdd = strength_update<double>(m, sc.dt, sg, Dd, depd, epsp, epsdot, dmg, T);
        pH = (float)pHd;
        dep = (float)depd;
#pragma unroll
        for (int k = 0; k < 6; k++) sdev.a[k] = (float)sdd.a[k];
      } else {
        pH = eos_pressure<float>(m, J, Jm1, rho, dmg, D.tr(), g.cellsize, T);
        if (hasT) pH += (float)m.temp_p[3] * ((float)m.temp_p[4] - T);
        sdev = strength_update<float>(m, dt, sig, D, dep, epsp, epsdot, dmg, T);
      }
      epsp += dep;
      const float tav = 1000.f * g.cellsize / (float)m.signal_velocity;
      epsdot -= epsdot * dt / tav;
      epsdot += dep / tav;
      epsdot = fmaxf(0.f, epsdot);
      if (m.damage >= 0) {
        float Tdm = a.thermal ? T : 0.f;
        damage_update<float>(m, dinit, dmg, pH, sdev, epsdot, dep, Tdm);
        P[PF_DMGI * ps + p] = dinit;
        P[PF_DMG * ps + p] = dmg;
      }
      if (hasT) {
        const float flow = (float)KMPM_SQRT_3_OVER_2 * sdev.norm();
        float gam = T < (float)m.temp_p[5] ? (float)m.temp_p[0] * flow * epsdot : 0.f;
        gam *= (TL ? vol0 : J * vol0) * (float)m.invcp;
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
        const float iG = dmg > 1e-10f ? 1.f / ((float)m.G * (1.f - dmg)) : 1.f / (float)m.G;
#pragma unroll
        for (int k = 0; k < 6; k++) P[(PF_STRAIN + k) * ps + p] = sdev.a[k] * iG + (k < 3 ? tr3 : 0.f);
      }
    }
#pragma unroll
    for (int k = 0; k < 6; k++) P[(PF_SIG + k) * ps + p] = sig.a[k];
    // ---- nodal-force operand for the next scatter
    if (TL) {
      if (!have_pk1) {
        // vol0 J (R sigma R^T) F^-T = vol0 (R sigma R^T) cof(F)
        float Sm[9] = {sig.a[0], sig.a[3], sig.a[4], sig.a[3], sig.a[1], sig.a[5], sig.a[4], sig.a[5], sig.a[2]};
        float RS[9], RSR[9];
        matmul3(R, Sm, RS);
        matmulT3(RS, R, RSR);
        matmul3(RSR, cofF, PK1);
      }
#pragma unroll
      for (int k = 0; k < 9; k++) P[(PF_PK + k) * ps + p] = PK1[k] * vol0;
    } else {
      const float vol = J * vol0;
#pragma unroll
      for (int k = 0; k < 6; k++) P[(PF_PK + k) * ps + p] = vol * sig.a[k];
    }
    if (THERMAL) {  // Solid::update_heat_flux (src/solid.cpp:2812-2839)
      const float f = (TL ? vol0 : J * vol0) * (float)(m.invcp * m.kappa);
#pragma unroll
      for (int c = 0; c < 3; c++) P[(PF_Q + c) * ps + p] = qg[c] * f;
    }
    // ---- wave speed and h ratio (src/solid.cpp:1376-1437)
    if (dmg < 1.f) {
      const float vx = P[PF_V * ps + p], vy = P[(PF_V + 1) * ps + p], vz = P[(PF_V + 2) * ps + p];
      const float c = sqrtf((float)(m.K + KMPM_FOUR_THIRD * m.G) / rho) + fmaxf(fmaxf(fabsf(vx), fabsf(vy)), fabsf(vz));
      if (isnan(c)) raise_error(a.err, ERR_NAN, p, sc.ntimestep);
      my_c = c;
      if (TL) my_h = fminf(1.f, min_abs_eig_real(H));
    }
  }
  // block reduction (order-free min / max)
  red_c[threadIdx.x] = my_c;
  red_h[threadIdx.x] = my_h;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red_c[threadIdx.x] = fmaxf(red_c[threadIdx.x], red_c[threadIdx.x + s]);
      red_h[threadIdx.x] = fminf(red_h[threadIdx.x], red_h[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.blk_c[blockIdx.x] = red_c[0];
    a.blk_h[blockIdx.x] = red_h[0];
  }
}

// ============================================================== instantiation
template <int DIM, int BASIS>
void fill_step_kernels(StepKernels &k) {
  k.p2g_mass = (void *)k_p2g<DIM, BASIS, P2G_MASS, false>;
  k.p2g_tl = (void *)k_p2g<DIM, BASIS, P2G_TL, false>;
  k.p2g_tl_th = (void *)k_p2g<DIM, BASIS, P2G_TL, true>;
  k.p2g_ul = (void *)k_p2g<DIM, BASIS, P2G_UL, false>;
  k.p2g_ul_th = (void *)k_p2g<DIM, BASIS, P2G_UL, true>;
  k.p2g_vel = (void *)k_p2g<DIM, BASIS, P2G_VEL, false>;
  k.p2g_vel_th = (void *)k_p2g<DIM, BASIS, P2G_VEL, true>;
  k.grid_mass = (void *)k_grid<DIM, BASIS, GM_MASS, true, false>;
  k.grid_upd[0][0] = (void *)k_grid<DIM, BASIS, GM_UPDATE, false, false>;
  k.grid_upd[0][1] = (void *)k_grid<DIM, BASIS, GM_UPDATE, false, true>;
  k.grid_upd[1][0] = (void *)k_grid<DIM, BASIS, GM_UPDATE, true, false>;
  k.grid_upd[1][1] = (void *)k_grid<DIM, BASIS, GM_UPDATE, true, true>;
  k.grid_vel[0][0] = (void *)k_grid<DIM, BASIS, GM_VEL, false, false>;
  k.grid_vel[0][1] = (void *)k_grid<DIM, BASIS, GM_VEL, false, true>;
  k.grid_vel[1][0] = (void *)k_grid<DIM, BASIS, GM_VEL, true, false>;
  k.grid_vel[1][1] = (void *)k_grid<DIM, BASIS, GM_VEL, true, true>;
  k.g2p1[0][0] = (void *)k_g2p1<DIM, BASIS, false, false>;
  k.g2p1[0][1] = (void *)k_g2p1<DIM, BASIS, false, true>;
  k.g2p1[1][0] = (void *)k_g2p1<DIM, BASIS, true, false>;
  k.g2p1[1][1] = (void *)k_g2p1<DIM, BASIS, true, true>;
  k.g2p2[0][0][0] = (void *)k_g2p2<DIM, BASIS, false, false, 0>;
  k.g2p2[0][1][0] = (void *)k_g2p2<DIM, BASIS, false, true, 0>;
  k.g2p2[1][0][0] = (void *)k_g2p2<DIM, BASIS, true, false, 0>;
  k.g2p2[1][1][0] = (void *)k_g2p2<DIM, BASIS, true, true, 0>;
  k.g2p2[0][0][1] = (void *)k_g2p2<DIM, BASIS, false, false, 1>;
  k.g2p2[0][1][1] = (void *)k_g2p2<DIM, BASIS, false, true, 1>;
  k.g2p2[1][0][1] = (void *)k_g2p2<DIM, BASIS, true, false, 1>;
  k.g2p2[1][1][1] = (void *)k_g2p2<DIM, BASIS, true, true, 1>;
}

}  // namespace kmpm
