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
#include "kmpm_async.cuh"
#include "kmpm_kernels.cuh"

namespace kmpm {

// ============================================================== P2G (scatter)
// One CTA of 8 warps per non-empty tile.  Warp w owns the x-slab of cells
// [w L, (w+1) L) of the tile and visits its cells in a fixed order; for every
// cell the lanes first stage the cell's particles (lane = particle: payload
// and the per-axis basis values, next cell prefetched into registers), then
// own the cell's stencil nodes (lane = node) and accumulate over the cell's
// particles in sorted order, then add the result into the warp's private
// slab footprint in shared memory.  After one barrier the slab footprints are
// summed in warp order into the tile's slice of the partial buffer.  No float
// atomics: the result is bit-reproducible.
// Contribution of one staged particle to this lane's stencil nodes.
template <int DIM, int S, int MODE, bool THERMAL, int Q, int QINP, int NSL, int NS, bool PAIR>
__device__ __forceinline__ void p2g_particle(float (&accr)[NSL][Q], const float *spay_j, const float2 *bj,
                                             const float *oj, float h, const int (&soff)[NSL][3], int lane) {
  constexpr int BM = p2g_base(MODE);
  constexpr bool AP = p2g_apic(MODE);
  float pay[QINP];
#pragma unroll
  for (int v = 0; v < QINP / 4; v++) {
    const float4 t = reinterpret_cast<const float4 *>(spay_j)[v];
    pay[4 * v] = t.x; pay[4 * v + 1] = t.y; pay[4 * v + 2] = t.z; pay[4 * v + 3] = t.w;
  }
  const float2 bx = bj[soff[0][0]];
  const float2 by = DIM >= 2 ? bj[S + soff[0][1]] : make_float2(1.f, 0.f);
  const float wxy = bx.x * by.x, gxy0 = bx.y * by.x, gxy1 = bx.x * by.y;
  if ((BM == P2G_TL || BM == P2G_UL || AP) && !THERMAL) {
    // the lane's nodes share (a, b): with w = wxy s_z and grad w =
    // (gxy0 s_z, gxy1 s_z, wxy s'_z), every term factors into a per-particle
    // part and s_z or s'_z:  m v w = s_z (wxy m v),
    // f_r -= s_z (T_r0 gxy0 + T_r1 gxy1) + s'_z (T_r2 wxy)  (T = vol0 PK1 or vol sigma),
    // and with external particle forces f_r += s_z (wxy mbp_r).
    // APIC adds m C (x_node - x_p) to m v: its x and y parts join the
    // per-particle term, its z part s_z (z_node - z_p) (wxy m C_r2) is per node;
    // x_node - x_p = h o + (x_w - x_p) with the staged offsets o of the weights.
    constexpr int OM = BM == P2G_UL ? 1 : 0;  // UL payload and sums start with the mass
    constexpr bool FORCE = BM != P2G_VEL;
    constexpr int NB = p2g_nin(BM, false);    // APIC: m C (9) and x_w - x_p (3) follow the base payload
    float q[4], t[3], t2[3], qc[3];
#pragma unroll
    for (int d = 0; d < 3 + OM; d++) q[d] = wxy * pay[d];
    if (AP) {
      const float *mC = pay + NB, *dw = pay + NB + 9;
      const float dxa = fmaf(oj[soff[0][0]], h, dw[0]), dyb = DIM >= 2 ? fmaf(oj[S + soff[0][1]], h, dw[1]) : 0.f;
#pragma unroll
      for (int r = 0; r < 3; r++) {
        q[OM + r] = fmaf(wxy, mC[3 * r] * dxa + mC[3 * r + 1] * dyb, q[OM + r]);
        qc[r] = wxy * mC[3 * r + 2];
      }
    }
    if (FORCE) {
#pragma unroll
      for (int r = 0; r < 3; r++) {
        float T0, T1, T2;
        if (BM == P2G_TL) {
          T0 = pay[3 + 3 * r]; T1 = pay[4 + 3 * r]; T2 = pay[5 + 3 * r];
        } else {  // symmetric sigma: xx yy zz xy xz yz
          const float *sg = pay + 4;
          T0 = r == 0 ? sg[0] : (r == 1 ? sg[3] : sg[4]);
          T1 = r == 0 ? sg[3] : (r == 1 ? sg[1] : sg[5]);
          T2 = r == 0 ? sg[4] : (r == 1 ? sg[5] : sg[2]);
        }
        t[r] = T0 * gxy0 + T1 * gxy1;
        // external particle force: f_r += s_z (wxy mbp_r)
        if (p2g_ext(MODE)) t[r] = fmaf(-wxy, pay[p2g_nin(MODE & ~(P2G_EXT | P2G_AXI), false) + r], t[r]);
        // axisymmetric hoop term (2-D, s_z = 1): f_0 -= w T_zz / r
        if (p2g_axi(MODE) && r == 0) t[0] = fmaf(wxy, pay[p2g_nin(MODE & ~P2G_AXI, false)], t[0]);
        t2[r] = T2 * wxy;
      }
    }
#pragma unroll
    for (int u = 0; u < NSL; u++) {
      if (!PAIR && lane + 32 * u >= NS) continue;
      const float2 bz = DIM == 3 ? bj[2 * S + soff[u][2]] : make_float2(1.f, 0.f);
#pragma unroll
      for (int d = 0; d < 3 + OM; d++) accr[u][d] = fmaf(bz.x, q[d], accr[u][d]);
      if (AP && DIM == 3) {
        const float bzd = bz.x * fmaf(oj[2 * S + soff[u][2]], h, pay[NB + 9 + 2]);
#pragma unroll
        for (int r = 0; r < 3; r++) accr[u][OM + r] = fmaf(bzd, qc[r], accr[u][OM + r]);
      }
      if (FORCE)
#pragma unroll
        for (int r = 0; r < 3; r++) accr[u][3 + OM + r] = fmaf(-bz.x, t[r], fmaf(-bz.y, t2[r], accr[u][3 + OM + r]));
    }
    return;
  }
#pragma unroll
  for (int u = 0; u < NSL; u++) {
    if (!PAIR && lane + 32 * u >= NS) continue;
    const float2 bz = DIM == 3 ? bj[2 * S + soff[u][2]] : make_float2(1.f, 0.f);
    // a pair the reference drops has w = 0 and, through the masked per-axis
    // slopes (Axis::eval), grad w = 0: it adds nothing, without a branch
    const float w = wxy * bz.x;
    const float gw[3] = {gxy0 * bz.x, gxy1 * bz.x, wxy * bz.y};
    p2g_accumulate<MODE, THERMAL, Q>(accr[u], pay, w, gw);
  }
}

// Resident blocks per SM the register budget is set for: for the plain 3-D
// mechanical scatters as many as their shared memory allows (four for the
// mass and velocity sums, three for the force scatters), one (no bound) for
// the others, whose larger payloads would spill.
template <int DIM, int MODE, bool THERMAL>
constexpr int p2g_min_blocks() {
  return (DIM >= 2 && !THERMAL && p2g_kind(MODE) == MODE && !p2g_apic(MODE))
             ? ((MODE == P2G_VEL || MODE == P2G_MASS) ? 4 : 3) : 1;
}

template <int DIM, int BASIS, int MODE, bool THERMAL>
__global__ void __launch_bounds__(256, (p2g_min_blocks<DIM, MODE, THERMAL>())) k_p2g(P2GArgs a) {
  using TS = TileShape<DIM, BASIS>;
  constexpr int S = TS::S, SC = TS::SC, LO = Stencil<BASIS>::LO;
  constexpr int TX = TS::TX, TY = TS::TY, TZ = TS::TZ, L = TS::L;
  constexpr int WX = TS::WX, WY = TS::WY, WZ = TS::WZ, FX = TS::FX, NW = TS::NW, NF = TS::NF, NS = TS::NS;
  constexpr int Q = p2g_nq(MODE, THERMAL);
  constexpr int QIN = p2g_nin(MODE, THERMAL);
  constexpr int QINP = (QIN + 3) & ~3;  // staged payload row, padded for float4 access
  constexpr int NSL = (NS + 31) / 32;  // stencil nodes per lane
  constexpr bool PAIR = (DIM == 3 && S == 4);  // lane owns (a,b,c) and (a,b,c+2)
  // stencils of at most 16 nodes: the warp splits into NG lane groups of GS
  // lanes on the same nodes; group g takes particles g, g + NG, ... of the
  // cell, and a fixed butterfly of shuffles adds the groups before the flush
  constexpr int GS = PAIR ? 32 : (NS <= 4 ? 4 : (NS <= 8 ? 8 : (NS <= 16 ? 16 : 32)));
  constexpr int NG = 32 / GS;
  constexpr int SLAB = (Q * NF + 3) & ~3;
  constexpr bool AP = p2g_apic(MODE);
  constexpr int STAGE = 32 * QINP + 32 * DIM * S * (AP ? 3 : 2);

  extern __shared__ __align__(16) float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *slab = smem + warp * SLAB;                                // Q * NF
  float *spay = smem + TS::NWARP * SLAB + warp * STAGE;                                // 32 * QINP
  float2 *sbas = reinterpret_cast<float2 *>(spay + 32 * QINP);                        // 32 * DIM * S
  float *sofs = reinterpret_cast<float *>(sbas + 32 * DIM * S);  // affine modes: 32 * DIM * S offsets

  const int2 td = a.tiles[blockIdx.x];
  const GridDev g = a.grids[td.x];
  const int tlin = td.y;
  const int tile_global = g.tile_off + tlin;
  if (a.tile_end[tile_global] == a.tile_start[tile_global] || run_finished(a.scalars)) return;
  int tc[3];
  tc[2] = DIM == 3 ? tlin % g.ntile[2] : 0;
  tc[1] = DIM >= 2 ? (DIM == 3 ? (tlin / g.ntile[2]) % g.ntile[1] : tlin % g.ntile[1]) : 0;
  tc[0] = DIM == 3 ? tlin / (g.ntile[1] * g.ntile[2]) : (DIM == 2 ? tlin / g.ntile[1] : tlin);
  const float h = g.cellsize / SC, ih = g.inv_cellsize;
  const int gn0 = g.n[0], gn1 = g.n[1], gn2 = g.n[2], gng0 = g.ng[0], gng1 = g.ng[1], gng2 = g.ng[2];
  const float glo0 = g.lo[0], glo1 = g.lo[1], glo2 = g.lo[2];
  const float *P = *a.Pp;
  const size_t ps = a.ps;

  for (int k = lane; k < Q * NF; k += 32) slab[k] = 0.f;

  // stencil slots (a, b, c) of this lane
  int soff[NSL][3];
#pragma unroll
  for (int u = 0; u < NSL; u++) {
    if (PAIR) {
      soff[u][0] = (lane & 15) >> 2; soff[u][1] = lane & 3; soff[u][2] = (lane >> 4) + 2 * u;
    } else {
      const int sidx = (NG > 1 ? lane % GS : lane) + 32 * u;
      if (DIM == 3) { soff[u][0] = sidx / (S * S); soff[u][1] = (sidx / S) % S; soff[u][2] = sidx % S; }
      else if (DIM == 2) { soff[u][0] = sidx / S; soff[u][1] = sidx % S; soff[u][2] = 0; }
      else { soff[u][0] = sidx; soff[u][1] = 0; soff[u][2] = 0; }
    }
  }
  const bool lane_active = PAIR || (NG > 1 ? lane % GS : lane) < NS;
  const int grp = lane / GS;

  // the k-th cell of this warp's slab: local cell index (lx*TY + ly)*TZ + lz
  const int cell_base = tile_global * TS::NCELL + warp * L * TY * TZ;
  // prefetch registers: one particle per lane
  float ppos[DIM], ppay[QIN];
  const bool use_u = a.pos_field == PF_X;
#define KMPM_LOAD_PARTICLE(p_)                                                                   \
  do {                                                                                         \
    const int pp_ = (p_);                                                                      \
    _Pragma("unroll") for (int d = 0; d < DIM; d++) ppos[d] =                                  \
        P[(PF_X0 + d) * ps + pp_] + (use_u ? P[(PF_X + d) * ps + pp_] : 0.f);                 \
    p2g_payload<MODE, THERMAL>(a, P, pp_, ppay);                                               \
  } while (0)

  int nstart = a.cell_start[cell_base];
  int ncount = a.cell_end[cell_base] - nstart;
  if (lane < ncount) KMPM_LOAD_PARTICLE(nstart + lane);
  for (int k = 0; k < TS::CPW; k++) {
    const int cstart = nstart, ccount = ncount;
    if (k + 1 < TS::CPW) {
      nstart = a.cell_start[cell_base + k + 1];
      ncount = a.cell_end[cell_base + k + 1] - nstart;
    }
    if (ccount == 0) {
      if (k + 1 < TS::CPW && lane < ncount) KMPM_LOAD_PARTICLE(nstart + lane);
      continue;
    }
    const int lc[3] = {warp * L + k / (TY * TZ), (k / TZ) % TY, k % TZ};
    int i0[3];
    const int tco[3] = {tc[0] * TX, tc[1] * TY, tc[2] * TZ};
#pragma unroll
    for (int d = 0; d < 3; d++) i0[d] = (d < DIM) ? (tco[d] + lc[d]) * SC - LO : 0;

    float accr[NSL][Q];
#pragma unroll
    for (int u = 0; u < NSL; u++)
#pragma unroll
      for (int q = 0; q < Q; q++) accr[u][q] = 0.f;

    for (int c0 = 0; c0 < ccount; c0 += 32) {
      const int cnt = min(32, ccount - c0);
      if (c0 > 0 && lane < cnt) KMPM_LOAD_PARTICLE(cstart + c0 + lane);  // cells with more than 32 particles
      // ---- stage (lane = particle)
      // this cell's positions stay in registers (the prefetch below reuses
      // ppos); the basis loop takes particle j's from lane j by shuffles
      const float cp0 = ppos[0], cp1 = DIM >= 2 ? ppos[DIM >= 2 ? 1 : 0] : 0.f, cp2 = DIM == 3 ? ppos[DIM == 3 ? 2 : 0] : 0.f;
      if (lane < cnt) {
#pragma unroll
        for (int v = 0; v < QINP / 4; v++)
          reinterpret_cast<float4 *>(spay + lane * QINP)[v] =
              make_float4(ppay[4 * v], 4 * v + 1 < QIN ? ppay[min(4 * v + 1, QIN - 1)] : 0.f,
                          4 * v + 2 < QIN ? ppay[min(4 * v + 2, QIN - 1)] : 0.f,
                          4 * v + 3 < QIN ? ppay[min(4 * v + 3, QIN - 1)] : 0.f);
      }
      __syncwarp();
      // prefetch the next cell while this one is computed
      if (c0 + 32 >= ccount && k + 1 < TS::CPW && lane < ncount) KMPM_LOAD_PARTICLE(nstart + lane);
      // ---- per (particle, axis, slot) basis values
      bool interior = false;
      if (BASIS == 1) {
        interior = cubic_interior(i0[0], gn0, gng0);
        if (DIM >= 2) interior = interior && cubic_interior(i0[1], gn1, gng1);
        if (DIM == 3) interior = interior && cubic_interior(i0[2], gn2, gng2);
      }
      if (interior) {
        for (int base = 0; base < cnt * DIM; base += 32) {
          const int it = base + lane;
          const int j = it < cnt * DIM ? it / DIM : 0, d = it % DIM;
          const float px = __shfl_sync(0xffffffffu, cp0, j), py = __shfl_sync(0xffffffffu, cp1, j),
                      pz = __shfl_sync(0xffffffffu, cp2, j);
          if (it >= cnt * DIM) continue;
          const int i0d = d == 0 ? i0[0] : (d == 1 ? i0[1] : i0[2]);
          const float lod = d == 0 ? glo0 : (d == 1 ? glo1 : glo2);
          const float t = cells_of(d == 0 ? px : (d == 1 ? py : pz), lod, ih);
          float sv[4], dsv[4];
          const float f = t - (float)(i0d + 1);
          cubic_weights(f, ih, sv, dsv);
          // (x_node - x_p) / h of the slots from the same f (see Axis::eval)
          if (AP) {
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
              const float o = (float)(kk - 1) - f;
              sofs[it * S + kk] = o;
              // MLS forces: the moment s (x_node - x_p) Di in place of the slope
              if (a.mls) dsv[kk] = sv[kk] * (o * h) * a.mls_di;
            }
          }
#pragma unroll
          for (int kk = 0; kk < 4; kk++) sbas[it * S + kk] = make_float2(sv[kk], dsv[kk]);
        }
      } else
      for (int base = 0; base < cnt * DIM * S; base += 32) {
        const int it = base + lane;
        const int j = it < cnt * DIM * S ? it / (DIM * S) : 0, d = (it / S) % DIM, kk = it % S;
        const float px = __shfl_sync(0xffffffffu, cp0, j), py = __shfl_sync(0xffffffffu, cp1, j),
                    pz = __shfl_sync(0xffffffffu, cp2, j);
        if (it >= cnt * DIM * S) continue;
        // per-axis constants selected without indexing local arrays
        const int i = (d == 0 ? i0[0] : (d == 1 ? i0[1] : i0[2])) + kk;
        const int nd = d == 0 ? gn0 : (d == 1 ? gn1 : gn2);
        const int ngd = d == 0 ? gng0 : (d == 1 ? gng1 : gng2);
        const float lod = d == 0 ? glo0 : (d == 1 ? glo1 : glo2);
        float sv = 0.f, dsv = 0.f, ov = 0.f;
        if (i >= 0 && i < nd) {
          const float r = node_offset_cells(d == 0 ? px : (d == 1 ? py : pz), lod, i, h, ih);
          basis<BASIS>(r, node_type<BASIS>(i, ngd), ih, sv, dsv);
          dsv = sv != 0.f ? dsv : 0.f;  // as Axis::eval
          ov = -r;
          // MLS forces (compute_external_and_internal_forces_nodes_UL_MLS,
          // src/solid.cpp:524-574): w Di (x_node - x_p) in place of grad w
          if (AP && a.mls) dsv = sv * (ov * h) * a.mls_di;
        }
        (void)px; (void)py; (void)pz;
        sbas[it] = make_float2(sv, dsv);
        if (AP) sofs[it] = ov;
      }
      __syncwarp();
      // ---- accumulate (lane = stencil node); two particles per iteration for ILP
      if (lane_active) {
        const int nl = NG > 1 ? lane % GS : lane;  // node slot of this lane
        if (NG == 1) {
          int j = 0;
          for (; j + 1 < cnt; j += 2) {
            p2g_particle<DIM, S, MODE, THERMAL, Q, QINP, NSL, NS, PAIR>(accr, spay + j * QINP, sbas + j * DIM * S,
                                                                        sofs + j * DIM * S, h, soff, nl);
            p2g_particle<DIM, S, MODE, THERMAL, Q, QINP, NSL, NS, PAIR>(accr, spay + (j + 1) * QINP, sbas + (j + 1) * DIM * S,
                                                                        sofs + (j + 1) * DIM * S, h, soff, nl);
          }
          if (j < cnt)
            p2g_particle<DIM, S, MODE, THERMAL, Q, QINP, NSL, NS, PAIR>(accr, spay + j * QINP, sbas + j * DIM * S,
                                                                        sofs + j * DIM * S, h, soff, nl);
        } else {
          int j = grp;
          for (; j + NG < cnt; j += 2 * NG) {
            p2g_particle<DIM, S, MODE, THERMAL, Q, QINP, NSL, NS, PAIR>(accr, spay + j * QINP, sbas + j * DIM * S,
                                                                        sofs + j * DIM * S, h, soff, nl);
            p2g_particle<DIM, S, MODE, THERMAL, Q, QINP, NSL, NS, PAIR>(accr, spay + (j + NG) * QINP, sbas + (j + NG) * DIM * S,
                                                                        sofs + (j + NG) * DIM * S, h, soff, nl);
          }
          if (j < cnt)
            p2g_particle<DIM, S, MODE, THERMAL, Q, QINP, NSL, NS, PAIR>(accr, spay + j * QINP, sbas + j * DIM * S,
                                                                        sofs + j * DIM * S, h, soff, nl);
        }
      }
      __syncwarp();
    }
    // ---- add the lane groups (fixed butterfly: the same order on every run)
    if (NG > 1) {
#pragma unroll
      for (int u = 0; u < NSL; u++)
#pragma unroll
        for (int q = 0; q < Q; q++)
#pragma unroll
          for (int o = GS; o < 32; o <<= 1) accr[u][q] += __shfl_xor_sync(0xffffffffu, accr[u][q], o);
    }
    // ---- add into this warp's slab footprint (only this warp writes it)
    if (lane_active && grp == 0) {
#pragma unroll
      for (int u = 0; u < NSL; u++) {
        if (!PAIR && lane + 32 * u >= NS) continue;
        const int fx = (lc[0] - warp * L) * SC + soff[u][0];
        const int fy = DIM >= 2 ? lc[1] * SC + soff[u][1] : 0;
        const int fz = DIM == 3 ? lc[2] * SC + soff[u][2] : 0;
        const int fi = (fx * WY + fy) * WZ + fz;
#pragma unroll
        for (int q = 0; q < Q; q++) slab[q * NF + fi] += accr[u][q];
      }
    }
    __syncwarp();
  }
#undef KMPM_LOAD_PARTICLE
  __syncthreads();
  // ---- sum the slabs in warp order into the tile footprint
  float *out = a.partial + (size_t)tile_global * a.pstride_tile;
  for (int k = threadIdx.x; k < Q * NW; k += blockDim.x) {
    const int q = k / NW, fi = k % NW;
    const int fx = fi / (WY * WZ), fyz = fi % (WY * WZ);
    float sum = 0.f;
#pragma unroll
    for (int w = 0; w < TS::NWARP; w++) {
      const int x = fx - w * L * SC;
      if (x >= 0 && x < FX) sum += smem[w * SLAB + q * NF + x * WY * WZ + fyz];
    }
    out[k] = sum;
  }
}

// ============================================================== P2G by cell rows
// The scatter of the 3-D four-wide stencils (cubic and quadratic B-splines)
// for the plain modes (TL and UL forces, the MUSL velocity re-map, without
// thermal, affine, contact or axisymmetric terms).  Same tiles, warps and
// slab footprints as k_p2g; the cells of warp w's x-layer are visited a z-row
// (4 cells, contiguous in the sorted order) at a time:
//   - stage (lane = particle): up to 32 particles of the row at once, each
//     lane its own particle's payload and the per-axis basis values of its
//     three axes, relative to its cell;
//   - accumulate (lane = (a, b, c) with a, b the stencil's x and y slots and
//     c in {0, 1}): the particles of the row's cells in sorted order, the
//     lane adding into z slots c and c + 2 of each.  Over the row those are
//     the nodes z = c .. c + 5 of the row's footprint, held in six register
//     accumulators: the cell lz adds to accumulators lz and lz + 2, a
//     compile-time index once the four cells are unrolled;
//   - flush once per row: lanes c = 1 hand their z = 1..5 sums to lanes c = 0
//     (a fixed shuffle), which add them into the warp's slab with their own.
// Every sum runs in a fixed order: the result is bit-reproducible.
template <int MODE, int Q>
__device__ __forceinline__ void p2g_row_particle(float (&A0)[Q], float (&A2)[Q], const float *pay, float2 bx,
                                                 float2 by, float2 bz0, float2 bz2) {
  constexpr int OM = MODE == P2G_UL ? 1 : 0;  // UL sums start with the mass
  constexpr bool FORCE = MODE != P2G_VEL;
  const float wxy = bx.x * by.x;
  float q[3 + OM];
#pragma unroll
  for (int d = 0; d < 3 + OM; d++) q[d] = wxy * pay[d];
  float t[3], t2[3];
  if (FORCE) {
    const float gxy0 = bx.y * by.x, gxy1 = bx.x * by.y;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      float T0, T1, T2;
      if (MODE == P2G_TL) {  // vol0 PK1, row-major
        T0 = pay[3 + 3 * r]; T1 = pay[4 + 3 * r]; T2 = pay[5 + 3 * r];
        t[r] = fmaf(T0, gxy0, T1 * gxy1);
      } else {  // vol sigma, symmetric xx yy zz xy xz yz
        const float *sg = pay + 4;
        T0 = r == 0 ? sg[0] : (r == 1 ? sg[3] : sg[4]);
        T1 = r == 0 ? sg[3] : (r == 1 ? sg[1] : sg[5]);
        T2 = r == 0 ? sg[4] : (r == 1 ? sg[5] : sg[2]);
        t[r] = T0 * gxy0 + T1 * gxy1;
      }
      t2[r] = T2 * wxy;
    }
  }
  if (MODE == P2G_TL || MODE == P2G_UL) {
    // packed pairs of neighbouring sums, each still a = fma(s, q, a) for the
    // momentum (and UL mass) sums and a = fma(-s, t, fma(-ds, t2, a)) for the
    // forces (fma(s, -t, .) rounds as fma(-s, t, .)):
    //   TL (6 sums): (p_x, p_y) (p_z, f_x) (f_y, f_z);
    //   UL (7 sums): (m, p_x) (p_y, p_z) (f_x, f_y) f_z
    const float nt[3] = {-t[0], -t[1], -t[2]};
    const auto slot = [&](float (&A)[Q], float2 bz) {
      const float2 s2 = bc2(bz.x), nd2 = bc2(-bz.y);
      if (MODE == P2G_TL) {
        A[3] = fmaf(-bz.y, t2[0], A[3]);
        float2 f12 = ffma2(nd2, make_float2(t2[1], t2[2]), make_float2(A[4], A[5]));
        const float2 p01 = ffma2(s2, make_float2(q[0], q[1]), make_float2(A[0], A[1]));
        const float2 p2f0 = ffma2(s2, make_float2(q[2], nt[0]), make_float2(A[2], A[3]));
        f12 = ffma2(s2, make_float2(nt[1], nt[2]), f12);
        A[0] = p01.x; A[1] = p01.y; A[2] = p2f0.x; A[3] = p2f0.y; A[4] = f12.x; A[5] = f12.y;
      } else {
        const float2 mp = ffma2(s2, make_float2(q[0], q[1]), make_float2(A[0], A[1]));
        const float2 pp = ffma2(s2, make_float2(q[2], q[3]), make_float2(A[2], A[3]));
        float2 f01 = ffma2(nd2, make_float2(t2[0], t2[1]), make_float2(A[4], A[5]));
        f01 = ffma2(s2, make_float2(nt[0], nt[1]), f01);
        A[6] = fmaf(-bz.x, t[2], fmaf(-bz.y, t2[2], A[6]));
        A[0] = mp.x; A[1] = mp.y; A[2] = pp.x; A[3] = pp.y; A[4] = f01.x; A[5] = f01.y;
      }
    };
    slot(A0, bz0);
    slot(A2, bz2);
    return;
  }
#pragma unroll
  for (int d = 0; d < 3 + OM; d++) {
    A0[d] = fmaf(bz0.x, q[d], A0[d]);
    A2[d] = fmaf(bz2.x, q[d], A2[d]);
  }
  if (FORCE)
#pragma unroll
    for (int r = 0; r < 3; r++) {
      A0[3 + OM + r] = fmaf(-bz0.x, t[r], fmaf(-bz0.y, t2[r], A0[3 + OM + r]));
      A2[3 + OM + r] = fmaf(-bz2.x, t[r], fmaf(-bz2.y, t2[r], A2[3 + OM + r]));
    }
}

template <int BASIS, int MODE>
__global__ void __launch_bounds__(256, (MODE == P2G_VEL ? 4 : 3)) k_p2g_row(P2GArgs a) {
  static_assert(Stencil<BASIS>::S == 4 && Stencil<BASIS>::SC == 1, "four-wide stencils");
  using TS = TileShape<3, BASIS>;
  constexpr int S = 4, LO = Stencil<BASIS>::LO;
  constexpr int TX = TS::TX, TY = TS::TY, TZ = TS::TZ;
  constexpr int WY = TS::WY, WZ = TS::WZ, NW = TS::NW, NF = TS::NF, FX = TS::FX;
  static_assert(TS::L == 1 && TZ == 4 && FX == 4, "one x-layer of 4 x 4 cells per warp");
  constexpr int Q = p2g_nq(MODE, false);
  constexpr int QIN = p2g_nin(MODE, false);
  constexpr int QINP = (QIN + 3) & ~3;
  constexpr int SLAB = (Q * NF + 3) & ~3;
  // basis rows of SROW float2 (one per staged particle, padded so that the
  // four slots of one particle fall in different banks)
  constexpr int SROW = 33;
  constexpr int STAGE = 32 * QINP + SROW * 3 * S * 2;

  extern __shared__ __align__(16) float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *slab = smem + warp * SLAB;
  float *spay = smem + TS::NWARP * SLAB + warp * STAGE;                  // [32][QINP]
  float2 *sbas = reinterpret_cast<float2 *>(spay + 32 * QINP);          // [axis][slot][SROW]

  const int2 td = a.tiles[blockIdx.x];
  const GridDev g = a.grids[td.x];
  const int tlin = td.y;
  const int tile_global = g.tile_off + tlin;
  if (a.tile_end[tile_global] == a.tile_start[tile_global] || run_finished(a.scalars)) return;
  const int tc2 = tlin % g.ntile[2], tc1 = (tlin / g.ntile[2]) % g.ntile[1], tc0 = tlin / (g.ntile[1] * g.ntile[2]);
  const float h = g.cellsize, ih = g.inv_cellsize;
  const float *P = *a.Pp;
  const size_t ps = a.ps;
  const bool use_u = a.pos_field == PF_X;
  {  // the tile's particle rows that the stage phase reads, into L2
    const int t0 = a.tile_start[tile_global], t1 = a.tile_end[tile_global];
    prefetch_rows_l2(P, ps, PF_X0, use_u ? 6 : 3, t0, t1);
    prefetch_rows_l2(P, ps, PF_V, 4, t0, t1);  // v, mass
    if (MODE != P2G_VEL) prefetch_rows_l2(P, ps, PF_PK, MODE == P2G_TL ? 9 : 6, t0, t1);
  }

  for (int k = lane; k < Q * NF; k += 32) slab[k] = 0.f;

  // this lane's stencil slots in the accumulate phase
  const int sa = lane >> 3, sb = (lane >> 1) & 3, sc = lane & 1;
  const float2 *px = sbas + (0 * S + sa) * SROW, *py = sbas + (1 * S + sb) * SROW;
  const float2 *pz0 = sbas + (2 * S + sc) * SROW, *pz2 = sbas + (2 * S + sc + 2) * SROW;
  const int i0x = (tc0 * TX + warp) - LO;
  // the particle ranges of the warp's TY x 4 cells (local index
  // (lx TY + ly) TZ + lz), in one load: lane k < 16 holds the start of cell
  // k, lane 16 + k its end
  static_assert(TY * TZ == 16, "16 cells per warp");
  const int cw = tile_global * TS::NCELL + warp * TY * TZ;
  const int cvw = lane < 16 ? a.cell_start[cw + lane] : a.cell_end[cw + lane - 16];

  for (int ly = 0; ly < TY; ly++) {
    // the row's four cells and their particle ranges [st, en); the non-empty
    // ones are contiguous in the sorted order (an empty cell's range is
    // st == en, of any value)
    int st[4], en[4], lo4[4];
    int rs = INT_MAX, re = INT_MIN;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      st[k] = __shfl_sync(0xffffffffu, cvw, ly * TZ + k);
      en[k] = __shfl_sync(0xffffffffu, cvw, 16 + ly * TZ + k);
      const bool full = en[k] > st[k];
      lo4[k] = full ? st[k] : INT_MAX;
      rs = full ? min(rs, st[k]) : rs;
      re = full ? max(re, en[k]) : re;
    }
    if (rs == INT_MAX) continue;
    const int i0y = (tc1 * TY + ly) - LO;
    float acc[6][Q];
#pragma unroll
    for (int m = 0; m < 6; m++)
#pragma unroll
      for (int qq = 0; qq < Q; qq++) acc[m][qq] = 0.f;

    for (int c0 = rs; c0 < re; c0 += 32) {
      const int cnt = min(32, re - c0);
      // ---- stage (lane = particle)
      if (lane < cnt) {
        const int p = c0 + lane;
        int lz = 0;  // the non-empty cell holding p: the last one starting at or before it
#pragma unroll
        for (int k = 1; k < 4; k++) lz = lo4[k] <= p ? k : lz;
        float pay[QIN];
        p2g_payload<MODE, false>(a, P, p, pay);
#pragma unroll
        for (int v = 0; v < QINP / 4; v++)
          reinterpret_cast<float4 *>(spay + lane * QINP)[v] =
              make_float4(pay[4 * v], 4 * v + 1 < QIN ? pay[min(4 * v + 1, QIN - 1)] : 0.f,
                          4 * v + 2 < QIN ? pay[min(4 * v + 2, QIN - 1)] : 0.f,
                          4 * v + 3 < QIN ? pay[min(4 * v + 3, QIN - 1)] : 0.f);
        const int i0[3] = {i0x, i0y, (tc2 * TZ + lz) - LO};
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const float xp = P[(PF_X0 + d) * ps + p] + (use_u ? P[(PF_X + d) * ps + p] : 0.f);
          const float lod = d == 0 ? g.lo[0] : (d == 1 ? g.lo[1] : g.lo[2]);
          const int nd = d == 0 ? g.n[0] : (d == 1 ? g.n[1] : g.n[2]);
          const int ngd = d == 0 ? g.ng[0] : (d == 1 ? g.ng[1] : g.ng[2]);
          float sv[S], dsv[S];
          if (BASIS == 1 && cubic_interior(i0[d], nd, ngd)) {
            cubic_weights(cells_of(xp, lod, ih) - (float)(i0[d] + 1), ih, sv, dsv);
          } else {
#pragma unroll
            for (int kk = 0; kk < S; kk++) {
              const int i = i0[d] + kk;
              sv[kk] = 0.f;
              dsv[kk] = 0.f;
              if (i >= 0 && i < nd) {
                const float r = node_offset_cells(xp, lod, i, h, ih);
                basis<BASIS>(r, node_type<BASIS>(i, ngd), ih, sv[kk], dsv[kk]);
                dsv[kk] = sv[kk] != 0.f ? dsv[kk] : 0.f;  // as Axis::eval
              }
            }
          }
#pragma unroll
          for (int kk = 0; kk < S; kk++) sbas[(d * S + kk) * SROW + lane] = make_float2(sv[kk], dsv[kk]);
        }
      }
      __syncwarp();
      // ---- accumulate (lane = node): cell after cell, particles in sorted order
#pragma unroll
      for (int lz = 0; lz < 4; lz++) {
        const int jlo = max(st[lz] - c0, 0), jhi = min(en[lz] - c0, cnt);
        for (int j = jlo; j < jhi; j++) {
          float pay[QINP];
#pragma unroll
          for (int v = 0; v < QINP / 4; v++) {
            const float4 t4 = reinterpret_cast<const float4 *>(spay + j * QINP)[v];
            pay[4 * v] = t4.x; pay[4 * v + 1] = t4.y; pay[4 * v + 2] = t4.z; pay[4 * v + 3] = t4.w;
          }
          p2g_row_particle<MODE, Q>(acc[lz], acc[lz + 2], pay, px[j], py[j], pz0[j], pz2[j]);
        }
      }
      __syncwarp();
    }
    // ---- flush: lanes c = 1 hold z = 1..6 as accumulators 0..5; their z = 1..5
    // join the c = 0 lanes' accumulators 1..5 (a fixed order)
#pragma unroll
    for (int m = 0; m < 5; m++)
#pragma unroll
      for (int qq = 0; qq < Q; qq++) {
        const float o = __shfl_xor_sync(0xffffffffu, acc[m][qq], 1);
        if (sc == 0) acc[m + 1][qq] += o;
      }
    const int fy = ly + sb;
#pragma unroll
    for (int m = 0; m < 6; m++) {
      if (sc == 1 && m < 5) continue;
      const int fz = m + sc;
      const int fi = (sa * WY + fy) * WZ + fz;
#pragma unroll
      for (int qq = 0; qq < Q; qq++) slab[qq * NF + fi] += acc[m][qq];
    }
    __syncwarp();
  }
  __syncthreads();
  // ---- sum the slabs in warp order into the tile footprint
  float *out = a.partial + (size_t)tile_global * a.pstride_tile;
  for (int k = threadIdx.x; k < Q * NW; k += blockDim.x) {
    const int qq = k / NW, fi = k % NW;
    const int fx = fi / (WY * WZ), fyz = fi % (WY * WZ);
    float sum = 0.f;
#pragma unroll
    for (int w = 0; w < TS::NWARP; w++) {
      const int x = fx - w;
      if (x >= 0 && x < FX) sum += smem[w * SLAB + qq * NF + x * WY * WZ + fyz];
    }
    out[k] = sum;
  }
}

// dynamic shared memory of k_p2g_force_row (bytes)
template <int BASIS> constexpr int p2g_force_row_smem() {
  using TS = TileShape<3, BASIS>;
  return 4 * TS::NWARP * (((3 * TS::NF + 3) & ~3) + 32 * 12 + 34 * 2 * 4 * 2 + 2 * 32 * 4);
}

// ============================================================== force-only P2G by half-warps
// The TLMPM force scatter of the momentum reuse (P2G_TL | P2G_FONLY): the
// tiles, warps, rows of four cells and slab footprints of k_p2g_row, with
// the row's particles shared between the two half-warps:
//   - stage (lane = particle): payload vol0 PK1 (9 floats) and the per-axis
//     values and slopes, the z axis as two float4 (s0 ds0 s1 ds1) (s2 ds2
//     s3 ds3) per particle;
//   - accumulate: half-warp h takes particles jlo + h, jlo + h + 2, ... of
//     each cell, in sorted order; lane (a, b) of a half adds into x slot a,
//     y slot b and all four z slots, seven register sums per force
//     component over the row's z nodes.  The per-particle terms of a lane
//     (the (a, b) products of PK1 with the x and y values and slopes) are
//     formed once for four slots, where k_p2g_row forms them for two;
//   - flush once per row: half 1's sums join half 0's by one shuffle, and
//     half 0 adds the row into the warp's slab.
// Every sum runs in a fixed order: the result is bit-reproducible.
template <int BASIS>
__global__ void __launch_bounds__(256, 4) k_p2g_force_row(P2GArgs a) {
  static_assert(Stencil<BASIS>::S == 4 && Stencil<BASIS>::SC == 1, "four-wide stencils");
  using TS = TileShape<3, BASIS>;
  constexpr int S = 4, LO = Stencil<BASIS>::LO;
  constexpr int TX = TS::TX, TY = TS::TY, TZ = TS::TZ;
  constexpr int WY = TS::WY, WZ = TS::WZ, NW = TS::NW, NF = TS::NF, FX = TS::FX;
  static_assert(TS::L == 1 && TZ == 4 && FX == 4, "one x-layer of 4 x 4 cells per warp");
  constexpr int Q = 3;
  constexpr int SLAB = (Q * NF + 3) & ~3;
  constexpr int SROW = 34;  // x, y rows of float2: the two halves' reads fall in different banks
  constexpr int STAGE = 32 * 12 + SROW * 2 * S * 2 + 2 * 32 * 4;
  static_assert(p2g_force_row_smem<BASIS>() == 4 * TS::NWARP * (SLAB + STAGE), "shared-memory size");

  extern __shared__ __align__(16) float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *slab = smem + warp * SLAB;
  float *spay = smem + TS::NWARP * SLAB + warp * STAGE;                 // [32][12]
  float2 *sbxy = reinterpret_cast<float2 *>(spay + 32 * 12);           // [axis x, y][slot][SROW]
  float4 *sbz = reinterpret_cast<float4 *>(sbxy + 2 * S * SROW);       // [pair][32]

  const int2 td = a.tiles[blockIdx.x];
  const GridDev g = a.grids[td.x];
  const int tlin = td.y;
  const int tile_global = g.tile_off + tlin;
  if (a.tile_end[tile_global] == a.tile_start[tile_global] || run_finished(a.scalars)) return;
  const int tc2 = tlin % g.ntile[2], tc1 = (tlin / g.ntile[2]) % g.ntile[1], tc0 = tlin / (g.ntile[1] * g.ntile[2]);
  const float h = g.cellsize, ih = g.inv_cellsize;
  const float *P = *a.Pp;
  const size_t ps = a.ps;
  {  // the tile's x0 and vol0 PK1 rows, into L2
    const int t0 = a.tile_start[tile_global], t1 = a.tile_end[tile_global];
    prefetch_rows_l2(P, ps, PF_X0, 3, t0, t1);
    prefetch_rows_l2(P, ps, PF_PK, 9, t0, t1);
  }

  for (int k = lane; k < Q * NF; k += 32) slab[k] = 0.f;

  // this lane's half and stencil slots in the accumulate phase
  const int hw = lane >> 4, sa = (lane >> 2) & 3, sb = lane & 3;
  const float2 *px = sbxy + (0 * S + sa) * SROW, *py = sbxy + (1 * S + sb) * SROW;
  const int i0x = (tc0 * TX + warp) - LO;
  // the particle ranges of the warp's TY x 4 cells, in one load: lane k < 16
  // holds the start of cell k, lane 16 + k its end
  static_assert(TY * TZ == 16, "16 cells per warp");
  const int cw = tile_global * TS::NCELL + warp * TY * TZ;
  const int cvw = lane < 16 ? a.cell_start[cw + lane] : a.cell_end[cw + lane - 16];

  for (int ly = 0; ly < TY; ly++) {
    // the row's four cells and their particle ranges (as k_p2g_row)
    int st[4], en[4], lo4[4];
    int rs = INT_MAX, re = INT_MIN;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      st[k] = __shfl_sync(0xffffffffu, cvw, ly * TZ + k);
      en[k] = __shfl_sync(0xffffffffu, cvw, 16 + ly * TZ + k);
      const bool full = en[k] > st[k];
      lo4[k] = full ? st[k] : INT_MAX;
      rs = full ? min(rs, st[k]) : rs;
      re = full ? max(re, en[k]) : re;
    }
    if (rs == INT_MAX) continue;
    const int i0y = (tc1 * TY + ly) - LO;
    float acc[7][Q];
#pragma unroll
    for (int m = 0; m < 7; m++)
#pragma unroll
      for (int qq = 0; qq < Q; qq++) acc[m][qq] = 0.f;

    for (int c0 = rs; c0 < re; c0 += 32) {
      const int cnt = min(32, re - c0);
      // ---- stage (lane = particle)
      if (lane < cnt) {
        const int p = c0 + lane;
        int lz = 0;
#pragma unroll
        for (int k = 1; k < 4; k++) lz = lo4[k] <= p ? k : lz;
        // every load of the particle before the first shared-memory store
        float pay[9], x0p[3];
#pragma unroll
        for (int k = 0; k < 9; k++) pay[k] = P[(PF_PK + k) * ps + p];
#pragma unroll
        for (int d = 0; d < 3; d++) x0p[d] = P[(PF_X0 + d) * ps + p];
        reinterpret_cast<float4 *>(spay + lane * 12)[0] = make_float4(pay[0], pay[1], pay[2], pay[3]);
        reinterpret_cast<float4 *>(spay + lane * 12)[1] = make_float4(pay[4], pay[5], pay[6], pay[7]);
        spay[lane * 12 + 8] = pay[8];
        const int i0[3] = {i0x, i0y, (tc2 * TZ + lz) - LO};
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const float xp = x0p[d];
          const float lod = d == 0 ? g.lo[0] : (d == 1 ? g.lo[1] : g.lo[2]);
          const int nd = d == 0 ? g.n[0] : (d == 1 ? g.n[1] : g.n[2]);
          const int ngd = d == 0 ? g.ng[0] : (d == 1 ? g.ng[1] : g.ng[2]);
          float sv[S], dsv[S];
          if (BASIS == 1 && cubic_interior(i0[d], nd, ngd)) {
            cubic_weights(cells_of(xp, lod, ih) - (float)(i0[d] + 1), ih, sv, dsv);
          } else {
#pragma unroll
            for (int kk = 0; kk < S; kk++) {
              const int i = i0[d] + kk;
              sv[kk] = 0.f;
              dsv[kk] = 0.f;
              if (i >= 0 && i < nd) {
                const float r = node_offset_cells(xp, lod, i, h, ih);
                basis<BASIS>(r, node_type<BASIS>(i, ngd), ih, sv[kk], dsv[kk]);
                dsv[kk] = sv[kk] != 0.f ? dsv[kk] : 0.f;  // as Axis::eval
              }
            }
          }
          if (d < 2) {
#pragma unroll
            for (int kk = 0; kk < S; kk++) sbxy[(d * S + kk) * SROW + lane] = make_float2(sv[kk], dsv[kk]);
          } else {
            sbz[lane] = make_float4(sv[0], dsv[0], sv[1], dsv[1]);
            sbz[32 + lane] = make_float4(sv[2], dsv[2], sv[3], dsv[3]);
          }
        }
      }
      __syncwarp();
      // ---- accumulate (half-warp = particle, lane = (x, y) slot pair)
#pragma unroll
      for (int lz = 0; lz < 4; lz++) {
        const int jlo = max(st[lz] - c0, 0), jhi = min(en[lz] - c0, cnt);
        for (int j = jlo + hw; j < jhi; j += 2) {
          const float4 pa = reinterpret_cast<const float4 *>(spay + j * 12)[0];
          const float4 pb = reinterpret_cast<const float4 *>(spay + j * 12)[1];
          const float p8 = spay[j * 12 + 8];
          const float T[9] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w, p8};
          const float2 bx = px[j], by = py[j];
          const float4 z01 = sbz[j], z23 = sbz[32 + j];
          const float zs[4] = {z01.x, z01.z, z23.x, z23.z}, zd[4] = {z01.y, z01.w, z23.y, z23.w};
          const float wxy = bx.x * by.x, gxy0 = bx.y * by.x, gxy1 = bx.x * by.y;
#pragma unroll
          for (int r = 0; r < 3; r++) {
            // f_r -= PK1(r, :) . grad w: the x and y parts t, the z part t2
            const float t = fmaf(T[3 * r], gxy0, T[3 * r + 1] * gxy1), t2 = T[3 * r + 2] * wxy;
#pragma unroll
            for (int c = 0; c < 4; c++) acc[lz + c][r] = fmaf(-zs[c], t, fmaf(-zd[c], t2, acc[lz + c][r]));
          }
        }
      }
      __syncwarp();
    }
    // ---- flush: half 1's sums join half 0's, which adds the row into the slab
#pragma unroll
    for (int m = 0; m < 7; m++)
#pragma unroll
      for (int qq = 0; qq < Q; qq++) acc[m][qq] += __shfl_xor_sync(0xffffffffu, acc[m][qq], 16);
    if (hw == 0) {
      const int fy = ly + sb;
#pragma unroll
      for (int m = 0; m < 7; m++) {
        const int fi = (sa * WY + fy) * WZ + m;
#pragma unroll
        for (int qq = 0; qq < Q; qq++) slab[qq * NF + fi] += acc[m][qq];
      }
    }
    __syncwarp();
  }
  __syncthreads();
  // ---- sum the slabs in warp order into the tile footprint
  float *out = a.partial + (size_t)tile_global * a.pstride_tile;
  for (int k = threadIdx.x; k < Q * NW; k += blockDim.x) {
    const int qq = k / NW, fi = k % NW;
    const int fx = fi / (WY * WZ), fyz = fi % (WY * WZ);
    float sum = 0.f;
#pragma unroll
    for (int w = 0; w < TS::NWARP; w++) {
      const int x = fx - w;
      if (x >= 0 && x < FX) sum += smem[w * SLAB + qq * NF + x * WY * WZ + fyz];
    }
    out[k] = sum;
  }
}

// ============================================================== velocity row scatter by half-warps
// The sums of compute_velocity_nodes (Σ w m v, the MUSL re-map) over the
// rows of four cells of k_p2g_row, the row's particles shared between the
// two half-warps as in k_p2g_force_row: half-warp hw takes particles
// jlo + hw, jlo + hw + 2, ... of each cell in sorted order, and lane (a, b)
// of a half adds into x slot a, y slot b and all four z slots, seven
// register sums per component over the row's z nodes.  The fused MUSL pass
// (k_g2p1_remap_row) and the velocity scatter (k_p2g_vel_row) share this
// code, so they give the same bits.  Staged per warp: m v (float4 per
// particle), the x and y weights in rows of VROW floats per slot (the two
// halves' reads fall in different banks), the four z weights as one float4.
constexpr int VROW = 36;
constexpr int VEL_STAGE = 32 * 4 + 2 * 4 * VROW + 32 * 4;  // floats per warp

__device__ __forceinline__ void vel_row_stage_basis(float *sbxy, float4 *sbz, int lane, const float (&sv)[3][4]) {
#pragma unroll
  for (int kk = 0; kk < 4; kk++) {
    sbxy[kk * VROW + lane] = sv[0][kk];
    sbxy[(4 + kk) * VROW + lane] = sv[1][kk];
  }
  sbz[lane] = make_float4(sv[2][0], sv[2][1], sv[2][2], sv[2][3]);
}

__device__ __forceinline__ void vel_row_accumulate(float (&acc)[7][3], const float *spay, const float *px,
                                                   const float *py, const float4 *sbz, const int (&st)[4],
                                                   const int (&en)[4], int c0, int cnt, int hw) {
#pragma unroll
  for (int lz = 0; lz < 4; lz++) {
    const int jlo = max(st[lz] - c0, 0), jhi = min(en[lz] - c0, cnt);
    for (int j = jlo + hw; j < jhi; j += 2) {
      const float4 t4 = reinterpret_cast<const float4 *>(spay)[j];
      const float wxy = px[j] * py[j];
      const float q[3] = {wxy * t4.x, wxy * t4.y, wxy * t4.z};
      const float4 z = sbz[j];
      const float zs[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
      for (int c = 0; c < 4; c++)
#pragma unroll
        for (int r = 0; r < 3; r++) acc[lz + c][r] = fmaf(zs[c], q[r], acc[lz + c][r]);
    }
  }
}

// flush of one row: half 1's sums join half 0's, which adds them into the
// warp's slab (x slot sa, y node ly + sb, z nodes 0..6 of the row)
template <int WY, int WZ, int NF>
__device__ __forceinline__ void vel_row_flush(float (&acc)[7][3], float *slab, int hw, int sa, int sb, int ly) {
#pragma unroll
  for (int m = 0; m < 7; m++)
#pragma unroll
    for (int r = 0; r < 3; r++) acc[m][r] += __shfl_xor_sync(0xffffffffu, acc[m][r], 16);
  if (hw == 0) {
#pragma unroll
    for (int m = 0; m < 7; m++) {
      const int fi = (sa * WY + ly + sb) * WZ + m;
#pragma unroll
      for (int r = 0; r < 3; r++) slab[r * NF + fi] += acc[m][r];
    }
  }
}

// The velocity scatter (P2G_VEL) of the plain 3-D four-wide modes: the tiles,
// warps, rows and slab footprints of k_p2g_row, the sums of vel_row_accumulate.
template <int BASIS>
__global__ void __launch_bounds__(256, 4) k_p2g_vel_row(P2GArgs a) {
  static_assert(Stencil<BASIS>::S == 4 && Stencil<BASIS>::SC == 1, "four-wide stencils");
  using TS = TileShape<3, BASIS>;
  constexpr int S = 4, LO = Stencil<BASIS>::LO;
  constexpr int TX = TS::TX, TY = TS::TY, TZ = TS::TZ;
  constexpr int WY = TS::WY, WZ = TS::WZ, NW = TS::NW, NF = TS::NF, FX = TS::FX;
  static_assert(TS::L == 1 && TZ == 4 && FX == 4, "one x-layer of 4 x 4 cells per warp");
  constexpr int Q = 3;
  constexpr int SLAB = (Q * NF + 3) & ~3;

  extern __shared__ __align__(16) float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *slab = smem + warp * SLAB;
  float *spay = smem + TS::NWARP * SLAB + warp * VEL_STAGE;  // [32][4]
  float *sbxy = spay + 32 * 4;                               // [axis x, y][slot][VROW]
  float4 *sbz = reinterpret_cast<float4 *>(sbxy + 2 * 4 * VROW);

  const int2 td = a.tiles[blockIdx.x];
  const GridDev g = a.grids[td.x];
  const int tlin = td.y;
  const int tile_global = g.tile_off + tlin;
  if (a.tile_end[tile_global] == a.tile_start[tile_global] || run_finished(a.scalars)) return;
  const int tc2 = tlin % g.ntile[2], tc1 = (tlin / g.ntile[2]) % g.ntile[1], tc0 = tlin / (g.ntile[1] * g.ntile[2]);
  const float h = g.cellsize, ih = g.inv_cellsize;
  const float *P = *a.Pp;
  const size_t ps = a.ps;
  const bool use_u = a.pos_field == PF_X;
  {  // the tile's particle rows that the stage phase reads, into L2
    const int t0 = a.tile_start[tile_global], t1 = a.tile_end[tile_global];
    prefetch_rows_l2(P, ps, PF_X0, use_u ? 6 : 3, t0, t1);
    prefetch_rows_l2(P, ps, PF_V, 4, t0, t1);  // v, mass
  }

  for (int k = lane; k < Q * NF; k += 32) slab[k] = 0.f;

  const int hw = lane >> 4, sa = (lane >> 2) & 3, sb = lane & 3;
  const float *px = sbxy + sa * VROW, *py = sbxy + (4 + sb) * VROW;
  const int i0x = (tc0 * TX + warp) - LO;
  // the particle ranges of the warp's TY x 4 cells, in one load (as k_p2g_force_row)
  static_assert(TY * TZ == 16, "16 cells per warp");
  const int cw = tile_global * TS::NCELL + warp * TY * TZ;
  const int cvw = lane < 16 ? a.cell_start[cw + lane] : a.cell_end[cw + lane - 16];

  for (int ly = 0; ly < TY; ly++) {
    int st[4], en[4], lo4[4];
    int rs = INT_MAX, re = INT_MIN;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      st[k] = __shfl_sync(0xffffffffu, cvw, ly * TZ + k);
      en[k] = __shfl_sync(0xffffffffu, cvw, 16 + ly * TZ + k);
      const bool full = en[k] > st[k];
      lo4[k] = full ? st[k] : INT_MAX;
      rs = full ? min(rs, st[k]) : rs;
      re = full ? max(re, en[k]) : re;
    }
    if (rs == INT_MAX) continue;
    const int i0y = (tc1 * TY + ly) - LO;
    float acc[7][Q];
#pragma unroll
    for (int m = 0; m < 7; m++)
#pragma unroll
      for (int qq = 0; qq < Q; qq++) acc[m][qq] = 0.f;

    for (int c0 = rs; c0 < re; c0 += 32) {
      const int cnt = min(32, re - c0);
      // ---- stage (lane = particle): m v and the weights
      if (lane < cnt) {
        const int p = c0 + lane;
        int lz = 0;
#pragma unroll
        for (int k = 1; k < 4; k++) lz = lo4[k] <= p ? k : lz;
        float pay[3];
        p2g_payload<P2G_VEL, false>(a, P, p, pay);
        reinterpret_cast<float4 *>(spay)[lane] = make_float4(pay[0], pay[1], pay[2], 0.f);
        const int i0[3] = {i0x, i0y, (tc2 * TZ + lz) - LO};
        float sv[3][S];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const float xp = P[(PF_X0 + d) * ps + p] + (use_u ? P[(PF_X + d) * ps + p] : 0.f);
          const float lod = d == 0 ? g.lo[0] : (d == 1 ? g.lo[1] : g.lo[2]);
          const int nd = d == 0 ? g.n[0] : (d == 1 ? g.n[1] : g.n[2]);
          const int ngd = d == 0 ? g.ng[0] : (d == 1 ? g.ng[1] : g.ng[2]);
          float dsv[S];
          if (BASIS == 1 && cubic_interior(i0[d], nd, ngd)) {
            cubic_weights(cells_of(xp, lod, ih) - (float)(i0[d] + 1), ih, sv[d], dsv);
          } else {
#pragma unroll
            for (int kk = 0; kk < S; kk++) {
              const int i = i0[d] + kk;
              sv[d][kk] = 0.f;
              dsv[kk] = 0.f;
              if (i >= 0 && i < nd) {
                const float r = node_offset_cells(xp, lod, i, h, ih);
                basis<BASIS>(r, node_type<BASIS>(i, ngd), ih, sv[d][kk], dsv[kk]);
              }
            }
          }
        }
        vel_row_stage_basis(sbxy, sbz, lane, sv);
      }
      __syncwarp();
      vel_row_accumulate(acc, spay, px, py, sbz, st, en, c0, cnt, hw);
      __syncwarp();
    }
    vel_row_flush<WY, WZ, NF>(acc, slab, hw, sa, sb, ly);
    __syncwarp();
  }
  __syncthreads();
  // ---- sum the slabs in warp order into the tile footprint
  float *out = a.partial + (size_t)tile_global * a.pstride_tile;
  for (int k = threadIdx.x; k < Q * NW; k += blockDim.x) {
    const int qq = k / NW, fi = k % NW;
    const int fx = fi / (WY * WZ), fyz = fi % (WY * WZ);
    float sum = 0.f;
#pragma unroll
    for (int w = 0; w < TS::NWARP; w++) {
      const int x = fx - w;
      if (x >= 0 && x < FX) sum += smem[w * SLAB + qq * NF + x * WY * WZ + fyz];
    }
    out[k] = sum;
  }
}

// ============================================================== 2-D P2G by cell rows
// The scatter of the 2-D four-wide stencils (cubic and quadratic B-splines)
// for the plain modes, on the tiles, warps and slab footprints of k_p2g (a
// warp owns two x-columns of 16 cells).  A column is visited in rows of 4
// cells along y (contiguous in the sorted order):
//   - stage (lane = particle): up to 32 particles of the row, each lane its
//     own particle's payload and per-axis basis values;
//   - accumulate: four lane groups of 8 take the row's particles in turn
//     (particle j of the row goes to group j mod 4, j counted from the row's
//     first particle); lane (a, c) of a group adds into x slot a and y slots
//     c and c + 2 of each of its particles, six register accumulators over
//     the row's y nodes c .. c + 5, as k_p2g_row does along z;
//   - flush once per row: a fixed butterfly adds the four groups, the c = 1
//     lanes hand their y = 1..5 sums to the c = 0 lanes, and group 0 adds
//     the row into the warp's slab.
// Every sum runs in a fixed order: the result is bit-reproducible.
__device__ __forceinline__ void raise_error(ErrState *e, int code, int p, long long step);  // (G2P below)

// dynamic shared memory of k_p2g_row2<.., P2G_VEL, REMAP> (bytes): the
// velocity scatter's, then the tile's node footprint (24 bytes per node)
template <int BASIS> constexpr int p2g_row2_remap_smem() {
  using TS = TileShape<2, BASIS>;
  constexpr int QINP = (p2g_nin(P2G_VEL, false) + 3) & ~3;
  return 4 * (TS::NWARP * (((3 * TS::NF + 3) & ~3) + 32 * QINP + 33 * 2 * 4 * 2) + 6 * ((TS::NW + 1) & ~1));
}

// REMAP (MODE P2G_VEL; 1 TLMPM, 2 ULMPM): the MUSL gather, particle update
// and re-map in one pass, as k_g2p1_remap_row does in 3-D.  The block stages
// its tile's node footprint of (v, v_update), and each particle's stage also
// gathers its 16 nodes there in k_g2p1's order, moves the particle and
// stages m v_new: the scatter that follows is this kernel's own, so the sums
// are those of k_g2p1 then the plain velocity scatter, bit for bit.
template <int BASIS, int MODE, int REMAP = 0>
__global__ void __launch_bounds__(256, (MODE == P2G_VEL || p2g_fonly(MODE) ? 4 : 3)) k_p2g_row2(P2GArgs a) {
  static_assert(REMAP == 0 || MODE == P2G_VEL, "the re-map pass is a velocity scatter");
  static_assert(Stencil<BASIS>::S == 4 && Stencil<BASIS>::SC == 1, "four-wide stencils");
  using TS = TileShape<2, BASIS>;
  constexpr int S = 4, LO = Stencil<BASIS>::LO;
  constexpr int TX = TS::TX, TY = TS::TY, L = TS::L;
  constexpr int WY = TS::WY, NW = TS::NW, NF = TS::NF, FX = TS::FX;
  static_assert(TY % 4 == 0 && TS::WZ == 1, "rows of 4 cells along y");
  constexpr int Q = p2g_nq(MODE, false);
  constexpr int QIN = p2g_nin(MODE, false);
  constexpr int QINP = (QIN + 3) & ~3;
  constexpr int SLAB = (Q * NF + 3) & ~3;
  constexpr int SROW = 33;
  constexpr int STAGE = 32 * QINP + SROW * 2 * S * 2;
  constexpr int OM = MODE == P2G_UL ? 1 : 0;  // UL sums start with the mass
  constexpr bool FORCE = MODE != P2G_VEL;
  // P2G_TL | P2G_FONLY (TLMPM MUSL momentum reuse): the force sums only, at
  // quantities 0..2, in the arithmetic and order of the P2G_TL force sums;
  // payload vol0 PK1
  constexpr bool FO = p2g_fonly(MODE);

  extern __shared__ __align__(16) float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *slab = smem + warp * SLAB;
  float *spay = smem + TS::NWARP * SLAB + warp * STAGE;           // [32][QINP]
  float2 *sbas = reinterpret_cast<float2 *>(spay + 32 * QINP);    // [axis][slot][SROW]

  const int2 td = a.tiles[blockIdx.x];
  const GridDev g = a.grids[td.x];
  const int tlin = td.y;
  const int tile_global = g.tile_off + tlin;
  if (a.tile_end[tile_global] == a.tile_start[tile_global] || run_finished(a.scalars)) return;
  const int tc1 = tlin % g.ntile[1], tc0 = tlin / g.ntile[1];
  const float h = g.cellsize, ih = g.inv_cellsize;
  float *P = *a.Pp;
  const size_t ps = a.ps;
  const bool use_u = a.pos_field == PF_X;
  constexpr int NWP = (NW + 1) & ~1;
  float4 *fpA = reinterpret_cast<float4 *>(smem + TS::NWARP * (SLAB + STAGE));  // (v, v_update.x)
  float2 *fpB = reinterpret_cast<float2 *>(fpA + NWP);                          // (v_update.y, v_update.z)
  float dt = 0.f, alpha = 0.f;
  long long nstep = 0;
  if (REMAP) {
    const StepScalars &sc0 = a.scalars[a.indep ? g.solid0 : 0];
    dt = (float)sc0.dt;
    nstep = sc0.ntimestep;
    alpha = a.pic_flip;
    prefetch_rows_l2(P, ps, PF_X0, PF_MASS + 1 - PF_X0, a.tile_start[tile_global], a.tile_end[tile_global]);
    // the tile's node footprint: nodes (tc TX - LO + fx, tc TY - LO + fy)
    const float4 *__restrict__ NA = a.nodeA + NODE_STRIDE * g.node_off;
    const int b0 = tc0 * TX - LO, b1 = tc1 * TY - LO;
    for (int e = threadIdx.x; e < NW; e += blockDim.x) {
      const int fy = e % WY, fx = e / WY;
      const int ix = b0 + fx, iy = b1 + fy;
      float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A;
      if (ix >= 0 && ix < g.n[0] && iy >= 0 && iy < g.n[1]) ld_node_pair(NA + NODE_STRIDE * (ix * g.n[1] + iy), A, B);
      fpA[e] = make_float4(A.x, A.y, A.z, B.x);
      fpB[e] = make_float2(B.y, B.z);
    }
    __syncthreads();
  }

  for (int k = lane; k < Q * NF; k += 32) slab[k] = 0.f;

  const int grp = lane >> 3, sa = (lane >> 1) & 3, sc = lane & 1;
  const float2 *px = sbas + (0 * S + sa) * SROW;
  const float2 *py0 = sbas + (1 * S + sc) * SROW, *py2 = sbas + (1 * S + sc + 2) * SROW;

  // the particle ranges of the warp's L x TY cells (local index lx' TY + ly),
  // in one load: lane k holds the start and the end of cell k
  static_assert(L * TY == 32, "32 cells per warp");
  const int cw = tile_global * TS::NCELL + warp * L * TY;
  const int cvs = a.cell_start[cw + lane], cve = a.cell_end[cw + lane];

  for (int lx = 0; lx < L; lx++) {
    const int i0x = (tc0 * TX + warp * L + lx) - LO;
    for (int ly0 = 0; ly0 < TY; ly0 += 4) {
      // the row's four cells and their ranges
      int st[4], en[4], lo4[4];
      int rs = INT_MAX, re = INT_MIN;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        st[k] = __shfl_sync(0xffffffffu, cvs, lx * TY + ly0 + k);
        en[k] = __shfl_sync(0xffffffffu, cve, lx * TY + ly0 + k);
        const bool full = en[k] > st[k];
        lo4[k] = full ? st[k] : INT_MAX;
        rs = full ? min(rs, st[k]) : rs;
        re = full ? max(re, en[k]) : re;
      }
      if (rs == INT_MAX) continue;
      float acc[6][Q];
#pragma unroll
      for (int m = 0; m < 6; m++)
#pragma unroll
        for (int qq = 0; qq < Q; qq++) acc[m][qq] = 0.f;

      for (int c0 = rs; c0 < re; c0 += 32) {
        const int cnt = min(32, re - c0);
        // ---- stage (lane = particle)
        if (lane < cnt) {
          const int p = c0 + lane;
          int ly = 0;  // the non-empty cell holding p: the last one starting at or before it
#pragma unroll
          for (int k = 1; k < 4; k++) ly = lo4[k] <= p ? k : ly;
          float pay[QIN];
          if (!REMAP) p2g_payload<MODE, false>(a, P, p, pay);
          const int i0[2] = {i0x, (tc1 * TY + ly0 + ly) - LO};
          float svs[2][S];
#pragma unroll
          for (int d = 0; d < 2; d++) {
            const float xp = P[(PF_X0 + d) * ps + p] + (use_u ? P[(PF_X + d) * ps + p] : 0.f);
            const float lod = d == 0 ? g.lo[0] : g.lo[1];
            const int nd = d == 0 ? g.n[0] : g.n[1];
            const int ngd = d == 0 ? g.ng[0] : g.ng[1];
            float sv[S], dsv[S];
            if (BASIS == 1 && cubic_interior(i0[d], nd, ngd)) {
              cubic_weights(cells_of(xp, lod, ih) - (float)(i0[d] + 1), ih, sv, dsv);
            } else {
#pragma unroll
              for (int kk = 0; kk < S; kk++) {
                const int i = i0[d] + kk;
                sv[kk] = 0.f;
                dsv[kk] = 0.f;
                if (i >= 0 && i < nd) {
                  const float r = node_offset_cells(xp, lod, i, h, ih);
                  basis<BASIS>(r, node_type<BASIS>(i, ngd), ih, sv[kk], dsv[kk]);
                  dsv[kk] = sv[kk] != 0.f ? dsv[kk] : 0.f;  // as Axis::eval
                }
              }
            }
#pragma unroll
            for (int kk = 0; kk < S; kk++) {
              sbas[(d * S + kk) * SROW + lane] = make_float2(sv[kk], dsv[kk]);
              svs[d][kk] = sv[kk];
            }
          }
          if (REMAP) {
            // k_g2p1's gather from the footprint: stencil node (i, j) is
            // footprint node (warp L + lx + i, ly0 + ly + j); w = s_x s_y (the
            // unit z weight of the 2-D gather leaves it exact)
            float vu[3] = {0.f, 0.f, 0.f}, va[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int i = 0; i < S; i++) {
#pragma unroll
              for (int j = 0; j < S; j++) {
                const float w = svs[0][i] * svs[1][j];
                const int fi = (warp * L + lx + i) * WY + (ly0 + ly + j);
                const float4 A = fpA[fi];
                const float2 B = fpB[fi];
                vu[0] = fmaf(w, A.w, vu[0]); vu[1] = fmaf(w, B.x, vu[1]); vu[2] = fmaf(w, B.y, vu[2]);
                va[0] = fmaf(w, A.x, va[0]); va[1] = fmaf(w, A.y, va[1]); va[2] = fmaf(w, A.z, va[2]);
              }
            }
            const float m = P[PF_MASS * ps + p];
            float xn[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
              const float up = P[(PF_X + d) * ps + p];
              const float v = P[(PF_V + d) * ps + p];
              const float vnew = (1.f - alpha) * vu[d] + alpha * (v + (vu[d] - va[d]));
              const float un = up + dt * vu[d];
              if (REMAP == 1) {
                P[(PF_X + d) * ps + p] = un;
              } else {
                P[(PF_XN + d) * ps + p] = un;
                xn[d] = P[(PF_X0 + d) * ps + p] + un;
              }
              P[(PF_V + d) * ps + p] = vnew;
              pay[d] = m * vnew;
            }
            if (REMAP == 2 && !(xn[0] >= a.boxlo[0] && xn[0] <= a.boxhi[0] && xn[1] >= a.boxlo[1] &&
                                xn[1] <= a.boxhi[1] && xn[2] >= a.boxlo[2] && xn[2] <= a.boxhi[2]))
              raise_error(a.err, ERR_LEFT, p, nstep);
          }
#pragma unroll
          for (int v = 0; v < QINP / 4; v++)
            reinterpret_cast<float4 *>(spay + lane * QINP)[v] =
                make_float4(pay[4 * v], 4 * v + 1 < QIN ? pay[min(4 * v + 1, QIN - 1)] : 0.f,
                            4 * v + 2 < QIN ? pay[min(4 * v + 2, QIN - 1)] : 0.f,
                            4 * v + 3 < QIN ? pay[min(4 * v + 3, QIN - 1)] : 0.f);
        }
        __syncwarp();
        // ---- accumulate: group grp takes particles j = grp, grp + 4, ... of
        // each cell's share of this chunk (c0 - rs is a multiple of 32)
#pragma unroll
        for (int ly = 0; ly < 4; ly++) {
          const int jlo = max(st[ly] - c0, 0), jhi = min(en[ly] - c0, cnt);
          for (int j = jlo + ((grp - jlo - (c0 - rs)) & 3); j < jhi; j += 4) {
            float pay[QINP];
#pragma unroll
            for (int v = 0; v < QINP / 4; v++) {
              const float4 t4 = reinterpret_cast<const float4 *>(spay + j * QINP)[v];
              pay[4 * v] = t4.x; pay[4 * v + 1] = t4.y; pay[4 * v + 2] = t4.z; pay[4 * v + 3] = t4.w;
            }
            const float2 bx = px[j], b0 = py0[j], b2 = py2[j];
            // momentum (and UL mass): w = sx sy; force: -(T[r][0] dsx sy + T[r][1] sx dsy)
            if (!FO) {
              float q[3 + OM];
#pragma unroll
              for (int d = 0; d < 3 + OM; d++) q[d] = bx.x * pay[d];
#pragma unroll
              for (int d = 0; d < 3 + OM; d++) {
                if (d == OM + 2) continue;  // v_z = 0 in 2-D: the sum stays 0
                acc[ly][d] = fmaf(b0.x, q[d], acc[ly][d]);
                acc[ly + 2][d] = fmaf(b2.x, q[d], acc[ly + 2][d]);
              }
            }
            if (FORCE) {
              constexpr int F0 = FO ? 0 : 3 + OM;  // the force sums' first quantity
#pragma unroll
              for (int r = 0; r < 2; r++) {
                float T0, T1;
                if (FO) {  // vol0 PK1, row-major, alone in the payload
                  T0 = pay[3 * r]; T1 = pay[1 + 3 * r];
                } else if (MODE == P2G_TL) {  // vol0 PK1, row-major
                  T0 = pay[3 + 3 * r]; T1 = pay[4 + 3 * r];
                } else {  // vol sigma, symmetric xx yy zz xy xz yz
                  const float *sg = pay + 4;
                  T0 = r == 0 ? sg[0] : sg[3];
                  T1 = r == 0 ? sg[3] : sg[1];
                }
                const float tx = T0 * bx.y, ty = T1 * bx.x;
                acc[ly][F0 + r] = fmaf(-b0.x, tx, fmaf(-b0.y, ty, acc[ly][F0 + r]));
                acc[ly + 2][F0 + r] = fmaf(-b2.x, tx, fmaf(-b2.y, ty, acc[ly + 2][F0 + r]));
              }
            }
          }
        }
        __syncwarp();
      }
      // ---- flush: add the four groups (fixed butterfly), then lanes c = 1
      // hand their y = 1..5 sums to the c = 0 lanes (a fixed order)
#pragma unroll
      for (int m = 0; m < 6; m++)
#pragma unroll
        for (int qq = 0; qq < Q; qq++) {
          acc[m][qq] += __shfl_xor_sync(0xffffffffu, acc[m][qq], 8);
          acc[m][qq] += __shfl_xor_sync(0xffffffffu, acc[m][qq], 16);
        }
#pragma unroll
      for (int m = 0; m < 5; m++)
#pragma unroll
        for (int qq = 0; qq < Q; qq++) {
          const float o = __shfl_xor_sync(0xffffffffu, acc[m][qq], 1);
          if (sc == 0) acc[m + 1][qq] += o;
        }
      if (grp == 0) {
#pragma unroll
        for (int m = 0; m < 6; m++) {
          if (sc == 1 && m < 5) continue;
          const int fy = ly0 + m + sc;
          const int fi = (lx + sa) * WY + fy;
#pragma unroll
          for (int qq = 0; qq < Q; qq++) slab[qq * NF + fi] += acc[m][qq];
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
  // ---- sum the slabs in warp order into the tile footprint
  float *out = a.partial + (size_t)tile_global * a.pstride_tile;
  for (int k = threadIdx.x; k < Q * NW; k += blockDim.x) {
    const int qq = k / NW, fi = k % NW;
    const int fx = fi / WY, fy = fi % WY;
    float sum = 0.f;
#pragma unroll
    for (int w = 0; w < TS::NWARP; w++) {
      const int x = fx - w * L;
      if (x >= 0 && x < FX) sum += smem[w * SLAB + qq * NF + x * WY + fy];
    }
    out[k] = sum;
  }
}

// ============================================================== grid
// Sum of the tile partials covering one node, in a fixed tile order.
template <int DIM, int BASIS, int Q, typename ACC>
__device__ __forceinline__ void gather_partials(const GridArgs &a, const GridDev &g, int li, const int *ix, ACC *sum) {
  using TS = TileShape<DIM, BASIS>;
  constexpr int SC = Stencil<BASIS>::SC, LO = Stencil<BASIS>::LO;
  const int T[3] = {TS::TX, TS::TY, TS::TZ}, W[3] = {TS::WX, TS::WY, TS::WZ};
  int tlo[3], thi[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (d < DIM) {
      // tile t covers nodes [t*T*SC - LO, t*T*SC - LO + W - 1]
      const int TN = T[d] * SC;
      const int hi = (ix[d] + LO) / TN;
      const int lo_num = ix[d] + LO - W[d] + 1;
      const int lo = lo_num <= 0 ? 0 : (lo_num + TN - 1) / TN;
      tlo[d] = max(lo, 0);
      thi[d] = min(hi, g.ntile[d] - 1);
    } else {
      tlo[d] = thi[d] = 0;
    }
  }
#pragma unroll
  for (int q = 0; q < Q; q++) sum[q] = ACC(0);
  for (int tx = tlo[0]; tx <= thi[0]; tx++)
    for (int ty = tlo[1]; ty <= thi[1]; ty++)
      for (int tz = tlo[2]; tz <= thi[2]; tz++) {
        const int tl = DIM == 3 ? (tx * g.ntile[1] + ty) * g.ntile[2] + tz : (DIM == 2 ? tx * g.ntile[1] + ty : tx);
        const int tg = g.tile_off + tl;
        if (a.tile_end[tg] == a.tile_start[tg]) continue;
        const int fl[3] = {ix[0] - (tx * TS::TX * SC - LO), DIM >= 2 ? ix[1] - (ty * TS::TY * SC - LO) : 0,
                           DIM == 3 ? ix[2] - (tz * TS::TZ * SC - LO) : 0};
        const int fi = (fl[0] * TS::WY + fl[1]) * TS::WZ + fl[2];
        const float *src = a.partial + (size_t)tg * a.pstride_tile;
#pragma unroll
        for (int q = 0; q < Q; q++) sum[q] += (ACC)src[q * TS::NW + fi];
      }
  (void)li;
}

// GM_MASS: nodal mass only (TL once).  GM_UPDATE: after the first scatter.
// GM_VEL: after the MUSL re-map (or USL: positions only).  R is the
// arithmetic of the nodal sums and of v = p/m (double for the FP64 islands).
template <int DIM, int BASIS, int GMODE, bool TL, bool THERMAL, typename R>
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
  const R dt = (R)sc.dt;

  if (GMODE == GM_MASS) {
    R s[1];
    gather_partials<DIM, BASIS, 1, R>(a, g, li, ix, s);
    float4 A = a.nodeA[NODE_STRIDE * node];
    A.w = (float)s[0];
    a.nodeA[NODE_STRIDE * node] = A;
    return;
  }
  if (GMODE == GM_STORE_P) {
    // the momentum of a P2G_VEL scatter of the current state into nodeP, as
    // GM_VEL keeps the re-map's (TLMPM, mechanical)
    R s[3];
    gather_partials<DIM, BASIS, 3, R>(a, g, li, ix, s);
    a.nodeP[node] = make_float4((float)s[0], (float)s[1], (float)s[2], 0.f);
    return;
  }
  if (GMODE == GM_UPDATE || GMODE == GM_UPDATE_F) {
    // quantities: TL [p3 f3 (+mT Qext Qint)]; UL [m p3 f3 (+...)];
    // GM_UPDATE_F (TL, mechanical): [f3], p as the last re-map summed it
    constexpr bool FO = GMODE == GM_UPDATE_F;
    static_assert(!FO || (TL && !THERMAL), "the momentum reuse is TLMPM and mechanical");
    constexpr int Q = FO ? 3 : TL ? (THERMAL ? 9 : 6) : (THERMAL ? 10 : 7);
    R s[Q];
    gather_partials<DIM, BASIS, Q, R>(a, g, li, ix, s);
    const int o = TL ? 0 : 1;
    float4 A = a.nodeA[NODE_STRIDE * node];
    const R m = TL ? (R)A.w : s[0];
    R v[3], f[3], mb[3] = {0, 0, 0}, vu[3];
    R pm[3];
    if (FO) {
      const float4 Pn = a.nodeP[node];
      pm[0] = Pn.x; pm[1] = Pn.y; pm[2] = Pn.z;
    } else {
#pragma unroll
      for (int d = 0; d < 3; d++) pm[d] = s[o + d];
    }
    // Solid::compute_velocity_nodes: v = p/m only where m > 0 (src/solid.cpp:357)
    const R im = m > R(0) ? R(1) / m : R(0);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      v[d] = pm[d] * im;
      f[d] = s[(FO ? 0 : o + 3) + d];
    }
    // body force on nodes with mass (src/fix_body_force.cpp:122-136)
    for (int k = a.fix_start[gi]; k < a.fix_start[gi] + a.fix_count[gi]; k++) {
      const FixDev &fx = a.fixes[k];
      if (fx.kind != 1 || !fx.mask[li] || !(m > R(0))) continue;
      for (int d = 0; d < 3; d++)
        if (fx.set[d]) mb[d] += (R)fx.c[d][0] * m;
    }
    // Grid::update_grid_velocities (src/grid.cpp:448-466)
#pragma unroll
    for (int d = 0; d < 3; d++) vu[d] = m != R(0) ? v[d] + dt * (f[d] + mb[d]) * im : v[d];
    R T = 0, Tu = 0;
    if constexpr (THERMAL && !FO) {
      T = s[o + 6] * im;
      Tu = m != R(0) ? T + dt * (s[o + 8] + s[o + 7]) * im : T;  // src/grid.cpp:1354-1361
    }
    // FixVelocityNodes::post_update_grid_state (src/fix_velocity_nodes.cpp:130-225)
    for (int k = a.fix_start[gi]; k < a.fix_start[gi] + a.fix_count[gi]; k++) {
      const FixDev &fx = a.fixes[k];
      if (fx.kind != 0 || !fx.mask[li]) continue;
      for (int d = 0; d < 3; d++)
        if (fx.set[d]) { vu[d] = (R)fx.now[d]; v[d] = (R)fx.prev[d]; }
    }
    a.nodeA[NODE_STRIDE * node] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)m);
    a.nodeB[NODE_STRIDE * node] = make_float4((float)vu[0], (float)vu[1], (float)vu[2], (float)Tu);
    if (THERMAL) a.nodeT[node] = (float)T;
    return;
  }
  // GM_VEL: MUSL velocities_to_grid (+ BCs on v) and TL grid positions
  float4 A = a.nodeA[NODE_STRIDE * node];
  R v[3] = {A.x, A.y, A.z};
  if (a.remap) {
    constexpr int Q = THERMAL ? 4 : 3;
    R s[Q];
    gather_partials<DIM, BASIS, Q, R>(a, g, li, ix, s);
    // the momentum sums before the BCs, for the next grid update (P2G_FONLY)
    if (TL && !THERMAL && a.nodeP) a.nodeP[node] = make_float4((float)s[0], (float)s[1], (float)s[2], 0.f);
    const R m = A.w;
    const R im = m > R(0) ? R(1) / m : R(0);
#pragma unroll
    for (int d = 0; d < 3; d++) v[d] = s[d] * im;
    if (THERMAL) a.nodeT[node] = (float)(s[3] * im);
    // FixVelocityNodes::post_velocities_to_grid (src/fix_velocity_nodes.cpp:227-271)
    for (int k = a.fix_start[gi]; k < a.fix_start[gi] + a.fix_count[gi]; k++) {
      const FixDev &fx = a.fixes[k];
      if (fx.kind != 0 || !fx.mask[li]) continue;
      for (int d = 0; d < 3; d++)
        if (fx.set[d]) v[d] = (R)fx.now[d];
    }
    a.nodeA[NODE_STRIDE * node] = make_float4((float)v[0], (float)v[1], (float)v[2], A.w);
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

// ---- node staging of the gathers
// Every 256-particle block of a gather kernel copies the nodes of the
// bounding box of its particles' stencils from HBM into shared memory once
// (zeros where the box leaves the grid), and each particle then reads its
// stencil nodes there, at compile-time offsets from one base.  Particles are
// sorted by (tile, cell), so a block's box is small (a block of a full 3-D
// tile spans two cell layers: 5 x 7 x 7 nodes); a block whose box holds more
// than G2P_STAGE_NODES nodes (it spans tiles far apart in the tile order)
// gathers from global memory instead.  The 8 particles of one cell read the
// same shared-memory words (broadcast), where the same loads through L1 had
// been bound by its wavefront rate.
// Block-wide bounding box [lo, lo + nb) of the stencil origins i0 of the
// block's particles, widened by the stencil width S; false if the block has
// no particle or the box holds more than cap nodes.  Every thread of the
// block must call it (it synchronises the block).
template <int DIM, int S>
__device__ __forceinline__ bool stage_box(bool valid, const int (&i0)[3], int cap, int (&lo)[3], int (&nb)[3],
                                          int &vol) {
  __shared__ int red[8][6];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int v[6];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    v[d] = valid ? i0[d] : INT_MAX;
    v[3 + d] = valid ? -i0[d] : INT_MAX;  // min of -i0 = -max
  }
#pragma unroll
  for (int k = 0; k < 6; k++) v[k] = __reduce_min_sync(0xffffffffu, v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 6; k++) red[warp][k] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 6; k++) {
    int m = red[0][k];
#pragma unroll
    for (int w = 1; w < 8; w++) m = min(m, red[w][k]);
    v[k] = m;
  }
  if (v[0] == INT_MAX) return false;
  long long vv = 1;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    lo[d] = d < DIM ? v[d] : 0;
    nb[d] = d < DIM ? -v[3 + d] - v[d] + S : 1;
    vv *= nb[d];
  }
  vol = (int)min(vv, (long long)INT_MAX);
  return vv <= cap;
}

// Box element e -> grid node (local index), or -1 outside the grid.
__device__ __forceinline__ int stage_node(const GridDev &g, const int (&lo)[3], const int (&nb)[3], int e) {
  const int c = e % nb[2], b = (e / nb[2]) % nb[1], a = e / (nb[1] * nb[2]);
  const int ix = lo[0] + a, iy = lo[1] + b, iz = lo[2] + c;
  if (ix < 0 || ix >= g.n[0] || iy < 0 || iy >= g.n[1] || iz < 0 || iz >= g.n[2]) return -1;
  return (ix * g.n[1] + iy) * g.n[2] + iz;
}

// grid_to_points + advance_particles (src/solid.cpp:576-635, 786-790)
// MINB: resident blocks per SM the register budget is set for (launch shape
// picked per run by the autotuner, kmpm_api.cu).  Dynamic shared memory:
// G2P_STAGE_NODES * 32 bytes (the staged v, v_update pairs).
template <int DIM, int BASIS, bool TL, bool THERMAL, int MINB = 4>
__global__ void __launch_bounds__(256, MINB) k_g2p1(PartArgs a) {
  extern __shared__ __align__(16) float4 g2p_stage[];
  if (run_finished(a.scalars)) return;
  RangeDev rd;
  const int p = range_particle(a, rd);
  const bool valid = p >= 0;
  float *P = *a.Pp;
  const GridDev g = a.grids[rd.grid];
  const StepScalars &sc = a.scalars[a.indep ? a.blk_range[blockIdx.x] : 0];
  const float dt = (float)sc.dt;
  const size_t ps = a.ps;
  const int pl = valid ? p : rd.start;  // a thread without a particle evaluates a stand-in (never written)
  float xp[3], up[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    up[d] = P[(PF_X + d) * ps + pl];
    xp[d] = P[(PF_X0 + d) * ps + pl] + (TL ? 0.f : up[d]);
  }
  PAxes<DIM, BASIS> ax;
  ax.eval(g, xp);
  constexpr int S = Stencil<BASIS>::S;
  constexpr int SY = DIM >= 2 ? S : 1, SZ = DIM == 3 ? S : 1;
  const float4 *__restrict__ NA = a.nodeA + NODE_STRIDE * g.node_off;  // v, v_update interleaved
  const int i0[3] = {ax.ax[0].i0, ax.ax[1].i0, ax.ax[2].i0};
  int lo[3], nb[3], vol;
  const bool staged = stage_box<DIM, S>(valid, i0, G2P_STAGE_NODES, lo, nb, vol);
  // mechanical runs stage the six values of a node as a float4 (v, v_update.x)
  // and a float2 (v_update.y, v_update.z) in two arrays: two loads of 6
  // shared-memory wavefronts per warp and node, where two float4 take 8;
  // thermal runs stage (v, -) and (v_update, T)
  float2 *stage2 = reinterpret_cast<float2 *>(g2p_stage + G2P_STAGE_NODES);
  if (staged) {
    for (int e = threadIdx.x; e < vol; e += blockDim.x) {
      const int n = stage_node(g, lo, nb, e);
      float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A;
      if (n >= 0) ld_node_pair(NA + NODE_STRIDE * n, A, B);
      if (THERMAL) {
        g2p_stage[2 * e] = A;
        g2p_stage[2 * e + 1] = B;
      } else {
        g2p_stage[e] = make_float4(A.x, A.y, A.z, B.x);
        stage2[e] = make_float2(B.y, B.z);
      }
    }
    __syncthreads();
  }
  if (!valid) return;
  float vu[3] = {0, 0, 0}, va[3] = {0, 0, 0}, Tp = 0.f;
  if (staged) {
    // stencil node (i, j, k) is box element base + (i nb1 + j) nb2 + k
    const int base = ((i0[0] - lo[0]) * nb[1] + (i0[1] - lo[1])) * nb[2] + (i0[2] - lo[2]);
#pragma unroll
    for (int i = 0; i < S; i++) {
#pragma unroll
      for (int j = 0; j < SY; j++) {
        const float sxy = ax.ax[0].s[i] * ax.ax[1].s[j];
        const int r = base + (i * nb[1] + j) * nb[2];
#pragma unroll
        for (int k = 0; k < SZ; k++) {
          const float w = sxy * ax.ax[2].s[k];
          float4 A, B;
          if (THERMAL) {
            A = g2p_stage[2 * (r + k)];
            B = g2p_stage[2 * (r + k) + 1];
          } else {
            const float4 A4 = g2p_stage[r + k];
            const float2 B2 = stage2[r + k];
            A = A4;
            B = make_float4(A4.w, B2.x, B2.y, 0.f);
          }
          vu[0] = fmaf(w, B.x, vu[0]); vu[1] = fmaf(w, B.y, vu[1]); vu[2] = fmaf(w, B.z, vu[2]);
          va[0] = fmaf(w, A.x, va[0]); va[1] = fmaf(w, A.y, va[1]); va[2] = fmaf(w, A.z, va[2]);
          if (THERMAL) Tp = fmaf(w, B.w, Tp);
        }
      }
    }
  } else {
    // branch-free gather from global memory: per-axis node indices clamped
    // into the grid (a node outside it has a zero value, so its clamped
    // stand-in contributes nothing)
    int cx[S], cy[SY], cz[SZ];
#pragma unroll
    for (int k = 0; k < S; k++) cx[k] = min(max(i0[0] + k, 0), g.n[0] - 1);
#pragma unroll
    for (int k = 0; k < SY; k++) cy[k] = min(max(i0[1] + k, 0), g.n[1] - 1);
#pragma unroll
    for (int k = 0; k < SZ; k++) cz[k] = min(max(i0[2] + k, 0), g.n[2] - 1);
#pragma unroll
    for (int i = 0; i < S; i++) {
#pragma unroll
      for (int j = 0; j < SY; j++) {
        const float sxy = ax.ax[0].s[i] * ax.ax[1].s[j];
        const int row = (cx[i] * g.n[1] + cy[j]) * g.n[2];
#pragma unroll
        for (int k = 0; k < SZ; k++) {
          const float w = sxy * ax.ax[2].s[k];
          float4 A, B;
          ld_node_pair(NA + NODE_STRIDE * (row + cz[k]), A, B);
          vu[0] = fmaf(w, B.x, vu[0]); vu[1] = fmaf(w, B.y, vu[1]); vu[2] = fmaf(w, B.z, vu[2]);
          va[0] = fmaf(w, A.x, va[0]); va[1] = fmaf(w, A.y, va[1]); va[2] = fmaf(w, A.z, va[2]);
          if (THERMAL) Tp = fmaf(w, B.w, Tp);
        }
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
    const float v = P[(PF_V + d) * ps + p];
    // v = (1-alpha) v_update + alpha (v + dt a), with dt a = sum w (v_update - v)
    // = sum w v_update - sum w v
    const float dv = vu[d] - va[d];
    const float vnew = (1.f - alpha) * vu[d] + alpha * (v + dv);
    if (TL) P[(PF_X + d) * ps + p] = up[d] + dt * vu[d];
    else {
      // ASFLIP moves the particle with the blended velocity
      // (update_particle_velocities_and_positions, src/solid.cpp:791-796) and
      // checks the box on the position before the move (src/solid.cpp:676-686)
      const float un = up[d] + dt * (a.asflip ? vnew : vu[d]);
      P[(PF_XN + d) * ps + p] = un;
      xn[d] = P[(PF_X0 + d) * ps + p] + (a.asflip ? up[d] : un);
    }
    P[(PF_V + d) * ps + p] = vnew;
  }
  if (THERMAL) P[PF_T * ps + p] = Tp;
  if (!TL) {
    if (!(xn[0] >= a.boxlo[0] && xn[0] <= a.boxhi[0] && xn[1] >= a.boxlo[1] && xn[1] <= a.boxhi[1] &&
          xn[2] >= a.boxlo[2] && xn[2] <= a.boxhi[2]))
      raise_error(a.err, ERR_LEFT, p, sc.ntimestep);
  }
}

// MUSL grid_to_points + advance_particles + velocities_to_grid in one pass
// (src/musl.cpp:59-67; src/tlmpm.cpp:418-452, src/ulmpm.cpp:442-496): the
// gather of k_g2p1 and the re-map scatter of k_p2g_row<.., P2G_VEL> for the
// particles of one tile, whose weights both phases share.  3-D, cubic and
// quadratic splines, FLIP/PIC transfers, mechanical runs.
//   - the tile's node footprint of (v, v_update) is staged in shared memory
//     once (a float4 (v, v_update.x) and a float2 (v_update.y, v_update.z)
//     per node);
//   - each warp walks its rows of cells as k_p2g_row does; in the stage phase
//     a lane evaluates its particle's basis values, gathers the 64 nodes from
//     the staged footprint in k_g2p1's order, writes the particle's new
//     velocity and position, and stages m v_new for the re-map;
//   - accumulate and flush as k_p2g_row<.., P2G_VEL>.
// Every sum has the order of the two separate kernels, so the results are
// the same bit for bit (KMPM_SPLIT_MUSL=1 selects the separate kernels).
template <int BASIS, bool TL>
__global__ void __launch_bounds__(256, 4) k_g2p1_remap_row(P2GArgs a) {
  static_assert(Stencil<BASIS>::S == 4 && Stencil<BASIS>::SC == 1, "four-wide stencils");
  using TS = TileShape<3, BASIS>;
  constexpr int S = 4, LO = Stencil<BASIS>::LO;
  constexpr int TX = TS::TX, TY = TS::TY, TZ = TS::TZ;
  constexpr int WY = TS::WY, WZ = TS::WZ, NW = TS::NW, NF = TS::NF, FX = TS::FX;
  static_assert(TS::L == 1 && TZ == 4 && FX == 4, "one x-layer of 4 x 4 cells per warp");
  constexpr int Q = 3;                       // m v
  constexpr int SLAB = (Q * NF + 3) & ~3;
  constexpr int STAGE = VEL_STAGE;
  constexpr int NWP = (NW + 1) & ~1;

  extern __shared__ __align__(16) float smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *slab = smem + warp * SLAB;
  float *spay = smem + TS::NWARP * SLAB + warp * STAGE;  // [32][4]
  float *sbxy = spay + 32 * 4;                           // [axis x, y][slot][VROW]
  float4 *sbz = reinterpret_cast<float4 *>(sbxy + 2 * 4 * VROW);
  float4 *fpA = reinterpret_cast<float4 *>(smem + TS::NWARP * (SLAB + STAGE));
  float2 *fpB = reinterpret_cast<float2 *>(fpA + NWP);

  const int2 td = a.tiles[blockIdx.x];
  const GridDev g = a.grids[td.x];
  const int tlin = td.y;
  const int tile_global = g.tile_off + tlin;
  if (a.tile_end[tile_global] == a.tile_start[tile_global] || run_finished(a.scalars)) return;
  const int tc2 = tlin % g.ntile[2], tc1 = (tlin / g.ntile[2]) % g.ntile[1], tc0 = tlin / (g.ntile[1] * g.ntile[2]);
  const float h = g.cellsize, ih = g.inv_cellsize;
  float *P = *a.Pp;
  const size_t ps = a.ps;
  const StepScalars &sc = a.scalars[a.indep ? g.solid0 : 0];
  const float dt = (float)sc.dt;
  const float alpha = a.pic_flip;
  // the tile's x0, u, v and mass rows, into L2 while the footprint is staged
  prefetch_rows_l2(P, ps, PF_X0, PF_MASS + 1 - PF_X0, a.tile_start[tile_global], a.tile_end[tile_global]);
  // the particle ranges of the warp's TY x 4 cells, in one load (as
  // k_p2g_force_row), issued before the footprint's loads and barrier
  static_assert(TY * TZ == 16, "16 cells per warp");
  const int cw = tile_global * TS::NCELL + warp * TY * TZ;
  const int cvw = lane < 16 ? a.cell_start[cw + lane] : a.cell_end[cw + lane - 16];

  for (int k = lane; k < Q * NF; k += 32) slab[k] = 0.f;
  // the tile's node footprint: nodes (tc TX - LO + fx, ...), fx < WX
  {
    const float4 *__restrict__ NA = a.nodeA + NODE_STRIDE * g.node_off;
    const int b0 = tc0 * TX - LO, b1 = tc1 * TY - LO, b2 = tc2 * TZ - LO;
    for (int e = threadIdx.x; e < NW; e += blockDim.x) {
      const int fz = e % WZ, fy = (e / WZ) % WY, fx = e / (WY * WZ);
      const int ix = b0 + fx, iy = b1 + fy, iz = b2 + fz;
      float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A;
      if (ix >= 0 && ix < g.n[0] && iy >= 0 && iy < g.n[1] && iz >= 0 && iz < g.n[2])
        ld_node_pair(NA + NODE_STRIDE * ((ix * g.n[1] + iy) * g.n[2] + iz), A, B);
      fpA[e] = make_float4(A.x, A.y, A.z, B.x);
      fpB[e] = make_float2(B.y, B.z);
    }
  }
  __syncthreads();

  const int hw = lane >> 4, sa = (lane >> 2) & 3, sb = lane & 3;
  const float *px = sbxy + sa * VROW, *py = sbxy + (4 + sb) * VROW;
  const int i0x = (tc0 * TX + warp) - LO;

  for (int ly = 0; ly < TY; ly++) {
    int st[4], en[4], lo4[4];
    int rs = INT_MAX, re = INT_MIN;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      st[k] = __shfl_sync(0xffffffffu, cvw, ly * TZ + k);
      en[k] = __shfl_sync(0xffffffffu, cvw, 16 + ly * TZ + k);
      const bool full = en[k] > st[k];
      lo4[k] = full ? st[k] : INT_MAX;
      rs = full ? min(rs, st[k]) : rs;
      re = full ? max(re, en[k]) : re;
    }
    if (rs == INT_MAX) continue;
    const int i0y = (tc1 * TY + ly) - LO;
    float acc[7][Q];
#pragma unroll
    for (int m = 0; m < 7; m++)
#pragma unroll
      for (int qq = 0; qq < Q; qq++) acc[m][qq] = 0.f;

    for (int c0 = rs; c0 < re; c0 += 32) {
      const int cnt = min(32, re - c0);
      // ---- stage (lane = particle): weights, gather, particle update, payload
      if (lane < cnt) {
        const int p = c0 + lane;
        int lz = 0;
#pragma unroll
        for (int k = 1; k < 4; k++) lz = lo4[k] <= p ? k : lz;
        const int i0[3] = {i0x, i0y, (tc2 * TZ + lz) - LO};
        float sv[3][S], up[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          up[d] = P[(PF_X + d) * ps + p];
          const float xp = P[(PF_X0 + d) * ps + p] + (TL ? 0.f : up[d]);
          const float lod = d == 0 ? g.lo[0] : (d == 1 ? g.lo[1] : g.lo[2]);
          const int nd = d == 0 ? g.n[0] : (d == 1 ? g.n[1] : g.n[2]);
          const int ngd = d == 0 ? g.ng[0] : (d == 1 ? g.ng[1] : g.ng[2]);
          float dsv[S];
          if (BASIS == 1 && cubic_interior(i0[d], nd, ngd)) {
            cubic_weights(cells_of(xp, lod, ih) - (float)(i0[d] + 1), ih, sv[d], dsv);
          } else {
#pragma unroll
            for (int kk = 0; kk < S; kk++) {
              const int i = i0[d] + kk;
              sv[d][kk] = 0.f;
              dsv[kk] = 0.f;
              if (i >= 0 && i < nd) {
                const float r = node_offset_cells(xp, lod, i, h, ih);
                basis<BASIS>(r, node_type<BASIS>(i, ngd), ih, sv[d][kk], dsv[kk]);
              }
            }
          }
        }
        vel_row_stage_basis(sbxy, sbz, lane, sv);
        // the gather of k_g2p1 from the footprint: stencil node (i, j, k) is
        // footprint node (warp + i, ly + j, lz + k)
        // in packed pairs (v_x, v_y), (v_z, vu_x), (vu_y, vu_z): the footprint's
        // node layout, each component summed as w * value in node order
        float2 g01 = make_float2(0.f, 0.f), g2u0 = g01, u12 = g01;
        {
          float2 sz2[S];
#pragma unroll
          for (int k = 0; k < S; k++) sz2[k] = bc2(sv[2][k]);
#pragma unroll
          for (int i = 0; i < S; i++) {
            const float2 sx2 = bc2(sv[0][i]);
#pragma unroll
            for (int j = 0; j < S; j++) {
              const float2 sxy = fmul2(sx2, bc2(sv[1][j]));
              const int r = ((warp + i) * WY + (ly + j)) * WZ + lz;
#pragma unroll
              for (int k = 0; k < S; k++) {
                const float2 w = fmul2(sxy, sz2[k]);
                const float4 A = fpA[r + k];
                g01 = ffma2(w, make_float2(A.x, A.y), g01);
                g2u0 = ffma2(w, make_float2(A.z, A.w), g2u0);
                u12 = ffma2(w, fpB[r + k], u12);
              }
            }
          }
        }
        const float va[3] = {g01.x, g01.y, g2u0.x}, vu[3] = {g2u0.y, u12.x, u12.y};
        const float m = P[PF_MASS * ps + p];
        float xn[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const float v = P[(PF_V + d) * ps + p];
          const float vnew = (1.f - alpha) * vu[d] + alpha * (v + (vu[d] - va[d]));
          const float un = up[d] + dt * vu[d];
          if (TL) {
            P[(PF_X + d) * ps + p] = un;
          } else {
            P[(PF_XN + d) * ps + p] = un;
            xn[d] = P[(PF_X0 + d) * ps + p] + un;
          }
          P[(PF_V + d) * ps + p] = vnew;
          spay[lane * 4 + d] = m * vnew;
        }
        if (!TL && !(xn[0] >= a.boxlo[0] && xn[0] <= a.boxhi[0] && xn[1] >= a.boxlo[1] && xn[1] <= a.boxhi[1] &&
                     xn[2] >= a.boxlo[2] && xn[2] <= a.boxhi[2]))
          raise_error(a.err, ERR_LEFT, p, sc.ntimestep);
      }
      __syncwarp();
      // ---- accumulate (half-warp = particle, lane = (x, y) slot pair)
      vel_row_accumulate(acc, spay, px, py, sbz, st, en, c0, cnt, hw);
      __syncwarp();
    }
    vel_row_flush<WY, WZ, NF>(acc, slab, hw, sa, sb, ly);
    __syncwarp();
  }
  __syncthreads();
  // ---- sum the slabs in warp order into the tile footprint
  float *out = a.partial + (size_t)tile_global * a.pstride_tile;
  for (int k = threadIdx.x; k < Q * NW; k += blockDim.x) {
    const int qq = k / NW, fi = k % NW;
    const int fx = fi / (WY * WZ), fyz = fi % (WY * WZ);
    float sum = 0.f;
#pragma unroll
    for (int w = 0; w < TS::NWARP; w++) {
      const int x = fx - w;
      if (x >= 0 && x < FX) sum += smem[w * SLAB + qq * NF + x * WY * WZ + fyz];
    }
    out[k] = sum;
  }
}
// dynamic shared memory of k_g2p1_remap_row (bytes)
template <int BASIS> constexpr int g2p1_remap_smem() {
  using TS = TileShape<3, BASIS>;
  return 4 * (TS::NWARP * (((3 * TS::NF + 3) & ~3) + VEL_STAGE) + 6 * ((TS::NW + 1) & ~1));
}

// Node sources of the velocity-gradient gather: (v, T) of stencil node
// (i, j, k) from the staged box in shared memory or from global memory
// (clamped indices).
struct GradFetchStage {
  const float4 *st;
  int base, nb1, nb2;
  __device__ __forceinline__ int row(int i, int j, int) const { return base + (i * nb1 + j) * nb2; }
  __device__ __forceinline__ float4 at(int row, int k) const { return st[row + k]; }
};
template <int S, bool THERMAL> struct GradFetchGlobal {
  const float4 *NV;   // v (or v_update) of the grid's nodes, stride NODE_STRIDE
  const float *NT;    // nodal T of the grid (thermal, not use_vu)
  int cx[S], cy[S], cz[S], n1, n2;
  bool use_vu;
  __device__ __forceinline__ int row(int i, int j, int) const { return (cx[i] * n1 + cy[j]) * n2; }
  __device__ __forceinline__ float4 at(int row, int k) const {
    float4 V = __ldg(NV + NODE_STRIDE * (row + cz[k]));
    if (THERMAL && !use_vu) V.w = NT[row + cz[k]];
    return V;
  }
};

// Sum-factorised gradient gather over the z slots: for every (i, j),
// A = sum_k s_z V and B = sum_k ds_z V, then grad v += (ds_x s_y A,
// s_x ds_y A, s_x s_y B) (dropped pairs add 0: see Axis::eval).  Also the
// thermal gradient (qg -= grad T) and, in 2-D, sum w v_r.
template <int DIM, int BASIS, bool THERMAL, bool PACK, typename F>
__device__ __forceinline__ void grad_gather(const PAxes<DIM, BASIS> &ax, const F &f, float (&G)[9], float (&qg)[3],
                                            float &vr) {
  constexpr int S = Stencil<BASIS>::S;
  constexpr int SY = DIM >= 2 ? S : 1, SZ = DIM == 3 ? S : 1;
  // the z sums in packed pairs over the node's (v_x, v_y) and (v_z, T)
#pragma unroll
  for (int i = 0; i < S; i++) {
    const float sx = ax.ax[0].s[i], dsx = ax.ax[0].ds[i];
#pragma unroll
    for (int j = 0; j < SY; j++) {
      const float sy = ax.ax[1].s[j], dsy = ax.ax[1].ds[j];
      const int row = f.row(i, j, 0);
      float A[3] = {0.f, 0.f, 0.f}, B[3] = {0.f, 0.f, 0.f}, AT = 0.f, BT = 0.f;
      if (PACK) {
        float2 A01 = make_float2(0.f, 0.f), A2T = A01, B01 = A01, B2T = A01;
#pragma unroll
        for (int k = 0; k < SZ; k++) {
          const float4 V = f.at(row, k);
          const float2 xy = make_float2(V.x, V.y), zt = make_float2(V.z, V.w);
          const float2 sz = bc2(ax.ax[2].s[k]);
          A01 = ffma2(sz, xy, A01);
          A2T = ffma2(sz, zt, A2T);
          if (DIM == 3) {
            const float2 dsz = bc2(ax.ax[2].ds[k]);
            B01 = ffma2(dsz, xy, B01);
            B2T = ffma2(dsz, zt, B2T);
          }
        }
        A[0] = A01.x; A[1] = A01.y; A[2] = A2T.x; B[0] = B01.x; B[1] = B01.y; B[2] = B2T.x; AT = A2T.y; BT = B2T.y;
      } else {
#pragma unroll
        for (int k = 0; k < SZ; k++) {
          const float sz = ax.ax[2].s[k], dsz = ax.ax[2].ds[k];
          const float4 V = f.at(row, k);
          const float vn[3] = {V.x, V.y, V.z};
#pragma unroll
          for (int r = 0; r < DIM; r++) {
            A[r] += sz * vn[r];
            if (DIM == 3) B[r] += dsz * vn[r];
          }
          if (THERMAL) {
            AT += sz * V.w;
            if (DIM == 3) BT += dsz * V.w;
          }
        }
      }
      const float sxy = sx * sy, gx = dsx * sy, gy = sx * dsy;
#pragma unroll
      for (int r = 0; r < DIM; r++) {
        G[3 * r] += gx * A[r];
        if (DIM >= 2) G[3 * r + 1] += gy * A[r];
        if (DIM == 3) G[3 * r + 2] += sxy * B[r];
      }
      if (DIM == 2) vr += sxy * A[0];  // sum w v_r (axisymmetric hoop rate)
      if (THERMAL) {
        qg[0] -= gx * AT;
        qg[1] -= gy * AT;
        qg[2] -= sxy * BT;
      }
    }
  }
}

// 3-D TLMPM: the node box that k_g2p2 stages for each 256-particle block, from
// the block's x0 (static, so computed once at setup): the box of stage_box
// over the same particles, stored as int4 (lo, vol or -1 if the block gathers
// from global memory) and int4 (nb, 0).
template <int DIM, int BASIS>
__global__ void __launch_bounds__(256) k_gather_box(PartArgs a, int4 *box) {
  RangeDev rd;
  const int p0 = range_particle(a, rd);
  const bool valid = p0 >= 0;
  const int p = valid ? p0 : rd.start;
  const float *P = *a.Pp;
  const GridDev g = a.grids[rd.grid];
  float xp[3];
#pragma unroll
  for (int d = 0; d < 3; d++) xp[d] = P[(PF_X0 + d) * a.ps + p];
  PAxes<DIM, BASIS> ax;
  ax.eval(g, xp);
  const int i0[3] = {ax.ax[0].i0, ax.ax[1].i0, ax.ax[2].i0};
  int lo[3] = {0, 0, 0}, nb[3] = {1, 1, 1}, vol = 0;
  const bool staged = stage_box<DIM, Stencil<BASIS>::S>(valid, i0, G2P_STAGE_NODES, lo, nb, vol);
  if (threadIdx.x == 0) {
    box[2 * blockIdx.x] = make_int4(lo[0], lo[1], lo[2], staged ? vol : -1);
    box[2 * blockIdx.x + 1] = make_int4(nb[0], nb[1], nb[2], 0);
  }
}

// rate of deformation + deformation gradient + stress + wave speed
// (src/solid.cpp:798-936, 1155-1438)
// QUEUE: also append every plastic step (undamaged particle) to the learned
// return map's queue with what k_learn_queue needs to redo its update
template <int DIM, int BASIS, bool TL, bool THERMAL, int PREC, int MINB = 3, int LAW = LAW_ANY, bool QUEUE = false>
__global__ void __launch_bounds__(256, MINB) k_g2p2(PartArgs a) {
  __shared__ float red_c[8], red_h[8];
  __shared__ __align__(8) unsigned long long state_bar;
  // G2P_STAGE_NODES (v, T) of the staged box; then, for the linear EOS +
  // Johnson-Cook kernels, the state rows (G2P2_STATE_ROWS x 256 floats)
  extern __shared__ __align__(16) float4 g2p_stage[];
  if (run_finished(a.scalars)) return;
  RangeDev rd;
  const int p0 = range_particle(a, rd);
  const bool valid = p0 >= 0;
  const int p = valid ? p0 : rd.start;  // a thread without a particle evaluates a stand-in (never written)
  float my_c = 0.f, my_h = 1.f;
  float *P = *a.Pp;
  const size_t ps = a.ps;
  // Linear EOS + Johnson-Cook (FP32): the block's 256-slot slices of the
  // state rows v .. damage (PF_V .. PF_DMG: 23 rows, contiguous in the field
  // order, each slice 1 KB at a 1 KB boundary, as the field stride and the
  // blocks are multiples of 256 slots) come into shared memory by bulk copies
  // (cp.async.bulk) on one mbarrier.  One thread issues them before the node
  // staging and the gather, which then hide their latency; each thread waits
  // (bounded) before its first state read.  A wait that runs out raises
  // ERR_TIMEOUT (the step fails) and waits once more, bounded, so that the
  // block does not end with copies in flight.
  constexpr bool TMA_STATE = LAW == LAW_EOS_LINEAR_JC && PREC == 0 && !QUEUE;
  static_assert(PF_DMG + 1 - PF_V == G2P2_STATE_ROWS, "state rows");
  float *sstate = reinterpret_cast<float *>(g2p_stage + G2P_STAGE_NODES);  // [row - PF_V][256]
  const uint32_t sbar = smem_u32(&state_bar);
  bool waited = false;  // this thread saw the copies complete
  // (thread 0 initialises the mbarrier and issues the copies in program
  // order; the other threads first touch it after the barrier of the node
  // staging, stage_box, which orders them after the initialisation)
  if (TMA_STATE && threadIdx.x == 0) {
    mbar_init(sbar, 1);
    mbar_fence_init();
    const int blk0 = rd.start + (blockIdx.x - rd.blk0) * 256;
    mbar_expect_tx(sbar, G2P2_STATE_ROWS * 1024);
    for (int r = 0; r < G2P2_STATE_ROWS; r++)
      bulk_g2s(smem_u32(sstate + r * 256), P + (size_t)(PF_V + r) * ps + blk0, 1024, sbar);
  }
  // a state value of this thread's particle: from the staged rows or global memory
  const auto st_ld = [&](int row) -> float {
    if (TMA_STATE && row >= PF_V && row <= PF_DMG) return sstate[(row - PF_V) * 256 + threadIdx.x];
    return P[(size_t)row * ps + p];
  };
  // the kernels compiled for one set of laws serve FLIP/PIC runs only (APIC
  // runs take the general ones): no affine moments, no per-slot offsets kept
  const bool apic = LAW != LAW_ANY ? false : a.apic != 0;
  const GridDev g = a.grids[rd.grid];
  constexpr int S = Stencil<BASIS>::S;
  constexpr int SY = DIM >= 2 ? S : 1, SZ = DIM == 3 ? S : 1;
  const float4 *__restrict__ NV = (a.use_vu ? a.nodeB : a.nodeA) + NODE_STRIDE * g.node_off;
  const auto stage_nodes = [&](const int (&lo)[3], const int (&nb)[3], int vol) {
    for (int e = threadIdx.x; e < vol; e += blockDim.x) {
      const int n = stage_node(g, lo, nb, e);
      float4 V = make_float4(0.f, 0.f, 0.f, 0.f);
      if (n >= 0) {
        V = __ldg(NV + NODE_STRIDE * n);
        if (THERMAL && !a.use_vu) V.w = a.nodeT[g.node_off + n];
      }
      g2p_stage[e] = V;
    }
  };
  float xp[3];
  PAxes<DIM, BASIS> ax;
  int lo[3], nb[3], vol;
  bool staged;
  if (TL && DIM == 3 && a.gbox) {
    // the block's box from setup: the particle's x0 loads and the block's
    // node loads start at once, and the basis overlaps them (3-D: in 2-D the
    // box's own load costs more than the shorter chain it saves)
    const int4 b0 = a.gbox[2 * blockIdx.x], b1 = a.gbox[2 * blockIdx.x + 1];
    lo[0] = b0.x; lo[1] = b0.y; lo[2] = b0.z;
    nb[0] = b1.x; nb[1] = b1.y; nb[2] = b1.z;
    vol = b0.w;
    staged = vol >= 0;
#pragma unroll
    for (int d = 0; d < 3; d++) xp[d] = P[(PF_X0 + d) * ps + p];
    if (staged) stage_nodes(lo, nb, vol);
    ax.eval(g, xp);
    __syncthreads();  // block-uniform; also orders every thread after the mbarrier's initialisation
  } else {
#pragma unroll
    for (int d = 0; d < 3; d++) xp[d] = P[(PF_X0 + d) * ps + p] + (TL ? 0.f : P[(PF_X + d) * ps + p]);
    ax.eval(g, xp);
    const int i0[3] = {ax.ax[0].i0, ax.ax[1].i0, ax.ax[2].i0};
    staged = stage_box<DIM, S>(valid, i0, G2P_STAGE_NODES, lo, nb, vol);
    if (staged) {
      stage_nodes(lo, nb, vol);
      __syncthreads();
    }
  }
  const int i0[3] = {ax.ax[0].i0, ax.ax[1].i0, ax.ax[2].i0};
  if (valid) {
    const int mi = rd.mat >= 0 ? rd.mat : a.solid_mat[__float_as_int(P[PF_SID * ps + p])];
    const MatDev &m = a.mats[mi];
    const StepScalars &sc = a.scalars[a.indep ? a.blk_range[blockIdx.x] : 0];
    const float dt = (float)sc.dt;
    // the state rows the EOS + strength update reads after the node gather
    // (material type 2): start their DRAM reads now, into L2, so that they
    // overlap the gather (a hint: no registers held)
    if (!TMA_STATE && (LAW != LAW_ANY || (PREC == 0 && m.type == 2))) {
      const int rows[] = {PF_H, PF_H + 1, PF_H + 2, PF_H + 3, PF_H + 4, PF_H + 5, PF_H + 6, PF_H + 7, PF_H + 8,
                          PF_SIG, PF_SIG + 1, PF_SIG + 2, PF_SIG + 3, PF_SIG + 4, PF_SIG + 5,
                          PF_EPSP, PF_EPSDOT, PF_DMG, PF_VOL0, PF_V, PF_V + 1, PF_V + 2};
      // each address is formed inside the asm block: the compiler must not keep
      // these 22 addresses live across the gather for the later loads
      const unsigned long long base = (unsigned long long)(P + p), row_bytes = 4ull * ps;
#pragma unroll
      for (int r : rows)
        asm volatile("{ .reg .u64 ad; mad.lo.u64 ad, %1, %2, %0; prefetch.global.L2 [ad]; }" ::"l"(base),
                     "l"(row_bytes), "l"((unsigned long long)r));
    }
    if ((BASIS == 0 || BASIS == 1 || BASIS == 3) && apic) {
      // APIC (compute_rate_deformation_gradient_{TL,UL}_APIC,
      // src/solid.cpp:1006-1153): grad v = sum w v_node (x_node - x_p)^T Di with
      // Di = 3 / cellsize^2 (cubic) or 4 / cellsize^2 (quadratic)
      // (Solid::compute_inertia_tensor, src/solid.cpp:1440-1478).
      // The per-axis moment s (x_node - x_p) Di takes the place of the slope;
      // x_p is x0 (TL), and for ULMPM the position the reference holds at this
      // point: before the move (USL) or after it (MUSL)
      // x_node - x_p = h o_k + (x_w - x_p): o_k from the weights (Axis::eval)
      // and, for ULMPM MUSL, the move x_w - x_p = u - u_moved of this step
      // (linear TLMPM: 16/4 or 16/3 over cellsize^2 by particles per cell, src/solid.cpp:1448-1462)
      const float Di = BASIS == 0 ? g.apic_di : (BASIS == 3 ? 4.f : 3.f) * g.inv_cellsize * g.inv_cellsize;
#pragma unroll
      for (int d = 0; d < DIM; d++) {
        const float dw = (TL || a.use_vu) ? 0.f : P[(PF_X + d) * ps + p] - P[(PF_XN + d) * ps + p];
#pragma unroll
        for (int k = 0; k < S; k++)
          ax.ax[d].ds[k] = ax.ax[d].s[k] * fmaf(ax.ax[d].o[k], g.cellsize, dw) * Di;
      }
    }
    float G[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float qg[3] = {0, 0, 0};
    float vr = 0.f;
    // the staged box in shared memory, or global memory with clamped indices
    // (see k_g2p1); a pair with a zero weight is dropped as in the
    // reference, so its slope is masked too
    if (staged) {
      GradFetchStage f{g2p_stage, ((i0[0] - lo[0]) * nb[1] + (i0[1] - lo[1])) * nb[2] + (i0[2] - lo[2]), nb[1],
                       nb[2]};
      grad_gather<DIM, BASIS, THERMAL, true>(ax, f, G, qg, vr);
    } else {
      GradFetchGlobal<S, THERMAL> f;
      f.NV = NV;
      f.NT = a.nodeT + g.node_off;
      f.n1 = g.n[1];
      f.n2 = g.n[2];
      f.use_vu = a.use_vu != 0;
#pragma unroll
      for (int k = 0; k < S; k++) {
        f.cx[k] = min(max(i0[0] + k, 0), g.n[0] - 1);
        f.cy[k] = SY > 1 ? min(max(i0[1] + k, 0), g.n[1] - 1) : 0;
        f.cz[k] = SZ > 1 ? min(max(i0[2] + k, 0), g.n[2] - 1) : 0;
      }
      grad_gather<DIM, BASIS, THERMAL, false>(ax, f, G, qg, vr);
    }
    if (DIM == 2 && a.axisym) {
      // Fdot(2,2) / L(2,2) += sum w v_r / r, r = x0_r (TL) or the x_r of the
      // rate (src/solid.cpp:818-829, 900-913; APIC 1046-1058, 1120-1132, where
      // Di(2,2) = 1 in 2-D)
      const float r = P[PF_X0 * ps + p] + (TL ? 0.f : P[(a.use_vu ? PF_X : PF_XN) * ps + p]);
      G[8] += vr / r;
    }
    if ((BASIS == 0 || BASIS == 1 || BASIS == 3) && apic)
#pragma unroll
      for (int k = 0; k < 9; k++) P[(PF_C + k) * ps + p] = G[k];  // C of the next transfers
    if (TMA_STATE) {
      waited = mbar_wait(sbar, 0);
      if (!waited) {
        raise_error(a.err, ERR_TIMEOUT, p, sc.ntimestep);
        waited = mbar_wait(sbar, 0);
      }
    }
    // ---- deformation gradient (src/solid.cpp:1155-1244), stored as H = F - I
    float H[9];
#pragma unroll
    for (int k = 0; k < 9; k++) H[k] = st_ld(PF_H + k);
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
    float dmg = st_ld(PF_DMG);
    if (J <= 0.f && dmg < 1.f) raise_error(a.err, ERR_J, p, sc.ntimestep);
    const float vol0 = st_ld(PF_VOL0);
    const float rho = m.f_rho0 / J;
    float R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    Sym<float> D;
#pragma unroll
    for (int k = 0; k < 6; k++) D.a[k] = 0.f;
    const bool nh = LAW == LAW_ANY && m.type == 1;
    if (!nh) {
      if (TL) {
        if (!polar_rotation(F, R)) {
          if (dmg < 1.f) raise_error(a.err, ERR_POLDEC, p, sc.ntimestep);
        }
        // L = Fdot F^-1 = Fdot cof(F)^T / J ; D = R^T sym(L) R, symmetric:
        // its upper triangle (xx yy zz xy xz yz) from (R^T sym(L)) R
        float L[9], RtL[9];
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
        const int di[6] = {0, 1, 2, 0, 0, 1}, dj[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
        for (int k = 0; k < 6; k++)
          D.a[k] = RtL[3 * di[k]] * R[dj[k]] + RtL[3 * di[k] + 1] * R[3 + dj[k]] + RtL[3 * di[k] + 2] * R[6 + dj[k]];
      } else {
        D.a[0] = G[0]; D.a[1] = G[4]; D.a[2] = G[8];
        D.a[3] = 0.5f * (G[1] + G[3]); D.a[4] = 0.5f * (G[2] + G[6]); D.a[5] = 0.5f * (G[5] + G[7]);
      }
    }
    // ---- stress (src/solid.cpp:1246-1374)
    Sym<float> sig;
#pragma unroll
    for (int k = 0; k < 6; k++) sig.a[k] = st_ld(PF_SIG + k);
    float PK1[9];
    bool have_pk1 = false;
    if (LAW == LAW_ANY && m.type == 0) {  // LINEAR
      const float G2 = 2.f * m.f_G, lam = m.f_lambda;
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
      const float Gm = m.f_G, lam = m.f_lambda;
      const float lnJ = log1pf(Jm1);
      // F - F^-T = H + F^-T H^T (no cancellation when F is close to I)
      float FiTHt[9];
      matmulT3(FiT, H, FiTHt);
#pragma unroll
      for (int k = 0; k < 9; k++) PK1[k] = Gm * (H[k] + FiTHt[k]) + lam * lnJ * FiT[k];
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
      const bool hasT = LAW == LAW_ANY && m.f_cp != 0.f;
      float T = hasT ? a.T_ref + P[PF_T * ps + p] : 0.f;  // PF_T holds T - T_ref
      float epsp = st_ld(PF_EPSP), epsdot = st_ld(PF_EPSDOT);
      // Johnson-Cook damage: on for its law set, else as the material says
      const bool dmg_law = law_damage(LAW) == 1 || (LAW == LAW_ANY && m.damage >= 0);
      float dinit = dmg_law ? P[PF_DMGI * ps + p] : 0.f;
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
        pH = eos_pressure<float, LAW>(m, J, Jm1, rho, dmg, D.tr(), g.cellsize, T);
        if (hasT) pH += m.f_temp_p[3] * (m.f_temp_p[4] - T);
        bool returned = false;
        sdev = strength_update<float, LAW>(m, dt, sig, D, dep, epsp, epsdot, dmg, T, &returned);
        if constexpr (QUEUE) {
          const bool enq = returned && dmg == 0.f;
          const unsigned act = __activemask();
          const unsigned want = __ballot_sync(act, enq);
          if (want) {
            const int lane = threadIdx.x & 31, leader = __ffs(want) - 1;
            int base = 0;
            if (lane == leader) {
              base = atomicAdd(a.lq_count, __popc(want));
              atomicAdd(&a.lq_stats[0], (unsigned long long)__popc(want));
            }
            base = __shfl_sync(act, base, leader);
            if (enq) {
              const long long j = base + __popc(want & ((1u << lane) - 1u)), cap = a.lq_cap;
              float *q = a.lq_f;
              a.lq_i[LQ_P * cap + j] = p;
              a.lq_i[LQ_MAT * cap + j] = mi;
              q[LQ_DT * cap + j] = dt;
              q[LQ_TAV * cap + j] = 1000.f * g.cellsize / m.f_signal_velocity;
#pragma unroll
              for (int k = 0; k < 6; k++) {
                q[(LQ_D + k) * cap + j] = D.a[k];
                q[(LQ_SIG + k) * cap + j] = sig.a[k];
              }
              q[LQ_EPSP * cap + j] = epsp;
              q[LQ_EPSDOT * cap + j] = epsdot;
              q[LQ_PH * cap + j] = pH;
              float tre = 0.f;
              if (a.track_strain)
#pragma unroll
                for (int k = 0; k < 3; k++) tre += P[(PF_STRAIN + k) * ps + p];
              q[LQ_TRE * cap + j] = tre;
#pragma unroll
              for (int k = 0; k < 9; k++) {
                q[(LQ_R + k) * cap + j] = R[k];
                q[(LQ_COF + k) * cap + j] = cofF[k];
              }
            }
          }
        }
      }
      epsp += dep;
      // relaxation of the plastic strain rate over tav = 1000 cellsize / c (one division)
      const float itav = m.f_signal_velocity / (1000.f * g.cellsize);
      epsdot -= epsdot * dt * itav;
      epsdot += dep * itav;
      epsdot = fmaxf(0.f, epsdot);
      if (dmg_law) {
        float Tdm = a.thermal ? a.T_ref + P[PF_T * ps + p] : 0.f;
        damage_update<float>(m, dinit, dmg, pH, sdev, epsdot, dep, Tdm);
        P[PF_DMGI * ps + p] = dinit;
        P[PF_DMG * ps + p] = dmg;
      }
      if (hasT) {
        const float flow = (float)KMPM_SQRT_3_OVER_2 * sdev.norm();
        float gam = T < m.f_temp_p[5] ? m.f_temp_p[0] * flow * epsdot : 0.f;
        gam *= (TL ? vol0 : J * vol0) * m.f_invcp;
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
    }
#pragma unroll
    for (int k = 0; k < 6; k++) P[(PF_SIG + k) * ps + p] = sig.a[k];
    // ---- nodal-force operand for the next scatter
    if (TL) {
      if (!have_pk1) {
        // vol0 J (R sigma R^T) F^-T = vol0 (R sigma R^T) cof(F); R sigma R^T
        // is symmetric: its upper triangle, mirrored
        float Sm[9] = {sig.a[0], sig.a[3], sig.a[4], sig.a[3], sig.a[1], sig.a[5], sig.a[4], sig.a[5], sig.a[2]};
        float RS[9], RSR[9];
        matmul3(R, Sm, RS);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = i; j < 3; j++) {
            RSR[3 * i + j] = RS[3 * i] * R[3 * j] + RS[3 * i + 1] * R[3 * j + 1] + RS[3 * i + 2] * R[3 * j + 2];
            RSR[3 * j + i] = RSR[3 * i + j];
          }
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
      const float f = (TL ? vol0 : J * vol0) * (m.f_invcp * m.f_kappa);
#pragma unroll
      for (int c = 0; c < 3; c++) P[(PF_Q + c) * ps + p] = qg[c] * f;
    }
    // ---- wave speed and h ratio (src/solid.cpp:1376-1437)
    if (dmg < 1.f) {
      const float vx = st_ld(PF_V), vy = st_ld(PF_V + 1), vz = st_ld(PF_V + 2);
      const float c = sqrtf(m.f_c2_rho0 * J) + fmaxf(fmaxf(fabsf(vx), fabsf(vy)), fabsf(vz));  // c2 / rho = c2 J / rho0
      if (isnan(c)) raise_error(a.err, ERR_NAN, p, sc.ntimestep);
      my_c = c;
      if (TL) {
        // the cubic only where this particle may hold its range's minimum
        // (HRange): elsewhere the range's bound, which k_h_exact checks
        const float hb = a.hr ? a.hr[a.blk_range[blockIdx.x]].bound : 2.f;
        my_h = (hb > 1.f || re_eig_lower_bound(H) < hb) ? fminf(1.f, min_abs_eig_real(H)) : hb;
      }
    }
  }
  // block reduction (order-free min / max): within each warp by shuffles,
  // then over the eight warps
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    my_c = fmaxf(my_c, __shfl_xor_sync(0xffffffffu, my_c, o));
    my_h = fminf(my_h, __shfl_xor_sync(0xffffffffu, my_h, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red_c[threadIdx.x >> 5] = my_c;
    red_h[threadIdx.x >> 5] = my_h;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float c = red_c[0], hh = red_h[0];
#pragma unroll
    for (int w = 1; w < 8; w++) {
      c = fmaxf(c, red_c[w]);
      hh = fminf(hh, red_h[w]);
    }
    a.blk_c[blockIdx.x] = c;
    a.blk_h[blockIdx.x] = hh;
    // every thread with a particle has passed its wait (the barrier above);
    // unless thread 0 saw the copies complete (a block of an empty range has
    // no particle), it waits for them (bounded) before the block ends
    if (TMA_STATE) {
      if (!waited) mbar_wait(sbar, 0);
      mbar_inval(sbar);
    }
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
  k.gather_box = (void *)k_gather_box<DIM, BASIS>;
  k.p2g_row_fonly = k.grid_upd_fonly = k.grid_store_p = nullptr;
  k.p2g_row_fonly_smem = 0;
  if constexpr (DIM == 3 && (BASIS == 1 || BASIS == 3)) {
    k.p2g_row_fonly = (void *)k_p2g_force_row<BASIS>;
    k.p2g_row_fonly_smem = p2g_force_row_smem<BASIS>();
    k.grid_upd_fonly = (void *)k_grid<DIM, BASIS, GM_UPDATE_F, true, false, float>;
    k.grid_store_p = (void *)k_grid<DIM, BASIS, GM_STORE_P, true, false, float>;
    k.p2g_row[0] = (void *)k_p2g_row<BASIS, P2G_TL>;
    k.p2g_row[1] = (void *)k_p2g_row<BASIS, P2G_UL>;
    k.p2g_row[2] = (void *)k_p2g_vel_row<BASIS>;
    k.g2p1_remap[0] = (void *)k_g2p1_remap_row<BASIS, false>;
    k.g2p1_remap[1] = (void *)k_g2p1_remap_row<BASIS, true>;
    k.g2p1_remap_smem = g2p1_remap_smem<BASIS>();
  } else if constexpr (DIM == 2 && (BASIS == 1 || BASIS == 3)) {
    k.g2p1_remap[0] = (void *)k_p2g_row2<BASIS, P2G_VEL, 2>;
    k.g2p1_remap[1] = (void *)k_p2g_row2<BASIS, P2G_VEL, 1>;
    k.g2p1_remap_smem = p2g_row2_remap_smem<BASIS>();
    k.p2g_row_fonly = (void *)k_p2g_row2<BASIS, P2G_TL | P2G_FONLY>;
    k.p2g_row_fonly_smem = 0;  // p2g_smem_bytes of the mode
    k.grid_upd_fonly = (void *)k_grid<DIM, BASIS, GM_UPDATE_F, true, false, float>;
    k.grid_store_p = (void *)k_grid<DIM, BASIS, GM_STORE_P, true, false, float>;
    k.p2g_row[0] = (void *)k_p2g_row2<BASIS, P2G_TL>;
    k.p2g_row[1] = (void *)k_p2g_row2<BASIS, P2G_UL>;
    k.p2g_row[2] = (void *)k_p2g_row2<BASIS, P2G_VEL>;
  } else {
    k.p2g_row[0] = k.p2g_row[1] = k.p2g_row[2] = nullptr;
    k.g2p1_remap[0] = k.g2p1_remap[1] = nullptr;
    k.g2p1_remap_smem = 0;
  }
  // APIC runs with the cubic and quadratic splines, and for TLMPM with the
  // linear basis (src/solid.cpp:1447-1473)
  if constexpr (BASIS == 1 || BASIS == 3) {
    k.p2g_tl_apic = (void *)k_p2g<DIM, BASIS, P2G_TL_APIC, false>;
    k.p2g_ul_apic = (void *)k_p2g<DIM, BASIS, P2G_UL_APIC, false>;
    k.p2g_vel_apic = (void *)k_p2g<DIM, BASIS, P2G_VEL_APIC, false>;
  } else if constexpr (BASIS == 0) {
    k.p2g_tl_apic = (void *)k_p2g<DIM, BASIS, P2G_TL_APIC, false>;
    k.p2g_vel_apic = (void *)k_p2g<DIM, BASIS, P2G_VEL_APIC, false>;
    k.p2g_ul_apic = nullptr;
  } else {
    k.p2g_tl_apic = k.p2g_ul_apic = k.p2g_vel_apic = nullptr;
  }
#define KMPM_AXI(ul, ap, ex, mode)                                                             \
  k.p2g_axi[ul][ap][ex] = (void *)k_p2g<DIM, BASIS, (mode) | P2G_AXI | ((ex) ? P2G_EXT : 0), false>;
  for (int u = 0; u < 2; u++)
    for (int ap = 0; ap < 2; ap++)
      for (int ex = 0; ex < 2; ex++) k.p2g_axi[u][ap][ex] = nullptr;
  if constexpr (DIM == 2) {  // axisymmetric runs are 2-D
    KMPM_AXI(0, 0, 0, P2G_TL) KMPM_AXI(0, 0, 1, P2G_TL) KMPM_AXI(1, 0, 0, P2G_UL) KMPM_AXI(1, 0, 1, P2G_UL)
    if constexpr (BASIS == 0 || BASIS == 1 || BASIS == 3) {
      KMPM_AXI(0, 1, 0, P2G_TL_APIC) KMPM_AXI(0, 1, 1, P2G_TL_APIC)
    }
    if constexpr (BASIS == 1 || BASIS == 3) {
      KMPM_AXI(1, 1, 0, P2G_UL_APIC) KMPM_AXI(1, 1, 1, P2G_UL_APIC)
    }
  }
#undef KMPM_AXI
  if constexpr (DIM >= 2) {  // contact fixes act in 2-D and 3-D runs
    k.p2g_tl_ext[0] = (void *)k_p2g<DIM, BASIS, P2G_TL | P2G_EXT, false>;
    k.p2g_tl_ext[1] = (void *)k_p2g<DIM, BASIS, P2G_TL | P2G_EXT, true>;
    k.p2g_ul_ext[0] = (void *)k_p2g<DIM, BASIS, P2G_UL | P2G_EXT, false>;
    k.p2g_ul_ext[1] = (void *)k_p2g<DIM, BASIS, P2G_UL | P2G_EXT, true>;
    if constexpr (BASIS == 1 || BASIS == 3) {
      k.p2g_tl_apic_ext = (void *)k_p2g<DIM, BASIS, P2G_TL_APIC | P2G_EXT, false>;
      k.p2g_ul_apic_ext = (void *)k_p2g<DIM, BASIS, P2G_UL_APIC | P2G_EXT, false>;
    } else if constexpr (BASIS == 0) {
      k.p2g_tl_apic_ext = (void *)k_p2g<DIM, BASIS, P2G_TL_APIC | P2G_EXT, false>;
      k.p2g_ul_apic_ext = nullptr;
    } else {
      k.p2g_tl_apic_ext = k.p2g_ul_apic_ext = nullptr;
    }
  } else {
    k.p2g_tl_ext[0] = k.p2g_tl_ext[1] = k.p2g_ul_ext[0] = k.p2g_ul_ext[1] = nullptr;
    k.p2g_tl_apic_ext = k.p2g_ul_apic_ext = nullptr;
  }
  k.grid_mass[0] = (void *)k_grid<DIM, BASIS, GM_MASS, true, false, float>;
  k.grid_mass[1] = (void *)k_grid<DIM, BASIS, GM_MASS, true, false, double>;
#define KMPM_GRID_SET(tl, th)                                                                  \
  k.grid_upd[tl][th][0] = (void *)k_grid<DIM, BASIS, GM_UPDATE, tl, th, float>;                \
  k.grid_upd[tl][th][1] = (void *)k_grid<DIM, BASIS, GM_UPDATE, tl, th, double>;               \
  k.grid_vel[tl][th][0] = (void *)k_grid<DIM, BASIS, GM_VEL, tl, th, float>;                   \
  k.grid_vel[tl][th][1] = (void *)k_grid<DIM, BASIS, GM_VEL, tl, th, double>;
  KMPM_GRID_SET(false, false)
  KMPM_GRID_SET(false, true)
  KMPM_GRID_SET(true, false)
  KMPM_GRID_SET(true, true)
#undef KMPM_GRID_SET
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
  // launch-shape candidates of the FP32 mechanical path (variant 0 = default)
#define KMPM_VAR_SET(tl)                                                                       \
  k.g2p1_v[tl][0] = (void *)k_g2p1<DIM, BASIS, tl, false, G2P1_MINB[0]>;                      \
  k.g2p1_v[tl][1] = (void *)k_g2p1<DIM, BASIS, tl, false, G2P1_MINB[1]>;                      \
  k.g2p1_v[tl][2] = (void *)k_g2p1<DIM, BASIS, tl, false, G2P1_MINB[2]>;                      \
  k.g2p2_v[tl][0] = (void *)k_g2p2<DIM, BASIS, tl, false, 0, G2P2_MINB[0]>;                   \
  k.g2p2_v[tl][1] = (void *)k_g2p2<DIM, BASIS, tl, false, 0, G2P2_MINB[1]>;                   \
  k.g2p2_v[tl][2] = (void *)k_g2p2<DIM, BASIS, tl, false, 0, G2P2_MINB[2]>;
  KMPM_VAR_SET(false)
  KMPM_VAR_SET(true)
#undef KMPM_VAR_SET
  for (int t = 0; t < 2; t++)
    for (int v = 0; v < G2P_NVAR; v++) k.g2p2_jc[t][v] = nullptr;
  if constexpr (DIM == 3) {  // the benchmark's material: linear EOS + Johnson-Cook
#define KMPM_JC_SET(tl)                                                                               \
  k.g2p2_jc[tl][0] = (void *)k_g2p2<DIM, BASIS, tl, false, 0, G2P2_MINB[0], LAW_EOS_LINEAR_JC>;        \
  k.g2p2_jc[tl][1] = (void *)k_g2p2<DIM, BASIS, tl, false, 0, G2P2_MINB[1], LAW_EOS_LINEAR_JC>;        \
  k.g2p2_jc[tl][2] = (void *)k_g2p2<DIM, BASIS, tl, false, 0, G2P2_MINB[2], LAW_EOS_LINEAR_JC>;
    KMPM_JC_SET(false)
    KMPM_JC_SET(true)
#undef KMPM_JC_SET
  }
  for (int v = 0; v < G2P_NVAR; v++) k.g2p2_jcq[v] = nullptr;
  for (int t = 0; t < 2; t++)
    for (int v = 0; v < G2P_NVAR; v++) k.g2p2_jcd[t][v] = k.g2p2_fl[t][v] = nullptr;
  if constexpr (DIM == 2 && BASIS == 1) {  // batches of damage bars
    k.g2p2_jcd[1][0] = (void *)k_g2p2<DIM, BASIS, true, false, 0, G2P2_MINB[0], LAW_EOS_SHOCK_JC_DMG>;
    k.g2p2_jcd[1][1] = (void *)k_g2p2<DIM, BASIS, true, false, 0, G2P2_MINB[1], LAW_EOS_SHOCK_JC_DMG>;
    k.g2p2_jcd[1][2] = (void *)k_g2p2<DIM, BASIS, true, false, 0, G2P2_MINB[2], LAW_EOS_SHOCK_JC_DMG>;
  }
  if constexpr (DIM == 3 && BASIS == 1) {  // fluids (ULMPM)
    k.g2p2_fl[0][0] = (void *)k_g2p2<DIM, BASIS, false, false, 0, G2P2_MINB[0], LAW_FLUID>;
    k.g2p2_fl[0][1] = (void *)k_g2p2<DIM, BASIS, false, false, 0, G2P2_MINB[1], LAW_FLUID>;
    k.g2p2_fl[0][2] = (void *)k_g2p2<DIM, BASIS, false, false, 0, G2P2_MINB[2], LAW_FLUID>;
  }
  if constexpr (DIM == 3 && BASIS == 1) {  // the learned return map's path
    k.g2p2_jcq[0] = (void *)k_g2p2<DIM, BASIS, true, false, 0, G2P2_MINB[0], LAW_EOS_LINEAR_JC, true>;
    k.g2p2_jcq[1] = (void *)k_g2p2<DIM, BASIS, true, false, 0, G2P2_MINB[1], LAW_EOS_LINEAR_JC, true>;
    k.g2p2_jcq[2] = (void *)k_g2p2<DIM, BASIS, true, false, 0, G2P2_MINB[2], LAW_EOS_LINEAR_JC, true>;
  }
}

}  // namespace kmpm
