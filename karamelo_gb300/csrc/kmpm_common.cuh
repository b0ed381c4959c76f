// kmpm_common.cuh -- data layout and device helpers shared by the kernels.
//
// Layout in HBM (one context):
//   particles: one FP32 structure of arrays, field f of particle p at
//              P[f * pstride + p]; each solid's particles are contiguous,
//              sorted by (tile, cell) of their reference (TL) or current (UL)
//              position, and padded to a multiple of 256 so that every
//              256-thread block of a particle kernel belongs to one solid;
//   nodes:     float4 A = (v, mass) and float4 B = (v_update, T_update) per
//              node, interleaved (A B A B ..., 32 bytes per node), grids
//              concatenated and padded to multiples of 256;
//   tiles:     a grid's cells are grouped in tiles of T^dim cells; the
//              scatter kernel writes each tile's footprint (the nodes its
//              particles touch) to its own slice of a partial buffer, and the
//              grid kernel adds the (at most 2^dim) slices covering a node in a
//              fixed order, so P2G is bit-reproducible without float atomics.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace kmpm {

// ------------------------------------------------------------------ fields
enum PField : int {
  PF_X0 = 0,        // 3
  PF_X = 3,         // 3: displacement x - x0 (weights of ULMPM use x0 + PF_X)
  PF_V = 6,         // 3
  PF_MASS = 9,
  PF_VOL0 = 10,
  PF_H = 11,        // 9: F - I (row-major)
  PF_SIG = 20,      // 6: xx yy zz xy xz yz
  PF_EPSP = 26,
  PF_EPSDOT = 27,
  PF_DMG = 28,
  PF_DMGI = 29,
  PF_T = 30,
  PF_GAMMA = 31,
  PF_Q = 32,        // 3
  PF_PK = 35,       // 9: TL vol0*PK1 (row-major) ; UL vol*sigma (first 6, sym order)
  PF_STRAIN = 44,   // 6: strain_el (sym order)
  PF_XN = 50,       // 3: ULMPM displacement after this step's move (weights use PF_X)
  PF_ORIG = 53,     // caller index (int bits)
  PF_SID = 54,      // solid id (int bits), ULMPM only
  PF_C = 55,        // APIC affine matrix (9, row-major): Fdot (TL) or L (UL) of the last stress update
  PF_COUNT = 64
};

// symmetric storage order: xx yy zz xy xz yz
__host__ __device__ inline int sym_index(int i, int j) {
  if (i == j) return i;
  int a = i < j ? i : j, b = i < j ? j : i;
  return a == 0 ? (b == 1 ? 3 : 4) : 5;
}

// ------------------------------------------------------------------ tables
struct GridDev {
  int n[3];          // local node counts (Grid::nx, ny, nz)
  int ng[3];         // global node counts (ntype of the boundary-modified cubic)
  int ncell[3];      // cells per dim
  int ntile[3];      // tiles per dim
  int node_off;      // first node in the global node arrays
  int tile_off;      // first tile in the global tile arrays
  int cell_off;      // first cell in the global cell arrays
  int solid0;        // first solid using this grid (for per-solid scalars)
  float lo[3];       // lower bound of the lattice
  float inv_cellsize;
  float cellsize;
  float apic_di;     // linear-basis APIC: Di of the grid's solid (16/4 or 16/3 over cellsize^2)
};

// A contiguous particle range that shares one grid: one per solid for TLMPM,
// one for all solids for ULMPM (whose particles are binned together).
struct RangeDev {
  int start, count;  // particle range in the global arrays
  int grid;
  int mat;           // material id, or -1: per particle through PF_SID
  int blk0, nblk;    // 256-particle blocks of this range
};

// Material in device form (Mat, src/material.h:45-68, and its laws)
struct MatDev {
  int type, eos, strength, damage, temp;
  double rho0, K, G, lambda, signal_velocity, cp, invcp, kappa;
  double eos_p[12], str_p[12], dam_p[8], temp_p[6];
  // FP32 copies for the FP32 path (no per-particle double conversions)
  float f_rho0, f_K, f_G, f_lambda, f_signal_velocity, f_cp, f_invcp, f_kappa, f_c2;  // f_c2 = K + 4G/3
  float f_eos_p[12], f_str_p[12], f_dam_p[8], f_temp_p[6];
  float f_c2_rho0;  // f_c2 / rho0: the squared wave speed is f_c2_rho0 J
};
template <typename R> struct MatP;
template <> struct MatP<float> {
  __device__ static const float *eos(const MatDev &m) { return m.f_eos_p; }
  __device__ static const float *str(const MatDev &m) { return m.f_str_p; }
  __device__ static const float *dam(const MatDev &m) { return m.f_dam_p; }
};
template <> struct MatP<double> {
  __device__ static const double *eos(const MatDev &m) { return m.eos_p; }
  __device__ static const double *str(const MatDev &m) { return m.str_p; }
  __device__ static const double *dam(const MatDev &m) { return m.dam_p; }
};

// Node vectors: v (A) and v_update (B) of node i interleaved at float4 2i and
// 2i + 1, 32 bytes per node, so that one 256-bit load reads both.
constexpr int NODE_STRIDE = 2;
__device__ __forceinline__ void ld_node_pair(const float4 *p, float4 &A, float4 &B) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(A.x), "=f"(A.y), "=f"(A.z), "=f"(A.w), "=f"(B.x), "=f"(B.y), "=f"(B.z), "=f"(B.w)
      : "l"(p));
}

// Per-solid time-step scalars kept on the device so a captured step replays.
struct StepScalars {
  double dt, time;
  long long ntimestep;
  double dtCFL;
  double maxtime;  // RunTime: a step runs only while time < maxtime (+inf for run(n))
};

// Every kernel of a step returns at once when the run has reached its end
// time, so a batch of captured steps never overshoots run_time's bound.
__device__ __forceinline__ bool run_finished(const StepScalars *s) { return !(s->time < s->maxtime); }

// A node fix (velocity_nodes / body_force) in device form.
struct FixDev {
  int kind, grid, set[3];
  double c[3][4];
  const uint8_t *mask;  // node mask of that grid (local node index)
  // velocity fixes: c0 + c1 t + c2 exp(c3 t) at this step's time and at the
  // time one dt earlier, evaluated once per step (k_fix_values) rather than
  // per masked node (an FP64 exp)
  double now[3], prev[3];
};

enum ErrCode : int {
  ERR_NONE = 0,
  ERR_J = 10,
  ERR_LEFT = 11,
  ERR_NAN = 12,
  ERR_POLDEC = 13,
  ERR_DTCFL = 14,
  ERR_TIMEOUT = 15,
};
struct ErrState {
  int code;
  int particle;
  long long step;
};

// ------------------------------------------------------------------ stencils
// Node stencil of a particle whose base cell index is c along one axis:
// nodes c*SC - LO + s for s in [0, S).  Linear (src/tlmpm.cpp:141-175): c,c+1.
// Cubic (src/tlmpm.cpp:209-245): c-1..c+2.  Bernstein (src/tlmpm.cpp:176-208):
// fine nodes 2c..2c+2 of the h/2 lattice.  Cells of the same colour
// (index mod C in every axis) have disjoint stencils.
template <int BASIS> struct Stencil;
template <> struct Stencil<0> { static constexpr int S = 2, LO = 0, SC = 1, C = 2; };
template <> struct Stencil<1> { static constexpr int S = 4, LO = 1, SC = 1, C = 4; };
template <> struct Stencil<2> { static constexpr int S = 3, LO = 0, SC = 2, C = 2; };
// quadratic B-spline: the cubic stencil (src/ulmpm.cpp:204-207, src/tlmpm.cpp:209-245)
template <> struct Stencil<3> { static constexpr int S = 4, LO = 1, SC = 1, C = 4; };

// Tiles of TX x TY x TZ cells.  The scatter kernel gives every warp of the
// tile an x-slab of L = TX / NWARP cell layers; the warp accumulates its slab
// into a private footprint (FX x WY x WZ nodes) in shared memory, cell after
// cell in a fixed order, and the slabs are then summed in warp order.
template <int DIM, int BASIS> struct TileShape {
  static constexpr int S = Stencil<BASIS>::S, SC = Stencil<BASIS>::SC;
  static constexpr int NWARP = 8;
  static constexpr int TX = DIM == 3 ? 8 : (DIM == 2 ? 16 : 64);
  static constexpr int TY = DIM == 3 ? 4 : (DIM == 2 ? 16 : 1);
  static constexpr int TZ = DIM == 3 ? 4 : 1;
  static constexpr int L = TX / NWARP;
  static constexpr int WX = (TX - 1) * SC + S;
  static constexpr int WY = DIM >= 2 ? (TY - 1) * SC + S : 1;
  static constexpr int WZ = DIM == 3 ? (TZ - 1) * SC + S : 1;
  static constexpr int FX = (L - 1) * SC + S;
  static constexpr int NW = WX * WY * WZ;   // tile footprint nodes
  static constexpr int NF = FX * WY * WZ;   // slab footprint nodes
  static constexpr int NS = DIM == 3 ? S * S * S : (DIM == 2 ? S * S : S);
  static constexpr int NCELL = TX * TY * TZ;
  static constexpr int CPW = L * TY * TZ;   // cells per warp
};

__host__ __device__ inline void tile_dims(int dim, int basis, int *t) {
  (void)basis;
  t[0] = dim == 3 ? 8 : (dim == 2 ? 16 : 64);
  t[1] = dim == 3 ? 4 : (dim == 2 ? 16 : 1);
  t[2] = dim == 3 ? 4 : 1;
}
__host__ __device__ inline int stencil_width(int basis) { return basis == 0 ? 2 : (basis == 2 ? 3 : 4); }
__host__ __device__ inline int stencil_lo(int basis) { return (basis == 1 || basis == 3) ? 1 : 0; }
__host__ __device__ inline int stencil_sc(int basis) { return basis == 2 ? 2 : 1; }

// ntype of a node along one axis (Grid::init, src/grid.cpp:228-240)
template <int BASIS> __device__ __forceinline__ int node_type(int i, int ng) {
  if (BASIS == 1 || BASIS == 3) return min(2, i) - min(ng - 1 - i, 2);
  if (BASIS == 2) return i & 1;
  return 0;
}

// ------------------------------------------------------------------ basis
// BasisFunction::*, src/basis_functions.h:21-138, in FP32.  Value and
// derivative (already multiplied by 1/cellsize).
template <int BASIS> __device__ __forceinline__ void basis(float r, int nt, float ih, float &s, float &ds);

template <> __device__ __forceinline__ void basis<0>(float r, int, float ih, float &s, float &ds) {
  float a = fabsf(r);
  s = a >= 1.f ? 0.f : 1.f - a;
  ds = (r >= 1.f || r <= -1.f || r == 0.f) ? 0.f : (r > 0.f ? -ih : ih);
}

template <> __device__ __forceinline__ void basis<1>(float r, int nt, float ih, float &s, float &ds) {
  if (r >= 1.f && r < 2.f) {
    if (nt == 1) { s = 0.f; ds = -ih; }
    else { s = ((-1.f / 6.f * r + 1.f) * r - 2.f) * r + 4.f / 3.f; ds = ih * ((-0.5f * r + 2.f) * r - 2.f); }
  } else if (r >= 0.f && r < 1.f) {
    if (nt == -2) { s = (1.f / 6.f * r * r - 1.f) * r + 1.f; ds = ih * (0.5f * r * r - 1.f); }
    else if (nt == 2) { s = 1.f; ds = ih; }
    else if (nt == 1) { s = (1.f / 3.f * r - 1.f) * r * r + 2.f / 3.f; ds = ih * r * (r - 2.f); }
    else { s = (0.5f * r - 1.f) * r * r + 2.f / 3.f; ds = ih * (1.5f * r - 2.f) * r; }
  } else if (r >= -1.f && r < 0.f) {
    if (nt == 2) { s = (-1.f / 6.f * r * r + 1.f) * r + 1.f; ds = ih * (-0.5f * r * r + 1.f); }
    else if (nt == -1) { s = (-1.f / 3.f * r - 1.f) * r * r + 2.f / 3.f; ds = ih * (-r - 2.f) * r; }
    else { s = (-0.5f * r - 1.f) * r * r + 2.f / 3.f; ds = ih * (-1.5f * r - 2.f) * r; }
  } else if (r >= -2.f && r < -1.f) {
    s = ((1.f / 6.f * r + 1.f) * r + 2.f) * r + 4.f / 3.f;
    ds = ih * ((0.5f * r + 2.f) * r + 2.f);
  } else {
    s = 0.f; ds = 0.f;
  }
}

template <> __device__ __forceinline__ void basis<2>(float r, int nt, float ih, float &s, float &ds) {
  float a = fabsf(r);
  if (a >= 1.f) { s = 0.f; ds = 0.f; return; }
  if (nt == 1) {
    s = a >= 0.5f ? 0.f : 0.5f - 2.f * r * r;
    ds = a > 0.5f ? 0.f : -4.f * r * ih;
  } else {
    s = (1.f - a) * (1.f - a);
    ds = r > 0.f ? -2.f * (1.f - r) * ih : 2.f * (1.f + r) * ih;
  }
}

// BasisFunction::quadratic_spline and its derivative, src/basis_functions.h:140-241
template <> __device__ __forceinline__ void basis<3>(float r, int nt, float ih, float &s, float &ds) {
  s = 0.f;
  ds = 0.f;
  if (nt == 0) {
    if (r >= 0.5f && r < 1.5f) { s = (0.5f * r - 1.5f) * r + 1.125f; ds = ih * (r - 1.5f); }
    else if (r >= -0.5f && r < 0.5f) { s = -r * r + 0.75f; ds = -2.f * ih * r; }
    else if (r >= -1.5f && r < 0.5f) { s = (0.5f * r + 1.5f) * r + 1.125f; ds = ih * (r + 1.5f); }
  } else if (nt == -2) {
    if (r >= 0.f && r < 0.5f) { s = 1.f - r; ds = -ih; }
    else if (r >= 0.5f && r < 1.5f) { s = (0.5f * r - 1.5f) * r + 1.125f; ds = ih * (r - 1.5f); }
  } else if (nt == -1) {
    if (r >= -1.f && r < -0.5f) { s = 1.f + r; ds = ih; }
    else if (r >= -0.5f && r < 0.5f) { s = -r * r + 0.75f; ds = -2.f * ih * r; }
    else if (r >= 0.5f && r < 1.5f) { s = (0.5f * r - 1.5f) * r + 1.125f; ds = ih * (r - 1.5f); }
  } else if (nt == 1) {
    if (r >= -1.5f && r < -0.5f) { s = (0.5f * r + 1.5f) * r + 1.125f; ds = ih * (r + 1.5f); }
    else if (r >= -0.5f && r < 0.5f) { s = -r * r + 0.75f; ds = -2.f * ih * r; }
    else if (r >= 0.5f && r < 1.f) { s = 1.f - r; ds = -ih; }
  } else {
    if (r >= -1.5f && r < -0.5f) { s = (0.5f * r + 1.5f) * r + 1.125f; ds = ih * (r + 1.5f); }
    else if (r >= -0.5f && r <= 0.f) { s = 1.f + r; ds = ih; }
  }
}

// Packed FP32 pairs (sm_100 and later): one instruction issues two IEEE
// single-precision operations, each rounded exactly as the scalar fmaf / fmul
// would round it, so a loop written with them gives the same bits as its
// scalar form while taking half the issue slots.  bc2(x) is the pair (x, x).
__device__ __forceinline__ float2 bc2(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) { return __fmul2_rn(a, b); }

// A particle's coordinate in cells, (x - lo) / h, and its offset from node i
// in cells, (x - (lo + i h)) / h, each rounded once: the multiplications are
// kept out of fused multiply-adds, so that every kernel that evaluates a
// particle's basis (the scatters, the gathers and the fused MUSL pass) gets
// the same weights bit for bit, whatever the compiler contracts around them.
__device__ __forceinline__ float cells_of(float x, float lo, float ih) { return __fmul_rn(x - lo, ih); }
__device__ __forceinline__ float node_offset_cells(float x, float lo, int i, float h, float ih) {
  return __fmul_rn(x - __fadd_rn(lo, __fmul_rn((float)i, h)), ih);
}

// Cubic B-spline values and slopes of the four nodes c-1..c+2 of a particle at
// fractional position f in cell c, when all four have ntype 0: the same
// polynomials as src/basis_functions.h:40-104 evaluated without branches.
__device__ __forceinline__ bool cubic_interior(int i0, int n, int ng) { return i0 >= 2 && i0 + 3 <= min(n - 1, ng - 3); }
__device__ __forceinline__ void cubic_weights(float f, float ih, float *s, float *ds) {
  const float g = 1.f - f, f2 = f * f, g2 = g * g;
  s[0] = g2 * g * (1.f / 6.f);
  s[1] = (0.5f * f - 1.f) * f2 + 2.f / 3.f;
  s[2] = (0.5f * g - 1.f) * g2 + 2.f / 3.f;
  s[3] = f2 * f * (1.f / 6.f);
  ds[0] = -0.5f * g2 * ih;
  ds[1] = (1.5f * f - 2.f) * f * ih;
  ds[2] = (2.f - 1.5f * g) * g * ih;
  ds[3] = 0.5f * f2 * ih;
}

// Per-axis stencil values of one particle: base node index i0 and, for each
// stencil slot s, the basis value and derivative (0 where the node is absent).
// The derivative is also set to 0 where the value is 0: the reference keeps a
// particle-node pair only when every 1-D value is non-zero (src/tlmpm.cpp:263,
// src/ulmpm.cpp:259-272), and with this masking every product of per-axis
// values and slopes that forms w or grad w of such a pair is 0, so no kernel
// needs a per-node test.  (The boundary-modified cubic spline at ntype 1 has a
// zero value with a non-zero slope; interior cubic values are zero only where
// their slope is zero too.)
//
// o[k] = (x_node - x_p) / h, formed from the same rounded operands as the
// value: the affine moments s (x_node - x_p) built from it keep the spline's
// linear reproduction sum_k s_k o_k = 0 to the rounding of s, where node and
// particle coordinates subtracted in FP32 would leave an error of one ulp of
// |x| (relative to h), which APIC transfers feed back step after step.
template <int BASIS> struct Axis {
  static constexpr int S = Stencil<BASIS>::S;
  int i0;
  float s[S], ds[S], o[S];
  __device__ __forceinline__ void eval(float xp, float lo, float ih, float h, int n, int ng) {
    // the reference truncates (src/tlmpm.cpp:145); the clamp keeps indices of a
    // non-finite or far-away position in range (such a particle raises an error)
    float t = fminf(fmaxf(cells_of(xp, lo, ih), -4.f), (float)(n + 4));
    int c = (int)t;
    i0 = c * Stencil<BASIS>::SC - Stencil<BASIS>::LO;
    if (BASIS == 1 && cubic_interior(i0, n, ng)) {
      const float f = t - (float)c;
      cubic_weights(f, ih, s, ds);
#pragma unroll
      for (int k = 0; k < S; k++) o[k] = (float)(k - 1) - f;
      return;
    }
#pragma unroll
    for (int k = 0; k < S; k++) {
      int i = i0 + k;
      if (i < 0 || i >= n) { s[k] = 0.f; ds[k] = 0.f; o[k] = 0.f; continue; }
      const float r = node_offset_cells(xp, lo, i, h, ih);
      basis<BASIS>(r, node_type<BASIS>(i, ng), ih, s[k], ds[k]);
      ds[k] = s[k] != 0.f ? ds[k] : 0.f;
      o[k] = -r;
    }
  }
  // 1-D (unused axis): weight 1, gradient 0, single slot at node 0
  __device__ __forceinline__ void unit() {
    i0 = 0;
#pragma unroll
    for (int k = 0; k < S; k++) { s[k] = k == 0 ? 1.f : 0.f; ds[k] = 0.f; o[k] = 0.f; }
  }
};

// ------------------------------------------------------------------ 3x3
struct f3x3 { float a[9]; };
__device__ __forceinline__ float det3(const float *m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}
// cofactor matrix: cof(M) = det(M) M^{-T}
__device__ __forceinline__ void cof3(const float *m, float *c) {
  c[0] = m[4] * m[8] - m[5] * m[7];
  c[1] = m[5] * m[6] - m[3] * m[8];
  c[2] = m[3] * m[7] - m[4] * m[6];
  c[3] = m[2] * m[7] - m[1] * m[8];
  c[4] = m[0] * m[8] - m[2] * m[6];
  c[5] = m[1] * m[6] - m[0] * m[7];
  c[6] = m[1] * m[5] - m[2] * m[4];
  c[7] = m[2] * m[3] - m[0] * m[5];
  c[8] = m[0] * m[4] - m[1] * m[3];
}
__device__ __forceinline__ double det3d(const double *m) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) + m[2] * (m[3] * m[7] - m[4] * m[6]);
}
__device__ __forceinline__ void cof3d(const double *m, double *c) {
  c[0] = m[4] * m[8] - m[5] * m[7];
  c[1] = m[5] * m[6] - m[3] * m[8];
  c[2] = m[3] * m[7] - m[4] * m[6];
  c[3] = m[2] * m[7] - m[1] * m[8];
  c[4] = m[0] * m[8] - m[2] * m[6];
  c[5] = m[1] * m[6] - m[0] * m[7];
  c[6] = m[1] * m[5] - m[2] * m[4];
  c[7] = m[2] * m[3] - m[0] * m[5];
  c[8] = m[0] * m[4] - m[1] * m[3];
}
__device__ __forceinline__ void matmul3(const float *a, const float *b, float *c) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}
// c = a^T b
__device__ __forceinline__ void matTmul3(const float *a, const float *b, float *c) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) c[3 * i + j] = a[i] * b[j] + a[3 + i] * b[3 + j] + a[6 + i] * b[6 + j];
}
// c = a b^T
__device__ __forceinline__ void matmulT3(const float *a, const float *b, float *c) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) c[3 * i + j] = a[3 * i] * b[3 * j] + a[3 * i + 1] * b[3 * j + 1] + a[3 * i + 2] * b[3 * j + 2];
}

// det(I + H) - 1 without cancellation: tr H + (sum of principal 2x2 minors) + det H
__device__ __forceinline__ float jm1_of_H(const float *H) {
  float tr = H[0] + H[4] + H[8];
  float m2 = H[0] * H[4] - H[1] * H[3] + H[0] * H[8] - H[2] * H[6] + H[4] * H[8] - H[5] * H[7];
  return tr + m2 + det3(H);
}

// Rotation factor of the polar decomposition F = R U (MPM_Math::PolDec,
// src/mpm_math.h:104-133) by the scaled Newton iteration of N. J. Higham,
// "Computing the polar decomposition -- with applications", SIAM J. Sci.
// Stat. Comput. 7 (1986): X <- (g X + X^-T / g)/2 with g = |det X|^(-1/3).
// For det F > 0 the limit is the unique proper rotation, which is what the
// reference's SVD route returns.  Returns false if det F <= 0.
__device__ inline bool polar_rotation(const float *F, float *R) {
  float X[9], C[9];
#pragma unroll
  for (int k = 0; k < 9; k++) X[k] = F[k];
  float d = det3(X);
  if (!(d > 0.f)) return false;
  // quadratic convergence: stop once the update is at FP32 rounding level
  // (|dX|_F < ~3e-7); the determinant scaling is dropped once |det X - 1| is
  // small, where it no longer accelerates the iteration
  for (int it = 0; it < 12; it++) {
    cof3(X, C);
    const float dx = X[0] * C[0] + X[1] * C[1] + X[2] * C[2];  // det X along the first row
    const float g = fabsf(dx - 1.f) > 1e-3f ? rcbrtf(fabsf(dx)) : 1.f;  // scaling |det X|^(-1/3) (Higham 1986, sec. 3)
    // X <- (g X + X^-T / g) / 2 with X^-T / g = C / (g det X); the halving,
    // exact, is folded into both factors
    const float gh = 0.5f * g, gih = 0.5f / (g * dx);
    float diff = 0.f;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const float xn = fmaf(gih, C[k], gh * X[k]);
      const float e = xn - X[k];
      diff = fmaf(e, e, diff);
      X[k] = xn;
    }
    if (diff < 1e-13f) break;
  }
#pragma unroll
  for (int k = 0; k < 9; k++) R[k] = X[k];
  return true;
}

// A lower bound of min |Re lambda(F)|, F = I + H.  For an eigenpair F x =
// lambda x of the real F, Re lambda = x* S x / x* x with S = sym(F), so every
// real part lies in the spectrum of S, which Gershgorin's discs bound from
// below: min_i (S_ii - sum_{j != i} |S_ij|).  A bound <= 0 says nothing.
__device__ __forceinline__ float re_eig_lower_bound(const float *H) {
  const float s01 = 0.5f * fabsf(H[1] + H[3]), s02 = 0.5f * fabsf(H[2] + H[6]), s12 = 0.5f * fabsf(H[5] + H[7]);
  const float l0 = 1.f + H[0] - s01 - s02, l1 = 1.f + H[4] - s01 - s12, l2 = 1.f + H[8] - s02 - s12;
  return fminf(l0, fminf(l1, l2));
}

// Real parts of the eigenvalues of F = I + H (the reference calls
// Eigen::EigenSolver, src/solid.cpp:1401-1409): the characteristic cubic of H
// solved in closed form (trigonometric form for three real roots, Cardano
// otherwise), shifted by 1.  Returns min |Re lambda|.
__device__ inline float min_abs_eig_real(const float *H) {
  float a2 = H[0] + H[4] + H[8];
  float a1 = H[0] * H[4] - H[1] * H[3] + H[0] * H[8] - H[2] * H[6] + H[4] * H[8] - H[5] * H[7];
  float a0 = det3(H);
  // mu^3 - a2 mu^2 + a1 mu - a0 = 0 ; mu = t + a2/3 (thirds and 27ths as
  // products with the rounded reciprocals)
  constexpr float third = 1.f / 3.f, r27 = 1.f / 27.f;
  float p = a1 - a2 * a2 * third;
  float q = -2.f * a2 * a2 * a2 * r27 + a2 * a1 * third - a0;
  float sh = a2 * third;
  float disc = q * q * 0.25f + p * p * p * r27;
  float m;
  if (disc <= 0.f) {
    float r = sqrtf(fmaxf(-p * third, 0.f));
    float arg = r > 0.f ? (-q / 2.f) / (r * r * r) : 0.f;
    arg = fminf(1.f, fmaxf(-1.f, arg));
    float phi = acosf(arg);
    // cos(phi/3 + 2 pi k/3) for k = 0, 1, 2 from one sine and cosine:
    // cos(a + 2pi/3) = -c/2 - (sqrt 3/2) s, cos(a + 4pi/3) = -c/2 + (sqrt 3/2) s
    float sn, cs;
    sincosf(phi * third, &sn, &cs);
    const float h3 = 0.866025403784439f * sn;
    float e0 = 1.f + sh + 2.f * r * cs;
    float e1 = 1.f + sh + 2.f * r * (-0.5f * cs - h3);
    float e2 = 1.f + sh + 2.f * r * (-0.5f * cs + h3);
    m = fminf(fabsf(e0), fminf(fabsf(e1), fabsf(e2)));
  } else {
    float sd = sqrtf(disc);
    float u = cbrtf(-q / 2.f + sd), v = cbrtf(-q / 2.f - sd);
    float mu = u + v + sh;
    float e_real = 1.f + mu;
    float e_pair = 1.f + (a2 - mu) / 2.f;
    m = fminf(fabsf(e_real), fabsf(e_pair));
  }
  return m;
}

// ------------------------------------------------------------------ constitutive
// The reference's truncated constants (src/solid.cpp:39-40, src/strength_jc.cpp:29)
#define KMPM_SQRT_3_OVER_2 1.224744871
#define KMPM_FOUR_THIRD 1.333333333333333333333333333333333333333

// Symmetric 3x3 in storage order xx yy zz xy xz yz
template <typename T> struct Sym {
  T a[6];
  __device__ __forceinline__ T tr() const { return a[0] + a[1] + a[2]; }
  __device__ __forceinline__ T norm() const {  // Frobenius norm of the full matrix
    return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + T(2) * (a[3] * a[3] + a[4] * a[4] + a[5] * a[5]));
  }
  __device__ __forceinline__ void dev() {
    T t = tr() / T(3);
    a[0] -= t; a[1] -= t; a[2] -= t;
  }
};

struct ConstitutiveIn {
  float J, Jm1, rho, cellsize;
};

// Constitutive laws the stress kernel is compiled for: LAW_ANY dispatches on
// the material at run time; LAW_EOS_LINEAR_JC fixes linear EOS +
// Johnson-Cook strength without damage or temperature (the copper bar), so
// that the other laws' code leaves the kernel.
// Stress kernels compiled for one set of laws (the others' code left out):
// LAW_ANY reads the laws from the material; the rest fix them at compile
// time, for runs whose every material is of that kind (no temperature law)
enum : int { LAW_ANY = 0, LAW_EOS_LINEAR_JC = 1, LAW_EOS_SHOCK_JC_DMG = 2, LAW_FLUID = 3 };
// the EOS, strength and damage law of a set (-1: read from the material;
// damage 1: Johnson-Cook damage, 0: none)
__host__ __device__ constexpr int law_eos(int law) { return law == 1 ? 0 : law == 2 ? 1 : law == 3 ? 2 : -1; }
__host__ __device__ constexpr int law_strength(int law) { return law == 1 || law == 2 ? 2 : law == 3 ? 4 : -1; }
__host__ __device__ constexpr int law_damage(int law) { return law == 2 ? 1 : law == 0 ? -1 : 0; }

// EOS::compute_pressure (src/eos_linear.cpp:71-74, src/eos_shock.cpp:99-133,
// src/eos_fluid.cpp:68-73); T is the particle temperature or 0.
template <typename R, int LAW = LAW_ANY>
__device__ inline R eos_pressure(const MatDev &m, R J, R Jm1, R rho, R damage, R trD, R cellsize, R T) {
  const auto *ep = MatP<R>::eos(m);
  const int eos = law_eos(LAW) >= 0 ? law_eos(LAW) : m.eos;
  if (eos == 0) return -R(ep[1]) * Jm1 * (R(1) - damage);
  // rho/rho0 = 1/J; the compressions below are written in J - 1 so that FP32
  // keeps them accurate when J is close to 1 (no 1/J - 1 cancellation)
  if (eos == 2) {  // K ((rho/rho0)^gamma - 1) = K expm1(-gamma log1p(J-1))
    return R(ep[1]) * expm1(-R(ep[2]) * log1p(Jm1));
  }
  R rho0 = ep[0], c0 = ep[2], S = ep[3], Gamma = ep[4], cv = ep[5], Tr = ep[6];
  R Q1 = ep[7], Q2 = ep[8];
  R mu = -Jm1 / J;  // rho/rho0 - 1
  R dd = R(1) - (S - R(1)) * mu;
  R pH = rho0 * c0 * c0 * mu * (R(1) + mu) / (dd * dd);
  R e = T > Tr ? cv * rho0 * (T - Tr) : R(0);
  R pF = pH + Gamma * e;
  if (damage > R(0) && pF < R(0)) pF = damage >= R(1) ? R(0) : pF * (R(1) - damage);
  if ((Q1 != R(0) || Q2 != R(0)) && trD < R(0))
    pF += rho * cellsize * (Q1 * cellsize * trD * trD - Q2 * c0 * sqrt(J) * trD);
  return pF;
}

// Strength::update_deviatoric_stress (src/strength_linear.cpp:59-71,
// src/strength_plastic.cpp:62-115, src/strength_jc.cpp:100-184,
// src/strength_swift.cpp:77-147, src/strength_fluid.cpp:46-58).
// sig: current sigma (full, symmetric storage), D: rate of deformation.
// Johnson-Cook flow stress at the start of the step
// (StrengthJohnsonCook::update_deviatoric_stress, src/strength_jc.cpp:120-150);
// p = (G, A, B, n, epsdot0, C, m, Tr, Tm)
template <typename R>
__device__ __forceinline__ R jc_flow_stress(const R *p, R epsp, R epsdot, R T) {
  R A = p[1], B = p[2], n = p[3], epsdot0 = p[4], C = p[5], mm = p[6], Tr = p[7], Tm = p[8];
  constexpr bool F32 = sizeof(R) == 4;
  // FP32: epsdot / epsdot0 as a product with 1 / epsdot0 (slot 9), and the
  // two powers of positive bases as exp2(y log2 x): relative error about
  // |y log2 x| ulp, 1e-6 at epsp = 1e-10 and 3e-7 for epsp above 0.1
  R ratio = F32 ? epsdot * p[9] : epsdot / epsdot0;
  ratio = ratio > R(1) ? ratio : R(1);
  R ys = epsp < R(1.0e-10) ? A : A + B * (F32 ? R(exp2f(float(n) * log2f(float(epsp)))) : pow(epsp, n));
  if (C != R(0)) ys *= F32 ? R(exp2f(float(C) * log2f(float(R(1) + ratio)))) : pow(R(1) + ratio, C);
  if (T < Tm) {
    if (mm != R(0) && T >= Tr) ys *= R(1) - pow((T - Tr) / (Tm - Tr), mm);
  } else {
    ys = R(0);
  }
  return ys;
}

template <typename R, int LAW = LAW_ANY>
__device__ inline Sym<R> strength_update(const MatDev &m, R dt, const Sym<R> &sig, const Sym<R> &D, R &dep, R epsp,
                                         R epsdot, R damage, R T, bool *returned = nullptr) {
  Sym<R> out;
  dep = R(0);
  const auto *p = MatP<R>::str(m);
  const int strength = law_strength(LAW) >= 0 ? law_strength(LAW) : m.strength;
  if (strength == 0) {  // linear: dev(sigma) + dt 2G(1-D) dev(D)
    Sym<R> s = sig, d = D;
    s.dev(); d.dev();
    R f = dt * R(2) * R(p[0]) * (R(1) - damage);
#pragma unroll
    for (int k = 0; k < 6; k++) out.a[k] = s.a[k] + f * d.a[k];
    return out;
  }
  if (strength == 4) {  // fluid: 2 mu dev(D)
    Sym<R> d = D;
    d.dev();
#pragma unroll
    for (int k = 0; k < 6; k++) out.a[k] = R(2) * R(p[0]) * d.a[k];
    return out;
  }
  if (strength == 1) {  // perfect plasticity
    R Gd = R(p[0]) * (R(1) - damage), syD = R(p[1]) * (R(1) - damage);
    Sym<R> s = sig, d = D;
    s.dev(); d.dev();
#pragma unroll
    for (int k = 0; k < 6; k++) out.a[k] = s.a[k] + dt * R(2) * Gd * d.a[k];
    R J2 = sqrt(R(1.5)) * out.norm();
    if (J2 < syD) return out;
    dep = (J2 - syD) / (R(3) * Gd);
    R sc = syD / J2;
#pragma unroll
    for (int k = 0; k < 6; k++) out.a[k] *= sc;
    return out;
  }
  // Johnson-Cook (2) and Swift (3): closed-form radial return
  if (damage >= R(1)) {
#pragma unroll
    for (int k = 0; k < 6; k++) out.a[k] = R(0);
    return out;
  }
  R G = p[0], ys;
  if (strength == 2) {
    ys = jc_flow_stress<R>(p, epsp, epsdot, T);
  } else {
    R A = p[1], B = p[2], C = p[3], n = p[4];
    ys = (epsp > R(1.0e-10) && epsp > C) ? A + B * pow(epsp - C, n) : A;
  }
  R Gd = G;
  if (damage > R(0)) { Gd *= (R(1) - damage); ys *= (R(1) - damage); }
  R f = dt * R(2) * Gd;
#pragma unroll
  for (int k = 0; k < 6; k++) out.a[k] = sig.a[k] + f * D.a[k];
  out.dev();
  R J2 = R(KMPM_SQRT_3_OVER_2) * out.norm();
  if (J2 < ys) return out;
  if (returned) *returned = true;  // the trial state reached the yield surface
  dep = (J2 - ys) / (R(3) * Gd);
  R sc = ys / J2;
#pragma unroll
  for (int k = 0; k < 6; k++) out.a[k] *= sc;
  return out;
}

// DamageJohnsonCook::compute_damage, src/damage_jc.cpp:91-143
template <typename R>
__device__ inline void damage_update(const MatDev &m, R &dinit, R &damage, R pH, const Sym<R> &sdev, R epsdot, R dep,
                                     R T) {
  const auto *p = MatP<R>::dam(m);
  if (dep == R(0) && damage >= R(1)) return;
  R vm = R(KMPM_SQRT_3_OVER_2) * sdev.norm();
  R triax = R(0);
  if (pH != R(0) && vm != R(0)) triax = -pH / (vm + R(0.001) * fabs(pH));
  if (triax <= R(-3)) { dinit = R(0); return; }
  R ef = R(p[0]) + R(p[1]) * exp(R(p[2]) * triax);
  if (R(p[3]) > R(0) && epsdot > R(p[5])) ef *= (R(1) + R(p[3]) * log(epsdot / R(p[5])));
  if (R(p[4]) > R(0) && T >= R(p[6])) ef *= R(1) + R(p[4]) * (T - R(p[6])) / (R(p[7]) - R(p[6]));
  dinit += dep / ef;
  if (dinit >= R(1)) {
    R dn = (dinit - R(1)) * R(10);
    damage = dn < R(1) ? dn : R(1);
  }
}

}  // namespace kmpm
