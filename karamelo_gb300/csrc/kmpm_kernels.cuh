// kmpm_kernels.cuh -- kernel argument blocks and the per-mode scatter payloads.
#pragma once
#include "kmpm_common.cuh"

namespace kmpm {

// scatter modes
enum P2GMode : int {
  P2G_MASS = 0,  // m                      (TLMPM: once, Solid::compute_mass_nodes)
  P2G_TL = 1,    // p, f_int (TL)          (+ mT, Qext, Qint when thermal)
  P2G_UL = 2,    // m, p, f_int (UL)       (+ mT, Qext, Qint)
  P2G_VEL = 3,   // p                      (MUSL re-map; + mT)
  // APIC (Solid::compute_velocity_nodes_APIC, src/solid.cpp:392-426): the
  // same sums with the particle velocity v + C (x_node - x_p); the payload
  // adds m C (9) and x_w - x_p (3), x_w the position of the weights
  P2G_TL_APIC = 4,
  P2G_UL_APIC = 5,
  P2G_VEL_APIC = 6,
  // flag on the force modes: the particle's external force mbp (3, contact
  // fixes) joins the payload and w mbp the force sums -- the grid's
  // f + mb of Grid::update_grid_velocities (src/grid.cpp:456), filled by
  // Solid::compute_external_forces_nodes (src/solid.cpp:428-449)
  P2G_EXT = 8,
  // flag on the force modes of axisymmetric runs: the hoop term
  // T_zz / r (1) joins the payload, and -w T_zz / r the radial force sums
  // (src/solid.cpp:472-475, 513-519, 565-571)
  P2G_AXI = 16,
  // flag on P2G_TL (TLMPM MUSL, FLIP/PIC, mechanical): the force sums only
  // (k_p2g_force_row).  TLMPM's weights and masses do not change, and no
  // velocity changes between a step's re-map and the next step's scatter, so
  // the nodal momentum of that scatter is the re-map's sum, bit for bit: the
  // velocity pass of the grid keeps it (GridArgs::nodeP) and the next grid
  // update reads it there
  P2G_FONLY = 32,
};
__host__ __device__ constexpr int p2g_kind(int mode) { return mode & 7; }
__host__ __device__ constexpr bool p2g_axi(int mode) { return (mode & P2G_AXI) != 0; }
__host__ __device__ constexpr int p2g_base(int mode) { return p2g_kind(mode) >= P2G_TL_APIC ? p2g_kind(mode) - 3 : p2g_kind(mode); }
__host__ __device__ constexpr bool p2g_apic(int mode) { return p2g_kind(mode) >= P2G_TL_APIC; }
__host__ __device__ constexpr bool p2g_ext(int mode) { return (mode & P2G_EXT) != 0; }
__host__ __device__ constexpr bool p2g_fonly(int mode) { return (mode & P2G_FONLY) != 0; }
// GM_UPDATE_F: the grid update after a P2G_FONLY scatter (momentum from
// nodeP); GM_STORE_P: the momentum sums of a P2G_VEL scatter into nodeP
enum GridMode : int { GM_MASS = 0, GM_UPDATE = 1, GM_VEL = 2, GM_UPDATE_F = 3, GM_STORE_P = 4 };

__host__ __device__ constexpr int p2g_nq(int mode, bool th) {
  return p2g_fonly(mode) ? 3
         : p2g_base(mode) == P2G_MASS  ? 1
         : p2g_base(mode) == P2G_TL ? (th ? 9 : 6)
         : p2g_base(mode) == P2G_UL ? (th ? 10 : 7)
                                    : (th ? 4 : 3);
}
__host__ __device__ constexpr int p2g_nin(int mode, bool th) {
  return p2g_fonly(mode) ? 9
         : (p2g_base(mode) == P2G_MASS  ? 1
          : p2g_base(mode) == P2G_TL ? (th ? 17 : 12)
          : p2g_base(mode) == P2G_UL ? (th ? 15 : 10)
                                     : (th ? 4 : 3)) +
         (p2g_apic(mode) ? 12 : 0) + (p2g_ext(mode) ? 3 : 0) + (p2g_axi(mode) ? 1 : 0);
}

struct P2GArgs {
  float *const *Pp;          // device pointer to the current particle buffer
  size_t ps;                 // particle field stride
  int pos_field;             // PF_X0 (TL) or PF_X (UL)
  const int2 *tiles;         // (grid, tile) of every non-empty tile
  const GridDev *grids;
  const int *cell_start, *cell_end;  // particle range of every cell (sorted order)
  float *partial;            // tile footprint slices
  size_t pstride_tile;       // floats per tile slice
  const int *tile_start, *tile_end;  // particle range of every tile (empty tiles are skipped)
  const StepScalars *scalars;
  int apic_pos;              // APIC: displacement field added to x0 for x_p (PF_X, PF_XN) or -1 (TL: x0)
                             // (pos_field is that of the weights)
  int mls;                   // ULMPM MLS: internal forces from moments, Di = mls_di
  float mls_di;
  const float *mbp;          // P2G_EXT: external particle forces, 3 rows of ps floats
  // the fused MUSL gather + re-map (k_g2p1_remap_row): what k_g2p1 reads
  const float4 *nodeA;       // v, v_update interleaved, stride NODE_STRIDE
  float pic_flip;
  float boxlo[3], boxhi[3];  // ULMPM: the domain the moved particles must stay in
  ErrState *err;
  int indep;                 // per-solid clocks (independent instances)
};

struct GridArgs {
  const GridDev *grids;
  const int *blk_grid, *grid_blk0;
  const float *partial;
  size_t pstride_tile;
  const int *tile_start, *tile_end;
  float4 *nodeA, *nodeB, *nodeX;  // nodeA / nodeB: one array, stride NODE_STRIDE
  float *nodeT;
  const FixDev *fixes;
  const int *fix_start, *fix_count;
  StepScalars *scalars;
  int indep;                 // per-solid clocks (independent instances)
  int remap;                 // GM_VEL: MUSL re-map (else positions only)
  // TLMPM MUSL momentum reuse (P2G_FONLY): GM_VEL stores the re-map's nodal
  // momentum sums (before the velocity BCs) here and GM_UPDATE_F reads them;
  // nullptr where the reuse is off
  float4 *nodeP;
};

struct HRange;  // the h-ratio bound of one range (below)

struct PartArgs {
  float *const *Pp;
  size_t ps;
  const RangeDev *ranges;
  const int *blk_range;
  const int *solid_mat;      // solid id -> material id (ULMPM per-particle lookup)
  const GridDev *grids;
  const MatDev *mats;
  const float4 *nodeA, *nodeB;  // one array, stride NODE_STRIDE
  const float *nodeT;
  StepScalars *scalars;
  ErrState *err;
  float *blk_c, *blk_h;
  float pic_flip;
  float T_ref;               // particle and nodal temperatures are stored as T - T_ref
  float boxlo[3], boxhi[3];
  int indep, use_vu, thermal, track_strain, dim;
  int tile_t[3];
  int apic;                  // APIC transfers: k_g2p2 forms grad v from moments and stores PF_C
  const HRange *hr;          // TLMPM, one clock: the h-ratio bound of each range (nullptr: solve every particle)
  int asflip;                // ULMPM ASFLIP: positions move with the blended velocity
  int axisym;                // 2-D axisymmetric: Fdot(2,2) / L(2,2) += v_r w / r
  // 3-D TLMPM: each 256-particle block's staged node box of the stress kernel's
  // gather, fixed by x0 (k_gather_box at setup): int4 (lo, vol or -1 when
  // not staged), int4 (nb, 0) per block; null: the kernel computes it
  const int4 *gbox;
  // queue of the plastic particle-steps for the learned return map (the
  // stress kernel's QUEUE variant writes it, k_learn_queue reads it):
  // LQ_NF float rows and LQ_NI int rows of lq_cap entries each
  float *lq_f;
  int *lq_i;
  int *lq_count;
  unsigned long long *lq_stats;
  long long lq_cap;
};
// queue rows: slot, material; dt, tav, D (6), sigma before the step (6),
// eps_p, eps_p rate, pressure, trace of strain_el, R (9), cof F (9)
enum { LQ_P = 0, LQ_MAT = 1, LQ_NI = 2 };
enum { LQ_DT = 0, LQ_TAV = 1, LQ_D = 2, LQ_SIG = 8, LQ_EPSP = 14, LQ_EPSDOT = 15, LQ_PH = 16, LQ_TRE = 17,
       LQ_R = 18, LQ_COF = 27, LQ_NF = 36 };

// The h ratio of the time step (TLMPM), per range: the smallest
// min(1, |Re lambda(F)|) over its particles (src/solid.cpp:1399-1409).  The
// stress kernel solves the characteristic cubic only for particles whose
// cheap lower bound (re_eig_lower_bound) lies below `bound`; the others
// report `bound`.  If the range's reduced minimum reaches `bound`, one of
// them may hold the true minimum, and k_h_exact recomputes the range from
// every particle: the result is the exact minimum whatever the bound.
struct HRange {
  float bound;  // this step's threshold: min(1, 1.001 x the last exact minimum); 0 at setup
  float hmin;   // the range's minimum of this step (exact once the step's dt is formed)
  float cmax;   // the range's largest wave speed of this step
  int need;     // 1: the reduced minimum reached the bound (k_h_exact recomputes it)
};

struct DtArgs {
  const RangeDev *ranges;
  const GridDev *grids;
  const float *blk_c, *blk_h;
  double *solid_dtcfl;
  StepScalars *scalars;
  ErrState *err;
  int nranges, indep, dt_constant;
  double dt_factor;
  int max_nblk;              // largest range, in 256-particle blocks (picks the reduction width)
  // TLMPM h ratio (nullptr for ULMPM and independent instances): per-range bounds, the list of the
  // ranges k_h_exact recomputes and its length, the particle state it reads
  HRange *hr;
  int *hflags, *nhflag;
  float *const *Pp;
  size_t ps;
  int exact_blocks;          // grid of k_h_exact
};

struct LaunchSet {
  int dummy;
};

// kernel entry points of one (dim, basis) instantiation
struct StepKernels {
  void *p2g_mass, *p2g_tl, *p2g_tl_th, *p2g_ul, *p2g_ul_th, *p2g_vel, *p2g_vel_th;
  // the row scatters (k_p2g_row, k_p2g_row2) of the plain TL, UL and
  // velocity modes: 2-D and 3-D cubic and quadratic splines (nullptr elsewhere)
  void *p2g_row[3];
  // the scatter of the force sums only (P2G_TL | P2G_FONLY: k_p2g_force_row
  // in 3-D, k_p2g_row2 in 2-D) and its dynamic shared memory (0: that of
  // p2g_smem_bytes), the grid update that takes the stored momentum
  // (GM_UPDATE_F) and the pass that stores the momentum of a velocity
  // scatter (GM_STORE_P): TLMPM, FP32, mechanical, cubic and quadratic
  // splines (nullptr elsewhere)
  void *p2g_row_fonly, *grid_upd_fonly, *grid_store_p;
  int p2g_row_fonly_smem;
  void *p2g_tl_apic, *p2g_ul_apic, *p2g_vel_apic;  // cubic spline only (nullptr otherwise)
  // the force scatters with external particle forces (P2G_EXT): [thermal]
  void *p2g_tl_ext[2], *p2g_ul_ext[2], *p2g_tl_apic_ext, *p2g_ul_apic_ext;
  // 2-D axisymmetric force scatters (P2G_AXI): [UL][APIC][EXT] (nullptr elsewhere)
  void *p2g_axi[2][2][2];
  void *grid_mass[2], *grid_upd[2][2][2], *grid_vel[2][2][2];
  void *g2p1[2][2], *g2p2[2][2][2];
  // launch-shape candidates [TL][variant] of the gathers (FP32, no thermal):
  // __launch_bounds__(256, G2P1_MINB[v] / G2P2_MINB[v]); variant 0 is the default
  void *g2p1_v[2][3], *g2p2_v[2][3];
  // the same stress-kernel shapes compiled for linear EOS + Johnson-Cook only
  // (LAW_EOS_LINEAR_JC; 3-D, nullptr elsewhere)
  void *g2p2_jc[2][3];
  void *g2p2_jcq[3];  // 3-D cubic TLMPM, linear EOS + Johnson-Cook, queueing plastic steps
  // compiled for shock EOS + Johnson-Cook + Johnson-Cook damage (2-D cubic
  // TLMPM) and for fluid EOS + fluid strength (3-D cubic ULMPM) [TL][variant]
  void *g2p2_jcd[2][3], *g2p2_fl[2][3];
  void *gather_box;  // TLMPM: the stress kernel's node box of every block (k_gather_box)
  // MUSL gather + re-map in one pass (k_g2p1_remap_row) [TL]: 3-D cubic and
  // quadratic splines (nullptr elsewhere), and its dynamic shared memory
  void *g2p1_remap[2];
  int g2p1_remap_smem;
};
constexpr int G2P_NVAR = 3;
// node staging of the gathers (k_g2p1, k_g2p2): nodes of a block's stencil
// bounding box copied into shared memory, and the dynamic shared memory of
// the two kernels (v and v_update pairs; one (v, T) vector)
constexpr int G2P_STAGE_NODES = 1024;
constexpr int G2P1_SMEM = G2P_STAGE_NODES * 32;
constexpr int G2P2_SMEM = G2P_STAGE_NODES * 16;
// the linear EOS + Johnson-Cook stress kernels also stage their particles'
// state rows v .. damage (PF_V .. PF_DMG), 256 floats each
constexpr int G2P2_STATE_ROWS = 23;
constexpr int G2P2_JC_SMEM = G2P2_SMEM + G2P2_STATE_ROWS * 256 * 4;
constexpr int G2P1_MINB[G2P_NVAR] = {4, 3, 6};
constexpr int G2P2_MINB[G2P_NVAR] = {3, 2, 4};

void get_step_kernels(int dim, int basis, StepKernels &k);
// particle downloads (kmpm_dump.cu): values per particle of a KMPM_P_* field
// (0 if unknown) and the gather of one solid's field into caller order, FP64
int dump_width(int field);
void launch_dump(const PartArgs &a, int ri, int count, int solid, int base, int field, int TL, int rotate,
                 double T_ref, double *out, cudaStream_t st);
// the inverse: one field of one solid from caller order (FP64, device) into its slots
void launch_load(const PartArgs &a, int ri, int count, int solid, int base, int field, int TL, double T_ref,
                 const double *in, cudaStream_t st);
int p2g_smem_bytes(int dim, int basis, int mode, bool thermal);

// kmpm_contact.cu: one contact fix between two solids (device form)
struct ContactDev {
  int kind;                  // KMPM_CONTACT_*
  int dim, thermal;
  int ul;                    // ULMPM: members are the slots of one range, told apart by PF_SID
  int sid1, sid2;            // solid ids (ULMPM member test)
  int start1, n1, start2, n2;  // TLMPM: the two solids' slot ranges; ULMPM: start1, n1 = the range
  int nmem;                  // members (n1 + n2 TLMPM, n1 ULMPM)
  int nb, key_bits;          // hash buckets (a power of two) and sort key bits (bucket nb = not a member)
  float mu, estar, alpha, hcoef, cmax, inv_cmax;
  float invcp1, invcp2;
  float boxlo[3];
  int *keys, *vals;          // bucket of every member, sorted with the member index
  int *bstart, *bend;        // member range of every bucket in sorted order
  float4 *ra, *rb;           // per member: (x, Rp), (v, m)
  int4 *rc;                  // per member: cell (3), tag (0 solid1, 1 solid2, -1 neither)
  double *blk, *ftot;        // per-block partial sums of the pair forces, their total
  float *mbp;                // 3 rows of ps floats: external particle forces
  int axisym;                // 2-D axisymmetric: the min-penetration Rp uses vol / r
};

// kmpm_misc.cu
// one solid's caller arrays (device copy, FP64: x0, x, v as n*3, mass, vol0)
// into its slots of the particle buffer
struct StageArgs {
  const double *in;
  int n, slot0, orig0, sid, ul, thermal;
  float T;
  size_t ps;
  float *P;
};
void launch_stage_solid(const StageArgs &a, cudaStream_t st);
// the error word into mapped host memory (read after a stream synchronize)
void launch_publish_err(const ErrState *d, ErrState *h_mapped, cudaStream_t st);
void launch_cell_keys(const PartArgs &a, int nblk, int *keys, int use_x0, cudaStream_t st, int pad_last = 0);
void launch_cell_ranges(const int *sorted_keys, int start, int n, int ncell_per_tile, int *cell_start, int *cell_end,
                        int *tile_start, int *tile_end, cudaStream_t st);
void launch_dt(const DtArgs &a, cudaStream_t st);
void launch_energy(const PartArgs &a, int nblk, double *blk, double *out, cudaStream_t st);
// stable LSD radix sort of (key, value) pairs by key, 8 bits per pass
struct RadixTemp {
  int *k1, *v1, *hist, *tot;
  int max_blocks;
};
void radix_sort(int *keys, int *vals, int n, int key_bits, RadixTemp &tmp, cudaStream_t st);
// kmpm_contact.cu: launches one contact's kernels on st; returns the number of launches
int launch_contact(const PartArgs &a, const ContactDev &c, RadixTemp &rt, cudaStream_t st);
void launch_iota(int *v, int n, cudaStream_t st);

// cell key of a position: global tile * cells per tile + cell within the
// tile (tile-major order), cells clamped to the lattice
__device__ __forceinline__ int cell_key(const GridDev &g, int T0, int T1, int T2, const float x[3], int dim) {
  int c[3] = {0, 0, 0};
#pragma unroll
  for (int d = 0; d < 3; d++)
    if (d < dim) c[d] = max(0, min((int)((x[d] - g.lo[d]) * g.inv_cellsize), g.ncell[d] - 1));
  const int tl = ((c[0] / T0) * g.ntile[1] + c[1] / T1) * g.ntile[2] + c[2] / T2;
  const int lc = ((c[0] % T0) * T1 + c[1] % T1) * T2 + c[2] % T2;
  return (g.tile_off + tl) * (T0 * T1 * T2) + lc;
}

// ULMPM re-binning as an update of the previous binning (kmpm_rebin.cu).
// keys / cell_start / cell_end hold a consistent binning of the current slot
// order on entry (sorted keys, and the ranges of those keys) and the binning
// by the new positions on exit; perm gets the stable-sort permutation.
constexpr int RB_CELLS_PER_THREAD = 16;
constexpr int RB_CHUNK = 256 * RB_CELLS_PER_THREAD;  // cells per block of the count / range kernels
struct RebinArgs {
  PartArgs pa;
  int grid, start, n;     // the particle range [start, start + n) on grid `grid`
  int ncell, ncell_pad;   // cells of all tiles; allocated (multiple of RB_CHUNK, > ncell)
  int ncpt;               // cells per tile
  int *keys;              // [n] cell of every slot, sorted
  int *knew;              // [n] cell of the new position
  unsigned *mflag;        // [nblk * 8] bit per slot: the cell changed
  int *cin, *cout;        // [ncell_pad] movers into / out of every cell (zero between steps)
  int *mpre;              // [ncell_pad] exclusive prefix of cin
  int *bsum;              // [2 * nchunk] per-chunk sums of the new counts and of cin (padded to 4096 ints)
  int *blkm;              // [nblk] movers per 256 slots (padded to 4096 ints)
  int *brun, *bsort;      // [n] movers grouped by destination cell; then sorted by slot in each group
  int *cell_start, *cell_end, *tile_start, *tile_end;
  int *perm;              // [n] source slot (relative to start) of every destination slot
};
int launch_rebin(const RebinArgs &r, cudaStream_t st);  // returns the number of launches
void launch_permute(float *const *src_pp, float *const *dst_pp, size_t ps, const int *perm, int start, int n,
                    const int *fields, int nfields, cudaStream_t st);
void launch_swap_ptrs(float **pp, cudaStream_t st);

// Starts the DRAM reads of particles [p0, p1) of field rows row0 .. row0 +
// nrows - 1 into L2, one prefetch per 128-byte line, spread over the block's
// threads.  A hint that holds no registers: a tile kernel issues it before
// staging its node footprint, so that the loads of its particle rows, row
// after row, find them in L2.  Field rows start on 1 KB boundaries (the field
// stride is a multiple of 256 particles), and every line lies inside its row.
__device__ __forceinline__ void prefetch_rows_l2(const float *P, size_t ps, int row0, int nrows, int p0, int p1) {
  if (p1 <= p0) return;
  const int l0 = p0 >> 5, nl = ((p1 - 1) >> 5) - l0 + 1;  // 32 floats per line
  const float *base = P + (size_t)row0 * ps + (size_t)l0 * 32;
  for (int e = threadIdx.x; e < nrows * nl; e += blockDim.x) {
    const int f = e / nl, l = e - f * nl;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (size_t)f * ps + (size_t)l * 32));
  }
}

static_assert(PF_X == PF_X0 + 3 && PF_V == PF_X + 3 && PF_MASS == PF_V + 3, "x0, u, v, mass rows are contiguous");

// ---- payload staged per particle for the scatter
template <int MODE_, bool TH>
__device__ __forceinline__ void p2g_payload(const P2GArgs &a, const float *P, int p, float *pay) {
  constexpr int MODE = p2g_base(MODE_);
  const size_t ps = a.ps;
  if (p2g_fonly(MODE_)) {  // vol0 PK1 only
#pragma unroll
    for (int k = 0; k < 9; k++) pay[k] = P[(PF_PK + k) * ps + p];
    return;
  }
  const float m = P[PF_MASS * ps + p];
  if (MODE == P2G_MASS) { pay[0] = m; return; }
  int o = 0;
  if (MODE == P2G_UL) pay[o++] = m;
#pragma unroll
  for (int d = 0; d < 3; d++) pay[o++] = m * P[(PF_V + d) * ps + p];
  if (MODE == P2G_TL) {
#pragma unroll
    for (int k = 0; k < 9; k++) pay[o++] = P[(PF_PK + k) * ps + p];
  } else if (MODE == P2G_UL) {
#pragma unroll
    for (int k = 0; k < 6; k++) pay[o++] = P[(PF_PK + k) * ps + p];
  }
  if (TH) {
    pay[o++] = m * P[PF_T * ps + p];
    if (MODE != P2G_VEL) {
      pay[o++] = P[PF_GAMMA * ps + p];
#pragma unroll
      for (int d = 0; d < 3; d++) pay[o++] = P[(PF_Q + d) * ps + p];
    }
  }
  if (p2g_apic(MODE_)) {
#pragma unroll
    for (int k = 0; k < 9; k++) pay[o++] = m * P[(PF_C + k) * ps + p];
    // x_w - x_p: the weights' position minus the affine one (ULMPM re-map:
    // u - u_moved; 0 where both are the same)
#pragma unroll
    for (int d = 0; d < 3; d++)
      pay[o++] = (a.apic_pos >= 0 && a.apic_pos != a.pos_field)
                     ? P[(a.pos_field + d) * ps + p] - P[(a.apic_pos + d) * ps + p] : 0.f;
  }
  if (p2g_ext(MODE_)) {
#pragma unroll
    for (int d = 0; d < 3; d++) pay[o++] = a.mbp[d * ps + p];
  }
  if (p2g_axi(MODE_)) {
    // T_zz / r: vol0 PK1(2,2) / x0_r (TL) or vol sigma(2,2) / x_r (UL)
    const float r = P[PF_X0 * ps + p] + (a.pos_field == PF_X ? P[PF_X * ps + p] : 0.f);
    pay[o++] = P[(PF_PK + (MODE == P2G_TL ? 8 : 2)) * ps + p] / r;
  }
}

// ---- contribution of one particle to one node
template <int MODE_, bool TH, int Q>
__device__ __forceinline__ void p2g_accumulate(float *acc, const float *pay, float w, const float *gw) {
  constexpr int MODE = p2g_base(MODE_);  // APIC modes never take this path (no thermal APIC)
  if (MODE == P2G_MASS) { acc[0] += w * pay[0]; return; }
  int o = 0, i = 0;
  if (MODE == P2G_UL) acc[o++] += w * pay[i++];
#pragma unroll
  for (int d = 0; d < 3; d++) acc[o++] += w * pay[i++];
  if (MODE == P2G_TL) {
    // f -= vol0PK1 * grad w  (src/solid.cpp:468)
#pragma unroll
    for (int d = 0; d < 3; d++) acc[o + d] -= pay[i + 3 * d] * gw[0] + pay[i + 3 * d + 1] * gw[1] + pay[i + 3 * d + 2] * gw[2];
    o += 3;
    i += 9;
  } else if (MODE == P2G_UL) {
    // f -= vol * sigma * grad w  (src/solid.cpp:508); sigma symmetric xx yy zz xy xz yz
    const float *s = pay + i;
    acc[o + 0] -= s[0] * gw[0] + s[3] * gw[1] + s[4] * gw[2];
    acc[o + 1] -= s[3] * gw[0] + s[1] * gw[1] + s[5] * gw[2];
    acc[o + 2] -= s[4] * gw[0] + s[5] * gw[1] + s[2] * gw[2];
    o += 3;
    i += 6;
  }
  if (TH) {
    acc[o++] += w * pay[i++];  // m T
    if (MODE != P2G_VEL) {
      acc[o++] += w * pay[i++];  // Qext: w gamma
      acc[o++] += gw[0] * pay[i] + gw[1] * pay[i + 1] + gw[2] * pay[i + 2];  // Qint: grad w . q
      i += 3;
    }
  }
  if (p2g_ext(MODE_)) {
    // f += w mbp (the force sums follow the momentum: index 3 TL, 4 UL)
    constexpr int FO = MODE == P2G_UL ? 4 : 3;
#pragma unroll
    for (int d = 0; d < 3; d++) acc[FO + d] += w * pay[i + d];
  }
}

}  // namespace kmpm
