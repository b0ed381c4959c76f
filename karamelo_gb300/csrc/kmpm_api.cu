// kmpm_api.cu -- the C ABI of include/kmpm.h: context, device layout, the
// per-step launch sequence (captured once as a CUDA graph and replayed), and
// the host<->device conversions between the caller's FP64 arrays and the
// device's FP32 structure of arrays.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/kmpm.h"
#include "kmpm_kernels.cuh"
#include "kmpm_learn.h"

using namespace kmpm;

namespace kmpm {
void launch_step_begin(StepScalars *s, int n, cudaStream_t st);
void launch_fix_values(FixDev *fixes, int nfix, const GridDev *grids, const StepScalars *scalars, int indep,
                       cudaStream_t st);
}

struct kmpm_ctx {
  kmpm_params prm{};
  std::string err;
  cudaStream_t st = nullptr;
  // ---- host-side definitions
  std::vector<MatDev> mats;
  struct HGrid {
    double lo[3];
    double cellsize;
    int n[3], ng[3];
  };
  std::vector<HGrid> hgrids;
  struct HSolid {
    int grid, mat, n;
    int np_per_cell = 0;  // Solid::np_per_cell (particles per cell per direction; linear APIC)
    double T0;
    // the caller's arrays, copied to the device as given (FP64: x0, x, v as
    // n*3, then mass, vol0); converted into the particle buffer at build
    double *d_in = nullptr;
  };
  std::vector<HSolid> hsolids;
  struct HFix {
    int kind, grid, set[3];
    std::vector<uint8_t> mask;
    double c[12];
  };
  std::vector<HFix> hfixes;
  bool built = false, fixes_dirty = true;
  // contact fixes: the pairs of solids, and their device state
  struct HContact {
    int kind, s1, s2;
    double mu;
  };
  std::vector<HContact> hcontacts;
  std::vector<double> mat_E, mat_nu;  // Mat::E, Mat::nu (derived from K and G for EOS materials)
  std::vector<ContactDev> contacts;
  float *d_mbp = nullptr;             // external particle forces, 3 rows of ps floats
  bool contacts_dirty = false;
  // the force scatter of this configuration (select_scatters) and the
  // non-affine one of the USF scheme's second pass, with their shared memory
  void *sc_force = nullptr, *sc_usf = nullptr;
  int smem_force = 0, smem_usf = 0;
  // ---- device layout
  size_t ps = 0;
  int nblk_p = 0;
  float *buf[2] = {nullptr, nullptr};
  float **d_pp = nullptr;  // d_pp[0] current buffer, d_pp[1] the other
  std::vector<RangeDev> ranges;
  std::vector<int> solid_range, solid_base;
  RangeDev *d_ranges = nullptr;
  int *d_blk_range = nullptr;
  int *d_solid_mat = nullptr;
  std::vector<GridDev> grids;
  GridDev *d_grids = nullptr;
  int *d_blk_grid = nullptr, *d_grid_blk0 = nullptr;
  int nblk_g = 0, nnodes_pad = 0;
  MatDev *d_mats = nullptr;
  float4 *nodeA = nullptr, *nodeB = nullptr, *nodeX = nullptr;
  float *nodeT = nullptr;
  // TLMPM MUSL force-only scatter and momentum reuse (P2G_FONLY): the step's
  // scatter sums the forces only (k_p2g_force_row) and the grid update takes
  // the nodal momentum from nodeP: the last re-map's sums, kept by the grid
  // velocity pass, or, where those are not the current state's, the sums of
  // a velocity scatter run first.  fonly: this configuration takes that path
  // (select_scatters); reuse_ok: the re-map's sums may be reused
  // (KMPM_NO_MOMENTUM_REUSE=1: never); p_valid: nodeP holds the sums of the
  // particles' current velocities (set by every step, cleared by anything
  // that changes the particle state between steps)
  float4 *nodeP = nullptr;
  bool fonly = false, reuse_ok = false, p_valid = false;
  int smem_fonly = 0;
  int tdim[3] = {0, 0, 0}, NCELL = 0, ntiles_total = 0;
  int2 *d_tiles = nullptr;
  int ntiles_launch = 0;
  int *d_cs = nullptr, *d_ce = nullptr, *d_ts = nullptr, *d_te = nullptr;
  float *partial = nullptr;
  size_t pstride_tile = 0;
  FixDev *d_fixes = nullptr;
  int nfix_dev = 0;
  int *d_fix_start = nullptr, *d_fix_count = nullptr;
  std::vector<uint8_t *> d_masks;
  StepScalars *d_scalars = nullptr;
  int nscalars = 1;
  double *d_dtcfl = nullptr;
  // TLMPM h ratio of the time step: per-range bounds, the flagged ranges
  // (HRange, k_h_exact) and the exact pass's grid
  HRange *d_hr = nullptr;
  int4 *d_gbox = nullptr;  // TLMPM: the stress kernel's node box of every block
  int *d_hflags = nullptr, *d_nhflag = nullptr;
  int exact_blocks = 0;
  bool exact_h = false;  // KMPM_EXACT_H=1: the cubic for every particle (no bounds)
  ErrState *d_err = nullptr;
  // host view of the error word: page-locked, mapped, written by a one-thread
  // kernel at the end of every run, so that reading it needs no copy engine
  // (a small copy would queue behind a dump's device-to-host copy)
  ErrState *h_err = nullptr, *h_err_dev = nullptr;
  double maxtime_dev = 1e300;  // StepScalars::maxtime as last written
  float *d_blk_c = nullptr, *d_blk_h = nullptr;
  double *d_eblk = nullptr, *d_eout = nullptr;
  int *d_keys = nullptr, *d_vals = nullptr;
  // ULMPM re-binning as an update of the last binning (launch_rebin); the
  // full radix sort of every key each step with KMPM_FULL_REBIN=1
  bool full_rebin = false;
  int ncell_pad = 0;
  int *d_knew = nullptr, *d_cin = nullptr, *d_cout = nullptr, *d_mpre = nullptr, *d_bsum = nullptr;
  int *d_blkm = nullptr, *d_brun = nullptr, *d_bsort = nullptr;
  unsigned *d_mflag = nullptr;
  RadixTemp rtmp{};
  int key_bits = 0;
  std::vector<int> ul_fields;
  StepKernels K{};
  cudaGraphExec_t gexec = nullptr;
  cudaGraphExec_t gexec_r = nullptr;  // the step with the momentum reuse (fonly and reuse_ok)
  bool graph_valid = false;
  int launches_per_step = 0;
  int smem[4][2] = {{0}};
  // per-kernel timing (kmpm_profile): events recorded between launches
  bool profiling = false;
  std::vector<cudaEvent_t> prof_ev;
  std::vector<std::string> prof_names;
  int prof_n = 0;
  // TLMPM keeps its binning order for the whole run: caller index of every slot
  std::vector<int> orig_cache, sid_cache;
  // temperatures are kept as T - T_ref in FP32 (T_ref: the first solid's
  // initial temperature in thermo-mechanical runs, 0 otherwise)
  double T_ref = 0;
  // learned return map: MODE_PLAIN, MODE_LOG (training pairs) or MODE_SUR
  int learn_mode = MODE_PLAIN;
  unsigned char *d_blob = nullptr;
  float sur_tol = 0.f;
  unsigned long long *d_lstats = nullptr, *d_log_count = nullptr;
  float *d_log = nullptr;
  long long log_cap = 0;
  uint32_t log_thresh = 0;
  unsigned long long log_seed = 0;
  LearnKernels LK{};
  // autotuner: chosen launch-shape variant of each gather kernel, its record
  int var_g2p1 = 0, var_g2p2 = 0;
  // learned return map on linear EOS + Johnson-Cook: the plain stress kernel
  // queues the plastic steps and k_learn_queue runs the network over them
  // (KMPM_SUR_FUSED=1: the fused k_g2p2_learn instead)
  float *d_lq_f = nullptr;
  int *d_lq_i = nullptr, *d_lq_count = nullptr;
  long long lq_cap = 0;
  int nsm = 0;
  int law = 0;           // the law set every material shares (LAW_*): the specialised stress kernels
  bool law_jc = false;  // every material is linear EOS + Johnson-Cook
  // plastic strain or damage was uploaded (a restart): those rows may be
  // non-zero whatever the laws, and are permuted with the others
  bool restored_state = false;
  bool tuned = false;
  long long runs = 0;
  std::string tuning = "{}";
  // device buffer of kmpm_download_particles (one field of one solid, FP64)
  double *d_dump = nullptr;
  size_t dump_cap = 0;
  // asynchronous downloads: gathers on the step stream, copies on cst, one
  // device buffer per download in flight (reused once its copy has ended)
  cudaStream_t cst = nullptr;
  struct AsyncBuf {
    double *buf = nullptr;
    size_t cap = 0;
    cudaEvent_t gathered = nullptr, copied = nullptr;
    bool busy = false;
    const double *dst = nullptr;  // the caller's buffer of the last copy
  };
  std::vector<AsyncBuf> abufs;
  bool fuse_remap = false;  // MUSL gather + re-map in one kernel (k_g2p1_remap_row)
  bool indep() const { return prm.independent != 0; }
  // affine transfers: APIC, and for ULMPM also AFLIP / ASFLIP / MLS
  // (src/ulmpm.cpp:79-85; TLMPM takes the affine path for APIC only, src/tlmpm.cpp:354)
  bool apic() const {
    return prm.transfer == KMPM_TRANSFER_APIC ||
           (prm.method == KMPM_ULMPM && prm.transfer >= KMPM_TRANSFER_AFLIP && prm.transfer <= KMPM_TRANSFER_MLS);
  }
  int smem_apic[3] = {0, 0, 0};  // dynamic shared memory of the APIC scatters (TL, UL, VEL)
  bool TL() const { return prm.method == KMPM_TLMPM; }
  bool musl() const { return prm.scheme == KMPM_MUSL; }
  bool usf() const { return prm.scheme == KMPM_USF; }
};

namespace {

int fail(kmpm_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                                \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return fail(c, KMPM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T> int dalloc(kmpm_ctx *c, T **p, size_t n) {
  CK(cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(n, 1)));
  CK(cudaMemsetAsync(*p, 0, sizeof(T) * std::max<size_t>(n, 1), c->st));
  return KMPM_OK;
}
#define DALLOC(p, n)                      \
  do {                                    \
    int r_ = dalloc(c, &(p), (n));        \
    if (r_ != KMPM_OK) return r_;         \
  } while (0)

template <typename T> void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

MatDev to_dev(const kmpm_material &m) {
  MatDev d{};
  d.type = m.type;
  d.eos = m.eos;
  d.strength = m.strength;
  d.damage = m.damage;
  d.temp = m.temp;
  for (int i = 0; i < 12; i++) { d.eos_p[i] = m.eos_p[i]; d.str_p[i] = m.str_p[i]; }
  for (int i = 0; i < 8; i++) d.dam_p[i] = m.dam_p[i];
  for (int i = 0; i < 6; i++) d.temp_p[i] = m.temp_p[i];
  // Mat::Mat, src/material.cpp:720-769
  if (m.type == KMPM_MAT_EOS_STRENGTH) {
    d.rho0 = m.eos_p[0];
    d.K = m.eos_p[1];
    d.G = m.str_p[0];
    d.lambda = d.K - 2 * d.G / 3;
    d.signal_velocity = std::sqrt((d.lambda + 2 * d.G) / d.rho0);
    if (m.temp >= 0) {
      d.cp = m.temp_p[1];
      d.invcp = 1.0 / d.cp;
      d.kappa = m.temp_p[2];
    }
  } else {
    d.rho0 = m.rho0;
    d.G = m.E / (2 * (1 + m.nu));
    d.lambda = m.E * m.nu / ((1 + m.nu) * (1 - 2 * m.nu));
    d.K = m.E / (3 * (1 - 2 * m.nu));
    d.signal_velocity = std::sqrt(d.K / d.rho0);
    d.cp = m.cp;
    d.invcp = m.cp != 0 ? 1.0 / m.cp : 0;
    d.kappa = m.kappa;
  }
  d.f_rho0 = (float)d.rho0; d.f_K = (float)d.K; d.f_G = (float)d.G; d.f_lambda = (float)d.lambda;
  d.f_signal_velocity = (float)d.signal_velocity; d.f_cp = (float)d.cp; d.f_invcp = (float)d.invcp;
  d.f_kappa = (float)d.kappa;
  d.f_c2 = (float)(d.K + 1.333333333333333333333333333333333333333 * d.G);  // src/solid.cpp:40 FOUR_THIRD
  for (int i = 0; i < 12; i++) { d.f_eos_p[i] = (float)d.eos_p[i]; d.f_str_p[i] = (float)d.str_p[i]; }
  for (int i = 0; i < 8; i++) d.f_dam_p[i] = (float)d.dam_p[i];
  for (int i = 0; i < 6; i++) d.f_temp_p[i] = (float)d.temp_p[i];
  // FP32 path: (K + 4G/3) / rho0, so that the wave speed is sqrt(f_c2_rho0 J)
  // with no division per particle; Johnson-Cook: 1 / epsdot0 in the free
  // parameter slot 9 (the FP64 path keeps the reference's quotients)
  d.f_c2_rho0 = (float)((d.K + 1.333333333333333333333333333333333333333 * d.G) / d.rho0);
  if (d.type == KMPM_MAT_EOS_STRENGTH && d.strength == 2 && d.str_p[4] != 0.0) d.f_str_p[9] = (float)(1.0 / d.str_p[4]);
  return d;
}

PartArgs part_args(kmpm_ctx *c) {
  PartArgs a{};
  a.Pp = c->d_pp;
  a.ps = c->ps;
  a.ranges = c->d_ranges;
  a.blk_range = c->d_blk_range;
  a.solid_mat = c->d_solid_mat;
  a.grids = c->d_grids;
  a.mats = c->d_mats;
  a.nodeA = c->nodeA;
  a.nodeB = c->nodeB;
  a.nodeT = c->nodeT;
  a.scalars = c->d_scalars;
  a.err = c->d_err;
  a.blk_c = c->d_blk_c;
  a.blk_h = c->d_blk_h;
  a.pic_flip = (float)c->prm.pic_flip;
  a.T_ref = (float)c->T_ref;
  for (int d = 0; d < 3; d++) {
    a.boxlo[d] = (float)c->prm.boxlo[d];
    a.boxhi[d] = (float)c->prm.boxhi[d];
  }
  a.indep = c->indep();
  a.use_vu = c->musl() ? 0 : 1;
  a.thermal = c->prm.thermal;
  a.track_strain = c->prm.track_strain;
  a.apic = c->apic() ? 1 : 0;
  a.hr = c->exact_h ? nullptr : c->d_hr;
  a.asflip = (!c->TL() && c->prm.transfer == KMPM_TRANSFER_ASFLIP) ? 1 : 0;
  a.axisym = c->prm.axisymmetric;
  a.dim = c->prm.dim;
  a.gbox = c->TL() ? c->d_gbox : nullptr;
  for (int d = 0; d < 3; d++) a.tile_t[d] = c->tdim[d];
  a.lq_f = c->d_lq_f;
  a.lq_i = c->d_lq_i;
  a.lq_count = c->d_lq_count;
  a.lq_stats = c->d_lstats;
  a.lq_cap = c->lq_cap;
  return a;
}

P2GArgs p2g_args(kmpm_ctx *c) {
  P2GArgs a{};
  a.Pp = c->d_pp;
  a.ps = c->ps;
  a.pos_field = c->TL() ? PF_X0 : PF_X;
  a.tiles = c->d_tiles;
  a.grids = c->d_grids;
  a.cell_start = c->d_cs;
  a.cell_end = c->d_ce;
  a.partial = c->partial;
  a.pstride_tile = c->pstride_tile;
  a.tile_start = c->d_ts;
  a.tile_end = c->d_te;
  a.scalars = c->d_scalars;
  a.apic_pos = -1;
  a.mls = (!c->TL() && c->prm.transfer == KMPM_TRANSFER_MLS) ? 1 : 0;
  a.mbp = c->d_mbp;
  a.nodeA = c->nodeA;
  a.pic_flip = (float)c->prm.pic_flip;
  for (int d = 0; d < 3; d++) {
    a.boxlo[d] = (float)c->prm.boxlo[d];
    a.boxhi[d] = (float)c->prm.boxhi[d];
  }
  a.err = c->d_err;
  a.indep = c->indep();
  {
    const double cs = c->hgrids.empty() ? 1.0 : c->hgrids[0].cellsize;
    a.mls_di = (float)((c->prm.basis == KMPM_BASIS_QUADRATIC ? 4.0 : 3.0) / (cs * cs));
  }
  return a;
}

GridArgs grid_args(kmpm_ctx *c, int remap) {
  GridArgs a{};
  a.grids = c->d_grids;
  a.blk_grid = c->d_blk_grid;
  a.grid_blk0 = c->d_grid_blk0;
  a.partial = c->partial;
  a.pstride_tile = c->pstride_tile;
  a.tile_start = c->d_ts;
  a.tile_end = c->d_te;
  a.nodeA = c->nodeA;
  a.nodeB = c->nodeB;
  a.nodeX = c->nodeX;
  a.nodeT = c->nodeT;
  a.fixes = c->d_fixes;
  a.fix_start = c->d_fix_start;
  a.fix_count = c->d_fix_count;
  a.scalars = c->d_scalars;
  a.indep = c->indep();
  a.remap = remap;
  a.nodeP = c->fonly ? c->nodeP : nullptr;
  return a;
}

DtArgs dt_args(kmpm_ctx *c) {
  DtArgs a{};
  a.ranges = c->d_ranges;
  a.grids = c->d_grids;
  a.blk_c = c->d_blk_c;
  a.blk_h = c->d_blk_h;
  a.solid_dtcfl = c->d_dtcfl;
  a.scalars = c->d_scalars;
  a.err = c->d_err;
  a.nranges = (int)c->ranges.size();
  a.hr = c->exact_h ? nullptr : c->d_hr;
  a.hflags = c->d_hflags;
  a.nhflag = c->d_nhflag;
  a.Pp = c->d_pp;
  a.ps = c->ps;
  a.exact_blocks = c->exact_blocks;
  a.indep = c->indep();
  a.dt_constant = c->prm.dt_constant;
  a.dt_factor = c->prm.dt_factor;
  a.max_nblk = 0;
  for (const auto &r : c->ranges) a.max_nblk = std::max(a.max_nblk, r.nblk);
  return a;
}

int launch(kmpm_ctx *c, void *fn, dim3 grid, dim3 block, size_t smem, void *arg) {
  void *args[] = {arg};
  CK(cudaLaunchKernel(fn, grid, block, args, smem, c->st));
  return KMPM_OK;
}
#define LAUNCH(fn, g, b, sm, arg)                               \
  do {                                                          \
    int r_ = launch(c, (fn), dim3(g), dim3(b), (sm), (void *)&(arg)); \
    if (r_ != KMPM_OK) return r_;                               \
    nl++;                                                       \
  } while (0)

// records a profiling event after the launches of one phase
int mark(kmpm_ctx *c, const char *name) {
  if (!c->profiling) return KMPM_OK;
  if ((int)c->prof_ev.size() <= c->prof_n) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    c->prof_ev.push_back(e);
  }
  if ((int)c->prof_names.size() <= c->prof_n) c->prof_names.push_back(name);
  else c->prof_names[c->prof_n] = name;
  CK(cudaEventRecord(c->prof_ev[c->prof_n], c->st));
  c->prof_n++;
  return KMPM_OK;
}
#define MARK(name)                  \
  do {                              \
    int r_ = mark(c, (name));       \
    if (r_ != KMPM_OK) return r_;   \
  } while (0)

// particle fields that live in the device buffer for this configuration
// (rows that stay zero for the whole run are left out: both buffers start
// zeroed, and the kernels only ever write zeros into them)
std::vector<int> active_fields(kmpm_ctx *c) {
  std::vector<int> f;
  auto add = [&](int base, int n) { for (int i = 0; i < n; i++) f.push_back(base + i); };
  bool plastic = false, damage = false;
  for (const auto &m : c->mats) {
    plastic = plastic || (m.type == KMPM_MAT_EOS_STRENGTH && m.strength >= 1 && m.strength <= 3);
    damage = damage || (m.type == KMPM_MAT_EOS_STRENGTH && m.damage >= 0);
  }
  add(PF_X0, 3); add(PF_X, 3); add(PF_V, 3); add(PF_MASS, 1); add(PF_VOL0, 1); add(PF_H, 9); add(PF_SIG, 6);
  if (plastic || c->learn_mode != MODE_PLAIN || c->restored_state) add(PF_EPSP, 2);
  if (damage || c->restored_state) add(PF_DMG, 2);
  add(PF_PK, c->TL() ? 9 : 6);  // ULMPM scatters vol sigma (6)
  add(PF_ORIG, 1); add(PF_SID, 1);
  bool thermal = c->prm.thermal;
  for (auto &m : c->mats) if (m.cp != 0) thermal = true;
  if (thermal) { add(PF_T, 2); add(PF_Q, 3); }
  if (c->prm.track_strain) add(PF_STRAIN, 6);
  if (!c->TL()) add(PF_XN, 3);
  if (c->apic()) add(PF_C, 9);
  return f;
}

// the fields ULMPM's re-binning permutes (destination << 8 | source): the
// moved displacement becomes the binned one
void set_ul_fields(kmpm_ctx *c) {
  c->ul_fields.clear();
  for (int f : active_fields(c)) {
    int src = (f >= PF_X && f < PF_X + 3) ? PF_XN + (f - PF_X) : f;
    c->ul_fields.push_back((f << 8) | src);
  }
}

// ---------------------------------------------------------------- build
int build(kmpm_ctx *c) {
  const int dim = c->prm.dim, basis = c->prm.basis;
  if (c->hsolids.empty()) return fail(c, KMPM_ERR_STATE, "no solid was added");
  get_step_kernels(dim, basis, c->K);
  // the plain 2-D and 3-D four-wide scatters by cell rows (KMPM_CELL_SCATTER=1: cell by cell)
  if (c->K.p2g_row[0]) {
    const char *ev = std::getenv("KMPM_CELL_SCATTER");
    if (!(ev && ev[0] == '1')) {
      c->K.p2g_tl = c->K.p2g_row[0];
      c->K.p2g_ul = c->K.p2g_row[1];
      c->K.p2g_vel = c->K.p2g_row[2];
    }
  }
  // MUSL with FLIP/PIC transfers on mechanical 3-D runs: the gather and the
  // re-map scatter in one pass (KMPM_SPLIT_MUSL=1 or KMPM_CELL_SCATTER=1:
  // the two kernels)
  {
    const char *es = std::getenv("KMPM_SPLIT_MUSL"), *ec = std::getenv("KMPM_CELL_SCATTER");
    c->fuse_remap = c->K.g2p1_remap[0] && c->musl() && !c->prm.thermal && !c->apic() && !(es && es[0] == '1') &&
                    !(ec && ec[0] == '1');
  }
  // the specialised stress kernels: every material of one law set (linear
  // EOS + Johnson-Cook; shock EOS + Johnson-Cook + Johnson-Cook damage; fluid
  // EOS + fluid strength), no temperature law
  {
    const auto kind = [](const MatDev &m) {
      if (m.type != KMPM_MAT_EOS_STRENGTH || m.temp >= 0 || m.cp != 0.0) return (int)LAW_ANY;
      if (m.eos == 0 && m.strength == 2 && m.damage < 0) return (int)LAW_EOS_LINEAR_JC;
      if (m.eos == 1 && m.strength == 2 && m.damage >= 0) return (int)LAW_EOS_SHOCK_JC_DMG;
      if (m.eos == 2 && m.strength == 4 && m.damage < 0) return (int)LAW_FLUID;
      return (int)LAW_ANY;
    };
    c->law = (c->prm.thermal || c->mats.empty()) ? (int)LAW_ANY : kind(c->mats[0]);
    for (const auto &m : c->mats)
      if (kind(m) != c->law) c->law = LAW_ANY;
    c->law_jc = c->law == LAW_EOS_LINEAR_JC;
  }
  tile_dims(dim, basis, c->tdim);
  c->NCELL = c->tdim[0] * c->tdim[1] * c->tdim[2];
  // ---- grids
  c->grids.clear();
  int node_off = 0, tile_off = 0;
  std::vector<int> blk_grid, grid_blk0;
  for (size_t gi = 0; gi < c->hgrids.size(); gi++) {
    const auto &h = c->hgrids[gi];
    GridDev g{};
    for (int d = 0; d < 3; d++) {
      g.n[d] = h.n[d];
      g.ng[d] = h.ng[d];
      g.lo[d] = (float)h.lo[d];
      int nc = basis == KMPM_BASIS_BERNSTEIN ? (h.n[d] + 1) / 2 : h.n[d];
      if (d >= dim) nc = 1;
      g.ncell[d] = std::max(nc, 1);
      g.ntile[d] = d < dim ? (g.ncell[d] + c->tdim[d] - 1) / c->tdim[d] : 1;
    }
    g.cellsize = (float)h.cellsize;
    g.inv_cellsize = (float)(1.0 / h.cellsize);
    g.apic_di = 0.f;
    g.node_off = node_off;
    g.tile_off = tile_off;
    g.cell_off = tile_off * c->NCELL;
    g.solid0 = 0;
    const int nn = h.n[0] * h.n[1] * h.n[2];
    const int nb = (nn + 255) / 256;
    grid_blk0.push_back((int)blk_grid.size());
    for (int b = 0; b < nb; b++) blk_grid.push_back((int)gi);
    node_off += nb * 256;
    tile_off += g.ntile[0] * g.ntile[1] * g.ntile[2];
    c->grids.push_back(g);
  }
  c->nnodes_pad = node_off;
  c->nblk_g = (int)blk_grid.size();
  c->ntiles_total = tile_off;
  if ((long long)c->ntiles_total * c->NCELL > (1LL << 30))
    return fail(c, KMPM_ERR_ARG, "grid too large for the cell binning");
  c->key_bits = 1;
  while ((1LL << c->key_bits) < (long long)c->ntiles_total * c->NCELL) c->key_bits++;
  // ---- particle ranges
  c->ranges.clear();
  c->solid_range.assign(c->hsolids.size(), 0);
  c->solid_base.assign(c->hsolids.size(), 0);
  int base = 0;
  for (size_t s = 0; s < c->hsolids.size(); s++) { c->solid_base[s] = base; base += c->hsolids[s].n; }
  std::vector<int> blk_range;
  int pstart = 0;
  auto add_range = [&](int grid, int mat, int count) {
    RangeDev r{};
    r.start = pstart;
    r.count = count;
    r.grid = grid;
    r.mat = mat;
    r.blk0 = (int)blk_range.size();
    r.nblk = std::max(1, (count + 255) / 256);
    for (int b = 0; b < r.nblk; b++) blk_range.push_back((int)c->ranges.size());
    pstart += r.nblk * 256;
    c->ranges.push_back(r);
  };
  if (c->TL()) {
    for (size_t s = 0; s < c->hsolids.size(); s++) {
      c->solid_range[s] = (int)c->ranges.size();
      add_range(c->hsolids[s].grid, c->hsolids[s].mat, c->hsolids[s].n);
    }
  } else {
    int mat = c->hsolids[0].mat;
    for (auto &s : c->hsolids) if (s.mat != mat) mat = -1;
    add_range(0, mat, base);
  }
  c->ps = pstart;
  c->nblk_p = (int)blk_range.size();
  if (c->TL())  // per-grid clock of independent solids: the range of the solid owning the grid
    for (size_t s = 0; s < c->hsolids.size(); s++) c->grids[c->hsolids[s].grid].solid0 = c->solid_range[s];
  if (c->apic() && basis == KMPM_BASIS_LINEAR) {
    // Solid::compute_inertia_tensor (src/solid.cpp:1447-1462): Di = 16/4 (one
    // particle per cell per direction) or 16/3 (two) over cellsize^2
    for (size_t s = 0; s < c->hsolids.size(); s++) {
      const int npc = c->hsolids[s].np_per_cell;
      if (npc != 1 && npc != 2)
        return fail(c, KMPM_ERR_ARG,
                    "Number of particle per cell not supported with linear shape functions and APIC "
                    "(kmpm_set_np_per_cell: 1 or 2)");
      const double cs = c->hgrids[c->hsolids[s].grid].cellsize;
      c->grids[c->hsolids[s].grid].apic_di = (float)((npc == 1 ? 16.0 / 4.0 : 16.0 / 3.0) / (cs * cs));
    }
  }
  // ---- device allocations
  DALLOC(c->buf[0], c->ps * PF_COUNT);
  DALLOC(c->buf[1], c->ps * PF_COUNT);
  DALLOC(c->d_pp, 2);
  {
    float *pp[2] = {c->buf[0], c->buf[1]};
    CK(cudaMemcpyAsync(c->d_pp, pp, sizeof(pp), cudaMemcpyHostToDevice, c->st));
  }
  DALLOC(c->d_ranges, c->ranges.size());
  CK(cudaMemcpyAsync(c->d_ranges, c->ranges.data(), sizeof(RangeDev) * c->ranges.size(), cudaMemcpyHostToDevice, c->st));
  DALLOC(c->d_blk_range, blk_range.size());
  CK(cudaMemcpyAsync(c->d_blk_range, blk_range.data(), sizeof(int) * blk_range.size(), cudaMemcpyHostToDevice, c->st));
  std::vector<int> smat(c->hsolids.size());
  for (size_t s = 0; s < c->hsolids.size(); s++) smat[s] = c->hsolids[s].mat;
  DALLOC(c->d_solid_mat, smat.size());
  CK(cudaMemcpyAsync(c->d_solid_mat, smat.data(), sizeof(int) * smat.size(), cudaMemcpyHostToDevice, c->st));
  DALLOC(c->d_grids, c->grids.size());
  CK(cudaMemcpyAsync(c->d_grids, c->grids.data(), sizeof(GridDev) * c->grids.size(), cudaMemcpyHostToDevice, c->st));
  DALLOC(c->d_blk_grid, blk_grid.size());
  CK(cudaMemcpyAsync(c->d_blk_grid, blk_grid.data(), sizeof(int) * blk_grid.size(), cudaMemcpyHostToDevice, c->st));
  DALLOC(c->d_grid_blk0, grid_blk0.size());
  CK(cudaMemcpyAsync(c->d_grid_blk0, grid_blk0.data(), sizeof(int) * grid_blk0.size(), cudaMemcpyHostToDevice, c->st));
  DALLOC(c->d_mats, c->mats.size());
  CK(cudaMemcpyAsync(c->d_mats, c->mats.data(), sizeof(MatDev) * c->mats.size(), cudaMemcpyHostToDevice, c->st));
  // v and v_update interleaved: nodeB is the odd float4s of the same array
  DALLOC(c->nodeA, (size_t)NODE_STRIDE * c->nnodes_pad);
  c->nodeB = c->nodeA + 1;
  DALLOC(c->nodeX, c->nnodes_pad);
  DALLOC(c->nodeT, c->nnodes_pad);
  if (c->TL() && c->musl()) DALLOC(c->nodeP, c->nnodes_pad);
  {
    std::vector<float4> X(c->nnodes_pad, make_float4(0, 0, 0, 0));
    for (size_t gi = 0; gi < c->hgrids.size(); gi++) {
      const auto &h = c->hgrids[gi];
      const double hh = basis == KMPM_BASIS_BERNSTEIN ? h.cellsize / 2 : h.cellsize;
      int l = 0;
      for (int i = 0; i < h.n[0]; i++)
        for (int j = 0; j < h.n[1]; j++)
          for (int k = 0; k < h.n[2]; k++, l++)
            X[c->grids[gi].node_off + l] = make_float4((float)(h.lo[0] + i * hh), dim >= 2 ? (float)(h.lo[1] + j * hh) : 0.f,
                                                       dim == 3 ? (float)(h.lo[2] + k * hh) : 0.f, 0.f);
    }
    CK(cudaMemcpyAsync(c->nodeX, X.data(), sizeof(float4) * X.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  const int ncells = c->ntiles_total * c->NCELL;
  // padded to whole chunks of the re-binning's cell kernels, with one cell
  // past the end (the total of the movers' prefix)
  c->ncell_pad = (ncells + RB_CHUNK) / RB_CHUNK * RB_CHUNK;
  DALLOC(c->d_cs, c->ncell_pad);
  DALLOC(c->d_ce, c->ncell_pad);
  DALLOC(c->d_ts, c->ntiles_total);
  DALLOC(c->d_te, c->ntiles_total);
  {
    int S = stencil_width(basis), SC = stencil_sc(basis);
    int NW = 1;
    for (int d = 0; d < dim; d++) NW *= (c->tdim[d] - 1) * SC + S;
    c->pstride_tile = (size_t)NW * 10;
  }
  DALLOC(c->partial, c->pstride_tile * c->ntiles_total);
  c->nscalars = c->indep() ? (int)c->ranges.size() : 1;
  DALLOC(c->d_scalars, c->nscalars);
  {
    StepScalars s0{};
    s0.dt = c->prm.dt;
    s0.time = 0;
    s0.ntimestep = 0;
    s0.dtCFL = 1e22;
    s0.maxtime = 1e300;
    std::vector<StepScalars> sv(c->nscalars, s0);
    CK(cudaMemcpyAsync(c->d_scalars, sv.data(), sizeof(StepScalars) * sv.size(), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  DALLOC(c->d_dtcfl, c->ranges.size());
  if (const char *ev = std::getenv("KMPM_EXACT_H"); ev && ev[0] == '1') c->exact_h = true;
  // one clock only: independent instances (each its own minimum over a
  // uniformly loaded solid) leave few particles to skip
  if (c->TL() && !c->indep()) {  // bounds 0: the first step takes the exact pass
    DALLOC(c->d_hr, c->ranges.size());
    DALLOC(c->d_hflags, c->ranges.size());
    DALLOC(c->d_nhflag, 1);
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    c->exact_blocks = 4 * nsm;
  }
  DALLOC(c->d_err, 1);
  CK(cudaHostAlloc((void **)&c->h_err, sizeof(ErrState), cudaHostAllocMapped));
  CK(cudaHostGetDevicePointer((void **)&c->h_err_dev, c->h_err, 0));
  std::memset((void *)c->h_err, 0, sizeof(ErrState));
  c->maxtime_dev = 1e300;
  DALLOC(c->d_blk_c, c->nblk_p);
  DALLOC(c->d_blk_h, c->nblk_p);
  DALLOC(c->d_eblk, 2 * c->nblk_p);
  DALLOC(c->d_eout, 2);
  DALLOC(c->d_keys, c->ps);
  DALLOC(c->d_vals, c->ps);
  DALLOC(c->rtmp.k1, c->ps);
  DALLOC(c->rtmp.v1, c->ps);
  DALLOC(c->rtmp.hist, 256 * ((c->ps + 2047) / 2048 + 1));
  DALLOC(c->rtmp.tot, 256);
  if (!c->TL()) {
    if (const char *ev = std::getenv("KMPM_FULL_REBIN"); ev && ev[0] == '1') c->full_rebin = true;
    const int n = c->ranges[0].count, nblk = (n + 255) / 256;
    DALLOC(c->d_knew, n);
    DALLOC(c->d_mflag, (size_t)nblk * 8);
    DALLOC(c->d_cin, c->ncell_pad);
    DALLOC(c->d_cout, c->ncell_pad);
    DALLOC(c->d_mpre, c->ncell_pad);
    // the single-block scans read whole 4096-int tiles
    DALLOC(c->d_bsum, (2 * (c->ncell_pad / RB_CHUNK) + 4095) / 4096 * 4096);
    DALLOC(c->d_blkm, (nblk + 4095) / 4096 * 4096);
    DALLOC(c->d_brun, n);
    DALLOC(c->d_bsort, n);
    // the binning the first step updates: every slot in cell 0 (keys are
    // zero), which the ranges say
    const int cs0 = c->ranges[0].start, ce0 = c->ranges[0].start + n;
    CK(cudaMemcpy(c->d_cs, &cs0, sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_ce, &ce0, sizeof(int), cudaMemcpyHostToDevice));
  }
  // ---- particle upload: each solid's caller arrays (already on the device,
  // kmpm_add_solid) converted into its slots; the other fields are zero
  c->T_ref = c->prm.thermal ? c->hsolids[0].T0 : 0.0;
  for (size_t s = 0; s < c->hsolids.size(); s++) {
    auto &S = c->hsolids[s];
    const RangeDev &r = c->ranges[c->TL() ? c->solid_range[s] : 0];
    StageArgs sa{};
    sa.in = S.d_in;
    sa.n = S.n;
    sa.slot0 = c->TL() ? r.start : r.start + c->solid_base[s];
    sa.orig0 = c->solid_base[s];
    sa.sid = (int)s;
    sa.ul = c->TL() ? 0 : 1;
    // Solid::populate sets T = T0 only for thermo-mechanical runs (src/solid.cpp:2297-2306)
    sa.thermal = c->prm.thermal;
    sa.T = (float)(S.T0 - c->T_ref);
    sa.ps = c->ps;
    sa.P = c->buf[0];
    launch_stage_solid(sa, c->st);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  for (auto &S : c->hsolids) dfree(S.d_in);
  // ---- kernel attributes
  const int modes[4] = {P2G_MASS, P2G_TL, P2G_UL, P2G_VEL};
  void *fns[4][2] = {{c->K.p2g_mass, c->K.p2g_mass}, {c->K.p2g_tl, c->K.p2g_tl_th}, {c->K.p2g_ul, c->K.p2g_ul_th},
                     {c->K.p2g_vel, c->K.p2g_vel_th}};
  for (int m = 0; m < 4; m++)
    for (int t = 0; t < 2; t++) {
      c->smem[m][t] = p2g_smem_bytes(dim, basis, modes[m], t == 1);
      CK(cudaFuncSetAttribute(fns[m][t], cudaFuncAttributeMaxDynamicSharedMemorySize, c->smem[m][t]));
    }
  if (c->fuse_remap)
    CK(cudaFuncSetAttribute(c->K.g2p1_remap[c->TL() ? 1 : 0], cudaFuncAttributeMaxDynamicSharedMemorySize,
                            c->K.g2p1_remap_smem));
  if (c->apic()) {
    const int am[3] = {P2G_TL_APIC, P2G_UL_APIC, P2G_VEL_APIC};
    void *af[3] = {c->K.p2g_tl_apic, c->K.p2g_ul_apic, c->K.p2g_vel_apic};
    for (int m = 0; m < 3; m++) {
      if (!af[m]) continue;  // linear basis: TLMPM modes only
      c->smem_apic[m] = p2g_smem_bytes(dim, basis, am[m], false);
      CK(cudaFuncSetAttribute(af[m], cudaFuncAttributeMaxDynamicSharedMemorySize, c->smem_apic[m]));
    }
  }
  set_ul_fields(c);
  // ---- TLMPM: bin once by x0 (static connectivity, src/tlmpm.cpp:339) and compute the nodal mass
  if (c->TL()) {
    PartArgs pa = part_args(c);
    // grids in range order keep the keys of range r below those of range r+1
    bool ordered = true;
    for (size_t r = 1; r < c->ranges.size(); r++) ordered = ordered && c->ranges[r].grid > c->ranges[r - 1].grid;
    if (const char *ev = std::getenv("KMPM_SORT_PER_RANGE"); ev && ev[0] == '1') ordered = false;
    std::vector<int2> tiles;
    if (ordered) {
      // one stable LSD radix sort of every slot on the device: the same
      // permutation as a stable sort of each range by cell key (padding
      // slots carry their grid's last key and stay at the end of their range)
      launch_cell_keys(pa, c->nblk_p, c->d_keys, 1, c->st, 1);
      launch_iota(c->d_vals, (int)c->ps, c->st);
      radix_sort(c->d_keys, c->d_vals, (int)c->ps, c->key_bits, c->rtmp, c->st);
      std::vector<int> fl;
      for (int f : active_fields(c)) fl.push_back((f << 8) | f);
      launch_permute(c->d_pp, c->d_pp + 1, c->ps, c->d_vals, 0, (int)c->ps, fl.data(), (int)fl.size(), c->st);
    } else {
      // grids out of range order: sort range by range
      launch_cell_keys(pa, c->nblk_p, c->d_keys, 1, c->st, 0);
      std::vector<int> fl;
      for (int f : active_fields(c)) fl.push_back((f << 8) | f);
      for (auto &r : c->ranges) {
        launch_iota(c->d_vals + r.start, r.count, c->st);
        radix_sort(c->d_keys + r.start, c->d_vals + r.start, r.count, c->key_bits, c->rtmp, c->st);
        launch_permute(c->d_pp, c->d_pp + 1, c->ps, c->d_vals + r.start, r.start, r.count, fl.data(), (int)fl.size(),
                       c->st);
      }
    }
    launch_swap_ptrs(c->d_pp, c->st);
    std::swap(c->buf[0], c->buf[1]);
    for (auto &r : c->ranges)
      launch_cell_ranges(c->d_keys + r.start, r.start, r.count, c->NCELL, c->d_cs, c->d_ce, c->d_ts, c->d_te, c->st);
    CK(cudaGetLastError());
    // the non-empty tiles, in grid then tile order
    {
      std::vector<int> ts(c->ntiles_total), te(c->ntiles_total);
      CK(cudaMemcpyAsync(ts.data(), c->d_ts, sizeof(int) * ts.size(), cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(te.data(), c->d_te, sizeof(int) * te.size(), cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      for (auto &r : c->ranges) {
        const GridDev &g = c->grids[r.grid];
        const int nt = g.ntile[0] * g.ntile[1] * g.ntile[2];
        for (int t = 0; t < nt; t++)
          if (te[g.tile_off + t] > ts[g.tile_off + t]) tiles.push_back(make_int2(r.grid, t));
      }
      // launch order: the fullest tiles first, so that the partly filled
      // tiles at the solids' surfaces fill the last wave of blocks (each tile
      // writes its own slice: the order changes no result).  The sort is
      // stable, so tiles of equal count, the full ones among them, keep their
      // grid order and their shared halo nodes stay in L2 between neighbours
      auto count = [&](int2 t) { const int tg = c->grids[t.x].tile_off + t.y; return te[tg] - ts[tg]; };
      std::stable_sort(tiles.begin(), tiles.end(), [&](int2 a, int2 b) { return count(a) > count(b); });
    }
    c->ntiles_launch = (int)tiles.size();
    DALLOC(c->d_tiles, tiles.size());
    CK(cudaMemcpyAsync(c->d_tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice, c->st));
    if (const char *ev = std::getenv("KMPM_CHECK_BINS"); ev && ev[0] == '1') {
      // self-check of the binning (setup only): sorted keys and the device cell
      // ranges against ranges recomputed on the host
      const size_t ncell = (size_t)c->ntiles_total * c->NCELL;
      std::vector<int> cs(ncell), ce(ncell), ts(c->ntiles_total), te(c->ntiles_total), dk(c->ps);
      CK(cudaMemcpyAsync(cs.data(), c->d_cs, sizeof(int) * ncell, cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(ce.data(), c->d_ce, sizeof(int) * ncell, cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(ts.data(), c->d_ts, sizeof(int) * ts.size(), cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(te.data(), c->d_te, sizeof(int) * te.size(), cudaMemcpyDeviceToHost, c->st));
      CK(cudaMemcpyAsync(dk.data(), c->d_keys, sizeof(int) * c->ps, cudaMemcpyDeviceToHost, c->st));
      CK(cudaStreamSynchronize(c->st));
      long long key_mismatch = 0, bad_cells = 0, total = 0, maxc = 0, bad_tiles = 0;
      std::vector<int> hs(ncell, 0), he(ncell, 0);
      for (auto &r : c->ranges)
        for (int i = 0; i < r.count; i++) {
          const int k = dk[r.start + i];
          if (i > 0 && dk[r.start + i - 1] > k) key_mismatch++;  // unsorted within a range
          if (i == 0 || dk[r.start + i - 1] != k) hs[k] = r.start + i;
          he[k] = r.start + i + 1;
        }
      size_t first_bad = ncell;
      for (size_t k = 0; k < ncell; k++) {
        const long long n = (long long)ce[k] - cs[k];
        total += n > 0 ? n : 0;
        maxc = std::max(maxc, n);
        if (cs[k] != hs[k] || ce[k] != he[k]) { bad_cells++; if (first_bad == ncell) first_bad = k; }
      }
      for (auto t : tiles) {
        const int tg = c->grids[t.x].tile_off + t.y;
        if (te[tg] <= ts[tg]) bad_tiles++;
      }
      std::fprintf(stderr,
                   "[kmpm bins] ps %zu cells %zu tiles %d launched %d particles-in-cells %lld max/cell %lld "
                   "unsorted %lld bad-cells %lld bad-tiles %lld",
                   c->ps, ncell, c->ntiles_total, c->ntiles_launch, total, maxc, key_mismatch, bad_cells, bad_tiles);
      if (first_bad < ncell)
        std::fprintf(stderr, " first bad cell %zu: dev [%d,%d) host [%d,%d)", first_bad, cs[first_bad], ce[first_bad],
                     hs[first_bad], he[first_bad]);
      std::fprintf(stderr, "\n");
    }
    // nodal mass, once (TLMPM::particles_to_grid, src/tlmpm.cpp:344-351)
    P2GArgs p = p2g_args(c);
    int nl = 0;
    LAUNCH(c->K.p2g_mass, c->ntiles_launch, 256, c->smem[0][0], p);
    GridArgs ga = grid_args(c, 0);
    LAUNCH(c->K.grid_mass[c->prm.precision == KMPM_PREC_FP64_ISLANDS ? 1 : 0], c->nblk_g, 256, 0, ga);
    // the stress kernel's node box of every block, fixed by x0 from here on
    if (const char *ev = std::getenv("KMPM_BOX_PER_LAUNCH"); dim == 3 && !(ev && ev[0] == '1')) {
      DALLOC(c->d_gbox, 2 * (size_t)c->nblk_p);
      PartArgs pb = part_args(c);
      pb.gbox = nullptr;
      int4 *box = c->d_gbox;
      void *args[] = {&pb, &box};
      CK(cudaLaunchKernel(c->K.gather_box, dim3(c->nblk_p), dim3(256), args, 0, c->st));
    }
    CK(cudaStreamSynchronize(c->st));
  } else {
    // ULMPM: every tile of the box grid is launched; empty ones return at once
    std::vector<int2> tiles;
    for (size_t gi = 0; gi < c->grids.size(); gi++) {
      const GridDev &g = c->grids[gi];
      for (int t = 0; t < g.ntile[0] * g.ntile[1] * g.ntile[2]; t++) tiles.push_back(make_int2((int)gi, t));
    }
    c->ntiles_launch = (int)tiles.size();
    DALLOC(c->d_tiles, tiles.size());
    CK(cudaMemcpyAsync(c->d_tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice, c->st));
  }
  c->built = true;
  return KMPM_OK;
}

int upload_fixes(kmpm_ctx *c) {
  for (auto *m : c->d_masks) cudaFree(m);
  c->d_masks.clear();
  dfree(c->d_fixes);
  dfree(c->d_fix_start);
  dfree(c->d_fix_count);
  std::vector<FixDev> fx;
  std::vector<int> start(c->hgrids.size(), 0), count(c->hgrids.size(), 0);
  for (size_t gi = 0; gi < c->hgrids.size(); gi++) {
    start[gi] = (int)fx.size();
    for (auto &h : c->hfixes) {
      if (h.grid != (int)gi) continue;
      FixDev f{};
      f.kind = h.kind;
      f.grid = h.grid;
      for (int d = 0; d < 3; d++) {
        f.set[d] = h.set[d];
        for (int k = 0; k < 4; k++) f.c[d][k] = h.c[4 * d + k];
      }
      uint8_t *m = nullptr;
      CK(cudaMalloc(&m, h.mask.size()));
      CK(cudaMemcpyAsync(m, h.mask.data(), h.mask.size(), cudaMemcpyHostToDevice, c->st));
      CK(cudaStreamSynchronize(c->st));
      c->d_masks.push_back(m);
      f.mask = m;
      fx.push_back(f);
    }
    count[gi] = (int)fx.size() - start[gi];
  }
  DALLOC(c->d_fixes, fx.size());
  c->nfix_dev = (int)fx.size();
  if (!fx.empty())
    CK(cudaMemcpyAsync(c->d_fixes, fx.data(), sizeof(FixDev) * fx.size(), cudaMemcpyHostToDevice, c->st));
  DALLOC(c->d_fix_start, start.size());
  DALLOC(c->d_fix_count, count.size());
  CK(cudaMemcpyAsync(c->d_fix_start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaMemcpyAsync(c->d_fix_count, count.data(), sizeof(int) * count.size(), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->fixes_dirty = false;
  c->graph_valid = false;
  return KMPM_OK;
}

void free_contacts(kmpm_ctx *c) {
  for (auto &d : c->contacts) {
    dfree(d.keys); dfree(d.vals); dfree(d.bstart); dfree(d.bend);
    dfree(d.ra); dfree(d.rb); dfree(d.rc); dfree(d.blk); dfree(d.ftot);
  }
  c->contacts.clear();
  dfree(c->d_mbp);
}

// device state of the contact fixes: member lists, hash buckets and the mbp rows
int setup_contacts(kmpm_ctx *c) {
  free_contacts(c);
  c->contacts_dirty = false;
  c->graph_valid = false;
  if (c->hcontacts.empty()) return KMPM_OK;
  const int dim = c->prm.dim;
  DALLOC(c->d_mbp, 3 * c->ps);
  CK(cudaMemsetAsync(c->d_mbp, 0, sizeof(float) * 3 * c->ps, c->st));
  for (const auto &h : c->hcontacts) {
    ContactDev d{};
    d.kind = h.kind;
    d.dim = dim;
    d.thermal = c->prm.thermal;
    d.ul = c->TL() ? 0 : 1;
    d.sid1 = h.s1;
    d.sid2 = h.s2;
    if (c->TL()) {
      const RangeDev &r1 = c->ranges[c->solid_range[h.s1]], &r2 = c->ranges[c->solid_range[h.s2]];
      d.start1 = r1.start; d.n1 = r1.count;
      d.start2 = r2.start; d.n2 = r2.count;
      d.nmem = r1.count + r2.count;
    } else {
      const RangeDev &r = c->ranges[0];
      d.start1 = r.start; d.n1 = r.count;
      d.start2 = 0; d.n2 = 0;
      d.nmem = r.count;
    }
    d.nb = 1024;
    while (d.nb < d.nmem) d.nb <<= 1;
    d.key_bits = 1;
    while ((1 << d.key_bits) <= d.nb) d.key_bits++;  // bucket nb marks non-members
    const int m1 = c->hsolids[h.s1].mat, m2 = c->hsolids[h.s2].mat;
    const double E1 = c->mat_E[m1], E2 = c->mat_E[m2], nu1 = c->mat_nu[m1], nu2 = c->mat_nu[m2];
    d.estar = (float)(1.0 / ((1 - nu1 * nu1) / E1 + (1 - nu2 * nu2) / E2));
    d.alpha = (float)(c->mats[m1].kappa / (c->mats[m1].kappa + c->mats[m2].kappa));
    d.invcp1 = (float)c->mats[m1].invcp;
    d.invcp2 = (float)c->mats[m2].invcp;
    d.mu = (float)h.mu;
    // four_thirds = 1.333333333 in both reference fixes; 0.25 pi in 2-D Hertz
    d.hcoef = (float)(dim == 3 ? 1.333333333 : 0.25 * M_PI);
    const double cmax = std::max(c->hgrids[c->hsolids[h.s1].grid].cellsize, c->hgrids[c->hsolids[h.s2].grid].cellsize);
    d.cmax = (float)cmax;
    d.inv_cmax = (float)(1.0 / cmax);
    for (int k = 0; k < 3; k++) d.boxlo[k] = (float)c->prm.boxlo[k];
    const int nblk = (d.nmem + 255) / 256;
    DALLOC(d.keys, std::max(d.nmem, 1));
    DALLOC(d.vals, std::max(d.nmem, 1));
    DALLOC(d.bstart, d.nb);
    DALLOC(d.bend, d.nb);
    DALLOC(d.ra, std::max(d.nmem, 1));
    DALLOC(d.rb, std::max(d.nmem, 1));
    DALLOC(d.rc, std::max(d.nmem, 1));
    DALLOC(d.blk, 3 * std::max(nblk, 1));
    DALLOC(d.ftot, 3);
    CK(cudaMemsetAsync(d.ftot, 0, 3 * sizeof(double), c->st));
    d.mbp = c->d_mbp;
    d.axisym = c->prm.axisymmetric;
    c->contacts.push_back(d);
  }
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

// The scatter kernel of one force mode: the mode's base (TL / UL), affine
// transfers, external particle forces (contact fixes) and the axisymmetric
// hoop term select the instantiation.
void *force_scatter_fn(const kmpm_ctx *c, int mode, bool th) {
  const StepKernels &K = c->K;
  const bool ul = p2g_base(mode) == P2G_UL, ap = p2g_apic(mode), ex = p2g_ext(mode);
  if (p2g_axi(mode)) return th ? nullptr : K.p2g_axi[ul][ap][ex];
  if (ex) {
    if (ap) return th ? nullptr : (ul ? K.p2g_ul_apic_ext : K.p2g_tl_apic_ext);
    return ul ? K.p2g_ul_ext[th] : K.p2g_tl_ext[th];
  }
  if (ap) return th ? nullptr : (ul ? K.p2g_ul_apic : K.p2g_tl_apic);
  return ul ? (th ? K.p2g_ul_th : K.p2g_ul) : (th ? K.p2g_tl_th : K.p2g_tl);
}

// launch shape v of the FP32 mechanical stress kernel, specialised to the
// materials where that applies
// the learned return map through the queue (plain stress kernel + k_learn_queue)
bool sur_queued(const kmpm_ctx *c) {
  if (c->learn_mode != MODE_SUR || !c->law_jc || !c->K.g2p2_jcq[0] || !c->LK.queue) return false;
  const char *ev = std::getenv("KMPM_SUR_FUSED");
  return !(ev && ev[0] == '1');
}

// dynamic shared memory of a stress kernel: the linear EOS + Johnson-Cook
// variants also stage their particles' state rows (G2P2_JC_SMEM)
int g2p2_smem(const kmpm_ctx *c, const void *fn) {
  for (int t = 0; t < 2; t++)
    for (int v = 0; v < G2P_NVAR; v++)
      if (fn && fn == c->K.g2p2_jc[t][v]) return G2P2_JC_SMEM;
  return G2P2_SMEM;
}

void *g2p2_variant(const kmpm_ctx *c, int v) {
  const bool TL = c->TL();
  if (!c->apic()) {
    if (c->law == LAW_EOS_LINEAR_JC && c->K.g2p2_jc[TL][v]) return c->K.g2p2_jc[TL][v];
    if (c->law == LAW_EOS_SHOCK_JC_DMG && c->K.g2p2_jcd[TL][v]) return c->K.g2p2_jcd[TL][v];
    if (c->law == LAW_FLUID && c->K.g2p2_fl[TL][v]) return c->K.g2p2_fl[TL][v];
  }
  return c->K.g2p2_v[TL][v];
}

int select_scatters(kmpm_ctx *c) {
  const bool TL = c->TL(), th = c->prm.thermal != 0;
  const int flags = (!c->contacts.empty() && c->prm.dim >= 2 ? P2G_EXT : 0) | (c->prm.axisymmetric ? P2G_AXI : 0);
  const int base = TL ? P2G_TL : P2G_UL;
  const int mode = (c->apic() ? base + 3 : base) | flags;
  const int mode_usf = base | flags;
  c->sc_force = force_scatter_fn(c, mode, th);
  c->sc_usf = force_scatter_fn(c, mode_usf, false);
  if (!c->sc_force || !c->sc_usf) return fail(c, KMPM_ERR_ARG, "no scatter kernel for this combination");
  c->smem_force = p2g_smem_bytes(c->prm.dim, c->prm.basis, mode, th);
  c->smem_usf = p2g_smem_bytes(c->prm.dim, c->prm.basis, mode_usf, false);
  CK(cudaFuncSetAttribute(c->sc_force, cudaFuncAttributeMaxDynamicSharedMemorySize, c->smem_force));
  CK(cudaFuncSetAttribute(c->sc_usf, cudaFuncAttributeMaxDynamicSharedMemorySize, c->smem_usf));
  // TLMPM MUSL with FLIP/PIC on the plain row scatter, mechanical, FP32: the
  // force-only scatter, with the momentum of the last re-map where it is the
  // current state's (KMPM_NO_MOMENTUM_REUSE=1: a velocity scatter every step)
  {
    const char *ev = std::getenv("KMPM_NO_MOMENTUM_REUSE");
    c->fonly = TL && c->musl() && !th && flags == 0 && !c->apic() && c->nodeP &&
               c->prm.precision == KMPM_PREC_FP32 && c->K.p2g_row_fonly && c->sc_force == c->K.p2g_row[0];
    c->reuse_ok = c->fonly && !(ev && ev[0] == '1');
    c->p_valid = false;
    if (c->fonly) {
      c->smem_fonly = c->K.p2g_row_fonly_smem > 0 ? c->K.p2g_row_fonly_smem
                                                  : p2g_smem_bytes(c->prm.dim, c->prm.basis, P2G_TL | P2G_FONLY, false);
      CK(cudaFuncSetAttribute(c->K.p2g_row_fonly, cudaFuncAttributeMaxDynamicSharedMemorySize, c->smem_fonly));
    }
  }
  return KMPM_OK;
}

// ---------------------------------------------------------------- one step
// USL::run (src/usl.cpp:43-92) / MUSL::run (src/musl.cpp:43-93)
// reuse (fonly configurations): nodeP holds the last re-map's momentum, which
// is the current state's, so no velocity scatter runs before the force scatter
int enqueue_step(kmpm_ctx *c, bool reuse = false) {
  int nl = 0;
  const bool TL = c->TL(), th = c->prm.thermal != 0, musl = c->musl();
  const int prec = c->prm.precision == KMPM_PREC_FP64_ISLANDS ? 1 : 0;
  PartArgs pa = part_args(c);
  MARK("begin");
  launch_step_begin(c->d_scalars, c->nscalars, c->st);
  if (c->nfix_dev > 0) {
    launch_fix_values(c->d_fixes, c->nfix_dev, c->d_grids, c->d_scalars, c->indep(), c->st);
    nl++;
  }
  nl++;
  if (!TL) {
    // compute_grid_weight_functions_and_gradients (src/ulmpm.cpp:88-337):
    // re-bin all particles by the cell of their current position
    const RangeDev &r = c->ranges[0];
    if (c->full_rebin) {
      launch_cell_keys(pa, c->nblk_p, c->d_keys, 0, c->st);
      launch_iota(c->d_vals, r.count, c->st);
      radix_sort(c->d_keys, c->d_vals, r.count, c->key_bits, c->rtmp, c->st);
      CK(cudaMemsetAsync(c->d_cs, 0, sizeof(int) * (size_t)c->ncell_pad, c->st));
      CK(cudaMemsetAsync(c->d_ce, 0, sizeof(int) * (size_t)c->ncell_pad, c->st));
      CK(cudaMemsetAsync(c->d_ts, 0, sizeof(int) * c->ntiles_total, c->st));
      CK(cudaMemsetAsync(c->d_te, 0, sizeof(int) * c->ntiles_total, c->st));
      launch_cell_ranges(c->d_keys, r.start, r.count, c->NCELL, c->d_cs, c->d_ce, c->d_ts, c->d_te, c->st);
      nl += 3 + 3 * ((c->key_bits + 7) / 8);
    } else {
      RebinArgs rb{};
      rb.pa = pa;
      rb.grid = r.grid; rb.start = r.start; rb.n = r.count;
      rb.ncell = c->ntiles_total * c->NCELL; rb.ncell_pad = c->ncell_pad; rb.ncpt = c->NCELL;
      rb.keys = c->d_keys; rb.knew = c->d_knew; rb.mflag = c->d_mflag;
      rb.cin = c->d_cin; rb.cout = c->d_cout; rb.mpre = c->d_mpre; rb.bsum = c->d_bsum; rb.blkm = c->d_blkm;
      rb.brun = c->d_brun; rb.bsort = c->d_bsort;
      rb.cell_start = c->d_cs; rb.cell_end = c->d_ce; rb.tile_start = c->d_ts; rb.tile_end = c->d_te;
      rb.perm = c->d_vals;
      nl += launch_rebin(rb, c->st);
    }
    launch_permute(c->d_pp, c->d_pp + 1, c->ps, c->d_vals, r.start, r.count, c->ul_fields.data(),
                   (int)c->ul_fields.size(), c->st);
    launch_swap_ptrs(c->d_pp, c->st);
    nl += 2;
    MARK("bin_sort");
  }
  // reset() + initial_integrate: the contact fixes fill mbp from the current
  // positions (src/musl.cpp:48-49, src/usl.cpp:48-49, src/usf.cpp:48-49)
  const bool ext = !c->contacts.empty() && c->prm.dim >= 2;
  if (ext) {
    CK(cudaMemsetAsync(c->d_mbp, 0, sizeof(float) * 3 * c->ps, c->st));
    for (const auto &cd : c->contacts) nl += launch_contact(pa, cd, c->rtmp, c->st);
    MARK("contact");
  }
  P2GArgs p = p2g_args(c);
  GridArgs g1 = grid_args(c, 0);
  const bool apic = c->apic();
  // particles_to_grid (APIC: compute_velocity_nodes_APIC with x_p = x0 (TL) or x (UL))
  p.apic_pos = TL ? -1 : PF_X;
  // (with w mbp added to the node forces when contacts exist, and the hoop
  // term in axisymmetric runs: select_scatters)
  if (c->fonly) {
    if (!reuse) {
      // compute_velocity_nodes: the sums the re-map forms (the velocity row
      // scatter), kept in nodeP
      LAUNCH(c->K.p2g_vel, c->ntiles_launch, 256, c->smem[3][0], p);
      LAUNCH(c->K.grid_store_p, c->nblk_g, 256, 0, g1);
      MARK("p2g_momentum");
    }
    // compute_internal_forces_nodes_TL
    LAUNCH(c->K.p2g_row_fonly, c->ntiles_launch, 256, c->smem_fonly, p);
    MARK("p2g_force");
  } else {
    LAUNCH(c->sc_force, c->ntiles_launch, 256, c->smem_force, p);
    MARK("p2g");
  }
  // update_grid_state + fixes
  LAUNCH(c->fonly ? c->K.grid_upd_fonly : c->K.grid_upd[TL][th][prec], c->nblk_g, 256, 0, g1);
  MARK("grid_update");
  if (c->usf()) {
    // USF::run (src/usf.cpp:43-86): the stress from the grid velocities of the
    // first scatter (compute_rate_deformation_gradient(true)), then the
    // forces of the new stress, the grid update and the particle update
    PartArgs ps = pa;
    ps.use_vu = 0;
    void *fs = (th || prec) ? c->K.g2p2[TL][th][prec] : g2p2_variant(c, c->var_g2p2);
    LAUNCH(fs, c->nblk_p, 256, g2p2_smem(c, fs), ps);
    MARK("g2p_stress");
    LAUNCH(c->sc_usf, c->ntiles_launch, 256, c->smem_usf, p);
    MARK("p2g_forces");
    LAUNCH(c->K.grid_upd[TL][th][prec], c->nblk_g, 256, 0, g1);
    MARK("grid_update2");
    LAUNCH(c->K.g2p1_v[TL][c->var_g2p1], c->nblk_p, 256, G2P1_SMEM, pa);
    MARK("g2p_advance");
    if (TL) {
      GridArgs g2 = grid_args(c, 0);
      LAUNCH(c->K.grid_vel[TL][th][prec], c->nblk_g, 256, 0, g2);
      MARK("grid_positions");
    }
    DtArgs da = dt_args(c);
    launch_dt(da, c->st);
    nl += c->d_hr && !c->exact_h ? 3 : 2;
    MARK("dt");
    CK(cudaGetLastError());
    c->launches_per_step = nl;
    return KMPM_OK;
  }
  if (c->fuse_remap) {
    // grid_to_points + advance_particles + velocities_to_grid in one pass
    // over the tiles, then post_velocities_to_grid (+ TL grid positions)
    LAUNCH(c->K.g2p1_remap[TL], c->ntiles_launch, 256, c->K.g2p1_remap_smem, p);
    MARK("g2p_advance_remap");
    GridArgs g2 = grid_args(c, 1);
    LAUNCH(c->K.grid_vel[TL][th][prec], c->nblk_g, 256, 0, g2);
    MARK("grid_velocity");
  } else {
    // grid_to_points + advance_particles
    LAUNCH(th ? c->K.g2p1[TL][th] : c->K.g2p1_v[TL][c->var_g2p1], c->nblk_p, 256, G2P1_SMEM, pa);
    MARK("g2p_advance");
    if (musl) {
      // velocities_to_grid + post_velocities_to_grid (+ TL grid positions)
      // APIC re-map: ULMPM takes x_p after the move, with this step's weights
      P2GArgs pv = p;
      pv.apic_pos = TL ? -1 : PF_XN;
      if (apic) LAUNCH(c->K.p2g_vel_apic, c->ntiles_launch, 256, c->smem_apic[2], pv);
      else LAUNCH(th ? c->K.p2g_vel_th : c->K.p2g_vel, c->ntiles_launch, 256, c->smem[3][th], pv);
      MARK("p2g_velocity");
      GridArgs g2 = grid_args(c, 1);
      LAUNCH(c->K.grid_vel[TL][th][prec], c->nblk_g, 256, 0, g2);
      MARK("grid_velocity");
    } else if (TL) {
      GridArgs g2 = grid_args(c, 0);
      LAUNCH(c->K.grid_vel[TL][th][prec], c->nblk_g, 256, 0, g2);
      MARK("grid_positions");
    }
  }
  // compute_rate_deformation_gradient + update_deformation_gradient + update_stress
  if (c->learn_mode == MODE_PLAIN) {
    void *fs = (th || prec) ? c->K.g2p2[TL][th][prec] : g2p2_variant(c, c->var_g2p2);
    LAUNCH(fs, c->nblk_p, 256, g2p2_smem(c, fs), pa);
  } else {
    LearnArgs la{};
    la.blob = c->d_blob;
    la.tol = c->sur_tol;
    la.stats = c->d_lstats;
    la.log = c->d_log;
    la.log_count = c->d_log_count;
    la.log_cap = c->log_cap;
    la.log_seed = c->log_seed;
    la.log_thresh = c->log_thresh;
    la.nblk = c->nblk_p;
    void *args[] = {&pa, &la};
    if (sur_queued(c)) {
      CK(cudaMemsetAsync(c->d_lq_count, 0, sizeof(int), c->st));
      LAUNCH(c->K.g2p2_jcq[c->var_g2p2], c->nblk_p, 256, G2P2_SMEM, pa);
      CK(cudaLaunchKernel(c->LK.queue, dim3(c->nsm), dim3(512), args, c->LK.sur_smem, c->st));
    } else if (c->learn_mode == MODE_SUR) {
      CK(cudaLaunchKernel(c->LK.sur, dim3((c->nblk_p + 1) / 2), dim3(512), args, c->LK.sur_smem, c->st));
    } else {
      CK(cudaLaunchKernel(c->LK.log, dim3(c->nblk_p), dim3(256), args, 0, c->st));
    }
    nl++;
  }
  MARK("g2p_stress");
  // update_time + adjust_dt
  DtArgs da = dt_args(c);
  launch_dt(da, c->st);
  nl += c->d_hr && !c->exact_h ? 3 : 2;
  MARK("dt");
  CK(cudaGetLastError());
  c->launches_per_step = nl;
  return KMPM_OK;
}

int capture_step(kmpm_ctx *c, bool reuse, cudaGraphExec_t *out) {
  if (*out) { cudaGraphExecDestroy(*out); *out = nullptr; }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
  int r = enqueue_step(c, reuse);
  cudaError_t e = cudaStreamEndCapture(c->st, &g);
  if (r != KMPM_OK) return r;
  if (e != cudaSuccess) return fail(c, KMPM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  CK(cudaGraphInstantiate(out, g, 0));
  cudaGraphDestroy(g);
  return KMPM_OK;
}

int ensure_graph(kmpm_ctx *c) {
  if (c->graph_valid) return KMPM_OK;
  c->p_valid = false;
  int r = capture_step(c, false, &c->gexec);
  if (r == KMPM_OK && c->reuse_ok) r = capture_step(c, true, &c->gexec_r);
  if (r != KMPM_OK) return r;
  c->graph_valid = true;
  return KMPM_OK;
}

// n replays of the step graph: the momentum-reuse step wherever the last
// re-map's sums are those of the current particle state
int launch_steps(kmpm_ctx *c, int n) {
  for (int i = 0; i < n; i++) {
    CK(cudaGraphLaunch(c->reuse_ok && c->p_valid ? c->gexec_r : c->gexec, c->st));
    c->p_valid = c->reuse_ok;
  }
  return KMPM_OK;
}

int check_error(kmpm_ctx *c) {
  launch_publish_err(c->d_err, c->h_err_dev, c->st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  ErrState e;
  std::memcpy(&e, (const void *)c->h_err, sizeof(e));
  if (e.code == 0) return KMPM_OK;
  char buf[256];
  const char *what = e.code == ERR_J ? "J<=0" : e.code == ERR_LEFT ? "particle left the domain"
                     : e.code == ERR_NAN ? "max_p_wave_speed is nan" : e.code == ERR_POLDEC ? "polar decomposition failed"
                     : "dtCFL == 0 or nan";
  std::snprintf(buf, sizeof(buf), "Error: %s (particle slot %d, step %lld)", what, e.particle, e.step);
  const int code = e.code == ERR_J ? KMPM_ERR_J : e.code == ERR_LEFT ? KMPM_ERR_LEFT_DOMAIN
                   : e.code == ERR_NAN ? KMPM_ERR_NAN : e.code == ERR_POLDEC ? KMPM_ERR_POLDEC
                   : e.code == ERR_TIMEOUT ? KMPM_ERR_TIMEOUT : KMPM_ERR_DTCFL;
  return fail(c, code, buf);
}

int prepare(kmpm_ctx *c) {
  if (!c->built) {
    int r = build(c);
    if (r != KMPM_OK) return r;
  }
  if (c->fixes_dirty) {
    int r = upload_fixes(c);
    if (r != KMPM_OK) return r;
  }
  if (c->contacts_dirty) {
    int r = setup_contacts(c);
    if (r != KMPM_OK) return r;
  }
  if (!c->graph_valid) {
    int r = select_scatters(c);
    if (r != KMPM_OK) return r;
  }
  if (sur_queued(c) && !c->d_lq_f) {  // room for every particle: the queue cannot overflow
    c->lq_cap = (long long)c->ps;
    DALLOC(c->d_lq_f, (size_t)LQ_NF * c->lq_cap);
    DALLOC(c->d_lq_i, (size_t)LQ_NI * c->lq_cap);
    DALLOC(c->d_lq_count, 1);
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaStreamSynchronize(c->st));
  }
  return ensure_graph(c);
}

// ---------------------------------------------------------------- autotuner
// Launch shape of the two gathers: resident blocks per SM, i.e. the register
// budget of k_g2p1 / k_g2p2 (G2P1_MINB / G2P2_MINB).  Every candidate runs on
// a scratch copy of the live particle state (the spare buffer), interleaved,
// three timed launches each after one untimed; the fastest mean is kept for
// the rest of the run.  The live state and the dt partials of the next step
// are untouched.
int autotune(kmpm_ctx *c) {
  c->tuned = true;
  if (c->prm.thermal || c->prm.precision != KMPM_PREC_FP32) return KMPM_OK;  // candidates exist for FP32 mechanics
  const double big = 1e300;
  CK(cudaMemcpyAsync((char *)c->d_scalars + offsetof(StepScalars, maxtime), &big, sizeof(double),
                     cudaMemcpyHostToDevice, c->st));
  c->maxtime_dev = big;
  float *pp[2] = {nullptr, nullptr};
  CK(cudaMemcpyAsync(pp, c->d_pp, sizeof(pp), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaMemcpyAsync(pp[1], pp[0], sizeof(float) * c->ps * PF_COUNT, cudaMemcpyDeviceToDevice, c->st));
  launch_swap_ptrs(c->d_pp, c->st);  // the candidates read and write the copy
  const bool TL = c->TL();
  PartArgs pa = part_args(c);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  double t[2][G2P_NVAR] = {{0}};
  const int k0 = c->fuse_remap ? 1 : 0;  // no separate gather kernel to tune
  for (int rep = 0; rep < 4; rep++)
    for (int k = k0; k < 2; k++)
      for (int v = 0; v < G2P_NVAR; v++) {
        void *fn = k == 0 ? c->K.g2p1_v[TL][v] : g2p2_variant(c, v);
        CK(cudaEventRecord(e0, c->st));
        int r = launch(c, fn, dim3(c->nblk_p), dim3(256), k == 0 ? G2P1_SMEM : g2p2_smem(c, fn), &pa);
        if (r != KMPM_OK) return r;
        CK(cudaEventRecord(e1, c->st));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0) t[k][v] += ms / 3.0;
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  launch_swap_ptrs(c->d_pp, c->st);
  CK(cudaMemsetAsync(c->d_err, 0, sizeof(ErrState), c->st));
  CK(cudaStreamSynchronize(c->st));
  int best[2] = {0, 0};
  for (int k = 0; k < 2; k++)
    for (int v = 1; v < G2P_NVAR; v++)
      if (t[k][v] < t[k][best[k]]) best[k] = v;
  c->var_g2p1 = best[0];
  c->var_g2p2 = best[1];
  char buf[512];
  char adv[160];
  if (c->fuse_remap)
    std::snprintf(adv, sizeof(adv), "{\"fused_with_remap\": true}");
  else
    std::snprintf(adv, sizeof(adv), "{\"min_blocks\": [%d, %d, %d], \"ms\": [%.4f, %.4f, %.4f], \"chosen\": %d}",
                  G2P1_MINB[0], G2P1_MINB[1], G2P1_MINB[2], t[0][0], t[0][1], t[0][2], G2P1_MINB[best[0]]);
  std::snprintf(buf, sizeof(buf),
                "{\"g2p_advance\": %s, "
                "\"g2p_stress\": {\"min_blocks\": [%d, %d, %d], \"ms\": [%.4f, %.4f, %.4f], \"chosen\": %d}}",
                adv, G2P2_MINB[0], G2P2_MINB[1], G2P2_MINB[2], t[1][0], t[1][1], t[1][2], G2P2_MINB[best[1]]);
  c->tuning = buf;
  c->graph_valid = false;
  return KMPM_OK;
}

// tune once, at the first run after at least one step (a state with motion)
// Launch shapes already chosen in this process, by problem signature
// (method, dim, basis, law specialisation, particle count to a factor of 2):
// a later context of the same problem takes the choice without its trial
// launches.
struct TuneKey {
  int tl, dim, basis, law, transfer, log2n;
  bool operator<(const TuneKey &o) const {
    return std::tie(tl, dim, basis, law, transfer, log2n) <
           std::tie(o.tl, o.dim, o.basis, o.law, o.transfer, o.log2n);
  }
};
std::mutex g_tune_mutex;
std::map<TuneKey, std::pair<std::pair<int, int>, std::string>> g_tune_cache;

TuneKey tune_key(const kmpm_ctx *c) {
  long long n = 0;
  for (const auto &r : c->ranges) n += r.count;
  int l = 0;
  while ((1LL << (l + 1)) <= std::max(n, 1LL)) l++;
  return TuneKey{c->TL() ? 1 : 0, c->prm.dim, c->prm.basis, c->law, c->prm.transfer, l};
}

int maybe_tune(kmpm_ctx *c) {
  const bool due = c->prm.autotune && !c->tuned && c->runs > 0;
  c->runs++;
  if (!due) return KMPM_OK;
  if (!c->prm.thermal && c->prm.precision == KMPM_PREC_FP32) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(tune_key(c));
    if (it != g_tune_cache.end()) {
      c->tuned = true;
      c->var_g2p1 = it->second.first.first;
      c->var_g2p2 = it->second.first.second;
      c->tuning = "{\"cached\": true, \"from\": " + it->second.second + "}";
      c->graph_valid = false;
      return ensure_graph(c);
    }
  }
  int r = autotune(c);
  if (r != KMPM_OK) return r;
  if (!c->prm.thermal && c->prm.precision == KMPM_PREC_FP32) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[tune_key(c)] = {{c->var_g2p1, c->var_g2p2}, c->tuning};
  }
  return ensure_graph(c);
}

int read_scalars(kmpm_ctx *c, StepScalars &s) {
  CK(cudaMemcpyAsync(&s, c->d_scalars, sizeof(s), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

}  // namespace

// ================================================================ C ABI
extern "C" {

int kmpm_create(const kmpm_params *params, kmpm_ctx **out) {
  if (!params || !out) return KMPM_ERR_ARG;
  *out = nullptr;
  const kmpm_params &p = *params;
  if (p.method != KMPM_TLMPM && p.method != KMPM_ULMPM) return KMPM_ERR_ARG;
  if (p.scheme != KMPM_USL && p.scheme != KMPM_MUSL && p.scheme != KMPM_USF) return KMPM_ERR_ARG;
  if (p.scheme == KMPM_USF && (p.transfer != KMPM_TRANSFER_FLIP || p.thermal)) return KMPM_ERR_ARG;
  if (p.basis < 0 || p.basis > 3 || p.dim < 1 || p.dim > 3) return KMPM_ERR_ARG;
  if (p.method == KMPM_ULMPM && p.basis == KMPM_BASIS_BERNSTEIN) return KMPM_ERR_ARG;
  if (p.independent && p.method != KMPM_TLMPM) return KMPM_ERR_ARG;  // ULMPM solids share one grid
  if (p.transfer < KMPM_TRANSFER_FLIP || p.transfer > KMPM_TRANSFER_MLS) return KMPM_ERR_ARG;
  if (p.transfer == KMPM_TRANSFER_MLS && p.method != KMPM_ULMPM) return KMPM_ERR_ARG;  // MLS is a ULMPM path
  if (p.axisymmetric && (p.dim != 2 || p.thermal)) return KMPM_ERR_ARG;  // 2-D, mechanical
  {
    // affine transfers: the cubic or quadratic spline, or the linear basis for
    // TLMPM (src/solid.cpp:1447-1473); mechanical runs
    const bool affine = p.transfer == KMPM_TRANSFER_APIC || (p.method == KMPM_ULMPM && p.transfer >= KMPM_TRANSFER_AFLIP);
    const bool basis_ok = p.basis == KMPM_BASIS_CUBIC || p.basis == KMPM_BASIS_QUADRATIC ||
                          (p.basis == KMPM_BASIS_LINEAR && p.method == KMPM_TLMPM);
    if (affine && (!basis_ok || p.thermal)) return KMPM_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return KMPM_ERR_CUDA;
  kmpm_ctx *c = new kmpm_ctx();
  c->prm = p;
  // APIC and MLS update v = v_update (src/tlmpm.cpp:82-84, src/ulmpm.cpp:79-82)
  if (p.transfer == KMPM_TRANSFER_APIC || p.transfer == KMPM_TRANSFER_MLS) c->prm.pic_flip = 0;
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return KMPM_ERR_CUDA;
  }
  *out = c;
  return KMPM_OK;
}

int kmpm_destroy(kmpm_ctx *c) {
  if (!c) return KMPM_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->gexec_r) cudaGraphExecDestroy(c->gexec_r);
  for (auto *m : c->d_masks) cudaFree(m);
  for (auto e : c->prof_ev) cudaEventDestroy(e);
  dfree(c->buf[0]); dfree(c->buf[1]); dfree(c->d_pp); dfree(c->d_ranges); dfree(c->d_blk_range);
  dfree(c->d_solid_mat); dfree(c->d_grids); dfree(c->d_blk_grid); dfree(c->d_grid_blk0); dfree(c->d_mats);
  c->nodeB = nullptr;  // inside nodeA's allocation
  dfree(c->nodeA); dfree(c->nodeX); dfree(c->nodeT); dfree(c->nodeP); dfree(c->d_tiles);
  dfree(c->d_cs); dfree(c->d_ce); dfree(c->d_ts); dfree(c->d_te); dfree(c->partial);
  dfree(c->d_fixes); dfree(c->d_fix_start); dfree(c->d_fix_count); dfree(c->d_scalars); dfree(c->d_dtcfl);
  dfree(c->d_hr); dfree(c->d_hflags); dfree(c->d_nhflag); dfree(c->d_gbox);
  dfree(c->d_dump);
  free_contacts(c);
  for (auto &S : c->hsolids) dfree(S.d_in);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->cst) cudaStreamSynchronize(c->cst);
  for (auto &b : c->abufs) {
    dfree(b.buf);
    if (b.gathered) cudaEventDestroy(b.gathered);
    if (b.copied) cudaEventDestroy(b.copied);
  }
  if (c->cst) cudaStreamDestroy(c->cst);
  dfree(c->d_blob); dfree(c->d_lstats); dfree(c->d_log_count); dfree(c->d_log);
  dfree(c->d_err); dfree(c->d_blk_c); dfree(c->d_blk_h); dfree(c->d_eblk); dfree(c->d_eout);
  dfree(c->d_lq_f); dfree(c->d_lq_i); dfree(c->d_lq_count);
  dfree(c->d_knew); dfree(c->d_mflag); dfree(c->d_cin); dfree(c->d_cout); dfree(c->d_mpre); dfree(c->d_bsum);
  dfree(c->d_blkm); dfree(c->d_brun); dfree(c->d_bsort);
  dfree(c->d_keys); dfree(c->d_vals); dfree(c->rtmp.k1); dfree(c->rtmp.v1); dfree(c->rtmp.hist); dfree(c->rtmp.tot);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return KMPM_OK;
}

const char *kmpm_last_error(const kmpm_ctx *c) { return c ? c->err.c_str() : "null context"; }

int kmpm_add_material(kmpm_ctx *c, const kmpm_material *m) {
  if (!c || !m) return KMPM_ERR_ARG;
  if (c->built) return fail(c, KMPM_ERR_STATE, "materials must be added before the first run");
  if (m->type < 0 || m->type > 2) return fail(c, KMPM_ERR_ARG, "unsupported material type (rigid has no GPU path)");
  if (m->type == KMPM_MAT_EOS_STRENGTH) {
    if (m->eos < 0 || m->eos > 2 || m->strength < 0 || m->strength > 4 || m->damage < -1 || m->damage > 0 ||
        m->temp < -1 || m->temp > 0)
      return fail(c, KMPM_ERR_ARG, "unsupported EOS / strength / damage / temperature law");
    if (m->strength == 2 && m->str_p[7] == m->str_p[8])
      return fail(c, KMPM_ERR_ARG, "Error: reference temperature Tr equals melting temperature Tm");
  }
  c->mats.push_back(to_dev(*m));
  // Mat::Mat (src/material.cpp:720-747): E and nu of an EOS material from K and G
  if (m->type == KMPM_MAT_EOS_STRENGTH) {
    const double K = m->eos_p[1], G = m->str_p[0];
    c->mat_E.push_back(9 * K * G / (3 * K + G));
    c->mat_nu.push_back((3 * K - 2 * G) / (2 * (3 * K + G)));
  } else {
    c->mat_E.push_back(m->E);
    c->mat_nu.push_back(m->nu);
  }
  return (int)c->mats.size() - 1;
}

int kmpm_add_grid(kmpm_ctx *c, const double lo[3], double cellsize, const int n[3], const int nglobal[3]) {
  if (!c || !lo || !n || !nglobal || !(cellsize > 0)) return KMPM_ERR_ARG;
  if (c->built) return fail(c, KMPM_ERR_STATE, "grids must be added before the first run");
  if (!c->TL() && !c->hgrids.empty()) return fail(c, KMPM_ERR_ARG, "ULMPM uses one grid");
  kmpm_ctx::HGrid g{};
  for (int d = 0; d < 3; d++) {
    g.lo[d] = lo[d];
    g.n[d] = d < c->prm.dim ? n[d] : 1;
    g.ng[d] = d < c->prm.dim ? nglobal[d] : 1;
    if (g.n[d] < 1) return fail(c, KMPM_ERR_ARG, "empty grid");
  }
  g.cellsize = cellsize;
  c->hgrids.push_back(g);
  return (int)c->hgrids.size() - 1;
}

int kmpm_add_solid(kmpm_ctx *c, int grid, int mat, int n, const double *x0, const double *x, const double *v,
                   const double *mass, const double *vol0, double T0) {
  if (!c || n <= 0 || !x0 || !x || !v || !mass || !vol0) return KMPM_ERR_ARG;
  if (c->built) return fail(c, KMPM_ERR_STATE, "solids must be added before the first run");
  if (grid < 0 || grid >= (int)c->hgrids.size() || mat < 0 || mat >= (int)c->mats.size())
    return fail(c, KMPM_ERR_ARG, "bad grid or material id");
  if (c->TL())
    for (auto &s : c->hsolids)
      if (s.grid == grid) return fail(c, KMPM_ERR_ARG, "each TLMPM solid owns its grid");
  kmpm_ctx::HSolid s;
  s.grid = grid; s.mat = mat; s.n = n; s.T0 = T0;
  // straight to the device (no host copy or conversion); the caller's
  // buffers are free again when this returns
  const size_t nn = (size_t)n;
  CK(cudaMalloc((void **)&s.d_in, sizeof(double) * 11 * nn));
  const struct { const double *src; size_t off, cnt; } parts[5] = {
      {x0, 0, 3 * nn}, {x, 3 * nn, 3 * nn}, {v, 6 * nn, 3 * nn}, {mass, 9 * nn, nn}, {vol0, 10 * nn, nn}};
  for (const auto &q : parts) {
    const cudaError_t e = cudaMemcpyAsync(s.d_in + q.off, q.src, sizeof(double) * q.cnt, cudaMemcpyHostToDevice, c->st);
    if (e != cudaSuccess) {
      cudaFree(s.d_in);
      return fail(c, KMPM_ERR_CUDA, std::string("solid upload: ") + cudaGetErrorString(e));
    }
  }
  const cudaError_t e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) {
    cudaFree(s.d_in);
    return fail(c, KMPM_ERR_CUDA, std::string("solid upload: ") + cudaGetErrorString(e));
  }
  c->hsolids.push_back(s);
  return (int)c->hsolids.size() - 1;
}

int kmpm_set_np_per_cell(kmpm_ctx *c, int solid, int np_per_cell) {
  if (!c || solid < 0 || solid >= (int)c->hsolids.size() || np_per_cell < 1) return KMPM_ERR_ARG;
  if (c->built) return fail(c, KMPM_ERR_STATE, "set before the first run");
  c->hsolids[solid].np_per_cell = np_per_cell;
  return KMPM_OK;
}

int kmpm_add_fix(kmpm_ctx *c, int kind, int grid, const unsigned char *node_mask, const int set[3], const double coef[12]) {
  if (!c || !node_mask || !set || !coef) return KMPM_ERR_ARG;
  if (kind != KMPM_FIX_VELOCITY_NODES && kind != KMPM_FIX_BODY_FORCE) return fail(c, KMPM_ERR_ARG, "unsupported fix");
  if (grid < 0 || grid >= (int)c->hgrids.size()) return fail(c, KMPM_ERR_ARG, "bad grid id");
  const auto &g = c->hgrids[grid];
  kmpm_ctx::HFix f{};
  f.kind = kind;
  f.grid = grid;
  for (int d = 0; d < 3; d++) f.set[d] = d < c->prm.dim ? set[d] : 0;
  for (int k = 0; k < 12; k++) f.c[k] = coef[k];
  if (kind == KMPM_FIX_BODY_FORCE)
    for (int d = 0; d < 3; d++)
      if (f.c[4 * d + 1] != 0 || f.c[4 * d + 2] != 0) return fail(c, KMPM_ERR_ARG, "body_force must be constant");
  f.mask.assign(node_mask, node_mask + (size_t)g.n[0] * g.n[1] * g.n[2]);
  c->hfixes.push_back(std::move(f));
  c->fixes_dirty = true;
  return (int)c->hfixes.size() - 1;
}

int kmpm_add_contact(kmpm_ctx *c, int kind, int solid1, int solid2, double mu) {
  if (!c) return KMPM_ERR_ARG;
  if (kind != KMPM_CONTACT_MIN_PENETRATION && kind != KMPM_CONTACT_HERTZ)
    return fail(c, KMPM_ERR_ARG, "unsupported contact style");
  const int ns = (int)c->hsolids.size();
  if (solid1 < 0 || solid1 >= ns || solid2 < 0 || solid2 >= ns) return fail(c, KMPM_ERR_ARG, "Error: solid unknown.");
  if (solid1 == solid2) return fail(c, KMPM_ERR_ARG, "a contact needs two different solids");
  if (c->indep()) return fail(c, KMPM_ERR_ARG, "independent batches take no contact fix");
  c->hcontacts.push_back({kind, solid1, solid2, kind == KMPM_CONTACT_MIN_PENETRATION ? mu : 0.0});
  c->contacts_dirty = true;
  return (int)c->hcontacts.size() - 1;
}

int kmpm_contact_force(kmpm_ctx *c, int k, double out[3]) {
  if (!c || !out || k < 0 || k >= (int)c->hcontacts.size()) return KMPM_ERR_ARG;
  if (k >= (int)c->contacts.size()) {
    out[0] = out[1] = out[2] = 0;
    return KMPM_OK;
  }
  CK(cudaMemcpyAsync(out, c->contacts[k].ftot, 3 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

static int set_maxtime(kmpm_ctx *c, double maxtime) {
  if (maxtime == c->maxtime_dev) return KMPM_OK;  // no copy between plain runs
  CK(cudaMemcpyAsync((char *)c->d_scalars + offsetof(StepScalars, maxtime), &maxtime, sizeof(double),
                     cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->maxtime_dev = maxtime;
  return KMPM_OK;
}

int kmpm_run(kmpm_ctx *c, int nsteps) {
  if (!c || nsteps < 0) return KMPM_ERR_ARG;
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  if (nsteps > 0) {
    r = maybe_tune(c);
    if (r != KMPM_OK) return r;
  }
  r = set_maxtime(c, 1e300);
  if (r != KMPM_OK) return r;
  r = launch_steps(c, nsteps);
  if (r != KMPM_OK) return r;
  return check_error(c);
}

// kmpm_run without the final wait: the steps' graph launches are queued and
// the error word is read by the next kmpm_sync / kmpm_run
int kmpm_run_async(kmpm_ctx *c, int nsteps) {
  if (!c || nsteps < 0) return KMPM_ERR_ARG;
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  if (nsteps > 0) {
    r = maybe_tune(c);
    if (r != KMPM_OK) return r;
  }
  r = set_maxtime(c, 1e300);
  if (r != KMPM_OK) return r;
  r = launch_steps(c, nsteps);
  if (r != KMPM_OK) return r;
  CK(cudaGetLastError());
  return KMPM_OK;
}

int kmpm_sync(kmpm_ctx *c) {
  if (!c) return KMPM_ERR_ARG;
  if (!c->built) return KMPM_OK;
  return check_error(c);
}

int kmpm_run_time(kmpm_ctx *c, double maxtime, int *nsteps_done) {
  if (!c) return KMPM_ERR_ARG;
  if (c->indep()) return fail(c, KMPM_ERR_ARG, "run_time needs one clock: not available for independent solids");
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  r = maybe_tune(c);
  if (r != KMPM_OK) return r;
  StepScalars s{};
  r = read_scalars(c, s);
  if (r != KMPM_OK) return r;
  const long long n0 = s.ntimestep;
  // RunTime::command (src/run_time.cpp:30-60): steps while time < maxtime.
  // The steps check the bound on the device, so a batch can be launched
  // without overshooting; the host only decides when to stop launching.
  r = set_maxtime(c, maxtime);
  if (r != KMPM_OK) return r;
  while (s.time < maxtime) {
    r = launch_steps(c, 64);
    if (r != KMPM_OK) return r;
    r = check_error(c);
    if (r != KMPM_OK) return r;
    r = read_scalars(c, s);
    if (r != KMPM_OK) return r;
  }
  r = set_maxtime(c, 1e300);
  if (r != KMPM_OK) return r;
  if (nsteps_done) *nsteps_done = (int)(s.ntimestep - n0);
  return KMPM_OK;
}

int kmpm_run_until(kmpm_ctx *c, int nsteps, double maxtime, int *nsteps_done) {
  if (!c || nsteps < 0) return KMPM_ERR_ARG;
  if (c->indep()) return fail(c, KMPM_ERR_ARG, "run_until needs one clock: not available for independent solids");
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  r = maybe_tune(c);
  if (r != KMPM_OK) return r;
  StepScalars s{};
  r = read_scalars(c, s);
  if (r != KMPM_OK) return r;
  const long long n0 = s.ntimestep;
  // at most nsteps steps of a RunTime::command (src/run_time.cpp:30-60): the
  // steps check the time bound on the device, so a batch never overshoots it
  r = set_maxtime(c, maxtime);
  if (r != KMPM_OK) return r;
  while (s.time < maxtime && s.ntimestep - n0 < nsteps) {
    const int k = (int)std::min<long long>(64, nsteps - (s.ntimestep - n0));
    r = launch_steps(c, k);
    if (r != KMPM_OK) return r;
    r = check_error(c);
    if (r != KMPM_OK) return r;
    r = read_scalars(c, s);
    if (r != KMPM_OK) return r;
  }
  r = set_maxtime(c, 1e300);
  if (r != KMPM_OK) return r;
  if (nsteps_done) *nsteps_done = (int)(s.ntimestep - n0);
  return KMPM_OK;
}

int kmpm_scalars(kmpm_ctx *c, double *time, double *dt, long long *ntimestep) {
  if (!c) return KMPM_ERR_ARG;
  StepScalars s{};
  if (c->built) {
    int r = read_scalars(c, s);
    if (r != KMPM_OK) return r;
  } else {
    s.dt = c->prm.dt;
  }
  if (time) *time = s.time;
  if (dt) *dt = s.dt;
  if (ntimestep) *ntimestep = s.ntimestep;
  return KMPM_OK;
}

// Copies the rows of the listed fields for slots [start, start+n) of the
// current particle buffer into H (H[f][slot - start]).
int kmpm_solid_scalars(kmpm_ctx *c, int solid, double *time, double *dt, long long *ntimestep) {
  if (!c || solid < 0 || solid >= (int)c->hsolids.size()) return KMPM_ERR_ARG;
  if (!c->built || !c->indep()) return kmpm_scalars(c, time, dt, ntimestep);
  StepScalars s{};
  CK(cudaMemcpyAsync(&s, c->d_scalars + c->solid_range[solid], sizeof(s), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (time) *time = s.time;
  if (dt) *dt = s.dt;
  if (ntimestep) *ntimestep = s.ntimestep;
  return KMPM_OK;
}

static int fetch_rows(kmpm_ctx *c, const std::vector<int> &fields, int start, int n,
                      std::vector<std::vector<float>> &H) {
  CK(cudaStreamSynchronize(c->st));
  float *cur = nullptr;
  CK(cudaMemcpyAsync(&cur, c->d_pp, sizeof(float *), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  H.assign(PF_COUNT, std::vector<float>());
  for (int f : fields) {
    H[f].resize(n);
    CK(cudaMemcpyAsync(H[f].data(), cur + (size_t)f * c->ps + start, sizeof(float) * n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  return KMPM_OK;
}

// caller index and solid of every slot of the range holding `solid`
static int slot_map(kmpm_ctx *c, const RangeDev &rg, std::vector<int> &orig, std::vector<int> &sid) {
  if (c->TL() && !c->orig_cache.empty()) {
    orig.assign(c->orig_cache.begin() + rg.start, c->orig_cache.begin() + rg.start + rg.count);
    sid.assign(c->sid_cache.begin() + rg.start, c->sid_cache.begin() + rg.start + rg.count);
    return KMPM_OK;
  }
  std::vector<std::vector<float>> H;
  int r = fetch_rows(c, {PF_ORIG, PF_SID}, rg.start, rg.count, H);
  if (r != KMPM_OK) return r;
  orig.resize(rg.count);
  sid.resize(rg.count);
  std::memcpy(orig.data(), H[PF_ORIG].data(), sizeof(int) * rg.count);
  std::memcpy(sid.data(), H[PF_SID].data(), sizeof(int) * rg.count);
  if (c->TL()) {  // static order: cache it for the whole run
    if (c->orig_cache.empty()) {
      c->orig_cache.assign(c->ps, -1);
      c->sid_cache.assign(c->ps, -1);
    }
    std::copy(orig.begin(), orig.end(), c->orig_cache.begin() + rg.start);
    std::copy(sid.begin(), sid.end(), c->sid_cache.begin() + rg.start);
    bool all = true;
    for (auto &q : c->ranges) if (c->orig_cache[q.start] < 0) all = false;
    if (!all) c->orig_cache.clear(), c->sid_cache.clear();
  }
  return KMPM_OK;
}

int kmpm_download_particles(kmpm_ctx *c, int solid, int field, double *out) {
  if (!c || !out || solid < 0 || solid >= (int)c->hsolids.size()) return KMPM_ERR_ARG;
  const auto &S = c->hsolids[solid];
  if (!c->built) {
    // the arrays as the caller gave them (x0, x, v at 0, 3n, 6n of the staging)
    const size_t off = field == KMPM_P_X0 ? 0 : field == KMPM_P_X ? 3 : field == KMPM_P_V ? 6 : 99;
    if (off == 99) return fail(c, KMPM_ERR_STATE, "field not available before the first run");
    CK(cudaMemcpyAsync(out, S.d_in + off * S.n, sizeof(double) * 3 * S.n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return KMPM_OK;
  }
  if (field == KMPM_P_STRAIN_EL && !c->prm.track_strain)
    return fail(c, KMPM_ERR_STATE, "strain_el is tracked only with track_strain");
  const int w = dump_width(field);
  if (w == 0) return fail(c, KMPM_ERR_ARG, "unknown particle field");
  // gathered into caller order and FP64 on the device (kmpm_dump.cu), then one copy
  const size_t need = (size_t)S.n * w;
  if (need > c->dump_cap) {
    dfree(c->d_dump);
    DALLOC(c->d_dump, need);
    c->dump_cap = need;
  }
  const int ri = c->TL() ? c->solid_range[solid] : 0;
  // TLMPM keeps sigma unrotated, except for neo-Hookean solids, whose R stays
  // the identity (src/solid.cpp:1220); ULMPM stores it in the current frame
  const int rotate = c->TL() && c->mats[S.mat].type != KMPM_MAT_NEO_HOOKEAN;
  launch_dump(part_args(c), ri, c->ranges[ri].count, solid, c->solid_base[solid], field, c->TL() ? 1 : 0, rotate,
              c->T_ref, c->d_dump, c->st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, c->d_dump, sizeof(double) * need, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

int kmpm_download_particles_async(kmpm_ctx *c, int solid, int field, double *out) {
  if (!c || !out || solid < 0 || solid >= (int)c->hsolids.size()) return KMPM_ERR_ARG;
  if (!c->built) return fail(c, KMPM_ERR_STATE, "no particle state before the first run");
  if (field == KMPM_P_STRAIN_EL && !c->prm.track_strain)
    return fail(c, KMPM_ERR_STATE, "strain_el is tracked only with track_strain");
  const int w = dump_width(field);
  if (w == 0) return fail(c, KMPM_ERR_ARG, "unknown particle field");
  const auto &S = c->hsolids[solid];
  const size_t need = (size_t)S.n * w;
  if (!c->cst) CK(cudaStreamCreateWithFlags(&c->cst, cudaStreamNonBlocking));
  // the smallest free buffer that holds the field (one whose copy has
  // ended), else a new one: a buffer is never freed and reallocated here,
  // as cudaFree would wait for every step the caller has queued
  kmpm_ctx::AsyncBuf *b = nullptr;
  for (auto &x : c->abufs) {
    if (x.busy && cudaEventQuery(x.copied) != cudaSuccess) continue;
    x.busy = false;
    if (x.cap >= need && (!b || x.cap < b->cap)) b = &x;
  }
  if (!b) {
    c->abufs.emplace_back();
    b = &c->abufs.back();
    CK(cudaEventCreateWithFlags(&b->gathered, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&b->copied, cudaEventDisableTiming));
    DALLOC(b->buf, need);
    b->cap = need;
  }
  const int ri = c->TL() ? c->solid_range[solid] : 0;
  const int rotate = c->TL() && c->mats[S.mat].type != KMPM_MAT_NEO_HOOKEAN;
  launch_dump(part_args(c), ri, c->ranges[ri].count, solid, c->solid_base[solid], field, c->TL() ? 1 : 0, rotate,
              c->T_ref, b->buf, c->st);
  CK(cudaGetLastError());
  CK(cudaEventRecord(b->gathered, c->st));
  CK(cudaStreamWaitEvent(c->cst, b->gathered, 0));
  CK(cudaMemcpyAsync(out, b->buf, sizeof(double) * need, cudaMemcpyDeviceToHost, c->cst));
  CK(cudaEventRecord(b->copied, c->cst));
  b->busy = true;
  for (auto &x : c->abufs)  // a buffer has one pending copy at a time
    if (&x != b && x.dst == out) x.dst = nullptr;
  b->dst = out;
  return KMPM_OK;
}

int kmpm_wait_download(kmpm_ctx *c, const double *out) {
  if (!c || !out) return KMPM_ERR_ARG;
  for (auto &b : c->abufs)
    if (b.dst == out) {
      if (b.busy) CK(cudaEventSynchronize(b.copied));
      b.busy = false;
      b.dst = nullptr;
    }
  return KMPM_OK;
}

int kmpm_sync_downloads(kmpm_ctx *c) {
  if (!c) return KMPM_ERR_ARG;
  if (c->cst) CK(cudaStreamSynchronize(c->cst));
  for (auto &b : c->abufs) b.busy = false;
  return KMPM_OK;
}

int kmpm_upload_particles(kmpm_ctx *c, int solid, int field, const double *in) {
  if (!c || !in || solid < 0 || solid >= (int)c->hsolids.size()) return KMPM_ERR_ARG;
  auto &S = c->hsolids[solid];
  if (!c->built) {
    // into the arrays kmpm_add_solid took (x0, x, v at 0, 3n, 6n)
    const size_t off = field == KMPM_P_X0 ? 0 : field == KMPM_P_X ? 3 : field == KMPM_P_V ? 6 : 99;
    if (off == 99) return fail(c, KMPM_ERR_STATE, "only x0, x and v can be uploaded before the first run");
    CK(cudaMemcpyAsync(S.d_in + off * S.n, in, sizeof(double) * 3 * S.n, cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    return KMPM_OK;
  }
  switch (field) {
    case KMPM_P_X: case KMPM_P_V: case KMPM_P_SIGMA: case KMPM_P_F: case KMPM_P_EPS_P: case KMPM_P_EPSDOT_P:
    case KMPM_P_DAMAGE: case KMPM_P_DAMAGE_INIT: case KMPM_P_T: case KMPM_P_STRAIN_EL:
      break;
    case KMPM_P_VOL0PK1:
      if (!c->TL()) return fail(c, KMPM_ERR_ARG, "vol0PK1 is TLMPM state");
      break;
    case KMPM_P_X0:
      return fail(c, KMPM_ERR_STATE, "x0 is fixed once the context is built (TLMPM bins by it)");
    default:
      return fail(c, KMPM_ERR_ARG, "this field cannot be uploaded");
  }
  if (field == KMPM_P_T && !c->prm.thermal) return fail(c, KMPM_ERR_STATE, "temperature needs a thermo-mechanical run");
  if ((field == KMPM_P_EPS_P || field == KMPM_P_EPSDOT_P || field == KMPM_P_DAMAGE || field == KMPM_P_DAMAGE_INIT) &&
      !c->restored_state) {
    c->restored_state = true;  // keep these rows through the re-binning from now on
    set_ul_fields(c);
    c->graph_valid = false;
  }
  if (field == KMPM_P_STRAIN_EL && !c->prm.track_strain)
    return fail(c, KMPM_ERR_STATE, "strain_el is tracked only with track_strain");
  const size_t need = (size_t)S.n * dump_width(field);
  if (need > c->dump_cap) {
    dfree(c->d_dump);
    DALLOC(c->d_dump, need);
    c->dump_cap = need;
  }
  CK(cudaMemcpyAsync(c->d_dump, in, sizeof(double) * need, cudaMemcpyHostToDevice, c->st));
  c->p_valid = false;  // the next scatter sums the momentum of the new state
  const int ri = c->TL() ? c->solid_range[solid] : 0;
  launch_load(part_args(c), ri, c->ranges[ri].count, solid, c->solid_base[solid], field, c->TL() ? 1 : 0, c->T_ref,
              c->d_dump, c->st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

int kmpm_set_scalars(kmpm_ctx *c, double time, double dt, long long ntimestep) {
  if (!c) return KMPM_ERR_ARG;
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  std::vector<StepScalars> sv(c->nscalars);
  CK(cudaMemcpyAsync(sv.data(), c->d_scalars, sizeof(StepScalars) * sv.size(), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (auto &x : sv) {
    x.time = time;
    x.dt = dt;
    x.ntimestep = ntimestep;
  }
  CK(cudaMemcpyAsync(c->d_scalars, sv.data(), sizeof(StepScalars) * sv.size(), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

// ---- device snapshot: header, field ids, scalars, particle rows, node arrays
struct SnapHeader {
  char magic[8];
  int version, method, dim, basis, nfields, nscalars, nnodes_pad, nsolids;
  unsigned long long ps;
};
static const char SNAP_MAGIC[8] = {'K', 'M', 'P', 'M', 'S', 'N', 'P', '1'};

static unsigned long long snap_bytes(kmpm_ctx *c, const std::vector<int> &fl) {
  return sizeof(SnapHeader) + sizeof(int) * fl.size() + sizeof(StepScalars) * c->nscalars +
         sizeof(float) * c->ps * fl.size() + (NODE_STRIDE + 1) * sizeof(float4) * (unsigned long long)c->nnodes_pad +
         sizeof(float) * (unsigned long long)c->nnodes_pad;
}

static int current_buffer(kmpm_ctx *c, float **cur) {
  CK(cudaMemcpyAsync(cur, c->d_pp, sizeof(float *), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

int kmpm_state_size(kmpm_ctx *c, unsigned long long *bytes) {
  if (!c || !bytes) return KMPM_ERR_ARG;
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  *bytes = snap_bytes(c, active_fields(c));
  return KMPM_OK;
}

int kmpm_save_state(kmpm_ctx *c, void *out, unsigned long long bytes) {
  if (!c || !out) return KMPM_ERR_ARG;
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  const std::vector<int> fl = active_fields(c);
  if (bytes < snap_bytes(c, fl)) return fail(c, KMPM_ERR_ARG, "snapshot buffer too small (kmpm_state_size)");
  char *o = (char *)out;
  SnapHeader h{};
  std::memcpy(h.magic, SNAP_MAGIC, 8);
  h.version = 1; h.method = c->prm.method; h.dim = c->prm.dim; h.basis = c->prm.basis;
  h.nfields = (int)fl.size(); h.nscalars = c->nscalars; h.nnodes_pad = c->nnodes_pad;
  h.nsolids = (int)c->hsolids.size(); h.ps = c->ps;
  std::memcpy(o, &h, sizeof(h)); o += sizeof(h);
  std::memcpy(o, fl.data(), sizeof(int) * fl.size()); o += sizeof(int) * fl.size();
  CK(cudaMemcpyAsync(o, c->d_scalars, sizeof(StepScalars) * c->nscalars, cudaMemcpyDeviceToHost, c->st));
  o += sizeof(StepScalars) * c->nscalars;
  float *cur = nullptr;
  r = current_buffer(c, &cur);
  if (r != KMPM_OK) return r;
  for (int f : fl) {
    CK(cudaMemcpyAsync(o, cur + (size_t)f * c->ps, sizeof(float) * c->ps, cudaMemcpyDeviceToHost, c->st));
    o += sizeof(float) * c->ps;
  }
  // v / v_update (interleaved) and x of the nodes
  CK(cudaMemcpyAsync(o, c->nodeA, sizeof(float4) * NODE_STRIDE * c->nnodes_pad, cudaMemcpyDeviceToHost, c->st));
  o += sizeof(float4) * NODE_STRIDE * c->nnodes_pad;
  CK(cudaMemcpyAsync(o, c->nodeX, sizeof(float4) * c->nnodes_pad, cudaMemcpyDeviceToHost, c->st));
  o += sizeof(float4) * c->nnodes_pad;
  CK(cudaMemcpyAsync(o, c->nodeT, sizeof(float) * c->nnodes_pad, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

int kmpm_load_state(kmpm_ctx *c, const void *in, unsigned long long bytes) {
  if (!c || !in) return KMPM_ERR_ARG;
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  if (bytes < sizeof(SnapHeader)) return fail(c, KMPM_ERR_ARG, "not a snapshot");
  const char *o = (const char *)in;
  SnapHeader h;
  std::memcpy(&h, o, sizeof(h));
  o += sizeof(h);
  if (std::memcmp(h.magic, SNAP_MAGIC, 8) != 0 || h.version != 1) return fail(c, KMPM_ERR_ARG, "not a snapshot");
  c->p_valid = false;  // the next scatter sums the momentum of the loaded state
  std::vector<int> fl = active_fields(c);
  if (h.nfields != (int)fl.size() && !c->restored_state) {
    // a snapshot of a context that had uploaded plastic strain or damage
    c->restored_state = true;
    std::vector<int> wide = active_fields(c);
    if (h.nfields == (int)wide.size()) {
      set_ul_fields(c);
      c->graph_valid = false;
      fl = wide;
    } else {
      c->restored_state = false;
    }
  }
  if (h.method != c->prm.method || h.dim != c->prm.dim || h.basis != c->prm.basis || h.nfields != (int)fl.size() ||
      h.nscalars != c->nscalars || h.nnodes_pad != c->nnodes_pad || h.nsolids != (int)c->hsolids.size() ||
      h.ps != c->ps || bytes < snap_bytes(c, fl))
    return fail(c, KMPM_ERR_ARG, "snapshot of a different setup");
  if (std::memcmp(o, fl.data(), sizeof(int) * fl.size()) != 0) return fail(c, KMPM_ERR_ARG, "snapshot fields differ");
  o += sizeof(int) * fl.size();
  CK(cudaMemcpyAsync(c->d_scalars, o, sizeof(StepScalars) * c->nscalars, cudaMemcpyHostToDevice, c->st));
  o += sizeof(StepScalars) * c->nscalars;
  float *cur = nullptr;
  r = current_buffer(c, &cur);
  if (r != KMPM_OK) return r;
  for (int f : fl) {
    CK(cudaMemcpyAsync(cur + (size_t)f * c->ps, o, sizeof(float) * c->ps, cudaMemcpyHostToDevice, c->st));
    o += sizeof(float) * c->ps;
  }
  CK(cudaMemcpyAsync(c->nodeA, o, sizeof(float4) * NODE_STRIDE * c->nnodes_pad, cudaMemcpyHostToDevice, c->st));
  o += sizeof(float4) * NODE_STRIDE * c->nnodes_pad;
  CK(cudaMemcpyAsync(c->nodeX, o, sizeof(float4) * c->nnodes_pad, cudaMemcpyHostToDevice, c->st));
  o += sizeof(float4) * c->nnodes_pad;
  CK(cudaMemcpyAsync(c->nodeT, o, sizeof(float) * c->nnodes_pad, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  // the slot maps of the host caches follow the restored order; maxtime
  // as written with the scalars
  c->orig_cache.clear();
  c->sid_cache.clear();
  StepScalars s0{};
  std::memcpy(&s0, (const char *)in + sizeof(SnapHeader) + sizeof(int) * fl.size(), sizeof(s0));
  c->maxtime_dev = s0.maxtime;
  return KMPM_OK;
}

int kmpm_download_grid(kmpm_ctx *c, int grid, int field, double *out) {
  if (!c || !out || grid < 0 || grid >= (int)c->hgrids.size()) return KMPM_ERR_ARG;
  if (!c->built) return fail(c, KMPM_ERR_STATE, "no grid state before the first run");
  CK(cudaStreamSynchronize(c->st));
  const GridDev &g = c->grids[grid];
  const int nn = g.n[0] * g.n[1] * g.n[2];
  std::vector<float4> A(nn), B(nn);
  std::vector<float> Tn(nn);
  if (field == KMPM_G_MASS || field == KMPM_G_V || field == KMPM_G_V_UPDATE) {
    const float4 *src = (field == KMPM_G_V_UPDATE ? c->nodeB : c->nodeA) + (size_t)NODE_STRIDE * g.node_off;
    CK(cudaMemcpy2DAsync(A.data(), sizeof(float4), src, NODE_STRIDE * sizeof(float4), sizeof(float4), nn,
                         cudaMemcpyDeviceToHost, c->st));
  }
  else if (field == KMPM_G_X)
    CK(cudaMemcpyAsync(A.data(), c->nodeX + g.node_off, sizeof(float4) * nn, cudaMemcpyDeviceToHost, c->st));
  else if (field == KMPM_G_T)
    CK(cudaMemcpyAsync(Tn.data(), c->nodeT + g.node_off, sizeof(float) * nn, cudaMemcpyDeviceToHost, c->st));
  else return fail(c, KMPM_ERR_ARG, "unknown grid field");
  CK(cudaStreamSynchronize(c->st));
  for (int i = 0; i < nn; i++) {
    if (field == KMPM_G_MASS) out[i] = A[i].w;
    else if (field == KMPM_G_T) out[i] = c->T_ref + Tn[i];
    else { out[3 * i] = A[i].x; out[3 * i + 1] = A[i].y; out[3 * i + 2] = A[i].z; }
  }
  return KMPM_OK;
}

int kmpm_energy(kmpm_ctx *c, double out[2]) {
  if (!c || !out) return KMPM_ERR_ARG;
  if (!c->built) return fail(c, KMPM_ERR_STATE, "no state before the first run");
  PartArgs pa = part_args(c);
  launch_energy(pa, c->nblk_p, c->d_eblk, c->d_eout, c->st);
  CK(cudaMemcpyAsync(out, c->d_eout, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

void *kmpm_stream(kmpm_ctx *c) { return c ? (void *)c->st : nullptr; }

int kmpm_profile(kmpm_ctx *c, int nsteps, double *phase_ms, int max_phases, int *nphases) {
  if (!c || nsteps <= 0 || !phase_ms || !nphases) return KMPM_ERR_ARG;
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  std::vector<double> acc;
  for (int s = 0; s < nsteps; s++) {
    c->profiling = true;
    c->prof_n = 0;
    r = enqueue_step(c, c->reuse_ok && c->p_valid);
    c->profiling = false;
    if (r != KMPM_OK) return r;
    c->p_valid = c->reuse_ok;
    CK(cudaStreamSynchronize(c->st));
    acc.resize(std::max<size_t>(acc.size(), c->prof_n), 0.0);
    for (int k = 1; k < c->prof_n; k++) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, c->prof_ev[k - 1], c->prof_ev[k]));
      acc[k - 1] += ms;
    }
  }
  const int n = std::min(c->prof_n - 1, max_phases);
  for (int k = 0; k < n; k++) phase_ms[k] = acc[k] / nsteps;
  *nphases = n;
  return check_error(c);
}

const char *kmpm_profile_phase(kmpm_ctx *c, int i) {
  if (!c || i < 0 || i + 1 >= (int)c->prof_names.size()) return "";
  return c->prof_names[i + 1].c_str();
}

int kmpm_launches_per_step(kmpm_ctx *c) { return c ? c->launches_per_step : 0; }

const char *kmpm_tuning(kmpm_ctx *c) { return c ? c->tuning.c_str() : "{}"; }

// ---------------------------------------------------------------- learned return map
static int learn_check(kmpm_ctx *c) {
  if (!c->TL() || c->prm.dim != 3 || c->prm.basis != KMPM_BASIS_CUBIC)
    return fail(c, KMPM_ERR_ARG, "the learned return map covers 3-D TLMPM with the cubic B-spline basis");
  if (c->prm.precision != KMPM_PREC_FP32 || c->prm.thermal || c->apic() || c->usf())
    return fail(c, KMPM_ERR_ARG,
                "the learned return map needs FP32, FLIP/PIC transfers, USL or MUSL and no thermo-mechanical coupling");
  for (const MatDev &m : c->mats)
    if (m.type != KMPM_MAT_EOS_STRENGTH || m.strength != 2)
      return fail(c, KMPM_ERR_ARG, "the learned return map needs eos-strength materials with Johnson-Cook strength");
  if (!c->LK.sur) get_learn_kernels(c->LK);
  return KMPM_OK;
}

int kmpm_log_start(kmpm_ctx *c, long long capacity, double fraction, unsigned long long seed) {
  if (!c || capacity < 1 || !(fraction > 0.0)) return KMPM_ERR_ARG;
  int r = learn_check(c);
  if (r != KMPM_OK) return r;
  if (capacity != c->log_cap) {
    dfree(c->d_log);
    DALLOC(c->d_log, (size_t)capacity * (mlp_nin() + mlp_nout()));
    c->log_cap = capacity;
  }
  if (!c->d_log_count) DALLOC(c->d_log_count, 1);
  CK(cudaMemsetAsync(c->d_log_count, 0, sizeof(unsigned long long), c->st));
  CK(cudaStreamSynchronize(c->st));
  c->log_thresh = fraction >= 1.0 ? 0xFFFFFFFFu : (uint32_t)(fraction * 4294967296.0);
  c->log_seed = seed;
  c->learn_mode = MODE_LOG;
  c->graph_valid = false;
  return KMPM_OK;
}

int kmpm_log_stop(kmpm_ctx *c) {
  if (!c) return KMPM_ERR_ARG;
  if (c->learn_mode == MODE_LOG) {
    c->learn_mode = MODE_PLAIN;
    c->graph_valid = false;
  }
  return KMPM_OK;
}

int kmpm_log_data(kmpm_ctx *c, const float **rows, long long *n) {
  if (!c || !rows || !n) return KMPM_ERR_ARG;
  *rows = c->d_log;
  *n = 0;
  if (!c->d_log_count) return KMPM_OK;
  unsigned long long cnt = 0;
  CK(cudaMemcpyAsync(&cnt, c->d_log_count, sizeof(cnt), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  *n = (long long)std::min<unsigned long long>(cnt, (unsigned long long)c->log_cap);
  return KMPM_OK;
}

int kmpm_jc_label(kmpm_ctx *c, int material, const float *X, long long n, float *Y) {
  if (!c || !X || !Y || n < 0 || material < 0 || material >= (int)c->mats.size()) return KMPM_ERR_ARG;
  const MatDev &m = c->mats[material];
  if (m.type != KMPM_MAT_EOS_STRENGTH || m.strength != 2) return fail(c, KMPM_ERR_ARG, "not a Johnson-Cook material");
  int r = prepare(c);
  if (r != KMPM_OK) return r;
  if (!c->LK.label) get_learn_kernels(c->LK);
  if (n == 0) return KMPM_OK;
  const MatDev *mats = c->d_mats;
  void *args[] = {(void *)&mats, &material, (void *)&X, &n, (void *)&Y};
  CK(cudaLaunchKernel(c->LK.label, dim3((unsigned)((n + 255) / 256)), dim3(256), args, 0, c->st));
  CK(cudaStreamSynchronize(c->st));
  return KMPM_OK;
}

int kmpm_set_surrogate(kmpm_ctx *c, kmpm_mlp *m, double tol) {
  if (!c) return KMPM_ERR_ARG;
  if (!m) {
    if (c->learn_mode == MODE_SUR) {
      c->learn_mode = MODE_PLAIN;
      c->graph_valid = false;
    }
    return KMPM_OK;
  }
  if (!(tol > 0.0)) return fail(c, KMPM_ERR_ARG, "tol must be positive");
  int r = learn_check(c);
  if (r != KMPM_OK) return r;
  const unsigned char *blob = nullptr;
  r = mlp_device_blob(m, &blob);
  if (r != KMPM_OK) return fail(c, r, std::string("network: ") + kmpm_mlp_last_error(m));
  if (!c->d_blob) DALLOC(c->d_blob, (size_t)mlp_blob_bytes());
  if (!c->d_lstats) DALLOC(c->d_lstats, 4);
  CK(cudaMemcpyAsync(c->d_blob, blob, (size_t)mlp_blob_bytes(), cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemsetAsync(c->d_lstats, 0, 4 * sizeof(unsigned long long), c->st));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaFuncSetAttribute(c->LK.sur, cudaFuncAttributeMaxDynamicSharedMemorySize, c->LK.sur_smem));
  CK(cudaFuncSetAttribute(c->LK.queue, cudaFuncAttributeMaxDynamicSharedMemorySize, c->LK.sur_smem));
  c->sur_tol = (float)tol;
  c->learn_mode = MODE_SUR;
  c->graph_valid = false;
  return KMPM_OK;
}

int kmpm_surrogate_stats(kmpm_ctx *c, long long out[4]) {
  if (!c || !out) return KMPM_ERR_ARG;
  unsigned long long v[4] = {0, 0, 0, 0};
  if (c->d_lstats) {
    CK(cudaMemcpyAsync(v, c->d_lstats, sizeof(v), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  for (int k = 0; k < 4; k++) out[k] = (long long)v[k];
  return KMPM_OK;
}

}  // extern "C"
