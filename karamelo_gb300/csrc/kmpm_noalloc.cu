// kmpm_noalloc.cu -- kmpm_p2g_mass_noalloc: the nodal-mass scatter
// (Solid::compute_mass_nodes, src/solid.cpp:317-335) for callers that cannot
// allocate device memory.
//
// Some host applications own all of their GPU memory through their own pool
// allocator and budget: they reserve the device memory up front and may not
// call cudaMalloc behind the pool's back (the call could fail once the pool
// holds the memory, and it would escape their accounting).  This entry point
// takes the caller's input and output buffers and keeps every intermediate
// array (binning keys, sort buffers, cell and tile ranges, the scatter's tile
// partials, an error counter) in one file-scope device array of fixed size
// instead.
//
// Properties of that array:
//   - it has a fixed size (KMPM_NOALLOC_SCRATCH_BYTES) and exists on every
//     GPU that loads this library until the process exits;
//   - its device address is looked up once per device, with that device
//     current, by the first call made on that device: make that first call
//     before any stream capture;
//   - all calls share it and it keeps the last call's contents, so this code
//     clears whatever must start at zero; two calls whose work overlaps on the
//     GPU (different streams, no ordering between them) race on it.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/kmpm.h"
#include "kmpm_step_impl.cuh"

namespace kmpm {

namespace {

constexpr size_t kScratchBytes = KMPM_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char *g_base[kMaxDevices] = {nullptr};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Layout of the scratch array for one call.
struct Carve {
  size_t off = 0;
  template <typename T> T *take(unsigned char *base, size_t n) {
    T *p = reinterpret_cast<T *>(base + off);
    off = align256(off + sizeof(T) * n);
    return p;
  }
};

// keys of the caller's particles (caller order); x is n*3 floats (x,y,z per
// particle).  A particle outside the grid's cells (or with a non-finite
// coordinate) is counted in *bad: its cell index is clamped only so that every
// access stays in bounds, and the call reports the count as an error.
__global__ void k_na_keys(const float *x, int n, const GridDev g, int dim, int t0, int t1, int t2, int *keys,
                          int *vals, int *bad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int T[3] = {t0, t1, t2};
  int c[3] = {0, 0, 0};
  bool inside = true;
  for (int d = 0; d < dim; d++) {
    const float t = (x[3 * p + d] - g.lo[d]) * g.inv_cellsize;
    inside = inside && t >= 0.f && t < (float)g.ncell[d];
    const int cd = (int)fminf(fmaxf(t, 0.f), (float)(g.ncell[d] - 1));
    c[d] = max(0, min(cd, g.ncell[d] - 1));
  }
  if (!inside) atomicAdd(bad, 1);
  const int tl = ((c[0] / T[0]) * g.ntile[1] + c[1] / T[1]) * g.ntile[2] + c[2] / T[2];
  const int lc = ((c[0] % T[0]) * T[1] + c[1] % T[1]) * T[2] + c[2] % T[2];
  keys[p] = tl * (T[0] * T[1] * T[2]) + lc;
  vals[p] = p;
}

// sorted structure of arrays: the fields the mass scatter reads
__global__ void k_na_gather(const float *x, const float *mass, const int *perm, int n, float *P, size_t ps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = perm[i];
  for (int d = 0; d < 3; d++) P[(PF_X0 + d) * ps + i] = x[3 * j + d];
  P[PF_MASS * ps + i] = mass[j];
}

__global__ void k_na_tiles(int2 *tiles, int ntiles) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ntiles) tiles[t] = make_int2(0, t);
}

// The grid description arrives by value (a kernel argument), so no host
// memory is read once the call has returned.
__global__ void k_na_init(GridDev gv, GridDev *gd, float **pp, float *P, StepScalars *sc, int *bad) {
  *gd = gv;
  *bad = 0;
  pp[0] = P;
  pp[1] = P;
  sc->dt = 0;
  sc->time = 0;
  sc->ntimestep = 0;
  sc->dtCFL = 0;
  sc->maxtime = 1e300;
}

// nodal sums of the tile partials, written to the caller's output
template <int DIM, int BASIS>
__global__ void k_na_grid_mass(GridArgs a, const GridDev *gp, float *out) {
  const GridDev g = *gp;
  const int li = blockIdx.x * blockDim.x + threadIdx.x;
  const int nn = g.n[0] * g.n[1] * g.n[2];
  if (li >= nn) return;
  int ix[3];
  ix[2] = li % g.n[2];
  ix[1] = (li / g.n[2]) % g.n[1];
  ix[0] = li / (g.n[1] * g.n[2]);
  float s[1];
  gather_partials<DIM, BASIS, 1, float>(a, g, li, ix, s);
  out[li] = s[0];
}

template <int DIM, int BASIS> struct NaKernels {
  static void *p2g() { return (void *)k_p2g<DIM, BASIS, P2G_MASS, false>; }
  static void *grid() { return (void *)k_na_grid_mass<DIM, BASIS>; }
};

void na_kernels(int dim, int basis, void **p2g, void **grid) {
  switch (basis == 3 ? 100 + dim : dim * 3 + basis) {
    case 3: *p2g = NaKernels<1, 0>::p2g(); *grid = NaKernels<1, 0>::grid(); break;
    case 4: *p2g = NaKernels<1, 1>::p2g(); *grid = NaKernels<1, 1>::grid(); break;
    case 5: *p2g = NaKernels<1, 2>::p2g(); *grid = NaKernels<1, 2>::grid(); break;
    case 6: *p2g = NaKernels<2, 0>::p2g(); *grid = NaKernels<2, 0>::grid(); break;
    case 7: *p2g = NaKernels<2, 1>::p2g(); *grid = NaKernels<2, 1>::grid(); break;
    case 8: *p2g = NaKernels<2, 2>::p2g(); *grid = NaKernels<2, 2>::grid(); break;
    case 9: *p2g = NaKernels<3, 0>::p2g(); *grid = NaKernels<3, 0>::grid(); break;
    case 10: *p2g = NaKernels<3, 1>::p2g(); *grid = NaKernels<3, 1>::grid(); break;
    case 11: *p2g = NaKernels<3, 2>::p2g(); *grid = NaKernels<3, 2>::grid(); break;
    // quadratic B-spline (basis 3): dim 1, 2, 3
    case 101: *p2g = NaKernels<1, 3>::p2g(); *grid = NaKernels<1, 3>::grid(); break;
    case 102: *p2g = NaKernels<2, 3>::p2g(); *grid = NaKernels<2, 3>::grid(); break;
    default: *p2g = NaKernels<3, 3>::p2g(); *grid = NaKernels<3, 3>::grid(); break;
  }
}

int set_err(char *err, int errlen, int code, const char *msg) {
  if (err && errlen > 0) {
    std::strncpy(err, msg, errlen - 1);
    err[errlen - 1] = 0;
  }
  return code;
}

}  // namespace
}  // namespace kmpm

using namespace kmpm;

extern "C" int kmpm_p2g_mass_noalloc(const float *x, const float *mass, int n, int dim, int basis, const double lo[3],
                                     double cellsize, const int nnodes[3], const int nglobal[3], float *node_mass,
                                     void *stream, char *err, int errlen) {
  if (!x || !mass || !node_mass || !lo || !nnodes || !nglobal || n < 0 || dim < 1 || dim > 3 || basis < 0 ||
      basis > 3 || !(cellsize > 0))
    return set_err(err, errlen, KMPM_ERR_ARG, "kmpm_p2g_mass_noalloc: bad argument");
  if (n > KMPM_NOALLOC_MAX_PARTICLES)
    return set_err(err, errlen, KMPM_ERR_ARG, "kmpm_p2g_mass_noalloc: more particles than KMPM_NOALLOC_MAX_PARTICLES");
  cudaStream_t st = (cudaStream_t)stream;
  // ---- grid and tiles
  int t[3];
  tile_dims(dim, basis, t);
  GridDev g{};
  long long nn = 1, ntiles = 1;
  for (int d = 0; d < 3; d++) {
    g.n[d] = d < dim ? nnodes[d] : 1;
    g.ng[d] = d < dim ? nglobal[d] : 1;
    if (g.n[d] < 1) return set_err(err, errlen, KMPM_ERR_ARG, "kmpm_p2g_mass_noalloc: empty grid");
    g.lo[d] = (float)lo[d];
    const int nc = d < dim ? (basis == 2 ? (g.n[d] + 1) / 2 : g.n[d]) : 1;
    g.ncell[d] = nc;
    g.ntile[d] = d < dim ? (nc + t[d] - 1) / t[d] : 1;
    nn *= g.n[d];
    ntiles *= g.ntile[d];
  }
  g.cellsize = (float)cellsize;
  g.inv_cellsize = (float)(1.0 / cellsize);
  const long long ncpt = (long long)t[0] * t[1] * t[2];
  const long long ncells = ntiles * ncpt;
  if (ncells > KMPM_NOALLOC_MAX_CELLS)
    return set_err(err, errlen, KMPM_ERR_ARG, "kmpm_p2g_mass_noalloc: grid has more cells than KMPM_NOALLOC_MAX_CELLS");
  const int S = stencil_width(basis), SC = stencil_sc(basis);
  long long NW = 1;
  for (int d = 0; d < dim; d++) NW *= (long long)(t[d] - 1) * SC + S;
  // ---- scratch base on this device (looked up once per device)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return set_err(err, errlen, KMPM_ERR_CUDA, "kmpm_p2g_mass_noalloc: no current CUDA device");
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_base[dev]) {
      void *ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) return set_err(err, errlen, KMPM_ERR_CUDA, cudaGetErrorString(e));
      g_base[dev] = (unsigned char *)ptr;
    }
    base = g_base[dev];
  }
  // ---- carve the scratch
  const size_t ps = align256((size_t)std::max(n, 1) * sizeof(float)) / sizeof(float);
  const int nblk_rs = (n + 2047) / 2048 + 1;
  Carve cv;
  float **pp = cv.take<float *>(base, 2);
  StepScalars *sc = cv.take<StepScalars>(base, 1);
  GridDev *gd = cv.take<GridDev>(base, 1);
  int *bad = cv.take<int>(base, 1);
  float *P = cv.take<float>(base, ps * (PF_MASS + 1));
  int *keys = cv.take<int>(base, n + 1), *vals = cv.take<int>(base, n + 1);
  RadixTemp rt{};
  rt.k1 = cv.take<int>(base, n + 1);
  rt.v1 = cv.take<int>(base, n + 1);
  rt.hist = cv.take<int>(base, 256 * (size_t)nblk_rs);
  rt.tot = cv.take<int>(base, 256);
  int *cs = cv.take<int>(base, ncells), *ce = cv.take<int>(base, ncells);
  int *ts = cv.take<int>(base, ntiles), *te = cv.take<int>(base, ntiles);
  int2 *tiles = cv.take<int2>(base, ntiles);
  float *partial = cv.take<float>(base, (size_t)ntiles * NW);
  if (cv.off > kScratchBytes)
    return set_err(err, errlen, KMPM_ERR_ARG, "kmpm_p2g_mass_noalloc: problem exceeds KMPM_NOALLOC_SCRATCH_BYTES");
  // ---- work (all on the caller's stream)
#define NA_CK(call)                                                                 \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) return set_err(err, errlen, KMPM_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)
  k_na_init<<<1, 1, 0, st>>>(g, gd, pp, P, sc, bad);
  // the previous call's cell and tile ranges must not leak into this one
  NA_CK(cudaMemsetAsync(cs, 0, sizeof(int) * ncells, st));
  NA_CK(cudaMemsetAsync(ce, 0, sizeof(int) * ncells, st));
  NA_CK(cudaMemsetAsync(ts, 0, sizeof(int) * ntiles, st));
  NA_CK(cudaMemsetAsync(te, 0, sizeof(int) * ntiles, st));
  if (n > 0) {
    k_na_keys<<<(n + 255) / 256, 256, 0, st>>>(x, n, g, dim, t[0], t[1], t[2], keys, vals, bad);
    int key_bits = 1;
    while ((1LL << key_bits) < ncells) key_bits++;
    radix_sort(keys, vals, n, key_bits, rt, st);
    k_na_gather<<<(n + 255) / 256, 256, 0, st>>>(x, mass, vals, n, P, ps);
    launch_cell_ranges(keys, 0, n, (int)ncpt, cs, ce, ts, te, st);
  }
  k_na_tiles<<<(int)((ntiles + 255) / 256), 256, 0, st>>>(tiles, (int)ntiles);
  void *kp2g = nullptr, *kgrid = nullptr;
  na_kernels(dim, basis, &kp2g, &kgrid);
  const int smem = p2g_smem_bytes(dim, basis, P2G_MASS, false);
  NA_CK(cudaFuncSetAttribute(kp2g, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  P2GArgs pa{};
  pa.Pp = pp;
  pa.ps = ps;
  pa.pos_field = PF_X0;
  pa.tiles = tiles;
  pa.grids = gd;
  pa.cell_start = cs;
  pa.cell_end = ce;
  pa.partial = partial;
  pa.pstride_tile = (size_t)NW;
  pa.tile_start = ts;
  pa.tile_end = te;
  pa.scalars = sc;
  {
    void *args[] = {&pa};
    NA_CK(cudaLaunchKernel(kp2g, dim3((unsigned)ntiles), dim3(256), args, smem, st));
  }
  GridArgs ga{};
  ga.grids = gd;
  ga.partial = partial;
  ga.pstride_tile = (size_t)NW;
  ga.tile_start = ts;
  ga.tile_end = te;
  ga.scalars = sc;
  {
    void *args[] = {&ga, &gd, &node_mass};
    NA_CK(cudaLaunchKernel(kgrid, dim3((unsigned)((nn + 255) / 256)), dim3(256), args, 0, st));
  }
  NA_CK(cudaGetLastError());
  // the count of particles outside the grid decides the status: wait for the
  // work and read it back (a four-byte copy into this stack frame)
  int nbad = 0;
  NA_CK(cudaMemcpyAsync(&nbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
#undef NA_CK
  if (nbad > 0) {
    char msg[160];
    std::snprintf(msg, sizeof msg, "kmpm_p2g_mass_noalloc: %d particle(s) outside the grid's cells", nbad);
    return set_err(err, errlen, KMPM_ERR_LEFT_DOMAIN, msg);
  }
  return KMPM_OK;
}
