// kmpm_rebin.cu -- ULMPM's per-step re-binning as an update of the previous
// binning.
//
// compute_grid_weight_functions_and_gradients (src/ulmpm.cpp:88-337)
// rebuilds every particle's node list each step.  Here the particles are
// kept sorted by cell (tile-major keys), and each step sorts them again by
// the cell of their new position, stably: particles of one cell keep their
// slot order, so every sum over a cell runs in a fixed order.
//
// Between two steps few particles cross a cell face.  Those that do are the
// "movers"; the others ("stayers") keep their key, so the stayers are still
// sorted by key in slot order.  The stable sort puts the particle of slot i
// and cell k at
//     (particles with cell < k) + (particles with cell k and slot < i),
// the first term being the exclusive prefix of the new per-cell counts, the
// second
//     clamp(stayers before slot i - stayers with cell < k, 0, stayers in k)
//   + (movers into k with slot < i).
// The new counts are the old ones (cell_end - cell_start) minus the movers
// out plus the movers in.  So the permutation is the one a stable LSD radix
// sort of the new keys gives, from streaming passes over the slots and the
// cells plus work on the movers alone.  On entry keys and the cell ranges
// must describe one binning of the current order (any sorted keys with their
// own ranges: the update stays exact, only more particles count as movers).
//
// Kernels, one launch each:
//   keys    new key per slot, mover bits, per-cell in / out counts (atomics
//           on movers only), movers per 256 slots;
//   count   per chunk of cells: sums of the new counts and of the movers in;
//   scan    one block: exclusive scans of the chunk sums and of the slot
//           blocks' mover counts;
//   ranges  per chunk: new cell and tile ranges, prefix of movers in; clears
//           the out counts;
//   group   movers into their destination cell's group (atomic slot, which
//           also clears the in counts);
//   order   each group sorted by slot (rank = members with a smaller slot);
//   place   destination of every slot; writes perm and the sorted keys.
#include "kmpm_kernels.cuh"

namespace kmpm {

namespace {

__device__ __forceinline__ int warp_excl_scan(int v, int lane, int &total) {
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

// exclusive scan of one value per thread over the block (NT threads, NT/32
// warps <= 32); every thread gets its prefix and the block total
template <int NT>
__device__ __forceinline__ int block_excl_scan(int v, int *sw, int &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int wt;
  const int ex = warp_excl_scan(v, lane, wt);
  if (lane == 0) sw[warp] = wt;
  __syncthreads();
  if (warp == 0) {
    const int w = lane < NT / 32 ? sw[lane] : 0;
    int t;
    const int wex = warp_excl_scan(w, lane, t);
    if (lane < NT / 32) sw[lane] = wex;
    if (lane == 0) sw[32] = t;
  }
  __syncthreads();
  const int r = ex + sw[warp];
  total = sw[32];
  __syncthreads();
  return r;
}

__device__ __forceinline__ int4 ld4(const int *p) { return *reinterpret_cast<const int4 *>(p); }
__device__ __forceinline__ void st4(int *p, int4 v) { *reinterpret_cast<int4 *>(p) = v; }
__device__ __forceinline__ int comp(const int4 &v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }

__global__ void __launch_bounds__(256) k_rebin_keys(RebinArgs r) {
  if (run_finished(r.pa.scalars)) return;
  const int i = blockIdx.x * 256 + threadIdx.x;
  const bool valid = i < r.n;
  int knew = 0, kold = 0;
  if (valid) {
    const GridDev &g = r.pa.grids[r.grid];
    const float *P = *r.pa.Pp;
    const size_t ps = r.pa.ps, p = (size_t)r.start + i;
    float x[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < 3; d++)
      if (d < r.pa.dim) x[d] = P[(PF_X0 + d) * ps + p] + P[(PF_XN + d) * ps + p];
    knew = cell_key(g, r.pa.tile_t[0], r.pa.tile_t[1], r.pa.tile_t[2], x, r.pa.dim);
    kold = r.keys[i];
    r.knew[i] = knew;
  }
  const bool mover = valid && knew != kold;
  const unsigned b = __ballot_sync(0xffffffffu, mover);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) r.mflag[i >> 5] = b;
  if (mover) {
    // one atomic per distinct cell of the warp (on the first step every
    // mover leaves cell 0)
    const unsigned act = __activemask();
    const unsigned pin = __match_any_sync(act, knew), pout = __match_any_sync(act, kold);
    if (lane == __ffs(pin) - 1) atomicAdd(&r.cin[knew], __popc(pin));
    if (lane == __ffs(pout) - 1) atomicAdd(&r.cout[kold], __popc(pout));
  }
  __shared__ int wc[8];
  if (lane == 0) wc[warp] = __popc(b);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
#pragma unroll
    for (int w = 0; w < 8; w++) s += wc[w];
    r.blkm[blockIdx.x] = s;
  }
}

// this thread's cells [c0, c0 + 16): new counts and movers in
__device__ __forceinline__ void cell_counts(const RebinArgs &r, int c0, int nc[RB_CELLS_PER_THREAD],
                                            int mi[RB_CELLS_PER_THREAD]) {
#pragma unroll
  for (int q = 0; q < RB_CELLS_PER_THREAD / 4; q++) {
    const int4 s = ld4(r.cell_start + c0 + 4 * q), e = ld4(r.cell_end + c0 + 4 * q);
    const int4 in = ld4(r.cin + c0 + 4 * q), out = ld4(r.cout + c0 + 4 * q);
#pragma unroll
    for (int j = 0; j < 4; j++) {
      mi[4 * q + j] = comp(in, j);
      nc[4 * q + j] = comp(e, j) - comp(s, j) - comp(out, j) + comp(in, j);
    }
  }
}

__global__ void __launch_bounds__(256) k_rebin_count(RebinArgs r) {
  if (run_finished(r.pa.scalars)) return;
  __shared__ int sw[33];
  const int c0 = blockIdx.x * RB_CHUNK + threadIdx.x * RB_CELLS_PER_THREAD;
  int nc[RB_CELLS_PER_THREAD], mi[RB_CELLS_PER_THREAD];
  cell_counts(r, c0, nc, mi);
  int sn = 0, sm = 0;
#pragma unroll
  for (int u = 0; u < RB_CELLS_PER_THREAD; u++) { sn += nc[u]; sm += mi[u]; }
  int tn, tm;
  block_excl_scan<256>(sn, sw, tn);
  block_excl_scan<256>(sm, sw, tm);
  if (threadIdx.x == 0) {
    r.bsum[2 * blockIdx.x] = tn;
    r.bsum[2 * blockIdx.x + 1] = tm;
  }
}

// exclusive scans in place by one block of 1024 threads, one int4 per thread
// per 4096-int tile (coalesced), with the running total carried across tiles.
// The arrays are padded to whole tiles; entries past the valid range only
// follow it, so whatever they hold does not change its prefixes.
__device__ void scan_ints(int *a, int n, int *sw) {
  int carry = 0;
  for (int base = 0; base < n; base += 4096) {
    const int4 v = ld4(a + base + 4 * threadIdx.x);
    int tot;
    const int e = block_excl_scan<1024>(v.x + v.y + v.z + v.w, sw, tot) + carry;
    st4(a + base + 4 * threadIdx.x, make_int4(e, e + v.x, e + v.x + v.y, e + v.x + v.y + v.z));
    carry += tot;
  }
}
// the same over pairs (a[2k], a[2k+1]), scanned as two sequences
__device__ void scan_pairs(int *a, int npairs, int *sw) {
  int c0 = 0, c1 = 0;
  for (int base = 0; base < npairs; base += 2048) {
    const int4 v = ld4(a + 2 * base + 4 * threadIdx.x);  // pairs base + 2t and base + 2t + 1
    int t0, t1;
    const int e0 = block_excl_scan<1024>(v.x + v.z, sw, t0) + c0;
    const int e1 = block_excl_scan<1024>(v.y + v.w, sw, t1) + c1;
    st4(a + 2 * base + 4 * threadIdx.x, make_int4(e0, e1, e0 + v.x, e1 + v.y));
    c0 += t0;
    c1 += t1;
  }
}

__global__ void __launch_bounds__(1024) k_rebin_scan(RebinArgs r, int nchunk, int nblk) {
  if (run_finished(r.pa.scalars)) return;
  __shared__ int sw[33];
  scan_pairs(r.bsum, nchunk, sw);
  scan_ints(r.blkm, nblk, sw);
}

__global__ void __launch_bounds__(256) k_rebin_ranges(RebinArgs r) {
  if (run_finished(r.pa.scalars)) return;
  __shared__ int sw[33];
  const int c0 = blockIdx.x * RB_CHUNK + threadIdx.x * RB_CELLS_PER_THREAD;
  int nc[RB_CELLS_PER_THREAD], mi[RB_CELLS_PER_THREAD];
  cell_counts(r, c0, nc, mi);
  int sn = 0, sm = 0;
#pragma unroll
  for (int u = 0; u < RB_CELLS_PER_THREAD; u++) { sn += nc[u]; sm += mi[u]; }
  int tn, tm;
  int pn = block_excl_scan<256>(sn, sw, tn) + r.bsum[2 * blockIdx.x] + r.start;
  int pm = block_excl_scan<256>(sm, sw, tm) + r.bsum[2 * blockIdx.x + 1];
  const int4 zero = make_int4(0, 0, 0, 0);
#pragma unroll
  for (int q = 0; q < RB_CELLS_PER_THREAD / 4; q++) {
    int s[4], e[4], m[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int u = 4 * q + j, k = c0 + u;
      s[j] = pn;
      e[j] = pn + nc[u];
      m[j] = pm;
      if (k < r.ncell) {
        if (k % r.ncpt == 0) r.tile_start[k / r.ncpt] = s[j];
        if (k % r.ncpt == r.ncpt - 1) r.tile_end[k / r.ncpt] = e[j];
      }
      pn += nc[u];
      pm += mi[u];
    }
    st4(r.cell_start + c0 + 4 * q, make_int4(s[0], s[1], s[2], s[3]));
    st4(r.cell_end + c0 + 4 * q, make_int4(e[0], e[1], e[2], e[3]));
    st4(r.mpre + c0 + 4 * q, make_int4(m[0], m[1], m[2], m[3]));
    st4(r.cout + c0 + 4 * q, zero);
  }
}

__global__ void __launch_bounds__(256) k_rebin_group(RebinArgs r) {
  if (run_finished(r.pa.scalars)) return;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= r.n) return;
  if (!((r.mflag[i >> 5] >> (i & 31)) & 1u)) return;
  const int k = r.knew[i];
  r.brun[r.mpre[k] + atomicSub(&r.cin[k], 1) - 1] = i;
}

__global__ void __launch_bounds__(256) k_rebin_order(RebinArgs r) {
  if (run_finished(r.pa.scalars)) return;
  const int m = r.mpre[r.ncell];  // movers in all cells (the padding cells have none)
  for (int j = blockIdx.x * 256 + threadIdx.x; j < m; j += gridDim.x * 256) {
    const int s = r.brun[j];
    const int k = r.knew[s];
    const int a = r.mpre[k], e = r.mpre[k + 1];
    int rank = 0;
    for (int q = a; q < e; q++) rank += r.brun[q] < s;
    r.bsort[a + rank] = s;
  }
}

__global__ void __launch_bounds__(256) k_rebin_place(RebinArgs r) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (run_finished(r.pa.scalars)) {  // the run has ended: keep the order
    if (i < r.n) r.perm[i] = i;
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned w = r.mflag[i >> 5];
  __shared__ int wc[8];
  if (lane == 0) wc[warp] = __popc(w);
  __syncthreads();
  int before = r.blkm[blockIdx.x] + __popc(w & ((1u << lane) - 1u));
  for (int q = 0; q < warp; q++) before += wc[q];
  if (i >= r.n) return;
  const int k = r.knew[i];
  const int cs = r.cell_start[k] - r.start, cnt = r.cell_end[k] - r.cell_start[k];
  const int mp = r.mpre[k], mc = r.mpre[k + 1] - mp;
  // stayers of cell k before slot i, then movers into k with a smaller slot
  const int a = min(max((i - before) - (cs - mp), 0), cnt - mc);
  int b = 0;
  for (int q = mp; q < mp + mc && r.bsort[q] < i; q++) b++;
  const int pos = cs + a + b;
  r.perm[pos] = i;
  r.keys[pos] = k;
}

}  // namespace

int launch_rebin(const RebinArgs &r, cudaStream_t st) {
  if (r.n <= 0) return 0;
  const int nblk = (r.n + 255) / 256;
  const int nchunk = r.ncell_pad / RB_CHUNK;
  k_rebin_keys<<<nblk, 256, 0, st>>>(r);
  k_rebin_count<<<nchunk, 256, 0, st>>>(r);
  k_rebin_scan<<<1, 1024, 0, st>>>(r, nchunk, nblk);
  k_rebin_ranges<<<nchunk, 256, 0, st>>>(r);
  k_rebin_group<<<nblk, 256, 0, st>>>(r);
  k_rebin_order<<<min(nblk, 152 * 8), 256, 0, st>>>(r);
  k_rebin_place<<<nblk, 256, 0, st>>>(r);
  return 7;
}

}  // namespace kmpm
