// Learned Johnson-Cook return map: a 15-128-128-128-7 MLP evaluated on the
// 5th-generation tensor cores (tcgen05.mma kind::f16, BF16 operands, FP32
// accumulators in tensor memory).
//
// The network stands in for the radial return of StrengthJohnsonCook::
// update_deviatoric_stress (src/strength_jc.cpp:100-184) on plastic steps:
//   inputs  (15): strain increment dt*D (6), Cauchy stress before the step (6),
//                 equivalent plastic strain, temperature, log(1 + epsdot_p/epsdot0)
//   outputs  (7): stress correction s_new - s_trial (6), plastic strain increment
// Inputs and outputs are normalised with per-feature affine maps stored with
// the weights.  Hidden layers use ReLU.
//
// Tile scheme (one CTA of NTILE*128 threads): thread i owns particle row
// i % 128 of M-tile i / 128.  Rows are written as BF16 into shared memory in
// the canonical K-major no-swizzle layout (8-row x 16-byte core matrices),
// one elected thread issues tcgen05.mma for every tile and commits to an
// mbarrier, and every warp reads its own 32 TMEM lanes back with tcgen05.ld
// for the bias + ReLU + BF16 epilogue, which becomes the next layer's A
// operand in place.  Waits on mbarriers are bounded.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

#include "kmpm_async.cuh"

namespace kmpm {
namespace mlp {

constexpr int NIN = 15, NOUT = 7, HID = 128;
// Layer 1 runs at ~16-bit input precision with BF16 operands: each normalised
// input x and weight w is split into hi = bf16(x) and lo = bf16(x - hi), and
// the product is accumulated as w_hi x_hi + w_hi x_lo + w_lo x_hi (the lo*lo
// term is below FP32 rounding of the sum).  The K = 48 row of the A operand is
//   [x_hi (15), 1 | x_lo (15), 0 | x_hi (15), 1]
// against the weight row [w_hi, b_hi | w_hi, 0 | w_lo, b_lo].
constexpr int K1 = 48;
constexpr int N4 = 16;  // layer-4 N: 7 outputs padded to the minimum MMA N
constexpr int NPARAMS = HID * NIN + HID + HID * HID + HID + HID * HID + HID + NOUT * HID + NOUT;  // 35975
// normalisation block: in_mean[15] in_std[15] out_mean[7] out_scale[7] env_lo[15] env_hi[15]
constexpr int NNORM = 4 * NIN + 2 * NOUT;  // 74

// ---- device image of the network (global blob == shared-memory image)
constexpr int W1_OFF = 0;                          // [128 x 48]  BF16
constexpr int W2_OFF = W1_OFF + HID * K1 * 2;      // [128 x 128] BF16
constexpr int W3_OFF = W2_OFF + HID * HID * 2;     // [128 x 128] BF16
constexpr int W4_OFF = W3_OFF + HID * HID * 2;     // [16 x 128]  BF16
constexpr int PAR_OFF = W4_OFF + N4 * HID * 2;     // FP32 block below
constexpr int P_B2 = 0, P_B3 = 128, P_B4 = 256, P_IN_MEAN = 272, P_IN_ISTD = 288, P_OUT_MEAN = 304,
              P_OUT_SCALE = 312, P_ENV_LO = 320, P_ENV_HI = 336, NPAR = 352;
constexpr int BLOB_BYTES = PAR_OFF + NPAR * 4;     // 83328
static_assert(BLOB_BYTES % 64 == 0, "blob copied in four 16-byte-multiple pieces");
static_assert(K1 * 128 * 2 <= HID * HID * 2, "layer-1 operand fits the activation buffer");
// ---- shared memory of a tile CTA
constexpr int ACT_OFF = (BLOB_BYTES + 1023) & ~1023;  // per M-tile: [128 x 128] BF16 = 32 KB
constexpr int ACT_BYTES = HID * HID * 2;
template <int NTILE> struct Smem {
  static constexpr int BAR_OFF = ACT_OFF + NTILE * ACT_BYTES;  // wbar, mbar (8 B each), tmem slot
  static constexpr int RED_OFF = BAR_OFF + 32;
  static constexpr int BYTES = RED_OFF + 2 * 32 * 4;
};

// byte offset of element (r, k) of an [R x K] BF16 operand in the canonical
// K-major layout without swizzle: core matrix (r/8, k/8) holds 8 rows of
// 16 bytes; core matrices adjacent in K are 128 B apart (LBO), 8-row groups
// K*16 B apart (SBO)
__host__ __device__ constexpr uint32_t canon_off(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor (tcgen05): start, LBO, SBO in 16-byte
// units, descriptor version 1 at bit 46, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor, kind::f16: D F32 (bit 4), A BF16 (bits 7-9 = 1),
// B BF16 (bits 10-12 = 1), both K-major, N/8 at bit 17, M/16 at bit 24
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// Per-CTA state of a tile kernel: barriers, TMEM base, error flag.
struct TileCtx {
  unsigned char *smem;
  uint32_t s_base, wbar, mbar, tmem;
  uint32_t phase;
  bool ok;
};

// Prologue, executed by every thread of the CTA: barrier init, weight copy
// (cp.async.bulk, completes on wbar), TMEM allocation by warp 0.
template <int NTILE>
__device__ __forceinline__ void tile_begin(TileCtx &t, unsigned char *smem, const unsigned char *blob) {
  using SM = Smem<NTILE>;
  t.smem = smem;
  t.s_base = smem_u32(smem);
  t.wbar = t.s_base + SM::BAR_OFF;
  t.mbar = t.wbar + 8;
  const uint32_t slot = t.wbar + 16;
  t.phase = 0;
  t.ok = true;
  if (threadIdx.x == 0) {
    mbar_init(t.wbar, 1);
    mbar_init(t.mbar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(t.wbar, BLOB_BYTES);
    constexpr uint32_t piece = BLOB_BYTES / 4;
#pragma unroll
    for (int i = 0; i < 4; i++) bulk_g2s(t.s_base + i * piece, blob + i * piece, piece, t.wbar);
  }
  if (threadIdx.x < 32) tmem_alloc(slot, NTILE * 128);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  t.tmem = *reinterpret_cast<volatile uint32_t *>(smem + SM::BAR_OFF + 16);
}

// Wait for the weights (every thread, bounded).  Must run before the CTA
// exits even when no tile is evaluated, so that no copy is left in flight.
__device__ __forceinline__ void tile_weights_ready(TileCtx &t, bool &weights_ready) {
  if (weights_ready) return;
  const bool ok = mbar_wait(t.wbar, 0);
  t.ok = __syncthreads_and(ok) && t.ok;
  weights_ready = true;
}

// Epilogue: free the tensor memory (warp 0) once every warp is done with it.
template <int NTILE>
__device__ __forceinline__ void tile_end(TileCtx &t) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32) tmem_dealloc(t.tmem, NTILE * 128);
}

// This thread's feature row (layer-1 A operand, hi/lo split as above).
// Returns whether every normalised input lies inside the training envelope.
__device__ __forceinline__ bool tile_put_features(TileCtx &t, const float (&x)[NIN], bool active) {
  const float *par = reinterpret_cast<const float *>(t.smem + PAR_OFF);
  float hi[16], lo[16];
  bool inside = true;
#pragma unroll
  for (int j = 0; j < NIN; j++) {
    const float xn = active ? (x[j] - par[P_IN_MEAN + j]) * par[P_IN_ISTD + j] : 0.f;
    inside = inside && xn >= par[P_ENV_LO + j] && xn <= par[P_ENV_HI + j];
    hi[j] = __bfloat162float(__float2bfloat16_rn(xn));
    lo[j] = xn - hi[j];
  }
  hi[NIN] = 1.f;
  lo[NIN] = 0.f;
  const int tile = threadIdx.x >> 7, row = threadIdx.x & 127;
  unsigned char *act = t.smem + ACT_OFF + tile * ACT_BYTES;
#pragma unroll
  for (int part = 0; part < 3; part++) {
    const float *v16 = part == 1 ? lo : hi;
#pragma unroll
    for (int c = 0; c < 2; c++) {
      uint4 v;
      v.x = pack_bf16(v16[8 * c + 0], v16[8 * c + 1]);
      v.y = pack_bf16(v16[8 * c + 2], v16[8 * c + 3]);
      v.z = pack_bf16(v16[8 * c + 4], v16[8 * c + 5]);
      v.w = pack_bf16(v16[8 * c + 6], v16[8 * c + 7]);
      *reinterpret_cast<uint4 *>(act + canon_off(row, 16 * part + 8 * c, K1)) = v;
    }
  }
  fence_proxy_async();
  return inside;
}

// Four layers over every M-tile of the CTA.  Called by all threads; on
// return y holds this thread's de-normalised outputs.  Returns false (for
// every thread) if an MMA completion wait ran out.
template <int NTILE>
__device__ __forceinline__ bool tile_forward(TileCtx &t, float (&y)[NOUT]) {
  const int warp = threadIdx.x >> 5;
  const int tile = warp >> 2, quarter = warp & 3, row = threadIdx.x & 127;
  const float *par = reinterpret_cast<const float *>(t.smem + PAR_OFF);
  unsigned char *act = t.smem + ACT_OFF + tile * ACT_BYTES;
  const uint32_t trow = t.tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(tile * 128);
#pragma unroll 1
  for (int l = 0; l < 4; l++) {
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && t.ok) {
      tc_fence_after();
      const int K = l == 0 ? K1 : HID, N = l == 3 ? N4 : HID;
      const uint32_t woff = l == 0 ? W1_OFF : (l == 1 ? W2_OFF : (l == 2 ? W3_OFF : W4_OFF));
      const uint32_t id = instr_desc(128, N);
#pragma unroll 1
      for (int tt = 0; tt < NTILE; tt++)
#pragma unroll 1
        for (int ks = 0; ks < K / 16; ks++) {
          const uint64_t ad = smem_desc(t.s_base + ACT_OFF + tt * ACT_BYTES + ks * 256, 128, K * 16);
          const uint64_t bd = smem_desc(t.s_base + woff + ks * 256, 128, K * 16);
          mma_bf16(t.tmem + tt * 128, ad, bd, id, ks > 0 ? 1u : 0u);
        }
      mma_commit(t.mbar);
    }
    bool ok = t.ok ? mbar_wait(t.mbar, t.phase) : false;
    t.phase ^= 1u;
    t.ok = __syncthreads_and(ok);
    if (!t.ok) return false;
    tc_fence_after();
    if (l < 3) {
      const float *bias = par + (l == 1 ? P_B2 : P_B3);
#pragma unroll 1
      for (int c = 0; c < 4; c++) {
        uint32_t v[32];
        tmem_ld32(trow + 32 * c, v);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 4; j++) {
          float h[8];
#pragma unroll
          for (int e = 0; e < 8; e++) {
            const float b = l == 0 ? 0.f : bias[32 * c + 8 * j + e];
            h[e] = fmaxf(__uint_as_float(v[8 * j + e]) + b, 0.f);
          }
          uint4 pk;
          pk.x = pack_bf16(h[0], h[1]);
          pk.y = pack_bf16(h[2], h[3]);
          pk.z = pack_bf16(h[4], h[5]);
          pk.w = pack_bf16(h[6], h[7]);
          *reinterpret_cast<uint4 *>(act + canon_off(row, 32 * c + 8 * j, HID)) = pk;
        }
      }
      fence_proxy_async();
    } else {
      uint32_t v[16];
      tmem_ld16(trow, v);
      tmem_wait_ld();
#pragma unroll
      for (int j = 0; j < NOUT; j++)
        y[j] = (__uint_as_float(v[j]) + par[P_B4 + j]) * par[P_OUT_SCALE + j] + par[P_OUT_MEAN + j];
    }
  }
  return true;
}

}  // namespace mlp
}  // namespace kmpm
