// The learned return map's network object: parameters, normalisation,
// training on the GPU (hand-written FP32 forward / backward / Adam kernels),
// FP32 and tensor-core (BF16, tcgen05) inference, and the device image that
// the learned G2P kernel loads.  No counterpart in the reference: Karamelo
// evaluates StrengthJohnsonCook::update_deviatoric_stress
// (src/strength_jc.cpp:100-184) directly.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/kmpm.h"
#include "kmpm_mlp.cuh"

namespace kmpm {
namespace mlp {

// flat FP32 parameter vector: W1[128x15] b1 W2[128x128] b2 W3[128x128] b3 W4[7x128] b4
constexpr int O_W1 = 0, O_B1 = O_W1 + HID * NIN, O_W2 = O_B1 + HID, O_B2 = O_W2 + HID * HID, O_W3 = O_B2 + HID,
              O_B3 = O_W3 + HID * HID, O_W4 = O_B3 + HID, O_B4 = O_W4 + NOUT * HID;
static_assert(O_B4 + NOUT == NPARAMS, "parameter layout");
constexpr int LAYER_IN[4] = {NIN, HID, HID, HID}, LAYER_OUT[4] = {HID, HID, HID, NOUT};
constexpr int O_W[4] = {O_W1, O_W2, O_W3, O_W4}, O_B[4] = {O_B1, O_B2, O_B3, O_B4};

// ------------------------------------------------------------------ kernels
// C[M x N] = op(A) op(B) (+ epilogue), row-major, 64 x 64 tiles, 4 x 4 per thread.
//   A(m,k) = TA ? A[k lda + m] : A[m lda + k];  B(k,n) = TB ? B[n ldb + k] : B[k ldb + n]
// EPI 0: store; 1: + bias, ReLU; 2: + bias; 3: * (mask > 0) (ReLU backward)
template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float *__restrict__ A, int lda,
                                              const float *__restrict__ B, int ldb, float *__restrict__ C, int ldc,
                                              const float *__restrict__ bias, const float *__restrict__ mask, int ldm) {
  __shared__ float As[16][64 + 4], Bs[16][64 + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int lin = threadIdx.x + 256 * e;
      int m, k;
      if (TA) { k = lin >> 6; m = lin & 63; } else { m = lin >> 4; k = lin & 15; }
      const int gm = m0 + m, gk = k0 + k;
      As[k][m] = (gm < M && gk < K) ? (TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk]) : 0.f;
      int n, kb;
      if (TB) { n = lin >> 4; kb = lin & 15; } else { kb = lin >> 6; n = lin & 63; }
      const int gn = n0 + n, gkb = k0 + kb;
      Bs[kb][n] = (gn < N && gkb < K) ? (TB ? B[(size_t)gn * ldb + gkb] : B[(size_t)gkb * ldb + gn]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (EPI == 1) v = fmaxf(v + bias[gn], 0.f);
      if (EPI == 2) v += bias[gn];
      if (EPI == 3) v = mask[(size_t)gm * ldm + gn] > 0.f ? v : 0.f;
      C[(size_t)gm * ldc + gn] = v;
    }
  }
}

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// normalised batch: rows drawn with replacement (idx = hash(seed, step, i) mod n)
// or, when step < 0, rows [first, first + B) in order
__global__ void k_batch(const float *__restrict__ X, const float *__restrict__ Y, long long n, int B, long long first,
                        unsigned long long seed, long long step, const float *__restrict__ norm, float *Xb, float *Yb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const long long r = step < 0 ? first + i : (long long)(splitmix64(seed ^ splitmix64((unsigned long long)step * 0x100000001ull + i)) % (unsigned long long)n);
  const float *in_mean = norm, *in_std = norm + NIN, *out_mean = norm + 2 * NIN, *out_scale = norm + 2 * NIN + NOUT;
#pragma unroll
  for (int j = 0; j < NIN; j++) {
    const float s = in_std[j];
    Xb[(size_t)i * NIN + j] = s > 0.f ? (X[r * NIN + j] - in_mean[j]) / s : 0.f;
  }
  if (Y)
#pragma unroll
    for (int j = 0; j < NOUT; j++) Yb[(size_t)i * NOUT + j] = (Y[r * NOUT + j] - out_mean[j]) / out_scale[j];
}

// dZ4 = 2 (Yh - Y) / (B NOUT); per-block partial sums of the squared error
__global__ void k_loss(const float *__restrict__ Yh, const float *__restrict__ Yb, int B, float *dZ, float *partial) {
  __shared__ float red[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float e2 = 0.f;
  if (i < B * NOUT) {
    const float d = Yh[i] - Yb[i];
    dZ[i] = 2.f * d / (float)(B * NOUT);
    e2 = d * d;
  }
  red[threadIdx.x] = e2;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// column sums of dZ [M x N] in two fixed-order passes (bias gradients)
__global__ void k_colsum_part(const float *__restrict__ dZ, int M, int N, int rows_per, float *part) {
  const int n = threadIdx.x + blockDim.x * blockIdx.y;
  if (n >= N) return;
  const int r0 = blockIdx.x * rows_per, r1 = min(M, r0 + rows_per);
  float s = 0.f;
  for (int r = r0; r < r1; r++) s += dZ[(size_t)r * N + n];
  part[(size_t)blockIdx.x * N + n] = s;
}
__global__ void k_colsum_final(const float *__restrict__ part, int nparts, int N, float *out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int q = 0; q < nparts; q++) s += part[(size_t)q * N + n];
  out[n] = s;
}

__global__ void k_adam(int n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// denormalise FP32 predictions
__global__ void k_denorm(const float *__restrict__ Yh, int B, const float *__restrict__ norm, float *Y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * NOUT) return;
  const int j = i % NOUT;
  Y[i] = Yh[i] * norm[2 * NIN + NOUT + j] + norm[2 * NIN + j];
}

// tensor-core inference of raw inputs (one row per thread, NTILE M-tiles per CTA)
template <int NTILE>
__global__ void __launch_bounds__(NTILE * 128, 1)
    k_mlp_infer(const unsigned char *blob, const float *__restrict__ X, long long n, float *__restrict__ Y,
                signed char *inside_out, int *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  TileCtx t;
  tile_begin<NTILE>(t, smem, blob);
  bool wready = false;
  tile_weights_ready(t, wready);
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  float x[NIN];
#pragma unroll
  for (int j = 0; j < NIN; j++) x[j] = active ? X[i * NIN + j] : 0.f;
  const bool inside = tile_put_features(t, x, active);
  float y[NOUT];
  const bool ok = t.ok && tile_forward<NTILE>(t, y);
  if (active && ok) {
#pragma unroll
    for (int j = 0; j < NOUT; j++) Y[i * NOUT + j] = y[j];
    if (inside_out) inside_out[i] = inside ? 1 : 0;
  }
  if (!ok && threadIdx.x == 0) atomicExch(status, 1);
  tile_end<NTILE>(t);
}

// ------------------------------------------------------------------ host
uint16_t bf16_bits(float f) {  // round to nearest even
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x7FFFFFu)) return 0x7FC0;
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

void build_blob(const float *params, const float *norm, std::vector<unsigned char> &blob) {
  blob.assign(BLOB_BYTES, 0);
  auto put = [&](int off, int r, int k, int K, float v) {
    const uint16_t b = bf16_bits(v);
    std::memcpy(&blob[off + canon_off(r, k, K)], &b, 2);
  };
  auto bf = [](float v) {
    const uint32_t u = (uint32_t)bf16_bits(v) << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
  };
  for (int r = 0; r < HID; r++) {
    // layer 1, hi/lo split (kmpm_mlp.cuh): [w_hi, b_hi | w_hi, 0 | w_lo, b_lo]
    for (int k = 0; k <= NIN; k++) {
      const float w = k < NIN ? params[O_W1 + r * NIN + k] : params[O_B1 + r];
      const float whi = bf(w), wlo = w - whi;
      put(W1_OFF, r, k, K1, whi);
      if (k < NIN) put(W1_OFF, r, 16 + k, K1, whi);
      put(W1_OFF, r, 32 + k, K1, wlo);
    }
    for (int k = 0; k < HID; k++) {
      put(W2_OFF, r, k, HID, params[O_W2 + r * HID + k]);
      put(W3_OFF, r, k, HID, params[O_W3 + r * HID + k]);
    }
  }
  for (int r = 0; r < N4; r++)
    for (int k = 0; k < HID; k++) put(W4_OFF, r, k, HID, r < NOUT ? params[O_W4 + r * HID + k] : 0.f);
  std::vector<float> par(NPAR, 0.f);
  for (int j = 0; j < HID; j++) { par[P_B2 + j] = params[O_B2 + j]; par[P_B3 + j] = params[O_B3 + j]; }
  for (int j = 0; j < NOUT; j++) par[P_B4 + j] = params[O_B4 + j];
  const float *in_mean = norm, *in_std = norm + NIN, *out_mean = norm + 2 * NIN, *out_scale = norm + 2 * NIN + NOUT;
  const float *env_lo = norm + 2 * NIN + 2 * NOUT, *env_hi = env_lo + NIN;
  for (int j = 0; j < NIN; j++) {
    par[P_IN_MEAN + j] = in_mean[j];
    par[P_IN_ISTD + j] = in_std[j] > 0.f ? 1.f / in_std[j] : 0.f;
    par[P_ENV_LO + j] = env_lo[j];
    par[P_ENV_HI + j] = env_hi[j];
  }
  for (int j = 0; j < NOUT; j++) { par[P_OUT_MEAN + j] = out_mean[j]; par[P_OUT_SCALE + j] = out_scale[j]; }
  std::memcpy(&blob[PAR_OFF], par.data(), NPAR * 4);
}

}  // namespace mlp
}  // namespace kmpm

using namespace kmpm::mlp;

struct kmpm_mlp {
  std::string err;
  cudaStream_t st = nullptr;
  int cap = 0;  // batch rows
  float *d_par = nullptr, *d_grad = nullptr, *d_m = nullptr, *d_v = nullptr, *d_norm = nullptr;
  float *d_xb = nullptr, *d_yb = nullptr, *d_a[3] = {nullptr, nullptr, nullptr}, *d_yh = nullptr;
  float *d_dz[2] = {nullptr, nullptr}, *d_dz4 = nullptr, *d_part = nullptr, *d_cpart = nullptr;
  unsigned char *d_blob = nullptr;
  int *d_status = nullptr;
  long long adam_t = 0;
  bool norm_set = false, blob_valid = false;
};

namespace {
int mfail(kmpm_mlp *m, int code, const std::string &msg) {
  if (m) m->err = msg;
  return code;
}
#define MCK(x)                                                                          \
  do {                                                                                  \
    cudaError_t e_ = (x);                                                               \
    if (e_ != cudaSuccess) return mfail(m, KMPM_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

constexpr int CPART_ROWS = 128;

void gemm(cudaStream_t st, bool ta, bool tb, int epi, int M, int N, int K, const float *A, int lda, const float *B,
          int ldb, float *C, int ldc, const float *bias = nullptr, const float *mask = nullptr, int ldm = 0) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
#define KMPM_GEMM(TA, TB, E) k_gemm<TA, TB, E><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, mask, ldm)
  if (!ta && tb) {
    if (epi == 1) KMPM_GEMM(false, true, 1);
    else if (epi == 2) KMPM_GEMM(false, true, 2);
    else KMPM_GEMM(false, true, 0);
  } else if (!ta && !tb) {
    if (epi == 3) KMPM_GEMM(false, false, 3);
    else KMPM_GEMM(false, false, 0);
  } else {
    KMPM_GEMM(true, false, 0);
  }
#undef KMPM_GEMM
}

// forward over B normalised rows in d_xb: activations in d_a[0..2], output in d_yh
void forward(kmpm_mlp *m, int B) {
  const float *in = m->d_xb;
  for (int l = 0; l < 3; l++) {
    gemm(m->st, false, true, 1, B, HID, LAYER_IN[l], in, LAYER_IN[l], m->d_par + O_W[l], LAYER_IN[l], m->d_a[l], HID,
         m->d_par + O_B[l]);
    in = m->d_a[l];
  }
  gemm(m->st, false, true, 2, B, NOUT, HID, in, HID, m->d_par + O_W4, HID, m->d_yh, NOUT, m->d_par + O_B4);
}

void colsum(kmpm_mlp *m, const float *dZ, int B, int N, float *out) {
  const int nparts = (B + CPART_ROWS - 1) / CPART_ROWS;
  k_colsum_part<<<dim3(nparts, (N + 127) / 128), 128, 0, m->st>>>(dZ, B, N, CPART_ROWS, m->d_cpart);
  k_colsum_final<<<(N + 127) / 128, 128, 0, m->st>>>(m->d_cpart, nparts, N, out);
}

// loss over the batch in d_xb / d_yb, gradients into d_grad
void backward(kmpm_mlp *m, int B) {
  k_loss<<<(B * NOUT + 255) / 256, 256, 0, m->st>>>(m->d_yh, m->d_yb, B, m->d_dz4, m->d_part);
  const float *dz = m->d_dz4;
  int nout = NOUT;
  for (int l = 3; l >= 0; l--) {
    const float *ain = l == 0 ? m->d_xb : m->d_a[l - 1];
    const int nin = LAYER_IN[l];
    // dW = dZ^T A_in, db = column sums of dZ
    gemm(m->st, true, false, 0, nout, nin, B, dz, nout, ain, nin, m->d_grad + O_W[l], nin);
    colsum(m, dz, B, nout, m->d_grad + O_B[l]);
    if (l == 0) break;
    // dZ_prev = (dZ W) * (A_in > 0)
    float *dzp = m->d_dz[l & 1];
    gemm(m->st, false, false, 3, B, nin, nout, dz, nout, m->d_par + O_W[l], nin, dzp, nin, nullptr, ain, nin);
    dz = dzp;
    nout = nin;
  }
}

int ensure_blob(kmpm_mlp *m) {
  if (m->blob_valid) return KMPM_OK;
  std::vector<float> par(NPARAMS), norm(NNORM);
  MCK(cudaMemcpyAsync(par.data(), m->d_par, sizeof(float) * NPARAMS, cudaMemcpyDeviceToHost, m->st));
  MCK(cudaMemcpyAsync(norm.data(), m->d_norm, sizeof(float) * NNORM, cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  std::vector<unsigned char> blob;
  build_blob(par.data(), norm.data(), blob);
  MCK(cudaMemcpyAsync(m->d_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, m->st));
  MCK(cudaStreamSynchronize(m->st));
  m->blob_valid = true;
  return KMPM_OK;
}
}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

int kmpm_mlp_create(int batch, kmpm_mlp **out) {
  if (!out || batch < 1 || batch > (1 << 20)) return KMPM_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return KMPM_ERR_CUDA;
  kmpm_mlp *m = new kmpm_mlp();
  m->cap = batch;
  MCK(cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking));
  const size_t B = (size_t)batch;
  MCK(cudaMalloc(&m->d_par, sizeof(float) * NPARAMS));
  MCK(cudaMalloc(&m->d_grad, sizeof(float) * NPARAMS));
  MCK(cudaMalloc(&m->d_m, sizeof(float) * NPARAMS));
  MCK(cudaMalloc(&m->d_v, sizeof(float) * NPARAMS));
  MCK(cudaMalloc(&m->d_norm, sizeof(float) * NNORM));
  MCK(cudaMalloc(&m->d_xb, sizeof(float) * B * NIN));
  MCK(cudaMalloc(&m->d_yb, sizeof(float) * B * NOUT));
  for (int l = 0; l < 3; l++) MCK(cudaMalloc(&m->d_a[l], sizeof(float) * B * HID));
  for (int l = 0; l < 2; l++) MCK(cudaMalloc(&m->d_dz[l], sizeof(float) * B * HID));
  MCK(cudaMalloc(&m->d_yh, sizeof(float) * B * NOUT));
  MCK(cudaMalloc(&m->d_dz4, sizeof(float) * B * NOUT));
  MCK(cudaMalloc(&m->d_part, sizeof(float) * ((B * NOUT + 255) / 256)));
  MCK(cudaMalloc(&m->d_cpart, sizeof(float) * ((B + CPART_ROWS - 1) / CPART_ROWS) * HID));
  MCK(cudaMalloc(&m->d_blob, BLOB_BYTES));
  MCK(cudaMalloc(&m->d_status, sizeof(int)));
  MCK(cudaMemsetAsync(m->d_par, 0, sizeof(float) * NPARAMS, m->st));
  MCK(cudaMemsetAsync(m->d_m, 0, sizeof(float) * NPARAMS, m->st));
  MCK(cudaMemsetAsync(m->d_v, 0, sizeof(float) * NPARAMS, m->st));
  // identity normalisation, unbounded envelope
  std::vector<float> norm(NNORM, 0.f);
  for (int j = 0; j < NIN; j++) { norm[NIN + j] = 1.f; norm[2 * NIN + 2 * NOUT + j] = -1e30f; norm[3 * NIN + 2 * NOUT + j] = 1e30f; }
  for (int j = 0; j < NOUT; j++) norm[2 * NIN + NOUT + j] = 1.f;
  MCK(cudaMemcpyAsync(m->d_norm, norm.data(), sizeof(float) * NNORM, cudaMemcpyHostToDevice, m->st));
  MCK(cudaStreamSynchronize(m->st));
  MCK(cudaFuncSetAttribute((const void *)k_mlp_infer<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, Smem<4>::BYTES));
  *out = m;
  return KMPM_OK;
}

void kmpm_mlp_destroy(kmpm_mlp *m) {
  if (!m) return;
  float *bufs[] = {m->d_par, m->d_grad, m->d_m, m->d_v, m->d_norm, m->d_xb, m->d_yb, m->d_a[0], m->d_a[1],
                   m->d_a[2], m->d_yh, m->d_dz[0], m->d_dz[1], m->d_dz4, m->d_part, m->d_cpart};
  for (float *b : bufs)
    if (b) cudaFree(b);
  if (m->d_blob) cudaFree(m->d_blob);
  if (m->d_status) cudaFree(m->d_status);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
}

const char *kmpm_mlp_last_error(const kmpm_mlp *m) { return m ? m->err.c_str() : "null network"; }

int kmpm_mlp_init(kmpm_mlp *m, unsigned long long seed) {
  if (!m) return KMPM_ERR_ARG;
  // He-uniform weights (bound sqrt(6 / fan_in)), zero biases; splitmix64 stream
  std::vector<float> par(NPARAMS, 0.f);
  unsigned long long s = seed;
  auto next = [&s]() {
    s += 0x9E3779B97F4A7C15ull;
    unsigned long long z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < 4; l++) {
    const double bound = std::sqrt(6.0 / LAYER_IN[l]);
    for (int i = 0; i < LAYER_OUT[l] * LAYER_IN[l]; i++) par[O_W[l] + i] = (float)((2.0 * next() - 1.0) * bound);
  }
  MCK(cudaMemcpyAsync(m->d_par, par.data(), sizeof(float) * NPARAMS, cudaMemcpyHostToDevice, m->st));
  MCK(cudaMemsetAsync(m->d_m, 0, sizeof(float) * NPARAMS, m->st));
  MCK(cudaMemsetAsync(m->d_v, 0, sizeof(float) * NPARAMS, m->st));
  MCK(cudaStreamSynchronize(m->st));
  m->adam_t = 0;
  m->blob_valid = false;
  return KMPM_OK;
}

int kmpm_mlp_set_params(kmpm_mlp *m, const float *params) {
  if (!m || !params) return KMPM_ERR_ARG;
  MCK(cudaMemcpyAsync(m->d_par, params, sizeof(float) * NPARAMS, cudaMemcpyHostToDevice, m->st));
  MCK(cudaStreamSynchronize(m->st));
  m->blob_valid = false;
  return KMPM_OK;
}

int kmpm_mlp_get_params(kmpm_mlp *m, float *params) {
  if (!m || !params) return KMPM_ERR_ARG;
  MCK(cudaMemcpyAsync(params, m->d_par, sizeof(float) * NPARAMS, cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  return KMPM_OK;
}

int kmpm_mlp_set_norm(kmpm_mlp *m, const float *norm) {
  if (!m || !norm) return KMPM_ERR_ARG;
  for (int j = 0; j < NOUT; j++)
    if (!(norm[2 * NIN + NOUT + j] > 0.f)) return mfail(m, KMPM_ERR_ARG, "output scales must be positive");
  for (int j = 0; j < NIN; j++)
    if (!(norm[NIN + j] >= 0.f)) return mfail(m, KMPM_ERR_ARG, "input scales must be non-negative");
  MCK(cudaMemcpyAsync(m->d_norm, norm, sizeof(float) * NNORM, cudaMemcpyHostToDevice, m->st));
  MCK(cudaStreamSynchronize(m->st));
  m->norm_set = true;
  m->blob_valid = false;
  return KMPM_OK;
}

int kmpm_mlp_get_norm(kmpm_mlp *m, float *norm) {
  if (!m || !norm) return KMPM_ERR_ARG;
  MCK(cudaMemcpyAsync(norm, m->d_norm, sizeof(float) * NNORM, cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  return KMPM_OK;
}

int kmpm_mlp_loss_grad(kmpm_mlp *m, const float *X, const float *Y, int n, float *loss, float *grad) {
  if (!m || !X || !Y || n < 1 || n > m->cap) return mfail(m, KMPM_ERR_ARG, "n must be in [1, batch]");
  k_batch<<<(n + 255) / 256, 256, 0, m->st>>>(X, Y, n, n, 0, 0, -1, m->d_norm, m->d_xb, m->d_yb);
  forward(m, n);
  backward(m, n);
  MCK(cudaGetLastError());
  const int nb = (n * NOUT + 255) / 256;
  std::vector<float> part(nb);
  MCK(cudaMemcpyAsync(part.data(), m->d_part, sizeof(float) * nb, cudaMemcpyDeviceToHost, m->st));
  if (grad) MCK(cudaMemcpyAsync(grad, m->d_grad, sizeof(float) * NPARAMS, cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  double s = 0;
  for (float v : part) s += v;
  if (loss) *loss = (float)(s / ((double)n * NOUT));
  return KMPM_OK;
}

int kmpm_mlp_train(kmpm_mlp *m, const float *X, const float *Y, long long n, const kmpm_train_opts *o,
                   float *loss_out) {
  if (!m || !X || !Y || !o || n < 1) return mfail(m, KMPM_ERR_ARG, "bad arguments");
  const int B = o->batch;
  if (B < 1 || B > m->cap || o->steps < 1 || !(o->lr > 0)) return mfail(m, KMPM_ERR_ARG, "bad training options");
  const int nb = (B * NOUT + 255) / 256;
  std::vector<float> part(nb);
  double ema = -1;
  for (long long s = 0; s < o->steps; s++) {
    // cosine decay from lr to lr * lr_final_ratio
    const double f = 0.5 * (1.0 + std::cos(M_PI * (double)s / (double)o->steps));
    const float lr = (float)(o->lr * (o->lr_final_ratio + (1.0 - o->lr_final_ratio) * f));
    k_batch<<<(B + 255) / 256, 256, 0, m->st>>>(X, Y, n, B, 0, o->seed, s, m->d_norm, m->d_xb, m->d_yb);
    forward(m, B);
    backward(m, B);
    m->adam_t++;
    const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)m->adam_t)));
    const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)m->adam_t)));
    k_adam<<<(NPARAMS + 255) / 256, 256, 0, m->st>>>(NPARAMS, m->d_par, m->d_grad, m->d_m, m->d_v, lr, 0.9f, 0.999f,
                                                      1e-8f, c1, c2);
    if (s + 1 == o->steps || (o->report_every > 0 && (s + 1) % o->report_every == 0)) {
      MCK(cudaMemcpyAsync(part.data(), m->d_part, sizeof(float) * nb, cudaMemcpyDeviceToHost, m->st));
      MCK(cudaStreamSynchronize(m->st));
      double sum = 0;
      for (float v : part) sum += v;
      const double l = sum / ((double)B * NOUT);
      ema = l;
      if (o->report_every > 0) std::fprintf(stderr, "[kmpm_mlp_train] step %lld loss %.4e lr %.2e\n", s + 1, l, lr);
    }
  }
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(m->st));
  m->blob_valid = false;
  if (loss_out) *loss_out = (float)ema;
  return KMPM_OK;
}

int kmpm_mlp_predict(kmpm_mlp *m, const float *X, long long n, float *Y) {
  if (!m || !X || !Y || n < 0) return KMPM_ERR_ARG;
  for (long long first = 0; first < n; first += m->cap) {
    const int B = (int)std::min<long long>(m->cap, n - first);
    k_batch<<<(B + 255) / 256, 256, 0, m->st>>>(X, nullptr, n, B, first, 0, -1, m->d_norm, m->d_xb, nullptr);
    forward(m, B);
    k_denorm<<<(B * NOUT + 255) / 256, 256, 0, m->st>>>(m->d_yh, B, m->d_norm, Y + first * NOUT);
  }
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(m->st));
  return KMPM_OK;
}

int kmpm_mlp_predict_tc(kmpm_mlp *m, const float *X, long long n, float *Y, signed char *inside) {
  if (!m || !X || !Y || n < 0) return KMPM_ERR_ARG;
  int r = ensure_blob(m);
  if (r != KMPM_OK) return r;
  if (n == 0) return KMPM_OK;
  MCK(cudaMemsetAsync(m->d_status, 0, sizeof(int), m->st));
  const long long nblk = (n + 511) / 512;
  k_mlp_infer<4><<<(unsigned)nblk, 512, Smem<4>::BYTES, m->st>>>(m->d_blob, X, n, Y, inside, m->d_status);
  MCK(cudaGetLastError());
  int status = 0;
  MCK(cudaMemcpyAsync(&status, m->d_status, sizeof(int), cudaMemcpyDeviceToHost, m->st));
  MCK(cudaStreamSynchronize(m->st));
  if (status) return mfail(m, KMPM_ERR_CUDA, "tensor-core inference: an MMA completion wait timed out");
  return KMPM_OK;
}

}  // extern "C"

// blob access for the simulation context (kmpm_set_surrogate)
namespace kmpm {
int mlp_device_blob(kmpm_mlp *m, const unsigned char **blob) {
  int r = ensure_blob(m);
  if (r != KMPM_OK) return r;
  *blob = m->d_blob;
  return KMPM_OK;
}
}  // namespace kmpm
