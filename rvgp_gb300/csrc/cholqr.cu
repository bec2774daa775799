// Cholesky QR step of the eigensolver's FP32 block in FP32 (internal).
//
// Given the FP64 Gram G = VᵀV of an N x p FP32 block with unit-norm columns,
// V <- V L⁻ᵀ with G = L Lᵀ:
//   chol32_gram   : one CTA factors G (rounded to FP32) in shared memory and
//                   inverts the factor's 32 x 32 diagonal blocks (chol32.cuh);
//   trsm_rows_f32 : row tiles of V solve X Lᵀ = V in place, 32 columns at a
//                   time: X_b = (V_b − X_{<b} L_{b,<b}ᵀ) L_bbᵀ⁻¹, the last
//                   product with the stored diagonal-block inverse.
// FP32 is enough for Cholesky QR run twice when cond(G) stays below ~1e7 (the
// second pass starts from a nearly orthonormal block); a non-positive pivot
// is reported so the caller can repeat the pass with the FP64 factorisation.
#include "common.cuh"
#include "linalg.cuh"
#include "chol32.cuh"

namespace rvgp {
namespace {

constexpr int kCholThreads = 512;
constexpr int kRows = 64;       // rows of V per CTA in the triangular solve
constexpr int kTrsmThreads = 256;
using chol32::FB;

size_t chol_smem(int p) { return sizeof(float) * ((size_t)p * chol32::lda32(p) + p) + 64; }

__global__ void __launch_bounds__(kCholThreads, 1)
    chol32_gram_kernel(const double* __restrict__ G, int p, float* __restrict__ L, float* __restrict__ Mb,
                       int* __restrict__ info) {
  extern __shared__ __align__(16) float A[];
  __shared__ int s_flag;
  const int ld = chol32::lda32(p);
  float* dinvL = A + (size_t)p * ld;
  const int nblk = (p + FB - 1) / FB;
  for (int i = threadIdx.x >> 5; i < p; i += kCholThreads / 32)
    for (int j = threadIdx.x & 31; j <= i; j += 32) A[i * ld + j] = (float)G[(size_t)i * p + j];
  __syncthreads();
  if (!chol32::chol32_cta<kCholThreads>(A, ld, p, dinvL, &s_flag)) {
    if (threadIdx.x == 0) *info = 1;
    return;
  }
  chol32::invert_diag_blocks(A, ld, p, nblk, dinvL);
  __syncthreads();
  for (int i = threadIdx.x >> 5; i < p; i += kCholThreads / 32)
    for (int j = threadIdx.x & 31; j < p; j += 32) L[(size_t)i * p + j] = j <= i ? A[i * ld + j] : 0.f;
  // Mb[b][i][c] (row-major 32 x 32): inverse of diagonal block b, zero-padded
  for (int e = threadIdx.x; e < nblk * FB * FB; e += kCholThreads) {
    const int b = e / (FB * FB), i = (e / FB) % FB, c = e % FB;
    const int j0 = b * FB;
    float v = 0.f;
    if (j0 + i < p && j0 + c < p) v = (c < i) ? A[(j0 + c) * ld + j0 + i] : (c == i ? dinvL[j0 + i] : 0.f);
    Mb[e] = v;
  }
  if (threadIdx.x == 0) *info = 0;
}

// X Lᵀ = V for a tile of kRows rows, in place.  Shared memory: the tile
// (kRows x ldx), the current block row of L (32 x lds) and the diagonal-block
// inverse (32 x 33).  Thread (r, cg) owns rows {r, r+32} x columns cg*4..+3 of
// the current 32-column panel.
__global__ void __launch_bounds__(kTrsmThreads)
    trsm_rows_kernel(float* __restrict__ V, int ldv, long long N, int p, const float* __restrict__ L,
                     const float* __restrict__ Mb) {
  extern __shared__ __align__(16) float sm[];
  const int ldx = p + 1;
  float* X = sm;                        // kRows x ldx
  float* Ls = X + kRows * ldx;          // FB x (p + 1)
  float* Ms = Ls + FB * (p + 1);        // FB x (FB + 1)
  const long long row0 = (long long)blockIdx.x * kRows;
  const int rows = (int)min((long long)kRows, N - row0);
  for (int e = threadIdx.x; e < kRows * p; e += kTrsmThreads) {
    const int r = e / p, c = e % p;
    X[r * ldx + c] = r < rows ? V[(row0 + r) * ldv + c] : 0.f;
  }
  const int tr = threadIdx.x >> 3;  // 0..31: rows tr, tr + 32
  const int cg = threadIdx.x & 7;   // columns cg*4 .. cg*4+3 of the panel
  const int nblk = (p + FB - 1) / FB;
  for (int b = 0; b < nblk; ++b) {
    const int c0 = b * FB, nb = min(FB, p - c0);
    __syncthreads();
    for (int e = threadIdx.x; e < nb * c0; e += kTrsmThreads) {
      const int i = e / c0, k = e % c0;
      Ls[i * (p + 1) + k] = L[(size_t)(c0 + i) * p + k];
    }
    for (int e = threadIdx.x; e < FB * FB; e += kTrsmThreads) Ms[(e / FB) * (FB + 1) + e % FB] = Mb[(size_t)b * FB * FB + e];
    __syncthreads();
    // Y = V_b - X_{<b} L_{b,<b}ᵀ
    float acc[2][4];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int c = cg * 4 + v;
        acc[u][v] = c < nb ? X[(tr + 32 * u) * ldx + c0 + c] : 0.f;
      }
    for (int k = 0; k < c0; ++k) {
      const float x0 = X[tr * ldx + k], x1 = X[(tr + 32) * ldx + k];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float l = Ls[(cg * 4 + v) * (p + 1) + k];
        acc[0][v] = fmaf(-x0, l, acc[0][v]);
        acc[1][v] = fmaf(-x1, l, acc[1][v]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int c = cg * 4 + v;
        if (c < nb) X[(tr + 32 * u) * ldx + c0 + c] = acc[u][v];
      }
    __syncthreads();
    // X_b = Y Mbᵀ: X[r][c0+c] = Σ_{c' <= c} Y[r][c'] Mb[c][c']
    float out[2][4];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) out[u][v] = 0.f;
    for (int cp = 0; cp < nb; ++cp) {
      const float y0 = X[tr * ldx + c0 + cp], y1 = X[(tr + 32) * ldx + c0 + cp];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float mv = Ms[(cg * 4 + v) * (FB + 1) + cp];  // zero where cp > c
        out[0][v] = fmaf(y0, mv, out[0][v]);
        out[1][v] = fmaf(y1, mv, out[1][v]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int c = cg * 4 + v;
        if (c < nb) X[(tr + 32 * u) * ldx + c0 + c] = out[u][v];
      }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < rows * p; e += kTrsmThreads) {
    const int r = e / p, c = e % p;
    V[(row0 + r) * ldv + c] = X[r * ldx + c];
  }
}

size_t trsm_smem(int p) { return sizeof(float) * ((size_t)kRows * (p + 1) + (size_t)FB * (p + 1) + FB * (FB + 1)); }

}  // namespace

int cholqr32_max_p() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  int p = 32;
  while (chol_smem(p + 4) <= (size_t)optin && trsm_smem(p + 4) <= (size_t)optin) p += 4;
  return p;
}

size_t cholqr32_workspace(int p) {
  const int nblk = (p + FB - 1) / FB;
  return sizeof(float) * ((size_t)p * p + (size_t)nblk * FB * FB) + 512;
}

int chol32_gram(const double* G, int p, float* L, float* Mb, int* info, cudaStream_t st) {
  const size_t smem = chol_smem(p);
  if (cudaFuncSetAttribute(chol32_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    set_error("chol32_gram: cannot reserve %zu bytes of shared memory", smem);
    return RVGP_ELAUNCH;
  }
  rvgp::note_launch();
  chol32_gram_kernel<<<1, kCholThreads, smem, st>>>(G, p, L, Mb, info);
  return check_launch("chol32_gram");
}

int trsm_rows_f32(float* V, int ldv, long long N, int p, const float* L, const float* Mb, cudaStream_t st) {
  const size_t smem = trsm_smem(p);
  if (cudaFuncSetAttribute(trsm_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    set_error("trsm_rows_f32: cannot reserve %zu bytes of shared memory", smem);
    return RVGP_ELAUNCH;
  }
  rvgp::note_launch();
  trsm_rows_kernel<<<ceil_div(N, kRows), kTrsmThreads, smem, st>>>(V, ldv, N, p, L, Mb);
  return check_launch("trsm_rows_f32");
}

}  // namespace rvgp
