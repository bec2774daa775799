// Cholesky QR step of the eigensolver's FP32 block in FP32 (internal).
//
// Given the FP64 Gram G = VᵀV of an N x p FP32 block, V <- V D L⁻ᵀ with
// D = diag(G)^-½ and D G D = L Lᵀ (Cholesky QR of the column-scaled block,
// the scaling folded into the two steps):
//   chol32_gram   : one CTA forms D G D (rounded to FP32), factors it in
//                   shared memory and inverts the factor's 32 x 32 diagonal
//                   blocks (chol32.cuh); D to d (p floats);
//   trsm_rows_f32 : row tiles of V D solve X Lᵀ = V D in place, 32 columns at
//                   a time: X_b = (Y_b − X_{<b} L_{b,<b}ᵀ) L_bbᵀ⁻¹, the last
//                   product with the stored diagonal-block inverse; d may be
//                   null (V already scaled).
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

size_t chol_smem(int p) { return sizeof(float) * ((size_t)p * chol32::lda32(p) + 2 * (size_t)p) + 64; }

__global__ void __launch_bounds__(kCholThreads, 1)
    chol32_gram_kernel(const double* __restrict__ G, int p, float* __restrict__ L, float* __restrict__ Mb,
                       float* __restrict__ d, float first_order, int* __restrict__ info) {
  extern __shared__ __align__(16) float A[];
  __shared__ int s_flag;
  __shared__ unsigned s_emax;
  const int ld = chol32::lda32(p);
  float* dinvL = A + (size_t)p * ld;
  const int nblk = (p + FB - 1) / FB;
  // D = diag(G)^-½ (0 for an empty column, whose zero pivot then fails)
  float* dsh = A + (size_t)p * ld + p;  // p floats past dinvL
  for (int i = threadIdx.x; i < p; i += kCholThreads) {
    const double g = G[(size_t)i * p + i];
    dsh[i] = g > 0.0 ? (float)(1.0 / sqrt(g)) : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.x >> 5; i < p; i += kCholThreads / 32)
    for (int j = threadIdx.x & 31; j <= i; j += 32)
      A[i * ld + j] = (i == j && dsh[i] > 0.f) ? 1.f : (float)G[(size_t)i * p + j] * dsh[i] * dsh[j];
  for (int i = threadIdx.x; i < p; i += kCholThreads) d[i] = dsh[i];
  if (threadIdx.x == 0) s_emax = 0u;
  __syncthreads();
  if (first_order > 0.f) {
    // a nearly orthonormal block: E = D G D - I small, and V D (I - E/2) is
    // orthonormal to O(|E|²); L receives B = D (I - E/2) (row-major, p x p)
    float em = 0.f;
    for (int i = threadIdx.x >> 5; i < p; i += kCholThreads / 32)
      for (int j = threadIdx.x & 31; j <= i; j += 32) em = fmaxf(em, fabsf(A[i * ld + j] - (i == j ? 1.f : 0.f)));
    atomicMax(&s_emax, __float_as_uint(em));  // non-negative floats order as their bits
    __syncthreads();
    if (__uint_as_float(s_emax) <= first_order) {
      for (int i = threadIdx.x >> 5; i < p; i += kCholThreads / 32)
        for (int j = threadIdx.x & 31; j < p; j += 32) {
          const float e = (i == j) ? 0.f : A[max(i, j) * ld + min(i, j)];
          L[(size_t)i * p + j] = dsh[i] * ((i == j ? 1.f : 0.f) - 0.5f * e);
        }
      if (threadIdx.x == 0) *info = 2;
      return;
    }
  }
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

// X Lᵀ = V D for a tile of kRows rows, in place.  Shared memory: the tile
// (kRows x ldx), the current block row of L (32 x ldx) and the diagonal-block
// inverse (32 x 36), with ldx = p rounded up to an odd multiple of 4 words so
// that the 16-byte loads along k below are conflict-free.  Thread (r, g) owns
// rows {r, r + 32} x columns {g, g + 8, g + 16, g + 24} of the current
// 32-column panel; operands are read as float4 along k (8 FMAs per load).
__host__ __device__ inline int ldx_of(int p) { return ((p + 3) / 4 % 2 == 1) ? (p + 3) / 4 * 4 : (p + 3) / 4 * 4 + 4; }
constexpr int kLdm = FB + 4;  // 36 = 4 x 9

__global__ void __launch_bounds__(kTrsmThreads)
    trsm_rows_kernel(float* __restrict__ V, int ldv, long long N, int p, const float* __restrict__ L,
                     const float* __restrict__ Mb, const float* __restrict__ d) {
  extern __shared__ __align__(16) float sm[];
  const int ldx = ldx_of(p);
  float* X = sm;                        // kRows x ldx
  float* Ls = X + kRows * ldx;          // FB x ldx
  float* Ms = Ls + FB * ldx;            // FB x kLdm
  float* sd = Ms + FB * kLdm;           // p column scales
  for (int c = threadIdx.x; c < p; c += kTrsmThreads) sd[c] = d ? d[c] : 1.f;
  __syncthreads();
  const long long row0 = (long long)blockIdx.x * kRows;
  const int rows = (int)min((long long)kRows, N - row0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // tile rows (p, ldv multiples of 4: float4 along the row), zero padding
  for (int r = warp; r < kRows; r += kTrsmThreads / 32)
    for (int c = 4 * lane; c < ldx; c += 128) {
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < rows && c < p) {
        v = *reinterpret_cast<const float4*>(V + (row0 + r) * ldv + c);
        v.x *= sd[c];
        v.y *= sd[c + 1];
        v.z *= sd[c + 2];
        v.w *= sd[c + 3];
      }
      *reinterpret_cast<float4*>(X + r * ldx + c) = v;
    }
  const int tr = threadIdx.x >> 3;  // 0..31: rows tr, tr + 32
  const int g = threadIdx.x & 7;    // columns g + 8v of the panel
  const int nblk = (p + FB - 1) / FB;
  for (int b = 0; b < nblk; ++b) {
    const int c0 = b * FB, nb = min(FB, p - c0);
    __syncthreads();
    for (int i = warp; i < FB; i += kTrsmThreads / 32)
      for (int k = 4 * lane; k < c0; k += 128)
        *reinterpret_cast<float4*>(Ls + i * ldx + k) =
            i < nb ? *reinterpret_cast<const float4*>(L + (size_t)(c0 + i) * p + k) : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int e = threadIdx.x; e < FB * FB; e += kTrsmThreads) Ms[(e / FB) * kLdm + e % FB] = Mb[(size_t)b * FB * FB + e];
    __syncthreads();
    // Y = V_b - X_{<b} L_{b,<b}ᵀ
    float acc[2][4];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = X[(tr + 32 * u) * ldx + c0 + g + 8 * v];
    for (int k = 0; k < c0; k += 4) {
      const float4 x0 = *reinterpret_cast<const float4*>(X + tr * ldx + k);
      const float4 x1 = *reinterpret_cast<const float4*>(X + (tr + 32) * ldx + k);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float4 l = *reinterpret_cast<const float4*>(Ls + (g + 8 * v) * ldx + k);
        acc[0][v] = fmaf(-x0.x, l.x, fmaf(-x0.y, l.y, fmaf(-x0.z, l.z, fmaf(-x0.w, l.w, acc[0][v]))));
        acc[1][v] = fmaf(-x1.x, l.x, fmaf(-x1.y, l.y, fmaf(-x1.z, l.z, fmaf(-x1.w, l.w, acc[1][v]))));
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) X[(tr + 32 * u) * ldx + c0 + g + 8 * v] = acc[u][v];
    __syncthreads();
    // X_b = Y Mbᵀ: X[r][c0+c] = Σ_{c' <= c} Y[r][c'] Mb[c][c'] (Mb is zero above its diagonal)
    float out[2][4];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) out[u][v] = 0.f;
#pragma unroll 2
    for (int cp = 0; cp < FB; cp += 4) {
      const float4 y0 = *reinterpret_cast<const float4*>(X + tr * ldx + c0 + cp);
      const float4 y1 = *reinterpret_cast<const float4*>(X + (tr + 32) * ldx + c0 + cp);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float4 mv = *reinterpret_cast<const float4*>(Ms + (g + 8 * v) * kLdm + cp);
        out[0][v] = fmaf(y0.w, mv.w, fmaf(y0.z, mv.z, fmaf(y0.y, mv.y, fmaf(y0.x, mv.x, out[0][v]))));
        out[1][v] = fmaf(y1.w, mv.w, fmaf(y1.z, mv.z, fmaf(y1.y, mv.y, fmaf(y1.x, mv.x, out[1][v]))));
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v)
        if (g + 8 * v < nb) X[(tr + 32 * u) * ldx + c0 + g + 8 * v] = out[u][v];
  }
  __syncthreads();
  for (int r = warp; r < rows; r += kTrsmThreads / 32)
    for (int c = 4 * lane; c < p; c += 128)
      *reinterpret_cast<float4*>(V + (row0 + r) * ldv + c) = *reinterpret_cast<const float4*>(X + r * ldx + c);
}

size_t trsm_smem(int p) {
  return sizeof(float) * ((size_t)(kRows + FB) * ldx_of(p) + FB * kLdm + (size_t)p) + 16;
}

}  // namespace

int cholqr32_max_p() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  int p = 32;
  // + 512: the factorisation's static shared memory
  while (chol_smem(p + 4) + 512 <= (size_t)optin && trsm_smem(p + 4) <= (size_t)optin) p += 4;
  return p;
}

size_t cholqr32_workspace(int p) {
  const int nblk = (p + FB - 1) / FB;
  return sizeof(float) * ((size_t)p * p + (size_t)nblk * FB * FB) + 512;
}

int chol32_gram(const double* G, int p, float* L, float* Mb, float* d, float first_order, int* info,
                cudaStream_t st) {
  const size_t smem = chol_smem(p);
  if (raise_dyn_smem((const void*)chol32_gram_kernel, (size_t)(smem)) != cudaSuccess) {
    set_error("chol32_gram: cannot reserve %zu bytes of shared memory", smem);
    return RVGP_ELAUNCH;
  }
  rvgp::note_launch();
  chol32_gram_kernel<<<1, kCholThreads, smem, st>>>(G, p, L, Mb, d, first_order, info);
  return check_launch("chol32_gram");
}

int trsm_rows_f32(float* V, int ldv, long long N, int p, const float* L, const float* Mb, const float* d,
                  cudaStream_t st) {
  RVGP_CHECK_ARG(p % 4 == 0 && ldv % 4 == 0 && (uintptr_t)V % 16 == 0 && (uintptr_t)L % 16 == 0,
                 "trsm_rows_f32: p=%d and ldv=%d must be multiples of 4, V and L 16-byte aligned", p, ldv);
  const size_t smem = trsm_smem(p);
  if (raise_dyn_smem((const void*)trsm_rows_kernel, (size_t)(smem)) != cudaSuccess) {
    set_error("trsm_rows_f32: cannot reserve %zu bytes of shared memory", smem);
    return RVGP_ELAUNCH;
  }
  rvgp::note_launch();
  trsm_rows_kernel<<<ceil_div(N, kRows), kTrsmThreads, smem, st>>>(V, ldv, N, p, L, Mb, d);
  return check_launch("trsm_rows_f32");
}

}  // namespace rvgp
