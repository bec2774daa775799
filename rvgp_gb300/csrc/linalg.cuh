// Dense linear algebra used by the eigensolver and the GP (internal API).
//
// Shapes are row-major with explicit leading dimensions.  The tall-skinny
// products (N up to millions, p, q up to ~1024) are the GEMM-shaped part of
// block subspace iteration and of the low-rank GP algebra; the p x p kernels
// (Cholesky, triangular inverse, symmetric Jacobi eigensolver) are the small
// dense steps.  Every reduction is in a fixed order (deterministic).
#pragma once
#include "common.cuh"

namespace rvgp {

// 1/sqrt(d) for d > 0 in FP64 with a short dependency chain: an FP32 estimate
// refined by two Newton-Raphson steps y <- y + (y/2)(1 - d y²), each three
// dependent FP64 operations (the FP64 divide and square root are long chains
// of dependent operations on GB300).  Falls back to 1/sqrt(d) when d is
// outside the normal FP32 range.  Relative error ~1e-16.
__device__ __forceinline__ double rsqrt_nr(double d) {
  if (!(d > 1e-30 && d < 1e30)) return 1.0 / sqrt(d);
  double y = (double)rsqrtf((float)d);
  double a = d * y;
  double r = fma(-a, y, 1.0);
  y = fma(0.5 * y, r, y);
  a = d * y;
  r = fma(-a, y, 1.0);
  return fma(0.5 * y, r, y);
}
// FP32: correctly rounded square root and divide (rsqrtf's extra ulps would
// accumulate over the many rotations of a Jacobi sweep).
__device__ __forceinline__ float rsqrt_nr(float d) { return 1.0f / sqrtf(d); }

// 1/x in FP64 with an FP32 estimate and two Newton steps y <- y (2 - x y).
__device__ __forceinline__ double rcp_nr(double x) {
  const double ax = fabs(x);
  if (!(ax > 1e-30 && ax < 1e30)) return 1.0 / x;
  double y = (double)(1.0f / (float)x);
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}
__device__ __forceinline__ float rcp_nr(float x) { return 1.0f / x; }

// C (p x q, ldc) = alpha * Aᵀ B + beta * C,  A: N x p (lda), B: N x q (ldb).
template <typename T>
size_t gram_workspace(long long N, int p, int q);
template <typename T>
int gram(const T* A, int lda, const T* B, int ldb, long long N, int p, int q, T* C, int ldc, T alpha, T beta,
         void* ws, size_t ws_bytes, cudaStream_t st);

// Same product for FP32 inputs with FP32 partial sums reduced in FP64 into an FP64 C.
int gram_f32_out64(const float* A, int lda, const float* B, int ldb, long long N, int p, int q, double* C, int ldc,
                   double alpha, double beta, void* ws, size_t ws_bytes, cudaStream_t st);

// C (p x q, ldc) = sum over splits of part[split][p][q] (FP32) in FP64.
int reduce_f32_splits_to_f64(const float* part, int splits, int p, int q, double* C, int ldc, cudaStream_t st);

// Tensor-core (tcgen05, split-TF32) forms of the FP32 tall products for
// p, q <= 256 (tc_gemm.cu).  They do not synchronise; a timed-out pipeline
// wait sets *err (device) to 1.
bool tc_supported(int p, int q);
// false when the environment sets RVGP_TENSOR_CORES=0 (CUDA-core products instead)
bool tc_enabled();
// C (p x q, FP64) = Aᵀ B, A: N x p, B: N x q.
size_t tc_gram_workspace(long long N, int p, int q);
int tc_gram_f32_out64(const float* A, int lda, const float* B, int ldb, long long N, int p, int q, double* C, int ldc,
                      int* err, void* ws, size_t ws_bytes, cudaStream_t st);
// C (N x q) = A (N x K, lda % 4 == 0 for vector loads) Bm (K x q).  C must not alias A.
size_t tc_gemm_workspace(int K, int q);
int tc_gemm_f32(const float* A, int lda, long long N, int K, const float* Bm, int ldb, int q, float* C, int ldc,
                int* err, void* ws, size_t ws_bytes, cudaStream_t st);

// C (N x q, ldc) = alpha * A (N x p, lda) * B (p x q, ldb) + beta * C.  C must not alias A or B.
template <typename T>
int gemm_nn(const T* A, int lda, const T* B, int ldb, long long N, int p, int q, T* C, int ldc, T alpha, T beta,
            cudaStream_t st);

// In-place lower Cholesky of the p x p matrix A (lda).  *info (device) = 0 or
// j+1 when the leading (j+1) x (j+1) minor is not positive definite.  The
// strict upper triangle is not referenced.
template <typename T>
int cholesky(T* A, int lda, int p, int* info, cudaStream_t st);

// Linv (p x p, ld) = inverse of the lower-triangular L (lower part used); the
// strict upper part of Linv is set to zero.
template <typename T>
int tri_inv_lower(const T* L, int ldl, int p, T* Linv, int ldi, cudaStream_t st);

// Symmetric eigendecomposition by parallel cyclic Jacobi: H (p x p, symmetric,
// destroyed) -> eigenvalues w (ascending) and eigenvectors V (p x p, columns).
// max_sweeps bounds the work; *sweeps_used (host) reports it.  tol: stop when
// off(H) <= tol * ||H||_F.
template <typename T>
size_t jacobi_workspace(int p);
template <typename T>
int jacobi_eigh(T* H, int p, T* w, T* V, int max_sweeps, double tol, int* sweeps_used, void* ws, size_t ws_bytes,
                cudaStream_t st);

// FP32 block Jacobi (64 <= p <= 2048): the eigendecomposition of jacobi_eigh
// (H read only) with two grid barriers per round of 32-wide block pairs.
size_t jacobi_block_workspace(int p);
int jacobi_block_eigh(const float* H, int p, float* w, float* V, int max_sweeps, double tol, int* sweeps_used,
                      void* ws, size_t ws_bytes, cudaStream_t st);

// Column utilities on X (N x b, ld).
template <typename T>
int col_norms(const T* X, int ld, long long N, int b, T* out, void* ws, size_t ws_bytes, cudaStream_t st);
template <typename T>
size_t col_norms_workspace(long long N, int b);
template <typename T>
int scale_cols(T* X, int ld, long long N, int b, const T* s, bool inverse, cudaStream_t st);

// FP32 Cholesky QR step (cholqr.cu): chol32_gram scales the p x p FP64 Gram
// G to unit diagonal (d = diag(G)^-½, p floats) and factors D G D in FP32 in
// one CTA, writing L (p x p, lower, ld p) and the inverses of its 32 x 32
// diagonal blocks (Mb, ceil(p/32) x 32 x 32); *info (device) = 0, or 1 for a
// non-positive pivot.  trsm_rows_f32 overwrites V (N x p, ld) with V D L⁻ᵀ
// (D = diag(d); d null: the identity).  Both need p <= cholqr32_max_p().
// With first_order > 0 and max |D G D - I| <= first_order, chol32_gram instead
// writes B = D (I - E/2), E = D G D - I, into L (row-major p x p) and sets
// *info = 2: V B is then orthonormal to O(|E|²) (one block product, no
// factorisation).
int cholqr32_max_p();
size_t cholqr32_workspace(int p);
int chol32_gram(const double* G, int p, float* L, float* Mb, float* d, float first_order, int* info,
                cudaStream_t st);
int trsm_rows_f32(float* V, int ldv, long long N, int p, const float* L, const float* Mb, const float* d,
                  cudaStream_t st);

// FP32 symmetric eigensolver with the matrix in one SM's shared memory
// (jacobi32.cu): H (p x p, FP32, not modified) -> eigenvalues w ascending and
// eigenvectors V (p x p, columns), parallel cyclic Jacobi stopping at
// off(H) <= tol ||H||_F or after max_sweeps sweeps.  p even, p <= jacobi32_max_p().
int jacobi32_max_p();
size_t jacobi32_workspace(int p, int max_sweeps);
int jacobi32_eigh(const float* H, int p, float* w, float* V, int max_sweeps, double tol, int* sweeps_used, void* ws,
                  size_t ws_bytes, cudaStream_t st);

// Dtype conversion of an N x b block (ld in/out).
int convert_f32_to_f64(const float* in, int ldi, double* out, int ldo, long long N, int b, cudaStream_t st);
int convert_f64_to_f32(const double* in, int ldi, float* out, int ldo, long long N, int b, cudaStream_t st);

}  // namespace rvgp
