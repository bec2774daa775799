// Dense GP with the squared-exponential (RBF) kernel on the scalar-Laplacian
// eigenbasis: the `kernel='rbf'` branch of RVGP/main.py:33-37, where GPflow's
// `kernels.RBF()` and `GPR` treat the D vector components as D independent
// outputs sharing one kernel over the N training points.
//
//   K_ij = v exp(−½ |x_i − x_j|² / ℓ²),  K_y = K + σ² I = L Lᵀ,  A = K_y⁻¹ Y (N x D)
//   LML = −½ Σ_c |L⁻¹ y_c|² − D Σ log diag L − ½ N D log 2π
//   ∂LML/∂θ = ½ Σ_ij G_ij ∂K_y,ij/∂θ,  G = A Aᵀ − D K_y⁻¹
//     ∂K/∂v = K/v,  ∂K/∂ℓ = K ∘ |x_i − x_j|² / ℓ³,  ∂K_y/∂σ² = I
// Posterior (predict_f, full_cov=False): mean = K(X*, X) A, var = v − |L⁻¹ K(X, x*)|².
//
// Everything is FP64 (K_y's condition number grows like v N/σ²).  Squared
// distances are direct differences (no |x|² + |x'|² − 2 x·x' cancellation).
// The explicit K_y⁻¹ = L⁻ᵀ L⁻¹ is the N³ step; N is limited by the one-CTA-row
// triangular inverse to 3072 training rows.
#include "common.cuh"
#include "linalg.cuh"
#include "fp64_gemm.cuh"
#include <math.h>
#include <algorithm>

namespace rvgp {
namespace {

constexpr int kMaxRows = 3072;
constexpr int kGradCTAs = 1024;

// K (N1 x N2, ldk) = v exp(−½ sqd/ℓ²); optionally sqd (ld ldk) and
// Ky = K + σ² I (ld ldk) for the lower triangle and diagonal.
__global__ void __launch_bounds__(256) rbf_matrix_kernel(const double* __restrict__ X1, int N1,
                                                         const double* __restrict__ X2, int N2, int m,
                                                         const double* __restrict__ theta, double* __restrict__ K,
                                                         int ldk, double* __restrict__ sqd, double* __restrict__ Ky) {
  __shared__ double A1[16][33], A2[16][33];
  const int t = threadIdx.x, hi = t >> 4, lo = t & 15;
  const int i0 = blockIdx.y * 16, j0 = blockIdx.x * 16;
  double acc = 0.0;
  for (int c0 = 0; c0 < m; c0 += 32) {
    for (int e = t; e < 16 * 32; e += 256) {
      const int r = e >> 5, c = e & 31;
      A1[r][c] = (i0 + r < N1 && c0 + c < m) ? X1[(size_t)(i0 + r) * m + c0 + c] : 0.0;
      A2[r][c] = (j0 + r < N2 && c0 + c < m) ? X2[(size_t)(j0 + r) * m + c0 + c] : 0.0;
    }
    __syncthreads();
    const int cn = min(32, m - c0);
    for (int c = 0; c < cn; ++c) {
      const double d = A1[hi][c] - A2[lo][c];
      acc = fma(d, d, acc);
    }
    __syncthreads();
  }
  const int i = i0 + hi, j = j0 + lo;
  if (i >= N1 || j >= N2) return;
  const double v = theta[0], l = theta[1];
  const double k = v * exp(-0.5 * acc / (l * l));
  const size_t e = (size_t)i * ldk + j;
  K[e] = k;
  if (sqd) sqd[e] = acc;
  if (Ky && j <= i) Ky[e] = i == j ? k + theta[2] : k;
}

// Per-CTA partial sums over its rows i (i = b, b + grid, ...) of
//   s0 = Σ_j G_ij K_ij,  s1 = Σ_j G_ij K_ij sqd_ij,  s2 = G_ii,   G = A Aᵀ − D K_y⁻¹
__global__ void __launch_bounds__(256) rbf_grad_partial(const double* __restrict__ K, const double* __restrict__ sqd,
                                                        const double* __restrict__ Kinv, const double* __restrict__ A,
                                                        int N, int D, double* __restrict__ part) {
  __shared__ double red[3][8];
  __shared__ double Ai[16];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x; i < N; i += gridDim.x) {
    __syncthreads();
    if (threadIdx.x < D) Ai[threadIdx.x] = A[(size_t)i * D + threadIdx.x];
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      double aa = 0.0;
      for (int c = 0; c < D; ++c) aa = fma(Ai[c], A[(size_t)j * D + c], aa);
      const size_t e = (size_t)i * N + j;
      const double g = fma(-(double)D, Kinv[e], aa);
      const double gk = g * K[e];
      s0 += gk;
      s1 = fma(gk, sqd[e], s1);
      if (j == i) s2 += g;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[0][w] = s0;
    red[1][w] = s1;
    red[2][w] = s2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double r = 0.0;
    for (int q = 0; q < 8; ++q) r += red[threadIdx.x][q];
    part[(size_t)blockIdx.x * 3 + threadIdx.x] = r;
  }
}

// One CTA: LML and its gradient [∂/∂v, ∂/∂ℓ, ∂/∂σ²] from L, T = L⁻¹Y and the partials.
__global__ void __launch_bounds__(256) rbf_final(const double* __restrict__ L, int N, const double* __restrict__ T,
                                                 int D, const double* __restrict__ part, int nparts,
                                                 const double* __restrict__ theta, const int* __restrict__ info,
                                                 double* __restrict__ out) {
  __shared__ double sh[5][8];
  double logdet = 0.0, quad = 0.0, p0 = 0.0, p1 = 0.0, p2 = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) logdet += log(L[(size_t)i * N + i]);
  for (long long e = threadIdx.x; e < (long long)N * D; e += blockDim.x) quad = fma(T[e], T[e], quad);
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
    p0 += part[(size_t)b * 3];
    p1 += part[(size_t)b * 3 + 1];
    p2 += part[(size_t)b * 3 + 2];
  }
  double v[5] = {logdet, quad, p0, p1, p2};
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int q = 0; q < 5; ++q) {
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if (lane == 0) sh[q][w] = v[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r[5];
    for (int q = 0; q < 5; ++q) {
      r[q] = 0.0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r[q] += sh[q][k];
    }
    const double kLog2Pi = 1.8378770664093453;  // log(2π)
    double lml = -0.5 * r[1] - D * r[0] - 0.5 * (double)N * D * kLog2Pi;
    if (*info != 0) lml = nan("");
    const double var = theta[0], l = theta[1];
    out[0] = lml;
    out[1] = 0.5 * r[2] / var;
    out[2] = 0.5 * r[3] / (l * l * l);
    out[3] = 0.5 * r[4];
  }
}

// var_j = v − Σ_i V_ij²  (V: N x Q, column j)
__global__ void rbf_var_cols(const double* __restrict__ V, int N, int Q, const double* __restrict__ theta,
                             double* __restrict__ var) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= Q) return;
  double s = 0.0;
  for (int i = 0; i < N; ++i) {
    const double x = V[(size_t)i * Q + j];
    s = fma(x, x, s);
  }
  var[j] = theta[0] - s;
}

struct RbfBuffers {
  double *K, *sqd, *L, *Kinv, *T, *part;
};

RbfBuffers rbf_carve(Workspace& w, long long N, int D) {
  RbfBuffers B;
  const size_t NN = (size_t)N * N;
  B.K = w.take<double>(NN);
  B.sqd = w.take<double>(NN);
  B.L = w.take<double>(NN);
  B.Kinv = w.take<double>(NN);
  B.T = w.take<double>((size_t)N * D);
  B.part = w.take<double>((size_t)kGradCTAs * 3);
  return B;
}

constexpr long long kPredictChunk = 8192;

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_rbf_workspace(long long N, int D) {
  Workspace w(nullptr, 0);
  rbf_carve(w, N, D);
  return w.used + 256;
}

RVGP_API size_t rvgp_rbf_state_size(long long N, int D) { return (size_t)N * N + (size_t)N * D; }

// K (N1 x N2) = v exp(−½ |x1_i − x2_j|²/ℓ²) for theta = [v, ℓ, σ²] (device).
RVGP_API int rvgp_rbf_matrix(const double* X1, long long N1, const double* X2, long long N2, int m,
                             const double* theta, double* K, void* stream) {
  RVGP_CHECK_ARG(X1 && X2 && theta && K && N1 >= 1 && N2 >= 1 && m >= 1, "rvgp_rbf_matrix: bad arguments");
  RVGP_CHECK_ARG(N1 <= 65535LL * 16 && N2 <= (1LL << 31) - 1, "rvgp_rbf_matrix: too many rows");
  note_launch();
  rbf_matrix_kernel<<<dim3(ceil_div(N2, 16), ceil_div(N1, 16)), 256, 0, as_stream(stream)>>>(
      X1, (int)N1, X2, (int)N2, m, theta, K, (int)N2, nullptr, nullptr);
  RVGP_LAUNCH_CHECK("rvgp_rbf_matrix");
  return RVGP_OK;
}

// LML of the D-output GP with the RBF kernel on the N x m inputs X, outputs Y
// (N x D), theta = [variance, lengthscale, noise] (device).  out (device, 4) =
// [LML, ∂/∂variance, ∂/∂lengthscale, ∂/∂noise], LML NaN when the Cholesky
// factorisation failed (*info, device, = failing pivot + 1).  state (device,
// rvgp_rbf_state_size(N, D)) = [L⁻¹ (N x N), A = K_y⁻¹Y (N x D)] for
// rvgp_rbf_predict.  N <= 3072.  Asynchronous on `stream`.
RVGP_API int rvgp_rbf_lml(const double* X, long long N, int m, const double* Y, int D, const double* theta,
                          double* out, double* state, int* info, void* ws, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(X && Y && theta && out && state && info && ws, "rvgp_rbf_lml: null argument");
  RVGP_CHECK_ARG(N >= 1 && N <= kMaxRows && m >= 1 && D >= 1 && D <= 16,
                 "rvgp_rbf_lml: bad sizes N=%lld (1..%d) m=%d D=%d (1..16)", N, kMaxRows, m, D);
  RVGP_CHECK_ARG(ws_bytes >= rvgp_rbf_workspace(N, D), "rvgp_rbf_lml: workspace too small");
  cudaStream_t st = as_stream(stream);
  Workspace w(ws, ws_bytes);
  RbfBuffers B = rbf_carve(w, N, D);
  const int n = (int)N;
  double* Li = state;
  double* A = state + (size_t)N * N;
  note_launch();
  rbf_matrix_kernel<<<dim3(ceil_div(n, 16), ceil_div(n, 16)), 256, 0, st>>>(X, n, X, n, m, theta, B.K, n, B.sqd,
                                                                           B.L);
  TRY_RC(cholesky<double>(B.L, n, n, info, st));
  TRY_RC(tri_inv_lower<double>(B.L, n, n, Li, n, st));
  // T = L⁻¹ Y, A = L⁻ᵀ T, K_y⁻¹ = L⁻ᵀ L⁻¹
  gemm64<false, false>(n, D, n, 1.0, Li, n, Y, D, 0.0, B.T, D, st);
  gemm64<true, false>(n, D, n, 1.0, Li, n, B.T, D, 0.0, A, D, st);
  gemm64<true, false>(n, n, n, 1.0, Li, n, Li, n, 0.0, B.Kinv, n, st);
  const int g = (int)std::min<long long>(kGradCTAs, N);
  note_launch();
  rbf_grad_partial<<<g, 256, 0, st>>>(B.K, B.sqd, B.Kinv, A, n, D, B.part);
  note_launch();
  rbf_final<<<1, 256, 0, st>>>(B.L, n, B.T, D, B.part, g, theta, info, out);
  RVGP_LAUNCH_CHECK("rvgp_rbf_lml");
  return RVGP_OK;
}

RVGP_API size_t rvgp_rbf_predict_workspace(long long Nte, long long N) {
  const long long c = std::min(Nte, kPredictChunk);
  return sizeof(double) * (size_t)(2 * c * N) + 512;
}

// Posterior mean (Nte x D) and marginal variance (Nte, no noise) at the rows
// Xs (Nte x m) from the state of rvgp_rbf_lml (same X, theta).
RVGP_API int rvgp_rbf_predict(const double* Xs, long long Nte, const double* X, long long N, int m, int D,
                              const double* theta, const double* state, double* mean, double* var, void* ws,
                              size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(Xs && X && theta && state && mean && var && ws, "rvgp_rbf_predict: null argument");
  RVGP_CHECK_ARG(Nte >= 1 && N >= 1 && N <= kMaxRows && m >= 1 && D >= 1 && D <= 16,
                 "rvgp_rbf_predict: bad sizes");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_rbf_predict_workspace(Nte, N), "rvgp_rbf_predict: workspace too small");
  cudaStream_t st = as_stream(stream);
  const int n = (int)N;
  const double* Li = state;
  const double* A = state + (size_t)N * N;
  const long long c = std::min(Nte, kPredictChunk);
  double* Ks = static_cast<double*>(ws);
  double* V = Ks + (size_t)c * N;
  for (long long r0 = 0; r0 < Nte; r0 += c) {
    const int rows = (int)std::min(c, Nte - r0);
    note_launch();
    rbf_matrix_kernel<<<dim3(ceil_div(n, 16), ceil_div(rows, 16)), 256, 0, st>>>(Xs + r0 * m, rows, X, n, m, theta,
                                                                                Ks, n, nullptr, nullptr);
    gemm64<false, false>(rows, D, n, 1.0, Ks, n, A, D, 0.0, mean + r0 * D, D, st);
    gemm64<false, true>(n, rows, n, 1.0, Li, n, Ks, n, 0.0, V, rows, st);
    note_launch();
    rbf_var_cols<<<ceil_div(rows, 256), 256, 0, st>>>(V, n, rows, theta, var + r0);
  }
  RVGP_LAUNCH_CHECK("rvgp_rbf_predict");
  return RVGP_OK;
}
