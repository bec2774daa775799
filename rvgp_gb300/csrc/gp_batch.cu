// Posterior means (and log marginal likelihoods) of B vector fields observed
// at the same training rows, with shared hyperparameters: the many-fields
// workload of RVGP's time-series use (one fit per time sample, e.g.
// examples/eeg_example/eeg_utils.py:26-35, interpolate_time_range), solved
// for all fields at once from the state of one rvgp_gp_lml evaluation.
//
// With the rank-m state (L_A⁻¹, r = √S) of the GP and Y (N x B) the fields'
// training rows, one column per field:
//   Bm = Φᵀ Y,  Z = L_A⁻¹ (r ∘ Bm),  W = L_A⁻ᵀ Z,  P = r ∘ W / σ²   (m x B)
//   mean = Φ* P                                                      (N* x B)
//   LML_b = −½ (|y_b|² − |z_b|²/σ²)/σ² − ½ (N log σ² + 2 Σ log diag L_A) − ½ N log 2π
// (Σ log diag L_A = −Σ log diag L_A⁻¹), the single-field formulas of the GP
// with the right-hand side replaced by a block of B columns: four FP64
// products for every field together.
#include "common.cuh"
#include "linalg.cuh"
#include "fp64_gemm.cuh"
#include <math.h>

namespace rvgp {
namespace {

// out (m x B) = X ∘ r (rows), times 1/σ² when `by_noise`
__global__ void scale_rows(const double* __restrict__ X, int m, int B, const double* __restrict__ r,
                           const double* __restrict__ theta, int by_noise, double* __restrict__ out) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)m * B) return;
  const double v = X[e] * r[e / B];
  out[e] = by_noise ? v / theta[3] : v;
}

// ld = Σ_l log diag(L_A⁻¹) (one CTA, fixed order)
__global__ void __launch_bounds__(256) state_logdiag(const double* __restrict__ Li, int m, double* __restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int l = threadIdx.x; l < m; l += blockDim.x) s += log(Li[(size_t)l * m + l]);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// LML of every field (thread per column b)
__global__ void batch_lml(const double* __restrict__ Y, long long N, int B, const double* __restrict__ Z, int m,
                          const double* __restrict__ ld, const double* __restrict__ theta, double* __restrict__ lml) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  double yy = 0.0, zz = 0.0;
  for (long long i = 0; i < N; ++i) yy = fma(Y[i * B + b], Y[i * B + b], yy);
  for (int l = 0; l < m; ++l) zz = fma(Z[(size_t)l * B + b], Z[(size_t)l * B + b], zz);
  const double s2 = theta[3];
  const double kLog2Pi = 1.8378770664093453;  // log(2π)
  lml[b] = -0.5 * (yy - zz / s2) / s2 - 0.5 * ((double)N * log(s2) - 2.0 * ld[0]) - 0.5 * (double)N * kLog2Pi;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_gp_posterior_batch_workspace(int m, int B) {
  Workspace w(nullptr, 0);
  w.take<double>((size_t)m * B);
  w.take<double>((size_t)m * B);
  w.take<double>((size_t)m * B);
  w.take<double>(1);
  return w.used + 256;
}

// Phi (N x m) and Y (N x B): the training rows and the B fields' values at
// them; state (rvgp_gp_state_size(m)) and theta (4) of an rvgp_gp_lml
// evaluation on the same rows; Phi_star (Nte x m).  mean (Nte x B); lml (B,
// optional).  Asynchronous on `stream`.
RVGP_API int rvgp_gp_posterior_batch(const double* Phi, long long N, int m, const double* Y, int B,
                                     const double* theta, const double* state, const double* Phi_star, long long Nte,
                                     double* mean, double* lml, void* ws, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(Phi && Y && theta && state && Phi_star && mean && ws, "rvgp_gp_posterior_batch: null argument");
  RVGP_CHECK_ARG(N >= 1 && N <= (1LL << 31) - 1 && m >= 1 && B >= 1 && Nte >= 1 && Nte <= 65535LL * 32,
                 "rvgp_gp_posterior_batch: bad sizes");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_gp_posterior_batch_workspace(m, B), "rvgp_gp_posterior_batch: workspace too small");
  cudaStream_t st = as_stream(stream);
  Workspace w(ws, ws_bytes);
  double* Bm = w.take<double>((size_t)m * B);
  double* Z = w.take<double>((size_t)m * B);
  double* W = w.take<double>((size_t)m * B);
  double* ld = w.take<double>(1);
  const double* Li = state;
  const double* r = state + (size_t)m * m + 2 * (size_t)m;  // state = [L_A⁻¹, sp, S, r, w]
  const int n = (int)N;
  const long long mB = (long long)m * B;
  gemm64<true, false>(m, B, n, 1.0, Phi, m, Y, B, 0.0, Bm, B, st);  // Bm = Φᵀ Y
  note_launch();
  scale_rows<<<ceil_div(mB, 256), 256, 0, st>>>(Bm, m, B, r, theta, 0, W);  // r ∘ Bm
  gemm64<false, false>(m, B, m, 1.0, Li, m, W, B, 0.0, Z, B, st);   // Z = L_A⁻¹ (r ∘ Bm)
  gemm64<true, false>(m, B, m, 1.0, Li, m, Z, B, 0.0, W, B, st);    // W = L_A⁻ᵀ Z
  note_launch();
  scale_rows<<<ceil_div(mB, 256), 256, 0, st>>>(W, m, B, r, theta, 1, Bm);  // P = r ∘ W / σ²
  gemm64<false, false>((int)Nte, B, m, 1.0, Phi_star, m, Bm, B, 0.0, mean, B, st);
  if (lml) {
    note_launch();
    state_logdiag<<<1, 256, 0, st>>>(Li, m, ld);
    note_launch();
    batch_lml<<<ceil_div(B, 128), 128, 0, st>>>(Y, N, B, Z, m, ld, theta, lml);
  }
  RVGP_LAUNCH_CHECK("rvgp_gp_posterior_batch");
  return RVGP_OK;
}
