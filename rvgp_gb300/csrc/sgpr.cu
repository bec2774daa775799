// Sparse variational GP with inducing points: the collapsed bound of GPflow
// 2.6.5 SGPR as built by RVGP/main.py:59-67,119-137 (manifold_SGPR), its
// gradient with respect to (ν, κ, σ_f, σ²) and to the inducing inputs Z, and
// the posterior it predicts with.
//
// With the spectral kernel K(X, X2) = X D X2ᵀ (D = diag S) every N-space
// quantity of the bound reduces, through C = ΦᵀΦ, b = Φᵀy and yᵀy (formed
// once), to M- and m-space algebra (M inducing rows, m eigenpairs):
//   Kuu = Z D Zᵀ + εI = L Lᵀ,  Ẑ = L⁻¹Z,  W = Ẑ D        (GPflow's A = W Φᵀ/σ)
//   Q0 = W C Wᵀ,  B = I + Q0/σ² = L_B L_Bᵀ,  β = W b,  t = L_B⁻¹ β,  g = L_B⁻ᵀ t
//   F = −½N log 2π − Σ log diag L_B − ½N log σ² − ½ yᵀy/σ² + ½ tᵀt/σ⁴
//       − ½ tr(DC)/σ² + ½ tr(Q0)/σ²
// Gradient (hand-derived adjoint; P = WᵀW = D Zᵀ Kuu⁻¹ Z D is the Nyström
// weight matrix, Q = Φ P Φᵀ):
//   ∂F/∂P = Γ = ½ u uᵀ + ½ HᵀH,  u = (b − C Wᵀ g/σ²)/σ²,  H = V C/σ²,  V = L_B⁻¹ W
//   ∂F/∂S_l = 2(Y Γ)_ll − (Y Γ Yᵀ)_ll − ½ C_ll/σ²,   Y = Ẑᵀ W = Zᵀ Kuu⁻¹ Z D
//   ∂F/∂σ² = ½[(M − N − tr B⁻¹)/σ² + yᵀy/σ⁴ − (tᵀt + gᵀg)/σ⁶ + (tr(DC) − tr Q0)/σ⁴]
//   ∂F/∂Z  = 2 Kuu⁻¹ Z D Γ (D − P) = (Lᵀ⁻¹ W)(u (Qu)ᵀ + HᵀH Q),  Q = D − WᵀW
// and the chain rule through S(ν, κ, σ_f).  Posterior (predict_f,
// full_cov=False): mean = Φ* μ, var = diag(Φ* Σ Φ*ᵀ) with μ = Vᵀ t/σ² and
// Σ = D − WᵀW + VᵀV, i.e. GPflow's diag K** + colsum(tmp2²) − colsum(tmp1²).
//
// Everything is FP64: the bound's Cholesky factors have condition numbers up
// to |Kuu|/ε.  The products use the FP64 GEMM and matrix-vector kernels of
// fp64_gemm.cuh; the two Cholesky factorisations (one CTA for M <= 160,
// blocked above) and triangular inverses are the library's FP64 ones.
#include "common.cuh"
#include "linalg.cuh"
#include "fp64_gemm.cuh"
#include <math.h>
#include <algorithm>

RVGP_API int rvgp_spectral_S(const double* evals, int m, const double* theta, double n_rows, int typ, double* S,
                             double* dS, double* tmp3m, void* stream);

namespace rvgp {
namespace {

// out (R x m) = X ∘ S (column scaling)
__global__ void scale_cols_copy(const double* __restrict__ X, long long R, int m, const double* __restrict__ S,
                                double* __restrict__ out) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= R * m) return;
  out[e] = X[e] * S[e % m];
}

// K += jitter I
__global__ void add_jitter(double* __restrict__ K, int M, double jitter) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < M) K[(size_t)i * M + i] += jitter;
}

// LB = I + Q0/σ²
__global__ void build_B(const double* __restrict__ Q0, int M, const double* __restrict__ theta,
                        double* __restrict__ LB) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)M * M) return;
  const int i = (int)(e / M), j = (int)(e % M);
  LB[e] = (i == j ? 1.0 : 0.0) + Q0[e] / theta[3];
}

// u = (b − y2/σ²)/σ²
__global__ void make_u(const double* __restrict__ b, const double* __restrict__ y2, int m,
                       const double* __restrict__ theta, double* __restrict__ u) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= m) return;
  const double s2 = theta[3];
  u[l] = (b[l] - y2[l] / s2) / s2;
}

// Q (m x m) += diag(S)
__global__ void add_diag_vec(double* __restrict__ Q, int m, const double* __restrict__ S) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l < m) Q[(size_t)l * m + l] += S[l];
}

// G2 = u (Qu)ᵀ + G2/σ⁴
__global__ void finish_G2(double* __restrict__ G2, int m, const double* __restrict__ u, const double* __restrict__ Qu,
                          const double* __restrict__ theta) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)m * m) return;
  const double s2 = theta[3];
  G2[e] = fma(u[e / m], Qu[e % m], G2[e] / (s2 * s2));
}

// x *= 1/σ²
__global__ void scale_by_inv_noise(double* __restrict__ x, int n, const double* __restrict__ theta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] /= theta[3];
}

// CTA-wide sum in a fixed order; only warp 0 adds the per-warp partials (every
// FP64 instruction costs the SM's shared FP64 pipe, so none is repeated)
__device__ double cta_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double r = lane < nw ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (lane == 0) sh[32] = r;
  }
  __syncthreads();
  const double r = sh[32];
  __syncthreads();
  return r;
}

struct FinalIn {
  const double *S, *dS, *C, *b, *yy, *theta;
  const double *LB, *LBi, *Q0, *t, *g, *u, *Yu, *YHt, *Hp;
  const int* info;
  double N;
  int M, m;
};

// One warp per row, spread over many CTAs: rows l < m give ∂F/∂S_l (into gS),
// rows m + i give the squared norm of row i of L_B⁻¹ (into rowsq).
//   ∂F/∂S_l = Yu_l u_l + Σ_k YHt_lk Hp_kl/σ⁴ − ½ Yu_l² − ½ Σ_k YHt_lk²/σ⁴ − ½ C_ll/σ²
__global__ void __launch_bounds__(256) sgpr_rows(FinalIn in, double* __restrict__ gS, double* __restrict__ rowsq) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int M = in.M, m = in.m;
  if (r >= m + M) return;
  if (r < m) {
    const int l = r;
    double cross = 0.0, sq = 0.0;
    for (int k = lane; k < M; k += 32) {
      const double a = in.YHt[(size_t)l * M + k];
      cross = fma(a, in.Hp[(size_t)k * m + l], cross);
      sq = fma(a, a, sq);
    }
    for (int o = 16; o > 0; o >>= 1) {
      cross += __shfl_xor_sync(0xffffffffu, cross, o);
      sq += __shfl_xor_sync(0xffffffffu, sq, o);
    }
    if (lane == 0) {
      const double inv2 = rcp_nr(in.theta[3]), inv4 = inv2 * inv2;
      const double yu = in.Yu[l];
      gS[l] = yu * in.u[l] + cross * inv4 - 0.5 * yu * yu - 0.5 * sq * inv4 - 0.5 * in.C[(size_t)l * m + l] * inv2;
    }
  } else {
    const int i = r - m;
    double sq = 0.0;
    for (int k = lane; k <= i; k += 32) {
      const double v = in.LBi[(size_t)i * M + k];
      sq = fma(v, v, sq);
    }
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (lane == 0) rowsq[i] = sq;
  }
}

// One CTA: the bound and the four hyperparameter gradients from the scalar
// sums, gS and rowsq (every sum in a fixed order).
__global__ void __launch_bounds__(256) sgpr_final(FinalIn in, const double* __restrict__ gS,
                                                  const double* __restrict__ rowsq, double* __restrict__ out) {
  __shared__ double sh[33];
  const int M = in.M, m = in.m;
  const double s2 = in.theta[3], s4 = s2 * s2;
  double logdet = 0.0, trQ0 = 0.0, tt = 0.0, gg = 0.0, trBi = 0.0, trDC = 0.0;
  for (int i = threadIdx.x; i < M; i += blockDim.x) {
    logdet += log(in.LB[(size_t)i * M + i]);
    trQ0 += in.Q0[(size_t)i * M + i];
    tt = fma(in.t[i], in.t[i], tt);
    gg = fma(in.g[i], in.g[i], gg);
    trBi += rowsq[i];
  }
  double d0 = 0.0, d1 = 0.0, d2 = 0.0;
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    trDC = fma(in.S[l], in.C[(size_t)l * m + l], trDC);
    d0 = fma(gS[l], in.dS[l], d0);
    d1 = fma(gS[l], in.dS[m + l], d1);
    d2 = fma(gS[l], in.dS[2 * m + l], d2);
  }
  logdet = cta_sum(logdet, sh);
  trQ0 = cta_sum(trQ0, sh);
  tt = cta_sum(tt, sh);
  gg = cta_sum(gg, sh);
  trBi = cta_sum(trBi, sh);
  trDC = cta_sum(trDC, sh);
  d0 = cta_sum(d0, sh);
  d1 = cta_sum(d1, sh);
  d2 = cta_sum(d2, sh);
  if (threadIdx.x == 0) {
    const double N = in.N, yy = in.yy[0];
    const double kLog2Pi = 1.8378770664093453;  // log(2π)
    double F = -0.5 * N * kLog2Pi - logdet - 0.5 * N * log(s2) - 0.5 * yy / s2 + 0.5 * tt / s4 - 0.5 * trDC / s2 +
               0.5 * trQ0 / s2;
    const double dn =
        0.5 * ((M - N - trBi) / s2 + yy / s4 - (tt + gg) / (s4 * s2) + (trDC - trQ0) / s4);
    if (in.info[0] != 0 || in.info[1] != 0) F = nan("");
    out[0] = F;
    out[1] = d0;
    out[2] = d1;
    out[3] = d2;
    out[4] = dn;
  }
}

struct Buffers {
  double *S, *dS, *tmp, *ZS, *K, *Li, *Zh, *W, *WC, *Q0, *LB, *LBi, *YHt, *X, *Qm, *G2, *HQ;
  double *beta, *t, *g, *x, *y2, *u, *Wu, *Yu, *Qu, *gS, *rowsq;
};

Buffers carve(Workspace& w, int M, int m) {
  Buffers B;
  const size_t Mm = (size_t)M * m, MM = (size_t)M * M, mm = (size_t)m * m;
  B.S = w.take<double>(m);
  B.dS = w.take<double>(3 * (size_t)m);
  B.tmp = w.take<double>(3 * (size_t)m);
  B.ZS = w.take<double>(Mm);
  B.K = w.take<double>(MM);
  B.Li = w.take<double>(MM);
  B.Zh = w.take<double>(Mm);
  B.W = w.take<double>(Mm);
  B.WC = w.take<double>(Mm);
  B.Q0 = w.take<double>(MM);
  B.LB = w.take<double>(MM);
  B.LBi = w.take<double>(MM);
  B.YHt = w.take<double>(Mm);
  B.X = w.take<double>(Mm);
  B.Qm = w.take<double>(mm);
  B.G2 = w.take<double>(mm);
  B.HQ = w.take<double>(Mm);
  B.beta = w.take<double>(M);
  B.t = w.take<double>(M);
  B.g = w.take<double>(M);
  B.x = w.take<double>(m);
  B.y2 = w.take<double>(m);
  B.u = w.take<double>(m);
  B.Wu = w.take<double>(M);
  B.Yu = w.take<double>(m);
  B.Qu = w.take<double>(m);
  B.gS = w.take<double>(m);
  B.rowsq = w.take<double>(M);
  return B;
}

constexpr int kMaxM = 3072;  // triangular inverse: two M-rows of FP64 per warp in 48 KB

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_sgpr_workspace(int M, int m) {
  Workspace w(nullptr, 0);
  carve(w, M, m);
  return w.used + 256;
}

RVGP_API size_t rvgp_sgpr_state_size(int m) { return (size_t)m * m + (size_t)m; }

// Bound and gradients at theta = [ν, κ, σ_f, σ²] (device, 4) for the M x m
// inducing inputs Z (device), given C = ΦᵀΦ (m x m), b = Φᵀy (m) and yᵀy (1)
// of the N training rows.  out (device, 5) = [F, ∂F/∂ν, ∂F/∂κ, ∂F/∂σ_f,
// ∂F/∂σ²]; F is NaN when a Cholesky factorisation failed (info (device, 2):
// Kuu, B; 0 or the failing pivot + 1).  dZ (device, M x m, optional) =
// ∂F/∂Z; state (device, rvgp_sgpr_state_size(m), optional) = [Σ (m x m), μ
// (m)] for rvgp_sgpr_predict.  Asynchronous on `stream`.
RVGP_API int rvgp_sgpr_elbo(const double* C, const double* b, const double* yy, long long N, int m, const double* Z,
                            int M, const double* evals, double n_rows, const double* theta, int typ, double jitter,
                            double* out, double* dZ, double* state, int* info, void* ws, size_t ws_bytes,
                            void* stream) {
  RVGP_CHECK_ARG(C && b && yy && Z && evals && theta && out && info && ws, "rvgp_sgpr_elbo: null argument");
  RVGP_CHECK_ARG(N >= 1 && m >= 1 && M >= 1 && M <= kMaxM, "rvgp_sgpr_elbo: bad sizes N=%lld m=%d M=%d (M <= %d)",
                 N, m, M, kMaxM);
  RVGP_CHECK_ARG(typ == 0 || typ == 1, "rvgp_sgpr_elbo: typ must be 0 (matern) or 1 (se)");
  RVGP_CHECK_ARG(jitter >= 0.0, "rvgp_sgpr_elbo: negative jitter");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_sgpr_workspace(M, m), "rvgp_sgpr_elbo: workspace too small");
  cudaStream_t st = as_stream(stream);
  Workspace w(ws, ws_bytes);
  Buffers B = carve(w, M, m);
  const long long Mm = (long long)M * m, MM = (long long)M * M, mm = (long long)m * m;
  TRY_RC(rvgp_spectral_S(evals, m, theta, n_rows, typ, B.S, B.dS, B.tmp, stream));
  // Kuu = Z D Zᵀ + εI = L Lᵀ;  Ẑ = L⁻¹ Z;  W = Ẑ D
  note_launch();
  scale_cols_copy<<<ceil_div(Mm, 256), 256, 0, st>>>(Z, M, m, B.S, B.ZS);
  gemm64<false, true>(M, M, m, 1.0, B.ZS, m, Z, m, 0.0, B.K, M, st);
  note_launch();
  add_jitter<<<ceil_div(M, 256), 256, 0, st>>>(B.K, M, jitter);
  TRY_RC(cholesky<double>(B.K, M, M, info, st));
  TRY_RC(tri_inv_lower<double>(B.K, M, M, B.Li, M, st));
  gemm64<false, false>(M, m, M, 1.0, B.Li, M, Z, m, 0.0, B.Zh, m, st);
  note_launch();
  scale_cols_copy<<<ceil_div(Mm, 256), 256, 0, st>>>(B.Zh, M, m, B.S, B.W);
  // Q0 = W C Wᵀ;  B = I + Q0/σ² = L_B L_Bᵀ
  gemm64<false, false>(M, m, m, 1.0, B.W, m, C, m, 0.0, B.WC, m, st);
  gemm64<false, true>(M, M, m, 1.0, B.WC, m, B.W, m, 0.0, B.Q0, M, st);
  note_launch();
  build_B<<<ceil_div(MM, 256), 256, 0, st>>>(B.Q0, M, theta, B.LB);
  TRY_RC(cholesky<double>(B.LB, M, M, info + 1, st));
  TRY_RC(tri_inv_lower<double>(B.LB, M, M, B.LBi, M, st));
  // β = W b, t = L_B⁻¹ β, g = L_B⁻ᵀ t;  V = L_B⁻¹ W (into ZS);  Hp = V C (into WC; H = Hp/σ²)
  double* V = B.ZS;
  double* Hp = B.WC;
  gemm64<false, false>(M, 1, m, 1.0, B.W, m, b, 1, 0.0, B.beta, 1, st);
  gemm64<false, false>(M, 1, M, 1.0, B.LBi, M, B.beta, 1, 0.0, B.t, 1, st);
  gemm64<true, false>(M, 1, M, 1.0, B.LBi, M, B.t, 1, 0.0, B.g, 1, st);
  gemm64<false, false>(M, m, M, 1.0, B.LBi, M, B.W, m, 0.0, V, m, st);
  gemm64<false, false>(M, m, m, 1.0, V, m, C, m, 0.0, Hp, m, st);
  // u = (b − C Wᵀ g/σ²)/σ²;  Yu = Ẑᵀ W u
  gemm64<true, false>(m, 1, M, 1.0, B.W, m, B.g, 1, 0.0, B.x, 1, st);
  gemm64<false, false>(m, 1, m, 1.0, C, m, B.x, 1, 0.0, B.y2, 1, st);
  note_launch();
  make_u<<<ceil_div(m, 256), 256, 0, st>>>(b, B.y2, m, theta, B.u);
  gemm64<false, false>(M, 1, m, 1.0, B.W, m, B.u, 1, 0.0, B.Wu, 1, st);
  gemm64<true, false>(m, 1, M, 1.0, B.Zh, m, B.Wu, 1, 0.0, B.Yu, 1, st);
  // YHt = Ẑᵀ (W Hpᵀ)  (m x M; the M x M product goes into K, whose factor is no longer needed)
  gemm64<false, true>(M, M, m, 1.0, B.W, m, Hp, m, 0.0, B.K, M, st);
  gemm64<true, false>(m, M, M, 1.0, B.Zh, m, B.K, M, 0.0, B.YHt, M, st);
  FinalIn fi{B.S, B.dS, C, b, yy, theta, B.LB, B.LBi, B.Q0, B.t, B.g, B.u, B.Yu, B.YHt, Hp, info, (double)N, M, m};
  note_launch();
  sgpr_rows<<<ceil_div((long long)(m + M) * 32, 256), 256, 0, st>>>(fi, B.gS, B.rowsq);
  note_launch();
  sgpr_final<<<1, 256, 0, st>>>(fi, B.gS, B.rowsq, out);
  if (dZ || state) {
    // Q = D − WᵀW
    gemm64<true, false>(m, m, M, -1.0, B.W, m, B.W, m, 0.0, B.Qm, m, st);
    note_launch();
    add_diag_vec<<<ceil_div(m, 256), 256, 0, st>>>(B.Qm, m, B.S);
  }
  if (dZ) {
    // ∂F/∂Z = (L⁻ᵀ W)(u (Qu)ᵀ + HᵀH Q)
    gemm64<false, false>(m, 1, m, 1.0, B.Qm, m, B.u, 1, 0.0, B.Qu, 1, st);
    gemm64<false, false>(M, m, m, 1.0, Hp, m, B.Qm, m, 0.0, B.HQ, m, st);
    gemm64<true, false>(m, m, M, 1.0, Hp, m, B.HQ, m, 0.0, B.G2, m, st);
    note_launch();
    finish_G2<<<ceil_div(mm, 256), 256, 0, st>>>(B.G2, m, B.u, B.Qu, theta);
    gemm64<true, false>(M, m, M, 1.0, B.Li, M, B.W, m, 0.0, B.X, m, st);
    gemm64<false, false>(M, m, m, 1.0, B.X, m, B.G2, m, 0.0, dZ, m, st);
  }
  if (state) {
    // Σ = Q + VᵀV;  μ = Vᵀ t/σ²
    cudaMemcpyAsync(state, B.Qm, sizeof(double) * mm, cudaMemcpyDeviceToDevice, st);
    gemm64<true, false>(m, m, M, 1.0, V, m, V, m, 1.0, state, m, st);
    gemm64<true, false>(m, 1, M, 1.0, V, m, B.t, 1, 0.0, state + mm, 1, st);
    note_launch();
    scale_by_inv_noise<<<ceil_div(m, 256), 256, 0, st>>>(state + mm, m, theta);
  }
  RVGP_LAUNCH_CHECK("rvgp_sgpr_elbo");
  return RVGP_OK;
}

namespace rvgp {
namespace {
// mean_i = φ_i·μ, var_i = φ_i·(Σ φ_i) given T = Φ* Σ (one warp per row)
__global__ void sgpr_rows(const double* __restrict__ Phi, const double* __restrict__ T, long long Nte, int m,
                          const double* __restrict__ mu, double* __restrict__ mean, double* __restrict__ var) {
  const long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= Nte) return;
  double a = 0.0, v = 0.0;
  for (int l = lane; l < m; l += 32) {
    const double p = Phi[r * m + l];
    a = fma(p, mu[l], a);
    v = fma(p, T[r * m + l], v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  if (lane == 0) {
    mean[r] = a;
    var[r] = v;
  }
}
}  // namespace
}  // namespace rvgp

RVGP_API size_t rvgp_sgpr_predict_workspace(long long Nte, int m) { return sizeof(double) * (size_t)Nte * m + 256; }

// Posterior mean and marginal variance (no noise) at the Nte x m spectral
// rows Phi_star (device), from the state written by rvgp_sgpr_elbo.
RVGP_API int rvgp_sgpr_predict(const double* Phi_star, long long Nte, int m, const double* state, double* mean,
                               double* var, void* ws, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(Phi_star && state && mean && var && ws && Nte >= 1 && m >= 1, "rvgp_sgpr_predict: bad arguments");
  RVGP_CHECK_ARG(Nte <= (1LL << 31) / 32 * 32, "rvgp_sgpr_predict: too many rows");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_sgpr_predict_workspace(Nte, m), "rvgp_sgpr_predict: workspace too small");
  cudaStream_t st = as_stream(stream);
  double* T = static_cast<double*>(ws);
  // rows in chunks that keep the GEMM grid's y extent within limits
  const long long chunk = 65535LL * kT;
  for (long long r0 = 0; r0 < Nte; r0 += chunk) {
    const int rows = (int)std::min<long long>(chunk, Nte - r0);
    gemm64<false, false>(rows, m, m, 1.0, Phi_star + r0 * m, m, state, m, 0.0, T + r0 * m, m, st);
  }
  note_launch();
  sgpr_rows<<<ceil_div(Nte * 32, 256), 256, 0, st>>>(Phi_star, T, Nte, m, state + (size_t)m * m, mean, var);
  RVGP_LAUNCH_CHECK("rvgp_sgpr_predict");
  return RVGP_OK;
}
