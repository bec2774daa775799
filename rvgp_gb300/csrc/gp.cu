// Spectral manifold kernel and the Gaussian-process likelihood / posterior.
//
// Kernel (RVGP/kernels.py:41-67): with eigenpairs (λ_l, φ_l) of the
// connection Laplacian lifted to ambient rows (RVGP/dataclass.py:57-59),
//   Matérn: s_l = (λ_l + 2ν/κ²)^(-ν);  SE: s_l = exp(-λ_l κ²/2)
//   S_l = σ_f · N_rows · s_l / Σ s,   K(X, X2) = (X S) X2ᵀ.
//
// GP (GPflow GPR as used by RVGP/main.py:55-116): y ~ N(0, Φ S Φᵀ + σ² I).
// Because K has rank m, every quantity is computed exactly in the m-space
// (Woodbury identity and matrix determinant lemma) from C = ΦᵀΦ, b = Φᵀy and
// yᵀy, which are formed once:
//   R = diag(√S),  A = I + R C R / σ² = L_A L_Aᵀ,  z = L_A⁻¹ R b,  w = A⁻¹ R b
//   log|K_y| = N log σ² + 2 Σ log diag L_A
//   yᵀK_y⁻¹y = (yᵀy − zᵀz / σ²) / σ²
//   Φᵀα = w / (r σ²)  (α = K_y⁻¹ y),   S_l (ΦᵀK_y⁻¹Φ)_ll = 1 − (A⁻¹)_ll
//   ∂LML/∂S_l = ½[(Φᵀα)_l² − (ΦᵀK_y⁻¹Φ)_ll]
//   ∂LML/∂σ²  = ½[αᵀα − tr K_y⁻¹],  αᵀα = (yᵀy − zᵀz/σ² − wᵀw/σ²)/σ⁴,
//                                    tr K_y⁻¹ = (N − m + tr A⁻¹)/σ²
// (the identities follow from A w = R b and R C R = σ²(A − I)), and the chain
// rule through S(ν, κ, σ_f) including the Σs normalisation.
// Posterior (predict_f, full_cov=False): mean = Φ* (S ∘ Φᵀα),
// var = diag(Φ* R A⁻¹ R Φ*ᵀ) = |L_A⁻¹ R φ*_i|² per test row.
// The m x m factorisation is FP64 in both forms (cond(A) grows like
// λ_max(RCR)/σ²); the tall products (C = ΦᵀΦ, Φ* Bᵀ) are FP32 in the mixed form.
#include "common.cuh"
#include <algorithm>
#include "linalg.cuh"
#include <math.h>
#include <float.h>

namespace rvgp {
namespace {

constexpr int kCTA = 1024;

__device__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

__device__ double block_max(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

// theta = [nu, kappa, sigma_f, noise]; S (m); dS (3 x m) = ∂S/∂(nu, kappa, sigma_f)
__global__ void __launch_bounds__(kCTA) spectral_S_kernel(const double* __restrict__ evals, int m,
                                                          const double* __restrict__ theta, double n_rows, int typ,
                                                          double* __restrict__ S, double* __restrict__ dS,
                                                          double* __restrict__ tmp) {
  __shared__ double sh[kCTA];
  const double nu = theta[0], kappa = theta[1], sf = theta[2];
  double* ls = tmp;          // log s_l
  double* gnu = tmp + m;     // ∂ log s_l / ∂nu
  double* gk = tmp + 2 * m;  // ∂ log s_l / ∂kappa
  double mx = -DBL_MAX;
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    const double lam = evals[l];
    double a, b, c;
    if (typ == 0) {
      const double u = lam + 2.0 * nu / (kappa * kappa);
      const double lu = log(u);
      a = -nu * lu;
      b = -lu - nu * (2.0 / (kappa * kappa)) / u;
      c = 4.0 * nu * nu / (kappa * kappa * kappa * u);
    } else {
      a = -0.5 * lam * kappa * kappa;
      b = 0.0;
      c = -lam * kappa;
    }
    ls[l] = a;
    gnu[l] = b;
    gk[l] = c;
    mx = fmax(mx, a);
  }
  mx = block_max(mx, sh);
  double z = 0.0;
  for (int l = threadIdx.x; l < m; l += blockDim.x) z += exp(ls[l] - mx);
  z = block_sum(z, sh);
  double mnu = 0.0, mk = 0.0;
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    const double w = exp(ls[l] - mx) / z;
    mnu += w * gnu[l];
    mk += w * gk[l];
  }
  mnu = block_sum(mnu, sh);
  mk = block_sum(mk, sh);
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    const double Sl = sf * n_rows * exp(ls[l] - mx) / z;
    S[l] = Sl;
    if (dS) {
      dS[l] = Sl * (gnu[l] - mnu);
      dS[m + l] = Sl * (gk[l] - mk);
      dS[2 * m + l] = Sl / sf;
    }
  }
}

__global__ void build_A(const double* __restrict__ C, int m, const double* __restrict__ S,
                        const double* __restrict__ theta, double* __restrict__ A) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)m * m) return;
  const int i = (int)(e / m), j = (int)(e % m);
  const double s2 = theta[3];
  A[e] = (i == j ? 1.0 : 0.0) + sqrt(S[i]) * C[e] * sqrt(S[j]) / s2;
}

// state layout (doubles): [0, m²) L_A⁻¹, then sp = S ∘ Φᵀα = r ∘ w / σ² (m), S (m),
// r (m), w = A⁻¹ R b (m).
//
// With w = A⁻¹ R b the Woodbury algebra collapses (A w = R b and
// R C R = σ²(A − I)):  Φᵀα = w / (r σ²),  diag(ΦᵀK⁻¹Φ)_l S_l = 1 − (A⁻¹)_ll,
// αᵀα = (yᵀy − zᵀz/σ² − wᵀw/σ²)/σ⁴ with z = L_A⁻¹ R b.  Every gradient term is
// then O(m) given L_A⁻¹ and is free of cancellation:
//   ∂LML/∂θ = ½ Σ_l [(w_l/σ²)² − (1 − (A⁻¹)_ll)] ∂log S_l/∂θ.

// z = L_A⁻¹ (r ∘ b): one warp per row k of L_A⁻¹
__global__ void lml_z(const double* __restrict__ Li, int m, const double* __restrict__ S,
                      const double* __restrict__ b, double* __restrict__ z, const int* __restrict__ info) {
  const int lane = threadIdx.x & 31;
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (k >= m || *info) return;
  double s = 0.0;
  for (int l = lane; l <= k; l += 32) s += Li[(size_t)k * m + l] * sqrt(S[l]) * b[l];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) z[k] = s;
}

// w = L_A⁻ᵀ z and (A⁻¹)_ll = Σ_k (L_A⁻¹)_kl²: one warp per column l
__global__ void lml_w_diag(const double* __restrict__ Li, int m, const double* __restrict__ z,
                           double* __restrict__ w, double* __restrict__ ainv_diag, const int* __restrict__ info) {
  const int lane = threadIdx.x & 31;
  const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (l >= m || *info) return;
  double s = 0.0, q = 0.0;
  for (int k = l + lane; k < m; k += 32) {
    const double v = Li[(size_t)k * m + l];
    s += v * z[k];
    q += v * v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    q += __shfl_xor_sync(0xffffffffu, q, o);
  }
  if (lane == 0) {
    w[l] = s;
    ainv_diag[l] = q;
  }
}

// LML, its gradient w.r.t. [nu, kappa, sigma_f, noise] and the predict state (one CTA)
__global__ void __launch_bounds__(kCTA) lml_final(const double* __restrict__ yy, long long N, int m,
                                                  const double* __restrict__ LA, const double* __restrict__ S,
                                                  const double* __restrict__ dS, const double* __restrict__ z,
                                                  const double* __restrict__ w, const double* __restrict__ ainv_diag,
                                                  const double* __restrict__ theta, const int* __restrict__ info,
                                                  double* __restrict__ state, double* __restrict__ out) {
  __shared__ double sh[kCTA];
  const double s2 = theta[3];
  if (*info != 0) {
    if (threadIdx.x == 0)
      for (int t = 0; t < 5; ++t) out[t] = nan("");
    return;
  }
  double* sp = state + (size_t)m * m;
  double* Sst = sp + m;
  double* r = Sst + m;
  double* wst = r + m;
  double zz = 0.0, ww = 0.0, logd = 0.0, tr = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    const double Sl = S[l], rl = sqrt(Sl), wl = w[l];
    zz += z[l] * z[l];
    ww += wl * wl;
    logd += log(LA[(size_t)l * m + l]);
    tr += ainv_diag[l];
    sp[l] = rl * wl / s2;
    Sst[l] = Sl;
    r[l] = rl;
    wst[l] = wl;
    // ½[(w_l/σ²)² − (1 − (A⁻¹)_ll)] · ∂S_l/∂θ / S_l
    const double q = 0.5 * ((wl / s2) * (wl / s2) - (1.0 - ainv_diag[l])) / Sl;
    g0 += q * dS[l];
    g1 += q * dS[m + l];
    g2 += q * dS[2 * m + l];
  }
  zz = block_sum(zz, sh);
  ww = block_sum(ww, sh);
  logd = block_sum(logd, sh);
  tr = block_sum(tr, sh);
  g0 = block_sum(g0, sh);
  g1 = block_sum(g1, sh);
  g2 = block_sum(g2, sh);
  if (threadIdx.x == 0) {
    const double Nd = (double)N;
    const double quad = (yy[0] - zz / s2) / s2;
    const double logdet = Nd * log(s2) + 2.0 * logd;
    out[0] = -0.5 * quad - 0.5 * logdet - 0.5 * Nd * log(2.0 * M_PI);
    out[1] = g0;
    out[2] = g1;
    out[3] = g2;
    const double a2 = (yy[0] - zz / s2 - ww / s2) / (s2 * s2);
    out[4] = 0.5 * (a2 - (Nd - m + tr) / s2);
  }
}

__device__ __forceinline__ double softplus_d(double u) { return u > 0.0 ? u + log1p(exp(-u)) : log1p(exp(u)); }
__device__ __forceinline__ double sigmoid_d(double u) {
  return u >= 0.0 ? 1.0 / (1.0 + exp(-u)) : exp(u) / (1.0 + exp(u));
}

// Adam on the unconstrained parameters u (value = softplus(u) + lower) minimising −LML.
// adam = [u(4), m(4), v(4)]; hyper = [lr, beta1, beta2, eps]; mask = trainable flags.
__global__ void adam_step(double* __restrict__ theta, double* __restrict__ adam, const double* __restrict__ lower,
                          const int* __restrict__ mask, const double* __restrict__ out, int step, double lr,
                          double beta1, double beta2, double eps, double* __restrict__ hist) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (hist) hist[step] = out[0];
  bool finite = true;
  for (int q = 0; q < 5; ++q) finite = finite && isfinite(out[q]);
  if (!finite) return;  // keep the parameters; the history records the failure
  const double b1t = 1.0 - pow(beta1, (double)(step + 1)), b2t = 1.0 - pow(beta2, (double)(step + 1));
  for (int q = 0; q < 4; ++q) {
    if (!mask[q]) continue;
    double* u = adam + q;
    double* m1 = adam + 4 + q;
    double* v1 = adam + 8 + q;
    const double g = -out[1 + q] * sigmoid_d(*u);  // d(−LML)/du
    *m1 = beta1 * *m1 + (1.0 - beta1) * g;
    *v1 = beta2 * *v1 + (1.0 - beta2) * g * g;
    *u -= lr * (*m1 / b1t) / (sqrt(*v1 / b2t) + eps);
    theta[q] = softplus_d(*u) + lower[q];
  }
}

__global__ void adam_init(const double* __restrict__ theta0, const double* __restrict__ lower,
                          double* __restrict__ theta, double* __restrict__ adam) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int q = 0; q < 4; ++q) {
    theta[q] = theta0[q];
    const double v = theta0[q] - lower[q];
    adam[q] = v > 30.0 ? v : log(expm1(fmax(v, 1e-300)));  // inverse softplus
    adam[4 + q] = 0.0;
    adam[8 + q] = 0.0;
  }
}

// Φ[(t*D + a), :] = src[(idx[t]*D + a), :],  y[(t*D + a)] = vec[idx[t]*D + a]
// part[c][j] = Σ over rows of chunk c of Phi[r][j] y[r] (j < m), and
// part[c][m] = Σ y[r]² over the chunk: grid (chunks, ceil((m + 1) / 32)), warp
// w takes rows r0 + w, r0 + w + 8, ... for columns 32 blockIdx.y + lane
// (coalesced); the 8 warp sums are added in a fixed order.
__global__ void __launch_bounds__(256) phity_partial(const double* __restrict__ Phi, const double* __restrict__ y,
                                                     long long N, int m, long long chunk, double* __restrict__ part) {
  __shared__ double sh[8][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.y * 32 + lane;
  const long long r0 = blockIdx.x * chunk, r1 = min(N, r0 + chunk);
  double s0 = 0.0, s1 = 0.0;
  if (j < m) {
    long long r = r0 + warp;
    for (; r + 8 < r1; r += 16) {
      s0 = fma(Phi[r * m + j], y[r], s0);
      s1 = fma(Phi[(r + 8) * m + j], y[r + 8], s1);
    }
    for (; r < r1; r += 8) s0 = fma(Phi[r * m + j], y[r], s0);
  } else if (j == m) {
    for (long long r = r0 + warp; r < r1; r += 8) s0 = fma(y[r], y[r], s0);
  }
  sh[warp][lane] = s0 + s1;
  __syncthreads();
  if (warp == 0 && j <= m) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += sh[w][lane];
    part[(size_t)blockIdx.x * (m + 1) + j] = t;
  }
}

// b[j] = Σ_c part[c][j] (j < m), yy = Σ_c part[c][m]
__global__ void phity_final(const double* __restrict__ part, int nchunk, int m, double* __restrict__ b,
                            double* __restrict__ yy) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j > m) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * (m + 1) + j];
  if (j < m)
    b[j] = s;
  else
    *yy = s;
}

int phity_chunks(long long N) { return (int)std::max<long long>(1, std::min<long long>(256, (N + 511) / 512)); }

__global__ void gather_rows(const double* __restrict__ src, int m, int D, const int* __restrict__ idx, int nt,
                            const double* __restrict__ vec, double* __restrict__ Phi, float* __restrict__ Phi32,
                            double* __restrict__ y) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long rows = (long long)nt * D;
  if (e >= rows * m) return;
  const long long row = e / m;
  const int j = (int)(e % m);
  const int t = (int)(row / D), a = (int)(row % D);
  const long long srow = (long long)idx[t] * D + a;
  const double v = src[srow * m + j];
  if (Phi) Phi[e] = v;
  if (Phi32) Phi32[e] = (float)v;
  if (y && j == 0) y[row] = vec[srow];
}

// out[(i*D + a), j] = Σ_q T[i, a, q] U[(i*d + q), j]
__global__ void lift_kernel(const double* __restrict__ T, int n, int D, int ld, int d, const double* __restrict__ U,
                            int m, double* __restrict__ out) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * D * m) return;
  const long long row = e / m;
  const int j = (int)(e % m);
  const int i = (int)(row / D), a = (int)(row % D);
  double s = 0.0;
  for (int q = 0; q < d; ++q) s += T[((size_t)i * D + a) * ld + q] * U[((size_t)i * d + q) * m + j];
  out[e] = s;
}

// ---------------------------------------------------------------- gauge-reduced rows
// The lifted rows of one point i are Φ_i = T_i U_i (D x m: gauge T_i, D x d,
// times the point's d rows U_i of the connection-Laplacian eigenvectors,
// RVGP/dataclass.py:57-59).  Hence, with G_i = T_iᵀT_i = L_i L_iᵀ (d x d):
//   Φ_iᵀΦ_i = (L_iᵀU_i)ᵀ(L_iᵀU_i),   Φ_iᵀy_i = (L_iᵀU_i)ᵀ(L_i⁻¹T_iᵀy_i),
// so C = ΦᵀΦ and b = Φᵀy come exactly from d rows per point instead of D, and
// yᵀy is summed over the full D-vectors.  kMaxLocalD bounds d.
constexpr int kMaxLocalD = 8;

// One warp per training point t (point i = idx[t]): L_t (d x d lower Cholesky
// factor of T_iᵀT_i, row-major), yt[t*d + q] = (L_t⁻¹ T_iᵀ y_i)_q and
// yyp[t] = |y_i|².  Lanes stride over the D coordinates; the d(d+1)/2 + d + 1
// sums are reduced by shuffles in a fixed order.
template <int d>
__global__ void local_factor_kernel(const double* __restrict__ T, int D, int ld, const int* __restrict__ idx,
                                    int nt, const double* __restrict__ vec, double* __restrict__ Lf,
                                    double* __restrict__ yt, double* __restrict__ yyp) {
  const int lane = threadIdx.x & 31;
  const long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (t >= nt) return;
  const long long i = idx[t];
  constexpr int NG = d * (d + 1) / 2;
  double g[NG], ty[d], yy = 0.0;
#pragma unroll
  for (int e = 0; e < NG; ++e) g[e] = 0.0;
#pragma unroll
  for (int q = 0; q < d; ++q) ty[q] = 0.0;
  for (int a = lane; a < D; a += 32) {
    const double* Ta = T + ((size_t)i * D + a) * ld;
    const double ya = vec ? vec[(size_t)i * D + a] : 0.0;
#pragma unroll
    for (int q = 0; q < d; ++q) {
      const double tq = Ta[q];
      ty[q] = fma(tq, ya, ty[q]);
#pragma unroll
      for (int r = 0; r <= q; ++r) g[q * (q + 1) / 2 + r] = fma(tq, Ta[r], g[q * (q + 1) / 2 + r]);
    }
    yy = fma(ya, ya, yy);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int e = 0; e < NG; ++e) g[e] += __shfl_xor_sync(0xffffffffu, g[e], o);
#pragma unroll
    for (int q = 0; q < d; ++q) ty[q] += __shfl_xor_sync(0xffffffffu, ty[q], o);
    yy += __shfl_xor_sync(0xffffffffu, yy, o);
  }
  if (lane != 0) return;
  // Cholesky of the packed lower triangle g (row q holds entries (q, 0..q))
  double L[d][d];
#pragma unroll
  for (int q = 0; q < d; ++q)
#pragma unroll
    for (int r = 0; r < d; ++r) L[q][r] = 0.0;
#pragma unroll
  for (int q = 0; q < d; ++q) {
#pragma unroll
    for (int r = 0; r <= q; ++r) {
      const int e = q * (q + 1) / 2 + r;
      double s = g[e];
      for (int k = 0; k < r; ++k) s -= L[q][k] * L[r][k];
      if (r == q)
        L[q][q] = sqrt(fmax(s, 0.0));
      else
        L[q][r] = s / L[r][r];
    }
  }
  // forward solve L x = Tᵀy
  for (int q = 0; q < d; ++q) {
    double s = ty[q];
    for (int k = 0; k < q; ++k) s -= L[q][k] * ty[k];
    ty[q] = s / L[q][q];
  }
  for (int q = 0; q < d; ++q) {
    for (int r = 0; r < d; ++r) Lf[((size_t)t * d + q) * d + r] = L[q][r];
    if (yt) yt[(size_t)t * d + q] = ty[q];
  }
  if (yyp) yyp[t] = yy;
}

// Ut[(t*d + q), j] = Σ_{r >= q} L_t[r][q] U[(idx[t]*d + r), j]   (= (L_tᵀ U_i)[q][j])
template <typename T>
__global__ void local_rows_kernel(const double* __restrict__ U, int m, int d, const int* __restrict__ idx, int nt,
                                  const double* __restrict__ Lf, T* __restrict__ Ut) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nt * d * m) return;
  const long long row = e / m;
  const int j = (int)(e % m);
  const long long t = row / d;
  const int q = (int)(row % d);
  const double* Ui = U + (size_t)idx[t] * d * m + j;
  const double* Lt = Lf + (size_t)t * d * d;
  double s = 0.0;
  for (int r = q; r < d; ++r) s = fma(Lt[r * d + q], Ui[(size_t)r * m], s);
  Ut[e] = (T)s;
}

// Rows U[(idx[t]*d + q), :] of the test points (FP64 or FP32 copy).
template <typename T>
__global__ void gather_local_rows(const double* __restrict__ U, int m, int d, const int* __restrict__ idx, int nt,
                                  T* __restrict__ out) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nt * d * m) return;
  const long long row = e / m;
  const int j = (int)(e % m);
  out[e] = (T)U[((size_t)idx[row / d] * d + row % d) * m + j];
}

// Fixed-order sum of v[0..n) by one CTA of 1024 threads: *out = Σ v.
__global__ void __launch_bounds__(1024) sum_fixed(const double* __restrict__ v, long long n, double* __restrict__ out) {
  __shared__ double sh[1024];
  double s = 0.0;
  for (long long k = threadIdx.x; k < n; k += 1024) s += v[k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// Posterior at the test points from Q = U_te Bt (rows t*d + q): warp per test
// point t (point i = idx[t]):
//   μ_loc[q] = Σ_j U[(i*d + q), j] sp_j,   M[q][r] = Σ_k Q[t*d + q][k] Q[t*d + r][k]
//   mean[t*D + a] = Σ_q T[i,a,q] μ_loc[q],  var[t*D + a] = Σ_{q,r} T[i,a,q] T[i,a,r] M[q][r]
// which equal mean = Φ*sp and var = |L_A⁻¹ R φ*|² of the lifted rows φ* = t_aᵀU_i.
template <int d, typename T>
__global__ void predict_local_kernel(const double* __restrict__ Tg, int D, int ld, const double* __restrict__ U,
                                     int m, const int* __restrict__ idx, int nt, const double* __restrict__ state,
                                     const T* __restrict__ Q, double* __restrict__ mean, double* __restrict__ var) {
  const int lane = threadIdx.x & 31;
  const long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (t >= nt) return;
  const long long i = idx[t];
  const double* sp = state + (size_t)m * m;
  constexpr int NG = d * (d + 1) / 2;
  double mu[d], M[NG];
#pragma unroll
  for (int q = 0; q < d; ++q) mu[q] = 0.0;
#pragma unroll
  for (int e = 0; e < NG; ++e) M[e] = 0.0;
  const double* Ui = U + (size_t)i * d * m;
  const T* Qt = Q + (size_t)t * d * m;
  for (int j = lane; j < m; j += 32) {
    const double s = sp[j];
    double qv[d];
#pragma unroll
    for (int q = 0; q < d; ++q) {
      mu[q] = fma(Ui[(size_t)q * m + j], s, mu[q]);
      qv[q] = (double)Qt[(size_t)q * m + j];
    }
#pragma unroll
    for (int q = 0; q < d; ++q)
#pragma unroll
      for (int r = 0; r <= q; ++r) M[q * (q + 1) / 2 + r] = fma(qv[q], qv[r], M[q * (q + 1) / 2 + r]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int q = 0; q < d; ++q) mu[q] += __shfl_xor_sync(0xffffffffu, mu[q], o);
#pragma unroll
    for (int e = 0; e < NG; ++e) M[e] += __shfl_xor_sync(0xffffffffu, M[e], o);
  }
  for (int a = lane; a < D; a += 32) {
    const double* Ta = Tg + ((size_t)i * D + a) * ld;
    double tv[d], mv = 0.0, vv = 0.0;
#pragma unroll
    for (int q = 0; q < d; ++q) tv[q] = Ta[q];
#pragma unroll
    for (int q = 0; q < d; ++q) {
      mv = fma(tv[q], mu[q], mv);
#pragma unroll
      for (int r = 0; r < q; ++r) vv = fma(2.0 * tv[q] * tv[r], M[q * (q + 1) / 2 + r], vv);
      vv = fma(tv[q] * tv[q], M[q * (q + 1) / 2 + q], vv);
    }
    mean[(size_t)t * D + a] = mv;
    var[(size_t)t * D + a] = vv;
  }
}

// Bt[l][k] = r_l L_A⁻¹[k][l]   (so that Φ* Bt = (L_A⁻¹ R Φ*ᵀ)ᵀ)
template <typename T>
__global__ void make_Bt(const double* __restrict__ state, int m, T* __restrict__ Bt) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)m * m) return;
  const int l = (int)(e / m), k = (int)(e % m);
  const double* r = state + (size_t)m * m + 2 * m;  // after L_A⁻¹, sp, S
  Bt[e] = (T)(k >= l ? r[l] * state[(size_t)k * m + l] : 0.0);
}

// mean_i = Σ_l Φ*_il sp_l  (sp = S ∘ Φᵀα) ; var_i = Σ_k P_ik²  (warp per row)
template <typename T>
__global__ void predict_rows(const double* __restrict__ Phi, long long Nte, int m, const double* __restrict__ state,
                             const T* __restrict__ P, double* __restrict__ mean, double* __restrict__ var) {
  const int lane = threadIdx.x & 31;
  const long long i = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (i >= Nte) return;
  const double* sp = state + (size_t)m * m;
  double sm = 0.0, sv = 0.0;
  for (int l = lane; l < m; l += 32) {
    sm += Phi[i * m + l] * sp[l];
    const double p = (double)P[i * m + l];
    sv += p * p;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sm += __shfl_xor_sync(0xffffffffu, sm, o);
    sv += __shfl_xor_sync(0xffffffffu, sv, o);
  }
  if (lane == 0) {
    mean[i] = sm;
    var[i] = sv;
  }
}

// C (N1 x N2) = (A diag(S)) Bᵀ
__global__ void __launch_bounds__(256) kernel_matrix(const double* __restrict__ A, long long N1,
                                                     const double* __restrict__ B, long long N2, int m,
                                                     const double* __restrict__ S, double* __restrict__ C) {
  __shared__ double As[64][17], Bs[64][17];
  const long long r0 = (long long)blockIdx.y * 64, c0 = (long long)blockIdx.x * 64;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < m; k0 += 16) {
    for (int e = threadIdx.x; e < 64 * 16; e += 256) {
      const int r = e / 16, c = e % 16;
      As[r][c] = (r0 + r < N1 && k0 + c < m) ? A[(r0 + r) * m + k0 + c] * S[k0 + c] : 0.0;
      Bs[r][c] = (c0 + r < N2 && k0 + c < m) ? B[(c0 + r) * m + k0 + c] : 0.0;
    }
    __syncthreads();
    for (int kk = 0; kk < 16; ++kk)
      for (int u = 0; u < 4; ++u)
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(As[ty * 4 + u][kk], Bs[tx * 4 + v][kk], acc[u][v]);
    __syncthreads();
  }
  for (int u = 0; u < 4; ++u)
    for (int v = 0; v < 4; ++v) {
      const long long r = r0 + ty * 4 + u, c = c0 + tx * 4 + v;
      if (r < N1 && c < N2) C[r * N2 + c] = acc[u][v];
    }
}

__global__ void kernel_diag(const double* __restrict__ A, long long N, int m, const double* __restrict__ S,
                            double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long i = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (i >= N) return;
  double s = 0.0;
  for (int l = lane; l < m; l += 32) s += A[i * m + l] * A[i * m + l] * S[l];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[i] = s;
}

struct LmlBufs {
  double *S, *dS, *stmp, *A, *z, *w, *ainv, *theta, *adam, *lower;
  int *info, *mask;
};

LmlBufs carve_lml(Workspace& ws, int m) {
  LmlBufs b;
  b.S = ws.take<double>(m);
  b.dS = ws.take<double>(3 * (size_t)m);
  b.stmp = ws.take<double>(3 * (size_t)m);
  b.A = ws.take<double>((size_t)m * m);
  b.z = ws.take<double>(m);
  b.w = ws.take<double>(m);
  b.ainv = ws.take<double>(m);
  b.theta = ws.take<double>(4);
  b.adam = ws.take<double>(12);
  b.lower = ws.take<double>(4);
  b.info = ws.take<int>(4);
  b.mask = ws.take<int>(4);
  return b;
}

// One likelihood + gradient evaluation at theta (device), all stream-ordered.
int lml_chain(const LmlBufs& B, const double* C, const double* b, const double* yy, long long N, int m,
              const double* evals, double n_rows, int typ, const double* theta, double* out, double* state,
              cudaStream_t st) {
  const long long mm = (long long)m * m;
  rvgp::note_launch(); spectral_S_kernel<<<1, kCTA, 0, st>>>(evals, m, theta, n_rows, typ, B.S, B.dS, B.stmp);
  rvgp::note_launch(); build_A<<<ceil_div(mm, 256), 256, 0, st>>>(C, m, B.S, theta, B.A);
  int rc = cholesky<double>(B.A, m, m, B.info, st);
  if (rc) return rc;
  rc = tri_inv_lower<double>(B.A, m, m, state, m, st);
  if (rc) return rc;
  const int wb = ceil_div((long long)m * 32, 256);
  rvgp::note_launch(); lml_z<<<wb, 256, 0, st>>>(state, m, B.S, b, B.z, B.info);
  rvgp::note_launch(); lml_w_diag<<<wb, 256, 0, st>>>(state, m, B.z, B.w, B.ainv, B.info);
  rvgp::note_launch(); lml_final<<<1, kCTA, 0, st>>>(yy, N, m, B.A, B.S, B.dS, B.z, B.w, B.ainv, theta, B.info, state,
                                                    out);
  return check_launch("lml_chain");
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API int rvgp_spectral_S(const double* evals, int m, const double* theta, double n_rows, int typ, double* S,
                             double* dS, double* tmp3m, void* stream) {
  RVGP_CHECK_ARG(evals && theta && S && tmp3m && m >= 1, "rvgp_spectral_S: bad arguments");
  RVGP_CHECK_ARG(typ == 0 || typ == 1, "rvgp_spectral_S: typ must be 0 (matern) or 1 (se)");
  rvgp::note_launch(); spectral_S_kernel<<<1, kCTA, 0, as_stream(stream)>>>(evals, m, theta, n_rows, typ, S, dS, tmp3m);
  RVGP_LAUNCH_CHECK("rvgp_spectral_S");
  return RVGP_OK;
}

RVGP_API int rvgp_lift(const double* T, int n, int D, int ld, int d, const double* U, int m, double* out,
                       void* stream) {
  RVGP_CHECK_ARG(T && U && out && d <= ld && d <= D, "rvgp_lift: bad arguments");
  rvgp::note_launch(); lift_kernel<<<ceil_div((long long)n * D * m, 256), 256, 0, as_stream(stream)>>>(T, n, D, ld, d, U, m, out);
  RVGP_LAUNCH_CHECK("rvgp_lift");
  return RVGP_OK;
}

RVGP_API int rvgp_gather_rows(const double* src, int m, int D, const int* idx, int nt, const double* vec, double* Phi,
                              float* Phi32, double* y, void* stream) {
  RVGP_CHECK_ARG(src && idx && m >= 1 && D >= 1, "rvgp_gather_rows: bad arguments");
  rvgp::note_launch(); gather_rows<<<ceil_div((long long)nt * D * m, 256), 256, 0, as_stream(stream)>>>(src, m, D, idx, nt, vec, Phi,
                                                                                    Phi32, y);
  RVGP_LAUNCH_CHECK("rvgp_gather_rows");
  return RVGP_OK;
}

RVGP_API size_t rvgp_gp_prepare_workspace(long long N, int m) {
  return std::max(gram_workspace<double>(N, m, m), gram_workspace<float>(N, m, m)) +
         sizeof(double) * (size_t)phity_chunks(N) * (m + 1) + 1024;
}

// C = ΦᵀΦ (m x m), b = Φᵀy (m), yy = yᵀy.  mode 1 uses Phi32 for C (FP32
// products, FP64-reduced partial sums); b and yy are FP64 in both modes.
RVGP_API int rvgp_gp_prepare(const double* Phi, const float* Phi32, const double* y, long long N, int m, int mode,
                             double* C, double* b, double* yy, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(Phi && y && C && b && yy && N >= 1 && m >= 1, "rvgp_gp_prepare: bad arguments");
  RVGP_CHECK_ARG(mode == 0 || Phi32, "rvgp_gp_prepare: mode 1 needs Phi32");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_gp_prepare_workspace(N, m), "rvgp_gp_prepare: workspace too small");
  cudaStream_t st = as_stream(stream);
  int rc;
  if (mode == 1)
    rc = gram_f32_out64(Phi32, m, Phi32, m, N, m, m, C, m, 1.0, 0.0, workspace, ws_bytes, st);
  else
    rc = gram<double>(Phi, m, Phi, m, N, m, m, C, m, 1.0, 0.0, workspace, ws_bytes, st);
  if (rc) return rc;
  // b and yy: one column reduction of [Phi y | y y] in FP64 (after the Gram's
  // scratch, which the Gram's reduction may still be reading in stream order)
  const size_t gbytes = std::max(gram_workspace<double>(N, m, m), gram_workspace<float>(N, m, m));
  double* part = reinterpret_cast<double*>(static_cast<char*>(workspace) + ((gbytes + 255) & ~size_t(255)));
  const int nc = phity_chunks(N);
  const long long chunk = (N + nc - 1) / nc;
  rvgp::note_launch();
  phity_partial<<<dim3(nc, ceil_div(m + 1, 32)), 256, 0, st>>>(Phi, y, N, m, chunk, part);
  rvgp::note_launch();
  phity_final<<<ceil_div(m + 1, 256), 256, 0, st>>>(part, nc, m, b, yy);
  RVGP_LAUNCH_CHECK("rvgp_gp_prepare");
  return RVGP_OK;
}

RVGP_API size_t rvgp_gp_lml_workspace(int m) {
  Workspace ws(nullptr, 0);
  carve_lml(ws, m);
  return ws.used;
}

RVGP_API size_t rvgp_gp_state_size(int m) { return (size_t)m * m + 4 * (size_t)m; }

// Log marginal likelihood and its gradient.  theta (device, 4 doubles) =
// [nu, kappa, sigma_f, noise variance]; out (device, 5 doubles) = [LML,
// ∂/∂nu, ∂/∂kappa, ∂/∂sigma_f, ∂/∂noise] (NaN when A is not positive definite).
// state (device, rvgp_gp_state_size(m) doubles) keeps what predict needs.
// Fully stream-ordered (no host synchronisation).
RVGP_API int rvgp_gp_lml(const double* C, const double* b, const double* yy, long long N, int m,
                         const double* evals, double n_rows, int typ, const double* theta, double* out, double* state,
                         void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(C && b && yy && evals && theta && out && state, "rvgp_gp_lml: null pointer");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_gp_lml_workspace(m), "rvgp_gp_lml: workspace too small");
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  LmlBufs B = carve_lml(ws, m);
  return lml_chain(B, C, b, yy, N, m, evals, n_rows, typ, theta, out, state, st);
}

// Hyperparameter learning on the device: `steps` Adam steps (Kingma & Ba, with
// bias correction) on the unconstrained parameters u, value = softplus(u) +
// lower, minimising −LML with the gradient above; no host synchronisation.
// theta0 (device, 4): start values [nu, kappa, sigma_f, noise]; lower / mask
// (host, 4 each): lower bounds and trainable flags; hyper = lr, beta1, beta2,
// eps.  theta_out (device, 4) = final values; hist (device, steps, optional) =
// LML before each step; out / state as for rvgp_gp_lml, evaluated at theta_out.
RVGP_API int rvgp_gp_fit_adam(const double* C, const double* b, const double* yy, long long N, int m,
                              const double* evals, double n_rows, int typ, const double* theta0, const double* lower,
                              const int* mask, int steps, double lr, double beta1, double beta2, double eps,
                              double* theta_out, double* hist, double* out, double* state, void* workspace,
                              size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(C && b && yy && evals && theta0 && lower && mask && theta_out && out && state,
                 "rvgp_gp_fit_adam: null pointer");
  RVGP_CHECK_ARG(steps >= 0 && ws_bytes >= rvgp_gp_lml_workspace(m), "rvgp_gp_fit_adam: bad steps or workspace");
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  LmlBufs B = carve_lml(ws, m);
  cudaMemcpyAsync(B.lower, lower, 4 * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(B.mask, mask, 4 * sizeof(int), cudaMemcpyHostToDevice, st);
  rvgp::note_launch(); adam_init<<<1, 32, 0, st>>>(theta0, B.lower, B.theta, B.adam);
  for (int s = 0; s < steps; ++s) {
    int rc = lml_chain(B, C, b, yy, N, m, evals, n_rows, typ, B.theta, out, state, st);
    if (rc) return rc;
    rvgp::note_launch(); adam_step<<<1, 32, 0, st>>>(B.theta, B.adam, B.lower, B.mask, out, s, lr, beta1, beta2, eps,
                                                     hist);
  }
  int rc = lml_chain(B, C, b, yy, N, m, evals, n_rows, typ, B.theta, out, state, st);
  if (rc) return rc;
  cudaMemcpyAsync(theta_out, B.theta, 4 * sizeof(double), cudaMemcpyDeviceToDevice, st);
  RVGP_LAUNCH_CHECK("rvgp_gp_fit_adam");
  return RVGP_OK;
}

RVGP_API size_t rvgp_gp_predict_workspace(long long Nte, int m, int mode) {
  return (mode == 1 ? sizeof(float) : sizeof(double)) * ((size_t)Nte * m + (size_t)m * m) + 1024;
}

// Posterior mean and marginal variance at Nte test rows (Phi_star, Nte x m;
// mode 1 also needs Phi_star32) from the state of the last rvgp_gp_lml call.
RVGP_API int rvgp_gp_predict(const double* Phi_star, const float* Phi_star32, long long Nte, int m, int mode,
                             const double* state, double* mean, double* var, void* workspace, size_t ws_bytes,
                             void* stream) {
  RVGP_CHECK_ARG(Phi_star && state && mean && var, "rvgp_gp_predict: null pointer");
  RVGP_CHECK_ARG(mode == 0 || Phi_star32, "rvgp_gp_predict: mode 1 needs Phi_star32");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_gp_predict_workspace(Nte, m, mode), "rvgp_gp_predict: workspace too small");
  cudaStream_t st = as_stream(stream);
  const long long mm = (long long)m * m;
  if (Nte == 0) return RVGP_OK;
  if (mode == 1) {
    Workspace ws(workspace, ws_bytes);
    float* Bt = ws.take<float>(mm);
    float* P = ws.take<float>((size_t)Nte * m);
    rvgp::note_launch(); make_Bt<float><<<ceil_div(mm, 256), 256, 0, st>>>(state, m, Bt);
    int rc = gemm_nn<float>(Phi_star32, m, Bt, m, Nte, m, m, P, m, 1.f, 0.f, st);
    if (rc) return rc;
    rvgp::note_launch(); predict_rows<float><<<ceil_div(Nte * 32, 256), 256, 0, st>>>(Phi_star, Nte, m, state, P, mean, var);
  } else {
    Workspace ws(workspace, ws_bytes);
    double* Bt = ws.take<double>(mm);
    double* P = ws.take<double>((size_t)Nte * m);
    rvgp::note_launch(); make_Bt<double><<<ceil_div(mm, 256), 256, 0, st>>>(state, m, Bt);
    int rc = gemm_nn<double>(Phi_star, m, Bt, m, Nte, m, m, P, m, 1.0, 0.0, st);
    if (rc) return rc;
    rvgp::note_launch(); predict_rows<double><<<ceil_div(Nte * 32, 256), 256, 0, st>>>(Phi_star, Nte, m, state, P, mean, var);
  }
  RVGP_LAUNCH_CHECK("rvgp_gp_predict");
  return RVGP_OK;
}

#define RVGP_LOCAL_D_DISPATCH(d, F) \
  switch (d) {                      \
    case 1: F(1); break;            \
    case 2: F(2); break;            \
    case 3: F(3); break;            \
    case 4: F(4); break;            \
    case 5: F(5); break;            \
    case 6: F(6); break;            \
    case 7: F(7); break;            \
    default: F(8); break;           \
  }

namespace {
struct LocalPrepareBufs {
  double *Lf, *yt, *yyp, *Ut;
  float* Ut32;
  void* gram_ws;
  size_t gram_bytes;
  double* part;
};
LocalPrepareBufs carve_local_prepare(Workspace& ws, int nt, int d, int m, int mode) {
  LocalPrepareBufs B;
  const long long rows = (long long)nt * d;
  B.Lf = ws.take<double>((size_t)nt * d * d);
  B.yt = ws.take<double>((size_t)rows);
  B.yyp = ws.take<double>((size_t)std::max(nt, 1));
  B.Ut = ws.take<double>((size_t)rows * m);
  B.Ut32 = mode == 1 ? ws.take<float>((size_t)rows * m) : nullptr;
  B.gram_bytes = mode == 1 ? gram_workspace<float>(rows, m, m) : gram_workspace<double>(rows, m, m);
  B.gram_ws = ws.take<char>(B.gram_bytes);
  B.part = ws.take<double>((size_t)phity_chunks(rows) * (m + 1));
  return B;
}
}  // namespace

RVGP_API size_t rvgp_gp_prepare_local_workspace(int nt, int d, int m, int mode) {
  Workspace ws(nullptr, 0);
  carve_local_prepare(ws, nt, d, m, mode);
  return ws.used + 256;
}

// C = ΦᵀΦ (m x m), b = Φᵀy (m) and yy = yᵀy for the lifted rows Φ of the
// training points idx (nt) without forming them: Φ_i = T_i U_i (gauges T,
// n x D x ld with d <= ld used columns; U, n*d x m, the eigenvectors of the
// connection Laplacian in local coordinates; vectors vec, n x D).  Per point
// the d x d Cholesky factor L_i of T_iᵀT_i gives the d rows L_iᵀU_i and the
// targets L_i⁻¹T_iᵀy_i whose Gram and products are exactly ΦᵀΦ and Φᵀy
// (RVGP/main.py:24-50 forms the D rows per point; the GP algebra only needs
// these three sums).  mode 1 forms C from FP32 rows with FP64-reduced partial
// sums; b and yy are FP64 in both modes.  Stream-ordered, no synchronisation.
RVGP_API int rvgp_gp_prepare_local(const double* T, int n, int D, int ld, int d, const double* U, int m,
                                   const int* idx, int nt, const double* vec, int mode, double* C, double* b,
                                   double* yy, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(T && U && idx && vec && C && b && yy, "rvgp_gp_prepare_local: null pointer");
  RVGP_CHECK_ARG(n >= 1 && D >= 1 && m >= 1 && nt >= 1 && d >= 1 && d <= ld && d <= D && d <= kMaxLocalD,
                 "rvgp_gp_prepare_local: bad sizes (d must be in [1, min(ld, D, %d)])", kMaxLocalD);
  RVGP_CHECK_ARG(mode == 0 || mode == 1, "rvgp_gp_prepare_local: mode must be 0 or 1");
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_gp_prepare_local_workspace(nt, d, m, mode),
                 "rvgp_gp_prepare_local: workspace too small");
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  LocalPrepareBufs B = carve_local_prepare(ws, nt, d, m, mode);
  const long long rows = (long long)nt * d;
  const int wb = ceil_div((long long)nt * 32, 256);
#define RVGP_LF(DD) local_factor_kernel<DD><<<wb, 256, 0, st>>>(T, D, ld, idx, nt, vec, B.Lf, B.yt, B.yyp)
  rvgp::note_launch();
  RVGP_LOCAL_D_DISPATCH(d, RVGP_LF)
#undef RVGP_LF
  rvgp::note_launch();
  local_rows_kernel<double><<<ceil_div(rows * m, 256), 256, 0, st>>>(U, m, d, idx, nt, B.Lf, B.Ut);
  int rc;
  if (mode == 1) {
    rvgp::note_launch();
    local_rows_kernel<float><<<ceil_div(rows * m, 256), 256, 0, st>>>(U, m, d, idx, nt, B.Lf, B.Ut32);
    rc = gram_f32_out64(B.Ut32, m, B.Ut32, m, rows, m, m, C, m, 1.0, 0.0, B.gram_ws, B.gram_bytes, st);
  } else {
    rc = gram<double>(B.Ut, m, B.Ut, m, rows, m, m, C, m, 1.0, 0.0, B.gram_ws, B.gram_bytes, st);
  }
  if (rc) return rc;
  const int nc = phity_chunks(rows);
  const long long chunk = (rows + nc - 1) / nc;
  rvgp::note_launch();
  phity_partial<<<dim3(nc, ceil_div(m + 1, 32)), 256, 0, st>>>(B.Ut, B.yt, rows, m, chunk, B.part);
  rvgp::note_launch();
  phity_final<<<ceil_div(m + 1, 256), 256, 0, st>>>(B.part, nc, m, b, yy);  // yy: |L⁻¹Tᵀy|², replaced next
  rvgp::note_launch();
  sum_fixed<<<1, 1024, 0, st>>>(B.yyp, nt, yy);
  RVGP_LAUNCH_CHECK("rvgp_gp_prepare_local");
  return RVGP_OK;
}

RVGP_API size_t rvgp_gp_predict_local_workspace(int nt, int d, int m, int mode) {
  const size_t s = mode == 1 ? sizeof(float) : sizeof(double);
  return s * (2 * (size_t)nt * d * m + (size_t)m * m) + 1024;
}

// Posterior mean and marginal variance (each nt x D, rows = test points idx,
// columns = ambient coordinates, as RVGP/main.py:102-116 reshapes them) from
// the state of the last likelihood evaluation, without forming the lifted
// rows: Q = U_te Bt (rows of U at the test points times r ∘ L_A⁻ᵀ), then per
// point the d x d Gram of its Q rows and the gauge's quadratic forms.  mode 1
// forms Q in FP32.  Stream-ordered, no synchronisation.
RVGP_API int rvgp_gp_predict_local(const double* T, int n, int D, int ld, int d, const double* U, int m,
                                   const int* idx, int nt, int mode, const double* state, double* mean, double* var,
                                   void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(T && U && idx && state && mean && var, "rvgp_gp_predict_local: null pointer");
  RVGP_CHECK_ARG(n >= 1 && D >= 1 && m >= 1 && nt >= 0 && d >= 1 && d <= ld && d <= D && d <= kMaxLocalD,
                 "rvgp_gp_predict_local: bad sizes");
  RVGP_CHECK_ARG(mode == 0 || mode == 1, "rvgp_gp_predict_local: mode must be 0 or 1");
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_gp_predict_local_workspace(nt, d, m, mode),
                 "rvgp_gp_predict_local: workspace too small");
  if (nt == 0) return RVGP_OK;
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  const long long rows = (long long)nt * d, mm = (long long)m * m;
  const int wb = ceil_div((long long)nt * 32, 256);
  int rc;
  if (mode == 1) {
    float* Bt = ws.take<float>(mm);
    float* Ut = ws.take<float>((size_t)rows * m);
    float* Q = ws.take<float>((size_t)rows * m);
    rvgp::note_launch(); make_Bt<float><<<ceil_div(mm, 256), 256, 0, st>>>(state, m, Bt);
    rvgp::note_launch(); gather_local_rows<float><<<ceil_div(rows * m, 256), 256, 0, st>>>(U, m, d, idx, nt, Ut);
    rc = gemm_nn<float>(Ut, m, Bt, m, rows, m, m, Q, m, 1.f, 0.f, st);
    if (rc) return rc;
#define RVGP_PL(DD) predict_local_kernel<DD, float><<<wb, 256, 0, st>>>(T, D, ld, U, m, idx, nt, state, Q, mean, var)
    rvgp::note_launch();
    RVGP_LOCAL_D_DISPATCH(d, RVGP_PL)
#undef RVGP_PL
  } else {
    double* Bt = ws.take<double>(mm);
    double* Ut = ws.take<double>((size_t)rows * m);
    double* Q = ws.take<double>((size_t)rows * m);
    rvgp::note_launch(); make_Bt<double><<<ceil_div(mm, 256), 256, 0, st>>>(state, m, Bt);
    rvgp::note_launch(); gather_local_rows<double><<<ceil_div(rows * m, 256), 256, 0, st>>>(U, m, d, idx, nt, Ut);
    rc = gemm_nn<double>(Ut, m, Bt, m, rows, m, m, Q, m, 1.0, 0.0, st);
    if (rc) return rc;
#define RVGP_PL(DD) predict_local_kernel<DD, double><<<wb, 256, 0, st>>>(T, D, ld, U, m, idx, nt, state, Q, mean, var)
    rvgp::note_launch();
    RVGP_LOCAL_D_DISPATCH(d, RVGP_PL)
#undef RVGP_PL
  }
  RVGP_LAUNCH_CHECK("rvgp_gp_predict_local");
  return RVGP_OK;
}

// K = (X S) X2ᵀ (N1 x N2) and its diagonal for X2 = X (RVGP/kernels.py:55-67).
RVGP_API int rvgp_kernel_matrix(const double* X, long long N1, const double* X2, long long N2, int m,
                                const double* S, double* K, void* stream) {
  RVGP_CHECK_ARG(X && X2 && S && K, "rvgp_kernel_matrix: null pointer");
  dim3 grid(ceil_div(N2, 64), ceil_div(N1, 64));
  rvgp::note_launch(); kernel_matrix<<<grid, 256, 0, as_stream(stream)>>>(X, N1, X2, N2, m, S, K);
  RVGP_LAUNCH_CHECK("rvgp_kernel_matrix");
  return RVGP_OK;
}

RVGP_API int rvgp_kernel_diag(const double* X, long long N, int m, const double* S, double* out, void* stream) {
  RVGP_CHECK_ARG(X && S && out, "rvgp_kernel_diag: null pointer");
  rvgp::note_launch(); kernel_diag<<<ceil_div(N * 32, 256), 256, 0, as_stream(stream)>>>(X, N, m, S, out);
  RVGP_LAUNCH_CHECK("rvgp_kernel_diag");
  return RVGP_OK;
}
