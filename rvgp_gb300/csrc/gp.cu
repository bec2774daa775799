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
//   R = diag(√S),  A = I + R C R / σ² = L_A L_Aᵀ
//   log|K_y| = N log σ² + 2 Σ log diag L_A
//   yᵀK_y⁻¹y = (yᵀy − |L_A⁻¹ R b|² / σ²) / σ²
//   Φᵀα = (b − C R A⁻¹ R b / σ²) / σ²                       (α = K_y⁻¹ y)
//   diag(ΦᵀK_y⁻¹Φ) = (diag C − diag(EᵀE) / σ²) / σ²,   E = L_A⁻¹ R C
//   ∂LML/∂S_l = ½[(Φᵀα)_l² − diag(ΦᵀK_y⁻¹Φ)_l]
//   ∂LML/∂σ²  = ½[αᵀα − tr K_y⁻¹],  tr K_y⁻¹ = (N − m + |L_A⁻¹|_F²)/σ²
// and the chain rule through S(ν, κ, σ_f) including the Σs normalisation.
// Posterior (predict_f, full_cov=False): mean = Φ* (S ∘ Φᵀα),
// var = diag(Φ* R A⁻¹ R Φ*ᵀ) = |L_A⁻¹ R φ*_i|² per test row.
// The m x m factorisation is FP64 in both forms (cond(A) grows like
// λ_max(RCR)/σ²); the tall products (C = ΦᵀΦ, Φ* Bᵀ) are FP32 in the mixed form.
#include "common.cuh"
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

// B (m x m) = diag(r) C with r = sqrt(S)
__global__ void scale_rows_sqrtS(const double* __restrict__ C, int m, const double* __restrict__ S,
                                 double* __restrict__ B) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)m * m) return;
  B[e] = sqrt(S[e / m]) * C[e];
}

// state layout (doubles): [0, m²) L_A⁻¹, then pa = Φᵀα (m), S (m), r (m), w (m)
__global__ void __launch_bounds__(kCTA) lml_epilogue(const double* __restrict__ C, const double* __restrict__ b,
                                                     const double* __restrict__ yy, long long N, int m,
                                                     const double* __restrict__ LA, const double* __restrict__ E,
                                                     const double* __restrict__ S, const double* __restrict__ dS,
                                                     const double* __restrict__ theta, const int* __restrict__ info,
                                                     double* __restrict__ state, double* __restrict__ tmp,
                                                     double* __restrict__ out) {
  __shared__ double sh[kCTA];
  const double s2 = theta[3];
  if (*info != 0) {
    if (threadIdx.x == 0)
      for (int t = 0; t < 5; ++t) out[t] = nan("");
    return;
  }
  const double* Li = state;  // L_A⁻¹ (lower)
  double* pa = state + (size_t)m * m;
  double* Sst = pa + m;
  double* r = Sst + m;
  double* w = r + m;
  double* z = tmp;
  double* rw = tmp + m;
  double* Crw = tmp + 2 * m;
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    r[l] = sqrt(S[l]);
    Sst[l] = S[l];
  }
  __syncthreads();
  // z = L_A⁻¹ (r ∘ b)
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    double s = 0.0;
    for (int l = 0; l <= k; ++l) s += Li[(size_t)k * m + l] * r[l] * b[l];
    z[k] = s;
  }
  __syncthreads();
  // w = L_A⁻ᵀ z = A⁻¹ R b ;  rw = r ∘ w
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    double s = 0.0;
    for (int k = l; k < m; ++k) s += Li[(size_t)k * m + l] * z[k];
    w[l] = s;
    rw[l] = r[l] * s;
  }
  __syncthreads();
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < m; ++j) s += C[(size_t)l * m + j] * rw[j];
    Crw[l] = s;
  }
  __syncthreads();
  double zz = 0.0, logd = 0.0, rwb = 0.0, rwCrw = 0.0, fro = 0.0;
  double g0 = 0.0, g1 = 0.0, g2 = 0.0;
  for (int l = threadIdx.x; l < m; l += blockDim.x) {
    zz += z[l] * z[l];
    logd += log(LA[(size_t)l * m + l]);
    rwb += rw[l] * b[l];
    rwCrw += rw[l] * Crw[l];
    const double p_l = (b[l] - Crw[l] / s2) / s2;
    pa[l] = p_l;
    double dm = 0.0;
    for (int k = 0; k < m; ++k) dm += E[(size_t)k * m + l] * E[(size_t)k * m + l];
    const double gl = 0.5 * (p_l * p_l - (C[(size_t)l * m + l] - dm / s2) / s2);
    g0 += gl * dS[l];
    g1 += gl * dS[m + l];
    g2 += gl * dS[2 * m + l];
  }
  for (long long e = threadIdx.x; e < (long long)m * m; e += blockDim.x) {
    const int i = (int)(e / m), j = (int)(e % m);
    if (j <= i) fro += Li[e] * Li[e];
  }
  zz = block_sum(zz, sh);
  logd = block_sum(logd, sh);
  rwb = block_sum(rwb, sh);
  rwCrw = block_sum(rwCrw, sh);
  fro = block_sum(fro, sh);
  g0 = block_sum(g0, sh);
  g1 = block_sum(g1, sh);
  g2 = block_sum(g2, sh);
  if (threadIdx.x == 0) {
    const double Nd = (double)N;
    const double quad = (yy[0] - zz / s2) / s2;
    const double logdet = Nd * log(s2) + 2.0 * logd;
    const double lml = -0.5 * quad - 0.5 * logdet - 0.5 * Nd * log(2.0 * M_PI);
    const double a2 = (yy[0] - 2.0 * rwb / s2 + rwCrw / (s2 * s2)) / (s2 * s2);
    const double trk = (Nd - m + fro) / s2;
    out[0] = lml;
    out[1] = g0;
    out[2] = g1;
    out[3] = g2;
    out[4] = 0.5 * (a2 - trk);
  }
}

// Φ[(t*D + a), :] = src[(idx[t]*D + a), :],  y[(t*D + a)] = vec[idx[t]*D + a]
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

// Bt[l][k] = r_l L_A⁻¹[k][l]   (so that Φ* Bt = (L_A⁻¹ R Φ*ᵀ)ᵀ)
template <typename T>
__global__ void make_Bt(const double* __restrict__ state, int m, T* __restrict__ Bt) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)m * m) return;
  const int l = (int)(e / m), k = (int)(e % m);
  const double* r = state + (size_t)m * m + 2 * m;  // after L_A⁻¹, pa, S
  Bt[e] = (T)(k >= l ? r[l] * state[(size_t)k * m + l] : 0.0);
}

// mean_i = Σ_l Φ*_il S_l pa_l ; var_i = Σ_k P_ik²  (warp per row)
template <typename T>
__global__ void predict_rows(const double* __restrict__ Phi, long long Nte, int m, const double* __restrict__ state,
                             const T* __restrict__ P, double* __restrict__ mean, double* __restrict__ var) {
  const int lane = threadIdx.x & 31;
  const long long i = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (i >= Nte) return;
  const double* pa = state + (size_t)m * m;
  const double* S = pa + m;
  double sm = 0.0, sv = 0.0;
  for (int l = lane; l < m; l += 32) {
    sm += Phi[i * m + l] * S[l] * pa[l];
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
  double *S, *dS, *stmp, *A, *B, *E, *etmp;
  int* info;
};

LmlBufs carve_lml(Workspace& ws, int m) {
  LmlBufs b;
  b.S = ws.take<double>(m);
  b.dS = ws.take<double>(3 * (size_t)m);
  b.stmp = ws.take<double>(3 * (size_t)m);
  b.A = ws.take<double>((size_t)m * m);
  b.B = ws.take<double>((size_t)m * m);
  b.E = ws.take<double>((size_t)m * m);
  b.etmp = ws.take<double>(3 * (size_t)m);
  b.info = ws.take<int>(4);
  return b;
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
  return gram_workspace<double>(N, m, m) + gram_workspace<float>(N, m, m) + 1024;
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
  rc = gram<double>(Phi, m, y, 1, N, m, 1, b, 1, 1.0, 0.0, workspace, ws_bytes, st);
  if (rc) return rc;
  rc = gram<double>(y, 1, y, 1, N, 1, 1, yy, 1, 1.0, 0.0, workspace, ws_bytes, st);
  if (rc) return rc;
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
  const long long mm = (long long)m * m;
  rvgp::note_launch(); spectral_S_kernel<<<1, kCTA, 0, st>>>(evals, m, theta, n_rows, typ, B.S, B.dS, B.stmp);
  rvgp::note_launch(); build_A<<<ceil_div(mm, 256), 256, 0, st>>>(C, m, B.S, theta, B.A);
  int rc = cholesky<double>(B.A, m, m, B.info, st);
  if (rc) return rc;
  rc = tri_inv_lower<double>(B.A, m, m, state, m, st);
  if (rc) return rc;
  rvgp::note_launch(); scale_rows_sqrtS<<<ceil_div(mm, 256), 256, 0, st>>>(C, m, B.S, B.B);
  rc = gemm_nn<double>(state, m, B.B, m, m, m, m, B.E, m, 1.0, 0.0, st);
  if (rc) return rc;
  rvgp::note_launch(); lml_epilogue<<<1, kCTA, 0, st>>>(C, b, yy, N, m, B.A, B.E, B.S, B.dS, theta, B.info, state, B.etmp, out);
  RVGP_LAUNCH_CHECK("rvgp_gp_lml");
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
