// Heat / vector diffusion on the graph and connection Laplacians.
//
// Replaces scalar_diffusion / vector_diffusion (RVGP/smoothing.py:8-63).  The
// reference forms the dense exponential scipy.linalg.expm(-t A) (O(N³), 10 s at
// n = 2000, infeasible beyond a few thousand points).  Here:
//
//  * exact action  y = exp(-tA) x  for symmetric PSD A with spectrum in [0, b]:
//    with s = 2A/b - I and α = t b / 2,
//        exp(-tA) = e^{-α} [ I_0(α) + 2 Σ_{k>=1} (-1)^k I_k(α) T_k(s) ]
//    (Chebyshev expansion of e^{-α s}; I_k modified Bessel functions).  The
//    scaled coefficients e^{-α} I_k(α) decay like exp(-k²/2α), so about
//    sqrt(2 α ln(1/ε)) terms suffice; each term is one fused block-sparse
//    product (three-term recurrence + accumulation).
//  * spectral form  y = Φ e^{-tΛ} Φᵀ x  on computed eigenpairs (the
//    method="spectral" branch of smoothing.py:17-32, written as intended).
//  * the normalisation of vector_diffusion (smoothing.py:59-62):
//        out * (e^{-tL}|x|) / ((e^{-tL}1) |out|)   per point.
#include "common.cuh"
#include "linalg.cuh"
#include <math.h>
#include <vector>

namespace rvgp {
namespace {

// Tn = al*(A Tc) + be*Tc + ga*Tp ;  Y += c * Tn   (b <= 4 columns, ld = b)
template <int DB>
__global__ void cheb_step(int n, const int* __restrict__ indptr, const int* __restrict__ indices,
                          const double* __restrict__ vals, const double* __restrict__ Tc, const double* __restrict__ Tp,
                          double* __restrict__ Tn, double* __restrict__ Y, int b, double al, double be, double ga,
                          double c) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * b) return;
  const int i = (int)(e / b), col = (int)(e % b);
  double acc[DB];
#pragma unroll
  for (int p = 0; p < DB; ++p) acc[p] = 0.0;
  for (int t = indptr[i]; t < indptr[i + 1]; ++t) {
    const int j = indices[t];
#pragma unroll
    for (int q = 0; q < DB; ++q) {
      const double x = Tc[((size_t)j * DB + q) * b + col];
#pragma unroll
      for (int p = 0; p < DB; ++p) acc[p] = fma(vals[((size_t)t * DB + p) * DB + q], x, acc[p]);
    }
  }
#pragma unroll
  for (int p = 0; p < DB; ++p) {
    const size_t r = ((size_t)i * DB + p) * b + col;
    double v = al * acc[p] + be * Tc[r];
    if (Tp) v += ga * Tp[r];
    Tn[r] = v;
    Y[r] += c * v;
  }
}

__global__ void axpby_init(const double* __restrict__ X, double* __restrict__ T0, double* __restrict__ Y, long long cnt,
                           double c0) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= cnt) return;
  T0[e] = X[e];
  Y[e] = c0 * X[e];
}

// e^{-α} I_k(α), k = 0..K, by Miller's backward recurrence normalised with
// e^{α} = I_0 + 2 Σ I_k.
std::vector<double> scaled_bessel(double alpha, int K) {
  std::vector<double> out(K + 1, 0.0);
  if (alpha <= 0.0) {
    out[0] = 1.0;
    return out;
  }
  const int start = K + 32 + (int)(10.0 * sqrt(K + alpha));
  std::vector<double> v(start + 2, 0.0);
  v[start + 1] = 0.0;
  v[start] = 1e-300;
  for (int k = start; k >= 1; --k) {
    v[k - 1] = (2.0 * k / alpha) * v[k] + v[k + 1];
    if (v[k - 1] > 1e250) {
      for (int j = k - 1; j <= start + 1; ++j) v[j] *= 1e-250;
    }
  }
  double norm = v[0];
  for (int k = 1; k <= start; ++k) norm += 2.0 * v[k];
  for (int k = 0; k <= K; ++k) out[k] = v[k] / norm;
  return out;
}

int terms_for(double alpha) {
  // Gaussian decay of e^{-α} I_k(α): exp(-k²/2α) < 1e-18 beyond sqrt(2 α · 41.4)
  int K = (int)ceil(sqrt(2.0 * alpha * 41.5)) + 16;
  if (alpha < 4.0) K = 40;
  return K;
}

__global__ void combine_vector_diffusion(const double* __restrict__ out_loc, const double* __restrict__ lsc, int n,
                                         int d, double* __restrict__ res) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // lsc[(i*2 + 0)] = e^{-tL}|x| ; lsc[(i*2 + 1)] = e^{-tL} 1
  double nrm = 0.0;
  for (int q = 0; q < d; ++q) nrm += out_loc[(size_t)i * 2 * d + q * 2] * out_loc[(size_t)i * 2 * d + q * 2];
  nrm = sqrt(nrm);
  const double f = lsc[(size_t)i * 2] / (lsc[(size_t)i * 2 + 1] * nrm);
  for (int q = 0; q < d; ++q) res[(size_t)i * d + q] = out_loc[(size_t)i * 2 * d + q * 2] * f;
}

__global__ void pack_columns(const double* __restrict__ x_loc, int n, int d, double* __restrict__ Xc,
                             double* __restrict__ Xs) {
  // Xc: (n*d, 2) = [x, 0]; Xs: (n, 2) = [|x_i|, 1]
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int q = 0; q < d; ++q) {
    const double v = x_loc[(size_t)i * d + q];
    Xc[((size_t)i * d + q) * 2] = v;
    Xc[((size_t)i * d + q) * 2 + 1] = 0.0;
    s += v * v;
  }
  Xs[(size_t)i * 2] = sqrt(s);
  Xs[(size_t)i * 2 + 1] = 1.0;
}

// exp(-t A) X = e^{-t mu} exp(-t (A - mu I)) X.  Shifting by mu <= λ_min keeps
// the slowest component O(1) through the sum: without it the terms (size
// ~1/sqrt(2πα)) cancel down to e^{-t λ_min} and the relative error grows like
// ε e^{t λ_min}.  The spectrum of A - mu I lies in [0, bound - mu].
template <int DB>
int run_expm(int n, const int* indptr, const int* indices, const double* vals, const double* X, int b, double t,
             double bound, double mu, bool rescale, double* Y, double* ws3, cudaStream_t st) {
  const long long cnt = (long long)n * DB * b;
  const double bp = bound - mu;
  const double alpha = 0.5 * t * bp;
  const int K = terms_for(alpha);
  std::vector<double> c = scaled_bessel(alpha, K);
  const double scale = rescale ? exp(-t * mu) : 1.0;
  for (double& v : c) v *= scale;
  double* T0 = ws3;
  double* T1 = ws3 + cnt;
  double* T2 = ws3 + 2 * cnt;
  const int grid = ceil_div(cnt / DB, 256);
  rvgp::note_launch(); axpby_init<<<ceil_div(cnt, 256), 256, 0, st>>>(X, T0, Y, cnt, c[0]);
  // T1 = s x = (2/b')(A - mu) x - x ; Y += -2 I_1 T1
  rvgp::note_launch(); cheb_step<DB><<<grid, 256, 0, st>>>(n, indptr, indices, vals, T0, nullptr, T1, Y, b, 2.0 / bp,
                                                           -(2.0 * mu / bp + 1.0), 0.0, -2.0 * c[1]);
  double *tp = T0, *tc = T1, *tn = T2;
  for (int k = 1; k < K; ++k) {
    const double ck = ((k + 1) % 2 ? -2.0 : 2.0) * c[k + 1];
    rvgp::note_launch(); cheb_step<DB><<<grid, 256, 0, st>>>(n, indptr, indices, vals, tc, tp, tn, Y, b, 4.0 / bp,
                                                             -(4.0 * mu / bp + 2.0), -1.0, ck);
    double* tmp = tp;
    tp = tc;
    tc = tn;
    tn = tmp;
  }
  return check_launch("rvgp_expm_action");
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_expm_action_workspace(int n, int DB, int b) { return sizeof(double) * 3 * (size_t)n * DB * b + 256; }

// Y = exp(-t A) X for the block-CSR A (n block rows, DB x DB blocks, spectrum
// in [shift, bound]); X, Y: (n*DB) x b row-major with ld = b, b <= 4.  shift:
// a lower bound of the spectrum (0 when unknown; λ_min gives full accuracy
// at large t).
RVGP_API int rvgp_expm_action(const int* indptr, const int* indices, const double* vals, int n, int DB, const double* X,
                              int b, double t, double bound, double shift, double* Y, void* workspace,
                              size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(indptr && indices && vals && X && Y && b >= 1 && b <= 4, "rvgp_expm_action: bad arguments");
  RVGP_CHECK_ARG(t >= 0 && bound > 0 && shift >= 0 && shift < bound,
                 "rvgp_expm_action: need t >= 0 and 0 <= shift < bound");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_expm_action_workspace(n, DB, b), "rvgp_expm_action: workspace too small");
  cudaStream_t st = as_stream(stream);
  double* ws3 = static_cast<double*>(workspace);
  switch (DB) {
    case 1: return run_expm<1>(n, indptr, indices, vals, X, b, t, bound, shift, true, Y, ws3, st);
    case 2: return run_expm<2>(n, indptr, indices, vals, X, b, t, bound, shift, true, Y, ws3, st);
    case 3: return run_expm<3>(n, indptr, indices, vals, X, b, t, bound, shift, true, Y, ws3, st);
    case 4: return run_expm<4>(n, indptr, indices, vals, X, b, t, bound, shift, true, Y, ws3, st);
  }
  set_error("rvgp_expm_action: block size %d unsupported", DB);
  return RVGP_ENOTSUP;
}

RVGP_API size_t rvgp_vector_diffusion_workspace(int n, int d) {
  const size_t c = (size_t)n * d * 2, s = (size_t)n * 2;
  return sizeof(double) * (2 * c + 2 * s) + rvgp_expm_action_workspace(n, d, 2) + rvgp_expm_action_workspace(n, 1, 2) +
         1024;
}

// vector_diffusion(x, t, Lc, L, normalise=True) with the exact exponential
// action: x_loc (n, d) -> out (n, d).  bound_L / bound_Lc: spectral upper
// bounds; shift_Lc: a lower bound of Lc's spectrum (its smallest eigenvalue).
// The factor e^{-t shift_Lc} cancels in the normalisation and is not applied.
RVGP_API int rvgp_vector_diffusion(const int* indptr, const int* indices, const double* L_vals, const double* Lc_vals,
                                   int n, int d, const double* x_loc, double t, double bound_L, double bound_Lc,
                                   double shift_Lc, double* out, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(ws_bytes >= rvgp_vector_diffusion_workspace(n, d), "rvgp_vector_diffusion: workspace too small");
  RVGP_CHECK_ARG(d >= 1 && d <= 4 && shift_Lc >= 0 && shift_Lc < bound_Lc, "rvgp_vector_diffusion: bad d or shift");
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  double* Xc = ws.take<double>((size_t)n * d * 2);
  double* Yc = ws.take<double>((size_t)n * d * 2);
  double* Xs = ws.take<double>((size_t)n * 2);
  double* Ys = ws.take<double>((size_t)n * 2);
  const size_t wc = rvgp_expm_action_workspace(n, d, 2), wsz = rvgp_expm_action_workspace(n, 1, 2);
  void* w1 = ws.take<char>(wc);
  void* w2 = ws.take<char>(wsz);
  rvgp::note_launch(); pack_columns<<<ceil_div(n, 128), 128, 0, st>>>(x_loc, n, d, Xc, Xs);
  double* w1d = static_cast<double*>(w1);
  int rc;
  switch (d) {
    case 1: rc = run_expm<1>(n, indptr, indices, Lc_vals, Xc, 2, t, bound_Lc, shift_Lc, false, Yc, w1d, st); break;
    case 2: rc = run_expm<2>(n, indptr, indices, Lc_vals, Xc, 2, t, bound_Lc, shift_Lc, false, Yc, w1d, st); break;
    case 3: rc = run_expm<3>(n, indptr, indices, Lc_vals, Xc, 2, t, bound_Lc, shift_Lc, false, Yc, w1d, st); break;
    default: rc = run_expm<4>(n, indptr, indices, Lc_vals, Xc, 2, t, bound_Lc, shift_Lc, false, Yc, w1d, st); break;
  }
  if (rc) return rc;
  rc = rvgp_expm_action(indptr, indices, L_vals, n, 1, Xs, 2, t, bound_L, 0.0, Ys, w2, wsz, stream);
  if (rc) return rc;
  rvgp::note_launch(); combine_vector_diffusion<<<ceil_div(n, 128), 128, 0, st>>>(Yc, Ys, n, d, out);
  RVGP_LAUNCH_CHECK("rvgp_vector_diffusion");
  return RVGP_OK;
}

RVGP_API size_t rvgp_spectral_diffusion_workspace(long long N, int m, int b) {
  return sizeof(double) * (size_t)m * b + gram_workspace<double>(N, m, b) + 512;
}

// Y = Φ diag(exp(-t λ)) Φᵀ X with orthonormal Φ (N x m); X, Y: N x b (ld = b).
__global__ void scale_by_exp(double* __restrict__ Z, int m, int b, const double* __restrict__ lam, double t) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)m * b) return;
  Z[e] *= exp(-t * lam[e / b]);
}

RVGP_API int rvgp_spectral_diffusion(const double* Phi, long long N, int m, const double* lam, const double* X, int b,
                                     double t, double* Y, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(Phi && lam && X && Y, "rvgp_spectral_diffusion: null pointer");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_spectral_diffusion_workspace(N, m, b), "rvgp_spectral_diffusion: workspace");
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  double* Z = ws.take<double>((size_t)m * b);
  const size_t gb = gram_workspace<double>(N, m, b);
  void* gw = ws.take<char>(gb);
  int rc = gram<double>(Phi, m, X, b, N, m, b, Z, b, 1.0, 0.0, gw, gb, st);
  if (rc) return rc;
  rvgp::note_launch(); scale_by_exp<<<ceil_div((long long)m * b, 256), 256, 0, st>>>(Z, m, b, lam, t);
  rc = gemm_nn<double>(Phi, m, Z, b, N, m, b, Y, b, 1.0, 0.0, st);
  if (rc) return rc;
  RVGP_LAUNCH_CHECK("rvgp_spectral_diffusion");
  return RVGP_OK;
}
