// Mixed-precision hyperparameter fit: every Adam step of the GP likelihood
// (GPflow GPR + RVGP ManifoldKernel as used by RVGP/main.py:55-95 and
// RVGP/kernels.py:41-53) inside ONE launch of ONE CTA.
//
// Why one CTA: each step is a chain of small dependent operations on the
// m x m capacitance matrix A = I + R C R / σ² (R = diag(√S)).  Across SMs every
// link of that chain costs a kernel launch or a grid barrier (microseconds);
// inside one SM it costs a __syncthreads (tens of nanoseconds).  FP32 keeps the
// arithmetic on the SM's 128 FP32 lanes; GB300 executes FP64 at a small
// fraction of that rate.
//
// Per step (FP64 unless noted):
//   1. S(θ), ∂S/∂(ν, κ, σ_f) as rvgp_spectral_S, with the log / exp of each
//      eigenvalue term in FP32 (the accuracy of the FP32 algebra below)
//   2. Jacobi scaling: Δ_l = A_ll = 1 + S_l C_ll/σ², h_l = √S_l /(σ √Δ_l);
//      Ã = Δ^-½ A Δ^-½ has unit diagonal, Ã_ij = C_ij h_i h_j   (FP32)
//   3. Ã = L Lᵀ, blocked right-looking Cholesky in shared memory, 32-wide
//      panels: one warp factors the diagonal block and inverts it, all warps
//      solve the panel and update the trailing matrix         (FP32)
//   4. M = L⁻¹ in place, block columns right to left           (FP32)
//   5. z̃ = M u with u = Δ^-½ R b,  w̃ = Mᵀ z̃,  c_l = Σ_k M_kl² = (Ã⁻¹)_ll (FP32)
//   6. w = Δ^-½ w̃ = A⁻¹ R b;  (A⁻¹)_ll = c_l/Δ_l;
//      1 - (A⁻¹)_ll = (Δ_l - 1 - (c_l - 1))/Δ_l   (no cancellation: Δ_l - 1 is
//      formed from S directly and c_l - 1 is small when Ã is near I);
//      LML and its gradient from the same identities as rvgp_gp_lml;
//      log|A| = Σ log Δ_l + 2 Σ log L_ll
//   7. Adam update of the unconstrained parameters (thread 0).
// A non-positive FP32 pivot (or a parameter value that makes S_l or Δ_l
// non-positive) stops the launch with a status the host reads; the caller then
// runs the FP64 form.  After the loop the host evaluates the FP64
// likelihood once at the final θ, so the returned out / state (and the
// posterior built from them) are FP64.
#include "common.cuh"
#include "linalg.cuh"
#include "chol32.cuh"
#include <math.h>
#include <stdlib.h>
#include <algorithm>
#include <float.h>

namespace rvgp {
namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
using chol32::FB;
using chol32::lda32;
constexpr int kLdT = FB + 4;  // T rows: 16-byte aligned

// shared-memory layout (bytes), doubles first
struct Layout {
  size_t S, dS, tmp, Dm1, invD, invS, isd, rb, w, cdg, red, th, adam, outv, A, T, u, z, c, L, total;
};

__host__ __device__ inline Layout layout(int m) {
  Layout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += (bytes + 15) & ~size_t(15);
    return at;
  };
  const size_t d = 8 * (size_t)m, f = 4 * (size_t)m;
  L.S = take(d);
  L.dS = take(3 * d);
  L.tmp = take(3 * d);
  L.Dm1 = take(d);
  L.invD = take(d);
  L.invS = take(d);
  L.isd = take(d);
  L.rb = take(d);
  L.w = take(d);
  L.cdg = take(d);
  L.red = take(8 * 8 * (kWarps + 1));
  L.th = take(8 * 4);
  L.adam = take(8 * 16);
  L.outv = take(8 * 8);
  L.A = take(4 * (size_t)m * lda32(m));
  L.T = take(4 * (size_t)m * kLdT);
  L.u = take(f);
  L.z = take(f);
  L.c = take(f);
  L.L = take(f);
  L.total = o;
  return L;
}

// FP64 reductions.  A warp-wide FP64 instruction costs the same however few
// of its lanes hold data, so only the nw warps that hold the m per-eigenpair
// values take part, and warp 0 combines their partial sums.  Fixed order:
// xor tree within a warp, then a xor tree over the warps' partials.  Every
// thread receives the results.  All threads must call these.
template <int NV>
__device__ __forceinline__ void cta_sum(double (&v)[NV], double* red, int nw) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < nw) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int q = 0; q < NV; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < NV; ++q) red[q * kWarps + warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double s = lane < nw ? red[q * kWarps + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) red[8 * kWarps + q] = s;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = red[8 * kWarps + q];
}

__device__ __forceinline__ double cta_max(double v, double* red, int nw) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < nw) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) red[warp] = v;
  }
  __syncthreads();
  if (warp == 0) {
    double s = lane < nw ? red[lane] : -DBL_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
    if (lane == 0) red[8 * kWarps + 7] = s;
  }
  __syncthreads();
  return red[8 * kWarps + 7];
}

// T[i - r0][c] = Σ_{k=r0}^{i} M[i][k] Lt[c][k] with Lt[c][k] = A[j0+c][k]
// (the block column's L, copied into the free upper triangle), 4 x 4 tiles,
// operands read as float4 along k (r0 and ld are multiples of 4); the entries
// of M beyond the diagonal (k > i, the upper triangle's contents) are masked.
__device__ void inverse_product(const float* A, int ld, int j0, int m, float* T) {
  const int r0 = j0 + FB;
  const int R = m - r0;
  const int TR = (R + 3) / 4;
  const int tiles = TR * (FB / 4);
  for (int t = threadIdx.x; t < tiles; t += kThreads) {
    const int ti = t / (FB / 4), tc = t % (FB / 4);
    const int i0 = r0 + 4 * ti, c0 = 4 * tc;
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
    int oa[4], ob[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      oa[u] = min(i0 + u, m - 1) * ld;
      ob[u] = (j0 + c0 + u) * ld;
    }
    const int kend = min(i0 + 3, m - 1);  // last k any row of the tile uses
    for (int k = r0; k <= kend; k += 4) {
      float4 b[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = *reinterpret_cast<const float4*>(A + ob[v] + k);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float4 a = *reinterpret_cast<const float4*>(A + oa[u] + k);
        const int i = i0 + u;  // mask M[i][k'] for k' > i
        if (k + 0 > i) a.x = 0.f;
        if (k + 1 > i) a.y = 0.f;
        if (k + 2 > i) a.z = 0.f;
        if (k + 3 > i) a.w = 0.f;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          acc[u][v] = fmaf(a.x, b[v].x, acc[u][v]);
          acc[u][v] = fmaf(a.y, b[v].y, acc[u][v]);
          acc[u][v] = fmaf(a.z, b[v].z, acc[u][v]);
          acc[u][v] = fmaf(a.w, b[v].w, acc[u][v]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (i0 + u < m)
#pragma unroll
        for (int v = 0; v < 4; ++v) T[(i0 + u - r0) * kLdT + c0 + v] = acc[u][v];
  }
}

// M[i][j0+c] = -Σ_{c' >= c} T[i - r0][c'] M11[c'][c] for rows i >= r0, 4 x 4
// tiles (M11 = the diagonal block's inverse, lower, in place).
__device__ void inverse_finish(float* A, int ld, int j0, int m, const float* T) {
  const int r0 = j0 + FB;
  const int R = m - r0;
  const int TR = (R + 3) / 4;
  const int tiles = TR * (FB / 4);
  const float* Mb = A + j0 * ld + j0;
  for (int t = threadIdx.x; t < tiles; t += kThreads) {
    const int ti = t / (FB / 4), tc = t % (FB / 4);
    const int i0 = r0 + 4 * ti, c0 = 4 * tc;
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
    int ri[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) ri[u] = min(i0 + u, m - 1) - r0;
#pragma unroll 2
    for (int cp = c0; cp < FB; ++cp) {
      float a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = T[ri[u] * kLdT + cp];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = (cp >= c0 + v) ? Mb[cp * ld + c0 + v] : 0.f;
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (i0 + u < m)
#pragma unroll
        for (int v = 0; v < 4; ++v) A[(i0 + u) * ld + j0 + c0 + v] = -acc[u][v];
  }
}

__global__ void __launch_bounds__(kThreads, 1)
    gp_fit_f32(const float* __restrict__ C32, const double* __restrict__ Cd, const double* __restrict__ bvec,
               const double* __restrict__ yy_p, long long N, int m, const double* __restrict__ evals, double n_rows,
               int typ, const double* __restrict__ theta0, const double* __restrict__ lower,
               const int* __restrict__ mask, int steps, double lr, double beta1, double beta2, double eps,
               double* __restrict__ theta_out, double* __restrict__ hist, int* __restrict__ status,
               int restarts_mode) {
  extern __shared__ __align__(16) unsigned char sm[];
  // CTA r runs restart r (independent fits of the same problem from their own start)
  theta0 += 4 * blockIdx.x;
  theta_out += 4 * blockIdx.x;
  if (hist) hist += (size_t)steps * blockIdx.x;
  status += blockIdx.x;
  const Layout Ly = layout(m);
  double* S = reinterpret_cast<double*>(sm + Ly.S);
  double* dS = reinterpret_cast<double*>(sm + Ly.dS);
  double* tmp = reinterpret_cast<double*>(sm + Ly.tmp);
  double* Dm1 = reinterpret_cast<double*>(sm + Ly.Dm1);
  double* invD = reinterpret_cast<double*>(sm + Ly.invD);
  double* invS = reinterpret_cast<double*>(sm + Ly.invS);
  double* isd = reinterpret_cast<double*>(sm + Ly.isd);
  double* rb = reinterpret_cast<double*>(sm + Ly.rb);
  double* wv = reinterpret_cast<double*>(sm + Ly.w);
  double* cdg = reinterpret_cast<double*>(sm + Ly.cdg);
  double* red = reinterpret_cast<double*>(sm + Ly.red);
  double* th = reinterpret_cast<double*>(sm + Ly.th);
  double* adam = reinterpret_cast<double*>(sm + Ly.adam);
  double* outv = reinterpret_cast<double*>(sm + Ly.outv);
  float* A = reinterpret_cast<float*>(sm + Ly.A);
  float* T = reinterpret_cast<float*>(sm + Ly.T);
  float* uf = reinterpret_cast<float*>(sm + Ly.u);
  float* hf = reinterpret_cast<float*>(sm + Ly.z);  // h_l while building Ã, then z̃
  float* cf = reinterpret_cast<float*>(sm + Ly.c);
  float* dinvL = reinterpret_cast<float*>(sm + Ly.L);
  float* zf = hf;
  __shared__ int s_bad, s_chol;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ld = lda32(m);
  const int nblk = (m + FB - 1) / FB;
  const int nw = (m + 31) / 32;  // warps holding the per-eigenpair values
  const double yy = yy_p[0];
  const double Nd = (double)N;
  for (int l = tid; l < m; l += kThreads) cdg[l] = Cd[(size_t)l * m + l];
  // row padding [m, ld) is read (and multiplied by masked zeros) by the float4
  // loops; it must hold finite values
  for (int e = tid; e < m * (ld - m); e += kThreads) A[(e / (ld - m)) * ld + m + e % (ld - m)] = 0.f;
  if (tid == 0) {
    s_bad = 0;
    for (int q = 0; q < 4; ++q) {
      th[q] = theta0[q];
      const double v = theta0[q] - lower[q];
      adam[q] = v > 30.0 ? v : log(expm1(fmax(v, 1e-300)));  // inverse softplus
      adam[4 + q] = 0.0;
      adam[8 + q] = 0.0;
    }
    adam[12] = 1.0;  // beta1^t
    adam[13] = 1.0;  // beta2^t
  }
  __syncthreads();
  for (int step = 0; step < steps; ++step) {
    const double nu = th[0], kappa = th[1], sf = th[2], s2 = th[3];
    // ---- 1. spectral weights and their derivatives (log domain), FP64
    double mx = -DBL_MAX;
    for (int l = tid; l < m; l += kThreads) {
      const double lam = evals[l];
      double a, b, c;
      if (typ == 0) {
        const double ik2 = rcp_nr(kappa * kappa);
        const double uu = lam + 2.0 * nu * ik2;
        const double iu = rcp_nr(uu);
        const double lu = (double)logf((float)uu);  // FP32 accuracy, as the m x m algebra
        a = -nu * lu;
        b = -lu - nu * (2.0 * ik2) * iu;
        c = 4.0 * nu * nu * ik2 * rcp_nr(kappa) * iu;
      } else {
        a = -0.5 * lam * kappa * kappa;
        b = 0.0;
        c = -lam * kappa;
      }
      tmp[l] = a;
      tmp[m + l] = b;
      tmp[2 * m + l] = c;
      mx = fmax(mx, a);
    }
    mx = cta_max(mx, red, nw);
    {
      double v[1] = {0.0};
      for (int l = tid; l < m; l += kThreads) {
        S[l] = (double)expf((float)(tmp[l] - mx));  // unnormalised weight (<= 1), normalised below
        v[0] += S[l];
      }
      cta_sum<1>(v, red, nw);
      const double iz = rcp_nr(v[0]);
      double g[2] = {0.0, 0.0};
      for (int l = tid; l < m; l += kThreads) {
        const double wl = S[l] * iz;
        g[0] += wl * tmp[m + l];
        g[1] += wl * tmp[2 * m + l];
      }
      cta_sum<2>(g, red, nw);
      const double is2 = rcp_nr(s2), isf = rcp_nr(sf);
      for (int l = tid; l < m; l += kThreads) {
        const double Sl = sf * n_rows * S[l] * iz;
        S[l] = Sl;
        dS[l] = Sl * (tmp[m + l] - g[0]);
        dS[m + l] = Sl * (tmp[2 * m + l] - g[1]);
        dS[2 * m + l] = Sl * isf;
        const double Bll = Sl * cdg[l] * is2;  // Δ_l - 1
        const double Dl = 1.0 + Bll;
        if (!(Sl > 0.0) || !(Dl > 0.0)) s_bad = 1;  // invalid parameters: A is not positive definite
        Dm1[l] = Bll;
        invD[l] = rcp_nr(Dl);
        invS[l] = rcp_nr(Sl);
        const double r_isd = rsqrt_nr(Dl);
        isd[l] = r_isd;
        const double rl = Sl * rsqrt_nr(Sl);
        rb[l] = rl * bvec[l];
        uf[l] = (float)(rb[l] * r_isd);
        hf[l] = sqrtf((float)(Sl * is2) * (float)invD[l]);  // √S_l /(σ √Δ_l)
      }
    }
    __syncthreads();
    if (s_bad) break;
    // ---- 2. scaled capacitance matrix (lower triangle, unit diagonal), FP32
    for (int i = warp; i < m; i += kWarps) {
      const float hi = hf[i];
#pragma unroll 4
      for (int j = lane; j <= i; j += 32) A[i * ld + j] = (j == i) ? 1.f : __ldg(C32 + (size_t)i * m + j) * hi * hf[j];
    }
    __syncthreads();
    // ---- 3. blocked Cholesky Ã = L Lᵀ
    if (!chol32::chol32_cta<kThreads>(A, ld, m, dinvL, &s_chol)) {
      if (tid == 0) s_bad = 1;
      break;
    }
    // ---- 4. M = L⁻¹ in place: the diagonal blocks' inverses (one warp each),
    // moved from the upper triangle to the lower; log L_ll for |Ã|
    chol32::invert_diag_blocks(A, ld, m, nblk, dinvL);
    __syncthreads();
    double logL = 0.0;
    for (int e = tid; e < nblk * FB * FB; e += kThreads) {
      const int jb = e / (FB * FB), r = (e / FB) % FB, c = e % FB;
      const int j0 = jb * FB, i = j0 + r, j = j0 + c;
      if (i < m && j < m) {
        if (c < r) A[i * ld + j] = A[j * ld + i];
        if (c == r) {
          A[i * ld + i] = dinvL[i];
          logL -= (double)logf(dinvL[i]);
        }
      }
    }
    __syncthreads();
    for (int jb = nblk - 2; jb >= 0; --jb) {
      const int j0 = jb * FB, r0 = j0 + FB;
      // the block column's L (rows >= r0) into the upper triangle, transposed
      for (int e = tid; e < (m - r0) * FB; e += kThreads) {
        const int k = r0 + e / FB, c = e % FB;
        A[(j0 + c) * ld + k] = A[k * ld + j0 + c];
      }
      __syncthreads();
      inverse_product(A, ld, j0, m, T);
      __syncthreads();
      inverse_finish(A, ld, j0, m, T);
      __syncthreads();
    }
    // ---- 5. z̃ = M u (warp per row), then w̃ = Mᵀ z̃ and column norms (warp per column)
    for (int i = warp; i < m; i += kWarps) {
      float s = 0.f;
      for (int k = lane; k <= i; k += 32) s = fmaf(A[i * ld + k], uf[k], s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) zf[i] = s;
    }
    __syncthreads();
    for (int l = warp; l < m; l += kWarps) {
      float s = 0.f, q = 0.f;
      for (int k = l + lane; k < m; k += 32) {
        const float v = A[k * ld + l];
        s = fmaf(v, zf[k], s);
        q = fmaf(v, v, q);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        q += __shfl_xor_sync(0xffffffffu, q, o);
      }
      if (lane == 0) {
        uf[l] = s;  // w̃_l (u is no longer needed)
        cf[l] = q;
      }
    }
    __syncthreads();
    // ---- 6. likelihood and gradient (FP64)
    {
      double v[7] = {0, 0, 0, 0, 0, 0, 0};  // zz, ww, log|Ã|/2 + log|Δ|, tr A⁻¹, g_nu, g_kappa, g_sf
      for (int l = tid; l < m; l += kThreads) {
        const double wl = (double)uf[l] * isd[l];
        wv[l] = wl;
        const double cl = (double)cf[l];
        v[0] += rb[l] * wl;
        v[1] += wl * wl;
        v[3] += cl * invD[l];
        const double one_minus = (Dm1[l] - (cl - 1.0)) * invD[l];
        const double wn = wl * rcp_nr(s2);
        const double q = 0.5 * (wn * wn - one_minus) * invS[l];
        v[4] += q * dS[l];
        v[5] += q * dS[m + l];
        v[6] += q * dS[2 * m + l];
        v[2] += (double)logf((float)(1.0 + Dm1[l]));
      }
      v[2] += 2.0 * logL;
      cta_sum<7>(v, red, nw);
      if (tid == 0) {
        const double zz = v[0], ww = v[1], logd = v[2], tr = v[3];
        const double is2 = rcp_nr(s2);
        const double quad = (yy - zz * is2) * is2;
        outv[0] = -0.5 * quad - 0.5 * (Nd * log(s2) + logd) - 0.5 * Nd * log(2.0 * M_PI);
        outv[1] = v[4];
        outv[2] = v[5];
        outv[3] = v[6];
        const double a2 = (yy - zz * is2 - ww * is2) * is2 * is2;
        outv[4] = 0.5 * (a2 - (Nd - m + tr) * is2);
        if (hist) hist[step] = outv[0];
        adam[12] *= beta1;
        adam[13] *= beta2;
      }
    }
    __syncthreads();
    // ---- 7. Adam on u (value = softplus(u) + lower), minimising -LML; lane q of
    // warp 0 updates parameter q: the FP64 form's adam_step with the moments in
    // FP64 and sigmoid / softplus / square root in FP32
    if (warp == 0 && lane < 4) {
      bool finite = true;
      for (int q = 0; q < 5; ++q) finite = finite && isfinite(outv[q]);
      const int q = lane;
      if (finite && mask[q]) {
        const double b1t = 1.0 - adam[12], b2t = 1.0 - adam[13];
        double* uq = adam + q;
        double* m1 = adam + 4 + q;
        double* v1 = adam + 8 + q;
        const float uf32 = (float)*uq;
        const double sig = (double)(1.0f / (1.0f + expf(-uf32)));
        const double g = -outv[1 + q] * sig;
        *m1 = beta1 * *m1 + (1.0 - beta1) * g;
        *v1 = beta2 * *v1 + (1.0 - beta2) * g * g;
        *uq -= lr * (*m1 / b1t) / ((double)sqrtf((float)(*v1 / b2t)) + eps);
        const float un = (float)*uq;
        const float sp = un > 15.f ? un + log1pf(expf(-un)) : log1pf(expf(un));
        th[q] = (double)sp + lower[q];
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (!s_bad || restarts_mode)
      for (int q = 0; q < 4; ++q) theta_out[q] = th[q];
    *status = s_bad;
  }
}

__global__ void to_f32(const double* __restrict__ in, long long n, float* __restrict__ out) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e < n) out[e] = (float)in[e];
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

namespace rvgp {
int gp_fit_cluster_max_m();
int gp_fit_cluster_launch(const float* C32, const double* C, const double* b, const double* yy, long long N, int m,
                          const double* evals, double n_rows, int typ, const double* theta0, const double* lower_dev,
                          const int* mask_dev, int steps, double lr, double beta1, double beta2, double eps,
                          double* theta_out, double* hist, int* status, cudaStream_t st, int restarts,
                          int restarts_mode, double* scratch);
size_t gp_fit_cluster_scratch(int m, int restarts);
}  // namespace rvgp

extern "C" size_t rvgp_gp_lml_workspace(int m);
extern "C" size_t rvgp_gp_state_size(int m);
extern "C" int rvgp_gp_lml(const double* C, const double* b, const double* yy, long long N, int m,
                           const double* evals, double n_rows, int typ, const double* theta, double* out,
                           double* state, void* workspace, size_t ws_bytes, void* stream);

// Largest m whose working set fits one SM's shared memory.
static int one_cta_max_m() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  int m = 8;
  while (layout(m + 1).total + 512 <= (size_t)optin) ++m;  // + the kernel's static shared memory
  return m;
}

// Largest m of the mixed fit: one CTA up to one SM's shared memory, then one
// thread-block cluster with the matrix spread over its CTAs (gp_cluster.cu).
RVGP_API int rvgp_gp_fit_mixed_max_m(void) { return std::max(one_cta_max_m(), gp_fit_cluster_max_m()); }

RVGP_API size_t rvgp_gp_fit_mixed_workspace(int m) {
  return rvgp_gp_lml_workspace(m) + sizeof(float) * (size_t)m * m + 4 * sizeof(double) +
         gp_fit_cluster_scratch(m, 1) + 6 * 256 + 64;
}

namespace {
struct FitBufs {
  void* lml_ws;
  float* C32;
  double* dl;
  int* dm;
  int* dstat;
  double* scratch;  // the wide cluster fit's FP64 arrays (m > 512)
};
FitBufs carve_fit(void* workspace, size_t ws_bytes, int m) {
  Workspace ws(workspace, ws_bytes);
  FitBufs f;
  f.lml_ws = ws.take<char>(rvgp_gp_lml_workspace(m));
  f.C32 = ws.take<float>((size_t)m * m);
  f.dl = ws.take<double>(4);
  f.dm = ws.take<int>(4);
  f.dstat = ws.take<int>(1);
  f.scratch = gp_fit_cluster_scratch(m, 1) ? ws.take<double>(gp_fit_cluster_scratch(m, 1) / sizeof(double)) : nullptr;
  return f;
}
}  // namespace

// Mixed-form Adam fit (see the top of this file), enqueued without waiting:
// arguments as rvgp_gp_fit_adam.  The workspace holds the fit's status until
// rvgp_gp_fit_adam_mixed_finish.  Requires m <= rvgp_gp_fit_mixed_max_m().
RVGP_API int rvgp_gp_fit_adam_mixed_launch(const double* C, const double* b, const double* yy, long long N, int m,
                                           const double* evals, double n_rows, int typ, const double* theta0,
                                           const double* lower, const int* mask, int steps, double lr, double beta1,
                                           double beta2, double eps, double* theta_out, double* hist,
                                           void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(C && b && yy && evals && theta0 && lower && mask && theta_out,
                 "rvgp_gp_fit_adam_mixed: null pointer");
  RVGP_CHECK_ARG(typ == 0 || typ == 1, "rvgp_gp_fit_adam_mixed: typ must be 0 (matern) or 1 (se)");
  RVGP_CHECK_ARG(steps >= 0 && workspace && ws_bytes >= rvgp_gp_fit_mixed_workspace(m),
                 "rvgp_gp_fit_adam_mixed: bad steps or workspace");
  const int mmax = rvgp_gp_fit_mixed_max_m();
  RVGP_CHECK_ARG(m >= 1 && m <= mmax, "rvgp_gp_fit_adam_mixed: m=%d exceeds the shared-memory limit %d", m, mmax);
  cudaStream_t st = as_stream(stream);
  FitBufs f = carve_fit(workspace, ws_bytes, m);
  cudaMemcpyAsync(f.dl, lower, 4 * sizeof(double), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(f.dm, mask, 4 * sizeof(int), cudaMemcpyHostToDevice, st);
  rvgp::note_launch();
  to_f32<<<ceil_div((long long)m * m, 256), 256, 0, st>>>(C, (long long)m * m, f.C32);
  // RVGP_GP_FIT_CLUSTER=1 selects the cluster kernel wherever it applies (tests)
  const char* force = getenv("RVGP_GP_FIT_CLUSTER");
  const bool cluster = m > one_cta_max_m() || (force && force[0] == '1' && m > 32 && m <= gp_fit_cluster_max_m());
  if (cluster) {
    const int rc = gp_fit_cluster_launch(f.C32, C, b, yy, N, m, evals, n_rows, typ, theta0, f.dl, f.dm, steps, lr,
                                         beta1, beta2, eps, theta_out, hist, f.dstat, st, 1, 0, f.scratch);
    if (rc != RVGP_OK) return rc;
    RVGP_LAUNCH_CHECK("rvgp_gp_fit_adam_mixed");
    return RVGP_OK;
  }
  const size_t smem = layout(m).total;
  if (raise_dyn_smem((const void*)gp_fit_f32, (size_t)(smem)) != cudaSuccess) {
    set_error("rvgp_gp_fit_adam_mixed: cannot reserve %zu bytes of shared memory", smem);
    return RVGP_ELAUNCH;
  }
  rvgp::note_launch();
  gp_fit_f32<<<1, kThreads, smem, st>>>(f.C32, C, b, yy, N, m, evals, n_rows, typ, theta0, f.dl, f.dm, steps, lr,
                                        beta1, beta2, eps, theta_out, hist, f.dstat, 0);
  RVGP_LAUNCH_CHECK("rvgp_gp_fit_adam_mixed");
  return RVGP_OK;
}

// Waits for the fit enqueued by rvgp_gp_fit_adam_mixed_launch on the same
// stream and workspace.  *status (host): 0 = done, and out / state hold the
// FP64 likelihood, gradient and posterior state at theta_out; 1 = an FP32
// pivot was not positive, nothing was written to theta_out / out / state and
// the caller should run rvgp_gp_fit_adam instead.
RVGP_API int rvgp_gp_fit_adam_mixed_finish(const double* C, const double* b, const double* yy, long long N, int m,
                                           const double* evals, double n_rows, int typ, const double* theta_out,
                                           double* out, double* state, int* status, void* workspace,
                                           size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(C && b && yy && evals && theta_out && out && state && status,
                 "rvgp_gp_fit_adam_mixed_finish: null pointer");
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_gp_fit_mixed_workspace(m), "rvgp_gp_fit_adam_mixed_finish: workspace");
  cudaStream_t st = as_stream(stream);
  FitBufs f = carve_fit(workspace, ws_bytes, m);
  int h = 0;
  if (read_back(&h, f.dstat, sizeof(int), st) != cudaSuccess) return check_launch("rvgp_gp_fit_adam_mixed");
  *status = h;
  if (h != 0) return RVGP_OK;
  // FP64 likelihood, gradient and posterior state at the final parameters
  return rvgp_gp_lml(C, b, yy, N, m, evals, n_rows, typ, theta_out, out, state, f.lml_ws, rvgp_gp_lml_workspace(m),
                     stream);
}

// rvgp_gp_fit_adam_mixed_launch followed by rvgp_gp_fit_adam_mixed_finish.
// Synchronises the stream (to read the status).
RVGP_API int rvgp_gp_fit_adam_mixed(const double* C, const double* b, const double* yy, long long N, int m,
                                    const double* evals, double n_rows, int typ, const double* theta0,
                                    const double* lower, const int* mask, int steps, double lr, double beta1,
                                    double beta2, double eps, double* theta_out, double* hist, double* out,
                                    double* state, int* status, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(out && state && status, "rvgp_gp_fit_adam_mixed: null pointer");
  const int rc = rvgp_gp_fit_adam_mixed_launch(C, b, yy, N, m, evals, n_rows, typ, theta0, lower, mask, steps, lr,
                                               beta1, beta2, eps, theta_out, hist, workspace, ws_bytes, stream);
  if (rc != RVGP_OK) return rc;
  return rvgp_gp_fit_adam_mixed_finish(C, b, yy, N, m, evals, n_rows, typ, theta_out, out, state, status, workspace,
                                       ws_bytes, stream);
}

// ------------------------------------------------------------------ many starts at once
// R independent mixed-form Adam fits of one problem from R starting points
// (the multi-start hyperparameter search of a batch of fields), then the FP64
// likelihood of every fit at its final parameters and the best of them, all
// enqueued without any host synchronisation (a stream capture may hold it).
//   theta0 (device, R x 4) starts; lower (device, 4) and mask (device, 4 ints)
//   as rvgp_gp_fit_adam; theta_out (device, R x 4) final parameters; hist
//   (device, R x steps, optional) FP32 LML before each step; lml (device, R)
//   FP64 LML at theta_out (-inf for a fit stopped by a non-positive FP32 pivot
//   or invalid parameters, status (device, R) = 1 for those); best (device, 1
//   int) index of the largest LML (lowest index on ties); theta_best
//   (device, 4) = its parameters.
// m <= rvgp_gp_fit_mixed_max_m(); one CTA per fit up to the one-SM limit,
// one thread-block cluster per fit above it.
RVGP_API size_t rvgp_gp_fit_restarts_workspace(int m, int R) {
  return rvgp_gp_lml_workspace(m) + sizeof(float) * (size_t)m * m + (size_t)rvgp_gp_state_size(m) * sizeof(double) +
         gp_fit_cluster_scratch(m, R) + 8 * sizeof(double) + 5 * 256;
}

namespace rvgp {
namespace {
__global__ void restarts_select(const double* __restrict__ outs, int R, const int* __restrict__ status,
                                const double* __restrict__ theta_out, double* __restrict__ lml, int* __restrict__ best,
                                double* __restrict__ theta_best) {
  if (threadIdx.x != 0) return;
  int bi = -1;
  double bv = -INFINITY;
  for (int r = 0; r < R; ++r) {
    const double v = (status[r] == 0 && isfinite(outs[5 * r])) ? outs[5 * r] : -INFINITY;
    lml[r] = v;
    if (bi < 0 || v > bv) {
      bi = r;
      bv = v;
    }
  }
  *best = bi;
  for (int q = 0; q < 4; ++q) theta_best[q] = theta_out[4 * bi + q];
}
}  // namespace
}  // namespace rvgp

RVGP_API int rvgp_gp_fit_restarts(const double* C, const double* b, const double* yy, long long N, int m,
                                  const double* evals, double n_rows, int typ, const double* theta0,
                                  const double* lower, const int* mask, int R, int steps, double lr, double beta1,
                                  double beta2, double eps, double* theta_out, double* hist, double* lml,
                                  int* status, double* outs, int* best, double* theta_best, void* workspace,
                                  size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(C && b && yy && evals && theta0 && lower && mask && theta_out && lml && status && outs && best &&
                     theta_best,
                 "rvgp_gp_fit_restarts: null pointer");
  RVGP_CHECK_ARG(typ == 0 || typ == 1, "rvgp_gp_fit_restarts: typ must be 0 (matern) or 1 (se)");
  RVGP_CHECK_ARG(R >= 1 && R <= 1024 && steps >= 0, "rvgp_gp_fit_restarts: bad R=%d or steps", R);
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_gp_fit_restarts_workspace(m, R), "rvgp_gp_fit_restarts: workspace");
  const int mmax = rvgp_gp_fit_mixed_max_m();
  RVGP_CHECK_ARG(m >= 1 && m <= mmax, "rvgp_gp_fit_restarts: m=%d exceeds the mixed fit's limit %d", m, mmax);
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  void* lml_ws = ws.take<char>(rvgp_gp_lml_workspace(m));
  float* C32 = ws.take<float>((size_t)m * m);
  double* state = ws.take<double>(rvgp_gp_state_size(m));
  const size_t scr = gp_fit_cluster_scratch(m, R);
  double* scratch = scr ? ws.take<double>(scr / sizeof(double)) : nullptr;
  rvgp::note_launch();
  to_f32<<<ceil_div((long long)m * m, 256), 256, 0, st>>>(C, (long long)m * m, C32);
  const char* force = getenv("RVGP_GP_FIT_CLUSTER");  // as for the single fit (tests)
  if (m > one_cta_max_m() || (force && force[0] == '1' && m > 32 && m <= gp_fit_cluster_max_m())) {
    TRY_RC(gp_fit_cluster_launch(C32, C, b, yy, N, m, evals, n_rows, typ, theta0, lower, mask, steps, lr, beta1,
                                 beta2, eps, theta_out, hist, status, st, R, 1, scratch));
  } else {
    const size_t smem = layout(m).total;
    if (raise_dyn_smem((const void*)gp_fit_f32, (size_t)(smem)) != cudaSuccess) {
      set_error("rvgp_gp_fit_restarts: cannot reserve %zu bytes of shared memory", smem);
      return RVGP_ELAUNCH;
    }
    rvgp::note_launch();
    gp_fit_f32<<<R, kThreads, smem, st>>>(C32, C, b, yy, N, m, evals, n_rows, typ, theta0, lower, mask, steps, lr,
                                          beta1, beta2, eps, theta_out, hist, status, 1);
  }
  RVGP_LAUNCH_CHECK("rvgp_gp_fit_restarts");
  // FP64 likelihood of every fit at its final parameters (the fits stopped
  // early keep finite parameters; their LML is discarded by the selection)
  for (int r = 0; r < R; ++r)
    TRY_RC(rvgp_gp_lml(C, b, yy, N, m, evals, n_rows, typ, theta_out + 4 * r, outs + 5 * r, state, lml_ws,
                       rvgp_gp_lml_workspace(m), stream));
  rvgp::note_launch();
  restarts_select<<<1, 32, 0, st>>>(outs, R, status, theta_out, lml, best, theta_best);
  RVGP_LAUNCH_CHECK("rvgp_gp_fit_restarts");
  return RVGP_OK;
}
