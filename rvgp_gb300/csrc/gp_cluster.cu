// Mixed-precision hyperparameter fit for m beyond one SM's shared memory:
// every Adam step of the GP likelihood (GPflow GPR + RVGP ManifoldKernel as
// used by RVGP/main.py:55-95 and RVGP/kernels.py:41-53) inside ONE launch of
// ONE thread-block cluster.
//
// The step is the same as the one-CTA fit (gp_mixed.cu): spectral weights in
// FP64, the Jacobi-scaled capacitance matrix Ã = Δ^-½ (I + R C R/σ²) Δ^-½ in
// FP32, Ã = L Lᵀ, M = L⁻¹, z̃ = M u, w̃ = Mᵀ z̃, c_l = Σ_k M_kl², then the
// likelihood, gradient and Adam update in FP64.  What changes is where Ã
// lives: the matrix is padded to mp = 32·nb (identity in the padding) and CTA
// r of the cluster (nb CTAs, nb = ⌈m/32⌉ ≤ 16) holds block row r (rows
// 32r..32r+31, all columns) in its shared memory.  CTAs read each other's
// block rows through distributed shared memory (DSMEM):
//   Cholesky, block column k = 0..nb-1:
//     CTA k factors its diagonal block (one warp)            | cluster barrier
//     CTAs r > k copy L_kk and solve their panel block       | cluster barrier
//     CTAs r > k copy the panel rows k+1..r and update their block row
//   inverse M = L⁻¹, block column j = nb-2..0 (diagonal blocks inverted first):
//     CTAs r > j copy column block j of L (rows j+1..r) and M_jj
//                                                            | cluster barrier
//     M_rj = -(Σ_{k=j+1}^{r} M_rk L_kj) M_jj (own block row only)
//   column sums of M and Mᵀz̃ over the block rows: each CTA sums its rows,
//   then every CTA adds the nb partial vectors in rank order.
// Every CTA computes the O(m) FP64 work itself from identical inputs, so the
// parameters, the decisions and the number of cluster barriers are identical
// in all CTAs.  A non-positive FP32 pivot or invalid parameters end the launch
// with status 1 (the host then runs the FP64 form); the final likelihood and
// posterior state are computed in FP64 by the host-side finish call, as for
// the one-CTA fit.
#include "common.cuh"
#include "linalg.cuh"
#include <cooperative_groups.h>
#include <math.h>
#include <float.h>

namespace cg = cooperative_groups;

namespace rvgp {
namespace {

constexpr int kNT = 512;
constexpr int kW = kNT / 32;
constexpr int FB = 32;
constexpr int kLdP = FB + 4;    // panel / block copies: 16-byte rows, ld/4 odd
constexpr int kMaxCluster = 16;
constexpr int kSlices = 4;      // K-split of the inverse product (kSlices x 64 threads)

__host__ __device__ inline int ld_rows(int mp) { return mp + 4; }  // mp % 32 == 0: ld/4 odd

struct CLayout {
  size_t Ar, P, Lk, dk, dinv, T, Tp, uf, hf, zt, part, pd, tmp, S, cdg, Dm1, isd, rb, red, th, adam, outv, flag, total;
};

__host__ __device__ inline CLayout clayout(int m, int nb) {
  CLayout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += (bytes + 15) & ~size_t(15);
    return at;
  };
  const int mp = nb * FB;
  const size_t d = 8 * (size_t)m;
  L.Ar = take(4 * (size_t)FB * ld_rows(mp));
  L.P = take(4 * (size_t)(mp - FB) * kLdP);   // rows of one column block, global row g at g - 32
  L.Lk = take(4 * (size_t)FB * kLdP);
  L.dk = take(4 * FB);
  L.dinv = take(4 * FB);
  L.T = take(4 * (size_t)FB * kLdP);
  L.Tp = take(4 * (size_t)kSlices * 64 * 16);  // K-split partial tiles of the inverse product
  L.uf = take(4 * (size_t)mp);
  L.hf = take(4 * (size_t)mp);
  L.zt = take(4 * FB);
  L.part = take(4 * 2 * (size_t)mp);          // [Σ_r M_rl z_r | Σ_r M_rl²] over the CTA's rows
  L.pd = take(8 * 2);                          // [log det of the own diagonal block, own pivot failure]
  L.tmp = take(3 * d);
  L.S = take(d);
  L.cdg = take(d);
  L.Dm1 = take(d);
  L.isd = take(d);
  L.rb = take(d);
  L.red = take(8 * 8 * (kW + 1));
  L.th = take(8 * 4);
  L.adam = take(8 * 16);
  L.outv = take(8 * 8);
  L.flag = take(16);
  L.total = o;
  return L;
}

// FP64 CTA reductions over the warps that hold the m per-eigenpair values
// (xor tree within a warp, then over the warps' partials; fixed order).
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
      for (int q = 0; q < NV; ++q) red[q * kW + warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double s = lane < nw ? red[q * kW + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) red[8 * kW + q] = s;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = red[8 * kW + q];
  __syncthreads();
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
    if (lane == 0) red[8 * kW + 7] = s;
  }
  __syncthreads();
  const double r = red[8 * kW + 7];
  __syncthreads();
  return r;
}

__device__ __forceinline__ float rsqrt_f(float d) {
  const float r = rsqrtf(d);
  return r * fmaf(-0.5f * d * r, r, 1.5f);
}

// One warp: Cholesky of the 32 x 32 block at columns c0.. of the CTA's rows
// (row r = A[r * ld + ...]).  Lane i keeps row i in registers; the pivot
// column reaches the lanes through a shared buffer.  Writes L into the block's
// lower triangle, 1/L_ii into dinv[i]; returns false on a non-positive pivot
// (the pivot is then clamped so the factorisation runs to its end).
__device__ bool diag_factor(float* A, int ld, int c0, float* dinv, float* lcol) {
  const int lane = threadIdx.x & 31;
  float a[FB];
#pragma unroll
  for (int c = 0; c < FB; ++c) a[c] = (c <= lane) ? A[lane * ld + c0 + c] : 0.f;
  bool ok = true;
#pragma unroll 1
  for (int j4 = 0; j4 < FB; j4 += 4) {
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int j = j4 + jj;
      const float d = __shfl_sync(0xffffffffu, a[jj], j);
      ok = ok && (d > 0.f);
      const float rs = rsqrt_f(fmaxf(d, FLT_MIN));
      const float l = (lane == j) ? d * rs : a[jj] * rs;
      if (lane >= j) A[lane * ld + c0 + j] = l;
      if (lane == j) dinv[j] = rs;
      __syncwarp();
      lcol[lane] = (lane > j) ? l : 0.f;
      __syncwarp();
      const float4* l4 = reinterpret_cast<const float4*>(lcol + j4);
#pragma unroll
      for (int q = (jj + 1) / 4; q < FB / 4; ++q) {
        const float4 v = q + j4 / 4 < FB / 4 ? l4[q] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (4 * q + 0 > jj) a[4 * q + 0] = fmaf(-l, v.x, a[4 * q + 0]);
        if (4 * q + 1 > jj) a[4 * q + 1] = fmaf(-l, v.y, a[4 * q + 1]);
        if (4 * q + 2 > jj) a[4 * q + 2] = fmaf(-l, v.z, a[4 * q + 2]);
        if (4 * q + 3 > jj) a[4 * q + 3] = fmaf(-l, v.w, a[4 * q + 3]);
      }
      __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < FB - 4; ++k) a[k] = a[k + 4];
#pragma unroll
    for (int k = FB - 4; k < FB; ++k) a[k] = 0.f;
  }
  __syncwarp();
  return __all_sync(0xffffffffu, ok);
}

// Rows of the CTA's block row, columns c0..c0+31 <- A L_kk⁻ᵀ (forward
// substitution per row; L_kk in Lk (ld kLdP), 1/diag in dk).  Warps 0..7 take
// four rows each.
__device__ void panel_solve_rows(float* A, int ld, int c0, const float* Lk, const float* dk) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp >= FB / 4) return;
  float lrow[FB];
#pragma unroll
  for (int c = 0; c < FB; ++c) lrow[c] = c < lane ? Lk[lane * kLdP + c] : 0.f;
  const float dl = dk[lane];
  const int r = 4 * warp;
  float x[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) x[q] = A[(r + q) * ld + c0 + lane];
#pragma unroll
  for (int c = 0; c < FB; ++c) {
    const float dc = __shfl_sync(0xffffffffu, dl, c);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float xc = __shfl_sync(0xffffffffu, x[q], c) * dc;
      x[q] = (lane == c) ? xc : fmaf(-xc, lrow[c], x[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) A[(r + q) * ld + c0 + lane] = x[q];
}

// A[r][32j + c] -= Σ_t A[r][c0 + t] P[(32j + c)][t] for the CTA's 32 rows and
// column blocks j in [j_lo, j_hi] (j_lo >= 1; P row g - 32 holds global row g):
// 4 x 4 register tiles, float4 operands.
__device__ void block_row_update(float* A, int ld, int c0, const float* P, int j_lo, int j_hi) {
  const int tiles = (j_hi - j_lo + 1) * 64;
  for (int t = threadIdx.x; t < tiles; t += kNT) {
    const int jb = j_lo + t / 64, tt = t % 64;
    const int r0 = 4 * (tt / 8), col0 = jb * FB + 4 * (tt % 8);
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
#pragma unroll 2
    for (int c = 0; c < FB; c += 4) {
      float4 b[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = *reinterpret_cast<const float4*>(P + (size_t)(col0 + v - FB) * kLdP + c);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float4 a = *reinterpret_cast<const float4*>(A + (r0 + u) * ld + c0 + c);
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
#pragma unroll
      for (int v = 0; v < 4; ++v) A[(r0 + u) * ld + col0 + v] -= acc[u][v];
  }
}

// Copy rows [g0, g1) (global row numbers, g0 >= 32), columns c0..c0+31 of the
// cluster's block rows into P[g - 32][0..31] (float4 reads through DSMEM; own
// rows locally).
__device__ void gather_panel(cg::cluster_group& cl, const float* Ar, int ld, int c0, int g0, int g1, float* P) {
  const int n4 = (g1 - g0) * (FB / 4);
  constexpr int U = 4;  // loads in flight per thread
  for (int e0 = threadIdx.x; e0 < n4; e0 += U * kNT) {
    float4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * kNT;
      if (e < n4) {
        const int g = g0 + e / (FB / 4), c = 4 * (e % (FB / 4));
        const float* src = cl.map_shared_rank(const_cast<float*>(Ar), (unsigned)(g / FB));
        v[u] = *reinterpret_cast<const float4*>(src + (g % FB) * ld + c0 + c);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * kNT;
      if (e < n4) {
        const int g = g0 + e / (FB / 4), c = 4 * (e % (FB / 4));
        *reinterpret_cast<float4*>(P + (size_t)(g - FB) * kLdP + c) = v[u];
      }
    }
  }
}

// One warp per diagonal block row of the CTA (warp 0): inverse M_rr of the
// factor's own diagonal block (lower, 1/L_ii on the diagonal), written over
// the block's lower triangle with zeros above.
__device__ void invert_own_diag(float* A, int ld, int c0, const float* dinv) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp != 0) return;
  float x[FB];
#pragma unroll
  for (int k = 0; k < FB; ++k) x[k] = (k == lane) ? 1.f : 0.f;
  const float dl = dinv[lane];
  for (int c = 0; c < FB; ++c) {
    const float lic = (lane > c) ? A[lane * ld + c0 + c] : 0.f;
    const float dc = __shfl_sync(0xffffffffu, dl, c);
#pragma unroll
    for (int k = 0; k < FB; ++k) {
      const float xck = __shfl_sync(0xffffffffu, x[k], c) * dc;
      x[k] = (lane == c) ? xck : fmaf(-lic, xck, x[k]);
    }
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < FB; ++k) A[lane * ld + c0 + k] = (k <= lane) ? x[k] : 0.f;
}

// T = Σ_{col = k0}^{k1-1} A[r][col] P[col - 32][c] (32 x 32, K split over
// kSlices groups of 64 threads; k0 >= 32), then
// A[r][c0 + c] = -Σ_{c' >= c} T[r][c'] Mj[c'][c].
__device__ void inverse_block(float* A, int ld, int c0, int k0, int k1, const float* P, const float* Mj, float* T,
                              float* Tp) {
  const int tile = threadIdx.x % 64, slice = threadIdx.x / 64;
  const int r0 = 4 * (tile / 8), cc0 = 4 * (tile % 8);
  const int K = k1 - k0;
  const int per = ((K + kSlices * 4 - 1) / (kSlices * 4)) * 4;  // multiple of 4
  const int ks = slice < kSlices ? k0 + slice * per : k1, ke = min(k1, ks + per);
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
  for (int k = ks; k < ke; k += 4) {
    float4 a[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = *reinterpret_cast<const float4*>(A + (r0 + u) * ld + k);
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const float4 b = *reinterpret_cast<const float4*>(P + (size_t)(k + kk - FB) * kLdP + cc0);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float av = kk == 0 ? a[u].x : kk == 1 ? a[u].y : kk == 2 ? a[u].z : a[u].w;
        acc[u][0] = fmaf(av, b.x, acc[u][0]);
        acc[u][1] = fmaf(av, b.y, acc[u][1]);
        acc[u][2] = fmaf(av, b.z, acc[u][2]);
        acc[u][3] = fmaf(av, b.w, acc[u][3]);
      }
    }
  }
  if (slice < kSlices)
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) Tp[(size_t)threadIdx.x * 16 + u * 4 + v] = acc[u][v];
  __syncthreads();
  for (int e = threadIdx.x; e < FB * FB; e += kNT) {
    const int r = e / FB, c = e % FB;
    const int t = (r / 4) * 8 + c / 4, q = (r % 4) * 4 + c % 4;
    float s = 0.f;
#pragma unroll
    for (int sl = 0; sl < kSlices; ++sl) s += Tp[(size_t)(sl * 64 + t) * 16 + q];
    T[r * kLdP + c] = s;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < FB * FB; e += kNT) {
    const int r = e / FB, c = e % FB;
    float s = 0.f;
    for (int cp = c; cp < FB; ++cp) s = fmaf(T[r * kLdP + cp], Mj[cp * kLdP + c], s);
    A[r * ld + c0 + c] = -s;
  }
}

// The per-eigenpair FP64 arrays of a fit step (shared or global memory).
struct FitVecs {
  double *tmp, *S, *cdg, *Dm1, *isd, *rb;  // tmp: 3m (log s_l, ∂/∂ν, ∂/∂κ); the others m
};

// Step phase 1: spectral weights S(θ) in the log domain (FP64; log / exp of
// each term in FP32, the accuracy of the FP32 algebra), Δ_l - 1, Δ_l^-½,
// r_l b_l, and the FP32 vectors u = Δ^-½ R b and h = √S/(σ √Δ) (zero in the
// padding [m, mp)).  flag[0] = 1 for parameters that make S or Δ
// non-positive.  Ends with a CTA barrier.  Every CTA of a cluster computes
// the same values from the same inputs.
__device__ void weights_phase(const FitVecs& V, const double* __restrict__ evals, const double* __restrict__ bvec,
                              int m, int mp, double n_rows, int typ, double nu, double kappa, double sf, double s2,
                              double* red, int nw, float* uf, float* hf, int* flag, double& g0, double& g1) {
  const int tid = threadIdx.x;
  double* tmp = V.tmp;
  double* S = V.S;
  const double* cdg = V.cdg;
  double* Dm1 = V.Dm1;
  double* isd = V.isd;
  double* rb = V.rb;
  double mx = -DBL_MAX;
  for (int l = tid; l < m; l += kNT) {
    const double lam = evals[l];
    double a, b, c;
    if (typ == 0) {
      const double ik2 = rcp_nr(kappa * kappa);
      const double uu = lam + 2.0 * nu * ik2;
      const double iu = rcp_nr(uu);
      const double lu = (double)logf((float)uu);
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
    for (int l = tid; l < m; l += kNT) {
      S[l] = (double)expf((float)(tmp[l] - mx));
      v[0] += S[l];
    }
    cta_sum<1>(v, red, nw);
    const double iz = rcp_nr(v[0]);
    double g[2] = {0.0, 0.0};
    for (int l = tid; l < m; l += kNT) {
      const double wl = S[l] * iz;
      g[0] += wl * tmp[m + l];
      g[1] += wl * tmp[2 * m + l];
    }
    cta_sum<2>(g, red, nw);
    g0 = g[0];
    g1 = g[1];
    const double is2 = rcp_nr(s2);
    for (int l = m + tid; l < mp; l += kNT) {  // padding of u and h (identity rows / columns)
      uf[l] = 0.f;
      hf[l] = 0.f;
    }
    for (int l = tid; l < m; l += kNT) {
      const double Sl = sf * n_rows * S[l] * iz;
      S[l] = Sl;
      const double Bll = Sl * cdg[l] * is2;  // Δ_l - 1
      const double Dl = 1.0 + Bll;
      if (!(Sl > 0.0) || !(Dl > 0.0)) flag[0] = 1;
      Dm1[l] = Bll;
      const double r_isd = rsqrt_nr(Dl);
      isd[l] = r_isd;
      const double rl = Sl * rsqrt_nr(Sl);
      rb[l] = rl * bvec[l];
      uf[l] = (float)(rb[l] * r_isd);
      hf[l] = sqrtf((float)(Sl * is2) * (float)(r_isd * r_isd));
    }
  }
  __syncthreads();
}

// Step phase 6: log marginal likelihood and its gradient (FP64) from w̃ (in
// uf), c_l = (Ã⁻¹)_ll (in hf) and the Cholesky log-determinant; thread 0
// writes outv, the history entry (when hist_at is given) and advances the
// Adam bias corrections; a failed pivot anywhere (fail) sets flag[0].  Ends
// with a CTA barrier.
__device__ void likelihood_phase(const FitVecs& V, int m, double yy, double Nd, double s2, double sf, double g0,
                                 double g1, double logd_chol, int fail, const float* uf, const float* hf, double* red,
                                 int nw, double* outv, double* adam, double beta1, double beta2, double* hist_at,
                                 int* flag) {
  const int tid = threadIdx.x;
  const double* tmp = V.tmp;
  const double* Dm1 = V.Dm1;
  const double* isd = V.isd;
  const double* rb = V.rb;
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int l = tid; l < m; l += kNT) {
    const double wl = (double)uf[l] * isd[l];
    const double cl_ = (double)hf[l];
    v[0] += rb[l] * wl;
    v[1] += wl * wl;
    const double iD = isd[l] * isd[l];
    v[3] += cl_ * iD;
    const double one_minus = (Dm1[l] - (cl_ - 1.0)) * iD;
    const double wn = wl * rcp_nr(s2);
    const double q = 0.5 * (wn * wn - one_minus);  // times ∂log S_l/∂θ
    v[4] += q * (tmp[m + l] - g0);
    v[5] += q * (tmp[2 * m + l] - g1);
    v[6] += q;
    v[2] += (double)logf((float)(1.0 + Dm1[l]));
  }
  cta_sum<7>(v, red, nw);
  if (tid == 0) {
    const double zz = v[0], ww = v[1], logd = v[2] + 2.0 * logd_chol, tr = v[3];
    const double is2 = rcp_nr(s2);
    const double quad = (yy - zz * is2) * is2;
    outv[0] = -0.5 * quad - 0.5 * (Nd * log(s2) + logd) - 0.5 * Nd * log(2.0 * M_PI);
    outv[1] = v[4];
    outv[2] = v[5];
    outv[3] = v[6] * rcp_nr(sf);
    const double a2 = (yy - zz * is2 - ww * is2) * is2 * is2;
    outv[4] = 0.5 * (a2 - (Nd - m + tr) * is2);
    if (hist_at) *hist_at = outv[0];
    adam[12] *= beta1;
    adam[13] *= beta2;
    if (fail) flag[0] = 1;
  }
  __syncthreads();
}

// Step phase 7: Adam on the unconstrained parameters (value = softplus(u) +
// lower), lane q of warp 0 for parameter q.  Ends with a CTA barrier.
__device__ void adam_phase(const double* outv, double* adam, double* th, const double* __restrict__ lower,
                           const int* __restrict__ mask, double lr, double beta1, double beta2, double eps) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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

__global__ void __launch_bounds__(kNT, 1)
    gp_fit_cluster(const float* __restrict__ C32, const double* __restrict__ Cd, const double* __restrict__ bvec,
                   const double* __restrict__ yy_p, long long N, int m, const double* __restrict__ evals,
                   double n_rows, int typ, const double* __restrict__ theta0, const double* __restrict__ lower,
                   const int* __restrict__ mask, int steps, double lr, double beta1, double beta2, double eps,
                   double* __restrict__ theta_out, double* __restrict__ hist, int* __restrict__ status,
                   int restarts_mode) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int nb = (int)cl.num_blocks();
  // cluster c of the grid runs restart c (independent fits from their own start)
  const int rs = blockIdx.x / nb;
  theta0 += 4 * rs;
  theta_out += 4 * rs;
  if (hist) hist += (size_t)steps * rs;
  status += rs;
  const int mp = nb * FB, ld = ld_rows(mp), i0 = rank * FB;
  extern __shared__ __align__(16) unsigned char sm[];
  const CLayout Ly = clayout(m, nb);
  float* Ar = reinterpret_cast<float*>(sm + Ly.Ar);
  float* P = reinterpret_cast<float*>(sm + Ly.P);
  float* Lk = reinterpret_cast<float*>(sm + Ly.Lk);
  float* dk = reinterpret_cast<float*>(sm + Ly.dk);
  float* dinv = reinterpret_cast<float*>(sm + Ly.dinv);
  float* T = reinterpret_cast<float*>(sm + Ly.T);
  float* Tp = reinterpret_cast<float*>(sm + Ly.Tp);
  float* uf = reinterpret_cast<float*>(sm + Ly.uf);
  float* hf = reinterpret_cast<float*>(sm + Ly.hf);
  float* zt = reinterpret_cast<float*>(sm + Ly.zt);
  float* part = reinterpret_cast<float*>(sm + Ly.part);
  double* pd = reinterpret_cast<double*>(sm + Ly.pd);
  double* tmp = reinterpret_cast<double*>(sm + Ly.tmp);
  double* S = reinterpret_cast<double*>(sm + Ly.S);
  double* cdg = reinterpret_cast<double*>(sm + Ly.cdg);
  double* Dm1 = reinterpret_cast<double*>(sm + Ly.Dm1);
  double* isd = reinterpret_cast<double*>(sm + Ly.isd);
  double* rb = reinterpret_cast<double*>(sm + Ly.rb);
  double* red = reinterpret_cast<double*>(sm + Ly.red);
  double* th = reinterpret_cast<double*>(sm + Ly.th);
  double* adam = reinterpret_cast<double*>(sm + Ly.adam);
  double* outv = reinterpret_cast<double*>(sm + Ly.outv);
  int* flag = reinterpret_cast<int*>(sm + Ly.flag);  // [0] invalid parameters / failed pivot, [1] own pivot failure
  __shared__ __align__(16) float lcol[2 * FB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = min(kW, (m + 31) / 32);
  const double yy = yy_p[0];
  const double Nd = (double)N;
  for (int l = tid; l < m; l += kNT) cdg[l] = Cd[(size_t)l * m + l];
  for (int l = m + tid; l < mp; l += kNT) {
    uf[l] = 0.f;
    hf[l] = 0.f;
  }
  for (int e = tid; e < FB * (ld - mp); e += kNT) Ar[(e / (ld - mp)) * ld + mp + e % (ld - mp)] = 0.f;
  for (int e = tid; e < 2 * FB; e += kNT) lcol[e] = 0.f;
  if (tid == 0) {
    flag[0] = 0;
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
  int done = 0;
  for (int step = 0; step < steps && !done; ++step) {
    const double nu = th[0], kappa = th[1], sf = th[2], s2 = th[3];
    double g0 = 0.0, g1 = 0.0;
    // ---- 1. spectral weights (FP64, log domain; every CTA computes all m)
    const FitVecs V{tmp, S, cdg, Dm1, isd, rb};
    int bad = 0;
    weights_phase(V, evals, bvec, m, mp, n_rows, typ, nu, kappa, sf, s2, red, nw, uf, hf, flag, g0, g1);
    __syncthreads();
    bad = flag[0];  // identical in every CTA (same FP64 inputs and code)
    if (bad) break;
    // ---- 2. own block row of the padded scaled capacitance matrix
    for (int r = warp; r < FB; r += kW) {
      const int i = i0 + r;
      const float hi = hf[i];
      for (int j = lane; j < mp; j += 32) {
        float v = 0.f;
        if (j == i)
          v = 1.f;
        else if (j < i && i < m)
          v = __ldg(C32 + (size_t)i * m + j) * hi * hf[j];
        Ar[r * ld + j] = v;
      }
    }
    if (tid == 0) flag[1] = 0;
    __syncthreads();
    // ---- 3. blocked Cholesky across the cluster
    for (int k = 0; k < nb; ++k) {
      if (rank == k && warp == 0) {
        const bool ok = diag_factor(Ar, ld, k * FB, dinv, lcol);
        if (!ok && lane == 0) flag[1] = 1;
      }
      cl.sync();
      if (rank > k) {
        const float* src = cl.map_shared_rank(Ar, (unsigned)k);
        const float* srcd = cl.map_shared_rank(dinv, (unsigned)k);
        for (int e = tid; e < FB * FB; e += kNT) Lk[(e / FB) * kLdP + e % FB] = src[(e / FB) * ld + k * FB + e % FB];
        if (tid < FB) dk[tid] = srcd[tid];
        __syncthreads();
        panel_solve_rows(Ar, ld, k * FB, Lk, dk);
      }
      cl.sync();
      if (rank > k) {
        gather_panel(cl, Ar, ld, k * FB, (k + 1) * FB, (rank + 1) * FB, P);
        __syncthreads();
        block_row_update(Ar, ld, k * FB, P, k + 1, rank);
      }
      __syncthreads();
    }
    // log-determinant of the own diagonal block, then its inverse in place
    double logL = 0.0;
    if (warp == 0) {
      double lg = (double)logf(dinv[lane]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lg += __shfl_xor_sync(0xffffffffu, lg, o);
      logL = -lg;
    }
    invert_own_diag(Ar, ld, i0, dinv);
    __syncthreads();
    cl.sync();
    // ---- 4. M = L⁻¹: block columns right to left
    for (int j = nb - 2; j >= 0; --j) {
      if (rank > j) {
        gather_panel(cl, Ar, ld, j * FB, (j + 1) * FB, (rank + 1) * FB, P);
        const float* src = cl.map_shared_rank(Ar, (unsigned)j);
        for (int e = tid; e < FB * FB; e += kNT) Lk[(e / FB) * kLdP + e % FB] = src[(e / FB) * ld + j * FB + e % FB];
      }
      cl.sync();  // every copy of column block j is done before it is overwritten
      if (rank > j) {
        __syncthreads();
        inverse_block(Ar, ld, j * FB, (j + 1) * FB, (rank + 1) * FB, P, Lk, T, Tp);
      }
      __syncthreads();
    }
    // ---- 5. z̃ = M u (own rows), partial column sums of M z̃ and M∘M
    for (int r = warp; r < FB; r += kW) {
      float s = 0.f;
      for (int k = lane; k <= i0 + r; k += 32) s = fmaf(Ar[r * ld + k], uf[k], s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) zt[r] = s;
    }
    __syncthreads();
    for (int l = tid; l < mp; l += kNT) {
      float s = 0.f, q = 0.f;
      if (l <= i0 + FB - 1)
        for (int r = 0; r < FB; ++r) {
          const float v = Ar[r * ld + l];
          s = fmaf(v, zt[r], s);
          q = fmaf(v, v, q);
        }
      part[l] = s;
      part[mp + l] = q;
    }
    if (tid == 0) {
      pd[0] = logL;
      pd[1] = (double)flag[1];
    }
    __syncthreads();
    cl.sync();
    // every CTA adds the partials in rank order: w̃ (into uf), c (into hf)
    for (int l = tid; l < mp; l += kNT) {
      float ps[kMaxCluster], pq[kMaxCluster];
#pragma unroll
      for (int c = 0; c < kMaxCluster; ++c) {  // all loads first, then the sums in rank order
        ps[c] = pq[c] = 0.f;
        if (c >= l / FB && c < nb) {
          const float* pc = cl.map_shared_rank(part, (unsigned)c);
          ps[c] = pc[l];
          pq[c] = pc[mp + l];
        }
      }
      float s = 0.f, q = 0.f;
#pragma unroll
      for (int c = 0; c < kMaxCluster; ++c) {
        s += ps[c];
        q += pq[c];
      }
      uf[l] = s;
      hf[l] = q;
    }
    double logd_chol = 0.0;
    int fail = 0;
    for (int c = 0; c < nb; ++c) {
      const double* pc = cl.map_shared_rank(pd, (unsigned)c);
      logd_chol += pc[0];
      fail |= pc[1] != 0.0;
    }
    __syncthreads();
    // ---- 6. likelihood and gradient (FP64)
    likelihood_phase(V, m, yy, Nd, s2, sf, g0, g1, logd_chol, fail, uf, hf, red, nw, outv, adam, beta1, beta2,
                     (hist && rank == 0) ? hist + step : nullptr, flag);
    __syncthreads();
    if (flag[0]) {
      done = 1;
      break;
    }
    // ---- 7. Adam (lane q of warp 0 updates parameter q)
    adam_phase(outv, adam, th, lower, mask, lr, beta1, beta2, eps);
    __syncthreads();
  }
  if (rank == 0 && tid == 0) {
    if (!flag[0] || restarts_mode)
      for (int q = 0; q < 4; ++q) theta_out[q] = th[q];
    *status = flag[0];
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

// ------------------------------------------------------------------ wide form
// m from 513 to 1024 (17..32 block rows) on one cluster of kWideCS = 16 CTAs:
// CTA r keeps block rows r and 31 - r (the second when it exists), so every
// CTA holds one short and one long row of the lower triangle and does about
// the same share of the work; each block row b is stored lower part only
// (columns 0 .. 32(b+1)-1, row stride 32(b+1) + 4), 136 KB for the pair.  The
// per-eigenpair FP64 arrays live in global memory (a slice per CTA), and
// column blocks are gathered kWideNP blocks at a time.  The barrier structure
// is the narrow form's: two cluster barriers per Cholesky block column, one
// per inverse block column (whose products go to a side buffer and are
// written in place only after it), one for the partial sums.
constexpr int kWideCS = 16;
constexpr int kWideNP = 4;
constexpr int kWideMaxNb = 2 * kWideCS;

__host__ __device__ constexpr int wide_owner(int b) { return b < kWideCS ? b : 2 * kWideCS - 1 - b; }
__host__ __device__ constexpr int wide_ld(int b) { return (b + 1) * FB + 4; }
// float offset of block row b in its owner's storage (the pair of a CTA r:
// row r at 0, row 31 - r after it)
__host__ __device__ constexpr int wide_off(int b) { return b < kWideCS ? 0 : FB * wide_ld(wide_owner(b)); }
constexpr int kWideAr = FB * (wide_ld(0) + wide_ld(kWideMaxNb - 1));  // the same for every pair r, 31 - r

struct WLayout {
  size_t Ar, P, Lk, dk, dinv, T, uf, hf, zt, part, pd, plog, red, th, adam, outv, flag, total;
};

__host__ __device__ inline WLayout wlayout() {
  WLayout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    size_t at = o;
    o += (bytes + 15) & ~size_t(15);
    return at;
  };
  const size_t mp = (size_t)kWideMaxNb * FB;
  L.Ar = take(4 * (size_t)kWideAr);
  L.P = take(4 * (size_t)kWideNP * FB * kLdP);
  L.Lk = take(4 * (size_t)FB * kLdP);
  L.dk = take(4 * FB);
  L.dinv = take(4 * 2 * FB);
  L.T = take(4 * 2 * (size_t)FB * kLdP);
  L.uf = take(4 * mp);
  L.hf = take(4 * mp);
  L.zt = take(4 * 2 * FB);
  L.part = take(4 * 2 * mp);
  L.pd = take(8 * 2);
  L.plog = take(8 * 2);
  L.red = take(8 * 8 * (kW + 1));
  L.th = take(8 * 4);
  L.adam = take(8 * 16);
  L.outv = take(8 * 8);
  L.flag = take(16);
  L.total = o;
  return L;
}

// panel_solve_rows for the eight warps [wbase, wbase + 8)
__device__ void panel_solve_rows_w(float* A, int ld, int c0, const float* Lk, const float* dk, int wbase) {
  const int lane = threadIdx.x & 31, warp = (threadIdx.x >> 5) - wbase;
  if (warp < 0 || warp >= FB / 4) return;
  float lrow[FB];
#pragma unroll
  for (int c = 0; c < FB; ++c) lrow[c] = c < lane ? Lk[lane * kLdP + c] : 0.f;
  const float dl = dk[lane];
  const int r = 4 * warp;
  float x[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) x[q] = A[(r + q) * ld + c0 + lane];
#pragma unroll
  for (int c = 0; c < FB; ++c) {
    const float dc = __shfl_sync(0xffffffffu, dl, c);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float xc = __shfl_sync(0xffffffffu, x[q], c) * dc;
      x[q] = (lane == c) ? xc : fmaf(-xc, lrow[c], x[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) A[(r + q) * ld + c0 + lane] = x[q];
}

// invert_own_diag by warp `wsel`
__device__ void invert_diag_w(float* A, int ld, int c0, const float* dinv, int wsel) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp != wsel) return;
  float x[FB];
#pragma unroll
  for (int k = 0; k < FB; ++k) x[k] = (k == lane) ? 1.f : 0.f;
  const float dl = dinv[lane];
  for (int c = 0; c < FB; ++c) {
    const float lic = (lane > c) ? A[lane * ld + c0 + c] : 0.f;
    const float dc = __shfl_sync(0xffffffffu, dl, c);
#pragma unroll
    for (int k = 0; k < FB; ++k) {
      const float xck = __shfl_sync(0xffffffffu, x[k], c) * dc;
      x[k] = (lane == c) ? xck : fmaf(-xck, lic, x[k]);
    }
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < FB; ++k) A[lane * ld + c0 + k] = (k <= lane) ? x[k] : 0.f;
}

// P[(b - b0) * 32 + r][0..31] = block (b, col) of the cluster's matrix for
// b in [b0, b0 + nblk) (float4 reads through DSMEM)
__device__ void gather_blocks_wide(cg::cluster_group& cl, const float* Ar, int b0, int nblk, int col, float* P) {
  const int n4 = nblk * FB * (FB / 4);
  constexpr int U = 4;
  for (int e0 = threadIdx.x; e0 < n4; e0 += U * kNT) {
    float4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * kNT;
      if (e < n4) {
        const int q = e / (FB / 4), c = 4 * (e % (FB / 4));
        const int b = b0 + q / FB, r = q % FB;
        const float* src = cl.map_shared_rank(const_cast<float*>(Ar), (unsigned)wide_owner(b)) + wide_off(b);
        v[u] = *reinterpret_cast<const float4*>(src + r * wide_ld(b) + col * FB + c);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * kNT;
      if (e < n4) {
        const int q = e / (FB / 4), c = 4 * (e % (FB / 4));
        *reinterpret_cast<float4*>(P + (size_t)q * kLdP + c) = v[u];
      }
    }
  }
}

__global__ void __launch_bounds__(kNT, 1)
    gp_fit_cluster_wide(const float* __restrict__ C32, const double* __restrict__ Cd, const double* __restrict__ bvec,
                        const double* __restrict__ yy_p, long long N, int m, const double* __restrict__ evals,
                        double n_rows, int typ, const double* __restrict__ theta0, const double* __restrict__ lower,
                        const int* __restrict__ mask, int steps, double lr, double beta1, double beta2, double eps,
                        double* __restrict__ theta_out, double* __restrict__ hist, int* __restrict__ status,
                        int restarts_mode, double* __restrict__ gscr) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int rs = blockIdx.x / kWideCS;  // cluster rs runs restart rs
  theta0 += 4 * rs;
  theta_out += 4 * rs;
  if (hist) hist += (size_t)steps * rs;
  status += rs;
  const int nb = (m + FB - 1) / FB;  // kWideCS < nb <= kWideMaxNb
  const int mp = nb * FB;
  int own[2] = {rank, 2 * kWideCS - 1 - rank};
  const int nown = own[1] < nb ? 2 : 1;
  const int bmax = own[nown - 1];  // the longer row
  extern __shared__ __align__(16) unsigned char sm[];
  const WLayout Ly = wlayout();
  float* Ar = reinterpret_cast<float*>(sm + Ly.Ar);
  float* P = reinterpret_cast<float*>(sm + Ly.P);
  float* Lk = reinterpret_cast<float*>(sm + Ly.Lk);
  float* dk = reinterpret_cast<float*>(sm + Ly.dk);
  float* dinv = reinterpret_cast<float*>(sm + Ly.dinv);
  float* T = reinterpret_cast<float*>(sm + Ly.T);
  float* uf = reinterpret_cast<float*>(sm + Ly.uf);
  float* hf = reinterpret_cast<float*>(sm + Ly.hf);
  float* zt = reinterpret_cast<float*>(sm + Ly.zt);
  float* part = reinterpret_cast<float*>(sm + Ly.part);
  double* pd = reinterpret_cast<double*>(sm + Ly.pd);
  double* plog = reinterpret_cast<double*>(sm + Ly.plog);
  double* red = reinterpret_cast<double*>(sm + Ly.red);
  double* th = reinterpret_cast<double*>(sm + Ly.th);
  double* adam = reinterpret_cast<double*>(sm + Ly.adam);
  double* outv = reinterpret_cast<double*>(sm + Ly.outv);
  int* flag = reinterpret_cast<int*>(sm + Ly.flag);
  __shared__ __align__(16) float lcol[2 * FB];
  double* gv = gscr + ((size_t)rs * kWideCS + rank) * 8 * (size_t)m;
  const FitVecs V{gv, gv + 3 * (size_t)m, gv + 4 * (size_t)m, gv + 5 * (size_t)m, gv + 6 * (size_t)m,
                  gv + 7 * (size_t)m};
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = min(kW, (m + 31) / 32);
  const double yy = yy_p[0];
  const double Nd = (double)N;
  auto row_base = [&](int slot) { return Ar + (slot == 0 ? 0 : FB * wide_ld(own[0])); };
  for (int l = tid; l < m; l += kNT) V.cdg[l] = Cd[(size_t)l * m + l];
  for (int l = m + tid; l < mp; l += kNT) {
    uf[l] = 0.f;
    hf[l] = 0.f;
  }
  for (int e = tid; e < kWideAr; e += kNT) Ar[e] = 0.f;
  for (int e = tid; e < 2 * FB; e += kNT) lcol[e] = 0.f;
  if (tid == 0) {
    flag[0] = 0;
    for (int q = 0; q < 4; ++q) {
      th[q] = theta0[q];
      const double v = theta0[q] - lower[q];
      adam[q] = v > 30.0 ? v : log(expm1(fmax(v, 1e-300)));  // inverse softplus
      adam[4 + q] = 0.0;
      adam[8 + q] = 0.0;
    }
    adam[12] = 1.0;
    adam[13] = 1.0;
  }
  __syncthreads();
  int done = 0;
  for (int step = 0; step < steps && !done; ++step) {
    const double nu = th[0], kappa = th[1], sf = th[2], s2 = th[3];
    double g0 = 0.0, g1 = 0.0;
    // ---- 1. spectral weights (FP64, every CTA computes all m)
    weights_phase(V, evals, bvec, m, mp, n_rows, typ, nu, kappa, sf, s2, red, nw, uf, hf, flag, g0, g1);
    __syncthreads();
    if (flag[0]) break;  // identical in every CTA
    // ---- 2. own block rows of the padded scaled capacitance matrix (lower parts)
    for (int q = warp; q < nown * FB; q += kW) {
      const int slot = q / FB, r = q % FB, b = own[slot];
      float* row = row_base(slot) + r * wide_ld(b);
      const int i = b * FB + r;
      const float hi = hf[i];
      for (int j = lane; j < (b + 1) * FB; j += 32) {
        float v = 0.f;
        if (j == i)
          v = 1.f;
        else if (j < i && i < m)
          v = __ldg(C32 + (size_t)i * m + j) * hi * hf[j];
        row[j] = v;
      }
    }
    if (tid == 0) flag[1] = 0;
    __syncthreads();
    // ---- 3. blocked Cholesky across the cluster
    for (int k = 0; k < nb; ++k) {
      if (wide_owner(k) == rank && warp == 0) {
        const int sk = k < kWideCS ? 0 : 1;
        const bool ok = diag_factor(row_base(sk), wide_ld(k), k * FB, dinv + sk * FB, lcol);
        if (!ok && lane == 0) flag[1] = 1;
      }
      cl.sync();
      const bool active = bmax > k;
      if (active) {
        const int ok_ = wide_owner(k), sk = k < kWideCS ? 0 : 1;
        const float* src = cl.map_shared_rank(Ar, (unsigned)ok_) + wide_off(k);
        const float* srcd = cl.map_shared_rank(dinv, (unsigned)ok_) + sk * FB;
        for (int e = tid; e < FB * FB; e += kNT)
          Lk[(e / FB) * kLdP + e % FB] = src[(e / FB) * wide_ld(k) + k * FB + e % FB];
        if (tid < FB) dk[tid] = srcd[tid];
        __syncthreads();
        for (int slot = 0; slot < nown; ++slot)
          if (own[slot] > k) panel_solve_rows_w(row_base(slot), wide_ld(own[slot]), k * FB, Lk, dk, 8 * slot);
      }
      cl.sync();
      if (active) {
        for (int jc = k + 1; jc <= bmax; jc += kWideNP) {
          const int jn = min(kWideNP, bmax - jc + 1);
          __syncthreads();  // the previous chunk's products are done with P
          gather_blocks_wide(cl, Ar, jc, jn, k, P);
          __syncthreads();
          // tiles: (slot, block j of the chunk, 4 x 4 tile); block (own[slot], j) needs j <= own[slot]
          const int tasks = nown * jn * 64;
          for (int t = tid; t < tasks; t += kNT) {
            const int slot = t / (jn * 64), jj = (t / 64) % jn, tt = t % 64;
            const int b = own[slot], j = jc + jj;
            if (b <= k || j > b) continue;
            float* A = row_base(slot);
            const int ldb = wide_ld(b);
            const int r0 = 4 * (tt / 8), cc = 4 * (tt % 8);
            float acc[4][4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
              for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
#pragma unroll 2
            for (int c = 0; c < FB; c += 4) {
              float4 bv[4];
#pragma unroll
              for (int v = 0; v < 4; ++v)
                bv[v] = *reinterpret_cast<const float4*>(P + (size_t)(jj * FB + cc + v) * kLdP + c);
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                const float4 a = *reinterpret_cast<const float4*>(A + (r0 + u) * ldb + k * FB + c);
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                  acc[u][v] = fmaf(a.x, bv[v].x, acc[u][v]);
                  acc[u][v] = fmaf(a.y, bv[v].y, acc[u][v]);
                  acc[u][v] = fmaf(a.z, bv[v].z, acc[u][v]);
                  acc[u][v] = fmaf(a.w, bv[v].w, acc[u][v]);
                }
              }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
              for (int v = 0; v < 4; ++v) A[(r0 + u) * ldb + j * FB + cc + v] -= acc[u][v];
          }
        }
      }
      __syncthreads();
    }
    // log-determinants of the own diagonal blocks, then their inverses in place
    if (warp < nown) {
      double lg = (double)logf(dinv[warp * FB + lane]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lg += __shfl_xor_sync(0xffffffffu, lg, o);
      if (lane == 0) plog[warp] = -lg;
    }
    for (int slot = 0; slot < nown; ++slot)
      invert_diag_w(row_base(slot), wide_ld(own[slot]), own[slot] * FB, dinv + slot * FB, slot);
    __syncthreads();
    const double logL = plog[0] + (nown > 1 ? plog[1] : 0.0);
    cl.sync();
    // ---- 4. M = L⁻¹: block columns right to left.  Thread t: slice t & 3
    // (one block of a gathered chunk), task t >> 2 = (slot, 4 x 4 tile); the
    // four slices of a task are adjacent lanes and are added by shuffles.
    for (int j = nb - 2; j >= 0; --j) {
      const bool active = bmax > j;
      const int slice = tid & 3, task = tid >> 2, slot = task >> 6, tt = task & 63;
      const bool mine = slot < nown && own[slot] > j;
      const int r0 = 4 * (tt / 8), cc = 4 * (tt % 8);
      float acc[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
      if (active) {
        const float* src = cl.map_shared_rank(Ar, (unsigned)wide_owner(j)) + wide_off(j);
        for (int e = tid; e < FB * FB; e += kNT)
          Lk[(e / FB) * kLdP + e % FB] = src[(e / FB) * wide_ld(j) + j * FB + e % FB];  // M_jj
        for (int jc = j + 1; jc <= bmax; jc += kWideNP) {
          const int jn = min(kWideNP, bmax - jc + 1);
          __syncthreads();
          gather_blocks_wide(cl, Ar, jc, jn, j, P);  // L blocks (kk, j)
          __syncthreads();
          const int kk = jc + slice;
          if (mine && slice < jn && kk <= own[slot]) {
            const float* A = row_base(slot);
            const int ldb = wide_ld(own[slot]);
            for (int t4 = 0; t4 < FB; t4 += 4) {
              float4 a[4];
#pragma unroll
              for (int u = 0; u < 4; ++u) a[u] = *reinterpret_cast<const float4*>(A + (r0 + u) * ldb + kk * FB + t4);
#pragma unroll
              for (int q = 0; q < 4; ++q) {
                const float4 bq = *reinterpret_cast<const float4*>(P + (size_t)(slice * FB + t4 + q) * kLdP + cc);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                  const float av = q == 0 ? a[u].x : q == 1 ? a[u].y : q == 2 ? a[u].z : a[u].w;
                  acc[u][0] = fmaf(av, bq.x, acc[u][0]);
                  acc[u][1] = fmaf(av, bq.y, acc[u][1]);
                  acc[u][2] = fmaf(av, bq.z, acc[u][2]);
                  acc[u][3] = fmaf(av, bq.w, acc[u][3]);
                }
              }
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          acc[u][v] += __shfl_xor_sync(0xffffffffu, acc[u][v], 1);
          acc[u][v] += __shfl_xor_sync(0xffffffffu, acc[u][v], 2);
        }
      if (mine && slice == 0)
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) T[(size_t)slot * FB * kLdP + (r0 + u) * kLdP + cc + v] = acc[u][v];
      __syncthreads();
      cl.sync();  // every read of column block j is done before it is overwritten
      if (active)
        for (int e = tid; e < nown * FB * FB; e += kNT) {
          const int sl = e / (FB * FB), r = (e / FB) % FB, c = e % FB;
          if (own[sl] <= j) continue;
          const float* Ts = T + (size_t)sl * FB * kLdP;
          float sacc = 0.f;
          for (int cp = c; cp < FB; ++cp) sacc = fmaf(Ts[r * kLdP + cp], Lk[cp * kLdP + c], sacc);
          row_base(sl)[r * wide_ld(own[sl]) + j * FB + c] = -sacc;
        }
      __syncthreads();
    }
    // ---- 5. z̃ = M u (own rows), partial column sums of M z̃ and M∘M
    for (int q = warp; q < nown * FB; q += kW) {
      const int slot = q / FB, r = q % FB, b = own[slot];
      const float* row = row_base(slot) + r * wide_ld(b);
      float s = 0.f;
      for (int k = lane; k <= b * FB + r; k += 32) s = fmaf(row[k], uf[k], s);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) zt[q] = s;
    }
    __syncthreads();
    for (int l = tid; l < mp; l += kNT) {
      float s = 0.f, q = 0.f;
      for (int slot = 0; slot < nown; ++slot) {
        const int b = own[slot];
        if (l >= (b + 1) * FB) continue;
        const float* A = row_base(slot);
        const int ldb = wide_ld(b);
        for (int r = 0; r < FB; ++r) {
          const float v = A[r * ldb + l];
          s = fmaf(v, zt[slot * FB + r], s);
          q = fmaf(v, v, q);
        }
      }
      part[l] = s;
      part[mp + l] = q;
    }
    if (tid == 0) {
      pd[0] = logL;
      pd[1] = (double)flag[1];
    }
    __syncthreads();
    cl.sync();
    for (int l = tid; l < mp; l += kNT) {
      float ps[kWideCS], pq[kWideCS];
#pragma unroll
      for (int c = 0; c < kWideCS; ++c) {
        const float* pc = cl.map_shared_rank(part, (unsigned)c);
        ps[c] = pc[l];
        pq[c] = pc[mp + l];
      }
      float s = 0.f, q = 0.f;
#pragma unroll
      for (int c = 0; c < kWideCS; ++c) {
        s += ps[c];
        q += pq[c];
      }
      uf[l] = s;
      hf[l] = q;
    }
    double logd_chol = 0.0;
    int fail = 0;
    for (int c = 0; c < kWideCS; ++c) {
      const double* pc = cl.map_shared_rank(pd, (unsigned)c);
      logd_chol += pc[0];
      fail |= pc[1] != 0.0;
    }
    __syncthreads();
    // ---- 6. likelihood and gradient, 7. Adam
    likelihood_phase(V, m, yy, Nd, s2, sf, g0, g1, logd_chol, fail, uf, hf, red, nw, outv, adam, beta1, beta2,
                     (hist && rank == 0) ? hist + step : nullptr, flag);
    __syncthreads();
    if (flag[0]) {
      done = 1;
      break;
    }
    adam_phase(outv, adam, th, lower, mask, lr, beta1, beta2, eps);
    __syncthreads();
  }
  if (rank == 0 && tid == 0) {
    if (!flag[0] || restarts_mode)
      for (int q = 0; q < 4; ++q) theta_out[q] = th[q];
    *status = flag[0];
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

}  // namespace

// Largest m the cluster fit handles on this device (0 when clusters of the
// needed size cannot be launched).
int gp_fit_cluster_max_m() {
  static int cached = -1;
  if (cached >= 0) return cached;
  int dev = 0, optin = 0;
  cached = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  if (cudaFuncSetAttribute(gp_fit_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int best = 0;
  for (int nb = 2; nb <= kMaxCluster; ++nb) {
    const int m = nb * FB;
    const size_t smem = clayout(m, nb).total;
    if (smem + 512 > (size_t)optin) break;
    if (raise_dyn_smem((const void*)gp_fit_cluster, (size_t)(smem)) != cudaSuccess) {
      cudaGetLastError();
      break;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nb);
    cfg.blockDim = dim3(kNT);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = nb;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, gp_fit_cluster, &cfg) != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      break;
    }
    best = m;
  }
  // the wide form, for 16 < nb <= 32, when the 16-block form fits
  if (best == kMaxCluster * FB && wlayout().total + 1024 <= (size_t)optin &&
      cudaFuncSetAttribute(gp_fit_cluster_wide, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
      raise_dyn_smem((const void*)gp_fit_cluster_wide, wlayout().total) == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kWideCS);
    cfg.blockDim = dim3(kNT);
    cfg.dynamicSmemBytes = wlayout().total;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kWideCS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, gp_fit_cluster_wide, &cfg) == cudaSuccess && nclusters >= 1)
      best = kWideMaxNb * FB;
  }
  cudaGetLastError();
  cached = best;
  return cached;
}

// Bytes of global scratch the cluster fit needs for `restarts` fits of size m
// (the wide form keeps its FP64 per-eigenpair arrays there: 8 m doubles per
// CTA and fit).
size_t gp_fit_cluster_scratch(int m, int restarts) {
  if (m <= kMaxCluster * FB) return 0;
  return (size_t)restarts * kWideCS * 8 * (size_t)m * sizeof(double);
}

// Enqueues the cluster fit (arguments as the one-CTA kernel; C32 = C in FP32).
int gp_fit_cluster_launch(const float* C32, const double* C, const double* b, const double* yy, long long N, int m,
                          const double* evals, double n_rows, int typ, const double* theta0, const double* lower_dev,
                          const int* mask_dev, int steps, double lr, double beta1, double beta2, double eps,
                          double* theta_out, double* hist, int* status, cudaStream_t st, int restarts,
                          int restarts_mode, double* scratch) {
  const int nb = (m + FB - 1) / FB;
  if (nb < 2 || nb > kWideMaxNb || m > gp_fit_cluster_max_m()) {
    set_error("gp_fit_cluster: m=%d outside the cluster fit's range", m);
    return RVGP_EARG;
  }
  if (nb > kMaxCluster) {
    if (!scratch) {
      set_error("gp_fit_cluster: m=%d needs %zu bytes of scratch", m, gp_fit_cluster_scratch(m, restarts));
      return RVGP_EARG;
    }
    const size_t smem = wlayout().total;
    if (raise_dyn_smem((const void*)gp_fit_cluster_wide, (size_t)(smem)) !=
        cudaSuccess) {
      set_error("gp_fit_cluster: cannot reserve %zu bytes of shared memory", smem);
      return RVGP_ELAUNCH;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kWideCS * restarts);  // one cluster per fit
    cfg.blockDim = dim3(kNT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kWideCS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    rvgp::note_launch();
    const cudaError_t e = cudaLaunchKernelEx(&cfg, gp_fit_cluster_wide, C32, C, b, yy, N, m, evals, n_rows, typ,
                                             theta0, lower_dev, mask_dev, steps, lr, beta1, beta2, eps, theta_out,
                                             hist, status, restarts_mode, scratch);
    if (e != cudaSuccess) {
      set_error("gp_fit_cluster: launch failed: %s", cudaGetErrorString(e));
      return RVGP_ELAUNCH;
    }
    return RVGP_OK;
  }
  const size_t smem = clayout(m, nb).total;
  if (raise_dyn_smem((const void*)gp_fit_cluster, (size_t)(smem)) != cudaSuccess) {
    set_error("gp_fit_cluster: cannot reserve %zu bytes of shared memory", smem);
    return RVGP_ELAUNCH;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nb * restarts);  // one cluster per fit
  cfg.blockDim = dim3(kNT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = nb;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  rvgp::note_launch();
  const cudaError_t e = cudaLaunchKernelEx(&cfg, gp_fit_cluster, C32, C, b, yy, N, m, evals, n_rows, typ, theta0,
                                           lower_dev, mask_dev, steps, lr, beta1, beta2, eps, theta_out, hist,
                                           status, restarts_mode);
  if (e != cudaSuccess) {
    set_error("gp_fit_cluster: launch failed: %s", cudaGetErrorString(e));
    return RVGP_ELAUNCH;
  }
  return RVGP_OK;
}

}  // namespace rvgp
