// Smallest eigenpairs of a sparse symmetric positive semi-definite block-CSR
// matrix by Chebyshev-filtered subspace iteration.
//
// Replaces compute_spectrum (RVGP/geometry.py:66-80), which calls ARPACK
// eigsh(which="SM") on the graph Laplacian L (n x n) and the connection
// Laplacian Lc (nd x nd).  Same result contract: the m algebraically smallest
// eigenvalues in ascending order and orthonormal eigenvectors (the caller
// applies the reference's sqrt(N) scaling through `scale`).
//
// Iteration (block of p = m + guard vectors, all bulk work on the device):
//   filter  : V <- p_k(A) V, the scaled Chebyshev polynomial of degree k that
//             damps [a, b] (a = largest Ritz value, b = Gershgorin bound) and
//             grows [0, a); 3-term recurrence fused into the SpMM.
//   orth    : column scaling + Cholesky QR twice (G = VᵀV, V <- V L⁻ᵀ).
//   RR      : W = A V, H = Vᵀ W, H = Q Θ Qᵀ (Jacobi), V <- V Q, W <- W Q.
//   check   : residuals |W_j - θ_j V_j|; stop when the first m are below
//             tol * b.
// Two precisions:
//   plain (mode 0): everything in FP64;
//   mixed (mode 1): SpMM and the tall products in FP32 (Gram partial sums
//             reduced in FP64), the p x p Cholesky in FP64, the Rayleigh-Ritz
//             eigensolve in FP32, then FP64 refinement iterations starting
//             from the FP32 subspace only if the FP64 tolerance asks for it.
#include "common.cuh"
#include "linalg.cuh"
#include <math.h>
#include <string.h>
#include <float.h>
#include <vector>
#include <algorithm>

namespace rvgp {
int bspmm_planned_f32(const void* plan, size_t plan_bytes, int n, int DB, long long nnz, const int* indptr,
                      const int* indices, const float* vals, const float* X, float* Y, const float* Z, int b, int ld,
                      float alpha, float beta, float gamma, cudaStream_t st);
int bspmm_planned_f64(const void* plan, size_t plan_bytes, int n, int DB, long long nnz, const int* indptr,
                      const int* indices, const double* vals, const double* X, double* Y, const double* Z, int b,
                      int ld, double alpha, double beta, double gamma, cudaStream_t st);
size_t spmm_plan_bytes(int n, int DB, long long nnz);
int spmm_plan_build(int n, int DB, const int* indptr, const int* indices, long long nnz, void* plan,
                    size_t plan_bytes, cudaStream_t st);

namespace {

// the tiled product's plan of the matrix (null: untiled variants)
struct SpmmPlan {
  const void* plan = nullptr;
  size_t bytes = 0;
  long long nnz = 0;
};

inline int spmm(const SpmmPlan& pl, int n, int DB, const int* ip, const int* ix, const float* v, const float* X,
                float* Y, const float* Z, int b, int ld, double al, double be, double ga, cudaStream_t st) {
  return bspmm_planned_f32(pl.plan, pl.bytes, n, DB, pl.nnz, ip, ix, v, X, Y, Z, b, ld, (float)al, (float)be,
                           (float)ga, st);
}
inline int spmm(const SpmmPlan& pl, int n, int DB, const int* ip, const int* ix, const double* v, const double* X,
                double* Y, const double* Z, int b, int ld, double al, double be, double ga, cudaStream_t st) {
  return bspmm_planned_f64(pl.plan, pl.bytes, n, DB, pl.nnz, ip, ix, v, X, Y, Z, b, ld, al, be, ga, st);
}

__global__ void gershgorin_kernel(int n, int DB, const int* __restrict__ indptr, const double* __restrict__ vals,
                                  double* __restrict__ part) {
  __shared__ double sh[256];
  double mx = 0.0;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < (long long)n * DB;
       r += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(r / DB), p = (int)(r % DB);
    double s = 0.0;
    for (int t = indptr[i]; t < indptr[i + 1]; ++t)
      for (int q = 0; q < DB; ++q) s += fabs(vals[((size_t)t * DB + p) * DB + q]);
    mx = fmax(mx, s);
  }
  sh[threadIdx.x] = mx;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__device__ __forceinline__ double hash_uniform(unsigned long long seed, unsigned long long a) {
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (a + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
}

// Start block: entry (r, j) is a hash of its position in the caller's row
// numbering, so a renumbered matrix (row r = original block row perm[r / DB])
// starts from the same block, permuted.
template <typename T>
__global__ void random_block(T* __restrict__ V, long long N, int p, int ld, unsigned long long seed,
                             const int* __restrict__ perm, int DB) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= N * p) return;
  const long long r = e / p;
  const int j = (int)(e % p);
  const long long ro = perm ? (long long)perm[r / DB] * DB + r % DB : r;
  V[r * ld + j] = (T)hash_uniform(seed, (unsigned long long)(ro * p + j));
}

// B (p x p, type T) = Linvᵀ, i.e. B[k][j] = Linv[j][k]
template <typename T>
__global__ void transpose_to(const double* __restrict__ A, int p, T* __restrict__ B) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)p * p) return;
  const int k = (int)(e / p), j = (int)(e % p);
  B[e] = (T)A[(size_t)j * p + k];
}

template <typename T>
__global__ void copy_to(const double* __restrict__ A, long long cnt, T* __restrict__ B) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e < cnt) B[e] = (T)A[e];
}

// Second Cholesky QR pass for blocks wider than the one-CTA FP32 path: with
// D = diag(G)^-½ and E = D G D - I, *emax = max |E| (as the bits of a
// non-negative float, which order like the values; zeroed by the caller).
__global__ void first_order_emax(const double* __restrict__ G, int p, unsigned* __restrict__ emax) {
  float em = 0.f;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)p * p;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / p), j = (int)(e % p);
    if (j >= i) continue;
    const double v = G[e] * rsqrt(G[(size_t)i * p + i]) * rsqrt(G[(size_t)j * p + j]);
    em = fmaxf(em, (float)fabs(v));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) em = fmaxf(em, __shfl_xor_sync(0xffffffffu, em, o));
  if ((threadIdx.x & 31) == 0) atomicMax(emax, __float_as_uint(em));
}

// B = D (I - E/2) (p x p, row-major, FP32): V B is orthonormal to O(|E|²)
__global__ void first_order_B(const double* __restrict__ G, int p, float* __restrict__ B) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)p * p) return;
  const int i = (int)(e / p), j = (int)(e % p);
  const double di = rsqrt(G[(size_t)i * p + i]);
  const double Eij = (i == j) ? 0.0 : G[e] * di * rsqrt(G[(size_t)j * p + j]);
  B[e] = (float)(di * ((i == j ? 1.0 : 0.0) - 0.5 * Eij));
}

// add shift * trace(G)/p to the diagonal (rescue for a numerically singular Gram)
__global__ void shift_diag(double* __restrict__ G, int p, double rel) {
  __shared__ double tr;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < p; ++i) s += G[(size_t)i * p + i];
    tr = s / p;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < p; i += blockDim.x) G[(size_t)i * p + i] += rel * tr;
}

// part[c][j] = sum over rows of chunk c of (W[r][j] - theta_j V[r][j])²:
// grid (chunks, ceil(b / 32)); warp w takes rows r0 + w, r0 + w + 8, ... for
// columns j = 32 blockIdx.y + lane (coalesced); the 8 warp sums are added in
// a fixed order.  FP32 blocks use FP32 fused differences (W and V are FP32
// already, so one rounding of d adds nothing to their own) with FP32 partial
// sums over the warp's rows.
template <typename T>
__global__ void __launch_bounds__(256) resid_partial(const T* __restrict__ W, const T* __restrict__ V,
                                                     const double* __restrict__ theta, int ld, long long N, int b,
                                                     long long chunk, double* __restrict__ part) {
  __shared__ double sh[8][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.y * 32 + lane;
  const long long r0 = blockIdx.x * chunk, r1 = min(N, r0 + chunk);
  double s = 0.0;
  if (j < b) {
    if constexpr (sizeof(T) == 4) {
      const float th = (float)theta[j];
      float a0 = 0.f, a1 = 0.f;
      long long r = r0 + warp;
      for (; r + 8 < r1; r += 16) {
        const float d0 = fmaf(-th, V[r * ld + j], W[r * ld + j]);
        const float d1 = fmaf(-th, V[(r + 8) * ld + j], W[(r + 8) * ld + j]);
        a0 = fmaf(d0, d0, a0);
        a1 = fmaf(d1, d1, a1);
      }
      for (; r < r1; r += 8) {
        const float d = fmaf(-th, V[r * ld + j], W[r * ld + j]);
        a0 = fmaf(d, d, a0);
      }
      s = (double)a0 + (double)a1;
    } else {
      const double th = theta[j];
      for (long long r = r0 + warp; r < r1; r += 8) {
        const double d = (double)W[r * ld + j] - th * (double)V[r * ld + j];
        s += d * d;
      }
    }
  }
  sh[warp][lane] = s;
  __syncthreads();
  if (warp == 0 && j < b) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += sh[w][lane];
    part[(size_t)blockIdx.x * b + j] = t;
  }
}

// Rayleigh quotients of the FP32 Ritz vectors: vᵀw and vᵀv per column (FP32
// products summed in FP64 per row chunk), then theta = vᵀw / vᵀv.  The FP32
// Jacobi's diagonal drifts with its rounding (~1e-4 relative at p ~ 500,
// growing with the rotations per index); the quotient's error is of the order
// of the squared residual.
__global__ void __launch_bounds__(256) rq_partial(const float* __restrict__ W, const float* __restrict__ V, int ld,
                                                  long long N, int b, long long chunk, double* __restrict__ part) {
  __shared__ double sh[2][8][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.y * 32 + lane;
  const long long r0 = blockIdx.x * chunk, r1 = min(N, r0 + chunk);
  double vw = 0.0, vv = 0.0;
  if (j < b) {
    for (long long r = r0 + warp; r < r1;) {
      float a0 = 0.f, a1 = 0.f;  // FP32 sums of at most 16 rows, then FP64
      for (int k = 0; k < 16 && r < r1; ++k, r += 8) {
        const float v = V[r * ld + j];
        a0 = fmaf(v, W[r * ld + j], a0);
        a1 = fmaf(v, v, a1);
      }
      vw += a0;
      vv += a1;
    }
  }
  sh[0][warp][lane] = vw;
  sh[1][warp][lane] = vv;
  __syncthreads();
  if (warp == 0 && j < b) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < 8; ++w) {
      t0 += sh[0][w][lane];
      t1 += sh[1][w][lane];
    }
    part[(size_t)blockIdx.x * 2 * b + j] = t0;
    part[(size_t)blockIdx.x * 2 * b + b + j] = t1;
  }
}

__global__ void rq_final(const double* __restrict__ part, int nchunk, int b, double* __restrict__ theta) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= b) return;
  double vw = 0.0, vv = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    vw += part[(size_t)c * 2 * b + j];
    vv += part[(size_t)c * 2 * b + b + j];
  }
  if (vv > 0.0) theta[j] = vw / vv;
}

__global__ void resid_final(const double* __restrict__ part, int nchunk, int b, double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= b) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * b + j];
  out[j] = sqrt(s);
}

template <typename T>
__global__ void write_output(const T* __restrict__ V, int ldv, long long N, int m, double scale, double* __restrict__ out,
                             int ldo, const int* __restrict__ perm, int DB, const int* __restrict__ colmap) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= N * m) return;
  const long long r = e / m;
  const int j = (int)(e % m);
  const long long ro = perm ? (long long)perm[r / DB] * DB + r % DB : r;
  out[ro * ldo + j] = scale * (double)V[r * ldv + colmap[j]];
}

// dst[r, d0 + j] = src[r, c0 + j], j < ncols (all column offsets and leading
// dimensions multiples of 4: float4 moves)
__global__ void copy_cols4(const float* __restrict__ src, int lds, int c0, float* __restrict__ dst, int ldd, int d0,
                           long long N, int ncols) {
  const int g = ncols / 4;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N * g;
       e += (long long)gridDim.x * blockDim.x) {
    const long long r = e / g;
    const int j = 4 * (int)(e % g);
    *reinterpret_cast<float4*>(dst + r * ldd + d0 + j) = *reinterpret_cast<const float4*>(src + r * lds + c0 + j);
  }
}

__global__ void sub_f32x4(float* __restrict__ X, const float* __restrict__ Y, long long n4) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n4;
       e += (long long)gridDim.x * blockDim.x) {
    float4 a = reinterpret_cast<float4*>(X)[e];
    const float4 b = reinterpret_cast<const float4*>(Y)[e];
    a.x -= b.x;
    a.y -= b.y;
    a.z -= b.z;
    a.w -= b.w;
    reinterpret_cast<float4*>(X)[e] = a;
  }
}

int resid_chunks(long long N) { return (int)std::max<long long>(1, std::min<long long>(512, (N + 1023) / 1024)); }

// ------------------------------------------------------------------------------ solver state
template <typename T>
struct Block {
  T *V, *W, *T1, *T2;  // N x p each, ld = p
};

struct Small {
  double *G, *H, *Q, *Linv, *theta, *res, *norms64;
  double *gersh, *resid_part;
  int* info;
  int* colmap;  // output column -> block column (Ritz values sorted)
  void* gram_ws;
  size_t gram_bytes;
  void* jac_ws;
  size_t jac_bytes;
  void* cn_ws;
  size_t cn_bytes;
  float* Bf;
  double* Bd;
  float *Hf, *thf;  // FP32 Rayleigh-Ritz matrix and its eigenvalues (mixed form)
  float *L32, *Mb32;  // FP32 Cholesky QR factor and its diagonal-block inverses
  float* d32;         // its column scaling diag(VᵀV)^-½
  int cholqr32;       // p fits the one-CTA FP32 Cholesky QR
  int jac32;          // p fits the one-CTA FP32 Jacobi
  int jacb;           // FP32 block Jacobi (wider p)
  void* jac32_ws;
  size_t jac32_bytes;
  float* nf;
  double* nd;
  int tc;             // FP32 tall products on the tensor cores (tc_gemm.cu)
  int* tc_err;        // raised by a tensor-core kernel whose pipeline wait timed out
  void* tc_ws;
  size_t tc_bytes;
};

struct Problem {
  int n, DB;
  long long N;
  const int *indptr, *indices;
  const double* v64;
  const float* v32;
  int m, p;
  SpmmPlan plan;
};

template <typename T>
const T* vals_of(const Problem& P);
template <>
const float* vals_of<float>(const Problem& P) { return P.v32; }
template <>
const double* vals_of<double>(const Problem& P) { return P.v64; }

template <typename T>
T* Bmat(Small& s);
template <>
float* Bmat<float>(Small& s) { return s.Bf; }
template <>
double* Bmat<double>(Small& s) { return s.Bd; }
template <typename T>
T* nrm(Small& s);
template <>
float* nrm<float>(Small& s) { return s.nf; }
template <>
double* nrm<double>(Small& s) { return s.nd; }

inline int gram_any(const float* A, const float* B, long long N, int p, double* C, Small& s, cudaStream_t st) {
  if (s.tc) return tc_gram_f32_out64(A, p, B, p, N, p, p, C, p, s.tc_err, s.tc_ws, s.tc_bytes, st);
  return gram_f32_out64(A, p, B, p, N, p, p, C, p, 1.0, 0.0, s.gram_ws, s.gram_bytes, st);
}
// C (N x p) = A (N x p) Bm (p x p), ld = p
inline int block_product(const float* A, const float* Bm, long long N, int p, float* C, Small& s, cudaStream_t st) {
  if (s.tc) return tc_gemm_f32(A, p, N, p, Bm, p, p, C, p, s.tc_err, s.tc_ws, s.tc_bytes, st);
  return gemm_nn<float>(A, p, Bm, p, N, p, p, C, p, 1.f, 0.f, st);
}
inline int block_product(const double* A, const double* Bm, long long N, int p, double* C, Small&, cudaStream_t st) {
  return gemm_nn<double>(A, p, Bm, p, N, p, p, C, p, 1.0, 0.0, st);
}
inline int gram_any(const double* A, const double* B, long long N, int p, double* C, Small& s, cudaStream_t st) {
  return gram<double>(A, p, B, p, N, p, p, C, p, 1.0, 0.0, s.gram_ws, s.gram_bytes, st);
}

constexpr int kFp32Sweeps = 12;
// second Cholesky QR pass: first-order correction when max |E| <= this (the
// result's departure from orthonormality is ~0.75 |E|², 7.5e-7 at the bound)
constexpr float kFirstOrderTol = 1e-3f;  // FP32 Jacobi sweeps are capped: off(H) stalls at FP32 rounding

#define TRY(x)                  \
  do {                          \
    int _s = (x);               \
    if (_s != RVGP_OK) return _s; \
  } while (0)

struct Stats {
  int iters = 0, spmm = 0, sweeps = 0, conv = 0, refine_iters = 0, chol_rescues = 0, locked = 0;
  float ms[4] = {0, 0, 0, 0};  // filter, orthonormalise, Rayleigh-Ritz tall products, Jacobi
};

// CUDA events at phase boundaries; elapsed times are collected after the
// synchronisation that ends every Rayleigh-Ritz step.
struct PhaseEvents {
  cudaEvent_t e[6];
  PhaseEvents() {
    for (auto& x : e) cudaEventCreate(&x);
  }
  ~PhaseEvents() {
    for (auto& x : e) cudaEventDestroy(x);
  }
  void collect(Stats& s) {
    float t;
    const int pairs[4][2] = {{0, 1}, {1, 2}, {2, 5}, {3, 4}};
    for (int q = 0; q < 4; ++q)
      if (cudaEventElapsedTime(&t, e[pairs[q][0]], e[pairs[q][1]]) == cudaSuccess) s.ms[q] += t;
    s.ms[2] -= (cudaEventElapsedTime(&t, e[3], e[4]) == cudaSuccess) ? t : 0.f;  // RR time excludes Jacobi
  }
};

// Chebyshev filter of degree deg on [a, b] with lower bound a0; result pointer returned in *out.
template <typename T>
int filter(const Problem& P, Block<T>& B, int deg, double a, double b, double a0, Stats& stt, cudaStream_t st) {
  const double e = (b - a) / 2, c = (b + a) / 2;
  double sigma = e / (a0 - c);
  const double tau = 2.0 / sigma;
  T *X = B.V, *Y = B.T1, *Z = B.T2;
  const T* vals = vals_of<T>(P);
  TRY(spmm(P.plan, P.n, P.DB, P.indptr, P.indices, vals, X, Y, (const T*)nullptr, P.p, P.p, sigma / e, -c * sigma / e, 0.0, st));
  ++stt.spmm;
  for (int i = 2; i <= deg; ++i) {
    const double sn = 1.0 / (tau - sigma);
    TRY(spmm(P.plan, P.n, P.DB, P.indptr, P.indices, vals, Y, Z, X, P.p, P.p, 2 * sn / e, -2 * c * sn / e, -sigma * sn, st));
    ++stt.spmm;
    T* t = X;
    X = Y;
    Y = Z;
    Z = t;
    sigma = sn;
  }
  // result in Y; make it V
  B.V = Y;
  B.T1 = X;
  B.T2 = Z;
  return RVGP_OK;
}

// V <- orthonormal basis of span(V): Cholesky QR with column scaling, twice.
// FP32 block: the scaling d = diag(VᵀV)^-½ is applied to the Gram inside the
// one-CTA FP32 factorisation and to V inside the triangular solve, so V is
// read twice per pass (Gram, solve).  Otherwise (or when an FP32 pivot fails)
// V is scaled explicitly and the FP64 Gram is factored in FP64.
template <typename T>
int orthonormalise(const Problem& P, Block<T>& B, Small& s, Stats& stt, cudaStream_t st) {
  const long long N = P.N;
  const int p = P.p;
  int rescues = 0;
  for (int pass = 0; pass < 2; ++pass) {
    if (sizeof(T) == 4 && s.cholqr32) {
      TRY(gram_any(B.V, B.V, N, p, s.G, s, st));
      // the second pass usually meets a block orthonormal to ~1e-4: a first-order
      // correction (one block product) then replaces factorisation and solve
      TRY(chol32_gram(s.G, p, s.L32, s.Mb32, s.d32, pass == 1 ? kFirstOrderTol : 0.f, s.info, st));
      int info32 = 0;
      if (read_back(&info32, s.info, sizeof(int), st) != cudaSuccess) return check_launch("orthonormalise");
      if (info32 == 2) {
        TRY(block_product(reinterpret_cast<const float*>(B.V), s.L32, N, p, reinterpret_cast<float*>(B.T1), s, st));
        std::swap(B.V, B.T1);
        continue;
      }
      if (info32 == 0) {
        TRY(trsm_rows_f32(reinterpret_cast<float*>(B.V), p, N, p, s.L32, s.Mb32, s.d32, st));
        continue;
      }
      // a failed FP32 pivot: the same pass in FP64 on the explicitly scaled block
    } else if (sizeof(T) == 4 && pass == 1) {
      // wide FP32 block: the second pass is usually a first-order correction
      // (one tensor-core block product) as in the one-CTA path above
      TRY(gram_any(B.V, B.V, N, p, s.G, s, st));
      cudaMemsetAsync(s.info + 1, 0, sizeof(unsigned), st);
      rvgp::note_launch();
      first_order_emax<<<std::min(4 * num_sms(), ceil_div((long long)p * p, 256)), 256, 0, st>>>(
          s.G, p, reinterpret_cast<unsigned*>(s.info + 1));
      unsigned bits = 0;
      if (read_back(&bits, s.info + 1, sizeof(unsigned), st) != cudaSuccess) return check_launch("orthonormalise");
      float emax;
      memcpy(&emax, &bits, sizeof(float));
      if (emax <= kFirstOrderTol) {
        rvgp::note_launch();
        first_order_B<<<ceil_div((long long)p * p, 256), 256, 0, st>>>(s.G, p, s.Bf);
        TRY(block_product(reinterpret_cast<const float*>(B.V), s.Bf, N, p, reinterpret_cast<float*>(B.T1), s, st));
        std::swap(B.V, B.T1);
        continue;
      }
      // not near orthonormal: the full pass below (its Gram is recomputed on the scaled block)
    }
    TRY(col_norms<T>(B.V, p, N, p, nrm<T>(s), s.cn_ws, s.cn_bytes, st));
    TRY(scale_cols<T>(B.V, p, N, p, nrm<T>(s), true, st));
    TRY(gram_any(B.V, B.V, N, p, s.G, s, st));
    TRY(cholesky<double>(s.G, p, p, s.info, st));
    int info = 0;
    if (read_back(&info, s.info, sizeof(int), st) != cudaSuccess) return check_launch("orthonormalise");
    if (info != 0) {
      // Numerically singular Gram (rounding of an ill-conditioned block made
      // it indefinite): shifted Cholesky QR on a fresh Gram, the shift raised
      // until the factorisation holds (10 u p ||V||² in FP32 terms is ~1e-4
      // at p = 1000); the shifted factor leaves a block of condition ~s^-½,
      // which two plain passes then orthonormalise.
      ++stt.chol_rescues;
      if (++rescues > 3) {
        set_error("eigensolver: Cholesky QR failed repeatedly (block lost rank)");
        return 1;
      }
      const double shifts[] = {sizeof(T) == 4 ? 1e-5 : 1e-12, 1e-4, 1e-3, 1e-2};
      for (double sh : shifts) {
        TRY(gram_any(B.V, B.V, N, p, s.G, s, st));
        rvgp::note_launch(); shift_diag<<<1, 256, 0, st>>>(s.G, p, sh);
        TRY(cholesky<double>(s.G, p, p, s.info, st));
        if (read_back(&info, s.info, sizeof(int), st) != cudaSuccess) return check_launch("orthonormalise");
        if (info == 0) break;
      }
      if (info != 0) {
        set_error("eigensolver: Cholesky QR failed (block lost rank)");
        return 1;
      }
      pass = -1;  // two clean passes after the rescue
    }
    TRY(tri_inv_lower<double>(s.G, p, p, s.Linv, p, st));
    rvgp::note_launch(); transpose_to<T><<<ceil_div((long long)p * p, 256), 256, 0, st>>>(s.Linv, p, Bmat<T>(s));
    TRY(block_product(B.V, Bmat<T>(s), N, p, B.T1, s, st));
    std::swap(B.V, B.T1);
  }
  return RVGP_OK;
}

// Rayleigh-Ritz: V, W = A V rotated to Ritz vectors; theta, residuals to host.
template <typename T>
int rayleigh_ritz(const Problem& P, Block<T>& B, Small& s, Stats& stt, int max_sweeps, std::vector<double>& theta,
                  std::vector<double>& res, PhaseEvents& ev, cudaStream_t st) {
  const long long N = P.N;
  const int p = P.p;
  TRY(spmm(P.plan, P.n, P.DB, P.indptr, P.indices, vals_of<T>(P), B.V, B.W, (const T*)nullptr, p, p, 1.0, 0.0, 0.0, st));
  ++stt.spmm;
  TRY(gram_any(B.V, B.W, N, p, s.H, s, st));
  int used = 0;
  cudaEventRecord(ev.e[3], st);
  if (sizeof(T) == 4) {
    // FP32 block: the FP64-reduced H is diagonalised in FP32 (an FP64 Jacobi
    // rotation costs ~64x an FP32 one on GB300).  Stop at off(H) <= 4e-6 ||H||_F,
    // below the FP32 stage's residual tolerance and above FP32 rounding.
    TRY(convert_f64_to_f32(s.H, p, s.Hf, p, p, p, st));
    // the one-sweep intermediate steps by block Jacobi (3.7x faster per sweep at
    // p = 1128; its FP32 rounding floor, ~5e-4 of ||H||, is irrelevant there and
    // the Ritz values are recomputed as Rayleigh quotients below); the full
    // step by the scalar kernel, whose floor is lower
    if (s.jacb && max_sweeps <= 1)
      TRY(jacobi_block_eigh(s.Hf, p, s.thf, s.Bf, max_sweeps, 4e-6, &used, s.jac_ws, s.jac_bytes, st));
    else if (s.jac32)
      TRY(jacobi32_eigh(s.Hf, p, s.thf, s.Bf, std::min(max_sweeps, kFp32Sweeps), 4e-6, &used, s.jac32_ws,
                        s.jac32_bytes, st));
    else
      TRY(jacobi_eigh<float>(s.Hf, p, s.thf, s.Bf, std::min(max_sweeps, kFp32Sweeps), 4e-6, &used, s.jac_ws,
                             s.jac_bytes, st));
    TRY(convert_f32_to_f64(s.thf, 1, s.theta, 1, p, 1, st));
  } else {
    TRY(jacobi_eigh<double>(s.H, p, s.theta, s.Q, max_sweeps, 1e-13, &used, s.jac_ws, s.jac_bytes, st));
    rvgp::note_launch(); copy_to<T><<<ceil_div((long long)p * p, 256), 256, 0, st>>>(s.Q, (long long)p * p, Bmat<T>(s));
  }
  cudaEventRecord(ev.e[4], st);
  stt.sweeps += used;
  TRY(block_product(B.V, Bmat<T>(s), N, p, B.T1, s, st));
  TRY(block_product(B.W, Bmat<T>(s), N, p, B.T2, s, st));
  std::swap(B.V, B.T1);
  std::swap(B.W, B.T2);
  const int nc = resid_chunks(N);
  const long long chunk = (N + nc - 1) / nc;
  if (sizeof(T) == 4) {
    rvgp::note_launch();
    rq_partial<<<dim3(nc, ceil_div(p, 32)), 256, 0, st>>>(reinterpret_cast<const float*>(B.W),
                                                          reinterpret_cast<const float*>(B.V), p, N, p, chunk,
                                                          s.resid_part);
    rvgp::note_launch(); rq_final<<<ceil_div(p, 256), 256, 0, st>>>(s.resid_part, nc, p, s.theta);
  }
  rvgp::note_launch();
  resid_partial<T><<<dim3(nc, ceil_div(p, 32)), 256, 0, st>>>(B.W, B.V, s.theta, p, N, p, chunk, s.resid_part);
  rvgp::note_launch(); resid_final<<<ceil_div(p, 256), 256, 0, st>>>(s.resid_part, nc, p, s.res);
  cudaEventRecord(ev.e[5], st);
  theta.resize(p);
  res.resize(p);
  if (read_back(theta.data(), s.theta, sizeof(double) * p, st) != cudaSuccess ||
      read_back(res.data(), s.res, sizeof(double) * p, st) != cudaSuccess)
    return check_launch("rayleigh_ritz");
  ev.collect(stt);
  return check_launch("rayleigh_ritz");
}

// Degree of the next filter on [a, b]: the m-th Ritz direction grows by about
// 2e4 against the edge a, the lowest one by at most `range` times the m-th and
// by at most `amp` in all.  `amp` bounds the spread of the filtered block's
// column norms along the Ritz directions, hence its condition number: an FP32
// block whose lowest directions outgrow the guard directions by much more
// than ~1e5 (with a Ritz basis only partly rotated) has a Gram matrix that
// its own rounding makes indefinite.
constexpr double kAmp32 = 1e5;  // largest filter gain of the FP32 stage

int choose_degree(const std::vector<double>& th, int m, double a, double b, double range, int cap, double amp) {
  const double e = (b - a) / 2, c = (b + a) / 2;
  const double xm = std::max(1.0 + 1e-6, (c - th[m - 1]) / e);
  const double x0 = std::max(xm, (c - std::min(th[0], th[m - 1])) / e);
  int deg = (int)ceil(log(2e4) / acosh(xm));
  const double gap = acosh(x0) - acosh(xm);
  if (gap > 0) deg = std::min(deg, (int)floor(log(range) / gap));
  deg = std::min(deg, (int)floor(acosh(amp) / acosh(x0)));
  return std::max(4, std::min(deg, cap));
}

// Runs iterations in precision T from the current B.V (orthonormalised inside).
template <typename T>
int iterate(const Problem& P, Block<T>& B, Small& s, Stats& stt, double bup, double tol, int max_iter, int first_deg,
            double range, std::vector<double>& theta, std::vector<double>& res, bool have_ritz, int* nconv_out,
            cudaStream_t st) {
  const int m = P.m, p = P.p;
  int nconv = 0;
  double a, a0;
  int deg = first_deg;
  if (have_ritz) {
    a = theta[p - 1];
    a0 = std::min(theta[0], 0.0) - 1e-3 * bup;
    deg = choose_degree(theta, m, a, bup, range, sizeof(T) == 4 ? 60 : 250, sizeof(T) == 4 ? kAmp32 : 1e300);
  } else {
    a = bup * std::min(0.5, std::max(4.0 * p / (double)P.N, 0.01));
    a0 = -1e-3 * bup;
  }
  PhaseEvents ev;
  // Intermediate Rayleigh-Ritz steps only partly diagonalise VᵀAV (a few Jacobi
  // sweeps): the filtered subspace does not depend on the basis inside it, and
  // rough Ritz values suffice for the filter bounds.  Once the residuals pass,
  // a full Rayleigh-Ritz step polishes the basis and the test is repeated.
  constexpr int kPartialSweeps = 1, kFullSweeps = 60;
  for (int it = 0; it < max_iter; ++it) {
    if (a >= bup * 0.999) a = bup * 0.5;
    cudaEventRecord(ev.e[0], st);
    TRY(filter<T>(P, B, deg, a, bup, a0, stt, st));
    cudaEventRecord(ev.e[1], st);
    TRY(orthonormalise<T>(P, B, s, stt, st));
    cudaEventRecord(ev.e[2], st);
    TRY(rayleigh_ritz<T>(P, B, s, stt, kPartialSweeps, theta, res, ev, st));
    ++stt.iters;
    nconv = 0;
    for (int j = 0; j < m; ++j)
      if (res[j] <= tol * bup) ++nconv;
    if (nconv == m) {
      for (int q = 0; q < 3; ++q) cudaEventRecord(ev.e[q], st);  // no filter / orthonormalisation time here
      TRY(rayleigh_ritz<T>(P, B, s, stt, kFullSweeps, theta, res, ev, st));
      nconv = 0;
      for (int j = 0; j < m; ++j)
        if (res[j] <= tol * bup) ++nconv;
      if (nconv == m) break;
    }
    a = theta[p - 1];
    a0 = std::min(theta[0], 0.0) - 1e-3 * bup;
    deg = choose_degree(theta, m, a, bup, range, sizeof(T) == 4 ? 60 : 250, sizeof(T) == 4 ? kAmp32 : 1e300);
  }
  *nconv_out = nconv;
  return RVGP_OK;
}

// The one-SM kernels of the FP32 stage by block width (the active width
// shrinks as eigenpairs are locked): Cholesky QR and Jacobi in one CTA when
// the width fits, block Jacobi above (RVGP_JACOBI_BLOCK=0: the scalar kernel).
void set_width_flags(Small& s, int w, int mode) {
  s.cholqr32 = (mode == 1 && w <= cholqr32_max_p()) ? 1 : 0;
  s.jac32 = (mode == 1 && w % 2 == 0 && w <= jacobi32_max_p()) ? 1 : 0;
  const char* e = getenv("RVGP_JACOBI_BLOCK");
  s.jacb = (mode == 1 && !s.jac32 && w >= 128 && jacobi_block_workspace(w) <= s.jac_bytes && !(e && e[0] == '0'))
               ? 1
               : 0;
}

// Va (N x pa) -= Vl (Vlᵀ Va), Vl the nl locked columns (ld ldl): one
// classical Gram-Schmidt pass against the locked vectors (tensor cores when
// the block products use them).  Tmp: N x pa scratch.
int project_out(const float* Vl, int ldl, int nl, float* Va, int pa, long long N, float* Tmp, Small& s,
                cudaStream_t st) {
  if (s.tc)
    TRY(tc_gram_f32_out64(Vl, ldl, Va, pa, N, nl, pa, s.G, pa, s.tc_err, s.tc_ws, s.tc_bytes, st));
  else
    TRY(gram_f32_out64(Vl, ldl, Va, pa, N, nl, pa, s.G, pa, 1.0, 0.0, s.gram_ws, s.gram_bytes, st));
  TRY(convert_f64_to_f32(s.G, pa, s.Bf, pa, nl, pa, st));
  if (s.tc) {
    TRY(tc_gemm_f32(Vl, ldl, N, nl, s.Bf, pa, pa, Tmp, pa, s.tc_err, s.tc_ws, s.tc_bytes, st));
    const long long n4 = N * pa / 4;
    rvgp::note_launch();
    sub_f32x4<<<(unsigned)std::min<long long>(8LL * num_sms(), ceil_div(n4, 256)), 256, 0, st>>>(Va, Tmp, n4);
    return check_launch("project_out");
  }
  return gemm_nn<float>(Vl, ldl, s.Bf, pa, N, nl, pa, Va, pa, -1.f, 1.f, st);
}

int copy_cols(const float* src, int lds, int c0, float* dst, int ldd, int d0, long long N, int ncols,
              cudaStream_t st) {
  if (ncols <= 0) return RVGP_OK;
  const long long g = N * (ncols / 4);
  rvgp::note_launch();
  copy_cols4<<<(unsigned)std::min<long long>(8LL * num_sms(), ceil_div(g, 256)), 256, 0, st>>>(src, lds, c0, dst, ldd,
                                                                                               d0, N, ncols);
  return check_launch("copy_cols");
}

// The FP32 stage with locking.  After each Rayleigh-Ritz step the leading
// active Ritz vectors whose residual is below a tenth of the tolerance (in
// multiples of 4, never beyond m) move to Vl and leave the iteration: the filter, the orthonormalisation,
// the Rayleigh-Ritz products and the Jacobi then run on the p - nl active
// columns, kept compact (ld = p - nl) so every kernel sees a plain block.
// After each filter the active block is projected against Vl twice
// (classical Gram-Schmidt twice: the filter amplifies the residual
// components along the locked directions most) before its Cholesky QR.  The
// filter degree still bounds the gain of the lowest Ritz value overall
// (locked or not), as without locking.  On return B.V is the N x p block
// [locked | active] (ld p), theta / res the matching values.
// lock at a tenth of the convergence tolerance (RVGP_EIG_LOCK_MARGIN overrides)
double lock_margin() {
  const char* e = getenv("RVGP_EIG_LOCK_MARGIN");
  return e ? atof(e) : 0.1;
}

int iterate_locked(const Problem& P, Block<float>& B, float* Vl, int ldl, Small& s, Stats& stt, double bup,
                   double tol, int max_iter, int first_deg, double range, std::vector<double>& theta,
                   std::vector<double>& res, int* nconv_out, cudaStream_t st) {
  const int m = P.m, p = P.p;
  const long long N = P.N;
  const char* le = getenv("RVGP_EIG_LOCK");
  const bool lock_on = !(le && le[0] == '0');
  int nl = 0;
  std::vector<double> th_l, res_l;
  Problem A = P;
  int nconv = 0;
  double a = bup * std::min(0.5, std::max(4.0 * p / (double)N, 0.01)), a0 = -1e-3 * bup;
  int deg = first_deg;
  PhaseEvents ev;
  constexpr int kPartialSweeps = 1, kFullSweeps = 60;
  for (int it = 0; it < max_iter; ++it) {
    const int pa = p - nl, ma = m - nl;
    A.p = pa;
    A.m = ma;
    set_width_flags(s, pa, 1);
    if (a >= bup * 0.999) a = bup * 0.5;
    cudaEventRecord(ev.e[0], st);
    TRY(filter<float>(A, B, deg, a, bup, a0, stt, st));
    cudaEventRecord(ev.e[1], st);
    for (int pass = 0; pass < 2 && nl > 0; ++pass) TRY(project_out(Vl, ldl, nl, B.V, pa, N, B.T1, s, st));
    TRY(orthonormalise<float>(A, B, s, stt, st));
    cudaEventRecord(ev.e[2], st);
    TRY(rayleigh_ritz<float>(A, B, s, stt, kPartialSweeps, theta, res, ev, st));
    ++stt.iters;
    nconv = 0;
    for (int j = 0; j < ma; ++j)
      if (res[j] <= tol * bup) ++nconv;
    if (nconv == ma) {
      for (int q = 0; q < 3; ++q) cudaEventRecord(ev.e[q], st);  // no filter / orthonormalisation time here
      TRY(rayleigh_ritz<float>(A, B, s, stt, kFullSweeps, theta, res, ev, st));
      nconv = 0;
      for (int j = 0; j < ma; ++j)
        if (res[j] <= tol * bup) ++nconv;
      if (nconv == ma) break;
    }
    if (lock_on) {
      // a locked vector is never polished again: lock only those whose
      // residual is well below the convergence tolerance
      int k = 0;
      const double lm = lock_margin();
      while (k < ma && res[k] <= lm * tol * bup) ++k;
      k = k / 4 * 4;
      if (k >= 8) {
        TRY(copy_cols(B.V, pa, 0, Vl, ldl, nl, N, k, st));
        TRY(copy_cols(B.V, pa, k, B.T1, pa - k, 0, N, pa - k, st));
        std::swap(B.V, B.T1);
        th_l.insert(th_l.end(), theta.begin(), theta.begin() + k);
        res_l.insert(res_l.end(), res.begin(), res.begin() + k);
        theta.erase(theta.begin(), theta.begin() + k);
        res.erase(res.begin(), res.begin() + k);
        nl += k;
        stt.locked = nl;
      }
    }
    const int pn = p - nl;
    const double lowest = nl > 0 ? std::min(th_l.front(), theta[0]) : theta[0];
    a = theta[pn - 1];
    a0 = std::min(lowest, 0.0) - 1e-3 * bup;
    std::vector<double> thd(theta);
    thd[0] = std::min(thd[0], lowest);
    deg = choose_degree(thd, m - nl, a, bup, range, 60, kAmp32);
  }
  if (nl > 0) {
    TRY(copy_cols(Vl, ldl, 0, B.T1, p, 0, N, nl, st));
    TRY(copy_cols(B.V, p - nl, 0, B.T1, p, nl, N, p - nl, st));
    std::swap(B.V, B.T1);
    th_l.insert(th_l.end(), theta.begin(), theta.end());
    res_l.insert(res_l.end(), res.begin(), res.end());
    theta.swap(th_l);
    res.swap(res_l);
  }
  set_width_flags(s, p, 1);
  nconv = 0;
  for (int j = 0; j < m; ++j)
    if (res[j] <= tol * bup) ++nconv;
  *nconv_out = nconv;
  return RVGP_OK;
}

struct Layout {
  Block<float> f;
  Block<double> d;
  Small s;
};

Layout carve(Workspace& ws, long long N, int p, int mode) {
  Layout L{};
  const size_t blk = (size_t)N * p;
  if (mode == 1) {
    L.f.V = ws.take<float>(blk);
    L.f.W = ws.take<float>(blk);
    L.f.T1 = ws.take<float>(blk);
    L.f.T2 = ws.take<float>(blk);
  }
  L.d.V = ws.take<double>(blk);
  L.d.W = ws.take<double>(blk);
  L.d.T1 = ws.take<double>(blk);
  L.d.T2 = ws.take<double>(blk);
  Small& s = L.s;
  const size_t pp = (size_t)p * p;
  s.G = ws.take<double>(pp);
  s.H = ws.take<double>(pp);
  s.Q = ws.take<double>(pp);
  s.Linv = ws.take<double>(pp);
  s.theta = ws.take<double>(p);
  s.res = ws.take<double>(p);
  s.norms64 = ws.take<double>(p);
  s.gersh = ws.take<double>(num_sms() * 2);
  s.resid_part = ws.take<double>((size_t)resid_chunks(N) * 2 * p);  // [vᵀw | vᵀv] partials, then the residual's
  s.info = ws.take<int>(4);
  s.colmap = ws.take<int>(p);
  s.Bf = ws.take<float>(pp);
  s.Bd = ws.take<double>(pp);
  s.nf = ws.take<float>(p);
  s.nd = ws.take<double>(p);
  s.Hf = ws.take<float>(pp);
  s.thf = ws.take<float>(p);
  s.L32 = ws.take<float>(pp);
  s.Mb32 = ws.take<float>((size_t)((p + 31) / 32) * 32 * 32);
  s.d32 = ws.take<float>(p);
  s.cholqr32 = 0;
  s.jac32 = 0;
  s.jacb = 0;
  s.jac32_bytes = jacobi32_workspace(p, kFp32Sweeps);
  s.jac32_ws = ws.take<char>(s.jac32_bytes);
  s.gram_bytes = std::max(gram_workspace<float>(N, p, p), gram_workspace<double>(N, p, p));
  // the locking projection's Grams are nl x (p - nl): their split counts grow
  // as nl shrinks, so size for every width the iteration can reach
  for (int w = 4; w < p; w += 4) s.gram_bytes = std::max(s.gram_bytes, gram_workspace<float>(N, w, p - w));
  s.gram_ws = ws.take<char>(s.gram_bytes);
  s.jac_bytes = jacobi_workspace<double>(p);
  s.jac_ws = ws.take<char>(s.jac_bytes);
  s.cn_bytes = std::max(col_norms_workspace<float>(N, p), col_norms_workspace<double>(N, p));
  s.cn_ws = ws.take<char>(s.cn_bytes);
  s.tc = 0;
  s.tc_err = ws.take<int>(1);
  s.tc_bytes = mode == 1 ? std::max(tc_gram_workspace(N, p, p), tc_gemm_workspace(p, p)) : 0;
  if (mode == 1)
    for (int w = 4; w < p; w += 4)
      s.tc_bytes = std::max(s.tc_bytes, std::max(tc_gram_workspace(N, w, p - w), tc_gemm_workspace(w, p - w)));
  s.tc_ws = ws.take<char>(s.tc_bytes);
  return L;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_eigsh_workspace(int n, int DB, int m, int p, int mode) {
  Workspace ws(nullptr, 0);
  carve(ws, (long long)n * DB, p, mode);
  return ws.used;
}

// Smallest m eigenpairs of the block-CSR matrix (n block rows, DB x DB blocks).
// vals64 is always required (Gershgorin bound, FP64 iterations); vals32 for
// mode 1.  p: block size (m < p <= N, p % 4 == 0).  mode: 0 plain FP64, 1 mixed.
// tol: FP64 residual tolerance relative to the Gershgorin bound; tol32 the
// FP32 stage's.  evals: m doubles ascending; evecs: N x m (ld_evecs) times
// `scale`.  stats (host, 16 ints, may be null): iterations, SpMM count, Jacobi
// sweeps, converged, FP64 refinement iterations, Cholesky rescues.
// Returns 0, or the number of unconverged eigenpairs (> 0).  Synchronises.
static int eigsh_impl(const int* indptr, const int* indices, const double* vals64, const float* vals32, int n,
                      int DB, int m, int p, int mode, double tol, double tol32, int max_iter,
                      unsigned long long seed, const int* perm, double* evals, double* evecs, int ld_evecs,
                      double scale, int* stats, void* workspace, size_t ws_bytes, void* stream) {
  const long long N = (long long)n * DB;
  RVGP_CHECK_ARG(indptr && indices && vals64 && evals && evecs, "rvgp_eigsh: null pointer");
  RVGP_CHECK_ARG(mode == 0 || (mode == 1 && vals32), "rvgp_eigsh: mode 1 needs FP32 values");
  RVGP_CHECK_ARG(m >= 1 && m < N - 1, "k must be less than ndim(A)-1, got k=%d", m);
  RVGP_CHECK_ARG(p > m && p <= N && p % 4 == 0 && p <= 2048, "rvgp_eigsh: block size p=%d invalid", p);
  RVGP_CHECK_ARG(DB >= 1 && DB <= 4, "rvgp_eigsh: block size %d unsupported", DB);
  size_t need = rvgp_eigsh_workspace(n, DB, m, p, mode);
  RVGP_CHECK_ARG(workspace && ws_bytes >= need, "rvgp_eigsh: workspace of %zu bytes needed", need);
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  Layout L = carve(ws, N, p, mode);
  Small& s = L.s;
  set_width_flags(s, p, mode);
  s.tc = (mode == 1 && s.tc_bytes > 0 && tc_enabled() && tc_supported(p, p)) ? 1 : 0;
  cudaMemsetAsync(s.tc_err, 0, sizeof(int), st);
  Problem P{n, DB, N, indptr, indices, vals64, vals32, m, p, SpmmPlan{}};
  Stats stt;
  // the product's plan (grouped and tiled forms, spmm.cu), in the workspace
  // beyond `need` when the caller sized it for one (rvgp_spmm_plan_bytes), on
  // request (RVGP_SPMM_PLAN=1): on GB300 both planned forms are slower than
  // the chunked variant (fewer resident warps, fewer gathers in flight), so
  // by default the tuner chooses among the plain variants only
  {
    const char* e = getenv("RVGP_SPMM_PLAN");
    int nnz = 0;
    if (e && e[0] == '1' && ws_bytes > need) {
      if (read_back(&nnz, indptr + n, sizeof(int), st) != cudaSuccess) return check_launch("rvgp_eigsh");
      const size_t pb = spmm_plan_bytes(n, DB, nnz);
      if (pb > 0 && ws.used + 256 + pb <= ws_bytes) {
        void* plan = ws.take<char>(pb);
        TRY(spmm_plan_build(n, DB, indptr, indices, nnz, plan, pb, st));
        P.plan = SpmmPlan{plan, pb, (long long)nnz};
      }
    }
  }

  // spectrum upper bound (Gershgorin)
  const int gb = std::min(num_sms() * 2, ceil_div(N, 256));
  rvgp::note_launch(); gershgorin_kernel<<<gb, 256, 0, st>>>(n, DB, indptr, vals64, s.gersh);
  std::vector<double> gp(gb);
  if (read_back(gp.data(), s.gersh, sizeof(double) * gb, st) != cudaSuccess) return check_launch("rvgp_eigsh");
  double bup = 0.0;
  for (double v : gp) bup = std::max(bup, v);
  bup = bup * (1.0 + 1e-12) + 1e-300;

  std::vector<double> theta, res;
  int nconv = 0;
  // degree of the first filter, from the random block (RVGP_EIG_FIRST_DEG overrides)
  const char* fd = getenv("RVGP_EIG_FIRST_DEG");
  const int first_deg = fd ? std::max(2, std::min(200, atoi(fd))) : 12;
  if (mode == 1) {
    rvgp::note_launch(); random_block<float><<<ceil_div(N * p, 256), 256, 0, st>>>(L.f.V, N, p, p, seed, perm, DB);
    // locked vectors live in the FP64 scratch block, unused until the refinement
    const int ldl = (m + 3) / 4 * 4;
    TRY(iterate_locked(P, L.f, reinterpret_cast<float*>(L.d.T2), ldl, s, stt, bup, tol32, max_iter, first_deg, 1e4,
                       theta, res, &nconv, st));
    // FP64 refinement from the FP32 subspace
    TRY(convert_f32_to_f64(L.f.V, p, L.d.V, p, N, p, st));
    nconv = 0;
    for (int j = 0; j < m; ++j)
      if (res[j] <= tol * bup) ++nconv;
    if (nconv < m) {
      std::sort(theta.begin(), theta.end());  // locked and active values: the degree rule wants them ordered
      const int before = stt.iters;
      TRY(iterate<double>(P, L.d, s, stt, bup, tol, max_iter, 4, 1e10, theta, res, true, &nconv, st));
      stt.refine_iters = stt.iters - before;
    }
  } else {
    rvgp::note_launch(); random_block<double><<<ceil_div(N * p, 256), 256, 0, st>>>(L.d.V, N, p, p, seed, perm, DB);
    TRY(iterate<double>(P, L.d, s, stt, bup, tol, max_iter, first_deg, 1e10, theta, res, false, &nconv, st));
  }
  stt.conv = nconv;
  // the m lowest Ritz values ascending (Rayleigh quotients can swap nearly
  // equal neighbours), ties by block column; their vectors by a column map
  std::vector<int> order(p);
  for (int j = 0; j < p; ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return theta[a] < theta[b]; });
  std::vector<double> ev(m);
  for (int j = 0; j < m; ++j) ev[j] = theta[order[j]];
  cudaMemcpyAsync(evals, ev.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s.colmap, order.data(), sizeof(int) * m, cudaMemcpyHostToDevice, st);
  rvgp::note_launch(); write_output<double><<<ceil_div(N * m, 256), 256, 0, st>>>(L.d.V, p, N, m, scale, evecs, ld_evecs, perm, DB, s.colmap);
  // the host vectors must outlive the copies from pageable memory
  if (cudaStreamSynchronize(st) != cudaSuccess) return check_launch("rvgp_eigsh");
  if (stats) {
    stats[0] = stt.iters;
    stats[1] = stt.spmm;
    stats[2] = stt.sweeps;
    stats[3] = stt.conv;
    stats[4] = stt.refine_iters;
    stats[5] = stt.chol_rescues;
    stats[6] = s.tc;
    stats[7] = P.plan.plan != nullptr;
    stats[12] = stt.locked;
    for (int q = 0; q < 4; ++q) stats[8 + q] = (int)(stt.ms[q] * 1000.f);  // microseconds per phase
  }
  RVGP_LAUNCH_CHECK("rvgp_eigsh");
  int tc_fail = 0;
  if (read_back(&tc_fail, s.tc_err, sizeof(int), st) != cudaSuccess) return check_launch("rvgp_eigsh");
  if (tc_fail) {
    set_error("eigensolver: a tensor-core pipeline wait timed out");
    return RVGP_ELAUNCH;
  }
  if (nconv < m) {
    set_error("eigensolver: %d of %d eigenpairs did not converge in %d iterations", m - nconv, m, max_iter);
    return m - nconv;
  }
  return RVGP_OK;
}

RVGP_API int rvgp_eigsh(const int* indptr, const int* indices, const double* vals64, const float* vals32, int n,
                        int DB, int m, int p, int mode, double tol, double tol32, int max_iter,
                        unsigned long long seed, double* evals, double* evecs, int ld_evecs, double scale, int* stats,
                        void* workspace, size_t ws_bytes, void* stream) {
  return eigsh_impl(indptr, indices, vals64, vals32, n, DB, m, p, mode, tol, tol32, max_iter, seed, nullptr, evals,
                    evecs, ld_evecs, scale, stats, workspace, ws_bytes, stream);
}

// The same solve on a renumbered matrix: block row r of (indptr, indices,
// vals) is block row perm[r] of the caller's matrix, columns renumbered
// alike (rvgp_permute_csr).  The start block is the caller-order one,
// permuted, and evecs rows come back in the caller's order, so the result
// equals rvgp_eigsh's on the original matrix up to summation order.
RVGP_API int rvgp_eigsh_ordered(const int* indptr, const int* indices, const double* vals64, const float* vals32,
                                int n, int DB, int m, int p, int mode, double tol, double tol32, int max_iter,
                                unsigned long long seed, const int* perm, double* evals, double* evecs, int ld_evecs,
                                double scale, int* stats, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(perm, "rvgp_eigsh_ordered: null permutation");
  return eigsh_impl(indptr, indices, vals64, vals32, n, DB, m, p, mode, tol, tol32, max_iter, seed, perm, evals,
                    evecs, ld_evecs, scale, stats, workspace, ws_bytes, stream);
}
