// Dense linear algebra kernels (see linalg.cuh).
#include "linalg.cuh"
#include "gridsync.cuh"
#include <math.h>
#include <limits.h>
#include <vector>
#include <mutex>
#include <atomic>
#include <map>
#include <algorithm>

namespace rvgp {
namespace {

constexpr int TB = 64;   // output tile edge
constexpr int BK = 16;   // reduction slab

// ------------------------------------------------------------------ C = Aᵀ B (split over N)
template <typename T>
__global__ void __launch_bounds__(256) gram_partial(const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb,
                                                    long long N, int p, int q, long long chunk, T* __restrict__ part) {
  __shared__ T As[BK][TB];
  __shared__ T Bs[BK][TB];
  const int i0 = blockIdx.x * TB, j0 = blockIdx.y * TB;
  const long long n0 = blockIdx.z * chunk;
  const long long n1 = min(N, n0 + chunk);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  for (long long nb = n0; nb < n1; nb += BK) {
    for (int e = threadIdx.x; e < BK * TB; e += 256) {
      const int r = e / TB, c = e % TB;
      const long long n = nb + r;
      As[r][c] = (n < n1 && i0 + c < p) ? A[n * lda + i0 + c] : T(0);
      Bs[r][c] = (n < n1 && j0 + c < q) ? B[n * ldb + j0 + c] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < BK; ++r) {
      T a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = As[r][ty * 4 + u];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = Bs[r][tx * 4 + v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = i0 + ty * 4 + u, j = j0 + tx * 4 + v;
      if (i < p && j < q) part[((size_t)blockIdx.z * p + i) * q + j] = acc[u][v];
    }
}

template <typename T>
__global__ void reduce_splits(const T* __restrict__ part, int splits, int p, int q, T* __restrict__ C, int ldc,
                              T alpha, T beta) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)p * q) return;
  const int i = (int)(e / q), j = (int)(e % q);
  T s = T(0);
  for (int t = 0; t < splits; ++t) s += part[((size_t)t * p + i) * q + j];
  T* c = C + (size_t)i * ldc + j;
  *c = beta == T(0) ? alpha * s : alpha * s + beta * (*c);
}

__global__ void reduce_splits_f32_to_f64(const float* __restrict__ part, int splits, int p, int q,
                                         double* __restrict__ C, int ldc, double alpha, double beta) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)p * q) return;
  const int i = (int)(e / q), j = (int)(e % q);
  // groups of eight splits are added in FP32 (at most 7 roundings of partials
  // of similar size, well below their own FP32 accumulation error), the
  // group sums in FP64 in a fixed order: few FP64 operations, 8 loads in flight
  const size_t stride = (size_t)p * q;
  const float* src = part + (size_t)i * q + j;
  double s = 0.0;
  int t = 0;
  for (; t + 8 <= splits; t += 8) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldg(src + (size_t)(t + u) * stride);
    s += (double)(((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7])));
  }
  for (; t < splits; ++t) s += (double)__ldg(src + (size_t)t * stride);
  double* c = C + (size_t)i * ldc + j;
  *c = beta == 0.0 ? alpha * s : alpha * s + beta * (*c);
}

}  // namespace

int reduce_f32_splits_to_f64(const float* part, int splits, int p, int q, double* C, int ldc, cudaStream_t st) {
  rvgp::note_launch();
  reduce_splits_f32_to_f64<<<ceil_div((long long)p * q, 256), 256, 0, st>>>(part, splits, p, q, C, ldc, 1.0, 0.0);
  return check_launch("reduce_f32_splits_to_f64");
}

namespace {

template <typename T>
int gram_splits(long long N, int p, int q) {
  const int tiles = ceil_div(p, TB) * ceil_div(q, TB);
  int s = ceil_div(4 * num_sms(), tiles);
  s = (int)std::min<long long>(s, std::max<long long>(1, N / 512));
  return std::max(1, std::min(s, 1024));
}

// ------------------------------------------------------------------ C = A B
template <typename T>
__global__ void __launch_bounds__(256) gemm_nn_kernel(const T* __restrict__ A, int lda, const T* __restrict__ B,
                                                      int ldb, long long N, int p, int q, T* __restrict__ C, int ldc,
                                                      T alpha, T beta) {
  __shared__ T As[TB][BK + 1];
  __shared__ T Bs[BK][TB];
  const long long r0 = (long long)blockIdx.x * TB;
  const int j0 = blockIdx.y * TB;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  for (int k0 = 0; k0 < p; k0 += BK) {
    for (int e = threadIdx.x; e < TB * BK; e += 256) {
      const int r = e / BK, c = e % BK;
      As[r][c] = (r0 + r < N && k0 + c < p) ? A[(r0 + r) * lda + k0 + c] : T(0);
      const int rb = e / TB, cb = e % TB;
      Bs[rb][cb] = (k0 + rb < p && j0 + cb < q) ? B[(size_t)(k0 + rb) * ldb + j0 + cb] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = As[ty * 4 + u][kk];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = Bs[kk][tx * 4 + v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const long long r = r0 + ty * 4 + u;
      const int j = j0 + tx * 4 + v;
      if (r < N && j < q) {
        T* c = C + r * ldc + j;
        *c = beta == T(0) ? alpha * acc[u][v] : alpha * acc[u][v] + beta * (*c);
      }
    }
}

// ------------------------------------------------------------------ Cholesky (one CTA)
template <typename T>
__global__ void __launch_bounds__(1024) chol_kernel(T* __restrict__ A, int lda, int p, int* __restrict__ info) {
  __shared__ int bad;
  if (threadIdx.x == 0) {
    bad = 0;
    *info = 0;
  }
  for (int j = 0; j < p; ++j) {
    __syncthreads();
    if (threadIdx.x == 0) {
      T d = A[(size_t)j * lda + j];
      if (!(d > T(0))) {
        bad = j + 1;
        *info = j + 1;
      } else {
        A[(size_t)j * lda + j] = sqrt(d);
      }
    }
    __syncthreads();
    if (bad) return;
    const T djj = A[(size_t)j * lda + j];
    for (int i = j + 1 + threadIdx.x; i < p; i += blockDim.x) A[(size_t)i * lda + j] /= djj;
    __syncthreads();
    const int m = p - j - 1;
    for (long long e = threadIdx.x; e < (long long)m * m; e += blockDim.x) {
      const int ii = (int)(e / m), kk = (int)(e % m);
      if (kk <= ii) {
        const int i = j + 1 + ii, k = j + 1 + kk;
        A[(size_t)i * lda + k] -= A[(size_t)i * lda + j] * A[(size_t)k * lda + j];
      }
    }
  }
}

// ------------------------------------------------------------------ blocked Cholesky (many CTAs)
constexpr int NB = 32;
// largest shared-memory footprint of the one-CTA Cholesky (p = 160 in FP64)
constexpr size_t kSmallCholSmem = 8 * (160 * 161 + 160);

// Factor the diagonal block [k0, k0+nb) in shared memory.  On GB300 a warp-wide
// FP64 instruction occupies its SM sub-partition's FP64 pipe for tens of
// cycles, so the work per pivot is spread over four warps (one per
// sub-partition) and the only serial FP64 chain is thread 0's pivot
// (short-chain 1/sqrt).  Pivot j: thread 0 forms 1/sqrt(d_j) and L_jj; after
// one barrier every thread scales column j-1 (read for the last time by the
// previous update) and applies the rank-1 update with the unscaled column j
// times 1/d_j, so each pivot costs two barriers.
template <typename T>
__global__ void __launch_bounds__(128) potrf_diag(T* __restrict__ A, int lda, int k0, int nb, int* __restrict__ info) {
  __shared__ T L[NB][NB + 1];
  __shared__ T sinv[NB];
  __shared__ int bad;
  if (*info) return;  // an earlier block already failed
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, c = e % nb;
    if (c <= i) L[i][c] = A[(size_t)(k0 + i) * lda + k0 + c];
  }
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (threadIdx.x == 0) {
      const T d = L[j][j];
      if (!(d > T(0))) {
        bad = 1;
        atomicCAS(info, 0, k0 + j + 1);
      } else {
        const T inv = rsqrt_nr(d);
        sinv[j] = inv;
        L[j][j] = d * inv;
      }
    }
    __syncthreads();
    if (bad) return;
    if (j > 0)
      for (int i = j + threadIdx.x; i < nb; i += blockDim.x) L[i][j - 1] *= sinv[j - 1];
    const T inv2 = sinv[j] * sinv[j];
    const int m = nb - j - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int ii = e / m, kk = e % m;
      if (kk <= ii) L[j + 1 + ii][j + 1 + kk] -= L[j + 1 + ii][j] * (L[j + 1 + kk][j] * inv2);
    }
    __syncthreads();
  }
  // column nb-1 has no rows below its pivot, so every column is final here
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, c = e % nb;
    if (c <= i) A[(size_t)(k0 + i) * lda + k0 + c] = L[i][c];
  }
}

// Whole-matrix Cholesky in one CTA with the lower triangle in shared memory
// (row stride p + 1), for p small enough to fit: one launch instead of three
// per 32-column block.  Column j: warp 0 forms 1/sqrt(d_j), L_jj and the
// scaled column (kept also in `col`); after a barrier every warp applies the
// rank-1 update to its rows of the trailing lower triangle; a second barrier
// ends the column.
template <typename T>
__global__ void __launch_bounds__(512) potrf_small(T* __restrict__ A, int lda, int p, int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char chol_smem[];
  T* L = reinterpret_cast<T*>(chol_smem);
  T* col = L + (size_t)p * (p + 1);
  __shared__ int bad;
  const int ld = p + 1;
  for (int i = threadIdx.x >> 5; i < p; i += blockDim.x >> 5)
    for (int c = threadIdx.x & 31; c <= i; c += 32) L[i * ld + c] = A[(size_t)i * lda + c];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = 0; j < p; ++j) {
    if (w == 0) {
      const T d = L[j * ld + j];
      if (!(d > T(0))) {
        if (lane == 0) {
          bad = 1;
          atomicCAS(info, 0, j + 1);
        }
      } else {
        const T r = rsqrt_nr(d);
        if (lane == 0) L[j * ld + j] = d * r;
        for (int i = j + 1 + lane; i < p; i += 32) {
          const T v = L[i * ld + j] * r;
          L[i * ld + j] = v;
          col[i] = v;
        }
      }
    }
    __syncthreads();
    if (bad) return;  // uniform: read after the barrier
    for (int i = j + 1 + w; i < p; i += nw) {
      const T ci = col[i];
      for (int k = j + 1 + lane; k <= i; k += 32) L[i * ld + k] -= ci * col[k];
    }
    __syncthreads();
  }
  for (int i = threadIdx.x >> 5; i < p; i += blockDim.x >> 5)
    for (int c = threadIdx.x & 31; c <= i; c += 32) A[(size_t)i * lda + c] = L[i * ld + c];
}

template <typename T>
size_t potrf_small_smem(int p) {
  return sizeof(T) * ((size_t)p * (p + 1) + p);
}

// panel: rows [k0+nb, p) of columns [k0, k0+nb) <- A L_kkᵀ⁻¹, one row per
// thread with the row in registers and the pivots' reciprocals in shared memory
template <typename T>
__global__ void __launch_bounds__(64) trsm_panel(T* __restrict__ A, int lda, int k0, int nb, int p,
                                                 const int* __restrict__ info) {
  __shared__ T L[NB][NB + 1];
  __shared__ T inv[NB];
  if (*info) return;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) L[e / nb][e % nb] = A[(size_t)(k0 + e / nb) * lda + k0 + e % nb];
  __syncthreads();
  for (int c = threadIdx.x; c < nb; c += blockDim.x) inv[c] = rcp_nr(L[c][c]);
  __syncthreads();
  const int r = k0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= p) return;
  T x[NB];
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    if (c < nb) {
      // four independent partial sums keep the dependent FP64 chain short
      T v0 = A[(size_t)r * lda + k0 + c], v1 = T(0), v2 = T(0), v3 = T(0);
#pragma unroll
      for (int t = 0; t < c; t += 4) {
        v0 -= x[t] * L[c][t];
        if (t + 1 < c) v1 -= x[t + 1] * L[c][t + 1];
        if (t + 2 < c) v2 -= x[t + 2] * L[c][t + 2];
        if (t + 3 < c) v3 -= x[t + 3] * L[c][t + 3];
      }
      x[c] = ((v0 + v1) + (v2 + v3)) * inv[c];
    }
  }
#pragma unroll
  for (int c = 0; c < NB; ++c)
    if (c < nb) A[(size_t)r * lda + k0 + c] = x[c];
}

// trailing update of the lower part: A_ij -= A_ik A_jkᵀ for blocks (i, j), j <= i, both > k
template <typename T>
__global__ void __launch_bounds__(256) syrk_update(T* __restrict__ A, int lda, int k0, int nb, int p,
                                                   const int* __restrict__ info) {
  __shared__ T Ai[NB][NB + 1], Aj[NB][NB + 1];
  if (*info) return;
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj > bi) return;
  const int r0 = k0 + nb + bi * NB, c0 = k0 + nb + bj * NB;
  for (int e = threadIdx.x; e < NB * nb; e += blockDim.x) {
    const int rr = e / nb, cc = e % nb;
    Ai[rr][cc] = r0 + rr < p ? A[(size_t)(r0 + rr) * lda + k0 + cc] : T(0);
    Aj[rr][cc] = c0 + rr < p ? A[(size_t)(c0 + rr) * lda + k0 + cc] : T(0);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
    const int rr = e / NB, cc = e % NB;
    const int i = r0 + rr, j = c0 + cc;
    if (i >= p || j >= p || j > i) continue;
    T s = T(0);
    for (int t = 0; t < nb; ++t) s += Ai[rr][t] * Aj[cc][t];
    A[(size_t)i * lda + j] -= s;
  }
}

// ------------------------------------------------------------------ triangular inverse (warp per column)
// Column j of L⁻¹ by column-oriented forward substitution: lane l owns the rows
// k ≡ l (mod 32) of the running right-hand side y (shared memory) and their
// reciprocal pivots.  Step i: the owner of row i forms x_i = y_i / L_ii, one
// shuffle broadcasts it, every lane updates its own rows y_k -= L_ki x_i.  No
// lane reads another lane's rows, so the dependent chain per step is a
// multiply, a shuffle and one multiply-add.
template <typename T>
__global__ void trinv_kernel(const T* __restrict__ L, int ldl, int p, T* __restrict__ X, int ldx, int warps) {
  extern __shared__ unsigned char smem_raw[];
  T* y = reinterpret_cast<T*>(smem_raw) + (size_t)(threadIdx.x >> 5) * 2 * p;
  T* rinv = y + p;
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * warps + (threadIdx.x >> 5);
  if (j >= p) return;
  for (int i = lane; i < j; i += 32) X[(size_t)i * ldx + j] = T(0);
  for (int k = j + ((lane - j) & 31); k < p; k += 32) {
    y[k] = k == j ? T(1) : T(0);
    rinv[k] = rcp_nr(L[(size_t)k * ldl + k]);
  }
  for (int i = j; i < p; ++i) {
    T xi = T(0);
    if (lane == (i & 31)) {
      xi = y[i] * rinv[i];
      X[(size_t)i * ldx + j] = xi;
    }
    xi = __shfl_sync(0xffffffffu, xi, i & 31);
    for (int k = i + 1 + ((lane - i - 1) & 31); k < p; k += 32) y[k] -= L[(size_t)k * ldl + i] * xi;
  }
}

// The same columns with the loads off the dependent chain: at step i the
// column i of L below the pivot (this lane's rows) is already in shared
// memory, copied by cp.async two steps earlier into a ring of three column
// buffers, so a step costs the pivot's multiply, one shuffle and the updates,
// not an L2 round trip.  The columns are read from a transposed copy (the
// strictly-lower part of L written into the strictly-upper part of the
// output first, `lower_to_upper`), so a step's copies are contiguous: a
// column of row-major L has one element per row, and at p = 800 its lines
// no longer stay in L1.  The output's upper part is zeroed afterwards.
// Every lane copies and reads only its own rows, so its own
// cp.async.wait_group orders the ring; the arithmetic and its order are the
// plain kernel's (the same bits).  One warp per CTA, so the heavy leading
// columns land on different SMs.
template <typename T>
__device__ __forceinline__ void cp_async_el(T* smem, const T* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(sizeof(T)) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// U[i][k] = L[k][i] for k > i (32 x 32 tiles through shared memory)
template <typename T>
__global__ void __launch_bounds__(256) lower_to_upper(const T* __restrict__ L, int ldl, int p, T* __restrict__ U,
                                                      int ldu) {
  __shared__ T tile[32][33];
  const int kb = blockIdx.y, ib = blockIdx.x;
  if (kb < ib) return;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += 8) {
    const int k = kb * 32 + r, i = ib * 32 + tx;
    tile[r][tx] = (k < p && i < p && k > i) ? L[(size_t)k * ldl + i] : T(0);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = ib * 32 + r, k = kb * 32 + tx;
    if (k < p && i < p && k > i) U[(size_t)i * ldu + k] = tile[tx][r];
  }
}

template <typename T>
__global__ void zero_strict_upper(T* __restrict__ X, int ldx, int p) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)p * p) return;
  const int i = (int)(e / p), j = (int)(e % p);
  if (j > i) X[(size_t)i * ldx + j] = T(0);
}

// LT: the transposed strictly-lower part of L (row c holds column c below
// its pivot), in the strictly-upper part of X itself: the kernel writes only
// the lower part of X, so the two never meet.
template <typename T>
__global__ void __launch_bounds__(32) trinv_pf_kernel(const T* __restrict__ L, int ldl, const T* LT, int ldt, int p,
                                                      T* X, int ldx) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* y = reinterpret_cast<T*>(smem_raw);
  T* rinv = y + p;
  T* ring = rinv + p;  // 3 x p
  const int lane = threadIdx.x;
  const int j = blockIdx.x;
  for (int k = j + ((lane - j) & 31); k < p; k += 32) {
    y[k] = k == j ? T(1) : T(0);
    rinv[k] = rcp_nr(L[(size_t)k * ldl + k]);
  }
  auto fetch = [&](int c) {  // column c below its pivot, this lane's rows, into slot c % 3
    if (c < p) {
      T* dst = ring + (size_t)(c % 3) * p;
      const T* src = LT + (size_t)c * ldt;
      for (int k = c + 1 + ((lane - c - 1) & 31); k < p; k += 32) cp_async_el(dst + k, src + k);
    }
    cp_async_commit();  // possibly empty: one group per column keeps the count
  };
  fetch(j);
  fetch(j + 1);
  for (int i = j; i < p; ++i) {
    fetch(i + 2);
    cp_async_wait<2>();  // column i (this lane's part) has landed
    T xi = T(0);
    if (lane == (i & 31)) {
      xi = y[i] * rinv[i];
      X[(size_t)i * ldx + j] = xi;
    }
    xi = __shfl_sync(0xffffffffu, xi, i & 31);
    const T* ci = ring + (size_t)(i % 3) * p;
    for (int k = i + 1 + ((lane - i - 1) & 31); k < p; k += 32) y[k] -= ci[k] * xi;
  }
  cp_async_wait<0>();
}

// ------------------------------------------------------------------ Jacobi eigensolver
template <typename T>
struct Eps;
template <> struct Eps<float> { static constexpr double v = 5.96e-8; };
template <> struct Eps<double> { static constexpr double v = 1.12e-16; };

// (c1, c2, P, Q) of index i for this round: new basis e'_i = c1 e_P + c2 e_Q
template <typename T>
__device__ __forceinline__ void rot_of(const T* __restrict__ H, int p, const int* __restrict__ partner, int i, T& c1,
                                       T& c2, int& P, int& Q) {
  const int m = partner[i];
  if (m == i || m >= p) {
    c1 = T(1);
    c2 = T(0);
    P = Q = i;
    return;
  }
  P = min(i, m);
  Q = max(i, m);
  const T a = H[(size_t)P * p + P], b = H[(size_t)Q * p + Q], c = H[(size_t)P * p + Q];
  T cs = T(1), sn = T(0);
  const double tiny = Eps<T>::v * 1e-3;
  if (c != T(0) && (double)c * (double)c > tiny * tiny * fabs((double)a) * fabs((double)b)) {
    // Rutishauser's stable rotation, with reciprocals / square roots from
    // short-chain Newton refinements: t = sign(θ)/(|θ| + sqrt(θ² + 1)).
    const T theta = (b - a) * rcp_nr(T(2) * c);
    T t;
    if (fabs((double)theta) > 1e15) {
      t = T(0.5) * rcp_nr(theta);  // sqrt(θ² + 1) = |θ| to working precision
    } else {
      const T q = fma(theta, theta, T(1));
      const T root = q * rsqrt_nr(q);
      t = (theta >= T(0) ? T(1) : T(-1)) * rcp_nr(fabs(theta) + root);
    }
    cs = rsqrt_nr(fma(t, t, T(1)));
    sn = t * cs;
  }
  if (i == P) {
    c1 = cs;
    c2 = -sn;
  } else {
    c1 = sn;
    c2 = cs;
  }
}

// per-index rotation coefficients of this round: coef[i] = (c1, c2), pq[i] = (P, Q)
template <typename T>
__global__ void jacobi_params(const T* __restrict__ H, int p, const int* __restrict__ partner, T* __restrict__ coef,
                              int2* __restrict__ pq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p) return;
  T c1, c2;
  int P, Q;
  rot_of(H, p, partner, i, c1, c2, P, Q);
  coef[2 * i] = c1;
  coef[2 * i + 1] = c2;
  pq[i] = make_int2(P, Q);
}

template <typename T>
__global__ void jacobi_round(const T* __restrict__ H, T* __restrict__ Hn, const T* __restrict__ V,
                             T* __restrict__ Vn, int p, const int* __restrict__ partner, const T* __restrict__ coef,
                             const int2* __restrict__ pq) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long pp = (long long)p * p;
  if (e < pp) {
    const int i = (int)(e / p), j = (int)(e % p);
    const T ci1 = coef[2 * i], ci2 = coef[2 * i + 1], cj1 = coef[2 * j], cj2 = coef[2 * j + 1];
    const int2 a = pq[i], b = pq[j];
    T v;
    if (i != j && partner[i] == j) {
      v = T(0);
    } else {
      v = ci1 * (cj1 * H[(size_t)a.x * p + b.x] + cj2 * H[(size_t)a.x * p + b.y]);
      if (ci2 != T(0)) v += ci2 * (cj1 * H[(size_t)a.y * p + b.x] + cj2 * H[(size_t)a.y * p + b.y]);
    }
    Hn[e] = v;
  } else if (e < 2 * pp) {
    const long long f = e - pp;
    const int r = (int)(f / p), i = (int)(f % p);
    const T c1 = coef[2 * i], c2 = coef[2 * i + 1];
    const int2 a = pq[i];
    T v = c1 * V[(size_t)r * p + a.x];
    if (c2 != T(0)) v += c2 * V[(size_t)r * p + a.y];
    Vn[f] = v;
  }
}

// H <- (H + Hᵀ)/2: rotations leave the antisymmetric part's norm unchanged, so
// rounding asymmetry must go before the off-norm test.
template <typename T>
__global__ void symmetrise(T* __restrict__ H, int p) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)p * p) return;
  const int i = (int)(e / p), j = (int)(e % p);
  if (j <= i) return;
  const T v = (H[(size_t)i * p + j] + H[(size_t)j * p + i]) * T(0.5);
  H[(size_t)i * p + j] = v;
  H[(size_t)j * p + i] = v;
}

template <typename T>
__global__ void set_identity(T* __restrict__ V, int p) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e < (long long)p * p) V[e] = (e / p == e % p) ? T(1) : T(0);
}

// off-diagonal and total squared Frobenius norms (one CTA, fixed order)
template <typename T>
__global__ void __launch_bounds__(1024) offnorm_kernel(const T* __restrict__ H, int p, double* __restrict__ out) {
  __shared__ double so[1024], st[1024];
  double off = 0.0, tot = 0.0;
  for (long long e = threadIdx.x; e < (long long)p * p; e += blockDim.x) {
    double v = (double)H[e];
    tot += v * v;
    if (e / p != e % p) off += v * v;
  }
  so[threadIdx.x] = off;
  st[threadIdx.x] = tot;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      so[threadIdx.x] += so[threadIdx.x + s];
      st[threadIdx.x] += st[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = so[0];
    out[1] = st[0];
  }
}

// sort the diagonal ascending (ties by index) and permute the columns of V (one CTA)
template <typename T>
__device__ void sort_eig_block(const T* __restrict__ H, const T* __restrict__ V, int p, T* __restrict__ w,
                               T* __restrict__ Vout, unsigned char* smem, int ld);

template <typename T>
__global__ void __launch_bounds__(1024) sort_eig(const T* __restrict__ H, const T* __restrict__ V, int p,
                                                 T* __restrict__ w, T* __restrict__ Vout) {
  extern __shared__ unsigned char smem[];
  sort_eig_block<T>(H, V, p, w, Vout, smem, p);
}

template <typename T>
__device__ void sort_eig_block(const T* __restrict__ H, const T* __restrict__ V, int p, T* __restrict__ w,
                               T* __restrict__ Vout, unsigned char* smem, int ld) {
  T* key = reinterpret_cast<T*>(smem);
  int* idx = reinterpret_cast<int*>(key + 2048);
  int P2 = 1;
  while (P2 < p) P2 <<= 1;
  for (int t = threadIdx.x; t < P2; t += blockDim.x) {
    key[t] = t < p ? H[(size_t)t * ld + t] : T(0);
    idx[t] = t < p ? t : INT_MAX;
  }
  __syncthreads();
  auto less = [&](int a, int b) {
    if (idx[a] == INT_MAX) return false;
    if (idx[b] == INT_MAX) return true;
    return key[a] < key[b] || (key[a] == key[b] && idx[a] < idx[b]);
  };
  for (int size = 2; size <= P2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < P2; t += blockDim.x) {
        const int o = t ^ stride;
        if (o > t) {
          const bool up = (t & size) == 0;
          if (up ? less(o, t) : less(t, o)) {
            T k = key[t];
            key[t] = key[o];
            key[o] = k;
            int x = idx[t];
            idx[t] = idx[o];
            idx[o] = x;
          }
        }
      }
      __syncthreads();
    }
  for (int t = threadIdx.x; t < p; t += blockDim.x) w[t] = key[t];
  for (long long e = threadIdx.x; e < (long long)p * p; e += blockDim.x) {
    const int r = (int)(e / p), c = (int)(e % p);
    Vout[e] = V[(size_t)r * ld + idx[c]];
  }
}

// The whole Jacobi eigensolve in one cooperative launch: symmetrise, then up to
// max_sweeps sweeps of p-1 rounds (rotation parameters, barrier, rotate H and
// V, barrier), with the off-norm test of each sweep reduced in a fixed order so
// every CTA takes the same decision; CTA 0 finally sorts.  Any barrier timeout
// makes every CTA leave early with *err set.
template <typename T>
__global__ void __launch_bounds__(256) jacobi_persistent(T* H, T* Hb, T* Va, T* Vb, int p,
                                                         const int* __restrict__ partner, int rounds, double* part,
                                                         int max_sweeps, double tol2, unsigned int* bar, int* err,
                                                         int* sweeps_out, T* w, T* Vout) {
  extern __shared__ unsigned char smem[];
  __shared__ double red[2][256];
  __shared__ double s_off, s_tot;
  T* coef = reinterpret_cast<T*>(smem);                      // 2p rotation coefficients
  int2* pq = reinterpret_cast<int2*>(coef + 2 * (size_t)p);  // p index pairs
  const unsigned G = gridDim.x;
  const long long pp = (long long)p * p;
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x, gsz = (long long)G * blockDim.x;
  for (long long e = gtid; e < pp; e += gsz) {
    const int i = (int)(e / p), j = (int)(e % p);
    if (j > i) {
      const T v = (H[(size_t)i * p + j] + H[(size_t)j * p + i]) * T(0.5);
      H[(size_t)i * p + j] = v;
      H[(size_t)j * p + i] = v;
    }
    Va[e] = i == j ? T(1) : T(0);
  }
  if (!grid_barrier(bar, err, G)) return;
  T *h0 = H, *h1 = Hb, *v0 = Va, *v1 = Vb;
  int used = 0;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (long long e = gtid; e < pp; e += gsz) {
      const double v = (double)h0[e];
      tot += v * v;
      if (e / p != e % p) off += v * v;
    }
    red[0][threadIdx.x] = off;
    red[1][threadIdx.x] = tot;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        red[0][threadIdx.x] += red[0][threadIdx.x + s];
        red[1][threadIdx.x] += red[1][threadIdx.x + s];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      part[2 * blockIdx.x] = red[0][0];
      part[2 * blockIdx.x + 1] = red[1][0];
    }
    if (!grid_barrier(bar, err, G)) return;
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (unsigned q = 0; q < G; ++q) {
        a += part[2 * q];
        b += part[2 * q + 1];
      }
      s_off = a;
      s_tot = b;
    }
    __syncthreads();
    if (!(s_off > tol2 * s_tot)) break;
    for (int r = 0; r < rounds; ++r) {
      const int* prt = partner + (size_t)r * p;
      // every CTA derives the round's p rotation coefficients itself (shared
      // memory): one grid barrier per round instead of two
      for (int i = threadIdx.x; i < p; i += blockDim.x) {
        T c1, c2;
        int P, Q;
        rot_of(h0, p, prt, i, c1, c2, P, Q);
        coef[2 * i] = c1;
        coef[2 * i + 1] = c2;
        pq[i] = make_int2(P, Q);
      }
      __syncthreads();
      for (long long e = gtid; e < 2 * pp; e += gsz) {
        if (e < pp) {
          const int i = (int)(e / p), j = (int)(e % p);
          const T ci1 = coef[2 * i], ci2 = coef[2 * i + 1], cj1 = coef[2 * j], cj2 = coef[2 * j + 1];
          const int2 a = pq[i], b = pq[j];
          T v;
          if (i != j && prt[i] == j) {
            v = T(0);
          } else {
            v = ci1 * (cj1 * h0[(size_t)a.x * p + b.x] + cj2 * h0[(size_t)a.x * p + b.y]);
            if (ci2 != T(0)) v += ci2 * (cj1 * h0[(size_t)a.y * p + b.x] + cj2 * h0[(size_t)a.y * p + b.y]);
          }
          h1[e] = v;
        } else {
          const long long f = e - pp;
          const int rr = (int)(f / p), i = (int)(f % p);
          const T c1 = coef[2 * i], c2 = coef[2 * i + 1];
          const int2 a = pq[i];
          T v = c1 * v0[(size_t)rr * p + a.x];
          if (c2 != T(0)) v += c2 * v0[(size_t)rr * p + a.y];
          v1[f] = v;
        }
      }
      if (!grid_barrier(bar, err, G)) return;
      T* t = h0;
      h0 = h1;
      h1 = t;
      t = v0;
      v0 = v1;
      v1 = t;
    }
    ++used;
  }
  if (blockIdx.x == 0) {
    sort_eig_block<T>(h0, v0, p, w, Vout, smem, p);
    if (threadIdx.x == 0) *sweeps_out = used;
  }
}

// ------------------------------------------------------------------ block Jacobi (FP32)
// The same eigendecomposition with far fewer grid-wide barriers: the index
// range (padded with zero rows and columns to P, a multiple of 64) is cut
// into blocks of 32, and a sweep pairs the blocks by the circle method (nb - 1
// rounds of nb / 2 disjoint pairs).  In a round, CTA k diagonalises the 64 x
// 64 principal submatrix of pair k by cyclic Jacobi in shared memory (the
// same rotation formula as the scalar kernel, 63 rounds of 32 rotations per
// inner sweep, until its off-diagonal part is below the outer tolerance) and
// publishes its orthogonal factor Q_k; then every 64 x 64 tile of H becomes
// Q_aᵀ H_ab Q_b and every 64-row tile of V becomes V Q_b, each tile read and
// written by one task (in place).  Two grid barriers per round: 2(nb - 1) per
// sweep instead of p - 1.  Zero padding never couples to the real indices, so
// V's leading p x p block holds the eigenvectors.
constexpr int kJB = 32;
constexpr int kJP = 2 * kJB;   // pair width
constexpr int kJLd = kJP + 1;  // shared-memory row stride
constexpr int kJbThreads = 1024;
constexpr int kJbMaxInner = 2;  // default inner sweeps per pair solve

__device__ __forceinline__ void jrot32(float a, float b, float c, float& cs, float& sn) {
  cs = 1.f;
  sn = 0.f;
  const double tiny = Eps<float>::v * 1e-3;
  if (c != 0.f && (double)c * (double)c > tiny * tiny * fabs((double)a) * fabs((double)b)) {
    const float theta = (b - a) * rcp_nr(2.f * c);
    float t;
    if (fabs((double)theta) > 1e15) {
      t = 0.5f * rcp_nr(theta);
    } else {
      const float q = fmaf(theta, theta, 1.f);
      const float root = q * rsqrt_nr(q);
      t = (theta >= 0.f ? 1.f : -1.f) * rcp_nr(fabsf(theta) + root);
    }
    cs = rsqrt_nr(fmaf(t, t, 1.f));
    sn = t * cs;
  }
}

// pair k of round r of the circle schedule over n (even) items
__device__ __forceinline__ int2 circle_pair(int n, int r, int k) {
  if (k == 0) return make_int2(min(r, n - 1), max(r, n - 1));
  const int a = (r + k) % (n - 1), b = (r - k + (n - 1)) % (n - 1);
  return make_int2(min(a, b), max(a, b));
}

// global index of local index l (0..63) of the pair of blocks (I, J)
__device__ __forceinline__ int pair_index(int I, int J, int l) { return l < kJB ? I * kJB + l : J * kJB + l - kJB; }

// sum over the CTA in a fixed order (warp shuffles, then warp 0)
__device__ __forceinline__ double cta_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < kJbThreads / 32; ++w) t += red[w];
  return t;
}

// Diagonalise the 64 x 64 principal submatrix of the pair (I, J); Q (64 x 64, global) <- its factor.
__device__ void jb_pair_solve(const float* __restrict__ H, int P, int I, int J, float* __restrict__ Qg, double tol2,
                              float* sm, double* red, int max_inner) {
  float* S = sm;
  float* S2 = S + kJP * kJLd;
  float* Q = S2 + kJP * kJLd;
  float* Q2 = Q + kJP * kJLd;
  float* cf = Q2 + kJP * kJLd;                    // per local index: c1, c2
  int* pq = reinterpret_cast<int*>(cf + 2 * kJP);  // per local index: P, Q, partner
  const int tid = threadIdx.x;
  for (int e = tid; e < kJP * kJP; e += kJbThreads) {
    const int r = e / kJP, c = e % kJP;
    const int gi = pair_index(I, J, r), gj = pair_index(I, J, c);
    S[r * kJLd + c] = 0.5f * (H[(size_t)gi * P + gj] + H[(size_t)gj * P + gi]);
    Q[r * kJLd + c] = r == c ? 1.f : 0.f;
  }
  __syncthreads();
  for (int sweep = 0; sweep < max_inner; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int e = tid; e < kJP * kJP; e += kJbThreads) {
      const double v = S[(e / kJP) * kJLd + e % kJP];
      tot += v * v;
      if (e / kJP != e % kJP) off += v * v;
    }
    off = cta_sum(off, red);
    tot = cta_sum(tot, red);
    if (!(off > tol2 * tot)) break;  // the same decision in every thread
    for (int rr = 0; rr < kJP - 1; ++rr) {
      if (tid < kJP / 2) {
        const int2 pr = circle_pair(kJP, rr, tid);
        float cs, sn;
        jrot32(S[pr.x * kJLd + pr.x], S[pr.y * kJLd + pr.y], S[pr.x * kJLd + pr.y], cs, sn);
        cf[2 * pr.x] = cs;
        cf[2 * pr.x + 1] = -sn;
        cf[2 * pr.y] = sn;
        cf[2 * pr.y + 1] = cs;
        pq[3 * pr.x] = pr.x;
        pq[3 * pr.x + 1] = pr.y;
        pq[3 * pr.x + 2] = pr.y;
        pq[3 * pr.y] = pr.x;
        pq[3 * pr.y + 1] = pr.y;
        pq[3 * pr.y + 2] = pr.x;
      }
      __syncthreads();
      for (int e = tid; e < kJP * kJP; e += kJbThreads) {
        const int i = e / kJP, j = e % kJP;
        const float ci1 = cf[2 * i], ci2 = cf[2 * i + 1], cj1 = cf[2 * j], cj2 = cf[2 * j + 1];
        const int aP = pq[3 * i], aQ = pq[3 * i + 1], bP = pq[3 * j], bQ = pq[3 * j + 1];
        float v;
        if (i != j && pq[3 * i + 2] == j) {
          v = 0.f;
        } else {
          v = ci1 * (cj1 * S[aP * kJLd + bP] + cj2 * S[aP * kJLd + bQ]);
          v += ci2 * (cj1 * S[aQ * kJLd + bP] + cj2 * S[aQ * kJLd + bQ]);
        }
        S2[i * kJLd + j] = v;
        Q2[i * kJLd + j] = cj1 * Q[i * kJLd + bP] + cj2 * Q[i * kJLd + bQ];
      }
      __syncthreads();
      float* t = S;
      S = S2;
      S2 = t;
      t = Q;
      Q = Q2;
      Q2 = t;
    }
  }
  for (int e = tid; e < kJP * kJP; e += kJbThreads) Qg[e] = Q[(e / kJP) * kJLd + e % kJP];
}

// X (64 x 64 tile: rows ri(l), columns ci(l) of a matrix with leading
// dimension P) <- Qaᵀ X Qb (Qa null: X Qb).  Each thread forms a 2 x 2 block.
__device__ void jb_apply_tile(float* __restrict__ X, int P, int rI, int rJ, int rows_contig, int cI, int cJ,
                              const float* __restrict__ Qa, const float* __restrict__ Qb, float* sm) {
  float* Xs = sm;
  float* A = Xs + kJP * kJLd;
  float* B = A + kJP * kJLd;
  float* T = B + kJP * kJLd;
  const int tid = threadIdx.x;
  auto grow = [&](int l) { return rows_contig >= 0 ? rows_contig + l : pair_index(rI, rJ, l); };
  for (int e = tid; e < kJP * kJP; e += kJbThreads) {
    const int r = e / kJP, c = e % kJP;
    Xs[r * kJLd + c] = X[(size_t)grow(r) * P + pair_index(cI, cJ, c)];
    B[r * kJLd + c] = Qb[e];
    if (Qa) A[r * kJLd + c] = Qa[e];
  }
  __syncthreads();
  constexpr int TB = 2;  // output block per thread
  const int i0 = TB * (tid / (kJP / TB)), j0 = TB * (tid % (kJP / TB));
  float acc[TB][TB];
  const float* src = Xs;
  if (Qa) {
#pragma unroll
    for (int u = 0; u < TB; ++u)
#pragma unroll
      for (int v = 0; v < TB; ++v) acc[u][v] = 0.f;
    for (int k = 0; k < kJP; ++k) {
      float a[TB], x[TB];
#pragma unroll
      for (int u = 0; u < TB; ++u) a[u] = A[k * kJLd + i0 + u];
#pragma unroll
      for (int v = 0; v < TB; ++v) x[v] = Xs[k * kJLd + j0 + v];
#pragma unroll
      for (int u = 0; u < TB; ++u)
#pragma unroll
        for (int v = 0; v < TB; ++v) acc[u][v] = fmaf(a[u], x[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < TB; ++u)
#pragma unroll
      for (int v = 0; v < TB; ++v) T[(i0 + u) * kJLd + j0 + v] = acc[u][v];
    __syncthreads();
    src = T;
  }
#pragma unroll
  for (int u = 0; u < TB; ++u)
#pragma unroll
    for (int v = 0; v < TB; ++v) acc[u][v] = 0.f;
  for (int k = 0; k < kJP; ++k) {
    float a[TB], b[TB];
#pragma unroll
    for (int u = 0; u < TB; ++u) a[u] = src[(i0 + u) * kJLd + k];
#pragma unroll
    for (int v = 0; v < TB; ++v) b[v] = B[k * kJLd + j0 + v];
#pragma unroll
    for (int u = 0; u < TB; ++u)
#pragma unroll
      for (int v = 0; v < TB; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < TB; ++u)
#pragma unroll
    for (int v = 0; v < TB; ++v) X[(size_t)grow(i0 + u) * P + pair_index(cI, cJ, j0 + v)] = acc[u][v];
  __syncthreads();  // the shared buffers are reused by the next task
}

__global__ void __launch_bounds__(kJbThreads) jacobi_block32(const float* __restrict__ H, int p, int P, float* Hp,
                                                             float* Vp, float* Qbuf, double* part, int max_sweeps,
                                                             double tol2, unsigned int* bar, int* err,
                                                             int* sweeps_out, float* w, float* Vout, int max_inner) {
  extern __shared__ __align__(16) unsigned char jsm[];
  __shared__ double red[kJbThreads / 32];
  __shared__ double s_off, s_tot;
  float* sm = reinterpret_cast<float*>(jsm);
  const unsigned G = gridDim.x;
  const int nb = P / kJB, npair = nb / 2;
  const long long PP = (long long)P * P;
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x, gsz = (long long)G * blockDim.x;
  for (long long e = gtid; e < PP; e += gsz) {
    const int i = (int)(e / P), j = (int)(e % P);
    Hp[e] = (i < p && j < p) ? 0.5f * (H[(size_t)i * p + j] + H[(size_t)j * p + i]) : 0.f;
    Vp[e] = i == j ? 1.f : 0.f;
  }
  if (!grid_barrier(bar, err, G)) return;
  int used = 0;
  const int ntask = npair * npair + (P / kJP) * npair;
  double prev_off = -1.0;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (long long e = gtid; e < PP; e += gsz) {
      const double v = (double)Hp[e];
      tot += v * v;
      if (e / P != e % P) off += v * v;
    }
    off = cta_sum(off, red);
    tot = cta_sum(tot, red);
    if (threadIdx.x == 0) {
      part[2 * blockIdx.x] = off;
      part[2 * blockIdx.x + 1] = tot;
    }
    if (!grid_barrier(bar, err, G)) return;
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (unsigned q = 0; q < G; ++q) {
        a += part[2 * q];
        b += part[2 * q + 1];
      }
      s_off = a;
      s_tot = b;
    }
    __syncthreads();
    if (!(s_off > tol2 * s_tot)) break;
    // the tile products leave an off-diagonal floor of ~64u||H|| (FP32 sums of
    // 64 terms) near the tolerance: from the third sweep on, one that did not
    // halve off(H)² stops (early sweeps reduce it by far more)
    if (sweep >= 2 && s_off > 0.5 * prev_off) break;
    prev_off = s_off;
    for (int r = 0; r < nb - 1; ++r) {
      for (int k = blockIdx.x; k < npair; k += G) {
        const int2 pr = circle_pair(nb, r, k);
        jb_pair_solve(Hp, P, pr.x, pr.y, Qbuf + (size_t)k * kJP * kJP, tol2, sm, red, max_inner);
        __syncthreads();
      }
      if (!grid_barrier(bar, err, G)) return;
      for (int t = blockIdx.x; t < ntask; t += G) {
        if (t < npair * npair) {
          const int a = t / npair, b = t % npair;
          const int2 pa = circle_pair(nb, r, a), pb = circle_pair(nb, r, b);
          jb_apply_tile(Hp, P, pa.x, pa.y, -1, pb.x, pb.y, Qbuf + (size_t)a * kJP * kJP,
                        Qbuf + (size_t)b * kJP * kJP, sm);
        } else {
          const int u = t - npair * npair;
          const int R = u / npair, b = u % npair;
          const int2 pb = circle_pair(nb, r, b);
          jb_apply_tile(Vp, P, 0, 0, R * kJP, pb.x, pb.y, nullptr, Qbuf + (size_t)b * kJP * kJP, sm);
        }
      }
      if (!grid_barrier(bar, err, G)) return;
    }
    ++used;
  }
  if (blockIdx.x == 0) {
    sort_eig_block<float>(Hp, Vp, p, w, Vout, jsm, P);
    if (threadIdx.x == 0) *sweeps_out = used;
  }
}

// round-robin (circle method) partner tables, cached per size
std::mutex g_sched_mu;
std::map<int, std::vector<int>> g_sched;

const std::vector<int>& schedule(int p) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  auto it = g_sched.find(p);
  if (it != g_sched.end()) return it->second;
  const int P = p + (p & 1);
  const int rounds = P - 1;
  std::vector<int> tab((size_t)rounds * p);
  for (int r = 0; r < rounds; ++r) {
    std::vector<int> part(P);
    part[P - 1] = r;
    part[r] = P - 1;
    for (int k = 1; k < P / 2; ++k) {
      int a = (r + k) % (P - 1), b = (r - k + (P - 1)) % (P - 1);
      part[a] = b;
      part[b] = a;
    }
    for (int i = 0; i < p; ++i) tab[(size_t)r * p + i] = part[i] >= p ? i : part[i];
  }
  return g_sched.emplace(p, std::move(tab)).first->second;
}

// ------------------------------------------------------------------ column utilities
template <typename T>
__global__ void colsq_partial(const T* __restrict__ X, int ld, long long N, int b, long long chunk, T* __restrict__ part) {
  const long long r0 = blockIdx.x * chunk, r1 = min(N, r0 + chunk);
  for (int j = threadIdx.x; j < b; j += blockDim.x) {
    T s = T(0);
    for (long long r = r0; r < r1; ++r) {
      T v = X[r * ld + j];
      s = fma(v, v, s);
    }
    part[(size_t)blockIdx.x * b + j] = s;
  }
}

template <typename T>
__global__ void colsq_final(const T* __restrict__ part, int nchunk, int b, T* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= b) return;
  T s = T(0);
  for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * b + j];
  out[j] = sqrt(s);
}

template <typename T>
__global__ void scale_cols_kernel(T* __restrict__ X, int ld, long long N, int b, const T* __restrict__ s, bool inv) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= N * b) return;
  const long long r = e / b;
  const int j = (int)(e % b);
  const T f = s[j];
  X[r * ld + j] = inv ? (f != T(0) ? X[r * ld + j] / f : T(0)) : X[r * ld + j] * f;
}

template <typename A, typename B>
__global__ void convert_kernel(const A* __restrict__ in, int ldi, B* __restrict__ out, int ldo, long long N, int b) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= N * b) return;
  const long long r = e / b;
  const int j = (int)(e % b);
  out[r * ldo + j] = (B)in[r * ldi + j];
}

int col_chunks(long long N) { return (int)std::max<long long>(1, std::min<long long>(1024, N / 64)); }

}  // namespace

// ------------------------------------------------------------------ host launchers
template <typename T>
size_t gram_workspace(long long N, int p, int q) {
  return sizeof(T) * (size_t)gram_splits<T>(N, p, q) * p * q + 256;
}

template <typename T>
int gram(const T* A, int lda, const T* B, int ldb, long long N, int p, int q, T* C, int ldc, T alpha, T beta,
         void* ws, size_t ws_bytes, cudaStream_t st) {
  const int splits = gram_splits<T>(N, p, q);
  if (ws_bytes < gram_workspace<T>(N, p, q)) {
    set_error("gram: workspace too small");
    return RVGP_EWORKSPACE;
  }
  const long long chunk = (N + splits - 1) / splits;
  dim3 grid(ceil_div(p, TB), ceil_div(q, TB), splits);
  T* part = static_cast<T*>(ws);
  rvgp::note_launch(); gram_partial<T><<<grid, 256, 0, st>>>(A, lda, B, ldb, N, p, q, chunk, part);
  rvgp::note_launch(); reduce_splits<T><<<ceil_div((long long)p * q, 256), 256, 0, st>>>(part, splits, p, q, C, ldc, alpha, beta);
  return check_launch("gram");
}

int gram_f32_out64(const float* A, int lda, const float* B, int ldb, long long N, int p, int q, double* C, int ldc,
                   double alpha, double beta, void* ws, size_t ws_bytes, cudaStream_t st) {
  const int splits = gram_splits<float>(N, p, q);
  if (ws_bytes < gram_workspace<float>(N, p, q)) {
    set_error("gram: workspace too small");
    return RVGP_EWORKSPACE;
  }
  const long long chunk = (N + splits - 1) / splits;
  dim3 grid(ceil_div(p, TB), ceil_div(q, TB), splits);
  float* part = static_cast<float*>(ws);
  rvgp::note_launch(); gram_partial<float><<<grid, 256, 0, st>>>(A, lda, B, ldb, N, p, q, chunk, part);
  rvgp::note_launch(); reduce_splits_f32_to_f64<<<ceil_div((long long)p * q, 256), 256, 0, st>>>(part, splits, p, q, C, ldc, alpha, beta);
  return check_launch("gram_f32_out64");
}

template <typename T>
int gemm_nn(const T* A, int lda, const T* B, int ldb, long long N, int p, int q, T* C, int ldc, T alpha, T beta,
            cudaStream_t st) {
  dim3 grid(ceil_div(N, TB), ceil_div(q, TB));
  rvgp::note_launch(); gemm_nn_kernel<T><<<grid, 256, 0, st>>>(A, lda, B, ldb, N, p, q, C, ldc, alpha, beta);
  return check_launch("gemm_nn");
}

template <typename T>
int cholesky(T* A, int lda, int p, int* info, cudaStream_t st) {
  cudaMemsetAsync(info, 0, sizeof(int), st);
  const size_t smem = potrf_small_smem<T>(p);
  if (smem <= kSmallCholSmem) {
    static std::atomic<bool> attr_set{false};  // per kernel; setting it twice is harmless
    if (!attr_set.load()) {
      if (raise_dyn_smem((const void*)potrf_small<T>, (size_t)(kSmallCholSmem)) !=
          cudaSuccess) {
        set_error("cholesky: cannot reserve %zu bytes of shared memory", kSmallCholSmem);
        return RVGP_ELAUNCH;
      }
      attr_set = true;
    }
    rvgp::note_launch(); potrf_small<T><<<1, 512, smem, st>>>(A, lda, p, info);
    return check_launch("cholesky");
  }
  for (int k0 = 0; k0 < p; k0 += NB) {
    const int nb = std::min(NB, p - k0);
    rvgp::note_launch(); potrf_diag<T><<<1, 128, 0, st>>>(A, lda, k0, nb, info);
    const int rest = p - k0 - nb;
    if (rest <= 0) break;
    const int rb = ceil_div(rest, NB);
    rvgp::note_launch(); trsm_panel<T><<<ceil_div(rest, 64), 64, 0, st>>>(A, lda, k0, nb, p, info);
    rvgp::note_launch(); syrk_update<T><<<dim3(rb, rb), 256, 0, st>>>(A, lda, k0, nb, p, info);
  }
  return check_launch("cholesky");
}

template <typename T>
int tri_inv_lower(const T* L, int ldl, int p, T* Linv, int ldi, cudaStream_t st) {
  const size_t pf_smem = sizeof(T) * 5 * (size_t)p;  // y, 1/L_kk and three columns
  if (pf_smem <= 200 * 1024) {
    if (raise_dyn_smem((const void*)trinv_pf_kernel<T>, pf_smem) != cudaSuccess) return check_launch("tri_inv_lower");
    const int nb = ceil_div(p, 32);
    rvgp::note_launch(); lower_to_upper<T><<<dim3(nb, nb), 256, 0, st>>>(L, ldl, p, Linv, ldi);
    rvgp::note_launch(); trinv_pf_kernel<T><<<p, 32, pf_smem, st>>>(L, ldl, Linv, ldi, p, Linv, ldi);
    rvgp::note_launch(); zero_strict_upper<T><<<ceil_div((long long)p * p, 256), 256, 0, st>>>(Linv, ldi, p);
    return check_launch("tri_inv_lower");
  }
  // shared memory: 2p values per warp, at most 48 KB per CTA
  const int warps = (int)std::max<size_t>(1, std::min<size_t>(4, (48 * 1024) / (2 * sizeof(T) * (size_t)p)));
  const size_t smem = sizeof(T) * 2 * (size_t)warps * p;
  rvgp::note_launch(); trinv_kernel<T><<<ceil_div(p, warps), 32 * warps, smem, st>>>(L, ldl, p, Linv, ldi, warps);
  return check_launch("tri_inv_lower");
}

constexpr int kMaxCoopGrid = 1024;

template <typename T>
size_t jacobi_workspace(int p) {
  const int P = p + (p & 1);
  return sizeof(T) * (size_t)p * p * 3 + sizeof(int) * (size_t)(P - 1) * p + 2 * sizeof(double) +
         sizeof(T) * 2 * (size_t)p + sizeof(int2) * (size_t)p + sizeof(double) * 2 * kMaxCoopGrid + sizeof(unsigned int) * (kMaxCoopGrid + 1) + 8192;
}

template <typename T>
int jacobi_eigh(T* H, int p, T* w, T* V, int max_sweeps, double tol, int* sweeps_used, void* ws, size_t ws_bytes,
                cudaStream_t st) {
  if (p < 1 || p > 2048) {
    set_error("jacobi_eigh: p=%d out of range", p);
    return RVGP_ENOTSUP;
  }
  if (ws_bytes < jacobi_workspace<T>(p)) {
    set_error("jacobi_eigh: workspace too small");
    return RVGP_EWORKSPACE;
  }
  Workspace W(ws, ws_bytes);
  T* Hb = W.take<T>((size_t)p * p);
  T* Va = W.take<T>((size_t)p * p);
  T* Vb = W.take<T>((size_t)p * p);
  const int P = p + (p & 1);
  const int rounds = P - 1;
  int* part = W.take<int>((size_t)rounds * p);
  double* nrm = W.take<double>(2);
  T* coef = W.take<T>(2 * (size_t)p);
  int2* pq = W.take<int2>(p);
  const std::vector<int>& tab = schedule(p);
  cudaMemcpyAsync(part, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice, st);
  const long long pp = (long long)p * p;

  // one cooperative launch for all sweeps when the device supports it
  double* gpart = W.take<double>(2 * (size_t)kMaxCoopGrid);
  unsigned int* bar = W.take<unsigned int>(kMaxCoopGrid + 1);
  int* flags = W.take<int>(2);  // [0] barrier error, [1] sweeps used
  // dynamic shared memory: the round's coefficients during the sweeps, the sort buffers at the end
  const size_t smem = std::max(sizeof(T) * 2 * (size_t)p + sizeof(int2) * (size_t)p,
                               2048 * sizeof(T) + 2048 * sizeof(int));
  // grid: about eight (FP32) or two (FP64) rotated elements per thread and
  // round; fewer CTAs make each round's grid barrier cheaper
  const long long per_cta = 256LL * (sizeof(T) == 4 ? 8 : 2);
  int G = smem <= 48 * 1024 ? std::min(cooperative_grid(jacobi_persistent<T>, 256, smem), kMaxCoopGrid) : 0;
  if (G > 0) G = (int)std::max<long long>(1, std::min<long long>(G, (2 * pp + per_cta - 1) / per_cta));
  if (G > 0 && p > 1) {
    cudaMemsetAsync(bar, 0, (G + 1) * sizeof(unsigned int), st);
    cudaMemsetAsync(flags, 0, 2 * sizeof(int), st);
    T* Hp = H;
    int pv = p, rv = rounds, ms = max_sweeps;
    double t2 = tol * tol;
    int* err_dev = flags;
    int* sweeps_dev = flags + 1;
    void* args[] = {&Hp, &Hb, &Va, &Vb, &pv, &part, &rv, &gpart, &ms, &t2, &bar, &err_dev, &sweeps_dev, &w, &V};
    rvgp::note_launch();
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)jacobi_persistent<T>, dim3(G), dim3(256), args, smem, st);
    if (e != cudaSuccess) {
      set_error("jacobi_eigh: cooperative launch failed: %s", cudaGetErrorString(e));
      return RVGP_ELAUNCH;
    }
    int hv[2] = {0, 0};
    if (read_back(hv, flags, sizeof(hv), st) != cudaSuccess) return check_launch("jacobi_eigh");
    if (hv[0] != 0) {
      set_error("jacobi_eigh: a grid barrier timed out");
      return RVGP_ELAUNCH;
    }
    if (sweeps_used) *sweeps_used = hv[1];
    return check_launch("jacobi_eigh");
  }

  rvgp::note_launch(); set_identity<T><<<ceil_div(pp, 256), 256, 0, st>>>(Va, p);
  rvgp::note_launch(); symmetrise<T><<<ceil_div(pp, 256), 256, 0, st>>>(H, p);
  T *h0 = H, *h1 = Hb, *v0 = Va, *v1 = Vb;
  int used = 0;
  for (int sweep = 0; sweep < max_sweeps && p > 1; ++sweep) {
    rvgp::note_launch(); offnorm_kernel<T><<<1, 1024, 0, st>>>(h0, p, nrm);
    double hn[2];
    if (read_back(hn, nrm, sizeof(hn), st) != cudaSuccess) return check_launch("jacobi_eigh");
    if (!(hn[0] > tol * tol * hn[1])) break;
    for (int r = 0; r < rounds; ++r) {
      rvgp::note_launch(); jacobi_params<T><<<ceil_div(p, 128), 128, 0, st>>>(h0, p, part + (size_t)r * p, coef, pq);
      rvgp::note_launch(); jacobi_round<T><<<ceil_div(2 * pp, 256), 256, 0, st>>>(h0, h1, v0, v1, p, part + (size_t)r * p, coef, pq);
      T* t = h0; h0 = h1; h1 = t;
      t = v0; v0 = v1; v1 = t;
    }
    ++used;
  }
  if (sweeps_used) *sweeps_used = used;
  rvgp::note_launch(); sort_eig<T><<<1, 1024, smem, st>>>(h0, v0, p, w, V);
  return check_launch("jacobi_eigh");
}

size_t jacobi_block_smem() {
  return std::max<size_t>(4 * sizeof(float) * kJP * kJLd + 2 * kJP * sizeof(float) + 3 * kJP * sizeof(int),
                          2048 * sizeof(float) + 2048 * sizeof(int));
}

size_t jacobi_block_workspace(int p) {
  const int P = (p + kJP - 1) / kJP * kJP;
  Workspace W(nullptr, 0);
  W.take<float>((size_t)P * P);
  W.take<float>((size_t)P * P);
  W.take<float>((size_t)(P / kJP) * kJP * kJP);
  W.take<double>(2 * (size_t)kMaxCoopGrid);
  W.take<unsigned int>(kMaxCoopGrid + 1);
  W.take<int>(2);
  return W.used;
}

// FP32 eigendecomposition by block Jacobi (see jacobi_block32): w ascending,
// V (p x p) the eigenvectors by column.  H is read only.  Returns
// RVGP_ENOTSUP when the cooperative launch cannot hold a CTA per block pair.
int jacobi_block_eigh(const float* H, int p, float* w, float* V, int max_sweeps, double tol, int* sweeps_used,
                      void* ws, size_t ws_bytes, cudaStream_t st) {
  if (p < kJP || p > 2048) {
    set_error("jacobi_block_eigh: p=%d out of range", p);
    return RVGP_ENOTSUP;
  }
  if (ws_bytes < jacobi_block_workspace(p)) {
    set_error("jacobi_block_eigh: workspace too small");
    return RVGP_EWORKSPACE;
  }
  const int P = (p + kJP - 1) / kJP * kJP;
  Workspace W(ws, ws_bytes);
  float* Hp = W.take<float>((size_t)P * P);
  float* Vp = W.take<float>((size_t)P * P);
  float* Qb = W.take<float>((size_t)(P / kJP) * kJP * kJP);
  double* part = W.take<double>(2 * (size_t)kMaxCoopGrid);
  unsigned int* bar = W.take<unsigned int>(kMaxCoopGrid + 1);
  int* flags = W.take<int>(2);
  const size_t smem = jacobi_block_smem();
  if (raise_dyn_smem((const void*)jacobi_block32, (size_t)(smem)) != cudaSuccess)
    return check_launch("jacobi_block_eigh");
  const int npair = P / kJP;
  const int ntask = npair * npair + (P / kJP) * npair;
  int G = std::min(std::min(cooperative_grid(jacobi_block32, kJbThreads, smem), kMaxCoopGrid), num_sms());
  G = std::min(G, ntask);
  if (G < npair) {
    set_error("jacobi_block_eigh: %d resident CTAs for %d block pairs", G, npair);
    return RVGP_ENOTSUP;
  }
  cudaMemsetAsync(bar, 0, (G + 1) * sizeof(unsigned int), st);
  cudaMemsetAsync(flags, 0, 2 * sizeof(int), st);
  int pv = p, Pv = P, ms = max_sweeps;
  double t2 = tol * tol;
  int* err_dev = flags;
  int* sweeps_dev = flags + 1;
  // inner sweeps per 64 x 64 pair solve (RVGP_JACOBI_BLOCK_INNER overrides)
  const char* ie = getenv("RVGP_JACOBI_BLOCK_INNER");
  int inner = ie ? std::max(1, std::min(8, atoi(ie))) : kJbMaxInner;
  void* args[] = {(void*)&H, &pv, &Pv, &Hp, &Vp, &Qb, &part, &ms, &t2, &bar, &err_dev, &sweeps_dev, &w, &V, &inner};
  rvgp::note_launch();
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)jacobi_block32, dim3(G), dim3(kJbThreads), args, smem, st);
  if (e != cudaSuccess) {
    set_error("jacobi_block_eigh: cooperative launch failed: %s", cudaGetErrorString(e));
    return RVGP_ELAUNCH;
  }
  int hv[2] = {0, 0};
  if (read_back(hv, flags, sizeof(hv), st) != cudaSuccess) return check_launch("jacobi_block_eigh");
  if (hv[0] != 0) {
    set_error("jacobi_block_eigh: a grid barrier timed out");
    return RVGP_ELAUNCH;
  }
  if (sweeps_used) *sweeps_used = hv[1];
  return check_launch("jacobi_block_eigh");
}

template <typename T>
size_t col_norms_workspace(long long N, int b) {
  return sizeof(T) * (size_t)col_chunks(N) * b + 256;
}

template <typename T>
int col_norms(const T* X, int ld, long long N, int b, T* out, void* ws, size_t ws_bytes, cudaStream_t st) {
  const int nc = col_chunks(N);
  if (ws_bytes < col_norms_workspace<T>(N, b)) {
    set_error("col_norms: workspace too small");
    return RVGP_EWORKSPACE;
  }
  const long long chunk = (N + nc - 1) / nc;
  T* part = static_cast<T*>(ws);
  rvgp::note_launch(); colsq_partial<T><<<nc, 256, 0, st>>>(X, ld, N, b, chunk, part);
  rvgp::note_launch(); colsq_final<T><<<ceil_div(b, 256), 256, 0, st>>>(part, nc, b, out);
  return check_launch("col_norms");
}

template <typename T>
int scale_cols(T* X, int ld, long long N, int b, const T* s, bool inverse, cudaStream_t st) {
  rvgp::note_launch(); scale_cols_kernel<T><<<ceil_div(N * b, 256), 256, 0, st>>>(X, ld, N, b, s, inverse);
  return check_launch("scale_cols");
}

int convert_f32_to_f64(const float* in, int ldi, double* out, int ldo, long long N, int b, cudaStream_t st) {
  rvgp::note_launch(); convert_kernel<float, double><<<ceil_div(N * b, 256), 256, 0, st>>>(in, ldi, out, ldo, N, b);
  return check_launch("convert");
}
int convert_f64_to_f32(const double* in, int ldi, float* out, int ldo, long long N, int b, cudaStream_t st) {
  rvgp::note_launch(); convert_kernel<double, float><<<ceil_div(N * b, 256), 256, 0, st>>>(in, ldi, out, ldo, N, b);
  return check_launch("convert");
}

#define INST(T)                                                                                                     \
  template size_t gram_workspace<T>(long long, int, int);                                                           \
  template int gram<T>(const T*, int, const T*, int, long long, int, int, T*, int, T, T, void*, size_t, cudaStream_t); \
  template int gemm_nn<T>(const T*, int, const T*, int, long long, int, int, T*, int, T, T, cudaStream_t);           \
  template int cholesky<T>(T*, int, int, int*, cudaStream_t);                                                       \
  template int tri_inv_lower<T>(const T*, int, int, T*, int, cudaStream_t);                                         \
  template size_t jacobi_workspace<T>(int);                                                                         \
  template int jacobi_eigh<T>(T*, int, T*, T*, int, double, int*, void*, size_t, cudaStream_t);                     \
  template size_t col_norms_workspace<T>(long long, int);                                                           \
  template int col_norms<T>(const T*, int, long long, int, T*, void*, size_t, cudaStream_t);                        \
  template int scale_cols<T>(T*, int, long long, int, const T*, bool, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_symeig_f32_workspace(int p) {
  if (p < 1 || p > 2048) return 0;
  return sizeof(float) * (size_t)p * p + 256 + std::max(jacobi_workspace<float>(p), jacobi_block_workspace(p));
}

// Eigendecomposition of a symmetric FP32 matrix H (p x p, read only; the
// Rayleigh-Ritz step of the eigensolver, whose reference is ARPACK inside
// scipy's eigsh, RVGP/geometry.py:73): w ascending, V (p x p) eigenvectors by
// column, up to max_sweeps sweeps until off(H) <= tol ||H||_F.  method 0:
// block Jacobi for p >= 64, else scalar; 1: scalar parallel Jacobi (one grid
// barrier per rotation round); 2: block Jacobi.  *sweeps_used (host, may be
// null).  Synchronises.
RVGP_API int rvgp_symeig_f32(const float* H, int p, float* w, float* V, int max_sweeps, double tol,
                             int* sweeps_used, int method, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(H && w && V && p >= 1 && p <= 2048 && max_sweeps >= 0, "rvgp_symeig_f32: bad arguments");
  RVGP_CHECK_ARG(method >= 0 && method <= 2, "rvgp_symeig_f32: method %d", method);
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_symeig_f32_workspace(p), "rvgp_symeig_f32: workspace");
  cudaStream_t st = as_stream(stream);
  const bool block = method == 2 || (method == 0 && p >= kJP);
  RVGP_CHECK_ARG(!block || p >= kJP, "rvgp_symeig_f32: the block form needs p >= %d", kJP);
  Workspace W(workspace, ws_bytes);
  float* Hc = W.take<float>((size_t)p * p);
  const size_t rest = ws_bytes - W.used;
  void* jws = W.take<char>(rest - 256);
  if (block) return jacobi_block_eigh(H, p, w, V, max_sweeps, tol, sweeps_used, jws, rest - 256, st);
  cudaMemcpyAsync(Hc, H, sizeof(float) * (size_t)p * p, cudaMemcpyDeviceToDevice, st);
  return jacobi_eigh<float>(Hc, p, w, V, max_sweeps, tol, sweeps_used, jws, rest - 256, st);
}

