// FP64 dense products for the small dense algebra of the GP models (sparse
// GP, RBF GP): tiled GEMM with transpose flags and matrix-vector kernels.
// Internal; every translation unit that includes it gets its own copy.
#pragma once
#include "common.cuh"
#include <algorithm>

namespace rvgp {
namespace {

// FP64 on GB300 issues about one warp instruction per ~19 SM cycles, so the
// products below are sized by FP64 instruction count: no lanes computing
// padding (dedicated matrix-vector kernels) and grids spread over all SMs
// (the output tile shrinks until there are enough CTAs).
constexpr int kT = 32;  // largest GEMM output tile

// C (R x Q) = alpha op(A) op(B) + beta C, row-major; op(A) is R x K, op(B) K x Q.
// TA: op(A)(i, k) = A[k * lda + i]; TB: op(B)(k, j) = B[j * ldb + k].
__device__ __forceinline__ void store_out(double* C, int ldc, int i, int j, double alpha, double beta, double acc) {
  double* c = C + (size_t)i * ldc + j;
  *c = beta == 0.0 ? alpha * acc : fma(beta, *c, alpha * acc);
}

// 32 x 32 outputs per CTA, 4 per thread
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm64_t32(int R, int Q, int K, double alpha, const double* __restrict__ A,
                                                  int lda, const double* __restrict__ B, int ldb, double beta,
                                                  double* __restrict__ C, int ldc) {
  __shared__ double As[kT][kT + 1];  // [i][k]
  __shared__ double Bs[kT][kT + 1];  // [k][j]
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int i0 = blockIdx.y * kT, j0 = blockIdx.x * kT;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k0 = 0; k0 < K; k0 += kT) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int a = ty + 8 * r;
      if (!TA) {
        const int i = i0 + a, k = k0 + tx;
        As[a][tx] = (i < R && k < K) ? A[(size_t)i * lda + k] : 0.0;
      } else {
        const int k = k0 + a, i = i0 + tx;
        As[tx][a] = (i < R && k < K) ? A[(size_t)k * lda + i] : 0.0;
      }
      if (!TB) {
        const int k = k0 + a, j = j0 + tx;
        Bs[a][tx] = (k < K && j < Q) ? B[(size_t)k * ldb + j] : 0.0;
      } else {
        const int j = j0 + a, k = k0 + tx;
        Bs[tx][a] = (k < K && j < Q) ? B[(size_t)j * ldb + k] : 0.0;
      }
    }
    __syncthreads();
    const int kn = min(kT, K - k0);
    for (int k = 0; k < kn; ++k) {
      const double bv = Bs[k][tx];
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[r] = fma(As[ty + 8 * r][k], bv, acc[r]);
    }
    __syncthreads();
  }
  const int j = j0 + tx;
  if (j >= Q) return;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ty + 8 * r;
    if (i < R) store_out(C, ldc, i, j, alpha, beta, acc[r]);
  }
}

// 16 x 16 outputs per CTA, one per thread
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm64_t16(int R, int Q, int K, double alpha, const double* __restrict__ A,
                                                  int lda, const double* __restrict__ B, int ldb, double beta,
                                                  double* __restrict__ C, int ldc) {
  __shared__ double As[16][17];  // [i][k]
  __shared__ double Bs[16][17];  // [k][j]
  const int t = threadIdx.x, hi = t >> 4, lo = t & 15;
  const int i0 = blockIdx.y * 16, j0 = blockIdx.x * 16;
  double acc = 0.0;
  for (int k0 = 0; k0 < K; k0 += 16) {
    if (!TA) {
      const int i = i0 + hi, k = k0 + lo;
      As[hi][lo] = (i < R && k < K) ? A[(size_t)i * lda + k] : 0.0;
    } else {
      const int k = k0 + hi, i = i0 + lo;
      As[lo][hi] = (i < R && k < K) ? A[(size_t)k * lda + i] : 0.0;
    }
    if (!TB) {
      const int k = k0 + hi, j = j0 + lo;
      Bs[hi][lo] = (k < K && j < Q) ? B[(size_t)k * ldb + j] : 0.0;
    } else {
      const int j = j0 + hi, k = k0 + lo;
      Bs[lo][hi] = (k < K && j < Q) ? B[(size_t)j * ldb + k] : 0.0;
    }
    __syncthreads();
    const int kn = min(16, K - k0);
    for (int k = 0; k < kn; ++k) acc = fma(As[hi][k], Bs[k][lo], acc);
    __syncthreads();
  }
  const int i = i0 + hi, j = j0 + lo;
  if (i < R && j < Q) store_out(C, ldc, i, j, alpha, beta, acc);
}

// 8 x 8 outputs per CTA, each summed by 4 threads over interleaved quarters of
// every 32-deep slab, then added in a fixed order
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm64_t8(int R, int Q, int K, double alpha, const double* __restrict__ A,
                                                 int lda, const double* __restrict__ B, int ldb, double beta,
                                                 double* __restrict__ C, int ldc) {
  __shared__ double As[8][33];  // [i][k]
  __shared__ double Bs[32][9];  // [k][j]
  __shared__ double red[4][64];
  const int t = threadIdx.x, o = t & 63, kg = t >> 6;
  const int oy = o >> 3, ox = o & 7;
  const int i0 = blockIdx.y * 8, j0 = blockIdx.x * 8;
  double acc = 0.0;
  for (int k0 = 0; k0 < K; k0 += 32) {
    if (!TA) {
      const int a = t >> 5, b = t & 31, i = i0 + a, k = k0 + b;
      As[a][b] = (i < R && k < K) ? A[(size_t)i * lda + k] : 0.0;
    } else {
      const int a = t & 7, b = t >> 3, i = i0 + a, k = k0 + b;
      As[a][b] = (i < R && k < K) ? A[(size_t)k * lda + i] : 0.0;
    }
    if (!TB) {
      const int a = t & 7, b = t >> 3, j = j0 + a, k = k0 + b;
      Bs[b][a] = (k < K && j < Q) ? B[(size_t)k * ldb + j] : 0.0;
    } else {
      const int a = t >> 5, b = t & 31, j = j0 + a, k = k0 + b;
      Bs[b][a] = (k < K && j < Q) ? B[(size_t)j * ldb + k] : 0.0;
    }
    __syncthreads();
    const int kn = min(32, K - k0);
    for (int k = kg; k < kn; k += 4) acc = fma(As[oy][k], Bs[k][ox], acc);
    __syncthreads();
  }
  red[kg][o] = acc;
  __syncthreads();
  if (t < 64) {
    const int i = i0 + oy, j = j0 + ox;
    if (i < R && j < Q) store_out(C, ldc, i, j, alpha, beta, ((red[0][o] + red[1][o]) + red[2][o]) + red[3][o]);
  }
}

// y (R, stride ldy) = alpha A x + beta y, A row-major (lda), x stride ldx: one warp per row
__global__ void __launch_bounds__(256) gemv64_n(int R, int K, double alpha, const double* __restrict__ A, int lda,
                                                const double* __restrict__ x, int ldx, double beta,
                                                double* __restrict__ y, int ldy) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= R) return;
  double s = 0.0;
  for (int k = lane; k < K; k += 32) s = fma(A[(size_t)i * lda + k], x[(size_t)k * ldx], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) store_out(y, ldy, i, 0, alpha, beta, s);
}

// y (R) = alpha Aᵀ x + beta y with A stored K x R (lda): 32 outputs per CTA,
// the 8 warps summing interleaved rows k, added in a fixed order
__global__ void __launch_bounds__(256) gemv64_t(int R, int K, double alpha, const double* __restrict__ A, int lda,
                                                const double* __restrict__ x, int ldx, double beta,
                                                double* __restrict__ y, int ldy) {
  __shared__ double red[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (i < R)
    for (int k = w; k < K; k += 8) s = fma(A[(size_t)k * lda + i], x[(size_t)k * ldx], s);
  red[w][lane] = s;
  __syncthreads();
  if (w == 0 && i < R) {
    double r = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) r += red[q][lane];
    store_out(y, ldy, i, 0, alpha, beta, r);
  }
}

long long tiles(int R, int Q, int T) { return (long long)ceil_div(R, T) * ceil_div(Q, T); }

// op(B) with one column (TB false, Q == 1) is a matrix-vector product; otherwise
// the output tile is the largest of 32, 16, 8 that still gives every SM a CTA.
template <bool TA, bool TB>
void gemm64(int R, int Q, int K, double alpha, const double* A, int lda, const double* B, int ldb, double beta,
            double* C, int ldc, cudaStream_t st) {
  note_launch();
  if (Q == 1 && !TB) {
    if (!TA)
      gemv64_n<<<ceil_div((long long)R * 32, 256), 256, 0, st>>>(R, K, alpha, A, lda, B, ldb, beta, C, ldc);
    else
      gemv64_t<<<ceil_div(R, 32), 256, 0, st>>>(R, K, alpha, A, lda, B, ldb, beta, C, ldc);
    return;
  }
  if (tiles(R, Q, 32) >= 2 * num_sms()) {
    gemm64_t32<TA, TB><<<dim3(ceil_div(Q, 32), ceil_div(R, 32)), 256, 0, st>>>(R, Q, K, alpha, A, lda, B, ldb, beta,
                                                                               C, ldc);
  } else if (tiles(R, Q, 16) >= num_sms()) {
    gemm64_t16<TA, TB><<<dim3(ceil_div(Q, 16), ceil_div(R, 16)), 256, 0, st>>>(R, Q, K, alpha, A, lda, B, ldb, beta,
                                                                               C, ldc);
  } else {
    gemm64_t8<TA, TB><<<dim3(ceil_div(Q, 8), ceil_div(R, 8)), 256, 0, st>>>(R, Q, K, alpha, A, lda, B, ldb, beta, C,
                                                                            ldc);
  }
}

}  // namespace
}  // namespace rvgp
