// Block-sparse times dense-block product with a fused three-term update:
//
//   Y = alpha * (A X) + beta * X + gamma * Z
//
// A: block CSR over n block-rows with DB x DB blocks (DB = 1 for the graph
// Laplacian L, DB = d for the connection Laplacian Lc; the products that
// scipy's ARPACK drives inside eigsh, RVGP/geometry.py:73, and the dense
// expm of RVGP/smoothing.py:15 become these).  X, Y, Z: (n*DB) x b row-major
// with leading dimension ld.  Z may be null (gamma ignored).
//
// Thread mapping: one thread per (block-row, group of V consecutive columns),
// V = 4 floats or 2 doubles (16-byte vector loads of X rows).  A row's gather
// of X hits L2: the whole block (n*DB*b*size) is sized to stay resident.  The
// gather is latency-bound, so each thread keeps several neighbours' loads in
// flight (the neighbour loop is unrolled with all loads ahead of the math).
// HBM traffic per product ≈ E*(DB²*sv + 4) + 2*n*DB*b*sx (+ Z).
#include "common.cuh"

namespace rvgp {
namespace {

template <typename T> struct Vec;
template <> struct Vec<float> { using type = float4; static constexpr int V = 4; };
template <> struct Vec<double> { using type = double2; static constexpr int V = 2; };

template <typename T>
__device__ __forceinline__ void vload(const T* p, T* out) {
  using VT = typename Vec<T>::type;
  VT v = *reinterpret_cast<const VT*>(p);
  const T* s = reinterpret_cast<const T*>(&v);
#pragma unroll
  for (int q = 0; q < Vec<T>::V; ++q) out[q] = s[q];
}

template <typename T>
__device__ __forceinline__ void vstore(T* p, const T* in) {
  using VT = typename Vec<T>::type;
  VT v;
  T* s = reinterpret_cast<T*>(&v);
#pragma unroll
  for (int q = 0; q < Vec<T>::V; ++q) s[q] = in[q];
  *reinterpret_cast<VT*>(p) = v;
}

template <typename T, int DB>
__global__ void __launch_bounds__(256) bspmm_kernel(int n, const int* __restrict__ indptr,
                                                    const int* __restrict__ indices, const T* __restrict__ vals,
                                                    const T* __restrict__ X, T* __restrict__ Y,
                                                    const T* __restrict__ Z, int b, int ld, T alpha, T beta, T gamma) {
  constexpr int V = Vec<T>::V;
  const int groups = b / V;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= (long long)n * groups) return;
  const int i = (int)(tid / groups);
  const int c0 = (int)(tid % groups) * V;
  T acc[DB][V];
#pragma unroll
  for (int p = 0; p < DB; ++p)
#pragma unroll
    for (int v = 0; v < V; ++v) acc[p][v] = T(0);
  const int s = indptr[i], e = indptr[i + 1];
  // U neighbours per iteration: all their index, block and X-row loads are
  // issued before the first multiply-add, so U gathers are in flight at once
  constexpr int U = DB <= 2 ? 4 : 2;
  int t = s;
  for (; t + U <= e; t += U) {
    int j[U];
#pragma unroll
    for (int u = 0; u < U; ++u) j[u] = __ldg(indices + t + u);
    T blk[U][DB * DB];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int pq = 0; pq < DB * DB; ++pq) blk[u][pq] = __ldg(vals + (size_t)(t + u) * DB * DB + pq);
    T x[U][DB][V];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int q = 0; q < DB; ++q) vload(X + ((size_t)j[u] * DB + q) * ld + c0, x[u][q]);
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int q = 0; q < DB; ++q)
#pragma unroll
        for (int p = 0; p < DB; ++p)
#pragma unroll
          for (int v = 0; v < V; ++v) acc[p][v] = fma(blk[u][p * DB + q], x[u][q][v], acc[p][v]);
  }
  for (; t < e; ++t) {
    const int j = __ldg(indices + t);
    T blk[DB * DB];
#pragma unroll
    for (int pq = 0; pq < DB * DB; ++pq) blk[pq] = __ldg(vals + (size_t)t * DB * DB + pq);
#pragma unroll
    for (int q = 0; q < DB; ++q) {
      T x[V];
      vload(X + ((size_t)j * DB + q) * ld + c0, x);
#pragma unroll
      for (int p = 0; p < DB; ++p)
#pragma unroll
        for (int v = 0; v < V; ++v) acc[p][v] = fma(blk[p * DB + q], x[v], acc[p][v]);
    }
  }
#pragma unroll
  for (int p = 0; p < DB; ++p) {
    const size_t row = ((size_t)i * DB + p) * ld + c0;
    T out[V], x[V];
#pragma unroll
    for (int v = 0; v < V; ++v) out[v] = alpha * acc[p][v];
    if (beta != T(0)) {
      vload(X + row, x);
#pragma unroll
      for (int v = 0; v < V; ++v) out[v] = fma(beta, x[v], out[v]);
    }
    if (Z && gamma != T(0)) {
      vload(Z + row, x);
#pragma unroll
      for (int v = 0; v < V; ++v) out[v] = fma(gamma, x[v], out[v]);
    }
    vstore(Y + row, out);
  }
}

template <typename T>
int launch(int n, int DB, const int* indptr, const int* indices, const T* vals, const T* X, T* Y, const T* Z, int b,
           int ld, T alpha, T beta, T gamma, cudaStream_t st) {
  constexpr int V = Vec<T>::V;
  RVGP_CHECK_ARG(b % V == 0 && ld % V == 0 && b <= ld, "rvgp_bspmm: b=%d and ld=%d must be multiples of %d", b, ld, V);
  RVGP_CHECK_ARG(((uintptr_t)X | (uintptr_t)Y | (uintptr_t)(Z ? Z : X)) % 16 == 0, "rvgp_bspmm: 16-byte alignment");
  long long threads = (long long)n * (b / V);
  int grid = ceil_div(threads, 256);
  switch (DB) {
    case 1: rvgp::note_launch(); bspmm_kernel<T, 1><<<grid, 256, 0, st>>>(n, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma); break;
    case 2: rvgp::note_launch(); bspmm_kernel<T, 2><<<grid, 256, 0, st>>>(n, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma); break;
    case 3: rvgp::note_launch(); bspmm_kernel<T, 3><<<grid, 256, 0, st>>>(n, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma); break;
    case 4: rvgp::note_launch(); bspmm_kernel<T, 4><<<grid, 256, 0, st>>>(n, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma); break;
    default: rvgp::set_error("rvgp_bspmm: block size %d not supported (1..4)", DB); return RVGP_ENOTSUP;
  }
  RVGP_LAUNCH_CHECK("rvgp_bspmm");
  return RVGP_OK;
}

}  // namespace

int bspmm_f32(int n, int DB, const int* indptr, const int* indices, const float* vals, const float* X, float* Y,
              const float* Z, int b, int ld, float alpha, float beta, float gamma, cudaStream_t st) {
  return launch<float>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
}
int bspmm_f64(int n, int DB, const int* indptr, const int* indices, const double* vals, const double* X, double* Y,
              const double* Z, int b, int ld, double alpha, double beta, double gamma, cudaStream_t st) {
  return launch<double>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
}

}  // namespace rvgp

RVGP_API int rvgp_bspmm_f32(int n, int DB, const int* indptr, const int* indices, const float* vals, const float* X,
                            float* Y, const float* Z, int b, int ld, float alpha, float beta, float gamma,
                            void* stream) {
  return rvgp::bspmm_f32(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, rvgp::as_stream(stream));
}

RVGP_API int rvgp_bspmm_f64(int n, int DB, const int* indptr, const int* indices, const double* vals,
                            const double* X, double* Y, const double* Z, int b, int ld, double alpha, double beta,
                            double gamma, void* stream) {
  return rvgp::bspmm_f64(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, rvgp::as_stream(stream));
}
