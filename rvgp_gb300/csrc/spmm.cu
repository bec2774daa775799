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
// Mapping: W lanes per block row (W = 32, or the smallest power of two
// covering the row's 16-byte column groups when there are fewer than 32, so
// narrow blocks put several rows in a warp); sub-lane l owns the groups
// l, l+W, ... (G per lane, V = 4 floats or 2 doubles per group).  A row's
// column indices and DB x DB blocks are loaded once per neighbour by the whole
// warp (one broadcast request each), so L1 wavefronts go almost entirely to
// the gathered X rows; the kernel is bound by those L1 wavefronts (each
// gathered row crosses the L1 data path once per use) and by L2 latency, so
// there is no unrolling: more resident warps hide the latency better than
// more loads in flight per warp.  Rows in a locality-preserving order
// (neighbouring rows share neighbours) raise the L1 hit rate.
// HBM traffic per product ≈ E*(DB²*sv + 4) + 2*n*DB*b*sx (+ Z).
#include "common.cuh"
#include "autotune.cuh"
#include <limits.h>
#include <algorithm>
#include <stdio.h>
#include <stdlib.h>

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

// the same load cached in L2 only (no L1 allocation)
template <typename T>
__device__ __forceinline__ void vload_cg(const T* p, T* out) {
  using VT = typename Vec<T>::type;
  VT v = __ldcg(reinterpret_cast<const VT*>(p));
  const T* s = reinterpret_cast<const T*>(&v);
#pragma unroll
  for (int q = 0; q < Vec<T>::V; ++q) out[q] = s[q];
}

template <typename T, bool CG>
__device__ __forceinline__ void vgather(const T* p, T* out) {
  if constexpr (CG)
    vload_cg(p, out);
  else
    vload(p, out);
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

// the DB x DB block of entry t, loaded by every lane of the warp (broadcast)
template <typename T, int DB>
__device__ __forceinline__ void load_block(const T* __restrict__ vals, int t, T* blk) {
  constexpr int NB = DB * DB;
  if constexpr ((NB * sizeof(T)) % 16 == 0) {
    using VT = typename Vec<T>::type;
    constexpr int V = Vec<T>::V;
    const VT* p = reinterpret_cast<const VT*>(vals + (size_t)t * NB);
#pragma unroll
    for (int c = 0; c < NB / V; ++c) {
      VT v = __ldg(p + c);
      const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
      for (int q = 0; q < V; ++q) blk[c * V + q] = e[q];
    }
  } else {
#pragma unroll
    for (int pq = 0; pq < NB; ++pq) blk[pq] = __ldg(vals + (size_t)t * NB + pq);
  }
}

template <typename T, int DB, int G>
__global__ void __launch_bounds__(256) bspmm_kernel(int n, const int* __restrict__ indptr,
                                                    const int* __restrict__ indices, const T* __restrict__ vals,
                                                    const T* __restrict__ X, T* __restrict__ Y,
                                                    const T* __restrict__ Z, int b, int ld, T alpha, T beta, T gamma,
                                                    int wshift) {
  constexpr int V = Vec<T>::V;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int W = 1 << wshift;
  const int i = (int)(warp * (32 >> wshift) + (lane >> wshift));
  const int sub = lane & (W - 1);
  if (i >= n) return;
  const int groups = b / V;
  bool on[G];
#pragma unroll
  for (int g = 0; g < G; ++g) on[g] = sub + W * g < groups;
  T acc[DB][G][V];
#pragma unroll
  for (int p = 0; p < DB; ++p)
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int v = 0; v < V; ++v) acc[p][g][v] = T(0);
  const int s = __ldg(indptr + i), e = __ldg(indptr + i + 1);
  for (int t = s; t < e; ++t) {
    const int j = __ldg(indices + t);
    T blk[DB * DB];
    load_block<T, DB>(vals, t, blk);
#pragma unroll
    for (int q = 0; q < DB; ++q) {
      const T* xr = X + ((size_t)j * DB + q) * ld;
#pragma unroll
      for (int g = 0; g < G; ++g) {
        if (!on[g]) continue;
        T x[V];
        vload(xr + (sub + W * g) * V, x);
#pragma unroll
        for (int p = 0; p < DB; ++p)
#pragma unroll
          for (int v = 0; v < V; ++v) acc[p][g][v] = fma(blk[p * DB + q], x[v], acc[p][g][v]);
      }
    }
  }
#pragma unroll
  for (int p = 0; p < DB; ++p)
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (!on[g]) continue;
      const size_t row = ((size_t)i * DB + p) * ld + (sub + W * g) * V;
      T out[V], x[V];
#pragma unroll
      for (int v = 0; v < V; ++v) out[v] = alpha * acc[p][g][v];
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

// Column-chunked form: warp w takes block row i = w / nch and the 32 column
// groups of chunk c = w % nch, one group per lane, so the accumulators stay at
// DB x V registers and every SM holds its full complement of warps; the chunks
// of a row are consecutive warps of one CTA (its indices and blocks come from
// L1 after the first).  U neighbours per iteration: all their loads are
// issued first, then the products in the row kernel's order (neighbour by
// neighbour, block column by block column), so every variant gives the same
// bits.
// RB: CTA = 8 consecutive rows x one column chunk, chunk-major grid (the
// rows of a CTA share most of their neighbours, and a chunk of X stays in L2
// while its row blocks run); otherwise the chunks of a row are consecutive
// warps.
template <typename T, int DB, int U, bool CG = false, bool RB = false>
__global__ void __launch_bounds__(256) bspmm_chunked_kernel(int n, int nch, const int* __restrict__ indptr,
                                                            const int* __restrict__ indices,
                                                            const T* __restrict__ vals, const T* __restrict__ X,
                                                            T* __restrict__ Y, const T* __restrict__ Z, int b, int ld,
                                                            T alpha, T beta, T gamma) {
  constexpr int V = Vec<T>::V;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  long long i;
  int chunk;
  if (RB) {
    const long long nrb = ((long long)n + 7) / 8;
    chunk = (int)(blockIdx.x / nrb);
    i = (blockIdx.x % nrb) * 8 + (threadIdx.x >> 5);
  } else {
    i = warp / nch;
    chunk = (int)(warp % nch);
  }
  if (i >= n) return;
  const int grp = chunk * 32 + lane;
  const bool on = grp < b / V;
  const int col = grp * V;
  T acc[DB][V];
#pragma unroll
  for (int p = 0; p < DB; ++p)
#pragma unroll
    for (int v = 0; v < V; ++v) acc[p][v] = T(0);
  const int s = __ldg(indptr + i), e = __ldg(indptr + i + 1);
  int t = s;
  for (; t + U <= e; t += U) {
    T blk[U][DB * DB], x[U][DB][V];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = __ldg(indices + t + u);
      load_block<T, DB>(vals, t + u, blk[u]);
      if (on)
#pragma unroll
        for (int q = 0; q < DB; ++q) vgather<T, CG>(X + ((size_t)j * DB + q) * ld + col, x[u][q]);
    }
    if (on)
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
    load_block<T, DB>(vals, t, blk);
    if (on)
#pragma unroll
      for (int q = 0; q < DB; ++q) {
        T x[V];
        vgather<T, CG>(X + ((size_t)j * DB + q) * ld + col, x);
#pragma unroll
        for (int p = 0; p < DB; ++p)
#pragma unroll
          for (int v = 0; v < V; ++v) acc[p][v] = fma(blk[p * DB + q], x[v], acc[p][v]);
      }
  }
  if (!on) return;
#pragma unroll
  for (int p = 0; p < DB; ++p) {
    const size_t row = ((size_t)i * DB + p) * ld + col;
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

// Tile-mapped form without staging: CTA (tile of 32 consecutive rows, one
// 128-byte column chunk), 8 lanes per row, chunk-major grid.  The rows of a
// tile share most of their neighbours (~131 distinct rows for ~570
// references at k = 15 on a surface, in the locality order), so after the
// first touch the gathered chunks come from L1, and no shared memory caps
// the occupancy.  Same accumulation order as the other variants.
template <typename T, int DB, int U, bool CG = false>
__global__ void __launch_bounds__(256) bspmm_tile_kernel(int n, int n_tiles, const int* __restrict__ indptr,
                                                         const int* __restrict__ indices, const T* __restrict__ vals,
                                                         const T* __restrict__ X, T* __restrict__ Y,
                                                         const T* __restrict__ Z, int b, int ld, T alpha, T beta,
                                                         T gamma) {
  constexpr int V = Vec<T>::V;
  constexpr int SEG = 128 / (int)sizeof(T);
  constexpr int G = SEG / V;  // 8 lanes per row
  const int tile = blockIdx.x % n_tiles, chunk = blockIdx.x / n_tiles;
  const int c0 = chunk * SEG;
  const int groups = min(G, (b - c0) / V);
  const int slot = threadIdx.x / G, g = threadIdx.x % G;
  const int i = tile * 32 + slot;
  if (i >= n) return;
  const bool on = g < groups;
  const int col = c0 + g * V;
  T acc[DB][V];
#pragma unroll
  for (int p = 0; p < DB; ++p)
#pragma unroll
    for (int v = 0; v < V; ++v) acc[p][v] = T(0);
  const int s = __ldg(indptr + i), e = __ldg(indptr + i + 1);
  int t = s;
  for (; t + U <= e; t += U) {
    T blk[U][DB * DB], x[U][DB][V];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = __ldg(indices + t + u);
      load_block<T, DB>(vals, t + u, blk[u]);
      if (on)
#pragma unroll
        for (int q = 0; q < DB; ++q) vgather<T, CG>(X + ((size_t)j * DB + q) * ld + col, x[u][q]);
    }
    if (on)
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
    load_block<T, DB>(vals, t, blk);
    if (on)
#pragma unroll
      for (int q = 0; q < DB; ++q) {
        T x[V];
        vgather<T, CG>(X + ((size_t)j * DB + q) * ld + col, x);
#pragma unroll
        for (int p = 0; p < DB; ++p)
#pragma unroll
          for (int v = 0; v < V; ++v) acc[p][v] = fma(blk[p * DB + q], x[v], acc[p][v]);
      }
  }
  if (!on) return;
#pragma unroll
  for (int p = 0; p < DB; ++p) {
    const size_t row = ((size_t)i * DB + p) * ld + col;
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

template <typename T, int U, bool CG = false>
int launch_tile(int n, int DB, const int* indptr, const int* indices, const T* vals, const T* X, T* Y, const T* Z,
                int b, int ld, T alpha, T beta, T gamma, cudaStream_t st) {
  constexpr int SEG = 128 / (int)sizeof(T);
  const int nt = (n + 31) / 32, nch = ceil_div(b, SEG);
  rvgp::note_launch();
#define RVGP_SPMM_T(DBv)                                                                                          \
  bspmm_tile_kernel<T, DBv, U, CG><<<(unsigned)((long long)nt * nch), 256, 0, st>>>(n, nt, indptr, indices, vals, X, Y, \
                                                                                 Z, b, ld, alpha, beta, gamma)
  switch (DB) {
    case 1: RVGP_SPMM_T(1); break;
    case 2: RVGP_SPMM_T(2); break;
    case 3: RVGP_SPMM_T(3); break;
    default: RVGP_SPMM_T(4);
  }
#undef RVGP_SPMM_T
  return check_launch("rvgp_bspmm");
}

template <typename T, int U, bool CG = false, bool RB = false>
int launch_chunked(int n, int DB, const int* indptr, const int* indices, const T* vals, const T* X, T* Y, const T* Z,
                   int b, int ld, T alpha, T beta, T gamma, cudaStream_t st) {
  constexpr int V = Vec<T>::V;
  const int nch = ceil_div(b / V, 32);
  const long long warps = (long long)n * nch;
  const int grid = RB ? (int)(((long long)n + 7) / 8 * nch) : ceil_div(warps * 32, 256);
  rvgp::note_launch();
#define RVGP_SPMM_C(DBv) \
  bspmm_chunked_kernel<T, DBv, U, CG, RB><<<grid, 256, 0, st>>>(n, nch, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma)
  switch (DB) {
    case 1: RVGP_SPMM_C(1); break;
    case 2: RVGP_SPMM_C(2); break;
    case 3: RVGP_SPMM_C(3); break;
    default: RVGP_SPMM_C(4);
  }
#undef RVGP_SPMM_C
  return check_launch("rvgp_bspmm");
}

template <typename T>
int launch_rows(int n, int DB, const int* indptr, const int* indices, const T* vals, const T* X, T* Y, const T* Z,
                int b, int ld, T alpha, T beta, T gamma, cudaStream_t st) {
  constexpr int V = Vec<T>::V;
  const int groups = b / V;
  const int G = groups <= 32 ? 1 : groups <= 64 ? 2 : groups <= 128 ? 4 : groups <= 256 ? 8 : 16;
  int wshift = 5;
  while (wshift > 0 && (1 << (wshift - 1)) >= groups) --wshift;
  const long long warps = ((long long)n + (32 >> wshift) - 1) / (32 >> wshift);
  const int grid = ceil_div(warps * 32, 256);
  rvgp::note_launch();
#define RVGP_SPMM_G(DBv, Gv) \
  bspmm_kernel<T, DBv, Gv><<<grid, 256, 0, st>>>(n, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, wshift)
#define RVGP_SPMM_DB(DBv)              \
  switch (G) {                         \
    case 1: RVGP_SPMM_G(DBv, 1); break; \
    case 2: RVGP_SPMM_G(DBv, 2); break; \
    case 4: RVGP_SPMM_G(DBv, 4); break; \
    case 8: RVGP_SPMM_G(DBv, 8); break; \
    default: RVGP_SPMM_G(DBv, 16);      \
  }
  switch (DB) {
    case 1: RVGP_SPMM_DB(1); break;
    case 2: RVGP_SPMM_DB(2); break;
    case 3: RVGP_SPMM_DB(3); break;
    default: RVGP_SPMM_DB(4);
  }
#undef RVGP_SPMM_DB
#undef RVGP_SPMM_G
  return check_launch("rvgp_bspmm");
}

// Column groups from which the chunked form is the default variant
// (RVGP_SPMM_CHUNK_MIN overrides it and turns the tuner off: 0 = always
// chunked, a large value = always row per warp).
int chunk_min_groups() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("RVGP_SPMM_CHUNK_MIN");
    v = e ? atoi(e) : 33;
  }
  return v;
}

bool overlaps(const void* a, const void* b, size_t bytes) {
  const char *x = static_cast<const char*>(a), *y = static_cast<const char*>(b);
  return x < y + bytes && y < x + bytes;
}

// Variants: 0 = row per warp (G groups per lane), 1 / 2 = column-chunked with
// 2 / 4 neighbours per iteration, 3 / 4 = tile-mapped with 2 / 4, 5 / 6 =
// chunked / tile-mapped (2 neighbours) with the neighbour gathers cached in
// L2 only (a gather that misses L1 costs the L1 data path a fill and a read;
// L2 has headroom), 7 = chunked with 8-row blocks per CTA, chunk-major.  The
// tuner (autotune.cuh) picks one per shape class (RVGP_SPMM_VARIANT=v forces
// one); the same bits come out of all eight.
template <typename T>
int run_variant(int v, int n, int DB, const int* indptr, const int* indices, const T* vals, const T* X, T* Y,
                const T* Z, int b, int ld, T alpha, T beta, T gamma, cudaStream_t st) {
  switch (v) {
    case 0: return launch_rows<T>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    case 1: return launch_chunked<T, 2>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    case 2: return launch_chunked<T, 4>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    case 3: return launch_tile<T, 2>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    case 4: return launch_tile<T, 4>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    case 5: return launch_chunked<T, 2, true>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    case 6: return launch_tile<T, 2, true>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    default:
      return launch_chunked<T, 2, false, true>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
  }
}

template <typename T>
int check_args(int DB, const T* X, const T* Y, const T* Z, int b, int ld) {
  constexpr int V = Vec<T>::V;
  RVGP_CHECK_ARG(b % V == 0 && ld % V == 0 && b <= ld, "rvgp_bspmm: b=%d and ld=%d must be multiples of %d", b, ld, V);
  RVGP_CHECK_ARG(((uintptr_t)X | (uintptr_t)Y | (uintptr_t)(Z ? Z : X)) % 16 == 0, "rvgp_bspmm: 16-byte alignment");
  RVGP_CHECK_ARG(b / V <= 32 * 16, "rvgp_bspmm: block width b=%d too large", b);
  RVGP_CHECK_ARG(DB >= 1 && DB <= 4, "rvgp_bspmm: block size %d not supported (1..4)", DB);
  return RVGP_OK;
}

template <typename T>
int launch(int n, int DB, const int* indptr, const int* indices, const T* vals, const T* X, T* Y, const T* Z, int b,
           int ld, T alpha, T beta, T gamma, cudaStream_t st) {
  constexpr int V = Vec<T>::V;
  if (int rc = check_args<T>(DB, X, Y, Z, b, ld)) return rc;
  const int groups = b / V;
  auto run = [&](int v) -> int {
    return run_variant<T>(v, n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
  };
  int def = groups >= chunk_min_groups() ? 1 : 0;
  if (const char* fv = getenv("RVGP_SPMM_VARIANT")) def = std::min(7, std::max(0, atoi(fv)));  // tests: one variant
  // tuning runs the product several times into Y: only when Y overlaps neither input
  const size_t bytes = (size_t)n * DB * ld * sizeof(T);
  const bool independent = !overlaps(Y, X, bytes) && !(Z && overlaps(Y, Z, bytes));
  int v = def;
  if (independent && getenv("RVGP_SPMM_CHUNK_MIN") == nullptr && getenv("RVGP_SPMM_VARIANT") == nullptr) {
    char key[160];
    snprintf(key, sizeof(key), "bspmm %s DB%d b%d n2^%d", sizeof(T) == 4 ? "f32" : "f64", DB, b,
             autotune::log2_bucket(n));
    v = autotune::tune(key, 8, def, st, 3, run);
    if (v < 0) return v;
  }
  return run(v);
}

// ------------------------------------------------------------ tiled form
// The product over one matrix is repeated hundreds of times (Chebyshev
// filter), so a plan built once per matrix pays: block rows are cut into
// tiles of kTileRows consecutive rows (in the locality-preserving order, a
// compact patch), and for every tile the sorted set of distinct block rows
// its entries reference (its halo, ~4x fewer than the references at k = 15
// on a surface) and, per entry, the position of its column in that set.
// CTA (tile, chunk) copies the halo's rows, one 128-byte column chunk of
// them, into shared memory (cp.async) and forms the tile's output rows from
// there; the grid runs chunk by chunk, so one chunk of X (n*DB*128 bytes)
// stays in L2 while the tiles that gather from it run, and X is read from
// HBM about once per product.  Tiles whose halo or entry count exceeds the
// shared-memory budget are marked (halo size -1) and gather from global
// memory.  Each output row accumulates neighbour by neighbour and block
// column by block column as the other variants do: the same bits.
constexpr int kTileRows = 32;
constexpr int kHaloRows = 576;      // halo rows x DB per tile (72 KB of 128-byte chunks)
constexpr int kPlanMaxEntries = 2048;
constexpr int kSegBytes = 128;
constexpr int kGroupRows = 4;       // block rows per group of the grouped form
constexpr int kMergeWindow = 64;    // look-ahead of the group merge

__host__ __device__ inline int plan_hmax(int DB) { return kHaloRows / DB; }
inline int plan_tiles(int n) { return (n + kTileRows - 1) / kTileRows; }
inline int plan_groups(int n) { return (n + kGroupRows - 1) / kGroupRows; }

// The plan holds both forms' data: per tile of kTileRows rows its halo and the
// local column of every entry (tiled form); per group of kGroupRows rows the
// merged neighbour list (grouped form).
struct PlanView {
  int* tile_h;
  int* halo;
  unsigned short* lidx;
  int* gcnt;  // merged entries of group g, at gcol[indptr[g * kGroupRows] ...]
  int* gcol;  // nnz slots: the merged entry's block column
  int* gidx;  // nnz x kGroupRows: per row of the group, its CSR entry at that column, or -1
};

size_t plan_bytes_needed(int n, int DB, long long nnz) {
  Workspace ws(nullptr, 0);
  ws.take<int>(plan_tiles(n));
  ws.take<int>((size_t)plan_tiles(n) * plan_hmax(DB));
  ws.take<unsigned short>((size_t)nnz);
  ws.take<int>(plan_groups(n));
  ws.take<int>((size_t)nnz);
  ws.take<int>((size_t)nnz * kGroupRows);
  return ws.used;
}

PlanView plan_view(void* plan, size_t bytes, int n, int DB, long long nnz) {
  Workspace ws(plan, bytes);
  PlanView v;
  v.tile_h = ws.take<int>(plan_tiles(n));
  v.halo = ws.take<int>((size_t)plan_tiles(n) * plan_hmax(DB));
  v.lidx = ws.take<unsigned short>((size_t)nnz);
  v.gcnt = ws.take<int>(plan_groups(n));
  v.gcol = ws.take<int>((size_t)nnz);
  v.gidx = ws.take<int>((size_t)nnz * kGroupRows);
  return v;
}

// ------------------------------------------------------------ grouped form
// The rows of a group (consecutive in the locality-preserving order) share
// most of their neighbours: at k = 15 on a surface, 4 rows reference ~54 %
// as many distinct block rows as entries.  The plan merges the group's CSR
// rows into one list of columns, each with the entry of every row that has
// it, by taking list heads only, so every row's entries stay in its CSR order
// (any order of the input rows is valid; when the rows are sorted by one
// key, as CSR rows are, the merge finds every shared column).  A head is
// taken together with the equal heads of the other rows unless it occurs
// further down one of them, in which case another head goes first; when every
// head does (rows in conflicting orders), the first row's head goes alone.
// The search looks kMergeWindow entries ahead (a hub row costs no more; a
// match further down is only a missed share).  One thread per group; the
// merged list of group g fills the group's own entry range, which it never
// outgrows (each merged entry takes at least one).
__global__ void __launch_bounds__(256) spmm_group_plan_kernel(int n, int ngroups, const int* __restrict__ indptr,
                                                              const int* __restrict__ indices, int* __restrict__ gcnt,
                                                              int* __restrict__ gcol, int* __restrict__ gidx) {
  constexpr int GR = kGroupRows;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngroups) return;
  const int i0 = g * GR;
  int ptr[GR], end[GR];
#pragma unroll
  for (int r = 0; r < GR; ++r) {
    const bool on = i0 + r < n;
    ptr[r] = on ? indptr[i0 + r] : 0;
    end[r] = on ? indptr[i0 + r + 1] : 0;
  }
  const int base = indptr[i0];
  int out = base;
  while (true) {
    int chosen = -1, first = -1;
#pragma unroll
    for (int r = 0; r < GR; ++r) {
      if (chosen >= 0 || ptr[r] >= end[r]) continue;
      if (first < 0) first = r;
      const int c = indices[ptr[r]];
      bool later = false;
#pragma unroll
      for (int q = 0; q < GR; ++q) {
        if (q == r || later) continue;
        const int t1 = min(end[q], ptr[q] + 1 + kMergeWindow);
        for (int t = ptr[q] + 1; t < t1; ++t)
          if (indices[t] == c) {
            later = true;
            break;
          }
      }
      if (!later) chosen = r;
    }
    if (first < 0) break;
    const bool alone = chosen < 0;
    if (alone) chosen = first;
    int c = 0;
#pragma unroll
    for (int r = 0; r < GR; ++r)
      if (r == chosen) c = indices[ptr[r]];
    int id[GR];
#pragma unroll
    for (int r = 0; r < GR; ++r) {
      const bool take = ptr[r] < end[r] && (alone ? r == chosen : indices[ptr[r]] == c);
      id[r] = take ? ptr[r] : -1;
      ptr[r] += take ? 1 : 0;
    }
    gcol[out] = c;
    *reinterpret_cast<int4*>(gidx + (size_t)out * GR) = make_int4(id[0], id[1], id[2], id[3]);
    ++out;
  }
  gcnt[g] = out - base;
}

// Warp per (group, 32-column-group chunk), as the chunked form, with the
// accumulators of the group's GR rows: a merged entry's X rows are gathered
// once and applied to every row that has the entry.  U entries per
// iteration, loads first; each row accumulates its own entries in CSR order,
// neighbour by neighbour and block column by block column: the same bits as
// the other variants.
template <typename T, int DB, int U>
__global__ void __launch_bounds__(256) bspmm_group_kernel(int n, int nch, const int* __restrict__ gcnt,
                                                          const int* __restrict__ gcol,
                                                          const int* __restrict__ gidx,
                                                          const int* __restrict__ indptr,
                                                          const T* __restrict__ vals, const T* __restrict__ X,
                                                          T* __restrict__ Y, const T* __restrict__ Z, int b, int ld,
                                                          T alpha, T beta, T gamma) {
  constexpr int V = Vec<T>::V;
  constexpr int GR = kGroupRows;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const long long g = warp / nch;
  const int chunk = (int)(warp % nch);
  if (g * GR >= n) return;
  const int grp = chunk * 32 + lane;
  const bool on = grp < b / V;
  const int col = grp * V;
  T acc[GR][DB][V];
#pragma unroll
  for (int r = 0; r < GR; ++r)
#pragma unroll
    for (int p = 0; p < DB; ++p)
#pragma unroll
      for (int v = 0; v < V; ++v) acc[r][p][v] = T(0);
  const int s = __ldg(indptr + g * GR), e = s + __ldg(gcnt + g);
  auto apply = [&](const int4& id4, const T (&x)[DB][V]) {
    const int id[GR] = {id4.x, id4.y, id4.z, id4.w};
#pragma unroll
    for (int r = 0; r < GR; ++r)
      if (id[r] >= 0) {  // uniform in the warp
        T blk[DB * DB];
        load_block<T, DB>(vals, id[r], blk);
#pragma unroll
        for (int q = 0; q < DB; ++q)
#pragma unroll
          for (int p = 0; p < DB; ++p)
#pragma unroll
            for (int v = 0; v < V; ++v) acc[r][p][v] = fma(blk[p * DB + q], x[q][v], acc[r][p][v]);
      }
  };
  int t = s;
  for (; t + U <= e; t += U) {
    T x[U][DB][V];
    int4 id[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = __ldg(gcol + t + u);
      id[u] = __ldg(reinterpret_cast<const int4*>(gidx) + t + u);
      if (on)
#pragma unroll
        for (int q = 0; q < DB; ++q) vgather<T, false>(X + ((size_t)j * DB + q) * ld + col, x[u][q]);
    }
    if (on)
#pragma unroll
      for (int u = 0; u < U; ++u) apply(id[u], x[u]);
  }
  for (; t < e; ++t) {
    T x[DB][V];
    const int j = __ldg(gcol + t);
    const int4 id = __ldg(reinterpret_cast<const int4*>(gidx) + t);
    if (on) {
#pragma unroll
      for (int q = 0; q < DB; ++q) vgather<T, false>(X + ((size_t)j * DB + q) * ld + col, x[q]);
      apply(id, x);
    }
  }
  if (!on) return;
#pragma unroll
  for (int r = 0; r < GR; ++r) {
    const long long i = g * GR + r;
    if (i >= n) break;
#pragma unroll
    for (int p = 0; p < DB; ++p) {
      const size_t row = ((size_t)i * DB + p) * ld + col;
      T out[V], x[V];
#pragma unroll
      for (int v = 0; v < V; ++v) out[v] = alpha * acc[r][p][v];
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
}

template <typename T, int U>
int launch_group(int n, int DB, const PlanView& pv, const int* indptr, const T* vals, const T* X, T* Y, const T* Z,
                 int b, int ld, T alpha, T beta, T gamma, cudaStream_t st) {
  constexpr int V = Vec<T>::V;
  const int nch = ceil_div(b / V, 32);
  const long long warps = (long long)plan_groups(n) * nch;
  const unsigned grid = (unsigned)ceil_div(warps * 32, 256ll);
  rvgp::note_launch();
  switch (DB) {
#define RVGP_GRP(DBv)                                                                                              \
  case DBv:                                                                                                        \
    bspmm_group_kernel<T, DBv, U><<<grid, 256, 0, st>>>(n, nch, pv.gcnt, pv.gcol, pv.gidx, indptr, vals, X, Y, Z,  \
                                                        b, ld, alpha, beta, gamma);                                \
    break;
    RVGP_GRP(1)
    RVGP_GRP(2)
    RVGP_GRP(3)
    default: RVGP_GRP(4)
#undef RVGP_GRP
  }
  return check_launch("rvgp_bspmm (grouped)");
}

__global__ void __launch_bounds__(256) spmm_plan_kernel(int n, int hmax, const int* __restrict__ indptr,
                                                        const int* __restrict__ indices, int* __restrict__ tile_h,
                                                        int* __restrict__ halo, unsigned short* __restrict__ lidx) {
  __shared__ int keys[kPlanMaxEntries];
  __shared__ int uniq[kPlanMaxEntries];
  __shared__ int wsum[8];
  const int tile = blockIdx.x, tid = threadIdx.x;
  const int i0 = tile * kTileRows, i1 = min(n, i0 + kTileRows);
  const int e0 = indptr[i0], ne = indptr[i1] - e0;
  if (ne > kPlanMaxEntries) {
    if (tid == 0) tile_h[tile] = -1;
    return;
  }
  int P2 = 1;
  while (P2 < ne) P2 <<= 1;
  for (int k = tid; k < P2; k += 256) keys[k] = k < ne ? indices[e0 + k] : INT_MAX;
  __syncthreads();
  for (int size = 2; size <= P2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int k = tid; k < P2 / 2; k += 256) {
        const int lo = 2 * stride * (k / stride) + (k % stride), hi = lo + stride;
        const bool asc = (lo & size) == 0;
        const int a = keys[lo], b = keys[hi];
        if ((a > b) == asc) {
          keys[lo] = b;
          keys[hi] = a;
        }
      }
      __syncthreads();
    }
  // distinct keys: exclusive scan of the first-occurrence flags, runs of
  // kPlanMaxEntries / 256 = 8 consecutive keys per thread
  constexpr int RUN = kPlanMaxEntries / 256;
  int flags[RUN], cnt = 0;
#pragma unroll
  for (int r = 0; r < RUN; ++r) {
    const int k = tid * RUN + r;
    flags[r] = (k < ne && (k == 0 || keys[k] != keys[k - 1])) ? 1 : 0;
    cnt += flags[r];
  }
  const int lane = tid & 31, warp = tid >> 5;
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  int base = 0, total = 0;
  for (int w = 0; w < 8; ++w) {
    if (w < warp) base += wsum[w];
    total += wsum[w];
  }
  int pos = base + incl - cnt;
#pragma unroll
  for (int r = 0; r < RUN; ++r)
    if (flags[r]) uniq[pos++] = keys[tid * RUN + r];
  __syncthreads();
  if (total > hmax) {
    if (tid == 0) tile_h[tile] = -1;
    return;
  }
  for (int k = tid; k < total; k += 256) halo[(size_t)tile * hmax + k] = uniq[k];
  for (int k = tid; k < ne; k += 256) {
    const int c = indices[e0 + k];
    int lo = 0, hi = total - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (uniq[mid] < c)
        lo = mid + 1;
      else
        hi = mid;
    }
    lidx[e0 + k] = (unsigned short)lo;
  }
  if (tid == 0) tile_h[tile] = total;
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename T, int DB, int U>
__global__ void __launch_bounds__(256) bspmm_tiled_kernel(int n, int n_tiles, const int* __restrict__ tile_h,
                                                          const int* __restrict__ halo,
                                                          const unsigned short* __restrict__ lidx,
                                                          const int* __restrict__ indptr,
                                                          const int* __restrict__ indices,
                                                          const T* __restrict__ vals, const T* __restrict__ X,
                                                          T* __restrict__ Y, const T* __restrict__ Z, int b, int ld,
                                                          T alpha, T beta, T gamma) {
  constexpr int V = Vec<T>::V;
  constexpr int SEG = kSegBytes / (int)sizeof(T);  // chunk width in elements
  constexpr int G = SEG / V;                       // lanes per row (8)
  constexpr int HM = kHaloRows / DB;
  extern __shared__ __align__(16) unsigned char tiled_smem[];
  T* xs = reinterpret_cast<T*>(tiled_smem);
  const int tile = blockIdx.x % n_tiles, chunk = blockIdx.x / n_tiles;
  const int c0 = chunk * SEG;
  const int groups = min(G, (b - c0) / V);
  const int h = __ldg(tile_h + tile);
  if (h > 0) {
    const int* hl = halo + (size_t)tile * HM;
    for (int e = threadIdx.x; e < h * DB * G; e += 256) {
      const int r = e / G, g = e % G;  // r = halo row * DB + q
      if (g < groups) {
        const int j = __ldg(hl + r / DB), q = r % DB;
        cp_async16(xs + (size_t)r * SEG + g * V, X + ((size_t)j * DB + q) * ld + c0 + g * V);
      }
    }
    cp_async_wait_all();
    __syncthreads();
  }
  const int slot = threadIdx.x / G, g = threadIdx.x % G;
  const int i = tile * kTileRows + slot;
  if (i >= n) return;  // no barrier below
  const bool on = g < groups;
  const bool staged = h >= 0;
  const int col = c0 + g * V;
  T acc[DB][V];
#pragma unroll
  for (int p = 0; p < DB; ++p)
#pragma unroll
    for (int v = 0; v < V; ++v) acc[p][v] = T(0);
  const int s = __ldg(indptr + i), e = __ldg(indptr + i + 1);
  int t = s;
  for (; t + U <= e; t += U) {
    T blk[U][DB * DB], x[U][DB][V];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      load_block<T, DB>(vals, t + u, blk[u]);
      if (on) {
        if (staged) {
          const int li = __ldg(lidx + t + u);
#pragma unroll
          for (int q = 0; q < DB; ++q) vload(xs + (size_t)(li * DB + q) * SEG + g * V, x[u][q]);
        } else {
          const int j = __ldg(indices + t + u);
#pragma unroll
          for (int q = 0; q < DB; ++q) vload(X + ((size_t)j * DB + q) * ld + col, x[u][q]);
        }
      }
    }
    if (on)
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
    T blk[DB * DB], x[DB][V];
    load_block<T, DB>(vals, t, blk);
    if (on) {
      if (staged) {
        const int li = __ldg(lidx + t);
#pragma unroll
        for (int q = 0; q < DB; ++q) vload(xs + (size_t)(li * DB + q) * SEG + g * V, x[q]);
      } else {
        const int j = __ldg(indices + t);
#pragma unroll
        for (int q = 0; q < DB; ++q) vload(X + ((size_t)j * DB + q) * ld + col, x[q]);
      }
#pragma unroll
      for (int q = 0; q < DB; ++q)
#pragma unroll
        for (int p = 0; p < DB; ++p)
#pragma unroll
          for (int v = 0; v < V; ++v) acc[p][v] = fma(blk[p * DB + q], x[q][v], acc[p][v]);
    }
  }
  if (!on) return;
#pragma unroll
  for (int p = 0; p < DB; ++p) {
    const size_t row = ((size_t)i * DB + p) * ld + col;
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

template <typename T, int DB>
int launch_tiled_db(int n, const PlanView& pv, const int* indptr, const int* indices, const T* vals, const T* X, T* Y,
                    const T* Z, int b, int ld, T alpha, T beta, T gamma, cudaStream_t st) {
  constexpr int SEG = kSegBytes / (int)sizeof(T);
  const int nt = plan_tiles(n), nch = ceil_div(b, SEG);
  const size_t smem = (size_t)kHaloRows / DB * DB * kSegBytes;
  if (raise_dyn_smem((const void*)bspmm_tiled_kernel<T, DB, 2>, smem) != cudaSuccess)
    return check_launch("rvgp_bspmm (tiled)");
  rvgp::note_launch();
  bspmm_tiled_kernel<T, DB, 2><<<(unsigned)((long long)nt * nch), 256, smem, st>>>(
      n, nt, pv.tile_h, pv.halo, pv.lidx, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma);
  return check_launch("rvgp_bspmm (tiled)");
}

// Through a plan: the eight plain variants, 8 = tiled (shared-memory halo),
// 9 / 10 = grouped with 2 / 1 merged entries per iteration.  The tuner picks
// one per shape class (RVGP_SPMM_VARIANT=v forces one); the same bits come
// out of all eleven.
template <typename T>
int launch_planned(const void* plan, size_t plan_bytes, int n, int DB, long long nnz, const int* indptr,
                   const int* indices, const T* vals, const T* X, T* Y, const T* Z, int b, int ld, T alpha, T beta,
                   T gamma, cudaStream_t st) {
  if (int rc = check_args<T>(DB, X, Y, Z, b, ld)) return rc;
  RVGP_CHECK_ARG(n >= 1 && nnz >= 0 && plan_bytes >= plan_bytes_needed(n, DB, nnz),
                 "rvgp_bspmm_planned: plan of %zu bytes needed", plan_bytes_needed(n, DB, nnz));
  const PlanView pv = plan_view(const_cast<void*>(plan), plan_bytes, n, DB, nnz);
  auto run = [&](int v) -> int {
    if (v < 8) return run_variant<T>(v, n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    if (v == 9) return launch_group<T, 2>(n, DB, pv, indptr, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    if (v == 10) return launch_group<T, 1>(n, DB, pv, indptr, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    switch (DB) {
      case 1: return launch_tiled_db<T, 1>(n, pv, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
      case 2: return launch_tiled_db<T, 2>(n, pv, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
      case 3: return launch_tiled_db<T, 3>(n, pv, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
      default: return launch_tiled_db<T, 4>(n, pv, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
    }
  };
  int def = 9;
  if (const char* fv = getenv("RVGP_SPMM_VARIANT")) def = std::min(10, std::max(0, atoi(fv)));
  const size_t bytes = (size_t)n * DB * ld * sizeof(T);
  const bool independent = !overlaps(Y, X, bytes) && !(Z && overlaps(Y, Z, bytes));
  int v = def;
  if (independent && getenv("RVGP_SPMM_CHUNK_MIN") == nullptr && getenv("RVGP_SPMM_VARIANT") == nullptr) {
    char key[160];
    snprintf(key, sizeof(key), "bspmm-plan %s DB%d b%d n2^%d", sizeof(T) == 4 ? "f32" : "f64", DB, b,
             autotune::log2_bucket(n));
    v = autotune::tune(key, 11, def, st, 3, run);
    if (v < 0) return v;
  }
  return run(v);
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

size_t spmm_plan_bytes(int n, int DB, long long nnz) {
  if (n < 1 || DB < 1 || DB > 4 || nnz < 0) return 0;
  return plan_bytes_needed(n, DB, nnz);
}

int spmm_plan_build(int n, int DB, const int* indptr, const int* indices, long long nnz, void* plan,
                    size_t plan_bytes, cudaStream_t st) {
  RVGP_CHECK_ARG(indptr && indices && plan, "rvgp_spmm_plan_build: null pointer");
  RVGP_CHECK_ARG(n >= 1 && DB >= 1 && DB <= 4 && nnz >= 0, "rvgp_spmm_plan_build: bad n=%d or DB=%d", n, DB);
  RVGP_CHECK_ARG(plan_bytes >= spmm_plan_bytes(n, DB, nnz), "rvgp_spmm_plan_build: plan of %zu bytes needed",
                 spmm_plan_bytes(n, DB, nnz));
  const PlanView pv = plan_view(plan, plan_bytes, n, DB, nnz);
  rvgp::note_launch();
  spmm_plan_kernel<<<plan_tiles(n), 256, 0, st>>>(n, plan_hmax(DB), indptr, indices, pv.tile_h, pv.halo, pv.lidx);
  rvgp::note_launch();
  spmm_group_plan_kernel<<<ceil_div(plan_groups(n), 256), 256, 0, st>>>(n, plan_groups(n), indptr, indices, pv.gcnt,
                                                                      pv.gcol, pv.gidx);
  return check_launch("rvgp_spmm_plan_build");
}

int bspmm_planned_f32(const void* plan, size_t plan_bytes, int n, int DB, long long nnz, const int* indptr,
                      const int* indices, const float* vals, const float* X, float* Y, const float* Z, int b, int ld,
                      float alpha, float beta, float gamma, cudaStream_t st) {
  if (!plan) return launch<float>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
  return launch_planned<float>(plan, plan_bytes, n, DB, nnz, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma,
                               st);
}
int bspmm_planned_f64(const void* plan, size_t plan_bytes, int n, int DB, long long nnz, const int* indptr,
                      const int* indices, const double* vals, const double* X, double* Y, const double* Z, int b,
                      int ld, double alpha, double beta, double gamma, cudaStream_t st) {
  if (!plan) return launch<double>(n, DB, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta, gamma, st);
  return launch_planned<double>(plan, plan_bytes, n, DB, nnz, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta,
                                gamma, st);
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

// Bytes of the planned product's plan for a block-CSR matrix of n block rows
// (DB x DB blocks) and nnz stored blocks.
RVGP_API size_t rvgp_spmm_plan_bytes(int n, int DB, long long nnz) { return rvgp::spmm_plan_bytes(n, DB, nnz); }

// Builds the plan (per tile of 32 block rows: its halo of distinct columns
// and the local column of every entry; per group of 4 block rows: the merged
// list of their columns with each row's entry there) into caller memory.
// Stream-ordered.
RVGP_API int rvgp_spmm_plan_build(int n, int DB, const int* indptr, const int* indices, long long nnz, void* plan,
                                  size_t plan_bytes, void* stream) {
  return rvgp::spmm_plan_build(n, DB, indptr, indices, nnz, plan, plan_bytes, rvgp::as_stream(stream));
}

// rvgp_bspmm_f32 / _f64 through a plan of the same matrix (null plan: the
// plain variants); the tuner also considers the tiled and grouped forms.
// The same bits as rvgp_bspmm_*.
RVGP_API int rvgp_bspmm_planned_f32(const void* plan, size_t plan_bytes, int n, int DB, long long nnz,
                                    const int* indptr, const int* indices, const float* vals, const float* X,
                                    float* Y, const float* Z, int b, int ld, float alpha, float beta, float gamma,
                                    void* stream) {
  return rvgp::bspmm_planned_f32(plan, plan_bytes, n, DB, nnz, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta,
                                 gamma, rvgp::as_stream(stream));
}
RVGP_API int rvgp_bspmm_planned_f64(const void* plan, size_t plan_bytes, int n, int DB, long long nnz,
                                    const int* indptr, const int* indices, const double* vals, const double* X,
                                    double* Y, const double* Z, int b, int ld, double alpha, double beta,
                                    double gamma, void* stream) {
  return rvgp::bspmm_planned_f64(plan, plan_bytes, n, DB, nnz, indptr, indices, vals, X, Y, Z, b, ld, alpha, beta,
                                 gamma, rvgp::as_stream(stream));
}
