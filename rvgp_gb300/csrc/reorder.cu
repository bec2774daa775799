// Locality-preserving renumbering of the points for the eigensolver's sparse
// products, and the matching permutations of a block-CSR matrix and of
// eigenvector rows.
//
// The block SpMM gathers, for every block row, the rows of X of all its
// neighbours.  In the caller's (arbitrary) point order consecutive block rows
// have unrelated neighbours, so every gather goes to L2.  Renumbered along a
// Morton (Z-order) curve of the coordinates, consecutive rows are spatial
// neighbours and share most of their neighbours, so a CTA that takes a run of
// consecutive rows finds most gathered rows already in L1.  The spectrum is
// invariant under the renumbering; eigenvectors are permuted back row by row.
//
// Morton code: the three coordinates of largest extent, 10 bits each, over
// the bounding box.  Sort: stable LSD radix sort of the 30-bit codes, 8 bits
// per pass (per-tile digit histograms, one exclusive scan, a stable
// scatter), so equal codes keep increasing point index and the order is
// deterministic.
#include "common.cuh"
#include "scan.cuh"
#include <float.h>
#include <vector>
#include <algorithm>
#include <cstring>

namespace rvgp {
namespace {

constexpr int kTile = 1024;   // keys per CTA in the radix passes
constexpr int kSortThreads = 256;
constexpr int kDigits = 256;

__device__ __forceinline__ unsigned long long ordered_bits(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_ordered(unsigned long long b) {
  return __longlong_as_double((long long)((b >> 63) ? (b & 0x7fffffffffffffffull) : ~b));
}

// per-dimension min and max (order-independent atomics on order-preserving bits)
__global__ void bbox_kernel(const double* __restrict__ X, int n, int D, unsigned long long* __restrict__ mm) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n * D;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e % D);
    const unsigned long long b = ordered_bits(X[e]);
    atomicMin(&mm[2 * j], b);
    atomicMax(&mm[2 * j + 1], b);
  }
}

// The same with per-thread extremes (D <= 256): T = a multiple of D threads
// per CTA and a grid stride that is one too, so every thread stays on one
// coordinate; the CTA combines its threads in shared memory and then makes
// one global atomic per coordinate (the per-element form above serialises on
// 2 D addresses).
__global__ void bbox_kernel_rows(const double* __restrict__ X, int n, int D, unsigned long long* __restrict__ mm) {
  __shared__ unsigned long long smin[256], smax[256];
  const int T = (blockDim.x / D) * D;
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    smin[j] = ~0ull;
    smax[j] = 0ull;
  }
  __syncthreads();
  if ((int)threadIdx.x < T) {
    const long long start = (long long)blockIdx.x * T + threadIdx.x;
    const long long stride = (long long)gridDim.x * T;
    unsigned long long lo = ~0ull, hi = 0ull;
    for (long long e = start; e < (long long)n * D; e += stride) {
      const unsigned long long b = ordered_bits(X[e]);
      lo = b < lo ? b : lo;
      hi = b > hi ? b : hi;
    }
    const int j = (int)(start % D);
    atomicMin(&smin[j], lo);
    atomicMax(&smax[j], hi);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    atomicMin(&mm[2 * j], smin[j]);
    atomicMax(&mm[2 * j + 1], smax[j]);
  }
}

__global__ void bbox_init(unsigned long long* mm, int D) {
  for (int j = threadIdx.x; j < D; j += blockDim.x) {
    mm[2 * j] = ~0ull;
    mm[2 * j + 1] = 0ull;
  }
}

__device__ __forceinline__ unsigned spread3(unsigned v) {  // 10 bits -> every third bit
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void morton_kernel(const double* __restrict__ X, int n, int D, int3 dims, int ndims,
                              const unsigned long long* __restrict__ mm, unsigned* __restrict__ key,
                              int* __restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int dd[3] = {dims.x, dims.y, dims.z};
  unsigned code = 0;
  for (int q = 0; q < ndims; ++q) {
    const int j = dd[q];
    const double lo = from_ordered(mm[2 * j]), hi = from_ordered(mm[2 * j + 1]);
    const double t = hi > lo ? (X[(size_t)i * D + j] - lo) / (hi - lo) : 0.0;
    const unsigned c = (unsigned)fmin(1023.0, fmax(0.0, t * 1024.0));
    code |= spread3(c) << q;
  }
  key[i] = code;
  val[i] = i;
}

// counts[d * ntiles + tile] = keys of this tile with digit d
__global__ void __launch_bounds__(kSortThreads) digit_hist(const unsigned* __restrict__ key, int n, int shift,
                                                           int ntiles, int* __restrict__ counts) {
  __shared__ int h[kDigits];
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) h[d] = 0;
  __syncthreads();
  const int base = blockIdx.x * kTile;
  for (int e = threadIdx.x; e < kTile && base + e < n; e += kSortThreads) atomicAdd(&h[(key[base + e] >> shift) & 255], 1);
  __syncthreads();
  for (int d = threadIdx.x; d < kDigits; d += kSortThreads) counts[d * ntiles + blockIdx.x] = h[d];
}

// stable scatter: thread d walks the tile in order and places its digit's keys
__global__ void __launch_bounds__(kDigits) digit_scatter(const unsigned* __restrict__ key, const int* __restrict__ val,
                                                        int n, int shift, int ntiles, const int* __restrict__ offs,
                                                        unsigned* __restrict__ okey, int* __restrict__ oval) {
  __shared__ unsigned sk[kTile];
  __shared__ int sv[kTile];
  const int base = blockIdx.x * kTile;
  const int cnt = min(kTile, n - base);
  for (int e = threadIdx.x; e < cnt; e += kDigits) {
    sk[e] = key[base + e];
    sv[e] = val[base + e];
  }
  __syncthreads();
  const unsigned d = threadIdx.x;
  int pos = offs[d * ntiles + blockIdx.x];
  for (int e = 0; e < cnt; ++e)
    if (((sk[e] >> shift) & 255u) == d) {
      okey[pos] = sk[e];
      oval[pos] = sv[e];
      ++pos;
    }
}

__global__ void invert_perm(const int* __restrict__ perm, int n, int* __restrict__ rank) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rank[perm[i]] = i;
}

// row lengths of the renumbered matrix
__global__ void perm_lengths(const int* __restrict__ indptr, const int* __restrict__ perm, int n,
                             int* __restrict__ len) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) len[r] = indptr[perm[r] + 1] - indptr[perm[r]];
}

// one warp per new row: copy its entries with renumbered columns
__global__ void perm_scatter(const int* __restrict__ indptr, const int* __restrict__ indices,
                             const double* __restrict__ v64, const float* __restrict__ v32, int DB,
                             const int* __restrict__ perm, const int* __restrict__ rank, const int* __restrict__ nptr,
                             int n, int* __restrict__ nidx, double* __restrict__ n64, float* __restrict__ n32) {
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= n) return;
  const int o = perm[r];
  const int s = indptr[o], e = indptr[o + 1], t0 = nptr[r];
  const int bb = DB * DB;
  for (int t = s + lane; t < e; t += 32) nidx[t0 + (t - s)] = rank[indices[t]];
  for (int q = lane; q < (e - s) * bb; q += 32) {
    n64[(size_t)t0 * bb + q] = v64[(size_t)s * bb + q];
    if (v32) n32[(size_t)t0 * bb + q] = v32[(size_t)s * bb + q];
  }
}

// dst[(i*DB + q), :] = src[(rank[i]*DB + q), :]  (rows of width m, ld each)
__global__ void unpermute_rows(const double* __restrict__ src, int lds, const int* __restrict__ rank, int n, int DB,
                               int m, double* __restrict__ dst, int ldd) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * DB * m) return;
  const long long row = e / m;
  const int j = (int)(e % m);
  const int i = (int)(row / DB), q = (int)(row % DB);
  dst[row * ldd + j] = src[((size_t)rank[i] * DB + q) * lds + j];
}

struct SortBufs {
  unsigned long long* mm;
  unsigned *k0, *k1;
  int *v0, *v1, *counts, *offs, *scan_ws;
};

SortBufs carve_sort(Workspace& ws, int n, int D) {
  SortBufs b;
  const int ntiles = ceil_div(n, kTile);
  b.mm = ws.take<unsigned long long>(2 * (size_t)D);
  b.k0 = ws.take<unsigned>(n);
  b.k1 = ws.take<unsigned>(n);
  b.v0 = ws.take<int>(n);
  b.v1 = ws.take<int>(n);
  b.counts = ws.take<int>((size_t)kDigits * ntiles);
  b.offs = ws.take<int>((size_t)kDigits * ntiles);
  b.scan_ws = ws.take<int>(scan_workspace(kDigits * ntiles) / sizeof(int) + 1);
  return b;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_locality_order_workspace(int n, int D) {
  Workspace ws(nullptr, 0);
  carve_sort(ws, n, D);
  return ws.used;
}

// perm (device, n): new position -> original point; rank (device, n): the
// inverse.  Synchronises once (reads the bounding box to pick the three
// coordinates of largest extent).
RVGP_API int rvgp_locality_order(const double* X, int n, int D, int* perm, int* rank, void* workspace,
                                 size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(X && perm && rank && n >= 1 && D >= 1, "rvgp_locality_order: bad arguments");
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_locality_order_workspace(n, D),
                 "rvgp_locality_order: workspace too small");
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  SortBufs b = carve_sort(ws, n, D);
  rvgp::note_launch();
  bbox_init<<<1, 128, 0, st>>>(b.mm, D);
  rvgp::note_launch();
  if (D <= 256)
    bbox_kernel_rows<<<std::min(num_sms() * 4, ceil_div((long long)n * D, 256)), 256, 0, st>>>(X, n, D, b.mm);
  else
    bbox_kernel<<<std::min(num_sms() * 4, ceil_div((long long)n * D, 256)), 256, 0, st>>>(X, n, D, b.mm);
  std::vector<unsigned long long> hm(2 * (size_t)D);
  if (read_back(hm.data(), b.mm, sizeof(unsigned long long) * 2 * D, st) != cudaSuccess) return check_launch("rvgp_locality_order");
  auto dec = [](unsigned long long v) {
    const unsigned long long bits = (v >> 63) ? (v & 0x7fffffffffffffffull) : ~v;
    double d;
    memcpy(&d, &bits, sizeof d);
    return d;
  };
  std::vector<int> order(D);
  for (int j = 0; j < D; ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return dec(hm[2 * a + 1]) - dec(hm[2 * a]) > dec(hm[2 * c + 1]) - dec(hm[2 * c]);
  });
  const int nd = std::min(3, D);
  int3 dims = make_int3(order[0], nd > 1 ? order[1] : 0, nd > 2 ? order[2] : 0);
  rvgp::note_launch();
  morton_kernel<<<ceil_div(n, 256), 256, 0, st>>>(X, n, D, dims, nd, b.mm, b.k0, b.v0);
  const int ntiles = ceil_div(n, kTile);
  unsigned *ka = b.k0, *kb = b.k1;
  int *va = b.v0, *vb = b.v1;
  for (int shift = 0; shift < 30; shift += 8) {
    rvgp::note_launch();
    digit_hist<<<ntiles, kSortThreads, 0, st>>>(ka, n, shift, ntiles, b.counts);
    exclusive_scan(b.counts, kDigits * ntiles, b.offs, nullptr, b.scan_ws, st);
    const bool last = shift + 8 >= 30;
    rvgp::note_launch();
    digit_scatter<<<ntiles, kDigits, 0, st>>>(ka, va, n, shift, ntiles, b.offs, kb, last ? perm : vb);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  rvgp::note_launch();
  invert_perm<<<ceil_div(n, 256), 256, 0, st>>>(perm, n, rank);
  RVGP_LAUNCH_CHECK("rvgp_locality_order");
  return RVGP_OK;
}

RVGP_API size_t rvgp_permute_csr_workspace(int n) {
  Workspace ws(nullptr, 0);
  ws.take<int>(n);
  ws.take<int>(scan_workspace(n) / sizeof(int) + 1);
  return ws.used;
}

// Renumbered block-CSR: new row r is old row perm[r]; columns c -> rank[c];
// each row's entries keep their order.  out_indptr (n+1), out_indices (nnz),
// out_vals64 (nnz*DB*DB) and, when vals32 is given, out_vals32.
RVGP_API int rvgp_permute_csr(int n, int DB, const int* indptr, const int* indices, const double* vals64,
                              const float* vals32, const int* perm, const int* rank, int* out_indptr,
                              int* out_indices, double* out_vals64, float* out_vals32, void* workspace,
                              size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(indptr && indices && vals64 && perm && rank && out_indptr && out_indices && out_vals64,
                 "rvgp_permute_csr: null pointer");
  RVGP_CHECK_ARG(!vals32 || out_vals32, "rvgp_permute_csr: vals32 needs out_vals32");
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_permute_csr_workspace(n), "rvgp_permute_csr: workspace too small");
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  int* len = ws.take<int>(n);
  int* sws = ws.take<int>(scan_workspace(n) / sizeof(int) + 1);
  rvgp::note_launch();
  perm_lengths<<<ceil_div(n, 256), 256, 0, st>>>(indptr, perm, n, len);
  exclusive_scan(len, n, out_indptr, out_indptr + n, sws, st);
  rvgp::note_launch();
  perm_scatter<<<ceil_div((long long)n * 32, 256), 256, 0, st>>>(indptr, indices, vals64, vals32, DB, perm, rank,
                                                                 out_indptr, n, out_indices, out_vals64, out_vals32);
  RVGP_LAUNCH_CHECK("rvgp_permute_csr");
  return RVGP_OK;
}

// dst (n*DB x m, ldd) rows in the original numbering from src rows in the new
// numbering: dst[(i*DB+q), :] = src[(rank[i]*DB+q), :].
RVGP_API int rvgp_unpermute_rows(const double* src, int lds, const int* rank, int n, int DB, int m, double* dst,
                                 int ldd, void* stream) {
  RVGP_CHECK_ARG(src && rank && dst && n >= 1 && DB >= 1 && m >= 1, "rvgp_unpermute_rows: bad arguments");
  rvgp::note_launch();
  unpermute_rows<<<ceil_div((long long)n * DB * m, 256), 256, 0, as_stream(stream)>>>(src, lds, rank, n, DB, m, dst,
                                                                                        ldd);
  RVGP_LAUNCH_CHECK("rvgp_unpermute_rows");
  return RVGP_OK;
}
