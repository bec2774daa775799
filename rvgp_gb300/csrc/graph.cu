// Symmetrised kNN graph in CSR form and its combinatorial Laplacian.
//
// Replaces the networkx/scipy graph handling of the reference:
//   A = kneighbors_graph(...) + I; G = nx.from_scipy_sparse_array(A)
//   (RVGP/geometry.py:103-112), the symmetrisation max(A, Aᵀ) done before the
//   Dijkstra and the transport loop (RVGP/lib/ptu_dijkstra.pyx:84-103), and
//   L = nx.laplacian_matrix(G) (RVGP/geometry.py:55-63).
//
// Output CSR: row i holds {i} ∪ knn(i) ∪ {j : i ∈ knn(j)}, column indices
// sorted ascending, every weight 1.  E = indptr[n] stored entries (self-loops
// included).  Laplacian values: deg_i on the diagonal (number of distinct
// neighbours; the self-loop cancels in D − A), −1 elsewhere.
#include "common.cuh"
#include "scan.cuh"
#include <limits.h>

namespace rvgp {
namespace {

constexpr int kSortCap = 512;   // rows up to this length are sorted by a warp in shared memory
constexpr int kWarpsPerCTA = 4;

__global__ void count_reverse(const int* __restrict__ knn, long long nk, int* __restrict__ rev) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nk; e += (long long)gridDim.x * blockDim.x)
    atomicAdd(&rev[knn[e]], 1);
}

__global__ void row_capacity(const int* __restrict__ rev, int n, int k, int* __restrict__ cap) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cap[i] = k + 1 + rev[i];
}

__global__ void fill_rows(const int* __restrict__ knn, int n, int k, const int* __restrict__ slot,
                          int* __restrict__ cursor, int* __restrict__ buf) {
  long long nk = (long long)n * k;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nk; e += (long long)gridDim.x * blockDim.x) {
    int i = (int)(e / k), r = (int)(e % k);
    int j = knn[e];
    buf[slot[i] + r] = j;
    if (r == 0) buf[slot[i] + k] = i;
    int pos = atomicAdd(&cursor[j], 1);
    buf[slot[j] + k + 1 + pos] = i;
  }
}

// One warp per row: sort, drop duplicates, write the unique count.
__global__ void sort_unique_rows(int n, const int* __restrict__ slot, const int* __restrict__ cap,
                                 int* __restrict__ buf, int* __restrict__ ucount) {
  __shared__ int sh[kWarpsPerCTA][kSortCap];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int row = blockIdx.x * kWarpsPerCTA + w;
  if (row >= n) return;
  int* r = buf + slot[row];
  const int len = cap[row];
  if (len <= kSortCap) {
    int p2 = 32;
    while (p2 < len) p2 <<= 1;
    for (int t = lane; t < p2; t += 32) sh[w][t] = t < len ? r[t] : INT_MAX;
    __syncwarp();
    for (int size = 2; size <= p2; size <<= 1) {
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int t = lane; t < p2; t += 32) {
          int o = t ^ stride;
          if (o > t) {
            bool up = (t & size) == 0;
            int a = sh[w][t], b = sh[w][o];
            if ((a > b) == up) {
              sh[w][t] = b;
              sh[w][o] = a;
            }
          }
        }
        __syncwarp();
      }
    }
    // compact unique values (ascending) back into the row
    int base = 0;
    for (int t0 = 0; t0 < len; t0 += 32) {
      int t = t0 + lane;
      bool keep = t < len && (t == 0 || sh[w][t] != sh[w][t - 1]);
      unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) r[base + __popc(m & ((1u << lane) - 1))] = sh[w][t];
      base += __popc(m);
    }
    if (lane == 0) ucount[row] = base;
  } else if (lane == 0) {
    // long row: serial shell sort in place, then compact
    for (int gap = len / 2; gap > 0; gap /= 2)
      for (int t = gap; t < len; ++t) {
        int v = r[t], s = t;
        while (s >= gap && r[s - gap] > v) {
          r[s] = r[s - gap];
          s -= gap;
        }
        r[s] = v;
      }
    int u = 0;
    for (int t = 0; t < len; ++t)
      if (t == 0 || r[t] != r[u - 1]) r[u++] = r[t];
    ucount[row] = u;
  }
}

__global__ void compact_rows(int n, const int* __restrict__ slot, const int* __restrict__ buf,
                             const int* __restrict__ indptr, int* __restrict__ indices,
                             const int* __restrict__ ucount, int* __restrict__ maxdeg) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kWarpsPerCTA + (threadIdx.x >> 5);
  if (row >= n) return;
  const int u = ucount[row];
  for (int t = lane; t < u; t += 32) indices[indptr[row] + t] = buf[slot[row] + t];
  if (lane == 0) atomicMax(maxdeg, u - 1);
}

__global__ void finish_indptr(int n, int* __restrict__ indptr, const int* __restrict__ total, int* __restrict__ e_out) {
  indptr[n] = *total;
  if (e_out) *e_out = *total;
}

struct GraphBufs {
  int *rev, *cap, *slot, *cursor, *buf, *ucount, *scan_ws, *total;
};

GraphBufs carve(Workspace& ws, int n, int k) {
  GraphBufs b;
  b.rev = ws.take<int>(n);
  b.cap = ws.take<int>(n);
  b.slot = ws.take<int>((size_t)n + 1);
  b.cursor = ws.take<int>(n);
  b.buf = ws.take<int>((size_t)n * (2 * k + 1));
  b.ucount = ws.take<int>(n);
  b.scan_ws = ws.take<int>(scan_workspace(n) / sizeof(int) + 1);
  b.total = ws.take<int>(2);
  return b;
}

__global__ void laplacian_values(int n, const int* __restrict__ indptr, const int* __restrict__ indices,
                                 double* __restrict__ vals) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * kWarpsPerCTA + (threadIdx.x >> 5);
  if (row >= n) return;
  const int s = indptr[row], e = indptr[row + 1];
  const double deg = (double)(e - s - 1);
  for (int t = s + lane; t < e; t += 32) vals[t] = indices[t] == row ? deg : -1.0;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_graph_workspace(int n, int k) {
  Workspace ws(nullptr, 0);
  carve(ws, n, k);
  return ws.used;
}

// knn: (n, k) int32 neighbour indices (device).  indptr: n+1 ints; indices:
// capacity n*(2k+1) ints.  e_out / maxdeg_out: one device int each (number of
// stored entries, largest degree excluding the self-loop).
RVGP_API int rvgp_graph_build(const int* knn, int n, int k, int* indptr, int* indices, int* e_out, int* maxdeg_out,
                              void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(knn && indptr && indices && maxdeg_out, "rvgp_graph_build: null pointer");
  RVGP_CHECK_ARG(n >= 2 && k >= 1 && k < n, "rvgp_graph_build: bad sizes n=%d k=%d", n, k);
  RVGP_CHECK_ARG((long long)n * (2 * k + 1) < INT_MAX, "rvgp_graph_build: graph too large for int32 indices");
  size_t need = rvgp_graph_workspace(n, k);
  RVGP_CHECK_ARG(workspace && ws_bytes >= need, "rvgp_graph_build: workspace of %zu bytes needed", need);
  cudaStream_t st = as_stream(stream);
  Workspace ws(workspace, ws_bytes);
  GraphBufs b = carve(ws, n, k);
  const long long nk = (long long)n * k;
  const int eb = min(ceil_div(nk, 256), num_sms() * 16);
  cudaMemsetAsync(b.rev, 0, sizeof(int) * n, st);
  cudaMemsetAsync(b.cursor, 0, sizeof(int) * n, st);
  cudaMemsetAsync(maxdeg_out, 0, sizeof(int), st);
  rvgp::note_launch(); count_reverse<<<eb, 256, 0, st>>>(knn, nk, b.rev);
  rvgp::note_launch(); row_capacity<<<ceil_div(n, 256), 256, 0, st>>>(b.rev, n, k, b.cap);
  exclusive_scan(b.cap, n, b.slot, nullptr, b.scan_ws, st);
  rvgp::note_launch(); fill_rows<<<eb, 256, 0, st>>>(knn, n, k, b.slot, b.cursor, b.buf);
  rvgp::note_launch(); sort_unique_rows<<<ceil_div(n, kWarpsPerCTA), 32 * kWarpsPerCTA, 0, st>>>(n, b.slot, b.cap, b.buf, b.ucount);
  exclusive_scan(b.ucount, n, indptr, b.total, b.scan_ws, st);
  rvgp::note_launch(); finish_indptr<<<1, 1, 0, st>>>(n, indptr, b.total, e_out);
  rvgp::note_launch(); compact_rows<<<ceil_div(n, kWarpsPerCTA), 32 * kWarpsPerCTA, 0, st>>>(n, b.slot, b.buf, indptr, indices, b.ucount,
                                                                         maxdeg_out);
  RVGP_LAUNCH_CHECK("rvgp_graph_build");
  return RVGP_OK;
}

// vals[e] for the CSR pattern above: deg_i on the diagonal, -1 off it.
RVGP_API int rvgp_laplacian_values(const int* indptr, const int* indices, int n, double* vals, void* stream) {
  RVGP_CHECK_ARG(indptr && indices && vals && n >= 1, "rvgp_laplacian_values: bad arguments");
  rvgp::note_launch(); laplacian_values<<<ceil_div(n, kWarpsPerCTA), 32 * kWarpsPerCTA, 0, as_stream(stream)>>>(n, indptr, indices, vals);
  RVGP_LAUNCH_CHECK("rvgp_laplacian_values");
  return RVGP_OK;
}
