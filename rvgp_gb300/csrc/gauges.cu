// Local tangent frames ("gauges") from geodesic neighbourhoods.
//
// Replaces the reference's native routine _geodesic_neigborhood_tangents
// (RVGP/lib/ptu_dijkstra.pyx:300-437) and its Fibonacci heap (pyx:444-690).
//
// Per point i (one thread per point, persistent grid):
//   1. Dijkstra over the unit-weight CSR graph from i until K+1 nodes are
//      scanned.  The heap is a replica of the reference's Fibonacci heap: the
//      same insert / remove_min / link / decrease_val steps in the same order,
//      on a per-thread node pool addressed through a small open-addressing hash
//      (global index -> pool slot).  Equal path lengths therefore leave the heap
//      in the same order as in the reference, and the K+1 scanned nodes are the
//      same set.  This is the one place where the steps of the reference's
//      algorithm must be reproduced, because the tie-breaking decides which
//      nodes at the boundary hop distance enter the neighbourhood.
//   2. Centre the D x (K+1) block of neighbourhood coordinates and take its
//      SVD by one-sided (Hestenes) Jacobi in FP64: on Mᵀ ((K+1) x D, rotations
//      accumulated into U) when D <= K+1, on M (D x (K+1)) otherwise.
//   3. Write the first d_out left singular vectors (tangents, (n, D, d_out))
//      and the c = min(D, K+1) singular values (Sigma, (n, c)), descending.
//      Each singular vector is signed so its largest-magnitude entry is
//      positive (the reference inherits LAPACK's arbitrary signs).
//
// Scratch is interleaved worker-minor (field[slot * W + worker]) so the SVD
// phase, where all threads walk the same loop, is coalesced.
#include "common.cuh"
#include <limits.h>

namespace rvgp {
namespace {

constexpr int NIL = -1;
constexpr int ST_SCANNED = 0, ST_NOT_IN_HEAP = 1, ST_IN_HEAP = 2;
constexpr int kRanks = 100;
constexpr int kThreads = 128;

struct GaugeLayout {
  int W;         // workers (threads with scratch)
  int pool;      // heap node slots per worker
  int hsize;     // hash slots per worker (power of two)
  int rows, cols;  // Jacobi matrix shape
  bool accumulate;  // path A (rotations accumulated into U)
};

struct Scratch {
  double* val;
  int *rank, *parent, *left, *right, *child, *state, *gidx;
  int *hkey, *hslot, *roots, *nbh;
  double *mat, *J;
};

Scratch carve(Workspace& ws, const GaugeLayout& L, int K) {
  Scratch s;
  size_t P = (size_t)L.pool * L.W;
  s.val = ws.take<double>(P);
  s.rank = ws.take<int>(P);
  s.parent = ws.take<int>(P);
  s.left = ws.take<int>(P);
  s.right = ws.take<int>(P);
  s.child = ws.take<int>(P);
  s.state = ws.take<int>(P);
  s.gidx = ws.take<int>(P);
  s.hkey = ws.take<int>((size_t)L.hsize * L.W);
  s.hslot = ws.take<int>((size_t)L.hsize * L.W);
  s.roots = ws.take<int>((size_t)kRanks * L.W);
  s.nbh = ws.take<int>((size_t)(K + 1) * L.W);
  s.mat = ws.take<double>((size_t)L.rows * L.cols * L.W);
  s.J = ws.take<double>((size_t)(L.accumulate ? L.cols * L.cols : 1) * L.W);
  return s;
}

// The heap of one worker.  Field f of pool slot v lives at f[v * W + w].
struct Heap {
  Scratch s;
  int W, w, pool, hsize, alloc, min_node;
  bool overflow;

  __host__ __device__ int& rank(int v) { return s.rank[(size_t)v * W + w]; }
  __host__ __device__ int& parent(int v) { return s.parent[(size_t)v * W + w]; }
  __host__ __device__ int& left(int v) { return s.left[(size_t)v * W + w]; }
  __host__ __device__ int& right(int v) { return s.right[(size_t)v * W + w]; }
  __host__ __device__ int& child(int v) { return s.child[(size_t)v * W + w]; }
  __host__ __device__ int& state(int v) { return s.state[(size_t)v * W + w]; }
  __host__ __device__ double& val(int v) { return s.val[(size_t)v * W + w]; }
  __host__ __device__ int& gidx(int v) { return s.gidx[(size_t)v * W + w]; }
  __host__ __device__ int& roots(int r) { return s.roots[(size_t)r * W + w]; }

  __host__ __device__ int hash_pos(int g) const { return (int)(((unsigned)g * 2654435761u) & (unsigned)(hsize - 1)); }

  // pool slot of global node g, allocated (and initialised) on first touch
  __host__ __device__ int slot_of(int g) {
    int h = hash_pos(g);
    for (int probe = 0; probe < hsize; ++probe) {
      size_t a = (size_t)h * W + w;
      int key = s.hkey[a];
      if (key == g) return s.hslot[a];
      if (key == NIL) {
        if (alloc >= pool) {
          overflow = true;
          return NIL;
        }
        int v = alloc++;
        s.hkey[a] = g;
        s.hslot[a] = v;
        gidx(v) = g;
        val(v) = 0.0;
        rank(v) = 0;
        state(v) = ST_NOT_IN_HEAP;
        parent(v) = left(v) = right(v) = child(v) = NIL;
        return v;
      }
      h = (h + 1) & (hsize - 1);
    }
    overflow = true;
    return NIL;
  }

  // empty the hash for the next point (every key inserted for this point is removed)
  __host__ __device__ void clear() {
    for (int v = 0; v < alloc; ++v) {
      int g = gidx(v);
      int h = hash_pos(g);
      for (int probe = 0; probe < hsize; ++probe) {
        size_t a = (size_t)h * W + w;
        if (s.hkey[a] == g) {
          s.hkey[a] = NIL;
          break;
        }
        h = (h + 1) & (hsize - 1);
      }
    }
    alloc = 0;
  }

  // sibling walks are bounded by the pool size; a longer walk marks overflow
  __host__ __device__ int rightmost(int v) {
    for (int g = 0; g < pool && right(v) != NIL; ++g) v = right(v);
    if (right(v) != NIL) overflow = true;
    return v;
  }
  __host__ __device__ int leftmost(int v) {
    for (int g = 0; g < pool && left(v) != NIL; ++g) v = left(v);
    if (left(v) != NIL) overflow = true;
    return v;
  }

  __host__ __device__ void add_sibling(int node, int sib) {
    int t = rightmost(node);
    right(t) = sib;
    left(sib) = t;
    right(sib) = NIL;
    parent(sib) = parent(node);
    if (parent(sib) != NIL) rank(parent(sib)) += 1;
  }

  __host__ __device__ void add_child(int node, int c) {
    parent(c) = node;
    if (child(node) != NIL) {
      add_sibling(child(node), c);
    } else {
      child(node) = c;
      right(c) = NIL;
      left(c) = NIL;
      rank(node) = 1;
    }
  }

  __host__ __device__ void unlink(int v) {
    int p = parent(v);
    if (p != NIL) {
      rank(p) -= 1;
      if (left(v) != NIL) child(p) = left(v);
      else if (right(v) != NIL) child(p) = right(v);
      else child(p) = NIL;
    }
    if (left(v) != NIL) right(left(v)) = right(v);
    if (right(v) != NIL) left(right(v)) = left(v);
    left(v) = NIL;
    right(v) = NIL;
    parent(v) = NIL;
  }

  __host__ __device__ void insert(int v) {
    if (min_node != NIL) {
      add_sibling(min_node, v);
      if (val(v) < val(min_node)) min_node = v;
    } else {
      min_node = v;
    }
  }

  __host__ __device__ void decrease(int v, double nv) {
    val(v) = nv;
    if (parent(v) != NIL && val(parent(v)) >= nv) {
      unlink(v);
      insert(v);
    } else if (val(min_node) > val(v)) {
      min_node = v;
    }
  }

  __host__ __device__ void link_root(int v) {
    for (int guard = 0; guard < pool + kRanks; ++guard) {
      int r = rank(v);
      if (r < 0 || r >= kRanks) { overflow = true; return; }
      int other = roots(r);
      if (other == NIL) {
        roots(r) = v;
        return;
      }
      roots(r) = NIL;
      if (val(v) < val(other) || v == min_node) {
        unlink(other);
        add_child(v, other);
      } else {
        unlink(v);
        add_child(other, v);
        v = other;
      }
    }
    overflow = true;
  }

  __host__ __device__ int remove_min() {
    int m = min_node, t, tr;
    if (child(m) != NIL) {
      t = leftmost(child(m));
      for (int g = 0; t != NIL; ++g) {
        if (g > pool) { overflow = true; return m; }
        tr = right(t);
        unlink(t);
        add_sibling(m, t);
        t = tr;
      }
      child(m) = NIL;
    }
    t = leftmost(m);
    if (t == m) {
      if (right(m) != NIL) {
        t = right(m);
      } else {
        min_node = NIL;
        return m;
      }
    }
    unlink(m);
    min_node = t;
    for (int r = 0; r < kRanks; ++r) roots(r) = NIL;
    for (int g = 0; t != NIL; ++g) {
      if (g > pool) { overflow = true; return m; }
      if (val(t) < val(min_node)) min_node = t;
      tr = right(t);
      link_root(t);
      if (overflow) return m;
      t = tr;
    }
    return m;
  }
};

// One-sided Jacobi on an r x c column-major matrix A (element (row, col) at
// A[(col * r + row) * W + w]); rotations optionally accumulated into J (c x c).
__host__ __device__ void hestenes(double* A, double* J, int r, int c, int W, int w) {
  auto a = [&](int col, int row) -> double& { return A[((size_t)col * r + row) * W + w]; };
  auto j = [&](int col, int row) -> double& { return J[((size_t)col * c + row) * W + w]; };
  if (J)
    for (int p = 0; p < c; ++p)
      for (int q = 0; q < c; ++q) j(p, q) = p == q ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < c - 1; ++p) {
      for (int q = p + 1; q < c; ++q) {
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int t = 0; t < r; ++t) {
          double x = a(p, t), y = a(q, t);
          al += x * x;
          be += y * y;
          ga += x * y;
        }
        if (ga == 0.0 || fabs(ga) <= 1e-15 * sqrt(al * be)) continue;
        rotated = true;
        double zeta = (be - al) / (2.0 * ga);
        double tt = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        double cs = 1.0 / sqrt(1.0 + tt * tt), sn = cs * tt;
        for (int t = 0; t < r; ++t) {
          double x = a(p, t), y = a(q, t);
          a(p, t) = cs * x - sn * y;
          a(q, t) = sn * x + cs * y;
        }
        if (J)
          for (int t = 0; t < c; ++t) {
            double x = j(p, t), y = j(q, t);
            j(p, t) = cs * x - sn * y;
            j(q, t) = sn * x + cs * y;
          }
      }
    }
    if (!rotated) break;
  }
}

// Everything for one point.  Returns 0, 1 (component smaller than K+1) or
// 2 (node pool overflow).  Host-callable so the exact device logic can be
// exercised on a CPU.
__host__ __device__ int gauge_point(int i, Heap& h, const double* __restrict__ X, int D,
                                    const int* __restrict__ indptr, const int* __restrict__ indices, int K,
                                    int d_out, const GaugeLayout& L, double* __restrict__ tangents,
                                    double* __restrict__ sigma, int* __restrict__ nbh_out) {
  Scratch& s = h.s;
  const int w = h.w;
  const int c = L.cols, r = L.rows;
  // ---- 1. geodesic neighbourhood (RVGP/lib/ptu_dijkstra.pyx:361-394)
  h.min_node = NIL;
  int si = h.slot_of(i);
  if (si == NIL) { h.clear(); h.overflow = false; return 2; }
  h.insert(si);
  int scanned = 0;
  while (h.min_node != NIL && scanned <= K && !h.overflow) {
    int v = h.remove_min();
    if (h.overflow) break;
    h.state(v) = ST_SCANNED;
    const int g = h.gidx(v);
    s.nbh[(size_t)scanned * L.W + w] = g;
    ++scanned;
    if (scanned <= K) {
      const double vv = h.val(v);
      for (int e = indptr[g]; e < indptr[g + 1]; ++e) {
        int su = h.slot_of(indices[e]);
        if (su == NIL) break;
        if (h.state(su) != ST_SCANNED) {
          double nv = vv + 1.0;  // connectivity graph: every weight is 1
          if (h.state(su) == ST_NOT_IN_HEAP) {
            h.state(su) = ST_IN_HEAP;
            h.val(su) = nv;
            h.insert(su);
          } else if (h.val(su) > nv) {
            h.decrease(su, nv);
          }
        }
      }
    }
  }
  const bool over = h.overflow;
  h.clear();
  h.overflow = false;
  if (over) return 2;
  if (scanned < K + 1) return 1;
  if (nbh_out)
    for (int q = 0; q <= K; ++q) nbh_out[(size_t)i * (K + 1) + q] = s.nbh[(size_t)q * L.W + w];

  // ---- 2. centred neighbourhood and its SVD (pyx:396-423)
  for (int p = 0; p < D; ++p) {
    double mean = 0.0;
    for (int q = 0; q <= K; ++q) mean += X[(size_t)s.nbh[(size_t)q * L.W + w] * D + p];
    mean /= (double)(K + 1);
    for (int q = 0; q <= K; ++q) {
      double v = X[(size_t)s.nbh[(size_t)q * L.W + w] * D + p] - mean;
      // path A: A = Mᵀ (rows = K+1, cols = D); path B: A = M (rows = D, cols = K+1)
      size_t e = L.accumulate ? ((size_t)p * r + q) : ((size_t)q * r + p);
      s.mat[e * L.W + w] = v;
    }
  }
  hestenes(s.mat, L.accumulate ? s.J : nullptr, r, c, L.W, w);

  // ---- 3. order by singular value, write Sigma and the leading vectors (pyx:425-434)
  int order[128];
  double sv[128];
  for (int p = 0; p < c; ++p) {
    double nrm = 0.0;
    for (int t = 0; t < r; ++t) {
      double x = s.mat[((size_t)p * r + t) * L.W + w];
      nrm += x * x;
    }
    double v = sqrt(nrm);
    int q = p;
    while (q > 0 && sv[q - 1] < v) {
      sv[q] = sv[q - 1];
      order[q] = order[q - 1];
      --q;
    }
    sv[q] = v;
    order[q] = p;
  }
  for (int q = 0; q < c; ++q) sigma[(size_t)i * c + q] = sv[q];
  for (int q = 0; q < d_out; ++q) {
    const int p = order[q];
    double big = 0.0;
    for (int t = 0; t < D; ++t) {
      double u = L.accumulate ? s.J[((size_t)p * c + t) * L.W + w] : s.mat[((size_t)p * r + t) * L.W + w] / sv[q];
      if (fabs(u) > fabs(big)) big = u;
    }
    const double sg = big < 0.0 ? -1.0 : 1.0;
    for (int t = 0; t < D; ++t) {
      double u = L.accumulate ? s.J[((size_t)p * c + t) * L.W + w] : s.mat[((size_t)p * r + t) * L.W + w] / sv[q];
      tangents[((size_t)i * D + t) * d_out + q] = sg * u;
    }
  }
  return 0;
}

__global__ void __launch_bounds__(kThreads) gauges_kernel(
    const double* __restrict__ X, int n, int D, const int* __restrict__ indptr, const int* __restrict__ indices,
    int K, int d_out, Scratch s, GaugeLayout L, double* __restrict__ tangents, double* __restrict__ sigma,
    int* __restrict__ nbh_out, int* __restrict__ status) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= L.W) return;
  Heap h;
  h.s = s;
  h.W = L.W;
  h.w = w;
  h.pool = L.pool;
  h.hsize = L.hsize;
  h.alloc = 0;
  h.overflow = false;
  for (int i = w; i < n; i += L.W) {
    int st = gauge_point(i, h, X, D, indptr, indices, K, d_out, L, tangents, sigma, nbh_out);
    if (st == 1) atomicMin(&status[0], i);
    if (st == 2) atomicMin(&status[2], i);
  }
}

GaugeLayout layout(int n, int D, int K, int maxdeg) {
  GaugeLayout L;
  L.W = min(n, kNumSMs * 256);
  L.pool = 1 + K * (maxdeg + 1);
  L.hsize = 64;
  while (L.hsize < 2 * L.pool) L.hsize <<= 1;
  L.accumulate = D <= K + 1;
  L.rows = L.accumulate ? K + 1 : D;
  L.cols = L.accumulate ? D : K + 1;
  return L;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_gauges_workspace(int n, int D, int K, int maxdeg) {
  GaugeLayout L = layout(n, D, K, maxdeg);
  Workspace ws(nullptr, 0);
  carve(ws, L, K);
  return ws.used;
}

// X: (n, D) f64.  CSR of the symmetrised graph (unit weights).  K: geodesic
// neighbourhood size (K+1 nodes are scanned).  maxdeg: largest degree excluding
// the self-loop (bounds the heap pool).  Outputs: tangents (n, D, d_out),
// sigma (n, min(D, K+1)), optional nbh_out (n, K+1) in scan order.
// status: 3 device ints, set to INT_MAX-like sentinels here and lowered to the
// first failing point: [0] component smaller than K+1, [2] heap pool overflow.
RVGP_API int rvgp_gauges(const double* X, int n, int D, const int* indptr, const int* indices, int K, int maxdeg,
                         int d_out, double* tangents, double* sigma, int* nbh_out, int* status, void* workspace,
                         size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(X && indptr && indices && tangents && sigma && status, "rvgp_gauges: null pointer");
  RVGP_CHECK_ARG(K >= 1 && K < n, "Geodesic neighborhood size must be less than the total number of samples");
  RVGP_CHECK_ARG(d_out >= 1 && d_out <= D && d_out <= K + 1, "rvgp_gauges: bad d_out=%d", d_out);
  RVGP_CHECK_ARG(D <= 128 && K + 1 <= 128, "rvgp_gauges: D and K+1 must be <= 128");
  RVGP_CHECK_ARG(maxdeg >= 1, "rvgp_gauges: bad maxdeg");
  size_t need = rvgp_gauges_workspace(n, D, K, maxdeg);
  RVGP_CHECK_ARG(workspace && ws_bytes >= need, "rvgp_gauges: workspace of %zu bytes needed", need);
  cudaStream_t st = as_stream(stream);
  GaugeLayout L = layout(n, D, K, maxdeg);
  Workspace ws(workspace, ws_bytes);
  Scratch s = carve(ws, L, K);
  cudaMemsetAsync(s.hkey, 0xFF, sizeof(int) * (size_t)L.hsize * L.W, st);
  cudaMemsetAsync(status, 0x7F, 3 * sizeof(int), st);
  rvgp::note_launch(); gauges_kernel<<<ceil_div(L.W, kThreads), kThreads, 0, st>>>(X, n, D, indptr, indices, K, d_out, s, L, tangents,
                                                               sigma, nbh_out, status);
  RVGP_LAUNCH_CHECK("rvgp_gauges");
  return RVGP_OK;
}
