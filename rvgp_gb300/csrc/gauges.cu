// Local tangent frames ("gauges") from geodesic neighbourhoods.
//
// Replaces the reference's native routine _geodesic_neigborhood_tangents
// (RVGP/lib/ptu_dijkstra.pyx:300-437) and its Fibonacci heap (pyx:444-690).
//
// Pipeline (three launches):
//   1. geodesic neighbourhood of every point (RVGP/lib/ptu_dijkstra.pyx:361-394):
//      Dijkstra over the unit-weight CSR graph from i until K+1 nodes are
//      scanned.  The heap is a replica of the reference's Fibonacci heap: the
//      same insert / remove_min / link / decrease_val steps in the same order,
//      on a node pool addressed through a small open-addressing hash (global
//      index -> pool slot).  Equal path lengths therefore leave the heap in the
//      same order as in the reference, and the K+1 scanned nodes are the same
//      set.  This is the one place where the steps of the reference's
//      algorithm must be reproduced, because the tie-breaking decides which
//      nodes at the boundary hop distance enter the neighbourhood.
//      One warp per point keeps the pool (256 slots, 16-bit links, 16 bytes
//      per node) and the hash in shared memory, so every link the heap follows
//      is a shared-memory access; a point whose search touches more nodes is
//      queued for
//   1b. the same search with the pool and hash in global memory, sized for
//      the worst case 1 + K(maxdeg + 1) (one thread per queued point);
//   2. one thread per point centres the D x (K+1) block M of neighbourhood
//      coordinates and takes its SVD in FP64 (pyx:396-434): when D <= K+1 by
//      one-sided (Hestenes) Jacobi on Mᵀ ((K+1) x D, rotations accumulated
//      into U); otherwise (ambient dimension above the neighbourhood size,
//      e.g. D = 64, K + 1 = 23) from the (K+1) x (K+1) Gram matrix MᵀM =
//      V Λ Vᵀ (Householder tridiagonalisation and implicit QL, symeig.cuh):
//      the columns of M V have norms σ_j (taken as the singular values, so
//      small ones keep an absolute accuracy ~ε σ₁ rather than the √ε σ₁ of
//      √λ_j) and are σ_j u_j.  It writes the first d_out left singular
//      vectors (tangents, (n, D, d_out)) and the c = min(D, K+1) singular
//      values (Sigma, (n, c)), descending.  Each singular vector is signed so
//      its largest-magnitude entry is positive (the reference inherits
//      LAPACK's arbitrary signs).
//
// Global scratch is interleaved worker-minor (field[slot * W + worker]) so the
// SVD phase, where all threads walk the same loop, is coalesced.
#include "common.cuh"
#include "symeig.cuh"
#include <limits.h>

namespace rvgp {
namespace {

constexpr int NIL = -1;
constexpr int ST_SCANNED = 0, ST_NOT_IN_HEAP = 1, ST_IN_HEAP = 2;
constexpr int kSvdThreads = 128;
constexpr int kPoolS = 256;     // shared-memory pool slots per point
constexpr int kHashS = 512;     // shared-memory hash slots per point
constexpr int kRanksS = 32;     // root-list ranks (a 256-node Fibonacci heap has rank < 12)
constexpr int kNbhWarps = 4;    // points (warps) per CTA in the shared-memory search
constexpr int kFbWorkers = 1024;  // threads of the global-memory search for queued points

// ------------------------------------------------------------------ node storage
// Global-memory scratch, interleaved worker-minor (field f of slot v at f[v * W + w]).
struct Scratch {
  double* val;
  int *rank, *parent, *left, *right, *child, *state, *gidx;
  int *hkey, *hslot, *roots;
  double *mat, *J;
};

struct GlobalStore {
  static constexpr int kRanks = 100;
  Scratch s;
  int W, w, pool, hsize;
  __host__ __device__ int& rank(int v) { return s.rank[(size_t)v * W + w]; }
  __host__ __device__ int& parent(int v) { return s.parent[(size_t)v * W + w]; }
  __host__ __device__ int& left(int v) { return s.left[(size_t)v * W + w]; }
  __host__ __device__ int& right(int v) { return s.right[(size_t)v * W + w]; }
  __host__ __device__ int& child(int v) { return s.child[(size_t)v * W + w]; }
  __host__ __device__ int& state(int v) { return s.state[(size_t)v * W + w]; }
  __host__ __device__ double& val(int v) { return s.val[(size_t)v * W + w]; }
  __host__ __device__ int& gidx(int v) { return s.gidx[(size_t)v * W + w]; }
  __host__ __device__ int& roots(int r) { return s.roots[(size_t)r * W + w]; }
  __host__ __device__ int& hkey(int h) { return s.hkey[(size_t)h * W + w]; }
  __host__ __device__ int& hslot(int h) { return s.hslot[(size_t)h * W + w]; }
  static constexpr bool kClearKeys = true;  // the hash is emptied key by key after each point
};

// One warp's pool in shared memory: 16-bit links and values (hop counts of
// at most K+1), 16 bytes per node.
struct SmemStore {
  static constexpr int kRanks = kRanksS;
  short *par, *lft, *rgt, *chd, *vl, *hs, *rt;
  unsigned char *rk, *stt;
  int *gi, *hk;
  int pool, hsize;
  __device__ unsigned char& rank(int v) { return rk[v]; }
  __device__ short& parent(int v) { return par[v]; }
  __device__ short& left(int v) { return lft[v]; }
  __device__ short& right(int v) { return rgt[v]; }
  __device__ short& child(int v) { return chd[v]; }
  __device__ unsigned char& state(int v) { return stt[v]; }
  __device__ short& val(int v) { return vl[v]; }
  __device__ int& gidx(int v) { return gi[v]; }
  __device__ short& roots(int r) { return rt[r]; }
  __device__ int& hkey(int h) { return hk[h]; }
  __device__ short& hslot(int h) { return hs[h]; }
  static constexpr bool kClearKeys = false;  // the warp resets the whole hash after each point
};

__host__ __device__ inline size_t smem_bytes_per_warp() {
  return (size_t)kPoolS * (5 * sizeof(short) + 2 + sizeof(int)) + (size_t)kHashS * (sizeof(int) + sizeof(short)) +
         kRanksS * sizeof(short) + 64;
}

// ------------------------------------------------------------------ the heap
// The Fibonacci heap of RVGP/lib/ptu_dijkstra.pyx:444-690 on a node pool (the
// same operations in the same order; node identity is the pool slot).
template <class Store>
struct Heap : Store {
  int alloc = 0, min_node = NIL;
  bool overflow = false;

  __host__ __device__ int hash_pos(int g) const {
    return (int)(((unsigned)g * 2654435761u) & (unsigned)(this->hsize - 1));
  }

  // pool slot of global node g, allocated (and initialised) on first touch
  __host__ __device__ int slot_of(int g) {
    int h = hash_pos(g);
    for (int probe = 0; probe < this->hsize; ++probe) {
      const int key = this->hkey(h);
      if (key == g) return this->hslot(h);
      if (key == NIL) {
        if (alloc >= this->pool) {
          overflow = true;
          return NIL;
        }
        const int v = alloc++;
        this->hkey(h) = g;
        this->hslot(h) = v;
        this->gidx(v) = g;
        this->val(v) = 0;
        this->rank(v) = 0;
        this->state(v) = ST_NOT_IN_HEAP;
        this->parent(v) = NIL;
        this->left(v) = NIL;
        this->right(v) = NIL;
        this->child(v) = NIL;
        return v;
      }
      h = (h + 1) & (this->hsize - 1);
    }
    overflow = true;
    return NIL;
  }

  // forget this point's nodes (global store: remove every key it inserted)
  __host__ __device__ void clear() {
    if (Store::kClearKeys)
      for (int v = 0; v < alloc; ++v) {
        const int g = this->gidx(v);
        int h = hash_pos(g);
        for (int probe = 0; probe < this->hsize; ++probe) {
          if (this->hkey(h) == g) {
            this->hkey(h) = NIL;
            break;
          }
          h = (h + 1) & (this->hsize - 1);
        }
      }
    alloc = 0;
  }

  // sibling walks are bounded by the pool size; a longer walk marks overflow
  __host__ __device__ int rightmost(int v) {
    for (int g = 0; g < this->pool && this->right(v) != NIL; ++g) v = this->right(v);
    if (this->right(v) != NIL) overflow = true;
    return v;
  }
  __host__ __device__ int leftmost(int v) {
    for (int g = 0; g < this->pool && this->left(v) != NIL; ++g) v = this->left(v);
    if (this->left(v) != NIL) overflow = true;
    return v;
  }

  __host__ __device__ void add_sibling(int node, int sib) {
    const int t = rightmost(node);
    this->right(t) = sib;
    this->left(sib) = t;
    this->right(sib) = NIL;
    this->parent(sib) = this->parent(node);
    if (this->parent(sib) != NIL) this->rank(this->parent(sib)) += 1;
  }

  __host__ __device__ void add_child(int node, int c) {
    this->parent(c) = node;
    if (this->child(node) != NIL) {
      add_sibling(this->child(node), c);
    } else {
      this->child(node) = c;
      this->right(c) = NIL;
      this->left(c) = NIL;
      this->rank(node) = 1;
    }
  }

  __host__ __device__ void unlink(int v) {
    const int p = this->parent(v);
    if (p != NIL) {
      this->rank(p) -= 1;
      if (this->left(v) != NIL) this->child(p) = this->left(v);
      else if (this->right(v) != NIL) this->child(p) = this->right(v);
      else this->child(p) = NIL;
    }
    if (this->left(v) != NIL) this->right(this->left(v)) = this->right(v);
    if (this->right(v) != NIL) this->left(this->right(v)) = this->left(v);
    this->left(v) = NIL;
    this->right(v) = NIL;
    this->parent(v) = NIL;
  }

  __host__ __device__ void insert(int v) {
    if (min_node != NIL) {
      add_sibling(min_node, v);
      if (this->val(v) < this->val(min_node)) min_node = v;
    } else {
      min_node = v;
    }
  }

  __host__ __device__ void decrease(int v, int nv) {
    this->val(v) = nv;
    if (this->parent(v) != NIL && this->val(this->parent(v)) >= nv) {
      unlink(v);
      insert(v);
    } else if (this->val(min_node) > this->val(v)) {
      min_node = v;
    }
  }

  __host__ __device__ void link_root(int v) {
    for (int guard = 0; guard < this->pool + Store::kRanks; ++guard) {
      const int r = this->rank(v);
      if (r < 0 || r >= Store::kRanks) {
        overflow = true;
        return;
      }
      const int other = this->roots(r);
      if (other == NIL) {
        this->roots(r) = v;
        return;
      }
      this->roots(r) = NIL;
      if (this->val(v) < this->val(other) || v == min_node) {
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
    const int m = min_node;
    int t, tr;
    if (this->child(m) != NIL) {
      t = leftmost(this->child(m));
      for (int g = 0; t != NIL; ++g) {
        if (g > this->pool) {
          overflow = true;
          return m;
        }
        tr = this->right(t);
        unlink(t);
        add_sibling(m, t);
        t = tr;
      }
      this->child(m) = NIL;
    }
    t = leftmost(m);
    if (t == m) {
      if (this->right(m) != NIL) {
        t = this->right(m);
      } else {
        min_node = NIL;
        return m;
      }
    }
    unlink(m);
    min_node = t;
    for (int r = 0; r < Store::kRanks; ++r) this->roots(r) = NIL;
    for (int g = 0; t != NIL; ++g) {
      if (g > this->pool) {
        overflow = true;
        return m;
      }
      if (this->val(t) < this->val(min_node)) min_node = t;
      tr = this->right(t);
      link_root(t);
      if (overflow) return m;
      t = tr;
    }
    return m;
  }
};

// The K+1 nodes scanned first by Dijkstra from i over the unit-weight graph
// (RVGP/lib/ptu_dijkstra.pyx:361-394), in scan order, into nbh_row.
// Returns 0, 1 (component smaller than K+1) or 2 (node pool overflow).
template <class Store>
__host__ __device__ int geodesic_nbh(Heap<Store>& h, int i, const int* __restrict__ indptr,
                                     const int* __restrict__ indices, int K, int* nbh_row) {
  h.min_node = NIL;
  const int si = h.slot_of(i);
  if (si == NIL) {
    h.clear();
    h.overflow = false;
    return 2;
  }
  h.insert(si);
  int scanned = 0;
  while (h.min_node != NIL && scanned <= K && !h.overflow) {
    const int v = h.remove_min();
    if (h.overflow) break;
    h.state(v) = ST_SCANNED;
    nbh_row[scanned++] = h.gidx(v);
    if (scanned <= K) {
      const int vv = h.val(v);
      for (int e = indptr[h.gidx(v)]; e < indptr[h.gidx(v) + 1]; ++e) {
        const int su = h.slot_of(indices[e]);
        if (su == NIL) break;
        if (h.state(su) != ST_SCANNED) {
          const int nv = vv + 1;  // connectivity graph: every weight is 1
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
  return scanned < K + 1 ? 1 : 0;
}

// One warp per point; lane 0 runs the search on the warp's shared-memory pool,
// the other lanes reset the hash afterwards.  Points that overflow the pool go
// to ovf_list for the global-memory search.
__global__ void __launch_bounds__(kNbhWarps * 32)
    geonbh_smem_kernel(int n, const int* __restrict__ indptr, const int* __restrict__ indices, int K,
                       int* __restrict__ nbh, int* __restrict__ status, int* __restrict__ ovf_count,
                       int* __restrict__ ovf_list) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned char* base = sm + wib * smem_bytes_per_warp();
  Heap<SmemStore> h;
  h.gi = reinterpret_cast<int*>(base);
  h.hk = h.gi + kPoolS;
  h.par = reinterpret_cast<short*>(h.hk + kHashS);
  h.lft = h.par + kPoolS;
  h.rgt = h.lft + kPoolS;
  h.chd = h.rgt + kPoolS;
  h.vl = h.chd + kPoolS;
  h.hs = h.vl + kPoolS;
  h.rt = h.hs + kHashS;
  h.rk = reinterpret_cast<unsigned char*>(h.rt + kRanksS);
  h.stt = h.rk + kPoolS;
  h.pool = kPoolS;
  h.hsize = kHashS;
  for (int q = lane; q < kHashS; q += 32) h.hk[q] = NIL;
  __syncwarp();
  const int warps = gridDim.x * kNbhWarps;
  for (int i = blockIdx.x * kNbhWarps + wib; i < n; i += warps) {
    int st = 0;
    if (lane == 0) st = geodesic_nbh(h, i, indptr, indices, K, nbh + (size_t)i * (K + 1));
    st = __shfl_sync(0xffffffffu, st, 0);
    for (int q = lane; q < kHashS; q += 32) h.hk[q] = NIL;
    __syncwarp();
    if (lane == 0) {
      if (st == 1) atomicMin(&status[0], i);
      if (st == 2) ovf_list[atomicAdd(ovf_count, 1)] = i;
    }
  }
}

// The same search with the worst-case pool in global memory, for the queued points.
__global__ void __launch_bounds__(128)
    geonbh_global_kernel(const int* __restrict__ indptr, const int* __restrict__ indices, int K, Scratch s, int W,
                         int pool, int hsize, const int* __restrict__ ovf_count, const int* __restrict__ ovf_list,
                         int* __restrict__ nbh, int* __restrict__ status) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= W) return;
  Heap<GlobalStore> h;
  h.s = s;
  h.W = W;
  h.w = w;
  h.pool = pool;
  h.hsize = hsize;
  const int cnt = *ovf_count;
  for (int q = w; q < cnt; q += W) {
    const int i = ovf_list[q];
    const int st = geodesic_nbh(h, i, indptr, indices, K, nbh + (size_t)i * (K + 1));
    if (st == 1) atomicMin(&status[0], i);
    if (st == 2) atomicMin(&status[2], i);
  }
}

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

struct GaugeLayout {
  int W;            // SVD workers (threads with scratch)
  int rows, cols;   // Jacobi matrix shape
  bool accumulate;  // path A (rotations accumulated into U)
  int Wf;           // workers of the global-memory search
  int pool, hsize;  // its worst-case pool and hash per worker
};

// SVD of the centred D x c block M (column q at mat[(q * D + t) * W + w],
// D > c) through its Gram matrix G = MᵀM (c x c at Jm, overwritten by its
// eigenvectors V): singular values |M v_j| (descending), left singular
// vectors M v_j / σ_j for the first d_out.
__host__ __device__ void gauge_svd_gram(int i, int D, int c, int d_out, const GaugeLayout& L, double* mat, double* Jm,
                                        int w, double* __restrict__ tangents, double* __restrict__ sigma) {
  const int W = L.W;
  auto m_ = [&](int q, int t) -> double& { return mat[((size_t)q * D + t) * W + w]; };
  struct Acc {
    double* p;
    int c, W, w;
    __host__ __device__ double& operator()(int a, int b) { return p[((size_t)a * c + b) * W + w]; }
  } g{Jm, c, W, w};
  for (int a = 0; a < c; ++a)
    for (int b = 0; b <= a; ++b) {
      double s = 0.0;
      for (int t = 0; t < D; ++t) s += m_(a, t) * m_(b, t);
      g(a, b) = s;
      g(b, a) = s;
    }
  double lam[128], e[128], sv[128];
  int order[128];
  symeig::eigh(g, c, lam, e);
  // σ_j = |M v_j| in the order of descending eigenvalue (ties keep column order)
  for (int j = 0; j < c; ++j) {
    double nrm = 0.0;
    for (int t = 0; t < D; ++t) {
      double u = 0.0;
      for (int a = 0; a < c; ++a) u += m_(a, t) * g(a, j);
      nrm += u * u;
    }
    const double v = sqrt(nrm);
    int q = j;
    while (q > 0 && (lam[order[q - 1]] < lam[j])) {
      order[q] = order[q - 1];
      --q;
    }
    order[q] = j;
    sv[j] = v;
  }
  for (int q = 0; q < c; ++q) sigma[(size_t)i * c + q] = sv[order[q]];
  for (int q = 0; q < d_out; ++q) {
    const int j = order[q];
    const double inv = 1.0 / sv[j];
    double big = 0.0;
    for (int t = 0; t < D; ++t) {
      double u = 0.0;
      for (int a = 0; a < c; ++a) u += m_(a, t) * g(a, j);
      u *= inv;
      if (fabs(u) > fabs(big)) big = u;
    }
    const double sg = big < 0.0 ? -1.0 : 1.0;
    for (int t = 0; t < D; ++t) {
      double u = 0.0;
      for (int a = 0; a < c; ++a) u += m_(a, t) * g(a, j);
      tangents[((size_t)i * D + t) * d_out + q] = sg * u * inv;
    }
  }
}

// Centring and SVD of point i's neighbourhood (pyx:396-434).
__host__ __device__ void gauge_svd(int i, const double* __restrict__ X, int D, int K, const int* __restrict__ nbh_row,
                                   int d_out, const GaugeLayout& L, double* mat, double* Jm, int w,
                                   double* __restrict__ tangents, double* __restrict__ sigma) {
  const int c = L.cols, r = L.rows;
  for (int p = 0; p < D; ++p) {
    double mean = 0.0;
    for (int q = 0; q <= K; ++q) mean += X[(size_t)nbh_row[q] * D + p];
    mean /= (double)(K + 1);
    for (int q = 0; q <= K; ++q) {
      const double v = X[(size_t)nbh_row[q] * D + p] - mean;
      // path A: A = Mᵀ (rows = K+1, cols = D); path B: A = M (rows = D, cols = K+1)
      const size_t e = L.accumulate ? ((size_t)p * r + q) : ((size_t)q * r + p);
      mat[e * L.W + w] = v;
    }
  }
  if (!L.accumulate) {
    gauge_svd_gram(i, D, c, d_out, L, mat, Jm, w, tangents, sigma);
    return;
  }
  hestenes(mat, L.accumulate ? Jm : nullptr, r, c, L.W, w);
  int order[128];
  double sv[128];
  for (int p = 0; p < c; ++p) {
    double nrm = 0.0;
    for (int t = 0; t < r; ++t) {
      const double x = mat[((size_t)p * r + t) * L.W + w];
      nrm += x * x;
    }
    const double v = sqrt(nrm);
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
      const double u = L.accumulate ? Jm[((size_t)p * c + t) * L.W + w] : mat[((size_t)p * r + t) * L.W + w] / sv[q];
      if (fabs(u) > fabs(big)) big = u;
    }
    const double sg = big < 0.0 ? -1.0 : 1.0;
    for (int t = 0; t < D; ++t) {
      const double u = L.accumulate ? Jm[((size_t)p * c + t) * L.W + w] : mat[((size_t)p * r + t) * L.W + w] / sv[q];
      tangents[((size_t)i * D + t) * d_out + q] = sg * u;
    }
  }
}

__global__ void __launch_bounds__(kSvdThreads)
    gauges_svd_kernel(const double* __restrict__ X, int n, int D, int K, const int* __restrict__ nbh, int d_out,
                      GaugeLayout L, double* __restrict__ mat, double* __restrict__ Jm,
                      double* __restrict__ tangents, double* __restrict__ sigma) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= L.W) return;
  for (int i = w; i < n; i += L.W) {
    const int* row = nbh + (size_t)i * (K + 1);
    if (row[K] < 0) continue;  // the search failed for this point (reported in status)
    gauge_svd(i, X, D, K, row, d_out, L, mat, Jm, w, tangents, sigma);
  }
}

GaugeLayout layout(int n, int D, int K, int maxdeg) {
  GaugeLayout L;
  L.W = min(n, num_sms() * 256);
  L.accumulate = D <= K + 1;
  L.rows = L.accumulate ? K + 1 : D;
  L.cols = L.accumulate ? D : K + 1;
  L.Wf = min(n, kFbWorkers);
  L.pool = 1 + K * (maxdeg + 1);
  L.hsize = 64;
  while (L.hsize < 2 * L.pool) L.hsize <<= 1;
  return L;
}

struct Bufs {
  Scratch s;  // global-memory search (Wf workers) + SVD matrices (W workers)
  int *nbh, *ovf_count, *ovf_list;
};

Bufs carve(Workspace& ws, const GaugeLayout& L, int n, int K, bool own_nbh) {
  Bufs b;
  const size_t P = (size_t)L.pool * L.Wf;
  b.s.val = ws.take<double>(P);
  b.s.rank = ws.take<int>(P);
  b.s.parent = ws.take<int>(P);
  b.s.left = ws.take<int>(P);
  b.s.right = ws.take<int>(P);
  b.s.child = ws.take<int>(P);
  b.s.state = ws.take<int>(P);
  b.s.gidx = ws.take<int>(P);
  b.s.hkey = ws.take<int>((size_t)L.hsize * L.Wf);
  b.s.hslot = ws.take<int>((size_t)L.hsize * L.Wf);
  b.s.roots = ws.take<int>((size_t)GlobalStore::kRanks * L.Wf);
  b.s.mat = ws.take<double>((size_t)L.rows * L.cols * L.W);
  b.s.J = ws.take<double>((size_t)L.cols * L.cols * L.W);  // rotations (D <= K+1) or the Gram matrix
  b.nbh = own_nbh ? ws.take<int>((size_t)n * (K + 1)) : nullptr;
  b.ovf_count = ws.take<int>(1);
  b.ovf_list = ws.take<int>(n);
  return b;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_gauges_workspace(int n, int D, int K, int maxdeg) {
  GaugeLayout L = layout(n, D, K, maxdeg);
  Workspace ws(nullptr, 0);
  carve(ws, L, n, K, true);
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
  Bufs b = carve(ws, L, n, K, true);
  int* nbh = nbh_out ? nbh_out : b.nbh;
  cudaMemsetAsync(status, 0x7F, 3 * sizeof(int), st);
  cudaMemsetAsync(b.ovf_count, 0, sizeof(int), st);
  cudaMemsetAsync(nbh, 0xFF, sizeof(int) * (size_t)n * (K + 1), st);
  cudaMemsetAsync(b.s.hkey, 0xFF, sizeof(int) * (size_t)L.hsize * L.Wf, st);
  const size_t smem = kNbhWarps * smem_bytes_per_warp();
  rvgp::note_launch();
  geonbh_smem_kernel<<<ceil_div(n, kNbhWarps), kNbhWarps * 32, smem, st>>>(n, indptr, indices, K, nbh, status,
                                                                           b.ovf_count, b.ovf_list);
  rvgp::note_launch();
  geonbh_global_kernel<<<ceil_div(L.Wf, 128), 128, 0, st>>>(indptr, indices, K, b.s, L.Wf, L.pool, L.hsize,
                                                           b.ovf_count, b.ovf_list, nbh, status);
  rvgp::note_launch();
  gauges_svd_kernel<<<ceil_div(L.W, kSvdThreads), kSvdThreads, 0, st>>>(X, n, D, K, nbh, d_out, L, b.s.mat, b.s.J,
                                                                        tangents, sigma);
  RVGP_LAUNCH_CHECK("rvgp_gauges");
  return RVGP_OK;
}
