// Exact k-nearest-neighbour search (replaces sklearn kneighbors_graph,
// RVGP/geometry.py:103-110, connectivity mode, include_self=False).
//
// Result contract: for every point q, the k indices j != q with the smallest
// FP64 squared distance  sum_j (x_qj - x_cj)^2  (coordinates summed in order,
// no fused multiply-add), ties broken by the lower index, listed in ascending
// (distance, index) order.
//
// Pipeline (all on the caller's stream):
//   1. prep     : bounding-box centre, FP32 centred copy padded to DP columns,
//                 radius R = max |x - c| (two-stage deterministic reductions).
//   2. screen   : FP32 brute force.  CTA = 128 queries x one slice of the
//                 candidates staged through shared memory; every query keeps its
//                 kc smallest FP32 squared distances in a register-resident
//                 sorted list (kc = k + 8 rounded up to 16, 32, 48 or 72).
//   3. finish   : merge the slices, rescore the kc survivors in exact FP64, sort
//                 by (d2, index) and certify: with u = 2^-24 the FP32 distance f
//                 of any pair satisfies  true >= (f/(1+g) - 4.01 u R)/(1+u),
//                 g = DP u/(1 - DP u).  If that lower bound for the kc-th FP32
//                 survivor exceeds the exact k-th distance, no non-survivor can
//                 enter the top k and the row is exact.  Otherwise the row is
//                 queued.
//   4. fallback : exact FP64 scan of the queued rows (one CTA per row).
#include "common.cuh"
#include "knn_top.cuh"
#include <float.h>
#include <limits.h>
#include <algorithm>
#include <mutex>

namespace rvgp {
namespace {

constexpr int kQB = 128;      // queries per CTA in the screen
constexpr int kTileElems = 8192;  // floats of candidate coordinates per shared-memory tile (32 KB)
constexpr int kExtra = 8;     // surplus survivors kept by the FP32 screen
constexpr int kMaxKC = 72;    // k + kExtra upper bound
constexpr int kFbThreads = 128;

__global__ void prep_minmax(const double* __restrict__ X, int n, int D, double* __restrict__ part) {
  // part[(block * D + j) * 2 + {0,1}] = min, max of column j over this block's rows
  extern __shared__ double sh[];
  for (int j = 0; j < D; ++j) {
    double lo = DBL_MAX, hi = -DBL_MAX;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      double v = X[(size_t)i * D + j];
      lo = fmin(lo, v);
      hi = fmax(hi, v);
    }
    sh[threadIdx.x] = lo;
    sh[blockDim.x + threadIdx.x] = hi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + s]);
        sh[blockDim.x + threadIdx.x] = fmax(sh[blockDim.x + threadIdx.x], sh[blockDim.x + threadIdx.x + s]);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      part[((size_t)blockIdx.x * D + j) * 2 + 0] = sh[0];
      part[((size_t)blockIdx.x * D + j) * 2 + 1] = sh[blockDim.x];
    }
    __syncthreads();
  }
}

__global__ void prep_centre(const double* __restrict__ part, int nblk, int D, double* __restrict__ centre) {
  int j = threadIdx.x;
  if (j >= D) return;
  double lo = DBL_MAX, hi = -DBL_MAX;
  for (int b = 0; b < nblk; ++b) {
    lo = fmin(lo, part[((size_t)b * D + j) * 2 + 0]);
    hi = fmax(hi, part[((size_t)b * D + j) * 2 + 1]);
  }
  centre[j] = 0.5 * (lo + hi);
}

__global__ void prep_copy(const double* __restrict__ X, int n, int D, int DP, const double* __restrict__ centre,
                          float* __restrict__ Xf, double* __restrict__ part_r2) {
  __shared__ double sh[256];
  double r2max = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double r2 = 0.0;
    for (int j = 0; j < DP; ++j) {
      double a = j < D ? X[(size_t)i * D + j] - centre[j] : 0.0;
      Xf[(size_t)i * DP + j] = (float)a;
      r2 += a * a;
    }
    r2max = fmax(r2max, r2);
  }
  sh[threadIdx.x] = r2max;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part_r2[blockIdx.x] = sh[0];
}

__global__ void prep_radius(const double* __restrict__ part_r2, int nblk, double* __restrict__ radius) {
  if (threadIdx.x != 0) return;
  double m = 0.0;
  for (int b = 0; b < nblk; ++b) m = fmax(m, part_r2[b]);
  // sqrt of an FP64 sum: inflate by a relative 1e-12 so R is an upper bound
  *radius = sqrt(m) * (1.0 + 1e-12);
}

// Splits per listed row when the screen runs over a list of nlist rows (the
// rows another screen's certificate could not settle): as many as the part
// buffers hold (cap_rows row-lists), at most smax.  The screen and the finish
// compute it alike from the device-side count.
__device__ __forceinline__ int list_splits(int nlist, long long cap_rows, int smax) {
  const long long s = nlist > 0 ? cap_rows / nlist : smax;
  return (int)max(1ll, min((long long)smax, s));
}

// One CTA's work: queries qi0 .. qi0 + kQB - 1 (list slots in list mode)
// against the candidates of split `split` of nsplit; their lists at
// part[(qi * nsplit + split) * KC] in list mode, else at the query's row.
template <int DP, int KC>
__device__ __forceinline__ void screen_block(float* tile, const float* __restrict__ Xf, int n, int qi0, int split,
                                             int nsplit, float* __restrict__ part_d, int* __restrict__ part_i,
                                             const int* __restrict__ qlist, int nlist) {
  constexpr int kTile = kTileElems / DP;
  const int qi = qi0 + threadIdx.x;
  const int q = qlist ? (qi < nlist ? qlist[qi] : n) : qi;
  const long long chunk = ((long long)n + nsplit - 1) / nsplit;
  const int c0 = (int)min((long long)n, split * chunk);
  const int c1 = (int)min((long long)n, c0 + chunk);
  float xq[DP];
#pragma unroll
  for (int j = 0; j < DP; ++j) xq[j] = q < n ? Xf[(size_t)q * DP + j] : 0.f;
  RegTop<KC> L;
  L.init();
  for (int t0 = c0; t0 < c1; t0 += kTile) {
    const int tn = min(kTile, c1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < tn * DP; e += kQB) tile[e] = Xf[(size_t)t0 * DP + e];
    __syncthreads();
    if (q < n) {
      for (int c = 0; c < tn; ++c) {
        float acc = 0.f;
#pragma unroll
        for (int j = 0; j < DP; ++j) {
          float df = xq[j] - tile[c * DP + j];
          acc = fmaf(df, df, acc);
        }
        const int ci = t0 + c;
        if (acc < L.worst() && ci != q) L.insert(acc, ci);
      }
    }
  }
  if (q < n) {
    const size_t base = ((size_t)(qlist ? qi : q) * nsplit + split) * KC;
#pragma unroll
    for (int r = 0; r < KC; ++r) {
      part_d[base + r] = L.d[r];
      part_i[base + r] = L.i[r];
    }
  }
}

// Every query (grid ceil(n / kQB) x nsplit), or, with qlist, the nq[0] listed
// rows: each CTA then takes (list block, split) items in turn, with
// list_splits(nq[0], cap_rows, nsplit) splits per row, so a short list still
// spreads over the whole GPU.
template <int DP, int KC>
__global__ void __launch_bounds__(kQB) knn_screen(const float* __restrict__ Xf, int n, int nsplit,
                                                  float* __restrict__ part_d, int* __restrict__ part_i,
                                                  const int* __restrict__ qlist, const int* __restrict__ nq,
                                                  long long cap_rows) {
  constexpr int kTile = kTileElems / DP;
  __shared__ float tile[kTile * DP];
  if (!qlist) {
    screen_block<DP, KC>(tile, Xf, n, blockIdx.x * kQB, blockIdx.y, nsplit, part_d, part_i, nullptr, 0);
    return;
  }
  const int nlist = *nq;
  const int S = list_splits(nlist, cap_rows, nsplit);
  const long long items = (long long)((nlist + kQB - 1) / kQB) * S;
  for (long long w = blockIdx.x; w < items; w += gridDim.x) {  // uniform in the CTA
    __syncthreads();  // the previous item's tile reads are done
    screen_block<DP, KC>(tile, Xf, n, (int)(w / S) * kQB, (int)(w % S), S, part_d, part_i, qlist, nlist);
  }
}

__device__ __forceinline__ double exact_d2(const double* __restrict__ X, int D, int a, int b) {
  double acc = 0.0;
  for (int j = 0; j < D; ++j) {
    double df = __dsub_rn(X[(size_t)a * D + j], X[(size_t)b * D + j]);
    acc = __dadd_rn(acc, __dmul_rn(df, df));
  }
  return acc;
}

__device__ __forceinline__ bool lex_less(double da, int ia, double db, int ib) {
  return da < db || (da == db && ia < ib);
}

// Keeps the kc smallest values seen (runtime kc, arrays in local memory; the
// merge runs once per query, so its cost is small next to the screen).
struct TopList {
  float d[kMaxKC];
  int i[kMaxKC];
  int cnt;
  int kc;
  float worst;
  int wpos;
  __device__ void init(int kc_) { cnt = 0; kc = kc_; worst = FLT_MAX; wpos = 0; }
  __device__ void refresh() {
    worst = d[0];
    wpos = 0;
    for (int r = 1; r < kc; ++r)
      if (d[r] > worst) { worst = d[r]; wpos = r; }
  }
  __device__ void push(float v, int idx) {
    if (cnt < kc) {
      d[cnt] = v;
      i[cnt] = idx;
      if (++cnt == kc) refresh();
    } else if (v < worst) {
      d[wpos] = v;
      i[wpos] = idx;
      refresh();
    }
  }
};

// r2q (optional): the tensor-core screen's |x'|² per query (knn_tc.cu): its
// certificate replaces the SIMT screen's; tcerr (optional): a raised flag of
// that screen sends every row to the exact scan.
__global__ void knn_finish(const double* __restrict__ X, int n, int D, int DP, int k, int kc, int nsplit,
                           const float* __restrict__ part_d, const int* __restrict__ part_i,
                           const double* __restrict__ radius, int* __restrict__ out_idx,
                           int* __restrict__ nflag, int* __restrict__ flag_list, const float* __restrict__ r2q,
                           const int* __restrict__ tcerr, const int* __restrict__ qlist, const int* __restrict__ nq,
                           long long cap_rows) {
  const int qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qlist ? qi >= *nq : qi >= n) return;
  const int q = qlist ? qlist[qi] : qi;
  if (qlist) nsplit = list_splits(*nq, cap_rows, nsplit);  // the list screen's layout
  TopList L;
  L.init(kc);
  const size_t base = (size_t)(qlist ? qi : q) * nsplit * kc;
  int total = 0;
  for (int e = 0; e < nsplit * kc; ++e) {
    int ci = part_i[base + e];
    if (ci < 0) continue;
    ++total;
    float v = part_d[base + e];
    if (L.cnt < kc || v < L.worst) L.push(v, ci);
  }
  const int cnt = L.cnt;
  double d2[kMaxKC];
  int id[kMaxKC];
  for (int r = 0; r < cnt; ++r) {
    double v = exact_d2(X, D, q, L.i[r]);
    int ci = L.i[r];
    int s = r;
    while (s > 0 && lex_less(v, ci, d2[s - 1], id[s - 1])) {
      d2[s] = d2[s - 1];
      id[s] = id[s - 1];
      --s;
    }
    d2[s] = v;
    id[s] = ci;
  }
  bool certified;
  if (total == n - 1 && cnt == total) {
    certified = true;  // every other point was rescored exactly
  } else {
    // here some slice kept a full list, so total >= kc and cnt == kc
    const double u = 5.9604644775390625e-08;  // 2^-24
    double lb;
    if (r2q) {
      // tensor-core screen: d'² >= (f² - 3 eps |x'|²) / (1 + 2 eps) on the
      // block-centred FP32 values, eps = 1e-4 (knn_tc.cu), then their own
      // rounding (u (|x'| + |y'|) <= u (2|x'| + d')) and the FP32 copy's
      const double eps = 1e-4, rq = (double)r2q[q] * (1.0 + 1e-6);
      const double lb2 = ((double)L.worst - 3.0 * eps * rq) / (1.0 + 2.0 * eps);
      const double dp = sqrt(fmax(lb2, 0.0));
      lb = (dp * (1.0 - u) - 2.0 * u * sqrt(rq) - 4.01 * u * radius[0]) / (1.0 + u);
    } else {
      const double g = DP * u / (1.0 - DP * u);
      const double f = sqrt((double)L.worst);
      lb = (f / (1.0 + g) - 4.01 * u * radius[0]) / (1.0 + u);
    }
    lb *= (1.0 - 1e-12);
    certified = lb > 0.0 && lb * lb > d2[k - 1] * (1.0 + 1e-12);
  }
  if (tcerr && *tcerr) certified = false;
  for (int r = 0; r < k; ++r) out_idx[(size_t)q * k + r] = r < cnt ? id[r] : -1;
  if (!certified) {
    int slot = atomicAdd(nflag, 1);
    flag_list[slot] = q;
  }
}

// Exact FP64 scan for the rows the certificate could not settle.
__global__ void __launch_bounds__(kFbThreads) knn_fallback(const double* __restrict__ X, int n, int D, int k,
                                                           const int* __restrict__ nflag,
                                                           const int* __restrict__ flag_list,
                                                           int* __restrict__ out_idx) {
  __shared__ double sd[kFbThreads];
  __shared__ int si[kFbThreads];
  __shared__ int st[kFbThreads];
  const int nf = *nflag;
  for (int f = blockIdx.x; f < nf; f += gridDim.x) {
    const int q = flag_list[f];
    double d2[kMaxKC];
    int id[kMaxKC];
    int cnt = 0;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      if (c == q) continue;
      double v = exact_d2(X, D, q, c);
      if (cnt == k && !lex_less(v, c, d2[k - 1], id[k - 1])) continue;
      int s = cnt < k ? cnt++ : k - 1;
      while (s > 0 && lex_less(v, c, d2[s - 1], id[s - 1])) {
        d2[s] = d2[s - 1];
        id[s] = id[s - 1];
        --s;
      }
      d2[s] = v;
      id[s] = c;
    }
    int head = 0;
    for (int r = 0; r < k; ++r) {
      sd[threadIdx.x] = head < cnt ? d2[head] : DBL_MAX;
      si[threadIdx.x] = head < cnt ? id[head] : INT_MAX;
      st[threadIdx.x] = threadIdx.x;
      __syncthreads();
      for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
          int o = threadIdx.x + s;
          if (lex_less(sd[o], si[o], sd[threadIdx.x], si[threadIdx.x])) {
            sd[threadIdx.x] = sd[o];
            si[threadIdx.x] = si[o];
            st[threadIdx.x] = st[o];
          }
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) out_idx[(size_t)q * k + r] = si[0];
      if (threadIdx.x == st[0]) ++head;
      __syncthreads();
    }
  }
}

int padded_dim(int D) {
  if (D <= 4) return 4;
  if (D <= 8) return 8;
  if (D <= 16) return 16;
  if (D <= 32) return 32;
  if (D <= 64) return 64;
  if (D <= 128) return 128;
  return -1;
}

// survivors kept per slice: k + kExtra rounded up to a register-list size
int kc_bucket(int k) {
  const int c = k + kExtra;
  return c <= 16 ? 16 : c <= 32 ? 32 : c <= 48 ? 48 : 72;
}

template <int KC>
void launch_screen(int DP, dim3 grid, cudaStream_t st, const float* Xf, int n, int nsplit, float* pd, int* pi,
                   const int* qlist = nullptr, const int* nq = nullptr, long long cap = 0) {
  switch (DP) {
    case 4: knn_screen<4, KC><<<grid, kQB, 0, st>>>(Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
    case 8: knn_screen<8, KC><<<grid, kQB, 0, st>>>(Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
    case 16: knn_screen<16, KC><<<grid, kQB, 0, st>>>(Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
    case 32: knn_screen<32, KC><<<grid, kQB, 0, st>>>(Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
    case 64: knn_screen<64, KC><<<grid, kQB, 0, st>>>(Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
    default: knn_screen<128, KC><<<grid, kQB, 0, st>>>(Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
  }
}

void screen_kc(int kc, int DP, dim3 grid, cudaStream_t st, const float* Xf, int n, int nsplit, float* pd, int* pi,
               const int* qlist = nullptr, const int* nq = nullptr, long long cap = 0) {
  switch (kc) {
    case 16: launch_screen<16>(DP, grid, st, Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
    case 32: launch_screen<32>(DP, grid, st, Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
    case 48: launch_screen<48>(DP, grid, st, Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
    default: launch_screen<72>(DP, grid, st, Xf, n, nsplit, pd, pi, qlist, nq, cap); break;
  }
}

struct KnnPlan {
  int DP, kc, nsplit, nblk_prep;
  bool tc;      // tensor-core screen (knn_tc.cu)
  int nsplit2;  // part-buffer room per row beside nsplit (the re-screen's list layout uses it)
};

// The tensor-core screen for 16 < D <= 64 (RVGP_KNN_TC=0, or
// RVGP_TENSOR_CORES=0, selects the SIMT screen); the allocation-free entry
// point keeps the SIMT screen (its scratch is fixed).
bool knn_tc_enabled(int D) {
  const char* e = getenv("RVGP_KNN_TC");
  const char* t = getenv("RVGP_TENSOR_CORES");
  return D > 16 && D <= 64 && !(e && e[0] == '0') && !(t && t[0] == '0');
}

KnnPlan plan(int n, int D, int k, bool allow_tc = true) {
  KnnPlan p;
  p.DP = padded_dim(D);
  p.kc = kc_bucket(k);
  p.tc = allow_tc && knn_tc_enabled(D);
  int qblocks = ceil_div(n, kQB);
  p.nsplit = max(1, min(16, ceil_div((p.tc ? 1 : 4) * num_sms(), qblocks)));
  p.nsplit2 = max(1, min(16, ceil_div(4 * num_sms(), qblocks)));
  p.nblk_prep = min(num_sms() * 2, max(1, ceil_div(n, 256)));
  return p;
}

struct KnnBufs {
  double *part_mm, *centre, *part_r2, *radius;
  float *Xf, *part_d, *r2q;
  int *part_i, *nflag, *flag_list, *order, *rank, *tcerr, *nflag2, *flag_list2;
  void* lo_ws;
  size_t lo_bytes;
};

}  // namespace
}  // namespace rvgp
extern "C" size_t rvgp_locality_order_workspace(int n, int D);
extern "C" int rvgp_locality_order(const double* X, int n, int D, int* perm, int* rank, void* workspace,
                                   size_t ws_bytes, void* stream);
namespace rvgp {
int knn_tc_screen_launch(int DP, int kc, const float* Xf, int n, const int* order, int nsplit, float* part_d,
                         int* part_i, float* r2q, int* err, cudaStream_t st);
namespace {

KnnBufs carve(Workspace& ws, const KnnPlan& p, int n, int D) {
  KnnBufs b;
  b.r2q = nullptr;
  b.order = b.rank = b.tcerr = b.nflag2 = b.flag_list2 = nullptr;
  b.lo_ws = nullptr;
  b.lo_bytes = 0;
  b.part_mm = ws.take<double>((size_t)p.nblk_prep * D * 2);
  b.centre = ws.take<double>(D);
  b.part_r2 = ws.take<double>(p.nblk_prep);
  b.radius = ws.take<double>(1);
  b.Xf = ws.take<float>((size_t)n * p.DP);
  const int ns = std::max(p.tc ? 2 * p.nsplit : p.nsplit, p.nsplit2);  // the TC screen writes two halves
  b.part_d = ws.take<float>((size_t)n * ns * p.kc);
  b.part_i = ws.take<int>((size_t)n * ns * p.kc);
  b.nflag = ws.take<int>(1);
  b.flag_list = ws.take<int>(n);
  if (p.tc) {
    b.nflag2 = ws.take<int>(1);
    b.flag_list2 = ws.take<int>(n);
    b.r2q = ws.take<float>(n);
    b.order = ws.take<int>(n);
    b.rank = ws.take<int>(n);
    b.tcerr = ws.take<int>(1);
    b.lo_bytes = rvgp_locality_order_workspace(n, D);
    b.lo_ws = ws.take<char>(b.lo_bytes);
  }
  return b;
}

size_t workspace_bytes(int n, int D, int k, bool allow_tc = true) {
  Workspace ws(nullptr, 0);
  carve(ws, plan(n, D, k, allow_tc), n, D);
  return ws.used;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

// Scratch bytes rvgp_knn needs, or 0 for a shape it does not support
// (n < 2, D outside [1, 128], k outside [1, n) or above its maximum).
RVGP_API size_t rvgp_knn_workspace(int n, int D, int k) {
  if (n < 2 || D < 1 || k < 1 || k >= n || padded_dim(D) < 0 || k + kExtra > kMaxKC) return 0;
  return workspace_bytes(n, D, k);
}

static int knn_impl(const double* X, int n, int D, int k, int* idx, void* workspace, size_t ws_bytes, void* stream,
                    bool allow_tc);

RVGP_API int rvgp_knn(const double* X, int n, int D, int k, int* idx, void* workspace, size_t ws_bytes,
                      void* stream) {
  return knn_impl(X, n, D, k, idx, workspace, ws_bytes, stream, true);
}

static int knn_impl(const double* X, int n, int D, int k, int* idx, void* workspace, size_t ws_bytes, void* stream,
                    bool allow_tc) {
  RVGP_CHECK_ARG(X && idx, "rvgp_knn: null pointer");
  RVGP_CHECK_ARG(n >= 2, "rvgp_knn: need at least 2 points, got %d", n);
  RVGP_CHECK_ARG(k >= 1 && k < n, "Expected n_neighbors < n_samples, got %d >= %d", k, n);
  RVGP_CHECK_ARG(k + kExtra <= kMaxKC, "rvgp_knn: k=%d exceeds the supported maximum %d", k, kMaxKC - kExtra);
  RVGP_CHECK_ARG(padded_dim(D) > 0, "rvgp_knn: ambient dimension %d > 128 is not supported", D);
  size_t need = workspace_bytes(n, D, k, allow_tc);
  RVGP_CHECK_ARG(workspace && ws_bytes >= need, "rvgp_knn: workspace of %zu bytes needed", need);
  cudaStream_t st = as_stream(stream);
  KnnPlan p = plan(n, D, k, allow_tc);
  Workspace ws(workspace, ws_bytes);
  KnnBufs b = carve(ws, p, n, D);
  rvgp::note_launch(); prep_minmax<<<p.nblk_prep, 256, 2 * 256 * sizeof(double), st>>>(X, n, D, b.part_mm);
  rvgp::note_launch(); prep_centre<<<1, 128, 0, st>>>(b.part_mm, p.nblk_prep, D, b.centre);
  rvgp::note_launch(); prep_copy<<<p.nblk_prep, 256, 0, st>>>(X, n, D, p.DP, b.centre, b.Xf, b.part_r2);
  rvgp::note_launch(); prep_radius<<<1, 32, 0, st>>>(b.part_r2, p.nblk_prep, b.radius);
  cudaMemsetAsync(b.nflag, 0, sizeof(int), st);
  if (p.tc) {
    // queries in the locality order: a block of 128 is a compact patch
    TRY_RC(rvgp_locality_order(X, n, D, b.order, b.rank, b.lo_ws, b.lo_bytes, stream));
    cudaMemsetAsync(b.tcerr, 0, sizeof(int), st);
    cudaMemsetAsync(b.nflag2, 0, sizeof(int), st);
    TRY_RC(knn_tc_screen_launch(p.DP, p.kc, b.Xf, n, b.order, p.nsplit, b.part_d, b.part_i, b.r2q, b.tcerr, st));
    rvgp::note_launch();
    knn_finish<<<ceil_div(n, 128), 128, 0, st>>>(X, n, D, p.DP, k, p.kc, 2 * p.nsplit, b.part_d, b.part_i, b.radius,
                                                 idx, b.nflag, b.flag_list, b.r2q, b.tcerr, nullptr, nullptr, 0);
    // rows the tensor-core certificate could not settle (a query block
    // straddling a jump of the Morton curve): the SIMT screen, whose
    // direct-difference certificate does not depend on the block, then the
    // exact scan for what remains.  The list is usually short (tens of rows
    // at n = 100 000), so its rows get up to one split per SM, as many as the
    // part buffers hold (list_splits).
    const int smax = num_sms();
    const long long cap = (long long)n * std::max(2 * p.nsplit, p.nsplit2);
    const int gx = (int)std::min<long long>((long long)ceil_div(n, kQB) * smax, 4ll * num_sms());
    rvgp::note_launch();
    screen_kc(p.kc, p.DP, dim3(gx, 1), st, b.Xf, n, smax, b.part_d, b.part_i, b.flag_list, b.nflag, cap);
    rvgp::note_launch();
    knn_finish<<<ceil_div(n, 128), 128, 0, st>>>(X, n, D, p.DP, k, p.kc, smax, b.part_d, b.part_i, b.radius, idx,
                                                 b.nflag2, b.flag_list2, nullptr, nullptr, b.flag_list, b.nflag, cap);
    rvgp::note_launch(); knn_fallback<<<num_sms(), kFbThreads, 0, st>>>(X, n, D, k, b.nflag2, b.flag_list2, idx);
  } else {
    dim3 grid(ceil_div(n, kQB), p.nsplit);
    rvgp::note_launch();
    screen_kc(p.kc, p.DP, grid, st, b.Xf, n, p.nsplit, b.part_d, b.part_i);
    rvgp::note_launch();
    knn_finish<<<ceil_div(n, 128), 128, 0, st>>>(X, n, D, p.DP, k, p.kc, p.nsplit, b.part_d, b.part_i, b.radius, idx,
                                                 b.nflag, b.flag_list, nullptr, nullptr, nullptr, nullptr, 0);
    rvgp::note_launch(); knn_fallback<<<num_sms(), kFbThreads, 0, st>>>(X, n, D, k, b.nflag, b.flag_list, idx);
  }
  RVGP_LAUNCH_CHECK("rvgp_knn");
  return RVGP_OK;
}

// ---------------------------------------------------------------------------
// kNN without any device allocation.
//
// For callers that cannot allocate device memory at the time they need a
// neighbour search: applications that reserve their whole device-memory
// budget at start-up and forbid later allocations, hosts that embed this
// library inside a framework owning the device memory pool without offering
// an allocator to plug in, and latency-critical loops where an allocation's
// implicit synchronisation is not acceptable.  They pass inputs and outputs
// only; the scratch comes from a fixed buffer compiled into this library.
//
// Limits and behaviour:
//  * the buffer holds kNoAllocScratchBytes (32 MiB); a problem whose scratch
//    (rvgp_knn_workspace(n, D, k)) is larger is rejected with an error.  Every
//    n up to 63,000 fits at D = 3, k = 20 (up to 32,500 at D = 64, k = 15);
//    query rvgp_knn_workspace for other shapes;
//  * the buffer is a file-scope device array, so every GPU that loads this
//    library keeps those 32 MiB until the process exits;
//  * the first call on a device looks up the buffer's device address with
//    that device current and caches it; make that first call before any
//    stream capture;
//  * all calls share the one buffer, which keeps the previous call's data:
//    the search overwrites every part it reads and zeroes its fallback
//    counter on each call, but two calls whose work overlaps on the GPU (on
//    different streams, or from different host threads) race on the buffer
//    and must be serialised by the caller.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_knn_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};
}  // namespace

RVGP_API int rvgp_knn_noalloc(const double* X, int n, int D, int k, int* idx, void* stream) {
  RVGP_CHECK_ARG(n >= 2 && k >= 1 && k < n && D >= 1, "rvgp_knn_noalloc: bad sizes n=%d D=%d k=%d", n, D, k);
  RVGP_CHECK_ARG(rvgp_knn_workspace(n, D, k) > 0,
                 "rvgp_knn_noalloc: unsupported shape n=%d, D=%d, k=%d (D must be <= 128, k <= %d)", n, D, k,
                 kMaxKC - kExtra);
  const size_t need = workspace_bytes(n, D, k, false);  // the SIMT screen: its scratch is the fixed buffer's
  RVGP_CHECK_ARG(need <= kNoAllocScratchBytes,
                 "rvgp_knn_noalloc: n=%d, D=%d, k=%d needs %zu bytes of scratch, more than the fixed %zu-byte "
                 "buffer; use rvgp_knn with a caller-provided workspace",
                 n, D, k, need, kNoAllocScratchBytes);
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    rvgp::set_error("rvgp_knn_noalloc: no usable current CUDA device");
    return RVGP_ELAUNCH;
  }
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_knn_scratch);
      if (e != cudaSuccess || !p) {
        rvgp::set_error("rvgp_knn_noalloc: device address of the scratch buffer unavailable: %s",
                        cudaGetErrorString(e));
        return RVGP_ELAUNCH;
      }
      g_scratch_ptr[dev] = p;
    }
    scratch = g_scratch_ptr[dev];
  }
  return knn_impl(X, n, D, k, idx, scratch, kNoAllocScratchBytes, stream, false);
}

// Number of rows the last rvgp_knn call on this workspace sent to the exact
// fallback (reads one int from the workspace; synchronises the stream).
RVGP_API int rvgp_knn_fallback_rows(int n, int D, int k, void* workspace, void* stream) {
  if (padded_dim(D) < 0 || k < 1 || k >= n) return -1;
  Workspace ws(workspace, SIZE_MAX);
  KnnBufs b = carve(ws, plan(n, D, k), n, D);
  int h = -1;
  // the tensor-core path's exact scan takes the rows its SIMT re-screen left
  if (read_back(&h, b.nflag2 ? b.nflag2 : b.nflag, sizeof(int), as_stream(stream)) != cudaSuccess) return -1;
  return h;
}
