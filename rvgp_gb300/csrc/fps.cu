// Greedy furthest-point sampling (RVGP/geometry.py:126-162).
//
// The reference forms the dense n x n distance matrix (sklearn
// pairwise_distances) and loops on the host.  Here distances are computed on
// the fly in exact FP64 (sqrt of the in-order sum of squared differences, no
// fused multiply-add), the running minimum lives in HBM, and each selection is
// one launch: every CTA first reduces the previous launch's per-CTA maxima (in
// a fixed order: largest distance, then lowest index, i.e. np.argmax's first
// maximum), the CTAs agree on the new point, then each updates its slice of
// the running minimum and publishes its own maximum.  The spacing stop
// (lambda / diameter < spacing) is evaluated on the device; later launches of
// a stopped run return at once.
#include "common.cuh"
#include "gridsync.cuh"
#include <float.h>
#include <limits.h>
#include <algorithm>

namespace rvgp {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double exact_dist(const double* __restrict__ X, int D, int a, int b) {
  double acc = 0.0;
  for (int j = 0; j < D; ++j) {
    const double df = __dsub_rn(X[(size_t)a * D + j], X[(size_t)b * D + j]);
    acc = __dadd_rn(acc, __dmul_rn(df, df));
  }
  return sqrt(acc);
}

struct Best {
  double v;
  int i;
};

__device__ __forceinline__ bool better(double v, int i, double bv, int bi) { return v > bv || (v == bv && i < bi); }

__device__ Best block_best(double v, int i, double* sv, int* si) {
  sv[threadIdx.x] = v;
  si[threadIdx.x] = i;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s && better(sv[threadIdx.x + s], si[threadIdx.x + s], sv[threadIdx.x], si[threadIdx.x])) {
      sv[threadIdx.x] = sv[threadIdx.x + s];
      si[threadIdx.x] = si[threadIdx.x + s];
    }
    __syncthreads();
  }
  Best b{sv[0], si[0]};
  __syncthreads();
  return b;
}

// it == 0: seed with `start`; it >= 1: select from the previous partials.
__global__ void __launch_bounds__(kThreads) fps_step(const double* __restrict__ X, int n, int D, int it, int start,
                                                     double* __restrict__ ds, const double* __restrict__ pv_prev,
                                                     const int* __restrict__ pi_prev, double* __restrict__ pv_next,
                                                     int* __restrict__ pi_next, int* __restrict__ perm,
                                                     double* __restrict__ lambdas, int* __restrict__ count,
                                                     const double* __restrict__ diam, double spacing) {
  __shared__ double sv[kThreads];
  __shared__ int si[kThreads];
  if (*count >= 0) return;  // stopped earlier
  int p;
  if (it == 0) {
    p = start;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      perm[0] = start;
      lambdas[0] = 0.0;
    }
  } else {
    double v = -DBL_MAX;
    int i = INT_MAX;
    for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
      if (better(pv_prev[b], pi_prev[b], v, i)) {
        v = pv_prev[b];
        i = pi_prev[b];
      }
    Best bb = block_best(v, i, sv, si);
    p = bb.i;
    if (diam && bb.v / diam[0] < spacing) {
      if (blockIdx.x == 0 && threadIdx.x == 0) *count = it;
      return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      perm[it] = p;
      lambdas[it] = bb.v;
    }
  }
  const long long chunk = ((long long)n + gridDim.x - 1) / gridDim.x;
  const long long r0 = blockIdx.x * chunk, r1 = min((long long)n, r0 + chunk);
  double v = -DBL_MAX;
  int vi = INT_MAX;
  for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const double d = exact_dist(X, D, p, (int)r);
    const double nd = it == 0 ? d : fmin(ds[r], d);
    ds[r] = nd;
    if (better(nd, (int)r, v, vi)) {
      v = nd;
      vi = (int)r;
    }
  }
  Best bb = block_best(v, vi, sv, si);
  if (threadIdx.x == 0) {
    pv_next[blockIdx.x] = bb.v;
    pi_next[blockIdx.x] = bb.i;
  }
}

// Largest pairwise exact distance (tiles of 128 x 128 points, per-CTA max).
__global__ void __launch_bounds__(kThreads) diameter_tiles(const double* __restrict__ X, int n, int D,
                                                           double* __restrict__ part) {
  __shared__ double sv[kThreads];
  __shared__ int si[kThreads];
  const long long ntile = (n + 127) / 128;
  double mx = 0.0;
  for (long long t = blockIdx.x; t < ntile * ntile; t += gridDim.x) {
    const int ta = (int)(t / ntile), tb = (int)(t % ntile);
    if (tb < ta) continue;
    for (int e = threadIdx.x; e < 128 * 128; e += blockDim.x) {
      const int a = ta * 128 + e / 128, b = tb * 128 + e % 128;
      if (a < n && b < n && b > a) mx = fmax(mx, exact_dist(X, D, a, b));
    }
  }
  Best bb = block_best(mx, 0, sv, si);
  if (threadIdx.x == 0) part[blockIdx.x] = bb.v;
}

__global__ void max_reduce(const double* __restrict__ part, int cnt, double* __restrict__ out) {
  __shared__ double sv[kThreads];
  __shared__ int si[kThreads];
  double m = 0.0;
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) m = fmax(m, part[i]);
  Best bb = block_best(m, 0, sv, si);
  if (threadIdx.x == 0) *out = bb.v;
}

int fps_grid(int n) { return std::max(1, std::min(num_sms() * 2, ceil_div(n, 1024))); }

// ---------------------------------------------------------------- persistent form
// One cooperative launch runs every selection.  Per selection each CTA
// reduces the previous selection's per-CTA maxima (double-buffered by the
// selection's parity; fixed order, largest distance then lowest index), so
// every CTA agrees on the new point p; then it updates the running minimum of
// its slice and publishes the slice's maximum; a bounded grid barrier ends
// the selection.  The new distance d(p, r) is screened in FP32 on the
// coordinates rounded to FP32: with u = 2^-24, R the largest norm of a point
// and D the dimension, |d32 - d| <= 4uR + (D/2 + 2)u d (rounding of the
// operands and of their differences, of the D-term sum and of the square
// root), which delta = 4u(2R√D + (D + 2) d32) exceeds; so
// d32 - delta > ds[r] proves d > ds[r] and the minimum keeps its
// value; only the other points get the exact FP64 distance of exact_dist.
// The stored minima are therefore the exact ones and the selections equal
// the one-launch-per-point form's.
__global__ void fps_prep(const double* __restrict__ X, int n, int D, int DP, float* __restrict__ X32,
                         double* __restrict__ r2max_part) {
  __shared__ double sv[kThreads];
  __shared__ int si[kThreads];
  double mx = 0.0;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < DP; ++j) {
      const float v = j < D ? (float)X[(size_t)r * D + j] : 0.f;
      X32[(size_t)r * DP + j] = v;
      s += (double)v * (double)v;
    }
    mx = fmax(mx, s);
  }
  Best bb = block_best(mx, 0, sv, si);
  if (threadIdx.x == 0) r2max_part[blockIdx.x] = bb.v;
}

__global__ void __launch_bounds__(kThreads) fps_persistent(const double* __restrict__ X, const float* __restrict__ X32,
                                                           int n, int D, int DP, int N_max, int start,
                                                           double* __restrict__ ds, double* __restrict__ pv,
                                                           int* __restrict__ pi, int* __restrict__ perm,
                                                           double* __restrict__ lambdas, int* __restrict__ count,
                                                           const double* __restrict__ diam, double spacing,
                                                           const double* __restrict__ r2max_part, int nprep,
                                                           unsigned int* __restrict__ flags, int* __restrict__ err,
                                                           long long* __restrict__ exact_evals) {
  __shared__ double sv[kThreads];
  __shared__ int si[kThreads];
  __shared__ int s_p, s_stop;
  const unsigned G = gridDim.x;
  unsigned epoch = 0;
  double r2 = 0.0;
  for (int b = 0; b < nprep; ++b) r2 = fmax(r2, r2max_part[b]);
  const double u = 5.9604644775390625e-8;  // 2^-24
  const float c0 = (float)(4.0 * u * 2.0 * sqrt(r2) * sqrt((double)D) * (1.0 + 1e-6));
  const float c1 = (float)(4.0 * u * (D + 2) * (1.0 + 1e-6));
  const long long chunk = ((long long)n + G - 1) / G;
  const long long r0 = blockIdx.x * chunk, r1 = min((long long)n, r0 + chunk);
  long long exact = 0;
  for (int it = 0; it < N_max; ++it) {
    if (threadIdx.x == 0) {
      s_stop = 0;
      if (it == 0) {
        s_p = start;
      }
    }
    if (it > 0) {
      const double* pvp = pv + (size_t)((it - 1) & 1) * G;
      const int* pip = pi + (size_t)((it - 1) & 1) * G;
      double v = -DBL_MAX;
      int i = INT_MAX;
      for (int b = threadIdx.x; b < (int)G; b += blockDim.x)
        if (better(pvp[b], pip[b], v, i)) {
          v = pvp[b];
          i = pip[b];
        }
      Best bb = block_best(v, i, sv, si);
      if (threadIdx.x == 0) {
        s_p = bb.i;
        if (diam && bb.v / diam[0] < spacing) {
          s_stop = 1;
          if (blockIdx.x == 0) *count = it;
        } else if (blockIdx.x == 0) {
          perm[it] = bb.i;
          lambdas[it] = bb.v;
        }
      }
    } else if (blockIdx.x == 0 && threadIdx.x == 0) {
      perm[0] = start;
      lambdas[0] = 0.0;
    }
    __syncthreads();
    if (s_stop) break;  // every CTA takes the same decision from the same partials
    const int p = s_p;
    float xp[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) xp[j] = j < DP ? X32[(size_t)p * DP + j] : 0.f;
    double v = -DBL_MAX;
    int vi = INT_MAX;
    for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      double nd;
      if (it == 0) {
        nd = exact_dist(X, D, p, (int)r);
        ++exact;
      } else {
        const double cur = ds[r];
        float s2 = 0.f;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          if (j < DP) {
            const float df = xp[j] - X32[(size_t)r * DP + j];
            s2 = fmaf(df, df, s2);
          }
        }
        const float d32 = sqrtf(s2);
        if ((double)(d32 - (c0 + c1 * d32)) > cur) {
          nd = cur;  // d(p, r) > ds[r] for certain: the minimum keeps its value
        } else {
          nd = fmin(cur, exact_dist(X, D, p, (int)r));
          ++exact;
        }
      }
      ds[r] = nd;
      if (better(nd, (int)r, v, vi)) {
        v = nd;
        vi = (int)r;
      }
    }
    Best bb = block_best(v, vi, sv, si);
    if (threadIdx.x == 0) {
      pv[(size_t)(it & 1) * G + blockIdx.x] = bb.v;
      pi[(size_t)(it & 1) * G + blockIdx.x] = bb.i;
    }
    if (!grid_barrier_flags(flags, epoch, err, G)) break;
  }
  if (exact_evals) atomicAdd((unsigned long long*)exact_evals, (unsigned long long)exact);
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_fps_workspace(int n) {
  const int G = fps_grid(n);
  return sizeof(double) * ((size_t)n + 2 * G + 4) + sizeof(int) * (2 * (size_t)G + 4) + 1024;
}

// perm (N_max ints), lambdas (N_max doubles): the reference's outputs.  diam:
// device pointer to the diameter for the spacing stop, or null to take all
// N_max points.  count (device int): number of points taken (N_max when no
// stop).  Launches once per point; the host thread does not synchronise.
RVGP_API int rvgp_fps(const double* X, int n, int D, int N_max, int start, const double* diam, double spacing,
                      int* perm, double* lambdas, int* count, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(X && perm && lambdas && count && n >= 1 && D >= 1, "rvgp_fps: bad arguments");
  RVGP_CHECK_ARG(N_max >= 1 && N_max <= n && start >= 0 && start < n, "rvgp_fps: bad N=%d or start=%d", N_max, start);
  RVGP_CHECK_ARG(ws_bytes >= rvgp_fps_workspace(n), "rvgp_fps: workspace too small");
  cudaStream_t st = as_stream(stream);
  const int G = fps_grid(n);
  Workspace ws(workspace, ws_bytes);
  double* ds = ws.take<double>(n);
  double* pv[2] = {ws.take<double>(G), ws.take<double>(G)};
  int* pi[2] = {ws.take<int>(G), ws.take<int>(G)};
  cudaMemsetAsync(count, 0xFF, sizeof(int), st);  // -1: running
  for (int it = 0; it < N_max; ++it) {
    rvgp::note_launch(); fps_step<<<G, kThreads, 0, st>>>(X, n, D, it, start, ds, pv[(it + 1) & 1], pi[(it + 1) & 1], pv[it & 1],
                                     pi[it & 1], perm, lambdas, count, diam, spacing);
  }
  RVGP_LAUNCH_CHECK("rvgp_fps");
  return RVGP_OK;
}

// The same selections in one cooperative launch (see fps_persistent); D <= 8.
// Grid: every CTA resident (the occupancy of the kernel times the SMs, at
// most one CTA per 1024 points).  exact_evals (device long long, optional):
// number of exact FP64 distances evaluated (the rest were screened out in
// FP32).  Returns RVGP_ELAUNCH if a grid barrier timed out.
RVGP_API size_t rvgp_fps_persistent_workspace(int n) {
  return sizeof(double) * ((size_t)n + 4 * (size_t)num_sms() * 8 + 16) + sizeof(float) * (size_t)n * 8 +
         sizeof(int) * (4 * (size_t)num_sms() * 8 + 16) + sizeof(unsigned) * ((size_t)num_sms() * 8 + 8) + 4096;
}

RVGP_API int rvgp_fps_persistent(const double* X, int n, int D, int N_max, int start, const double* diam,
                                 double spacing, int* perm, double* lambdas, int* count, long long* exact_evals,
                                 void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(X && perm && lambdas && count && n >= 1 && D >= 1 && D <= 8, "rvgp_fps_persistent: bad arguments");
  RVGP_CHECK_ARG(N_max >= 1 && N_max <= n && start >= 0 && start < n, "rvgp_fps_persistent: bad N=%d or start=%d",
                 N_max, start);
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_fps_persistent_workspace(n), "rvgp_fps_persistent: workspace");
  cudaStream_t st = as_stream(stream);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fps_persistent, kThreads, 0) != cudaSuccess ||
      per_sm < 1) {
    set_error("rvgp_fps_persistent: occupancy query failed");
    return RVGP_ELAUNCH;
  }
  const int G = std::max(1, std::min(std::min(per_sm, 8) * num_sms(), ceil_div(n, 1024)));
  const int DP = D <= 4 ? 4 : 8;
  const int nprep = std::min(num_sms() * 2, ceil_div(n, kThreads));
  Workspace ws(workspace, ws_bytes);
  double* ds = ws.take<double>(n);
  double* pv = ws.take<double>(2 * (size_t)G);
  int* pi = ws.take<int>(2 * (size_t)G);
  float* X32 = ws.take<float>((size_t)n * DP);
  double* r2part = ws.take<double>(nprep);
  unsigned* flags = ws.take<unsigned>((size_t)G + 1);
  int* err = ws.take<int>(1);
  cudaMemsetAsync(count, 0xFF, sizeof(int), st);  // -1: all N_max taken unless the spacing stop fires
  cudaMemsetAsync(flags, 0, sizeof(unsigned) * ((size_t)G + 1), st);
  cudaMemsetAsync(err, 0, sizeof(int), st);
  if (exact_evals) cudaMemsetAsync(exact_evals, 0, sizeof(long long), st);
  rvgp::note_launch();
  fps_prep<<<nprep, kThreads, 0, st>>>(X, n, D, DP, X32, r2part);
  void* args[] = {(void*)&X, (void*)&X32, (void*)&n, (void*)&D, (void*)&DP, (void*)&N_max, (void*)&start,
                  (void*)&ds, (void*)&pv, (void*)&pi, (void*)&perm, (void*)&lambdas, (void*)&count, (void*)&diam,
                  (void*)&spacing, (void*)&r2part, (void*)&nprep, (void*)&flags, (void*)&err, (void*)&exact_evals};
  rvgp::note_launch();
  if (cudaLaunchCooperativeKernel((const void*)fps_persistent, G, kThreads, args, 0, st) != cudaSuccess)
    return check_launch("rvgp_fps_persistent");
  RVGP_LAUNCH_CHECK("rvgp_fps_persistent");
  int h = 0;
  if (read_back(&h, err, sizeof(int), st) != cudaSuccess) return check_launch("rvgp_fps_persistent");
  if (h) {
    set_error("rvgp_fps_persistent: a grid barrier timed out");
    return RVGP_ELAUNCH;
  }
  return RVGP_OK;
}

RVGP_API size_t rvgp_diameter_workspace(int n) { return sizeof(double) * num_sms() * 4 + 256; }

RVGP_API int rvgp_diameter(const double* X, int n, int D, double* out, void* workspace, size_t ws_bytes,
                           void* stream) {
  RVGP_CHECK_ARG(X && out && n >= 1, "rvgp_diameter: bad arguments");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_diameter_workspace(n), "rvgp_diameter: workspace too small");
  cudaStream_t st = as_stream(stream);
  double* part = static_cast<double*>(workspace);
  rvgp::note_launch(); diameter_tiles<<<num_sms() * 4, kThreads, 0, st>>>(X, n, D, part);
  rvgp::note_launch(); max_reduce<<<1, kThreads, 0, st>>>(part, num_sms() * 4, out);
  RVGP_LAUNCH_CHECK("rvgp_diameter");
  return RVGP_OK;
}

// ------------------------------------------------------------ spatial form
// The same selections with the update confined to where it can change
// anything.  Selecting p with value r = max_x ds[x] lowers ds[x] only where
// d(p, x) < ds[x] <= r.  Points are renumbered along a Morton curve
// (rvgp_locality_order) and cut into blocks of 32 and superblocks of 32
// blocks, each with its bounding box (FP32, rounded outwards, so it contains
// the FP64 points) and the maximum of ds over it (value, then lowest
// original index).  One CTA runs all selections with no grid barrier:
//  A. the next point is the maximum over the superblock maxima (shared
//     memory), compared as integer keys: the bits of a non-negative double
//     order like its value, then the original index;
//  B. superblocks whose box may come closer to p than their maximum are
//     listed: the FP32 box distance lb32 with the certified margin
//     δ = 4u(2R√D + (D+2)·lb32) (u = 2^-24, R the largest point norm: the
//     roundings of p, of the differences, squares, sum and square root), so a
//     superblock is skipped only when lb32 − δ > its maximum for certain;
//  C. a warp owns each listed superblock: the same test per block, then the
//     points of the blocks that pass (lane per point, loads of several
//     blocks in flight) get the FP32 distance with the same margin and, only
//     where it cannot exclude a new minimum, the exact FP64 distance
//     (exact_dist's order); the blocks' maxima stay in the lanes' registers
//     and reduce to the superblock's, whose maximising point's coordinates go
//     to shared memory for step A.
// The stored minima are bit-identical to the other forms', so the three
// forms select the same points with the same lambdas.
namespace rvgp {
namespace {
constexpr int kSpThreads = 512;
constexpr int kBlk = 32;  // points per block
constexpr int kSup = 32;  // blocks per superblock

// (value bits, original index, position): value >= 0, so its bits order like it
struct Key {
  unsigned long long v;
  int orig, pos;
};
__device__ __forceinline__ bool kbetter(const Key& a, const Key& b) {
  return a.v > b.v || (a.v == b.v && a.orig < b.orig);
}
__device__ __forceinline__ Key kpad() { return Key{0ull, INT_MAX, 0}; }
__device__ __forceinline__ Key kof(double v, int orig, int pos) {
  return Key{(unsigned long long)__double_as_longlong(v), orig, pos};
}
__device__ __forceinline__ Key warp_maxk(Key a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Key b{__shfl_xor_sync(0xffffffffu, a.v, o), __shfl_xor_sync(0xffffffffu, a.orig, o),
          __shfl_xor_sync(0xffffffffu, a.pos, o)};
    if (kbetter(b, a)) a = b;
  }
  return a;
}

// FP32 distance from p to the box [lo, hi] and its certified error bound
template <int D>
__device__ __forceinline__ float box_lb32(const float* p, const float* lo, const float* hi) {
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < D; ++j) {
    const float e = fmaxf(0.f, fmaxf(lo[j] - p[j], p[j] - hi[j]));
    s = fmaf(e, e, s);
  }
  return sqrtf(s);
}

// Points in Morton order (FP64 and FP32), ds from the start point, per-block
// FP32 boxes (outward) and maxima (warp per block); the largest squared norm.
__global__ void fps_sp_blocks(const double* __restrict__ X, const int* __restrict__ order, int n, int D, int start,
                              double* __restrict__ Xs, float* __restrict__ Xs32, double* __restrict__ ds,
                              float* __restrict__ box, double* __restrict__ bmax, int* __restrict__ borig,
                              int* __restrict__ bpos, unsigned long long* __restrict__ r2max) {
  const int warp = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  const int nb = (n + kBlk - 1) / kBlk;
  if (warp >= nb) return;
  const int q = warp * kBlk + lane;
  const bool on = q < n;
  const int o = on ? order[q] : 0;
  Key m = kpad();
  double r2 = 0.0;
  if (on) {
    for (int j = 0; j < D; ++j) {
      const double x = X[(size_t)o * D + j];
      Xs[(size_t)q * D + j] = x;
      Xs32[(size_t)q * D + j] = (float)x;
      r2 += x * x;
    }
    const double d = exact_dist(X, D, start, o);
    ds[q] = d;
    m = kof(d, o, q);
  }
  m = warp_maxk(m);
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) r2 = fmax(r2, __shfl_xor_sync(0xffffffffu, r2, s));
  for (int j = 0; j < D; ++j) {
    double lo = on ? X[(size_t)o * D + j] : DBL_MAX, hi = on ? X[(size_t)o * D + j] : -DBL_MAX;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, s));
      hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, s));
    }
    if (lane == 0) {
      box[(size_t)warp * 2 * D + j] = __double2float_rd(lo);
      box[(size_t)warp * 2 * D + D + j] = __double2float_ru(hi);
    }
  }
  if (lane == 0) {
    bmax[warp] = __longlong_as_double((long long)m.v);
    borig[warp] = m.orig;
    bpos[warp] = m.pos;
    atomicMax(r2max, (unsigned long long)__double_as_longlong(r2));
  }
}

// Superblock boxes and maxima, and the coordinates of each superblock's
// maximising point (warp per superblock).
__global__ void fps_sp_super(int nb, int D, const double* __restrict__ Xs, const float* __restrict__ box,
                             const double* __restrict__ bmax, const int* __restrict__ borig,
                             const int* __restrict__ bpos, float* __restrict__ sbox, double* __restrict__ smax,
                             int* __restrict__ sorig, int* __restrict__ spos, double* __restrict__ sxy) {
  const int warp = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  const int ns = (nb + kSup - 1) / kSup;
  if (warp >= ns) return;
  const int b = warp * kSup + lane;
  const bool on = b < nb;
  Key m = on ? kof(bmax[b], borig[b], bpos[b]) : kpad();
  m = warp_maxk(m);
  for (int j = 0; j < D; ++j) {
    float lo = on ? box[(size_t)b * 2 * D + j] : FLT_MAX, hi = on ? box[(size_t)b * 2 * D + D + j] : -FLT_MAX;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
      lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, s));
      hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, s));
    }
    if (lane == 0) {
      sbox[(size_t)warp * 2 * D + j] = lo;
      sbox[(size_t)warp * 2 * D + D + j] = hi;
    }
  }
  if (lane == 0) {
    smax[warp] = __longlong_as_double((long long)m.v);
    sorig[warp] = m.orig;
    spos[warp] = m.pos;
  }
  if (lane < D) sxy[(size_t)warp * D + lane] = Xs[(size_t)m.pos * D + lane];
}

template <int D>
__global__ void __launch_bounds__(kSpThreads, 1)
    fps_sp_select(const double* __restrict__ Xs, const float* __restrict__ Xs32, const int* __restrict__ order,
                  int n, int N_max, double* __restrict__ ds, const float* __restrict__ box,
                  double* __restrict__ bmax, int* __restrict__ borig, int* __restrict__ bpos,
                  const float* __restrict__ sbox_g, const double* __restrict__ smax_g,
                  const int* __restrict__ sorig_g, const int* __restrict__ spos_g, const double* __restrict__ sxy_g,
                  const unsigned long long* __restrict__ r2max, int* __restrict__ perm,
                  double* __restrict__ lambdas, int* __restrict__ count, const double* __restrict__ diam,
                  double spacing, long long* __restrict__ exact_evals) {
  constexpr int GB = D <= 4 ? 4 : 2;  // blocks whose points are loaded together
  constexpr int NW = kSpThreads / 32;
  extern __shared__ __align__(16) unsigned char fsm[];
  const int nb = (n + kBlk - 1) / kBlk, ns = (nb + kSup - 1) / kSup;
  double* sxy = reinterpret_cast<double*>(fsm);          // ns x D
  double* smax = sxy + (size_t)ns * D;                    // ns
  float* sbox = reinterpret_cast<float*>(smax + ns);      // ns x 2D
  int* sorig = reinterpret_cast<int*>(sbox + (size_t)ns * 2 * D);  // ns
  int* spos = sorig + ns;                                  // ns
  int* slist = spos + ns;                                  // ns
  __shared__ double s_p[D];
  __shared__ unsigned long long s_wv[NW];
  __shared__ int s_wo[NW], s_ws[NW];
  __shared__ int s_ns, s_stop;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int s = tid; s < ns; s += kSpThreads) {
    for (int j = 0; j < 2 * D; ++j) sbox[(size_t)s * 2 * D + j] = sbox_g[(size_t)s * 2 * D + j];
    for (int j = 0; j < D; ++j) sxy[(size_t)s * D + j] = sxy_g[(size_t)s * D + j];
    smax[s] = smax_g[s];
    sorig[s] = sorig_g[s];
    spos[s] = spos_g[s];
  }
  const double R = sqrt(__longlong_as_double((long long)*r2max));
  const float u = 5.9604644775390625e-8f;  // 2^-24
  const float c0 = (float)(4.0 * 5.9604644775390625e-8 * 2.0 * R * sqrt((double)D) * (1.0 + 1e-6));
  const float c1 = (float)(4.0 * 5.9604644775390625e-8 * (D + 2) * (1.0 + 1e-6));
  (void)u;
  long long exact = 0;
  __syncthreads();
  for (int it = 1; it < N_max; ++it) {
    // ---- A. the next point: maximum over the superblock maxima (pos = superblock)
    Key m = kpad();
    for (int s = tid; s < ns; s += kSpThreads) {
      const Key c = kof(smax[s], sorig[s], s);
      if (kbetter(c, m)) m = c;
    }
    m = warp_maxk(m);
    if (lane == 0) {
      s_wv[warp] = m.v;
      s_wo[warp] = m.orig;
      s_ws[warp] = m.pos;
    }
    __syncthreads();
    if (warp == 0) {
      Key w = lane < NW ? Key{s_wv[lane], s_wo[lane], s_ws[lane]} : kpad();
      w = warp_maxk(w);  // the same in every lane
      if (lane == 0) {
        const double v = __longlong_as_double((long long)w.v);
        s_stop = 0;
        s_ns = 0;
        if (diam && v / diam[0] < spacing) {
          s_stop = 1;
          *count = it;
        } else {
          perm[it] = w.orig;
          lambdas[it] = v;
        }
      }
      if (lane < D) s_p[lane] = sxy[(size_t)w.pos * D + lane];
    }
    __syncthreads();
    if (s_stop) break;
    double p[D];
    float p32[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      p[j] = s_p[j];
      p32[j] = (float)p[j];
    }
    // ---- B. superblocks that may hold a point whose minimum p can lower
    for (int s = tid; s < ns; s += kSpThreads) {
      const float lb = box_lb32<D>(p32, sbox + (size_t)s * 2 * D, sbox + (size_t)s * 2 * D + D);
      if (!((double)(lb - (c0 + c1 * lb)) > smax[s])) slist[atomicAdd(&s_ns, 1)] = s;
    }
    __syncthreads();
    // ---- C. each listed superblock by one warp
    const int nsl = s_ns;
    for (int e = warp; e < nsl; e += NW) {
      const int sb = slist[e];
      const int b = sb * kSup + lane;
      const bool valid = b < nb;
      Key bm = kpad();
      bool need = false;
      if (valid) {
        const double bv = bmax[b];
        bm = kof(bv, borig[b], bpos[b]);
        const float lb = box_lb32<D>(p32, box + (size_t)b * 2 * D, box + (size_t)b * 2 * D + D);
        need = !((double)(lb - (c0 + c1 * lb)) > bv);
      }
      unsigned mask = __ballot_sync(0xffffffffu, need);
      while (mask) {  // warp-uniform
        int bl[GB];
#pragma unroll
        for (int t = 0; t < GB; ++t) {
          bl[t] = -1;
          if (mask) {
            bl[t] = __ffs(mask) - 1;
            mask &= mask - 1;
          }
        }
        double cur[GB];
        float x[GB][D];
        int q[GB], o[GB];
#pragma unroll
        for (int t = 0; t < GB; ++t) {
          q[t] = bl[t] >= 0 ? (sb * kSup + bl[t]) * kBlk + lane : n;
          if (q[t] < n) {
            cur[t] = ds[q[t]];
            o[t] = order[q[t]];
#pragma unroll
            for (int j = 0; j < D; ++j) x[t][j] = Xs32[(size_t)q[t] * D + j];
          }
        }
#pragma unroll
        for (int t = 0; t < GB; ++t) {
          if (bl[t] < 0) break;  // warp-uniform
          Key mm = kpad();
          if (q[t] < n) {
            double c = cur[t];
            if (c > 0.0) {
              float s2 = 0.f;
#pragma unroll
              for (int j = 0; j < D; ++j) {
                const float df = p32[j] - x[t][j];
                s2 = fmaf(df, df, s2);
              }
              const float d32 = sqrtf(s2);
              if (!((double)(d32 - (c0 + c1 * d32)) > c)) {  // cannot rule out a new minimum
                double acc = 0.0;
#pragma unroll
                for (int j = 0; j < D; ++j) {
                  const double df = __dsub_rn(p[j], Xs[(size_t)q[t] * D + j]);
                  acc = __dadd_rn(acc, __dmul_rn(df, df));
                }
                const double d = sqrt(acc);
                ++exact;
                if (d < c) {
                  c = d;
                  ds[q[t]] = d;
                }
              }
            }
            mm = kof(c, o[t], q[t]);
          }
          mm = warp_maxk(mm);
          const int bb = sb * kSup + bl[t];
          if (lane == bl[t]) bm = mm;
          if (lane == 0) {
            bmax[bb] = __longlong_as_double((long long)mm.v);
            borig[bb] = mm.orig;
            bpos[bb] = mm.pos;
          }
        }
      }
      const Key sm = warp_maxk(bm);
      if (lane == 0) {
        smax[sb] = __longlong_as_double((long long)sm.v);
        sorig[sb] = sm.orig;
        spos[sb] = sm.pos;
      }
      if (lane < D) sxy[(size_t)sb * D + lane] = Xs[(size_t)sm.pos * D + lane];
    }
    __syncthreads();
  }
  if (exact_evals) atomicAdd((unsigned long long*)exact_evals, (unsigned long long)exact);
}

__global__ void write_first(int* perm, double* lambdas, int start) {
  if (threadIdx.x == 0) {
    perm[0] = start;
    lambdas[0] = 0.0;
  }
}

__global__ void add_ll(long long* p, long long v) { *p += v; }

size_t fps_sp_smem(int n, int D) {
  const int nb = (n + kBlk - 1) / kBlk, ns = (nb + kSup - 1) / kSup;
  return (size_t)ns * (D * sizeof(double) + sizeof(double) + 2 * D * sizeof(float) + 3 * sizeof(int));
}

struct SpBufs {
  int *order, *rank, *borig, *bpos, *sorig, *spos;
  double *Xs, *ds, *bmax, *smax, *sxy;
  float *Xs32, *box, *sbox;
  unsigned long long* r2max;
  void* lo_ws;
  size_t lo_bytes;
};
}  // namespace
}  // namespace rvgp

extern "C" size_t rvgp_locality_order_workspace(int n, int D);
extern "C" int rvgp_locality_order(const double* X, int n, int D, int* perm, int* rank, void* workspace,
                                   size_t ws_bytes, void* stream);

namespace {
// one carve for the size query and the call
rvgp::SpBufs carve_sp(Workspace& ws, int n, int D) {
  using namespace rvgp;
  const int nb = (n + kBlk - 1) / kBlk, ns = (nb + kSup - 1) / kSup;
  SpBufs b;
  b.order = ws.take<int>(n);
  b.rank = ws.take<int>(n);
  b.Xs = ws.take<double>((size_t)n * D);
  b.Xs32 = ws.take<float>((size_t)n * D);
  b.ds = ws.take<double>(n);
  b.box = ws.take<float>((size_t)nb * 2 * D);
  b.bmax = ws.take<double>(nb);
  b.borig = ws.take<int>(nb);
  b.bpos = ws.take<int>(nb);
  b.sbox = ws.take<float>((size_t)ns * 2 * D);
  b.sxy = ws.take<double>((size_t)ns * D);
  b.smax = ws.take<double>(ns);
  b.sorig = ws.take<int>(ns);
  b.spos = ws.take<int>(ns);
  b.r2max = ws.take<unsigned long long>(1);
  b.lo_bytes = rvgp_locality_order_workspace(n, D);
  b.lo_ws = ws.take<char>(b.lo_bytes);
  return b;
}
}  // namespace

// Largest n the spatial form takes for dimension D (its superblock table
// must fit one SM's shared memory), 0 when D is outside 1..8.
RVGP_API int rvgp_fps_spatial_max_n(int D) {
  if (D < 1 || D > 8) return 0;
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return 0;
  const size_t per = D * sizeof(double) + sizeof(double) + 2 * D * sizeof(float) + 3 * sizeof(int);
  const long long ns = ((long long)optin - 2048) / (long long)per;
  return (int)std::min<long long>(INT_MAX / 2, ns * rvgp::kBlk * rvgp::kSup);
}

RVGP_API size_t rvgp_fps_spatial_workspace(int n, int D) {
  if (n < 1 || D < 1 || D > 8) return 0;
  Workspace ws(nullptr, 0);
  carve_sp(ws, n, D);
  return ws.used;
}

// Same arguments and results as rvgp_fps_persistent; n <= rvgp_fps_spatial_max_n(D).
RVGP_API int rvgp_fps_spatial(const double* X, int n, int D, int N_max, int start, const double* diam,
                              double spacing, int* perm, double* lambdas, int* count, long long* exact_evals,
                              void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(X && perm && lambdas && count && n >= 1 && D >= 1 && D <= 8, "rvgp_fps_spatial: bad arguments");
  RVGP_CHECK_ARG(N_max >= 1 && N_max <= n && start >= 0 && start < n, "rvgp_fps_spatial: bad N=%d or start=%d",
                 N_max, start);
  RVGP_CHECK_ARG(n <= rvgp_fps_spatial_max_n(D), "rvgp_fps_spatial: n=%d above the limit %d for D=%d", n,
                 rvgp_fps_spatial_max_n(D), D);
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_fps_spatial_workspace(n, D), "rvgp_fps_spatial: workspace");
  using namespace rvgp;
  cudaStream_t st = as_stream(stream);
  const int nb = (n + kBlk - 1) / kBlk, ns = (nb + kSup - 1) / kSup;
  Workspace ws(workspace, ws_bytes);
  const SpBufs B = carve_sp(ws, n, D);
  TRY_RC(rvgp_locality_order(X, n, D, B.order, B.rank, B.lo_ws, B.lo_bytes, stream));
  cudaMemsetAsync(count, 0xFF, sizeof(int), st);  // -1: all N_max taken unless the spacing stop fires
  cudaMemsetAsync(B.r2max, 0, sizeof(unsigned long long), st);
  if (exact_evals) cudaMemsetAsync(exact_evals, 0, sizeof(long long), st);
  rvgp::note_launch();
  fps_sp_blocks<<<ceil_div((long long)nb * 32, 256), 256, 0, st>>>(X, B.order, n, D, start, B.Xs, B.Xs32, B.ds,
                                                                    B.box, B.bmax, B.borig, B.bpos, B.r2max);
  rvgp::note_launch();
  fps_sp_super<<<ceil_div((long long)ns * 32, 256), 256, 0, st>>>(nb, D, B.Xs, B.box, B.bmax, B.borig, B.bpos,
                                                                   B.sbox, B.smax, B.sorig, B.spos, B.sxy);
  rvgp::note_launch();
  write_first<<<1, 32, 0, st>>>(perm, lambdas, start);
  if (N_max > 1) {
    const size_t smem = fps_sp_smem(n, D);
#define RVGP_FPS_SP(Dv)                                                                                        \
  case Dv: {                                                                                                   \
    if (raise_dyn_smem((const void*)fps_sp_select<Dv>, (size_t)(smem)) !=    \
        cudaSuccess)                                                                                           \
      return check_launch("rvgp_fps_spatial");                                                                 \
    rvgp::note_launch();                                                                                       \
    fps_sp_select<Dv><<<1, kSpThreads, smem, st>>>(B.Xs, B.Xs32, B.order, n, N_max, B.ds, B.box, B.bmax,       \
                                                   B.borig, B.bpos, B.sbox, B.smax, B.sorig, B.spos, B.sxy,    \
                                                   B.r2max, perm, lambdas, count, diam, spacing, exact_evals); \
    break;                                                                                                     \
  }
    switch (D) {
      RVGP_FPS_SP(1)
      RVGP_FPS_SP(2)
      RVGP_FPS_SP(3)
      RVGP_FPS_SP(4)
      RVGP_FPS_SP(5)
      RVGP_FPS_SP(6)
      RVGP_FPS_SP(7)
      default: RVGP_FPS_SP(8)
    }
#undef RVGP_FPS_SP
  }
  RVGP_LAUNCH_CHECK("rvgp_fps_spatial");
  if (exact_evals) {
    // the n distances from the start point
    rvgp::note_launch();
    add_ll<<<1, 1, 0, st>>>(exact_evals, (long long)n);
  }
  return RVGP_OK;
}
