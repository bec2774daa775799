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
