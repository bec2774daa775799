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
