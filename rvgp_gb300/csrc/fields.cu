// Per-point field operations and the manifold-dimension estimate.
//
//   manifold_dimension  RVGP/geometry.py:83-97
//   project_to_manifold RVGP/geometry.py:165-168   v <- T Tᵀ v
//   express_in_local_frame RVGP/geometry.py:171-175  c = Tᵀ v  /  v = T c
//   row normalisation   RVGP/dataclass.py:103 (v /= |v|)
#include "common.cuh"
#include <math.h>

namespace rvgp {
namespace {

constexpr int kCTA = 1024;
constexpr int kMaxC = 128;

// One CTA: normalised cumulative explained variance per point, mean - std over
// points per column (two passes, fixed order), first column >= frac.
__global__ void __launch_bounds__(kCTA) dimension_kernel(const double* __restrict__ sigma, int n, int c, double frac,
                                                         double* __restrict__ var_exp, int* __restrict__ dim) {
  __shared__ double sh[kCTA];
  __shared__ double mean[kMaxC];
  auto cum = [&](int i, int j) {
    double tot = 0.0, run = 0.0;
    for (int q = 0; q < c; ++q) {
      double s = sigma[(size_t)i * c + q];
      tot += s * s;
      if (q <= j) run += s * s;
    }
    return run / tot;
  };
  for (int j = 0; j < c; ++j) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += cum(i, j);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) mean[j] = sh[0] / n;
    __syncthreads();
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double d = cum(i, j) - mean[j];
      v += d * d;
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
    }
    if (threadIdx.x == 0) var_exp[j] = mean[j] - sqrt(sh[0] / n);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int d = -1;
    for (int j = 0; j < c; ++j)
      if (var_exp[j] >= frac) {
        d = j + 1;
        break;
      }
    *dim = d;
  }
}

// mode 0: out = T Tᵀ v (n, D); mode 1: out = Tᵀ v (n, d); mode 2: out = T v (v: (n, d), out (n, D))
__global__ void frame_kernel(const double* __restrict__ T, int n, int D, int ld, int d, const double* __restrict__ v,
                             int mode, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double c[8];
  if (mode == 2) {
    for (int q = 0; q < d; ++q) c[q] = v[(size_t)i * d + q];
  } else {
    for (int q = 0; q < d; ++q) {
      double s = 0.0;
      for (int a = 0; a < D; ++a) s += T[((size_t)i * D + a) * ld + q] * v[(size_t)i * D + a];
      c[q] = s;
    }
  }
  if (mode == 1) {
    for (int q = 0; q < d; ++q) out[(size_t)i * d + q] = c[q];
    return;
  }
  for (int a = 0; a < D; ++a) {
    double s = 0.0;
    for (int q = 0; q < d; ++q) s += c[q] * T[((size_t)i * D + a) * ld + q];
    out[(size_t)i * D + a] = s;
  }
}

__global__ void normalise_rows(double* __restrict__ v, int n, int D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int a = 0; a < D; ++a) s += v[(size_t)i * D + a] * v[(size_t)i * D + a];
  s = sqrt(s);
  for (int a = 0; a < D; ++a) v[(size_t)i * D + a] /= s;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

// var_exp: c doubles (device); dim: one device int (-1 if no column reaches frac).
RVGP_API int rvgp_manifold_dimension(const double* sigma, int n, int c, double frac, double* var_exp, int* dim,
                                     void* stream) {
  RVGP_CHECK_ARG(sigma && var_exp && dim && n >= 1 && c >= 1 && c <= kMaxC, "rvgp_manifold_dimension: bad arguments");
  rvgp::note_launch(); dimension_kernel<<<1, kCTA, 0, as_stream(stream)>>>(sigma, n, c, frac, var_exp, dim);
  RVGP_LAUNCH_CHECK("rvgp_manifold_dimension");
  return RVGP_OK;
}

// mode 0 project (n, D) -> (n, D); 1 to local frame (n, D) -> (n, d); 2 from local frame (n, d) -> (n, D).
RVGP_API int rvgp_frame_map(const double* T, int n, int D, int ld, int d, const double* v, int mode, double* out,
                            void* stream) {
  RVGP_CHECK_ARG(T && v && out && d >= 1 && d <= 8 && d <= ld && mode >= 0 && mode <= 2, "rvgp_frame_map: bad args");
  rvgp::note_launch(); frame_kernel<<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(T, n, D, ld, d, v, mode, out);
  RVGP_LAUNCH_CHECK("rvgp_frame_map");
  return RVGP_OK;
}

RVGP_API int rvgp_normalise_rows(double* v, int n, int D, void* stream) {
  RVGP_CHECK_ARG(v && n >= 0 && D >= 1, "rvgp_normalise_rows: bad arguments");
  rvgp::note_launch(); normalise_rows<<<ceil_div(n, 128), 128, 0, as_stream(stream)>>>(v, n, D);
  RVGP_LAUNCH_CHECK("rvgp_normalise_rows");
  return RVGP_OK;
}
