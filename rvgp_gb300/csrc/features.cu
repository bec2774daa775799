// Vector-field features: divergence and curl estimates from the k nearest
// neighbours of every point (examples/eeg_example/eeg_utils.py:46-80,
// compute_vectorfield_features), for B fields on the same points in one launch.
//
// With unit vectors u = v/|v| and, for each neighbour i of point j,
// Δp = p_i − p_j and Δu = u_i − u_ref:
//   div_j  = (1/k) Σ_i (Δu·Δp) / |Δp|²,   curl_j = (1/k) Σ_i (Δu × Δp) / |Δp|²
// u_ref is u_j, or, as the reference computes it, u_0 (the unit vector of
// point 0 for every j).
#include "common.cuh"
#include "linalg.cuh"
#include <math.h>

namespace rvgp {
namespace {

// Three passes, so that no FP64 division or square root is repeated per field
// (on GB300 every FP64 warp instruction occupies the SM's FP64 pipe for
// ~19 cycles, and a division is a long FP64 sequence):
//   geometry (per point and neighbour, shared by all fields): e = Δp / |Δp|²,
//     with |Δp|² formed as the square of the norm, as the reference does;
//   unit vectors (per field and point): u = v · 1/|v|;
//   features (per field and point): div += Δu·e, curl += Δu × e, times 1/k.

__global__ void vf_geometry(const double* __restrict__ P, int n, const int* __restrict__ nbr, int k,
                            double* __restrict__ e) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)n * k) return;
  const int j = (int)(t / k), i = nbr[t];
  const double dx = P[(size_t)i * 3] - P[(size_t)j * 3], dy = P[(size_t)i * 3 + 1] - P[(size_t)j * 3 + 1],
               dz = P[(size_t)i * 3 + 2] - P[(size_t)j * 3 + 2];
  const double r = sqrt(dx * dx + dy * dy + dz * dz);
  const double w = 1.0 / (r * r);
  e[t * 3] = dx * w;
  e[t * 3 + 1] = dy * w;
  e[t * 3 + 2] = dz * w;
}

__global__ void vf_unit(const double* __restrict__ V, long long rows, double* __restrict__ U) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= rows) return;
  const double x = V[t * 3], y = V[t * 3 + 1], z = V[t * 3 + 2];
  const double s = rsqrt_nr(x * x + y * y + z * z);
  U[t * 3] = x * s;
  U[t * 3 + 1] = y * s;
  U[t * 3 + 2] = z * s;
}

// one thread per (field b, point j)
__global__ void __launch_bounds__(256) vf_features_kernel(const double* __restrict__ U, int n,
                                                          const double* __restrict__ E, int B,
                                                          const int* __restrict__ nbr, int k, int ref_first,
                                                          double inv_k, double* __restrict__ div,
                                                          double* __restrict__ curl) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)B * n) return;
  const int b = (int)(t / n), j = (int)(t % n);
  const double* Ub = U + (size_t)b * n * 3;
  const double* ur = Ub + (size_t)(ref_first ? 0 : j) * 3;
  const double rx = ur[0], ry = ur[1], rz = ur[2];
  double dv = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0;
  for (int q = 0; q < k; ++q) {
    const size_t s = (size_t)j * k + q;
    const double* ui = Ub + (size_t)nbr[s] * 3;
    const double ex = E[s * 3], ey = E[s * 3 + 1], ez = E[s * 3 + 2];
    const double ax = ui[0] - rx, ay = ui[1] - ry, az = ui[2] - rz;
    dv += ax * ex + ay * ey + az * ez;
    c0 += ay * ez - az * ey;
    c1 += az * ex - ax * ez;
    c2 += ax * ey - ay * ex;
  }
  div[t] = dv * inv_k;
  curl[t * 3] = c0 * inv_k;
  curl[t * 3 + 1] = c1 * inv_k;
  curl[t * 3 + 2] = c2 * inv_k;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

RVGP_API size_t rvgp_vectorfield_features_workspace(int n, int B, int k) {
  return sizeof(double) * ((size_t)n * k * 3 + (size_t)B * n * 3) + 512;
}

// P (n x 3), V (B x n x 3), nbr (n x k, the k nearest neighbours of every
// point, excluding the point) -> div (B x n), curl (B x n x 3).  ref_first = 1
// takes the reference vector of every point from point 0, as the reference does.
RVGP_API int rvgp_vectorfield_features(const double* P, int n, const double* V, int B, const int* nbr, int k,
                                       int ref_first, double* div, double* curl, void* ws, size_t ws_bytes,
                                       void* stream) {
  RVGP_CHECK_ARG(P && V && nbr && div && curl && ws && n >= 1 && B >= 1 && k >= 1,
                 "rvgp_vectorfield_features: bad arguments");
  RVGP_CHECK_ARG(ws_bytes >= rvgp_vectorfield_features_workspace(n, B, k),
                 "rvgp_vectorfield_features: workspace too small");
  cudaStream_t st = as_stream(stream);
  Workspace w(ws, ws_bytes);
  double* E = w.take<double>((size_t)n * k * 3);
  double* U = w.take<double>((size_t)B * n * 3);
  note_launch();
  vf_geometry<<<ceil_div((long long)n * k, 256), 256, 0, st>>>(P, n, nbr, k, E);
  note_launch();
  vf_unit<<<ceil_div((long long)B * n, 256), 256, 0, st>>>(V, (long long)B * n, U);
  note_launch();
  vf_features_kernel<<<ceil_div((long long)B * n, 256), 256, 0, st>>>(U, n, E, B, nbr, k, ref_first ? 1 : 0,
                                                                       1.0 / k, div, curl);
  RVGP_LAUNCH_CHECK("rvgp_vectorfield_features");
  return RVGP_OK;
}
