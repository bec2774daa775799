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
#include <math.h>

namespace rvgp {
namespace {

__device__ __forceinline__ void unit3(const double* v, double* u) {
  const double nrm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  u[0] = v[0] / nrm;
  u[1] = v[1] / nrm;
  u[2] = v[2] / nrm;
}

// one thread per (field b, point j)
__global__ void __launch_bounds__(256) vf_features_kernel(const double* __restrict__ P, int n,
                                                          const double* __restrict__ V, int B,
                                                          const int* __restrict__ nbr, int k, int ref_first,
                                                          double* __restrict__ div, double* __restrict__ curl) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)B * n) return;
  const int b = (int)(e / n), j = (int)(e % n);
  const double* Vb = V + (size_t)b * n * 3;
  double ur[3];
  unit3(Vb + (size_t)(ref_first ? 0 : j) * 3, ur);
  const double px = P[(size_t)j * 3], py = P[(size_t)j * 3 + 1], pz = P[(size_t)j * 3 + 2];
  double dv = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0;
  for (int q = 0; q < k; ++q) {
    const int i = nbr[(size_t)j * k + q];
    const double dx = P[(size_t)i * 3] - px, dy = P[(size_t)i * 3 + 1] - py, dz = P[(size_t)i * 3 + 2] - pz;
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    const double r2 = r * r;
    double ui[3];
    unit3(Vb + (size_t)i * 3, ui);
    const double ax = ui[0] - ur[0], ay = ui[1] - ur[1], az = ui[2] - ur[2];
    dv += (ax * dx + ay * dy + az * dz) / r2;
    c0 += (ay * dz - az * dy) / r2;
    c1 += (az * dx - ax * dz) / r2;
    c2 += (ax * dy - ay * dx) / r2;
  }
  div[e] = dv / k;
  curl[e * 3] = c0 / k;
  curl[e * 3 + 1] = c1 / k;
  curl[e * 3 + 2] = c2 / k;
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

// P (n x 3), V (B x n x 3), nbr (n x k, the k nearest neighbours of every
// point, excluding the point) -> div (B x n), curl (B x n x 3).  ref_first = 1
// takes the reference vector of every point from point 0, as the reference does.
RVGP_API int rvgp_vectorfield_features(const double* P, int n, const double* V, int B, const int* nbr, int k,
                                       int ref_first, double* div, double* curl, void* stream) {
  RVGP_CHECK_ARG(P && V && nbr && div && curl && n >= 1 && B >= 1 && k >= 1,
                 "rvgp_vectorfield_features: bad arguments");
  note_launch();
  vf_features_kernel<<<ceil_div((long long)B * n, 256), 256, 0, as_stream(stream)>>>(P, n, V, B, nbr, k,
                                                                                      ref_first ? 1 : 0, div, curl);
  RVGP_LAUNCH_CHECK("rvgp_vectorfield_features");
  return RVGP_OK;
}
