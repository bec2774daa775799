// Per-edge parallel transport and the block connection Laplacian.
//
// Replaces _parallel_transport_dijkstra (RVGP/lib/ptu_dijkstra.pyx:221-293),
// expand_edge_index (pyx:202-214) and compute_connection_laplacian
// (RVGP/geometry.py:14-52, normalization=None).
//
// For every stored entry (i, j) of the symmetrised CSR, in CSR order:
//   M = T_iᵀ T_j (d x d),  R_ij = U Vᵀ  where  M = U S Vᵀ,
// i.e. the orthogonal polar factor of M (the closest orthogonal matrix; a
// reflection when det M < 0, as LAPACK's U Vᵀ is).  For d = 2 it is closed
// form: (M + det(M) M^-ᵀ)/|..| reduces to
//   det >= 0: [[a+d, b-c], [c-b, a+d]] / hypot(a+d, c-b)
//   det <  0: [[a-d, b+c], [b+c, d-a]] / hypot(a-d, b+c).
// For d > 2 a one-sided Jacobi SVD of M gives U and V.
//
// The connection Laplacian is stored as block CSR with the graph's pattern:
// block (i, j) = L_ij R_ij, i.e. deg_i R_ii on the diagonal and -R_ij off it,
// in FP64 and an FP32 copy for the mixed-precision products.
#include "common.cuh"

namespace rvgp {
namespace {

constexpr int kWarps = 4;
constexpr int kMaxD = 8;

__device__ void polar2(const double* m, double* R) {
  const double a = m[0], b = m[1], c = m[2], d = m[3];
  const double det = a * d - b * c;
  if (det >= 0.0) {
    double x = a + d, y = c - b, h = hypot(x, y);
    if (h == 0.0) { R[0] = 1; R[1] = 0; R[2] = 0; R[3] = 1; return; }
    x /= h; y /= h;
    R[0] = x; R[1] = -y; R[2] = y; R[3] = x;
  } else {
    double x = a - d, y = b + c, h = hypot(x, y);
    x /= h; y /= h;
    R[0] = x; R[1] = y; R[2] = y; R[3] = -x;
  }
}

// General d: M = U S Vᵀ by one-sided Jacobi on M (columns), V = accumulated rotations.
__device__ void polar_general(const double* m, int d, double* R) {
  double A[kMaxD * kMaxD], V[kMaxD * kMaxD];  // column-major: A[col*d + row]
  for (int p = 0; p < d; ++p)
    for (int q = 0; q < d; ++q) {
      A[q * d + p] = m[p * d + q];
      V[q * d + p] = p == q ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rot = false;
    for (int p = 0; p < d - 1; ++p)
      for (int q = p + 1; q < d; ++q) {
        double al = 0, be = 0, ga = 0;
        for (int t = 0; t < d; ++t) {
          al += A[p * d + t] * A[p * d + t];
          be += A[q * d + t] * A[q * d + t];
          ga += A[p * d + t] * A[q * d + t];
        }
        if (ga == 0.0 || fabs(ga) <= 1e-15 * sqrt(al * be)) continue;
        rot = true;
        double zeta = (be - al) / (2 * ga);
        double tt = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1 + zeta * zeta));
        double cs = 1 / sqrt(1 + tt * tt), sn = cs * tt;
        for (int t = 0; t < d; ++t) {
          double x = A[p * d + t], y = A[q * d + t];
          A[p * d + t] = cs * x - sn * y;
          A[q * d + t] = sn * x + cs * y;
          x = V[p * d + t];
          y = V[q * d + t];
          V[p * d + t] = cs * x - sn * y;
          V[q * d + t] = sn * x + cs * y;
        }
      }
    if (!rot) break;
  }
  // U columns = A columns / norms; R = U Vᵀ
  for (int p = 0; p < d; ++p) {
    double nrm = 0;
    for (int t = 0; t < d; ++t) nrm += A[p * d + t] * A[p * d + t];
    nrm = sqrt(nrm);
    for (int t = 0; t < d; ++t) A[p * d + t] = nrm > 0 ? A[p * d + t] / nrm : (t == p ? 1.0 : 0.0);
  }
  for (int p = 0; p < d; ++p)
    for (int q = 0; q < d; ++q) {
      double s = 0;
      for (int k = 0; k < d; ++k) s += A[k * d + p] * V[k * d + q];
      R[p * d + q] = s;
    }
}

__global__ void connections_kernel(const double* __restrict__ T, int n, int D, int ld, int d,
                                   const int* __restrict__ indptr, const int* __restrict__ indices,
                                   double* __restrict__ R, double* __restrict__ lc64, float* __restrict__ lc32) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (i >= n) return;
  const int s = indptr[i], e = indptr[i + 1];
  const double deg = (double)(e - s - 1);
  for (int t = s + lane; t < e; t += 32) {
    const int j = indices[t];
    double m[kMaxD * kMaxD], r[kMaxD * kMaxD];
    for (int p = 0; p < d; ++p)
      for (int q = 0; q < d; ++q) {
        double acc = 0.0;
        for (int k = 0; k < D; ++k) acc += T[((size_t)i * D + k) * ld + p] * T[((size_t)j * D + k) * ld + q];
        m[p * d + q] = acc;
      }
    if (d == 1) r[0] = m[0] >= 0.0 ? 1.0 : -1.0;
    else if (d == 2) polar2(m, r);
    else polar_general(m, d, r);
    const double scale = j == i ? deg : -1.0;
    for (int pq = 0; pq < d * d; ++pq) {
      size_t o = (size_t)t * d * d + pq;
      if (R) R[o] = r[pq];
      const double v = scale * r[pq];
      if (lc64) lc64[o] = v;
      if (lc32) lc32[o] = (float)v;
    }
  }
}

}  // namespace
}  // namespace rvgp

using namespace rvgp;

// T: tangents (n, D, ld) f64, the first d columns used.  R: (E, d, d) f64
// transports in CSR order.  lc64 / lc32: block-CSR values of the connection
// Laplacian (E, d, d), either may be null.
RVGP_API int rvgp_connections(const double* T, int n, int D, int ld, int d, const int* indptr, const int* indices,
                              double* R, double* lc64, float* lc32, void* stream) {
  RVGP_CHECK_ARG(T && indptr && indices, "rvgp_connections: null pointer");
  RVGP_CHECK_ARG(d >= 1 && d <= kMaxD && d <= D && d <= ld,
                 "Embedding dimension must be less or equal to the ambient dimension of input data");
  rvgp::note_launch(); connections_kernel<<<ceil_div(n, kWarps), 32 * kWarps, 0, as_stream(stream)>>>(T, n, D, ld, d, indptr, indices, R,
                                                                                  lc64, lc32);
  RVGP_LAUNCH_CHECK("rvgp_connections");
  return RVGP_OK;
}
