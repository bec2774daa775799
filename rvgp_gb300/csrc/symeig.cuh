// Eigen-decomposition of a small dense symmetric matrix in FP64, one thread
// per matrix (internal; used by the gauges for the Gram matrix of a
// neighbourhood).
//
// Householder reduction to tridiagonal form, accumulating the orthogonal
// transformation, then the implicit QL iteration with Wilkinson-type shifts on
// the tridiagonal matrix, applying every plane rotation to the accumulated
// basis (the classical two-stage method for symmetric matrices, O(4n³/3) +
// O(3n³) flops instead of the O(n³) per sweep of cyclic Jacobi).
//
// The matrix is reached through an accessor a(i, j) (row i, column j), so the
// caller chooses the storage (the gauges keep it in interleaved global
// scratch).  On return a(i, j) holds component i of eigenvector j and w[j]
// its eigenvalue (unsorted).  Returns false if some eigenvalue needed more
// than 60 QL iterations.
#pragma once
#include <math.h>

namespace rvgp {
namespace symeig {

template <class Acc>
__host__ __device__ void householder_tridiagonal(Acc& a, int n, double* w, double* e) {
  for (int i = n - 1; i >= 1; --i) {
    const int l = i - 1;
    double h = 0.0;
    if (l > 0) {
      double scale = 0.0;
      for (int k = 0; k <= l; ++k) scale += fabs(a(i, k));
      if (scale == 0.0) {
        e[i] = a(i, l);
      } else {
        // u = row i (columns 0..l) scaled; H = |u|²/2 after the shift of u_l
        for (int k = 0; k <= l; ++k) {
          a(i, k) /= scale;
          h += a(i, k) * a(i, k);
        }
        double f = a(i, l);
        double g = f >= 0.0 ? -sqrt(h) : sqrt(h);
        e[i] = scale * g;
        h -= f * g;
        a(i, l) = f - g;
        f = 0.0;
        for (int j = 0; j <= l; ++j) {
          a(j, i) = a(i, j) / h;  // u / H, kept for the accumulation below
          g = 0.0;                // (A u)_j from the lower triangle
          for (int k = 0; k <= j; ++k) g += a(j, k) * a(i, k);
          for (int k = j + 1; k <= l; ++k) g += a(k, j) * a(i, k);
          e[j] = g / h;  // p = A u / H
          f += e[j] * a(i, j);
        }
        const double hh = f / (h + h);  // K = uᵀp / 2H
        for (int j = 0; j <= l; ++j) {  // A <- A - u qᵀ - q uᵀ, q = p - K u
          f = a(i, j);
          e[j] = g = e[j] - hh * f;
          for (int k = 0; k <= j; ++k) a(j, k) -= (f * e[k] + g * a(i, k));
        }
      }
    } else {
      e[i] = a(i, l);
    }
    w[i] = h;
  }
  w[0] = 0.0;
  e[0] = 0.0;
  // accumulate Q = P_1 P_2 ... in place (rows / columns 0..i-1 hold the
  // reflectors, w[i] != 0 marks a non-trivial one)
  for (int i = 0; i < n; ++i) {
    const int l = i - 1;
    if (w[i] != 0.0) {
      for (int j = 0; j <= l; ++j) {
        double g = 0.0;
        for (int k = 0; k <= l; ++k) g += a(i, k) * a(k, j);
        for (int k = 0; k <= l; ++k) a(k, j) -= g * a(k, i);
      }
    }
    w[i] = a(i, i);
    a(i, i) = 1.0;
    for (int j = 0; j <= l; ++j) {
      a(j, i) = 0.0;
      a(i, j) = 0.0;
    }
  }
}

// Implicit QL on the tridiagonal (w diagonal, e[1..n-1] sub-diagonal as
// produced above); rotations applied to the columns of a.
template <class Acc>
__host__ __device__ bool tridiagonal_ql(Acc& a, int n, double* w, double* e) {
  for (int i = 1; i < n; ++i) e[i - 1] = e[i];
  e[n - 1] = 0.0;
  bool ok = true;
  for (int l = 0; l < n; ++l) {
    int iter = 0, m;
    do {
      for (m = l; m < n - 1; ++m) {  // first negligible off-diagonal at or after l
        const double dd = fabs(w[m]) + fabs(w[m + 1]);
        if (fabs(e[m]) <= 1e-16 * dd) break;
      }
      if (m != l) {
        if (iter++ == 60) {
          ok = false;
          break;
        }
        double g = (w[l + 1] - w[l]) / (2.0 * e[l]);  // shift from the leading 2 x 2 block
        double r = hypot(g, 1.0);
        g = w[m] - w[l] + e[l] / (g + (g >= 0.0 ? fabs(r) : -fabs(r)));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        bool deflated = false;
        for (i = m - 1; i >= l; --i) {
          double f = s * e[i];
          const double b = c * e[i];
          e[i + 1] = r = hypot(f, g);
          if (r == 0.0) {  // underflow: the rotation splits the matrix
            w[i + 1] -= p;
            e[m] = 0.0;
            deflated = true;
            break;
          }
          s = f / r;
          c = g / r;
          g = w[i + 1] - p;
          r = (w[i] - g) * s + 2.0 * c * b;
          p = s * r;
          w[i + 1] = g + p;
          g = c * r - b;
          for (int k = 0; k < n; ++k) {
            f = a(k, i + 1);
            a(k, i + 1) = s * a(k, i) + c * f;
            a(k, i) = c * a(k, i) - s * f;
          }
        }
        if (deflated) continue;
        w[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
  }
  return ok;
}

template <class Acc>
__host__ __device__ bool eigh(Acc& a, int n, double* w, double* e) {
  householder_tridiagonal(a, n, w, e);
  return tridiagonal_ql(a, n, w, e);
}

}  // namespace symeig
}  // namespace rvgp
