// FP32 Cholesky of a small symmetric positive definite matrix held in one
// SM's shared memory (internal; used by the mixed-precision GP fit and the
// eigensolver's Cholesky QR).
//
// A is m x m, row-major with stride ld (lda32(m)), lower triangle used.  The
// factorisation is blocked in 32-wide panels: warp 0 factors the diagonal
// block (chol_diag_block), all warps solve the panel below it (panel_solve)
// and update the trailing matrix in 4 x 4 register tiles (trailing_update);
// chol32_cta runs the whole sequence with CTA barriers.  invert_diag_blocks
// forms the inverses of the factor's diagonal blocks, one warp per block.
#pragma once
#include "common.cuh"
#include <float.h>
#include <limits.h>

namespace rvgp {
namespace chol32 {

constexpr int FB = 32;  // panel width (one warp)

// Row stride: a multiple of 4 (16-byte rows for float4 loads) with ld/4 odd,
// so eight consecutive rows read as float4 fall in eight distinct 4-bank groups.
__host__ __device__ inline int lda32(int m) {
  int q = (m + 3) / 4;
  if (q % 2 == 0) ++q;
  return 4 * q;
}

// 1/sqrt(d) in FP32: hardware estimate plus one Newton step.
__device__ __forceinline__ float rsqrt_f(float d) {
  const float r = rsqrtf(d);
  return r * fmaf(-0.5f * d * r, r, 1.5f);
}

// One warp: Cholesky of the nb x nb diagonal block at (j0, j0) of A.  Lane i
// keeps row i in registers; pivots are processed four at a time with compile-
// time register indices, then the row shifts left by four, so the code stays
// small enough for the instruction cache.  Each pivot's column of L goes to a
// per-CTA shared buffer once (one store per lane) and comes back as 16-byte
// broadcast loads: register a[k] holds column j4 + k, so the entries it needs
// are buffer words j4 + k, chunk (j4 + k) / 4 with a compile-time component.
// Entries above the diagonal are updated too but never feed a stored value
// (the buffer holds zeros for rows <= the pivot).  Writes L into the block's
// lower triangle and 1/L_ii into dinvL.  Returns false on a non-positive pivot.
// Only one warp of a CTA may be inside this function at a time.
__device__ inline bool chol_diag_block(float* A, int ld, int j0, int nb, float* dinvL) {
  __shared__ __align__(16) float lcol[2 * FB];  // column j of L (rows 0..31), zeros beyond
  const int lane = threadIdx.x & 31;
  float a[FB];
#pragma unroll
  for (int c = 0; c < FB; ++c) a[c] = (lane < nb && c <= lane) ? A[(j0 + lane) * ld + j0 + c] : 0.f;
  lcol[FB + lane] = 0.f;
  bool ok = true;
  for (int j4 = 0; j4 < nb; j4 += 4) {
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int j = j4 + jj;
      if (j < nb) {
        const float d = __shfl_sync(0xffffffffu, a[jj], j);
        ok = ok && (d > 0.f);
        const float rs = rsqrt_f(fmaxf(d, FLT_MIN));
        const float l = (lane == j) ? d * rs : a[jj] * rs;  // L_ij for lane i >= j
        if (lane >= j && lane < nb) A[(j0 + lane) * ld + j0 + j] = l;
        if (lane == j) dinvL[j0 + j] = rs;
        __syncwarp();
        lcol[lane] = (lane > j && lane < nb) ? l : 0.f;
        __syncwarp();
        const float4* l4 = reinterpret_cast<const float4*>(lcol + j4);
#pragma unroll
        for (int q = (jj + 1) / 4; q < FB / 4; ++q) {
          const float4 v = l4[q];  // L_{j4+4q+c, j}
          if (4 * q + 0 > jj) a[4 * q + 0] = fmaf(-l, v.x, a[4 * q + 0]);
          if (4 * q + 1 > jj) a[4 * q + 1] = fmaf(-l, v.y, a[4 * q + 1]);
          if (4 * q + 2 > jj) a[4 * q + 2] = fmaf(-l, v.z, a[4 * q + 2]);
          if (4 * q + 3 > jj) a[4 * q + 3] = fmaf(-l, v.w, a[4 * q + 3]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < FB - 4; ++k) a[k] = a[k + 4];
#pragma unroll
    for (int k = FB - 4; k < FB; ++k) a[k] = 0.f;
  }
  __syncwarp();
  return __all_sync(0xffffffffu, ok);
}

// Rows [j0+32, m) of block column j0 <- A21 L11⁻ᵀ, i.e. for every row the
// forward substitution L11 x = a.  A warp takes four rows at a time (four
// independent dependency chains), lane c holds column c; lane c' keeps row c'
// of L11 in registers; x_c reaches the other lanes by shuffle.
template <int NT>
__device__ void panel_solve(float* A, int ld, int j0, int m, const float* dinvL) {
  constexpr int kWarps = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r0 = j0 + FB;
  if (r0 >= m) return;
  float lrow[FB];
#pragma unroll
  for (int c = 0; c < FB; ++c) lrow[c] = c < lane ? A[(j0 + lane) * ld + j0 + c] : 0.f;
  const float dl = dinvL[j0 + lane];
  for (int r = r0 + 4 * warp; r < m; r += 4 * kWarps) {
    float x[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) x[q] = (r + q < m) ? A[(r + q) * ld + j0 + lane] : 0.f;
#pragma unroll
    for (int c = 0; c < FB; ++c) {
      const float dc = __shfl_sync(0xffffffffu, dl, c);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float xc = __shfl_sync(0xffffffffu, x[q], c) * dc;
        x[q] = (lane == c) ? xc : fmaf(-xc, lrow[c], x[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (r + q < m) A[(r + q) * ld + j0 + lane] = x[q];
  }
}

// Trailing update of the lower part: A[i][k] -= Σ_c L[i][j0+c] L[k][j0+c] for
// r0 <= k <= i < m, 4 x 4 register tiles, operands read as float4 along c.
// Tiles are numbered row by row over the lower triangle (t -> (ti, tk), tk <=
// ti); this call does tiles t0 + first, t0 + first + stride, ... below t1.
__device__ inline void update_tiles(float* A, int ld, int j0, int m, int t0, int t1, int first, int stride) {
  const int r0 = j0 + FB;
  const int R = m - r0;
  if (R <= 0) return;
  const int TR = (R + 3) / 4;
  const int tiles = min(t1, TR * (TR + 1) / 2);
  for (int t = t0 + first; t < tiles; t += stride) {
    int ti = (int)((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
    while (ti * (ti + 1) / 2 > t) --ti;
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    const int tk = t - ti * (ti + 1) / 2;
    const int i0 = r0 + 4 * ti, k0 = r0 + 4 * tk;
    float acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
    int oa[4], ob[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      oa[u] = min(i0 + u, m - 1) * ld + j0;
      ob[u] = min(k0 + u, m - 1) * ld + j0;
    }
#pragma unroll 1
    for (int c = 0; c < FB; c += 4) {
      float4 b[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = *reinterpret_cast<const float4*>(A + ob[v] + c);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float4 a = *reinterpret_cast<const float4*>(A + oa[u] + c);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          acc[u][v] = fmaf(a.x, b[v].x, acc[u][v]);
          acc[u][v] = fmaf(a.y, b[v].y, acc[u][v]);
          acc[u][v] = fmaf(a.z, b[v].z, acc[u][v]);
          acc[u][v] = fmaf(a.w, b[v].w, acc[u][v]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int i = i0 + u, k = k0 + v;
        if (i < m && k <= i) A[i * ld + k] -= acc[u][v];
      }
  }
}

template <int NT>
__device__ void trailing_update(float* A, int ld, int j0, int m) {
  update_tiles(A, ld, j0, m, 0, INT_MAX, threadIdx.x, NT);
}

// Warp w < nblk: inverse Mb of the factor's diagonal block w by solving
// L X = I with lane i holding row i of X in registers: step c scales row c
// (lane c) and every lane i > c subtracts L_ic times it (shuffled).  Mb is
// written transposed into the block's strict upper triangle (Mb[i][c] at
// A[j0+c][j0+i], i > c); its diagonal is dinvL.
__device__ inline void invert_diag_blocks(float* A, int ld, int m, int nblk, const float* dinvL) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp >= nblk) return;
  const int j0 = warp * FB, nb = min(FB, m - j0);
  float x[FB];
#pragma unroll
  for (int k = 0; k < FB; ++k) x[k] = (k == lane) ? 1.f : 0.f;
  const float dl = lane < nb ? dinvL[j0 + lane] : 0.f;
  for (int c = 0; c < nb; ++c) {
    const float lic = (lane > c && lane < nb) ? A[(j0 + lane) * ld + j0 + c] : 0.f;
    const float dc = __shfl_sync(0xffffffffu, dl, c);
#pragma unroll
    for (int k = 0; k < FB; ++k) {
      const float xck = __shfl_sync(0xffffffffu, x[k], c) * dc;  // row c of X, final
      x[k] = (lane == c) ? xck : fmaf(-lic, xck, x[k]);
    }
  }
  __syncwarp();
  if (lane < nb)
#pragma unroll
    for (int k = 0; k < FB; ++k)
      if (k < lane) A[(j0 + k) * ld + j0 + lane] = x[k];  // Mb[lane][k] -> upper (k, lane)
}


// The blocked factorisation of the lower triangle of A in place (all threads
// of the CTA call it).  dinvL[i] = 1/L_ii.  Returns false (on every thread) if
// a pivot was not positive; *s_flag is a shared int the CTA uses for that.
// Lookahead: after panel jb is solved, warp 0 applies panel jb's update to the
// next diagonal block and factors it while the other warps update the rest of
// the trailing matrix, so the diagonal chain overlaps the largest updates.
template <int NT>
__device__ bool chol32_cta(float* A, int ld, int m, float* dinvL, int* s_flag) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nblk = (m + FB - 1) / FB;
  if (threadIdx.x == 0) *s_flag = 0;
  __syncthreads();
  if (warp == 0 && !chol_diag_block(A, ld, 0, min(FB, m), dinvL) && lane == 0) *s_flag = 1;
  __syncthreads();
  if (*s_flag) return false;
  for (int jb = 0; jb + 1 < nblk; ++jb) {
    const int j0 = jb * FB, r0 = j0 + FB;
    const int nb1 = min(FB, m - r0);
    panel_solve<NT>(A, ld, j0, m, dinvL);
    __syncthreads();
    // tiles of the next diagonal block: tile rows ti < ceil(nb1 / 4)
    const int tr1 = (nb1 + 3) / 4;
    const int tdiag = tr1 * (tr1 + 1) / 2;
    if (warp % 4 == 0) {
      // warps 0, 4, 8, ... (all on warp 0's scheduler: warp w issues on
      // sub-partition w % 4) update the next diagonal block's tiles together;
      // then warp 0 factors it while the others stay idle, so the
      // latency-bound diagonal chain is not starved
      static_assert(NT % 128 == 0, "chol32_cta: NT must be a multiple of 128");
      constexpr int kDiagW = NT / 128;
      update_tiles(A, ld, j0, m, 0, tdiag, (warp / 4) * 32 + lane, kDiagW * 32);
      asm volatile("bar.sync 1, %0;" ::"n"(kDiagW * 32) : "memory");
      if (warp == 0 && !chol_diag_block(A, ld, r0, nb1, dinvL) && lane == 0) *s_flag = 1;
    } else {
      constexpr int kUpd = NT / 32 - NT / 128;
      update_tiles(A, ld, j0, m, tdiag, INT_MAX, (warp - warp / 4 - 1) * 32 + lane, kUpd * 32);
    }
    __syncthreads();
    if (*s_flag) return false;
  }
  return true;
}

}  // namespace chol32
}  // namespace rvgp
