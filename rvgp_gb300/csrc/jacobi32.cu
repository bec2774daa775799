// FP32 symmetric eigensolver for the eigensolver's Rayleigh-Ritz step
// (internal): parallel cyclic Jacobi with the whole p x p matrix in one SM's
// shared memory.
//
// A multi-SM Jacobi pays a grid barrier and two L2 round trips per round
// (p - 1 rounds per sweep).  Here a round costs one CTA barrier: the p/2
// rotations of a round (circle-method pairing) act on disjoint index pairs,
// so the two-sided update H <- Jᵀ H J splits into independent 2 x 2 blocks
// (pair a, pair b) that one thread reads, rotates and writes in place.  Only
// the upper triangle is stored (a block and its transpose share storage).
// The eigenvector matrix is not carried along: every round's (cos, sin) are
// logged, and jacobi32_replay rotates rows of V = I independently (one CTA
// per four rows), which also applies the final sort by eigenvalue.
//
// Convergence test after each sweep: off(H)² <= tol² ||H||_F² (FP32 sums).
#include "common.cuh"
#include "linalg.cuh"
#include <float.h>
#include <algorithm>
#include <cstdint>

namespace rvgp {
namespace {

constexpr int kThreads = 1024;
constexpr int kReplayRows = 4;
constexpr int kReplayThreads = 128;

__host__ __device__ inline int ldh_of(int p) { return p + 1; }

// pair k of round r of the circle method on p (even) indices, as (min, max)
__device__ __forceinline__ int2 pair_of(int r, int k, int p) {
  int a, b;
  if (k == 0) {
    a = r;
    b = p - 1;
  } else {
    a = (r + k) % (p - 1);
    b = (r - k + p - 1) % (p - 1);
  }
  return a < b ? make_int2(a, b) : make_int2(b, a);
}

// shared memory: H (p x ldh), the round's pairs as float4 (c, s, P, Q), the
// reduction scratch, and the (a, b) block table (2 bytes per block, a <= b <
// p/2), which the final sort's keys overlay once the sweeps are done
size_t jac_smem(int p) {
  const size_t np = p / 2, nblk = np * (np + 1) / 2;
  size_t P2 = 1;
  while (P2 < (size_t)p) P2 <<= 1;
  const size_t table = std::max(sizeof(uint16_t) * nblk, (sizeof(float) + sizeof(int)) * P2);
  return sizeof(float) * (size_t)p * ldh_of(p) + 16 * np + sizeof(float) * 64 + table + 256;
}

// Rutishauser's rotation annihilating H_PQ: cos, sin with t = sign(θ)/(|θ| + sqrt(θ²+1)).
__device__ __forceinline__ void rotation(float hpp, float hqq, float hpq, float& c, float& s) {
  c = 1.f;
  s = 0.f;
  if (hpq != 0.f && fabsf(hpq) > 1e-30f * sqrtf(fabsf(hpp) * fabsf(hqq) + 1e-38f)) {
    const float theta = (hqq - hpp) / (2.f * hpq);
    const float t = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(fmaf(theta, theta, 1.f)));
    c = 1.f / sqrtf(fmaf(t, t, 1.f));
    s = t * c;
  }
}

__global__ void __launch_bounds__(kThreads, 1)
    jacobi32_kernel(const float* __restrict__ Hin, int p, int max_sweeps, float tol2, float* __restrict__ log,
                    int* __restrict__ sweeps_out, float* __restrict__ w, int* __restrict__ perm) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ldh = ldh_of(p);
  const int np = p / 2, rounds = p - 1;
  const int nblk = np * (np + 1) / 2;
  float* H = reinterpret_cast<float*>(smraw);
  float4* pd = reinterpret_cast<float4*>(H + (size_t)p * ldh + ((4 - (p * ldh) % 4) % 4));  // (c, s, P, Q)
  float* red = reinterpret_cast<float*>(pd + np);                 // 64
  uint16_t* table = reinterpret_cast<uint16_t*>(red + 64);        // nblk blocks (a | b << 8)
  float* key = reinterpret_cast<float*>(table);                   // final sort, overlays the table
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // symmetric storage: element (i, j) lives at (min, max) in the upper triangle
  auto idx = [&](int i, int j) { return min(i, j) * ldh + max(i, j); };
  for (int e = tid; e < p * p; e += kThreads) {
    const int i = e / p, j = e % p;
    if (i <= j) H[i * ldh + j] = 0.5f * (Hin[(size_t)i * p + j] + Hin[(size_t)j * p + i]);
  }
  // block table: row a holds blocks (a, a) .. (a, np - 1) from offset a np - a (a - 1) / 2
  for (int a = tid; a < np; a += kThreads) {
    const int off = a * np - a * (a - 1) / 2;
    for (int b = a; b < np; ++b) table[off + b - a] = (uint16_t)(a | (b << 8));
  }
  __syncthreads();
  int used = 0;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    // off-diagonal and total squared norms
    float off = 0.f, tot = 0.f;
    for (int e = tid; e < p * p; e += kThreads) {
      const int i = e / p, j = e % p;
      if (i > j) continue;
      const float v = H[i * ldh + j];
      const float w2 = (i == j) ? v * v : 2.f * v * v;  // the upper entry stands for both
      tot += w2;
      if (i != j) off += w2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if (lane == 0) {
      red[warp] = off;
      red[32 + warp] = tot;
    }
    __syncthreads();
    if (warp == 0) {
      float a = red[lane], b = red[32 + lane];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
      }
      if (lane == 0) {
        red[0] = a;
        red[32] = b;
      }
    }
    __syncthreads();
    const bool done = !(red[0] > tol2 * red[32]);
    __syncthreads();
    if (done) break;
    for (int r = 0; r < rounds; ++r) {
      float* lg = log + ((size_t)sweep * rounds + r) * 2 * np;
      for (int k = tid; k < np; k += kThreads) {
        const int2 q = pair_of(r, k, p);
        float c, s;
        rotation(H[q.x * ldh + q.x], H[q.y * ldh + q.y], H[q.x * ldh + q.y], c, s);  // q.x < q.y
        pd[k] = make_float4(c, s, __int_as_float(q.x), __int_as_float(q.y));
        lg[2 * k] = c;
        lg[2 * k + 1] = s;
      }
      __syncthreads();
      // the round's blocks (a, b), a <= b, dealt evenly over the threads
      for (int t = tid; t < nblk; t += kThreads) {
        const uint16_t e = table[t];
        const int a = e & 255, b = e >> 8;
        const float4 PA = pd[a], PB = pd[b];
        const float ca = PA.x, sa = PA.y, cb = PB.x, sb = PB.y;
        if (sa == 0.f && sb == 0.f) continue;  // both rotations are the identity
        const int ax = __float_as_int(PA.z), ay = __float_as_int(PA.w);
        const int bx = __float_as_int(PB.z), by = __float_as_int(PB.w);
        if (a == b) {
          const float x00 = H[ax * ldh + ax], x01 = H[ax * ldh + ay], x11 = H[ay * ldh + ay];
          const float t00 = ca * x00 - sa * x01, t01 = sa * x00 + ca * x01;
          const float t10 = ca * x01 - sa * x11, t11 = sa * x01 + ca * x11;
          H[ax * ldh + ax] = ca * t00 - sa * t10;
          H[ay * ldh + ay] = sa * t01 + ca * t11;
          H[ax * ldh + ay] = 0.f;  // ax < ay
        } else {
          const int i00 = idx(ax, bx), i01 = idx(ax, by), i10 = idx(ay, bx), i11 = idx(ay, by);
          const float x00 = H[i00], x01 = H[i01], x10 = H[i10], x11 = H[i11];
          // T = X J_b, J = [[c, s], [-s, c]]; H' = J_aᵀ T
          const float t00 = cb * x00 - sb * x01, t01 = sb * x00 + cb * x01;
          const float t10 = cb * x10 - sb * x11, t11 = sb * x10 + cb * x11;
          H[i00] = ca * t00 - sa * t10;
          H[i01] = ca * t01 - sa * t11;
          H[i10] = sa * t00 + ca * t10;
          H[i11] = sa * t01 + ca * t11;
        }
      }
      __syncthreads();
    }
    ++used;
  }
  // sort the diagonal ascending, ties by index (bitonic over a power of two)
  int P2 = 1;
  while (P2 < p) P2 <<= 1;
  int* key_idx = reinterpret_cast<int*>(key + P2);
  for (int t = tid; t < P2; t += kThreads) {
    key[t] = t < p ? H[t * ldh + t] : FLT_MAX;
    key_idx[t] = t < p ? t : INT_MAX;
  }
  __syncthreads();
  for (int size = 2; size <= P2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = tid; t < P2; t += kThreads) {
        const int o = t ^ stride;
        if (o > t) {
          const bool up = (t & size) == 0;
          const int it = key_idx[t], io = key_idx[o];
          const bool o_less = io != INT_MAX && (it == INT_MAX || key[o] < key[t] || (key[o] == key[t] && io < it));
          const bool t_less = it != INT_MAX && (io == INT_MAX || key[t] < key[o] || (key[t] == key[o] && it < io));
          if (up ? o_less : t_less) {
            const float kk = key[t];
            key[t] = key[o];
            key[o] = kk;
            key_idx[t] = io;
            key_idx[o] = it;
          }
        }
      }
      __syncthreads();
    }
  for (int t = tid; t < p; t += kThreads) {
    w[t] = key[t];
    perm[t] = key_idx[t];
  }
  if (tid == 0) *sweeps_out = used;
}

// V (p x p) = product of the logged rotations applied to I, columns permuted
// by perm: CTA b owns rows 4b..4b+3 of V in shared memory; each round's p/2
// rotations act on disjoint column pairs (one thread each).  The log is
// staged kChunk rounds at a time so its L2 latency is paid once per chunk.
constexpr int kChunk = 16;

__global__ void __launch_bounds__(kReplayThreads)
    jacobi32_replay(const float* __restrict__ log, int p, const int* __restrict__ sweeps, const int* __restrict__ perm,
                    float* __restrict__ V) {
  extern __shared__ float sm[];
  const int np = p / 2, rounds = p - 1;
  float* v = sm;                          // kReplayRows x p
  float* lg = sm + kReplayRows * p;       // kChunk x 2np
  const int row0 = blockIdx.x * kReplayRows;
  for (int e = threadIdx.x; e < kReplayRows * p; e += kReplayThreads) {
    const int r = e / p, j = e % p;
    v[e] = (row0 + r == j) ? 1.f : 0.f;
  }
  const long long total = (long long)(*sweeps) * rounds;
  for (long long t0 = 0; t0 < total; t0 += kChunk) {
    const int nr = (int)min((long long)kChunk, total - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < nr * 2 * np; e += kReplayThreads) lg[e] = log[(size_t)t0 * 2 * np + e];
    __syncthreads();
    for (int q = 0; q < nr; ++q) {
      const int r = (int)((t0 + q) % rounds);
      for (int k = threadIdx.x; k < np; k += kReplayThreads) {
        const int2 pr = pair_of(r, k, p);
        const float c = lg[q * 2 * np + 2 * k], s = lg[q * 2 * np + 2 * k + 1];
#pragma unroll
        for (int rr = 0; rr < kReplayRows; ++rr) {
          const float a = v[rr * p + pr.x], b = v[rr * p + pr.y];
          v[rr * p + pr.x] = c * a - s * b;  // e'_P = c e_P - s e_Q
          v[rr * p + pr.y] = s * a + c * b;  // e'_Q = s e_P + c e_Q
        }
      }
      __syncthreads();
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kReplayRows * p; e += kReplayThreads) {
    const int r = e / p, j = e % p;
    if (row0 + r < p) V[(size_t)(row0 + r) * p + j] = v[r * p + perm[j]];
  }
}

}  // namespace

int jacobi32_max_p() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  int p = 2;
  while (jac_smem(p + 2) <= (size_t)optin) p += 2;
  return p;
}

size_t jacobi32_workspace(int p, int max_sweeps) {
  return sizeof(float) * (size_t)max_sweeps * (p - 1) * p + sizeof(int) * (size_t)(p + 4) + 512;
}

int jacobi32_eigh(const float* H, int p, float* w, float* V, int max_sweeps, double tol, int* sweeps_used, void* ws,
                  size_t ws_bytes, cudaStream_t st) {
  if (p < 2 || p % 2 != 0 || p > jacobi32_max_p()) {
    set_error("jacobi32_eigh: p=%d must be even and at most %d", p, jacobi32_max_p());
    return RVGP_ENOTSUP;
  }
  if (ws_bytes < jacobi32_workspace(p, max_sweeps)) {
    set_error("jacobi32_eigh: workspace too small");
    return RVGP_EWORKSPACE;
  }
  Workspace W(ws, ws_bytes);
  float* lg = W.take<float>((size_t)max_sweeps * (p - 1) * p);
  int* perm = W.take<int>(p);
  int* sw = W.take<int>(4);
  const size_t smem = jac_smem(p);
  if (raise_dyn_smem((const void*)jacobi32_kernel, (size_t)(smem)) != cudaSuccess) {
    set_error("jacobi32_eigh: cannot reserve %zu bytes of shared memory", smem);
    return RVGP_ELAUNCH;
  }
  rvgp::note_launch();
  jacobi32_kernel<<<1, kThreads, smem, st>>>(H, p, max_sweeps, (float)(tol * tol), lg, sw, w, perm);
  rvgp::note_launch();
  jacobi32_replay<<<ceil_div(p, kReplayRows), kReplayThreads, sizeof(float) * (kReplayRows * p + kChunk * p), st>>>(
      lg, p, sw, perm, V);
  if (sweeps_used) {
    int h = 0;
    if (read_back(&h, sw, sizeof(int), st) != cudaSuccess) return check_launch("jacobi32_eigh");
    *sweeps_used = h;
  }
  return check_launch("jacobi32_eigh");
}

}  // namespace rvgp
