// Tensor-core screen of the exact kNN search (knn.cu, step 2) for ambient
// dimensions 17..64 (padded to DP = 32 or 64): the squared distances of a
// block of 128 queries to tiles of 128 candidates as
//     f² = |x'|² + |y'|² − 2 x'·y'
// with x', y' the FP32 coordinates minus the block's own centre c (the mean
// of its 128 queries), and x'·y' from split-TF32 tcgen05 MMAs (x' = hi + lo,
// A B ≈ Ahi Bhi + Ahi Blo + Alo Bhi, FP32 accumulators in TMEM).  Queries are
// taken in the locality (Morton) order, so a block is a compact patch and
// |x'| is its radius scale.  Candidates are taken in the same order and each
// split visits its tiles outwards from the query block's own position, so the
// first tiles hold most of a block's neighbours: the kc-th distance, the
// insertion threshold, is tight after a few tiles and later insertions (a
// divergent register shift of the whole list) are rare.  Which candidates
// tie at the kc-th value may depend on the visiting order; the certificate
// below does not.
//
// Error bound (per pair, on the FP32 centred values): the dropped lo·lo term
// and the TF32 truncation of lo, ≤ 1.2e-6 |x'||y'|; at most 3·64 FP32
// accumulation roundings (truncation assumed), ≤ 2.3e-5 |x'||y'|; the two
// FP32 norms, ≤ 64u each; the final sums, 4u — in all |f² − d'²| ≤
// 2.9e-5 (|x'|² + |y'|²).  With ε = 1e-4 and |y'|² ≤ 2d'² + 2|x'|²:
//     d'² ≥ (f² − 3ε|x'|²) / (1 + 2ε),
// monotone in f², so the kc-th survivor's f² bounds every non-survivor; the
// finish kernel turns it into a certificate with the FP32 copy's own rounding
// (4.01 u R, as for the SIMT screen) and per-query |x'|² (r2q).
//
// CTA: 416 threads.  Warps 0-7: epilogue, two per SMSP (the epilogue is
// latency-bound with one): warp w owns query rows 32 (w % 4) .. = TMEM lanes
// and the column half w / 4 of every tile, each thread a register top-kc
// list for its row and half (of positions in the order, turned into point
// indices when written; the two halves are written as two splits); warps
// 0-3 also stage the queries.  Warps 8-11: producers, thread r stages
// candidate row r of a tile (centred, split, 128-byte-swizzled K-major) and
// its squared norm; warp 12: one thread issues the MMAs.  Two candidate
// buffers and two TMEM accumulators; mbarriers: staged[b] (4 producer
// warps), full[b] (MMA commit), free[b] (8 epilogue warps).  Every wait is
// bounded; on a timeout the CTA raises the error flag, drains its MMAs and
// frees its TMEM.
#include "common.cuh"
#include "knn_top.cuh"
#include "tcgen05.cuh"
#include <float.h>

namespace rvgp {
namespace {

constexpr int kTQ = 128;             // queries per CTA (MMA M)
constexpr int kTC = 128;             // candidates per tile (MMA N)
constexpr int kEpiWarps = 8;           // two per SMSP: column halves of each tile
constexpr int kTThreads = (kEpiWarps + 4 + 1) * 32;  // + 4 producer warps + the MMA warp
constexpr uint32_t kTTmemCols = 256;  // two 128-column accumulators
constexpr long long kTWait = 1ll << 22;
constexpr int kSlabBytes = kTQ * 128;  // one 32-element K slab of a 128-row operand

// Tile visited i-th of ntiles: t0, t0+1, t0-1, t0+2, ... then the rest of
// the longer side.
__device__ __forceinline__ int tile_of(int i, int t0, int ntiles) {
  const int m = min(t0, ntiles - 1 - t0);
  if (i <= 2 * m) {
    const int j = (i + 1) >> 1;
    return (i & 1) ? t0 + j : t0 - j;
  }
  const int r = i - 2 * m;
  return (ntiles - 1 - t0 > t0) ? t0 + m + r : t0 - m - r;
}

__device__ __forceinline__ uint8_t* align1k(uint8_t* p) {
  const uint32_t a = tc::smem_u32(p);
  return p + (((a + 1023u) & ~1023u) - a);
}

// hi / lo TF32 parts of 4 consecutive K elements (chunk kc of slab s) of row r
__device__ __forceinline__ void put4(uint8_t* hi, uint8_t* lo, int r, int s, int kc, float4 v) {
  float4 h, l;
  h.x = tc::to_tf32(v.x);
  h.y = tc::to_tf32(v.y);
  h.z = tc::to_tf32(v.z);
  h.w = tc::to_tf32(v.w);
  l.x = v.x - h.x;
  l.y = v.y - h.y;
  l.z = v.z - h.z;
  l.w = v.w - h.w;
  const int off = s * kSlabBytes + r * 128 + ((kc ^ (r & 7)) << 4);
  *reinterpret_cast<float4*>(hi + off) = h;
  *reinterpret_cast<float4*>(lo + off) = l;
}

template <int DP, int KC>
__global__ void __launch_bounds__(kTThreads, 1)
    knn_tc_screen(const float* __restrict__ Xf, int n, const int* __restrict__ order, int nsplit,
                  float* __restrict__ part_d, int* __restrict__ part_i, float* __restrict__ r2q,
                  int* __restrict__ err) {
  constexpr int NS = DP / 32;                 // K slabs
  constexpr int OPB = NS * kSlabBytes;        // one split (hi or lo) of a 128-row operand
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bar[7];                 // staged[2], full[2], free[2], drain
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  __shared__ float cen[DP];
  __shared__ float cn[2][kTC];
  __shared__ float s_qn[kTQ];  // each query's |x'|², for both epilogue warps of its row
  __shared__ int s_q[kTQ];     // and its point index (-1 past the end)
  uint8_t* smem = align1k(smem_raw);
  uint8_t* Ahi = smem;
  uint8_t* Alo = Ahi + OPB;
  uint8_t* Bb = Alo + OPB;                    // buffer b: hi at Bb + 2 b OPB, lo after it
                                              // then the epilogue's hit staging
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int qb = blockIdx.x, split = blockIdx.y;
  const int q0 = qb * kTQ, nq = min(kTQ, n - q0);
  const long long chunk = ((long long)n + nsplit - 1) / nsplit;
  const int c0 = (int)min((long long)n, split * chunk), c1 = (int)min((long long)n, c0 + chunk);
  const int ntiles = (c1 - c0 + kTC - 1) / kTC;
  // first tile: the one holding this block's own first position, or the
  // split's end nearest to it
  const int t0 = ntiles > 0 ? max(0, min(ntiles - 1, (q0 - c0) / kTC)) : 0;

  if (warp == 0) {
    tc::tmem_alloc(&tmem_slot, kTTmemCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&bar[b], 4);
      tc::mbar_init(&bar[2 + b], 1);
      tc::mbar_init(&bar[4 + b], kEpiWarps);
    }
    tc::mbar_init(&bar[6], 1);
    tc::fence_mbar_init();
    s_fail = 0;
  }
  // the block's centre: mean of its queries (fixed order)
  for (int j = tid; j < DP; j += kTThreads) {
    float s = 0.f;
    for (int i = 0; i < nq; ++i) s += Xf[(size_t)order[q0 + i] * DP + j];
    cen[j] = s / (float)nq;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  // A operand (query rows, centred) and each query's |x'|², by the epilogue threads
  float qn = 0.f;
  int q = -1;
  if (warp < 4) {
    const int i = tid;
    const bool on = i < nq;
    q = on ? order[q0 + i] : -1;
#pragma unroll
    for (int s = 0; s < NS; ++s)
#pragma unroll
      for (int kc = 0; kc < 8; ++kc) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (on) {
          const float4 x = *reinterpret_cast<const float4*>(Xf + (size_t)q * DP + s * 32 + kc * 4);
          const int j = s * 32 + kc * 4;
          v = make_float4(x.x - cen[j], x.y - cen[j + 1], x.z - cen[j + 2], x.w - cen[j + 3]);
          qn = fmaf(v.x, v.x, qn);
          qn = fmaf(v.y, v.y, qn);
          qn = fmaf(v.z, v.z, qn);
          qn = fmaf(v.w, v.w, qn);
        }
        put4(Ahi, Alo, i, s, kc, v);
      }
    if (on && split == 0) r2q[q] = qn;
    s_qn[i] = qn;
    s_q[i] = q;
  }
  tc::fence_async_smem();
  __syncthreads();

  if (warp < kEpiWarps) {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. (its query rows)
    // and columns [64 h, 64 h + 64) of each tile, h = w / 4; the two halves of
    // a row keep their own lists, written as two splits
    const int row = (warp & 3) * 32 + lane, half = warp >> 2, e = warp * 32 + lane;
    const float qn_r = s_qn[row];
    const int q_r = s_q[row];
    RegTop<KC> L;
    L.init();
    // columns per TMEM load: 16 where the k-list leaves the registers
    constexpr int kCh = KC > 48 ? 8 : 16;
    float* sd = reinterpret_cast<float*>(Bb + 4 * OPB);  // kCh x 256 hit staging
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    for (int t = 0; t < ntiles; ++t) {
      const int b = t & 1;
      bool ok = true;
      // staged[b] too: it orders the producers' norms cn[b] before these reads
      // (its phase cannot move on before this warp releases the buffer)
      for (int which = 0; which < 2 && ok; ++which)
        for (long long w = 0; !tc::mbar_try_wait(&bar[which == 0 ? b : 2 + b], (t >> 1) & 1); ++w)
          if (w > kTWait || *((volatile int*)&s_fail)) {
            ok = false;
            break;
          }
      if (!ok) {
        s_fail = 1;
        break;
      }
      tc::fence_after_sync();
      const int cb = c0 + tile_of(t, t0, ntiles) * kTC;
      const int qp = q0 + row;  // this query's own position
#pragma unroll 1
      for (int c = half * (kTC / 2); c < (half + 1) * (kTC / 2); c += kCh) {
        float v[kCh];
        if constexpr (kCh == 16) tc::tmem_ld16(trow + (uint32_t)(b * kTC + c), v);
        else tc::tmem_ld8(trow + (uint32_t)(b * kTC + c), v);
        // unrolled: f² and a mask of the columns under the threshold at the
        // chunk's start (a superset of those that insert)
        const float wst = L.worst();
        uint32_t mask = 0;
#pragma unroll
        for (int g = 0; g < kCh / 4; ++g) {
          const float4 nv = *reinterpret_cast<const float4*>(&cn[b][c + 4 * g]);
          const float nn[4] = {nv.x, nv.y, nv.z, nv.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            v[4 * g + u] = fmaf(-2.f, v[4 * g + u], qn_r + nn[u]);
            mask |= (v[4 * g + u] < wst ? 1u : 0u) << (4 * g + u);
          }
        }
        // rare after the first tiles: the hits go through shared memory to a
        // loop with one insertion site (one copy of the register shift)
        if (mask) {
#pragma unroll
          for (int j = 0; j < kCh; ++j) sd[j * (kEpiWarps * 32) + e] = v[j];
          while (mask) {
            const int j = __ffs(mask) - 1;
            mask &= mask - 1;
            const float d2 = sd[j * (kEpiWarps * 32) + e];
            const int cand = cb + c + j;
            if (d2 < L.worst() && cand < c1 && cand != qp) L.insert(d2, cand);
          }
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&bar[4 + b]);
    }
    if (q_r >= 0) {
      const size_t base = ((size_t)q_r * (2 * nsplit) + 2 * split + half) * KC;
#pragma unroll
      for (int r = 0; r < KC; ++r) {
        part_d[base + r] = L.d[r];
        part_i[base + r] = L.i[r] >= 0 ? order[L.i[r]] : -1;
      }
    }
  } else if (warp < kEpiWarps + 4) {
    // ---- producers: thread r stages candidate row r of each tile; the next
    // tile's row is loaded into registers before the next buffer wait
    const int r = tid - kEpiWarps * 32;
    float4 nxt[NS * 8];
    auto fetch = [&](int t) {
      const int cand = c0 + tile_of(t, t0, ntiles) * kTC + r;
      const float* y = cand < c1 ? Xf + (size_t)order[cand] * DP : nullptr;
#pragma unroll
      for (int e = 0; e < NS * 8; ++e)
        nxt[e] = y ? *reinterpret_cast<const float4*>(y + e * 4) : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    if (ntiles > 0) fetch(0);
    for (int t = 0; t < ntiles; ++t) {
      const int b = t & 1;
      if (t >= 2) {
        bool ok = true;
        for (long long w = 0; !tc::mbar_try_wait(&bar[4 + b], ((t - 2) >> 1) & 1); ++w)
          if (w > kTWait || *((volatile int*)&s_fail)) {
            ok = false;
            break;
          }
        if (!ok) {
          s_fail = 1;
          break;
        }
      }
      const bool on = c0 + tile_of(t, t0, ntiles) * kTC + r < c1;
      uint8_t* hi = Bb + 2 * b * OPB;
      uint8_t* lo = hi + OPB;
      float nrm = 0.f;
#pragma unroll
      for (int s = 0; s < NS; ++s)
#pragma unroll
        for (int kc = 0; kc < 8; ++kc) {
          const float4 y = nxt[s * 8 + kc];
          const int j = s * 32 + kc * 4;
          const float4 v = on ? make_float4(y.x - cen[j], y.y - cen[j + 1], y.z - cen[j + 2], y.w - cen[j + 3])
                              : make_float4(0.f, 0.f, 0.f, 0.f);
          nrm = fmaf(v.x, v.x, nrm);
          nrm = fmaf(v.y, v.y, nrm);
          nrm = fmaf(v.z, v.z, nrm);
          nrm = fmaf(v.w, v.w, nrm);
          put4(hi, lo, r, s, kc, v);
        }
      cn[b][r] = on ? nrm : FLT_MAX;
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&bar[b]);
      if (t + 1 < ntiles) fetch(t + 1);  // in flight during the next buffer wait
    }
  } else if (lane == 0) {
    // ---- MMA issuer
    const uint32_t idesc = tc::idesc_tf32(kTQ, kTC);
    const uint32_t ah = tc::smem_u32(Ahi), al = tc::smem_u32(Alo);
    for (int t = 0; t < ntiles; ++t) {
      const int b = t & 1;
      bool ok = true;
      for (long long w = 0; !tc::mbar_try_wait(&bar[b], (t >> 1) & 1); ++w)
        if (w > kTWait || *((volatile int*)&s_fail)) {
          ok = false;
          break;
        }
      if (!ok) {
        s_fail = 1;
        break;
      }
      tc::fence_after_sync();
      const uint32_t bh = tc::smem_u32(Bb + 2 * b * OPB), bl = bh + OPB;
      const uint32_t d = tmem + (uint32_t)(b * kTC);
#pragma unroll
      for (int s = 0; s < NS; ++s)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint32_t o = s * kSlabBytes + kk * 32;
          tc::mma_tf32(d, tc::desc_sw128(ah + o), tc::desc_sw128(bh + o), idesc, (s == 0 && kk == 0) ? 0u : 1u);
          tc::mma_tf32(d, tc::desc_sw128(ah + o), tc::desc_sw128(bl + o), idesc, 1u);
          tc::mma_tf32(d, tc::desc_sw128(al + o), tc::desc_sw128(bh + o), idesc, 1u);
        }
      tc::mma_commit(&bar[2 + b]);
    }
  }
  // every MMA issued has completed before TMEM is released: on the normal
  // path the epilogue waited for the last tile; after a timeout the issuer
  // commits once more and waits (bounded)
  __syncthreads();
  if (s_fail && warp == kEpiWarps + 4 && lane == 0) {
    tc::mma_commit(&bar[6]);
    tc::mbar_wait(&bar[6], 0, kTWait);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kTTmemCols);
  if (tid == 0 && s_fail) atomicExch(err, 1);
}

template <int DP>
int launch_dp(int kc, dim3 grid, size_t smem, cudaStream_t st, const float* Xf, int n, const int* order, int nsplit,
              float* pd, int* pi, float* r2q, int* err) {
#define RVGP_KTC(KCv)                                                                                              \
  case KCv: {                                                                                                      \
    if (raise_dyn_smem((const void*)knn_tc_screen<DP, KCv>, smem) != cudaSuccess)                               \
      return check_launch("knn_tc_screen");                                                                        \
    rvgp::note_launch();                                                                                           \
    knn_tc_screen<DP, KCv><<<grid, kTThreads, smem, st>>>(Xf, n, order, nsplit, pd, pi, r2q, err);                 \
    break;                                                                                                         \
  }
  switch (kc) {
    RVGP_KTC(16)
    RVGP_KTC(32)
    RVGP_KTC(48)
    default: RVGP_KTC(72)
  }
#undef RVGP_KTC
  return check_launch("knn_tc_screen");
}

}  // namespace

// The screen's launch (kc in 16/32/48/72; DP 32 or 64): part_d / part_i
// (n x 2 nsplit x kc, the candidates' f² and indices: each split's two column
// halves), r2q (n) = |x'|².
int knn_tc_screen_launch(int DP, int kc, const float* Xf, int n, const int* order, int nsplit, float* part_d,
                         int* part_i, float* r2q, int* err, cudaStream_t st) {
  const int NS = DP / 32;
  // A hi/lo + two B buffers of hi/lo + the epilogue's 16 x 256 hit staging
  const size_t smem = 1024 + (size_t)2 * NS * kSlabBytes * 3 + (size_t)16 * kEpiWarps * 32 * sizeof(float);
  dim3 grid((n + kTQ - 1) / kTQ, nsplit);
  if (DP == 32) return launch_dp<32>(kc, grid, smem, st, Xf, n, order, nsplit, part_d, part_i, r2q, err);
  return launch_dp<64>(kc, grid, smem, st, Xf, n, order, nsplit, part_d, part_i, r2q, err);
}

}  // namespace rvgp
