// Tall FP32 products of the eigensolver on the tensor cores (tcgen05, TMEM
// accumulators), with FP32-level accuracy from split TF32 operands:
// x = hi + lo, hi = tf32(x), lo = x - hi, and A B ~ Ahi Bhi + Ahi Blo + Alo Bhi
// (the dropped Alo Blo and the TF32 truncation of lo are ~2^-21 relative).
//
//   tc_gram_f32_out64 : C (p x q, FP64) = Aᵀ B for tall A (N x p), B (N x q).
//                       CTA = (128-row tile of C, split of the N rows); FP32
//                       partials in TMEM, summed over the splits in FP64 (the
//                       Gram matrices of the Cholesky QR and Rayleigh-Ritz
//                       steps).  For Aᵀ A with p <= 256 the row slabs are
//                       bulk-copied by the TMA engine and converted from
//                       shared memory; wider products run as column blocks
//                       of C (at most 256 columns, one TMEM accumulator).
//   tc_gemm_f32       : C (N x q) = A (N x K) Bm (K x q).  CTA = 128-row tile
//                       of A and C (block rotations V Q, W Q); K streams in
//                       slabs, q > 256 runs as column blocks of C.
//
// Both stream 32-wide K slabs through a two-stage shared-memory pipeline
// (even slabs accumulate in one TMEM accumulator, odd slabs in another):
// every thread stages its share of the next slab (hi / lo split, swizzled
// K-major layout, tcgen05.cuh) while the tensor core runs the MMAs of the
// current one; one thread issues the MMAs (12 per slab: 4 K steps x 3
// products) and commits them to the slab buffer's mbarrier, which the stagers
// wait on before they overwrite that buffer.  Waits are bounded: on a timeout
// the kernel raises a flag in the workspace, finishes and frees its TMEM.
#include "common.cuh"
#include "linalg.cuh"
#include "tcgen05.cuh"
#include <cstdlib>

namespace rvgp {
namespace {

constexpr int kThreads = 512;
constexpr int kSlab = 32;                     // K elements per slab (128 bytes)
constexpr int kTileM = 128;                   // MMA M
constexpr uint32_t kAccCols = 256;            // FP32 accumulator columns (N <= 256)
constexpr uint32_t kTmemCols = 2 * kAccCols;   // two accumulators, alternating slabs (half the FP32 sum chain)
constexpr long long kWaitLimit = 1ll << 20;   // mbarrier polls before giving up

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  const uint32_t a = tc::smem_u32(p);
  return p + (((a + 1023u) & ~1023u) - a);
}

// hi / lo TF32 parts of 4 consecutive K elements of operand row r, chunk kc
__device__ __forceinline__ void put_chunk(uint8_t* hi, uint8_t* lo, int r, int kc, float4 v) {
  float4 h, l;
  h.x = tc::to_tf32(v.x);
  h.y = tc::to_tf32(v.y);
  h.z = tc::to_tf32(v.z);
  h.w = tc::to_tf32(v.w);
  l.x = v.x - h.x;
  l.y = v.y - h.y;
  l.z = v.z - h.z;
  l.w = v.w - h.w;
  const int off = r * 128 + ((kc ^ (r & 7)) << 4);
  *reinterpret_cast<float4*>(hi + off) = h;
  *reinterpret_cast<float4*>(lo + off) = l;
}

// 12 MMAs of one slab: D (+)= Ahi Bhi + Ahi Blo + Alo Bhi over 4 K steps
__device__ __forceinline__ void slab_mmas(uint32_t tmem, uint32_t ahi, uint32_t alo, uint32_t bhi, uint32_t blo,
                                          uint32_t idesc, bool first) {
  tc::fence_after_sync();
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const uint32_t o = kk * 32;
    tc::mma_tf32(tmem, tc::desc_sw128(ahi + o), tc::desc_sw128(bhi + o), idesc, (first && kk == 0) ? 0u : 1u);
    tc::mma_tf32(tmem, tc::desc_sw128(ahi + o), tc::desc_sw128(blo + o), idesc, 1u);
    tc::mma_tf32(tmem, tc::desc_sw128(alo + o), tc::desc_sw128(bhi + o), idesc, 1u);
  }
}

// TMEM -> global: warp w reads lanes 32*(w%4).. and every (kThreads/128)-th
// 8-column chunk, starting at chunk w/4, of the nacc (0..2) accumulators and
// adds them; row i of the tile goes to out + i*ldo (columns < ncols, rows < nrows)
__device__ __forceinline__ void epilogue(uint32_t tmem, int nacc, int Npad, float* out, long long ldo, int nrows,
                                         int ncols) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int quarter = warp & 3, group = warp >> 2, ngroups = kThreads / 128;
  const int i = quarter * 32 + lane;
  for (int c = group * 8; c < Npad; c += ngroups * 8) {
    float v[8], w[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) v[t] = 0.f;
    for (int a = 0; a < nacc; ++a) {
      tc::tmem_ld8(tmem + ((uint32_t)(quarter * 32) << 16) + a * kAccCols + (uint32_t)c, w);
#pragma unroll
      for (int t = 0; t < 8; ++t) v[t] += w[t];
    }
    if (i < nrows) {
      float* o = out + (long long)i * ldo + c;
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (c + t < ncols) o[t] = v[t];
    }
  }
}

// bar[0..1]: MMA completion per stage; bar[2]: drain barrier of the failure path
__device__ __forceinline__ void setup(uint64_t* bar, uint32_t* tmem_slot, int* s_fail) {
  if ((threadIdx.x >> 5) == 0) {
    tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_init(&bar[2], 1);
    tc::fence_mbar_init();
    *s_fail = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// Every thread learns whether a pipeline wait timed out; the epilogue runs
// only if none did.
__device__ __forceinline__ bool pipeline_ok(const int* s_fail) {
  __syncthreads();
  return *s_fail == 0;
}

// After a timed-out wait, thread 0 (the MMA issuer) commits once more and
// waits (bounded) until every MMA it issued has completed, so TMEM is freed
// only when nothing writes it any more; `full` / `nfull` / `last` name the
// bulk-copy barriers and the parity of the last copy issued into each, which
// are waited on likewise before the CTA's shared memory is released.
__device__ __forceinline__ void teardown(uint32_t tmem, uint64_t* bar, const int* s_fail, int* err,
                                         uint64_t* full = nullptr, int nfull = 0, const int* last = nullptr) {
  if (*s_fail && threadIdx.x == 0) {
    tc::mma_commit(&bar[2]);
    tc::mbar_wait(&bar[2], 0, kWaitLimit);
    for (int k = 0; k < nfull; ++k)
      if (last[k] >= 0) tc::mbar_wait(&full[k], (uint32_t)last[k], kWaitLimit);
  }
  tc::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tmem, kTmemCols);
  if (threadIdx.x == 0 && *s_fail) atomicExch(err, 1);
}

// ---------------------------------------------------------------- C = Aᵀ B
// grid (ceil(p / 128), splits), 512 threads.  B image: Brows (<= 256) x 128 B
// per part; when SAME (B = A) the A operand is rows [i0, i0 + 128) of the B
// image.  Thread t stages B-image row j = t % 256, chunks 4 (t / 256) .. +3
// (4 loads each, coalesced over j) and, not SAME, A-image row t % 128, chunks
// 2 (t / 128) .. +1.  Two register sets hold the next two slabs, so a slab's
// global loads are issued two slabs before their conversion.
struct GramRegs {
  float4 b[4];
  float4 a[2];
};

template <bool SAME>
__global__ void __launch_bounds__(kThreads, 1)
    tc_gram_kernel(const float* __restrict__ A, int lda, const float* __restrict__ B, int ldb, long long N, int p,
                   int q, int Npad, int Brows, long long rows_per, float* __restrict__ part, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bar[3];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  uint8_t* smem = align1024(smem_raw);
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * kTileM;
  const long long r_begin = (long long)blockIdx.y * rows_per;
  const long long r_end = min(N, r_begin + rows_per);
  const int nslabs = r_end > r_begin ? (int)((r_end - r_begin + kSlab - 1) / kSlab) : 0;
  const int bbytes = Brows * 128;
  const int abytes = SAME ? 0 : kTileM * 128;
  const int stage_bytes = 2 * bbytes + 2 * abytes;
  setup(bar, &tmem_slot, &s_fail);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::idesc_tf32(kTileM, Npad);
  const int jb = tid & 255, kb0 = (tid >> 8) * 4;       // B-image row and first chunk
  const int ia = tid & 127, ka0 = (tid >> 7) * 2;       // A-image row and first chunk
  const bool bon = jb < q, bput = jb < Brows, aon = !SAME && i0 + ia < p;
  auto load = [&](GramRegs& R, int s) {
    const long long r0 = r_begin + (long long)s * kSlab;
    const int nr = (int)min((long long)kSlab, r_end - r0);  // rows of this slab
    const float* bp = B + r0 * ldb + jb;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float* vv = reinterpret_cast<float*>(&R.b[c]);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int rr = (kb0 + c) * 4 + t;
        vv[t] = (bon && rr < nr) ? __ldg(bp + (long long)rr * ldb) : 0.f;
      }
    }
    if (!SAME) {
      const float* ap = A + r0 * lda + i0 + ia;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        float* vv = reinterpret_cast<float*>(&R.a[c]);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int rr = (ka0 + c) * 4 + t;
          vv[t] = (aon && rr < nr) ? __ldg(ap + (long long)rr * lda) : 0.f;
        }
      }
    }
  };
  auto step = [&](GramRegs& R, int s) {
    const int buf = s & 1;
    uint8_t* st = smem + buf * stage_bytes;
    if (s >= 2 && !tc::mbar_wait(&bar[buf], ((s - 2) >> 1) & 1, kWaitLimit)) s_fail = 1;
    if (bput) {
#pragma unroll
      for (int c = 0; c < 4; ++c) put_chunk(st, st + bbytes, jb, kb0 + c, R.b[c]);
    }
    if (!SAME) {
      uint8_t* ah = st + 2 * bbytes;
#pragma unroll
      for (int c = 0; c < 2; ++c) put_chunk(ah, ah + abytes, ia, ka0 + c, R.a[c]);
    }
    if (s + 2 < nslabs) load(R, s + 2);
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      const uint32_t bh = tc::smem_u32(st), bl = bh + bbytes;
      const uint32_t ahi = SAME ? bh + i0 * 128 : bh + 2 * bbytes;
      const uint32_t alo = SAME ? bl + i0 * 128 : ahi + abytes;
      slab_mmas(tmem + (s & 1) * kAccCols, ahi, alo, bh, bl, idesc, s < 2);
      tc::mma_commit(&bar[buf]);
    }
  };
  GramRegs R0, R1;
  if (nslabs > 0) load(R0, 0);
  if (nslabs > 1) load(R1, 1);
  for (int s = 0; s < nslabs; s += 2) {
    step(R0, s);
    if (s + 1 < nslabs) step(R1, s + 1);
  }
  if (nslabs > 0 && !tc::mbar_wait(&bar[(nslabs - 1) & 1], ((nslabs - 1) >> 1) & 1, kWaitLimit)) s_fail = 1;
  tc::fence_after_sync();
  if (pipeline_ok(&s_fail)) epilogue(tmem, min(nslabs, 2), Npad, part + ((size_t)blockIdx.y * p + i0) * q, q, p - i0, q);
  teardown(tmem, bar, &s_fail, err);
}

// ---------------------------------------------------------------- C = A Bm
// B image (built once per call): per slab, [hi | lo] each Npad x 128 B, the
// operand rows being the columns of Bm (element (j, k) = Bm[k][j]).
__global__ void build_bimg(const float* __restrict__ Bm, int ldb, int K, int q, int Npad, int kslabs,
                           uint8_t* __restrict__ img) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)kslabs * Npad * 8) return;
  const int s = (int)(idx / (Npad * 8));
  const int rem = (int)(idx % (Npad * 8));
  const int j = rem / 8, kc = rem % 8;
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (j < q) {
    float* vv = reinterpret_cast<float*>(&v);
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int k = s * kSlab + kc * 4 + t;
      if (k < K) vv[t] = Bm[(size_t)k * ldb + j];
    }
  }
  uint8_t* base = img + (size_t)s * 2 * Npad * 128;
  put_chunk(base, base + (size_t)Npad * 128, j, kc, v);
}

// grid ceil(N / 128), 512 threads.  The pre-split B image of slab s (one
// contiguous block) is fetched by the TMA engine (bulk copy, completion on
// full[s % 2]) as soon as the MMAs of slab s - 1 have released its stage;
// thread t stages A rows (t / 8) + 64 c (c < 2), chunk t % 8, from registers
// loaded two slabs ahead.
struct GemmRegs {
  float4 a[2];
};

__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const float* __restrict__ A, int lda, long long N, int K, const uint8_t* __restrict__ img, int Npad,
                   int q, float* __restrict__ C, int ldc, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bar[3], full[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  uint8_t* smem = align1024(smem_raw);
  const int tid = threadIdx.x;
  const long long row0 = (long long)blockIdx.x * kTileM;
  const int kslabs = (K + kSlab - 1) / kSlab;
  const int abytes = kTileM * 128, bbytes = Npad * 128;
  const uint32_t bimg = 2u * bbytes;
  const int stage_bytes = 2 * abytes + 2 * bbytes;
  if (tid == 0) {
    tc::mbar_init(&full[0], 1);
    tc::mbar_init(&full[1], 1);
  }
  setup(bar, &tmem_slot, &s_fail);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::idesc_tf32(kTileM, Npad);
  const bool vec_ok = (lda % 4) == 0;
  const int kc = tid & 7, ra0 = tid >> 3;
  auto issue_b = [&](int s) {
    uint8_t* st = smem + (s & 1) * stage_bytes;
    tc::mbar_expect_tx(&full[s & 1], bimg);
    tc::bulk_g2s(st + 2 * abytes, img + (size_t)s * bimg, bimg, &full[s & 1]);
  };
  auto load = [&](GemmRegs& R, int s) {
    const int k = s * kSlab + kc * 4;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const long long row = row0 + ra0 + 64 * c;
      R.a[c] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (row < N) {
        const float* a = A + row * lda + k;
        if (vec_ok && k + 3 < K) {
          R.a[c] = __ldg(reinterpret_cast<const float4*>(a));
        } else {
          float* vv = reinterpret_cast<float*>(&R.a[c]);
#pragma unroll
          for (int t = 0; t < 4; ++t)
            if (k + t < K) vv[t] = __ldg(a + t);
        }
      }
    }
  };
  auto step = [&](GemmRegs& R, int s) {
    const int buf = s & 1;
    uint8_t* st = smem + buf * stage_bytes;
    if (s >= 2 && !tc::mbar_wait(&bar[buf], ((s - 2) >> 1) & 1, kWaitLimit)) s_fail = 1;
#pragma unroll
    for (int c = 0; c < 2; ++c) put_chunk(st, st + abytes, ra0 + 64 * c, kc, R.a[c]);
    if (s + 2 < kslabs) load(R, s + 2);
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      if (!tc::mbar_wait(&full[buf], (s >> 1) & 1, kWaitLimit)) s_fail = 1;
      const uint32_t ah = tc::smem_u32(st), al = ah + abytes;
      const uint32_t bh = ah + 2 * abytes, bl = bh + bbytes;
      slab_mmas(tmem + (s & 1) * kAccCols, ah, al, bh, bl, idesc, s < 2);
      tc::mma_commit(&bar[buf]);
      if (s >= 1 && s + 1 < kslabs) {  // stage (s + 1) % 2 is free once the MMAs of slab s - 1 are done
        if (!tc::mbar_wait(&bar[(s + 1) & 1], ((s - 1) >> 1) & 1, kWaitLimit)) s_fail = 1;
        issue_b(s + 1);
      }
    }
  };
  if (tid == 0) {
    if (kslabs > 0) issue_b(0);
    if (kslabs > 1) issue_b(1);
  }
  GemmRegs R0, R1;
  if (kslabs > 0) load(R0, 0);
  if (kslabs > 1) load(R1, 1);
  for (int s = 0; s < kslabs; s += 2) {
    step(R0, s);
    if (s + 1 < kslabs) step(R1, s + 1);
  }
  if (kslabs > 0 && !tc::mbar_wait(&bar[(kslabs - 1) & 1], ((kslabs - 1) >> 1) & 1, kWaitLimit)) s_fail = 1;
  tc::fence_after_sync();
  const int nrows = (int)min((long long)kTileM, N - row0);
  if (pipeline_ok(&s_fail)) epilogue(tmem, min(kslabs, 2), Npad, C + row0 * ldc, ldc, nrows, q);
  // the last B-image copy into each stage: slab s uses full[s % 2], phase s / 2
  int last[2];
  for (int k = 0; k < 2; ++k) {
    const int sl = kslabs - 1 - ((kslabs - 1 - k) % 2 + 2) % 2;
    last[k] = sl >= 0 ? (sl >> 1) & 1 : -1;
  }
  teardown(tmem, bar, &s_fail, err, full, 2, last);
}

// ---------------------------------------------------------------- C = Aᵀ A, bulk-copied row slabs
// A's rows of a slab are one contiguous block (lda % 4 == 0): the TMA engine
// copies it raw into a three-slab ring (completion on full[s % 3]), three
// slabs ahead; the threads convert it from shared memory into the swizzled
// hi / lo image (thread t: image row t % 256, chunks 4 (t / 256) .. +3).
__global__ void __launch_bounds__(kThreads, 1)
    tc_gram_bulk_kernel(const float* __restrict__ A, int lda, long long N, int p, int Npad, int Brows,
                        long long rows_per, int raw_pad, float* __restrict__ part, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bar[3], full[3];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  uint8_t* smem = align1024(smem_raw);
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * kTileM;
  const long long r_begin = (long long)blockIdx.y * rows_per;
  const long long r_end = min(N, r_begin + rows_per);
  const int nslabs = r_end > r_begin ? (int)((r_end - r_begin + kSlab - 1) / kSlab) : 0;
  const int bbytes = Brows * 128;
  uint8_t* raw = smem;                       // 3 x raw_pad
  uint8_t* imgs = smem + 3 * (size_t)raw_pad;  // 2 x (hi | lo)
  if (tid == 0)
    for (int k = 0; k < 3; ++k) tc::mbar_init(&full[k], 1);
  setup(bar, &tmem_slot, &s_fail);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::idesc_tf32(kTileM, Npad);
  const int jb = tid & 255, kb0 = (tid >> 8) * 4;
  auto rows_of = [&](int s) { return (int)min((long long)kSlab, r_end - (r_begin + (long long)s * kSlab)); };
  auto issue_raw = [&](int s) {
    const uint32_t bytes = (uint32_t)rows_of(s) * lda * 4u;
    tc::mbar_expect_tx(&full[s % 3], bytes);
    tc::bulk_g2s(raw + (size_t)(s % 3) * raw_pad, A + (r_begin + (long long)s * kSlab) * lda, bytes, &full[s % 3]);
  };
  if (tid == 0)
    for (int k = 0; k < 3 && k < nslabs; ++k) issue_raw(k);
  for (int s = 0; s < nslabs; ++s) {
    const int buf = s & 1;
    uint8_t* st = imgs + (size_t)buf * 2 * bbytes;
    if (!tc::mbar_wait(&full[s % 3], (s / 3) & 1, kWaitLimit)) s_fail = 1;
    if (s >= 2 && !tc::mbar_wait(&bar[buf], ((s - 2) >> 1) & 1, kWaitLimit)) s_fail = 1;
    const float* rs = reinterpret_cast<const float*>(raw + (size_t)(s % 3) * raw_pad);
    const int nr = rows_of(s);
    if (jb < Brows) {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float4 v;
        float* vv = reinterpret_cast<float*>(&v);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int rr = (kb0 + c) * 4 + t;
          vv[t] = (jb < p && rr < nr) ? rs[rr * lda + jb] : 0.f;
        }
        put_chunk(st, st + bbytes, jb, kb0 + c, v);
      }
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      const uint32_t bh = tc::smem_u32(st), bl = bh + bbytes;
      slab_mmas(tmem + (s & 1) * kAccCols, bh + i0 * 128, bl + i0 * 128, bh, bl, idesc, s < 2);
      tc::mma_commit(&bar[buf]);
      if (s + 3 < nslabs) issue_raw(s + 3);  // every thread has read raw slot s % 3
    }
  }
  if (nslabs > 0 && !tc::mbar_wait(&bar[(nslabs - 1) & 1], ((nslabs - 1) >> 1) & 1, kWaitLimit)) s_fail = 1;
  tc::fence_after_sync();
  if (pipeline_ok(&s_fail)) epilogue(tmem, min(nslabs, 2), Npad, part + ((size_t)blockIdx.y * p + i0) * p, p, p - i0, p);
  // the last raw copy into each ring slot: slab s uses full[s % 3], phase s / 3
  int last[3];
  for (int k = 0; k < 3; ++k) {
    const int sl = nslabs - 1 - ((nslabs - 1 - k) % 3 + 3) % 3;
    last[k] = sl >= 0 ? (sl / 3) & 1 : -1;
  }
  teardown(tmem, bar, &s_fail, err, full, 3, last);
}

int pad16(int q) { return (q + 15) / 16 * 16; }

// At least 120 KB, so no two CTAs share an SM (each holds all 512 TMEM columns).
constexpr size_t kMinSmem = 120 * 1024;
size_t gram_smem(bool same, int p, int q) {
  const int Npad = pad16(q);
  const int Brows = same ? std::max(Npad, ceil_div(p, kTileM) * kTileM) : Npad;
  const size_t stage = 2 * (size_t)Brows * 128 + (same ? 0 : 2 * (size_t)kTileM * 128);
  return std::max(kMinSmem, 2 * stage + 1024);
}
int raw_pad_bytes(int lda) { return (kSlab * lda * 4 + 1023) / 1024 * 1024; }
size_t gram_bulk_smem(int p, int lda) {
  const int Brows = std::max(pad16(p), ceil_div(p, kTileM) * kTileM);
  return std::max(kMinSmem, 3 * (size_t)raw_pad_bytes(lda) + 2 * 2 * (size_t)Brows * 128 + 1024);
}
size_t gemm_smem(int q) {
  return std::max(kMinSmem, 2 * (2 * (size_t)kTileM * 128 + 2 * (size_t)pad16(q) * 128) + 1024);
}

struct GramPlan {
  int mtiles, splits;
  long long rows_per;
};
GramPlan gram_plan(long long N, int p) {
  GramPlan g;
  g.mtiles = ceil_div(p, kTileM);
  const int want = std::max(1, num_sms() / g.mtiles);
  long long rows = (N + want - 1) / want;
  rows = std::max<long long>(kSlab, (rows + kSlab - 1) / kSlab * kSlab);
  g.rows_per = rows;
  g.splits = (int)((N + rows - 1) / rows);
  return g;
}

int set_smem(const void* fn, size_t bytes, const char* what) {
  if (raise_dyn_smem((const void*)fn, (size_t)(bytes)) != cudaSuccess) {
    set_error("%s: cannot reserve %zu bytes of shared memory", what, bytes);
    return RVGP_ELAUNCH;
  }
  return RVGP_OK;
}

}  // namespace

bool tc_enabled() {
  const char* e = getenv("RVGP_TENSOR_CORES");
  return !(e && e[0] == '0');
}

// Products wider than one accumulator (256 FP32 columns) run as column blocks
// of at most kColBlock output columns; K (the summed dimension) and the rows
// of the Gram's first operand are not limited.
constexpr int kColBlock = 256;
constexpr int kMaxWidth = 2048;

bool tc_supported(int p, int q) {
  int dev = 0, optin = 0;
  if (p < 1 || q < 1 || p > kMaxWidth || q > kMaxWidth) return false;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
  const int pb = std::min(p, kColBlock), qb = std::min(q, kColBlock);
  return gram_smem(true, pb, qb) <= (size_t)optin && gram_smem(false, pb, qb) <= (size_t)optin &&
         gemm_smem(qb) <= (size_t)optin;
}

size_t tc_gram_workspace(long long N, int p, int q) {
  const GramPlan g = gram_plan(N, p);
  return sizeof(float) * (size_t)g.splits * p * std::min(q, kColBlock) + 512;
}

static int tc_gram_block(const float* A, int lda, const float* B, int ldb, long long N, int p, int q, double* C,
                         int ldc, int* err, void* ws, size_t ws_bytes, cudaStream_t st);

int tc_gram_f32_out64(const float* A, int lda, const float* B, int ldb, long long N, int p, int q, double* C, int ldc,
                      int* err, void* ws, size_t ws_bytes, cudaStream_t st) {
  RVGP_CHECK_ARG(p >= 1 && q >= 1 && p <= kMaxWidth && q <= kMaxWidth && N >= 1, "tc_gram: p=%d q=%d out of range",
                 p, q);
  RVGP_CHECK_ARG(ws && ws_bytes >= tc_gram_workspace(N, p, q), "tc_gram: workspace too small");
  if (p <= kColBlock && q <= kColBlock) return tc_gram_block(A, lda, B, ldb, N, p, q, C, ldc, err, ws, ws_bytes, st);
  // column blocks of C (the split partials of one block are reduced before the
  // next block reuses the workspace, in stream order); the first operand's
  // 128-row tiles span all of p, so every block runs the two-operand kernel
  for (int j0 = 0; j0 < q; j0 += kColBlock) {
    const int qb = std::min(kColBlock, q - j0);
    TRY_RC(tc_gram_block(A, lda, B + j0, ldb, N, p, qb, C + j0, ldc, err, ws, ws_bytes, st));
  }
  return RVGP_OK;
}

static int tc_gram_block(const float* A, int lda, const float* B, int ldb, long long N, int p, int q, double* C,
                         int ldc, int* err, void* ws, size_t ws_bytes, cudaStream_t st) {
  const GramPlan g = gram_plan(N, p);
  float* part = static_cast<float*>(ws);
  const bool same = (A == B && lda == ldb && p == q);
  const int Npad = pad16(q);
  const int Brows = same ? std::max(Npad, g.mtiles * kTileM) : Npad;
  const size_t smem = gram_smem(same, p, q);
  dim3 grid(g.mtiles, g.splits);
  int optin = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t bsmem = gram_bulk_smem(p, lda);
  if (same && lda % 4 == 0 && (uintptr_t)A % 16 == 0 && bsmem <= (size_t)optin) {
    TRY_RC(set_smem((const void*)tc_gram_bulk_kernel, bsmem, "tc_gram"));
    rvgp::note_launch();
    tc_gram_bulk_kernel<<<grid, kThreads, bsmem, st>>>(A, lda, N, p, Npad, Brows, g.rows_per, raw_pad_bytes(lda),
                                                        part, err);
  } else if (same) {
    TRY_RC(set_smem((const void*)tc_gram_kernel<true>, smem, "tc_gram"));
    rvgp::note_launch();
    tc_gram_kernel<true><<<grid, kThreads, smem, st>>>(A, lda, B, ldb, N, p, q, Npad, Brows, g.rows_per, part, err);
  } else {
    TRY_RC(set_smem((const void*)tc_gram_kernel<false>, smem, "tc_gram"));
    rvgp::note_launch();
    tc_gram_kernel<false><<<grid, kThreads, smem, st>>>(A, lda, B, ldb, N, p, q, Npad, Brows, g.rows_per, part, err);
  }
  RVGP_LAUNCH_CHECK("tc_gram");
  return reduce_f32_splits_to_f64(part, g.splits, p, q, C, ldc, st);
}

size_t tc_gemm_workspace(int K, int q) {
  return (size_t)ceil_div(K, kSlab) * 2 * pad16(std::min(q, kColBlock)) * 128 + 512;
}

int tc_gemm_f32(const float* A, int lda, long long N, int K, const float* Bm, int ldb, int q, float* C, int ldc,
                int* err, void* ws, size_t ws_bytes, cudaStream_t st) {
  RVGP_CHECK_ARG(K >= 1 && q >= 1 && K <= kMaxWidth && q <= kMaxWidth && N >= 1, "tc_gemm: K=%d q=%d out of range",
                 K, q);
  RVGP_CHECK_ARG(ws && ws_bytes >= tc_gemm_workspace(K, q), "tc_gemm: workspace too small");
  RVGP_CHECK_ARG((uintptr_t)A % 16 == 0, "tc_gemm: A must be 16-byte aligned");
  // output column blocks of at most 256 (one accumulator each); the B image
  // of a block is rebuilt in the workspace after the previous block's kernel
  // (stream order)
  for (int j0 = 0; j0 < q; j0 += kColBlock) {
    const int qb = std::min(kColBlock, q - j0);
    const int Npad = pad16(qb), kslabs = ceil_div(K, kSlab);
    uint8_t* img = static_cast<uint8_t*>(ws);
    rvgp::note_launch();
    build_bimg<<<ceil_div((long long)kslabs * Npad * 8, 256), 256, 0, st>>>(Bm + j0, ldb, K, qb, Npad, kslabs, img);
    const size_t smem = gemm_smem(qb);
    TRY_RC(set_smem((const void*)tc_gemm_kernel, smem, "tc_gemm"));
    rvgp::note_launch();
    tc_gemm_kernel<<<ceil_div(N, kTileM), kThreads, smem, st>>>(A, lda, N, K, img, Npad, qb, C + j0, ldc, err);
    RVGP_LAUNCH_CHECK("tc_gemm");
  }
  return RVGP_OK;
}

}  // namespace rvgp

using namespace rvgp;

// ------------------------------------------------------------------ C ABI (synchronous, for tests and tools)
RVGP_API size_t rvgp_tc_gram_workspace(long long N, int p, int q) { return tc_gram_workspace(N, p, q) + 256; }

RVGP_API int rvgp_tc_gram_f32(const float* A, int lda, const float* B, int ldb, long long N, int p, int q, double* C,
                              int ldc, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(A && B && C, "rvgp_tc_gram_f32: null pointer");
  RVGP_CHECK_ARG(tc_supported(p, q), "rvgp_tc_gram_f32: p=%d, q=%d not supported by the tensor-core path", p, q);
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_tc_gram_workspace(N, p, q), "rvgp_tc_gram_f32: workspace too small");
  cudaStream_t st = as_stream(stream);
  int* err = static_cast<int*>(workspace);
  cudaMemsetAsync(err, 0, sizeof(int), st);
  const int rc = tc_gram_f32_out64(A, lda, B, ldb, N, p, q, C, ldc, err, static_cast<char*>(workspace) + 256,
                                   ws_bytes - 256, st);
  if (rc != RVGP_OK) return rc;
  int h = 0;
  if (read_back(&h, err, sizeof(int), st) != cudaSuccess) return check_launch("rvgp_tc_gram_f32");
  if (h) {
    set_error("rvgp_tc_gram_f32: a tensor-core pipeline wait timed out");
    return RVGP_ELAUNCH;
  }
  return RVGP_OK;
}

RVGP_API size_t rvgp_tc_gemm_workspace(int K, int q) { return tc_gemm_workspace(K, q) + 256; }

RVGP_API int rvgp_tc_gemm_f32(const float* A, int lda, long long N, int K, const float* Bm, int ldb, int q, float* C,
                              int ldc, void* workspace, size_t ws_bytes, void* stream) {
  RVGP_CHECK_ARG(A && Bm && C, "rvgp_tc_gemm_f32: null pointer");
  RVGP_CHECK_ARG(tc_supported(K, q), "rvgp_tc_gemm_f32: K=%d, q=%d not supported by the tensor-core path", K, q);
  RVGP_CHECK_ARG(workspace && ws_bytes >= rvgp_tc_gemm_workspace(K, q), "rvgp_tc_gemm_f32: workspace too small");
  cudaStream_t st = as_stream(stream);
  int* err = static_cast<int*>(workspace);
  cudaMemsetAsync(err, 0, sizeof(int), st);
  const int rc = tc_gemm_f32(A, lda, N, K, Bm, ldb, q, C, ldc, err, static_cast<char*>(workspace) + 256,
                             ws_bytes - 256, st);
  if (rc != RVGP_OK) return rc;
  int h = 0;
  if (read_back(&h, err, sizeof(int), st) != cudaSuccess) return check_launch("rvgp_tc_gemm_f32");
  if (h) {
    set_error("rvgp_tc_gemm_f32: a tensor-core pipeline wait timed out");
    return RVGP_ELAUNCH;
  }
  return RVGP_OK;
}
