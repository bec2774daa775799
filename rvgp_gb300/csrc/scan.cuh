// Deterministic exclusive prefix sum over int32 (three kernels, no atomics).
#pragma once
#include "common.cuh"

namespace rvgp {
// internal linkage: every translation unit that includes this gets its own copy
namespace {

constexpr int kScanBlock = 1024;  // elements per CTA in the first pass (256 threads x 4)

__global__ void scan_blocks(const int* __restrict__ in, int n, int* __restrict__ out, int* __restrict__ sums) {
  __shared__ int sh[256];
  const int base = blockIdx.x * kScanBlock + threadIdx.x * 4;
  int v[4], s = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    v[r] = base + r < n ? in[base + r] : 0;
    s += v[r];
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < 256; off <<= 1) {
    int t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  int run = sh[threadIdx.x] - s;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    if (base + r < n) out[base + r] = run;
    run += v[r];
  }
  if (threadIdx.x == 255) sums[blockIdx.x] = sh[255];
}

// single CTA: exclusive scan of the per-block sums in place; total to *total
__global__ void scan_sums(int* __restrict__ sums, int nb, int* __restrict__ total) {
  __shared__ int sh[1024];
  int carry = 0;
  for (int c0 = 0; c0 < nb; c0 += 1024) {
    int i = c0 + threadIdx.x;
    int v = i < nb ? sums[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      int t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) sums[i] = carry + sh[threadIdx.x] - v;
    int blk_total = sh[1023];
    __syncthreads();
    carry += blk_total;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void scan_add(int* __restrict__ out, int n, const int* __restrict__ sums) {
  const int base = blockIdx.x * kScanBlock + threadIdx.x * 4;
  const int add = sums[blockIdx.x];
#pragma unroll
  for (int r = 0; r < 4; ++r)
    if (base + r < n) out[base + r] += add;
}

size_t scan_workspace(int n) { return sizeof(int) * (size_t)(ceil_div(n, kScanBlock) + 1); }

// out[i] = sum_{j<i} in[j] for i < n; *total (device) = sum of all (may be nullptr).
void exclusive_scan(const int* in, int n, int* out, int* total, int* ws, cudaStream_t st) {
  int nb = ceil_div(n, kScanBlock);
  rvgp::note_launch(); scan_blocks<<<nb, 256, 0, st>>>(in, n, out, ws);
  rvgp::note_launch(); scan_sums<<<1, 1024, 0, st>>>(ws, nb, total);
  rvgp::note_launch(); scan_add<<<nb, 256, 0, st>>>(out, n, ws);
}

}  // namespace
}  // namespace rvgp
