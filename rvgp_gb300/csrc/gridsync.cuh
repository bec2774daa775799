// Software grid barrier for persistent kernels launched cooperatively
// (cudaLaunchCooperativeKernel guarantees every CTA of the grid is resident,
// so the barrier cannot wait on a CTA that never runs).
//
// Every wait is bounded: after kSpinLimit polls the barrier sets *err and
// returns false, and every later barrier of the same launch returns false at
// once, so a kernel that checks the result leaves its loops and exits instead
// of hanging the device.  The host turns a non-zero *err into an error status.
#pragma once
#include "common.cuh"

namespace rvgp {

constexpr unsigned long long kSpinLimit = 1ull << 25;

// bar[0] = arrival count, bar[1] = generation; both zero before the launch.
__device__ __forceinline__ bool grid_barrier(unsigned int* bar, int* err, unsigned int nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    if (*((volatile int*)err) != 0) {
      ok = 0;
    } else {
      volatile unsigned int* vgen = bar + 1;
      const unsigned int g = *vgen;
      __threadfence();
      if (atomicAdd(bar, 1u) == nblocks - 1) {
        atomicExch(bar, 0u);
        __threadfence();
        atomicAdd(bar + 1, 1u);
      } else {
        unsigned long long spins = 0;
        while (*vgen == g) {
          if (++spins > kSpinLimit || *((volatile int*)err) != 0) {
            atomicExch(err, 1);
            ok = 0;
            break;
          }
          __nanosleep(32);
        }
      }
      __threadfence();
    }
  }
  __syncthreads();
  return ok != 0;
}

// Contention-free variant: flags[b] (b < G) = last epoch CTA b arrived at,
// flags[G] = last released epoch, all zero before the launch; `epoch` is a
// per-CTA register counter starting at 0.  CTA 0's threads poll the arrival
// slots in parallel, then publish the release; every wait is bounded.
__device__ __forceinline__ bool grid_barrier_flags(unsigned int* flags, unsigned int& epoch, int* err,
                                                   unsigned int G) {
  __shared__ int ok;
  ++epoch;
  __syncthreads();
  volatile unsigned int* vf = flags;
  volatile int* verr = err;
  if (threadIdx.x == 0) {
    __threadfence();
    vf[blockIdx.x] = epoch;
  }
  if (blockIdx.x == 0) {
    int good = 1;
    for (unsigned int b = threadIdx.x; b < G && good; b += blockDim.x) {
      unsigned long long spins = 0;
      while (vf[b] < epoch) {
        if (++spins > kSpinLimit || *verr != 0) {
          good = 0;
          break;
        }
        __nanosleep(16);
      }
    }
    good = __syncthreads_and(good);
    if (threadIdx.x == 0) {
      if (!good) atomicExch(err, 1);
      __threadfence();
      vf[G] = epoch;
      ok = good;
    }
  } else if (threadIdx.x == 0) {
    ok = 1;
    unsigned long long spins = 0;
    while (vf[G] < epoch) {
      if (++spins > kSpinLimit || *verr != 0) {
        atomicExch(err, 1);
        ok = 0;
        break;
      }
      __nanosleep(16);
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// Largest grid of `threads`-thread CTAs of `kernel` that is co-resident.
template <typename K>
int cooperative_grid(K kernel, int threads, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0, coop = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  if (!coop || per_sm < 1) return 0;
  return sms;  // one CTA per SM: enough parallelism for these small problems
}

}  // namespace rvgp
