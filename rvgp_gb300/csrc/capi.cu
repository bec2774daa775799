// Error state and library-level entry points of librvgp_gb300.
#include <mutex>
#include <map>
#include "common.cuh"
#include <string.h>
#include <atomic>

namespace rvgp {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int num_sms() {
  constexpr int kMaxDevices = 64, kDefault = 152;
  static std::atomic<int> cache[kMaxDevices] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return kDefault;  // no device (host-only size queries): the GB300 count
  }
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
    cudaGetLastError();
    v = kDefault;
  }
  cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return RVGP_ELAUNCH;
  }
  return RVGP_OK;
}

}  // namespace rvgp

RVGP_API const char* rvgp_last_error(void) { return rvgp::g_err; }

RVGP_API int rvgp_abi_version(void) { return 1; }

// Kernels launched by this library since it was loaded (all host threads).
RVGP_API long long rvgp_launch_count(void) { return rvgp::g_launches.load(std::memory_order_relaxed); }

namespace rvgp {
cudaError_t raise_dyn_smem(const void* fn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> set;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = set[{dev, fn}];
  if (bytes <= cur) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}
}  // namespace rvgp

