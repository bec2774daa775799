// Error state and library-level entry points of librvgp_gb300.
#include "common.cuh"
#include <string.h>
#include <atomic>

namespace rvgp {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

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
