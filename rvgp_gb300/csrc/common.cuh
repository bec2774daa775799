// Shared definitions for the RVGP GB300 kernels (sm_103a).
//
// Every exported entry point follows one convention: device pointers and
// sizes in, an opaque stream (cudaStream_t passed as void*) and, where a
// kernel needs scratch, a caller-provided workspace with a size query.  The
// return value is 0 on success, > 0 for numerical information (documented per
// call) and < 0 for bad arguments or launch failures; rvgp_last_error()
// returns the message of the last failure on the calling host thread.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>
#include <stddef.h>

#define RVGP_OK 0
#define RVGP_EARG (-1)
#define RVGP_ELAUNCH (-2)
#define RVGP_EWORKSPACE (-3)
#define RVGP_ENOTSUP (-4)

#define RVGP_API extern "C" __attribute__((visibility("default")))

namespace rvgp {

void set_error(const char* fmt, ...);
int check_launch(const char* what);
// process-wide count of kernel launches made by this library (diagnostics)
void note_launch();

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Bump allocator over a caller-provided workspace.  Every carve-out is
// 256-byte aligned.  With base == nullptr it only measures.
struct Workspace {
  char* base;
  size_t cap;
  size_t used = 0;
  Workspace(void* b, size_t c) : base(static_cast<char*>(b)), cap(c) {}
  template <typename T>
  T* take(size_t count) {
    size_t off = (used + 255) & ~size_t(255);
    used = off + count * sizeof(T);
    return base ? reinterpret_cast<T*>(base + off) : nullptr;
  }
  bool ok() const { return base == nullptr || used <= cap; }
};

// Device-to-host read of results queued on `st`: waits for the stream first
// and copies after.  A copy into pageable host memory issued while the
// stream is still busy blocks the CUDA calls of every other host thread
// until it completes; waiting in cudaStreamSynchronize does not.
inline cudaError_t read_back(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Streaming multiprocessors of the current device (queried once per device
// and cached; 152 on GB300, 2 dies x 76).  Host-side planning of grids and of
// the workspaces that depend on them uses it; every entry point recomputes
// its workspace need on the device it runs on.
int num_sms();

// Raise (never lower) a kernel's dynamic shared-memory limit on the current
// device: the limit is a per-function setting shared by every host thread,
// so two threads launching one kernel with different sizes must not set it
// down under each other's launch.
cudaError_t raise_dyn_smem(const void* fn, size_t bytes);

}  // namespace rvgp

#define RVGP_CHECK_ARG(cond, ...)        \
  do {                                   \
    if (!(cond)) {                       \
      rvgp::set_error(__VA_ARGS__);      \
      return RVGP_EARG;                  \
    }                                    \
  } while (0)

#define TRY_RC(x)               \
  do {                          \
    int _rc = (x);              \
    if (_rc != RVGP_OK) return _rc; \
  } while (0)

#define RVGP_LAUNCH_CHECK(what)                         \
  do {                                                  \
    int _st = rvgp::check_launch(what);                 \
    if (_st != RVGP_OK) return _st;                     \
  } while (0)
