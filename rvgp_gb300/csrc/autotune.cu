// Launch-configuration autotuner with an on-disk cache (see autotune.cuh).
#include "autotune.cuh"
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <map>
#include <mutex>
#include <vector>

namespace rvgp {
namespace autotune {
namespace {

std::mutex g_mu;
std::map<std::string, int> g_cache;
bool g_loaded = false;
std::string g_path;

void ensure_dir(const std::string& file) {
  std::string dir;
  for (size_t i = 1; i < file.size(); ++i)
    if (file[i] == '/') {
      dir = file.substr(0, i);
      mkdir(dir.c_str(), 0755);  // an existing directory is fine
    }
}

void load_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const char* e = getenv("RVGP_AUTOTUNE_CACHE");
  if (e && e[0]) {
    g_path = e;
  } else {
    const char* x = getenv("XDG_CACHE_HOME");
    const char* h = getenv("HOME");
    g_path = (x && x[0]) ? std::string(x) + "/rvgp_gb300/autotune.txt"
                         : std::string(h && h[0] ? h : "/tmp") + "/.cache/rvgp_gb300/autotune.txt";
  }
  FILE* f = fopen(g_path.c_str(), "r");
  if (!f) return;
  char line[1024];
  while (fgets(line, sizeof(line), f)) {
    // "key words ... choice t0 t1 ...": the key is everything before the
    // field that starts with '#', written as "key # choice t0 ..."
    char* hash = strstr(line, " # ");
    if (!hash) continue;
    *hash = 0;
    const int choice = atoi(hash + 3);
    if (choice >= 0) g_cache[line] = choice;
  }
  fclose(f);
}

void append_locked(const std::string& key, int choice, const std::vector<float>& ms) {
  ensure_dir(g_path);
  FILE* f = fopen(g_path.c_str(), "a");
  if (!f) return;  // a read-only home: the choice still holds for this process
  fprintf(f, "%s # %d", key.c_str(), choice);
  for (float t : ms) fprintf(f, " %.4f", t);
  fprintf(f, "\n");
  fclose(f);
}

}  // namespace

bool enabled() {
  const char* e = getenv("RVGP_AUTOTUNE");
  return !(e && e[0] == '0');
}

const char* cache_path() {
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  return g_path.c_str();
}

int lookup(const std::string& key) {
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  auto it = g_cache.find(key);
  return it == g_cache.end() ? -1 : it->second;
}

int log2_bucket(long long x) {
  int b = 0;
  while (x > 1) {
    x >>= 1;
    ++b;
  }
  return b;
}

int tune(const std::string& key, int nvar, int default_choice, cudaStream_t st, int reps,
         const std::function<int(int)>& run) {
  if (!enabled() || nvar <= 1) return default_choice;
  const int cached = lookup(key);
  if (cached >= 0 && cached < nvar) return cached;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return default_choice;
  }
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    return default_choice;
  }
  std::vector<float> ms(nvar, 0.f);
  int best = default_choice;
  for (int v = 0; v < nvar; ++v) {
    int rc = run(v);  // warm-up (and the launch check)
    if (rc != RVGP_OK) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; ++r) run(v);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    ms[v] = t / reps;
  }
  best = 0;
  for (int v = 1; v < nvar; ++v)
    if (ms[v] < ms[best]) best = v;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::lock_guard<std::mutex> lk(g_mu);
  load_locked();
  g_cache[key] = best;
  append_locked(key, best, ms);
  return best;
}

}  // namespace autotune
}  // namespace rvgp

RVGP_API const char* rvgp_autotune_cache_path(void) { return rvgp::autotune::cache_path(); }

// Cached variant for a key (see autotune.cuh), or -1.
RVGP_API int rvgp_autotune_lookup(const char* key) { return key ? rvgp::autotune::lookup(key) : -1; }
