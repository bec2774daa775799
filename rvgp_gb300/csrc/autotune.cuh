// Launch-configuration autotuner with an on-disk cache (internal).
//
// A kernel with several launch variants that compute the same result (the
// same arithmetic in the same order, so the choice never changes a result)
// asks tune(key, ...) for the variant to run.  The first call with a key times
// every variant on the caller's stream with CUDA events (one warm-up run and
// `reps` timed runs each) and keeps the fastest; later calls, in this process
// or in any process that reads the same cache file, reuse it.  The key names
// the kernel and the shape class (e.g. "bspmm f32 DB2 b564 n2^17 deg16").
//
// The cache is one text file, a line "key choice t0 t1 ..." (milliseconds
// per variant) per entry: $RVGP_AUTOTUNE_CACHE, else
// $XDG_CACHE_HOME/rvgp_gb300/autotune.txt, else ~/.cache/rvgp_gb300/autotune.txt.
// Tuning needs host synchronisation, so it is skipped (the default variant
// runs, nothing is stored) while the stream is being captured into a CUDA
// graph, and when RVGP_AUTOTUNE=0.
#pragma once
#include "common.cuh"
#include <functional>
#include <string>

namespace rvgp {
namespace autotune {

bool enabled();
const char* cache_path();
// cached choice for key, or -1
int lookup(const std::string& key);
// run(v) enqueues variant v on st and returns an RVGP status; returns the
// chosen variant (default_choice when tuning is off or not possible), or a
// negative status if a variant failed to launch.
int tune(const std::string& key, int nvar, int default_choice, cudaStream_t st, int reps,
         const std::function<int(int)>& run);
// power-of-two bucket of x (shape classes)
int log2_bucket(long long x);

}  // namespace autotune
}  // namespace rvgp
