// Register-resident top-k list shared by the kNN screens (knn.cu, knn_tc.cu).
#pragma once
#include <float.h>

namespace rvgp {

// The KC smallest (value, index) pairs seen, ascending, held in registers:
// every position is a compile-time index, so nothing spills to local memory.
// Empty slots hold (FLT_MAX, -1).
template <int KC>
struct RegTop {
  float d[KC];
  int i[KC];
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int r = 0; r < KC; ++r) {
      d[r] = FLT_MAX;
      i[r] = -1;
    }
  }
  __device__ __forceinline__ float worst() const { return d[KC - 1]; }
  // Insert keeping the order (equal values stay in arrival order); call only
  // when v < worst().  Each position decides from the old values of itself and
  // its predecessor, so the KC selects are independent of one another.
  __device__ __forceinline__ void insert(float v, int idx) {
#pragma unroll
    for (int r = KC - 1; r > 0; --r) {
      const bool shift = d[r - 1] > v;
      const bool here = d[r] > v;
      d[r] = shift ? d[r - 1] : (here ? v : d[r]);
      i[r] = shift ? i[r - 1] : (here ? idx : i[r]);
    }
    if (d[0] > v) {
      d[0] = v;
      i[0] = idx;
    }
  }
};

}  // namespace rvgp
