// Exact Euclidean kNN (see knn.cu).
#pragma once

#include "internal.h"

namespace bhg {

struct KnnWorkspace {
  DevBuf xf, norms, cand, thr, fails, counters;
  int64_t last_fallback_rows = 0;
  void release() {
    xf.release();
    norms.release();
    cand.release();
    thr.release();
    fails.release();
  }
};

// Writes, per row of X (n x dim, row-major), the k nearest other rows ordered
// by (distance, index) and their distances. Returns the number of rows that
// needed the exact fallback (synchronises the stream).
template <class T>
int64_t knn_euclidean(const T* X, int64_t n, int dim, int k, uint32_t* out_idx, T* out_dist, KnnWorkspace& ws,
                      cudaStream_t s);

}  // namespace bhg
