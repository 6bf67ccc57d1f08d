// Exact Euclidean kNN (see knn.cu).
#pragma once

#include <vector>

#include "internal.h"
#include "knn_tc.h"

namespace bhg {

struct KnnWorkspace {
  DevBuf xf, norms, cand, thr, fails, counters, blk, tc_blk, slices, fbound, list, over;
  KnnTcScratch tc;
  int64_t last_fallback_rows = 0;
  int last_fallback_slices = 1;  // candidate slices of the last brute force
  int64_t last_brute_rows = 0;   // rows of the last call that took the brute force
  // candidate pass: -1 the default (tensor cores unless BHTSNE_KNN_SIMT is
  // set), 0 tensor cores, 1 CUDA cores; both give the same neighbours
  int pass = -1;
  void release() {
    xf.release();
    norms.release();
    cand.release();
    thr.release();
    fails.release();
    blk.release();
    tc_blk.release();
    slices.release();
    fbound.release();
    list.release();
    over.release();
    tc.release();
  }
};

// Writes, per row of X (n x dim, row-major), the k nearest other rows ordered
// by (distance, index) and their distances. Returns the number of rows that
// needed the exact fallback (synchronises the stream).
template <class T>
int64_t knn_euclidean(const T* X, int64_t n, int dim, int k, uint32_t* out_idx, T* out_dist, KnnWorkspace& ws,
                      cudaStream_t s);

// The same over many independent point sets stored back to back (set j owns
// rows off[j]..off[j+1]; seg_of[row] is the set of a row, off is also given on
// the device as d_off): every row gets its k nearest rows of its own set, as
// global row indices. All sets share dim and k.
template <class T>
int64_t knn_euclidean_segmented(const T* X, int64_t total, int dim, int k, const std::vector<int64_t>& off,
                                const int64_t* d_off, const uint32_t* d_seg_of, uint32_t* out_idx, T* out_dist,
                                KnnWorkspace& ws, cudaStream_t s);

}  // namespace bhg
