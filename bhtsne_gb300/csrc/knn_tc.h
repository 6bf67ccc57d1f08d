// Tensor-core candidate pass of the exact kNN (see knn_tc.cu).
#pragma once

#include <cmath>
#include <vector>

#include "internal.h"

namespace bhg {

struct KnnTcScratch {
  DevBuf xhi, err;  // xhi: rows padded to a multiple of 16 dimensions when needed
  DevBuf split;     // candidate tiles split into TF32 hi / lo (resident form)
  DevBuf tile_base; // first split tile of each point set (segmented calls)
  bool last_resident = false;  // the last call ran the resident form
  bool last_segmented = false;
  int64_t last_n = 0;
  int last_dim = 0;
  const float* last_xp = nullptr;  // its rows (padded to 16 dimensions when needed)
  void release() {
    xhi.release();
    split.release();
    tile_base.release();
  }
};

// Per query of X (n x dim, FP32): the indices of its 128 candidates with the
// smallest |q|^2 + |c|^2 - 2 q.c (3xTF32 tensor-core dot products), sorted by
// (value, index), into cand[q * 128 ..], and the 128-th value into thr[q]
// (INFINITY when fewer candidates exist). Blocks of 128 queries; with a block
// table (blk_q0, blk_job, seg_off, and the host copy of the set offsets in
// off) block b takes queries blk_q0[b].. of set blk_job[b] and scans only
// that set's rows. Rows of at most 128 dimensions run the resident form
// (query tile in tensor memory, candidate tiles split once into hi / lo and
// streamed by bulk copies: 2 n dim_pad floats of scratch), wider rows the
// staged form. Synchronises the stream.
void knn_tc_candidates(const float* X, int64_t n, int dim, const float* norms, const int64_t* blk_q0,
                       const int32_t* blk_job, const int64_t* seg_off, const std::vector<int64_t>* off,
                       int64_t nblocks, uint32_t* cand, float* thr, KnnTcScratch& ws, cudaStream_t s);

// Bounded re-scan after a resident, unsegmented knn_tc_candidates call on the
// same rows (its split tiles are reused): for listed row i (row qrows[i] of
// X), every j with candidate value <= qbound[i], in index order, into
// list[i * cap ..], and their count (which may exceed cap) into list_cnt[i].
// Candidate values are those of knn_tc_candidates, so a row's true
// neighbours, whose values the certificate's error bound keeps below
// qbound[i], are all listed when the count is at most cap. Synchronises.
bool knn_tc_can_bound(const KnnTcScratch& ws, int64_t n, int dim);
void knn_tc_bounded(int64_t n, int dim, const float* norms, const uint32_t* qrows, const float* qbound, int64_t nq,
                    uint32_t* list, uint32_t* list_cnt, int cap, KnnTcScratch& ws, cudaStream_t s);

// Error coefficient of the tensor-core candidate values: |v - d^2| <= coef *
// (|q|^2 + r^2) for candidates within radius r of the origin.
inline double knn_tc_error_coef(int dim) {
  const int dim_pad = (dim + 15) / 16 * 16;
  return 2.0 * (std::ldexp(1.0, -19) + (3.0 * dim_pad + 8.0) * std::ldexp(1.0, -23) + (dim + 8.0) * std::ldexp(1.0, -24));
}

}  // namespace bhg
