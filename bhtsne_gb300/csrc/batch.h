// Batched Barnes-Hut stages (see batch.cu).
#pragma once

#include "affinity.h"
#include "bh.h"
#include "knn.h"

namespace bhg {

// Affinities of several independent point sets built together: one
// block-diagonal CSR over their rows stacked in order (group numbering).
template <class T>
struct GroupCsr {
  DevBuf rows, cols, vals;
  std::vector<uint64_t> rows_h;  // host copy of the row offsets
  int64_t nnz = 0;
};

template <class T>
struct AffinityScratch {
  DevBuf g_off, g_of, kidx, kdist, kp, xin;
  KnnWorkspace knn;
  SymWorkspace<T> sym;
  void release() {
    kidx.release();
    kdist.release();
    kp.release();
    xin.release();
    knn.release();
    sym.release();
  }
};

// Dense Euclidean sets X[g] (device, n[g] x dim each, one dim for all): the
// segmented kNN over their stacked rows, then group_affinities_from_knn.
template <class T>
void group_affinities_euclidean(const std::vector<const T*>& X, const std::vector<int64_t>& n, int dim, int64_t k,
                                T perplexity, GroupCsr<T>& out, AffinityScratch<T>& ws, cudaStream_t s);

// search_beta + symmetrize (build_affinities, src/lib.rs:1061-1127) over a
// stacked kNN table already in ws.kidx / ws.kdist (tot rows of k, indices in
// group numbering): every set's rows, columns and values are those of its own
// fit, shifted to its place in the group.
template <class T>
void group_affinities_from_knn(int64_t tot, int64_t k, T perplexity, GroupCsr<T>& out, AffinityScratch<T>& ws,
                               cudaStream_t s);

// Per-job bounding box (one block per job), recentring by the job's mean first
// when apply_mean; boxes[j] gets the job's quantisation and half-width table.
// Jobs with active[j] == 0 (when active is given) are not recentred.
template <class T>
void batch_box(int D, T* y, const int64_t* off, int K, bool apply_mean, BoxParams<T>* boxes, int bits, cudaStream_t s,
               const uint8_t* active = nullptr);

// Per-job Morton codes, sort by (job, code), and the forest of per-job trees
// in ws (tiles: the job-relative prefix-sum tiles of the same offsets).
// jobkey ends up holding the job of every sorted position.
template <class T>
void batch_sort_and_build(int D, const T* y, int64_t total, int K, const uint32_t* job_of, const int64_t* off,
                          const BoxParams<T>* boxes, BhWorkspace<T>& ws, DevBuf& codes, DevBuf& jobkey,
                          DevBuf& jobkey_alt, const SegTiles& tiles, cudaStream_t s);

// z[j] = sum of q over job j's points (FP64, one block per job).
template <class T>
void batch_z(const T* q, const int64_t* off, int K, double* z, cudaStream_t s);

// Fused gradient step with the job's 1/Z, learning rate and momentum; points
// of jobs with active[j] == 0 (when active is given) are left untouched.
template <class T>
void batch_update(int D, T* y, const T* pos, const T* neg, T* uy, T* gains, int64_t total, const uint32_t* job_of,
                  const double* z, const T* lr, const T* momentum, cudaStream_t s, const uint8_t* active = nullptr);

// Appends a job's CSR to the block-diagonal matrix (row offsets + row_add,
// columns + col_add), and the inverse extraction.
void batch_append_csr(const uint64_t* rows, const uint32_t* cols, int64_t n, int64_t nnz, uint64_t row_add,
                      uint32_t col_add, uint64_t* rows_out, uint32_t* cols_out, cudaStream_t s);
void batch_extract_csr(const uint64_t* rows, const uint32_t* cols, int64_t n, int64_t nnz, uint64_t row_sub,
                       uint32_t col_sub, uint64_t* rows_out, uint32_t* cols_out, cudaStream_t s);
// normalize_p_values of every job (job j's values are nnz_off[j]..nnz_off[j+1]).
template <class T>
void batch_normalize(T* vals, const int64_t* nnz_off, int K, T exaggeration, bool unexaggerate, cudaStream_t s);
// out[e] = in[e] + add (kNN indices moved to a job's place in a group).
void batch_offset_indices(const uint32_t* in, int64_t count, uint32_t add, uint32_t* out, cudaStream_t s);
void batch_fill_job(uint32_t* job_of, int64_t lo, int64_t hi, uint32_t j, cudaStream_t s);

}  // namespace bhg
