// Batched Barnes-Hut stages (see batch.cu).
#pragma once

#include "bh.h"

namespace bhg {

// Per-job bounding box (one block per job), recentring by the job's mean first
// when apply_mean; boxes[j] gets the job's quantisation and half-width table.
template <class T>
void batch_box(int D, T* y, const int64_t* off, int K, bool apply_mean, BoxParams<T>* boxes, int bits, cudaStream_t s);

// Per-job Morton codes, sort by (job, code), and the forest of per-job trees
// in ws. jobkey ends up holding the job of every sorted position.
template <class T>
void batch_sort_and_build(int D, const T* y, int64_t total, int K, const uint32_t* job_of, const int64_t* off,
                          const BoxParams<T>* boxes, BhWorkspace<T>& ws, DevBuf& codes, DevBuf& jobkey,
                          DevBuf& jobkey_alt, cudaStream_t s);

// z[j] = sum of q over job j's points (FP64, one block per job).
template <class T>
void batch_z(const T* q, const int64_t* off, int K, double* z, cudaStream_t s);

// Fused gradient step with the job's 1/Z, learning rate and momentum.
template <class T>
void batch_update(int D, T* y, const T* pos, const T* neg, T* uy, T* gains, int64_t total, const uint32_t* job_of,
                  const double* z, const T* lr, const T* momentum, cudaStream_t s);

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
