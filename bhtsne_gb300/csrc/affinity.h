// Affinity kernels (see affinity.cu).
#pragma once

#include "internal.h"

namespace bhg {

constexpr int kMaxSortK = 1024;

template <class T>
struct SymWorkspace {
  DevBuf keys, keys_alt, ev, ev_alt, count, sort_tmp;
  void release() {
    keys.release();
    keys_alt.release();
    ev.release();
    ev_alt.release();
    sort_tmp.release();
  }
};

// Conditional P per row from neighbour distances (n rows of k).
template <class T>
void launch_search_beta(const T* dist, int64_t n, int64_t k, T perplexity, T* p, int32_t* iters, cudaStream_t s);

// Sorts each kNN row by column (in place) and emits + sorts the symmetric
// entries into ws; returns nnz (synchronises the stream).
template <class T>
int64_t symmetrize(uint32_t* cols, T* vals, int64_t n, int k, SymWorkspace<T>& ws, cudaStream_t s);

// Writes the CSR arrays (rows n+1, cols nnz, vals nnz, halved) from ws.
template <class T>
void symmetrize_finish(const SymWorkspace<T>& ws, int64_t n, int64_t nnz, uint64_t* rows, uint32_t* cols_out,
                       T* vals_out, cudaStream_t s);

// FP64 sum of n values into *out (device).
template <class T>
void launch_sum(const T* v, int64_t n, double* out, DevBuf& tmp, cudaStream_t s);

// v *= exaggeration / (sum(v) + eps).
template <class T>
void launch_normalize(T* v, int64_t n, T exaggeration, double* sum_dev, DevBuf& tmp, cudaStream_t s);

template <class T>
void launch_scale(T* v, int64_t n, T scale, cudaStream_t s);

template <class T>
void launch_scaled_copy(const T* v, int64_t n, T scale, T* out, cudaStream_t s);

}  // namespace bhg
