// Per-epoch kernels (see epoch.cu).
#pragma once

#include "internal.h"

namespace bhg {

struct UpdateScratch {
  DevBuf part, done, mean_sum;
  bool zeroed = false;
  const double* mean() const { return static_cast<const double*>(mean_sum.ptr); }
};

template <class T>
void launch_attractive(int D, const uint64_t* rows, const uint32_t* cols, const T* vals, const T* y, int64_t n, T* pos,
                       cudaStream_t s);

// Fused gradient step; neg == nullptr means pos already holds the gradient.
// The reciprocal normaliser is 1 / (T)*z, or inv_norm when z is null.
// Leaves sum(y_new) per axis in us.mean_sum.
template <class T>
void launch_update(int D, T* y, const T* pos, const T* neg, T* uy, T* gains, int64_t n, const double* z, T inv_norm,
                   T lr, T momentum, UpdateScratch& us, cudaStream_t s);

template <class T>
void launch_kl_sparse(int D, const uint64_t* rows, const uint32_t* cols, const T* vals, const T* y, int64_t n,
                      const double* z, bool quirk, double* out, DevBuf& tmp, cudaStream_t s);

template <class T>
void launch_dense_distance(const T* X, int64_t n, int dim, bool squared, T* dist, cudaStream_t s);

template <class T>
void launch_dense_symmetrize(T* p, int64_t n, cudaStream_t s);

template <class T>
void launch_exact_z(int D, const T* y, int64_t n, double* z, DevBuf& tmp, cudaStream_t s);

template <class T>
void launch_exact_grad(int D, const T* y, const T* p, int64_t n, const double* z, T* dy, cudaStream_t s);

template <class T>
void launch_exact_kl(int D, const T* y, const T* p, int64_t n, const double* z, double* out, DevBuf& tmp,
                     cudaStream_t s);

}  // namespace bhg
