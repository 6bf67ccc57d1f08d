// Per-epoch kernels (see epoch.cu).
#pragma once

#include "internal.h"

namespace bhg {

struct UpdateScratch {
  DevBuf part, done, mean_sum;
  bool zeroed = false;
  const double* mean() const { return static_cast<const double*>(mean_sum.ptr); }
};

// Attractive forces over bounded tasks: every CSR row is cut into tasks of at
// most task_len entries (64, 128 or 256: 2, 4 or 8 per lane), one warp per
// task. A row of one task writes its slot directly; the tasks of a longer row
// write partial sums that a second kernel adds in task order, so results do
// not depend on scheduling (they do depend on task_len, which sets how a row's
// terms are grouped). Built once per CSR layout (one host synchronisation),
// replayed every epoch.
constexpr int kAttrTaskLen = 128;  // the default task length
// Component layout (component_order) for fits of at least this many points:
// below it y stays in cache whatever the layout.
constexpr int64_t kComponentMinN = 65536;
struct AttrTasks {
  DevBuf tasks, off, cnt, longs, nlong_dev, part, scan_tmp;
  int64_t ntasks = 0, nlong = 0, n = 0;
  int D = 0;
  int task_len = kAttrTaskLen;
  uint64_t gen = ~0ull;  // layout generation the tasks were built for
};

template <class T>
void build_attr_tasks(AttrTasks& at, int D, const uint64_t* rows, int64_t n, cudaStream_t s,
                      int task_len = kAttrTaskLen);

template <class T>
void launch_attractive_tasks(const AttrTasks& at, const uint32_t* cols, const T* vals, const T* y, T* pos,
                             cudaStream_t s);

// random_init (the reference's is unseeded, src/tsne/mod.rs:142-147): a
// seeded Box-Muller N(0, 1e-4) over the LCG s <- 6364136223846793005 s +
// 1442695040888963407, values 2i and 2i + 1 from states 2i + 1 and 2i + 2.
template <class T>
void launch_random_init(T* y, int64_t count, uint64_t seed, cudaStream_t s);

// Locality renumbering of the device-resident optimisation state. The points
// are re-laid out in `order` (a permutation of the current slots, e.g. the
// Morton order of the embedding); ext[s] is the point (CSR row) held by slot
// s, inv its inverse, and cols the CSR columns translated to slots.
// Locality layout of the embedding state: slot s holds the point ext[s]
// (inv is the inverse map). rows/cols/vals are P in slot order: row s is the
// CSR row of ext[s] with columns as slots, sorted within the row.
struct Renumbering {
  bool active = false;
  DevBuf ext, ext_alt, inv, rows, cols, vals, len, scan_tmp;
  DevBuf long_rows;  // u32 count, then the slots of the rows longer than the register sort takes
};

template <class T>
void launch_renumber(int D, const uint32_t* order, int64_t n, Renumbering& r, T* y, T* uy, T* gains, T* tmp_a, T* tmp_b,
                     T* tmp_c, const uint64_t* rows, const uint32_t* cols, const T* vals, int64_t nnz, cudaStream_t s);

// Component layout: the connected components of the (symmetric) CSR graph of
// P, found by minimum-label propagation (called at a fit's first periodic
// re-layout point). When the graph splits into
// components of at most n / 4 points each, `order` receives the points
// grouped by component (the component of the smallest index first), in index
// order within each, and the call returns true. A layout in that order keeps
// every row's columns inside its component's slot range, so the attractive
// pass's gathers of y stay within a few hundred kilobytes. False (order
// unspecified) for a graph with a larger component; `largest` receives the
// size of the largest component (0 when propagation did not settle).
struct ComponentScratch {
  DevBuf label, count, keys, keys_alt, vals_alt, flag, sort_tmp;
  void release() {
    label.release();
    count.release();
    keys.release();
    keys_alt.release();
    vals_alt.release();
    flag.release();
    sort_tmp.release();
  }
};
bool component_order(const uint64_t* rows, const uint32_t* cols, int64_t n, DevBuf& order, ComponentScratch& cs,
                     int64_t* largest, cudaStream_t s);
// out[s] = inv[order[s]]: an order of CSR rows as an order of the current slots.
void launch_compose_order(const uint32_t* order, const uint32_t* inv, int64_t n, uint32_t* out, cudaStream_t s);

// out[ext[s]] = y[s]: back to the caller's point order.
template <class T>
void launch_unpermute(int D, const T* y, const uint32_t* ext, int64_t n, T* out, cudaStream_t s);

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
