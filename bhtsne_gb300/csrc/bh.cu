// Barnes-Hut repulsion on the GPU: bounding box, Morton codes, radix sort,
// a parallel build of the reference's compressed 2^D-tree, centre-of-mass
// summaries, and a stackless per-point traversal.
//
// Reference behaviour restated (bhtsne 0.7.10):
//  * bounding box, quantisation scale and per-level half widths:
//    src/tsne/arena.rs:65-94, :154-174; quantize: src/tsne/morton.rs:103-120;
//    encoders: src/tsne/morton/d2.rs:5-47, src/tsne/morton/d3.rs:5-50.
//  * tree shape: src/tsne/arena.rs:197-259. A node whose Morton range holds
//    more than one distinct code becomes internal at the tightest D-bit level
//    that splits the range; its children are the non-empty orthants at that
//    level; a run of equal codes is a leaf.
//  * leaf centre of mass = mean of members (:264-284); internal = count
//    weighted mean (:289-309).
//  * traversal: :338-392 (skip the leaf at zero distance; descend while
//    half_width^2[level] >= theta^2 * dist^2; accumulate count/(1+d^2)).
//
// GPU construction (no sequential breadth-first walk):
//  * For sorted codes c[0..N), the boundary between s-1 and s (c[s-1] != c[s])
//    has level l = bits-1 - msb(c[s-1]^c[s])/D. The internal node that owns
//    the boundary is the Morton cell at depth l holding c[s]; its range
//    [a, e) is found by binary search for the cell's first and one-past-last
//    codes. The boundary is the node's representative when c[s-1] lies in the
//    first child of that cell, so every internal node is emitted exactly once.
//  * Nodes are laid out in depth-first preorder, i.e. by (range start, level).
//    A bitmask per start position records the levels of the internal nodes
//    starting there; an exclusive scan of (popcount + run-start flag) gives
//    every node its index, and the index one past a node's subtree ("skip")
//    is simply the scan value at the node's range end.
//  * Internal centres of mass come from FP64 prefix sums of the Z-ordered
//    points, (S[e] - S[a]) / (e - a), which equals the count-weighted mean of
//    the children. Leaves are summed in T exactly like the reference so that
//    a singleton leaf's centre is bit-identical to its point (the self test).
#include "bh.h"

#include <type_traits>
#include "bh_dev.cuh"

namespace bhg {

namespace {

constexpr int kThreads = 256;
constexpr int kTraverseMax = 512;
static_assert(kBhThreads == 128, "bh_sizes sizes the Z partials for traversal blocks of at least 128 threads");

// ---------------------------------------------------------------------------
// Recentre (optional) + per-axis bounding box; the last block to finish
// derives the tree parameters. Also used by the FIt-SNE path (min/max only).
// ---------------------------------------------------------------------------
template <class T, int D>
__global__ void recenter_bbox_kernel(T* __restrict__ y, int64_t n, const double* __restrict__ mean_sum,
                                     int apply_mean, T* __restrict__ part_min, T* __restrict__ part_max,
                                     unsigned* __restrict__ done, BoxParams<T>* __restrict__ out, int bits) {
  __shared__ T smin[D][32], smax[D][32];
  __shared__ bool last;
  T mean[D];
  if (apply_mean) {
#pragma unroll
    for (int a = 0; a < D; ++a) mean[a] = (T)mean_sum[a] / (T)n;
  }
  T mn[D], mx[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    mn[a] = Lim<T>::max();
    mx[a] = -Lim<T>::max();
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      T v = y[i * D + a];
      if (apply_mean) {
        v = v - mean[a];
        y[i * D + a] = v;
      }
      mn[a] = fmin(mn[a], v);
      mx[a] = fmax(mx[a], v);
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    T m0 = warp_min(mn[a]), m1 = warp_max(mx[a]);
    if (lane == 0) {
      smin[a][w] = m0;
      smax[a][w] = m1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      T m0 = smin[a][0], m1 = smax[a][0];
      for (int q = 1; q < nw; ++q) {
        m0 = fmin(m0, smin[a][q]);
        m1 = fmax(m1, smax[a][q]);
      }
      part_min[blockIdx.x * D + a] = m0;
      part_max[blockIdx.x * D + a] = m1;
    }
    __threadfence();
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ T shr[32];
  T fmn[D], fmx[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    fmn[a] = block_min_parts<T>(part_min, gridDim.x, D, a, Lim<T>::max(), shr);
    fmx[a] = block_max_parts<T>(part_max, gridDim.x, D, a, -Lim<T>::max(), shr);
  }
  if (threadIdx.x == 0) {
    const T scale = (T)(double)(1ULL << bits);
    T max_extent = T(0);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const T ext = fmx[a] - fmn[a];
      out->mn[a] = fmn[a];
      out->mx[a] = fmx[a];
      out->inv_scale[a] = ext > T(0) ? scale / ext : T(0);
      max_extent = fmax(max_extent, ext);
    }
    for (int a = D; a < 8; ++a) {
      out->mn[a] = T(0);
      out->mx[a] = T(0);
      out->inv_scale[a] = T(0);
    }
    out->max_extent = max_extent;
    for (int l = 0; l <= bits; ++l) {
      const T hw = max_extent / (T)(double)(1ULL << (l + 1));
      out->hw2[l] = hw * hw;
    }
    *done = 0;
  }
}

// Morton codes of the points in index order. 64-bit codes go to keys; 128-bit
// codes (D >= 5) are split into lo (also copied to keys, the first sort key)
// and hi.
template <class T, int D>
__global__ void morton_kernel(const T* __restrict__ y, int64_t n, const BoxParams<T>* __restrict__ prm,
                              uint64_t* __restrict__ keys, uint32_t* __restrict__ idx, uint64_t* __restrict__ lo_out,
                              uint64_t* __restrict__ hi_out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  constexpr int B = MortonD<D>::BITS;
  const uint32_t max_bucket = (uint32_t)((1ULL << B) - 1);
  uint32_t q[D];
#pragma unroll
  for (int a = 0; a < D; ++a) q[a] = quantize<T>(y[i * D + a], prm->mn[a], prm->inv_scale[a], max_bucket);
  const typename MortonD<D>::Code c = MortonD<D>::encode(q);
  if constexpr (sizeof(c) == 8) {
    keys[i] = (uint64_t)c;
  } else {
    keys[i] = (uint64_t)c;
    lo_out[i] = (uint64_t)c;
    hi_out[i] = (uint64_t)(c >> 64);
  }
  idx[i] = (uint32_t)i;
}

__global__ void gather_u64_kernel(const uint32_t* __restrict__ perm, const uint64_t* __restrict__ src, int64_t n,
                                  uint64_t* __restrict__ out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) out[s] = src[perm[s]];
}

__global__ void compose_wide_kernel(const uint32_t* __restrict__ perm, const uint64_t* __restrict__ lo,
                                    const uint64_t* __restrict__ hi, int64_t n, u128* __restrict__ out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) {
    const uint32_t p = perm[s];
    out[s] = ((u128)hi[p] << 64) | (u128)lo[p];
  }
}

// ---------------------------------------------------------------------------
// FP64 prefix sums of the Z-ordered points (for internal centres of mass).
// ---------------------------------------------------------------------------
constexpr int kPsThreads = 256;
constexpr int kPsItems = 8;
constexpr int kPsTile = kPsThreads * kPsItems;
static_assert(kPsTile == kBhPrefixTile, "bh_sizes sizes the prefix-sum partials by this tile");

template <class T, int D>
__global__ void prefix_reduce_kernel(const T* __restrict__ y, const uint32_t* __restrict__ perm, int64_t n,
                                     double* __restrict__ part) {
  __shared__ double sh[D][kPsThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kPsTile;
  double s[D];
#pragma unroll
  for (int a = 0; a < D; ++a) s[a] = 0.0;
  for (int i = 0; i < kPsItems; ++i) {
    const int64_t p = base + (int64_t)i * kPsThreads + threadIdx.x;
    if (p < n) {
      const int64_t src = perm[p];
#pragma unroll
      for (int a = 0; a < D; ++a) s[a] += (double)y[src * D + a];
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    double v = warp_sum(s[a]);
    if (lane == 0) sh[a][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < D) {
    double t = 0.0;
    for (int q = 0; q < kPsThreads / 32; ++q) t += sh[threadIdx.x][q];
    part[blockIdx.x * D + threadIdx.x] = t;
  }
}

// Exclusive scan of the per-tile partials (one block, chunks of blockDim
// carried in order; deterministic).
template <int D>
__global__ void prefix_partials_kernel(double* __restrict__ part, int64_t nparts) {
  __shared__ double wsum[D][32];
  __shared__ double carry[D], ctot[D];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x < D) carry[threadIdx.x] = 0.0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < nparts; c0 += blockDim.x) {
    const int64_t b = c0 + threadIdx.x;
    double v[D], x[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      v[a] = b < nparts ? part[b * D + a] : 0.0;
      x[a] = v[a];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(kFull, x[a], o);
        if (lane >= o) x[a] += y;
      }
      if (lane == 31) wsum[a][w] = x[a];
    }
    __syncthreads();
    if (threadIdx.x < D) {
      double run = 0.0;
      const int nw = blockDim.x >> 5;
      for (int q = 0; q < nw; ++q) {
        const double t = wsum[threadIdx.x][q];
        wsum[threadIdx.x][q] = run;
        run += t;
      }
      ctot[threadIdx.x] = run;
    }
    __syncthreads();
    if (b < nparts) {
#pragma unroll
      for (int a = 0; a < D; ++a) part[b * D + a] = carry[a] + wsum[a][w] + (x[a] - v[a]);
    }
    __syncthreads();
    if (threadIdx.x < D) carry[threadIdx.x] += ctot[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x < D) part[nparts * D + threadIdx.x] = carry[threadIdx.x];
}

// Writes the Z-ordered points (T) and their exclusive FP64 prefix sums S[0..n].
template <class T, int D>
__global__ void prefix_apply_kernel(const T* __restrict__ y, const uint32_t* __restrict__ perm, int64_t n,
                                    const double* __restrict__ part, int64_t nparts, T* __restrict__ ys,
                                    double* __restrict__ pre) {
  __shared__ double sh[D][kPsThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kPsTile + (int64_t)threadIdx.x * kPsItems;
  double v[kPsItems][D];
  double s[D];
#pragma unroll
  for (int a = 0; a < D; ++a) s[a] = 0.0;
#pragma unroll
  for (int i = 0; i < kPsItems; ++i) {
    const int64_t p = base + i;
    if (p < n) {
      const int64_t src = perm[p];
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const T t = y[src * D + a];
        ys[p * D + a] = t;
        v[i][a] = (double)t;
        s[a] += v[i][a];
      }
    } else {
#pragma unroll
      for (int a = 0; a < D; ++a) v[i][a] = 0.0;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    x[a] = s[a];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(kFull, x[a], o);
      if (lane >= o) x[a] += t;
    }
    if (lane == 31) sh[a][w] = x[a];
  }
  __syncthreads();
  if (threadIdx.x < D) {
    double run = 0.0;
    for (int q = 0; q < kPsThreads / 32; ++q) {
      const double t = sh[threadIdx.x][q];
      sh[threadIdx.x][q] = run;
      run += t;
    }
  }
  __syncthreads();
  double run[D];
#pragma unroll
  for (int a = 0; a < D; ++a) run[a] = x[a] - s[a] + sh[a][w] + part[blockIdx.x * D + a];
#pragma unroll
  for (int i = 0; i < kPsItems; ++i) {
    const int64_t p = base + i;
    if (p < n) {
#pragma unroll
      for (int a = 0; a < D; ++a) {
        pre[p * D + a] = run[a];
        run[a] += v[i][a];
      }
    }
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
#pragma unroll
    for (int a = 0; a < D; ++a) pre[n * D + a] = part[nparts * D + a];
  }
}

// Job-relative prefix sums for a batch of independent sets: every tile
// starts at its set's first position and a set's carry starts at zero, so the
// sums (and the centres of mass taken from them) are those of the set alone.
// pre holds n_j + 1 entries per set j: position p of set j is entry p + j.
template <class T, int D>
__global__ void seg_prefix_reduce_kernel(const T* __restrict__ y, const uint32_t* __restrict__ perm,
                                         const int64_t* __restrict__ tile_start, const int64_t* __restrict__ tile_end,
                                         double* __restrict__ part) {
  __shared__ double sh[D][kPsThreads / 32];
  const int64_t base = tile_start[blockIdx.x], lim = tile_end[blockIdx.x];
  double s[D];
#pragma unroll
  for (int a = 0; a < D; ++a) s[a] = 0.0;
  for (int i = 0; i < kPsItems; ++i) {
    const int64_t p = base + (int64_t)i * kPsThreads + threadIdx.x;
    if (p < lim) {
      const int64_t src = perm[p];
#pragma unroll
      for (int a = 0; a < D; ++a) s[a] += (double)y[src * D + a];
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    double v = warp_sum(s[a]);
    if (lane == 0) sh[a][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < D) {
    double t = 0.0;
    for (int q = 0; q < kPsThreads / 32; ++q) t += sh[threadIdx.x][q];
    part[blockIdx.x * D + threadIdx.x] = t;
  }
}

// One thread per set: exclusive scan of its tile sums; set totals to tot.
template <int D>
__global__ void seg_prefix_partials_kernel(double* __restrict__ part, const int32_t* __restrict__ job_tile, int K,
                                           double* __restrict__ tot) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K) return;
  double carry[D];
#pragma unroll
  for (int a = 0; a < D; ++a) carry[a] = 0.0;
  for (int b = job_tile[j]; b < job_tile[j + 1]; ++b) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const double v = part[b * D + a];
      part[b * D + a] = carry[a];
      carry[a] += v;
    }
  }
#pragma unroll
  for (int a = 0; a < D; ++a) tot[j * D + a] = carry[a];
}

template <class T, int D>
__global__ void seg_prefix_apply_kernel(const T* __restrict__ y, const uint32_t* __restrict__ perm,
                                        const int64_t* __restrict__ tile_start, const int64_t* __restrict__ tile_end,
                                        const int32_t* __restrict__ tile_job, const int32_t* __restrict__ job_tile,
                                        const double* __restrict__ part, const double* __restrict__ tot,
                                        T* __restrict__ ys, double* __restrict__ pre) {
  __shared__ double sh[D][kPsThreads / 32];
  const int64_t lim = tile_end[blockIdx.x];
  const int64_t base = tile_start[blockIdx.x] + (int64_t)threadIdx.x * kPsItems;
  const int64_t jj = tile_job[blockIdx.x];
  double v[kPsItems][D];
  double s[D];
#pragma unroll
  for (int a = 0; a < D; ++a) s[a] = 0.0;
#pragma unroll
  for (int i = 0; i < kPsItems; ++i) {
    const int64_t p = base + i;
    if (p < lim) {
      const int64_t src = perm[p];
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const T t = y[src * D + a];
        ys[p * D + a] = t;
        v[i][a] = (double)t;
        s[a] += v[i][a];
      }
    } else {
#pragma unroll
      for (int a = 0; a < D; ++a) v[i][a] = 0.0;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double x[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    x[a] = s[a];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(kFull, x[a], o);
      if (lane >= o) x[a] += t;
    }
    if (lane == 31) sh[a][w] = x[a];
  }
  __syncthreads();
  if (threadIdx.x < D) {
    double run = 0.0;
    for (int q = 0; q < kPsThreads / 32; ++q) {
      const double t = sh[threadIdx.x][q];
      sh[threadIdx.x][q] = run;
      run += t;
    }
  }
  __syncthreads();
  double run[D];
#pragma unroll
  for (int a = 0; a < D; ++a) run[a] = x[a] - s[a] + sh[a][w] + part[blockIdx.x * D + a];
#pragma unroll
  for (int i = 0; i < kPsItems; ++i) {
    const int64_t p = base + i;
    if (p < lim) {
#pragma unroll
      for (int a = 0; a < D; ++a) {
        pre[(p + jj) * D + a] = run[a];
        run[a] += v[i][a];
      }
    }
  }
  if (threadIdx.x == 0 && (int64_t)blockIdx.x == (int64_t)job_tile[jj + 1] - 1) {
#pragma unroll
    for (int a = 0; a < D; ++a) pre[(lim + jj) * D + a] = tot[jj * D + a];
  }
}

// ---------------------------------------------------------------------------
// Tree build.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void seg_bounds(const Segs& sg, int64_t s, int64_t n, int64_t* lo, int64_t* hi) {
  if (sg.job) {
    const uint64_t j = sg.job[s];
    *lo = sg.off[j];
    *hi = sg.off[j + 1];
  } else {
    *lo = 0;
    *hi = n;
  }
}

__device__ __forceinline__ bool same_set(const Segs& sg, int64_t a, int64_t b) {
  return !sg.job || sg.job[a] == sg.job[b];
}

template <int D>
__global__ void tree_mark_kernel(const typename MortonD<D>::Code* __restrict__ codes, int64_t n,
                                 uint32_t* __restrict__ mask, Segs sg) {
  typedef typename MortonD<D>::Code Code;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s <= 0 || s >= n) return;
  if (!same_set(sg, s - 1, s)) return;
  const Code c0 = codes[s - 1], c1 = codes[s];
  if (c0 == c1) return;
  constexpr int B = MortonD<D>::BITS;
  const int l = boundary_level<D>(c0, c1);
  int64_t lo, hi, a, e;
  seg_bounds(sg, s, n, &lo, &hi);
  cell_range_near<D>(codes, lo, hi, c1, l, s, &a, &e, false);
  const int sh1 = D * (B - l - 1);
  if ((c0 >> sh1) == (codes[a] >> sh1)) atomicOr(&mask[a], 1u << l);
}

template <class Code>
__global__ void tree_count_kernel(const Code* __restrict__ codes, int64_t n, const uint32_t* __restrict__ mask,
                                  uint32_t* __restrict__ cnt, Segs sg) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const bool run_start = s == 0 || !same_set(sg, s - 1, s) || codes[s - 1] != codes[s];
  cnt[s] = (uint32_t)__popc(mask[s]) + (run_start ? 1u : 0u);
}

template <class T, int D>
__global__ void tree_emit_kernel(const typename MortonD<D>::Code* __restrict__ codes, int64_t n,
                                 const uint32_t* __restrict__ mask, const uint64_t* __restrict__ base,
                                 const T* __restrict__ ys, const double* __restrict__ pre, TreeNodes<T, D> nodes,
                                 Segs sg) {
  typedef typename MortonD<D>::Code Code;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  constexpr int B = MortonD<D>::BITS;
  const Code c1 = codes[s];
  const bool set_start = s == 0 || !same_set(sg, s - 1, s);
  const bool run_start = set_start || codes[s - 1] != c1;
  int64_t lo, hi;
  seg_bounds(sg, s, n, &lo, &hi);
  if (!set_start && run_start) {
    const Code c0 = codes[s - 1];
    const int l = boundary_level<D>(c0, c1);
    int64_t a, e;
    cell_range_near<D>(codes, lo, hi, c1, l, s, &a, &e, true);
    const int sh1 = D * (B - l - 1);
    if ((c0 >> sh1) == (codes[a] >> sh1)) {
      const uint32_t m = mask[a];
      const int64_t idx = (int64_t)base[a] + __popc(m & ((1u << l) - 1u));
      if (idx >= 2 * n) return;  // cannot happen for a well-formed build; never write out of bounds
      const double cnt = (double)(e - a);
      const int64_t jj = sg.tile_job ? (int64_t)sg.job[s] : 0;  // job-relative prefix layout
      T com[D];
#pragma unroll
      for (int q = 0; q < D; ++q) com[q] = (T)((pre[(e + jj) * D + q] - pre[(a + jj) * D + q]) / cnt);
      nodes.write(idx, com, (T)(uint32_t)(e - a), l, (uint32_t)base[e]);
    }
  }
  if (run_start) {
    int64_t e = s + 1;
    if (e < hi && codes[e] == c1) {
      // duplicate codes: find the run end within the set
      int64_t a = e, b = hi;
      while (a < b) {
        const int64_t mid = (a + b) >> 1;
        if (codes[mid] <= c1) a = mid + 1;
        else b = mid;
      }
      e = a;
    }
    const uint32_t m = mask[s];
    const int64_t idx = (int64_t)base[s] + __popc(m);
    if (idx >= 2 * n) return;
    const uint32_t count = (uint32_t)(e - s);
    T com[D];
    if (count == 1) {
#pragma unroll
      for (int q = 0; q < D; ++q) com[q] = ys[s * D + q];
    } else {
      T acc[D];
#pragma unroll
      for (int q = 0; q < D; ++q) acc[q] = T(0);
      for (int64_t p = s; p < e; ++p) {
#pragma unroll
        for (int q = 0; q < D; ++q) acc[q] += ys[p * D + q];
      }
      const T inv = T(1) / (T)count;
#pragma unroll
      for (int q = 0; q < D; ++q) com[q] = acc[q] * inv;
    }
    nodes.write(idx, com, (T)count, -1, (uint32_t)base[e]);
  }
}

// ---------------------------------------------------------------------------
// Traversal: one thread per query point, queries taken in Z-order so that a
// warp walks neighbouring paths. Writes the repulsive force and per-point q,
// and reduces Z = sum q in FP64 (deterministic: per-block partials reduced in
// block order by the last block).
// ---------------------------------------------------------------------------
template <class T, int D>
__global__ void __launch_bounds__(kTraverseMax) bh_traverse_kernel(const T* __restrict__ y, const uint32_t* __restrict__ perm,
                                                               int64_t n, TreeNodes<T, D> nodes, const uint64_t* __restrict__ n_nodes_p,
                                                               int64_t max_nodes, const BoxParams<T>* __restrict__ prm,
                                                               T theta_sq, T* __restrict__ neg, T* __restrict__ qout,
                                                               double* __restrict__ zpart, unsigned* __restrict__ done,
                                                               double* __restrict__ z_out, Segs sg,
                                                               const BoxParams<T>* __restrict__ boxes,
                                                               const uint64_t* __restrict__ base) {
  __shared__ double sh[32];
  __shared__ bool last;
  __shared__ T hw2s[40];
  if (!sg.job && threadIdx.x < 40) hw2s[threadIdx.x] = prm->hw2[threadIdx.x];
  __syncthreads();
  nodes.hw2 = hw2s;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double qd = 0.0;
  if (t < n) {
    const int64_t pi = perm[t];
    T qv[D];
#pragma unroll
    for (int a = 0; a < D; ++a) qv[a] = y[pi * D + a];
    const uint64_t m_raw = *n_nodes_p;
    uint32_t M = (uint32_t)(m_raw < (uint64_t)max_nodes ? m_raw : (uint64_t)max_nodes);
    uint32_t root = 0;
    if (sg.job) {
      // this query's own tree: nodes [base[off[j]], base[off[j+1]])
      const uint64_t j = sg.job[t];
      root = (uint32_t)base[sg.off[j]];
      const uint32_t end = (uint32_t)base[sg.off[j + 1]];
      M = end < M ? end : M;
      nodes.hw2 = boxes[j].hw2;
    }
    T f[D];
#pragma unroll
    for (int a = 0; a < D; ++a) f[a] = T(0);
    T q = T(0);
    // 2-D single precision: the displacement and its squares in paired
    // f32x2 instructions (each half the scalar operation, so the same values
    // as the per-axis code). The force update stays scalar: a paired multiply
    // feeding a paired add was measured to round as one fused multiply-add
    // despite the .rn modifiers, which the reference's f += m * d never does.
    constexpr bool kPair = D == 2 && std::is_same<T, float>::value;
    F32x2 q2 = {0ull};
    if constexpr (kPair) q2 = f2_make((float)qv[0], (float)qv[D - 1]);
    // Software-pipelined walk: both possible successors of the current node
    // (i + 1 if it is opened, its skip target if it is summarised) are loaded
    // before the decision, so the next visit never waits on a dependent load.
    uint32_t i = root;
    typename TreeNodes<T, D>::Raw cur = nodes.load(root < M ? root : 0);
    while (i < M) {
      const uint32_t w = nodes.word(cur);
      const bool leaf = w == kLeafWord;
      const uint32_t sk_raw = leaf ? i + 1 : (w >> 5);
      // skip > i by construction; max() keeps the walk finite regardless.
      const uint32_t sk = sk_raw > i ? sk_raw : i + 1;
      // i + 1 <= M and the node array holds M + 1 entries (a spare past the
      // last node), so neither load needs a clamp beyond sk <= M
      const typename TreeNodes<T, D>::Raw nxt_open = nodes.load(i + 1);
      const typename TreeNodes<T, D>::Raw nxt_skip = leaf ? nxt_open : nodes.load(sk < M ? sk : M);
      T com[D], mass, r2;
      nodes.decode(cur, com, &mass, &r2);
      T disp[D];
      T dist = T(0);
      F32x2 d2 = {0ull};
      if constexpr (kPair) {
        d2 = f2_sub(q2, f2_make((float)com[0], (float)com[D - 1]));
        const F32x2 s2 = f2_mul(d2, d2);
        dist = (T)(f2_lo(s2) + f2_hi(s2));  // (0 + dx^2) + dy^2, as the per-axis sum
      } else {
#pragma unroll
        for (int a = 0; a < D; ++a) {
          disp[a] = qv[a] - com[a];
          dist += disp[a] * disp[a];
        }
      }
      if (r2 >= theta_sq * dist) {
        i = i + 1;
        cur = nxt_open;
        continue;
      }
      i = sk;
      cur = nxt_skip;
      if (r2 < T(0) && dist == T(0)) continue;
      const T inv = rcp_rn(T(1) + dist);
      T m = mass * inv;
      q += m;
      m = m * inv;
      if constexpr (kPair) {
        f[0] += m * (T)f2_lo(d2);
        f[D - 1] += m * (T)f2_hi(d2);
      } else {
#pragma unroll
        for (int a = 0; a < D; ++a) f[a] += m * disp[a];
      }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) neg[pi * D + a] = f[a];
    if (qout) qout[pi] = q;
    qd = (double)q;
  }
  const double bs = block_sum(qd, sh);
  if (threadIdx.x == 0) {
    zpart[blockIdx.x] = bs;
    __threadfence();
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    const double z = block_sum_parts(zpart, gridDim.x, 1, 0, sh);
    if (threadIdx.x == 0) {
      *z_out = z;
      *done = 0;
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host orchestration.
// ---------------------------------------------------------------------------
template <class T>
void launch_recenter_bbox(int D, T* y, int64_t n, const double* mean_sum, bool apply_mean, BhWorkspace<T>& ws,
                          int bits, cudaStream_t s) {
  const int grid =
      (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kThreads), sm_grid(2, (int)kBhBoxBlocksMax)));
  ws.zero_counters(s);
  T* pmin = ws.part_min.template as<T>();
  T* pmax = ws.part_max.template as<T>();
  with_dim<1, 7>(D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    recenter_bbox_kernel<T, DD><<<grid, kThreads, 0, s>>>(y, n, mean_sum, apply_mean ? 1 : 0, pmin, pmax,
                                                          ws.done.template as<unsigned>(),
                                                          ws.params.template as<BoxParams<T>>(), bits);
  });
  BHG_LAUNCH_CHECK();
}

template <class T>
void BhWorkspace<T>::reserve(int64_t n_, int D_) {
  n = n_;
  D = D_;
  const BhSizes z = bh_sizes<T>(n, D);
  keys.ensure(z.keys);
  keys_alt.ensure(z.keys);
  perm.ensure(z.perm);
  perm_alt.ensure(z.perm);
  ys.ensure(z.ys);
  pre.ensure(z.pre);
  pre_part.ensure(z.pre_part);
  mask.ensure(z.mask);
  cnt.ensure(z.cnt);
  base.ensure(z.base);
  geom.ensure(z.geom);
  if (z.word) word.ensure(z.word);
  if (z.wide) {
    wide.ensure(z.wide);
    lo_orig.ensure(z.wide / 2);
    hi_orig.ensure(z.wide / 2);
  }
  part_min.ensure(z.part);
  part_max.ensure(z.part);
  done.ensure(z.small);
  zdone.ensure(z.small);
  params.ensure(z.params);
  zpart.ensure(z.zpart);
  zval.ensure(z.zval);
}

template <class T, int D>
static TreeNodes<T, D> nodes_of(BhWorkspace<T>& ws) {
  TreeNodes<T, D> t;
  t.hw2 = nullptr;
  if constexpr (D == 2) {
    t.geom = ws.geom.template as<Node2<T>>();
  } else if constexpr (D == 3) {
    t.geom = ws.geom.template as<Quad<T>>();
    t.words = ws.word.template as<uint32_t>();
  } else {
    t.geom = ws.geom.template as<Oct<T>>();
    t.words = ws.word.template as<uint32_t>();
  }
  return t;
}

// Sorted codes as the tree kernels read them.
template <class T, int D>
static const typename MortonD<D>::Code* sorted_codes(BhWorkspace<T>& ws) {
  return static_cast<const typename MortonD<D>::Code*>(D >= 5 ? ws.wide.ptr : ws.keys.ptr);
}

template <class T, int D>
static void build_from_sorted_impl(BhWorkspace<T>& ws, const T* y, int64_t n, const Segs& sg, cudaStream_t s);

template <class T, int D>
static void bh_build_impl(BhWorkspace<T>& ws, const T* y, int64_t n, cudaStream_t s) {
  constexpr int B = MortonD<D>::BITS;
  const unsigned g = (unsigned)ceil_div(n, kThreads);
  uint64_t* lo = D >= 5 ? ws.lo_orig.template as<uint64_t>() : nullptr;
  uint64_t* hi = D >= 5 ? ws.hi_orig.template as<uint64_t>() : nullptr;
  morton_kernel<T, D><<<g, kThreads, 0, s>>>(y, n, ws.params.template as<BoxParams<T>>(), ws.keys.template as<uint64_t>(),
                                             ws.perm.template as<uint32_t>(), lo, hi);
  BHG_LAUNCH_CHECK();
  if constexpr (D * B <= 64) {
    radix_sort_pairs<uint32_t>(ws.keys.template as<uint64_t>(), ws.perm.template as<uint32_t>(),
                               ws.keys_alt.template as<uint64_t>(), ws.perm_alt.template as<uint32_t>(), n, 0, D * B,
                               ws.sort_tmp, s);
  } else {
    // 128-bit codes: stable LSD sort on the low word, then on the high word
    radix_sort_pairs<uint32_t>(ws.keys.template as<uint64_t>(), ws.perm.template as<uint32_t>(),
                               ws.keys_alt.template as<uint64_t>(), ws.perm_alt.template as<uint32_t>(), n, 0, 64,
                               ws.sort_tmp, s);
    gather_u64_kernel<<<g, kThreads, 0, s>>>(ws.perm.template as<uint32_t>(), hi, n, ws.keys.template as<uint64_t>());
    BHG_LAUNCH_CHECK();
    radix_sort_pairs<uint32_t>(ws.keys.template as<uint64_t>(), ws.perm.template as<uint32_t>(),
                               ws.keys_alt.template as<uint64_t>(), ws.perm_alt.template as<uint32_t>(), n, 0,
                               D * B - 64, ws.sort_tmp, s);
    compose_wide_kernel<<<g, kThreads, 0, s>>>(ws.perm.template as<uint32_t>(), lo, hi, n,
                                               ws.wide.template as<u128>());
    BHG_LAUNCH_CHECK();
  }
  build_from_sorted_impl<T, D>(ws, y, n, Segs(), s);
}

template <class T, int D>
static void build_from_sorted_impl(BhWorkspace<T>& ws, const T* y, int64_t n, const Segs& sg, cudaStream_t s) {
  const unsigned g = (unsigned)ceil_div(n, kThreads);
  if (sg.tile_job) {
    const int64_t nt = sg.ntiles;
    double* part = static_cast<double*>(ws.pre_part.ensure((size_t)(nt + 1) * D * sizeof(double)));
    double* tot = static_cast<double*>(ws.seg_tot.ensure((size_t)std::max(sg.K, 1) * D * sizeof(double)));
    double* pre = static_cast<double*>(ws.pre.ensure((size_t)(n + sg.K) * D * sizeof(double)));
    seg_prefix_reduce_kernel<T, D><<<(unsigned)nt, kPsThreads, 0, s>>>(y, ws.perm.template as<uint32_t>(),
                                                                        sg.tile_start, sg.tile_end, part);
    BHG_LAUNCH_CHECK();
    seg_prefix_partials_kernel<D><<<(unsigned)ceil_div(sg.K, 128), 128, 0, s>>>(part, sg.job_tile, sg.K, tot);
    BHG_LAUNCH_CHECK();
    seg_prefix_apply_kernel<T, D><<<(unsigned)nt, kPsThreads, 0, s>>>(
        y, ws.perm.template as<uint32_t>(), sg.tile_start, sg.tile_end, sg.tile_job, sg.job_tile, part, tot,
        ws.ys.template as<T>(), pre);
    BHG_LAUNCH_CHECK();
  } else {
    const int64_t np = ceil_div(n, kPsTile);
    prefix_reduce_kernel<T, D><<<(unsigned)np, kPsThreads, 0, s>>>(y, ws.perm.template as<uint32_t>(), n,
                                                                    ws.pre_part.template as<double>());
    BHG_LAUNCH_CHECK();
    prefix_partials_kernel<D><<<1, 1024, 0, s>>>(ws.pre_part.template as<double>(), np);
    BHG_LAUNCH_CHECK();
    prefix_apply_kernel<T, D><<<(unsigned)np, kPsThreads, 0, s>>>(y, ws.perm.template as<uint32_t>(), n,
                                                                   ws.pre_part.template as<double>(), np,
                                                                   ws.ys.template as<T>(), ws.pre.template as<double>());
    BHG_LAUNCH_CHECK();
  }
  BHG_CUDA(cudaMemsetAsync(ws.mask.ptr, 0, (size_t)n * 4, s));
  const typename MortonD<D>::Code* codes = sorted_codes<T, D>(ws);
  tree_mark_kernel<D><<<g, kThreads, 0, s>>>(codes, n, ws.mask.template as<uint32_t>(), sg);
  BHG_LAUNCH_CHECK();
  tree_count_kernel<<<g, kThreads, 0, s>>>(codes, n, ws.mask.template as<uint32_t>(), ws.cnt.template as<uint32_t>(), sg);
  BHG_LAUNCH_CHECK();
  scan_u32_to_u64(ws.cnt.template as<uint32_t>(), ws.base.template as<uint64_t>(), n, ws.scan_tmp, s);
  tree_emit_kernel<T, D><<<g, kThreads, 0, s>>>(codes, n, ws.mask.template as<uint32_t>(),
                                                ws.base.template as<uint64_t>(), ws.ys.template as<T>(),
                                                ws.pre.template as<double>(), nodes_of<T, D>(ws), sg);
  BHG_LAUNCH_CHECK();
}

template <class T>
void bh_build(BhWorkspace<T>& ws, int D, const T* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  if (n > kMaxTreePoints) throw Error(ST_EINVAL, "error: the GPU Barnes-Hut arena holds at most 2^26 - 1 points.");
  with_dim<2, 7>(D, "error: Barnes-Hut covers D in 2..7.", [&](auto dc) {
    bh_build_impl<T, decltype(dc)::value>(ws, y, n, s);
  });
}

template <class T>
void bh_build_from_sorted(BhWorkspace<T>& ws, int D, const T* y, int64_t n, const Segs& segs, cudaStream_t s) {
  if (n <= 0) return;
  if (n > kMaxTreePoints) throw Error(ST_EINVAL, "error: the GPU Barnes-Hut arena holds at most 2^26 - 1 points.");
  if (D == 2) build_from_sorted_impl<T, 2>(ws, y, n, segs, s);
  else if (D == 3) build_from_sorted_impl<T, 3>(ws, y, n, segs, s);
  else throw Error(ST_EINVAL, "error: the batched Barnes-Hut path covers D in {2, 3}.");
}

template <class T>
void bh_traverse(BhWorkspace<T>& ws, int D, const T* y, int64_t n, T theta, T* neg, T* qout, cudaStream_t s,
                 const Segs& segs, const BoxParams<T>* boxes) {
  if (n <= 0) {
    BHG_CUDA(cudaMemsetAsync(ws.zval.ptr, 0, sizeof(double), s));
    return;
  }
  ws.zero_counters(s);
  const int bt = ws.traverse_threads == 128 || ws.traverse_threads == 512 ? ws.traverse_threads : 256;
  const unsigned g = (unsigned)ceil_div(n, bt);
  const T theta_sq = theta * theta;
  const uint64_t* M = ws.base.template as<uint64_t>() + n;
  with_dim<2, 7>(D, "error: Barnes-Hut covers D in 2..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    bh_traverse_kernel<T, DD><<<g, bt, 0, s>>>(
        y, ws.perm.template as<uint32_t>(), n, nodes_of<T, DD>(ws), M, 2 * n, ws.params.template as<BoxParams<T>>(),
        theta_sq, neg, qout, ws.zpart.template as<double>(), ws.zdone.template as<unsigned>(),
        ws.zval.template as<double>(), segs, boxes, ws.base.template as<uint64_t>());
  });
  BHG_LAUNCH_CHECK();
}

template <class T>
int bh_bits(int D) {
  int b = 0;
  with_dim<2, 7>(D, "error: Barnes-Hut covers D in 2..7.", [&](auto dc) { b = MortonD<decltype(dc)::value>::BITS; });
  return b;
}

void SegTiles::build(const std::vector<int64_t>& off, cudaStream_t s) {
  K = (int)off.size() - 1;
  std::vector<int64_t> st, en;
  std::vector<int32_t> tj, jt(K + 1, 0);
  for (int j = 0; j < K; ++j) {
    jt[j] = (int32_t)st.size();
    for (int64_t p = off[j]; p < off[j + 1]; p += kPsTile) {
      st.push_back(p);
      en.push_back(std::min<int64_t>(p + kPsTile, off[j + 1]));
      tj.push_back(j);
    }
  }
  jt[K] = (int32_t)st.size();
  ntiles = (int64_t)st.size();
  const size_t a = ((size_t)ntiles * 8 + 255) / 256 * 256;
  const size_t b = ((size_t)ntiles * 4 + 255) / 256 * 256;
  char* base = static_cast<char*>(buf.ensure(2 * a + b + (size_t)(K + 1) * 4 + 256));
  BHG_CUDA(cudaMemcpyAsync(base, st.data(), (size_t)ntiles * 8, cudaMemcpyHostToDevice, s));
  BHG_CUDA(cudaMemcpyAsync(base + a, en.data(), (size_t)ntiles * 8, cudaMemcpyHostToDevice, s));
  BHG_CUDA(cudaMemcpyAsync(base + 2 * a, tj.data(), (size_t)ntiles * 4, cudaMemcpyHostToDevice, s));
  BHG_CUDA(cudaMemcpyAsync(base + 2 * a + b, jt.data(), (size_t)(K + 1) * 4, cudaMemcpyHostToDevice, s));
  BHG_CUDA(cudaStreamSynchronize(s));
}

void SegTiles::fill(Segs& sg) const {
  const size_t a = ((size_t)ntiles * 8 + 255) / 256 * 256;
  const size_t b = ((size_t)ntiles * 4 + 255) / 256 * 256;
  char* base = static_cast<char*>(buf.ptr);
  sg.tile_start = reinterpret_cast<const int64_t*>(base);
  sg.tile_end = reinterpret_cast<const int64_t*>(base + a);
  sg.tile_job = reinterpret_cast<const int32_t*>(base + 2 * a);
  sg.job_tile = reinterpret_cast<const int32_t*>(base + 2 * a + b);
  sg.ntiles = ntiles;
  sg.K = K;
}

// The last-block counters start at zero once; every kernel that uses one
// leaves it at zero. Zeroed on the caller's stream (a plain cudaMemset runs on
// the legacy stream, which does not order against non-blocking streams).
template <class T>
void BhWorkspace<T>::zero_counters(cudaStream_t s) {
  if (zeroed) return;
  BHG_CUDA(cudaMemsetAsync(done.ptr, 0, 64, s));
  BHG_CUDA(cudaMemsetAsync(zdone.ptr, 0, 64, s));
  zeroed = true;
}

template struct BhWorkspace<float>;
template struct BhWorkspace<double>;
template void launch_recenter_bbox<float>(int, float*, int64_t, const double*, bool, BhWorkspace<float>&, int, cudaStream_t);
template void launch_recenter_bbox<double>(int, double*, int64_t, const double*, bool, BhWorkspace<double>&, int,
                                           cudaStream_t);
template void bh_build<float>(BhWorkspace<float>&, int, const float*, int64_t, cudaStream_t);
template void bh_build<double>(BhWorkspace<double>&, int, const double*, int64_t, cudaStream_t);
template void bh_traverse<float>(BhWorkspace<float>&, int, const float*, int64_t, float, float*, float*, cudaStream_t,
                                 const Segs&, const BoxParams<float>*);
template void bh_traverse<double>(BhWorkspace<double>&, int, const double*, int64_t, double, double*, double*,
                                  cudaStream_t, const Segs&, const BoxParams<double>*);
template void bh_build_from_sorted<float>(BhWorkspace<float>&, int, const float*, int64_t, const Segs&, cudaStream_t);
template void bh_build_from_sorted<double>(BhWorkspace<double>&, int, const double*, int64_t, const Segs&, cudaStream_t);
template int bh_bits<float>(int);
template int bh_bits<double>(int);

}  // namespace bhg
