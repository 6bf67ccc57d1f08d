// bhtsne oracle: a CPU restatement of the bhtsne 0.7.10 fitting path.
//
// TEST INFRASTRUCTURE ONLY. This file is the correctness checker for the CUDA
// library and the timed CPU baseline ("port") of bench.py. It is never linked
// into, loaded by, or called from the product library (bhtsne_gb300/), and the
// product path never falls back to it.
//
// Each routine restates one function of the Rust reference, cited as
// path:line within the reference crate. Arithmetic is kept in the reference's
// own order and precision (T = f32 or f64, sequential sums where the reference
// sums sequentially, no fused multiply-add: build with -ffp-contract=off) so
// that single-threaded results reproduce the reference's operation sequence.
// Parallel loops (OpenMP) only split independent per-row work; every
// reduction is sequential, so results do not depend on the thread count.
//
// Deviations, each deliberate:
//  * kNN is exact brute force ordered by (distance, index) instead of the
//    randomised VP-tree (src/tsne/vptree.rs:101-319); the reference's own
//    tests (src/test.rs:866-928) establish that the two give the same lists.
//  * The FFT is this file's own mixed-radix complex transform in place of
//    rustfft/realfft (src/tsne/fft.rs); a linear convolution is independent
//    of the transform used, up to rounding.
//  * The unstable Morton sort (src/tsne/arena.rs:191) is made deterministic by
//    ordering equal codes by point index, one of the orders it may produce.
//  * random_init (src/tsne/mod.rs:142-147) is unseeded in the reference; here
//    it is a seeded Box-Muller N(0, 1e-4) so runs repeat.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

template <class T>
struct Num {
  static T max() { return std::numeric_limits<T>::max(); }
  // Rust `Float::min_positive_value()`: the smallest positive normal.
  static T min_pos() { return std::numeric_limits<T>::min(); }
  static T eps() { return std::numeric_limits<T>::epsilon(); }
};

// Rust `signum`: +1 for +0.0 and positives, -1 for -0.0 and negatives, NaN for NaN.
template <class T>
static inline T signum(T x) {
  if (std::isnan(x)) return x;
  return std::copysign(T(1), x);
}

// rayon's par_iter().sum() (src/tsne/mod.rs:288, :597-601, :603-617, :668,
// :774; src/tsne/interpolation.rs:309-328; src/lib.rs:589) splits the slice in
// halves across the thread pool and adds the halves' sums. Its split points
// follow the pool size and work stealing, so the reference's own result varies
// with the thread count; restated here as a balanced tree of halves with
// leaves of at most 256 values summed in order, in T: the accuracy of a
// parallel reduction (error growing with log n, not with n), independent of
// the thread count. Sums the reference forms sequentially stay sequential.
template <class T>
T tree_sum(const T* v, int64_t n) {
  if (n <= 256) {
    T s = T(0);
    for (int64_t i = 0; i < n; ++i) s = s + v[i];
    return s;
  }
  const int64_t h = n / 2;
  return tree_sum(v, h) + tree_sum(v + h, n - h);
}

// Rust `f32::min` / `f32::max` return the non-NaN operand.
template <class T>
static inline T fmin_(T a, T b) { return std::fmin(a, b); }
template <class T>
static inline T fmax_(T a, T b) { return std::fmax(a, b); }

// ---------------------------------------------------------------------------
// Perplexity check: src/tsne/mod.rs:55-59.
// `n_samples - 1 < 3 * perplexity.as_()` where as_() truncates toward zero.
// ---------------------------------------------------------------------------
template <class T>
bool perplexity_ok(T perplexity, int64_t n_samples) {
  // usize arithmetic in Rust: n_samples - 1 underflows (panics in debug) for 0.
  if (n_samples < 1) return false;
  int64_t as_usize = perplexity > T(0) ? (int64_t)perplexity : 0;
  return !((n_samples - 1) < 3 * as_usize);
}

// ---------------------------------------------------------------------------
// Brute-force kNN with the reference test metric (src/test.rs:856-862,
// src/test.rs:866-881): distance = sqrt(sum over dims, in order, of (a-b)^2),
// ordered by (distance, index), self excluded.
// ---------------------------------------------------------------------------
template <class T>
T euclidean(const T* a, const T* b, int32_t dim) {
  T s = T(0);
  for (int32_t c = 0; c < dim; ++c) {
    T d = a[c] - b[c];
    s = s + d * d;
  }
  return std::sqrt(s);
}

template <class T>
void knn_brute(const T* X, int64_t n, int32_t dim, int32_t k, uint32_t* idx, T* dist) {
#pragma omp parallel
  {
    std::vector<std::pair<T, uint32_t>> row;
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i) {
      row.clear();
      for (int64_t j = 0; j < n; ++j) {
        if (j == i) continue;
        row.emplace_back(euclidean(X + i * dim, X + j * dim, dim), (uint32_t)j);
      }
      std::partial_sort(row.begin(), row.begin() + k, row.end(),
                        [](const std::pair<T, uint32_t>& a, const std::pair<T, uint32_t>& b) {
                          if (a.first < b.first) return true;
                          if (b.first < a.first) return false;
                          return a.second < b.second;
                        });
      for (int32_t c = 0; c < k; ++c) {
        idx[i * k + c] = row[c].second;
        dist[i * k + c] = row[c].first;
      }
    }
  }
}

// The same neighbours for selected query rows only (a bounded max-heap by
// (distance, index) instead of a partial sort of the whole row): the k
// smallest pairs in that order, which is what knn_brute returns for the row.
template <class T>
void knn_brute_rows(const T* X, int64_t n, int32_t dim, int32_t k, const int64_t* rows, int64_t nrows,
                    uint32_t* idx, T* dist) {
  auto less = [](const std::pair<T, uint32_t>& a, const std::pair<T, uint32_t>& b) {
    if (a.first < b.first) return true;
    if (b.first < a.first) return false;
    return a.second < b.second;
  };
#pragma omp parallel
  {
    std::vector<std::pair<T, uint32_t>> heap;
#pragma omp for schedule(dynamic, 4)
    for (int64_t r = 0; r < nrows; ++r) {
      const int64_t i = rows[r];
      heap.clear();
      for (int64_t j = 0; j < n; ++j) {
        if (j == i) continue;
        std::pair<T, uint32_t> c(euclidean(X + i * dim, X + j * dim, dim), (uint32_t)j);
        if ((int32_t)heap.size() < k) {
          heap.push_back(c);
          std::push_heap(heap.begin(), heap.end(), less);
        } else if (less(c, heap.front())) {
          std::pop_heap(heap.begin(), heap.end(), less);
          heap.back() = c;
          std::push_heap(heap.begin(), heap.end(), less);
        }
      }
      std::sort_heap(heap.begin(), heap.end(), less);
      for (int32_t c = 0; c < k; ++c) {
        idx[r * k + c] = heap[c].second;
        dist[r * k + c] = heap[c].first;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// search_beta: src/tsne/mod.rs:201-275.
// ---------------------------------------------------------------------------
template <class T>
int search_beta(T* p, const T* d, int64_t k, T perplexity) {
  bool found = false;
  T beta = T(1);
  T min_beta = -Num<T>::max();
  T max_beta = Num<T>::max();
  const T tolerance = T(1e-5);
  int iteration = 0;
  T sum = T(0);
  const T two = T(2);
  while (!found && iteration < 200) {
    for (int64_t j = 0; j < k; ++j) p[j] = std::exp(-beta * (d[j] * d[j]));
    T s = T(0);
    for (int64_t j = 0; j < k; ++j) s = s + p[j];
    sum = s + Num<T>::min_pos();
    T entropy = T(0);
    for (int64_t j = 0; j < k; ++j) entropy = entropy + beta * p[j] * (d[j] * d[j]);
    entropy = entropy / sum + std::log(sum);
    T diff = entropy - std::log(perplexity);
    if (diff < tolerance && -diff < tolerance) {
      found = true;
    } else {
      if (diff > T(0)) {
        min_beta = beta;
        if (max_beta == Num<T>::max() || max_beta == -Num<T>::max())
          beta *= two;
        else
          beta = (beta + max_beta) / two;
      } else {
        max_beta = beta;
        if (min_beta == -Num<T>::max() || min_beta == Num<T>::max())
          beta /= two;
        else
          beta = (beta + min_beta) / two;
      }
      if (std::isinf(beta) && beta > T(0)) beta = Num<T>::max();
      if (std::isinf(beta) && beta < T(0)) beta = -Num<T>::max();
    }
    iteration += 1;
  }
  for (int64_t j = 0; j < k; ++j) p[j] /= sum + Num<T>::eps();
  return iteration;
}

// ---------------------------------------------------------------------------
// normalize_p_values: src/tsne/mod.rs:284-293; stop_lying: src/tsne/mod.rs:525-531.
// ---------------------------------------------------------------------------
template <class T>
void normalize_p(T* p, int64_t nnz, T exaggeration) {
  const T s = tree_sum(p, nnz);
  T scale = exaggeration / (s + Num<T>::eps());
  for (int64_t e = 0; e < nnz; ++e) p[e] *= scale;
}

template <class T>
void stop_lying(T* p, int64_t nnz, T exaggeration) {
  T scale = T(1) / exaggeration;
  for (int64_t e = 0; e < nnz; ++e) p[e] *= scale;
}

// ---------------------------------------------------------------------------
// symmetrize_sparse_matrix: src/tsne/mod.rs:306-406. Rows of the kNN table are
// sorted by column, then the symmetric CSR is emitted by the sequential
// count-and-fill walk, which fixes the in-row entry order.
// ---------------------------------------------------------------------------
template <class T>
void symmetrize(std::vector<uint32_t> cols, std::vector<T> vals, int64_t n, int64_t k,
                std::vector<uint64_t>& rows_out, std::vector<uint32_t>& cols_out,
                std::vector<T>& vals_out) {
#pragma omp parallel
  {
    std::vector<std::pair<uint32_t, T>> row;
#pragma omp for
    for (int64_t r = 0; r < n; ++r) {
      row.clear();
      for (int64_t c = 0; c < k; ++c) row.emplace_back(cols[r * k + c], vals[r * k + c]);
      std::sort(row.begin(), row.end(),
                [](const std::pair<uint32_t, T>& a, const std::pair<uint32_t, T>& b) {
                  return a.first < b.first;
                });
      for (int64_t c = 0; c < k; ++c) {
        cols[r * k + c] = row[c].first;
        vals[r * k + c] = row[c].second;
      }
    }
  }
  auto find = [&](int64_t row, uint32_t target, int64_t* at) -> bool {
    const uint32_t* b = cols.data() + row * k;
    const uint32_t* e = b + k;
    const uint32_t* it = std::lower_bound(b, e, target);
    if (it != e && *it == target) {
      *at = it - b;
      return true;
    }
    return false;
  };
  std::vector<uint64_t> row_counts(n, 0);
  for (int64_t r = 0; r < n; ++r) {
    for (int64_t i = r * k; i < (r + 1) * k; ++i) {
      row_counts[r] += 1;
      int64_t at;
      if (!find(cols[i], (uint32_t)r, &at)) row_counts[cols[i]] += 1;
    }
  }
  rows_out.assign(n + 1, 0);
  for (int64_t r = 0; r < n; ++r) rows_out[r + 1] = rows_out[r] + row_counts[r];
  uint64_t total = rows_out[n];
  cols_out.assign(total, 0);
  vals_out.assign(total, T(0));
  std::vector<uint64_t> offset(n, 0);
  for (int64_t r = 0; r < n; ++r) {
    for (int64_t i = r * k; i < (r + 1) * k; ++i) {
      int64_t c = cols[i];
      int64_t m_off;
      bool present = find(c, (uint32_t)r, &m_off);
      if (present) {
        if (r <= c) {
          cols_out[rows_out[r] + offset[r]] = (uint32_t)c;
          cols_out[rows_out[c] + offset[c]] = (uint32_t)r;
          int64_t m = c * k + m_off;
          vals_out[rows_out[r] + offset[r]] = vals[i] + vals[m];
          vals_out[rows_out[c] + offset[c]] = vals[i] + vals[m];
        }
      } else {
        cols_out[rows_out[r] + offset[r]] = (uint32_t)c;
        cols_out[rows_out[c] + offset[c]] = (uint32_t)r;
        vals_out[rows_out[r] + offset[r]] = vals[i];
        vals_out[rows_out[c] + offset[c]] = vals[i];
      }
      if (!present || r <= c) {
        offset[r] += 1;
        if (c != r) offset[c] += 1;
      }
    }
  }
  const T half = T(0.5);
  for (auto& v : vals_out) v *= half;
}

// ---------------------------------------------------------------------------
// Morton codecs: src/tsne/morton/d2.rs:5-47, src/tsne/morton/d3.rs:5-50, and
// quantize: src/tsne/morton.rs:103-120.
// ---------------------------------------------------------------------------
static inline uint64_t part1by1(uint64_t x) {
  x &= 0x00000000ffffffffULL;
  x = (x | (x << 16)) & 0x0000ffff0000ffffULL;
  x = (x | (x << 8)) & 0x00ff00ff00ff00ffULL;
  x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0fULL;
  x = (x | (x << 2)) & 0x3333333333333333ULL;
  return (x | (x << 1)) & 0x5555555555555555ULL;
}
static inline uint64_t part1by2(uint64_t x) {
  x &= 0x1fffffULL;
  x = (x | (x << 32)) & 0x001f00000000ffffULL;
  x = (x | (x << 16)) & 0x001f0000ff0000ffULL;
  x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
  return (x | (x << 2)) & 0x1249249249249249ULL;
}

// Codecs of src/tsne/morton/d2.rs-d7.rs: bits per axis 32, 21, 16, 25, 21,
// 18 for D = 2..7; u64 words up to D = 4, u128 beyond. Bit b of axis a is
// code bit b * D + a.
typedef unsigned __int128 u128;

template <class C, int D, uint32_t B>
static C interleave(const uint32_t* c) {
  C code = 0;
  for (uint32_t b = 0; b < B; ++b)
    for (int a = 0; a < D; ++a) code |= (C)((c[a] >> b) & 1u) << (b * D + a);
  return code;
}

template <int D>
struct MortonSpec;
template <>
struct MortonSpec<2> {
  static constexpr uint32_t BITS = 32;
  typedef uint64_t Code;
  static uint64_t encode(const uint32_t* c) { return part1by1(c[0]) | (part1by1(c[1]) << 1); }
};
template <>
struct MortonSpec<3> {
  static constexpr uint32_t BITS = 21;
  typedef uint64_t Code;
  static uint64_t encode(const uint32_t* c) {
    return part1by2(c[0]) | (part1by2(c[1]) << 1) | (part1by2(c[2]) << 2);
  }
};
template <>
struct MortonSpec<4> {
  static constexpr uint32_t BITS = 16;
  typedef uint64_t Code;
  static Code encode(const uint32_t* c) { return interleave<Code, 4, 16>(c); }
};
template <>
struct MortonSpec<5> {
  static constexpr uint32_t BITS = 25;
  typedef u128 Code;
  static Code encode(const uint32_t* c) { return interleave<Code, 5, 25>(c); }
};
template <>
struct MortonSpec<6> {
  static constexpr uint32_t BITS = 21;
  typedef u128 Code;
  static Code encode(const uint32_t* c) { return interleave<Code, 6, 21>(c); }
};
template <>
struct MortonSpec<7> {
  static constexpr uint32_t BITS = 18;
  typedef u128 Code;
  static Code encode(const uint32_t* c) { return interleave<Code, 7, 18>(c); }
};

static inline uint32_t msb_position(uint64_t x) { return 63u - (uint32_t)__builtin_clzll(x); }
static inline uint32_t msb_position(u128 x) {
  const uint64_t hi = (uint64_t)(x >> 64);
  return hi ? 64u + msb_position(hi) : msb_position((uint64_t)x);
}

// Calls f(std::integral_constant<int, D>()) for D in [lo, hi]; false otherwise.
template <int lo, int hi, class F>
static bool with_d(int D, F&& f) {
  bool ok = true;
  switch (D) {
    case 1: if constexpr (lo <= 1 && 1 <= hi) f(std::integral_constant<int, 1>()); else ok = false; break;
    case 2: if constexpr (lo <= 2 && 2 <= hi) f(std::integral_constant<int, 2>()); else ok = false; break;
    case 3: if constexpr (lo <= 3 && 3 <= hi) f(std::integral_constant<int, 3>()); else ok = false; break;
    case 4: if constexpr (lo <= 4 && 4 <= hi) f(std::integral_constant<int, 4>()); else ok = false; break;
    case 5: if constexpr (lo <= 5 && 5 <= hi) f(std::integral_constant<int, 5>()); else ok = false; break;
    case 6: if constexpr (lo <= 6 && 6 <= hi) f(std::integral_constant<int, 6>()); else ok = false; break;
    case 7: if constexpr (lo <= 7 && 7 <= hi) f(std::integral_constant<int, 7>()); else ok = false; break;
    default: ok = false;
  }
  return ok;
}

template <class T>
static inline uint32_t quantize_axis(T v, T mn, T inv_scale, uint32_t max_bucket) {
  T scaled = std::floor((v - mn) * inv_scale);
  if (scaled > T(0)) {
    // num_traits to_u64(): None when the value does not fit in a u64.
    if (!(scaled < T(18446744073709551616.0))) return max_bucket;
    uint64_t q = (uint64_t)scaled;
    return (uint32_t)std::min<uint64_t>(q, max_bucket);
  }
  return 0;
}

uint64_t encode2(const uint32_t* c) { return MortonSpec<2>::encode(c); }
uint64_t encode3(const uint32_t* c) { return MortonSpec<3>::encode(c); }

// ---------------------------------------------------------------------------
// Arena: src/tsne/arena.rs:37-43 (Node), :65-94 (bounding_box), :137-328 (rebuild),
// :338-392 (compute_non_edge_forces), :398-427 (compute_edge_forces).
// ---------------------------------------------------------------------------
static const uint32_t SENTINEL = 0xffffffffu;

template <class T, int D>
struct Node {
  T com[D];
  uint32_t count;
  uint32_t first_child;
  uint8_t child_count;
  uint8_t level;
};

template <class T, int D>
struct Arena {
  std::vector<Node<T, D>> nodes;
  std::vector<std::pair<uint32_t, uint32_t>> ranges;
  typedef typename MortonSpec<D>::Code Code;
  std::vector<std::pair<Code, uint32_t>> sorted;
  std::vector<T> level_half_width_sq;

  void rebuild(const T* y, int64_t n) {
    const uint32_t bits = MortonSpec<D>::BITS;
    nodes.clear();
    ranges.clear();
    sorted.clear();
    if (n == 0) {
      level_half_width_sq.clear();
      return;
    }
    T mn[D], mx[D];
    for (int a = 0; a < D; ++a) {
      mn[a] = Num<T>::max();
      mx[a] = -Num<T>::max();
    }
    for (int64_t i = 0; i < n; ++i)
      for (int a = 0; a < D; ++a) {
        mn[a] = fmin_(mn[a], y[i * D + a]);
        mx[a] = fmax_(mx[a], y[i * D + a]);
      }
    T extent[D], inv_scale[D];
    const T scale = T((double)(1ULL << bits));
    const uint32_t max_bucket = (uint32_t)((1ULL << bits) - 1);
    for (int a = 0; a < D; ++a) {
      extent[a] = mx[a] - mn[a];
      inv_scale[a] = extent[a] > T(0) ? scale / extent[a] : T(0);
    }
    T max_extent = T(0);
    for (int a = 0; a < D; ++a) max_extent = fmax_(max_extent, extent[a]);
    level_half_width_sq.clear();
    for (uint32_t level = 0; level <= bits; ++level) {
      T hw = max_extent / T((double)(1ULL << (level + 1)));
      level_half_width_sq.push_back(hw * hw);
    }
    sorted.resize(n);
#pragma omp parallel for if (n >= 4096)
    for (int64_t i = 0; i < n; ++i) {
      uint32_t q[D];
      for (int a = 0; a < D; ++a) q[a] = quantize_axis(y[i * D + a], mn[a], inv_scale[a], max_bucket);
      sorted[i] = {MortonSpec<D>::encode(q), (uint32_t)i};
    }
    std::sort(sorted.begin(), sorted.end());

    nodes.reserve(2 * n - 1);
    ranges.reserve(2 * n - 1);
    Node<T, D> root{};
    root.count = (uint32_t)n;
    root.first_child = SENTINEL;
    root.child_count = 0;
    root.level = (uint8_t)bits;
    nodes.push_back(root);
    ranges.push_back({0u, (uint32_t)n});
    const Code mask = ((Code)1 << D) - 1;
    size_t node = 0;
    while (node < nodes.size()) {
      uint32_t start = ranges[node].first, end = ranges[node].second;
      if (end - start <= 1 || sorted[start].first == sorted[end - 1].first) {
        node += 1;
        continue;
      }
      const Code x = sorted[start].first ^ sorted[end - 1].first;
      uint32_t highest = msb_position(x);
      uint32_t level = (bits - 1) - highest / D;
      uint32_t shift = D * (bits - 1 - level);
      nodes[node].level = (uint8_t)level;
      uint32_t first_child = (uint32_t)nodes.size();
      uint32_t child_count = 0;
      uint32_t cs = start;
      while (cs < end) {
        const Code group = (sorted[cs].first >> shift) & mask;
        uint32_t ce = cs + 1;
        while (ce < end && ((sorted[ce].first >> shift) & mask) == group) ce += 1;
        Node<T, D> c{};
        c.count = ce - cs;
        c.first_child = SENTINEL;
        c.child_count = 0;
        c.level = (uint8_t)bits;
        nodes.push_back(c);
        ranges.push_back({cs, ce});
        child_count += 1;
        cs = ce;
      }
      nodes[node].first_child = first_child;
      nodes[node].child_count = (uint8_t)child_count;
      node += 1;
    }
    const int64_t nn = (int64_t)nodes.size();
#pragma omp parallel for if (nn >= 4096)
    for (int64_t v = 0; v < nn; ++v) {
      Node<T, D>& nd = nodes[v];
      if (nd.first_child != SENTINEL) continue;
      T c[D];
      for (int a = 0; a < D; ++a) c[a] = T(0);
      for (uint32_t s = ranges[v].first; s < ranges[v].second; ++s) {
        const T* p = y + (int64_t)sorted[s].second * D;
        for (int a = 0; a < D; ++a) c[a] += p[a];
      }
      T inv = T(1) / T(nd.count);
      for (int a = 0; a < D; ++a) nd.com[a] = c[a] * inv;
    }
    for (int64_t v = nn - 1; v >= 0; --v) {
      Node<T, D>& nd = nodes[v];
      if (nd.first_child == SENTINEL) continue;
      T total = T(nd.count);
      T c[D];
      for (int a = 0; a < D; ++a) c[a] = T(0);
      for (uint32_t ch = nd.first_child; ch < nd.first_child + nd.child_count; ++ch) {
        T w = T(nodes[ch].count);
        for (int a = 0; a < D; ++a) c[a] += nodes[ch].com[a] * w;
      }
      T inv = T(1) / total;
      for (int a = 0; a < D; ++a) nd.com[a] = c[a] * inv;
    }
  }

  void non_edge_forces(int64_t index, T theta_sq, const T* y, T* neg, T* q_sum,
                       std::vector<uint32_t>& stack) const {
    if (nodes.empty()) return;
    const T* q = y + index * D;
    size_t top = 0;
    if (stack.size() < 64) stack.resize(64);
    stack[top++] = 0;
    while (top > 0) {
      top -= 1;
      const Node<T, D>& nd = nodes[stack[top]];
      T disp[D];
      T dist = T(0);
      for (int a = 0; a < D; ++a) {
        T delta = q[a] - nd.com[a];
        disp[a] = delta;
        dist += delta * delta;
      }
      if (nd.first_child == SENTINEL) {
        if (dist == T(0)) continue;
      } else if (level_half_width_sq[nd.level] >= theta_sq * dist) {
        if (stack.size() < top + nd.child_count + 1) stack.resize(2 * (top + nd.child_count + 1));
        for (uint32_t c = 0; c < nd.child_count; ++c) stack[top++] = nd.first_child + c;
        continue;
      }
      T inverse = T(1) / (T(1) + dist);
      T magnitude = T(nd.count) * inverse;
      *q_sum += magnitude;
      magnitude = magnitude * inverse;
      for (int a = 0; a < D; ++a) neg[a] += magnitude * disp[a];
    }
  }

  // The same walk counting theta tests (node visits) and accepted cells
  // (interactions); the self leaf and its duplicates are visited, not counted.
  void count_visits(int64_t index, T theta_sq, const T* y, int64_t* visits, int64_t* interactions,
                    std::vector<uint32_t>& stack) const {
    if (nodes.empty()) return;
    const T* q = y + index * D;
    size_t top = 0;
    if (stack.size() < 64) stack.resize(64);
    stack[top++] = 0;
    while (top > 0) {
      top -= 1;
      const Node<T, D>& nd = nodes[stack[top]];
      *visits += 1;
      T dist = T(0);
      for (int a = 0; a < D; ++a) {
        T delta = q[a] - nd.com[a];
        dist += delta * delta;
      }
      if (nd.first_child == SENTINEL) {
        if (dist == T(0)) continue;
      } else if (level_half_width_sq[nd.level] >= theta_sq * dist) {
        if (stack.size() < top + nd.child_count + 1) stack.resize(2 * (top + nd.child_count + 1));
        for (uint32_t c = 0; c < nd.child_count; ++c) stack[top++] = nd.first_child + c;
        continue;
      }
      *interactions += 1;
    }
  }
};

template <class T, int D>
void edge_forces_row(int64_t index, const T* y, const uint64_t* rows, const uint32_t* cols,
                     const T* vals, T* pos) {
  const T* s = y + index * D;
  for (uint64_t e = rows[index]; e < rows[index + 1]; ++e) {
    const T* o = y + (int64_t)cols[e] * D;
    T disp[D];
    T dist = T(0);
    for (int a = 0; a < D; ++a) {
      T delta = s[a] - o[a];
      disp[a] = delta;
      dist += delta * delta;
    }
    T factor = vals[e] / (dist + T(1));
    for (int a = 0; a < D; ++a) pos[a] += factor * disp[a];
  }
}

template <class T, int D>
void edge_forces(const T* y, int64_t n, const uint64_t* rows, const uint32_t* cols, const T* vals,
                 T* pos) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    T row[D];
    for (int a = 0; a < D; ++a) row[a] = T(0);
    edge_forces_row<T, D>(i, y, rows, cols, vals, row);
    for (int a = 0; a < D; ++a) pos[i * D + a] = row[a];
  }
}

// BarnesHutRepulsion::step (src/repulsion.rs:95-158) without the attractive
// half: rebuild, per-point traversal, sequential Z. Returns Z (not 1/Z).
template <class T, int D>
T bh_repulsion(Arena<T, D>& arena, const T* y, int64_t n, T theta, T* neg, T* q_sums) {
  arena.rebuild(y, n);
  const T theta_sq = theta * theta;
#pragma omp parallel
  {
    std::vector<uint32_t> stack(256);
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
      T row[D];
      for (int a = 0; a < D; ++a) row[a] = T(0);
      T q = T(0);
      arena.non_edge_forces(i, theta_sq, y, row, &q, stack);
      for (int a = 0; a < D; ++a) neg[i * D + a] = row[a];
      q_sums[i] = q;
    }
  }
  T z = T(0);
  for (int64_t i = 0; i < n; ++i) z = z + q_sums[i];
  return z;
}

// Work of one Barnes-Hut repulsion pass at y: theta tests and accepted cells
// summed over all points (measurement aid for the traversal's rate).
template <class T, int D>
void bh_count(const T* y, int64_t n, T theta, int64_t* visits_out, int64_t* interactions_out) {
  Arena<T, D> a;
  a.rebuild(y, n);
  const T theta_sq = theta * theta;
  int64_t vis = 0, inter = 0;
#pragma omp parallel reduction(+ : vis, inter)
  {
    std::vector<uint32_t> stack(256);
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) a.count_visits(i, theta_sq, y, &vis, &inter, stack);
  }
  *visits_out = vis;
  *interactions_out = inter;
}

// ---------------------------------------------------------------------------
// Complex FFT for 7-smooth lengths (own mixed-radix decimation in time),
// standing in for rustfft/realfft behind src/tsne/fft.rs:20-247.
// ---------------------------------------------------------------------------
template <class T>
struct Fft1 {
  int n = 0;
  std::vector<int> radices;
  std::vector<std::complex<T>> tw;  // exp(-2 pi i k / n)
  void plan(int len) {
    n = len;
    radices.clear();
    int m = len;
    for (int p : {4, 2, 3, 5, 7}) {
      while (m % p == 0) {
        radices.push_back(p);
        m /= p;
      }
    }
    if (m != 1) radices.push_back(m);  // generic DFT for a leftover factor
    tw.resize(n);
    for (int k = 0; k < n; ++k) {
      double ang = -2.0 * M_PI * (double)k / (double)n;
      tw[k] = std::complex<T>((T)std::cos(ang), (T)std::sin(ang));
    }
  }
  // Recursive Cooley-Tukey; `sign` = -1 forward, +1 inverse (unnormalised).
  void rec(const std::complex<T>* in, int stride, std::complex<T>* out, int len, int ri,
           bool inverse, std::vector<std::complex<T>>& tmp) const {
    if (len == 1) {
      out[0] = in[0];
      return;
    }
    int p = radices[ri];
    int m = len / p;
    for (int r = 0; r < p; ++r) rec(in + r * stride, stride * p, out + r * m, m, ri + 1, inverse, tmp);
    // Butterflies: X[k + q m] = sum_r W_len^{r (k + q m)} Y_r[k]
    int tstep = n / len;
    std::vector<std::complex<T>> y(p);
    for (int kk = 0; kk < m; ++kk) {
      for (int r = 0; r < p; ++r) {
        std::complex<T> w = tw[(size_t)((int64_t)r * kk * tstep % n)];
        if (inverse) w = std::conj(w);
        y[r] = out[r * m + kk] * w;
      }
      for (int q = 0; q < p; ++q) {
        std::complex<T> acc(0, 0);
        for (int r = 0; r < p; ++r) {
          std::complex<T> w = tw[(size_t)((int64_t)r * q * m * tstep % n)];
          if (inverse) w = std::conj(w);
          acc += y[r] * w;
        }
        tmp[q] = acc;
      }
      for (int q = 0; q < p; ++q) out[q * m + kk] = tmp[q];
    }
  }
  void run(std::complex<T>* data, int stride, bool inverse, std::vector<std::complex<T>>& a,
           std::vector<std::complex<T>>& b) const {
    a.resize(n);
    b.resize(n);
    std::vector<std::complex<T>> tmp(8 + (radices.empty() ? 0 : *std::max_element(radices.begin(), radices.end())));
    for (int i = 0; i < n; ++i) a[i] = data[(size_t)i * stride];
    rec(a.data(), 1, b.data(), n, 0, inverse, tmp);
    for (int i = 0; i < n; ++i) data[(size_t)i * stride] = b[i];
  }
};

template <class T>
void fft_nd(std::vector<std::complex<T>>& grid, int len, int dims, bool inverse, const Fft1<T>& f) {
  if (dims == 1) {
    std::vector<std::complex<T>> a, b;
    f.run(grid.data(), 1, inverse, a, b);
    return;
  }
  // dims == 2: rows then columns.
#pragma omp parallel
  {
    std::vector<std::complex<T>> a, b;
#pragma omp for
    for (int r = 0; r < len; ++r) f.run(grid.data() + (size_t)r * len, 1, inverse, a, b);
#pragma omp for
    for (int c = 0; c < len; ++c) f.run(grid.data() + c, len, inverse, a, b);
  }
}

// ---------------------------------------------------------------------------
// FIt-SNE interpolation: src/tsne/interpolation.rs:100-134 (repulsive_forces),
// :162-187 (locate_points), :198-226 (build_kernel_spectrum), :247-269
// (spread_charges), :273-278 (multiply), :282-301 (gather), :305-332
// (reconstruct), :337-389 (bounds, box_count, next_smooth, signed_lag),
// :395-441 (Lagrange basis), :446-481 (charges, node_of_combo).
// ---------------------------------------------------------------------------
static const int INTERP_POINTS = 3;
static const int MIN_BOXES = 10;
static const int MAX_BOXES = 1000;

int64_t next_smooth(int64_t n) {
  int64_t cand = std::max<int64_t>(n, 1);
  for (;;) {
    int64_t v = cand;
    for (int p : {2, 3, 5, 7})
      while (v % p == 0) v /= p;
    if (v == 1) return cand;
    cand += 1;
  }
}

template <class T>
int64_t box_count(T extent) {
  T scaled = std::ceil(extent / T(1.0));
  int64_t s = 0;
  if (scaled > T(0)) {
    // `as usize` saturates.
    s = scaled >= T(9.2e18) ? INT64_MAX : (int64_t)scaled;
  }
  return std::min<int64_t>(std::max<int64_t>(s, MIN_BOXES), MAX_BOXES);
}

template <class T>
struct Lagrange {
  T nodes[INTERP_POINTS];
  T inv_denom[INTERP_POINTS];
  Lagrange() {
    const T half = T(0.5);
    const T p_recip = T(1) / T(INTERP_POINTS);
    for (int k = 0; k < INTERP_POINTS; ++k) nodes[k] = (T(k) + half) * p_recip;
    for (int k = 0; k < INTERP_POINTS; ++k) {
      T denom = T(1);
      for (int m = 0; m < INTERP_POINTS; ++m)
        if (m != k) denom = denom * (nodes[k] - nodes[m]);
      inv_denom[k] = T(1) / denom;
    }
  }
  void weights(T local, T* out) const {
    for (int k = 0; k < INTERP_POINTS; ++k) {
      T num = T(1);
      for (int m = 0; m < INTERP_POINTS; ++m)
        if (m != k) num = num * (local - nodes[m]);
      out[k] = num * inv_denom[k];
    }
  }
};

struct FitGridInfo {
  int64_t boxes, nodes, fft_len;
  double min, box_width, spacing;
};

template <class T, int D>
T fit_repulsion(const T* y, int64_t n, T* neg, FitGridInfo* info) {
  if (n == 0) return T(0);
  T lo = std::numeric_limits<T>::infinity(), hi = -std::numeric_limits<T>::infinity();
  for (int64_t e = 0; e < n * D; ++e) {
    lo = fmin_(lo, y[e]);
    hi = fmax_(hi, y[e]);
  }
  T extent = fmax_(hi - lo, Num<T>::min_pos());
  int64_t boxes = box_count(extent);
  int64_t nodes = boxes * INTERP_POINTS;
  int64_t len = next_smooth(2 * nodes - 1);
  T box_width = extent / T(boxes);
  T spacing = box_width / T(INTERP_POINTS);
  if (info) {
    info->boxes = boxes;
    info->nodes = nodes;
    info->fft_len = len;
    info->min = (double)lo;
    info->box_width = (double)box_width;
    info->spacing = (double)spacing;
  }
  // locate_points
  const T inv_box_width = T(1) / box_width;
  const int64_t last_box = boxes - 1;
  Lagrange<T> basis;
  std::vector<int64_t> box_index(n * D);
  std::vector<T> weights(n * D * INTERP_POINTS);
#pragma omp parallel for if (n >= 4096)
  for (int64_t i = 0; i < n; ++i) {
    for (int a = 0; a < D; ++a) {
      T offset = (y[i * D + a] - lo) * inv_box_width;
      T b = std::floor(offset);
      int64_t bid = 0;
      if (b > T(0)) bid = std::min<int64_t>(b >= T(9.2e18) ? last_box : (int64_t)b, last_box);
      box_index[i * D + a] = bid;
      T local = offset - T((double)bid);
      basis.weights(local, &weights[(i * D + a) * INTERP_POINTS]);
    }
  }
  // build_kernel_spectrum
  int64_t total = 1;
  for (int a = 0; a < D; ++a) total *= len;
  std::vector<std::complex<T>> kernel(total);
  for (int64_t flat = 0; flat < total; ++flat) {
    T sq = T(0);
    int64_t rem = flat;
    for (int a = 0; a < D; ++a) {
      int64_t coord = rem % len;
      rem /= len;
      int64_t lag = coord <= len / 2 ? coord : coord - len;
      T disp = spacing * T((double)lag);
      sq = sq + disp * disp;
    }
    T cauchy = T(1) / (T(1) + sq);
    kernel[flat] = std::complex<T>(cauchy * cauchy, T(0));
  }
  Fft1<T> f;
  f.plan((int)len);
  fft_nd(kernel, (int)len, D, false, f);
  const T inv_total = T(1) / T((double)total);
  for (auto& v : kernel) v = v * inv_total;
  // convolve_terms
  const int combos = D == 1 ? 3 : 9;
  std::vector<T> potentials(n * (D + 2));
  std::vector<std::complex<T>> grid(total);
  auto node_of_combo = [&](int combo, int64_t i, int64_t* flat, T* w) {
    int rem = combo;
    int64_t fl = 0;
    T wt = T(1);
    for (int a = 0; a < D; ++a) {
      int k = rem % INTERP_POINTS;
      rem /= INTERP_POINTS;
      int64_t nd = box_index[i * D + a] * INTERP_POINTS + k;
      fl = fl * len + nd;
      wt = wt * weights[(i * D + a) * INTERP_POINTS + k];
    }
    *flat = fl;
    *w = wt;
  };
  for (int term = 0; term < D + 2; ++term) {
    std::fill(grid.begin(), grid.end(), std::complex<T>(0, 0));
    for (int64_t i = 0; i < n; ++i) {
      T charge;
      if (term == 0)
        charge = T(1);
      else if (term <= D)
        charge = y[i * D + term - 1];
      else {
        charge = T(0);
        for (int a = 0; a < D; ++a) charge = charge + y[i * D + a] * y[i * D + a];
      }
      for (int c = 0; c < combos; ++c) {
        int64_t fl;
        T w;
        node_of_combo(c, i, &fl, &w);
        grid[fl] = std::complex<T>(grid[fl].real() + w * charge, T(0));
      }
    }
    fft_nd(grid, (int)len, D, false, f);
    for (int64_t e = 0; e < total; ++e) grid[e] = grid[e] * kernel[e];
    fft_nd(grid, (int)len, D, true, f);
#pragma omp parallel for if (n >= 4096)
    for (int64_t i = 0; i < n; ++i) {
      T phi = T(0);
      for (int c = 0; c < combos; ++c) {
        int64_t fl;
        T w;
        node_of_combo(c, i, &fl, &w);
        phi = phi + w * grid[fl].real();
      }
      potentials[i * (D + 2) + term] = phi;
    }
  }
  // reconstruct
  const T two = T(2);
  std::vector<T> z_terms((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    const T* phi = &potentials[i * (D + 2)];
    T density = phi[0];
    T sqn = phi[D + 1];
    T norm_sq = T(0), cross = T(0);
    for (int a = 0; a < D; ++a) {
      T fm = phi[1 + a];
      neg[i * D + a] = y[i * D + a] * density - fm;
      norm_sq = norm_sq + y[i * D + a] * y[i * D + a];
      cross = cross + y[i * D + a] * fm;
    }
    z_terms[i] = (T(1) + norm_sq) * density - two * cross + sqn;
  }
  return tree_sum(z_terms.data(), n) - T((double)n);
}

// ---------------------------------------------------------------------------
// gradient_descent_step: src/tsne/mod.rs:470-516; update_solution: :423-451;
// zero_mean: :534-568. Gain constants: src/tsne/mod.rs:29-31.
// ---------------------------------------------------------------------------
template <class T>
void gradient_step(T* y, const T* pos, const T* neg, T* uy, T* gains, int64_t len, T lr,
                   T momentum, T inv_norm) {
  const T inc = T(0.2), dec = T(0.8), floor_ = T(0.01);
#pragma omp parallel for if (len >= 8192)
  for (int64_t e = 0; e < len; ++e) {
    T g = pos[e] - neg[e] * inv_norm;
    T gn = (signum(g) != signum(uy[e])) ? gains[e] + inc : gains[e] * dec;
    if (gn < floor_) gn = floor_;
    gains[e] = gn;
    uy[e] = momentum * uy[e] - lr * gn * g;
    y[e] += uy[e];
  }
}

template <class T>
void update_solution(T* y, const T* dy, T* uy, T* gains, int64_t len, T lr, T momentum) {
  const T inc = T(0.2), dec = T(0.8), floor_ = T(0.01);
  for (int64_t e = 0; e < len; ++e) {
    T gn = (signum(dy[e]) != signum(uy[e])) ? gains[e] + inc : gains[e] * dec;
    if (gn < floor_) gn = floor_;
    gains[e] = gn;
    uy[e] = momentum * uy[e] - lr * gn * dy[e];
    y[e] += uy[e];
  }
}

template <class T>
void zero_mean(T* y, int64_t n, int D) {
  std::vector<T> mean(D, T(0));
  for (int64_t i = 0; i < n; ++i)
    for (int a = 0; a < D; ++a) mean[a] += y[i * D + a];
  T nn = T((double)n);
  for (int a = 0; a < D; ++a) mean[a] /= nn;
  for (int64_t i = 0; i < n; ++i)
    for (int a = 0; a < D; ++a) y[i * D + a] -= mean[a];
}

// ---------------------------------------------------------------------------
// KL divergence: sparse_kl_divergence src/tsne/mod.rs:738-775. With `quirk`
// the value read is p_values[row] exactly as the reference does (:768-770);
// without it, the CSR entry's own value.
// ---------------------------------------------------------------------------
template <class T, int D>
T sparse_kl(const uint64_t* rows, const uint32_t* cols, const T* vals, const T* y, int64_t n,
            T inv_q_sum, bool quirk) {
  std::vector<T> partial(n, T(0));
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    T cost = T(0);
    for (uint64_t e = rows[i]; e < rows[i + 1]; ++e) {
      const T* a = y + i * D;
      const T* b = y + (int64_t)cols[e] * D;
      T q = T(0);
      for (int c = 0; c < D; ++c) {
        T d = a[c] - b[c];
        q = q + d * d;
      }
      q = (T(1) / (T(1) + q)) * inv_q_sum;
      T p = quirk ? vals[i] : vals[e];
      cost += p * std::log((p + Num<T>::min_pos()) / (q + Num<T>::min_pos()));
    }
    partial[i] = cost;
  }
  return tree_sum(partial.data(), n);
}

// evaluate_error (exact KL): src/tsne/mod.rs:579-618.
template <class T, int D>
T exact_kl(const T* p, const T* y, int64_t n) {
  std::vector<T> dist((size_t)(n * n), T(0));
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = i + 1; j < n; ++j) {
      T s = T(0);
      for (int c = 0; c < D; ++c) {
        T d = y[i * D + c] - y[j * D + c];
        s = s + d * d;
      }
      dist[i * n + j] = s;
      dist[j * n + i] = s;
    }
  std::vector<T> terms((size_t)(n * n));
  for (int64_t e = 0; e < n * n; ++e) terms[e] = T(1) / (T(1) + dist[e]);
  const T inv = T(1) / tree_sum(terms.data(), n * n);
  for (int64_t e = 0; e < n * n; ++e) {
    T q = T(1) / (T(1) + dist[e]) * inv;
    terms[e] = p[e] * std::log((p[e] + Num<T>::min_pos()) / (q + Num<T>::min_pos()));
  }
  return tree_sum(terms.data(), n * n);
}

// The exact method's joint P before normalisation: src/lib.rs:512-554. The
// caller's distance closure is evaluated on the strict upper triangle and
// mirrored, the diagonal stays zero (src/tsne/mod.rs:161-189); search_beta runs
// over each full row, the zero self-distance included, so p_ii is not zero;
// then p_ij + p_ji is stored on both sides, without the sparse path's halving.
template <class T>
void exact_affinities(const T* dist_in, int64_t n, T perplexity, T* p, std::vector<T>& distances) {
  distances.assign((size_t)(n * n), T(0));
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = i + 1; j < n; ++j) {
      distances[i * n + j] = dist_in[i * n + j];
      distances[j * n + i] = dist_in[i * n + j];
    }
  std::fill(p, p + n * n, T(0));
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) search_beta(&p[i * n], &distances[i * n], n, perplexity);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = i + 1; j < n; ++j) {
      T s = p[j * n + i];
      p[i * n + j] += s;
      p[j * n + i] = p[i * n + j];
    }
}

// One exact gradient: src/lib.rs:567-619. Squared embedding distances on the
// upper triangle, mirrored; q = 1 / (1 + d) over all n^2 entries, the diagonal
// included (q_ii = 1, so Z counts n); Z summed in T; then
// dy_i += (y_i - y_j) (p_ij - q_ij / Z) q_ij over every j. dy is overwritten.
// Returns Z.
template <class T, int D>
T exact_gradient(const T* p, const T* y, int64_t n, T* dy, std::vector<T>& distances, std::vector<T>& q) {
  const int64_t pe = n * n;
  distances.assign((size_t)pe, T(0));
  q.resize((size_t)pe);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = i + 1; j < n; ++j) {
      T s = T(0);
      for (int c = 0; c < D; ++c) {
        T d = y[i * D + c] - y[j * D + c];
        s = s + d * d;
      }
      distances[i * n + j] = s;
    }
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = i + 1; j < n; ++j) distances[j * n + i] = distances[i * n + j];
  for (int64_t e = 0; e < pe; ++e) q[e] = T(1) / (T(1) + distances[e]);
  const T qs = tree_sum(q.data(), pe);
  const T inv = T(1) / qs;
  std::fill(dy, dy + n * D, T(0));
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = 0; j < n; ++j) {
      T m = (p[i * n + j] - q[i * n + j] * inv) * q[i * n + j];
      for (int c = 0; c < D; ++c) dy[i * D + c] += (y[i * D + c] - y[j * D + c]) * m;
    }
  return qs;
}

// ---------------------------------------------------------------------------
// The tSNE builder state machine: src/lib.rs:149-176 (fields), :241-266
// (defaults), :489-646 (exact), :652-659 (learning rate), :663-685
// (finalize_p_and_seed), :701-1014 (approximate fits and run_loop), :1019-1051
// (affinities / with_affinities), :1061-1127 (build_affinities), :1162-1179
// (epoch_tail), :1182-1248 (validation and cache), :1254-1268 (neighbor copy).
// ---------------------------------------------------------------------------
enum FitKind { FIT_NONE = 0, FIT_EXACT = 1, FIT_BH = 2, FIT_INTERP = 3 };

typedef void (*epoch_cb_t)(int64_t epoch, const void* y, void* user);

struct Status {
  int code = 0;
  std::string msg;
};

template <class T>
struct TSNE {
  int D;
  int64_t n;
  bool has_lr = false;
  T learning_rate = T(0);
  int64_t epochs = 1000;
  T momentum = T(0.5), final_momentum = T(0.8);
  int64_t momentum_switch_epoch = 250, stop_lying_epoch = 250;
  T early_exaggeration = T(12.0);
  T perplexity = T(20.0);
  std::vector<T> p_values;
  std::vector<uint64_t> p_rows;
  std::vector<uint32_t> p_columns;
  std::vector<T> y, dy, uy, gains;
  epoch_cb_t cb = nullptr;
  void* cb_user = nullptr;
  bool has_init = false;
  std::vector<T> initial;
  bool stop_lying_fired = false;
  bool has_cached_perplexity = false;
  T cached_perplexity = T(0);
  int fit = FIT_NONE;
  T fit_theta = T(0);
  uint64_t seed = 0x6268747336e65ULL;
  Status st;

  TSNE(int D_, int64_t n_) : D(D_), n(n_) {}

  int fail(const std::string& m) {
    st.code = 22;
    st.msg = m;
    return 22;
  }

  T resolve_lr() const {
    if (has_lr) return learning_rate;
    T a = T((double)n) / early_exaggeration / T(4.0);
    return fmax_(a, T(50.0));
  }

  void random_init() {
    // Seeded Box-Muller, N(0, 1e-4); the reference draws from an unseeded rng.
    uint64_t s = seed;
    auto next = [&]() {
      s = s * 6364136223846793005ULL + 1442695040888963407ULL;
      return ((s >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (size_t e = 0; e < y.size(); e += 2) {
      double u1 = next(), u2 = next();
      double r = std::sqrt(-2.0 * std::log(u1));
      y[e] = T(1e-4 * r * std::cos(2 * M_PI * u2));
      if (e + 1 < y.size()) y[e + 1] = T(1e-4 * r * std::sin(2 * M_PI * u2));
    }
  }

  int finalize_p_and_seed(int64_t grad_entries) {
    normalize_p(p_values.data(), (int64_t)p_values.size(), early_exaggeration);
    if (stop_lying_epoch == 0) stop_lying(p_values.data(), (int64_t)p_values.size(), early_exaggeration);
    if (has_init) {
      has_init = false;
      if ((int64_t)initial.size() != grad_entries) {
        char buf[256];
        snprintf(buf, sizeof buf, "error: initial embedding has %zu values, expected n_samples * D = %lld",
                 initial.size(), (long long)grad_entries);
        initial.clear();
        return fail(buf);
      }
      std::copy(initial.begin(), initial.end(), y.begin());
      initial.clear();
    } else {
      random_init();
    }
    return 0;
  }

  void epoch_tail(int64_t epoch) {
    if (epoch == stop_lying_epoch && epoch != 0) {
      stop_lying(p_values.data(), (int64_t)p_values.size(), early_exaggeration);
      stop_lying_fired = true;
    }
    if (epoch == momentum_switch_epoch) momentum = final_momentum;
    if (cb) cb(epoch, y.data(), cb_user);
  }

  // build_affinities from a kNN table (the *_with_neighbors filler and the
  // brute-force Euclidean filler share it).
  void build_affinities(const uint32_t* idx, const T* dist, int64_t k) {
    const int64_t grad_entries = n * D;
    y.resize(grad_entries, T(0));
    uy.resize(grad_entries, T(0));
    gains.resize(grad_entries, T(1));
    std::vector<T> p(n * k, T(0));
    std::vector<uint32_t> cols(idx, idx + n * k);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) search_beta(&p[i * k], dist + i * k, k, perplexity);
    symmetrize<T>(std::move(cols), std::move(p), n, k, p_rows, p_columns, p_values);
    has_cached_perplexity = true;
    cached_perplexity = perplexity;
  }

  bool has_cached_affinities() const {
    return !p_rows.empty() && (int64_t)p_rows.size() == n + 1 && has_cached_perplexity &&
           cached_perplexity == perplexity;
  }

  bool cached_match_neighbors(const uint32_t* idx, int64_t k) const {
    if (p_rows.empty() || (int64_t)p_rows.size() != n + 1 || !has_cached_perplexity ||
        cached_perplexity != perplexity)
      return false;
    for (int64_t i = 0; i < n; ++i) {
      uint64_t s = p_rows[i], e = p_rows[i + 1];
      if ((int64_t)(e - s) != k) return false;
      for (int64_t j = 0; j < k; ++j)
        if (p_columns[s + j] != idx[i * k + j]) return false;
    }
    return true;
  }

  template <int DD>
  int run_loop(int kind, T theta) {
    const int64_t ge = n * DD;
    std::vector<T> pos(ge, T(0)), neg(ge, T(0)), q_sums(n, T(0));
    const T lr = resolve_lr();
    Arena<T, (DD >= 2 ? DD : 2)> arena;
    for (int64_t epoch = 0; epoch < epochs; ++epoch) {
      T inv_norm = T(0);
      if (kind == FIT_BH) {
        if constexpr (DD >= 2) {
          edge_forces<T, DD>(y.data(), n, p_rows.data(), p_columns.data(), p_values.data(), pos.data());
          T z = bh_repulsion<T, DD>(arena, y.data(), n, theta, neg.data(), q_sums.data());
          inv_norm = T(1) / z;
        }
      } else {
        edge_forces<T, DD>(y.data(), n, p_rows.data(), p_columns.data(), p_values.data(), pos.data());
        T z = fit_repulsion_dispatch<DD>(y.data(), neg.data());
        inv_norm = T(1) / z;
      }
      gradient_step(y.data(), pos.data(), neg.data(), uy.data(), gains.data(), ge, lr, momentum, inv_norm);
      zero_mean(y.data(), n, DD);
      epoch_tail(epoch);
    }
    dy.clear();
    uy.clear();
    gains.clear();
    fit = kind;
    fit_theta = theta;
    return 0;
  }

  template <int DD>
  T fit_repulsion_dispatch(const T* yy, T* neg) {
    if constexpr (DD == 1 || DD == 2) return fit_repulsion<T, DD>(yy, n, neg, nullptr);
    return T(0);
  }

  int dispatch_loop(int kind, T theta) {
    if (kind == FIT_BH) {
      int rc = 0;
      if (!with_d<2, 7>(D, [&](auto dc) { rc = run_loop<decltype(dc)::value>(kind, theta); }))
        return fail("error: Barnes-Hut covers D in 2..7.");
      return rc;
    }
    if (D == 1) return run_loop<1>(kind, theta);
    if (D == 2) return run_loop<2>(kind, theta);
    return fail("error: FIt-SNE is restricted to D in {1, 2}.");
  }

  int prepare_cached() {
    stop_lying_fired = false;
    const int64_t ge = n * D;
    y.resize(ge, T(0));
    uy.resize(ge, T(0));
    gains.resize(ge, T(1));
    return finalize_p_and_seed(ge);
  }

  int validate(int kind, T theta) {
    if (kind == FIT_BH && !(theta > T(0)))
      return fail("error: theta value must be greater than 0.0.\n            A value of 0.0 corresponds to using the exact version of the algorithm.");
    if (!perplexity_ok(perplexity, n))
      return fail("error: the provided perplexity is too large for the number of data points.\n");
    return 0;
  }

  // barnes_hut / fit_sne over a dense Euclidean dataset (src/lib.rs:701-742, :835-871).
  int fit_euclidean(int kind, T theta, const T* X, int32_t dim) {
    if (int rc = validate(kind, theta)) return rc;
    if (has_cached_affinities()) {
      if (int rc = prepare_cached()) return rc;
      return dispatch_loop(kind, theta);
    }
    int64_t k = (int64_t)(T(3.0) * perplexity);
    std::vector<uint32_t> idx(n * k);
    std::vector<T> dist(n * k);
    knn_brute(X, n, dim, (int32_t)k, idx.data(), dist.data());
    build_affinities(idx.data(), dist.data(), k);
    if (int rc = finalize_p_and_seed(n * D)) return rc;
    return dispatch_loop(kind, theta);
  }

  // *_with_neighbors: src/lib.rs:757-772, :884-894, :922-951.
  int fit_with_neighbors(int kind, T theta, const uint64_t* idx64, const T* dist, int64_t rows,
                         int64_t k) {
    if (kind == FIT_BH) {
      if (int rc = validate(kind, theta)) return rc;
    }
    if (rows != n) {
      char buf[200];
      snprintf(buf, sizeof buf, "error: neighbors has %lld rows, expected one per sample = %lld",
               (long long)rows, (long long)n);
      return fail(buf);
    }
    if (k <= 0) return fail("error: every neighbors row must have the same length, greater than zero.");
    std::vector<uint32_t> idx(n * k);
    for (int64_t e = 0; e < n * k; ++e) idx[e] = (uint32_t)idx64[e];
    bool hit = true;
    for (int64_t e = 0; e < n * k; ++e)
      if (idx64[e] > 0xffffffffULL) hit = false;
    if (hit && cached_match_neighbors(idx.data(), k)) {
      if (int rc = prepare_cached()) return rc;
      return dispatch_loop(kind, theta);
    }
    for (int64_t e = 0; e < n * k; ++e)
      if (idx64[e] >= (uint64_t)n) {
        char buf[200];
        snprintf(buf, sizeof buf,
                 "error: a neighbor index is out of range, every index must be < n_samples = %lld.",
                 (long long)n);
        return fail(buf);
      }
    build_affinities(idx.data(), dist, k);
    if (int rc = finalize_p_and_seed(n * D)) return rc;
    return dispatch_loop(kind, theta);
  }

  // exact over a dense distance matrix computed by the caller's closure
  // (src/lib.rs:489-646). `dist` is n*n with a zero diagonal.
  int exact_with_distances(const T* dist_in) {
    if (!perplexity_ok(perplexity, n))
      return fail("error: the provided perplexity is too large for the number of data points.\n");
    const int64_t ge = n * D, pe = n * n;
    y.resize(ge, T(0));
    dy.assign(ge, T(0));
    uy.resize(ge, T(0));
    gains.resize(ge, T(1));
    p_values.assign(pe, T(0));
    std::vector<T> distances, q;
    exact_affinities(dist_in, n, perplexity, p_values.data(), distances);
    if (int rc = finalize_p_and_seed(ge)) return rc;
    const T lr = resolve_lr();
    for (int64_t epoch = 0; epoch < epochs; ++epoch) {
      with_d<1, 7>(D, [&](auto dc) {
        exact_gradient<T, decltype(dc)::value>(p_values.data(), y.data(), n, dy.data(), distances, q);
      });
      update_solution(y.data(), dy.data(), uy.data(), gains.data(), ge, lr, momentum);
      std::fill(dy.begin(), dy.end(), T(0));
      zero_mean(y.data(), n, D);
      epoch_tail(epoch);
    }
    dy.clear();
    uy.clear();
    gains.clear();
    fit = FIT_EXACT;
    return 0;
  }

  // kl_divergence: src/lib.rs:448-477.
  bool kl(bool quirk, T* out) {
    if (fit == FIT_NONE) return false;
    if (fit == FIT_EXACT) {
      with_d<1, 7>(D, [&](auto dc) { *out = exact_kl<T, decltype(dc)::value>(p_values.data(), y.data(), n); });
      return true;
    }
    T z;
    std::vector<T> neg(n * D), qs(n);
    if (fit == FIT_BH) {
      with_d<2, 7>(D, [&](auto dc) {
        constexpr int DD = decltype(dc)::value;
        Arena<T, DD> a;
        bh_repulsion<T, DD>(a, y.data(), n, fit_theta, neg.data(), qs.data());
      });
      // evaluate_error_approximately sums the q_sums in parallel (src/tsne/mod.rs:668)
      z = tree_sum(qs.data(), n);
    } else {
      if (D == 1) z = fit_repulsion<T, 1>(y.data(), n, neg.data(), nullptr);
      else z = fit_repulsion<T, 2>(y.data(), n, neg.data(), nullptr);
    }
    T inv = T(1) / z;
    with_d<1, 7>(D, [&](auto dc) {
      *out = sparse_kl<T, decltype(dc)::value>(p_rows.data(), p_columns.data(), p_values.data(), y.data(), n, inv, quirk);
    });
    return true;
  }
};

}  // namespace orc

// ===========================================================================
// extern "C" surface, driven from Python (ctypes) by tests and bench.py.
// dtype: 0 = f32, 1 = f64. T-typed buffers are passed as void*.
// ===========================================================================
using namespace orc;

extern "C" {

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

#define ORC_T(dtype, ...) \
  do {                     \
    if ((dtype) == 0) {    \
      typedef float T;     \
      __VA_ARGS__;         \
    } else {               \
      typedef double T;    \
      __VA_ARGS__;         \
    }                      \
  } while (0)

void orc_knn(int dtype, const void* X, int64_t n, int32_t dim, int32_t k, uint32_t* idx, void* dist) {
  ORC_T(dtype, knn_brute<T>((const T*)X, n, dim, k, idx, (T*)dist));
}

void orc_knn_rows(int dtype, const void* X, int64_t n, int32_t dim, int32_t k, const int64_t* rows, int64_t nrows,
                  uint32_t* idx, void* dist) {
  ORC_T(dtype, knn_brute_rows<T>((const T*)X, n, dim, k, rows, nrows, idx, (T*)dist));
}

int orc_search_beta(int dtype, const void* dist, int64_t n, int32_t k, double perplexity, void* p,
                    int32_t* iterations) {
  int worst = 0;
  ORC_T(dtype, {
    for (int64_t i = 0; i < n; ++i) {
      int it = search_beta<T>((T*)p + i * k, (const T*)dist + i * k, k, (T)perplexity);
      if (iterations) iterations[i] = it;
      worst = std::max(worst, it);
    }
  });
  return worst;
}

int64_t orc_symmetrize(int dtype, const uint32_t* cols, const void* p, int64_t n, int32_t k,
                       uint64_t* rows_out, uint32_t* cols_out, void* vals_out) {
  int64_t nnz = 0;
  ORC_T(dtype, {
    std::vector<uint64_t> r;
    std::vector<uint32_t> c;
    std::vector<T> v;
    symmetrize<T>(std::vector<uint32_t>(cols, cols + n * k),
                  std::vector<T>((const T*)p, (const T*)p + n * k), n, k, r, c, v);
    nnz = (int64_t)c.size();
    if (rows_out) std::copy(r.begin(), r.end(), rows_out);
    if (cols_out) std::copy(c.begin(), c.end(), cols_out);
    if (vals_out) std::copy(v.begin(), v.end(), (T*)vals_out);
  });
  return nnz;
}

void orc_normalize(int dtype, void* vals, int64_t nnz, double exaggeration) {
  ORC_T(dtype, normalize_p<T>((T*)vals, nnz, (T)exaggeration));
}

int orc_edge_forces(int dtype, int32_t D, const void* y, int64_t n, const uint64_t* rows,
                    const uint32_t* cols, const void* vals, void* pos) {
  ORC_T(dtype, {
    if (!with_d<1, 7>(D, [&](auto dc) {
          edge_forces<T, decltype(dc)::value>((const T*)y, n, rows, cols, (const T*)vals, (T*)pos);
        }))
      return 22;
  });
  return 0;
}

// Returns Z through z_out; neg and q_sums per point.
int orc_bh_repulsion(int dtype, int32_t D, const void* y, int64_t n, double theta, void* neg,
                     void* q_sums, double* z_out) {
  ORC_T(dtype, {
    T z = T(0);
    if (!with_d<2, 7>(D, [&](auto dc) {
          constexpr int DD = decltype(dc)::value;
          Arena<T, DD> a;
          z = bh_repulsion<T, DD>(a, (const T*)y, n, (T)theta, (T*)neg, (T*)q_sums);
        }))
      return 22;
    *z_out = (double)z;
  });
  return 0;
}

// Theta tests and accepted cells of one Barnes-Hut repulsion pass at y.
int orc_bh_interactions(int dtype, int32_t D, const void* y, int64_t n, double theta, int64_t* visits_out,
                        int64_t* interactions_out) {
  ORC_T(dtype, {
    if (!with_d<2, 7>(D, [&](auto dc) {
          constexpr int DD = decltype(dc)::value;
          bh_count<T, DD>((const T*)y, n, (T)theta, visits_out, interactions_out);
        }))
      return 22;
  });
  return 0;
}

// Dumps the arena: returns the node count; arrays may be NULL for a size query.
int64_t orc_bh_tree(int dtype, int32_t D, const void* y, int64_t n, void* com, uint32_t* count,
                    uint8_t* level, uint32_t* first_child, uint8_t* child_count, uint32_t* range_start,
                    uint32_t* range_end) {
  int64_t nn = -1;
  ORC_T(dtype, {
    auto dump = [&](auto& a, int DD) {
      nn = (int64_t)a.nodes.size();
      for (int64_t v = 0; v < nn; ++v) {
        if (com)
          for (int c = 0; c < DD; ++c) ((T*)com)[v * DD + c] = a.nodes[v].com[c];
        if (count) count[v] = a.nodes[v].count;
        if (level) level[v] = a.nodes[v].level;
        if (first_child) first_child[v] = a.nodes[v].first_child;
        if (child_count) child_count[v] = a.nodes[v].child_count;
        if (range_start) range_start[v] = a.ranges[v].first;
        if (range_end) range_end[v] = a.ranges[v].second;
      }
    };
    with_d<2, 7>(D, [&](auto dc) {
      constexpr int DD = decltype(dc)::value;
      Arena<T, DD> a;
      a.rebuild((const T*)y, n);
      dump(a, DD);
    });
  });
  return nn;
}

// FIt-SNE repulsion at a fixed embedding; grid_out (6 doubles): boxes, nodes,
// fft_len, min, box_width, spacing.
int orc_fit_repulsion(int dtype, int32_t D, const void* y, int64_t n, void* neg, double* z_out,
                      double* grid_out) {
  FitGridInfo info{};
  ORC_T(dtype, {
    T z;
    if (D == 1) z = fit_repulsion<T, 1>((const T*)y, n, (T*)neg, &info);
    else if (D == 2) z = fit_repulsion<T, 2>((const T*)y, n, (T*)neg, &info);
    else return 22;
    *z_out = (double)z;
  });
  if (grid_out) {
    grid_out[0] = (double)info.boxes;
    grid_out[1] = (double)info.nodes;
    grid_out[2] = (double)info.fft_len;
    grid_out[3] = info.min;
    grid_out[4] = info.box_width;
    grid_out[5] = info.spacing;
  }
  return 0;
}

void orc_gradient_step(int dtype, void* y, const void* pos, const void* neg, void* uy, void* gains,
                       int64_t len, double lr, double momentum, double inv_norm) {
  ORC_T(dtype, gradient_step<T>((T*)y, (const T*)pos, (const T*)neg, (T*)uy, (T*)gains, len, (T)lr,
                                (T)momentum, (T)inv_norm));
}

int orc_exact_affinities(int dtype, const void* dist, int64_t n, double perplexity, void* p) {
  ORC_T(dtype, {
    std::vector<T> distances;
    exact_affinities<T>((const T*)dist, n, (T)perplexity, (T*)p, distances);
  });
  return 0;
}

double orc_exact_gradient(int dtype, int32_t D, const void* p, const void* y, int64_t n, void* dy) {
  double z = 0;
  ORC_T(dtype, {
    std::vector<T> distances, q;
    with_d<1, 7>(D, [&](auto dc) {
      z = (double)exact_gradient<T, decltype(dc)::value>((const T*)p, (const T*)y, n, (T*)dy, distances, q);
    });
  });
  return z;
}

void orc_zero_mean(int dtype, void* y, int64_t n, int32_t D) {
  ORC_T(dtype, zero_mean<T>((T*)y, n, D));
}

double orc_sparse_kl(int dtype, int32_t D, const uint64_t* rows, const uint32_t* cols,
                     const void* vals, const void* y, int64_t n, double inv_q_sum, int quirk) {
  double out = 0;
  ORC_T(dtype, {
    with_d<1, 7>(D, [&](auto dc) {
      out = sparse_kl<T, decltype(dc)::value>(rows, cols, (const T*)vals, (const T*)y, n, (T)inv_q_sum, quirk != 0);
    });
  });
  return out;
}

// Morton code of D coordinates (D = 2..7) as two 64-bit halves.
int orc_morton(int32_t D, const uint32_t* c, uint64_t* lo, uint64_t* hi) {
  bool ok = with_d<2, 7>(D, [&](auto dc) {
    const auto code = MortonSpec<decltype(dc)::value>::encode(c);
    *lo = (uint64_t)code;
    *hi = (uint64_t)((u128)code >> 64);
  });
  return ok ? 0 : 22;
}

uint64_t orc_morton2(uint32_t a, uint32_t b) {
  uint32_t c[2] = {a, b};
  return encode2(c);
}
uint64_t orc_morton3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t q[3] = {a, b, c};
  return encode3(q);
}
uint32_t orc_quantize_f32(float v, float mn, float inv_scale, uint32_t max_bucket) {
  return quantize_axis<float>(v, mn, inv_scale, max_bucket);
}
int64_t orc_next_smooth(int64_t n) { return next_smooth(n); }

// Circular convolution through the oracle FFT, for the FFT known-answer tests
// (round trip and convolution against a direct sum, src/tsne/fft.rs:255-333).
void orc_fft_f64(double* re, double* im, int32_t len, int32_t dims, int32_t inverse) {
  int64_t total = dims == 1 ? len : (int64_t)len * len;
  std::vector<std::complex<double>> g(total);
  for (int64_t e = 0; e < total; ++e) g[e] = {re[e], im[e]};
  Fft1<double> f;
  f.plan(len);
  fft_nd(g, len, dims, inverse != 0, f);
  for (int64_t e = 0; e < total; ++e) {
    re[e] = g[e].real();
    im[e] = g[e].imag();
  }
}

void orc_lagrange_weights(double local, double* out3) {
  Lagrange<double> b;
  b.weights(local, out3);
}

// ---- builder handle --------------------------------------------------------
struct orc_tsne {
  int dtype;
  void* impl;
};

orc_tsne* orc_tsne_new(int dtype, int32_t D, int64_t n) {
  orc_tsne* h = new orc_tsne;
  h->dtype = dtype;
  if (dtype == 0) h->impl = new TSNE<float>(D, n);
  else h->impl = new TSNE<double>(D, n);
  return h;
}

void orc_tsne_free(orc_tsne* h) {
  if (!h) return;
  if (h->dtype == 0) delete (TSNE<float>*)h->impl;
  else delete (TSNE<double>*)h->impl;
  delete h;
}

#define ORC_H(h, ...)                          \
  do {                                         \
    if ((h)->dtype == 0) {                     \
      typedef float T;                         \
      TSNE<T>* t = (TSNE<T>*)(h)->impl;        \
      __VA_ARGS__;                             \
    } else {                                   \
      typedef double T;                        \
      TSNE<T>* t = (TSNE<T>*)(h)->impl;        \
      __VA_ARGS__;                             \
    }                                          \
  } while (0)

const char* orc_tsne_last_error(orc_tsne* h) {
  const char* m = "";
  ORC_H(h, m = t->st.msg.c_str());
  return m;
}

// Setters mirror src/lib.rs:277-435; `what` names the field.
int orc_tsne_set(orc_tsne* h, const char* what, double v) {
  std::string w(what);
  ORC_H(h, {
    if (w == "learning_rate") {
      t->has_lr = true;
      t->learning_rate = (T)v;
    } else if (w == "epochs") t->epochs = (int64_t)v;
    else if (w == "momentum") t->momentum = (T)v;
    else if (w == "final_momentum") t->final_momentum = (T)v;
    else if (w == "momentum_switch_epoch") t->momentum_switch_epoch = (int64_t)v;
    else if (w == "stop_lying_epoch") t->stop_lying_epoch = (int64_t)v;
    else if (w == "early_exaggeration") t->early_exaggeration = (T)v;
    else if (w == "perplexity") t->perplexity = (T)v;
    else if (w == "seed") t->seed = (uint64_t)v;
    else return 22;
  });
  return 0;
}

double orc_tsne_get(orc_tsne* h, const char* what) {
  std::string w(what);
  double out = NAN;
  ORC_H(h, {
    if (w == "momentum") out = (double)t->momentum;
    else if (w == "perplexity") out = (double)t->perplexity;
    else if (w == "learning_rate") out = (double)t->resolve_lr();
    else if (w == "stop_lying_fired") out = t->stop_lying_fired ? 1.0 : 0.0;
    else if (w == "nnz") out = (double)t->p_values.size();
  });
  return out;
}

void orc_tsne_set_initial_embedding(orc_tsne* h, const void* y, int64_t len) {
  ORC_H(h, {
    t->has_init = true;
    t->initial.assign((const T*)y, (const T*)y + len);
  });
}

void orc_tsne_set_epoch_callback(orc_tsne* h, epoch_cb_t cb, void* user) {
  ORC_H(h, {
    t->cb = cb;
    t->cb_user = user;
  });
}

// method: 1 = exact (X is the dense distance matrix), 2 = Barnes-Hut, 3 = FIt-SNE.
int orc_tsne_fit_euclidean(orc_tsne* h, int method, double theta, const void* X, int32_t dim) {
  int rc = 0;
  ORC_H(h, rc = t->fit_euclidean(method, (T)theta, (const T*)X, dim));
  return rc;
}

int orc_tsne_fit_with_neighbors(orc_tsne* h, int method, double theta, const uint64_t* idx,
                                const void* dist, int64_t rows, int64_t k) {
  int rc = 0;
  ORC_H(h, rc = t->fit_with_neighbors(method, (T)theta, idx, (const T*)dist, rows, k));
  return rc;
}

int orc_tsne_exact(orc_tsne* h, const void* dist_matrix) {
  int rc = 0;
  ORC_H(h, rc = t->exact_with_distances((const T*)dist_matrix));
  return rc;
}

void orc_tsne_embedding(orc_tsne* h, void* out) {
  ORC_H(h, std::copy(t->y.begin(), t->y.end(), (T*)out));
}

int orc_tsne_kl(orc_tsne* h, int quirk, double* out) {
  int has = 0;
  ORC_H(h, {
    T v;
    has = t->kl(quirk != 0, &v) ? 1 : 0;
    if (has) *out = (double)v;
  });
  return has;
}

// affinities(): src/lib.rs:1019-1037. Returns nnz, or -1 when absent.
int64_t orc_tsne_affinities(orc_tsne* h, uint64_t* rows, uint32_t* cols, void* vals, double* perplexity) {
  int64_t nnz = -1;
  ORC_H(h, {
    if (t->p_rows.empty()) return -1;
    nnz = (int64_t)t->p_values.size();
    if (rows) std::copy(t->p_rows.begin(), t->p_rows.end(), rows);
    if (cols) std::copy(t->p_columns.begin(), t->p_columns.end(), cols);
    if (vals) {
      if (t->stop_lying_fired) std::copy(t->p_values.begin(), t->p_values.end(), (T*)vals);
      else {
        T scale = T(1) / t->early_exaggeration;
        for (int64_t e = 0; e < nnz; ++e) ((T*)vals)[e] = t->p_values[e] * scale;
      }
    }
    if (perplexity) *perplexity = (double)t->perplexity;
  });
  return nnz;
}

void orc_tsne_with_affinities(orc_tsne* h, const uint64_t* rows, int64_t n_rows, const uint32_t* cols,
                              const void* vals, int64_t nnz, double perplexity) {
  ORC_H(h, {
    t->perplexity = (T)perplexity;
    t->p_rows.assign(rows, rows + n_rows);
    t->p_columns.assign(cols, cols + nnz);
    t->p_values.assign((const T*)vals, (const T*)vals + nnz);
    t->has_cached_perplexity = true;
    t->cached_perplexity = t->perplexity;
  });
}

// Copies the current P values (as stored, exaggeration included) for tests.
int64_t orc_tsne_p_values(orc_tsne* h, void* vals) {
  int64_t nnz = 0;
  ORC_H(h, {
    nnz = (int64_t)t->p_values.size();
    if (vals) std::copy(t->p_values.begin(), t->p_values.end(), (T*)vals);
  });
  return nnz;
}

}  // extern "C"
