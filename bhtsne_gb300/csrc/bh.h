// Barnes-Hut tree types and launchers (see bh.cu for the algorithm).
#pragma once

#include <type_traits>

#include "internal.h"

namespace bhg {

// Per-epoch box parameters, written on the device by the bounding-box kernel.
template <class T>
struct BoxParams {
  T mn[8];
  T mx[8];
  T inv_scale[8];
  T max_extent;
  T hw2[40];  // squared half width per level, src/tsne/arena.rs:167-174
};

template <class T>
struct alignas(16) Quad {
  T x, y, z, w;
};

// Packed level + skip word: internal nodes hold (skip << 5) | level, leaves
// hold all ones (their skip is always index + 1 and they have no level). Five
// bits cover every level (at most 31, for D = 2); 27 bits of skip bound the
// arena at 2^27 - 1 nodes, i.e. N < 2^26 points.
constexpr uint32_t kLeafWord = 0xffffffffu;
constexpr int64_t kMaxTreePoints = (1LL << 26) - 1;

template <class T>
struct alignas(16) Node2 {
  T x, y, mass;
  typename std::conditional<sizeof(T) == 4, uint32_t, uint64_t>::type w;
};

// Node storage, depth-first preorder. D = 2: one 16-byte (f32) record
// {x, y, mass, word}, a single load per visit. D = 3: {x, y, z, mass} plus a
// separate word array. D = 4..7: {centre[D], mass} padded to 8 values plus a
// word array. The squared half width of an internal node's level is read from
// a per-launch table (BoxParams::hw2, staged in shared memory).
template <class T>
struct alignas(8 * sizeof(T)) Oct {
  T v[8];
};

template <class T, int D>
struct TreeNodes {
  static_assert(D >= 4 && D <= 7, "generic node layout is for D = 4..7");
  Oct<T>* geom;
  uint32_t* words;
  const T* hw2;
  struct Raw {
    Oct<T> g;
    uint32_t w;
  };
  __device__ __forceinline__ Raw load(uint32_t i) const {
    Raw r;
    r.g = geom[i];
    r.w = words[i];
    return r;
  }
  __device__ __forceinline__ uint32_t word(const Raw& r) const { return r.w; }
  __device__ __forceinline__ void decode(const Raw& r, T* c, T* mass, T* r2) const {
#pragma unroll
    for (int a = 0; a < D; ++a) c[a] = r.g.v[a];
    *mass = r.g.v[D];
    *r2 = r.w == kLeafWord ? T(-1) : hw2[r.w & 31u];
  }
  __device__ __forceinline__ void write(int64_t i, const T* c, T mass, int level, uint32_t sk) const {
    Oct<T> g;
#pragma unroll
    for (int a = 0; a < 8; ++a) g.v[a] = a < D ? c[a < D ? a : 0] : (a == D ? mass : T(0));
    geom[i] = g;
    words[i] = level < 0 ? kLeafWord : ((sk << 5) | (uint32_t)level);
  }
};

template <class T>
struct TreeNodes<T, 2> {
  Node2<T>* geom;
  const T* hw2;  // shared-memory copy of BoxParams::hw2 inside the traversal
  typedef Node2<T> Raw;
  __device__ __forceinline__ Raw load(uint32_t i) const { return geom[i]; }
  __device__ __forceinline__ uint32_t word(const Raw& r) const { return (uint32_t)r.w; }
  __device__ __forceinline__ void decode(const Raw& g, T* c, T* mass, T* r2) const {
    c[0] = g.x;
    c[1] = g.y;
    *mass = g.mass;
    const uint32_t w = (uint32_t)g.w;
    *r2 = w == kLeafWord ? T(-1) : hw2[w & 31u];
  }
  __device__ __forceinline__ void write(int64_t i, const T* c, T mass, int level, uint32_t sk) const {
    Node2<T> g;
    g.x = c[0];
    g.y = c[1];
    g.mass = mass;
    g.w = level < 0 ? kLeafWord : ((sk << 5) | (uint32_t)level);
    geom[i] = g;
  }
  __device__ __forceinline__ void read(uint32_t i, T* c, T* mass, T* r2, uint32_t* sk) const {
    const Node2<T> g = geom[i];
    c[0] = g.x;
    c[1] = g.y;
    *mass = g.mass;
    const uint32_t w = (uint32_t)g.w;
    const bool leaf = w == kLeafWord;
    *r2 = leaf ? T(-1) : hw2[w & 31u];
    *sk = leaf ? i + 1 : (w >> 5);
  }
};

template <class T>
struct TreeNodes<T, 3> {
  Quad<T>* geom;
  uint32_t* words;
  const T* hw2;
  struct Raw {
    Quad<T> g;
    uint32_t w;
  };
  __device__ __forceinline__ Raw load(uint32_t i) const {
    Raw r;
    r.g = geom[i];
    r.w = words[i];
    return r;
  }
  __device__ __forceinline__ uint32_t word(const Raw& r) const { return r.w; }
  __device__ __forceinline__ void decode(const Raw& r, T* c, T* mass, T* r2) const {
    c[0] = r.g.x;
    c[1] = r.g.y;
    c[2] = r.g.z;
    *mass = r.g.w;
    *r2 = r.w == kLeafWord ? T(-1) : hw2[r.w & 31u];
  }
  __device__ __forceinline__ void write(int64_t i, const T* c, T mass, int level, uint32_t sk) const {
    Quad<T> g;
    g.x = c[0];
    g.y = c[1];
    g.z = c[2];
    g.w = mass;
    geom[i] = g;
    words[i] = level < 0 ? kLeafWord : ((sk << 5) | (uint32_t)level);
  }
  __device__ __forceinline__ void read(uint32_t i, T* c, T* mass, T* r2, uint32_t* sk) const {
    const Quad<T> g = geom[i];
    const uint32_t w = words[i];
    c[0] = g.x;
    c[1] = g.y;
    c[2] = g.z;
    *mass = g.w;
    const bool leaf = w == kLeafWord;
    *r2 = leaf ? T(-1) : hw2[w & 31u];
    *sk = leaf ? i + 1 : (w >> 5);
  }
};

// Launch shapes that fix scratch sizes: points per prefix-sum tile of the
// centre-of-mass sums, the most blocks of the bounding-box reduction (it runs
// two per SM, up to this many), and the smallest threads per block of the
// traversal (one Z partial per block).
constexpr int64_t kBhPrefixTile = 2048;
constexpr int64_t kBhBoxBlocksMax = 1024;
constexpr int64_t kBhThreads = 128;

// Bytes of each Barnes-Hut workspace buffer for n points in D dimensions.
// BhWorkspace::reserve requests exactly these, and callers that carve a
// workspace out of fixed memory size their slices from the same table.
struct BhSizes {
  size_t keys, perm, ys, pre, pre_part, mask, cnt, base, geom, word, wide, part, small, params, zpart, zval;
};
template <class T>
constexpr BhSizes bh_sizes(int64_t n, int D) {
  const int64_t nn = n > 1 ? n : 1;
  // one spare node past the largest tree: the traversal loads node i + 1
  // while at the last node i = M - 1
  const int64_t max_nodes = 2 * nn + 1;
  BhSizes z{};
  z.keys = (size_t)nn * 8;
  z.perm = (size_t)nn * 4;
  z.ys = (size_t)nn * D * sizeof(T);
  z.pre = (size_t)(nn + 1) * D * sizeof(double);
  z.pre_part = (size_t)((nn + kBhPrefixTile - 1) / kBhPrefixTile + 1) * D * sizeof(double);
  z.mask = (size_t)nn * 4;
  z.cnt = (size_t)nn * 4;
  z.base = (size_t)(nn + 1) * 8;
  z.geom = (size_t)max_nodes * (D == 2 ? sizeof(Node2<T>) : D == 3 ? sizeof(Quad<T>) : sizeof(Oct<T>));
  z.word = D == 2 ? 0 : (size_t)max_nodes * sizeof(uint32_t);
  z.wide = D >= 5 ? (size_t)nn * 16 : 0;  // also lo_orig and hi_orig at half this each
  z.part = (size_t)kBhBoxBlocksMax * 8 * sizeof(T);
  z.small = 64;
  z.params = sizeof(BoxParams<T>);
  z.zpart = (size_t)((nn + kBhThreads - 1) / kBhThreads + 1) * sizeof(double);
  z.zval = sizeof(double);
  return z;
}

template <class T>
struct BhWorkspace {
  int64_t n = 0;
  int D = 0;
  bool zeroed = false;
  int traverse_threads = 256;  // threads per block of the traversal: 128, 256 or 512
  DevBuf keys, keys_alt, perm, perm_alt, ys, pre, pre_part, mask, cnt, base, geom, word;
  DevBuf wide, lo_orig, hi_orig;  // 128-bit codes (D >= 5): sorted codes and the unsorted halves
  DevBuf seg_tot;                 // per-set coordinate sums (job-relative prefix sums)
  DevBuf part_min, part_max, done, zdone, params, zpart, zval, sort_tmp, scan_tmp;
  void reserve(int64_t n, int D);
  void zero_counters(cudaStream_t s);
  const double* z() const { return static_cast<const double*>(zval.ptr); }
  uint64_t* node_count() const { return static_cast<uint64_t*>(base.ptr) + n; }
};

// Independent point sets laid out back to back (a batch of fits): job[s] is
// the set of sorted position s and off[j]..off[j+1] the positions of set j.
// Both null means one set spanning everything. The tile table cuts every set
// into prefix-sum tiles that start at the set's first position (tile t spans
// tile_start[t]..tile_end[t] of set tile_job[t]; set j owns tiles
// job_tile[j]..job_tile[j+1]), so each set's centres of mass are summed
// exactly as if it were alone (see SegTiles).
struct Segs {
  const uint64_t* job = nullptr;
  const int64_t* off = nullptr;
  const int64_t* tile_start = nullptr;
  const int64_t* tile_end = nullptr;
  const int32_t* tile_job = nullptr;
  const int32_t* job_tile = nullptr;
  int64_t ntiles = 0;
  int K = 0;
};

// Device tile table for Segs, built on the host from the set offsets.
struct SegTiles {
  DevBuf buf;
  int64_t ntiles = 0;
  int K = 0;
  void build(const std::vector<int64_t>& off, cudaStream_t s);
  void fill(Segs& sg) const;
};

// Recentres y by mean_sum/n when apply_mean, then writes BoxParams (bits = Morton
// bits per axis for the tree's half-width table; any value for FIt-SNE).
template <class T>
void launch_recenter_bbox(int D, T* y, int64_t n, const double* mean_sum, bool apply_mean, BhWorkspace<T>& ws,
                          int bits, cudaStream_t s);

// Builds the tree over y (BoxParams must be current).
template <class T>
void bh_build(BhWorkspace<T>& ws, int D, const T* y, int64_t n, cudaStream_t s);

// Tree build from codes already sorted into ws.keys with the point order in
// ws.perm (one forest of independent trees when segs are given).
template <class T>
void bh_build_from_sorted(BhWorkspace<T>& ws, int D, const T* y, int64_t n, const Segs& segs, cudaStream_t s);

// Repulsive forces (neg, original order), optional per-point q, and Z into
// ws.zval. With segs, each query walks only its own set's tree, whose level
// half widths come from boxes[set].
template <class T>
void bh_traverse(BhWorkspace<T>& ws, int D, const T* y, int64_t n, T theta, T* neg, T* qout, cudaStream_t s,
                 const Segs& segs = Segs(), const BoxParams<T>* boxes = nullptr);

template <class T>
int bh_bits(int D);

}  // namespace bhg
