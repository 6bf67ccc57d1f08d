// Barnes-Hut tree types and launchers (see bh.cu for the algorithm).
#pragma once

#include <type_traits>

#include "internal.h"

namespace bhg {

// Per-epoch box parameters, written on the device by the bounding-box kernel.
template <class T>
struct BoxParams {
  T mn[3];
  T mx[3];
  T inv_scale[3];
  T max_extent;
  T hw2[40];  // squared half width per level, src/tsne/arena.rs:167-174
};

template <class T>
struct alignas(16) Quad {
  T x, y, z, w;
};

template <class T>
struct RSkip {
  T r2;
  uint32_t skip;
};

// Node storage, depth-first preorder. D = 2: geom = {x, y, mass, r2} plus a
// skip array. D = 3: geom = {x, y, z, mass} plus {r2, skip}. r2 < 0 marks a
// leaf; r2 >= 0 is the half-width^2 of the node's level.
template <class T, int D>
struct TreeNodes;

template <class T>
struct TreeNodes<T, 2> {
  Quad<T>* geom;
  uint32_t* skip;
  __device__ __forceinline__ void write(int64_t i, const T* c, T mass, T r2, uint32_t sk) const {
    Quad<T> g;
    g.x = c[0];
    g.y = c[1];
    g.z = mass;
    g.w = r2;
    geom[i] = g;
    skip[i] = sk;
  }
  __device__ __forceinline__ void read(uint32_t i, T* c, T* mass, T* r2, uint32_t* sk) const {
    const Quad<T> g = geom[i];
    *sk = __ldg(skip + i);
    c[0] = g.x;
    c[1] = g.y;
    *mass = g.z;
    *r2 = g.w;
  }
};

template <class T>
struct TreeNodes<T, 3> {
  Quad<T>* geom;
  RSkip<T>* rs;
  __device__ __forceinline__ void write(int64_t i, const T* c, T mass, T r2, uint32_t sk) const {
    Quad<T> g;
    g.x = c[0];
    g.y = c[1];
    g.z = c[2];
    g.w = mass;
    geom[i] = g;
    RSkip<T> r;
    r.r2 = r2;
    r.skip = sk;
    rs[i] = r;
  }
  __device__ __forceinline__ void read(uint32_t i, T* c, T* mass, T* r2, uint32_t* sk) const {
    const Quad<T> g = geom[i];
    const RSkip<T> r = rs[i];
    c[0] = g.x;
    c[1] = g.y;
    c[2] = g.z;
    *mass = g.w;
    *r2 = r.r2;
    *sk = r.skip;
  }
};

template <class T>
struct BhWorkspace {
  int64_t n = 0;
  int D = 0;
  bool zeroed = false;
  DevBuf keys, keys_alt, perm, perm_alt, ys, pre, pre_part, mask, cnt, base, geom, aux;
  DevBuf part_min, part_max, done, zdone, params, zpart, zval, sort_tmp, scan_tmp;
  void reserve(int64_t n, int D);
  const double* z() const { return static_cast<const double*>(zval.ptr); }
  uint64_t* node_count() const { return static_cast<uint64_t*>(base.ptr) + n; }
};

// Recentres y by mean_sum/n when apply_mean, then writes BoxParams (bits = Morton
// bits per axis for the tree's half-width table; any value for FIt-SNE).
template <class T>
void launch_recenter_bbox(int D, T* y, int64_t n, const double* mean_sum, bool apply_mean, BhWorkspace<T>& ws,
                          int bits, cudaStream_t s);

// Builds the tree over y (BoxParams must be current).
template <class T>
void bh_build(BhWorkspace<T>& ws, int D, const T* y, int64_t n, cudaStream_t s);

// Repulsive forces (neg, original order), optional per-point q, and Z into ws.zval.
template <class T>
void bh_traverse(BhWorkspace<T>& ws, int D, const T* y, int64_t n, T theta, T* neg, T* qout, cudaStream_t s);

template <class T>
int bh_bits(int D);

}  // namespace bhg
