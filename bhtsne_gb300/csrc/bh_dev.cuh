// Device helpers shared by the single-fit and batched Barnes-Hut builds:
// Morton codecs (src/tsne/morton/d2.rs:5-47, d3.rs:5-50), quantisation
// (src/tsne/morton.rs:103-120), and the Morton-cell range search used by the
// parallel tree construction.
#pragma once

#include "bh.h"

namespace bhg {

template <int D>
struct MortonD;
template <>
struct MortonD<2> {
  static constexpr int BITS = 32;
  __device__ static uint64_t part(uint64_t x) {
    x &= 0x00000000ffffffffULL;
    x = (x | (x << 16)) & 0x0000ffff0000ffffULL;
    x = (x | (x << 8)) & 0x00ff00ff00ff00ffULL;
    x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0fULL;
    x = (x | (x << 2)) & 0x3333333333333333ULL;
    return (x | (x << 1)) & 0x5555555555555555ULL;
  }
  __device__ static uint64_t encode(const uint32_t* c) { return part(c[0]) | (part(c[1]) << 1); }
};
template <>
struct MortonD<3> {
  static constexpr int BITS = 21;
  __device__ static uint64_t part(uint64_t x) {
    x &= 0x1fffffULL;
    x = (x | (x << 32)) & 0x001f00000000ffffULL;
    x = (x | (x << 16)) & 0x001f0000ff0000ffULL;
    x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
    return (x | (x << 2)) & 0x1249249249249249ULL;
  }
  __device__ static uint64_t encode(const uint32_t* c) {
    return part(c[0]) | (part(c[1]) << 1) | (part(c[2]) << 2);
  }
};

template <class T>
__device__ __forceinline__ uint32_t quantize(T v, T mn, T inv_scale, uint32_t max_bucket) {
  const T scaled = floor((v - mn) * inv_scale);
  if (scaled > T(0)) {
    if (!(scaled < T(18446744073709551616.0))) return max_bucket;
    const uint64_t q = (uint64_t)scaled;
    return q < (uint64_t)max_bucket ? (uint32_t)q : max_bucket;
  }
  return 0u;
}

__device__ __forceinline__ int64_t lower_bound_u64(const uint64_t* __restrict__ c, int64_t lo, int64_t hi,
                                                   uint64_t key) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (c[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <int D>
__device__ __forceinline__ int boundary_level(uint64_t c0, uint64_t c1) {
  constexpr int B = MortonD<D>::BITS;
  const int highest = 63 - __clzll((long long)(c0 ^ c1));
  return (B - 1) - highest / D;
}

// Range [a, e) of the depth-l Morton cell holding code c.
// Range [a, e) of the depth-l Morton cell holding code c, searched within [lo, hi).
template <int D>
__device__ __forceinline__ void cell_range_in(const uint64_t* __restrict__ codes, int64_t lo, int64_t hi,
                                              uint64_t c, int l, int64_t* a, int64_t* e) {
  constexpr int B = MortonD<D>::BITS;
  if (l == 0) {
    *a = lo;
    *e = hi;
    return;
  }
  const int shift = D * (B - l);
  const uint64_t prefix = c >> shift;
  *a = lower_bound_u64(codes, lo, hi, prefix << shift);
  const uint64_t limit = ~0ULL >> shift;
  if (prefix >= limit) *e = hi;
  else *e = lower_bound_u64(codes, *a, hi, (prefix + 1) << shift);
}

template <int D>
__device__ __forceinline__ void cell_range(const uint64_t* __restrict__ codes, int64_t n, uint64_t c, int l,
                                           int64_t* a, int64_t* e) {
  constexpr int B = MortonD<D>::BITS;
  if (l == 0) {
    *a = 0;
    *e = n;
    return;
  }
  const int shift = D * (B - l);
  const uint64_t prefix = c >> shift;
  *a = lower_bound_u64(codes, 0, n, prefix << shift);
  const uint64_t limit = ~0ULL >> shift;  // largest prefix representable
  if (prefix >= limit) *e = n;
  else *e = lower_bound_u64(codes, *a, n, (prefix + 1) << shift);
}


}  // namespace bhg
