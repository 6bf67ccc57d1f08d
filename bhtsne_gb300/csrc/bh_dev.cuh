// Device helpers shared by the single-fit and batched Barnes-Hut builds:
// Morton codecs (src/tsne/morton/d2.rs:5-47, d3.rs:5-50, d4.rs:5-45 and the
// 128-bit codecs of d5.rs-d7.rs), quantisation (src/tsne/morton.rs:103-120),
// and the Morton-cell range search used by the parallel tree construction.
#pragma once

#include "bh.h"

namespace bhg {

typedef unsigned __int128 u128;

// Bits per axis and code word per output dimension, as in the reference:
// D = 2: 32 bits (u64), 3: 21 (u64), 4: 16 (u64), 5: 25, 6: 21, 7: 18 (u128).
// Bit b of axis a lands at code bit b * D + a (axis 0 least significant).
template <int D>
struct MortonD;
template <>
struct MortonD<2> {
  static constexpr int BITS = 32;
  typedef uint64_t Code;
  __device__ static uint64_t part(uint64_t x) {
    x &= 0x00000000ffffffffULL;
    x = (x | (x << 16)) & 0x0000ffff0000ffffULL;
    x = (x | (x << 8)) & 0x00ff00ff00ff00ffULL;
    x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0fULL;
    x = (x | (x << 2)) & 0x3333333333333333ULL;
    return (x | (x << 1)) & 0x5555555555555555ULL;
  }
  __device__ static Code encode(const uint32_t* c) { return part(c[0]) | (part(c[1]) << 1); }
};
template <>
struct MortonD<3> {
  static constexpr int BITS = 21;
  typedef uint64_t Code;
  __device__ static uint64_t part(uint64_t x) {
    x &= 0x1fffffULL;
    x = (x | (x << 32)) & 0x001f00000000ffffULL;
    x = (x | (x << 16)) & 0x001f0000ff0000ffULL;
    x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
    return (x | (x << 2)) & 0x1249249249249249ULL;
  }
  __device__ static Code encode(const uint32_t* c) {
    return part(c[0]) | (part(c[1]) << 1) | (part(c[2]) << 2);
  }
};
template <>
struct MortonD<4> {
  static constexpr int BITS = 16;
  typedef uint64_t Code;
  // 16 bits spread to every fourth bit.
  __device__ static uint64_t part(uint64_t x) {
    x &= 0xffffULL;
    x = (x | (x << 24)) & 0x000000ff000000ffULL;
    x = (x | (x << 12)) & 0x000f000f000f000fULL;
    x = (x | (x << 6)) & 0x0303030303030303ULL;
    return (x | (x << 3)) & 0x1111111111111111ULL;
  }
  __device__ static Code encode(const uint32_t* c) {
    return part(c[0]) | (part(c[1]) << 1) | (part(c[2]) << 2) | (part(c[3]) << 3);
  }
};
template <int D, int B>
struct MortonWide {
  static constexpr int BITS = B;
  typedef u128 Code;
  __device__ static Code encode(const uint32_t* c) {
    uint64_t lo = 0, hi = 0;
#pragma unroll
    for (int b = 0; b < B; ++b)
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const int pos = b * D + a;
        const uint64_t bit = (c[a] >> b) & 1u;
        if (pos < 64) lo |= bit << pos;
        else hi |= bit << (pos - 64);
      }
    return ((u128)hi << 64) | (u128)lo;
  }
};
template <>
struct MortonD<5> : MortonWide<5, 25> {};
template <>
struct MortonD<6> : MortonWide<6, 21> {};
template <>
struct MortonD<7> : MortonWide<7, 18> {};

__device__ __forceinline__ int msb_pos(uint64_t x) { return 63 - __clzll((long long)x); }
__device__ __forceinline__ int msb_pos(u128 x) {
  const uint64_t hi = (uint64_t)(x >> 64);
  return hi ? 64 + msb_pos(hi) : msb_pos((uint64_t)x);
}

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

template <class C>
__device__ __forceinline__ int64_t lower_bound_code(const C* __restrict__ c, int64_t lo, int64_t hi, C key) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (c[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Level at which two distinct codes part: the depth of their deepest common cell.
template <int D>
__device__ __forceinline__ int boundary_level(typename MortonD<D>::Code c0, typename MortonD<D>::Code c1) {
  constexpr int B = MortonD<D>::BITS;
  return (B - 1) - msb_pos(c0 ^ c1) / D;
}

// First index in [lo, s] whose code is >= key, given codes[s] >= key: a
// galloping search leftwards from s (about 2 log2 of the distance probes,
// the same answer as a binary search over [lo, s]).
template <class C>
__device__ __forceinline__ int64_t gallop_down(const C* __restrict__ c, int64_t lo, int64_t s, C key) {
  int64_t good = s, bad = lo - 1, step = 1;
  while (good - step >= lo) {
    const int64_t probe = good - step;
    if (c[probe] < key) {
      bad = probe;
      break;
    }
    good = probe;
    step <<= 1;
  }
  return lower_bound_code<C>(c, bad + 1, good, key);
}

// First index in (s, hi) whose code is >= key, or hi, given codes[s] < key:
// a galloping search rightwards from s.
template <class C>
__device__ __forceinline__ int64_t gallop_up(const C* __restrict__ c, int64_t s, int64_t hi, C key) {
  int64_t bad = s, good = hi, step = 1;
  while (bad + step < hi) {
    const int64_t probe = bad + step;
    if (c[probe] >= key) {
      good = probe;
      break;
    }
    bad = probe;
    step <<= 1;
  }
  return lower_bound_code<C>(c, bad + 1, good, key);
}

// Range [a, e) of the depth-l Morton cell holding code c = codes[s], within
// [lo, hi): galloping searches outwards from s. With need_end false only *a
// is computed.
template <int D>
__device__ __forceinline__ void cell_range_near(const typename MortonD<D>::Code* __restrict__ codes, int64_t lo,
                                                int64_t hi, typename MortonD<D>::Code c, int l, int64_t s,
                                                int64_t* a, int64_t* e, bool need_end) {
  typedef typename MortonD<D>::Code Code;
  constexpr int B = MortonD<D>::BITS;
  if (l == 0) {
    *a = lo;
    *e = hi;
    return;
  }
  const int shift = D * (B - l);
  const Code prefix = c >> shift;
  *a = gallop_down<Code>(codes, lo, s, prefix << shift);
  if (!need_end) return;
  const Code limit = ~(Code)0 >> shift;  // largest prefix representable
  if (prefix >= limit) *e = hi;
  else *e = gallop_up<Code>(codes, s, hi, (prefix + 1) << shift);
}

}  // namespace bhg
