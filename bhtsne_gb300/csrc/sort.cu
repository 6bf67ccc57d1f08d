// Device-wide exclusive scans and a stable LSD radix sort of (u64 key, payload)
// pairs. Used every Barnes-Hut epoch to put the Morton codes in Z-order (the
// role of `par_sort_unstable_by_key` at src/tsne/arena.rs:191 of the
// reference) and once per fit to order the symmetric affinity entries.
//
// The sort takes 8-bit digits over tiles of 2048 keys, three kernels a pass:
//  * a histogram per tile (warp-aggregated shared atomics) that also adds
//    its counts into per-super-tile totals (32 tiles each, digit-major);
//  * an exclusive scan of the super-tile totals (one block while the table
//    is small), which also clears them for the next pass;
//  * a scatter: each tile adds the counts of the earlier tiles of its super
//    tile to get its output offsets, ranks its keys stably in shared memory
//    (each warp with __match_any_sync, then one prefix over warps and
//    digits) and writes them out in sorted order, so that each digit's run
//    is one contiguous, coalesced store.
//
// From 131,072 keys (the Morton codes of a large fit, every epoch) a pass is
// one kernel instead: one histogram kernel first counts every pass's digits
// (the key multiset is the same in every pass), and in each pass a tile takes
// its number from an atomic counter, counts its digits, publishes them, and
// learns the counts of all earlier tiles by decoupled look-back (Merrill and
// Garland's single-pass prefix scan): it walks back over the earlier tiles'
// published words, adding aggregates until it meets an inclusive prefix.
// Tiles are numbered in the order blocks start, so every tile a block waits
// on belongs to a block already running. Every wait is bounded; a wait that
// runs out raises the library's sort fault word (radix_sort_fault_take)
// instead of hanging.
#include <cstdlib>

#include "internal.h"

namespace bhg {

namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class In>
__global__ void scan_reduce_kernel(const In* __restrict__ in, int64_t n, uint64_t* __restrict__ partial) {
  __shared__ double sh_unused[1];
  (void)sh_unused;
  __shared__ uint64_t warp_tot[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int64_t p = base + (int64_t)i * kScanThreads + threadIdx.x;
    if (p < n) s += (uint64_t)in[p];
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint64_t v = threadIdx.x < kScanThreads / 32 ? warp_tot[threadIdx.x] : 0;
    v = warp_sum(v);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
  }
}

// Exclusive scan of the per-tile partials by one block, carrying across chunks.
__global__ void scan_partials_kernel(uint64_t* __restrict__ partial, int64_t nparts, uint64_t* __restrict__ total) {
  __shared__ uint64_t warp_tot[32];
  __shared__ uint64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t c0 = 0; c0 < nparts; c0 += blockDim.x) {
    int64_t p = c0 + threadIdx.x;
    uint64_t v = p < nparts ? partial[p] : 0;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      const int nw = blockDim.x >> 5;
      uint64_t t = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(kFull, t, o);
        if (lane >= o) t += y;
      }
      if (lane < nw) warp_tot[lane] = t;
    }
    __syncthreads();
    uint64_t excl = x - v + (w > 0 ? warp_tot[w - 1] : 0) + carry;
    if (p < nparts) partial[p] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

template <class In>
__global__ void scan_apply_kernel(const In* __restrict__ in, uint64_t* __restrict__ out, int64_t n,
                                  const uint64_t* __restrict__ partial) {
  __shared__ uint64_t warp_tot[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint64_t v[kScanItems];
  uint64_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int64_t p = base + i;
    v[i] = p < n ? (uint64_t)in[p] : 0;
    s += v[i];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint64_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    uint64_t t = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint64_t y = __shfl_up_sync(kFull, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  uint64_t run = x - s + (w > 0 ? warp_tot[w - 1] : 0) + partial[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int64_t p = base + i;
    if (p < n) out[p] = run;
    run += v[i];
  }
}

// Blocked layout: each thread owns kScanItems consecutive inputs (scan_apply)
// while scan_reduce reads strided; both cover the same tile, so the tile sums agree.
template <class In>
void scan_impl(const In* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  const int64_t nb = ceil_div(n, kScanTile);
  uint64_t* partial = static_cast<uint64_t*>(tmp.ensure((size_t)(nb + 1) * sizeof(uint64_t)));
  if (n > 0) {
    scan_reduce_kernel<In><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, partial);
    BHG_LAUNCH_CHECK();
  }
  scan_partials_kernel<<<1, 1024, 0, s>>>(partial, nb, out + n);
  BHG_LAUNCH_CHECK();
  if (n > 0) {
    scan_apply_kernel<In><<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, partial);
    BHG_LAUNCH_CHECK();
  }
}

// ---------------------------------------------------------------------------
// radix sort
// ---------------------------------------------------------------------------
constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsRounds = 8;                       // rounds of 32 keys per warp
constexpr int kRsWarpSpan = 32 * kRsRounds;        // 256 consecutive keys per warp
constexpr int kRsTile = kRsThreads * kRsRounds;    // 2048 keys per tile
constexpr int kRsSup = 32;                         // tiles per super-tile
constexpr int kRsInlineSup = 32;                   // up to this many super-tiles, the scatter scans them itself
constexpr int kSpineThreads = 1024;
constexpr int64_t kSpineMax = (int64_t)1 << 16;    // largest super-tile table scanned by one block

// Per-tile digit counts (tile-major: counts[b * 256 + d]), also added into
// the super-tile totals sup[d * ns + b / kRsSup].
__global__ void __launch_bounds__(kRsThreads) rs_hist_kernel(const uint64_t* __restrict__ keys, int64_t n, int shift,
                                                             uint32_t* __restrict__ counts, uint32_t* __restrict__ sup,
                                                             int64_t ns) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
#pragma unroll
  for (int i = 0; i < kRsRounds; ++i) {
    const int64_t p = base + (int64_t)i * kRsThreads + threadIdx.x;
    const unsigned d = p < n ? ((unsigned)(keys[p] >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(kFull, d);
    if (d < 256u && lane == __ffs(peers) - 1) atomicAdd(&h[d], (unsigned)__popc(peers));
  }
  __syncthreads();
  const uint32_t c = h[threadIdx.x];
  counts[(int64_t)blockIdx.x * 256 + threadIdx.x] = c;
  if (c) atomicAdd(&sup[(int64_t)threadIdx.x * ns + blockIdx.x / kRsSup], c);
}

// Exclusive scan of m u32 values into u64 offsets by one block, in coalesced
// rounds of 1024; clears the input afterwards when `clear` is set.
__global__ void __launch_bounds__(kSpineThreads) rs_spine_kernel(uint32_t* __restrict__ vals, int64_t m,
                                                                 uint64_t* __restrict__ offsets, int clear) {
  __shared__ uint64_t wt[kSpineThreads / 32];
  __shared__ uint64_t carry;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t r0 = 0; r0 < m; r0 += kSpineThreads) {
    const int64_t i = r0 + threadIdx.x;
    const uint64_t v = i < m ? vals[i] : 0;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wt[w] = x;
    __syncthreads();
    if (w == 0) {
      uint64_t t = wt[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(kFull, t, o);
        if (lane >= o) t += y;
      }
      wt[lane] = t;
    }
    __syncthreads();
    const uint64_t c0 = carry;
    if (i < m) {
      offsets[i] = c0 + x - v + (w > 0 ? wt[w - 1] : 0);
      if (clear) vals[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry = c0 + wt[31];
    __syncthreads();
  }
}

template <class V>
struct RsSmem {
  uint64_t key[kRsTile];
  V val[kRsTile];
  uint32_t wcnt[kRsWarps][256];  // per warp and digit: count, then exclusive offset within the digit
  uint32_t tstart[256];          // first position of each digit in the sorted tile
  uint64_t gbase[256];           // first output position of the tile's keys of each digit
  uint32_t wtot[kRsWarps];
};

// One pass over tile blockIdx.x: output offsets from the super-tile prefix
// and the earlier tiles of the super-tile, a stable rank in shared memory,
// and a coalesced write-out.
template <class V>
__global__ void __launch_bounds__(kRsThreads, 4) rs_scatter_kernel(const uint64_t* __restrict__ kin, const V* __restrict__ vin,
                                                                uint64_t* __restrict__ kout, V* __restrict__ vout, int64_t n,
                                                                int shift, const uint32_t* __restrict__ counts,
                                                                const uint64_t* __restrict__ sup_off,
                                                                const uint32_t* __restrict__ sup, int64_t ns,
                                                                uint32_t* __restrict__ sup_clear) {
  __shared__ RsSmem<V> sm;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t b = blockIdx.x;
  const int64_t tile = b * kRsTile;
  const int64_t wbase = tile + (int64_t)w * kRsWarpSpan;
  uint64_t k[kRsRounds];
  V v[kRsRounds];
  uint32_t rk[kRsRounds];
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t p = wbase + r * 32 + lane;
    k[r] = 0;
    v[r] = V{};
    if (p < n) {
      k[r] = kin[p];
      v[r] = vin[p];
    }
  }
  {
    const int64_t s0 = (b / kRsSup) * kRsSup;
    const int nq = (int)(b - s0);
    uint64_t g;
    if (sup_off) {
      g = sup_off[(int64_t)tid * ns + b / kRsSup];
    } else {
      // few super-tiles: digit totals, their exclusive scan over the block,
      // and this digit's earlier super-tiles
      const int S = (int)(b / kRsSup);
      uint32_t st[kRsInlineSup];
#pragma unroll
      for (int q = 0; q < kRsInlineSup; ++q) st[q] = q < ns ? sup[(int64_t)tid * ns + q] : 0u;
      uint32_t tot = 0, pre = 0;
#pragma unroll
      for (int q = 0; q < kRsInlineSup; ++q) {
        tot += st[q];
        pre += q < S ? st[q] : 0u;
      }
      uint32_t x = tot;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) sm.wtot[w] = x;
      __syncthreads();
      uint32_t add = 0;
      for (int q = 0; q < w; ++q) add += sm.wtot[q];
      g = (uint64_t)(x - tot + add) + pre;
      __syncthreads();
      if (b == 0 && sup_clear)
        for (int64_t i = tid; i < 256 * ns; i += kRsThreads) sup_clear[i] = 0;
    }
    uint32_t c[kRsSup - 1];
#pragma unroll
    for (int q = 0; q < kRsSup - 1; ++q) c[q] = q < nq ? counts[(s0 + q) * 256 + tid] : 0u;
#pragma unroll
    for (int q = 0; q < kRsSup - 1; ++q) g += c[q];
    sm.gbase[tid] = g;
  }
#pragma unroll
  for (int q = 0; q < kRsWarps; ++q) sm.wcnt[q][tid] = 0;
  __syncthreads();
  // rank among the warp's earlier keys of the same digit (round r, lane l is
  // key wbase + 32 r + l: input order)
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t p = wbase + r * 32 + lane;
    const unsigned d = p < n ? ((unsigned)(k[r] >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(kFull, d);
    const uint32_t prior = d < 256u ? sm.wcnt[w][d] : 0u;
    __syncwarp();
    if (d < 256u && lane == __ffs(peers) - 1) sm.wcnt[w][d] = prior + (uint32_t)__popc(peers);
    __syncwarp();
    rk[r] = prior + (uint32_t)__popc(peers & lt);
  }
  __syncthreads();
  // thread tid owns digit tid: offsets across warps, then the digit starts
  {
    uint32_t tot = 0;
#pragma unroll
    for (int q = 0; q < kRsWarps; ++q) {
      const uint32_t c = sm.wcnt[q][tid];
      sm.wcnt[q][tid] = tot;
      tot += c;
    }
    uint32_t x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sm.wtot[w] = x;
    __syncthreads();
    uint32_t add = 0;
    for (int q = 0; q < w; ++q) add += sm.wtot[q];
    sm.tstart[tid] = x - tot + add;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t p = wbase + r * 32 + lane;
    if (p < n) {
      const unsigned d = (unsigned)(k[r] >> shift) & 255u;
      const uint32_t lp = sm.tstart[d] + sm.wcnt[w][d] + rk[r];
      sm.key[lp] = k[r];
      sm.val[lp] = v[r];
    }
  }
  __syncthreads();
  // write out in sorted order: consecutive positions of a digit go to
  // consecutive output positions
  const int64_t left = n - tile;
  const int cnt = left < kRsTile ? (int)left : kRsTile;
#pragma unroll 4
  for (int i = tid; i < cnt; i += kRsThreads) {
    const uint64_t key = sm.key[i];
    const unsigned d = (unsigned)(key >> shift) & 255u;
    const uint64_t gp = sm.gbase[d] + (uint64_t)(i - (int)sm.tstart[d]);
    kout[gp] = key;
    vout[gp] = sm.val[i];
  }
}

// ---- single-pass variant -------------------------------------------------------
__device__ uint32_t g_radix_fault;  // raised by a look-back wait that ran out

constexpr uint32_t kOsAgg = 1u << 30;  // word holds the tile's own count
constexpr uint32_t kOsInc = 2u << 30;  // word holds the inclusive prefix through the tile
constexpr uint32_t kOsMask = (1u << 30) - 1u;
constexpr long long kOsSpinLimit = 1LL << 22;
constexpr int kOsMaxPass = 8;
constexpr int kOsLook = 8;  // earlier tiles' words a look-back step loads at once

// Digit counts of passes 0 .. npass-1 (digit shift begin_bit + 8 q) in one read.
__global__ void __launch_bounds__(256) os_hist_kernel(const uint64_t* __restrict__ keys, int64_t n, int begin_bit,
                                                      int npass, uint32_t* __restrict__ ghist) {
  __shared__ uint32_t h[kOsMaxPass][256];
  for (int i = threadIdx.x; i < kOsMaxPass * 256; i += blockDim.x) h[i / 256][i % 256] = 0;
  __syncthreads();
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[p];
    for (int q = 0; q < npass; ++q) atomicAdd(&h[q][(unsigned)(k >> (begin_bit + 8 * q)) & 255u], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < npass * 256; i += blockDim.x) {
    const uint32_t c = h[i / 256][i % 256];
    if (c) atomicAdd(&ghist[i], c);
  }
}

// Exclusive scan of each pass's 256 digit counts (block q: pass q).
__global__ void __launch_bounds__(256) os_base_kernel(const uint32_t* __restrict__ ghist, uint32_t* __restrict__ base) {
  __shared__ uint32_t wt[8];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const uint32_t v = ghist[blockIdx.x * 256 + tid];
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wt[w] = x;
  __syncthreads();
  uint32_t add = 0;
  for (int q = 0; q < w; ++q) add += wt[q];
  base[blockIdx.x * 256 + tid] = x - v + add;
}

__device__ __forceinline__ uint32_t os_load(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void os_store(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One pass: tile number from *ticket, stable rank in shared memory as in
// rs_scatter_kernel, output offsets from the pass's digit bases plus the
// counts of the earlier tiles (look-back over status, one word per tile and
// digit), coalesced write-out.
template <class V>
__global__ void __launch_bounds__(kRsThreads, 4) os_pass_kernel(const uint64_t* __restrict__ kin, const V* __restrict__ vin,
                                                             uint64_t* __restrict__ kout, V* __restrict__ vout, int64_t n,
                                                             int shift, const uint32_t* __restrict__ dbase,
                                                             uint32_t* __restrict__ status, uint32_t* __restrict__ ticket) {
  __shared__ RsSmem<V> sm;
  __shared__ uint32_t tile_no;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const unsigned lt = (1u << lane) - 1u;
  if (tid == 0) tile_no = atomicAdd(ticket, 1u);
#pragma unroll
  for (int q = 0; q < kRsWarps; ++q) sm.wcnt[q][tid] = 0;
  __syncthreads();
  const int64_t b = tile_no;
  const int64_t tile = b * kRsTile;
  const int64_t wbase = tile + (int64_t)w * kRsWarpSpan;
  uint64_t k[kRsRounds];
  V v[kRsRounds];
  uint32_t rk[kRsRounds];
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t p = wbase + r * 32 + lane;
    k[r] = 0;
    v[r] = V{};
    if (p < n) {
      k[r] = kin[p];
      v[r] = vin[p];
    }
  }
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t p = wbase + r * 32 + lane;
    const unsigned d = p < n ? ((unsigned)(k[r] >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(kFull, d);
    const uint32_t prior = d < 256u ? sm.wcnt[w][d] : 0u;
    __syncwarp();
    if (d < 256u && lane == __ffs(peers) - 1) sm.wcnt[w][d] = prior + (uint32_t)__popc(peers);
    __syncwarp();
    rk[r] = prior + (uint32_t)__popc(peers & lt);
  }
  __syncthreads();
  // thread tid owns digit tid: the tile's count, offsets across warps
  uint32_t tot = 0;
#pragma unroll
  for (int q = 0; q < kRsWarps; ++q) {
    const uint32_t c = sm.wcnt[q][tid];
    sm.wcnt[q][tid] = tot;
    tot += c;
  }
  // publish, look back, publish the inclusive prefix
  uint32_t* st = status + b * 256 + tid;
  uint32_t excl = 0;
  if (b == 0) {
    os_store(st, kOsInc | tot);
  } else {
    os_store(st, kOsAgg | tot);
    // Walk back kOsLook tiles per step: their words are loaded together, then
    // taken in tile order (a word read early is at worst an aggregate where
    // the tile has since published its prefix: the sum is the same). Tile 0
    // always holds an inclusive prefix, so the walk ends there at the latest.
    bool done = false;
    for (int64_t pb = b - 1; !done; pb -= kOsLook) {
      uint32_t wv[kOsLook];
#pragma unroll
      for (int i = 0; i < kOsLook; ++i) wv[i] = pb - i >= 0 ? os_load(status + (pb - i) * 256 + tid) : kOsInc;
#pragma unroll
      for (int i = 0; i < kOsLook; ++i) {
        if (done) break;
        uint32_t word = wv[i];
        long long spins = 0;
        while ((word & ~kOsMask) == 0u) {
          if (++spins >= kOsSpinLimit) {
            atomicExch(&g_radix_fault, 1u);
            break;
          }
          word = os_load(status + (pb - i) * 256 + tid);
        }
        excl += word & kOsMask;
        done = (word & ~kOsMask) != kOsAgg;  // an inclusive prefix (or a wait that ran out)
      }
    }
    os_store(st, kOsInc | (excl + tot));
  }
  sm.gbase[tid] = (uint64_t)dbase[tid] + excl;
  {
    uint32_t x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sm.wtot[w] = x;
    __syncthreads();
    uint32_t add = 0;
    for (int q = 0; q < w; ++q) add += sm.wtot[q];
    sm.tstart[tid] = x - tot + add;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRsRounds; ++r) {
    const int64_t p = wbase + r * 32 + lane;
    if (p < n) {
      const unsigned d = (unsigned)(k[r] >> shift) & 255u;
      const uint32_t lp = sm.tstart[d] + sm.wcnt[w][d] + rk[r];
      sm.key[lp] = k[r];
      sm.val[lp] = v[r];
    }
  }
  __syncthreads();
  const int64_t left = n - tile;
  const int cnt = left < kRsTile ? (int)left : kRsTile;
#pragma unroll 4
  for (int i = tid; i < cnt; i += kRsThreads) {
    const uint64_t key = sm.key[i];
    const unsigned d = (unsigned)(key >> shift) & 255u;
    const uint64_t gp = sm.gbase[d] + (uint64_t)(i - (int)sm.tstart[d]);
    kout[gp] = key;
    vout[gp] = sm.val[i];
  }
}

}  // namespace

// Bytes the single-pass variant keeps in the sort's scratch: the tickets, the
// digit counts and bases of every pass, then the look-back words of every pass
// (one per tile and digit).
static size_t os_tmp_bytes(int64_t n, int npass) {
  const int64_t nb = ceil_div(n, kRsTile);
  return 256 + (size_t)2 * kOsMaxPass * 256 * 4 + (size_t)npass * nb * 256 * 4;
}

bool radix_sort_fault_take(cudaStream_t s) {
  uint32_t h = 0, zero = 0;
  BHG_CUDA(cudaMemcpyFromSymbolAsync(&h, g_radix_fault, 4, 0, cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaMemcpyToSymbolAsync(g_radix_fault, &zero, 4, 0, cudaMemcpyHostToDevice, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  return h != 0;
}

template <class V>
static void radix_sort_onesweep(uint64_t* keys, V* vals, uint64_t* keys_alt, V* vals_alt, int64_t n, int begin_bit,
                                int end_bit, DevBuf& tmp, cudaStream_t s) {
  const int npass = (end_bit - begin_bit + 7) / 8;
  const int64_t nb = ceil_div(n, kRsTile);
  char* base = static_cast<char*>(tmp.ensure(std::max(os_tmp_bytes(n, npass), radix_sort_tmp_bytes(n))));
  uint32_t* tickets = reinterpret_cast<uint32_t*>(base) + 8;    // words 8 .. 15
  uint32_t* ghist = reinterpret_cast<uint32_t*>(base + 256);
  uint32_t* dbase = ghist + kOsMaxPass * 256;
  uint32_t* status = dbase + kOsMaxPass * 256;
  // tickets, counts and look-back words start at zero (one memset; the fault word is left alone)
  BHG_CUDA(cudaMemsetAsync(tickets, 0, 256 - 32 + (size_t)2 * kOsMaxPass * 256 * 4 + (size_t)npass * nb * 256 * 4, s));
  os_hist_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n, 256), sm_grid(4, 4096)), 256, 0, s>>>(keys, n, begin_bit,
                                                                                               npass, ghist);
  BHG_LAUNCH_CHECK();
  os_base_kernel<<<(unsigned)npass, 256, 0, s>>>(ghist, dbase);
  BHG_LAUNCH_CHECK();
  uint64_t *ki = keys, *ko = keys_alt;
  V *vi = vals, *vo = vals_alt;
  for (int q = 0; q < npass; ++q) {
    os_pass_kernel<V><<<(unsigned)nb, kRsThreads, 0, s>>>(ki, vi, ko, vo, n, begin_bit + 8 * q, dbase + q * 256,
                                                          status + (int64_t)q * nb * 256, tickets + q);
    BHG_LAUNCH_CHECK();
    std::swap(ki, ko);
    std::swap(vi, vo);
  }
  if (npass & 1) {
    BHG_CUDA(cudaMemcpyAsync(keys, ki, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    BHG_CUDA(cudaMemcpyAsync(vals, vi, (size_t)n * sizeof(V), cudaMemcpyDeviceToDevice, s));
  }
}

void scan_u32_to_u64(const uint32_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  scan_impl<uint32_t>(in, out, n, tmp, s);
}

void scan_u64(const uint64_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  scan_impl<uint64_t>(in, out, n, tmp, s);
}

template <class V>
void radix_sort_pairs(uint64_t* keys, V* vals, uint64_t* keys_alt, V* vals_alt, int64_t n, int begin_bit,
                      int end_bit, DevBuf& tmp, cudaStream_t s) {
  if (n <= 1 || begin_bit >= end_bit) return;
  // BHTSNE_SORT_ONESWEEP=0 keeps the three-kernel passes at every size (for
  // comparing the two; both are stable, so they give the same permutation)
  const char* os_env = getenv("BHTSNE_SORT_ONESWEEP");
  const bool os_off = os_env && atoi(os_env) == 0;
  if (!os_off && n >= kOnesweepMin && n <= kOnesweepMax && end_bit - begin_bit <= 8 * kOsMaxPass) {
    radix_sort_onesweep<V>(keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, tmp, s);
    return;
  }
  static_assert(kRsTile == kRadixTile && kRsSup == kRadixSup && kScanTile == kRadixScanTile,
                "radix_sort_tmp_bytes describes this layout");
  const int64_t nb = ceil_div(n, kRsTile);
  const int64_t ns = ceil_div(nb, kRsSup);
  const int64_t ms = 256 * ns;
  // tmp layout: tile counts (u32, 256 nb) | super-tile totals (u32, ms) |
  // super-tile offsets (u64, ms + 1; with the inline spine, the second
  // super-tile table) | scan scratch
  const size_t cb = radix_round256((size_t)nb * 256 * 4);
  const size_t sb = radix_round256((size_t)ms * 4);
  const size_t ob = radix_round256((size_t)(ms + 1) * 8);
  char* base = static_cast<char*>(tmp.ensure(radix_sort_tmp_bytes(n)));
  uint32_t* counts = reinterpret_cast<uint32_t*>(base);
  uint32_t* sup = reinterpret_cast<uint32_t*>(base + cb);
  uint64_t* sup_off = reinterpret_cast<uint64_t*>(base + cb + sb);
  uint64_t* partial = reinterpret_cast<uint64_t*>(base + cb + sb + ob);
  const bool inline_spine = ns <= kRsInlineSup;
  const bool one_block = ms <= kSpineMax;
  // inline spine: two super-tile tables used in turn; the scatter of one
  // pass clears the table the next pass's histogram fills
  uint32_t* sup2 = reinterpret_cast<uint32_t*>(base + cb + sb);
  BHG_CUDA(cudaMemsetAsync(sup, 0, (size_t)(inline_spine ? 2 * sb : ms * 4), s));

  uint64_t *ki = keys, *ko = keys_alt;
  V *vi = vals, *vo = vals_alt;
  int passes = 0;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    rs_hist_kernel<<<(unsigned)nb, kRsThreads, 0, s>>>(ki, n, shift, counts, sup, ns);
    BHG_LAUNCH_CHECK();
    if (inline_spine) {
      rs_scatter_kernel<V><<<(unsigned)nb, kRsThreads, 0, s>>>(ki, vi, ko, vo, n, shift, counts, nullptr, sup, ns,
                                                               sup2);
      BHG_LAUNCH_CHECK();
      std::swap(sup, sup2);
      std::swap(ki, ko);
      std::swap(vi, vo);
      ++passes;
      continue;
    }
    if (one_block) {
      rs_spine_kernel<<<1, kSpineThreads, 0, s>>>(sup, ms, sup_off, 1);
      BHG_LAUNCH_CHECK();
    } else {
      const int64_t nsb = ceil_div(ms, kScanTile);
      scan_reduce_kernel<uint32_t><<<(unsigned)nsb, kScanThreads, 0, s>>>(sup, ms, partial);
      BHG_LAUNCH_CHECK();
      scan_partials_kernel<<<1, 1024, 0, s>>>(partial, nsb, sup_off + ms);
      BHG_LAUNCH_CHECK();
      scan_apply_kernel<uint32_t><<<(unsigned)nsb, kScanThreads, 0, s>>>(sup, sup_off, ms, partial);
      BHG_LAUNCH_CHECK();
      BHG_CUDA(cudaMemsetAsync(sup, 0, (size_t)ms * 4, s));
    }
    rs_scatter_kernel<V><<<(unsigned)nb, kRsThreads, 0, s>>>(ki, vi, ko, vo, n, shift, counts, sup_off, nullptr, ns,
                                                             nullptr);
    BHG_LAUNCH_CHECK();
    std::swap(ki, ko);
    std::swap(vi, vo);
    ++passes;
  }
  if (passes & 1) {
    BHG_CUDA(cudaMemcpyAsync(keys, ki, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
    BHG_CUDA(cudaMemcpyAsync(vals, vi, (size_t)n * sizeof(V), cudaMemcpyDeviceToDevice, s));
  }
}

template void radix_sort_pairs<uint32_t>(uint64_t*, uint32_t*, uint64_t*, uint32_t*, int64_t, int, int, DevBuf&,
                                         cudaStream_t);
template void radix_sort_pairs<float>(uint64_t*, float*, uint64_t*, float*, int64_t, int, int, DevBuf&, cudaStream_t);
template void radix_sort_pairs<double>(uint64_t*, double*, uint64_t*, double*, int64_t, int, int, DevBuf&,
                                       cudaStream_t);

}  // namespace bhg
