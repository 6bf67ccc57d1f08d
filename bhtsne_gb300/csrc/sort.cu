// Device-wide exclusive scans and a stable LSD radix sort of (u64 key, payload)
// pairs. Used every Barnes-Hut epoch to put the Morton codes in Z-order (the
// role of `par_sort_unstable_by_key` at src/tsne/arena.rs:191 of the
// reference) and once per fit to order the symmetric affinity entries.
//
// The sort is three kernels per 8-bit digit: a per-tile histogram, one scan of
// the digit-major count table, and a stable scatter in which each warp ranks
// its keys with __match_any_sync. Tiles are 4096 keys, read in coalesced
// rounds of 256.
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
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsWarps = kRsThreads / 32;

__global__ void rs_hist_kernel(const uint64_t* __restrict__ keys, int64_t n, int shift, uint32_t* __restrict__ counts,
                               int64_t nblocks) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kRsTile;
#pragma unroll 4
  for (int i = 0; i < kRsItems; ++i) {
    int64_t p = base + (int64_t)i * kRsThreads + threadIdx.x;
    if (p < n) atomicAdd(&h[(unsigned)(keys[p] >> shift) & 255u], 1u);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

template <class V>
__global__ void __launch_bounds__(kRsThreads) rs_scatter_kernel(const uint64_t* __restrict__ kin, const V* __restrict__ vin,
                                                                uint64_t* __restrict__ kout, V* __restrict__ vout, int64_t n,
                                                                int shift, const uint64_t* __restrict__ offsets,
                                                                int64_t nblocks) {
  __shared__ uint32_t cnt[kRsWarps][256];
  __shared__ uint64_t off[kRsWarps][256];
  __shared__ uint64_t base[256];
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  base[tid] = offsets[(int64_t)tid * nblocks + blockIdx.x];
#pragma unroll
  for (int q = 0; q < kRsWarps; ++q) cnt[q][tid] = 0;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  const int64_t tile = (int64_t)blockIdx.x * kRsTile;
  for (int i = 0; i < kRsItems; ++i) {
    const int64_t p = tile + (int64_t)i * kRsThreads + tid;
    const bool valid = p < n;
    uint64_t k = 0;
    V v{};
    if (valid) {
      k = kin[p];
      v = vin[p];
    }
    const unsigned d = valid ? ((unsigned)(k >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(kFull, d);
    const unsigned rank = __popc(peers & lt);
    if (valid && rank == 0) cnt[w][d] = __popc(peers);
    __syncthreads();
    {
      uint64_t run = base[tid];
#pragma unroll
      for (int q = 0; q < kRsWarps; ++q) {
        const uint32_t c = cnt[q][tid];
        off[q][tid] = run;
        run += c;
        cnt[q][tid] = 0;
      }
      base[tid] = run;
    }
    __syncthreads();
    if (valid) {
      const uint64_t pos = off[w][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
  }
}

}  // namespace

void scan_u32_to_u64(const uint32_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  scan_impl<uint32_t>(in, out, n, tmp, s);
}

void scan_u64(const uint64_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s) {
  scan_impl<uint64_t>(in, out, n, tmp, s);
}

template <class V>
void radix_sort_pairs(uint64_t* keys, V* vals, uint64_t* keys_alt, V* vals_alt, int64_t n, int begin_bit,
                      int end_bit, DevBuf& tmp, cudaStream_t s) {
  if (n <= 1) return;
  const int64_t nb = ceil_div(n, kRsTile);
  const int64_t ncount = 256 * nb;
  // tmp layout: counts (u32, ncount) | offsets (u64, ncount+1) | scan scratch
  const size_t counts_bytes = ((size_t)ncount * 4 + 255) / 256 * 256;
  const size_t off_bytes = ((size_t)(ncount + 1) * 8 + 255) / 256 * 256;
  const int64_t scan_parts = ceil_div(ncount, kScanTile) + 1;
  char* base = static_cast<char*>(tmp.ensure(counts_bytes + off_bytes + (size_t)scan_parts * 8 + 256));
  uint32_t* counts = reinterpret_cast<uint32_t*>(base);
  uint64_t* offsets = reinterpret_cast<uint64_t*>(base + counts_bytes);
  uint64_t* partial = reinterpret_cast<uint64_t*>(base + counts_bytes + off_bytes);

  uint64_t *ki = keys, *ko = keys_alt;
  V *vi = vals, *vo = vals_alt;
  int passes = 0;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    rs_hist_kernel<<<(unsigned)nb, kRsThreads, 0, s>>>(ki, n, shift, counts, nb);
    BHG_LAUNCH_CHECK();
    const int64_t sb = ceil_div(ncount, kScanTile);
    scan_reduce_kernel<uint32_t><<<(unsigned)sb, kScanThreads, 0, s>>>(counts, ncount, partial);
    BHG_LAUNCH_CHECK();
    scan_partials_kernel<<<1, 1024, 0, s>>>(partial, sb, offsets + ncount);
    BHG_LAUNCH_CHECK();
    scan_apply_kernel<uint32_t><<<(unsigned)sb, kScanThreads, 0, s>>>(counts, offsets, ncount, partial);
    BHG_LAUNCH_CHECK();
    rs_scatter_kernel<V><<<(unsigned)nb, kRsThreads, 0, s>>>(ki, vi, ko, vo, n, shift, offsets, nb);
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
