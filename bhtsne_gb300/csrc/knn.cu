// Exact k-nearest neighbours for dense Euclidean data, the GPU replacement of
// the VP-tree search (src/tsne/vptree.rs:274-319 of bhtsne 0.7.10) for
// `barnes_hut` / `fit_sne` over a Euclidean metric closure.
//
// Result contract (the reference's brute-force test helper,
// src/test.rs:856-881): distance = sqrt(sum over dimensions, in order, of
// (a - b)^2) rounded in T at every step; neighbours ordered by (distance,
// index); the query itself excluded.
//
// Pipeline:
//  1. candidates: a register-tiled FP32 pass computes |q|^2 + |c|^2 - 2 q.c
//     for 64 queries x 128 candidates per tile and keeps, per query, the C
//     smallest (C = 128 or 256, C > k) in a sorted list in shared memory.
//  2. re-rank: the exact distance of every candidate is recomputed in the
//     reference's operation order, the list is sorted by (distance, index)
//     and the first k are kept.
//  3. certification: a neighbour outside the candidate list has an
//     approximate squared distance >= the list's C-th value, and the FP32
//     error of that approximation is below (4 dim + 16) u (|q|^2 + max|x|^2).
//     When the exact k-th squared distance is below that bound the row is
//     provably exact; otherwise the row is recomputed by an exact brute-force
//     warp over all points. Either way the output equals brute force.
#include "knn.h"

#include <algorithm>
#include <cfloat>
#include <cstdlib>
#include <type_traits>

namespace bhg {

namespace {

constexpr int QB = 64;    // queries per block
constexpr int CB = 128;   // candidates per tile
constexpr int DK = 32;    // dimensions per candidate chunk
constexpr int kThreads = 256;
constexpr uint32_t SENT = 0xffffffffu;
// sliced certified fallback: at most kMaxSlices slices of at least kMinSlice
// candidates, scratch of at most kSliceScratchMax bytes
constexpr int kMaxSlices = 16;
constexpr int64_t kMinSlice = 4096;
constexpr size_t kSliceScratchMax = (size_t)1 << 30;
// bounded re-scan: at most kListCap listed candidates per failing row, lists
// of at most kListBytesMax bytes in all
constexpr int kListCap = 2048;
constexpr size_t kListBytesMax = (size_t)1 << 30;

__global__ void sq_norm_kernel(const float* __restrict__ X, int64_t n, int dim, float* __restrict__ norms,
                               unsigned* __restrict__ max_bits) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  float s = 0.f;
  for (int d = lane; d < dim; d += 32) {
    const float v = X[i * dim + d];
    s = fmaf(v, v, s);
  }
  s = warp_sum(s);
  if (lane == 0) {
    norms[i] = s;
    atomicMax(max_bits, __float_as_uint(s));
  }
}

template <class T>
__global__ void to_f32_kernel(const T* __restrict__ X, int64_t count, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)X[i];
}

// Warp-cooperative insertion of (v, j) into a sorted list (v, j ascending) of
// capacity cap holding *len entries.
template <class V>
__device__ __forceinline__ bool lt_pair(V a, uint32_t ai, V b, uint32_t bi) {
  return a < b || (a == b && ai < bi);
}

template <class V>
__device__ void warp_insert(V* lv, uint32_t* li, int* len_p, int cap, V v, uint32_t j, int lane) {
  const int len = *len_p;
  if (len == cap && !lt_pair(v, j, lv[cap - 1], li[cap - 1])) return;
  int pos = 0;
  for (int b = 0; b < len; b += 32) {
    const int e = b + lane;
    const bool less = e < len && lt_pair(lv[e], li[e], v, j);
    pos += __popc(__ballot_sync(kFull, less));
  }
  const int top = len < cap ? len : cap - 1;  // last index to move from (exclusive bound handled below)
  for (int b = ((top - 1) >> 5) << 5; b >= 0 && top > 0; b -= 32) {
    const int e = b + lane;
    V tv{};
    uint32_t tj = 0;
    const bool mv = e >= pos && e < top;
    if (mv) {
      tv = lv[e];
      tj = li[e];
    }
    __syncwarp();
    if (mv) {
      lv[e + 1] = tv;
      li[e + 1] = tj;
    }
    __syncwarp();
    if (b == 0) break;
  }
  if (lane == 0) {
    lv[pos] = v;
    li[pos] = j;
    *len_p = len < cap ? len + 1 : cap;
  }
  __syncwarp();
}

// Register-tiled distance tile: 64 queries x 128 candidates per step, 4 x 8
// values per thread, dimensions consumed in order in chunks of 32. With
// EXACT = false a value is |q|^2 + |c|^2 - 2 q.c (FP32 FMA, the candidate
// pass); with EXACT = true it is the reference's distance sqrt(sum_d (q-c)^2)
// rounded at every step (the certified fallback), and the kept list is the
// answer. Queries are rows q0.. of X, or the rows listed in `qrows`.
//
// dynamic shared layout: Qs[dim][QB] | Cs[DK][CB] | S[QB][CB+1] | lv[QB][C] | li[QB][C] | len[QB] | qn[QB]
//
// Segmented form (blk_q0 != nullptr, candidate pass only): X holds many
// independent point sets back to back, set j owning rows seg_off[j]..
// seg_off[j+1]; block b takes the queries blk_q0[b].. of set blk_job[b] and
// scans that set's rows only. Indices stay global.
//
// Sliced form (slice_len > 0, EXACT with qrows only): block (x, y) scans the
// candidates y slice_len .. (y + 1) slice_len - 1 only and writes its list of
// `cap` (index, distance), padded with (SENT, +inf), to row r = x QB + q of
// slice_idx / slice_val at [(r gridDim.y + y) cap]; slice_merge_kernel then
// merges the slices' lists.
template <int C, bool EXACT>
__global__ void __launch_bounds__(kThreads, 1) knn_tile_kernel(const float* __restrict__ X, int64_t n, int dim,
                                                               const float* __restrict__ norms,
                                                               const uint32_t* __restrict__ qrows, int64_t nq, int cap,
                                                               uint32_t* __restrict__ out_idx,
                                                               float* __restrict__ out_val,
                                                               const int64_t* __restrict__ blk_q0 = nullptr,
                                                               const int32_t* __restrict__ blk_job = nullptr,
                                                               const int64_t* __restrict__ seg_off = nullptr,
                                                               int64_t slice_len = 0,
                                                               uint32_t* __restrict__ slice_idx = nullptr,
                                                               float* __restrict__ slice_val = nullptr) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* Qs = reinterpret_cast<float*>(smem);
  float* Cs = Qs + (size_t)dim * QB;
  float* S = Cs + DK * CB;
  float* lv = S + QB * (CB + 1);
  uint32_t* li = reinterpret_cast<uint32_t*>(lv + QB * C);
  int* len = reinterpret_cast<int*>(li + QB * C);
  float* qn = reinterpret_cast<float*>(len + QB);
  __shared__ int64_t qidx[QB];

  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int tq = tid >> 4, tc = tid & 15;
  int64_t q0 = (int64_t)blockIdx.x * QB, lo = 0, hi = n;
  if (blk_q0) {
    const int jb = blk_job[blockIdx.x];
    q0 = blk_q0[blockIdx.x];
    lo = seg_off[jb];
    hi = seg_off[jb + 1];
  }
  if (tid < QB) {
    const int64_t r = q0 + tid;
    if (blk_q0) qidx[tid] = r < hi ? r : -1;
    else qidx[tid] = r < nq ? (qrows ? (int64_t)qrows[r] : r) : -1;
    len[tid] = 0;
  }
  if (slice_len > 0) {
    lo = (int64_t)blockIdx.y * slice_len;
    hi = lo + slice_len < n ? lo + slice_len : n;
  }
  __syncthreads();
  for (int e = tid; e < QB * dim; e += kThreads) {
    const int q = e / dim, d = e % dim;
    const int64_t qi = qidx[q];
    Qs[d * QB + q] = qi >= 0 ? X[qi * dim + d] : 0.f;
  }
  if (tid < QB) qn[tid] = (!EXACT && qidx[tid] >= 0) ? norms[qidx[tid]] : 0.f;

  // Candidate chunk staging: thread t owns candidate c = t % CB and 4-dim
  // groups (t / CB) * 4 + 8 g, loaded as float4 when the row allows it.
  const bool vec4 = (dim & 3) == 0;
  float pre[16];
  auto load_chunk = [&](int64_t c0, int d0) {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const int c = tid % CB;
      const int dq = (tid / CB) * 4 + 8 * g;
      const int64_t j = c0 + c;
      const int d = d0 + dq;
      if (j < hi && vec4 && d + 3 < dim) {
        const float4 v = *reinterpret_cast<const float4*>(X + j * dim + d);
        pre[4 * g + 0] = v.x;
        pre[4 * g + 1] = v.y;
        pre[4 * g + 2] = v.z;
        pre[4 * g + 3] = v.w;
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) pre[4 * g + i] = (j < hi && d + i < dim) ? X[j * dim + d + i] : 0.f;
      }
    }
  };
  auto store_chunk = [&]() {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const int c = tid % CB;
      const int dq = (tid / CB) * 4 + 8 * g;
#pragma unroll
      for (int i = 0; i < 4; ++i) Cs[(dq + i) * CB + c] = pre[4 * g + i];
    }
  };

  const int nchunks = (dim + DK - 1) / DK;
  load_chunk(lo, 0);
  for (int64_t c0 = lo; c0 < hi; c0 += CB) {
    float acc[4][8];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    for (int ch = 0; ch < nchunks; ++ch) {
      const int d0 = ch * DK;
      __syncthreads();
      store_chunk();
      __syncthreads();
      // prefetch the next chunk (next dims, or the next candidate tile's first dims)
      if (ch + 1 < nchunks) load_chunk(c0, d0 + DK);
      else if (c0 + CB < hi) load_chunk(c0 + CB, 0);
      const int dmax = min(DK, dim - d0);
      for (int dd = 0; dd < dmax; ++dd) {
        const float4 a4 = *reinterpret_cast<const float4*>(Qs + (d0 + dd) * QB + tq * 4);
        const float4 b0 = *reinterpret_cast<const float4*>(Cs + dd * CB + tc * 4);
        const float4 b1 = *reinterpret_cast<const float4*>(Cs + dd * CB + 64 + tc * 4);
        const float av[4] = {a4.x, a4.y, a4.z, a4.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 8; ++b) {
            if (EXACT) {
              const float t = av[a] - bv[b];
              acc[a][b] = __fadd_rn(acc[a][b], __fmul_rn(t, t));
            } else {
              acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
            }
          }
      }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int q = tq * 4 + a;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const int c = b < 4 ? tc * 4 + b : 64 + tc * 4 + (b - 4);
        float v;
        if (EXACT) {
          v = sqrtf(acc[a][b]);
        } else {
          const int64_t j = c0 + c;
          const float cn = j < hi ? norms[j] : 0.f;
          v = qn[q] + cn - 2.f * acc[a][b];
        }
        S[q * (CB + 1) + c] = v;
      }
    }
    __syncthreads();
    for (int qq = 0; qq < QB / 8; ++qq) {
      const int q = w * (QB / 8) + qq;
      const int64_t qi = qidx[q];
      if (qi < 0) continue;
      float* qlv = lv + q * C;
      uint32_t* qli = li + q * C;
#pragma unroll
      for (int part = 0; part < CB / 32; ++part) {
        const int c = part * 32 + lane;
        const int64_t j = c0 + c;
        const float v = S[q * (CB + 1) + c];
        const int L = len[q];
        bool ok = j < hi && j != qi;
        if (ok && L == cap) ok = lt_pair(v, (uint32_t)j, qlv[cap - 1], qli[cap - 1]);
        unsigned mask = __ballot_sync(kFull, ok);
        while (mask) {
          const int src = __ffs(mask) - 1;
          mask &= mask - 1;
          const float vv = __shfl_sync(kFull, v, src);
          const uint32_t jj = (uint32_t)(c0 + part * 32 + src);
          warp_insert<float>(qlv, qli, &len[q], cap, vv, jj, lane);
        }
      }
    }
  }
  __syncthreads();
  for (int qq = 0; qq < QB / 8; ++qq) {
    const int q = w * (QB / 8) + qq;
    const int64_t qi = qidx[q];
    if (qi < 0) continue;
    const int L = len[q];
    if (EXACT && slice_len > 0) {
      const size_t base = ((size_t)(q0 + q) * gridDim.y + blockIdx.y) * cap;
      for (int t = lane; t < cap; t += 32) {
        slice_idx[base + t] = t < L ? li[q * C + t] : SENT;
        slice_val[base + t] = t < L ? lv[q * C + t] : INFINITY;
      }
    } else if (EXACT) {
      for (int t = lane; t < cap; t += 32) {
        out_idx[qi * cap + t] = li[q * C + t];
        out_val[qi * cap + t] = lv[q * C + t];
      }
    } else {
      for (int t = lane; t < C; t += 32) out_idx[qi * C + t] = t < L ? li[q * C + t] : SENT;
      if (lane == 0) out_val[qi] = L == C ? lv[q * C + C - 1] : INFINITY;
    }
  }
}

// Merge of the sliced fallback's lists: one warp per listed row; lane l < S
// follows slice l's sorted list, and each of the k steps takes the smallest
// head (distance bits, index) over the warp. Distances are >= 0, so their
// bit patterns order like the values; (SENT, +inf) pads sort last.
__global__ void slice_merge_kernel(const uint32_t* __restrict__ slice_idx, const float* __restrict__ slice_val,
                                   const uint32_t* __restrict__ rows, int64_t nrows, int S, int k,
                                   uint32_t* __restrict__ out_idx, float* __restrict__ out_dist) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  const int64_t qi = rows[r];
  const size_t base = ((size_t)r * S + (lane < S ? lane : 0)) * k;
  int p = 0;
  auto head = [&]() -> unsigned long long {
    if (lane >= S || p >= k) return ~0ull;
    return ((unsigned long long)__float_as_uint(slice_val[base + p]) << 32) | slice_idx[base + p];
  };
  unsigned long long h = head();
  for (int t = 0; t < k; ++t) {
    unsigned long long m = h;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(kFull, m, o);
      m = x < m ? x : m;
    }
    if (lane == 0) {
      out_idx[qi * k + t] = (uint32_t)(m & 0xffffffffull);
      out_dist[qi * k + t] = __uint_as_float((uint32_t)(m >> 32));
    }
    if (h == m) {
      ++p;
      h = head();
    }
  }
}

// Candidate pass with buffered selection (C = kSelC, dim <= kSelDimMax).
// Distances as in knn_tile_kernel (same FP32 values, so the same candidate
// list and threshold); only the selection differs. Per query, a buffer of 2C
// (value, index) pairs in shared memory holds the C best so far (sorted, from
// the last merge) followed by unsorted appends that beat the current C-th
// best. Appends cost one ballot per 32 candidates; when the next 32 could
// overflow the buffer, the owning warp bitonic-sorts it by (value, index) and
// keeps the first C. Every rejected candidate is no better than a C-th best
// of its time, hence no better than the final C-th: the list and threshold
// equal those of one sorted insertion per candidate.
constexpr int kSelC = 128;
constexpr int kSelDimMax = 128;

__device__ __forceinline__ void sel_merge(float* bv, uint32_t* bi, int& c, float& tv, uint32_t& ti, int lane) {
  constexpr int B = 2 * kSelC;
  for (int t = c + lane; t < B; t += 32) {
    bv[t] = INFINITY;
    bi[t] = SENT;
  }
  __syncwarp();
  for (int size = 2; size <= B; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < B / 2; t += 32) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const float a = bv[lo], b = bv[hi];
        const uint32_t ia = bi[lo], ib = bi[hi];
        if (lt_pair(b, ib, a, ia) == up) {
          bv[lo] = b;
          bv[hi] = a;
          bi[lo] = ib;
          bi[hi] = ia;
        }
      }
      __syncwarp();
    }
  }
  c = c < kSelC ? c : kSelC;
  if (c == kSelC) {
    tv = bv[kSelC - 1];
    ti = bi[kSelC - 1];
  }
}

// dynamic shared layout: Qs[dim][QB] | Cs[DK][CB] | S[QB][CB+1] | bv[QB][2C] | bi[QB][2C]
__global__ void __launch_bounds__(kThreads, 1) knn_cand_kernel(const float* __restrict__ X, int64_t n, int dim,
                                                               const float* __restrict__ norms,
                                                               uint32_t* __restrict__ out_idx,
                                                               float* __restrict__ out_thr,
                                                               const int64_t* __restrict__ blk_q0,
                                                               const int32_t* __restrict__ blk_job,
                                                               const int64_t* __restrict__ seg_off) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* Qs = reinterpret_cast<float*>(smem);
  float* Cs = Qs + (size_t)dim * QB;
  float* S = Cs + DK * CB;
  float* bv = S + QB * (CB + 1);
  uint32_t* bi = reinterpret_cast<uint32_t*>(bv + QB * 2 * kSelC);
  __shared__ int64_t qidx[QB];
  __shared__ float qn[QB];
  constexpr int QW = QB / 8;  // queries per warp in the selection

  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int tq = tid >> 4, tc = tid & 15;
  int64_t q0 = (int64_t)blockIdx.x * QB, lo = 0, hi = n;
  if (blk_q0) {
    const int jb = blk_job[blockIdx.x];
    q0 = blk_q0[blockIdx.x];
    lo = seg_off[jb];
    hi = seg_off[jb + 1];
  }
  if (tid < QB) {
    const int64_t r = q0 + tid;
    qidx[tid] = r < hi ? r : -1;
    qn[tid] = r < hi ? norms[r] : 0.f;
  }
  __syncthreads();
  for (int e = tid; e < QB * dim; e += kThreads) {
    const int q = e / dim, d = e % dim;
    const int64_t qi = qidx[q];
    Qs[d * QB + q] = qi >= 0 ? X[qi * dim + d] : 0.f;
  }

  const bool vec4 = (dim & 3) == 0;
  float pre[16];
  auto load_chunk = [&](int64_t c0, int d0) {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const int c = tid % CB;
      const int dq = (tid / CB) * 4 + 8 * g;
      const int64_t j = c0 + c;
      const int d = d0 + dq;
      if (j < hi && vec4 && d + 3 < dim) {
        const float4 v = *reinterpret_cast<const float4*>(X + j * dim + d);
        pre[4 * g + 0] = v.x;
        pre[4 * g + 1] = v.y;
        pre[4 * g + 2] = v.z;
        pre[4 * g + 3] = v.w;
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) pre[4 * g + i] = (j < hi && d + i < dim) ? X[j * dim + d + i] : 0.f;
      }
    }
  };
  auto store_chunk = [&]() {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const int c = tid % CB;
      const int dq = (tid / CB) * 4 + 8 * g;
#pragma unroll
      for (int i = 0; i < 4; ++i) Cs[(dq + i) * CB + c] = pre[4 * g + i];
    }
  };

  int cnt[QW];
  float tv[QW];
  uint32_t ti[QW];
#pragma unroll
  for (int qq = 0; qq < QW; ++qq) {
    cnt[qq] = 0;
    tv[qq] = INFINITY;
    ti[qq] = SENT;
  }

  const int nchunks = (dim + DK - 1) / DK;
  load_chunk(lo, 0);
  for (int64_t c0 = lo; c0 < hi; c0 += CB) {
    float acc[4][8];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    for (int ch = 0; ch < nchunks; ++ch) {
      const int d0 = ch * DK;
      __syncthreads();
      store_chunk();
      __syncthreads();
      if (ch + 1 < nchunks) load_chunk(c0, d0 + DK);
      else if (c0 + CB < hi) load_chunk(c0 + CB, 0);
      const int dmax = min(DK, dim - d0);
      for (int dd = 0; dd < dmax; ++dd) {
        const float4 a4 = *reinterpret_cast<const float4*>(Qs + (d0 + dd) * QB + tq * 4);
        const float4 b0 = *reinterpret_cast<const float4*>(Cs + dd * CB + tc * 4);
        const float4 b1 = *reinterpret_cast<const float4*>(Cs + dd * CB + 64 + tc * 4);
        const float av[4] = {a4.x, a4.y, a4.z, a4.w};
        const float bv8[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(av[a], bv8[b], acc[a][b]);
      }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int q = tq * 4 + a;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const int c = b < 4 ? tc * 4 + b : 64 + tc * 4 + (b - 4);
        const int64_t j = c0 + c;
        const float cn = j < hi ? norms[j] : 0.f;
        S[q * (CB + 1) + c] = qn[q] + cn - 2.f * acc[a][b];
      }
    }
    __syncthreads();
#pragma unroll
    for (int qq = 0; qq < QW; ++qq) {
      const int q = w * QW + qq;
      const int64_t qi = qidx[q];
      if (qi < 0) continue;
      float* qbv = bv + (size_t)q * 2 * kSelC;
      uint32_t* qbi = bi + (size_t)q * 2 * kSelC;
#pragma unroll
      for (int part = 0; part < CB / 32; ++part) {
        if (cnt[qq] > 2 * kSelC - 32) sel_merge(qbv, qbi, cnt[qq], tv[qq], ti[qq], lane);
        const int c = part * 32 + lane;
        const int64_t j = c0 + c;
        const float v = S[q * (CB + 1) + c];
        const bool ok = j < hi && j != qi && lt_pair(v, (uint32_t)j, tv[qq], ti[qq]);
        const unsigned m = __ballot_sync(kFull, ok);
        if (ok) {
          const int at = cnt[qq] + __popc(m & ((1u << lane) - 1u));
          qbv[at] = v;
          qbi[at] = (uint32_t)j;
        }
        cnt[qq] += __popc(m);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int qq = 0; qq < QW; ++qq) {
    const int q = w * QW + qq;
    const int64_t qi = qidx[q];
    if (qi < 0) continue;
    float* qbv = bv + (size_t)q * 2 * kSelC;
    uint32_t* qbi = bi + (size_t)q * 2 * kSelC;
    sel_merge(qbv, qbi, cnt[qq], tv[qq], ti[qq], lane);
    for (int t = lane; t < kSelC; t += 32) out_idx[qi * kSelC + t] = t < cnt[qq] ? qbi[t] : SENT;
    if (lane == 0) out_thr[qi] = cnt[qq] == kSelC ? qbv[kSelC - 1] : INFINITY;
  }
}

// Exact distance in the reference's order (sequential over dimensions, T).
template <class T>
__device__ __forceinline__ T exact_d2(const T* __restrict__ a, const T* __restrict__ b, int dim) {
  T s = T(0);
  for (int d = 0; d < dim; ++d) {
    const T t = a[d] - b[d];
    s = s + t * t;
  }
  return s;
}

// One warp per query: exact distances of the C candidates, bitonic sort by
// (distance, index), first k out, certification.
template <class T, int C>
__global__ void knn_rerank_kernel(const T* __restrict__ X, int64_t n, int dim, int k, const uint32_t* __restrict__ cand,
                                  const float* __restrict__ thr, const float* __restrict__ norms,
                                  const unsigned* __restrict__ max_bits, uint32_t* __restrict__ out_idx,
                                  T* __restrict__ out_dist, uint32_t* __restrict__ fail_list,
                                  unsigned* __restrict__ fail_count, double ecoef,
                                  float* __restrict__ fail_bound = nullptr) {
  constexpr int W = 4;
  __shared__ T sd[W][C];
  __shared__ T sd2[W][C];
  __shared__ uint32_t sj[W][C];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t qi = (int64_t)blockIdx.x * W + w;
  if (qi >= n) return;
  const T* xq = X + qi * dim;
  for (int t = lane; t < C; t += 32) {
    const uint32_t j = cand[qi * C + t];
    T d2 = (T)INFINITY, d = (T)INFINITY;
    if (j != SENT) {
      d2 = exact_d2<T>(xq, X + (int64_t)j * dim, dim);
      d = dsqrt(d2);
    }
    sd[w][t] = d;
    sd2[w][t] = d2;
    sj[w][t] = j;
  }
  __syncwarp();
  for (int size = 2; size <= C; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < C / 2; t += 32) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const bool gt = lt_pair(sd[w][hi], sj[w][hi], sd[w][lo], sj[w][lo]);
        if (gt == up) {
          T a = sd[w][lo];
          sd[w][lo] = sd[w][hi];
          sd[w][hi] = a;
          a = sd2[w][lo];
          sd2[w][lo] = sd2[w][hi];
          sd2[w][hi] = a;
          const uint32_t b = sj[w][lo];
          sj[w][lo] = sj[w][hi];
          sj[w][hi] = b;
        }
      }
      __syncwarp();
    }
  }
  for (int t = lane; t < k; t += 32) {
    out_idx[qi * k + t] = sj[w][t];
    out_dist[qi * k + t] = sd[w][t];
  }
  if (lane == 0) {
    // A point c outside the candidate list that ranked within the first k
    // would have true |q - c|^2 <= d2k, hence |c| <= |q| + sqrt(d2k), so the
    // FP32 error of its candidate value is at most E below; yet that value is
    // >= th. Certified when d2k (inflated by its own rounding) + E < th.
    const float th = thr[qi];
    bool ok = true;
    double bound = 0.0;
    if (!isinf(th)) {
      const double u = 1.0 / 16777216.0;
      const double g = (dim + 2.0) * u;
      const double qn = (double)norms[qi] * (1.0 + g);
      const double d2k = (double)sd2[w][k - 1] * (1.0 + g) * (1.0 + 16.0 * u);
      const double r = sqrt(qn) + sqrt(d2k);
      const double E = ecoef * (qn + r * r);
      bound = d2k + E;
      ok = bound < (double)th;
    }
    if (!ok) {
      const unsigned f = atomicAdd(fail_count, 1u);
      fail_list[f] = (uint32_t)qi;
      // every true neighbour's candidate value is at most bound (rounded up)
      if (fail_bound) fail_bound[f] = __double2float_ru(bound);
    }
  }
}

// Exact re-rank of a bounded re-scan: one warp per listed row r (row
// rows[r] of X) over its list of list_cnt[r] candidates (index order), with
// the sorted list of size k in shared memory by (distance, index). A row
// whose list overflowed cap (or holds fewer than k others) goes to over[].
template <class T>
__global__ void knn_list_rerank_kernel(const T* __restrict__ X, int dim, int k, const uint32_t* __restrict__ rows,
                                       int64_t nrows, const uint32_t* __restrict__ list,
                                       const uint32_t* __restrict__ list_cnt, int cap, uint32_t* __restrict__ out_idx,
                                       T* __restrict__ out_dist, uint32_t* __restrict__ over,
                                       unsigned* __restrict__ over_count) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int W = 4;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* lv = reinterpret_cast<T*>(smem) + (size_t)w * k;
  uint32_t* li = reinterpret_cast<uint32_t*>(reinterpret_cast<T*>(smem) + (size_t)W * k) + (size_t)w * k;
  __shared__ int len[W];
  const int64_t r = (int64_t)blockIdx.x * W + w;
  if (r >= nrows) return;
  const int64_t qi = rows[r];
  const uint32_t cnt = list_cnt[r];
  if (cnt > (uint32_t)cap) {
    if (lane == 0) over[atomicAdd(over_count, 1u)] = (uint32_t)qi;
    return;
  }
  if (lane == 0) len[w] = 0;
  __syncwarp();
  const T* xq = X + qi * dim;
  const uint32_t* lr = list + (size_t)r * cap;
  for (uint32_t b = 0; b < cnt; b += 32) {
    const uint32_t e = b + lane;
    const uint32_t j = e < cnt ? lr[e] : 0u;
    bool ok = e < cnt && (int64_t)j != qi;
    T d = T(0);
    if (ok) d = dsqrt(exact_d2<T>(xq, X + (int64_t)j * dim, dim));
    if (ok && len[w] == k) ok = lt_pair(d, j, lv[k - 1], li[k - 1]);
    unsigned mask = __ballot_sync(kFull, ok);
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const T dv = __shfl_sync(kFull, d, src);
      const uint32_t jv = __shfl_sync(kFull, j, src);
      warp_insert<T>(lv, li, &len[w], k, dv, jv, lane);
    }
  }
  if (len[w] < k) {
    if (lane == 0) over[atomicAdd(over_count, 1u)] = (uint32_t)qi;
    return;
  }
  for (int t = lane; t < k; t += 32) {
    out_idx[qi * k + t] = li[t];
    out_dist[qi * k + t] = lv[t];
  }
}

// Exact brute force for the listed queries, one warp per query, list of size k
// kept sorted in shared memory by (distance, index).
// With seg_off, a query of set j = seg_of[qi] scans rows seg_off[j]..seg_off[j+1] only.
template <class T>
__global__ void knn_exact_kernel(const T* __restrict__ X, int64_t n, int dim, int k, const uint32_t* __restrict__ rows,
                                 const unsigned* __restrict__ nrows_p, int64_t nrows_fixed,
                                 uint32_t* __restrict__ out_idx, T* __restrict__ out_dist,
                                 const int64_t* __restrict__ seg_off = nullptr,
                                 const uint32_t* __restrict__ seg_of = nullptr) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int W = 4;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* lv = reinterpret_cast<T*>(smem) + (size_t)w * k;
  uint32_t* li = reinterpret_cast<uint32_t*>(reinterpret_cast<T*>(smem) + (size_t)W * k) + (size_t)w * k;
  __shared__ int len[W];
  const int64_t nrows = nrows_p ? (int64_t)*nrows_p : nrows_fixed;
  const int64_t r = (int64_t)blockIdx.x * W + w;
  if (r >= nrows) return;
  const int64_t qi = rows ? (int64_t)rows[r] : r;
  if (lane == 0) len[w] = 0;
  __syncwarp();
  const T* xq = X + qi * dim;
  int64_t lo = 0, hi = n;
  if (seg_off) {
    lo = seg_off[seg_of[qi]];
    hi = seg_off[seg_of[qi] + 1];
  }
  for (int64_t b = lo; b < hi; b += 32) {
    const int64_t j = b + lane;
    T d = T(0);
    bool ok = j < hi && j != qi;
    if (ok) d = dsqrt(exact_d2<T>(xq, X + j * dim, dim));
    if (ok && len[w] == k) ok = lt_pair(d, (uint32_t)j, lv[k - 1], li[k - 1]);
    unsigned mask = __ballot_sync(kFull, ok);
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const T dv = __shfl_sync(kFull, d, src);
      warp_insert<T>(lv, li, &len[w], k, dv, (uint32_t)(b + src), lane);
    }
  }
  for (int t = lane; t < k; t += 32) {
    out_idx[qi * k + t] = li[t];
    out_dist[qi * k + t] = lv[t];
  }
}

// The candidate pass runs on the tensor cores unless BHTSNE_KNN_SIMT is set
// (the FP32 CUDA-core kernels, kept for comparison).
bool use_tensor_cores() {
  static const bool simt = getenv("BHTSNE_KNN_SIMT") != nullptr;
  return !simt;
}

// BHTSNE_KNN_RESCAN=0 sends every row that fails the certificate straight to
// the brute force (read on every call).
bool rescan_enabled() {
  const char* e = getenv("BHTSNE_KNN_RESCAN");
  return !(e && e[0] == '0');
}

size_t sel_smem_bytes(int dim) {
  return ((size_t)dim * QB + DK * CB + QB * (CB + 1)) * 4 + (size_t)QB * 2 * kSelC * 8;
}

}  // namespace

template <class T>
int64_t knn_euclidean(const T* X, int64_t n, int dim, int k, uint32_t* out_idx, T* out_dist, KnnWorkspace& ws,
                      cudaStream_t s) {
  if (k <= 0 || k > n - 1) throw Error(ST_EINVAL, "error: k must be in [1, n_samples - 1].");
  const int C = k <= 96 ? 128 : (k <= 224 ? 256 : 0);
  const int qdim_max = C == 128 ? 256 : 128;
  const bool use_candidates = C != 0 && dim <= qdim_max && n > C;
  unsigned* fail_count = static_cast<unsigned*>(ws.counters.ensure(64));
  BHG_CUDA(cudaMemsetAsync(fail_count, 0, 64, s));
  if (!use_candidates) {
    const size_t smem = (size_t)4 * k * (sizeof(T) + sizeof(uint32_t));
    if (smem > 48 * 1024)
      BHG_CUDA(cudaFuncSetAttribute(knn_exact_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    knn_exact_kernel<T><<<(unsigned)ceil_div(n, 4), 128, smem, s>>>(X, n, dim, k, nullptr, nullptr, n, out_idx, out_dist);
    BHG_LAUNCH_CHECK();
    return n;
  }
  const float* Xf;
  if constexpr (std::is_same<T, float>::value) {
    Xf = X;
  } else {
    float* tmp = static_cast<float*>(ws.xf.ensure((size_t)n * dim * sizeof(float)));
    to_f32_kernel<T><<<1024, 256, 0, s>>>(X, n * dim, tmp);
    BHG_LAUNCH_CHECK();
    Xf = tmp;
  }
  float* norms = static_cast<float*>(ws.norms.ensure((size_t)n * sizeof(float)));
  unsigned* max_bits = fail_count + 1;
  sq_norm_kernel<<<(unsigned)ceil_div(n * 32, 256), 256, 0, s>>>(Xf, n, dim, norms, max_bits);
  BHG_LAUNCH_CHECK();
  uint32_t* cand = static_cast<uint32_t*>(ws.cand.ensure((size_t)n * C * sizeof(uint32_t)));
  float* thr = static_cast<float*>(ws.thr.ensure((size_t)n * sizeof(float)));
  uint32_t* fails = static_cast<uint32_t*>(ws.fails.ensure((size_t)n * sizeof(uint32_t)));
  const size_t smem = ((size_t)dim * QB + DK * CB + QB * (CB + 1) + (size_t)QB * C * 2 + 2 * QB) * 4;
  const unsigned grid = (unsigned)ceil_div(n, QB);
  const double simt_coef = (4.0 * dim + 16.0) / 16777216.0;
  float* fbound = nullptr;  // per failing row: the bound of the bounded re-scan
  if (C == 128 && (ws.pass == 0 || (ws.pass < 0 && use_tensor_cores()))) {
    knn_tc_candidates(Xf, n, dim, norms, nullptr, nullptr, nullptr, nullptr, ceil_div(n, 128), cand, thr, ws.tc, s);
    if (knn_tc_can_bound(ws.tc, n, dim) && rescan_enabled()) fbound = static_cast<float*>(ws.fbound.ensure((size_t)n * 4));
    knn_rerank_kernel<T, 128><<<(unsigned)ceil_div(n, 4), 128, 0, s>>>(X, n, dim, k, cand, thr, norms, max_bits, out_idx,
                                                                       out_dist, fails, fail_count,
                                                                       knn_tc_error_coef(dim), fbound);
  } else if (C == 128 && dim <= kSelDimMax) {
    const size_t ssmem = sel_smem_bytes(dim);
    BHG_CUDA(cudaFuncSetAttribute(knn_cand_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssmem));
    knn_cand_kernel<<<grid, kThreads, ssmem, s>>>(Xf, n, dim, norms, cand, thr, nullptr, nullptr, nullptr);
    BHG_LAUNCH_CHECK();
    knn_rerank_kernel<T, 128><<<(unsigned)ceil_div(n, 4), 128, 0, s>>>(X, n, dim, k, cand, thr, norms, max_bits, out_idx,
                                                                       out_dist, fails, fail_count, simt_coef);
  } else if (C == 128) {
    BHG_CUDA(cudaFuncSetAttribute(knn_tile_kernel<128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    knn_tile_kernel<128, false><<<grid, kThreads, smem, s>>>(Xf, n, dim, norms, nullptr, n, 128, cand, thr);
    BHG_LAUNCH_CHECK();
    knn_rerank_kernel<T, 128><<<(unsigned)ceil_div(n, 4), 128, 0, s>>>(X, n, dim, k, cand, thr, norms, max_bits, out_idx,
                                                                       out_dist, fails, fail_count, simt_coef);
  } else {
    BHG_CUDA(cudaFuncSetAttribute(knn_tile_kernel<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    knn_tile_kernel<256, false><<<grid, kThreads, smem, s>>>(Xf, n, dim, norms, nullptr, n, 256, cand, thr);
    BHG_LAUNCH_CHECK();
    knn_rerank_kernel<T, 256><<<(unsigned)ceil_div(n, 4), 128, 0, s>>>(X, n, dim, k, cand, thr, norms, max_bits, out_idx,
                                                                       out_dist, fails, fail_count, simt_coef);
  }
  BHG_LAUNCH_CHECK();
  unsigned nfail = 0;
  BHG_CUDA(cudaMemcpyAsync(&nfail, fail_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  // Exact brute force for the listed rows: the tiled kernel computing the
  // reference's exact distances (f32), or one warp per row (f64).
  auto brute = [&](const uint32_t* rows, unsigned nrows) {
    if constexpr (std::is_same<T, float>::value) {
      // With few rows (under a few waves of blocks) the candidate range is
      // split into S slices, each block scanning one slice, and the slices'
      // lists merged: S chosen to minimise the waves per slice length.
      const unsigned fgrid = (unsigned)ceil_div(nrows, QB);
      const int sms = device_sm_count();
      int S = 1;
      double best = (double)ceil_div((int64_t)fgrid, sms);
      for (int cand_s = 2; cand_s <= kMaxSlices; ++cand_s) {
        if (n / cand_s < kMinSlice || (size_t)nrows * cand_s * k * 8 > kSliceScratchMax) break;
        const double waves = (double)ceil_div((int64_t)fgrid * cand_s, sms) / cand_s;
        if (waves < best - 1e-9) {
          best = waves;
          S = cand_s;
        }
      }
      int64_t slice_len = 0;
      uint32_t* sidx = nullptr;
      float* sval = nullptr;
      if (S > 1) {
        slice_len = ceil_div(ceil_div(n, S), CB) * CB;
        S = (int)ceil_div(n, slice_len);
        sidx = static_cast<uint32_t*>(ws.slices.ensure((size_t)nrows * S * k * 8));
        sval = reinterpret_cast<float*>(sidx + (size_t)nrows * S * k);
      }
      const dim3 g2(fgrid, (unsigned)S);
      if (C == 128) {
        BHG_CUDA(cudaFuncSetAttribute(knn_tile_kernel<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        knn_tile_kernel<128, true><<<g2, kThreads, smem, s>>>(X, n, dim, norms, rows, nrows, k, out_idx, out_dist,
                                                              nullptr, nullptr, nullptr, slice_len, sidx, sval);
      } else {
        BHG_CUDA(cudaFuncSetAttribute(knn_tile_kernel<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        knn_tile_kernel<256, true><<<g2, kThreads, smem, s>>>(X, n, dim, norms, rows, nrows, k, out_idx, out_dist,
                                                              nullptr, nullptr, nullptr, slice_len, sidx, sval);
      }
      BHG_LAUNCH_CHECK();
      if (S > 1) {
        slice_merge_kernel<<<(unsigned)ceil_div((int64_t)nrows * 32, 256), 256, 0, s>>>(sidx, sval, rows, nrows, S, k,
                                                                                        out_idx, out_dist);
        BHG_LAUNCH_CHECK();
      }
      ws.last_fallback_slices = S;
    } else {
      const size_t esmem = (size_t)4 * k * (sizeof(T) + sizeof(uint32_t));
      if (esmem > 48 * 1024)
        BHG_CUDA(cudaFuncSetAttribute(knn_exact_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem));
      knn_exact_kernel<T><<<(unsigned)ceil_div(nrows, 4), 128, esmem, s>>>(X, n, dim, k, rows, nullptr, nrows, out_idx,
                                                                          out_dist);
      BHG_LAUNCH_CHECK();
    }
  };
  ws.last_fallback_slices = 1;
  ws.last_brute_rows = 0;
  if (nfail > 0) {
    // Bounded re-scan: the rows that failed the certificate take every
    // candidate whose tensor-core value is within their bound (a superset of
    // their true neighbours) and re-rank that list exactly; rows whose list
    // overflows take the brute force.
    int cap = 0;
    if (fbound) {
      cap = (int)std::min<int64_t>(kListCap, (int64_t)(kListBytesMax / ((size_t)nfail * 4)) / 32 * 32);
      if (cap < 4 * 128) cap = 0;
    }
    if (cap > 0) {
      uint32_t* list = static_cast<uint32_t*>(ws.list.ensure((size_t)nfail * (cap + 1) * 4));
      uint32_t* list_cnt = list + (size_t)nfail * cap;
      knn_tc_bounded(n, dim, norms, fails, fbound, nfail, list, list_cnt, cap, ws.tc, s);
      unsigned* over_count = fail_count + 2;
      uint32_t* over = static_cast<uint32_t*>(ws.over.ensure((size_t)nfail * 4));
      const size_t esmem = (size_t)4 * k * (sizeof(T) + sizeof(uint32_t));
      if (esmem > 48 * 1024)
        BHG_CUDA(cudaFuncSetAttribute(knn_list_rerank_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem));
      knn_list_rerank_kernel<T><<<(unsigned)ceil_div(nfail, 4), 128, esmem, s>>>(X, dim, k, fails, nfail, list, list_cnt,
                                                                                cap, out_idx, out_dist, over, over_count);
      BHG_LAUNCH_CHECK();
      unsigned nover = 0;
      BHG_CUDA(cudaMemcpyAsync(&nover, over_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaStreamSynchronize(s));
      if (nover > 0) brute(over, nover);
      ws.last_brute_rows = nover;
    } else {
      brute(fails, nfail);
      ws.last_brute_rows = nfail;
    }
  }
  ws.last_fallback_rows = nfail;
  return (int64_t)nfail;
}

template <class T>
int64_t knn_euclidean_segmented(const T* X, int64_t total, int dim, int k, const std::vector<int64_t>& off,
                                const int64_t* d_off, const uint32_t* d_seg_of, uint32_t* out_idx, T* out_dist,
                                KnnWorkspace& ws, cudaStream_t s) {
  const int K = (int)off.size() - 1;
  for (int j = 0; j < K; ++j)
    if (k <= 0 || k > off[j + 1] - off[j] - 1) throw Error(ST_EINVAL, "error: k must be in [1, n_samples - 1].");
  const int C = k <= 96 ? 128 : (k <= 224 ? 256 : 0);
  const int qdim_max = C == 128 ? 256 : 128;
  if (C == 0 || dim > qdim_max)
    throw Error(ST_EINVAL, "error: the segmented kNN covers k <= 224 and dim <= " + std::to_string(qdim_max) + ".");
  unsigned* fail_count = static_cast<unsigned*>(ws.counters.ensure(64));
  BHG_CUDA(cudaMemsetAsync(fail_count, 0, 64, s));
  const float* Xf;
  if constexpr (std::is_same<T, float>::value) {
    Xf = X;
  } else {
    float* tmp = static_cast<float*>(ws.xf.ensure((size_t)total * dim * sizeof(float)));
    to_f32_kernel<T><<<1024, 256, 0, s>>>(X, total * dim, tmp);
    BHG_LAUNCH_CHECK();
    Xf = tmp;
  }
  float* norms = static_cast<float*>(ws.norms.ensure((size_t)total * sizeof(float)));
  unsigned* max_bits = fail_count + 1;
  sq_norm_kernel<<<(unsigned)ceil_div(total * 32, 256), 256, 0, s>>>(Xf, total, dim, norms, max_bits);
  BHG_LAUNCH_CHECK();
  // block table, largest sets first (each of their blocks scans the most candidates)
  std::vector<int> order(K);
  for (int j = 0; j < K; ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return off[a + 1] - off[a] > off[b + 1] - off[b]; });
  std::vector<int64_t> q0;
  std::vector<int32_t> bj;
  for (int j : order)
    for (int64_t q = off[j]; q < off[j + 1]; q += QB) {
      q0.push_back(q);
      bj.push_back(j);
    }
  const int64_t nblk = (int64_t)q0.size();
  int64_t* d_q0 = static_cast<int64_t*>(ws.blk.ensure((size_t)nblk * (8 + 4)));
  int32_t* d_bj = reinterpret_cast<int32_t*>(d_q0 + nblk);
  BHG_CUDA(cudaMemcpyAsync(d_q0, q0.data(), (size_t)nblk * 8, cudaMemcpyHostToDevice, s));
  BHG_CUDA(cudaMemcpyAsync(d_bj, bj.data(), (size_t)nblk * 4, cudaMemcpyHostToDevice, s));
  uint32_t* cand = static_cast<uint32_t*>(ws.cand.ensure((size_t)total * C * sizeof(uint32_t)));
  float* thr = static_cast<float*>(ws.thr.ensure((size_t)total * sizeof(float)));
  uint32_t* fails = static_cast<uint32_t*>(ws.fails.ensure((size_t)total * sizeof(uint32_t)));
  const size_t smem = ((size_t)dim * QB + DK * CB + QB * (CB + 1) + (size_t)QB * C * 2 + 2 * QB) * 4;
  const double simt_coef = (4.0 * dim + 16.0) / 16777216.0;
  if (C == 128 && (ws.pass == 0 || (ws.pass < 0 && use_tensor_cores()))) {
    // 128-query blocks per set, largest sets first
    std::vector<int64_t> tq0;
    std::vector<int32_t> tbj;
    for (int j : order)
      for (int64_t q = off[j]; q < off[j + 1]; q += 128) {
        tq0.push_back(q);
        tbj.push_back(j);
      }
    const int64_t tn = (int64_t)tq0.size();
    int64_t* t_q0 = static_cast<int64_t*>(ws.tc_blk.ensure((size_t)tn * (8 + 4)));
    int32_t* t_bj = reinterpret_cast<int32_t*>(t_q0 + tn);
    BHG_CUDA(cudaMemcpyAsync(t_q0, tq0.data(), (size_t)tn * 8, cudaMemcpyHostToDevice, s));
    BHG_CUDA(cudaMemcpyAsync(t_bj, tbj.data(), (size_t)tn * 4, cudaMemcpyHostToDevice, s));
    knn_tc_candidates(Xf, total, dim, norms, t_q0, t_bj, d_off, &off, tn, cand, thr, ws.tc, s);
    knn_rerank_kernel<T, 128><<<(unsigned)ceil_div(total, 4), 128, 0, s>>>(X, total, dim, k, cand, thr, norms, max_bits,
                                                                           out_idx, out_dist, fails, fail_count,
                                                                           knn_tc_error_coef(dim));
  } else if (C == 128 && dim <= kSelDimMax) {
    const size_t ssmem = sel_smem_bytes(dim);
    BHG_CUDA(cudaFuncSetAttribute(knn_cand_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssmem));
    knn_cand_kernel<<<(unsigned)nblk, kThreads, ssmem, s>>>(Xf, total, dim, norms, cand, thr, d_q0, d_bj, d_off);
    BHG_LAUNCH_CHECK();
    knn_rerank_kernel<T, 128><<<(unsigned)ceil_div(total, 4), 128, 0, s>>>(X, total, dim, k, cand, thr, norms, max_bits,
                                                                           out_idx, out_dist, fails, fail_count, simt_coef);
  } else if (C == 128) {
    BHG_CUDA(cudaFuncSetAttribute(knn_tile_kernel<128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    knn_tile_kernel<128, false><<<(unsigned)nblk, kThreads, smem, s>>>(Xf, total, dim, norms, nullptr, total, 128, cand,
                                                                      thr, d_q0, d_bj, d_off);
    BHG_LAUNCH_CHECK();
    knn_rerank_kernel<T, 128><<<(unsigned)ceil_div(total, 4), 128, 0, s>>>(X, total, dim, k, cand, thr, norms, max_bits,
                                                                           out_idx, out_dist, fails, fail_count, simt_coef);
  } else {
    BHG_CUDA(cudaFuncSetAttribute(knn_tile_kernel<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    knn_tile_kernel<256, false><<<(unsigned)nblk, kThreads, smem, s>>>(Xf, total, dim, norms, nullptr, total, 256, cand,
                                                                      thr, d_q0, d_bj, d_off);
    BHG_LAUNCH_CHECK();
    knn_rerank_kernel<T, 256><<<(unsigned)ceil_div(total, 4), 128, 0, s>>>(X, total, dim, k, cand, thr, norms, max_bits,
                                                                           out_idx, out_dist, fails, fail_count, simt_coef);
  }
  BHG_LAUNCH_CHECK();
  unsigned nfail = 0;
  BHG_CUDA(cudaMemcpyAsync(&nfail, fail_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  if (nfail > 0) {
    const size_t esmem = (size_t)4 * k * (sizeof(T) + sizeof(uint32_t));
    if (esmem > 48 * 1024)
      BHG_CUDA(cudaFuncSetAttribute(knn_exact_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem));
    knn_exact_kernel<T><<<(unsigned)ceil_div(nfail, 4), 128, esmem, s>>>(X, total, dim, k, fails, nullptr, nfail, out_idx,
                                                                        out_dist, d_off, d_seg_of);
    BHG_LAUNCH_CHECK();
  }
  ws.last_fallback_rows = nfail;
  return (int64_t)nfail;
}

template int64_t knn_euclidean<float>(const float*, int64_t, int, int, uint32_t*, float*, KnnWorkspace&, cudaStream_t);
template int64_t knn_euclidean<double>(const double*, int64_t, int, int, uint32_t*, double*, KnnWorkspace&,
                                       cudaStream_t);

template int64_t knn_euclidean_segmented<float>(const float*, int64_t, int, int, const std::vector<int64_t>&,
                                                 const int64_t*, const uint32_t*, uint32_t*, float*, KnnWorkspace&,
                                                 cudaStream_t);
template int64_t knn_euclidean_segmented<double>(const double*, int64_t, int, int, const std::vector<int64_t>&,
                                                  const int64_t*, const uint32_t*, uint32_t*, double*, KnnWorkspace&,
                                                  cudaStream_t);

}  // namespace bhg
