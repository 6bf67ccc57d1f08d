// Attractive forces over a 2-D blocked copy of P: compute_edge_forces
// (src/tsne/arena.rs:398-427), pos_i = sum_{j in row i} p_ij / (1 + |y_i - y_j|^2) (y_i - y_j).
//
// The points are cut into blocks of B = 2^tile_log consecutive slots. Entry
// (i, j) of P lives in tile (row block of i, column block of j); within a tile
// the entries keep the order of their rows (and, within a row, the row's own
// entry order). A unit of work is one row block and a range of its column
// tiles. For each column tile the unit's CTA copies that block of y into
// shared memory with one bulk copy (TMA engine, mbarrier), double-buffered so
// the next tile's copy overlaps the current tile's entries, and every y[j]
// gather of the tile reads shared memory. The CSR stream is the only DRAM
// traffic; y moves from L2 in whole 2^tile_log-point blocks instead of one
// 32-byte sector per gather.
//
// Arithmetic and determinism. Each entry's term is computed exactly as in
// compute_edge_forces. A row's terms within one tile are summed by one warp
// (a segmented scan over lanes), added once to the row's accumulator in
// shared memory; tiles are taken in order, and the partial sums of a row
// block's units are added in unit order by the reduce kernel. So the result
// is the same on every run; only the summation order differs from the
// reference's sequential row sum (within its rounding).
//
// Bounded waits: every mbarrier wait polls at most 2^22 times; on a timeout the
// CTA raises the fault word, loads its tiles with plain loads from then on,
// and before it exits waits once more (bounded) for copies still in flight.
// The host reads the fault word after the epochs and reports BHTSNE_ETIMEDOUT.
#include "epoch.h"

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <type_traits>

namespace bhg {

namespace {

constexpr int kBlkThreads = 512;
constexpr int kBlkWarps = kBlkThreads / 32;
constexpr int kBlkRounds = 8;     // rounds of 32 entries a warp loads ahead
constexpr int kSegPerBlock = 64;  // row segments per row block in the build
constexpr int kBuildWarps = 4;    // segments per CTA in the build

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int spin = 0; spin < (1 << 22); ++spin) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Build: per (row block, column tile, row segment) counts, one scan, then a
// stable scatter (one warp per row segment, rows in order).
// ---------------------------------------------------------------------------

// One warp per row segment of B / kSegPerBlock rows; hist holds one counter
// per column tile (per warp) in shared memory.
__global__ void blk_count_kernel(const uint64_t* __restrict__ rows, const uint32_t* __restrict__ cols, int64_t n,
                                 int tile_log, int nb, int64_t nseg, uint32_t* __restrict__ cnt) {
  extern __shared__ uint32_t hist[];  // kBuildWarps x nb
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t seg = (int64_t)blockIdx.x * kBuildWarps + warp;
  uint32_t* h = hist + (size_t)warp * nb;
  for (int c = lane; c < nb; c += 32) h[c] = 0;
  __syncwarp();
  const int64_t seg_rows = ((int64_t)1 << tile_log) / kSegPerBlock;
  if (seg < nseg) {
    const int64_t s0 = seg * seg_rows, s1 = min(s0 + seg_rows, n);
    for (int64_t r = s0; r < s1; ++r) {
      const uint64_t e1 = rows[r + 1];
      for (uint64_t eb = rows[r]; eb < e1; eb += 32) {
        const uint64_t e = eb + lane;
        uint32_t ct = 0xffffffffu;
        if (e < e1) ct = cols[e] >> tile_log;
        // one shared-memory atomic per column tile and chunk
        const uint32_t grp = __match_any_sync(kFull, ct);
        if (e < e1 && (grp & ((1u << lane) - 1u)) == 0) atomicAdd(&h[ct], (uint32_t)__popc(grp));
      }
    }
  }
  __syncwarp();
  if (seg < nseg) {
    const int64_t rb = seg / kSegPerBlock, sl = seg % kSegPerBlock;
    for (int c = lane; c < nb; c += 32) cnt[((size_t)rb * nb + c) * kSegPerBlock + sl] = h[c];
  }
}

// Rows of a segment in order; a chunk of 32 entries at a time, grouped by
// column tile with __match_any_sync so that each tile's entries keep the
// row's entry order.
template <class T>
__global__ void blk_scatter_kernel(const uint64_t* __restrict__ rows, const uint32_t* __restrict__ cols,
                                   const T* __restrict__ vals, int64_t n, int tile_log, int nb, int64_t nseg,
                                   const uint64_t* __restrict__ base, uint32_t* __restrict__ out_idx,
                                   T* __restrict__ out_val) {
  extern __shared__ unsigned long long cursor_all[];  // kBuildWarps x nb
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t seg = (int64_t)blockIdx.x * kBuildWarps + warp;
  if (seg >= nseg) return;  // uniform per warp; no block-wide barrier follows
  unsigned long long* cur = cursor_all + (size_t)warp * nb;
  const int64_t rb = seg / kSegPerBlock, sl = seg % kSegPerBlock;
  for (int c = lane; c < nb; c += 32) cur[c] = base[((size_t)rb * nb + c) * kSegPerBlock + sl];
  __syncwarp();
  const int64_t seg_rows = ((int64_t)1 << tile_log) / kSegPerBlock;
  const uint32_t bmask = (1u << tile_log) - 1u;
  const int64_t s0 = seg * seg_rows, s1 = min(s0 + seg_rows, n);
  const uint32_t lt = (1u << lane) - 1u;
  for (int64_t r = s0; r < s1; ++r) {
    const uint32_t local_row = (uint32_t)(r & bmask);
    const uint64_t e0 = rows[r], e1 = rows[r + 1];
    for (uint64_t eb = e0; eb < e1; eb += 32) {
      const uint64_t e = eb + lane;
      const bool act = e < e1;
      uint32_t ct = 0xffffffffu, lc = 0;
      T v = T(0);
      if (act) {
        const uint32_t c = cols[e];
        ct = c >> tile_log;
        lc = c & bmask;
        v = vals[e];
      }
      const uint32_t grp = __match_any_sync(kFull, ct);
      if (act) {
        const unsigned long long pos = cur[ct] + (unsigned long long)__popc(grp & lt);
        out_idx[pos] = (local_row << tile_log) | lc;
        out_val[pos] = v;
      }
      __syncwarp();
      if (act && (grp & lt) == 0) cur[ct] += (unsigned long long)__popc(grp);
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------
// The pass.
// ---------------------------------------------------------------------------
template <class T, int D>
__global__ void __launch_bounds__(kBlkThreads, 2) attractive_blocked_kernel(
    const uint64_t* __restrict__ base, const uint32_t* __restrict__ idx, const T* __restrict__ val,
    const T* __restrict__ y, int64_t n, int tile_log, int nb, int groups, T* __restrict__ part,
    unsigned* __restrict__ counter, int* __restrict__ fault) {
  extern __shared__ __align__(128) unsigned char blk_smem[];
  const int64_t B = (int64_t)1 << tile_log;
  T* tile_buf = reinterpret_cast<T*>(blk_smem);  // 2 x B x D
  T* acc = tile_buf + 2 * B * D;                 // B x D
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int unit_sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t bmask = (uint32_t)B - 1u;
  const int64_t units = (int64_t)nb * groups;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  uint32_t ph0 = 0u, ph1 = 0u;  // mbarrier phase parity of each tile buffer
  bool tma_ok = true;  // cleared after a wait timed out: tiles then come from global memory
  for (;;) {
    __syncthreads();  // the previous unit is finished by every warp
    if (threadIdx.x == 0) unit_sh = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int64_t u = unit_sh;
    if (u >= units) break;
    const int rb = (int)(u / groups), g = (int)(u % groups);
    const int ct0 = (int)((int64_t)nb * g / groups), ct1 = (int)((int64_t)nb * (g + 1) / groups);
    const int64_t row0 = (int64_t)rb * B;
    for (int64_t k = threadIdx.x; k < B * D; k += blockDim.x) acc[k] = T(0);
    // a tile's points: [ct * B, min(ct * B + B, n)); the bulk copy takes the
    // whole 16-byte part, plain loads the rest
    auto issue = [&](int ct, int buf) {
      const int64_t p0 = (int64_t)ct * B;
      const int64_t pts = min(B, n - p0);
      const uint32_t bytes = (uint32_t)(pts * D * sizeof(T)) & ~15u;
      if (threadIdx.x == 0 && bytes > 0 && tma_ok) {
        const uint32_t bar = smem_u32(&bars[buf]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(tile_buf + (size_t)buf * B * D)),
                     "l"(y + p0 * D), "r"(bytes), "r"(bar)
                     : "memory");
      }
    };
    auto finish = [&](int ct, int buf) {
      // wait for the bulk part, then load the tail (and everything after a timeout) directly
      const int64_t p0 = (int64_t)ct * B;
      const int64_t pts = min(B, n - p0);
      const uint32_t bytes = (uint32_t)(pts * D * sizeof(T)) & ~15u;
      int64_t from = 0;
      if (bytes > 0 && tma_ok) {
        const bool ok = mbar_wait(smem_u32(&bars[buf]), buf ? ph1 : ph0);
        if (buf) ph1 ^= 1u;
        else ph0 ^= 1u;
        if (__syncthreads_or(!ok)) {
          tma_ok = false;
          if (threadIdx.x == 0) atomicExch(fault, 1);
        } else {
          from = bytes / sizeof(T);
        }
      }
      T* dst = tile_buf + (size_t)buf * B * D;
      for (int64_t k = from + threadIdx.x; k < pts * D; k += blockDim.x) dst[k] = y[p0 * D + k];
      __syncthreads();
    };
    if (ct0 < ct1) issue(ct0, 0);
    for (int ct = ct0; ct < ct1; ++ct) {
      const int buf = (ct - ct0) & 1;
      if (ct + 1 < ct1) issue(ct + 1, buf ^ 1);  // that buffer's last reader finished at the previous barrier
      finish(ct, buf);
      const T* ty = tile_buf + (size_t)buf * B * D;
      const uint64_t tk = ((uint64_t)rb * nb + ct) * kSegPerBlock;
      const uint64_t e0 = base[tk], e1 = base[tk + kSegPerBlock];
      // warp w takes entries [e0 + w * len, e0 + (w + 1) * len), both ends moved
      // forward to the next row start, so that each row of the tile is summed by
      // exactly one warp
      const uint64_t len = (e1 - e0 + kBlkWarps - 1) / kBlkWarps;
      auto row_start = [&](uint64_t e) -> uint64_t {
        // first entry >= e that starts a row (or e1)
        while (e < e1 && e > e0) {
          const uint64_t q = e + lane;
          const uint32_t r_here = q < e1 ? (idx[q] >> tile_log) : 0xffffffffu;
          const uint32_t r_prev = q < e1 ? (idx[q - 1] >> tile_log) : 0xfffffffeu;
          const uint32_t starts = __ballot_sync(kFull, q >= e1 || r_here != r_prev);
          if (starts) return e + (uint64_t)(__ffs(starts) - 1);
          e += 32;
        }
        return e < e1 ? e : e1;
      };
      const uint64_t wb = row_start(min(e0 + (uint64_t)warp * len, e1));
      const uint64_t we = row_start(min(e0 + (uint64_t)(warp + 1) * len, e1));
      T carry[D];
#pragma unroll
      for (int a = 0; a < D; ++a) carry[a] = T(0);
      uint32_t carry_row = 0xffffffffu;
      for (uint64_t eb0 = wb; eb0 < we; eb0 += 32 * kBlkRounds) {
        // the loads of kBlkRounds rounds first (streamed past L1), then the
        // rounds themselves: enough bytes in flight per warp to cover DRAM latency
        uint32_t wv[kBlkRounds];
        T pv[kBlkRounds];
#pragma unroll
        for (int u = 0; u < kBlkRounds; ++u) {
          const uint64_t e = eb0 + 32 * u + lane;
          wv[u] = 0xffffffffu;
          pv[u] = T(0);
          if (e < we) {
            wv[u] = __ldcs(idx + e);
            pv[u] = __ldcs(val + e);
          }
        }
        // the first row of the batch after this one (for the last round's carry)
        const uint64_t nb0 = eb0 + 32 * kBlkRounds;
        const uint32_t after = (nb0 < we && lane == 0) ? (__ldg(idx + nb0) >> tile_log) : 0xffffffffu;
        const uint32_t after_row = __shfl_sync(kFull, after, 0);
#pragma unroll
        for (int u = 0; u < kBlkRounds; ++u) {
          const uint64_t eb = eb0 + 32 * u;
          if (eb >= we) break;  // uniform
          const bool act = wv[u] != 0xffffffffu;
          const uint32_t row = act ? (wv[u] >> tile_log) : 0xffffffffu;
          T c[D];
#pragma unroll
          for (int a = 0; a < D; ++a) c[a] = T(0);
          if (act) {
            const uint32_t col = wv[u] & bmask;
            T disp[D];
            T dist = T(0);
#pragma unroll
            for (int a = 0; a < D; ++a) {
              disp[a] = y[(row0 + row) * D + a] - ty[(size_t)col * D + a];
              dist += disp[a] * disp[a];
            }
            const T factor = pv[u] / (dist + T(1));
#pragma unroll
            for (int a = 0; a < D; ++a) c[a] = factor * disp[a];
          }
          // segmented inclusive scan over lanes (segments = runs of one row)
          const uint32_t prev_row = __shfl_up_sync(kFull, row, 1);
          const bool head = lane == 0 || prev_row != row;
          const uint32_t heads = __ballot_sync(kFull, head);
          const int seg_start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
          // the carry of the previous round joins the first segment when it continues that row
          if (lane == 0 && row == carry_row) {
#pragma unroll
            for (int a = 0; a < D; ++a) c[a] = carry[a] + c[a];
          }
          for (int o = 1; o < 32; o <<= 1) {
            const bool take = lane - o >= seg_start;
            if (!__any_sync(kFull, take)) break;
#pragma unroll
            for (int a = 0; a < D; ++a) {
              const T up = __shfl_up_sync(kFull, c[a], o);
              if (take) c[a] += up;
            }
          }
          const uint32_t next_row = __shfl_down_sync(kFull, row, 1);
          const bool tail = act && (lane == 31 || next_row != row);
          // the last segment may continue in the next round: it becomes the carry
          const uint32_t last_row = __shfl_sync(kFull, row, 31);
          uint32_t nrow = after_row;  // the next round's first row
          if (u + 1 < kBlkRounds) {
            const uint32_t wn = __shfl_sync(kFull, wv[u + 1 < kBlkRounds ? u + 1 : u], 0);
            nrow = (eb + 32 < we) ? (wn >> tile_log) : 0xffffffffu;
          }
          const bool cont = (eb + 32 < we) && nrow == last_row;
#pragma unroll
          for (int a = 0; a < D; ++a) carry[a] = __shfl_sync(kFull, c[a], 31);
          carry_row = cont ? last_row : 0xffffffffu;
          if (tail && !(cont && lane == 31)) {
#pragma unroll
            for (int a = 0; a < D; ++a) acc[(size_t)row * D + a] += c[a];
          }
        }
      }
      __syncthreads();  // every warp is done with this tile buffer
    }
    T* out = part + (size_t)u * B * D;
    for (int64_t k = threadIdx.x; k < B * D; k += blockDim.x) out[k] = acc[k];
  }
  if (!tma_ok) {
    // a timed-out copy may still be in flight: wait for both buffers, bounded
    mbar_wait(smem_u32(&bars[0]), ph0);
    mbar_wait(smem_u32(&bars[1]), ph1);
  }
}

// pos of row block rb = the unit partials in unit order; resets the work counter.
template <class T, int D>
__global__ void blk_reduce_kernel(const T* __restrict__ part, int64_t n, int tile_log, int groups, T* __restrict__ pos,
                                  unsigned* __restrict__ counter) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *counter = 0u;
  if (i >= n * D) return;
  const int64_t row = i / D, a = i % D;
  const int64_t rb = row >> tile_log, lr = row & (((int64_t)1 << tile_log) - 1);
  const int64_t B = (int64_t)1 << tile_log;
  T s = T(0);
  for (int g = 0; g < groups; ++g) s += part[(((size_t)rb * groups + g) * B + lr) * D + a];
  pos[i] = s;
}

}  // namespace

template <class T, int D>
static void prepare_blocked_d(AttrBlocks& ab) {
  const int64_t B = (int64_t)1 << ab.tile_log;
  const size_t smem = (size_t)3 * B * D * sizeof(T);
  static std::atomic<int> configured[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if ((size_t)configured[dev].load() < smem) {
    BHG_CUDA(cudaFuncSetAttribute(attractive_blocked_kernel<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    configured[dev].store((int)smem);
  }
  int per_sm = 0;
  BHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, attractive_blocked_kernel<T, D>, kBlkThreads, smem));
  const int64_t units = (int64_t)ab.nb * ab.groups;
  ab.grid = (int)std::min<int64_t>(units, (int64_t)std::max(per_sm, 1) * device_sm_count());
  ab.smem = smem;
}

template <class T, int D>
static void launch_blocked_d(const AttrBlocks& ab, const T* y, T* pos, cudaStream_t s) {
  attractive_blocked_kernel<T, D><<<(unsigned)ab.grid, kBlkThreads, ab.smem, s>>>(
      static_cast<const uint64_t*>(ab.base.ptr), static_cast<const uint32_t*>(ab.idx.ptr),
      static_cast<const T*>(ab.val.ptr), y, ab.n, ab.tile_log, ab.nb, ab.groups, static_cast<T*>(ab.part.ptr),
      static_cast<unsigned*>(ab.counter.ptr), static_cast<int*>(ab.counter.ptr) + 1);
  BHG_LAUNCH_CHECK();
  blk_reduce_kernel<T, D><<<(unsigned)ceil_div(ab.n * D, 256), 256, 0, s>>>(
      static_cast<const T*>(ab.part.ptr), ab.n, ab.tile_log, ab.groups, pos, static_cast<unsigned*>(ab.counter.ptr));
  BHG_LAUNCH_CHECK();
}

int attr_blocks_tile_log(int D, size_t value_bytes, int64_t n) {
  const char* env = getenv("BHTSNE_ATTR_BLOCKED");
  if (env && atoi(env) == 0) return 0;
  if (D < 1 || D > 3) return 0;
  // two tile buffers and the accumulators in at most 100 KB of shared memory
  // (two CTAs per SM)
  int tl = 14;
  while (tl > 8 && (size_t)3 * ((size_t)1 << tl) * D * value_bytes > (size_t)100 * 1024) --tl;
  // enough row blocks to fill the device; below that the plain task pass is better
  if ((n >> tl) < 8) return 0;
  // the build's counters: nb^2 x kSegPerBlock
  const int64_t nb = (n + ((int64_t)1 << tl) - 1) >> tl;
  if (nb > 1024) return 0;
  return tl;
}

template <class T>
void build_attr_blocks(AttrBlocks& ab, int D, const uint64_t* rows, const uint32_t* cols, const T* vals, int64_t n,
                       int64_t nnz, int tile_log, cudaStream_t s) {
  ab.tile_log = 0;
  ab.n = n;
  ab.D = D;
  ab.nnz = nnz;
  if (tile_log <= 0 || n <= 0) return;
  const int64_t B = (int64_t)1 << tile_log;
  const int nb = (int)((n + B - 1) / B);
  const int64_t nseg = (int64_t)nb * kSegPerBlock;
  const size_t ncnt = (size_t)nb * nb * kSegPerBlock;
  uint32_t* cnt = static_cast<uint32_t*>(ab.cnt.ensure(ncnt * 4));
  uint64_t* base = static_cast<uint64_t*>(ab.base.ensure((ncnt + 1) * 8));
  const unsigned grid = (unsigned)ceil_div(nseg, kBuildWarps);
  const size_t hist_smem = (size_t)kBuildWarps * nb * 4;
  if (hist_smem > 48 * 1024)
    BHG_CUDA(cudaFuncSetAttribute(blk_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hist_smem));
  blk_count_kernel<<<grid, kBuildWarps * 32, hist_smem, s>>>(rows, cols, n, tile_log, nb, nseg, cnt);
  BHG_LAUNCH_CHECK();
  scan_u32_to_u64(cnt, base, (int64_t)ncnt, ab.scan_tmp, s);
  uint32_t* oidx = static_cast<uint32_t*>(ab.idx.ensure((size_t)std::max<int64_t>(nnz, 1) * 4));
  T* oval = static_cast<T*>(ab.val.ensure((size_t)std::max<int64_t>(nnz, 1) * sizeof(T)));
  const size_t cur_smem = (size_t)kBuildWarps * nb * 8;
  if (cur_smem > 48 * 1024)
    BHG_CUDA(cudaFuncSetAttribute(blk_scatter_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cur_smem));
  blk_scatter_kernel<T><<<grid, kBuildWarps * 32, cur_smem, s>>>(rows, cols, vals, n, tile_log, nb, nseg, base, oidx,
                                                                 oval);
  BHG_LAUNCH_CHECK();
  ab.nb = nb;
  // units: one row block and a range of its column tiles, about four per SM
  const int sms = device_sm_count();
  ab.groups = (int)std::min<int64_t>(nb, std::max<int64_t>(1, ceil_div((int64_t)4 * sms, nb)));
  ab.part.ensure((size_t)nb * ab.groups * B * D * sizeof(T));
  unsigned* counter = static_cast<unsigned*>(ab.counter.ensure(64));
  BHG_CUDA(cudaMemsetAsync(counter, 0, 64, s));  // work counter, fault word
  ab.tile_log = tile_log;
  with_dim<1, 3>(D, "error: the blocked attractive pass covers D in 1..3.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    prepare_blocked_d<T, DD>(ab);
  });
}

bool attr_blocks_fault(const AttrBlocks& ab, cudaStream_t s) {
  if (ab.tile_log <= 0) return false;
  int f = 0;
  BHG_CUDA(cudaMemcpyAsync(&f, static_cast<int*>(ab.counter.ptr) + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  return f != 0;
}

template <class T>
void launch_attractive_blocked(const AttrBlocks& ab, const T* y, T* pos, cudaStream_t s) {
  if (ab.tile_log <= 0) throw Error(ST_EINTERNAL, "error: the blocked attractive pass was not built.");
  with_dim<1, 3>(ab.D, "error: the blocked attractive pass covers D in 1..3.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    launch_blocked_d<T, DD>(ab, y, pos, s);
  });
}

#define BHG_INST_BLK(T)                                                                                           \
  template void build_attr_blocks<T>(AttrBlocks&, int, const uint64_t*, const uint32_t*, const T*, int64_t, int64_t, \
                                     int, cudaStream_t);                                                           \
  template void launch_attractive_blocked<T>(const AttrBlocks&, const T*, T*, cudaStream_t);
BHG_INST_BLK(float)
BHG_INST_BLK(double)

}  // namespace bhg
