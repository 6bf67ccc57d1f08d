// Tensor-core candidate pass of the exact kNN (see knn.cu for the pipeline).
//
// The distance tile |q|^2 + |c|^2 - 2 q.c of 128 queries x 128 candidates is
// a GEMM: q.c runs on the 5th-generation tensor cores (tcgen05.mma,
// kind::tf32, accumulator in tensor memory). TF32 keeps 10 mantissa bits, so
// every FP32 operand x is split as x = hi + lo (hi = x rounded to TF32, lo =
// x - hi, exact in FP32) and q.c = hi.hi + hi.lo + lo.hi (the lo.lo term is
// below 2^-22 |q||c|): three MMAs per k-step give FP32-level products. The
// re-rank recomputes every candidate exactly and the certificate accounts for
// this pass's error bound, so the neighbour lists stay exact.
//
// One CTA = 128 queries (one per selection thread and per tensor-memory
// lane) against every candidate row of its point set, in tiles of 128; see
// knn_tc_pipe_kernel for the warp roles. Operand tiles use the no-swizzle
// K-major core-matrix layout (8 rows x 16 bytes per core matrix). Every wait
// on an mbarrier is bounded; on timeout the CTA raises the error flag, stops
// issuing work and releases its tensor memory.
#include "knn_tc.h"

#include <cfloat>

namespace bhg {

namespace {

constexpr int TQ = 128;     // queries per CTA (= MMA M)
constexpr int TC = 128;     // candidates per tile (= MMA N)
constexpr int HEAPC = 128;  // candidates kept per query
constexpr uint32_t SENTI = 0xffffffffu;
constexpr long long kSpinLimit = 1LL << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// no-swizzle K-major shared-memory matrix descriptor: start, leading (K)
// byte offset between adjacent core matrices in K, stride byte offset between
// adjacent 8-row groups, descriptor version 1
__device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// kind::tf32 instruction descriptor: FP32 accumulator, TF32 A and B, both
// K-major, N = TC, M = TQ.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC >> 3) << 17) | ((uint32_t)(TQ >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool lt_vi(float a, uint32_t ai, float b, uint32_t bi) {
  return a < b || (a == b && ai < bi);
}

// Max-heap of (value, index) per thread, element i of thread t at [i * TQ + t].
__device__ __forceinline__ void heap_sift_down(float* hv, uint32_t* hi, int t, int cnt, int i) {
  float v = hv[i * TQ + t];
  uint32_t x = hi[i * TQ + t];
  for (;;) {
    int c = 2 * i + 1;
    if (c >= cnt) break;
    float cv = hv[c * TQ + t];
    uint32_t cx = hi[c * TQ + t];
    if (c + 1 < cnt) {
      const float rv = hv[(c + 1) * TQ + t];
      const uint32_t rx = hi[(c + 1) * TQ + t];
      if (lt_vi(cv, cx, rv, rx)) {
        c = c + 1;
        cv = rv;
        cx = rx;
      }
    }
    if (!lt_vi(v, x, cv, cx)) break;
    hv[i * TQ + t] = cv;
    hi[i * TQ + t] = cx;
    i = c;
  }
  hv[i * TQ + t] = v;
  hi[i * TQ + t] = x;
}

__device__ __forceinline__ void heap_push(float* hv, uint32_t* hi, int t, int& cnt, float v, uint32_t x) {
  int i = cnt++;
  while (i > 0) {
    const int p = (i - 1) >> 1;
    const float pv = hv[p * TQ + t];
    const uint32_t px = hi[p * TQ + t];
    if (!lt_vi(pv, px, v, x)) break;
    hv[i * TQ + t] = pv;
    hi[i * TQ + t] = px;
    i = p;
  }
  hv[i * TQ + t] = v;
  hi[i * TQ + t] = x;
}

// ---------------------------------------------------------------------------
// Pipelined form. 8 warps split the work:
//   warps 0-3  selection: thread t owns query row t (TMEM lane t), reads the
//              128 dot products of a finished tile from one of two TMEM
//              accumulators and keeps its best 128 in a max-heap in shared
//              memory (the fast path compares against the root in registers);
//   warp 4     one thread issues the MMAs: per candidate tile and 16-dim
//              chunk, 2 k-steps x 3 MMAs;
//   warps 5-7  stage 16-dim chunks of the query and candidate rows, split into
//              TF32 hi / lo parts on the fly from the FP32 rows, into a
//              3-deep shared-memory ring.
// mbarriers: full[s] (producers -> MMA), empty[s] (MMA commit -> producers),
// acc_full[b] (MMA commit -> selection), acc_free[b] (selection -> MMA).
// The selection of tile t overlaps the staging and MMAs of tile t + 1.
// ---------------------------------------------------------------------------
constexpr int PK = 16;                     // dimensions per ring stage
constexpr int NST = 2;                     // ring depth
constexpr int kProducers = 96;
constexpr int kPipeThreads = 256;
constexpr int kSubTile = TQ * PK * 4;      // 8 KB: 128 rows x 16 dims
constexpr int kStageBytes = 4 * kSubTile;  // query hi, query lo, candidate hi, candidate lo
constexpr int kBuf = 32;                   // pending candidates per query between heap merges
constexpr int kLd = 16;                    // accumulator columns read per tcgen05.ld
constexpr size_t kPipeSmem = (size_t)HEAPC * TQ * 8 + (size_t)kBuf * TQ * 8 + (size_t)NST * kStageBytes;

struct PipeBars {
  uint64_t full[NST], empty[NST], acc_full[2], acc_free[2];
};

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(mbar) : "memory");
}

// Bounded wait; false (and the abort flag raised) when it runs out or
// another role already aborted.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity, volatile int* abort_flag, int* err) {
  long long spins = 0;
  while (!mbar_try_wait(mbar, parity)) {
    if (*abort_flag) return false;
    if (++spins >= kSpinLimit) {
      *abort_flag = 1;
      atomicExch(err, 1);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t b = __float_as_uint(x);
  if ((b & 0x7f800000u) != 0x7f800000u) b = (b + 0x1000u) & 0xffffe000u;
  return __uint_as_float(b);
}

// Rows [q0, q0 + 128) (queries) and [c0, c0 + 128) (candidates) x dims
// [d0, d0 + 16) of Xp (row-major, ld = dim_pad, zero padded), split into hi /
// lo core-matrix sub-tiles at dst (query hi, query lo, candidate hi, candidate
// lo); rows >= row_end are 0. All loads are issued before the first store.
// A warp takes 8 rows x the four 16-byte pieces of their chunk: its loads
// touch 8 cache lines (not 32), and lanes 8q .. 8q + 7 hold piece q of the 8
// rows, so each quarter-warp phase of its 16-byte stores fills one whole core
// matrix (128 contiguous bytes, no bank conflict).
constexpr int kStageIters = (2 * TQ * (PK / 4) + kProducers - 1) / kProducers;
static_assert(PK == 16 && TQ % 8 == 0 && kProducers % 32 == 0, "stage_split's lane layout: 4 pieces per row, whole warps");

__device__ __forceinline__ void stage_split(const float* __restrict__ Xp, int64_t q0, int64_t c0, int64_t row_end,
                                            int dim_pad, int d0, unsigned char* dst, int p) {
  float4 x[kStageIters];
#pragma unroll
  for (int u = 0; u < kStageIters; ++u) {
    const int idx = p + u * kProducers;
    x[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (idx < 2 * TQ * (PK / 4)) {
      const int half = idx / (TQ * (PK / 4)), rem = idx % (TQ * (PK / 4));
      const int r = 8 * (rem >> 5) + (rem & 7), k4 = (rem >> 3) & 3;
      const int64_t row = (half ? c0 : q0) + r;
      if (row < row_end) x[u] = __ldg(reinterpret_cast<const float4*>(Xp + row * dim_pad + d0) + k4);
    }
  }
#pragma unroll
  for (int u = 0; u < kStageIters; ++u) {
    const int idx = p + u * kProducers;
    if (idx < 2 * TQ * (PK / 4)) {
      const int half = idx / (TQ * (PK / 4)), rem = idx % (TQ * (PK / 4));
      const int r = 8 * (rem >> 5) + (rem & 7), k4 = (rem >> 3) & 3;
      float4 h, l;
      h.x = tf32_hi(x[u].x);
      h.y = tf32_hi(x[u].y);
      h.z = tf32_hi(x[u].z);
      h.w = tf32_hi(x[u].w);
      l.x = x[u].x - h.x;
      l.y = x[u].y - h.y;
      l.z = x[u].z - h.z;
      l.w = x[u].w - h.w;
      const int off = ((r >> 3) * (PK / 4) + k4) * 128 + (r & 7) * 16;
      unsigned char* base = dst + (size_t)half * 2 * kSubTile;
      *reinterpret_cast<float4*>(base + off) = h;
      *reinterpret_cast<float4*>(base + kSubTile + off) = l;
    }
  }
}

__global__ void __launch_bounds__(kPipeThreads, 1)
    knn_tc_pipe_kernel(const float* __restrict__ Xp, int64_t n, int dim_pad, const float* __restrict__ norms,
                       uint32_t* __restrict__ out_idx, float* __restrict__ out_thr, const int64_t* __restrict__ blk_q0,
                       const int32_t* __restrict__ blk_job, const int64_t* __restrict__ seg_off, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  float* hv = reinterpret_cast<float*>(smem);
  uint32_t* hx = reinterpret_cast<uint32_t*>(hv + HEAPC * TQ);
  uint2* pend = reinterpret_cast<uint2*>(hx + HEAPC * TQ);  // [kBuf][TQ] pending (value bits, index)
  unsigned char* ring = reinterpret_cast<unsigned char*>(pend + kBuf * TQ);
  __shared__ __align__(8) PipeBars bars;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5;
  int64_t q0 = (int64_t)blockIdx.x * TQ, lo = 0, hi = n;
  if (blk_q0) {
    const int jb = blk_job[blockIdx.x];
    q0 = blk_q0[blockIdx.x];
    lo = seg_off[jb];
    hi = seg_off[jb + 1];
  }
  const int64_t ntiles = (hi - lo + TC - 1) / TC;
  const int nch = dim_pad / PK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(2 * TC)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < NST; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bars.full[i])), "r"(kProducers) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.empty[i])) : "memory");
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.acc_full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bars.acc_free[b])), "r"(TQ) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp >= 5) {
    // ---- producers
    const int p = tid - 5 * 32;
    int64_t it = 0;
    for (int64_t t = 0; t < ntiles && !abort_flag; ++t) {
      const int64_t c0 = lo + t * TC;
      for (int ch = 0; ch < nch; ++ch, ++it) {
        const int st = (int)(it % NST);
        const uint32_t par = (uint32_t)(((it / NST) & 1) ^ 1);
        if (!mbar_wait_bounded(smem_u32(&bars.empty[st]), par, &abort_flag, err)) break;
        stage_split(Xp, q0, c0, hi, dim_pad, ch * PK, ring + (size_t)st * kStageBytes, p);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(smem_u32(&bars.full[st]));
      }
    }
  } else if (warp == 4) {
    // ---- MMA issue (one thread)
    if ((tid & 31) == 0) {
      int64_t it = 0;
      for (int64_t t = 0; t < ntiles && !abort_flag; ++t) {
        const int b = (int)(t & 1);
        if (!mbar_wait_bounded(smem_u32(&bars.acc_free[b]), (uint32_t)(((t >> 1) & 1) ^ 1), &abort_flag, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem + (uint32_t)(b * TC);
        bool ok = true;
        for (int ch = 0; ch < nch; ++ch, ++it) {
          const int st = (int)(it % NST);
          if (!mbar_wait_bounded(smem_u32(&bars.full[st]), (uint32_t)((it / NST) & 1), &abort_flag, err)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t base = smem_u32(ring + (size_t)st * kStageBytes);
          const uint32_t ah = base, al = base + kSubTile, bh = base + 2 * kSubTile, bl = base + 3 * kSubTile;
#pragma unroll
          for (int ks = 0; ks < PK / 8; ++ks) {
            const uint32_t koff = (uint32_t)(ks * 2) * 128;
            const uint32_t sbo = (PK / 4) * 128;
            const uint64_t dah = make_desc(ah + koff, 128, sbo);
            const uint64_t dal = make_desc(al + koff, 128, sbo);
            const uint64_t dbh = make_desc(bh + koff, 128, sbo);
            const uint64_t dbl = make_desc(bl + koff, 128, sbo);
            mma_tf32(dacc, dah, dbh, (ch > 0 || ks > 0) ? 1u : 0u);
            mma_tf32(dacc, dah, dbl, 1u);
            mma_tf32(dacc, dal, dbh, 1u);
          }
          mma_commit(smem_u32(&bars.empty[st]));
        }
        if (!ok) break;
        mma_commit(smem_u32(&bars.acc_full[b]));
      }
    }
  } else {
    // ---- selection: query row tid. Candidates that beat the current C-th
    // best (the heap root, in registers) are appended to a per-thread pending
    // list; when any lane's list could overflow on the next read, the whole
    // warp merges its lists into the heaps together, so lanes insert in
    // lockstep instead of one divergent heap update per candidate.
    const int64_t qi = q0 + tid;
    const bool qvalid = qi < hi;
    const float qn = qvalid ? norms[qi] : 0.f;
    int cnt = 0, np = 0;
    float rootv = INFINITY;
    uint32_t rootx = SENTI;
    auto merge = [&]() {
      const int rounds = __reduce_max_sync(0xffffffffu, (unsigned)np);
      for (int i = 0; i < rounds; ++i) {
        if (i < np) {
          const uint2 e = pend[i * TQ + tid];
          const float v = __uint_as_float(e.x);
          if (cnt < HEAPC) {
            heap_push(hv, hx, tid, cnt, v, e.y);
          } else if (lt_vi(v, e.y, hv[tid], hx[tid])) {
            hv[tid] = v;
            hx[tid] = e.y;
            heap_sift_down(hv, hx, tid, cnt, 0);
          }
        }
      }
      np = 0;
      if (cnt == HEAPC) {
        rootv = hv[tid];
        rootx = hx[tid];
      }
    };
    for (int64_t t = 0; t < ntiles; ++t) {
      const int b = (int)(t & 1);
      if (!mbar_wait_bounded(smem_u32(&bars.acc_full[b]), (uint32_t)((t >> 1) & 1), &abort_flag, err)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int64_t c0 = lo + t * TC;
#pragma unroll 1
      for (int cb = 0; cb < TC; cb += kLd) {
        uint32_t r[kLd];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * TC + cb);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (__any_sync(0xffffffffu, np > kBuf - kLd)) merge();
        if (qvalid) {
#pragma unroll
          for (int c = 0; c < kLd; ++c) {
            const int64_t j = c0 + cb + c;
            const float v = qn + __ldg(norms + (j < hi ? j : lo)) - 2.f * __uint_as_float(r[c]);
            const uint32_t x = (uint32_t)j;
            if (j < hi && j != qi && lt_vi(v, x, rootv, rootx)) {
              pend[np * TQ + tid] = make_uint2(__float_as_uint(v), x);
              ++np;
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(smem_u32(&bars.acc_free[b]));
    }
    merge();
    if (qvalid && !abort_flag) {
      const int full = cnt;
      for (int m = cnt; m > 1; --m) {
        const float v0 = hv[tid];
        const uint32_t x0 = hx[tid];
        hv[tid] = hv[(m - 1) * TQ + tid];
        hx[tid] = hx[(m - 1) * TQ + tid];
        hv[(m - 1) * TQ + tid] = v0;
        hx[(m - 1) * TQ + tid] = x0;
        heap_sift_down(hv, hx, tid, m - 1, 0);
      }
      for (int t = 0; t < HEAPC; ++t) out_idx[qi * HEAPC + t] = t < full ? hx[t * TQ + tid] : SENTI;
      out_thr[qi] = full == HEAPC ? hv[(HEAPC - 1) * TQ + tid] : INFINITY;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC) : "memory");
  }
}

// X (n x dim) copied to rows of dim_pad with zero padding.
__global__ void pad_rows_kernel(const float* __restrict__ X, int64_t n, int dim, int dim_pad, float* __restrict__ out) {
  const int64_t total = n * dim_pad;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / dim_pad;
    const int d = (int)(e % dim_pad);
    out[e] = d < dim ? X[r * dim + d] : 0.f;
  }
}

}  // namespace

void knn_tc_candidates(const float* X, int64_t n, int dim, const float* norms, const int64_t* blk_q0,
                       const int32_t* blk_job, const int64_t* seg_off, int64_t nblocks, uint32_t* cand, float* thr,
                       KnnTcScratch& ws, cudaStream_t s) {
  const int dim_pad = (dim + PK - 1) / PK * PK;
  int* err = static_cast<int*>(ws.err.ensure(64));
  BHG_CUDA(cudaMemsetAsync(err, 0, 4, s));
  const float* Xp = X;
  if (dim_pad != dim) {
    float* pad = static_cast<float*>(ws.xhi.ensure((size_t)n * dim_pad * 4));
    pad_rows_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n * dim_pad, 256), sm_grid(8, 8192)), 256, 0, s>>>(X, n, dim, dim_pad,
                                                                                                    pad);
    BHG_LAUNCH_CHECK();
    Xp = pad;
  }
  BHG_CUDA(cudaFuncSetAttribute(knn_tc_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPipeSmem));
  knn_tc_pipe_kernel<<<(unsigned)nblocks, kPipeThreads, kPipeSmem, s>>>(Xp, n, dim_pad, norms, cand, thr, blk_q0,
                                                                        blk_job, seg_off, err);
  BHG_LAUNCH_CHECK();
  int herr = 0;
  BHG_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(ST_ETIMEDOUT, "error: the tensor-core kNN pass timed out waiting for its MMAs.");
}

}  // namespace bhg
