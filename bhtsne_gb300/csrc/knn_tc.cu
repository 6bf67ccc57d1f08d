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
// lane) against every candidate row of its point set, in tiles of 128. Two
// forms compute the same products in the same order:
//  - resident (rows of at most 128 dimensions): the query tile's hi / lo
//    parts sit in tensor memory for the whole CTA (the MMA's A operand), and
//    the candidate tiles come, split into hi / lo in advance, by bulk copies
//    (TMA engine) into a 4-deep shared-memory ring;
//  - staged (wider rows): producer warps split query and candidate chunks
//    from the FP32 rows into a 2-deep ring for every candidate tile.
// Operand tiles in shared memory use the no-swizzle K-major core-matrix
// layout (8 rows x 16 bytes per core matrix). Every wait on an mbarrier is
// bounded; on timeout the CTA raises the error flag, stops issuing work, waits
// (bounded) for its copies and MMAs in flight and releases its tensor memory.
#include "knn_tc.h"

#include <cfloat>
#include <cstdlib>

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

// A and B from shared memory
__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

// A from tensor memory (row i of A in lane i, one element per column), B from
// shared memory
__device__ __forceinline__ void mma_tf32_ta(uint32_t tmem, uint32_t a_tmem, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(tmem),
      "r"(a_tmem), "l"(b), "r"(kIdesc), "r"(accumulate));
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

// Bounded wait that ignores the abort flag: the exit path's wait for work
// already in flight (copies, MMAs), which completes whatever the other roles do.
__device__ __forceinline__ void mbar_drain(uint32_t mbar, uint32_t parity, int* err) {
  long long spins = 0;
  while (!mbar_try_wait(mbar, parity)) {
    if (++spins >= kSpinLimit) {
      atomicExch(err, 1);
      return;
    }
  }
}

__device__ __forceinline__ bool lt_vi(float a, uint32_t ai, float b, uint32_t bi) {
  return a < b || (a == b && ai < bi);
}

// Paired single-precision add and fused multiply-add (sm_100 and later):
// each lane is the scalar IEEE operation rounded to nearest.
__device__ __forceinline__ unsigned long long pk2(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk2(unsigned long long x, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x));
}
__device__ __forceinline__ unsigned long long add2(unsigned long long x, unsigned long long y) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(x), "l"(y));
  return r;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long x, unsigned long long y, unsigned long long z) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(x), "l"(y), "l"(z));
  return r;
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t b = __float_as_uint(x);
  if ((b & 0x7f800000u) != 0x7f800000u) b = (b + 0x1000u) & 0xffffe000u;
  return __uint_as_float(b);
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

constexpr int PK = 16;                     // dimensions per ring stage
constexpr int kSubTile = TQ * PK * 4;      // 8 KB: 128 rows x 16 dims
constexpr int kBuf = 32;                   // pending candidates per query between heap merges
constexpr int kLd = 16;                    // accumulator columns read per tcgen05.ld
constexpr size_t kSelSmem = (size_t)HEAPC * TQ * 8 + (size_t)kBuf * TQ * 8;  // heaps + pending lists

// staged form
constexpr int NST = 2;                     // ring depth
constexpr int kProducers = 96;
constexpr int kPipeThreads = 256;
constexpr int kStageBytes = 4 * kSubTile;  // query hi, query lo, candidate hi, candidate lo
constexpr size_t kPipeSmem = kSelSmem + (size_t)NST * kStageBytes;

// resident form
constexpr int NSR = 4;                     // ring depth
constexpr int kResThreads = 192;
constexpr int kResStage = 2 * kSubTile;    // candidate hi, candidate lo: 16 KB
constexpr size_t kResSmem = kSelSmem + (size_t)NSR * kResStage;
constexpr int kResDimMax = 128;
// tensor-memory columns: accumulators 0 .. 2 TC - 1, then the query tile's hi
// and lo parts, kResDimMax columns each (512 in all)
constexpr uint32_t kColQhi = 2 * TC, kColQlo = 2 * TC + kResDimMax, kResCols = 2 * TC + 2 * kResDimMax;
static_assert(kResCols == 512, "the resident form takes the whole tensor memory of its SM");
static_assert(kResSmem <= 227 * 1024 && kPipeSmem <= 227 * 1024, "shared memory per CTA");

// 16 consecutive accumulator columns of the warp's 32 lanes (asynchronous:
// tcgen05.wait::ld, then regs_ready, before the registers are read)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

// Ties the registers of a tcgen05.ld to the preceding tcgen05.wait::ld, so
// no read of them is scheduled before the wait.
__device__ __forceinline__ void regs_ready(uint32_t (&r)[16]) {
#pragma unroll
  for (int i = 0; i < 16; ++i) asm volatile("" : "+r"(r[i]));
}

// ---------------------------------------------------------------------------
// Selection role (warps 0-3, thread t = query row q0 + t = TMEM lane t): reads
// the 128 dot products d of a finished tile from one of two TMEM accumulators,
// forms v = (|q|^2 + |c|^2) - 2 d and keeps its best 128 (value, index) in a
// max-heap in shared memory. Candidates that beat the current 128-th best
// (the heap root, in registers) are appended to a per-thread pending list;
// when any lane's list could overflow on the next read, the whole warp merges
// its lists into the heaps together, so lanes insert in lockstep instead of
// one divergent heap update per candidate. Tiles that lie wholly inside the
// point set and do not hold the CTA's own queries (every tile but the
// diagonal one and a partial last one) take a path without index checks;
// tnorm, when given, holds each split tile's 128 squared norms (read as
// float4). Writes the sorted list and the threshold of its query.
// ---------------------------------------------------------------------------
__device__ void selection_role(uint32_t tmem, uint64_t* acc_full, uint64_t* acc_free, unsigned char* smem, int64_t q0,
                               int64_t lo, int64_t hi, int64_t ntiles, const float* __restrict__ norms,
                               const float* __restrict__ tnorm, int64_t tb, uint32_t* __restrict__ out_idx,
                               float* __restrict__ out_thr, volatile int* abort_flag, int* err) {
  float* hv = reinterpret_cast<float*>(smem);
  uint32_t* hx = reinterpret_cast<uint32_t*>(hv + HEAPC * TQ);
  uint2* pend = reinterpret_cast<uint2*>(hx + HEAPC * TQ);  // [kBuf][TQ] pending (value bits, index)
  const int tid = threadIdx.x, warp = tid >> 5;
  const int64_t qi = q0 + tid;
  const bool qvalid = qi < hi;
  const float qn = qvalid ? norms[qi] : 0.f;
  int cnt = 0, np = 0;
  float rootv = INFINITY;
  uint32_t rootx = SENTI;
  // In a tile without the query's own row and past the set's end, every
  // candidate's index exceeds every heap entry's (the scan runs in index
  // order), so (v, x) beats the root iff v < rootv once the heap is full, and
  // always while it is not: the test is v <= lim.
  float lim = INFINITY;
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
      lim = nextafterf(rootv, -INFINITY);
    }
  };
  for (int64_t t = 0; t < ntiles; ++t) {
    const int b = (int)(t & 1);
    if (!mbar_wait_bounded(smem_u32(&acc_full[b]), (uint32_t)((t >> 1) & 1), abort_flag, err)) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int64_t c0 = lo + t * TC;
    const bool fast = c0 + TC <= hi && (c0 + TC <= q0 || q0 + TQ <= c0);  // uniform over the CTA
    // 16 dot products of columns cb .. cb + 15 against the root
    auto chunk = [&](const uint32_t* r, int cb) {
      if (__any_sync(0xffffffffu, np > kBuf - kLd)) merge();
      if (!qvalid) return;
      const uint32_t x0 = (uint32_t)(c0 + cb);
      if (fast) {
        float cn[kLd];
        if (tnorm) {
          const float4* tn = reinterpret_cast<const float4*>(tnorm + (size_t)(tb + t) * TC + cb);
#pragma unroll
          for (int i = 0; i < kLd / 4; ++i) {
            const float4 v4 = __ldg(tn + i);
            cn[4 * i] = v4.x;
            cn[4 * i + 1] = v4.y;
            cn[4 * i + 2] = v4.z;
            cn[4 * i + 3] = v4.w;
          }
        } else {
#pragma unroll
          for (int c = 0; c < kLd; ++c) cn[c] = __ldg(norms + x0 + c);
        }
        // all 16 values first (independent), one test of their minimum
        // against the root, and only then the per-value tests and appends as
        // predicated stores (no branch per value)
        // v = (qn + cn) - 2 d, two values per instruction: qn + cn rounded,
        // then 2 d is exact, so the fused multiply-add rounds once more
        float v[kLd];
        const unsigned long long qq = pk2(qn, qn), m2 = pk2(-2.f, -2.f);
#pragma unroll
        for (int c = 0; c < kLd; c += 2) {
          const unsigned long long s2 = add2(qq, pk2(cn[c], cn[c + 1]));
          upk2(fma2(m2, pk2(__uint_as_float(r[c]), __uint_as_float(r[c + 1])), s2), v[c], v[c + 1]);
        }
        float m8[kLd / 2];
#pragma unroll
        for (int c = 0; c < kLd / 2; ++c) m8[c] = fminf(v[2 * c], v[2 * c + 1]);
#pragma unroll
        for (int w2 = kLd / 4; w2 >= 1; w2 >>= 1)
#pragma unroll
          for (int c = 0; c < w2; ++c) m8[c] = fminf(m8[2 * c], m8[2 * c + 1]);
        if (m8[0] <= lim) {
          uint32_t at = smem_u32(pend + (size_t)np * TQ + tid);
#pragma unroll
          for (int c = 0; c < kLd; ++c) {
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.le.f32 p, %2, %3;\n\t@p st.shared.v2.u32 [%0], {%4, %5};\n\t"
                "@p add.u32 %0, %0, %6;\n\t@p add.s32 %1, %1, 1;\n\t}\n"
                : "+r"(at), "+r"(np)
                : "f"(v[c]), "f"(lim), "r"(__float_as_uint(v[c])), "r"(x0 + c), "n"(TQ * (int)sizeof(uint2))
                : "memory");
          }
        }
      } else {
#pragma unroll
        for (int c = 0; c < kLd; ++c) {
          const int64_t j = c0 + cb + c;
          const bool in = j < hi && j != qi;
          const float v = fmaf(-2.f, __uint_as_float(r[c]), qn + __ldg(norms + (in ? j : qi)));
          if (in && lt_vi(v, (uint32_t)j, rootv, rootx)) {
            pend[np * TQ + tid] = make_uint2(__float_as_uint(v), (uint32_t)j);
            ++np;
          }
        }
      }
    };
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * TC);
#pragma unroll 1
    for (int cb = 0; cb < TC; cb += kLd) {
      uint32_t r[kLd];
      tmem_ld16(lane_base + (uint32_t)cb, r);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      regs_ready(r);
      chunk(r, cb);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    mbar_arrive(smem_u32(&acc_free[b]));
  }
  merge();
  if (qvalid && !*abort_flag) {
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

// ---------------------------------------------------------------------------
// Bounded role (warps 0-3 of the resident form's bounded re-scan, thread t =
// listed query slot q0 + t): every candidate j < hi whose value v (computed as
// in selection_role) is <= B goes to the query's list, in index order; the
// count, which may exceed cap, to *cnt_out.
// ---------------------------------------------------------------------------
__device__ void bound_role(uint32_t tmem, uint64_t* acc_full, uint64_t* acc_free, bool qvalid, int64_t hi,
                           int64_t ntiles, float qn, float B, const float* __restrict__ tnorm,
                           uint32_t* __restrict__ my_list, int cap, uint32_t* __restrict__ cnt_out,
                           volatile int* abort_flag, int* err) {
  const int warp = threadIdx.x >> 5;
  uint32_t cnt = 0;
  for (int64_t t = 0; t < ntiles; ++t) {
    const int b = (int)(t & 1);
    if (!mbar_wait_bounded(smem_u32(&acc_full[b]), (uint32_t)((t >> 1) & 1), abort_flag, err)) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int64_t c0 = t * TC;
    const bool full = c0 + TC <= hi;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * TC);
#pragma unroll 1
    for (int cb = 0; cb < TC; cb += kLd) {
      uint32_t r[kLd];
      tmem_ld16(lane_base + (uint32_t)cb, r);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      regs_ready(r);
      if (!qvalid) continue;
      const float4* tn = reinterpret_cast<const float4*>(tnorm + (size_t)t * TC + cb);
      float v[kLd];
#pragma unroll
      for (int i = 0; i < kLd / 4; ++i) {
        const float4 v4 = __ldg(tn + i);
        v[4 * i] = fmaf(-2.f, __uint_as_float(r[4 * i]), qn + v4.x);
        v[4 * i + 1] = fmaf(-2.f, __uint_as_float(r[4 * i + 1]), qn + v4.y);
        v[4 * i + 2] = fmaf(-2.f, __uint_as_float(r[4 * i + 2]), qn + v4.z);
        v[4 * i + 3] = fmaf(-2.f, __uint_as_float(r[4 * i + 3]), qn + v4.w);
      }
      float m8[kLd / 2];
#pragma unroll
      for (int c = 0; c < kLd / 2; ++c) m8[c] = fminf(v[2 * c], v[2 * c + 1]);
#pragma unroll
      for (int w2 = kLd / 4; w2 >= 1; w2 >>= 1)
#pragma unroll
        for (int c = 0; c < w2; ++c) m8[c] = fminf(m8[2 * c], m8[2 * c + 1]);
      if (m8[0] <= B) {
#pragma unroll
        for (int c = 0; c < kLd; ++c) {
          const int64_t j = c0 + cb + c;
          if (v[c] <= B && (full || j < hi)) {
            if (cnt < (uint32_t)cap) my_list[cnt] = (uint32_t)j;
            ++cnt;
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    mbar_arrive(smem_u32(&acc_free[b]));
  }
  if (qvalid && !*abort_flag) *cnt_out = cnt;
}

// ---------------------------------------------------------------------------
// Staged form. 8 warps split the work:
//   warps 0-3  selection (selection_role);
//   warp 4     one thread issues the MMAs: per candidate tile and 16-dim
//              chunk, 2 k-steps x 3 MMAs;
//   warps 5-7  stage 16-dim chunks of the query and candidate rows, split into
//              TF32 hi / lo parts on the fly from the FP32 rows, into a
//              2-deep shared-memory ring.
// mbarriers: full[s] (producers -> MMA), empty[s] (MMA commit -> producers),
// acc_full[b] (MMA commit -> selection), acc_free[b] (selection -> MMA).
// The selection of tile t overlaps the staging and MMAs of tile t + 1.
// ---------------------------------------------------------------------------
struct PipeBars {
  uint64_t full[NST], empty[NST], acc_full[2], acc_free[2], done;
};

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
  unsigned char* ring = smem + kSelSmem;
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
    // a CTA that starts after another one timed out does no work
    abort_flag = *reinterpret_cast<volatile int*>(err) ? 1 : 0;
    for (int i = 0; i < NST; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bars.full[i])), "r"(kProducers) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.empty[i])) : "memory");
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.acc_full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bars.acc_free[b])), "r"(TQ) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.done)) : "memory");
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
      // every MMA issued has completed before the tensor memory is released
      mma_commit(smem_u32(&bars.done));
      mbar_drain(smem_u32(&bars.done), 0, err);
    }
  } else {
    selection_role(tmem, bars.acc_full, bars.acc_free, smem, q0, lo, hi, ntiles, norms, nullptr, 0, out_idx, out_thr,
                   &abort_flag, err);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Resident form. 6 warps:
//   warps 0-3  write their query rows' hi / lo parts into tensor memory
//              (columns kColQhi.. and kColQlo..), then selection_role;
//   warp 4     one thread issues the MMAs (A from tensor memory, B from the
//              ring): per candidate tile and 16-dim chunk, 2 k-steps x 3 MMAs,
//              in the staged form's order;
//   warp 5     one thread issues the bulk copies of the candidate chunks
//              (16 KB each, hi and lo, from the split tiles) into the ring.
// mbarriers: full[s] (copy bytes landed -> MMA), empty[s] (MMA commit ->
// copier), acc_full / acc_free as in the staged form, qready (query in tensor
// memory -> MMA), done (last MMAs -> exit).
// ---------------------------------------------------------------------------
struct ResBars {
  uint64_t full[NSR], empty[NSR], acc_full[2], acc_free[2], qready, done;
};

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
      "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
      : "memory");
}

// Xs: split candidate tiles, tile T's chunk ch at Xs + (T * nch + ch) * 16 KB
// (hi sub-tile, then lo), and their squared norms, 128 per tile, in tnorm;
// tiles of the point set of block b numbered from tile_base[blk_job[b]] (from
// 0 without a block table).
// BOUND: the bounded re-scan of the listed rows ba.qrows (see bound_role)
// over every row of X, instead of the candidate lists.
struct BoundArgs {
  const uint32_t* qrows = nullptr;
  const float* qbound = nullptr;
  int64_t nq = 0;
  uint32_t* list = nullptr;
  uint32_t* list_cnt = nullptr;
  int cap = 0;
};

template <bool BOUND>
__global__ void __launch_bounds__(kResThreads, 1)
    knn_tc_res_kernel(const float* __restrict__ Xp, const float* __restrict__ Xs, const float* __restrict__ tnorm,
                      int64_t n, int dim_pad,
                      const float* __restrict__ norms, uint32_t* __restrict__ out_idx, float* __restrict__ out_thr,
                      const int64_t* __restrict__ blk_q0, const int32_t* __restrict__ blk_job,
                      const int64_t* __restrict__ seg_off, const int64_t* __restrict__ tile_base, int* __restrict__ err,
                      BoundArgs ba) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* ring = smem + kSelSmem;
  __shared__ __align__(8) ResBars bars;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int64_t q0 = (int64_t)blockIdx.x * TQ, lo = 0, hi = n, tb = 0;
  if (!BOUND && blk_q0) {
    const int jb = blk_job[blockIdx.x];
    q0 = blk_q0[blockIdx.x];
    lo = seg_off[jb];
    hi = seg_off[jb + 1];
    tb = tile_base[jb];
  }
  const int64_t ntiles = (hi - lo + TC - 1) / TC;
  const int nch = dim_pad / PK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kResCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    // a CTA that starts after another one timed out does no work
    abort_flag = *reinterpret_cast<volatile int*>(err) ? 1 : 0;
    for (int i = 0; i < NSR; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.full[i])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.empty[i])) : "memory");
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.acc_full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bars.acc_free[b])), "r"(TQ) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bars.qready)), "r"(TQ) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars.done)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == 5) {
    // ---- bulk copies of the candidate chunks (one thread)
    if (lane == 0) {
      int64_t it = 0;
      bool ok = true;
      for (int64_t t = 0; t < ntiles && ok && !abort_flag; ++t) {
        const float* tile = Xs + (size_t)(tb + t) * nch * (kResStage / 4);
        for (int ch = 0; ch < nch; ++ch) {
          const int st = (int)(it % NSR);
          const uint32_t par = (uint32_t)(((it / NSR) & 1) ^ 1);
          if (!mbar_wait_bounded(smem_u32(&bars.empty[st]), par, &abort_flag, err)) {
            ok = false;
            break;
          }
          const uint32_t fb = smem_u32(&bars.full[st]);
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(kResStage) : "memory");
          asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                           smem_u32(ring + (size_t)st * kResStage)),
                       "l"(tile + (size_t)ch * (kResStage / 4)), "r"(kResStage), "r"(fb)
                       : "memory");
          ++it;
        }
      }
      // the copies still in flight land before the CTA exits
      for (int64_t j = it > NSR ? it - NSR : 0; j < it; ++j)
        mbar_drain(smem_u32(&bars.full[j % NSR]), (uint32_t)((j / NSR) & 1), err);
    }
  } else if (warp == 4) {
    // ---- MMA issue (one thread)
    if (lane == 0) {
      bool ok = mbar_wait_bounded(smem_u32(&bars.qready), 0, &abort_flag, err);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      int64_t it = 0;
      for (int64_t t = 0; t < ntiles && ok && !abort_flag; ++t) {
        const int b = (int)(t & 1);
        if (!mbar_wait_bounded(smem_u32(&bars.acc_free[b]), (uint32_t)(((t >> 1) & 1) ^ 1), &abort_flag, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem + (uint32_t)(b * TC);
        for (int ch = 0; ch < nch; ++ch, ++it) {
          const int st = (int)(it % NSR);
          if (!mbar_wait_bounded(smem_u32(&bars.full[st]), (uint32_t)((it / NSR) & 1), &abort_flag, err)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t bh = smem_u32(ring + (size_t)st * kResStage), bl = bh + kSubTile;
#pragma unroll
          for (int ks = 0; ks < PK / 8; ++ks) {
            const uint32_t koff = (uint32_t)(ks * 2) * 128;
            const uint32_t sbo = (PK / 4) * 128;
            const uint64_t dbh = make_desc(bh + koff, 128, sbo);
            const uint64_t dbl = make_desc(bl + koff, 128, sbo);
            const uint32_t col = (uint32_t)(ch * PK + ks * 8);
            mma_tf32_ta(dacc, tmem + kColQhi + col, dbh, (ch > 0 || ks > 0) ? 1u : 0u);
            mma_tf32_ta(dacc, tmem + kColQhi + col, dbl, 1u);
            mma_tf32_ta(dacc, tmem + kColQlo + col, dbh, 1u);
          }
          mma_commit(smem_u32(&bars.empty[st]));
        }
        if (!ok) break;
        mma_commit(smem_u32(&bars.acc_full[b]));
      }
      // every MMA issued has completed before the tensor memory is released
      mma_commit(smem_u32(&bars.done));
      mbar_drain(smem_u32(&bars.done), 0, err);
    }
  } else {
    // ---- query row q0 + tid (listed row ba.qrows[q0 + tid] when BOUND) into
    // tensor memory lane tid, then selection
    const int64_t slot = q0 + tid;
    const bool qvalid = BOUND ? slot < ba.nq : slot < hi;
    const int64_t qi = BOUND ? (qvalid ? (int64_t)ba.qrows[slot] : 0) : slot;
    const float4* xq = reinterpret_cast<const float4*>(Xp + (qvalid ? qi : 0) * dim_pad);
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int ch = 0; ch < nch; ++ch) {
      uint32_t h[16], l[16];
#pragma unroll
      for (int i4 = 0; i4 < 4; ++i4) {
        const float4 v = qvalid ? __ldg(xq + ch * 4 + i4) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float hx = tf32_hi(x[e]);
          h[4 * i4 + e] = __float_as_uint(hx);
          l[4 * i4 + e] = __float_as_uint(x[e] - hx);
        }
      }
      tmem_st16(lane_base + kColQhi + (uint32_t)(ch * PK), h);
      tmem_st16(lane_base + kColQlo + (uint32_t)(ch * PK), l);
    }
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    mbar_arrive(smem_u32(&bars.qready));
    if (BOUND)
      bound_role(tmem, bars.acc_full, bars.acc_free, qvalid, hi, ntiles, qvalid ? norms[qi] : 0.f,
                 qvalid ? ba.qbound[slot] : 0.f, tnorm, ba.list + (size_t)(qvalid ? slot : 0) * ba.cap, ba.cap,
                 ba.list_cnt + (qvalid ? slot : 0), &abort_flag, err);
    else
      selection_role(tmem, bars.acc_full, bars.acc_free, smem, q0, lo, hi, ntiles, norms, tnorm, tb, out_idx, out_thr,
                     &abort_flag, err);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kResCols) : "memory");
  }
}

// Candidate tiles split into TF32 hi / lo core-matrix sub-tiles (the resident
// form's copy source). Tile T covers rows row0(T) .. row0(T) + 127 of its
// point set (zero beyond the set's end): row0 = 128 T without a set table,
// else set j = the last with tile_base[j] <= T and row0 = seg_off[j] + 128
// (T - tile_base[j]). One thread per 16-byte piece of a row; the first piece's
// thread also copies the row's squared norm into tnorm[128 T + r].
__global__ void split_tiles_kernel(const float* __restrict__ Xp, const float* __restrict__ norms, int64_t n,
                                   int dim_pad, const int64_t* __restrict__ seg_off,
                                   const int64_t* __restrict__ tile_base, int nseg, int64_t ntile,
                                   float* __restrict__ out, float* __restrict__ tnorm) {
  const int q4 = dim_pad / 4, nch = dim_pad / PK;
  const int64_t total = ntile * TC * q4;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(e % q4);
    const int64_t rt = e / q4;
    const int r = (int)(rt % TC);
    const int64_t T = rt / TC;
    int64_t row0 = T * TC, rend = n;
    if (tile_base) {
      int a = 0, b = nseg - 1;
      while (a < b) {
        const int m = (a + b + 1) >> 1;
        if (tile_base[m] <= T) a = m;
        else b = m - 1;
      }
      row0 = seg_off[a] + (T - tile_base[a]) * TC;
      rend = seg_off[a + 1];
    }
    const int64_t row = row0 + r;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (row < rend) v = __ldg(reinterpret_cast<const float4*>(Xp + row * dim_pad) + q);
    if (q == 0) tnorm[T * TC + r] = row < rend ? norms[row] : 0.f;
    float4 h, l;
    h.x = tf32_hi(v.x);
    h.y = tf32_hi(v.y);
    h.z = tf32_hi(v.z);
    h.w = tf32_hi(v.w);
    l.x = v.x - h.x;
    l.y = v.y - h.y;
    l.z = v.z - h.z;
    l.w = v.w - h.w;
    const int ch = q >> 2, k4 = q & 3;
    float* base = out + ((size_t)T * nch + ch) * (kResStage / 4);
    const int off = (((r >> 3) * (PK / 4) + k4) * 128 + (r & 7) * 16) / 4;
    *reinterpret_cast<float4*>(base + off) = h;
    *reinterpret_cast<float4*>(base + kSubTile / 4 + off) = l;
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

// BHTSNE_KNN_TC_STAGED=1 selects the staged form for every width (the two
// forms give the same candidate lists); read on every call.
bool staged_forced() {
  const char* e = getenv("BHTSNE_KNN_TC_STAGED");
  return e && *e && *e != '0';
}

}  // namespace

void knn_tc_candidates(const float* X, int64_t n, int dim, const float* norms, const int64_t* blk_q0,
                       const int32_t* blk_job, const int64_t* seg_off, const std::vector<int64_t>* off,
                       int64_t nblocks, uint32_t* cand, float* thr, KnnTcScratch& ws, cudaStream_t s) {
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
  const bool resident = dim_pad <= kResDimMax && !staged_forced();
  ws.last_resident = resident;
  ws.last_n = n;
  ws.last_dim = dim;
  ws.last_segmented = off != nullptr;
  ws.last_xp = Xp;
  if (resident) {
    // candidate tiles per point set, numbered set after set
    const int64_t* tbase = nullptr;
    int64_t ntile = ceil_div(n, TC);
    int nseg = 0;
    if (off) {
      nseg = (int)off->size() - 1;
      std::vector<int64_t> tb(nseg + 1);
      tb[0] = 0;
      for (int j = 0; j < nseg; ++j) tb[j + 1] = tb[j] + ceil_div((*off)[j + 1] - (*off)[j], TC);
      ntile = tb[nseg];
      int64_t* d_tb = static_cast<int64_t*>(ws.tile_base.ensure((size_t)(nseg + 1) * 8));
      BHG_CUDA(cudaMemcpyAsync(d_tb, tb.data(), (size_t)(nseg + 1) * 8, cudaMemcpyHostToDevice, s));
      tbase = d_tb;
    }
    const int nch = dim_pad / PK;
    float* Xs = static_cast<float*>(ws.split.ensure((size_t)ntile * (nch * kResStage + TC * 4)));
    float* tnorm = Xs + (size_t)ntile * nch * (kResStage / 4);
    split_tiles_kernel<<<(unsigned)std::min<int64_t>(ceil_div(ntile * TC * (dim_pad / 4), 256), sm_grid(8, 8192)), 256, 0,
                         s>>>(Xp, norms, n, dim_pad, seg_off, tbase, nseg, ntile, Xs, tnorm);
    BHG_LAUNCH_CHECK();
    BHG_CUDA(cudaFuncSetAttribute(knn_tc_res_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kResSmem));
    knn_tc_res_kernel<false><<<(unsigned)nblocks, kResThreads, kResSmem, s>>>(Xp, Xs, tnorm, n, dim_pad, norms, cand, thr,
                                                                              blk_q0, blk_job, seg_off, tbase, err,
                                                                              BoundArgs{});
    BHG_LAUNCH_CHECK();
  } else {
    BHG_CUDA(cudaFuncSetAttribute(knn_tc_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPipeSmem));
    knn_tc_pipe_kernel<<<(unsigned)nblocks, kPipeThreads, kPipeSmem, s>>>(Xp, n, dim_pad, norms, cand, thr, blk_q0,
                                                                          blk_job, seg_off, err);
    BHG_LAUNCH_CHECK();
  }
  int herr = 0;
  BHG_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(ST_ETIMEDOUT, "error: the tensor-core kNN pass timed out waiting for its MMAs.");
}

bool knn_tc_can_bound(const KnnTcScratch& ws, int64_t n, int dim) {
  return ws.last_resident && !ws.last_segmented && ws.last_n == n && ws.last_dim == dim && ws.split.ptr != nullptr;
}

void knn_tc_bounded(int64_t n, int dim, const float* norms, const uint32_t* qrows, const float* qbound, int64_t nq,
                    uint32_t* list, uint32_t* list_cnt, int cap, KnnTcScratch& ws, cudaStream_t s) {
  if (!knn_tc_can_bound(ws, n, dim)) throw Error(ST_EINTERNAL, "error: the bounded kNN re-scan needs the resident pass.");
  const int dim_pad = (dim + PK - 1) / PK * PK;
  const int64_t ntile = ceil_div(n, TC);
  const float* Xs = static_cast<const float*>(ws.split.ptr);
  const float* tnorm = Xs + (size_t)ntile * (dim_pad / PK) * (kResStage / 4);
  int* err = static_cast<int*>(ws.err.ensure(64));
  BHG_CUDA(cudaMemsetAsync(err, 0, 4, s));
  BoundArgs ba;
  ba.qrows = qrows;
  ba.qbound = qbound;
  ba.nq = nq;
  ba.list = list;
  ba.list_cnt = list_cnt;
  ba.cap = cap;
  BHG_CUDA(cudaFuncSetAttribute(knn_tc_res_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kResSmem));
  knn_tc_res_kernel<true><<<(unsigned)ceil_div(nq, TQ), kResThreads, kResSmem, s>>>(
      ws.last_xp, Xs, tnorm, n, dim_pad, norms, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, err, ba);
  BHG_LAUNCH_CHECK();
  int herr = 0;
  BHG_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(ST_ETIMEDOUT, "error: the tensor-core kNN re-scan timed out waiting for its MMAs.");
}

}  // namespace bhg
