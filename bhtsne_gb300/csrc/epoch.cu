// Per-epoch kernels shared by every fitting method: the attractive CSR pass,
// the fused gains/momentum update with the FP64 mean for recentring, the
// sparse KL divergence, and the dense O(N^2) kernels of the exact method.
//
// Reference behaviour restated (bhtsne 0.7.10):
//  * compute_edge_forces: src/tsne/arena.rs:398-427,
//    pos_i = sum_{j in row i} p_ij / (1 + |y_i - y_j|^2) (y_i - y_j).
//  * gradient_descent_step: src/tsne/mod.rs:470-516 (g = pos - neg / Z;
//    gain + 0.2 on a sign change of (g, u), else * 0.8, floored at 0.01;
//    u = mu u - lr gain g; y += u), update_solution: :423-451 (exact method,
//    g = dy), zero_mean: :534-568, constants :29-31.
//  * sparse_kl_divergence: src/tsne/mod.rs:738-775, including the indexing of
//    the value array by row number (:768-770) when `quirk` is set.
//  * exact epoch: src/lib.rs:567-638 (Q includes the diagonal, Z includes N,
//    dy_i = sum_j (p_ij - q_ij / Z) q_ij (y_i - y_j)); evaluate_error:
//    src/tsne/mod.rs:579-618; dense symmetrisation: src/lib.rs:548-554.
#include "epoch.h"

#include <cstdint>
#include <cstdlib>
#include <type_traits>

namespace bhg {

namespace {

// y[j] as one 2-wide load when D = 2 and y is aligned for it (VEC), else per axis.
template <class T, int D, bool VEC>
__device__ __forceinline__ void load_point(const T* __restrict__ y, int64_t j, T (&v)[D]) {
  if constexpr (VEC && D == 2 && std::is_same<T, float>::value) {
    const float2 t = __ldg(reinterpret_cast<const float2*>(y) + j);
    v[0] = t.x;
    v[1] = t.y;
  } else if constexpr (VEC && D == 2 && std::is_same<T, double>::value) {
    const double2 t = __ldg(reinterpret_cast<const double2*>(y) + j);
    v[0] = t.x;
    v[1] = t.y;
  } else {
#pragma unroll
    for (int a = 0; a < D; ++a) v[a] = y[j * D + a];
  }
}

// ---------------------------------------------------------------------------
// Attractive forces over bounded tasks (see AttrTasks). A task is at most
// kU x 32 entries: each lane issues its kU column/value loads (streaming, so
// that L1 keeps the gathered y lines) and kU gathers at once.
// ---------------------------------------------------------------------------
struct AttrTask {
  uint64_t begin;  // first CSR entry
  uint32_t slot;
  uint32_t len;    // entries; bit 31: the row has several tasks (write a partial)
};

constexpr uint32_t kPartialBit = 0x80000000u;

// The terms of a task's entries lane + 32 u, u < NU, added to acc. Entries
// past the task's end add exactly zero, so running NU = ceil(len / 32) steps
// instead of kU gives the same sums.
template <class T, int D, bool VEC, int NU>
__device__ __forceinline__ void attr_accumulate(uint64_t begin, int len, int64_t slot, int lane,
                                                const uint32_t* __restrict__ cols, const T* __restrict__ vals,
                                                const T* __restrict__ y, const T (&yi)[D], T (&acc)[D]) {
  uint32_t j[NU];
  T p[NU];
  T yj[NU][D];
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    const int e = lane + 32 * u;
    j[u] = e < len ? __ldcs(cols + begin + e) : (uint32_t)slot;
    p[u] = e < len ? __ldcs(vals + begin + e) : T(0);
  }
#pragma unroll
  for (int u = 0; u < NU; ++u) load_point<T, D, VEC>(y, (int64_t)j[u], yj[u]);
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    T disp[D];
    T dist = T(0);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      disp[a] = yi[a] - yj[u][a];
      dist += disp[a] * disp[a];
    }
    const T factor = p[u] / (dist + T(1));
#pragma unroll
    for (int a = 0; a < D; ++a) acc[a] += factor * disp[a];
  }
}

template <class T, int D, bool VEC, int kU>
__global__ void __launch_bounds__(256) attractive_task_kernel(const AttrTask* __restrict__ tasks, int64_t ntasks,
                                                              const uint32_t* __restrict__ cols,
                                                              const T* __restrict__ vals, const T* __restrict__ y,
                                                              T* __restrict__ pos, T* __restrict__ part) {
  const int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= ntasks) return;  // uniform per warp
  const AttrTask tk = tasks[t];
  const int len = (int)(tk.len & ~kPartialBit);
  const int64_t slot = tk.slot;
  T yi[D], acc[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    yi[a] = y[slot * D + a];
    acc[a] = T(0);
  }
  // as many steps of 32 entries as the task holds (uniform per warp)
  switch ((len + 31) >> 5) {
    case 0:
      break;
    case 1:
      attr_accumulate<T, D, VEC, 1>(tk.begin, len, slot, lane, cols, vals, y, yi, acc);
      break;
    case 2:
      if constexpr (kU >= 2) attr_accumulate<T, D, VEC, 2>(tk.begin, len, slot, lane, cols, vals, y, yi, acc);
      break;
    case 3:
      if constexpr (kU >= 3) attr_accumulate<T, D, VEC, 3>(tk.begin, len, slot, lane, cols, vals, y, yi, acc);
      break;
    case 4:
      if constexpr (kU >= 4) attr_accumulate<T, D, VEC, 4>(tk.begin, len, slot, lane, cols, vals, y, yi, acc);
      break;
    case 5:
      if constexpr (kU >= 5) attr_accumulate<T, D, VEC, 5>(tk.begin, len, slot, lane, cols, vals, y, yi, acc);
      break;
    case 6:
      if constexpr (kU >= 6) attr_accumulate<T, D, VEC, 6>(tk.begin, len, slot, lane, cols, vals, y, yi, acc);
      break;
    case 7:
      if constexpr (kU >= 7) attr_accumulate<T, D, VEC, 7>(tk.begin, len, slot, lane, cols, vals, y, yi, acc);
      break;
    default:
      if constexpr (kU >= 8) attr_accumulate<T, D, VEC, 8>(tk.begin, len, slot, lane, cols, vals, y, yi, acc);
      break;
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[a] += __shfl_xor_sync(kFull, acc[a], o);
  }
  if (lane == 0) {
    T* out = (tk.len & kPartialBit) ? part + t * D : pos + slot * D;
#pragma unroll
    for (int a = 0; a < D; ++a) out[a] = acc[a];
  }
}

// Rows of several tasks: the partial sums in task order.
template <class T, int D>
__global__ void attractive_fixup_kernel(const uint32_t* __restrict__ longs, int64_t nlong,
                                        const uint64_t* __restrict__ off, const T* __restrict__ part,
                                        T* __restrict__ pos) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlong) return;
  const int64_t slot = longs[i];
  T acc[D];
#pragma unroll
  for (int a = 0; a < D; ++a) acc[a] = T(0);
  for (uint64_t t = off[slot]; t < off[slot + 1]; ++t) {
#pragma unroll
    for (int a = 0; a < D; ++a) acc[a] += part[t * D + a];
  }
#pragma unroll
  for (int a = 0; a < D; ++a) pos[slot * D + a] = acc[a];
}

__global__ void task_count_kernel(const uint64_t* __restrict__ rows, int64_t n, int task_len,
                                  uint32_t* __restrict__ cnt) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint64_t len = rows[s + 1] - rows[s];
  cnt[s] = len <= (uint64_t)task_len ? 1u : (uint32_t)((len + task_len - 1) / task_len);
}

__global__ void task_fill_kernel(const uint64_t* __restrict__ rows, int64_t n, int task_len,
                                 const uint64_t* __restrict__ off, AttrTask* __restrict__ tasks,
                                 uint32_t* __restrict__ longs, unsigned long long* __restrict__ nlong) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint64_t r0 = rows[s], len = rows[s + 1] - r0;
  const uint64_t t0 = off[s], c = off[s + 1] - t0;
  const uint32_t flag = c > 1 ? kPartialBit : 0u;
  for (uint64_t q = 0; q < c; ++q) {
    const uint64_t b = q * (uint64_t)task_len;
    const uint64_t l = len - b < (uint64_t)task_len ? len - b : (uint64_t)task_len;
    tasks[t0 + q] = AttrTask{r0 + b, (uint32_t)s, (uint32_t)l | flag};
  }
  if (c > 1) longs[atomicAdd(nlong, 1ull)] = (uint32_t)s;
}

// ---------------------------------------------------------------------------
// Seeded initial embedding. Pair i needs LCG states 2i + 1 and 2i + 2: the
// state 2i is reached from the seed by composing the affine step with itself
// (binary powers, O(log i)), so every pair is independent.
// ---------------------------------------------------------------------------
constexpr uint64_t kLcgMul = 6364136223846793005ULL, kLcgAdd = 1442695040888963407ULL;

__device__ __forceinline__ uint64_t lcg_jump(uint64_t state, uint64_t steps) {
  uint64_t acc_mul = 1, acc_add = 0, cur_mul = kLcgMul, cur_add = kLcgAdd;
  while (steps) {
    if (steps & 1) {
      acc_mul *= cur_mul;
      acc_add = acc_add * cur_mul + cur_add;
    }
    cur_add = (cur_mul + 1) * cur_add;
    cur_mul *= cur_mul;
    steps >>= 1;
  }
  return acc_mul * state + acc_add;
}

template <class T>
__global__ void random_init_kernel(T* __restrict__ y, int64_t count, uint64_t seed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (2 * i >= count) return;
  const uint64_t s1 = lcg_jump(seed, 2 * (uint64_t)i + 1);
  const uint64_t s2 = s1 * kLcgMul + kLcgAdd;
  const double u1 = ((double)(s1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double u2 = ((double)(s2 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double r = sqrt(-2.0 * log(u1));
  const double a = 2 * 3.14159265358979323846 * u2;
  y[2 * i] = (T)(1e-4 * r * cos(a));
  if (2 * i + 1 < count) y[2 * i + 1] = (T)(1e-4 * r * sin(a));
}

// ---------------------------------------------------------------------------
// Renumbering of the embedding layout (see launch_renumber).
// ---------------------------------------------------------------------------
template <class T, int D>
__global__ void renumber_gather_kernel(const uint32_t* __restrict__ order, const uint32_t* __restrict__ ext_old,
                                       int64_t n, const T* __restrict__ y, const T* __restrict__ uy,
                                       const T* __restrict__ gains, T* __restrict__ y2, T* __restrict__ uy2,
                                       T* __restrict__ g2, uint32_t* __restrict__ ext_new) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int64_t o = order[s];
  ext_new[s] = ext_old ? ext_old[o] : (uint32_t)o;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    y2[s * D + a] = y[o * D + a];
    uy2[s * D + a] = uy[o * D + a];
    g2[s * D + a] = gains[o * D + a];
  }
}

// Connected components by minimum-label propagation (component_order). A
// warp per row takes the smallest label among the row and its columns; a
// label only ever decreases, so the fixed point (each component labelled by
// its smallest index) does not depend on the order in which rows update.
__global__ void cc_init_kernel(uint32_t* __restrict__ label, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) label[i] = (uint32_t)i;
}

__global__ void cc_step_kernel(const uint64_t* __restrict__ rows, const uint32_t* __restrict__ cols, int64_t n,
                               uint32_t* label, int* __restrict__ changed) {
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;  // uniform per warp
  const uint32_t own = label[i];
  uint32_t m = own;
  for (uint64_t e = rows[i] + lane; e < rows[i + 1]; e += 32) {
    const uint32_t l = label[cols[e]];
    m = l < m ? l : m;
  }
  m = __reduce_min_sync(kFull, m);
  if (lane == 0 && m < own) {
    atomicMin(&label[i], m);
    *changed = 1;
  }
}

// label[i] = label[label[i]] (pointer jumping: labels fall toward the root
// of their chain in fewer propagation rounds)
__global__ void cc_jump_kernel(uint32_t* label, int64_t n, int* __restrict__ changed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t l = label[i];
  const uint32_t ll = label[l];
  if (ll < l) {
    atomicMin(&label[i], ll);
    *changed = 1;
  }
}

__global__ void cc_count_kernel(const uint32_t* __restrict__ label, int64_t n, uint32_t* __restrict__ count,
                                uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  atomicAdd(&count[label[i]], 1u);
  keys[i] = label[i];
  vals[i] = (uint32_t)i;
}

__global__ void cc_max_kernel(const uint32_t* __restrict__ count, int64_t n, unsigned* __restrict__ out) {
  unsigned m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = count[i] > m ? count[i] : m;
  m = __reduce_max_sync(kFull, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void compose_kernel(const uint32_t* __restrict__ order, const uint32_t* __restrict__ inv, int64_t n,
                               uint32_t* __restrict__ out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) out[s] = inv[order[s]];
}

__global__ void invert_kernel(const uint32_t* __restrict__ ext, int64_t n, uint32_t* __restrict__ inv) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) inv[ext[s]] = (uint32_t)s;
}

__global__ void slot_len_kernel(const uint64_t* __restrict__ rows, const uint32_t* __restrict__ row_of_slot, int64_t n,
                                uint32_t* __restrict__ len) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int64_t r = row_of_slot[s];
  len[s] = (uint32_t)(rows[r + 1] - rows[r]);
}

// One warp per slot: the CSR row of row_of_slot[s] moved to slot order with
// its columns mapped to slots and sorted by slot, so that a warp's neighbour
// gathers fall on few cache lines. Columns within a row are distinct, so the
// order is unique whatever the sorting network. Rows of at most kSlotRegMax
// entries sort in registers (slot_rows_short_kernel), which lists the longer
// ones (hub points of the kNN graph); those sort in shared memory up to
// kSlotSortMax entries (slot_rows_long_kernel), and rows longer still keep
// their order (only locality is lost: sorting them as well saved 2 % of the
// attractive pass and cost more than that in the re-layout).
constexpr int kSlotRegMax = 256;
constexpr int kSlotSortMax = 1024;
constexpr int kSlotWarps = 4;

// Bitonic sort of one row of L <= 32 E entries held E per lane: element e of
// the padded row is register e % E of lane e / E. Strides below E compare
// registers within a lane; larger strides pair lane l with lane l ^ (stride /
// E) by shuffles (the partner's value from before the step).
template <class T, int E>
__device__ __forceinline__ void slot_row_sort_regs(const uint32_t* __restrict__ crow, const T* __restrict__ vrow, int L,
                                                   const uint32_t* __restrict__ inv, uint32_t* __restrict__ cout,
                                                   T* __restrict__ vout, int lane) {
  uint32_t k[E];
  T v[E];
#pragma unroll
  for (int r = 0; r < E; ++r) {
    const int e = lane * E + r;
    k[r] = e < L ? inv[crow[e]] : 0xffffffffu;  // padding sorts last
    v[r] = e < L ? vrow[e] : T(0);
  }
#pragma unroll
  for (int size = 2; size <= 32 * E; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride < E) {
#pragma unroll
        for (int r = 0; r < E; ++r) {
          if (r & stride) continue;
          const bool up = ((lane * E + r) & size) == 0;
          const uint32_t a = k[r], b = k[r | stride];
          if ((a > b) == up) {
            k[r] = b;
            k[r | stride] = a;
            const T t = v[r];
            v[r] = v[r | stride];
            v[r | stride] = t;
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < E; ++r) {
          const int e = lane * E + r;
          const uint32_t pk = __shfl_xor_sync(kFull, k[r], stride / E);
          const T pv = __shfl_xor_sync(kFull, v[r], stride / E);
          // the lower element of an ascending pair (or the upper of a
          // descending one) keeps the minimum
          const bool take_min = ((e & stride) == 0) == ((e & size) == 0);
          if (take_min ? pk < k[r] : pk > k[r]) {
            k[r] = pk;
            v[r] = pv;
          }
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < E; ++r) {
    const int e = lane * E + r;
    if (e < L) {
      cout[e] = k[r];
      vout[e] = v[r];
    }
  }
}

template <class T>
__global__ void __launch_bounds__(256, 4) slot_rows_short_kernel(
    const uint64_t* __restrict__ rows, const uint32_t* __restrict__ cols, const T* __restrict__ vals,
    const uint32_t* __restrict__ row_of_slot, const uint32_t* __restrict__ inv, int64_t n,
    const uint64_t* __restrict__ rows_s, uint32_t* __restrict__ cols_s, T* __restrict__ vals_s,
    uint32_t* __restrict__ long_rows) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t slot = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; slot < n; slot += nwarps) {
    const int64_t r = row_of_slot[slot];
    const int64_t e0 = (int64_t)rows[r];
    const int L = (int)(rows[r + 1] - rows[r] > (uint64_t)kSlotRegMax ? kSlotRegMax + 1 : rows[r + 1] - rows[r]);
    if (L > kSlotRegMax) {  // listed for slot_rows_long_kernel
      if (lane == 0) long_rows[1 + atomicAdd(long_rows, 1u)] = (uint32_t)slot;
      continue;
    }
    const int64_t o = (int64_t)rows_s[slot];
    if (L <= 1) {
      if (L == 1 && lane == 0) {
        cols_s[o] = inv[cols[e0]];
        vals_s[o] = vals[e0];
      }
    } else if (L <= 32) {
      slot_row_sort_regs<T, 1>(cols + e0, vals + e0, L, inv, cols_s + o, vals_s + o, lane);
    } else if (L <= 64) {
      slot_row_sort_regs<T, 2>(cols + e0, vals + e0, L, inv, cols_s + o, vals_s + o, lane);
    } else if (L <= 128) {
      slot_row_sort_regs<T, 4>(cols + e0, vals + e0, L, inv, cols_s + o, vals_s + o, lane);
    } else {
      slot_row_sort_regs<T, 8>(cols + e0, vals + e0, L, inv, cols_s + o, vals_s + o, lane);
    }
  }
}

// The listed rows, one warp each: a bitonic sort over the next power of two
// >= L in the warp's shared-memory slice.
template <class T>
__global__ void __launch_bounds__(kSlotWarps * 32) slot_rows_long_kernel(
    const uint64_t* __restrict__ rows, const uint32_t* __restrict__ cols, const T* __restrict__ vals,
    const uint32_t* __restrict__ row_of_slot, const uint32_t* __restrict__ inv, const uint32_t* __restrict__ long_rows,
    const uint64_t* __restrict__ rows_s, uint32_t* __restrict__ cols_s, T* __restrict__ vals_s) {
  __shared__ uint32_t sk[kSlotWarps][kSlotSortMax];
  __shared__ T sv[kSlotWarps][kSlotSortMax];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t count = long_rows[0];
  const uint32_t nwarps = gridDim.x * kSlotWarps;
  for (uint32_t q = blockIdx.x * kSlotWarps + w; q < count; q += nwarps) {
    const int64_t slot = long_rows[1 + q];
    const int64_t r = row_of_slot[slot];
    const int64_t e0 = (int64_t)rows[r];
    const int64_t L = (int64_t)(rows[r + 1] - rows[r]);
    const int64_t o = (int64_t)rows_s[slot];
    if (L > kSlotSortMax) {
      for (int64_t t = lane; t < L; t += 32) {
        cols_s[o + t] = inv[cols[e0 + t]];
        vals_s[o + t] = vals[e0 + t];
      }
      continue;
    }
    int P = 32;
    while (P < L) P <<= 1;
    for (int t = lane; t < P; t += 32) {
      sk[w][t] = t < L ? inv[cols[e0 + t]] : 0xffffffffu;  // padding sorts last
      sv[w][t] = t < L ? vals[e0 + t] : T(0);
    }
    __syncwarp();
    for (int size = 2; size <= P; size <<= 1) {
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int t = lane; t < P / 2; t += 32) {
          const int lo = 2 * t - (t & (stride - 1));
          const int hi = lo + stride;
          const bool up = (lo & size) == 0;
          const uint32_t a = sk[w][lo], b = sk[w][hi];
          if ((a > b) == up) {
            sk[w][lo] = b;
            sk[w][hi] = a;
            const T va = sv[w][lo];
            sv[w][lo] = sv[w][hi];
            sv[w][hi] = va;
          }
        }
        __syncwarp();
      }
    }
    for (int t = lane; t < L; t += 32) {
      cols_s[o + t] = sk[w][t];
      vals_s[o + t] = sv[w][t];
    }
    __syncwarp();
  }
}

template <class T, int D>
__global__ void unpermute_kernel(const T* __restrict__ y, const uint32_t* __restrict__ ext, int64_t n,
                                 T* __restrict__ out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int64_t r = ext[s];
#pragma unroll
  for (int a = 0; a < D; ++a) out[r * D + a] = y[s * D + a];
}

// Fused update over points; neg may be null (exact method: pos holds dy).
// Accumulates sum(y_new) per axis in FP64 into mean_sum (deterministic: the
// last block reduces the per-block partials in block order).
template <class T, int D>
__global__ void __launch_bounds__(256) update_kernel(T* __restrict__ y, const T* __restrict__ pos, const T* __restrict__ neg,
                                                     T* __restrict__ uy, T* __restrict__ gains, int64_t n,
                                                     const double* __restrict__ z, T inv_norm_arg, T lr, T momentum,
                                                     double* __restrict__ part, unsigned* __restrict__ done,
                                                     double* __restrict__ mean_sum) {
  __shared__ double sh[D][32];
  __shared__ bool last;
  const T inc = (T)0.2, dec = (T)0.8, floor_ = (T)0.01;
  const T inv_norm = neg ? (z ? T(1) / (T)(*z) : inv_norm_arg) : T(0);
  double s[D];
#pragma unroll
  for (int a = 0; a < D; ++a) s[a] = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const int64_t e = i * D + a;
      const T g = neg ? pos[e] - neg[e] * inv_norm : pos[e];
      const T u = uy[e];
      T gn = (signum(g) != signum(u)) ? gains[e] + inc : gains[e] * dec;
      if (gn < floor_) gn = floor_;
      gains[e] = gn;
      const T un = momentum * u - lr * gn * g;
      uy[e] = un;
      const T yn = y[e] + un;
      y[e] = yn;
      s[a] += (double)yn;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double v = warp_sum(s[a]);
    if (lane == 0) sh[a][w] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double t = 0.0;
      for (int q = 0; q < nw; ++q) t += sh[a][q];
      part[blockIdx.x * D + a] = t;
    }
    __threadfence();
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    __shared__ double shr[32];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const double t = block_sum_parts(part, gridDim.x, D, a, shr);
      if (threadIdx.x == 0) mean_sum[a] = t;
    }
    if (threadIdx.x == 0) *done = 0;
  }
}

template <class T, int D>
__global__ void kl_sparse_kernel(const uint64_t* __restrict__ rows, const uint32_t* __restrict__ cols,
                                 const T* __restrict__ vals, const T* __restrict__ y, int64_t n,
                                 const double* __restrict__ z, int quirk, double* __restrict__ part) {
  __shared__ double sh[32];
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  const T inv_q_sum = T(1) / (T)(*z);
  double acc = 0.0;
  for (int64_t row = gw; row < n; row += nw) {
    T cost = T(0);
    const int64_t e0 = (int64_t)rows[row], e1 = (int64_t)rows[row + 1];
    for (int64_t e = e0 + lane; e < e1; e += 32) {
      const int64_t j = cols[e];
      T q = T(0);
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const T d = y[row * D + a] - y[j * D + a];
        q = q + d * d;
      }
      q = (T(1) / (T(1) + q)) * inv_q_sum;
      const T p = quirk ? vals[row] : vals[e];
      cost += p * dlog((p + Lim<T>::min_pos()) / (q + Lim<T>::min_pos()));
    }
    acc += (double)cost;
  }
  const double bs = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = bs;
}

__global__ void reduce_parts_kernel(const double* __restrict__ part, int nparts, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += part[b];
    *out = s;
  }
}

// ---------------------------------------------------------------------------
// Exact (dense) method.
// ---------------------------------------------------------------------------
template <class T>
__global__ void dense_distance_kernel(const T* __restrict__ X, int64_t n, int dim, int squared, T* __restrict__ dist) {
  const int64_t i = blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || j >= n) return;
  if (j == i) {
    dist[i * n + j] = T(0);
    return;
  }
  // Evaluate on the upper triangle only and mirror (src/tsne/mod.rs:161-189).
  const int64_t a = j > i ? i : j, b = j > i ? j : i;
  T s = T(0);
  for (int c = 0; c < dim; ++c) {
    const T d = X[a * dim + c] - X[b * dim + c];
    s = s + d * d;
  }
  dist[i * n + j] = squared ? s : dsqrt(s);
}

template <class T>
__global__ void dense_symmetrize_kernel(T* __restrict__ p, int64_t n) {
  const int64_t i = blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || j >= n || j <= i) return;
  const T v = p[i * n + j] + p[j * n + i];
  p[i * n + j] = v;
  p[j * n + i] = v;
}

// Z = sum over all (i, j) including the diagonal of 1 / (1 + |y_i - y_j|^2).
template <class T, int D>
__global__ void exact_z_kernel(const T* __restrict__ y, int64_t n, double* __restrict__ part) {
  __shared__ double sh[32];
  const int64_t i = blockIdx.x;
  T yi[D];
#pragma unroll
  for (int a = 0; a < D; ++a) yi[a] = y[i * D + a];
  double acc = 0.0;
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    T d = T(0);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const T t = yi[a] - y[j * D + a];
      d = d + t * t;
    }
    acc += (double)(T(1) / (T(1) + d));
  }
  const double bs = block_sum(acc, sh);
  if (threadIdx.x == 0) part[i] = bs;
}

template <class T, int D>
__global__ void exact_grad_kernel(const T* __restrict__ y, const T* __restrict__ p, int64_t n,
                                  const double* __restrict__ z, T* __restrict__ dy) {
  __shared__ double sh[32];
  const int64_t i = blockIdx.x;
  const T inv = T(1) / (T)(*z);
  T yi[D], acc[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    yi[a] = y[i * D + a];
    acc[a] = T(0);
  }
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    T d = T(0);
    T diff[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      diff[a] = yi[a] - y[j * D + a];
      d = d + diff[a] * diff[a];
    }
    const T q = T(1) / (T(1) + d);
    const T m = (p[i * n + j] - q * inv) * q;
#pragma unroll
    for (int a = 0; a < D; ++a) acc[a] += diff[a] * m;
  }
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double bs = block_sum((double)acc[a], sh);
    if (threadIdx.x == 0) dy[i * D + a] = (T)bs;
    __syncthreads();
  }
}

template <class T, int D>
__global__ void exact_kl_kernel(const T* __restrict__ y, const T* __restrict__ p, int64_t n,
                                const double* __restrict__ z, double* __restrict__ part) {
  __shared__ double sh[32];
  const int64_t i = blockIdx.x;
  const T inv = T(1) / (T)(*z);
  T yi[D];
#pragma unroll
  for (int a = 0; a < D; ++a) yi[a] = y[i * D + a];
  double acc = 0.0;
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    T d = T(0);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const T t = yi[a] - y[j * D + a];
      d = d + t * t;
    }
    const T q = T(1) / (T(1) + d) * inv;
    const T pv = p[i * n + j];
    acc += (double)(pv * dlog((pv + Lim<T>::min_pos()) / (q + Lim<T>::min_pos())));
  }
  const double bs = block_sum(acc, sh);
  if (threadIdx.x == 0) part[i] = bs;
}

constexpr int kUpdBlocksMax = 1024;  // partials of the update's mean (two blocks per SM)

}  // namespace

template <class T>
void launch_random_init(T* y, int64_t count, uint64_t seed, cudaStream_t s) {
  if (count <= 0) return;
  random_init_kernel<T><<<(unsigned)ceil_div(ceil_div(count, 2), 256), 256, 0, s>>>(y, count, seed);
  BHG_LAUNCH_CHECK();
}

template <class T>
void build_attr_tasks(AttrTasks& at, int D, const uint64_t* rows, int64_t n, cudaStream_t s, int task_len) {
  if (task_len != 64 && task_len != 128 && task_len != 256) task_len = kAttrTaskLen;
  at.D = D;
  at.n = n;
  at.task_len = task_len;
  at.ntasks = at.nlong = 0;
  if (n <= 0) return;
  const unsigned g = (unsigned)ceil_div(n, 256);
  uint32_t* cnt = static_cast<uint32_t*>(at.cnt.ensure((size_t)n * 4));
  uint64_t* off = static_cast<uint64_t*>(at.off.ensure((size_t)(n + 1) * 8));
  task_count_kernel<<<g, 256, 0, s>>>(rows, n, task_len, cnt);
  BHG_LAUNCH_CHECK();
  scan_u32_to_u64(cnt, off, n, at.scan_tmp, s);
  uint64_t total = 0;
  BHG_CUDA(cudaMemcpyAsync(&total, off + n, 8, cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  at.ntasks = (int64_t)total;
  AttrTask* tasks = static_cast<AttrTask*>(at.tasks.ensure((size_t)at.ntasks * sizeof(AttrTask)));
  uint32_t* longs = static_cast<uint32_t*>(at.longs.ensure((size_t)n * 4));
  unsigned long long* nl = static_cast<unsigned long long*>(at.nlong_dev.ensure(8));
  BHG_CUDA(cudaMemsetAsync(nl, 0, 8, s));
  task_fill_kernel<<<g, 256, 0, s>>>(rows, n, task_len, off, tasks, longs, nl);
  BHG_LAUNCH_CHECK();
  unsigned long long nlong = 0;
  BHG_CUDA(cudaMemcpyAsync(&nlong, nl, 8, cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  at.nlong = (int64_t)nlong;
  at.part.ensure((size_t)at.ntasks * D * sizeof(T));
}

template <class T, int D>
static void launch_attractive_tasks_d(const AttrTasks& at, const uint32_t* cols, const T* vals, const T* y, T* pos,
                                      cudaStream_t s) {
  const bool vec = D == 2 && (reinterpret_cast<uintptr_t>(y) % (2 * sizeof(T))) == 0;
  const unsigned grid = (unsigned)ceil_div(at.ntasks, 8);
  const AttrTask* tasks = static_cast<const AttrTask*>(at.tasks.ptr);
  T* part = static_cast<T*>(at.part.ptr);
  auto go = [&](auto ku) {
    constexpr int KU = decltype(ku)::value;
    if (vec) attractive_task_kernel<T, D, true, KU><<<grid, 256, 0, s>>>(tasks, at.ntasks, cols, vals, y, pos, part);
    else attractive_task_kernel<T, D, false, KU><<<grid, 256, 0, s>>>(tasks, at.ntasks, cols, vals, y, pos, part);
  };
  if (at.task_len == 64) go(std::integral_constant<int, 2>());
  else if (at.task_len == 256) go(std::integral_constant<int, 8>());
  else go(std::integral_constant<int, 4>());
  BHG_LAUNCH_CHECK();
  if (at.nlong > 0) {
    attractive_fixup_kernel<T, D><<<(unsigned)ceil_div(at.nlong, 256), 256, 0, s>>>(
        static_cast<const uint32_t*>(at.longs.ptr), at.nlong, static_cast<const uint64_t*>(at.off.ptr), part, pos);
    BHG_LAUNCH_CHECK();
  }
}

template <class T>
void launch_attractive_tasks(const AttrTasks& at, const uint32_t* cols, const T* vals, const T* y, T* pos,
                             cudaStream_t s) {
  if (at.ntasks <= 0) return;
  with_dim<1, 7>(at.D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    launch_attractive_tasks_d<T, DD>(at, cols, vals, y, pos, s);
  });
}

template <class T>
void launch_renumber(int D, const uint32_t* order, int64_t n, Renumbering& r, T* y, T* uy, T* gains, T* tmp_a, T* tmp_b,
                     T* tmp_c, const uint64_t* rows, const uint32_t* cols, const T* vals, int64_t nnz, cudaStream_t s) {
  const unsigned g = (unsigned)ceil_div(n, 256);
  uint32_t* ext_new = static_cast<uint32_t*>(r.ext_alt.ensure((size_t)n * 4));
  const uint32_t* ext_old = r.active ? r.ext.template as<uint32_t>() : nullptr;
  with_dim<1, 7>(D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    renumber_gather_kernel<T, DD><<<g, 256, 0, s>>>(order, ext_old, n, y, uy, gains, tmp_a, tmp_b, tmp_c, ext_new);
  });
  BHG_LAUNCH_CHECK();
  const size_t bytes = (size_t)n * D * sizeof(T);
  BHG_CUDA(cudaMemcpyAsync(y, tmp_a, bytes, cudaMemcpyDeviceToDevice, s));
  BHG_CUDA(cudaMemcpyAsync(uy, tmp_b, bytes, cudaMemcpyDeviceToDevice, s));
  BHG_CUDA(cudaMemcpyAsync(gains, tmp_c, bytes, cudaMemcpyDeviceToDevice, s));
  r.ext.ensure((size_t)n * 4);
  BHG_CUDA(cudaMemcpyAsync(r.ext.ptr, ext_new, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
  uint32_t* inv = static_cast<uint32_t*>(r.inv.ensure((size_t)n * 4));
  invert_kernel<<<g, 256, 0, s>>>(r.ext.template as<uint32_t>(), n, inv);
  BHG_LAUNCH_CHECK();
  // CSR in slot order with slot columns, sorted within each row
  uint32_t* len = static_cast<uint32_t*>(r.len.ensure((size_t)n * 4));
  slot_len_kernel<<<g, 256, 0, s>>>(rows, r.ext.template as<uint32_t>(), n, len);
  BHG_LAUNCH_CHECK();
  uint64_t* rows_s = static_cast<uint64_t*>(r.rows.ensure((size_t)(n + 1) * 8));
  scan_u32_to_u64(len, rows_s, n, r.scan_tmp, s);
  uint32_t* cols_s = static_cast<uint32_t*>(r.cols.ensure((size_t)std::max<int64_t>(nnz, 1) * 4));
  T* vals_s = static_cast<T*>(r.vals.ensure((size_t)std::max<int64_t>(nnz, 1) * sizeof(T)));
  if (nnz > 0) {
    uint32_t* long_rows = static_cast<uint32_t*>(r.long_rows.ensure((size_t)(n + 1) * 4));
    BHG_CUDA(cudaMemsetAsync(long_rows, 0, 4, s));
    slot_rows_short_kernel<T><<<(unsigned)std::min<int64_t>(ceil_div(n, 8), sm_grid(4, 4096)), 256, 0, s>>>(
        rows, cols, vals, r.ext.template as<uint32_t>(), inv, n, rows_s, cols_s, vals_s, long_rows);
    BHG_LAUNCH_CHECK();
    slot_rows_long_kernel<T><<<(unsigned)std::min<int64_t>(ceil_div(n, kSlotWarps), sm_grid(8, 8192)), kSlotWarps * 32, 0, s>>>(
        rows, cols, vals, r.ext.template as<uint32_t>(), inv, long_rows, rows_s, cols_s, vals_s);
    BHG_LAUNCH_CHECK();
  }
  r.active = true;
}

void launch_compose_order(const uint32_t* order, const uint32_t* inv, int64_t n, uint32_t* out, cudaStream_t s) {
  compose_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(order, inv, n, out);
  BHG_LAUNCH_CHECK();
}

bool component_order(const uint64_t* rows, const uint32_t* cols, int64_t n, DevBuf& order, ComponentScratch& cs,
                     int64_t* largest, cudaStream_t s) {
  *largest = 0;
  if (n < 2) return false;
  const unsigned g = (unsigned)ceil_div(n, 256);
  uint32_t* label = static_cast<uint32_t*>(cs.label.ensure((size_t)n * 4));
  int* flag = static_cast<int*>(cs.flag.ensure(64));
  cc_init_kernel<<<g, 256, 0, s>>>(label, n);
  BHG_LAUNCH_CHECK();
  // Each round at least halves the distance of every label chain to its root
  // or settles; a kNN graph's components have small diameters. Rounds are
  // bounded, and a graph that has not settled is left in its current layout.
  bool settled = false;
  for (int round = 0; round < 64 && !settled; ++round) {
    BHG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), s));
    cc_step_kernel<<<(unsigned)ceil_div(n * 32, 256), 256, 0, s>>>(rows, cols, n, label, flag);
    BHG_LAUNCH_CHECK();
    cc_jump_kernel<<<g, 256, 0, s>>>(label, n, flag);
    BHG_LAUNCH_CHECK();
    int h = 0;
    BHG_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    BHG_CUDA(cudaStreamSynchronize(s));
    settled = h == 0;
  }
  if (!settled) return false;
  uint32_t* count = static_cast<uint32_t*>(cs.count.ensure((size_t)n * 4));
  uint64_t* keys = static_cast<uint64_t*>(cs.keys.ensure((size_t)n * 8));
  uint32_t* vals = static_cast<uint32_t*>(order.ensure((size_t)n * 4));
  BHG_CUDA(cudaMemsetAsync(count, 0, (size_t)n * 4, s));
  cc_count_kernel<<<g, 256, 0, s>>>(label, n, count, keys, vals);
  BHG_LAUNCH_CHECK();
  unsigned* mx = reinterpret_cast<unsigned*>(flag) + 1;
  BHG_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned), s));
  cc_max_kernel<<<(unsigned)std::min<int64_t>(g, sm_grid(4, 4096)), 256, 0, s>>>(count, n, mx);
  BHG_LAUNCH_CHECK();
  unsigned hmax = 0;
  BHG_CUDA(cudaMemcpyAsync(&hmax, mx, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  *largest = hmax;
  if ((int64_t)hmax > n / 4) return false;
  int bits = 1;
  while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)n) ++bits;
  radix_sort_pairs<uint32_t>(keys, vals, static_cast<uint64_t*>(cs.keys_alt.ensure((size_t)n * 8)),
                             static_cast<uint32_t*>(cs.vals_alt.ensure((size_t)n * 4)), n, 0, bits, cs.sort_tmp, s);
  return true;
}

template <class T>
void launch_unpermute(int D, const T* y, const uint32_t* ext, int64_t n, T* out, cudaStream_t s) {
  const unsigned g = (unsigned)ceil_div(n, 256);
  with_dim<1, 7>(D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    unpermute_kernel<T, DD><<<g, 256, 0, s>>>(y, ext, n, out);
  });
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_update(int D, T* y, const T* pos, const T* neg, T* uy, T* gains, int64_t n, const double* z, T inv_norm,
                   T lr, T momentum, UpdateScratch& us, cudaStream_t s) {
  double* part = static_cast<double*>(us.part.ensure(kUpdBlocksMax * 8 * sizeof(double)));
  unsigned* done = static_cast<unsigned*>(us.done.ensure(64));
  if (!us.zeroed) {
    BHG_CUDA(cudaMemsetAsync(done, 0, 64, s));
    us.zeroed = true;
  }
  double* mean_sum = static_cast<double*>(us.mean_sum.ensure(8 * sizeof(double)));
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), sm_grid(2, kUpdBlocksMax)));
  with_dim<1, 7>(D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    update_kernel<T, DD><<<grid, 256, 0, s>>>(y, pos, neg, uy, gains, n, z, inv_norm, lr, momentum, part, done, mean_sum);
  });
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_kl_sparse(int D, const uint64_t* rows, const uint32_t* cols, const T* vals, const T* y, int64_t n,
                      const double* z, bool quirk, double* out, DevBuf& tmp, cudaStream_t s) {
  const int blocks = sm_grid(2, 1024);
  double* part = static_cast<double*>(tmp.ensure(blocks * sizeof(double)));
  with_dim<1, 7>(D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    kl_sparse_kernel<T, DD><<<blocks, 256, 0, s>>>(rows, cols, vals, y, n, z, quirk ? 1 : 0, part);
  });
  BHG_LAUNCH_CHECK();
  reduce_parts_kernel<<<1, 32, 0, s>>>(part, blocks, out);
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_dense_distance(const T* X, int64_t n, int dim, bool squared, T* dist, cudaStream_t s) {
  dim3 g((unsigned)ceil_div(n, 256), (unsigned)n);
  dense_distance_kernel<T><<<g, 256, 0, s>>>(X, n, dim, squared ? 1 : 0, dist);
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_dense_symmetrize(T* p, int64_t n, cudaStream_t s) {
  dim3 g((unsigned)ceil_div(n, 256), (unsigned)n);
  dense_symmetrize_kernel<T><<<g, 256, 0, s>>>(p, n);
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_exact_z(int D, const T* y, int64_t n, double* z, DevBuf& tmp, cudaStream_t s) {
  double* part = static_cast<double*>(tmp.ensure(n * sizeof(double)));
  with_dim<1, 7>(D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    exact_z_kernel<T, DD><<<(unsigned)n, 256, 0, s>>>(y, n, part);
  });
  BHG_LAUNCH_CHECK();
  reduce_parts_kernel<<<1, 32, 0, s>>>(part, (int)n, z);
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_exact_grad(int D, const T* y, const T* p, int64_t n, const double* z, T* dy, cudaStream_t s) {
  with_dim<1, 7>(D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    exact_grad_kernel<T, DD><<<(unsigned)n, 256, 0, s>>>(y, p, n, z, dy);
  });
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_exact_kl(int D, const T* y, const T* p, int64_t n, const double* z, double* out, DevBuf& tmp,
                     cudaStream_t s) {
  double* part = static_cast<double*>(tmp.ensure(n * sizeof(double)));
  with_dim<1, 7>(D, "error: the embedding dimension must be in 1..7.", [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    exact_kl_kernel<T, DD><<<(unsigned)n, 256, 0, s>>>(y, p, n, z, part);
  });
  BHG_LAUNCH_CHECK();
  reduce_parts_kernel<<<1, 32, 0, s>>>(part, (int)n, out);
  BHG_LAUNCH_CHECK();
}

#define BHG_INST(T)                                                                                                  \
  template void launch_renumber<T>(int, const uint32_t*, int64_t, Renumbering&, T*, T*, T*, T*, T*, T*,              \
                                   const uint64_t*, const uint32_t*, const T*, int64_t, cudaStream_t);               \
  template void launch_unpermute<T>(int, const T*, const uint32_t*, int64_t, T*, cudaStream_t);                      \
  template void build_attr_tasks<T>(AttrTasks&, int, const uint64_t*, int64_t, cudaStream_t, int);                   \
  template void launch_random_init<T>(T*, int64_t, uint64_t, cudaStream_t);                                          \
  template void launch_attractive_tasks<T>(const AttrTasks&, const uint32_t*, const T*, const T*, T*, cudaStream_t); \
  template void launch_update<T>(int, T*, const T*, const T*, T*, T*, int64_t, const double*, T, T, T, UpdateScratch&,  \
                                 cudaStream_t);                                                                      \
  template void launch_kl_sparse<T>(int, const uint64_t*, const uint32_t*, const T*, const T*, int64_t,             \
                                    const double*, bool, double*, DevBuf&, cudaStream_t);                            \
  template void launch_dense_distance<T>(const T*, int64_t, int, bool, T*, cudaStream_t);                            \
  template void launch_dense_symmetrize<T>(T*, int64_t, cudaStream_t);                                               \
  template void launch_exact_z<T>(int, const T*, int64_t, double*, DevBuf&, cudaStream_t);                           \
  template void launch_exact_grad<T>(int, const T*, const T*, int64_t, const double*, T*, cudaStream_t);             \
  template void launch_exact_kl<T>(int, const T*, const T*, int64_t, const double*, double*, DevBuf&, cudaStream_t);
BHG_INST(float)
BHG_INST(double)

}  // namespace bhg
