// Affinity construction on the GPU: the perplexity bisection per row, the
// symmetric CSR build, and the normalisation / exaggeration scalings.
//
// Reference behaviour restated (bhtsne 0.7.10):
//  * search_beta: src/tsne/mod.rs:201-275. p = exp(-beta * d^2) with d the
//    metric distance; sum += min_positive; H = sum(beta p d^2)/sum + ln sum;
//    stop when |H - ln(perplexity)| < 1e-5 or after 200 iterations; beta
//    doubles/halves until bracketed, then bisects; finally p /= sum + eps.
//    Sums are sequential in T as in the reference (see search_beta_kernel).
//  * symmetrize_sparse_matrix: src/tsne/mod.rs:306-406. The reference emits,
//    for every directed kNN edge i->j, the entries (i, j) and (j, i) with value
//    p_ij + p_ji when i and j list each other (once, from the side i < j) and
//    p_ij otherwise, then halves every value. Its sequential fill orders each
//    row r as: columns n < r with r in N(n) (ascending), then r's own sorted
//    neighbours minus the mutual ones below r, then columns n > r listing r
//    that r does not list (ascending). Sorting the emitted entries by
//    (row, group, column), group in {0, 1, 2} for those three runs,
//    reproduces that order exactly, so the CSR arrays (and the KL quirk that
//    indexes the value array by row number) match the reference entry for
//    entry.
//  * normalize_p_values: src/tsne/mod.rs:284-293; stop_lying: :525-531.
#include "affinity.h"

#include <cmath>
#include <mutex>

namespace bhg {

namespace {

// 2^(i / 256), i < 256, in double: the table of exp_table_f32 (filled once per
// device by launch_search_beta).
constexpr int kExpTab = 256;
__device__ double g_exp2_tab[kExpTab];

// ---------------------------------------------------------------------------
// search_beta: one warp per row. The lanes evaluate the kernel values of the
// row in parallel and park them in the output row; lane 0 then forms both
// sums sequentially in index order, in T, exactly as the reference folds
// them. exp and ln are evaluated in FP64 and rounded to T, which reproduces
// the correctly rounded single-precision libm results the reference gets on
// the host; the bisection's 1e-5 stopping test is sensitive to last-ulp
// differences, so this is what keeps P within 1e-5 of the reference.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T exp_rn(T x) {
  return (T)exp((double)x);
}

// exp(x) of a single-precision x <= 0, computed in FP64 with few FP64
// operations by Tang's table-driven method: x = (256 m + i) ln2 / 256 + r
// with |r| <= ln2 / 512 (i and m from a single-precision product, whose
// rounding moves that bound by under 0.5 %), exp(x) = 2^m 2^(i/256) exp(r),
// and exp(r) - 1 by its Taylor series to r^4 (the next term is below 2^-54
// relative). The FP64 value is within a few units in its last place of
// exp(x), so its rounding to single precision is the correctly rounded result
// but when exp(x) lies that close to a rounding boundary, as with exp((double)x)
// itself. Below -110 the result rounds to zero.
__device__ __forceinline__ float exp_table_f32(float x) {
  if (!(x >= -110.f)) return x != x ? x : 0.f;
  const float tf = x * 369.32993046757463f;  // 256 / ln 2
  const int nn = __float2int_rn(tf);
  const int i = nn & (kExpTab - 1), m = nn >> 8;
  // r = x - nn ln2 / 256, ln2 / 256 as a double pair (Cody and Waite)
  const double ln2_256_hi = 0.0027076061740622863, ln2_256_lo = 9.058776616587108e-20;
  double r = fma(-(double)nn, ln2_256_hi, (double)x);
  r = fma(-(double)nn, ln2_256_lo, r);
  double q = fma(r, 1.0 / 24.0, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  q = fma(q, r, 1.0);
  const double pr = q * r;  // exp(r) - 1
  const double ti = __ldg(g_exp2_tab + i);
  const double y = fma(ti, pr, ti);
  return (float)(y * __hiloint2double((m + 1023) << 20, 0));
}
template <class T>
__device__ __forceinline__ T exp_beta(T x) {
  return exp_rn<T>(x);
}
template <>
__device__ __forceinline__ float exp_beta<float>(float x) {
  return exp_table_f32(x);
}
template <class T>
__device__ __forceinline__ T log_rn(T x) {
  return (T)log((double)x);
}

template <class T>
__global__ void search_beta_kernel(const T* __restrict__ dist, int64_t n, int64_t k, T perplexity,
                                   T* __restrict__ p, int32_t* __restrict__ iters) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const T* d = dist + row * k;
  T* out = p + row * k;
  bool found = false;
  T beta = T(1), min_beta = -Lim<T>::max(), max_beta = Lim<T>::max();
  const T tolerance = (T)1e-5;
  const T two = T(2);
  const T ln_perp = log_rn(perplexity);
  T sum = T(0);
  int iteration = 0;
  while (!found && iteration < 200) {
    for (int64_t j = lane; j < k; j += 32) {
      const T dj = d[j];
      out[j] = exp_beta<T>(-beta * (dj * dj));
    }
    __syncwarp();
    T s = T(0), e = T(0);
    if (lane == 0) {
      for (int64_t j = 0; j < k; ++j) s = s + out[j];
      for (int64_t j = 0; j < k; ++j) {
        const T dj = d[j];
        e = e + beta * out[j] * (dj * dj);
      }
    }
    s = __shfl_sync(kFull, s, 0);
    e = __shfl_sync(kFull, e, 0);
    sum = s + Lim<T>::min_pos();
    T entropy = e / sum + log_rn(sum);
    const T diff = entropy - ln_perp;
    if (diff < tolerance && -diff < tolerance) {
      found = true;
    } else {
      if (diff > T(0)) {
        min_beta = beta;
        if (max_beta == Lim<T>::max() || max_beta == -Lim<T>::max()) beta *= two;
        else beta = (beta + max_beta) / two;
      } else {
        max_beta = beta;
        if (min_beta == -Lim<T>::max() || min_beta == Lim<T>::max()) beta /= two;
        else beta = (beta + min_beta) / two;
      }
      if (isinf(beta) && beta > T(0)) beta = Lim<T>::max();
      if (isinf(beta) && beta < T(0)) beta = -Lim<T>::max();
    }
    ++iteration;
    __syncwarp();
  }
  const T denom = sum + Lim<T>::eps();
  for (int64_t j = lane; j < k; j += 32) out[j] = out[j] / denom;
  if (iters && lane == 0) iters[row] = iteration;
}

// ---------------------------------------------------------------------------
// Row sort by column: one warp per row, bitonic sort in shared memory over a
// power-of-two padded copy (k <= kMaxSortK).
// ---------------------------------------------------------------------------
constexpr int kSortWarps = 4;

template <class T>
__global__ void sort_rows_kernel(uint32_t* __restrict__ cols, T* __restrict__ vals, int64_t n, int k, int P) {
  extern __shared__ unsigned char smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * kSortWarps + w;
  uint32_t* sc = reinterpret_cast<uint32_t*>(smem) + w * P;
  T* sv = reinterpret_cast<T*>(reinterpret_cast<uint32_t*>(smem) + kSortWarps * P) + w * P;
  if (row >= n) return;
  for (int j = lane; j < P; j += 32) {
    if (j < k) {
      sc[j] = cols[row * k + j];
      sv[j] = vals[row * k + j];
    } else {
      sc[j] = 0xffffffffu;
      sv[j] = T(0);
    }
  }
  __syncwarp();
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < P / 2; t += 32) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const uint32_t a = sc[lo], b = sc[hi];
        if ((a > b) == up) {
          sc[lo] = b;
          sc[hi] = a;
          const T va = sv[lo];
          sv[lo] = sv[hi];
          sv[hi] = va;
        }
      }
      __syncwarp();
    }
  }
  for (int j = lane; j < k; j += 32) {
    cols[row * k + j] = sc[j];
    vals[row * k + j] = sv[j];
  }
}

// ---------------------------------------------------------------------------
// Emission of the two directed entries of every kNN edge.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t find_in_row(const uint32_t* __restrict__ row, int k, uint32_t target) {
  int lo = 0, hi = k;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (row[mid] < target) lo = mid + 1;
    else hi = mid;
  }
  return (lo < k && row[lo] == target) ? lo : -1;
}

template <class T>
__global__ void emit_entries_kernel(const uint32_t* __restrict__ cols, const T* __restrict__ vals, int64_t n, int k,
                                    int cbits, uint64_t* __restrict__ keys, T* __restrict__ ev,
                                    unsigned long long* __restrict__ nnz) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = n * (int64_t)k;
  unsigned count = 0;
  if (e < total) {
    const uint64_t r = (uint64_t)(e / k);
    const uint32_t j = cols[e];
    const int64_t m = find_in_row(cols + (int64_t)j * k, k, (uint32_t)r);
    const bool mutual = m >= 0;
    const uint64_t sentinel = ~0ULL;
    if (mutual && r > j) {
      keys[2 * e] = sentinel;
      keys[2 * e + 1] = sentinel;
      ev[2 * e] = T(0);
      ev[2 * e + 1] = T(0);
    } else {
      const T v = mutual ? vals[e] + vals[(int64_t)j * k + m] : vals[e];
      const uint64_t g_rev = r < j ? 0 : 2;
      keys[2 * e] = (r << (cbits + 2)) | (1ULL << cbits) | (uint64_t)j;
      keys[2 * e + 1] = ((uint64_t)j << (cbits + 2)) | (g_rev << cbits) | r;
      ev[2 * e] = v;
      ev[2 * e + 1] = v;
      count = 2;
    }
  }
  // warp-aggregated count
  unsigned c = warp_sum(count);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(nnz, (unsigned long long)c);
}

template <class T>
__global__ void finish_csr_kernel(const uint64_t* __restrict__ keys, const T* __restrict__ ev, int64_t nnz, int cbits,
                                  uint32_t* __restrict__ cols_out, T* __restrict__ vals_out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  cols_out[e] = (uint32_t)(keys[e] & ((1ULL << cbits) - 1));
  vals_out[e] = ev[e] * T(0.5);
}

__global__ void row_ptr_kernel(const uint64_t* __restrict__ keys, int64_t nnz, int64_t n, int cbits,
                               uint64_t* __restrict__ rows) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r > n) return;
  if (r == n) {
    rows[n] = (uint64_t)nnz;
    return;
  }
  const uint64_t key = (uint64_t)r << (cbits + 2);
  int64_t lo = 0, hi = nnz;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  rows[r] = (uint64_t)lo;
}

// ---------------------------------------------------------------------------
// Sum of values (FP64, deterministic two-level) and scaling.
// ---------------------------------------------------------------------------
template <class T>
__global__ void sum_partial_kernel(const T* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += (double)v[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void sum_final_kernel(const double* __restrict__ part, int nparts, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += part[b];
    *out = s;
  }
}

// p *= exaggeration / (sum + eps), computed in T like the reference.
template <class T>
__global__ void normalize_kernel(T* __restrict__ v, int64_t n, const double* __restrict__ sum, T exaggeration) {
  const T scale = exaggeration / ((T)*sum + Lim<T>::eps());
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= scale;
}

template <class T>
__global__ void scale_kernel(T* __restrict__ v, int64_t n, T scale) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= scale;
}

template <class T>
__global__ void scaled_copy_kernel(const T* __restrict__ v, int64_t n, T scale, T* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = v[i] * scale;
}

int bits_for(int64_t n) {
  int b = 1;
  while ((1LL << b) < n) ++b;
  return b;
}

constexpr int kSumBlocksMax = 1024;  // partials of launch_sum (two blocks per SM)

}  // namespace

template <class T>
void launch_search_beta(const T* dist, int64_t n, int64_t k, T perplexity, T* p, int32_t* iters, cudaStream_t s) {
  if (n <= 0) return;
  {
    // the exp table of this device, once
    static std::mutex mu;
    static bool filled[256] = {};
    int dev = 0;
    BHG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 256 && !filled[dev]) {
      double tab[kExpTab];
      for (int i = 0; i < kExpTab; ++i) tab[i] = std::exp2((double)i / kExpTab);
      BHG_CUDA(cudaMemcpyToSymbol(g_exp2_tab, tab, sizeof tab));
      filled[dev] = true;
    }
  }
  const int threads = 256;
  const unsigned grid = (unsigned)ceil_div(n * 32, threads);
  search_beta_kernel<T><<<grid, threads, 0, s>>>(dist, n, k, perplexity, p, iters);
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_sum(const T* v, int64_t n, double* out, DevBuf& tmp, cudaStream_t s) {
  const int blocks = sm_grid(2, kSumBlocksMax);
  double* part = static_cast<double*>(tmp.ensure(kSumBlocksMax * sizeof(double)));
  sum_partial_kernel<T><<<blocks, 256, 0, s>>>(v, n, part);
  BHG_LAUNCH_CHECK();
  sum_final_kernel<<<1, 32, 0, s>>>(part, blocks, out);
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_normalize(T* v, int64_t n, T exaggeration, double* sum_dev, DevBuf& tmp, cudaStream_t s) {
  launch_sum<T>(v, n, sum_dev, tmp, s);
  normalize_kernel<T><<<sm_grid(2, kSumBlocksMax), 256, 0, s>>>(v, n, sum_dev, exaggeration);
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_scale(T* v, int64_t n, T scale, cudaStream_t s) {
  if (n <= 0) return;
  scale_kernel<T><<<sm_grid(2, kSumBlocksMax), 256, 0, s>>>(v, n, scale);
  BHG_LAUNCH_CHECK();
}

template <class T>
void launch_scaled_copy(const T* v, int64_t n, T scale, T* out, cudaStream_t s) {
  if (n <= 0) return;
  scaled_copy_kernel<T><<<sm_grid(2, kSumBlocksMax), 256, 0, s>>>(v, n, scale, out);
  BHG_LAUNCH_CHECK();
}

template <class T>
int64_t symmetrize(uint32_t* cols, T* vals, int64_t n, int k, SymWorkspace<T>& ws, cudaStream_t s) {
  if (k > kMaxSortK) throw Error(ST_EINVAL, "error: the GPU affinity build supports at most 1024 neighbours per row.");
  int P = 1;
  while (P < k) P <<= 1;
  const size_t smem = (size_t)kSortWarps * P * (sizeof(uint32_t) + sizeof(T));
  if (smem > 48 * 1024) BHG_CUDA(cudaFuncSetAttribute(sort_rows_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  sort_rows_kernel<T><<<(unsigned)ceil_div(n, kSortWarps), kSortWarps * 32, smem, s>>>(cols, vals, n, k, P);
  BHG_LAUNCH_CHECK();
  const int64_t total = n * (int64_t)k;
  const int64_t m = 2 * total;
  const int cbits = bits_for(n);
  ws.keys.ensure(m * 8);
  ws.keys_alt.ensure(m * 8);
  ws.ev.ensure(m * sizeof(T));
  ws.ev_alt.ensure(m * sizeof(T));
  ws.count.ensure(64);
  BHG_CUDA(cudaMemsetAsync(ws.count.ptr, 0, 8, s));
  emit_entries_kernel<T><<<(unsigned)ceil_div(total, 256), 256, 0, s>>>(cols, vals, n, k, cbits, ws.keys.template as<uint64_t>(),
                                                                      ws.ev.template as<T>(),
                                                                      ws.count.template as<unsigned long long>());
  BHG_LAUNCH_CHECK();
  radix_sort_pairs<T>(ws.keys.template as<uint64_t>(), ws.ev.template as<T>(), ws.keys_alt.template as<uint64_t>(),
                      ws.ev_alt.template as<T>(), m, 0, 2 * cbits + 2, ws.sort_tmp, s);
  unsigned long long nnz = 0;
  BHG_CUDA(cudaMemcpyAsync(&nnz, ws.count.ptr, 8, cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  return (int64_t)nnz;
}

template <class T>
void symmetrize_finish(const SymWorkspace<T>& ws, int64_t n, int64_t nnz, uint64_t* rows, uint32_t* cols_out,
                       T* vals_out, cudaStream_t s) {
  const int cbits = bits_for(n);
  if (nnz > 0) {
    finish_csr_kernel<T><<<(unsigned)ceil_div(nnz, 256), 256, 0, s>>>(ws.keys.template as<uint64_t>(), ws.ev.template as<T>(), nnz,
                                                                     cbits, cols_out, vals_out);
    BHG_LAUNCH_CHECK();
  }
  row_ptr_kernel<<<(unsigned)ceil_div(n + 1, 256), 256, 0, s>>>(ws.keys.template as<uint64_t>(), nnz, n, cbits, rows);
  BHG_LAUNCH_CHECK();
}

#define BHG_INST(T)                                                                                          \
  template void launch_search_beta<T>(const T*, int64_t, int64_t, T, T*, int32_t*, cudaStream_t);            \
  template void launch_sum<T>(const T*, int64_t, double*, DevBuf&, cudaStream_t);                            \
  template void launch_normalize<T>(T*, int64_t, T, double*, DevBuf&, cudaStream_t);                         \
  template void launch_scale<T>(T*, int64_t, T, cudaStream_t);                                               \
  template void launch_scaled_copy<T>(const T*, int64_t, T, T*, cudaStream_t);                               \
  template int64_t symmetrize<T>(uint32_t*, T*, int64_t, int, SymWorkspace<T>&, cudaStream_t);               \
  template void symmetrize_finish<T>(const SymWorkspace<T>&, int64_t, int64_t, uint64_t*, uint32_t*, T*,     \
                                     cudaStream_t);
BHG_INST(float)
BHG_INST(double)

}  // namespace bhg
