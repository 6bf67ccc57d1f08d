// Batched Barnes-Hut fitting: many independent embeddings of uneven size are
// stepped together, one launch per stage for the whole batch.
//
// Layout: the jobs' points are stored back to back (job j owns rows
// off[j]..off[j+1]); job_of[g] is the job of point g. The affinity matrices
// form one block-diagonal CSR with global column indices. Each epoch:
//   per-job box (+ recentre)   batch_box_kernel, one block per job
//   per-job Morton codes       batch_morton_kernel (the job's own box)
//   sort by (job, code)        radix sort on the code, then a stable radix
//                              sort on the job id (job_key / gather_codes)
//   forest of per-job trees    bh_build_from_sorted with Segs (bh.cu)
//   traversal                  bh_traverse with Segs: each query walks only
//                              its own job's tree with its job's half widths
//   per-job Z                  batch_z_kernel, one block per job, FP64
//   attractive                 attractive pass on the block-diagonal CSR
//   update                     batch_update_kernel with the job's 1/Z and lr
// Every per-job quantity (box, tree, Z, mean) is computed exactly as for a
// single fit of that job; only reduction orders differ.
#include "batch.h"

#include "bh_dev.cuh"

namespace bhg {

namespace {

template <class T, int D>
__global__ void batch_box_kernel(T* __restrict__ y, const int64_t* __restrict__ off, int apply_mean,
                                 BoxParams<T>* __restrict__ boxes, int bits, const uint8_t* __restrict__ active) {
  __shared__ double sh[32];
  __shared__ T shr[32];
  __shared__ double means[D];
  const int j = blockIdx.x;
  const int64_t lo = off[j], hi = off[j + 1];
  const int64_t n = hi - lo;
  if (active && !active[j]) apply_mean = 0;
  T mean[D];
#pragma unroll
  for (int a = 0; a < D; ++a) mean[a] = T(0);
  if (apply_mean && n > 0) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      double s = 0.0;
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += (double)y[i * D + a];
      s = block_sum(s, sh);
      if (threadIdx.x == 0) means[a] = s;
      __syncthreads();
      mean[a] = (T)means[a] / (T)n;
    }
  }
  T mn[D], mx[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    mn[a] = Lim<T>::max();
    mx[a] = -Lim<T>::max();
  }
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
      T v = y[i * D + a];
      if (apply_mean) {
        v = v - mean[a];
        y[i * D + a] = v;
      }
      mn[a] = fmin(mn[a], v);
      mx[a] = fmax(mx[a], v);
    }
  }
  T fmn[D], fmx[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    T v = warp_min(mn[a]);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) shr[w] = v;
    __syncthreads();
    v = Lim<T>::max();
    for (int q = 0; q < (int)((blockDim.x + 31) >> 5); ++q) v = fmin(v, shr[q]);
    fmn[a] = v;
    v = warp_max(mx[a]);
    __syncthreads();
    if (lane == 0) shr[w] = v;
    __syncthreads();
    v = -Lim<T>::max();
    for (int q = 0; q < (int)((blockDim.x + 31) >> 5); ++q) v = fmax(v, shr[q]);
    fmx[a] = v;
  }
  if (threadIdx.x == 0) {
    BoxParams<T>* out = boxes + j;
    const T scale = (T)(double)(1ULL << bits);
    T max_extent = T(0);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const T ext = fmx[a] - fmn[a];
      out->mn[a] = fmn[a];
      out->mx[a] = fmx[a];
      out->inv_scale[a] = ext > T(0) ? scale / ext : T(0);
      max_extent = fmax(max_extent, ext);
    }
    for (int a = D; a < 8; ++a) {
      out->mn[a] = T(0);
      out->mx[a] = T(0);
      out->inv_scale[a] = T(0);
    }
    out->max_extent = max_extent;
    for (int l = 0; l <= bits; ++l) {
      const T hw = max_extent / (T)(double)(1ULL << (l + 1));
      out->hw2[l] = hw * hw;
    }
  }
}

template <class T, int D>
__global__ void batch_morton_kernel(const T* __restrict__ y, int64_t total, const uint32_t* __restrict__ job_of,
                                    const BoxParams<T>* __restrict__ boxes, uint64_t* __restrict__ keys,
                                    uint64_t* __restrict__ codes, uint32_t* __restrict__ perm) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  constexpr int B = MortonD<D>::BITS;
  const uint32_t max_bucket = (uint32_t)((1ULL << B) - 1);
  const BoxParams<T>* p = boxes + job_of[g];
  uint32_t q[D];
#pragma unroll
  for (int a = 0; a < D; ++a) q[a] = quantize<T>(y[g * D + a], p->mn[a], p->inv_scale[a], max_bucket);
  const uint64_t c = MortonD<D>::encode(q);
  keys[g] = c;
  codes[g] = c;
  perm[g] = (uint32_t)g;
}

__global__ void job_key_kernel(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ job_of, int64_t total,
                               uint64_t* __restrict__ jobkey) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < total) jobkey[s] = job_of[perm[s]];
}

__global__ void gather_codes_kernel(const uint32_t* __restrict__ perm, const uint64_t* __restrict__ codes,
                                    int64_t total, uint64_t* __restrict__ keys) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < total) keys[s] = codes[perm[s]];
}

template <class T>
__global__ void batch_z_kernel(const T* __restrict__ q, const int64_t* __restrict__ off, double* __restrict__ z) {
  __shared__ double sh[32];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int64_t i = off[j] + threadIdx.x; i < off[j + 1]; i += blockDim.x) s += (double)q[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) z[j] = s;
}

template <class T, int D>
__global__ void batch_update_kernel(T* __restrict__ y, const T* __restrict__ pos, const T* __restrict__ neg,
                                    T* __restrict__ uy, T* __restrict__ gains, int64_t total,
                                    const uint32_t* __restrict__ job_of, const double* __restrict__ z,
                                    const T* __restrict__ lr, const T* __restrict__ momentum,
                                    const uint8_t* __restrict__ active) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const uint32_t j = job_of[i];
  if (active && !active[j]) return;
  const T inv_norm = T(1) / (T)z[j];
  const T l = lr[j], mom = momentum[j];
  const T inc = (T)0.2, dec = (T)0.8, floor_ = (T)0.01;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const int64_t e = i * D + a;
    const T g = pos[e] - neg[e] * inv_norm;
    const T u = uy[e];
    T gn = (signum(g) != signum(u)) ? gains[e] + inc : gains[e] * dec;
    if (gn < floor_) gn = floor_;
    gains[e] = gn;
    const T un = mom * u - l * gn * g;
    uy[e] = un;
    y[e] = y[e] + un;
  }
}

// CSR of one job appended to the block-diagonal matrix.
__global__ void offset_rows_kernel(const uint64_t* __restrict__ rows, int64_t n, uint64_t add,
                                   uint64_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = rows[i] + add;
}

__global__ void offset_cols_kernel(const uint32_t* __restrict__ cols, int64_t nnz, uint32_t add,
                                   uint32_t* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = cols[e] + add;
}

__global__ void sub_rows_kernel(const uint64_t* __restrict__ rows, int64_t n1, uint64_t sub, uint64_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n1) out[i] = rows[i] - sub;
}

__global__ void sub_cols_kernel(const uint32_t* __restrict__ cols, int64_t nnz, uint32_t sub, uint32_t* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = cols[e] - sub;
}

// normalize_p_values per job: p *= exaggeration / (sum + eps) in T, the sum in
// FP64 over the job's slice; then p *= 1 / exaggeration when lying is off.
template <class T>
__global__ void batch_normalize_kernel(T* __restrict__ v, const int64_t* __restrict__ nnz_off, T exaggeration,
                                       int unexaggerate) {
  __shared__ double sh[32];
  __shared__ double total;
  const int j = blockIdx.x;
  const int64_t lo = nnz_off[j], hi = nnz_off[j + 1];
  double s = 0.0;
  for (int64_t e = lo + threadIdx.x; e < hi; e += blockDim.x) s += (double)v[e];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) total = s;
  __syncthreads();
  const T scale = exaggeration / ((T)total + Lim<T>::eps());
  const T un = T(1) / exaggeration;
  for (int64_t e = lo + threadIdx.x; e < hi; e += blockDim.x) {
    T x = v[e] * scale;
    if (unexaggerate) x *= un;
    v[e] = x;
  }
}

__global__ void offset_u32_kernel(const uint32_t* __restrict__ in, int64_t count, uint32_t add,
                                  uint32_t* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = in[e] + add;
}

__global__ void fill_job_kernel(uint32_t* __restrict__ job_of, int64_t lo, int64_t hi, uint32_t j) {
  const int64_t i = lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < hi) job_of[i] = j;
}

int bits_for(int64_t v) {
  int b = 1;
  while ((1LL << b) <= v) ++b;
  return b;
}

}  // namespace

template <class T>
void batch_box(int D, T* y, const int64_t* off, int K, bool apply_mean, BoxParams<T>* boxes, int bits, cudaStream_t s,
               const uint8_t* active) {
  if (K <= 0) return;
  if (D == 2) batch_box_kernel<T, 2><<<K, 256, 0, s>>>(y, off, apply_mean ? 1 : 0, boxes, bits, active);
  else batch_box_kernel<T, 3><<<K, 256, 0, s>>>(y, off, apply_mean ? 1 : 0, boxes, bits, active);
  BHG_LAUNCH_CHECK();
}

template <class T>
void batch_sort_and_build(int D, const T* y, int64_t total, int K, const uint32_t* job_of, const int64_t* off,
                          const BoxParams<T>* boxes, BhWorkspace<T>& ws, DevBuf& codes, DevBuf& jobkey,
                          DevBuf& jobkey_alt, const SegTiles& tiles, cudaStream_t s) {
  const unsigned g = (unsigned)ceil_div(total, 256);
  uint64_t* cd = static_cast<uint64_t*>(codes.ensure((size_t)total * 8));
  uint64_t* jk = static_cast<uint64_t*>(jobkey.ensure((size_t)total * 8));
  uint64_t* jka = static_cast<uint64_t*>(jobkey_alt.ensure((size_t)total * 8));
  int B;
  if (D == 2) {
    batch_morton_kernel<T, 2><<<g, 256, 0, s>>>(y, total, job_of, boxes, ws.keys.template as<uint64_t>(), cd,
                                                ws.perm.template as<uint32_t>());
    B = 32;
  } else {
    batch_morton_kernel<T, 3><<<g, 256, 0, s>>>(y, total, job_of, boxes, ws.keys.template as<uint64_t>(), cd,
                                                ws.perm.template as<uint32_t>());
    B = 21;
  }
  BHG_LAUNCH_CHECK();
  radix_sort_pairs<uint32_t>(ws.keys.template as<uint64_t>(), ws.perm.template as<uint32_t>(),
                             ws.keys_alt.template as<uint64_t>(), ws.perm_alt.template as<uint32_t>(), total, 0, D * B,
                             ws.sort_tmp, s);
  job_key_kernel<<<g, 256, 0, s>>>(ws.perm.template as<uint32_t>(), job_of, total, jk);
  BHG_LAUNCH_CHECK();
  const int jbits = bits_for(K > 1 ? K - 1 : 1);
  radix_sort_pairs<uint32_t>(jk, ws.perm.template as<uint32_t>(), jka, ws.perm_alt.template as<uint32_t>(), total, 0,
                             ((jbits + 7) / 8) * 8, ws.sort_tmp, s);
  gather_codes_kernel<<<g, 256, 0, s>>>(ws.perm.template as<uint32_t>(), cd, total, ws.keys.template as<uint64_t>());
  BHG_LAUNCH_CHECK();
  Segs sg;
  sg.job = jk;
  sg.off = off;
  tiles.fill(sg);
  bh_build_from_sorted<T>(ws, D, y, total, sg, s);
}

template <class T>
void batch_z(const T* q, const int64_t* off, int K, double* z, cudaStream_t s) {
  if (K <= 0) return;
  batch_z_kernel<T><<<K, 256, 0, s>>>(q, off, z);
  BHG_LAUNCH_CHECK();
}

template <class T>
void batch_update(int D, T* y, const T* pos, const T* neg, T* uy, T* gains, int64_t total, const uint32_t* job_of,
                  const double* z, const T* lr, const T* momentum, cudaStream_t s, const uint8_t* active) {
  const unsigned g = (unsigned)ceil_div(total, 256);
  if (D == 2)
    batch_update_kernel<T, 2><<<g, 256, 0, s>>>(y, pos, neg, uy, gains, total, job_of, z, lr, momentum, active);
  else
    batch_update_kernel<T, 3><<<g, 256, 0, s>>>(y, pos, neg, uy, gains, total, job_of, z, lr, momentum, active);
  BHG_LAUNCH_CHECK();
}

void batch_append_csr(const uint64_t* rows, const uint32_t* cols, int64_t n, int64_t nnz, uint64_t row_add,
                      uint32_t col_add, uint64_t* rows_out, uint32_t* cols_out, cudaStream_t s) {
  offset_rows_kernel<<<(unsigned)ceil_div(n + 1, 256), 256, 0, s>>>(rows, n + 1, row_add, rows_out);
  BHG_LAUNCH_CHECK();
  if (nnz > 0) {
    offset_cols_kernel<<<(unsigned)std::min<int64_t>(ceil_div(nnz, 256), sm_grid(4, 4096)), 256, 0, s>>>(cols, nnz, col_add,
                                                                                                 cols_out);
    BHG_LAUNCH_CHECK();
  }
}

void batch_extract_csr(const uint64_t* rows, const uint32_t* cols, int64_t n, int64_t nnz, uint64_t row_sub,
                       uint32_t col_sub, uint64_t* rows_out, uint32_t* cols_out, cudaStream_t s) {
  sub_rows_kernel<<<(unsigned)ceil_div(n + 1, 256), 256, 0, s>>>(rows, n + 1, row_sub, rows_out);
  BHG_LAUNCH_CHECK();
  if (nnz > 0) {
    sub_cols_kernel<<<(unsigned)std::min<int64_t>(ceil_div(nnz, 256), sm_grid(4, 4096)), 256, 0, s>>>(cols, nnz, col_sub,
                                                                                              cols_out);
    BHG_LAUNCH_CHECK();
  }
}

template <class T>
void batch_normalize(T* vals, const int64_t* nnz_off, int K, T exaggeration, bool unexaggerate, cudaStream_t s) {
  if (K <= 0) return;
  batch_normalize_kernel<T><<<K, 512, 0, s>>>(vals, nnz_off, exaggeration, unexaggerate ? 1 : 0);
  BHG_LAUNCH_CHECK();
}

void batch_offset_indices(const uint32_t* in, int64_t count, uint32_t add, uint32_t* out, cudaStream_t s) {
  if (count <= 0) return;
  offset_u32_kernel<<<(unsigned)std::min<int64_t>(ceil_div(count, 256), sm_grid(8, 8192)), 256, 0, s>>>(in, count, add, out);
  BHG_LAUNCH_CHECK();
}

void batch_fill_job(uint32_t* job_of, int64_t lo, int64_t hi, uint32_t j, cudaStream_t s) {
  if (hi <= lo) return;
  fill_job_kernel<<<(unsigned)ceil_div(hi - lo, 256), 256, 0, s>>>(job_of, lo, hi, j);
  BHG_LAUNCH_CHECK();
}

template <class T>
void group_affinities_from_knn(int64_t tot, int64_t k, T perplexity, GroupCsr<T>& out, AffinityScratch<T>& ws,
                               cudaStream_t s) {
  uint32_t* kidx = ws.kidx.template as<uint32_t>();
  T* kdist = ws.kdist.template as<T>();
  ws.kp.ensure((size_t)tot * k * sizeof(T));
  launch_search_beta<T>(kdist, tot, k, perplexity, ws.kp.template as<T>(), nullptr, s);
  const int64_t nnz = symmetrize<T>(kidx, ws.kp.template as<T>(), tot, (int)k, ws.sym, s);
  out.rows.ensure((size_t)(tot + 1) * 8);
  out.cols.ensure((size_t)std::max<int64_t>(nnz, 1) * 4);
  out.vals.ensure((size_t)std::max<int64_t>(nnz, 1) * sizeof(T));
  symmetrize_finish<T>(ws.sym, tot, nnz, out.rows.template as<uint64_t>(), out.cols.template as<uint32_t>(),
                       out.vals.template as<T>(), s);
  out.rows_h.resize(tot + 1);
  BHG_CUDA(cudaMemcpyAsync(out.rows_h.data(), out.rows.ptr, (size_t)(tot + 1) * 8, cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  out.nnz = nnz;
  ws.sym.release();
  ws.kp.release();
}

template <class T>
void group_affinities_euclidean(const std::vector<const T*>& X, const std::vector<int64_t>& n, int dim, int64_t k,
                                T perplexity, GroupCsr<T>& out, AffinityScratch<T>& ws, cudaStream_t s) {
  const int G = (int)n.size();
  std::vector<int64_t> goff(G + 1, 0);
  for (int g = 0; g < G; ++g) goff[g + 1] = goff[g] + n[g];
  const int64_t tot = goff[G];
  int64_t* d_off = static_cast<int64_t*>(ws.g_off.ensure(goff.size() * 8));
  BHG_CUDA(cudaMemcpyAsync(d_off, goff.data(), goff.size() * 8, cudaMemcpyHostToDevice, s));
  uint32_t* gof = static_cast<uint32_t*>(ws.g_of.ensure((size_t)tot * 4));
  for (int g = 0; g < G; ++g) batch_fill_job(gof, goff[g], goff[g + 1], (uint32_t)g, s);
  T* Xs = static_cast<T*>(ws.xin.ensure((size_t)tot * dim * sizeof(T)));
  for (int g = 0; g < G; ++g)
    BHG_CUDA(cudaMemcpyAsync(Xs + goff[g] * dim, X[g], (size_t)n[g] * dim * sizeof(T), cudaMemcpyDeviceToDevice, s));
  uint32_t* kidx = static_cast<uint32_t*>(ws.kidx.ensure((size_t)tot * k * 4));
  T* kdist = static_cast<T*>(ws.kdist.ensure((size_t)tot * k * sizeof(T)));
  knn_euclidean_segmented<T>(Xs, tot, dim, (int)k, goff, d_off, gof, kidx, kdist, ws.knn, s);
  ws.xin.release();
  ws.knn.release();
  group_affinities_from_knn<T>(tot, k, perplexity, out, ws, s);
}

#define BHG_INST(T)                                                                                                  \
  template void batch_box<T>(int, T*, const int64_t*, int, bool, BoxParams<T>*, int, cudaStream_t, const uint8_t*); \
  template void batch_sort_and_build<T>(int, const T*, int64_t, int, const uint32_t*, const int64_t*,               \
                                        const BoxParams<T>*, BhWorkspace<T>&, DevBuf&, DevBuf&, DevBuf&,             \
                                        const SegTiles&, cudaStream_t);                                              \
  template void batch_z<T>(const T*, const int64_t*, int, double*, cudaStream_t);                                    \
  template void batch_normalize<T>(T*, const int64_t*, int, T, bool, cudaStream_t);                                  \
  template void batch_update<T>(int, T*, const T*, const T*, T*, T*, int64_t, const uint32_t*, const double*,        \
                                const T*, const T*, cudaStream_t, const uint8_t*);
BHG_INST(float)
BHG_INST(double)
template void group_affinities_from_knn<float>(int64_t, int64_t, float, GroupCsr<float>&, AffinityScratch<float>&,
                                               cudaStream_t);
template void group_affinities_from_knn<double>(int64_t, int64_t, double, GroupCsr<double>&, AffinityScratch<double>&,
                                                cudaStream_t);
template void group_affinities_euclidean<float>(const std::vector<const float*>&, const std::vector<int64_t>&, int,
                                                int64_t, float, GroupCsr<float>&, AffinityScratch<float>&,
                                                cudaStream_t);
template void group_affinities_euclidean<double>(const std::vector<const double*>&, const std::vector<int64_t>&, int,
                                                 int64_t, double, GroupCsr<double>&, AffinityScratch<double>&,
                                                 cudaStream_t);

}  // namespace bhg
