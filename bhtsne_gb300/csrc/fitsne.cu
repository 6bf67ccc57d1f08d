// FIt-SNE repulsion on the GPU: Lagrange spread onto an equispaced grid, FFT
// convolution with the squared Cauchy kernel, gather, and reconstruction of
// the forces and Z.
//
// Reference behaviour restated (bhtsne 0.7.10, src/tsne/interpolation.rs):
//  * square domain over the joint coordinate range, extent floored at
//    min_positive (:115-116); boxes = clamp(ceil(extent / 1), 10, 1000)
//    (:353-358); 3 Lagrange nodes per box at (k + 1/2)/3 (:395-441);
//    locate_points (:162-187); charges [1, y_1..y_D, |y|^2] (:446-456);
//    tensor-product weights, axis 0 the slow grid index (:462-481);
//    kernel (1 + spacing^2 lag^2)^-2 over signed lags (:198-226);
//    reconstruct (:305-332): F_i = y_i phi_0 - phi_{1+d},
//    Z = sum_i [(1 + |y_i|^2) phi_0 - 2 y_i . phi_1 + phi_{D+1}] - N.
//
// GPU choices:
//  * The transform length is the next power of two >= 2 nodes - 1 rather than
//    the reference's 7-smooth length. Any length >= 2 nodes - 1 yields the
//    same linear convolution on the node window (charges are zero padded and
//    wrapped lags are never read), so only rounding differs.
//  * The kernel is real and even, so its spectrum is real: two real charge
//    grids are packed as the real and imaginary parts of one complex grid and
//    convolved together (D + 2 terms -> 2 complex transforms). The pairs are
//    (s, y_1) and (y_2, |y|^2 / s) with s a power of two near max |y|, so both
//    halves of a pair have similar magnitude and neither one's rounding noise
//    swamps the other; scaling by a power of two is exact.
//  * 2-D transforms are row FFTs plus tiled transposes. Forward transforms
//    leave their spectra in bit-reversed order and the inverse transforms read
//    that order, so there is no reordering pass; the spectrum also stays in
//    transposed layout, which is harmless because the kernel spectrum goes
//    through the same pipeline and is symmetric in its two axes. Rows that
//    are known to be zero (charges) or unused (potentials) are skipped.
//  * The spread scatters with 64-bit integer atomics on a fixed-point grid
//    (units of 2^-fix_shift, chosen so no partial sum can overflow), so the
//    accumulated charges do not depend on the order of the atomics and the fit
//    is reproducible run to run like the reference's sequential spread; the
//    gather re-derives each point's boxes and weights instead of storing them.
#include "fitsne.h"

#include <cmath>
#include <vector>

namespace bhg {

namespace {

template <class T>
struct Cx;
template <>
struct Cx<float> {
  typedef float2 type;
};
template <>
struct Cx<double> {
  typedef double2 type;
};

// Complex arithmetic of the transforms. The FFT is this library's own (the
// reference uses rustfft), so its rounding is free: the product uses fused
// multiply-adds, and f32 sums and differences use the paired f32x2
// instructions (one instruction for both parts). The spread, the kernel
// values and the gather keep the reference's arithmetic.
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  float2 r;
  r.x = __fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y));
  r.y = __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x));
  return r;
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  double2 r;
  r.x = __fma_rn(a.x, b.x, -__dmul_rn(a.y, b.y));
  r.y = __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x));
  return r;
}

template <class T>
struct Lagrange3 {
  T node[3];
  T inv_denom[3];
  __device__ Lagrange3() {
    const T half = T(0.5);
    const T p_recip = T(1) / T(3);
#pragma unroll
    for (int k = 0; k < 3; ++k) node[k] = (T(k) + half) * p_recip;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      T denom = T(1);
#pragma unroll
      for (int m = 0; m < 3; ++m)
        if (m != k) denom = denom * (node[k] - node[m]);
      inv_denom[k] = T(1) / denom;
    }
  }
  __device__ __forceinline__ void weights(T local, T* out) const {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      T num = T(1);
#pragma unroll
      for (int m = 0; m < 3; ++m)
        if (m != k) num = num * (local - node[m]);
      out[k] = num * inv_denom[k];
    }
  }
};

// Grid parameters of the current embedding. With cap_L > 0 the grid must fit
// a cap_L transform: when it does not, out->need_L records the length needed,
// *overflow is raised and the box count is cut so every later kernel stays
// inside the capacity (that epoch's result is discarded by the caller).
template <class T, int D>
__global__ void fit_params_kernel(const BoxParams<T>* __restrict__ box, int64_t n_points, FitParams<T>* __restrict__ out,
                                  int cap_L, int* __restrict__ overflow) {
  if (threadIdx.x != 0) return;
  T lo = box->mn[0], hi = box->mx[0];
#pragma unroll
  for (int a = 1; a < D; ++a) {
    lo = fmin(lo, box->mn[a]);
    hi = fmax(hi, box->mx[a]);
  }
  const T extent = fmax(hi - lo, Lim<T>::min_pos());
  const T scaled = ceil(extent / T(1.0));
  int64_t boxes = 0;
  if (scaled > T(0)) boxes = scaled >= T(9.0e18) ? INT64_MAX : (int64_t)scaled;
  boxes = boxes < 10 ? 10 : (boxes > 1000 ? 1000 : boxes);
  int nodes = (int)boxes * 3;
  // the shorter of the next power of two and the next 3 * 2^j (>= 24)
  int L = 16;
  while (L < 2 * nodes - 1) L <<= 1;
  int L3 = 24;
  while (L3 < 2 * nodes - 1) L3 <<= 1;
  if (L3 < L) L = L3;
  out->need_L = L;
  if (cap_L > 0 && L > cap_L) {
    *overflow = 1;
    boxes = cap_L / 6 > 1 ? cap_L / 6 : 1;
    nodes = (int)boxes * 3;
    L = cap_L;
  }
  const T box_width = extent / (T)(double)boxes;
  T m = fmax(fmax(fabs(lo), fabs(hi)), T(1));
  int ex = 0;
  frexp(m, &ex);
  out->scale = ldexp(T(1), ex);
  // |charge| <= 2 scale and sum_combos |w| <= 3.5^D, so every partial sum is
  // below 3.5^D * 2 scale * n; keep it under 2^62.
  const double bound = pow(3.5, (double)D) * 2.0 * (double)out->scale * (double)(n_points > 0 ? n_points : 1);
  int eb = 0;
  frexp(bound, &eb);
  out->fix_shift = 62 - eb;
  out->up = (T)ldexp(1.0, out->fix_shift);
  out->down = (T)ldexp(1.0, -out->fix_shift);
  out->lo = lo;
  out->extent = extent;
  out->box_width = box_width;
  out->inv_box_width = T(1) / box_width;
  out->spacing = box_width / T(3);
  out->boxes = (int)boxes;
  out->nodes = nodes;
  out->L = L;
}

template <class T>
__device__ __forceinline__ void locate(T v, const FitParams<T>& p, const Lagrange3<T>& lb, int* box, T* w) {
  const T offset = (v - p.lo) * p.inv_box_width;
  const T b = floor(offset);
  const int64_t last = p.boxes - 1;
  int64_t id = 0;
  if (b > T(0)) {
    id = b >= T(9.0e18) ? last : (int64_t)b;
    if (id > last) id = last;
  }
  *box = (int)id;
  const T local = offset - (T)(int)id;  // id < 1000: exact either way
  lb.weights(local, w);
}

// A charge already scaled by 2^fix_shift (exact: a power of two) rounded to the
// nearest integer. f32 goes through integer operations (no FP64 pipe); the
// result equals the FP64 conversion of the same value.
__device__ __forceinline__ long long to_fixed(float x) { return f32_to_i64_rn(x); }
__device__ __forceinline__ long long to_fixed(double x) { return __double2ll_rn(x); }

// Charges of one point in fixed point: 3^D nodes x (D + 2) values. Integer
// sums are exact and order-free, so the grid does not depend on how the adds
// are grouped.
template <class T, int D>
__global__ void spread_kernel(const T* __restrict__ y, int64_t n, const FitParams<T>* __restrict__ prm,
                              long long* __restrict__ acc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = i < n;
  const FitParams<T> p = *prm;
  const Lagrange3<T> lb;
  const int L = p.L;
  constexpr int combos = D == 1 ? 3 : 9;
  constexpr int NV = D + 2;
  int box[D];
  T w[D][3];
  T yv[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    yv[a] = valid ? y[i * D + a] : T(0);
    locate<T>(yv[a], p, lb, &box[a], w[a]);
  }
  T sq = T(0);
#pragma unroll
  for (int a = 0; a < D; ++a) sq = sq + yv[a] * yv[a];
  long long v[combos][NV];
#pragma unroll
  for (int c = 0; c < combos; ++c) {
    int rem = c;
    T wt = T(1);
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const int k = rem % 3;
      rem /= 3;
      wt = wt * w[a][k];
    }
    v[c][0] = to_fixed((wt * p.scale) * p.up);
    v[c][1] = to_fixed((wt * yv[0]) * p.up);
    if (D == 2) v[c][D] = to_fixed((wt * yv[D - 1]) * p.up);
    v[c][NV - 1] = to_fixed((wt * (sq / p.scale)) * p.up);
    if (!valid) {
#pragma unroll
      for (int q = 0; q < NV; ++q) v[c][q] = 0;
    }
  }
  // Points are mostly in Z-order (the layout is renumbered by Morton order),
  // so runs of lanes share a box and so all 3^D target cells: sum each run in
  // registers (segmented reduction to the run's first lane) and let that lane
  // alone issue the atomics. A warp with many runs adds directly.
  long long key = valid ? (long long)box[0] : -1 - (long long)lane;
  if (D == 2 && valid) key = key * 4096 + box[D - 1];
  const long long prev = __shfl_up_sync(0xffffffffu, key, 1);
  const bool head = lane == 0 || prev != key;
  const unsigned heads = __ballot_sync(0xffffffffu, head);
  const bool combine = __popc(heads) <= 16;
  if (combine) {
    const int run = __popc(heads & ((2u << lane) - 1u));
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int orun = __shfl_down_sync(0xffffffffu, run, off);
      const bool take = lane + off < 32 && orun == run;
#pragma unroll
      for (int c = 0; c < combos; ++c)
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          const long long o = __shfl_down_sync(0xffffffffu, v[c][q], off);
          if (take) v[c][q] += o;
        }
    }
  }
  if (!valid || (combine && !head)) return;
#pragma unroll
  for (int c = 0; c < combos; ++c) {
    int rem = c;
    int64_t flat = 0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const int k = rem % 3;
      rem /= 3;
      flat = flat * L + (box[a] * 3 + k);
    }
    unsigned long long* cell = reinterpret_cast<unsigned long long*>(acc + 4 * flat);
#pragma unroll
    for (int q = 0; q < NV; ++q) atomicAdd(cell + q, (unsigned long long)v[c][q]);
  }
}






__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
      "add.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 pa, pb, pr;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
      "sub.rn.f32x2 pr, pa, pb;\n\tmov.b64 {%0, %1}, pr;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  a.x += b.x;
  a.y += b.y;
  return a;
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) {
  a.x -= b.x;
  a.y -= b.y;
  return a;
}
template <class T2>
__device__ __forceinline__ T2 shfl_xor2(T2 v, int m) {
  v.x = __shfl_xor_sync(kFull, v.x, m);
  v.y = __shfl_xor_sync(kFull, v.y, m);
  return v;
}

__device__ __forceinline__ uint32_t fft_smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// The row into shared memory with one bulk copy (TMA engine) completing on an
// mbarrier; the wait is bounded: on timeout *fault is raised and false returned.
__device__ __forceinline__ bool fft_load_row(void* smem_dst, const void* gsrc, uint32_t bytes, uint64_t* bar,
                                             int* fault) {
  const uint32_t b = fft_smem_addr(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     fft_smem_addr(smem_dst)),
                 "l"(gsrc), "r"(bytes), "r"(b)
                 : "memory");
  }
  long long spins = 0;
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(b)
        : "memory");
    if (ok) return true;
    if (++spins >= (1LL << 24)) {
      atomicExch(fault, 1);
      return false;
    }
  }
}

// Fixed-point charges -> the two packed complex grids: the first `nodes`
// entries of the rows < nodes (one row for D = 1) with row stride L, the
// cells the spread can reach. clear_cells_kernel then zeroes those cells
// (write-only), so the accumulator is zero again for the next spread.
// Fixed-point value times 2^-fix_shift in T: one rounding of the exact
// product (the scale is a power of two), without the FP64 pipe for f32.
__device__ __forceinline__ float unfix_value(long long v, float down) { return i64_to_f32_rn(v) * down; }
__device__ __forceinline__ double unfix_value(long long v, double down) { return (double)v * down; }

template <class T, int D>
__global__ void clear_cells_kernel(long long* __restrict__ acc, const FitParams<T>* __restrict__ prm) {
  const int nodes = prm->nodes;
  const int r = (int)blockIdx.y, c = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (r >= (D == 1 ? 1 : nodes) || c >= nodes) return;
  longlong2* cell = reinterpret_cast<longlong2*>(acc + 4 * ((int64_t)r * prm->L + c));
  __stcs(cell, make_longlong2(0, 0));
  __stcs(cell + 1, make_longlong2(0, 0));
}

template <class T, int D>
__global__ void charges_kernel(const long long* __restrict__ acc, const FitParams<T>* __restrict__ prm,
                               typename Cx<T>::type* __restrict__ g0, typename Cx<T>::type* __restrict__ g1) {
  // one cell per thread: row blockIdx.y, column blockIdx.x * blockDim.x +
  // threadIdx.x (the grid covers the capacity; blocks past nodes exit)
  const int nodes = prm->nodes;
  const int r = (int)blockIdx.y, c = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (r >= (D == 1 ? 1 : nodes) || c >= nodes) return;
  const T down = prm->down;
  const int L = prm->L;
  {
    const int64_t flat = (int64_t)r * L + c;
    const longlong2* cell = reinterpret_cast<const longlong2*>(acc + 4 * flat);
    const longlong2 p = __ldcs(cell), q = __ldcs(cell + 1);
    typename Cx<T>::type a, b;
    a.x = unfix_value(p.x, down);
    a.y = unfix_value(p.y, down);
    b.x = unfix_value(q.x, down);
    b.y = unfix_value(q.y, down);
    g0[flat] = a;
    g1[flat] = b;
  }
}

// 1-D grids (at most 3000 nodes): the linear convolution of the three charge
// rows with the squared Cauchy kernel, summed directly in FP64 instead of by
// f32 transforms. The kernel values are the reference's (computed in T as the
// transform path builds its rows), the charges the exact fixed-point sums; the
// result is the convolution the transforms compute, without their rounding,
// which the 1-D Z terms (|y|^2 phi_0 against phi_2, both near 1e6 at the
// 1000-box cap) would amplify to percent level.
// tab: kernel K(lag) at [0, nodes), charge row k at [cap (1 + k), + nodes),
// potential k at [cap (4 + k), + nodes).
template <class T>
__global__ void conv1d_prep_kernel(const long long* __restrict__ acc, const FitParams<T>* __restrict__ prm, int cap,
                                   double* __restrict__ tab) {
  const int nodes = prm->nodes;
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= nodes) return;
  const T dc = prm->spacing * (T)(double)i;
  T sq = T(0);
  sq = sq + dc * dc;
  const T cauchy = T(1) / (T(1) + sq);
  tab[i] = (double)(cauchy * cauchy);
  const double down = (double)prm->down;  // a power of two
#pragma unroll
  for (int k = 0; k < 3; ++k) tab[(int64_t)cap * (1 + k) + i] = (double)acc[4 * (int64_t)i + k] * down;
}

// One warp per output node j: lanes take the source nodes i = lane + 32 t,
// then a fixed shuffle tree adds the 32 partial sums (deterministic). The
// node potentials stay in FP64 (tab at [cap (4 + k), + nodes)) for the
// gather, which interpolates them in FP64.
template <class T>
__global__ void conv1d_direct_kernel(double* __restrict__ tab, const FitParams<T>* __restrict__ prm, int cap) {
  const int nodes = prm->nodes;
  const int j = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= nodes) return;  // uniform per warp
  const double* q0 = tab + cap;
  const double* q1 = tab + 2 * (int64_t)cap;
  const double* q2 = tab + 3 * (int64_t)cap;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int i = lane; i < nodes; i += 32) {
    const double k = tab[j > i ? j - i : i - j];
    s0 = fma(k, q0[i], s0);
    s1 = fma(k, q1[i], s1);
    s2 = fma(k, q2[i], s2);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(kFull, s0, o);
    s1 += __shfl_xor_sync(kFull, s1, o);
    s2 += __shfl_xor_sync(kFull, s2, o);
  }
  if (lane == 0) {
    tab[4 * (int64_t)cap + j] = s0;
    tab[5 * (int64_t)cap + j] = s1;
    tab[6 * (int64_t)cap + j] = s2;
  }
}

// Stages of a power-of-two transform of length L = 2^log2L in place in
// shared memory. Forward transforms are decimation in frequency (natural order
// in, bit-reversed spectrum out), inverse transforms decimation in time (bit-
// reversed in, natural out): no reordering pass exists, every spectrum (the
// Cauchy kernel's included) is held in the same bit-reversed layout, and
// pointwise products are unaffected. Stages of span >= 64 run in shared memory
// two at a time (radix 2^2: four elements through both stages in registers),
// where consecutive lanes touch consecutive elements; stages of span <= 32 run
// in registers across a warp with shuffles (lane l holds element 32 g + l).
// tw holds the twiddles stage by stage: W_S^k at tw[S / 2 - 1 + k] for every
// power of two S <= cap and k < S / 2, so the butterflies of a stage, whose
// positions are consecutive across lanes, read consecutive entries (a strided
// view of one W_cap table costs one L1 wavefront per lane at the short spans).

template <class T2>
__device__ __forceinline__ T2 twid(const T2* __restrict__ tw, int S, int k) {
  return tw[(S >> 1) - 1 + k];
}

// DIF stages of spans L .. 2^(small + 1) of `nsub` consecutive rows of
// length L held back to back, ending with a barrier.
template <class T2>
__device__ __forceinline__ void dif_smem_stages(T2* s, int L, int log2L, int small, const T2* __restrict__ tw,
                                                int nsub) {
  int lg = log2L;
  if (((log2L - small) & 1) != 0) {
    // one radix-2 stage of span L
    const int half = L >> 1;
#pragma unroll 2
    for (int b0 = threadIdx.x; b0 < nsub * half; b0 += blockDim.x) {
      const int b = b0 & (half - 1);
      T2* r = s + (b0 >> (log2L - 1)) * L;
      const T2 a = r[b], c = r[b + half];
      r[b] = cadd(a, c);
      r[b + half] = cmul(csub(a, c), twid(tw, L, b));
    }
    __syncthreads();
    lg -= 1;
  }
  for (; lg - 1 > small; lg -= 2) {
    // stages of spans S = 2^lg and S/2: quarter q = S/4
    const int q = 1 << (lg - 2);
#pragma unroll 2
    for (int b0 = threadIdx.x; b0 < nsub * (L >> 2); b0 += blockDim.x) {
      const int b = b0 & ((L >> 2) - 1);
      const int pos = b & (q - 1);
      const int i = (b0 >> (log2L - 2)) * L + ((b >> (lg - 2)) << lg) + pos;
      const T2 wa = twid(tw, 1 << lg, pos);  // W_S^pos
      T2 wb;                         // W_S^(pos+q) = W_S^pos * (-i)
      wb.x = wa.y;
      wb.y = -wa.x;
      const T2 wc = twid(tw, 1 << (lg - 1), pos);  // W_(S/2)^pos
      const T2 x0 = s[i], x1 = s[i + q], x2 = s[i + 2 * q], x3 = s[i + 3 * q];
      const T2 y0 = cadd(x0, x2), y2 = cmul(csub(x0, x2), wa);
      const T2 y1 = cadd(x1, x3), y3 = cmul(csub(x1, x3), wb);
      s[i] = cadd(y0, y1);
      s[i + q] = cmul(csub(y0, y1), wc);
      s[i + 2 * q] = cadd(y2, y3);
      s[i + 3 * q] = cmul(csub(y2, y3), wc);
    }
    __syncthreads();
  }
}

// DIT stages (conjugate twiddles) of spans 2^(small + 1) .. L, each pass
// ending with a barrier. Stages lg and lg + 1 together: a group of 4h
// elements, h = 2^(lg-1); stage lg uses W_2h^pos for both of its pairs,
// stage lg + 1 uses W_4h^pos and W_4h^(pos+h) = W_4h^pos * W_4^1, an exact
// quarter turn.
template <class T2>
__device__ __forceinline__ void dit_smem_stages(T2* s, int L, int log2L, int small, const T2* __restrict__ tw,
                                                int nsub) {
  int lg = small + 1;
  for (; lg + 1 <= log2L; lg += 2) {
    const int h = 1 << (lg - 1);
#pragma unroll 2
    for (int b0 = threadIdx.x; b0 < nsub * (L >> 2); b0 += blockDim.x) {
      const int b = b0 & ((L >> 2) - 1);
      const int pos = b & (h - 1);
      const int i = (b0 >> (log2L - 2)) * L + ((b >> (lg - 1)) << (lg + 1)) + pos;
      T2 w1 = twid(tw, 1 << lg, pos);
      T2 w2 = twid(tw, 1 << (lg + 1), pos);
      w1.y = -w1.y;
      w2.y = -w2.y;
      T2 w3;  // conjugate quarter turn: W_4^-1 = +i
      w3.x = -w2.y;
      w3.y = w2.x;
      T2 x0 = s[i], x1 = s[i + h], x2 = s[i + 2 * h], x3 = s[i + 3 * h];
      T2 t = cmul(x1, w1);
      x1 = csub(x0, t);
      x0 = cadd(x0, t);
      t = cmul(x3, w1);
      x3 = csub(x2, t);
      x2 = cadd(x2, t);
      t = cmul(x2, w2);
      s[i] = cadd(x0, t);
      s[i + 2 * h] = csub(x0, t);
      t = cmul(x3, w3);
      s[i + h] = cadd(x1, t);
      s[i + 3 * h] = csub(x1, t);
    }
    __syncthreads();
  }
  for (; lg <= log2L; ++lg) {
    const int half = 1 << (lg - 1);
#pragma unroll 2
    for (int b0 = threadIdx.x; b0 < nsub * (L >> 1); b0 += blockDim.x) {
      const int b = b0 & ((L >> 1) - 1);
      const int pos = b & (half - 1);
      const int i = (b0 >> (log2L - 1)) * L + ((b >> (lg - 1)) << lg) + pos;
      const int j = i + half;
      T2 w = twid(tw, 1 << lg, pos);
      w.y = -w.y;
      const T2 u = s[i];
      const T2 v = cmul(s[j], w);
      s[i] = cadd(u, v);
      s[j] = csub(u, v);
    }
    __syncthreads();
  }
}

// Lengths L = 3 M: a radix-3 stage of span L splits the row into three
// consecutive power-of-two rows of length M (decimation in frequency:
// position k M + p then holds frequency 3 bitrev(p) + k), and the inverse
// ends with the matching combination. tw3 holds W_cap3^k for k < cap3 and
// tws3 = cap3 / L. W_3 = -1/2 - i sqrt(3)/2.
template <class T2, class T>
__device__ __forceinline__ void r3_dif_stage(T2* s, int M, const T2* __restrict__ tw3, int tws3) {
  const T h = T(0.86602540378443864676);
  for (int n = threadIdx.x; n < M; n += blockDim.x) {
    const T2 x0 = s[n], x1 = s[n + M], x2 = s[n + 2 * M];
    const T2 a = cadd(x1, x2), b = csub(x1, x2);
    T2 t, u;
    t.x = x0.x - T(0.5) * a.x;
    t.y = x0.y - T(0.5) * a.y;
    u.x = h * b.y;  // -i sqrt(3)/2 (x1 - x2)
    u.y = -(h * b.x);
    s[n] = cadd(x0, a);
    s[n + M] = cmul(cadd(t, u), tw3[n * tws3]);
    s[n + 2 * M] = cmul(csub(t, u), tw3[2 * n * tws3]);
  }
  __syncthreads();
}

template <class T2, class T>
__device__ __forceinline__ void r3_dit_stage(T2* s, int M, const T2* __restrict__ tw3, int tws3) {
  const T h = T(0.86602540378443864676);
  for (int n = threadIdx.x; n < M; n += blockDim.x) {
    T2 w1 = tw3[n * tws3], w2 = tw3[2 * n * tws3];
    w1.y = -w1.y;
    w2.y = -w2.y;
    const T2 z0 = s[n], t1 = cmul(s[n + M], w1), t2 = cmul(s[n + 2 * M], w2);
    const T2 a = cadd(t1, t2), b = csub(t1, t2);
    T2 t, v;
    t.x = z0.x - T(0.5) * a.x;
    t.y = z0.y - T(0.5) * a.y;
    v.x = -(h * b.y);  // +i sqrt(3)/2 (t1 - t2)
    v.y = h * b.x;
    s[n] = cadd(z0, a);
    s[n + M] = cadd(t, v);
    s[n + 2 * M] = csub(t, v);
  }
  __syncthreads();
}

// This lane's twiddle for each register stage k (span 2^k): W_(2^k)^(lane
// mod 2^(k-1)) in the upper lane of each butterfly (lane bit k-1 set), 1 in
// the lower lane, so both lanes run the same instructions (below).
template <class T2>
__device__ __forceinline__ void lane_twiddles(int lane, int small, const T2* __restrict__ tw, T2 (&w)[5]) {
#pragma unroll
  for (int k = 1; k <= 5; ++k) {
    w[k - 1].x = 1;
    w[k - 1].y = 0;
    if (k <= small && (lane & (1 << (k - 1)))) w[k - 1] = twid(tw, 1 << k, lane & ((1 << (k - 1)) - 1));
  }
}

// +1 in the lower lane of a span-2^k butterfly, -1 in the upper one.
template <class T>
__device__ __forceinline__ T lane_sign(int lane, int k) {
  return (lane & (1 << (k - 1))) ? T(-1) : T(1);
}

// s x + o for both parts (one rounding each).
__device__ __forceinline__ float2 sfma2(float s, float2 x, float2 o) {
  float2 r;
  r.x = __fmaf_rn(s, x.x, o.x);
  r.y = __fmaf_rn(s, x.y, o.y);
  return r;
}
__device__ __forceinline__ double2 sfma2(double s, double2 x, double2 o) {
  double2 r;
  r.x = __fma_rn(s, x.x, o.x);
  r.y = __fma_rn(s, x.y, o.y);
  return r;
}

// DIF spans 2^small .. 2 on one element per lane (w from lane_twiddles). The
// lower lane of a butterfly keeps x + o, the upper one (o - x) w: both compute
// (o + s x) w with s = +-1 and w = 1 in the lower lane, without a branch.
template <class T2>
__device__ __forceinline__ T2 dif_reg_stages(T2 x, int lane, int small, const T2 (&w)[5]) {
  typedef decltype(x.x) T;
#pragma unroll
  for (int k = 5; k >= 1; --k) {
    if (k > small) continue;
    const T2 o = shfl_xor2(x, 1 << (k - 1));
    x = cmul(sfma2(lane_sign<T>(lane, k), x, o), w[k - 1]);
  }
  return x;
}

// DIT spans 2 .. 2^small on one element per lane (w from lane_twiddles, used
// conjugated): the upper lane sends t = x conj(w) and keeps o - t, the lower
// sends t = x and keeps x + o; both compute t = x conj(w), then o + s t.
template <class T2>
__device__ __forceinline__ T2 dit_reg_stages(T2 x, int lane, int small, const T2 (&w)[5]) {
  typedef decltype(x.x) T;
#pragma unroll
  for (int k = 1; k <= 5; ++k) {
    if (k > small) continue;
    T2 wc = w[k - 1];
    wc.y = -wc.y;
    const T2 t = cmul(x, wc);
    const T2 o = shfl_xor2(t, 1 << (k - 1));
    x = sfma2(lane_sign<T>(lane, k), t, o);
  }
  return x;
}

// Source of a row entering a transform: 0 -> data (one bulk copy); 1 -> row
// `row` of the squared Cauchy kernel over signed lags, computed in place (the
// arithmetic of the reference's kernel build, src/tsne/interpolation.rs:198-
// 226); 2 -> a charge row of data: its first `nodes` entries by bulk copy,
// zeros after them. False when a bulk copy timed out.
template <class T>
__device__ __forceinline__ bool fft_fill_row(typename Cx<T>::type* s, const typename Cx<T>::type* d, int src, int row,
                                             int L, int D, const FitParams<T>* __restrict__ prm, uint64_t* bar,
                                             int* fault) {
  typedef typename Cx<T>::type T2;
  if (src == 0) return fft_load_row(s, d, (uint32_t)(L * sizeof(T2)), bar, fault);
  if (src == 1) {
    const T spacing = prm->spacing;
    const int lr = row <= L / 2 ? row : row - L;
    const T dr = spacing * (T)lr;
    for (int c = threadIdx.x; c < L; c += blockDim.x) {
      const int lc = c <= L / 2 ? c : c - L;
      const T dc = spacing * (T)lc;
      T sq = T(0);
      sq = sq + dc * dc;
      if (D == 2) sq = sq + dr * dr;
      const T cauchy = T(1) / (T(1) + sq);
      T2 v;
      v.x = cauchy * cauchy;
      v.y = T(0);
      s[c] = v;
    }
  } else {
    // the first `nodes` entries (rounded up to 16 bytes), zeros after them
    const int nodes = prm->nodes;
    const uint32_t bytes = ((uint32_t)(nodes * sizeof(T2)) + 15u) & ~15u;
    if (!fft_load_row(s, d, bytes, bar, fault)) return false;
    for (int c = nodes + (int)threadIdx.x; c < L; c += blockDim.x) {
      T2 v;
      v.x = T(0);
      v.y = T(0);
      s[c] = v;
    }
  }
  __syncthreads();
  return true;
}

// Wide register phase (sub-rows of M >= 128): each lane holds the four
// elements 32 k + lane (k = 0..3) of a group of 128, so the stages of spans
// 128 and 64 are butterflies inside the lane and spans <= 32 are shuffles.
// w128 = W_128^lane and w64 = W_64^lane; W_128^(32 + lane) = w128 * (-i).
template <class T2>
__device__ __forceinline__ void dif_wide_stages(T2 (&x)[4], int lane, const T2 (&w)[5], T2 w64, T2 w128) {
  T2 w128b;
  w128b.x = w128.y;
  w128b.y = -w128.x;
  const T2 a = cadd(x[0], x[2]), b = cmul(csub(x[0], x[2]), w128);
  const T2 c = cadd(x[1], x[3]), d = cmul(csub(x[1], x[3]), w128b);
  x[0] = cadd(a, c);
  x[1] = cmul(csub(a, c), w64);
  x[2] = cadd(b, d);
  x[3] = cmul(csub(b, d), w64);
#pragma unroll
  for (int k = 0; k < 4; ++k) x[k] = dif_reg_stages(x[k], lane, 5, w);
}

template <class T2>
__device__ __forceinline__ void dit_wide_stages(T2 (&x)[4], int lane, const T2 (&w)[5], T2 w64, T2 w128) {
#pragma unroll
  for (int k = 0; k < 4; ++k) x[k] = dit_reg_stages(x[k], lane, 5, w);
  T2 c64 = w64, c128 = w128, c128b;
  c64.y = -c64.y;
  c128.y = -c128.y;
  c128b.x = -c128.y;  // conj(W_128^(32 + lane)) = conj(w128) * (+i)
  c128b.y = c128.x;
  T2 t = cmul(x[1], c64);
  x[1] = csub(x[0], t);
  x[0] = cadd(x[0], t);
  t = cmul(x[3], c64);
  x[3] = csub(x[2], t);
  x[2] = cadd(x[2], t);
  t = cmul(x[2], c128);
  x[2] = csub(x[0], t);
  x[0] = cadd(x[0], t);
  t = cmul(x[3], c128b);
  x[3] = csub(x[1], t);
  x[1] = cadd(x[1], t);
}

constexpr int kFftThreads = 512;

// Row geometry: L = nsub * M with M a power of two and nsub 1 or 3.
template <class T>
struct FftRow {
  typedef typename Cx<T>::type T2;
  int L, M, nsub, log2M, small, G, ngroups, tws3, lane, warp, nw;
  bool lane_ok, wide;
  __device__ FftRow(int L_, int cap_L) : L(L_) {
    nsub = (L % 3 == 0) ? 3 : 1;
    M = L / nsub;
    log2M = 0;
    while ((1 << log2M) < M) ++log2M;
    wide = log2M >= 7;  // groups of 128: stages of span <= 128 in registers
    small = wide ? 7 : (log2M < 5 ? log2M : 5);
    G = 1 << small;
    ngroups = L >> small;
    tws3 = nsub == 3 ? (3 * (cap_L >> 2)) / L : 0;
    lane = threadIdx.x & 31;
    warp = threadIdx.x >> 5;
    nw = blockDim.x >> 5;
    lane_ok = wide || lane < G;
  }
  // The frequency a forward transform leaves at position p, and the position
  // of frequency f: sub-row k of a 3 M row holds frequencies 3 m + k at the
  // bit-reversed positions of m; a power-of-two row is bit-reversed.
  __device__ int freq_at(int p) const {
    const int k = nsub == 3 ? p / M : 0;
    const int m = (int)(__brev((unsigned)(p - k * M)) >> (32 - log2M));
    return nsub == 3 ? 3 * m + k : m;
  }
  __device__ int pos_of(int f) const {
    const int k = nsub == 3 ? f % 3 : 0;
    const int m = nsub == 3 ? f / 3 : f;
    return k * M + (int)(__brev((unsigned)m) >> (32 - log2M));
  }
  // W_128^lane, W_64^lane of the sub-row length (wide mode)
  __device__ void wide_twiddles(const T2* __restrict__ tw, T2* w64, T2* w128) const {
    *w64 = twid(tw, 64, lane);
    *w128 = twid(tw, 128, lane);
  }
};

// Rows of length L (from the parameters), row b at data + b L; rows: 0 -> L
// rows, 1 -> `nodes` rows, 2 -> one row. The row arrives in shared memory by
// one bulk copy.
template <class T>
__global__ void __launch_bounds__(kFftThreads, sizeof(T) == 4 ? 3 : 1) fft_rows_kernel(typename Cx<T>::type* __restrict__ data,
                                                              const FitParams<T>* __restrict__ prm, int rows_sel,
                                                              const typename Cx<T>::type* __restrict__ tw,
                                                              const typename Cx<T>::type* __restrict__ tw3, int cap_L,
                                                              int inverse, int* __restrict__ fault, int src,
                                                              T* __restrict__ khat_out) {
  typedef typename Cx<T>::type T2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint64_t load_bar;
  const int L = prm->L;
  const int rows = rows_sel == 0 ? L : (rows_sel == 1 ? prm->nodes : 1);
  if ((int)blockIdx.x >= rows) return;
  const FftRow<T> r(L, cap_L);
  T2* s = reinterpret_cast<T2*>(smem_raw);
  T2* d = data + (int64_t)blockIdx.x * L;
  T2 w[5];
  lane_twiddles(r.lane, r.wide ? 5 : r.small, tw, w);
  T2 w64, w128;
  if (r.wide) r.wide_twiddles(tw, &w64, &w128);
  T2 zero;
  zero.x = T(0);
  zero.y = T(0);
  const int D = rows_sel == 2 ? 1 : 2;
  if (!fft_fill_row<T>(s, d, inverse ? 0 : src, (int)blockIdx.x, L, D, prm, &load_bar, fault)) return;
  if (!inverse) {
    if (r.nsub == 3) r3_dif_stage<T2, T>(s, r.M, tw3, r.tws3);
    dif_smem_stages(s, r.M, r.log2M, r.small, tw, r.nsub);
    // khat_out: the real part scaled by 1 / L^D (the kernel spectrum)
    // (L^D < 2^31 is exact as an int, so no FP64 conversion is needed)
    const T inv_total = khat_out ? T(1) / (T)(D == 1 ? L : L * L) : T(0);
    T* kr = khat_out ? khat_out + (int64_t)blockIdx.x * L : nullptr;
    for (int g = r.warp; g < r.ngroups; g += r.nw) {
      if (r.wide) {
        T2 x[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = s[g * 128 + 32 * k + r.lane];
        dif_wide_stages(x, r.lane, w, w64, w128);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int e = g * 128 + 32 * k + r.lane;
          if (kr) kr[e] = x[k].x * inv_total;
          else d[e] = x[k];
        }
        continue;
      }
      const T2 x = dif_reg_stages(r.lane_ok ? s[g * r.G + r.lane] : zero, r.lane, r.small, w);
      if (r.lane_ok) {
        if (kr) kr[g * r.G + r.lane] = x.x * inv_total;
        else d[g * r.G + r.lane] = x;
      }
    }
    return;
  }
  for (int g = r.warp; g < r.ngroups; g += r.nw) {
    if (r.wide) {
      T2 x[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) x[k] = s[g * 128 + 32 * k + r.lane];
      dit_wide_stages(x, r.lane, w, w64, w128);
#pragma unroll
      for (int k = 0; k < 4; ++k) s[g * 128 + 32 * k + r.lane] = x[k];
      continue;
    }
    const T2 x = dit_reg_stages(r.lane_ok ? s[g * r.G + r.lane] : zero, r.lane, r.small, w);
    if (r.lane_ok) s[g * r.G + r.lane] = x;
  }
  __syncthreads();
  dit_smem_stages(s, r.M, r.log2M, r.small, tw, r.nsub);
  if (r.nsub == 3) r3_dit_stage<T2, T>(s, r.M, tw3, r.tws3);
  // the potentials of the node rows: only their first `nodes` columns are read
  const int keep = rows_sel == 1 ? prm->nodes : L;
  for (int i = threadIdx.x; i < keep; i += blockDim.x) d[i] = s[i];
}

// The kernel spectrum in 2-D from real transforms packed two to a complex
// one. The kernel K(i, j) = (1 + spacing^2 (lag(i)^2 + lag(j)^2))^-2 is real
// and even in both indices, so every transform of its rows (and then of its
// columns) is real: rows a and b packed as a + i b transform to A + i B with
// A and B the two real transforms. Only rows 0 .. L/2 are distinct (row L - r
// equals row r).
//  pass 0: block b transforms kernel rows 2b and 2b + 1 (<= L/2) and writes
//          the two real rows of `out` (row stride L);
//  pass 1: block b takes the rows of the transposed table `in` (row p holds
//          column p for rows 0 .. L/2, stride L) at the positions of the
//          frequencies 2b and 2b + 1 (<= L/2), extends each evenly to length L,
//          transforms the pair and writes those rows of the spectrum times
//          `scale` (1 / L^2). Rows of frequencies above L/2 equal the rows of
//          L minus them and are not written: the convolution pass reads the
//          mirrored row (kspec_row).
// The spectrum is symmetric, so its rows and columns need no distinction.
template <class T>
__global__ void __launch_bounds__(kFftThreads, sizeof(T) == 4 ? 3 : 1) kspec_kernel(int pass, const FitParams<T>* __restrict__ prm,
                                                           const typename Cx<T>::type* __restrict__ tw,
                                                           const typename Cx<T>::type* __restrict__ tw3, int cap_L,
                                                           const T* __restrict__ in, T* __restrict__ out) {
  typedef typename Cx<T>::type T2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = prm->L, half = L / 2;
  const int b = (int)blockIdx.x;
  const FftRow<T> r(L, cap_L);
  // pass 0: kernel rows (lags); pass 1: table rows at the frequencies' positions
  const int f1 = 2 * b, f2 = 2 * b + 1;
  if (f1 > half) return;
  const bool two = f2 <= half;
  const int r1 = pass == 0 ? f1 : r.pos_of(f1);
  const int r2 = pass == 0 ? f2 : (two ? r.pos_of(f2) : r1);
  T2* s = reinterpret_cast<T2*>(smem_raw);
  T2 w[5];
  lane_twiddles(r.lane, r.wide ? 5 : r.small, tw, w);
  T2 w64, w128;
  if (r.wide) r.wide_twiddles(tw, &w64, &w128);
  T2 zero;
  zero.x = T(0);
  zero.y = T(0);
  if (pass == 0) {
    const T spacing = prm->spacing;
    const int l1 = r1 <= half ? r1 : r1 - L, l2 = r2 <= half ? r2 : r2 - L;
    const T d1 = spacing * (T)l1, d2 = spacing * (T)l2;
    for (int c = threadIdx.x; c < L; c += blockDim.x) {
      const int lc = c <= half ? c : c - L;
      const T dc = spacing * (T)lc;  // |lc| <= L/2: exact in T
      T sq1 = T(0), sq2 = T(0);
      sq1 = sq1 + dc * dc;
      sq1 = sq1 + d1 * d1;
      sq2 = sq2 + dc * dc;
      sq2 = sq2 + d2 * d2;
      const T c1 = T(1) / (T(1) + sq1), c2 = T(1) / (T(1) + sq2);
      T2 v;
      v.x = c1 * c1;
      v.y = two ? c2 * c2 : T(0);
      s[c] = v;
    }
  } else {
    const T* a = in + (int64_t)r1 * L;
    const T* c = in + (int64_t)r2 * L;  // r1 again when there is one row
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
      const int e = i <= half ? i : L - i;
      T2 v;
      v.x = a[e];
      v.y = c[e];
      s[i] = v;
    }
  }
  __syncthreads();
  if (r.nsub == 3) r3_dif_stage<T2, T>(s, r.M, tw3, r.tws3);
  dif_smem_stages(s, r.M, r.log2M, r.small, tw, r.nsub);
  const T scale = pass == 0 ? T(1) : T(1) / (T)(L * L);
  T* o1 = out + (int64_t)r1 * L;
  T* o2 = out + (int64_t)r2 * L;
  for (int g = r.warp; g < r.ngroups; g += r.nw) {
    if (r.wide) {
      T2 x[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) x[k] = s[g * 128 + 32 * k + r.lane];
      dif_wide_stages(x, r.lane, w, w64, w128);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int e = g * 128 + 32 * k + r.lane;
        o1[e] = x[k].x * scale;
        if (two) o2[e] = x[k].y * scale;
      }
      continue;
    }
    const T2 x = dif_reg_stages(r.lane_ok ? s[g * r.G + r.lane] : zero, r.lane, r.small, w);
    if (r.lane_ok) {
      o1[g * r.G + r.lane] = x.x * scale;
      if (two) o2[g * r.G + r.lane] = x.y * scale;
    }
  }
}

// out[c][r] = in[r][c] for the real table of pass 0 above: rows r <= L/2,
// columns c < L, row stride L in and out.
template <class T>
__global__ void transpose_half_kernel(const T* __restrict__ in, const FitParams<T>* __restrict__ prm,
                                      T* __restrict__ out) {
  __shared__ T tile[32][33];
  const int L = prm->L, rows = L / 2 + 1;
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  if (c0 >= L || r0 >= rows) return;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    tile[k][threadIdx.x] = (r < rows && c < L) ? in[(int64_t)r * L + c] : T(0);
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (c < L && r < rows) out[(int64_t)c * L + r] = tile[threadIdx.x][k];
  }
}

// Convolution of rows with the kernel spectrum: forward transform, product
// with the real spectrum row (khat, bit-reversed like the row), inverse
// transform, in one pass over each row. The forward transform's last stages
// and the inverse's first stages act on the same positions in registers, so
// the product sits between them without a shared-memory round trip. Only the
// first `nodes` entries of each output row are stored (all that is read
// afterwards). rows_sel: 0 -> L rows (2-D, second axis), 2 -> one row (1-D).
template <class T>
__global__ void __launch_bounds__(kFftThreads, sizeof(T) == 4 ? 3 : 1) fft_conv_rows_kernel(typename Cx<T>::type* __restrict__ data,
                                                                   const T* __restrict__ khat,
                                                                   const FitParams<T>* __restrict__ prm, int rows_sel,
                                                                   const typename Cx<T>::type* __restrict__ tw,
                                                                   const typename Cx<T>::type* __restrict__ tw3,
                                                                   int cap_L, int* __restrict__ fault, int src) {
  typedef typename Cx<T>::type T2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint64_t load_bar;
  const int L = prm->L;
  const int rows = rows_sel == 0 ? L : 1;
  if ((int)blockIdx.x >= rows) return;
  const int keep = prm->nodes;
  const FftRow<T> r(L, cap_L);
  T2* s = reinterpret_cast<T2*>(smem_raw);
  T2* d = data + (int64_t)blockIdx.x * L;
  // the spectrum row of this row's frequency (2-D: rows of frequencies above
  // L/2 are the rows of L minus them, see kspec_kernel)
  int krow = (int)blockIdx.x;
  if (rows_sel == 0) {
    const int f = r.freq_at(krow);
    if (f > L / 2) krow = r.pos_of(L - f);
  }
  const T* kr = khat + (int64_t)krow * L;
  T2 w[5];
  lane_twiddles(r.lane, r.wide ? 5 : r.small, tw, w);
  T2 w64, w128;
  if (r.wide) r.wide_twiddles(tw, &w64, &w128);
  T2 zero;
  zero.x = T(0);
  zero.y = T(0);
  if (!fft_fill_row<T>(s, d, src, (int)blockIdx.x, L, rows_sel == 2 ? 1 : 2, prm, &load_bar, fault)) return;
  if (r.nsub == 3) r3_dif_stage<T2, T>(s, r.M, tw3, r.tws3);
  dif_smem_stages(s, r.M, r.log2M, r.small, tw, r.nsub);
  for (int g = r.warp; g < r.ngroups; g += r.nw) {
    if (r.wide) {
      T2 x[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) x[k] = s[g * 128 + 32 * k + r.lane];
      dif_wide_stages(x, r.lane, w, w64, w128);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const T kv = kr[g * 128 + 32 * k + r.lane];
        x[k].x *= kv;
        x[k].y *= kv;
      }
      dit_wide_stages(x, r.lane, w, w64, w128);
#pragma unroll
      for (int k = 0; k < 4; ++k) s[g * 128 + 32 * k + r.lane] = x[k];
      continue;
    }
    const int e = g * r.G + r.lane;
    T2 x = dif_reg_stages(r.lane_ok ? s[e] : zero, r.lane, r.small, w);
    const T k = r.lane_ok ? kr[e] : T(0);
    x.x *= k;
    x.y *= k;
    x = dit_reg_stages(x, r.lane, r.small, w);
    if (r.lane_ok) s[e] = x;
  }
  __syncthreads();
  dit_smem_stages(s, r.M, r.log2M, r.small, tw, r.nsub);
  if (r.nsub == 3) r3_dit_stage<T2, T>(s, r.M, tw3, r.tws3);
  for (int i = threadIdx.x; i < keep; i += blockDim.x) d[i] = s[i];
}

// out[c][r] = in[r][c] for r < rows_in (zero for rows_in <= r < out_cols),
// c < cols; rows of length L in and out. Sizes from the parameters: sel 0 ->
// L, 1 -> nodes (out_sel 1: output rows end at column nodes, for a consumer
// that fills the rest with zeros itself). Blocks past the current sizes exit.
template <class T>
__global__ void transpose_kernel(const typename Cx<T>::type* __restrict__ in, const FitParams<T>* __restrict__ prm,
                                 int rows_sel, int cols_sel, int out_sel, typename Cx<T>::type* __restrict__ out) {
  typedef typename Cx<T>::type T2;
  __shared__ T2 tile[32][33];
  const int L = prm->L;
  const int rows_in = rows_sel == 0 ? L : prm->nodes;
  const int cols = cols_sel == 0 ? L : prm->nodes;
  const int out_cols = out_sel == 0 ? L : prm->nodes;
  const int64_t ld_in = L, ld_out = L;
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  if (c0 >= cols || r0 >= out_cols) return;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    T2 v;
    v.x = T(0);
    v.y = T(0);
    if (r < rows_in && c < cols) v = in[(int64_t)r * ld_in + c];
    tile[k][threadIdx.x] = v;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (c < cols && r < out_cols) out[(int64_t)c * ld_out + r] = tile[threadIdx.x][k];
  }
}

// phi64 (1-D): the node potentials in FP64, potential k at phi64[k stride +
// node], interpolated in FP64 (the forces rounded to T once); otherwise the
// potentials of the packed complex grids g0, g1 in T.
template <class T, int D>
__global__ void gather_kernel(const T* __restrict__ y, int64_t n, const FitParams<T>* __restrict__ prm,
                              const typename Cx<T>::type* __restrict__ g0, const typename Cx<T>::type* __restrict__ g1,
                              const double* __restrict__ phi64, int phi_stride, T* __restrict__ neg,
                              double* __restrict__ zpart, unsigned* __restrict__ done, double* __restrict__ z_out) {
  __shared__ double sh[32];
  __shared__ bool last;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double zi = 0.0;
  if (i < n) {
    const FitParams<T> p = *prm;
    const Lagrange3<T> lb;
    const int L = p.L;
    int box[D];
    T w[D][3];
    T yv[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      yv[a] = y[i * D + a];
      locate<T>(yv[a], p, lb, &box[a], w[a]);
    }
    constexpr int combos = D == 1 ? 3 : 9;
    bool in_fp64 = false;
    if constexpr (D == 1) {
      if (phi64 != nullptr) {
        double pd[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int64_t node = (int64_t)box[0] * 3 + c;
          const double wt = (double)w[0][c];
#pragma unroll
          for (int t = 0; t < 3; ++t) pd[t] += wt * phi64[(int64_t)t * phi_stride + node];
        }
        const double dens = pd[0] / (double)p.scale;
        const double sqp = pd[2] * (double)p.scale;
        const double yd = (double)yv[0];
        neg[i] = (T)(yd * dens - pd[1]);
        zi = (1.0 + yd * yd) * dens - 2.0 * yd * pd[1] + sqp;
        in_fp64 = true;
      }
    }
    if (!in_fp64) {
      T phi[D + 2];
#pragma unroll
      for (int t = 0; t < D + 2; ++t) phi[t] = T(0);
#pragma unroll
      for (int c = 0; c < combos; ++c) {
        int rem = c;
        int64_t flat = 0;
        T wt = T(1);
#pragma unroll
        for (int a = 0; a < D; ++a) {
          const int k = rem % 3;
          rem /= 3;
          flat = flat * L + (box[a] * 3 + k);
          wt = wt * w[a][k];
        }
        const typename Cx<T>::type a0 = g0[flat], a1 = g1[flat];
        phi[0] = phi[0] + wt * a0.x;
        phi[1] = phi[1] + wt * a0.y;
        phi[2] = phi[2] + wt * a1.x;
        if (D == 2) phi[3] = phi[3] + wt * a1.y;
      }
      phi[0] = phi[0] / p.scale;
      phi[D + 1] = phi[D + 1] * p.scale;
      const T density = phi[0];
      const T sqp = phi[D + 1];
      // Z's per-point term cancels terms of order |y|^2 phi_0; it is assembled
      // in FP64 from the interpolated potentials (the forces stay in T).
      double norm_sq = 0.0, cross = 0.0;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const T fm = phi[1 + a];
        neg[i * D + a] = yv[a] * density - fm;
        norm_sq += (double)yv[a] * (double)yv[a];
        cross += (double)yv[a] * (double)fm;
      }
      zi = (1.0 + norm_sq) * (double)density - 2.0 * cross + (double)sqp;
    }
  }
  const double bs = block_sum(zi, sh);
  if (threadIdx.x == 0) {
    zpart[blockIdx.x] = bs;
    __threadfence();
    last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    const double z = block_sum_parts(zpart, gridDim.x, 1, 0, sh);
    if (threadIdx.x == 0) {
      *z_out = z - (double)n;
      *done = 0;
    }
  }
}


}  // namespace

// W_cap3^k for k < cap3 = 3 cap_L / 4 (the full circle): the radix-3 stage of
// any length 3 * 2^j <= cap3.
template <class T>
const typename FitWorkspace<T>::T2* FitWorkspace<T>::twiddles3(int cap_L, cudaStream_t s) {
  const int c3 = 3 * (cap_L / 4);
  if (tw3_len != c3) {
    std::vector<T2> h(c3 > 0 ? c3 : 1);
    for (int k = 0; k < c3; ++k) {
      const double ang = -2.0 * M_PI * (double)k / (double)c3;
      h[k].x = (T)std::cos(ang);
      h[k].y = (T)std::sin(ang);
    }
    tw3.ensure(h.size() * sizeof(T2));
    BHG_CUDA(cudaMemcpyAsync(tw3.ptr, h.data(), h.size() * sizeof(T2), cudaMemcpyHostToDevice, s));
    tw3_len = c3;
  }
  return tw3.template as<T2>();
}

template <class T>
const typename FitWorkspace<T>::T2* FitWorkspace<T>::twiddles(int L, cudaStream_t s) {
  if (tw_len != L) {
    // W_S^k = exp(-2 pi i k / S) at S / 2 - 1 + k, for S = 2 .. L
    std::vector<T2> h(L > 1 ? L - 1 : 1);
    for (int S = 2; S <= L; S <<= 1)
      for (int k = 0; k < S / 2; ++k) {
        const double ang = -2.0 * M_PI * (double)k / (double)S;
        h[S / 2 - 1 + k].x = (T)std::cos(ang);
        h[S / 2 - 1 + k].y = (T)std::sin(ang);
      }
    tw.ensure(h.size() * sizeof(T2));
    // on the stream of the FFTs that read it (the legacy stream would not
    // order against a non-blocking one); the pageable source is staged
    // before the call returns
    BHG_CUDA(cudaMemcpyAsync(tw.ptr, h.data(), h.size() * sizeof(T2), cudaMemcpyHostToDevice, s));
    tw_len = L;
  }
  return tw.template as<T2>();
}

// src: 0 -> rows of `data`, 1 -> Cauchy kernel rows, 2 -> charge rows of
// `data` (entries past `nodes` are zero); khat_out: write the scaled real part
// there instead of the complex result (forward only).
template <class T>
static void fft_rows(FitWorkspace<T>& ws, typename Cx<T>::type* data, const FitParams<T>* dp, int rows_sel, int cap_L,
                     bool inverse, cudaStream_t s, int src = 0, T* khat_out = nullptr) {
  const int threads = std::min(kFftThreads, std::max(32, cap_L / 4));
  const size_t smem = (size_t)cap_L * sizeof(typename Cx<T>::type);
  const int grid = rows_sel == 2 ? 1 : cap_L;
  fft_rows_kernel<T><<<grid, threads, smem, s>>>(data, dp, rows_sel, ws.twiddles(cap_L, s), ws.twiddles3(cap_L, s),
                                                  cap_L, inverse ? 1 : 0,
                                                  ws.flag.template as<int>() + 1, src, khat_out);
  BHG_LAUNCH_CHECK();
}

template <class T>
static void fft_conv_rows(FitWorkspace<T>& ws, typename Cx<T>::type* data, const T* khat, const FitParams<T>* dp,
                          int rows_sel, int cap_L, cudaStream_t s, int src = 0) {
  const int threads = std::min(kFftThreads, std::max(32, cap_L / 4));
  const size_t smem = (size_t)cap_L * sizeof(typename Cx<T>::type);
  const int grid = rows_sel == 2 ? 1 : cap_L;
  fft_conv_rows_kernel<T><<<grid, threads, smem, s>>>(data, khat, dp, rows_sel, ws.twiddles(cap_L, s),
                                                       ws.twiddles3(cap_L, s), cap_L,
                                                       ws.flag.template as<int>() + 1, src);
  BHG_LAUNCH_CHECK();
}

template <class T>
static void transpose(const typename Cx<T>::type* in, const FitParams<T>* dp, int rows_sel, int cols_sel,
                      typename Cx<T>::type* out, int cap_L, cudaStream_t s, int out_sel = 0) {
  dim3 b(32, 8);
  dim3 g((unsigned)ceil_div(cap_L, 32), (unsigned)ceil_div(cap_L, 32));
  transpose_kernel<T><<<g, b, 0, s>>>(in, dp, rows_sel, cols_sel, out_sel, out);
  BHG_LAUNCH_CHECK();
}

template <class T>
void FitWorkspace<T>::reserve(int D, int64_t n, int cap) {
  if (cap < 16 || (cap & (cap - 1)) != 0) throw Error(ST_EINTERNAL, "error: FIt-SNE capacity must be a power of two.");
  typedef typename Cx<T>::type C2;
  const int64_t total = D == 1 ? (int64_t)cap : (int64_t)cap * cap;
  params.ensure(sizeof(FitParams<T>));
  g0.ensure(total * sizeof(C2));
  g1.ensure(total * sizeof(C2));
  h0.ensure(total * sizeof(C2));
  h1.ensure(total * sizeof(C2));
  khat.ensure(total * sizeof(T));
  // the spread reaches rows < nodes <= cap / 2 of an L <= cap grid
  const int64_t cells = D == 1 ? (int64_t)cap : (int64_t)(cap / 2 + 1) * cap;
  const size_t acc_before = acc.bytes;
  acc.ensure((size_t)cells * 4 * sizeof(long long));
  if (acc.bytes != acc_before) acc_clean = nullptr;  // new memory: cleared before its first spread
  zpart.ensure((ceil_div(std::max<int64_t>(n, 1), 256) + 1) * sizeof(double));
  if (D == 1) direct.ensure((size_t)7 * cap * sizeof(double));
  flag.ensure(64);
  done.ensure(64);
  if ((size_t)cap * sizeof(C2) >= 40 * 1024) {  // set outside any stream capture
    BHG_CUDA(cudaFuncSetAttribute(fft_rows_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    BHG_CUDA(cudaFuncSetAttribute(fft_conv_rows_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    BHG_CUDA(cudaFuncSetAttribute(kspec_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  }
  cap_L = cap;
}

template <class T>
int fit_needed_length(FitWorkspace<T>& ws, int D, int64_t n, const BoxParams<T>* box, cudaStream_t s) {
  ws.params.ensure(sizeof(FitParams<T>));
  FitParams<T>* dp = ws.params.template as<FitParams<T>>();
  if (D == 1) fit_params_kernel<T, 1><<<1, 32, 0, s>>>(box, n, dp, 0, nullptr);
  else fit_params_kernel<T, 2><<<1, 32, 0, s>>>(box, n, dp, 0, nullptr);
  BHG_LAUNCH_CHECK();
  FitParams<T> hp;
  BHG_CUDA(cudaMemcpyAsync(&hp, dp, sizeof(hp), cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  return hp.L;
}

template <class T>
void fit_repulsion_cap(FitWorkspace<T>& ws, int D, const T* y, int64_t n, const BoxParams<T>* box, T* neg,
                       double* z_out, cudaStream_t s) {
  typedef typename Cx<T>::type T2;
  const int cap = ws.cap_L;
  FitParams<T>* dp = ws.params.template as<FitParams<T>>();
  if (D == 1) fit_params_kernel<T, 1><<<1, 32, 0, s>>>(box, n, dp, cap, ws.flag.template as<int>());
  else fit_params_kernel<T, 2><<<1, 32, 0, s>>>(box, n, dp, cap, ws.flag.template as<int>());
  BHG_LAUNCH_CHECK();
  T2* g0 = ws.g0.template as<T2>();
  T2* g1 = ws.g1.template as<T2>();
  T2* h0 = ws.h0.template as<T2>();
  T2* h1 = ws.h1.template as<T2>();
  T* khat = ws.khat.template as<T>();

  // kernel spectrum (real, pre-scaled by 1/L^2): the kernel rows are made in
  // the first transform and the last one writes the scaled real part. It is
  // symmetric in its axes, so it serves the transposed spectrum layout. (1-D:
  // the convolution is summed directly, conv1d_*.)
  if (D == 2) {
    // packed real transforms (kspec_kernel); g0 and h0 serve as real tables
    T* a = reinterpret_cast<T*>(g0);
    T* at = reinterpret_cast<T*>(h0);
    const int threads = std::min(kFftThreads, std::max(32, cap / 4));
    const size_t smem = (size_t)cap * sizeof(T2);
    kspec_kernel<T><<<(unsigned)(cap / 4 + 1), threads, smem, s>>>(0, dp, ws.twiddles(cap, s), ws.twiddles3(cap, s),
                                                                 cap, nullptr, a);
    BHG_LAUNCH_CHECK();
    dim3 tb(32, 8), tg((unsigned)ceil_div(cap, 32), (unsigned)ceil_div(cap / 2 + 1, 32));
    transpose_half_kernel<T><<<tg, tb, 0, s>>>(a, dp, at);
    BHG_LAUNCH_CHECK();
    kspec_kernel<T><<<(unsigned)(cap / 4 + 1), threads, smem, s>>>(1, dp, ws.twiddles(cap, s), ws.twiddles3(cap, s),
                                                                 cap, at, khat);
    BHG_LAUNCH_CHECK();
  }

  // charges: spread into the fixed-point accumulator; charges_kernel (2-D) or
  // conv1d_prep_kernel (1-D) converts, clear_cells_kernel clears the cells the
  // spread can reach (so the accumulator is zeroed here only when newly
  // allocated)
  long long* acc = ws.acc.template as<long long>();
  if (ws.acc_clean != ws.acc.ptr) {
    BHG_CUDA(cudaMemsetAsync(ws.acc.ptr, 0, ws.acc.bytes, s));
    ws.acc_clean = ws.acc.ptr;
  }
  if (n > 0) {
    if (D == 1) spread_kernel<T, 1><<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(y, n, dp, acc);
    else spread_kernel<T, 2><<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(y, n, dp, acc);
    BHG_LAUNCH_CHECK();
  }

  {
    // nodes <= cap / 2 (L <= cap, L >= 2 nodes - 1)
    const dim3 cg((unsigned)ceil_div(cap / 2, 256), D == 1 ? 1u : (unsigned)(cap / 2));
    if (D == 1) {
      conv1d_prep_kernel<T><<<cg, 256, 0, s>>>(acc, dp, cap, ws.direct.template as<double>());
      clear_cells_kernel<T, 1><<<cg, 256, 0, s>>>(acc, dp);
    } else {
      charges_kernel<T, 2><<<cg, 256, 0, s>>>(acc, dp, g0, g1);
      clear_cells_kernel<T, 2><<<cg, 256, 0, s>>>(acc, dp);
    }
  }
  BHG_LAUNCH_CHECK();

  T2 *r0, *r1;
  if (D == 1) {
    conv1d_direct_kernel<T><<<(unsigned)ceil_div((int64_t)(cap / 2) * 32, 256), 256, 0, s>>>(
        ws.direct.template as<double>(), dp, cap);
    BHG_LAUNCH_CHECK();
    r0 = g0;
    r1 = g1;
  } else {
    // forward: rows n0 < nodes, transpose to [k1][n0], rows over n0
    fft_rows<T>(ws, g0, dp, 1, cap, false, s, 2);
    fft_rows<T>(ws, g1, dp, 1, cap, false, s, 2);
    // (columns n0 >= nodes are zero: not written, filled in by the next pass)
    transpose<T>(g0, dp, 1, 0, h0, cap, s, 1);
    transpose<T>(g1, dp, 1, 0, h1, cap, s, 1);
    // product with the kernel spectrum and inverse over k0 (columns n0 <
    // nodes kept), transpose back, rows over k1
    fft_conv_rows<T>(ws, h0, khat, dp, 0, cap, s, 2);
    fft_conv_rows<T>(ws, h1, khat, dp, 0, cap, s, 2);
    transpose<T>(h0, dp, 0, 1, g0, cap, s);
    transpose<T>(h1, dp, 0, 1, g1, cap, s);
    fft_rows<T>(ws, g0, dp, 1, cap, true, s);
    fft_rows<T>(ws, g1, dp, 1, cap, true, s);
    r0 = g0;
    r1 = g1;
  }

  if (!ws.done_zeroed) {
    BHG_CUDA(cudaMemsetAsync(ws.done.ptr, 0, 64, s));
    ws.done_zeroed = true;
  }
  if (n > 0) {
    const unsigned g = (unsigned)ceil_div(n, 256);
    if (D == 1)
      gather_kernel<T, 1><<<g, 256, 0, s>>>(y, n, dp, r0, r1, ws.direct.template as<double>() + 4 * (int64_t)cap, cap,
                                            neg, ws.zpart.template as<double>(), ws.done.template as<unsigned>(),
                                            z_out);
    else
      gather_kernel<T, 2><<<g, 256, 0, s>>>(y, n, dp, r0, r1, nullptr, 0, neg, ws.zpart.template as<double>(),
                                            ws.done.template as<unsigned>(), z_out);
    BHG_LAUNCH_CHECK();
  } else {
    BHG_CUDA(cudaMemsetAsync(z_out, 0, sizeof(double), s));
  }
}

template <class T>
FitGrid fit_repulsion(FitWorkspace<T>& ws, int D, const T* y, int64_t n, const BoxParams<T>* box, T* neg, double* z_out,
                      cudaStream_t s) {
  const int L = fit_needed_length<T>(ws, D, n, box, s);
  int cap = 16;  // capacities are powers of two (the twiddle tables assume it)
  while (cap < L) cap <<= 1;
  ws.reserve(D, n, std::max(ws.cap_L, cap));
  BHG_CUDA(cudaMemsetAsync(ws.flag.template as<int>() + 1, 0, sizeof(int), s));
  fit_repulsion_cap<T>(ws, D, y, n, box, neg, z_out, s);
  FitParams<T> hp;
  int fault = 0;
  BHG_CUDA(cudaMemcpyAsync(&hp, ws.params.ptr, sizeof(hp), cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaMemcpyAsync(&fault, ws.flag.template as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  if (fault) throw Error(ST_ETIMEDOUT, "error: an FFT row load timed out.");
  FitGrid fg;
  fg.boxes = hp.boxes;
  fg.nodes = hp.nodes;
  fg.fft_len = hp.L;
  fg.lo = (double)hp.lo;
  fg.box_width = (double)hp.box_width;
  fg.spacing = (double)hp.spacing;
  return fg;
}

template struct FitWorkspace<float>;
template struct FitWorkspace<double>;
template FitGrid fit_repulsion<float>(FitWorkspace<float>&, int, const float*, int64_t, const BoxParams<float>*, float*,
                                      double*, cudaStream_t);
template FitGrid fit_repulsion<double>(FitWorkspace<double>&, int, const double*, int64_t, const BoxParams<double>*,
                                       double*, double*, cudaStream_t);
template void fit_repulsion_cap<float>(FitWorkspace<float>&, int, const float*, int64_t, const BoxParams<float>*,
                                       float*, double*, cudaStream_t);
template void fit_repulsion_cap<double>(FitWorkspace<double>&, int, const double*, int64_t, const BoxParams<double>*,
                                        double*, double*, cudaStream_t);
template int fit_needed_length<float>(FitWorkspace<float>&, int, int64_t, const BoxParams<float>*, cudaStream_t);
template int fit_needed_length<double>(FitWorkspace<double>&, int, int64_t, const BoxParams<double>*, cudaStream_t);

}  // namespace bhg
