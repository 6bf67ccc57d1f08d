// Shared device/host helpers for the bhtsne GB300 library.
//
// Every translation unit is compiled with -fmad=false so that, like the Rust
// reference (which never contracts a*b+c), each product and sum is rounded on
// its own; kernels that want a fused multiply-add ask for it explicitly.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace bhg {

// Status codes of the C ABI (errno-like values).
enum : int {
  ST_OK = 0,
  ST_ENOMEM = 12,
  ST_EINVAL = 22,
  ST_ETIMEDOUT = 110,
  ST_ECUDA = 1001,
  ST_EINTERNAL = 1002,
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void throw_cuda(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof buf, "CUDA error %s (%s) at %s:%d: %s", cudaGetErrorName(e), cudaGetErrorString(e),
           file, line, what);
  throw Error(e == cudaErrorMemoryAllocation ? ST_ENOMEM : ST_ECUDA, buf);
}

#define BHG_CUDA(call)                                                   \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) ::bhg::throw_cuda(e_, #call, __FILE__, __LINE__); \
  } while (0)

// Every kernel launch in the library is followed by this check, which also
// counts launches (bhtsne_launch_count).
extern std::atomic<long long> g_launches;
#define BHG_LAUNCH_CHECK()                                   \
  do {                                                       \
    ::bhg::g_launches.fetch_add(1, std::memory_order_relaxed); \
    BHG_CUDA(cudaGetLastError());                            \
  } while (0)

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// 1 / x rounded to nearest: the same value as the IEEE quotient T(1) / x.
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }

// Two single-precision values in one 64-bit register pair, for the paired
// f32x2 instructions of sm_100 and later: each lane of a paired add, subtract
// or multiply is the scalar IEEE operation rounded to nearest. A paired
// multiply whose result feeds a paired add can still be fused into one
// multiply-add by the assembler (measured: f += m * d accumulated with
// mul.rn.f32x2 / add.rn.f32x2 rounds like fma), so no such chain is written.
struct F32x2 {
  unsigned long long v;
};
__device__ __forceinline__ F32x2 f2_make(float a, float b) {
  F32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float f2_lo(F32x2 x) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
  (void)b;
  return a;
}
__device__ __forceinline__ float f2_hi(F32x2 x) {
  float a, b;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
  (void)a;
  return b;
}
__device__ __forceinline__ F32x2 f2_sub(F32x2 x, F32x2 y) {
  F32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(x.v), "l"(y.v));
  return r;
}
__device__ __forceinline__ F32x2 f2_mul(F32x2 x, F32x2 y) {
  F32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(x.v), "l"(y.v));
  return r;
}

// Conversions between f32 and int64 with round-to-nearest-even, written with
// 32/64-bit integer operations only (the hardware conversions of 64-bit
// integers are slow on this part). f32_to_i64_rn saturates like the IEEE
// conversion (NaN and -inf to INT64_MIN, +inf to INT64_MAX).
__host__ __device__ __forceinline__ uint32_t f32_bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  __builtin_memcpy(&b, &x, 4);
  return b;
#endif
}

__host__ __device__ __forceinline__ float f32_from_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  __builtin_memcpy(&x, &b, 4);
  return x;
#endif
}

__host__ __device__ __forceinline__ float i64_to_f32_rn(long long v) {
  const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  if (a == 0) return 0.0f;
#ifdef __CUDA_ARCH__
  const int e = 63 - __clzll((long long)a);  // position of the leading one
#else
  const int e = 63 - __builtin_clzll(a);
#endif
  unsigned long long m;
  uint32_t ex = (uint32_t)(e + 127);
  if (e <= 23) {
    m = a << (23 - e);
  } else {
    const int sh = e - 23;
    m = a >> sh;
    const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (m & 1))) ++m;
    if (m == (1ull << 24)) {  // rounded up to the next power of two
      m >>= 1;
      ++ex;
    }
  }
  return f32_from_bits((v < 0 ? 0x80000000u : 0u) | (ex << 23) | ((uint32_t)m & 0x7FFFFFu));
}

__host__ __device__ __forceinline__ long long f32_to_i64_rn(float x) {
  const uint32_t b = f32_bits(x);
  const uint32_t ex = (b >> 23) & 0xFFu;
  const bool neg = (b >> 31) != 0;
  if (ex < 126) return 0;  // |x| < 0.5
  if (ex >= 190) {         // |x| >= 2^63, inf, NaN
    const bool nan = ex == 255 && (b & 0x7FFFFFu) != 0;
    return (neg || nan) ? (long long)0x8000000000000000ull : 0x7FFFFFFFFFFFFFFFll;
  }
  const unsigned long long m = (b & 0x7FFFFFu) | 0x800000u;
  const int k = (int)ex - 150;  // x = m 2^k
  unsigned long long a;
  if (k >= 0) {
    a = m << k;
  } else {
    const int sh = -k;  // 1 .. 24
    a = m >> sh;
    const unsigned long long rem = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (a & 1))) ++a;
  }
  return neg ? (long long)(0ull - a) : (long long)a;
}

// Numeric limits usable on the device.
template <class T>
struct Lim;
template <>
struct Lim<float> {
  __host__ __device__ static constexpr float max() { return 3.40282347e+38f; }
  __host__ __device__ static constexpr float min_pos() { return 1.17549435e-38f; }
  __host__ __device__ static constexpr float eps() { return 1.1920929e-07f; }
};
template <>
struct Lim<double> {
  __host__ __device__ static constexpr double max() { return 1.7976931348623157e+308; }
  __host__ __device__ static constexpr double min_pos() { return 2.2250738585072014e-308; }
  __host__ __device__ static constexpr double eps() { return 2.220446049250313e-16; }
};

__device__ __forceinline__ float dexp(float x) { return expf(x); }
__device__ __forceinline__ double dexp(double x) { return exp(x); }
__device__ __forceinline__ float dlog(float x) { return logf(x); }
__device__ __forceinline__ double dlog(double x) { return log(x); }
__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }

template <class V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

template <class V>
__device__ __forceinline__ V warp_min(V v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

template <class V>
__device__ __forceinline__ V warp_max(V v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// Block-wide sum of a double, result valid in thread 0. `sh` holds >= 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    r = lane < nw ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;
}

// Block-wide reduction of `count` per-block partials part[b * stride + off],
// all threads of the calling block participating (call from every thread of
// a block-uniform branch). The order is fixed, so results are deterministic.
__device__ __forceinline__ double block_sum_parts(const double* part, unsigned count, unsigned stride, unsigned off,
                                                  double* sh) {
  double s = 0.0;
  for (unsigned b = threadIdx.x; b < count; b += blockDim.x) s += ((const volatile double*)part)[b * stride + off];
  return block_sum(s, sh);
}

template <class V>
__device__ __forceinline__ V block_min_parts(const V* part, unsigned count, unsigned stride, unsigned off, V init,
                                             V* sh) {
  V s = init;
  for (unsigned b = threadIdx.x; b < count; b += blockDim.x) s = fmin(s, ((const volatile V*)part)[b * stride + off]);
  s = warp_min(s);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = s;
  __syncthreads();
  V r = init;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)((blockDim.x + 31) >> 5); ++q) r = fmin(r, sh[q]);
  return r;
}

template <class V>
__device__ __forceinline__ V block_max_parts(const V* part, unsigned count, unsigned stride, unsigned off, V init,
                                             V* sh) {
  V s = init;
  for (unsigned b = threadIdx.x; b < count; b += blockDim.x) s = fmax(s, ((const volatile V*)part)[b * stride + off]);
  s = warp_max(s);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = s;
  __syncthreads();
  V r = init;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)((blockDim.x + 31) >> 5); ++q) r = fmax(r, sh[q]);
  return r;
}

// Rust `signum`: +1 for +0.0 and positives, -1 for -0.0 and negatives, NaN for NaN.
// Calls f(std::integral_constant<int, D>()) for a runtime D in [lo, hi]
// (lo >= 1, hi <= 7); throws EINVAL with msg otherwise.
template <int lo, int hi, class F>
inline void with_dim(int D, const char* msg, F&& f) {
  if (D < lo || D > hi) throw Error(ST_EINVAL, msg);
  switch (D) {
    case 1: if constexpr (lo <= 1 && 1 <= hi) f(std::integral_constant<int, 1>()); break;
    case 2: if constexpr (lo <= 2 && 2 <= hi) f(std::integral_constant<int, 2>()); break;
    case 3: if constexpr (lo <= 3 && 3 <= hi) f(std::integral_constant<int, 3>()); break;
    case 4: if constexpr (lo <= 4 && 4 <= hi) f(std::integral_constant<int, 4>()); break;
    case 5: if constexpr (lo <= 5 && 5 <= hi) f(std::integral_constant<int, 5>()); break;
    case 6: if constexpr (lo <= 6 && 6 <= hi) f(std::integral_constant<int, 6>()); break;
    case 7: if constexpr (lo <= 7 && 7 <= hi) f(std::integral_constant<int, 7>()); break;
    default: throw Error(ST_EINVAL, msg);
  }
}

template <class T>
__device__ __forceinline__ T signum(T x) {
  return isnan(x) ? x : copysign(T(1), x);
}

}  // namespace bhg
