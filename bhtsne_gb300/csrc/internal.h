// Host-side declarations shared between the translation units of the library.
// Everything here is internal; the public surface is include/bhtsne_gpu.h.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

namespace bhg {

// ---- device buffers ---------------------------------------------------------
// Stream that orders the DevBuf allocations and frees of the calling thread.
// The API entry points and the server's threads set it to the stream their
// work runs on; allocations then come from the device's stream-ordered pool
// (cudaMallocAsync / cudaFreeAsync), so freeing a buffer never waits for the
// rest of the device, as a plain cudaFree does. Without a scope, plain
// cudaMalloc / cudaFree.
extern thread_local cudaStream_t g_alloc_stream;

struct AllocStreamScope {
  cudaStream_t prev;
  explicit AllocStreamScope(cudaStream_t s) : prev(g_alloc_stream) { g_alloc_stream = s; }
  ~AllocStreamScope() { g_alloc_stream = prev; }
  AllocStreamScope(const AllocStreamScope&) = delete;
  AllocStreamScope& operator=(const AllocStreamScope&) = delete;
};

// A grow-only device allocation owned by a context or a fit workspace. A
// buffer allocated on a stream is freed on that stream (after its work), so
// it must be used on that stream, or on another one only after synchronising.
//
// A borrowed buffer is a view of memory owned elsewhere (a slice of a fixed
// scratch array): it is never freed, and a request for more than it holds
// throws BHTSNE_EINTERNAL instead of reallocating, so code running on borrowed
// buffers can never allocate.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  bool async = false;
  bool borrowed = false;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr && !borrowed) {
      if (async) cudaFreeAsync(ptr, stream);
      else cudaFree(ptr);
    }
    ptr = nullptr;
    bytes = 0;
    async = false;
    stream = nullptr;
    borrowed = false;
  }
  // Makes this buffer a view of `bytes` bytes at `p`, owned by the caller.
  void borrow(void* p, size_t b) {
    release();
    ptr = p;
    bytes = b;
    borrowed = true;
  }
  void* ensure(size_t want) {
    if (want <= bytes && ptr) return ptr;
    if (borrowed) throw Error(ST_EINTERNAL, "error: a fixed scratch buffer is smaller than this call needs.");
    release();
    size_t b = want < 256 ? 256 : want;
    if (g_alloc_stream) {
      BHG_CUDA(cudaMallocAsync(&ptr, b, g_alloc_stream));
      stream = g_alloc_stream;
      async = true;
    } else {
      BHG_CUDA(cudaMalloc(&ptr, b));
    }
    bytes = b;
    return ptr;
  }
  template <class V>
  V* as() const { return static_cast<V*>(ptr); }
  void swap(DevBuf& o) {
    std::swap(ptr, o.ptr);
    std::swap(bytes, o.bytes);
    std::swap(stream, o.stream);
    std::swap(async, o.async);
    std::swap(borrowed, o.borrowed);
  }
};

// Streaming multiprocessors of the current device, looked up once per device.
inline int device_sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

// A grid of per_sm blocks for every SM of the current device, at most cap
// (for grid-stride kernels and for reductions whose partials are sized by cap).
inline int sm_grid(int per_sm, int cap) {
  const int g = per_sm * device_sm_count();
  return g < cap ? g : cap;
}

// write_csv of a host embedding (io.cu); returns a status, the message in
// bhtsne_io_last_error.
int write_csv_file(const void* embedding, int64_t n, int32_t embed_dim, int dtype, const char* path);
// Sets the message of a host-only call (read by bhtsne_io_last_error).
void set_host_error(const std::string& msg);

// Keeps the freed memory of the device's default pool cached (no release
// back to the driver at synchronisations), once per device.
void keep_pool_cached(int device);

// ---- scan ---------------------------------------------------------------------
// Exclusive prefix sum of n values (u32 in, u64 out); out has n+1 entries, out[n]
// is the total. `tmp` is scratch owned by the caller.
void scan_u32_to_u64(const uint32_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s);
void scan_u64(const uint64_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s);

// ---- radix sort -----------------------------------------------------------------
// Stable LSD sort of (u64 key, payload) pairs on key bits [begin_bit, end_bit).
// Sorted data ends in (keys, vals); (keys_alt, vals_alt) are scratch of equal size.
// `tmp` holds radix_sort_tmp_bytes(n): per-tile digit counts (tiles of 2048
// keys), two super-tile tables (32 tiles each; the second doubles as the
// u64 super-tile offsets) and the scan's per-block partials.
constexpr int64_t kRadixTile = 2048, kRadixSup = 32, kRadixScanTile = 4096;
constexpr size_t radix_round256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t radix_sort_tmp_bytes(int64_t n) {
  return radix_round256((size_t)((n + kRadixTile - 1) / kRadixTile) * 256 * 4) +
         radix_round256((size_t)(((n + kRadixTile - 1) / kRadixTile + kRadixSup - 1) / kRadixSup) * 256 * 4) +
         radix_round256((size_t)((((n + kRadixTile - 1) / kRadixTile + kRadixSup - 1) / kRadixSup) * 256 + 1) * 8) +
         (size_t)(((((n + kRadixTile - 1) / kRadixTile + kRadixSup - 1) / kRadixSup) * 256 + kRadixScanTile - 1) /
                      kRadixScanTile +
                  1) *
             8 +
         256;
}
// From kOnesweepMin to kOnesweepMax keys a pass is one kernel (decoupled
// look-back); `tmp` then grows to hold the look-back words. A look-back wait
// that runs out (which would mean a fault, not slow progress) raises a
// library-wide fault word instead of hanging; radix_sort_fault_take reads and
// clears it (synchronising s).
constexpr int64_t kOnesweepMin = 131072, kOnesweepMax = (int64_t)1 << 24;
template <class V>
void radix_sort_pairs(uint64_t* keys, V* vals, uint64_t* keys_alt, V* vals_alt, int64_t n, int begin_bit,
                      int end_bit, DevBuf& tmp, cudaStream_t s);
bool radix_sort_fault_take(cudaStream_t s);

}  // namespace bhg
