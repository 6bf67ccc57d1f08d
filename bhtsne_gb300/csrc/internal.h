// Host-side declarations shared between the translation units of the library.
// Everything here is internal; the public surface is include/bhtsne_gpu.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.cuh"

namespace bhg {

// ---- device buffers ---------------------------------------------------------
// A grow-only device allocation owned by a context or a fit workspace.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  void* ensure(size_t want) {
    if (want <= bytes && ptr) return ptr;
    release();
    size_t b = want < 256 ? 256 : want;
    BHG_CUDA(cudaMalloc(&ptr, b));
    bytes = b;
    return ptr;
  }
  template <class V>
  V* as() const { return static_cast<V*>(ptr); }
  void swap(DevBuf& o) {
    void* p = ptr;
    size_t b = bytes;
    ptr = o.ptr;
    bytes = o.bytes;
    o.ptr = p;
    o.bytes = b;
  }
};

// ---- scan ---------------------------------------------------------------------
// Exclusive prefix sum of n values (u32 in, u64 out); out has n+1 entries, out[n]
// is the total. `tmp` is scratch owned by the caller.
void scan_u32_to_u64(const uint32_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s);
void scan_u64(const uint64_t* in, uint64_t* out, int64_t n, DevBuf& tmp, cudaStream_t s);

// ---- radix sort -----------------------------------------------------------------
// Stable LSD sort of (u64 key, payload) pairs on key bits [begin_bit, end_bit).
// Sorted data ends in (keys, vals); (keys_alt, vals_alt) are scratch of equal size.
template <class V>
void radix_sort_pairs(uint64_t* keys, V* vals, uint64_t* keys_alt, V* vals_alt, int64_t n, int begin_bit,
                      int end_bit, DevBuf& tmp, cudaStream_t s);

}  // namespace bhg
