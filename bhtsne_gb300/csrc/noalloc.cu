// Allocation-free Barnes-Hut repulsion: bhtsne_bh_repulsion_noalloc.
//
// Some callers cannot call cudaMalloc: code that records work into a CUDA
// stream capture (cudaMalloc is not a stream operation and may not run while
// a capture is open), hosts that hand the library a fixed device-memory budget
// from their own pool, or latency-sensitive loops where an allocation may
// synchronise the device. This entry point serves them. Inputs and outputs are
// device buffers owned by the caller; every scratch buffer the tree build and
// traversal need lives in one file-scope device array of fixed size, so the
// call performs no device allocation, no free, and no allocating library call.
//
// Limits and sharing:
//  * f32, D = 2, 2 <= n <= kNoAllocMaxPoints (32768 points); larger inputs
//    (and null pointers or theta <= 0) are rejected with BHTSNE_EINVAL.
//  * The array (kNoAllocBytes, about 3.5 MB) is held by every GPU that loads
//    the library until the process exits.
//  * All calls share the array and it keeps the previous call's contents; the
//    call clears what must start at zero. Calls whose work overlaps on the GPU
//    (for example on two streams at once) race on the array: serialise them.
//  * The first call on a device resolves the array's device address for that
//    device (cudaGetSymbolAddress, with that device current); make that first
//    call before any stream capture that should contain later calls.
#include <mutex>
#include <string>

#include "../../include/bhtsne_gpu.h"
#include "bh.h"

namespace bhg {
namespace {

constexpr int64_t kNoAllocMaxPoints = 32768;

// Slice sizes, each rounded up to 256 bytes. The Barnes-Hut buffers come from
// the same table BhWorkspace::reserve allocates from (bh_sizes), the sort and
// scan scratch from the sizes their launchers request, so the carve cannot
// fall behind a change of tile size; and every slice is a borrowed DevBuf,
// which throws instead of reallocating if a request ever exceeds it.
constexpr size_t al(size_t b) { return (b + 255) / 256 * 256; }
constexpr int64_t kN = kNoAllocMaxPoints;
constexpr BhSizes kBh = bh_sizes<float>(kN, 2);
static_assert(kBh.word == 0 && kBh.wide == 0, "D = 2 needs no word or 128-bit code arrays");
constexpr size_t kSzKeys = al(kBh.keys), kSzPerm = al(kBh.perm), kSzYs = al(kBh.ys), kSzPre = al(kBh.pre),
                 kSzPrePart = al(kBh.pre_part), kSzMask = al(kBh.mask), kSzCnt = al(kBh.cnt), kSzBase = al(kBh.base),
                 kSzGeom = al(kBh.geom), kSzPart = al(kBh.part), kSzSmall = al(kBh.small),
                 kSzParams = al(kBh.params), kSzZpart = al(kBh.zpart), kSzZval = al(kBh.zval),
                 kSzSort = al(radix_sort_tmp_bytes(kN)),
                 kSzScan = al((size_t)((kN + kRadixScanTile - 1) / kRadixScanTile + 1) * 8);
constexpr size_t kNoAllocBytes = 2 * kSzKeys + 2 * kSzPerm + kSzYs + kSzPre + kSzPrePart + kSzMask + kSzCnt + kSzBase +
                                 kSzGeom + 2 * kSzPart + 2 * kSzSmall + kSzParams + kSzZpart + kSzZval + kSzSort +
                                 kSzScan;
static_assert(kNoAllocBytes < 4 * 1024 * 1024, "the fixed scratch array stays under 4 MB");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_mu;
void* g_addr[128] = {nullptr};

// Device address of the scratch array on the current device, resolved once.
void* scratch_address(std::string* err) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) {
    *err = "error: no current CUDA device.";
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      *err = std::string("error: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
      return nullptr;
    }
    g_addr[dev] = p;
  }
  return g_addr[dev];
}

// Points a DevBuf at a slice of the array without taking ownership.
void view(DevBuf& b, unsigned char*& cur, size_t bytes) {
  b.borrow(cur, bytes);
  cur += bytes;
}

}  // namespace
}  // namespace bhg

using namespace bhg;

extern "C" {

int bhtsne_bh_repulsion_noalloc(const float* y, int64_t n, double theta, float* neg, double* z, void* stream) {
  // Argument errors are reported by status alone (no handle to hold a message).
  if (!y || !neg || !z || n < 2 || n > kNoAllocMaxPoints || !(theta > 0)) return BHTSNE_EINVAL;
  std::string err;
  void* base = scratch_address(&err);
  if (!base) return BHTSNE_ECUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BhWorkspace<float> ws;
  unsigned char* cur = static_cast<unsigned char*>(base);
  view(ws.keys, cur, kSzKeys);
  view(ws.keys_alt, cur, kSzKeys);
  view(ws.perm, cur, kSzPerm);
  view(ws.perm_alt, cur, kSzPerm);
  view(ws.ys, cur, kSzYs);
  view(ws.pre, cur, kSzPre);
  view(ws.pre_part, cur, kSzPrePart);
  view(ws.mask, cur, kSzMask);
  view(ws.cnt, cur, kSzCnt);
  view(ws.base, cur, kSzBase);
  view(ws.geom, cur, kSzGeom);
  view(ws.part_min, cur, kSzPart);
  view(ws.part_max, cur, kSzPart);
  view(ws.done, cur, kSzSmall);
  view(ws.zdone, cur, kSzSmall);
  view(ws.params, cur, kSzParams);
  view(ws.zpart, cur, kSzZpart);
  view(ws.zval, cur, kSzZval);
  view(ws.sort_tmp, cur, kSzSort);
  view(ws.scan_tmp, cur, kSzScan);
  int rc = BHTSNE_OK;
  try {
    // Every request of the normal path goes through the borrowed slices:
    // one that does not fit throws BHTSNE_EINTERNAL, nothing is allocated.
    ws.reserve(n, 2);
    ws.zeroed = true;
    // The completion tickets of the last-block reductions must start at zero.
    BHG_CUDA(cudaMemsetAsync(ws.done.ptr, 0, kSzSmall, s));
    BHG_CUDA(cudaMemsetAsync(ws.zdone.ptr, 0, kSzSmall, s));
    // Same stages as the Barnes-Hut step of bhtsne_gradient: box, tree, traversal.
    float* yy = const_cast<float*>(y);
    launch_recenter_bbox<float>(2, yy, n, nullptr, false, ws, bh_bits<float>(2), s);
    bh_build<float>(ws, 2, y, n, s);
    bh_traverse<float>(ws, 2, y, n, (float)theta, neg, nullptr, s);
    BHG_CUDA(cudaMemcpyAsync(z, ws.zval.ptr, sizeof(double), cudaMemcpyDeviceToDevice, s));
  } catch (const Error& e) {
    rc = e.code;
  }
  // The borrowed slices are detached, never freed, when ws goes out of scope.
  return rc;
}

}  // extern "C"
