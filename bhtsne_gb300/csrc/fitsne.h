// FIt-SNE repulsion (see fitsne.cu).
#pragma once

#include "bh.h"

namespace bhg {

// Transform lengths are the shorter of the next power of two and the next
// 3 * 2^j >= 2 nodes - 1; the capacity is a power of two, at most 8192 (boxes
// <= 1000 per axis, 3 nodes per box: 6144 or shorter is used).
constexpr int kFitMaxL = 8192;

template <class T>
struct FitParams {
  T lo, extent, box_width, inv_box_width, spacing;
  T scale;  // power of two >= max |y|: balances the magnitudes of packed terms
  int boxes, nodes, L;
  int need_L;     // transform length the embedding needs (L unless the capacity was too small)
  int fix_shift;  // charges are accumulated as integers in units of 2^-fix_shift
  T up, down;     // 2^fix_shift and 2^-fix_shift
};

struct FitGrid {
  int boxes = 0, nodes = 0, fft_len = 0;
  double lo = 0, box_width = 0, spacing = 0;
};

template <class T>
struct FitWorkspace {
  typedef typename std::conditional<sizeof(T) == 4, float2, double2>::type T2;
  DevBuf params, g0, g1, h0, h1, khat, tw, tw3, zpart, done, acc, flag;
  DevBuf direct;  // 1-D: FP64 kernel table and charge rows of the direct convolution
  int tw_len = 0, tw3_len = 0;
  const void* acc_clean = nullptr;  // acc allocation known to be all zero
  int cap_L = 0;  // transform length the buffers hold
  bool done_zeroed = false;
  const T2* twiddles(int L, cudaStream_t s);
  const T2* twiddles3(int cap_L, cudaStream_t s);
  // Buffers for transforms up to cap (a power of two) at n points.
  void reserve(int D, int64_t n, int cap);
};

// Repulsive forces (neg) and Z (z_out, device) at y; `box` must hold the
// current per-axis bounds. Synchronises once to size the grid.
template <class T>
FitGrid fit_repulsion(FitWorkspace<T>& ws, int D, const T* y, int64_t n, const BoxParams<T>* box, T* neg, double* z_out,
                      cudaStream_t s);

// The same without a host synchronisation (graph-capturable): every size is
// read on the device from the current parameters, within the reserved
// capacity ws.cap_L. If the embedding needs a longer transform, the flag
// ws.flag (int) is raised and the result is not valid; the caller grows the
// capacity (fit_needed_length) and repeats the step.
template <class T>
void fit_repulsion_cap(FitWorkspace<T>& ws, int D, const T* y, int64_t n, const BoxParams<T>* box, T* neg,
                       double* z_out, cudaStream_t s);

// Transform length the current embedding needs (synchronises).
template <class T>
int fit_needed_length(FitWorkspace<T>& ws, int D, int64_t n, const BoxParams<T>* box, cudaStream_t s);

}  // namespace bhg
