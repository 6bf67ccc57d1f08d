// Autotuned launch shapes (see tune.cu).
#pragma once

#include <string>

#include "internal.h"

namespace bhg {

struct TuneKnobs {
  int attr_task_len = 128;  // entries per attractive task: 64, 128 or 256
  int bh_threads = 256;     // threads per block of the traversal: 128, 256 or 512
  int knn_pass = -1;        // -1 default, 0 tensor cores, 1 CUDA cores
  bool tuned = false;
};

// The knobs for (value type, D, N) on the current device: tuned or defaults.
TuneKnobs tune_lookup(int dtype, int D, int64_t n);
// Reads BHTSNE_TUNE_FILE into the table, once per process (if it exists).
void tune_load_env_once();
// Times every candidate on synthetic data of that shape (k neighbours per
// row; dim > 0 also tunes the kNN pass) and stores the fastest; writes
// BHTSNE_TUNE_FILE when set. report receives the timings.
int tune_run(int dtype, int D, int64_t n, int k, int dim, cudaStream_t s, std::string* report);
// {"key": ..., "knobs": {...}} for (value type, D, N) on the current device.
std::string tune_describe(int dtype, int D, int64_t n);
int tune_load(const char* path, std::string* err);
int tune_save(const char* path, std::string* err);

}  // namespace bhg
