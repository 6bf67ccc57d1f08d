// Autotuning of launch shapes (no reference counterpart).
//
// Three knobs, each chosen by timing every candidate on the device:
//  * attr_task_len: entries per task of the attractive pass (64, 128, 256),
//    i.e. how many loads each lane has in flight. It sets how a row's terms
//    are grouped, so it moves results by rounding (all within the reference's
//    own summation error) but is fixed for a whole fit.
//  * bh_threads: threads per block of the Barnes-Hut traversal (128, 256,
//    512); one query per thread, so the forces do not depend on it.
//  * knn_pass: the kNN candidate pass on the tensor cores or on the CUDA
//    cores; both give the same (exact) neighbour lists.
// The chosen values are kept per (GPU name, value type, D, N bucket = floor
// log2 N) in a process-wide table. BHTSNE_TUNE_FILE names a JSON file that
// the first context created reads into the table and bhtsne_tune writes it
// back to; bhtsne_tune_load / bhtsne_tune_save do the same on demand. A fit
// looks its knobs up once, when it starts; missing entries give the defaults
// (128, 256, tensor cores).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bhtsne_gpu.h"
#include "bh.h"
#include "epoch.h"
#include "knn.h"
#include "tune.h"

namespace bhg {

namespace {

std::mutex g_tune_mu;
std::map<std::string, TuneKnobs>& table() {
  static std::map<std::string, TuneKnobs> t;
  return t;
}

std::string gpu_name() {
  int dev = 0;
  cudaDeviceProp p;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "none";
  std::string s(p.name);
  for (char& c : s)
    if (c == '|' || c == '"' || c == '\\') c = '_';
  return s;
}

int bucket_of(int64_t n) {
  int b = 0;
  while (n > 1) {
    n >>= 1;
    ++b;
  }
  return b;
}

std::string key_of(int dtype, int D, int64_t n) {
  return gpu_name() + "|" + (dtype == BHTSNE_F64 ? "f64" : "f32") + "|D" + std::to_string(D) + "|n2^" +
         std::to_string(bucket_of(n));
}

std::string knobs_json(const TuneKnobs& k) {
  char buf[160];
  snprintf(buf, sizeof buf, "{\"attr_task_len\": %d, \"bh_threads\": %d, \"knn_pass\": \"%s\", \"tuned\": %s}",
           k.attr_task_len, k.bh_threads, k.knn_pass == 1 ? "cuda_cores" : k.knn_pass == 0 ? "tensor_cores" : "default",
           k.tuned ? "true" : "false");
  return buf;
}

// The file: one JSON object, key -> {"attr_task_len": a, "bh_threads": b, "knn_pass": 0|1}.
std::string table_json() {
  std::string s = "{\n";
  bool first = true;
  for (const auto& kv : table()) {
    if (!kv.second.tuned) continue;
    if (!first) s += ",\n";
    first = false;
    char buf[512];
    snprintf(buf, sizeof buf, "  \"%s\": {\"attr_task_len\": %d, \"bh_threads\": %d, \"knn_pass\": %d}",
             kv.first.c_str(), kv.second.attr_task_len, kv.second.bh_threads, kv.second.knn_pass);
    s += buf;
  }
  s += "\n}\n";
  return s;
}

// Reads what table_json writes (keys without quotes or backslashes, integer values).
bool parse_table(const std::string& s, std::map<std::string, TuneKnobs>* out) {
  size_t p = s.find('{');
  if (p == std::string::npos) return false;
  ++p;
  for (;;) {
    const size_t q0 = s.find('"', p);
    if (q0 == std::string::npos) return true;
    const size_t q1 = s.find('"', q0 + 1);
    const size_t b0 = s.find('{', q1 == std::string::npos ? q0 : q1);
    const size_t b1 = s.find('}', b0 == std::string::npos ? q0 : b0);
    if (q1 == std::string::npos || b0 == std::string::npos || b1 == std::string::npos) return false;
    const std::string key = s.substr(q0 + 1, q1 - q0 - 1);
    const std::string body = s.substr(b0 + 1, b1 - b0 - 1);
    TuneKnobs k;
    auto field = [&](const char* name, int* v) {
      const size_t f = body.find(std::string("\"") + name + "\"");
      if (f == std::string::npos) return false;
      const size_t c = body.find(':', f);
      if (c == std::string::npos) return false;
      *v = std::atoi(body.c_str() + c + 1);
      return true;
    };
    if (!field("attr_task_len", &k.attr_task_len) || !field("bh_threads", &k.bh_threads) ||
        !field("knn_pass", &k.knn_pass))
      return false;
    k.tuned = true;
    (*out)[key] = k;
    p = b1 + 1;
  }
}

int load_file(const char* path, std::string* err) {
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    *err = std::string("error: cannot open ") + path;
    return BHTSNE_EIO;
  }
  std::string s;
  char chunk[4096];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) s.append(chunk, got);
  std::fclose(f);
  std::map<std::string, TuneKnobs> m;
  if (!parse_table(s, &m)) {
    *err = std::string("error: ") + path + " is not a tuning table.";
    return BHTSNE_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (const auto& kv : m) table()[kv.first] = kv.second;
  return BHTSNE_OK;
}

int save_file(const char* path, std::string* err) {
  std::string s;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    s = table_json();
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    *err = std::string("error: cannot create ") + path;
    return BHTSNE_EIO;
  }
  const bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
  const bool closed = std::fclose(f) == 0;
  if (!ok || !closed) {
    *err = std::string("error: cannot write ") + path;
    return BHTSNE_EIO;
  }
  return BHTSNE_OK;
}

// ---- synthetic problems ------------------------------------------------------
__device__ __forceinline__ uint32_t mix32(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return (uint32_t)x;
}

// Points in a few Gaussian-like clusters (sum of uniforms), spread over a
// square of side ~sqrt(n): the shapes an embedding takes after the
// exaggeration phase.
template <class T>
__global__ void synth_points_kernel(T* y, int64_t n, int D) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double side = sqrt((double)n) * 0.5;
  const uint32_t c = mix32(0x9e3779b97f4a7c15ULL ^ (uint64_t)i) % 64u;
  for (int a = 0; a < D; ++a) {
    const double centre = ((double)(mix32((uint64_t)c * 131 + a) % 10000u) / 10000.0 - 0.5) * side;
    double u = 0;
    for (int r = 0; r < 4; ++r) u += (double)(mix32(((uint64_t)i << 8) ^ (uint64_t)(a * 8 + r) ^ 0x5bd1e995ULL) % 65536u) / 65536.0;
    y[i * D + a] = (T)(centre + (u - 2.0) * side * 0.05);
  }
}

// k distinct-looking random columns per row (a kNN-shaped CSR), value 1 / (n k).
template <class T>
__global__ void synth_csr_kernel(uint64_t* rows, uint32_t* cols, T* vals, int64_t n, int k) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  rows[i] = (uint64_t)i * k;
  if (i == n) return;
  for (int j = 0; j < k; ++j) {
    cols[i * k + j] = mix32(((uint64_t)i << 20) ^ (uint64_t)j ^ 0x2545f4914f6cdd1dULL) % (uint32_t)n;
    vals[i * k + j] = (T)(1.0 / ((double)n * k));
  }
}

template <class F>
float time_ms(cudaStream_t s, int reps, F&& f) {
  f();  // warm-up
  cudaEvent_t a, b;
  BHG_CUDA(cudaEventCreate(&a));
  BHG_CUDA(cudaEventCreate(&b));
  BHG_CUDA(cudaEventRecord(a, s));
  for (int r = 0; r < reps; ++r) f();
  BHG_CUDA(cudaEventRecord(b, s));
  BHG_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  BHG_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

template <class T>
TuneKnobs tune_impl(int D, int64_t n, int k, int dim, cudaStream_t s, std::string* report) {
  TuneKnobs best;
  AllocStreamScope scope(s);
  char line[256];
  DevBuf y, rows, cols, vals, pos;
  y.ensure((size_t)n * D * sizeof(T));
  rows.ensure((size_t)(n + 1) * 8);
  cols.ensure((size_t)n * k * 4);
  vals.ensure((size_t)n * k * sizeof(T));
  pos.ensure((size_t)n * D * sizeof(T));
  synth_points_kernel<T><<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(y.as<T>(), n, D);
  BHG_LAUNCH_CHECK();
  synth_csr_kernel<T><<<(unsigned)ceil_div(n + 1, 256), 256, 0, s>>>(rows.as<uint64_t>(), cols.as<uint32_t>(),
                                                                     vals.as<T>(), n, k);
  BHG_LAUNCH_CHECK();
  // attractive pass
  float best_ms = 1e30f;
  for (int len : {64, 128, 256}) {
    AttrTasks at;
    build_attr_tasks<T>(at, D, rows.as<uint64_t>(), n, s, len);
    const float ms = time_ms(s, 5, [&] {
      launch_attractive_tasks<T>(at, cols.as<uint32_t>(), vals.as<T>(), y.as<T>(), pos.as<T>(), s);
    });
    snprintf(line, sizeof line, "attr_task_len %d: %.4f ms; ", len, ms);
    *report += line;
    if (ms < best_ms) {
      best_ms = ms;
      best.attr_task_len = len;
    }
  }
  // Barnes-Hut traversal (D = 2..7)
  if (D >= 2 && D <= 7) {
    BhWorkspace<T> ws;
    ws.reserve(n, D);
    launch_recenter_bbox<T>(D, y.as<T>(), n, nullptr, false, ws, bh_bits<T>(D), s);
    bh_build<T>(ws, D, y.as<T>(), n, s);
    best_ms = 1e30f;
    for (int bt : {128, 256, 512}) {
      ws.traverse_threads = bt;
      const float ms = time_ms(s, 3, [&] { bh_traverse<T>(ws, D, y.as<T>(), n, (T)0.5, pos.as<T>(), nullptr, s); });
      snprintf(line, sizeof line, "bh_threads %d: %.4f ms; ", bt, ms);
      *report += line;
      if (ms < best_ms) {
        best_ms = ms;
        best.bh_threads = bt;
      }
    }
  }
  // kNN candidate pass on a sample of synthetic data of the given dimension
  if (dim > 0) {
    const int64_t ns = n < 32768 ? n : 32768;
    const int kk = std::min<int>(k, (int)ns - 1);
    DevBuf x, idx, dst;
    x.ensure((size_t)ns * dim * sizeof(T));
    idx.ensure((size_t)ns * kk * 4);
    dst.ensure((size_t)ns * kk * sizeof(T));
    synth_points_kernel<T><<<(unsigned)ceil_div(ns, 256), 256, 0, s>>>(x.as<T>(), ns, dim);
    BHG_LAUNCH_CHECK();
    best_ms = 1e30f;
    for (int pass : {0, 1}) {
      KnnWorkspace kw;
      kw.pass = pass;
      const float ms = time_ms(s, 1, [&] {
        knn_euclidean<T>(x.as<T>(), ns, dim, kk, idx.as<uint32_t>(), dst.as<T>(), kw, s);
      });
      snprintf(line, sizeof line, "knn_pass %s: %.3f ms; ", pass ? "cuda_cores" : "tensor_cores", ms);
      *report += line;
      if (ms < best_ms) {
        best_ms = ms;
        best.knn_pass = pass;
      }
    }
  }
  best.tuned = true;
  return best;
}

}  // namespace

TuneKnobs tune_lookup(int dtype, int D, int64_t n) {
  const std::string key = key_of(dtype, D, n);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = table().find(key);
  return it == table().end() ? TuneKnobs() : it->second;
}

void tune_load_env_once() {
  static std::once_flag once;
  std::call_once(once, [] {
    const char* path = getenv("BHTSNE_TUNE_FILE");
    if (!path) return;
    FILE* f = std::fopen(path, "rb");
    if (!f) return;  // not written yet
    std::fclose(f);
    std::string err;
    load_file(path, &err);
  });
}

int tune_run(int dtype, int D, int64_t n, int k, int dim, cudaStream_t s, std::string* report) {
  if (n < 64 || k < 1 || D < 1 || D > 7 || dim < 0) throw Error(ST_EINVAL, "error: invalid tuning arguments.");
  TuneKnobs best;
  if (dtype == BHTSNE_F64) best = tune_impl<double>(D, n, k, dim, s, report);
  else best = tune_impl<float>(D, n, k, dim, s, report);
  const std::string key = key_of(dtype, D, n);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    table()[key] = best;
  }
  if (const char* path = getenv("BHTSNE_TUNE_FILE")) {
    std::string err;
    const int rc = save_file(path, &err);
    if (rc != BHTSNE_OK) throw Error(rc, err);
  }
  return BHTSNE_OK;
}

std::string tune_describe(int dtype, int D, int64_t n) {
  const TuneKnobs k = tune_lookup(dtype, D, n);
  return "{\"key\": \"" + key_of(dtype, D, n) + "\", \"knobs\": " + knobs_json(k) + "}";
}

int tune_load(const char* path, std::string* err) { return load_file(path, err); }
int tune_save(const char* path, std::string* err) { return save_file(path, err); }

}  // namespace bhg

extern "C" {

int bhtsne_tune_config(int dtype, int32_t embed_dim, int64_t n, char* json, int64_t len) {
  if (!json || len <= 0) {
    bhg::set_host_error("error: invalid tune_config arguments.");
    return BHTSNE_EINVAL;
  }
  const std::string d = bhg::tune_describe(dtype, embed_dim, n);
  if ((int64_t)d.size() + 1 > len) {
    bhg::set_host_error("error: the buffer is too small for the configuration.");
    return BHTSNE_EINVAL;
  }
  std::memcpy(json, d.c_str(), d.size() + 1);
  return BHTSNE_OK;
}

int bhtsne_tune_load(const char* path) {
  if (!path) {
    bhg::set_host_error("error: the path is null.");
    return BHTSNE_EINVAL;
  }
  std::string err;
  const int rc = bhg::tune_load(path, &err);
  if (rc != BHTSNE_OK) bhg::set_host_error(err);
  return rc;
}

int bhtsne_tune_save(const char* path) {
  if (!path) {
    bhg::set_host_error("error: the path is null.");
    return BHTSNE_EINVAL;
  }
  std::string err;
  const int rc = bhg::tune_save(path, &err);
  if (rc != BHTSNE_OK) bhg::set_host_error(err);
  return rc;
}

}  // extern "C"
