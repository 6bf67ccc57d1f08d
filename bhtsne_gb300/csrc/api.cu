// C ABI of the library (include/bhtsne_gpu.h): the tSNE builder state machine
// and the stage entry points.
//
// The handle mirrors the reference builder (bhtsne 0.7.10, src/lib.rs):
// fields :149-176, defaults :241-266, setters :277-435, finishers :489-951,
// affinity cache :1019-1051 and :1192-1248, epoch tail :1162-1179. Device
// state (P, y, velocity, gains and every scratch buffer) stays resident in the
// handle; host memory is touched only for the caller's inputs and outputs and
// for the optional per-epoch callback snapshot.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bhtsne_gpu.h"
#include "affinity.h"
#include "bh.h"
#include "epoch.h"
#include "fitsne.h"
#include "knn.h"
#include "tune.h"
#include "batch.h"

using namespace bhg;

namespace bhg {
std::atomic<long long> g_launches{0};
thread_local cudaStream_t g_alloc_stream = nullptr;

void keep_pool_cached(int device) {
  static std::mutex m;
  static bool done[128] = {};
  std::lock_guard<std::mutex> lk(m);
  if (device < 0 || device >= 128 || done[device]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done[device] = true;
}
}  // namespace bhg

struct bhtsne_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t knn_fallback_rows = 0;  // rows of the last kNN on this context that failed the certificate
  int64_t knn_brute_rows = 0;     // of those, the rows recomputed by brute force
};

namespace bhg {
int ctx_device(const bhtsne_ctx* ctx) { return ctx->device; }

// A context whose stream has the given priority (lower numbers run first);
// used by the server for its FIt-SNE workers.
int ctx_create_with_priority(int device, int priority, bhtsne_ctx** out) {
  if (!out) return BHTSNE_EINVAL;
  *out = nullptr;
  bhtsne_ctx* c = new bhtsne_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, priority) != cudaSuccess) {
    delete c;
    return BHTSNE_ECUDA;
  }
  keep_pool_cached(device);
  tune_load_env_once();
  *out = c;
  return BHTSNE_OK;
}
}  // namespace bhg

namespace {

const char* kVersion = "bhtsne-gb300 0.1.0 (restates bhtsne 0.7.10)";

template <class T>
struct State {
  int D = 2;
  int64_t n = 0;
  // sparse P (CSR)
  bool has_sparse = false;
  int64_t sparse_rows = 0;  // number of row offsets held (n + 1 when usable)
  int64_t nnz = 0;
  DevBuf rows, cols, vals;
  // dense P (exact)
  bool has_dense = false;
  DevBuf pdense;
  // optimisation state
  DevBuf y, uy, gains, pos, neg, zbuf, klbuf, tmp, tmp2;
  DevBuf kidx, kdist, kp, xin, yext, ckpt;
  Renumbering rn;  // locality layout of y/uy/gains (see launch_renumber)
  // component layout of the current fit (component_order): the points grouped
  // by connected component of P, laid out once at epoch 0 instead of the
  // periodic Morton re-layout
  bool comp_mode = false;     // the component layout is active
  bool comp_decided = false;  // the first periodic re-layout point has chosen the layout
  bool comp_eligible = false; // this fit may use the component layout
  int64_t comp_largest = 0;
  DevBuf comp_order, comp_slots;
  ComponentScratch comp;
  AttrTasks at;    // attractive-pass tasks of the current CSR layout
  int task_len = kAttrTaskLen;  // the tuned task length of the current fit
  uint64_t layout_gen = 0;
  // y in the caller's point order (a copy when the layout is renumbered).
  const T* y_external(cudaStream_t s) {
    if (!rn.active) return y.template as<T>();
    T* out = static_cast<T*>(yext.ensure((size_t)n * D * sizeof(T)));
    launch_unpermute<T>(D, y.template as<T>(), rn.ext.template as<uint32_t>(), n, out, s);
    return out;
  }
  BhWorkspace<T> bh;
  FitWorkspace<T> fit;
  UpdateScratch us;
  SymWorkspace<T> sym;
  KnnWorkspace knn;
};

template <class T>
void upload(DevBuf& b, const void* src, size_t bytes, cudaStream_t s) {
  b.ensure(bytes);
  if (bytes) BHG_CUDA(cudaMemcpyAsync(b.ptr, src, bytes, cudaMemcpyHostToDevice, s));
}

template <class T>
__global__ void fill_kernel(T* p, int64_t n, T v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

__global__ void match_neighbors_kernel(const uint64_t* __restrict__ rows, const uint32_t* __restrict__ cols, int64_t n,
                                       int64_t k, const uint32_t* __restrict__ idx, int* __restrict__ mismatch) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * k) return;
  const int64_t i = e / k, j = e % k;
  const uint64_t s = rows[i], t = rows[i + 1];
  if ((int64_t)(t - s) != k || cols[s + j] != idx[e]) *mismatch = 1;
}


}  // namespace

struct bhtsne_tsne {
  bhtsne_ctx* ctx = nullptr;
  int dtype = BHTSNE_F32;
  int D = 2;
  int64_t n = 0;
  // builder fields (values rounded through T at the setter)
  bool has_lr = false;
  double lr = 0;
  int64_t epochs = 1000;
  double momentum = 0.5, final_momentum = 0.8;
  int64_t momentum_switch_epoch = 250, stop_lying_epoch = 250;
  double early_exaggeration = 12.0, perplexity = 20.0;
  bhtsne_epoch_cb cb = nullptr;
  void* user = nullptr;
  bool has_init = false;
  std::vector<unsigned char> init;
  int64_t init_len = 0;
  bool caller_init = false;  // the current fit started from the caller's embedding
  bool comp_layout = false;  // the last fit used the component layout
  int64_t comp_largest = 0;
  bool stop_lying_fired = false;
  bool has_cached_perplexity = false;
  double cached_perplexity = 0;
  int fit = 0;
  double fit_theta = 0;
  uint64_t seed = 0x6268747336e65ULL;
  // armed loop (for advance)
  bool armed = false;
  int loop_kind = 0;
  double loop_theta = 0, loop_lr = 0;
  int64_t cursor = 0;
  // timings
  double aff_ms = 0, loop_ms = 0;
  int64_t loop_epochs = 0;
  bool profile = false;
  double phase_ms[BHTSNE_PHASES] = {0, 0, 0, 0};
  int64_t phase_epochs = 0;
  double relayout_ms = 0;  // locality re-layouts of the last finisher or advance call
  int64_t relayouts = 0;
  // CUDA graph of one epoch body (Barnes-Hut and exact), re-captured when the
  // momentum changes or a new fit starts.
  cudaGraphExec_t graph = nullptr;
  double graph_momentum = 0;
  int64_t graph_kernels = 0;
  void drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
  }
  std::string err;
  State<float>* sf = nullptr;
  State<double>* sd = nullptr;
};

namespace {

double tcast(const bhtsne_tsne* t, double v) { return t->dtype == BHTSNE_F32 ? (double)(float)v : v; }

[[noreturn]] void invalid(const std::string& m) { throw Error(ST_EINVAL, m); }

template <class F>
int guard_ctx(bhtsne_ctx* ctx, F&& f) {
  if (!ctx) return BHTSNE_EINVAL;
  AllocStreamScope scope(ctx->stream);
  try {
    BHG_CUDA(cudaSetDevice(ctx->device));
    f();
    ctx->err.clear();
    return BHTSNE_OK;
  } catch (const Error& e) {
    ctx->err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    ctx->err = e.what();
    return BHTSNE_EINTERNAL;
  }
}

template <class F>
int guard(bhtsne_tsne* t, F&& f) {
  if (!t) return BHTSNE_EINVAL;
  AllocStreamScope scope(t->ctx->stream);
  try {
    BHG_CUDA(cudaSetDevice(t->ctx->device));
    f();
    return BHTSNE_OK;
  } catch (const Error& e) {
    t->err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    t->err = e.what();
    return BHTSNE_EINTERNAL;
  }
}

// check_perplexity: src/tsne/mod.rs:55-59.
void check_perplexity(const bhtsne_tsne* t) {
  const double perp = t->perplexity;
  const int64_t as_usize = perp > 0 ? (int64_t)perp : 0;
  if (t->n < 1 || (t->n - 1) < 3 * as_usize)
    invalid("error: the provided perplexity is too large for the number of data points.\n");
}

// validate_fit_params: src/lib.rs:1182-1189.
void validate_fit_params(const bhtsne_tsne* t, double theta) {
  if (!(theta > 0))
    invalid(
        "error: theta value must be greater than 0.0.\n            A value of 0.0 corresponds to using the exact "
        "version of the algorithm.");
  check_perplexity(t);
}

template <class T>
State<T>& st(bhtsne_tsne* t);
template <>
State<float>& st<float>(bhtsne_tsne* t) {
  return *t->sf;
}
template <>
State<double>& st<double>(bhtsne_tsne* t) {
  return *t->sd;
}

template <class T>
T resolve_lr(const bhtsne_tsne* t) {
  if (t->has_lr) return (T)t->lr;
  const T a = (T)(double)t->n / (T)t->early_exaggeration / (T)4.0;
  return a > (T)50.0 ? a : (T)50.0;
}


// finalize_p_and_seed: src/lib.rs:663-685 (plus the optimisation buffers that
// the reference resizes in build_affinities / prepare_cached).
template <class T>
void finalize_p_and_seed(bhtsne_tsne* t, bool dense) {
  State<T>& S = st<T>(t);
  cudaStream_t s = t->ctx->stream;
  const int64_t ge = t->n * t->D;
  T* p = dense ? S.pdense.template as<T>() : S.vals.template as<T>();
  const int64_t np = dense ? t->n * t->n : S.nnz;
  launch_normalize<T>(p, np, (T)t->early_exaggeration, S.zbuf.template as<double>() + 2, S.tmp, s);
  if (t->stop_lying_epoch == 0) launch_scale<T>(p, np, T(1) / (T)t->early_exaggeration, s);
  S.y.ensure(ge * sizeof(T));
  t->caller_init = t->has_init;
  if (t->has_init) {
    t->has_init = false;
    if (t->init_len != ge) {
      const int64_t got = t->init_len;
      t->init.clear();
      invalid("error: initial embedding has " + std::to_string(got) + " values, expected n_samples * D = " +
              std::to_string(ge));
    }
    BHG_CUDA(cudaMemcpyAsync(S.y.ptr, t->init.data(), ge * sizeof(T), cudaMemcpyHostToDevice, s));
    BHG_CUDA(cudaStreamSynchronize(s));
    t->init.clear();
  } else {
    launch_random_init<T>(S.y.template as<T>(), ge, t->seed, s);
  }
  S.uy.ensure(ge * sizeof(T));
  S.gains.ensure(ge * sizeof(T));
  BHG_CUDA(cudaMemsetAsync(S.uy.ptr, 0, ge * sizeof(T), s));
  fill_kernel<T><<<256, 256, 0, s>>>(S.gains.template as<T>(), ge, T(1));
  BHG_LAUNCH_CHECK();
}

template <class T>
void ensure_state(bhtsne_tsne* t) {
  State<T>& S = st<T>(t);
  S.D = t->D;
  S.n = t->n;
  const int64_t ge = std::max<int64_t>(t->n * t->D, 1);
  S.pos.ensure(ge * sizeof(T));
  S.neg.ensure(ge * sizeof(T));
  S.zbuf.ensure(16 * sizeof(double));
  S.klbuf.ensure(16 * sizeof(double));
}

// build_affinities: src/lib.rs:1061-1127, from a device kNN table in S.kidx / S.kdist.
template <class T>
void build_affinities(bhtsne_tsne* t, int64_t k) {
  State<T>& S = st<T>(t);
  cudaStream_t s = t->ctx->stream;
  const int64_t n = t->n;
  S.kp.ensure(n * k * sizeof(T));
  launch_search_beta<T>(S.kdist.template as<T>(), n, k, (T)t->perplexity, S.kp.template as<T>(), nullptr, s);
  const int64_t nnz = symmetrize<T>(S.kidx.template as<uint32_t>(), S.kp.template as<T>(), n, (int)k, S.sym, s);
  S.rows.ensure((n + 1) * 8);
  S.cols.ensure(std::max<int64_t>(nnz, 1) * 4);
  S.vals.ensure(std::max<int64_t>(nnz, 1) * sizeof(T));
  symmetrize_finish<T>(S.sym, n, nnz, S.rows.template as<uint64_t>(), S.cols.template as<uint32_t>(),
                       S.vals.template as<T>(), s);
  BHG_CUDA(cudaStreamSynchronize(s));
  S.sym.release();
  S.kp.release();
  S.nnz = nnz;
  S.has_sparse = true;
  S.sparse_rows = n + 1;
  t->has_cached_perplexity = true;
  t->cached_perplexity = t->perplexity;
}

template <class T>
void epoch_tail(bhtsne_tsne* t, int64_t epoch, std::vector<T>& snap) {
  State<T>& S = st<T>(t);
  cudaStream_t s = t->ctx->stream;
  if (epoch == t->stop_lying_epoch && epoch != 0) {
    const T scale = T(1) / (T)t->early_exaggeration;
    if (t->loop_kind == BHTSNE_METHOD_EXACT) launch_scale<T>(S.pdense.template as<T>(), t->n * t->n, scale, s);
    else launch_scale<T>(S.vals.template as<T>(), S.nnz, scale, s);
    if (S.rn.active && t->loop_kind != BHTSNE_METHOD_EXACT) launch_scale<T>(S.rn.vals.template as<T>(), S.nnz, scale, s);
    t->stop_lying_fired = true;
  }
  if (epoch == t->momentum_switch_epoch) t->momentum = t->final_momentum;
  if (t->cb) {
    snap.resize(t->n * t->D);
    BHG_CUDA(cudaMemcpyAsync(snap.data(), S.y_external(s), snap.size() * sizeof(T), cudaMemcpyDeviceToHost, s));
    BHG_CUDA(cudaStreamSynchronize(s));
    t->cb(epoch, snap.data(), t->user);
  }
}

template <class T>
int bits_for_method(const bhtsne_tsne* t) {
  return (t->loop_kind == BHTSNE_METHOD_BARNES_HUT) ? bh_bits<T>(t->D) : 32;
}

// The epoch loop body of run_loop (src/lib.rs:961-1014) and of exact's loop
// (src/lib.rs:567-638), on device-resident state.
template <class T>
void advance_impl(bhtsne_tsne* t, int64_t epochs) {
  State<T>& S = st<T>(t);
  cudaStream_t s = t->ctx->stream;
  const int64_t n = t->n;
  const int D = t->D;
  const T lr = (T)t->loop_lr;
  const int bits = bits_for_method<T>(t);
  std::vector<T> snap;
  S.bh.reserve(n, D);
  cudaEvent_t e0, e1;
  BHG_CUDA(cudaEventCreate(&e0));
  BHG_CUDA(cudaEventCreate(&e1));
  BHG_CUDA(cudaEventRecord(e0, s));
  T* y = S.y.template as<T>();
  double* z = S.zbuf.template as<double>();
  // Optional phase profiling: 5 events per epoch bound the 4 phases.
  const bool prof = t->profile;
  std::vector<cudaEvent_t> ev;
  if (prof) {
    ev.resize((size_t)epochs * (BHTSNE_PHASES + 1));
    for (auto& e : ev) BHG_CUDA(cudaEventCreate(&e));
  }
  auto mark = [&](int64_t k, int ph) {
    if (prof) BHG_CUDA(cudaEventRecord(ev[(size_t)k * (BHTSNE_PHASES + 1) + ph], s));
  };
  // Graph replay of the epoch body: Barnes-Hut and exact epochs have a fixed
  // launch sequence (the node count is read on the device), so after one
  // eager epoch has sized every buffer the body is captured once and
  // replayed. Off while profiling or when a callback needs per-epoch copies.
  static const bool graphs_off = getenv("BHTSNE_NO_GRAPH") != nullptr;
  const bool graphable = !graphs_off && !prof && !t->cb && t->loop_kind != BHTSNE_METHOD_FIT_SNE;
  const bool graphable_fit = !graphs_off && !prof && !t->cb && t->loop_kind == BHTSNE_METHOD_FIT_SNE;
  // Locality renumbering: every kRenumberEvery epochs the sparse methods re-lay
  // out y / uy / gains in the Morton order of the current embedding so that a
  // row's neighbour gathers in the attractive pass stay close in memory.
  const char* rev = getenv("BHTSNE_RENUMBER_EVERY");
  const int64_t renumber_every = rev ? atoll(rev) : 50;
  const bool sparse = t->loop_kind != BHTSNE_METHOD_EXACT;
  // Tasks of the current CSR layout, rebuilt (outside any capture) when the
  // layout changes: at a fit's start and at each renumbering.
  auto ensure_tasks = [&]() {
    if (!sparse || S.at.gen == S.layout_gen) return;
    build_attr_tasks<T>(S.at, D, (S.rn.active ? S.rn.rows : S.rows).template as<uint64_t>(), n, s, S.task_len);
    S.at.gen = S.layout_gen;
  };
  auto attractive = [&]() {
    if (S.rn.active)
      launch_attractive_tasks<T>(S.at, S.rn.cols.template as<uint32_t>(), S.rn.vals.template as<T>(), y,
                                 S.pos.template as<T>(), s);
    else
      launch_attractive_tasks<T>(S.at, S.cols.template as<uint32_t>(), S.vals.template as<T>(), y,
                                 S.pos.template as<T>(), s);
  };
  // CUDA events around each re-layout, read after the loop's final sync.
  std::vector<cudaEvent_t> rl_ev;
  auto maybe_renumber = [&](int64_t epoch) {
    if (S.comp_mode) return;  // laid out once by component: no periodic re-layout
    if (!sparse || renumber_every <= 0 || epoch % renumber_every != 0) return;
    // The first periodic re-layout point (epoch 50 by default) chooses the
    // layout for the rest of the fit: grouped by component when P's graph
    // splits into small components, else the Morton order of the embedding
    // every period. Fits shorter than a period never pay for the components.
    if (epoch > 0 && S.comp_eligible && !S.comp_decided) {
      S.comp_decided = true;
      S.comp_mode = component_order(S.rows.template as<uint64_t>(), S.cols.template as<uint32_t>(), n, S.comp_order,
                                    S.comp, &S.comp_largest, s);
      S.comp.release();
      t->comp_layout = S.comp_mode;
      t->comp_largest = S.comp_largest;
    }
    if (S.comp_mode) {
      // the state is in the caller's order, or in a Morton layout from epoch 0
      // (a warm start): the component order is of CSR rows, so compose it
      // with the current slot map
      const bool was_active = S.rn.active;
      rl_ev.resize(rl_ev.size() + 2);
      BHG_CUDA(cudaEventCreate(&rl_ev[rl_ev.size() - 2]));
      BHG_CUDA(cudaEventCreate(&rl_ev[rl_ev.size() - 1]));
      BHG_CUDA(cudaEventRecord(rl_ev[rl_ev.size() - 2], s));
      const uint32_t* order = S.comp_order.template as<uint32_t>();
      if (was_active) {
        uint32_t* o2 = static_cast<uint32_t*>(S.comp_slots.ensure((size_t)n * 4));
        launch_compose_order(order, S.rn.inv.template as<uint32_t>(), n, o2, s);
        order = o2;
      }
      launch_renumber<T>(D, order, n, S.rn, y, S.uy.template as<T>(),
                         S.gains.template as<T>(), S.pos.template as<T>(), S.neg.template as<T>(),
                         static_cast<T*>(S.yext.ensure((size_t)n * D * sizeof(T))), S.rows.template as<uint64_t>(),
                         S.cols.template as<uint32_t>(), S.vals.template as<T>(), S.nnz, s);
      launch_recenter_bbox<T>(D, y, n, nullptr, false, S.bh, bits, s);
      ++S.layout_gen;
      ensure_tasks();
      BHG_CUDA(cudaEventRecord(rl_ev.back(), s));
      if (!was_active) t->drop_graph();
      return;
    }
    // At epoch 0 only a caller's embedding (a warm start) has a layout worth
    // following; the seeded random start has none. A re-layout costs about as
    // much as the attractive passes of a re-layout period save, so a warm
    // start that runs fewer epochs than one period (in this call: a finisher
    // or an advance) keeps the caller's order.
    if (epoch == 0 && (!t->caller_init || epochs < renumber_every)) return;
    if (D < 2 || D > 3) return;
    rl_ev.resize(rl_ev.size() + 2);
    BHG_CUDA(cudaEventCreate(&rl_ev[rl_ev.size() - 2]));
    BHG_CUDA(cudaEventCreate(&rl_ev[rl_ev.size() - 1]));
    BHG_CUDA(cudaEventRecord(rl_ev[rl_ev.size() - 2], s));
    // the Morton order of the current y (the Barnes-Hut build computes it every
    // epoch; the FIt-SNE loop builds it here)
    if (t->loop_kind != BHTSNE_METHOD_BARNES_HUT || epoch == 0) {
      launch_recenter_bbox<T>(D, y, n, nullptr, false, S.bh, bh_bits<T>(D), s);
      bh_build<T>(S.bh, D, y, n, s);
    }
    const bool was_active = S.rn.active;
    launch_renumber<T>(D, S.bh.perm.template as<uint32_t>(), n, S.rn, y, S.uy.template as<T>(), S.gains.template as<T>(),
                       S.pos.template as<T>(), S.neg.template as<T>(), static_cast<T*>(S.yext.ensure((size_t)n * D * sizeof(T))),
                       S.rows.template as<uint64_t>(), S.cols.template as<uint32_t>(), S.vals.template as<T>(), S.nnz, s);
    if (t->loop_kind != BHTSNE_METHOD_BARNES_HUT || epoch == 0)
      launch_recenter_bbox<T>(D, y, n, nullptr, false, S.bh, bits, s);
    ++S.layout_gen;
    ensure_tasks();
    BHG_CUDA(cudaEventRecord(rl_ev.back(), s));
    if (!was_active) t->drop_graph();  // the attractive pass now reads the slot arrays
  };
  ensure_tasks();
  auto fit_body = [&](T mom) {
    fit_repulsion_cap<T>(S.fit, D, y, n, S.bh.params.template as<BoxParams<T>>(), S.neg.template as<T>(), z, s);
    attractive();
    launch_update<T>(D, y, S.pos.template as<T>(), S.neg.template as<T>(), S.uy.template as<T>(),
                     S.gains.template as<T>(), n, z, T(0), lr, mom, S.us, s);
    launch_recenter_bbox<T>(D, y, n, S.us.mean(), true, S.bh, bits, s);
  };
  auto body = [&](T mom) {
    if (t->loop_kind == BHTSNE_METHOD_BARNES_HUT) {
      bh_build<T>(S.bh, D, y, n, s);
      bh_traverse<T>(S.bh, D, y, n, (T)t->loop_theta, S.neg.template as<T>(), nullptr, s);
      attractive();
      launch_update<T>(D, y, S.pos.template as<T>(), S.neg.template as<T>(), S.uy.template as<T>(),
                       S.gains.template as<T>(), n, S.bh.z(), T(0), lr, mom, S.us, s);
    } else {
      launch_exact_z<T>(D, y, n, z, S.tmp, s);
      launch_exact_grad<T>(D, y, S.pdense.template as<T>(), n, z, S.pos.template as<T>(), s);
      launch_update<T>(D, y, S.pos.template as<T>(), nullptr, S.uy.template as<T>(), S.gains.template as<T>(), n,
                       nullptr, T(0), lr, mom, S.us, s);
    }
    launch_recenter_bbox<T>(D, y, n, S.us.mean(), true, S.bh, bits, s);
  };
  // FIt-SNE without a host synchronisation per epoch: the grid sizes are read
  // on the device within a reserved transform capacity, so the epoch body is
  // a graph too. Epochs run in chunks (up to 25, ending before a renumbering
  // and at an epoch whose tail changes P or the momentum); after a chunk one
  // synchronisation checks the capacity flag. If the embedding outgrew the
  // capacity, the chunk's starting state is restored, the capacity doubled
  // and the chunk repeated, so results never depend on the capacity.
  if (graphable_fit && epochs > 0) {
    FitWorkspace<T>& fw = S.fit;
    const size_t ybytes = (size_t)n * D * sizeof(T);
    T* ck = static_cast<T*>(S.ckpt.ensure(3 * ybytes));
    int64_t k = 0;
    bool eager_next = true;
    while (k < epochs) {
      const int64_t epoch = t->cursor;
      if (epoch == 0) launch_recenter_bbox<T>(D, y, n, nullptr, false, S.bh, bits, s);
      maybe_renumber(epoch);
      int64_t len = std::min<int64_t>(25, epochs - k);
      for (int64_t i = 0; i < len; ++i) {
        const int64_t e = epoch + i;
        if (i > 0 && renumber_every > 0 && e % renumber_every == 0) {
          len = i;
          break;
        }
        if ((e == t->stop_lying_epoch && e != 0) || e == t->momentum_switch_epoch) {
          len = i + 1;
          break;
        }
      }
      if (fw.cap_L == 0) {
        const int need = fit_needed_length<T>(fw, D, n, S.bh.params.template as<BoxParams<T>>(), s);
        int cap = 64;
        while (cap < 2 * need && cap < kFitMaxL) cap <<= 1;
        fw.reserve(D, n, cap);
        t->drop_graph();
        eager_next = true;
      }
      BHG_CUDA(cudaMemcpyAsync(ck, y, ybytes, cudaMemcpyDeviceToDevice, s));
      BHG_CUDA(cudaMemcpyAsync(ck + (size_t)n * D, S.uy.ptr, ybytes, cudaMemcpyDeviceToDevice, s));
      BHG_CUDA(cudaMemcpyAsync(ck + 2 * (size_t)n * D, S.gains.ptr, ybytes, cudaMemcpyDeviceToDevice, s));
      BHG_CUDA(cudaMemsetAsync(fw.flag.ptr, 0, 2 * sizeof(int), s));  // capacity flag, FFT fault word
      const T mom = (T)t->momentum;
      for (int64_t i = 0; i < len; ++i) {
        if (eager_next) {
          fit_body(mom);
          eager_next = false;
          continue;
        }
        if (!t->graph || t->graph_momentum != t->momentum) {
          t->drop_graph();
          cudaGraph_t g;
          const long long before = g_launches.load();
          BHG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
          fit_body(mom);
          BHG_CUDA(cudaStreamEndCapture(s, &g));
          t->graph_kernels = g_launches.load() - before;
          g_launches.fetch_sub(t->graph_kernels);
          BHG_CUDA(cudaGraphInstantiate(&t->graph, g, 0));
          BHG_CUDA(cudaGraphDestroy(g));
          t->graph_momentum = t->momentum;
        }
        BHG_CUDA(cudaGraphLaunch(t->graph, s));
        g_launches.fetch_add(t->graph_kernels);
      }
      int flags[2] = {0, 0};
      FitParams<T> hp;
      BHG_CUDA(cudaMemcpyAsync(flags, fw.flag.ptr, sizeof(flags), cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaMemcpyAsync(&hp, fw.params.ptr, sizeof(hp), cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaStreamSynchronize(s));
      if (flags[1]) throw Error(ST_ETIMEDOUT, "error: an FFT row load timed out.");
      const int over = flags[0];
      if (over) {
        BHG_CUDA(cudaMemcpyAsync(y, ck, ybytes, cudaMemcpyDeviceToDevice, s));
        BHG_CUDA(cudaMemcpyAsync(S.uy.ptr, ck + (size_t)n * D, ybytes, cudaMemcpyDeviceToDevice, s));
        BHG_CUDA(cudaMemcpyAsync(S.gains.ptr, ck + 2 * (size_t)n * D, ybytes, cudaMemcpyDeviceToDevice, s));
        launch_recenter_bbox<T>(D, y, n, nullptr, false, S.bh, bits, s);
        fw.reserve(D, n, std::min(2 * fw.cap_L, kFitMaxL));
        t->drop_graph();
        eager_next = true;
        continue;
      }
      for (int64_t i = 0; i < len; ++i) epoch_tail<T>(t, epoch + i, snap);
      t->cursor += len;
      k += len;
      if (2 * hp.need_L > fw.cap_L && fw.cap_L < kFitMaxL) {
        int cap = fw.cap_L;
        while (cap < 2 * hp.need_L && cap < kFitMaxL) cap <<= 1;
        fw.reserve(D, n, cap);
        t->drop_graph();
        eager_next = true;
      }
    }
  }
  bool warmed = false;
  for (int64_t k = graphable_fit ? epochs : 0; k < epochs; ++k) {
    const int64_t epoch = t->cursor;
    if (epoch == 0) launch_recenter_bbox<T>(D, y, n, nullptr, false, S.bh, bits, s);
    maybe_renumber(epoch);
    const T mom = (T)t->momentum;
    if (graphable && warmed) {
      if (!t->graph || t->graph_momentum != t->momentum) {
        t->drop_graph();
        cudaGraph_t g;
        const long long before = g_launches.load();
        BHG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
        body(mom);
        BHG_CUDA(cudaStreamEndCapture(s, &g));
        t->graph_kernels = g_launches.load() - before;
        g_launches.fetch_sub(t->graph_kernels);
        BHG_CUDA(cudaGraphInstantiate(&t->graph, g, 0));
        BHG_CUDA(cudaGraphDestroy(g));
        t->graph_momentum = t->momentum;
      }
      BHG_CUDA(cudaGraphLaunch(t->graph, s));
      g_launches.fetch_add(t->graph_kernels);
      epoch_tail<T>(t, epoch, snap);
      t->cursor += 1;
      continue;
    }
    warmed = true;
    mark(k, 0);
    if (t->loop_kind == BHTSNE_METHOD_BARNES_HUT) {
      bh_build<T>(S.bh, D, y, n, s);
      mark(k, 1);
      bh_traverse<T>(S.bh, D, y, n, (T)t->loop_theta, S.neg.template as<T>(), nullptr, s);
      mark(k, 2);
      attractive();
      mark(k, 3);
      launch_update<T>(D, y, S.pos.template as<T>(), S.neg.template as<T>(), S.uy.template as<T>(),
                       S.gains.template as<T>(), n, S.bh.z(), T(0), lr, mom, S.us, s);
    } else if (t->loop_kind == BHTSNE_METHOD_FIT_SNE) {
      mark(k, 1);
      fit_repulsion<T>(S.fit, D, y, n, S.bh.params.template as<BoxParams<T>>(), S.neg.template as<T>(), z, s);
      mark(k, 2);
      attractive();
      mark(k, 3);
      launch_update<T>(D, y, S.pos.template as<T>(), S.neg.template as<T>(), S.uy.template as<T>(),
                       S.gains.template as<T>(), n, z, T(0), lr, mom, S.us, s);
    } else {
      mark(k, 1);
      launch_exact_z<T>(D, y, n, z, S.tmp, s);
      launch_exact_grad<T>(D, y, S.pdense.template as<T>(), n, z, S.pos.template as<T>(), s);
      mark(k, 2);
      mark(k, 3);
      launch_update<T>(D, y, S.pos.template as<T>(), nullptr, S.uy.template as<T>(), S.gains.template as<T>(), n,
                       nullptr, T(0), lr, mom, S.us, s);
    }
    launch_recenter_bbox<T>(D, y, n, S.us.mean(), true, S.bh, bits, s);
    mark(k, 4);
    epoch_tail<T>(t, epoch, snap);
    t->cursor += 1;
  }
  BHG_CUDA(cudaEventRecord(e1, s));
  BHG_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  BHG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  BHG_CUDA(cudaEventDestroy(e0));
  BHG_CUDA(cudaEventDestroy(e1));
  t->loop_ms = ms;
  t->loop_epochs = epochs;
  t->relayout_ms = 0;
  t->relayouts = (int64_t)rl_ev.size() / 2;
  for (size_t i = 0; i + 1 < rl_ev.size(); i += 2) {
    float rm = 0;
    BHG_CUDA(cudaEventElapsedTime(&rm, rl_ev[i], rl_ev[i + 1]));
    t->relayout_ms += rm;
  }
  for (auto& e : rl_ev) cudaEventDestroy(e);
  if (prof) {
    for (int ph = 0; ph < BHTSNE_PHASES; ++ph) t->phase_ms[ph] = 0;
    for (int64_t k = 0; k < epochs; ++k)
      for (int ph = 0; ph < BHTSNE_PHASES; ++ph) {
        float pm = 0;
        BHG_CUDA(cudaEventElapsedTime(&pm, ev[(size_t)k * (BHTSNE_PHASES + 1) + ph],
                                      ev[(size_t)k * (BHTSNE_PHASES + 1) + ph + 1]));
        t->phase_ms[ph] += pm;
      }
    for (auto& e : ev) cudaEventDestroy(e);
    t->phase_epochs = epochs;
  }
  // the Barnes-Hut tree builds of large fits sort with look-back waits; one
  // that ran out (a fault, not slowness) left an unsorted tree: report it
  if (t->loop_kind == BHTSNE_METHOD_BARNES_HUT && n >= kOnesweepMin && radix_sort_fault_take(s))
    throw Error(ST_ETIMEDOUT, "error: a radix sort look-back wait timed out.");
}

template <class T>
void run_loop(bhtsne_tsne* t, int kind, double theta) {
  t->drop_graph();
  st<T>(t).rn.active = false;  // the fit starts from y in the caller's order
  ++st<T>(t).layout_gen;
  // Component layout for Barnes-Hut fits of large, clustered inputs: at the
  // first periodic re-layout point, when P's graph splits into components of
  // at most n / 4 points, the points are grouped by component once (every
  // row's columns then lie within its component's slots) instead of being
  // re-laid out in Morton order every 50 epochs (maybe_renumber).
  // BHTSNE_COMPONENT_LAYOUT=0 turns it off, =2 lifts the size threshold.
  {
    State<T>& S = st<T>(t);
    const char* cl = getenv("BHTSNE_COMPONENT_LAYOUT");
    const bool comp_off = cl && atoi(cl) == 0;
    const bool comp_force = cl && atoi(cl) == 2;
    S.comp_mode = false;
    S.comp_decided = false;
    S.comp_largest = 0;
    S.comp_eligible = !comp_off && kind == BHTSNE_METHOD_BARNES_HUT && S.has_sparse && (t->D == 2 || t->D == 3) &&
                      (comp_force || t->n >= kComponentMinN);
    t->comp_layout = false;
    t->comp_largest = 0;
  }
  // launch shapes of this fit: tuned for (T, D, N) on this device, or the defaults
  const TuneKnobs kn = tune_lookup(t->dtype, t->D, t->n);
  st<T>(t).task_len = kn.attr_task_len;
  st<T>(t).bh.traverse_threads = kn.bh_threads;
  t->armed = true;
  t->loop_kind = kind;
  t->loop_theta = theta;
  t->loop_lr = (double)resolve_lr<T>(t);
  t->cursor = 0;
  advance_impl<T>(t, t->epochs);
  t->fit = kind;
  t->fit_theta = theta;
}

template <class T>
bool has_cached_affinities(bhtsne_tsne* t) {
  State<T>& S = st<T>(t);
  return S.has_sparse && S.sparse_rows == t->n + 1 && t->has_cached_perplexity &&
         t->cached_perplexity == t->perplexity;
}

// prepare_cached + run_cached: src/lib.rs:1227-1248.
template <class T>
void run_cached(bhtsne_tsne* t, int kind, double theta) {
  t->stop_lying_fired = false;
  ensure_state<T>(t);
  finalize_p_and_seed<T>(t, false);
  run_loop<T>(t, kind, theta);
}

template <class T>
void timed_affinities(bhtsne_tsne* t, const std::function<void()>& f) {
  cudaStream_t s = t->ctx->stream;
  cudaEvent_t e0, e1;
  BHG_CUDA(cudaEventCreate(&e0));
  BHG_CUDA(cudaEventCreate(&e1));
  BHG_CUDA(cudaEventRecord(e0, s));
  f();
  BHG_CUDA(cudaEventRecord(e1, s));
  BHG_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  BHG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  t->aff_ms = ms;
}

// barnes_hut / fit_sne over a dense Euclidean dataset: src/lib.rs:701-742, :835-871.
template <class T>
void fit_euclidean(bhtsne_tsne* t, int kind, double theta, const void* data, int32_t dim) {
  if (kind == BHTSNE_METHOD_BARNES_HUT) validate_fit_params(t, theta);
  else check_perplexity(t);
  if (has_cached_affinities<T>(t)) {
    run_cached<T>(t, kind, theta);
    return;
  }
  if (!data || dim <= 0) invalid("error: data must be a non-empty n_samples x dim array.");
  State<T>& S = st<T>(t);
  ensure_state<T>(t);
  cudaStream_t s = t->ctx->stream;
  const int64_t n = t->n;
  const int64_t k = (int64_t)((T)3.0 * (T)t->perplexity);
  timed_affinities<T>(t, [&] {
    upload<T>(S.xin, data, (size_t)n * dim * sizeof(T), s);
    S.kidx.ensure(n * k * 4);
    S.kdist.ensure(n * k * sizeof(T));
    S.knn.pass = tune_lookup(t->dtype, t->D, n).knn_pass;
    t->ctx->knn_fallback_rows = knn_euclidean<T>(S.xin.template as<T>(), n, dim, (int)k,
                                                 S.kidx.template as<uint32_t>(), S.kdist.template as<T>(), S.knn, s);
    t->ctx->knn_brute_rows = S.knn.last_brute_rows;
    S.xin.release();
    S.knn.release();
    build_affinities<T>(t, k);
  });
  S.kidx.release();
  S.kdist.release();
  finalize_p_and_seed<T>(t, false);
  run_loop<T>(t, kind, theta);
}

// *_with_neighbors: src/lib.rs:757-772, :884-894, :922-951.
template <class T>
void fit_with_neighbors(bhtsne_tsne* t, int kind, double theta, const uint64_t* idx, const void* dist, int64_t rows,
                        int64_t k) {
  if (kind == BHTSNE_METHOD_BARNES_HUT) validate_fit_params(t, theta);
  const int64_t n = t->n;
  if (rows != n)
    invalid("error: neighbors has " + std::to_string(rows) + " rows, expected one per sample = " + std::to_string(n));
  if (k <= 0 || !idx || !dist) invalid("error: every neighbors row must have the same length, greater than zero.");
  State<T>& S = st<T>(t);
  ensure_state<T>(t);
  cudaStream_t s = t->ctx->stream;
  // Indices are compared and stored as u32 (the reference's `index as u32`).
  std::vector<uint32_t> idx32((size_t)(n * k));
  bool in_range = true;
  for (int64_t e = 0; e < n * k; ++e) {
    idx32[e] = (uint32_t)idx[e];
    in_range &= idx[e] < (uint64_t)n;
  }
  S.kidx.ensure(n * k * 4);
  BHG_CUDA(cudaMemcpyAsync(S.kidx.ptr, idx32.data(), n * k * 4, cudaMemcpyHostToDevice, s));
  // cached_affinities_match_neighbors: src/lib.rs:1201-1220.
  if (S.has_sparse && S.sparse_rows == n + 1 && t->has_cached_perplexity && t->cached_perplexity == t->perplexity) {
    int* mm = static_cast<int*>(S.tmp2.ensure(64));
    BHG_CUDA(cudaMemsetAsync(mm, 0, 4, s));
    match_neighbors_kernel<<<(unsigned)ceil_div(n * k, 256), 256, 0, s>>>(S.rows.template as<uint64_t>(),
                                                                          S.cols.template as<uint32_t>(), n, k,
                                                                          S.kidx.template as<uint32_t>(), mm);
    BHG_LAUNCH_CHECK();
    int h = 1;
    BHG_CUDA(cudaMemcpyAsync(&h, mm, 4, cudaMemcpyDeviceToHost, s));
    BHG_CUDA(cudaStreamSynchronize(s));
    if (h == 0) {
      S.kidx.release();
      run_cached<T>(t, kind, theta);
      return;
    }
  }
  if (!in_range)
    invalid("error: a neighbor index is out of range, every index must be < n_samples = " + std::to_string(n) + ".");
  timed_affinities<T>(t, [&] {
    upload<T>(S.kdist, dist, (size_t)n * k * sizeof(T), s);
    build_affinities<T>(t, k);
  });
  S.kidx.release();
  S.kdist.release();
  finalize_p_and_seed<T>(t, false);
  run_loop<T>(t, kind, theta);
}

// exact: src/lib.rs:489-646, given the dense distance matrix on the device in S.pdense.
template <class T>
void exact_from_device_distances(bhtsne_tsne* t) {
  State<T>& S = st<T>(t);
  cudaStream_t s = t->ctx->stream;
  const int64_t n = t->n;
  timed_affinities<T>(t, [&] {
    // search_beta over full rows, diagonal (distance 0) included.
    S.kp.ensure(n * n * sizeof(T));
    launch_search_beta<T>(S.pdense.template as<T>(), n, n, (T)t->perplexity, S.kp.template as<T>(), nullptr, s);
    S.pdense.swap(S.kp);
    S.kp.release();
    launch_dense_symmetrize<T>(S.pdense.template as<T>(), n, s);
  });
  S.has_dense = true;
  // The reference reuses p_values for the dense matrix; the sparse cache is
  // no longer valid after an exact fit.
  S.has_sparse = false;
  finalize_p_and_seed<T>(t, true);
  run_loop<T>(t, BHTSNE_METHOD_EXACT, 0.0);
}

template <class T>
void exact_euclidean(bhtsne_tsne* t, const void* data, int32_t dim, int32_t squared) {
  check_perplexity(t);
  if (!data || dim <= 0) invalid("error: data must be a non-empty n_samples x dim array.");
  State<T>& S = st<T>(t);
  ensure_state<T>(t);
  cudaStream_t s = t->ctx->stream;
  const int64_t n = t->n;
  upload<T>(S.xin, data, (size_t)n * dim * sizeof(T), s);
  S.pdense.ensure(n * n * sizeof(T));
  launch_dense_distance<T>(S.xin.template as<T>(), n, dim, squared != 0, S.pdense.template as<T>(), s);
  S.xin.release();
  exact_from_device_distances<T>(t);
}

template <class T>
__global__ void mirror_upper_kernel(T* d, int64_t n) {
  const int64_t i = blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || j >= n) return;
  if (j == i) d[i * n + j] = T(0);
  else if (j < i) d[i * n + j] = d[j * n + i];
}

template <class T>
void exact_distances(bhtsne_tsne* t, const void* dist) {
  check_perplexity(t);
  State<T>& S = st<T>(t);
  ensure_state<T>(t);
  cudaStream_t s = t->ctx->stream;
  const int64_t n = t->n;
  upload<T>(S.pdense, dist, (size_t)n * n * sizeof(T), s);
  dim3 g((unsigned)ceil_div(n, 256), (unsigned)n);
  mirror_upper_kernel<T><<<g, 256, 0, s>>>(S.pdense.template as<T>(), n);
  BHG_LAUNCH_CHECK();
  exact_from_device_distances<T>(t);
}

// kl_divergence: src/lib.rs:448-477.
template <class T>
bool kl(bhtsne_tsne* t, bool quirk, double* out) {
  if (t->fit == 0) return false;
  State<T>& S = st<T>(t);
  cudaStream_t s = t->ctx->stream;
  const int64_t n = t->n;
  const int D = t->D;
  T* y = const_cast<T*>(S.y_external(s));
  double* z = S.klbuf.template as<double>();
  double* res = z + 1;
  if (t->fit == BHTSNE_METHOD_EXACT) {
    launch_exact_z<T>(D, y, n, z, S.tmp, s);
    launch_exact_kl<T>(D, y, S.pdense.template as<T>(), n, z, res, S.tmp2, s);
  } else {
    S.bh.reserve(n, D);
    if (t->fit == BHTSNE_METHOD_BARNES_HUT) {
      launch_recenter_bbox<T>(D, y, n, nullptr, false, S.bh, bh_bits<T>(D), s);
      bh_build<T>(S.bh, D, y, n, s);
      bh_traverse<T>(S.bh, D, y, n, (T)t->fit_theta, S.neg.template as<T>(), nullptr, s);
      BHG_CUDA(cudaMemcpyAsync(z, S.bh.z(), sizeof(double), cudaMemcpyDeviceToDevice, s));
    } else {
      launch_recenter_bbox<T>(D, y, n, nullptr, false, S.bh, 32, s);
      fit_repulsion<T>(S.fit, D, y, n, S.bh.params.template as<BoxParams<T>>(), S.neg.template as<T>(), z, s);
    }
    launch_kl_sparse<T>(D, S.rows.template as<uint64_t>(), S.cols.template as<uint32_t>(), S.vals.template as<T>(), y, n,
                        z, quirk, res, S.tmp2, s);
  }
  BHG_CUDA(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, s));
  BHG_CUDA(cudaStreamSynchronize(s));
  return true;
}

template <class T>
void new_state(bhtsne_tsne* t);
template <>
void new_state<float>(bhtsne_tsne* t) {
  t->sf = new State<float>();
}
template <>
void new_state<double>(bhtsne_tsne* t) {
  t->sd = new State<double>();
}

#define DISPATCH(t, ...)            \
  do {                              \
    if ((t)->dtype == BHTSNE_F32) { \
      typedef float T;              \
      __VA_ARGS__;                  \
    } else {                        \
      typedef double T;             \
      __VA_ARGS__;                  \
    }                               \
  } while (0)

#define DISPATCH_DT(dt, ...)   \
  do {                         \
    if ((dt) == BHTSNE_F32) {  \
      typedef float T;         \
      __VA_ARGS__;             \
    } else {                   \
      typedef double T;        \
      __VA_ARGS__;             \
    }                          \
  } while (0)

}  // namespace

// ===========================================================================
extern "C" {

const char* bhtsne_version(void) { return kVersion; }

int bhtsne_ctx_create(int device, bhtsne_ctx** out) {
  if (!out) return BHTSNE_EINVAL;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return BHTSNE_ECUDA;
  if (device < 0 || device >= count) return BHTSNE_EINVAL;
  bhtsne_ctx* c = new bhtsne_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return BHTSNE_ECUDA;
  }
  keep_pool_cached(device);
  tune_load_env_once();
  *out = c;
  return BHTSNE_OK;
}

int bhtsne_ctx_destroy(bhtsne_ctx* ctx) {
  if (!ctx) return BHTSNE_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return BHTSNE_OK;
}

const char* bhtsne_ctx_last_error(const bhtsne_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int bhtsne_tune(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, int64_t n, int32_t k, int32_t dim) {
  std::string report;
  const int rc = guard_ctx(ctx, [&] {
    if (dtype != BHTSNE_F32 && dtype != BHTSNE_F64) invalid("error: dtype must be BHTSNE_F32 or BHTSNE_F64.");
    tune_run(dtype, embed_dim, n, k, dim, ctx->stream, &report);
  });
  if (rc == BHTSNE_OK) ctx->err = report;  // the timings, readable through bhtsne_ctx_last_error
  return rc;
}

int bhtsne_ctx_knn_fallback_rows(const bhtsne_ctx* ctx, int64_t* rows) {
  if (!ctx || !rows) return BHTSNE_EINVAL;
  *rows = ctx->knn_fallback_rows;
  return BHTSNE_OK;
}

int bhtsne_ctx_knn_brute_rows(const bhtsne_ctx* ctx, int64_t* rows) {
  if (!ctx || !rows) return BHTSNE_EINVAL;
  *rows = ctx->knn_brute_rows;
  return BHTSNE_OK;
}

int bhtsne_tsne_new(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, int64_t n_samples, bhtsne_tsne** out) {
  if (!ctx || !out) return BHTSNE_EINVAL;
  *out = nullptr;
  if (dtype != BHTSNE_F32 && dtype != BHTSNE_F64) {
    ctx->err = "error: dtype must be BHTSNE_F32 or BHTSNE_F64.";
    return BHTSNE_EINVAL;
  }
  if (embed_dim < 1 || embed_dim > 7) {
    ctx->err = "error: the embedding dimension must be in 1..7.";
    return BHTSNE_EINVAL;
  }
  if (n_samples < 0 || n_samples > 0x7fffffffLL) {
    ctx->err = "error: n_samples must be in [0, 2^31).";
    return BHTSNE_EINVAL;
  }
  bhtsne_tsne* t = new bhtsne_tsne();
  t->ctx = ctx;
  t->dtype = dtype;
  t->D = embed_dim;
  t->n = n_samples;
  t->momentum = tcast(t, 0.5);
  t->final_momentum = tcast(t, 0.8);
  t->early_exaggeration = tcast(t, 12.0);
  t->perplexity = tcast(t, 20.0);
  DISPATCH(t, new_state<T>(t));
  *out = t;
  return BHTSNE_OK;
}

int bhtsne_tsne_free(bhtsne_tsne* t) {
  if (!t) return BHTSNE_OK;
  cudaSetDevice(t->ctx->device);
  t->drop_graph();
  delete t->sf;
  delete t->sd;
  delete t;
  return BHTSNE_OK;
}

const char* bhtsne_tsne_last_error(const bhtsne_tsne* t) { return t ? t->err.c_str() : "null handle"; }

int bhtsne_tsne_learning_rate(bhtsne_tsne* t, double v) {
  if (!t) return BHTSNE_EINVAL;
  t->has_lr = true;
  t->lr = tcast(t, v);
  return BHTSNE_OK;
}
int bhtsne_tsne_epochs(bhtsne_tsne* t, int64_t v) {
  if (!t || v < 0) return BHTSNE_EINVAL;
  t->epochs = v;
  return BHTSNE_OK;
}
int bhtsne_tsne_momentum(bhtsne_tsne* t, double v) {
  if (!t) return BHTSNE_EINVAL;
  t->momentum = tcast(t, v);
  return BHTSNE_OK;
}
int bhtsne_tsne_final_momentum(bhtsne_tsne* t, double v) {
  if (!t) return BHTSNE_EINVAL;
  t->final_momentum = tcast(t, v);
  return BHTSNE_OK;
}
int bhtsne_tsne_momentum_switch_epoch(bhtsne_tsne* t, int64_t v) {
  if (!t || v < 0) return BHTSNE_EINVAL;
  t->momentum_switch_epoch = v;
  return BHTSNE_OK;
}
int bhtsne_tsne_stop_lying_epoch(bhtsne_tsne* t, int64_t v) {
  if (!t || v < 0) return BHTSNE_EINVAL;
  t->stop_lying_epoch = v;
  return BHTSNE_OK;
}
int bhtsne_tsne_early_exaggeration(bhtsne_tsne* t, double v) {
  if (!t) return BHTSNE_EINVAL;
  t->early_exaggeration = tcast(t, v);
  return BHTSNE_OK;
}
int bhtsne_tsne_perplexity(bhtsne_tsne* t, double v) {
  if (!t) return BHTSNE_EINVAL;
  t->perplexity = tcast(t, v);
  return BHTSNE_OK;
}
int bhtsne_tsne_epoch_callback(bhtsne_tsne* t, bhtsne_epoch_cb cb, void* user) {
  if (!t) return BHTSNE_EINVAL;
  t->cb = cb;
  t->user = user;
  return BHTSNE_OK;
}
int bhtsne_tsne_initial_embedding(bhtsne_tsne* t, const void* y, int64_t len) {
  if (!t || len < 0 || (len > 0 && !y)) return BHTSNE_EINVAL;
  const size_t es = t->dtype == BHTSNE_F32 ? 4 : 8;
  t->init.assign((const unsigned char*)y, (const unsigned char*)y + (size_t)len * es);
  t->init_len = len;
  t->has_init = true;
  return BHTSNE_OK;
}
int bhtsne_tsne_random_seed(bhtsne_tsne* t, uint64_t seed) {
  if (!t) return BHTSNE_EINVAL;
  t->seed = seed;
  return BHTSNE_OK;
}

int bhtsne_tsne_exact_euclidean(bhtsne_tsne* t, const void* data, int32_t dim, int32_t squared) {
  return guard(t, [&] { DISPATCH(t, exact_euclidean<T>(t, data, dim, squared)); });
}
int bhtsne_tsne_exact_distances(bhtsne_tsne* t, const void* distances) {
  return guard(t, [&] {
    if (!distances) invalid("error: distances must be an n_samples x n_samples array.");
    DISPATCH(t, exact_distances<T>(t, distances));
  });
}
int bhtsne_tsne_barnes_hut_euclidean(bhtsne_tsne* t, double theta, const void* data, int32_t dim) {
  return guard(t, [&] {
    if (t->D < 2 || t->D > 7) invalid("error: Barnes-Hut covers D in 2..7.");
    DISPATCH(t, fit_euclidean<T>(t, BHTSNE_METHOD_BARNES_HUT, tcast(t, theta), data, dim));
  });
}
int bhtsne_tsne_barnes_hut_with_neighbors(bhtsne_tsne* t, double theta, const uint64_t* indices, const void* distances,
                                          int64_t rows, int64_t k) {
  return guard(t, [&] {
    if (t->D < 2 || t->D > 7) invalid("error: Barnes-Hut covers D in 2..7.");
    DISPATCH(t, fit_with_neighbors<T>(t, BHTSNE_METHOD_BARNES_HUT, tcast(t, theta), indices, distances, rows, k));
  });
}
int bhtsne_tsne_fit_sne_euclidean(bhtsne_tsne* t, const void* data, int32_t dim) {
  return guard(t, [&] {
    if (t->D < 1 || t->D > 2) invalid("error: FIt-SNE is restricted to D in {1, 2}.");
    DISPATCH(t, fit_euclidean<T>(t, BHTSNE_METHOD_FIT_SNE, 0.0, data, dim));
  });
}
int bhtsne_tsne_fit_sne_with_neighbors(bhtsne_tsne* t, const uint64_t* indices, const void* distances, int64_t rows,
                                       int64_t k) {
  return guard(t, [&] {
    if (t->D < 1 || t->D > 2) invalid("error: FIt-SNE is restricted to D in {1, 2}.");
    DISPATCH(t, fit_with_neighbors<T>(t, BHTSNE_METHOD_FIT_SNE, 0.0, indices, distances, rows, k));
  });
}

int bhtsne_tsne_write_csv(bhtsne_tsne* t, const char* path) {
  return guard(t, [&] {
    if (!path) invalid("error: the path is null.");
    DISPATCH(t, {
      State<T>& S = st<T>(t);
      const size_t bytes = (size_t)t->n * t->D * sizeof(T);
      // before a fit the reference's embedding is empty: only the header is written
      const bool fitted = S.y.ptr && S.y.bytes >= bytes;
      std::vector<T> h(fitted ? (size_t)t->n * t->D : 0);
      if (fitted) {
        BHG_CUDA(cudaMemcpyAsync(h.data(), S.y_external(t->ctx->stream), bytes, cudaMemcpyDeviceToHost,
                                 t->ctx->stream));
        BHG_CUDA(cudaStreamSynchronize(t->ctx->stream));
      }
      const int rc = write_csv_file(h.data(), fitted ? t->n : 0, t->D, t->dtype, path);
      if (rc != BHTSNE_OK) throw Error(rc, bhtsne_io_last_error());
    });
  });
}

int bhtsne_tsne_embedding(bhtsne_tsne* t, void* out) {
  return guard(t, [&] {
    if (!out) invalid("error: output buffer is null.");
    DISPATCH(t, {
      State<T>& S = st<T>(t);
      const size_t bytes = (size_t)t->n * t->D * sizeof(T);
      if (!S.y.ptr || S.y.bytes < bytes) {
        // The reference returns an empty vector before a fit.
        return;
      }
      BHG_CUDA(cudaMemcpyAsync(out, S.y_external(t->ctx->stream), bytes, cudaMemcpyDeviceToHost, t->ctx->stream));
      BHG_CUDA(cudaStreamSynchronize(t->ctx->stream));
    });
  });
}

int bhtsne_tsne_kl_divergence(bhtsne_tsne* t, int32_t quirk, double* out, int32_t* has_value) {
  return guard(t, [&] {
    double v = 0;
    bool has = false;
    DISPATCH(t, has = kl<T>(t, quirk != 0, &v));
    if (has_value) *has_value = has ? 1 : 0;
    if (out && has) *out = v;
  });
}

int bhtsne_tsne_affinities(bhtsne_tsne* t, uint64_t* rows, uint32_t* columns, void* values, int64_t* nnz,
                           double* perplexity, int32_t* has_value) {
  return guard(t, [&] {
    DISPATCH(t, {
      State<T>& S = st<T>(t);
      if (has_value) *has_value = S.has_sparse ? 1 : 0;
      if (!S.has_sparse) return;
      if (nnz) *nnz = S.nnz;
      if (perplexity) *perplexity = t->perplexity;
      cudaStream_t s = t->ctx->stream;
      if (rows) BHG_CUDA(cudaMemcpyAsync(rows, S.rows.ptr, S.sparse_rows * 8, cudaMemcpyDeviceToHost, s));
      if (columns) BHG_CUDA(cudaMemcpyAsync(columns, S.cols.ptr, S.nnz * 4, cudaMemcpyDeviceToHost, s));
      if (values) {
        if (t->stop_lying_fired) {
          BHG_CUDA(cudaMemcpyAsync(values, S.vals.ptr, S.nnz * sizeof(T), cudaMemcpyDeviceToHost, s));
        } else {
          T* tmp = static_cast<T*>(S.tmp2.ensure(std::max<int64_t>(S.nnz, 1) * sizeof(T)));
          launch_scaled_copy<T>(S.vals.template as<T>(), S.nnz, T(1) / (T)t->early_exaggeration, tmp, s);
          BHG_CUDA(cudaMemcpyAsync(values, tmp, S.nnz * sizeof(T), cudaMemcpyDeviceToHost, s));
        }
      }
      BHG_CUDA(cudaStreamSynchronize(s));
    });
  });
}

int bhtsne_tsne_with_affinities(bhtsne_tsne* t, const uint64_t* rows, int64_t n_rows, const uint32_t* columns,
                                const void* values, int64_t nnz, double perplexity) {
  return guard(t, [&] {
    if (n_rows < 1 || nnz < 0 || !rows || (nnz > 0 && (!columns || !values)))
      invalid("error: affinities must hold row offsets, columns and values.");
    DISPATCH(t, {
      State<T>& S = st<T>(t);
      ensure_state<T>(t);
      cudaStream_t s = t->ctx->stream;
      upload<T>(S.rows, rows, n_rows * 8, s);
      S.cols.ensure(std::max<int64_t>(nnz, 1) * 4);
      S.vals.ensure(std::max<int64_t>(nnz, 1) * sizeof(T));
      if (nnz > 0) {
        BHG_CUDA(cudaMemcpyAsync(S.cols.ptr, columns, nnz * 4, cudaMemcpyHostToDevice, s));
        BHG_CUDA(cudaMemcpyAsync(S.vals.ptr, values, nnz * sizeof(T), cudaMemcpyHostToDevice, s));
      }
      BHG_CUDA(cudaStreamSynchronize(s));
      S.nnz = nnz;
      S.sparse_rows = n_rows;
      S.has_sparse = true;
      t->perplexity = tcast(t, perplexity);
      t->has_cached_perplexity = true;
      t->cached_perplexity = t->perplexity;
    });
  });
}

int bhtsne_tsne_advance(bhtsne_tsne* t, int64_t epochs) {
  return guard(t, [&] {
    if (!t->armed) invalid("error: advance needs a completed fit on this handle.");
    if (epochs < 0) invalid("error: epochs must be >= 0.");
    DISPATCH(t, advance_impl<T>(t, epochs));
  });
}

int bhtsne_tsne_profile(bhtsne_tsne* t, int32_t enable) {
  if (!t) return BHTSNE_EINVAL;
  t->profile = enable != 0;
  return BHTSNE_OK;
}

int bhtsne_tsne_layout_info(const bhtsne_tsne* t, int32_t* component_layout, int64_t* largest_component) {
  if (!t) return BHTSNE_EINVAL;
  if (component_layout) *component_layout = t->comp_layout ? 1 : 0;
  if (largest_component) *largest_component = t->comp_largest;
  return BHTSNE_OK;
}

int bhtsne_tsne_relayout_times(const bhtsne_tsne* t, double* ms, int64_t* count) {
  if (!t) return BHTSNE_EINVAL;
  if (ms) *ms = t->relayout_ms;
  if (count) *count = t->relayouts;
  return BHTSNE_OK;
}

int bhtsne_tsne_phase_times(const bhtsne_tsne* t, double* ms, int64_t* epochs) {
  if (!t) return BHTSNE_EINVAL;
  if (ms)
    for (int ph = 0; ph < BHTSNE_PHASES; ++ph) ms[ph] = t->phase_ms[ph];
  if (epochs) *epochs = t->phase_epochs;
  return BHTSNE_OK;
}

int64_t bhtsne_launch_count(void) { return (int64_t)g_launches.load(); }

int bhtsne_tsne_timings(const bhtsne_tsne* t, double* affinity_ms, double* loop_ms, int64_t* loop_epochs) {
  if (!t) return BHTSNE_EINVAL;
  if (affinity_ms) *affinity_ms = t->aff_ms;
  if (loop_ms) *loop_ms = t->loop_ms;
  if (loop_epochs) *loop_epochs = t->loop_epochs;
  return BHTSNE_OK;
}

// ---- stage entry points ----------------------------------------------------
int bhtsne_knn_euclidean(bhtsne_ctx* ctx, int dtype, const void* data, int64_t n, int32_t dim, int32_t k,
                         uint32_t* indices, void* distances) {
  return guard_ctx(ctx, [&] {
    if (!data || !indices || !distances || n < 2 || dim <= 0) invalid("error: invalid kNN arguments.");
    DISPATCH_DT(dtype, {
      cudaStream_t s = ctx->stream;
      DevBuf x, idx, dist;
      KnnWorkspace ws;
      upload<T>(x, data, (size_t)n * dim * sizeof(T), s);
      idx.ensure((size_t)n * k * 4);
      dist.ensure((size_t)n * k * sizeof(T));
      ctx->knn_fallback_rows = knn_euclidean<T>(x.as<T>(), n, dim, k, idx.as<uint32_t>(), dist.as<T>(), ws, s);
      ctx->knn_brute_rows = ws.last_brute_rows;
      BHG_CUDA(cudaMemcpyAsync(indices, idx.ptr, (size_t)n * k * 4, cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaMemcpyAsync(distances, dist.ptr, (size_t)n * k * sizeof(T), cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaStreamSynchronize(s));
    });
  });
}

int bhtsne_conditional_p(bhtsne_ctx* ctx, int dtype, const void* distances, int64_t n, int32_t k, double perplexity,
                         void* p, int32_t* iterations) {
  return guard_ctx(ctx, [&] {
    if (!distances || !p || n < 0 || k <= 0) invalid("error: invalid conditional P arguments.");
    DISPATCH_DT(dtype, {
      cudaStream_t s = ctx->stream;
      DevBuf d, out, it;
      upload<T>(d, distances, (size_t)n * k * sizeof(T), s);
      out.ensure((size_t)n * k * sizeof(T));
      if (iterations) it.ensure((size_t)n * 4);
      launch_search_beta<T>(d.as<T>(), n, k, (T)perplexity, out.as<T>(), iterations ? it.as<int32_t>() : nullptr, s);
      BHG_CUDA(cudaMemcpyAsync(p, out.ptr, (size_t)n * k * sizeof(T), cudaMemcpyDeviceToHost, s));
      if (iterations) BHG_CUDA(cudaMemcpyAsync(iterations, it.ptr, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaStreamSynchronize(s));
    });
  });
}

int bhtsne_symmetrize(bhtsne_ctx* ctx, int dtype, const uint32_t* columns, const void* p, int64_t n, int32_t k,
                      uint64_t* rows_out, uint32_t* columns_out, void* values_out, int64_t* nnz) {
  return guard_ctx(ctx, [&] {
    if (!columns || !p || n < 1 || k <= 0) invalid("error: invalid symmetrize arguments.");
    DISPATCH_DT(dtype, {
      cudaStream_t s = ctx->stream;
      DevBuf c, v, r, co, vo;
      SymWorkspace<T> ws;
      upload<T>(c, columns, (size_t)n * k * 4, s);
      upload<T>(v, p, (size_t)n * k * sizeof(T), s);
      const int64_t m = symmetrize<T>(c.as<uint32_t>(), v.as<T>(), n, k, ws, s);
      if (nnz) *nnz = m;
      if (rows_out || columns_out || values_out) {
        r.ensure((n + 1) * 8);
        co.ensure(std::max<int64_t>(m, 1) * 4);
        vo.ensure(std::max<int64_t>(m, 1) * sizeof(T));
        symmetrize_finish<T>(ws, n, m, r.as<uint64_t>(), co.as<uint32_t>(), vo.as<T>(), s);
        if (rows_out) BHG_CUDA(cudaMemcpyAsync(rows_out, r.ptr, (n + 1) * 8, cudaMemcpyDeviceToHost, s));
        if (columns_out && m) BHG_CUDA(cudaMemcpyAsync(columns_out, co.ptr, m * 4, cudaMemcpyDeviceToHost, s));
        if (values_out && m) BHG_CUDA(cudaMemcpyAsync(values_out, vo.ptr, m * sizeof(T), cudaMemcpyDeviceToHost, s));
      }
      BHG_CUDA(cudaStreamSynchronize(s));
    });
  });
}

int bhtsne_gradient(bhtsne_ctx* ctx, int dtype, int32_t method, int32_t embed_dim, const void* y, int64_t n,
                    const uint64_t* rows, const uint32_t* columns, const void* values, int64_t nnz, double theta,
                    void* pos, void* neg, double* z) {
  return guard_ctx(ctx, [&] {
    if (!y || n < 1 || !pos) invalid("error: invalid gradient arguments.");
    if (embed_dim < 1 || embed_dim > 7) invalid("error: the embedding dimension must be in 1..7.");
    DISPATCH_DT(dtype, {
      cudaStream_t s = ctx->stream;
      const int D = embed_dim;
      DevBuf yd, rd, cd, vd, pd, nd, zd, tmp;
      BhWorkspace<T> bh;
      FitWorkspace<T> fw;
      const TuneKnobs kn = tune_lookup(dtype, D, n);
      bh.traverse_threads = kn.bh_threads;
      upload<T>(yd, y, (size_t)n * D * sizeof(T), s);
      pd.ensure((size_t)n * D * sizeof(T));
      nd.ensure((size_t)n * D * sizeof(T));
      zd.ensure(64);
      if (method == BHTSNE_METHOD_EXACT) {
        upload<T>(vd, values, (size_t)n * n * sizeof(T), s);
        launch_exact_z<T>(D, yd.as<T>(), n, zd.as<double>(), tmp, s);
        launch_exact_grad<T>(D, yd.as<T>(), vd.as<T>(), n, zd.as<double>(), pd.as<T>(), s);
      } else {
        if (!rows || (nnz > 0 && (!columns || !values))) invalid("error: the sparse affinities are required.");
        upload<T>(rd, rows, (size_t)(n + 1) * 8, s);
        upload<T>(cd, columns, (size_t)std::max<int64_t>(nnz, 0) * 4, s);
        upload<T>(vd, values, (size_t)std::max<int64_t>(nnz, 0) * sizeof(T), s);
        bh.reserve(n, D);
        if (method == BHTSNE_METHOD_BARNES_HUT) {
          if (D < 2) invalid("error: Barnes-Hut covers D in 2..7.");
          if (!(theta > 0)) invalid("error: theta value must be greater than 0.0.");
          launch_recenter_bbox<T>(D, yd.as<T>(), n, nullptr, false, bh, bh_bits<T>(D), s);
          bh_build<T>(bh, D, yd.as<T>(), n, s);
          bh_traverse<T>(bh, D, yd.as<T>(), n, (T)theta, nd.as<T>(), nullptr, s);
          BHG_CUDA(cudaMemcpyAsync(zd.ptr, bh.z(), 8, cudaMemcpyDeviceToDevice, s));
        } else if (method == BHTSNE_METHOD_FIT_SNE) {
          if (D > 2) invalid("error: FIt-SNE is restricted to D in {1, 2}.");
          launch_recenter_bbox<T>(D, yd.as<T>(), n, nullptr, false, bh, 32, s);
          fit_repulsion<T>(fw, D, yd.as<T>(), n, bh.params.template as<BoxParams<T>>(), nd.as<T>(), zd.as<double>(), s);
        } else {
          invalid("error: unknown method.");
        }
        AttrTasks at;
        build_attr_tasks<T>(at, D, rd.as<uint64_t>(), n, s, kn.attr_task_len);
        launch_attractive_tasks<T>(at, cd.as<uint32_t>(), vd.as<T>(), yd.as<T>(), pd.as<T>(), s);
        if (neg) BHG_CUDA(cudaMemcpyAsync(neg, nd.ptr, (size_t)n * D * sizeof(T), cudaMemcpyDeviceToHost, s));
      }
      BHG_CUDA(cudaMemcpyAsync(pos, pd.ptr, (size_t)n * D * sizeof(T), cudaMemcpyDeviceToHost, s));
      double zh = 0;
      BHG_CUDA(cudaMemcpyAsync(&zh, zd.ptr, 8, cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaStreamSynchronize(s));
      if (z) *z = zh;
    });
  });
}

int bhtsne_update(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, void* y, const void* pos, const void* neg, void* uy,
                  void* gains, int64_t n, double learning_rate, double momentum, double inverse_z) {
  return guard_ctx(ctx, [&] {
    if (!y || !pos || !uy || !gains || n < 1) invalid("error: invalid update arguments.");
    if (embed_dim < 1 || embed_dim > 7) invalid("error: the embedding dimension must be in 1..7.");
    DISPATCH_DT(dtype, {
      cudaStream_t s = ctx->stream;
      const int D = embed_dim;
      const size_t bytes = (size_t)n * D * sizeof(T);
      DevBuf yd, pd, nd, ud, gd;
      UpdateScratch us;
      BhWorkspace<T> bh;
      bh.reserve(n, D);
      upload<T>(yd, y, bytes, s);
      upload<T>(pd, pos, bytes, s);
      if (neg) upload<T>(nd, neg, bytes, s);
      upload<T>(ud, uy, bytes, s);
      upload<T>(gd, gains, bytes, s);
      launch_update<T>(D, yd.as<T>(), pd.as<T>(), neg ? nd.as<T>() : nullptr, ud.as<T>(), gd.as<T>(), n, nullptr,
                       (T)inverse_z, (T)learning_rate, (T)momentum, us, s);
      launch_recenter_bbox<T>(D, yd.as<T>(), n, us.mean(), true, bh, 32, s);
      BHG_CUDA(cudaMemcpyAsync(y, yd.ptr, bytes, cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaMemcpyAsync(uy, ud.ptr, bytes, cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaMemcpyAsync(gains, gd.ptr, bytes, cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaStreamSynchronize(s));
    });
  });
}

}  // extern "C"

// ===========================================================================
// Batches of independent fits.
// ===========================================================================
struct bhtsne_batch {
  bhtsne_ctx* ctx = nullptr;
  int dtype = BHTSNE_F32;
  int D = 2;
  bhtsne_batch_params prm;
  std::string err;
  void* impl = nullptr;
};

namespace {

template <class T>
struct BatchJob {
  int64_t n = 0;
  int kind = 0;  // 0: dense Euclidean data, 1: kNN table
  int32_t dim = 0;
  int64_t k = 0;
  DevBuf in_a, in_b;  // data, or (u32 indices, T distances) until prepared
  bool has_init = false;
  std::vector<T> init;
  std::shared_ptr<GroupCsr<T>> group;
  int64_t goff = 0;  // first row of this job in its group
};

template <class T>
struct BatchImpl {
  std::vector<std::unique_ptr<BatchJob<T>>> jobs;
  int K = 0;
  int64_t total = 0, nnz = 0;
  std::vector<int64_t> off, nnz_off;
  DevBuf d_off, job_of, rows, cols, vals, y, uy, gains, pos, neg, q, z, lr, mom, boxes, codes, jobkey, jobkey_alt;
  DevBuf tmp, d_nnz_off;
  AttrTasks at;  // attractive-pass tasks of the block-diagonal CSR
  BhWorkspace<T> ws;
  SegTiles tiles;
  AffinityScratch<T> aff;
  bool fitted = false;
  double aff_ms = 0, loop_ms = 0;
  cudaGraphExec_t graph = nullptr;
  ~BatchImpl() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

template <class F>
int guard_batch(bhtsne_batch* b, F&& f) {
  if (!b) return BHTSNE_EINVAL;
  AllocStreamScope scope(b->ctx->stream);
  try {
    BHG_CUDA(cudaSetDevice(b->ctx->device));
    f();
    return BHTSNE_OK;
  } catch (const Error& e) {
    b->err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    b->err = e.what();
    return BHTSNE_EINTERNAL;
  }
}

template <class T>
BatchImpl<T>& bimpl(bhtsne_batch* b) {
  return *static_cast<BatchImpl<T>*>(b->impl);
}

void batch_check_job(const bhtsne_batch* b, int64_t n) {
  const double perp = b->prm.perplexity;
  const int64_t as_usize = perp > 0 ? (int64_t)perp : 0;
  if (n < 2 || (n - 1) < 3 * as_usize)
    invalid("error: the provided perplexity is too large for the number of data points.\n");
}

template <class T>
int64_t batch_add_with_neighbors(bhtsne_batch* b, const uint64_t* idx, const void* dist, int64_t n, int64_t k) {
  BatchImpl<T>& B = bimpl<T>(b);
  batch_check_job(b, n);
  if (k <= 0 || !idx || !dist) invalid("error: every neighbors row must have the same length, greater than zero.");
  std::vector<uint32_t> idx32((size_t)(n * k));
  for (int64_t e = 0; e < n * k; ++e) {
    if (idx[e] >= (uint64_t)n)
      invalid("error: a neighbor index is out of range, every index must be < n_samples = " + std::to_string(n) + ".");
    idx32[e] = (uint32_t)idx[e];
  }
  cudaStream_t s = b->ctx->stream;
  auto job = std::make_unique<BatchJob<T>>();
  job->n = n;
  job->kind = 1;
  job->k = k;
  upload<T>(job->in_a, idx32.data(), (size_t)n * k * 4, s);
  upload<T>(job->in_b, dist, (size_t)n * k * sizeof(T), s);
  BHG_CUDA(cudaStreamSynchronize(s));
  B.jobs.push_back(std::move(job));
  B.fitted = false;
  return (int64_t)B.jobs.size() - 1;
}

template <class T>
int64_t batch_add_euclidean(bhtsne_batch* b, const void* data, int64_t n, int32_t dim) {
  BatchImpl<T>& B = bimpl<T>(b);
  batch_check_job(b, n);
  if (!data || dim <= 0) invalid("error: data must be a non-empty n_samples x dim array.");
  cudaStream_t s = b->ctx->stream;
  auto job = std::make_unique<BatchJob<T>>();
  job->n = n;
  job->kind = 0;
  job->dim = dim;
  job->k = (int64_t)((T)3.0 * (T)b->prm.perplexity);
  upload<T>(job->in_a, data, (size_t)n * dim * sizeof(T), s);
  BHG_CUDA(cudaStreamSynchronize(s));
  B.jobs.push_back(std::move(job));
  B.fitted = false;
  return (int64_t)B.jobs.size() - 1;
}

// Affinities of every job not yet prepared, one group per (input kind, dim or
// k): segmented kNN over the group's concatenated rows (Euclidean jobs), then
// search_beta and symmetrize once over the group (build_affinities,
// src/lib.rs:1061-1127, for every job at once; the block-diagonal structure
// keeps each job's rows, columns and values those of its own fit).
template <class T>
void batch_prepare(bhtsne_batch* b) {
  BatchImpl<T>& B = bimpl<T>(b);
  cudaStream_t s = b->ctx->stream;
  std::vector<std::pair<std::pair<int, int64_t>, std::vector<int>>> groups;
  for (int j = 0; j < (int)B.jobs.size(); ++j) {
    const BatchJob<T>& J = *B.jobs[j];
    if (J.group) continue;
    const std::pair<int, int64_t> key(J.kind, J.kind == 0 ? (int64_t)J.dim * 4096 + J.k : J.k);
    auto it = std::find_if(groups.begin(), groups.end(), [&](const auto& g) { return g.first == key; });
    if (it == groups.end()) groups.push_back({key, {j}});
    else it->second.push_back(j);
  }
  for (auto& gr : groups) {
    const std::vector<int>& js = gr.second;
    const int G = (int)js.size();
    const BatchJob<T>& J0 = *B.jobs[js[0]];
    const int64_t k = J0.k;
    std::vector<int64_t> goff(G + 1, 0), ns(G);
    for (int g = 0; g < G; ++g) {
      ns[g] = B.jobs[js[g]]->n;
      goff[g + 1] = goff[g] + ns[g];
    }
    const int64_t tot = goff[G];
    auto grp = std::make_shared<GroupCsr<T>>();
    if (J0.kind == 0) {
      std::vector<const T*> X(G);
      for (int g = 0; g < G; ++g) X[g] = B.jobs[js[g]]->in_a.template as<T>();
      group_affinities_euclidean<T>(X, ns, J0.dim, k, (T)b->prm.perplexity, *grp, B.aff, s);
    } else {
      uint32_t* kidx = static_cast<uint32_t*>(B.aff.kidx.ensure((size_t)tot * k * 4));
      T* kdist = static_cast<T*>(B.aff.kdist.ensure((size_t)tot * k * sizeof(T)));
      for (int g = 0; g < G; ++g) {
        const BatchJob<T>& J = *B.jobs[js[g]];
        batch_offset_indices(J.in_a.template as<uint32_t>(), J.n * k, (uint32_t)goff[g], kidx + goff[g] * k, s);
        BHG_CUDA(cudaMemcpyAsync(kdist + goff[g] * k, J.in_b.ptr, (size_t)J.n * k * sizeof(T), cudaMemcpyDeviceToDevice,
                                 s));
      }
      group_affinities_from_knn<T>(tot, k, (T)b->prm.perplexity, *grp, B.aff, s);
    }
    for (int g = 0; g < G; ++g) {
      BatchJob<T>& J = *B.jobs[js[g]];
      J.group = grp;
      J.goff = goff[g];
      J.in_a.release();
      J.in_b.release();
    }
  }
  B.aff.release();
}

template <class T>
__global__ void batch_fill_kernel(T* p, int64_t n, T v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

// Lockstep Barnes-Hut fit of every job (run_loop, src/lib.rs:961-1014, per job).
template <class T>
void batch_fit(bhtsne_batch* b) {
  BatchImpl<T>& B = bimpl<T>(b);
  cudaStream_t s = b->ctx->stream;
  const int D = b->D;
  const bhtsne_batch_params& P = b->prm;
  if (B.jobs.empty()) invalid("error: the batch has no jobs.");
  if (!(P.theta > 0))
    invalid("error: theta value must be greater than 0.0.\n            A value of 0.0 corresponds to using the exact "
            "version of the algorithm.");
  cudaEvent_t e0, e1;
  BHG_CUDA(cudaEventCreate(&e0));
  BHG_CUDA(cudaEventCreate(&e1));
  BHG_CUDA(cudaEventRecord(e0, s));
  batch_prepare<T>(b);
  B.K = (int)B.jobs.size();
  B.off.assign(B.K + 1, 0);
  B.nnz_off.assign(B.K + 1, 0);
  for (int j = 0; j < B.K; ++j) {
    const BatchJob<T>& J = *B.jobs[j];
    B.off[j + 1] = B.off[j] + J.n;
    B.nnz_off[j + 1] = B.nnz_off[j] + (int64_t)(J.group->rows_h[J.goff + J.n] - J.group->rows_h[J.goff]);
  }
  B.total = B.off[B.K];
  B.nnz = B.nnz_off[B.K];
  const int64_t total = B.total;
  // block-diagonal CSR of the whole batch, rows and columns renumbered from
  // each job's place in its group to its place in the batch
  B.rows.ensure((size_t)(total + 1) * 8);
  B.cols.ensure((size_t)std::max<int64_t>(B.nnz, 1) * 4);
  B.vals.ensure((size_t)std::max<int64_t>(B.nnz, 1) * sizeof(T));
  B.job_of.ensure((size_t)total * 4);
  for (int j = 0; j < B.K; ++j) {
    const BatchJob<T>& J = *B.jobs[j];
    const uint64_t gs = J.group->rows_h[J.goff];
    const int64_t nnz_j = B.nnz_off[j + 1] - B.nnz_off[j];
    batch_append_csr(J.group->rows.template as<uint64_t>() + J.goff, J.group->cols.template as<uint32_t>() + gs, J.n,
                     nnz_j, (uint64_t)B.nnz_off[j] - gs, (uint32_t)(B.off[j] - J.goff),
                     B.rows.template as<uint64_t>() + B.off[j], B.cols.template as<uint32_t>() + B.nnz_off[j], s);
    if (nnz_j)
      BHG_CUDA(cudaMemcpyAsync(B.vals.template as<T>() + B.nnz_off[j], J.group->vals.template as<T>() + gs,
                               nnz_j * sizeof(T), cudaMemcpyDeviceToDevice, s));
    batch_fill_job(B.job_of.template as<uint32_t>(), B.off[j], B.off[j + 1], (uint32_t)j, s);
  }
  // normalize_p_values per job (src/tsne/mod.rs:284-293), then stop_lying if disabled
  upload<T>(B.d_nnz_off, B.nnz_off.data(), B.nnz_off.size() * 8, s);
  batch_normalize<T>(B.vals.template as<T>(), B.d_nnz_off.template as<int64_t>(), B.K, (T)P.early_exaggeration,
                     P.stop_lying_epoch == 0, s);
  upload<T>(B.d_off, B.off.data(), B.off.size() * 8, s);
  B.tiles.build(B.off, s);
  // seeds, velocity, gains, per-job learning rate and momentum
  const size_t ybytes = (size_t)total * D * sizeof(T);
  T* yd = static_cast<T*>(B.y.ensure(ybytes));
  std::vector<T> lrh(B.K), momh(B.K, (T)P.momentum);
  for (int j = 0; j < B.K; ++j) {
    BatchJob<T>& J = *B.jobs[j];
    T* dst = yd + B.off[j] * D;
    if (J.has_init) {
      BHG_CUDA(cudaMemcpyAsync(dst, J.init.data(), J.init.size() * sizeof(T), cudaMemcpyHostToDevice, s));
      J.has_init = false;
    } else {
      launch_random_init<T>(dst, J.n * D, P.seed + (uint64_t)j, s);
    }
    if (P.learning_rate > 0) lrh[j] = (T)P.learning_rate;
    else {
      const T a = (T)(double)J.n / (T)P.early_exaggeration / (T)4.0;
      lrh[j] = a > (T)50.0 ? a : (T)50.0;
    }
  }
  BHG_CUDA(cudaStreamSynchronize(s));  // the host copies of initial embeddings are staged
  B.uy.ensure(ybytes);
  B.gains.ensure(ybytes);
  B.pos.ensure(ybytes);
  B.neg.ensure(ybytes);
  B.q.ensure((size_t)total * sizeof(T));
  BHG_CUDA(cudaMemsetAsync(B.uy.ptr, 0, ybytes, s));
  batch_fill_kernel<T><<<256, 256, 0, s>>>(B.gains.template as<T>(), total * D, T(1));
  BHG_LAUNCH_CHECK();
  upload<T>(B.lr, lrh.data(), B.K * sizeof(T), s);
  upload<T>(B.mom, momh.data(), B.K * sizeof(T), s);
  B.z.ensure((size_t)B.K * 8);
  B.boxes.ensure((size_t)B.K * sizeof(BoxParams<T>));
  B.ws.reserve(total, D);
  BHG_CUDA(cudaEventRecord(e1, s));
  BHG_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  BHG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  B.aff_ms += ms;

  // epoch loop
  const int bits = D == 2 ? 32 : 21;
  T* y = B.y.template as<T>();
  build_attr_tasks<T>(B.at, D, B.rows.template as<uint64_t>(), total, s);
  BoxParams<T>* boxes = B.boxes.template as<BoxParams<T>>();
  const int64_t* off = B.d_off.template as<int64_t>();
  auto body = [&]() {
    batch_sort_and_build<T>(D, y, total, B.K, B.job_of.template as<uint32_t>(), off, boxes, B.ws, B.codes, B.jobkey,
                            B.jobkey_alt, B.tiles, s);
    Segs sg;
    sg.job = B.jobkey.template as<uint64_t>();
    sg.off = off;
    bh_traverse<T>(B.ws, D, y, total, (T)P.theta, B.neg.template as<T>(), B.q.template as<T>(), s, sg, boxes);
    batch_z<T>(B.q.template as<T>(), off, B.K, B.z.template as<double>(), s);
    launch_attractive_tasks<T>(B.at, B.cols.template as<uint32_t>(), B.vals.template as<T>(), y,
                               B.pos.template as<T>(), s);
    batch_update<T>(D, y, B.pos.template as<T>(), B.neg.template as<T>(), B.uy.template as<T>(),
                    B.gains.template as<T>(), total, B.job_of.template as<uint32_t>(), B.z.template as<double>(),
                    B.lr.template as<T>(), B.mom.template as<T>(), s);
    batch_box<T>(D, y, off, B.K, true, boxes, bits, s);
  };
  if (B.graph) {
    cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
  }
  int64_t graph_kernels = 0;
  BHG_CUDA(cudaEventRecord(e0, s));
  batch_box<T>(D, y, off, B.K, false, boxes, bits, s);
  for (int64_t epoch = 0; epoch < P.epochs; ++epoch) {
    if (epoch == 0) {
      body();
    } else {
      if (!B.graph) {
        cudaGraph_t g;
        const long long before = g_launches.load();
        BHG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
        body();
        BHG_CUDA(cudaStreamEndCapture(s, &g));
        graph_kernels = g_launches.load() - before;
        g_launches.fetch_sub(graph_kernels);
        BHG_CUDA(cudaGraphInstantiate(&B.graph, g, 0));
        BHG_CUDA(cudaGraphDestroy(g));
      }
      BHG_CUDA(cudaGraphLaunch(B.graph, s));
      g_launches.fetch_add(graph_kernels);
    }
    // epoch_tail (src/lib.rs:1162-1179), for every job at once
    if (epoch == P.stop_lying_epoch && epoch != 0)
      launch_scale<T>(B.vals.template as<T>(), B.nnz, T(1) / (T)P.early_exaggeration, s);
    if (epoch == P.momentum_switch_epoch) {
      batch_fill_kernel<T><<<(unsigned)std::max<int64_t>(1, ceil_div(B.K, 256)), 256, 0, s>>>(
          B.mom.template as<T>(), B.K, (T)P.final_momentum);
      BHG_LAUNCH_CHECK();
    }
  }
  BHG_CUDA(cudaEventRecord(e1, s));
  BHG_CUDA(cudaEventSynchronize(e1));
  BHG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  B.loop_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B.fitted = true;
}

// KL of one job: its slice of the batch in a temporary single-fit handle.
template <class T>
double batch_kl(bhtsne_batch* b, int64_t j, bool quirk) {
  BatchImpl<T>& B = bimpl<T>(b);
  if (!B.fitted || j < 0 || j >= B.K) invalid("error: no fitted job with that index.");
  cudaStream_t s = b->ctx->stream;
  const int64_t n = B.off[j + 1] - B.off[j], nnz = B.nnz_off[j + 1] - B.nnz_off[j];
  bhtsne_tsne t;
  t.ctx = b->ctx;
  t.dtype = b->dtype;
  t.D = b->D;
  t.n = n;
  new_state<T>(&t);
  std::unique_ptr<State<T>> hold(&st<T>(&t));
  State<T>& S = *hold;
  S.n = n;
  S.D = b->D;
  ensure_state<T>(&t);
  S.rows.ensure((size_t)(n + 1) * 8);
  S.cols.ensure((size_t)std::max<int64_t>(nnz, 1) * 4);
  S.vals.ensure((size_t)std::max<int64_t>(nnz, 1) * sizeof(T));
  batch_extract_csr(B.rows.template as<uint64_t>() + B.off[j], B.cols.template as<uint32_t>() + B.nnz_off[j], n, nnz,
                    (uint64_t)B.nnz_off[j], (uint32_t)B.off[j], S.rows.template as<uint64_t>(),
                    S.cols.template as<uint32_t>(), s);
  if (nnz)
    BHG_CUDA(cudaMemcpyAsync(S.vals.ptr, B.vals.template as<T>() + B.nnz_off[j], nnz * sizeof(T),
                             cudaMemcpyDeviceToDevice, s));
  S.y.ensure((size_t)n * b->D * sizeof(T));
  BHG_CUDA(cudaMemcpyAsync(S.y.ptr, B.y.template as<T>() + B.off[j] * b->D, (size_t)n * b->D * sizeof(T),
                           cudaMemcpyDeviceToDevice, s));
  S.nnz = nnz;
  S.has_sparse = true;
  S.sparse_rows = n + 1;
  t.fit = BHTSNE_METHOD_BARNES_HUT;
  t.fit_theta = b->prm.theta;
  double out = 0;
  kl<T>(&t, quirk, &out);
  return out;
}

}  // namespace

extern "C" {

void bhtsne_batch_params_default(bhtsne_batch_params* p) {
  if (!p) return;
  p->perplexity = 20.0;
  p->epochs = 1000;
  p->learning_rate = 0.0;
  p->momentum = 0.5;
  p->final_momentum = 0.8;
  p->momentum_switch_epoch = 250;
  p->stop_lying_epoch = 250;
  p->early_exaggeration = 12.0;
  p->theta = 0.5;
  p->seed = 0x6268747336e65ULL;
}

int bhtsne_batch_new(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, const bhtsne_batch_params* p, bhtsne_batch** out) {
  if (!ctx || !out) return BHTSNE_EINVAL;
  *out = nullptr;
  if (dtype != BHTSNE_F32 && dtype != BHTSNE_F64) {
    ctx->err = "error: dtype must be BHTSNE_F32 or BHTSNE_F64.";
    return BHTSNE_EINVAL;
  }
  if (embed_dim < 2 || embed_dim > 3) {
    ctx->err = "error: the batched Barnes-Hut path covers D in {2, 3}.";
    return BHTSNE_EINVAL;
  }
  bhtsne_batch* b = new bhtsne_batch();
  b->ctx = ctx;
  b->dtype = dtype;
  b->D = embed_dim;
  bhtsne_batch_params_default(&b->prm);
  if (p) b->prm = *p;
  if (dtype == BHTSNE_F32) b->impl = new BatchImpl<float>();
  else b->impl = new BatchImpl<double>();
  *out = b;
  return BHTSNE_OK;
}

int bhtsne_batch_free(bhtsne_batch* b) {
  if (!b) return BHTSNE_OK;
  cudaSetDevice(b->ctx->device);
  if (b->dtype == BHTSNE_F32) delete static_cast<BatchImpl<float>*>(b->impl);
  else delete static_cast<BatchImpl<double>*>(b->impl);
  delete b;
  return BHTSNE_OK;
}

const char* bhtsne_batch_last_error(const bhtsne_batch* b) { return b ? b->err.c_str() : "null batch"; }

int bhtsne_batch_add_euclidean(bhtsne_batch* b, const void* data, int64_t n, int32_t dim, int64_t* job) {
  return guard_batch(b, [&] {
    int64_t j = -1;
    DISPATCH_DT(b->dtype, j = batch_add_euclidean<T>(b, data, n, dim));
    if (job) *job = j;
  });
}

int bhtsne_batch_add_with_neighbors(bhtsne_batch* b, const uint64_t* indices, const void* distances, int64_t n,
                                    int64_t k, int64_t* job) {
  return guard_batch(b, [&] {
    int64_t j = -1;
    DISPATCH_DT(b->dtype, j = batch_add_with_neighbors<T>(b, indices, distances, n, k));
    if (job) *job = j;
  });
}

int bhtsne_batch_initial_embedding(bhtsne_batch* b, int64_t job, const void* y) {
  return guard_batch(b, [&] {
    DISPATCH_DT(b->dtype, {
      BatchImpl<T>& B = bimpl<T>(b);
      if (job < 0 || job >= (int64_t)B.jobs.size() || !y) invalid("error: no job with that index.");
      BatchJob<T>& J = *B.jobs[job];
      J.init.assign((const T*)y, (const T*)y + J.n * b->D);
      J.has_init = true;
    });
  });
}

int bhtsne_batch_fit(bhtsne_batch* b) {
  return guard_batch(b, [&] { DISPATCH_DT(b->dtype, batch_fit<T>(b)); });
}

int64_t bhtsne_batch_jobs(const bhtsne_batch* b) {
  if (!b) return -1;
  if (b->dtype == BHTSNE_F32) return (int64_t)static_cast<BatchImpl<float>*>(b->impl)->jobs.size();
  return (int64_t)static_cast<BatchImpl<double>*>(b->impl)->jobs.size();
}

int bhtsne_batch_embedding(bhtsne_batch* b, int64_t job, void* out) {
  return guard_batch(b, [&] {
    DISPATCH_DT(b->dtype, {
      BatchImpl<T>& B = bimpl<T>(b);
      if (!B.fitted || job < 0 || job >= B.K || !out) invalid("error: no fitted job with that index.");
      const size_t bytes = (size_t)(B.off[job + 1] - B.off[job]) * b->D * sizeof(T);
      BHG_CUDA(cudaMemcpyAsync(out, B.y.template as<T>() + B.off[job] * b->D, bytes, cudaMemcpyDeviceToHost,
                               b->ctx->stream));
      BHG_CUDA(cudaStreamSynchronize(b->ctx->stream));
    });
  });
}

int bhtsne_batch_kl_divergence(bhtsne_batch* b, int64_t job, int32_t quirk, double* out) {
  return guard_batch(b, [&] {
    double v = 0;
    DISPATCH_DT(b->dtype, v = batch_kl<T>(b, job, quirk != 0));
    if (out) *out = v;
  });
}

int bhtsne_batch_timings(const bhtsne_batch* b, double* affinity_ms, double* loop_ms) {
  if (!b) return BHTSNE_EINVAL;
  double a = 0, l = 0;
  if (b->dtype == BHTSNE_F32) {
    a = static_cast<BatchImpl<float>*>(b->impl)->aff_ms;
    l = static_cast<BatchImpl<float>*>(b->impl)->loop_ms;
  } else {
    a = static_cast<BatchImpl<double>*>(b->impl)->aff_ms;
    l = static_cast<BatchImpl<double>*>(b->impl)->loop_ms;
  }
  if (affinity_ms) *affinity_ms = a;
  if (loop_ms) *loop_ms = l;
  return BHTSNE_OK;
}

}  // extern "C"
