// Serving: continuous batching of embedding requests on one GPU.
//
// The reference fits one embedding per `tSNE` builder (src/lib.rs:149-1249)
// and has no server; this is the request loop around the same fits.
//
//   submit -> queue -> admission (FIFO, by estimated device footprint against
//   a byte budget) -> Barnes-Hut requests join the running batch, FIt-SNE
//   requests go to worker streams -> result.
//
// Barnes-Hut executor (one host thread, its own stream): the in-flight jobs
// are packed back to back (job j owns rows off[j]..off[j+1]) and stepped in
// lockstep, one launch per stage per epoch for all of them (the kernels of
// batch.cu: per-job box, per-job Morton trees, segmented traversal, per-job
// Z, attractive pass over the block-diagonal P, per-job update), the epoch
// body captured as a CUDA graph. Every job keeps its own epoch counter: the
// reference's epoch_tail (src/lib.rs:1162-1179) runs per job between epochs
// (its P slice scaled by 1/exaggeration and its momentum switched at its
// epoch 250), and a job that reaches its epoch count is frozen by an active
// flag. Every round_epochs epochs (or when jobs finished) the batch is
// repacked: finished jobs leave with their embedding and KL, admitted ones
// enter with their affinities built together (segmented kNN, one
// search_beta + symmetrize pass), survivors keep their state.
//
// FIt-SNE executor: fit_workers host threads, each with its own context and
// stream, run FIt-SNE requests through the builder path, so their work
// overlaps the Barnes-Hut batch on the device.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "../../include/bhtsne_gpu.h"
#include "batch.h"
#include "epoch.h"

namespace bhg {
int ctx_device(const bhtsne_ctx* ctx);
int ctx_create_with_priority(int device, int priority, bhtsne_ctx** out);
}

using namespace bhg;

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}


struct Request {
  int64_t id = 0;
  int method = 0;
  int64_t n = 0;
  int32_t dim = 0;
  int64_t epochs = 0;
  uint64_t seed = 0;
  bool want_kl = false;
  std::vector<unsigned char> data;
  int state = BHTSNE_JOB_QUEUED;
  std::vector<unsigned char> emb;
  double kl = NAN;
  std::string err;
  double t_submit = 0, t_done = 0;
  int64_t footprint = 0;
};

// A Barnes-Hut job in the packed batch.
template <class T>
struct Slot {
  Request* req = nullptr;
  int64_t n = 0, nnz = 0;
  DevBuf rows, cols, vals;  // its P in local numbering, normalised, exaggerated
  int64_t epoch = 0;        // epochs completed
  bool lying = true;
  bool active = true;
  T lr = T(0);
  int64_t off = 0, nnz_off = 0;  // place in the packing
};

constexpr double kExaggeration = 12.0;
constexpr int64_t kSwitchEpoch = 250;
constexpr double kMomentum = 0.5, kFinalMomentum = 0.8;

}  // namespace

struct bhtsne_server {
  bhtsne_ctx* ctx = nullptr;
  int device = 0;
  int dtype = BHTSNE_F32;
  int D = 2;
  bhtsne_server_params prm{};
  int64_t budget = 0;
  std::mutex m;
  std::condition_variable cv_bh, cv_run, cv_fit, cv_done;
  std::deque<Request*> queue;
  std::map<int64_t, std::unique_ptr<Request>> reqs;
  std::deque<Request*> bh_pending, fit_pending;
  int64_t next_id = 1;
  int64_t used = 0, peak = 0, done = 0, in_flight = 0;
  double batch_points_sum = 0;
  int64_t batch_epochs = 0;
  double t_round = 0, t_repack = 0, t_prepare = 0, t_fit = 0;  // host seconds per executor
  bool stop = false;
  std::string err;
  std::vector<std::thread> threads;
  void* engine = nullptr;  // BhEngine<T>

  int64_t footprint(int64_t n, int32_t dim) const {
    const int64_t sz = dtype == BHTSNE_F32 ? 4 : 8;
    const int64_t k = (int64_t)(3.0 * prm.perplexity);
    return n * (dim * sz + k * (40 + 4 * sz) + 600) + (1 << 20);
  }

  // Admits queued requests in order while they fit the budget (a request
  // larger than the whole budget is admitted alone). Caller holds m.
  void try_admit() {
    while (!queue.empty()) {
      Request* r = queue.front();
      if (used > 0 && used + r->footprint > budget) break;
      queue.pop_front();
      used += r->footprint;
      peak = std::max(peak, used);
      r->state = BHTSNE_JOB_RUNNING;
      ++in_flight;
      if (r->method == BHTSNE_METHOD_FIT_SNE) {
        fit_pending.push_back(r);
        cv_fit.notify_one();
      } else {
        bh_pending.push_back(r);
        cv_bh.notify_one();
      }
    }
  }

  void finish(Request* r, const std::string& error) {
    std::lock_guard<std::mutex> lk(m);
    r->state = error.empty() ? BHTSNE_JOB_DONE : BHTSNE_JOB_FAILED;
    r->err = error;
    r->t_done = now_s();
    used -= r->footprint;
    --in_flight;
    ++done;
    try_admit();
    cv_done.notify_all();
  }
};

namespace {

// Streams of the engine; declared first so that they outlive every buffer
// that is freed on them.
struct EngineStreams {
  cudaStream_t s = nullptr, ps = nullptr;
  ~EngineStreams() {
    if (s) cudaStreamSynchronize(s), cudaStreamDestroy(s);
    if (ps) cudaStreamSynchronize(ps), cudaStreamDestroy(ps);
  }
};

template <class T>
struct BhEngine {
  EngineStreams streams;
  bhtsne_server* sv;
  cudaStream_t& s = streams.s;
  std::vector<std::unique_ptr<Slot<T>>> slots;
  int64_t total = 0, nnz = 0;
  DevBuf d_off, job_of, rows, cols, vals, y, uy, gains, y2, uy2, g2, pos, neg, q, z, lr, mom, active, boxes;
  AttrTasks attr;  // attractive-pass tasks of the packed CSR, rebuilt at each repack
  DevBuf codes, jobkey, jobkey_alt, klbuf, kltmp, ykl;
  BhWorkspace<T> ws, kws;
  SegTiles tiles;
  // affinity preparation runs on its own thread and stream, overlapping the
  // batch's epochs; prepared jobs wait in `ready` for the next repack
  cudaStream_t& ps = streams.ps;
  AffinityScratch<T> paff;
  DevBuf psum, ptmp;
  std::vector<std::unique_ptr<Slot<T>>> ready;
  cudaGraphExec_t graph = nullptr;
  int64_t graph_kernels = 0;

  explicit BhEngine(bhtsne_server* server) : sv(server) {
    BHG_CUDA(cudaSetDevice(sv->device));
    // stream priorities: FIt-SNE workers (small, host-synchronised epochs)
    // first, then the batch's epochs, then affinity preparation (long kNN
    // launches), so freed SMs go to the latency-bound work first
    int lo = 0, hi = 0;
    BHG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    const int mid = lo + (hi - lo) / 2;
    BHG_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, mid == hi ? lo : mid));
    BHG_CUDA(cudaStreamCreateWithPriority(&ps, cudaStreamNonBlocking, lo));
  }
  ~BhEngine() {
    cudaSetDevice(sv->device);
    if (graph) cudaGraphExecDestroy(graph);
  }

  // Embedding (and KL) of a finished job, then it leaves the batch.
  void retire(Slot<T>& sl) {
    Request* r = sl.req;
    const int D = sv->D;
    const size_t ybytes = (size_t)sl.n * D * sizeof(T);
    r->emb.resize(ybytes);
    BHG_CUDA(cudaMemcpyAsync(r->emb.data(), y.template as<T>() + sl.off * D, ybytes, cudaMemcpyDeviceToHost, s));
    if (r->want_kl) {
      // kl_divergence (src/lib.rs:448-477): Z from a fresh tree over the
      // final embedding, the reference-compatible sparse KL over the job's P
      T* yk = static_cast<T*>(ykl.ensure(ybytes));
      BHG_CUDA(cudaMemcpyAsync(yk, y.template as<T>() + sl.off * D, ybytes, cudaMemcpyDeviceToDevice, s));
      kws.reserve(sl.n, D);
      launch_recenter_bbox<T>(D, yk, sl.n, nullptr, false, kws, bh_bits<T>(D), s);
      bh_build<T>(kws, D, yk, sl.n, s);
      bh_traverse<T>(kws, D, yk, sl.n, (T)sv->prm.theta, static_cast<T*>(neg.ptr), nullptr, s);
      double* res = static_cast<double*>(klbuf.ensure(64));
      launch_kl_sparse<T>(D, sl.rows.template as<uint64_t>(), sl.cols.template as<uint32_t>(),
                          vals.template as<T>() + sl.nnz_off, yk, sl.n, kws.z(), true, res, kltmp, s);
      double h = 0;
      BHG_CUDA(cudaMemcpyAsync(&h, res, sizeof(double), cudaMemcpyDeviceToHost, s));
      BHG_CUDA(cudaStreamSynchronize(s));
      r->kl = h;
    }
    BHG_CUDA(cudaStreamSynchronize(s));
  }

  // Affinities of newly admitted requests (grouped by input dim), their P
  // normalised and exaggerated (normalize_p_values, src/tsne/mod.rs:284-293).
  std::vector<std::unique_ptr<Slot<T>>> prepare(const std::vector<Request*>& fresh) {
    cudaStream_t s = ps;
    DevBuf& sumtmp = psum;
    DevBuf& tmp = ptmp;
    AffinityScratch<T>& aff = paff;
    std::vector<std::unique_ptr<Slot<T>>> out;
    std::map<int32_t, std::vector<Request*>> by_dim;
    for (Request* r : fresh) by_dim[r->dim].push_back(r);
    const int64_t k = (int64_t)((T)3.0 * (T)sv->prm.perplexity);
    for (auto& kv : by_dim) {
      const std::vector<Request*>& rs = kv.second;
      const int G = (int)rs.size();
      std::vector<DevBuf> xs(G);
      std::vector<const T*> X(G);
      std::vector<int64_t> ns(G);
      for (int g = 0; g < G; ++g) {
        const size_t bytes = rs[g]->data.size();
        xs[g].ensure(bytes);
        BHG_CUDA(cudaMemcpyAsync(xs[g].ptr, rs[g]->data.data(), bytes, cudaMemcpyHostToDevice, s));
        X[g] = xs[g].template as<T>();
        ns[g] = rs[g]->n;
      }
      GroupCsr<T> grp;
      group_affinities_euclidean<T>(X, ns, kv.first, k, (T)sv->prm.perplexity, grp, aff, s);
      xs.clear();
      int64_t goff = 0;
      for (int g = 0; g < G; ++g) {
        auto sl = std::make_unique<Slot<T>>();
        sl->req = rs[g];
        sl->n = ns[g];
        const uint64_t gs = grp.rows_h[goff], ge = grp.rows_h[goff + ns[g]];
        sl->nnz = (int64_t)(ge - gs);
        sl->rows.ensure((size_t)(sl->n + 1) * 8);
        sl->cols.ensure((size_t)std::max<int64_t>(sl->nnz, 1) * 4);
        sl->vals.ensure((size_t)std::max<int64_t>(sl->nnz, 1) * sizeof(T));
        batch_extract_csr(grp.rows.template as<uint64_t>() + goff, grp.cols.template as<uint32_t>() + gs, sl->n,
                          sl->nnz, gs, (uint32_t)goff, sl->rows.template as<uint64_t>(),
                          sl->cols.template as<uint32_t>(), s);
        if (sl->nnz)
          BHG_CUDA(cudaMemcpyAsync(sl->vals.ptr, grp.vals.template as<T>() + gs, sl->nnz * sizeof(T),
                                   cudaMemcpyDeviceToDevice, s));
        double* sum = static_cast<double*>(sumtmp.ensure(64));
        launch_normalize<T>(sl->vals.template as<T>(), sl->nnz, (T)kExaggeration, sum, tmp, s);
        const T a = (T)(double)sl->n / (T)kExaggeration / (T)4.0;  // resolve_learning_rate
        sl->lr = a > (T)50.0 ? a : (T)50.0;
        goff += ns[g];
        out.push_back(std::move(sl));
      }
      BHG_CUDA(cudaStreamSynchronize(s));
    }
    aff.release();
    return out;
  }

  // Rebuilds the packing from the surviving slots (state copied from the old
  // packing) and the fresh ones (seeded), retiring the finished jobs first.
  void repack(std::vector<std::unique_ptr<Slot<T>>> fresh) {
    const int D = sv->D;
    BHG_CUDA(cudaStreamSynchronize(s));
    std::vector<std::unique_ptr<Slot<T>>> keep;
    std::vector<Request*> finished;
    for (auto& sl : slots) {
      if (sl->active) {
        keep.push_back(std::move(sl));
      } else {
        std::string e;
        try {
          retire(*sl);
        } catch (const std::exception& ex) {
          e = ex.what();
        }
        finished.push_back(sl->req);
        sl.reset();
        sv->finish(finished.back(), e);
      }
    }
    slots.clear();
    if (graph) {
      cudaGraphExecDestroy(graph);
      graph = nullptr;
    }
    const size_t es = sizeof(T);
    int64_t tot = 0, nz = 0;
    for (auto& sl : keep) tot += sl->n, nz += sl->nnz;
    for (auto& sl : fresh) tot += sl->n, nz += sl->nnz;
    if (tot == 0) {
      total = 0;
      return;
    }
    y2.ensure((size_t)tot * D * es);
    uy2.ensure((size_t)tot * D * es);
    g2.ensure((size_t)tot * D * es);
    // survivors keep their state
    int64_t at = 0;
    for (auto& sl : keep) {
      const size_t b = (size_t)sl->n * D * es;
      BHG_CUDA(cudaMemcpyAsync(y2.template as<T>() + at * D, y.template as<T>() + sl->off * D, b,
                               cudaMemcpyDeviceToDevice, s));
      BHG_CUDA(cudaMemcpyAsync(uy2.template as<T>() + at * D, uy.template as<T>() + sl->off * D, b,
                               cudaMemcpyDeviceToDevice, s));
      BHG_CUDA(cudaMemcpyAsync(g2.template as<T>() + at * D, gains.template as<T>() + sl->off * D, b,
                               cudaMemcpyDeviceToDevice, s));
      at += sl->n;
    }
    // fresh jobs: random_init (seeded Box-Muller, N(0, 1e-4)), zero velocity, unit gains
    const int64_t fresh_rows = tot - at;
    if (fresh_rows > 0) {
      const size_t cnt_all = (size_t)fresh_rows * D;
      int64_t p = 0;
      for (auto& sl : fresh) {
        const int64_t cnt = sl->n * D;
        launch_random_init<T>(y2.template as<T>() + at * D + p, cnt, sl->req->seed, s);
        p += cnt;
      }
      BHG_CUDA(cudaMemsetAsync(uy2.template as<T>() + at * D, 0, cnt_all * es, s));
      std::vector<T> ones(cnt_all, T(1));
      BHG_CUDA(cudaMemcpyAsync(g2.template as<T>() + at * D, ones.data(), ones.size() * es, cudaMemcpyHostToDevice, s));
      BHG_CUDA(cudaStreamSynchronize(s));
    }
    y.swap(y2);
    uy.swap(uy2);
    gains.swap(g2);
    for (auto& sl : keep) slots.push_back(std::move(sl));
    for (auto& sl : fresh) slots.push_back(std::move(sl));
    const int K = (int)slots.size();
    std::vector<int64_t> off(K + 1, 0);
    std::vector<T> lrh(K), momh(K);
    std::vector<uint8_t> act(K, 1);
    rows.ensure((size_t)(tot + 1) * 8);
    cols.ensure((size_t)std::max<int64_t>(nz, 1) * 4);
    vals.ensure((size_t)std::max<int64_t>(nz, 1) * es);
    job_of.ensure((size_t)tot * 4);
    int64_t nzo = 0;
    for (int j = 0; j < K; ++j) {
      Slot<T>& sl = *slots[j];
      sl.off = off[j];
      sl.nnz_off = nzo;
      off[j + 1] = off[j] + sl.n;
      batch_append_csr(sl.rows.template as<uint64_t>(), sl.cols.template as<uint32_t>(), sl.n, sl.nnz, (uint64_t)nzo,
                       (uint32_t)sl.off, rows.template as<uint64_t>() + sl.off, cols.template as<uint32_t>() + nzo, s);
      if (sl.nnz) {
        if (sl.lying)
          BHG_CUDA(cudaMemcpyAsync(vals.template as<T>() + nzo, sl.vals.ptr, sl.nnz * es, cudaMemcpyDeviceToDevice, s));
        else
          launch_scaled_copy<T>(sl.vals.template as<T>(), sl.nnz, T(1) / (T)kExaggeration, vals.template as<T>() + nzo,
                                s);
      }
      batch_fill_job(job_of.template as<uint32_t>(), sl.off, off[j + 1], (uint32_t)j, s);
      lrh[j] = sl.lr;
      momh[j] = sl.epoch > kSwitchEpoch ? (T)kFinalMomentum : (T)kMomentum;
      nzo += sl.nnz;
    }
    total = tot;
    nnz = nz;
    build_attr_tasks<T>(attr, sv->D, rows.template as<uint64_t>(), tot, s);
    BHG_CUDA(cudaMemcpyAsync(d_off.ensure(off.size() * 8), off.data(), off.size() * 8, cudaMemcpyHostToDevice, s));
    tiles.build(off, s);
    BHG_CUDA(cudaMemcpyAsync(lr.ensure(K * es), lrh.data(), K * es, cudaMemcpyHostToDevice, s));
    BHG_CUDA(cudaMemcpyAsync(mom.ensure(K * es), momh.data(), K * es, cudaMemcpyHostToDevice, s));
    BHG_CUDA(cudaMemcpyAsync(active.ensure(K), act.data(), K, cudaMemcpyHostToDevice, s));
    pos.ensure((size_t)tot * D * es);
    neg.ensure((size_t)tot * D * es);
    q.ensure((size_t)tot * es);
    z.ensure((size_t)K * 8);
    boxes.ensure((size_t)K * sizeof(BoxParams<T>));
    ws.reserve(tot, D);
    batch_box<T>(D, y.template as<T>(), d_off.template as<int64_t>(), K, false, boxes.template as<BoxParams<T>>(),
                 bh_bits<T>(D), s, active.template as<uint8_t>());
    BHG_CUDA(cudaStreamSynchronize(s));
  }

  void body() {
    const int D = sv->D;
    const int K = (int)slots.size();
    T* yp = y.template as<T>();
    BoxParams<T>* bx = boxes.template as<BoxParams<T>>();
    const int64_t* off = d_off.template as<int64_t>();
    const uint8_t* act = active.template as<uint8_t>();
    batch_sort_and_build<T>(D, yp, total, K, job_of.template as<uint32_t>(), off, bx, ws, codes, jobkey, jobkey_alt,
                            tiles, s);
    Segs sg;
    sg.job = jobkey.template as<uint64_t>();
    sg.off = off;
    bh_traverse<T>(ws, D, yp, total, (T)sv->prm.theta, neg.template as<T>(), q.template as<T>(), s, sg, bx);
    batch_z<T>(q.template as<T>(), off, K, z.template as<double>(), s);
    launch_attractive_tasks<T>(attr, cols.template as<uint32_t>(), vals.template as<T>(), yp, pos.template as<T>(), s);
    batch_update<T>(D, yp, pos.template as<T>(), neg.template as<T>(), uy.template as<T>(), gains.template as<T>(), total,
                    job_of.template as<uint32_t>(), z.template as<double>(), lr.template as<T>(), mom.template as<T>(),
                    s, act);
    batch_box<T>(D, yp, off, K, true, bx, bh_bits<T>(D), s, act);
  }

  // Up to round_epochs epochs of every active job. A job that reaches its
  // epoch count is frozen at once and leaves at the next repack.
  void round() {
    bool eager = graph == nullptr;
    for (int e = 0; e < sv->prm.round_epochs; ++e) {
      if (eager) {
        body();
        eager = false;
      } else {
        if (!graph) {
          cudaGraph_t g;
          const long long before = g_launches.load();
          BHG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
          body();
          BHG_CUDA(cudaStreamEndCapture(s, &g));
          graph_kernels = g_launches.load() - before;
          g_launches.fetch_sub(graph_kernels);
          BHG_CUDA(cudaGraphInstantiate(&graph, g, 0));
          BHG_CUDA(cudaGraphDestroy(g));
        }
        BHG_CUDA(cudaGraphLaunch(graph, s));
        g_launches.fetch_add(graph_kernels);
      }
      {
        std::lock_guard<std::mutex> lk(sv->m);
        sv->batch_points_sum += (double)total;
        sv->batch_epochs += 1;
      }
      // epoch_tail per job (src/lib.rs:1162-1179)
      bool any_active = false;
      for (int j = 0; j < (int)slots.size(); ++j) {
        Slot<T>& sl = *slots[j];
        if (!sl.active) continue;
        const int64_t ep = sl.epoch;
        if (ep == kSwitchEpoch && ep != 0 && sl.lying) {
          launch_scale<T>(vals.template as<T>() + sl.nnz_off, sl.nnz, T(1) / (T)kExaggeration, s);
          sl.lying = false;
        }
        if (ep == kSwitchEpoch) {
          const T fm = (T)kFinalMomentum;
          BHG_CUDA(cudaMemcpyAsync(mom.template as<T>() + j, &fm, sizeof(T), cudaMemcpyHostToDevice, s));
        }
        sl.epoch = ep + 1;
        if (sl.epoch >= sl.req->epochs) {
          sl.active = false;
          const uint8_t zero = 0;
          BHG_CUDA(cudaMemcpyAsync(active.template as<uint8_t>() + j, &zero, 1, cudaMemcpyHostToDevice, s));
        } else {
          any_active = true;
        }
      }
      if (!any_active) break;
      {
        std::lock_guard<std::mutex> lk(sv->m);
        if (sv->stop) break;
      }
    }
    BHG_CUDA(cudaStreamSynchronize(s));
  }

  void fail_all(const std::string& e) {
    for (auto& sl : slots) sv->finish(sl->req, e);
    slots.clear();
    total = 0;
    if (graph) {
      cudaGraphExecDestroy(graph);
      graph = nullptr;
    }
  }

  // Preparer thread: affinities of admitted requests, handed to the batch.
  void prepare_loop() {
    BHG_CUDA(cudaSetDevice(sv->device));
    AllocStreamScope scope(ps);
    for (;;) {
      std::vector<Request*> fresh;
      {
        std::unique_lock<std::mutex> lk(sv->m);
        sv->cv_bh.wait(lk, [&] { return sv->stop || !sv->bh_pending.empty(); });
        if (sv->stop) break;
        fresh.assign(sv->bh_pending.begin(), sv->bh_pending.end());
        sv->bh_pending.clear();
      }
      std::vector<std::unique_ptr<Slot<T>>> prepared;
      const double t0 = now_s();
      try {
        prepared = prepare(fresh);
      } catch (const std::exception& ex) {
        for (Request* r : fresh) sv->finish(r, ex.what());
        continue;
      }
      std::lock_guard<std::mutex> lk(sv->m);
      sv->t_prepare += now_s() - t0;
      for (auto& p : prepared) ready.push_back(std::move(p));
      sv->cv_run.notify_all();
    }
  }

  // Batch thread: repack when jobs arrive or leave, then a round of epochs.
  void loop() {
    BHG_CUDA(cudaSetDevice(sv->device));
    AllocStreamScope scope(s);
    for (;;) {
      std::vector<std::unique_ptr<Slot<T>>> fresh;
      bool have_work = false;
      {
        std::unique_lock<std::mutex> lk(sv->m);
        sv->cv_run.wait(lk, [&] { return sv->stop || !ready.empty() || !slots.empty(); });
        if (sv->stop) break;
        for (auto& p : ready) fresh.push_back(std::move(p));
        ready.clear();
      }
      try {
        bool need_repack = !fresh.empty();
        for (auto& sl : slots) need_repack = need_repack || !sl->active;
        const double t0 = now_s();
        if (need_repack) repack(std::move(fresh));
        const double t1 = now_s();
        for (auto& sl : slots) have_work = have_work || sl->active;
        if (have_work) round();
        std::lock_guard<std::mutex> lk(sv->m);
        sv->t_repack += t1 - t0;
        sv->t_round += now_s() - t1;
      } catch (const std::exception& ex) {
        fail_all(ex.what());
      }
    }
    std::lock_guard<std::mutex> lk(sv->m);
    for (auto& sl : slots) {
      sl->req->state = BHTSNE_JOB_FAILED;
      sl->req->err = "error: the server was shut down.";
    }
  }
};

// One FIt-SNE request through the builder on the worker's own context.
template <class T>
void run_fit_request(bhtsne_server* sv, bhtsne_ctx* wctx, Request* r) {
  bhtsne_tsne* t = nullptr;
  std::string e;
  auto check = [&](int rc) {
    if (rc != BHTSNE_OK && e.empty()) e = t ? bhtsne_tsne_last_error(t) : "error: bhtsne_tsne_new failed.";
    return rc == BHTSNE_OK;
  };
  if (check(bhtsne_tsne_new(wctx, sv->dtype, sv->D, r->n, &t)) && check(bhtsne_tsne_perplexity(t, sv->prm.perplexity)) &&
      check(bhtsne_tsne_epochs(t, r->epochs)) && check(bhtsne_tsne_random_seed(t, r->seed)) &&
      check(bhtsne_tsne_fit_sne_euclidean(t, r->data.data(), r->dim))) {
    r->emb.resize((size_t)r->n * sv->D * sizeof(T));
    if (check(bhtsne_tsne_embedding(t, r->emb.data())) && r->want_kl) {
      double v = 0;
      int32_t has = 0;
      if (check(bhtsne_tsne_kl_divergence(t, 1, &v, &has))) r->kl = v;
    }
  }
  if (t) bhtsne_tsne_free(t);
  sv->finish(r, e);
}

template <class T>
void fit_worker(bhtsne_server* sv) {
  bhtsne_ctx* wctx = nullptr;
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  const int rc = ctx_create_with_priority(sv->device, hi, &wctx);
  for (;;) {
    Request* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(sv->m);
      sv->cv_fit.wait(lk, [&] { return sv->stop || !sv->fit_pending.empty(); });
      if (sv->stop) break;
      r = sv->fit_pending.front();
      sv->fit_pending.pop_front();
    }
    const double t0 = now_s();
    if (rc != BHTSNE_OK) sv->finish(r, "error: a FIt-SNE worker could not create its context.");
    else run_fit_request<T>(sv, wctx, r);
    std::lock_guard<std::mutex> lk(sv->m);
    sv->t_fit += now_s() - t0;
  }
  if (wctx) bhtsne_ctx_destroy(wctx);
}

template <class T>
void start(bhtsne_server* sv) {
  auto* eng = new BhEngine<T>(sv);
  sv->engine = eng;
  sv->threads.emplace_back([eng] { eng->loop(); });
  sv->threads.emplace_back([eng] { eng->prepare_loop(); });
  for (int w = 0; w < sv->prm.fit_workers; ++w) sv->threads.emplace_back([sv] { fit_worker<T>(sv); });
}

}  // namespace

extern "C" {

void bhtsne_server_params_default(bhtsne_server_params* p) {
  if (!p) return;
  p->perplexity = 30.0;
  p->theta = 0.5;
  p->hbm_budget_bytes = 0;
  p->round_epochs = 25;
  p->fit_workers = 2;
}

int bhtsne_server_new(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, const bhtsne_server_params* p,
                      bhtsne_server** out) {
  if (!ctx || !out) return BHTSNE_EINVAL;
  *out = nullptr;
  if ((dtype != BHTSNE_F32 && dtype != BHTSNE_F64) || embed_dim < 2 || embed_dim > 3) return BHTSNE_EINVAL;
  bhtsne_server_params prm;
  bhtsne_server_params_default(&prm);
  if (p) prm = *p;
  if (!(prm.theta > 0) || !(prm.perplexity > 0) || prm.round_epochs < 1 || prm.fit_workers < 0 ||
      3.0 * prm.perplexity > 224.0)
    return BHTSNE_EINVAL;
  auto* sv = new bhtsne_server();
  sv->ctx = ctx;
  sv->device = ctx_device(ctx);
  sv->dtype = dtype;
  sv->D = embed_dim;
  sv->prm = prm;
  try {
    BHG_CUDA(cudaSetDevice(sv->device));
    size_t fr = 0, totb = 0;
    BHG_CUDA(cudaMemGetInfo(&fr, &totb));
    sv->budget = prm.hbm_budget_bytes > 0 ? prm.hbm_budget_bytes : (int64_t)(0.9 * (double)fr);
    if (dtype == BHTSNE_F32) start<float>(sv);
    else start<double>(sv);
  } catch (const std::exception& e) {
    delete sv;
    return BHTSNE_ECUDA;
  }
  *out = sv;
  return BHTSNE_OK;
}

int bhtsne_server_free(bhtsne_server* sv) {
  if (!sv) return BHTSNE_OK;
  {
    std::lock_guard<std::mutex> lk(sv->m);
    sv->stop = true;
    for (Request* r : sv->queue) {
      r->state = BHTSNE_JOB_FAILED;
      r->err = "error: the server was shut down.";
    }
    sv->queue.clear();
  }
  sv->cv_bh.notify_all();
  sv->cv_run.notify_all();
  sv->cv_fit.notify_all();
  for (auto& t : sv->threads) t.join();
  if (sv->dtype == BHTSNE_F32) delete static_cast<BhEngine<float>*>(sv->engine);
  else delete static_cast<BhEngine<double>*>(sv->engine);
  delete sv;
  return BHTSNE_OK;
}

const char* bhtsne_server_last_error(const bhtsne_server* sv) { return sv ? sv->err.c_str() : "null server"; }

int bhtsne_server_submit(bhtsne_server* sv, const bhtsne_request* r, int64_t* id) {
  if (!sv || !r) return BHTSNE_EINVAL;
  auto fail = [&](const std::string& m) {
    std::lock_guard<std::mutex> lk(sv->m);
    sv->err = m;
    return BHTSNE_EINVAL;
  };
  if (!r->data || r->n < 2 || r->dim < 1) return fail("error: a request needs n >= 2 rows of dim >= 1 values.");
  const int64_t as_usize = (int64_t)sv->prm.perplexity;
  if (r->n - 1 < 3 * as_usize || r->n - 1 < (int64_t)(3.0 * sv->prm.perplexity))
    return fail("error: the provided perplexity is too large for the number of data points.\n");
  if (r->method != BHTSNE_METHOD_BARNES_HUT && r->method != BHTSNE_METHOD_FIT_SNE)
    return fail("error: a request's method is Barnes-Hut or FIt-SNE.");
  if (r->method == BHTSNE_METHOD_FIT_SNE && sv->D > 2) return fail("error: FIt-SNE is restricted to D in {1, 2}.");
  if (r->method == BHTSNE_METHOD_BARNES_HUT && r->n > kMaxTreePoints)
    return fail("error: the GPU Barnes-Hut arena holds at most 2^26 - 1 points.");
  if (r->epochs < 1) return fail("error: a request needs at least one epoch.");
  auto req = std::make_unique<Request>();
  req->method = r->method;
  req->n = r->n;
  req->dim = r->dim;
  req->epochs = r->epochs;
  req->seed = r->seed;
  req->want_kl = r->want_kl != 0;
  const size_t bytes = (size_t)r->n * r->dim * (sv->dtype == BHTSNE_F32 ? 4 : 8);
  req->data.assign(static_cast<const unsigned char*>(r->data), static_cast<const unsigned char*>(r->data) + bytes);
  req->footprint = sv->footprint(r->n, r->dim);
  std::lock_guard<std::mutex> lk(sv->m);
  if (sv->stop) {
    sv->err = "error: the server was shut down.";
    return BHTSNE_EINVAL;
  }
  req->id = sv->next_id++;
  req->t_submit = now_s();
  if (id) *id = req->id;
  Request* raw = req.get();
  sv->reqs[req->id] = std::move(req);
  sv->queue.push_back(raw);
  sv->try_admit();
  return BHTSNE_OK;
}

int bhtsne_server_poll(bhtsne_server* sv, int64_t id, int32_t* state) {
  if (!sv) return BHTSNE_EINVAL;
  std::lock_guard<std::mutex> lk(sv->m);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) {
    sv->err = "error: no request with that id.";
    return BHTSNE_EINVAL;
  }
  if (state) *state = it->second->state;
  return BHTSNE_OK;
}

int bhtsne_server_wait(bhtsne_server* sv, int64_t id, double timeout_s) {
  if (!sv) return BHTSNE_EINVAL;
  std::unique_lock<std::mutex> lk(sv->m);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) {
    sv->err = "error: no request with that id.";
    return BHTSNE_EINVAL;
  }
  Request* r = it->second.get();
  auto finished = [&] { return r->state == BHTSNE_JOB_DONE || r->state == BHTSNE_JOB_FAILED; };
  if (timeout_s < 0) {
    sv->cv_done.wait(lk, finished);
  } else if (!sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished)) {
    return BHTSNE_ETIMEDOUT;
  }
  return BHTSNE_OK;
}

int bhtsne_server_result(bhtsne_server* sv, int64_t id, void* embedding, double* kl, double* latency_ms) {
  if (!sv) return BHTSNE_EINVAL;
  std::lock_guard<std::mutex> lk(sv->m);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) {
    sv->err = "error: no request with that id.";
    return BHTSNE_EINVAL;
  }
  Request* r = it->second.get();
  if (r->state == BHTSNE_JOB_FAILED) {
    sv->err = r->err;
    sv->reqs.erase(it);
    return BHTSNE_EINVAL;
  }
  if (r->state != BHTSNE_JOB_DONE) {
    sv->err = "error: the request has not finished.";
    return BHTSNE_EINVAL;
  }
  if (embedding) std::memcpy(embedding, r->emb.data(), r->emb.size());
  if (kl) *kl = r->kl;
  if (latency_ms) *latency_ms = 1e3 * (r->t_done - r->t_submit);
  sv->reqs.erase(it);
  return BHTSNE_OK;
}

int bhtsne_server_timings(bhtsne_server* sv, double* round_s, double* repack_s, double* prepare_s, double* fit_s) {
  if (!sv) return BHTSNE_EINVAL;
  std::lock_guard<std::mutex> lk(sv->m);
  if (round_s) *round_s = sv->t_round;
  if (repack_s) *repack_s = sv->t_repack;
  if (prepare_s) *prepare_s = sv->t_prepare;
  if (fit_s) *fit_s = sv->t_fit;
  return BHTSNE_OK;
}

int bhtsne_server_stats(bhtsne_server* sv, int64_t* done, int64_t* in_flight, int64_t* peak_bytes,
                        double* mean_batch_points) {
  if (!sv) return BHTSNE_EINVAL;
  std::lock_guard<std::mutex> lk(sv->m);
  if (done) *done = sv->done;
  if (in_flight) *in_flight = sv->in_flight;
  if (peak_bytes) *peak_bytes = sv->peak;
  if (mean_batch_points) *mean_batch_points = sv->batch_epochs ? sv->batch_points_sum / sv->batch_epochs : 0.0;
  return BHTSNE_OK;
}

}  // extern "C"
