"""t-SNE epochs/s at 1M points on one GB300 (Barnes-Hut, theta 0.5, 2-D).

Workload (the 1M-point configuration): N = 1,000,000 points, input dim 128,
float32, a 100-cluster mixture with Student-t (nu = 5) radial spread and
centres ~ N(0, 8^2 I); perplexity 30 (k = 90); Barnes-Hut theta 0.5 into 2-D.
Both arms start from the same seeded normal embedding (sigma 1e-4) and time the same
window of the fit: --steps epochs after --burn-in (250, the end of the early
exaggeration) and --warmup epochs, i.e. epochs 255-274 by default. A "step"
is one optimisation epoch (tree build, traversal, attractive pass, fused
update + recentre) over the full 1M-point embedding.

  value  : epochs/s over the window with the affinities and embedding resident
           in HBM, timed with CUDA events on the library's stream
           (bhtsne_tsne_advance), with the locality re-layout (one every 50
           epochs, timed by CUDA events in the same run) charged pro rata.
  e2e    : the same window through the C ABI as a user calls it: a warm start
           from the window's first embedding (with_affinities from pinned host
           CSR, initial_embedding, barnes_hut with the exaggeration over and the
           final momentum, embedding()), every copy inside the timed region.
  roofline: the dominant epoch phase's algorithmic bytes per launch over its
           live CUDA-event time, against the measured HBM copy peak.
  cpu_baseline: the oracle (C++/OpenMP restatement) on epochs from the
           window's last embedding.
  parity : the 1M-point kNN on sampled rows against the oracle's brute force,
           the certificate's fallback rows, the gradient at the window's last
           embedding against the oracle; final-KL gaps of the 5k and 70k fits.
  clocks : nvidia-smi samples taken during the timed epochs.
  batched / serving: the 512-job batch and the request stream against the
           same work run one job at a time through the builder.

--impl reference times the CPU restatement of the reference (oracle/, C++
with OpenMP on every host core) on the same workload and window: one
continuous fit from the same initial embedding, epochs 255-274 timed inside
it. Run with --gpus N for N independent replicas (the path does not shard; one
process per GPU under torchrun).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "t-SNE epochs/s @1M pts (Barnes-Hut theta 0.5, 2-D)"
UNIT = "epochs/s"
RENUMBER_PERIOD = 50  # epochs between locality renumberings (library default)
INIT_SEED = 42


def initial_embedding(n, D=2, seed=INIT_SEED):
    """Seeded normal start with mean 0 and standard deviation 1e-4, the
    distribution of the reference's random_init (src/tsne/mod.rs:142-147,
    rand_distr Normal::new(0.0, 1e-4)); both arms start from it."""
    return np.random.default_rng(seed).normal(0.0, 1e-4, size=(n, D)).astype(np.float32)


def workload_config(args, ws):
    """The config both arms report (identical keys and values)."""
    first = args.burn_in + args.warmup
    return {"workload": "bh2d_1M_d128", "n_points": args.n, "input_dim": 128, "clusters": 100,
            "perplexity": 30.0, "k": 90, "theta": 0.5, "embed_dim": 2,
            "window": "epochs %d-%d of one fit from a seeded normal start (sigma 1e-4)" % (first, first + args.steps - 1),
            "l2": "inputs larger than L2 (CSR P of about 1.4 GB per epoch)",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}


def pinned_copy(a):
    """A copy of `a` in page-locked host memory (through torch), or `a` itself
    where pinning is unavailable; returns (array, pinned?)."""
    try:
        import torch
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        out = t.numpy().view(a.dtype).reshape(a.shape)  # the view keeps the tensor alive
        out[...] = a
        return out, True
    except Exception:
        return a, False


def make_workload(n, dim=128, clusters=100, seed=1003):
    """100-cluster Student-t (nu=5) mixture, centres ~ N(0, 8^2 I), equal weights."""
    rng = np.random.default_rng(seed)
    centres = rng.normal(0.0, 8.0, size=(clusters, dim)).astype(np.float32)
    lab = rng.integers(0, clusters, size=n)
    g = rng.standard_normal(size=(n, dim), dtype=np.float32)
    w = (rng.chisquare(5.0, size=n) / 5.0).astype(np.float32)
    X = centres[lab] + g / np.sqrt(w)[:, None]
    return np.ascontiguousarray(X, dtype=np.float32), lab


def within_cluster_knn(X, lab, k):
    """kNN restricted to each generating cluster (BLAS distances); used only to
    give the CPU arm its affinity input. In this mixture the clusters are far
    apart, so it coincides with the global kNN up to rounding ties."""
    n = X.shape[0]
    idx = np.zeros((n, k), np.uint64)
    dist = np.zeros((n, k), np.float32)
    for c in np.unique(lab):
        members = np.nonzero(lab == c)[0]
        Xc = X[members].astype(np.float32)
        sq = (Xc * Xc).sum(1)
        for s in range(0, len(members), 4096):
            blk = Xc[s:s + 4096]
            d2 = sq[s:s + 4096, None] + sq[None, :] - 2.0 * (blk @ Xc.T)
            np.maximum(d2, 0, out=d2)
            rows = np.arange(blk.shape[0])
            d2[rows, rows + s] = np.inf
            part = np.argpartition(d2, k, axis=1)[:, :k]
            pd = np.take_along_axis(d2, part, 1)
            order = np.argsort(pd, axis=1, kind="stable")
            part = np.take_along_axis(part, order, 1)
            idx[members[s:s + 4096]] = members[part]
            dist[members[s:s + 4096]] = np.sqrt(np.take_along_axis(pd, order, 1))
    return idx, dist


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_and_max(value, ws):
    """Barrier + max over ranks (gloo over the host; each rank runs its own GPU)."""
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")
    t = torch.tensor([value], dtype=torch.float64)
    dist.barrier()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    import bhtsne_gb300 as bg
    ws, rank, local = dist_info()
    n = args.n
    X, lab = make_workload(n, seed=args.seed)
    ctx = bg.Context(local)
    perp, theta = 30.0, 0.5
    y0 = initial_embedding(n, seed=INIT_SEED + rank)
    t = bg.TSNE(X, D=2, ctx=ctx).perplexity(perp).epochs(0).initial_embedding(y0)
    t0 = time.time()
    t.barnes_hut(theta)  # kNN + affinities + seeding, no epochs
    setup_s = time.time() - t0
    knn_fallback_fit = ctx.knn_fallback_rows()
    tm = t.timings()
    # burn-in past the early-exaggeration phase (epochs 0..249) and warm-up;
    # untimed. The window then covers the same epochs as the reference arm's.
    t.advance(args.burn_in)
    t.advance(args.warmup)
    y_start = t.embedding().reshape(n, 2)  # first embedding of the window (for the e2e leg)
    launches0 = ctx.lib.bhtsne_launch_count()
    barrier_and_max(0.0, ws)
    with ClockSampler(local) as clk:
        t.advance(args.steps)  # timed: CUDA events on the library's stream, epoch graphs replayed
    launches = ctx.lib.bhtsne_launch_count() - launches0
    loop_ms = t.timings()["loop_ms"]
    loop_ms = barrier_and_max(loop_ms, ws)
    window_relayouts = t.relayout_times()["count"]
    layout = t.layout_info()  # chosen at the first re-layout point (epoch 50), inside the burn-in
    # the embedding after the window: the CPU baseline, the work count and the
    # gradient parity check start from it; copied out after the timed region
    y_end = t.embedding().reshape(n, 2)
    # per-phase device times from a separate profiled pass (events between
    # phases force eager launches, so it is not the timed region)
    t.profile(True)
    t.advance(max(3, min(args.steps, 10)))
    t.profile(False)
    ph = t.phase_times()
    # one whole period of the locality renumbering (y, uy, gains and the CSR are
    # re-laid out in Morton order every 50 epochs, the library default), starting
    # with one: its re-layout time is charged to `value` pro rata
    cur = args.burn_in + args.warmup + args.steps + max(3, min(args.steps, 10))
    if (-cur) % RENUMBER_PERIOD:
        t.advance((-cur) % RENUMBER_PERIOD)
    t.advance(RENUMBER_PERIOD)
    period_ms = barrier_and_max(t.timings()["loop_ms"], ws)
    rl = t.relayout_times()
    relayout_ms = barrier_and_max(rl["ms"] / max(rl["count"], 1), ws)
    p0 = cur + (-cur) % RENUMBER_PERIOD
    period = {"value": round(ws * RENUMBER_PERIOD / (period_ms / 1e3), 3), "unit": UNIT,
              "window": "epochs %d-%d, %s" % (p0, p0 + RENUMBER_PERIOD - 1,
                                               "component layout (no periodic re-layout)" if layout["component_layout"]
                                               else "one locality re-layout at the start"),
              "relayout_ms": round(relayout_ms, 3)}
    aff = t.affinities()
    nnz = int(aff.values.size)
    # re-layouts in the window itself are already inside loop_ms; the others
    # are charged at one per RENUMBER_PERIOD epochs
    charged_ms = relayout_ms * (args.steps / RENUMBER_PERIOD - window_relayouts)
    value = ws * args.steps / ((loop_ms + max(charged_ms, 0.0)) / 1e3)
    window_value = ws * args.steps / (loop_ms / 1e3)

    # roofline: dominant phase of the epoch
    peak, peak_kind = measured_peaks()
    per = {k: ph[k] / max(ph["epochs"], 1) for k in ("tree", "repulsion", "attractive", "update")}
    # the roofline object describes the dominant HBM-bound phase (attractive
    # pass, update, tree build); the traversal is latency/L2-bound (its L1 hit
    # rate is 97 %) and is reported by its interaction rate under `traversal`
    dom_all = max(per, key=per.get)
    dom = max(("attractive", "update", "tree"), key=per.get)
    D = 2
    alg = {
        # traversal: queries (perm + y), every node once (16 B geometry + 4 B skip), forces out
        "repulsion": 4 * n + 4 * n * D + 20 * (2 * n - 1) + 4 * n * D,
        # CSR attractive: row offsets, (col, val) per entry, y once, forces out
        "attractive": 8 * (n + 1) + 8 * nnz + 4 * n * D + 4 * n * D,
        # update + recentre: 32 N D + 8 N D (+ bbox, included in the recentre read)
        "update": 32 * n * D + 8 * n * D,
        # Morton + sort: y in, 8 radix passes over (u64 key, u32 idx)
        "tree": 4 * n * D + 12 * n * 2 * 8,
    }
    achieved = alg[dom] / (per[dom] / 1e3) / 1e9
    # DRAM bytes (read + write) per launch from one ncu capture of the same
    # kernel at N = 300,000 in the component layout (435.7 MB for 52,492,156
    # CSR entries), scaled by this run's entries; null for the other phases
    traffic = {"attractive": int(435.65e6 * nnz / 52492156)}
    roofline = {"kernel": {"repulsion": "bh_traverse_kernel", "attractive": "attractive_task_kernel+attractive_fixup_kernel",
                           "update": "update_kernel+recenter_bbox_kernel", "tree": "morton+radix sort+tree build"}[dom],
                "bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": traffic.get(dom), "peak_source": peak_kind,
                "algorithmic_bytes": alg[dom], "ms_per_launch": round(per[dom], 4),
                "dominant_phase": dom_all,
                "note": "the dominant HBM-bound phase; the Barnes-Hut traversal (%.3f ms per epoch) is latency/L2-bound "
                        "and is reported under `traversal` by its interaction rate" % per["repulsion"]}
    att_gbs = alg["attractive"] / (per["attractive"] / 1e3) / 1e9

    # e2e: the same window through the C ABI with host buffers: a warm start
    # from the window's first embedding, exaggeration over (stop_lying_epoch 0)
    # and the final momentum, as epochs 255.. of the fit run
    rows_h, pin_rows = pinned_copy(aff.rows)
    cols_h, pin_cols = pinned_copy(aff.columns)
    vals_h, pin_vals = pinned_copy(aff.values)
    y_in, pin_y = pinned_copy(np.ascontiguousarray(y_start))
    aff_h = bg.SparseAffinities(rows_h, cols_h, vals_h, aff.perplexity)
    emb = np.empty(n * 2, np.float32)
    emb, _ = pinned_copy(emb)
    h2d = rows_h.nbytes + cols_h.nbytes + vals_h.nbytes + y_in.nbytes
    # the whole user-side call sequence, repeated (a single ~50 ms sample is at
    # the mercy of the host); the median of the repetitions is reported
    e2e_runs = []
    for _ in range(args.e2e_reps):
        t2 = bg.TSNE(n, D=2, ctx=ctx).epochs(args.steps).stop_lying_epoch(0).momentum(0.8)
        barrier_and_max(0.0, ws)
        w0 = time.perf_counter()
        t2.with_affinities(aff_h)
        t2.initial_embedding(y_in)
        t2.barnes_hut(theta)
        t2.embedding_into(emb)
        e2e_s = time.perf_counter() - w0
        e2e_runs.append(barrier_and_max(e2e_s, ws))
        t2.close()
    e2e_s = statistics.median(e2e_runs)
    e2e = {"value": round(ws * args.steps / e2e_s, 3), "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
           "d2h_bytes_per_step": emb.nbytes // args.steps,
           "samples": [round(ws * args.steps / x, 1) for x in e2e_runs], "statistic": "median",
           "pinned": bool(pin_rows and pin_cols and pin_vals and pin_y),
           "note": "with_affinities(host CSR) + initial_embedding(window start) + barnes_hut(epochs=steps, "
                   "stop_lying_epoch 0, momentum 0.8) + embedding(); affinity normalisation, the warm start's "
                   "re-layout and all copies inside the timed region"}
    del rows_h, cols_h, vals_h, aff_h

    parity = None
    if rank == 0 and not args.no_parity:
        parity = parity_1m(args, ctx, X, aff, y_end, knn_fallback_fit)
    del X

    batched = None
    if args.batch_jobs > 0:
        batched = run_batched(args, ctx)
    serving = None
    if args.serve_requests > 0:
        serving = run_serving(args, ctx)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample(aff, y_end, args.cpu_epochs, count_at=y_end)
    traversal = None
    if cpu and "bh_work_per_epoch" in cpu:
        w = cpu["bh_work_per_epoch"]
        sec = per["repulsion"] / 1e3
        traversal = {"kernel": "bh_traverse_kernel", "bound": "latency / L2 (ncu: 97 % L1 hits, issue-bound)",
                     "ms_per_launch": round(per["repulsion"], 4), "interactions_per_epoch": w["interactions"],
                     "theta_tests_per_epoch": w["theta_tests"],
                     "interactions_per_s": round(w["interactions"] / sec, 1),
                     "theta_tests_per_s": round(w["theta_tests"] / sec, 1),
                     "note": "work counted by the oracle's walk of the same tree and theta test at the embedding "
                             "after the timed window, over the profiled repulsion time"}
    configs = run_configs(args, ctx, aff, rank) if args.configs else None
    if configs and parity is not None:
        for key in ("c1_5k", "c2_70k_bh", "c2_70k_fit"):
            if key in configs.get("parity", {}):
                parity[key] = configs["parity"][key]

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * ws * args.steps / value / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, ws),
        "nnz": nnz,
        "window_only": {"value": round(window_value, 3), "relayouts_in_window": window_relayouts,
                        "relayout_ms_charged": round(max(charged_ms, 0.0), 3),
                        "note": "the timed window alone; `value` adds the periodic re-layouts (one per %d epochs in "
                                "the Morton layout, none in the component layout)" % RENUMBER_PERIOD},
        "layout": {"component_layout": layout["component_layout"], "largest_component": layout["largest_component"],
                   "note": "component layout: the points grouped once by connected component of P's graph; "
                           "otherwise re-laid out in the embedding's Morton order every 50 epochs"},
        "e2e": e2e,
        "roofline": roofline,
        "roofline_attractive": {"achieved": round(att_gbs, 2), "peak": peak, "unit": "GB/s",
                                "frac": round(att_gbs / peak, 4)},
        "phase_ms_per_epoch": {k: round(v, 4) for k, v in per.items()},
        "epochs_per_s_incl_renumbering": period,
        "traversal": traversal,
        "setup_s": round(setup_s, 3), "affinity_ms": round(tm["affinity_ms"], 2),
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if parity:
        out["parity"] = parity
    if batched:
        out["batched"] = batched
    if serving:
        out["serving"] = serving
    if cpu:
        out["cpu_baseline"] = cpu
    if configs:
        configs.pop("parity", None)
        out["configs"] = configs
    if rank == 0:
        print(json.dumps(out))


def parity_1m(args, ctx, X, aff, y_end, knn_fallback_fit):
    """Parity at the 1M-point size: the GPU kNN (tensor-core candidates, exact
    re-rank and certificate) on sampled query rows against the oracle's brute
    force over all 1M candidates, bit for bit; the certificate's fallback
    rows; and the Barnes-Hut gradient at the window's last embedding against
    the oracle (P un-exaggerated, theta 0.5)."""
    import bhtsne_gb300 as bg
    from oracle import pyoracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    n = X.shape[0]
    out = {}
    rows = np.sort(np.random.default_rng(2026).choice(n, args.parity_rows, replace=False))
    gi, gd = bg.knn_euclidean(X, 90, ctx=ctx)
    fb, fbb = ctx.knn_fallback_rows(), ctx.knn_brute_rows()
    w0 = time.perf_counter()
    oi, od = O.knn_rows(X, 90, rows)
    same = np.all(gi[rows] == oi, axis=1) & np.all(gd[rows] == od, axis=1)
    out["c3_knn"] = {"rows_checked": int(rows.size), "rows_bit_exact": int(same.sum()),
                     "fallback_rows": int(fb), "brute_rows": int(fbb), "fallback_rows_fit": int(knn_fallback_fit),
                     "oracle_s": round(time.perf_counter() - w0, 2),
                     "note": "random query rows, brute force over all %d candidates, (distance, index) order" % n}
    del gi, gd
    vals = O.normalize(aff.values, 1.0)
    y = np.ascontiguousarray(y_end, dtype=np.float32)
    pos, neg, z = bg.gradient(bg.METHOD_BARNES_HUT, y, aff.rows, aff.columns, vals, theta=0.5, ctx=ctx)
    opos = O.edge_forces(y, aff.rows, aff.columns, vals)
    oneg, oq, oz = O.bh_repulsion(y, 0.5)
    # the reference sums Z sequentially in f32 (src/repulsion.rs:155); the GPU
    # sums it in FP64: both against the FP64 sum of the oracle's per-point terms
    z64 = float(oq.astype(np.float64).sum())
    # the same Barnes-Hut pass evaluated in f64 by the oracle: the repulsive
    # forces of both f32 passes (the GPU's FP64 centres of mass, the oracle's
    # f32 ones) against it
    oneg64, _, _ = O.bh_repulsion(y.astype(np.float64), 0.5)
    g = pos.astype(np.float64) - neg.astype(np.float64) / z
    og = opos.astype(np.float64) - oneg.astype(np.float64) / oz
    out["c3_gradient"] = {"embedding": "after the timed window (epoch %d)" % (args.burn_in + args.warmup + args.steps),
                          "rel_l2_gradient": float("%.3g" % rel_l2(g, og)),
                          "rel_l2_attractive": float("%.3g" % rel_l2(pos, opos)),
                          "rel_l2_repulsive": float("%.3g" % rel_l2(neg, oneg)),
                          "rel_l2_repulsive_vs_f64_pass": {"gpu": float("%.3g" % rel_l2(neg, oneg64)),
                                                          "oracle_f32": float("%.3g" % rel_l2(oneg, oneg64))},
                          "z_rel_vs_fp64_sum": float("%.3g" % (abs(z - z64) / z64)),
                          "oracle_f32_sequential_z_rel_vs_fp64_sum": float("%.3g" % (abs(oz - z64) / z64)),
                          "bar": 1e-4}
    return out


def make_c1_workload(n=5000, dim=50, seed=1001):
    """10 equal-weight isotropic components, means ~ N(0, 10^2 I), unit variance."""
    rng = np.random.default_rng(seed)
    centres = rng.normal(0.0, 10.0, size=(10, dim))
    lab = rng.integers(0, 10, size=n)
    return (centres[lab] + rng.normal(size=(n, dim))).astype(np.float32)


def make_c2_workload(n=70_000, dim=20, seed=1002):
    """10 anisotropic clusters (per-axis std 1/sqrt(i+1)), centres ~ N(0, 5^2 I),
    weights ~ Dirichlet(2 * 1_10): the shape of MNIST after PCA to 20."""
    rng = np.random.default_rng(seed)
    centres = rng.normal(0.0, 5.0, size=(10, dim))
    w = rng.dirichlet(np.full(10, 2.0))
    lab = rng.choice(10, size=n, p=w)
    std = 1.0 / np.sqrt(np.arange(dim) + 1.0)
    return (centres[lab] + rng.normal(size=(n, dim)) * std).astype(np.float32)


def exact_gradient_f64(y, rows, cols, vals):
    """The t-SNE gradient direction pos - neg / Z of the sparse-P objective in
    FP64, all pairs (O(N^2), small N): pos_i = sum_j p_ij q_ij (y_i - y_j),
    neg_i = sum_{j != i} q_ij^2 (y_i - y_j), Z = sum_{i != j} q_ij. Returns
    (pos, neg / Z)."""
    y = y.astype(np.float64)
    n, D = y.shape
    r = np.repeat(np.arange(n), np.diff(rows.astype(np.int64)))
    d = y[r] - y[cols.astype(np.int64)]
    q = 1.0 / (1.0 + (d * d).sum(1))
    pos = np.zeros_like(y)
    np.add.at(pos, r, (vals.astype(np.float64) * q)[:, None] * d)
    neg = np.zeros_like(y)
    z = 0.0
    for a in range(0, n, 1024):
        diff = y[a:a + 1024, None, :] - y[None, :, :]
        qq = 1.0 / (1.0 + (diff * diff).sum(2))
        idx = np.arange(a, min(a + 1024, n))
        qq[idx - a, idx] = 0.0
        z += qq.sum()
        neg[a:a + 1024] = ((qq * qq)[:, :, None] * diff).sum(1)
    return pos, neg / z


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def timed_epochs(t, args):
    """Burn-in, warm-up, then args.steps timed epochs (graph replay) and a
    profiled pass for the phase split; returns epochs/s and phases (ms)."""
    t.advance(args.burn_in)
    t.advance(args.warmup)
    t.advance(args.steps)
    ms = t.timings()["loop_ms"] / args.steps
    t.profile(True)
    t.advance(10)
    ph = t.phase_times()
    t.profile(False)
    return round(1e3 / ms, 3), {k: round(v / 10, 4) for k, v in ph.items() if k != "epochs"}


def kl_gap(g, o):
    """Both KL forms of a GPU fit `g` and an oracle fit `o`, and their gaps."""
    out = {}
    for name, quirk in (("reference_compatible", True), ("true", False)):
        kg, ko = g.kl_divergence(quirk), o.kl_divergence(quirk)
        out[name] = {"gpu": round(kg, 6), "oracle": round(ko, 6), "gap": float("%.3g" % (abs(kg - ko) / abs(ko)))}
    return out


def run_configs(args, ctx, aff, rank):
    """The other configurations of the path, each measured here: 1M points in
    3-D Barnes-Hut and 2-D FIt-SNE (on the 1M affinities), the 70k MNIST-shape
    fits and the 5k fit, each against the oracle from the same kNN table and
    initial embedding (final KL, both forms), and the 5k error against an FP64
    all-pairs gradient."""
    import bhtsne_gb300 as bg
    out = {"parity": {}}
    n = aff.rows.size - 1
    for name, D, method in (("bh3d_1M", 3, "bh"), ("fitsne2d_1M", 2, "fit")):
        t = bg.TSNE(n, D=D, ctx=ctx).with_affinities(aff).epochs(0).initial_embedding(initial_embedding(n, D))
        t.barnes_hut(0.5) if method == "bh" else t.fit_sne()
        eps, ph = timed_epochs(t, args)
        out[name] = {"epochs_per_s": eps, "phase_ms_per_epoch": ph, "burn_in_epochs": args.burn_in,
                     "steps": args.steps, "note": "affinities of the 1M bh2d workload"}
        del t
    with_oracle = rank == 0 and not args.no_cpu
    if with_oracle:
        from oracle import pyoracle as O
        O.build()
        O.set_threads(os.cpu_count() or 1)

    X2 = make_c2_workload()
    n2 = X2.shape[0]
    y2 = initial_embedding(n2, seed=7)
    c2 = {"workload": "70k x 20, 10 anisotropic clusters, Dirichlet(2) weights, perplexity 30, 2-D, 1000 epochs"}
    gi2, gd2 = bg.knn_euclidean(X2, 90, ctx=ctx) if with_oracle else (None, None)
    for method in ("bh", "fit"):
        t = bg.TSNE(X2, D=2, ctx=ctx).perplexity(30).epochs(1000).initial_embedding(y2)
        w0 = time.perf_counter()
        t.barnes_hut(0.5) if method == "bh" else t.fit_sne()
        t.embedding()
        wall = time.perf_counter() - w0
        tm = t.timings()
        c2[method] = {"fit_s": round(wall, 3), "setup_ms": round(tm["affinity_ms"], 1),
                      "epochs_per_s": round(1e3 * tm["loop_epochs"] / tm["loop_ms"], 2),
                      "kl": round(t.kl_divergence(True), 5)}
        if with_oracle:
            # the oracle fit from the same kNN table (the GPU's, bit-exact with
            # brute force) and the same initial embedding, all host cores
            h = O.TSNE(n2).perplexity(30).epochs(1000).initial_embedding(y2)
            w0 = time.perf_counter()
            if method == "bh":
                h.barnes_hut_with_neighbors(0.5, gi2.astype(np.uint64), gd2)
            else:
                h.fit_sne_with_neighbors(gi2.astype(np.uint64), gd2)
            cpu_s = time.perf_counter() - w0
            c2[method]["cpu_fit_s"] = round(cpu_s, 2)
            c2[method]["cpu_epochs_per_s"] = round(1000 / cpu_s, 2)
            out["parity"]["c2_70k_" + method] = kl_gap(t, h)
            del h
        del t
    if with_oracle:
        c2["cpu_cores"] = os.cpu_count() or 1
        c2["cpu_note"] = "oracle fits include their affinity build (search_beta, symmetrisation)"
    out["c2_70k"] = c2

    X1 = make_c1_workload()
    y1 = initial_embedding(X1.shape[0], seed=5)
    if with_oracle:
        # C1 as specified: 5k x 50, BH theta 0.5, 1000 epochs, reference defaults
        g = bg.TSNE(X1, D=2, ctx=ctx).perplexity(30).epochs(1000).initial_embedding(y1)
        g.barnes_hut(0.5)
        gi1, gd1 = bg.knn_euclidean(X1, 90, ctx=ctx)
        h = O.TSNE(X1.shape[0]).perplexity(30).epochs(1000).initial_embedding(y1)
        h.barnes_hut_with_neighbors(0.5, gi1.astype(np.uint64), gd1)
        out["parity"]["c1_5k"] = kl_gap(g, h)
        del g, h

    # C1: the gradient at a fixed Y against FP64 all pairs. At epoch 100 (P
    # exaggerated x12, the embedding still moving) the full direction pos -
    # neg / Z; at the converged embedding of epoch 1000 pos and neg / Z nearly
    # cancel, so there the approximated term neg / Z is compared.
    t = bg.TSNE(X1, D=2, ctx=ctx).perplexity(30).epochs(100).initial_embedding(y1)
    t.barnes_hut(0.5)
    y100 = t.embedding().reshape(-1, 2)
    t.advance(900)
    y1000 = t.embedding().reshape(-1, 2)
    a1 = t.affinities()
    vals = a1.values.astype(np.float64)
    vals = vals / vals.sum()
    acc = {"workload": "5k x 50, 10 components, perplexity 30; Y of a Barnes-Hut fit at epochs 100 and 1000",
           "reference": "FP64 all pairs"}
    cases = (("epoch_100_gradient", y100, (12.0 * vals).astype(np.float32)),
             ("epoch_1000_repulsion", y1000, vals.astype(np.float32)))
    for label, yy, pv in cases:
        p64, r64 = exact_gradient_f64(yy, a1.rows, a1.columns, pv)
        for name, m in (("bh_theta_0.5_f32", bg.METHOD_BARNES_HUT), ("fitsne_f32", bg.METHOD_FIT_SNE)):
            pos, neg, z = bg.gradient(m, yy, a1.rows, a1.columns, pv, theta=0.5, ctx=ctx)
            rep = neg.astype(np.float64) / z
            err = rel_l2(pos.astype(np.float64) - rep, p64 - r64) if label.endswith("gradient") else rel_l2(rep, r64)
            acc.setdefault(label, {})[name] = round(err, 6)
    out["c1_5k_vs_fp64_exact"] = acc
    return out


def make_batch_workload(jobs=512, dim=32, seed=2024):
    """Per-job N log-uniform in [500, 50000]; each job a Gaussian mixture of
    5-20 equal-weight unit-variance components with centres ~ N(0, 10^2 I)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(500), np.log(50000), size=jobs)).astype(int)
    data = []
    for n in sizes:
        c = int(rng.integers(5, 21))
        centres = rng.normal(0.0, 10.0, size=(c, dim)).astype(np.float32)
        lab = rng.integers(0, c, size=n)
        data.append(np.ascontiguousarray(centres[lab] + rng.standard_normal(size=(n, dim), dtype=np.float32)))
    return data


def run_batched(args, ctx):
    """512 independent embeddings: one bhtsne_batch (segmented kNN/affinities,
    lockstep epochs with per-job trees, one graph per epoch) against the same
    512 run one at a time through the plain builder. Both arms start from host
    arrays and end with every embedding back on the host."""
    import bhtsne_gb300 as bg
    data = make_batch_workload(args.batch_jobs)
    E, perp, theta = args.batch_epochs, 30.0, 0.5
    w0 = time.perf_counter()
    b = bg.Batch(perplexity=perp, epochs=E, theta=theta, seed=11, ctx=ctx)
    for X in data:
        b.add(X)
    b.fit()
    embs = [b.embedding(j) for j in range(len(data))]
    batched_s = time.perf_counter() - w0
    aff_ms, loop_ms = b.timings()
    kl_b = [b.kl_divergence(j) for j in range(len(data))]
    del embs
    b.close()
    lat, kl_p = [], []
    w0 = time.perf_counter()
    for j, X in enumerate(data):
        t = bg.TSNE(X, ctx=ctx).perplexity(perp).epochs(E).random_seed(11 + j)
        t.barnes_hut(theta)
        t.embedding()
        lat.append(time.perf_counter() - w0)
        kl_p.append(t.kl_divergence())
        t.close()
    plain_s = time.perf_counter() - w0
    gap = np.abs(np.array(kl_b) - np.array(kl_p)) / np.abs(np.array(kl_p))
    J = len(data)
    return {
        "workload": f"{J} jobs, N log-uniform [500, 50000] (total {sum(len(x) for x in data)} points), input dim 32, "
                    f"5-20 component mixtures, perplexity {perp}, BH theta {theta}, 2-D, {E} epochs",
        "jobs_per_s": round(J / batched_s, 3), "plain_jobs_per_s": round(J / plain_s, 3),
        "speedup_vs_plain": round(plain_s / batched_s, 3),
        "batched_s": round(batched_s, 3), "plain_s": round(plain_s, 3),
        "batched_affinity_ms": round(aff_ms, 1), "batched_epoch_loop_ms": round(loop_ms, 1),
        "latency_s": {"batched_p50": round(batched_s, 3), "batched_p99": round(batched_s, 3),
                      "plain_p50": round(float(np.percentile(lat, 50)), 3),
                      "plain_p99": round(float(np.percentile(lat, 99)), 3),
                      "note": "all jobs submitted at t=0; lockstep batch returns every job at the end"},
        "kl_gap": {"mean": round(float(gap.mean()), 5), "p99": round(float(np.percentile(gap, 99)), 5),
                   "max": round(float(gap.max()), 5),
                   "aggregate": round(abs(sum(kl_b) - sum(kl_p)) / abs(sum(kl_p)), 6),
                   "within_1pct": int((gap <= 0.01).sum())},
    }


def run_batched_only(args, ctx):
    """The batched arm of the 512-job comparison alone (the same jobs, settings
    and seed as run_batched), for launch lists and profiles."""
    import bhtsne_gb300 as bg
    data = make_batch_workload(args.batch_jobs)
    w0 = time.perf_counter()
    b = bg.Batch(perplexity=30.0, epochs=args.batch_epochs, theta=0.5, seed=11, ctx=ctx)
    for X in data:
        b.add(X)
    b.fit()
    for j in range(len(data)):
        b.embedding(j)
    aff_ms, loop_ms = b.timings()
    b.close()
    return {"jobs": len(data), "points": int(sum(len(x) for x in data)), "epochs": args.batch_epochs,
            "total_s": round(time.perf_counter() - w0, 3), "affinity_ms": round(aff_ms, 1), "loop_ms": round(loop_ms, 1)}


def make_serving_workload(requests, seed=2025):
    """Requests with N log-uniform in [1000, 300000], input dim 50, each a
    10-component Gaussian mixture (centres ~ N(0, 10^2 I), unit variance);
    method Barnes-Hut or FIt-SNE with probability 1/2."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(requests):
        n = int(np.exp(rng.uniform(np.log(1000), np.log(300000))))
        centres = rng.normal(0.0, 10.0, size=(10, 50)).astype(np.float32)
        lab = rng.integers(0, 10, size=n)
        X = np.ascontiguousarray(centres[lab] + rng.standard_normal(size=(n, 50), dtype=np.float32))
        method = "bh" if rng.random() < 0.5 else "fit"
        out.append((X, method, 1000 + i))
    return out


def run_serving(args, ctx):
    """The request stream through bhtsne_server (continuous batching) against
    the same stream served one request at a time by the plain builder. Both
    arms see the same Poisson arrivals; latency = completion - arrival."""
    import bhtsne_gb300 as bg
    reqs = make_serving_workload(args.serve_requests)
    E = args.serve_epochs
    rng = np.random.default_rng(77)
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, size=len(reqs)))
    budget = int(args.serve_budget_gb * 1e9) if args.serve_budget_gb > 0 else 0
    sv = bg.Server(ctx=ctx, perplexity=30.0, theta=0.5, fit_workers=args.serve_fit_workers, hbm_budget_bytes=budget)
    ids = [None] * len(reqs)
    w0 = time.perf_counter()
    for i, (X, method, seed) in enumerate(reqs):
        delay = arrivals[i] - (time.perf_counter() - w0)
        if delay > 0:
            time.sleep(delay)
        ids[i] = sv.submit(X, method, epochs=E, seed=seed, want_kl=True)
    lat_s, kl_s = [], []
    for i in ids:
        sv.wait(i)
        _, kl, lat = sv.result(i)
        lat_s.append(lat / 1e3)
        kl_s.append(kl)
    served_s = time.perf_counter() - w0
    st = sv.stats()
    sv.close()
    # plain arm: one request at a time, in arrival order
    lat_p, kl_p = [], []
    w0 = time.perf_counter()
    for i, (X, method, seed) in enumerate(reqs):
        now = time.perf_counter() - w0
        if now < arrivals[i]:
            time.sleep(arrivals[i] - now)
        t = bg.TSNE(X, ctx=ctx).perplexity(30.0).epochs(E).random_seed(seed)
        t.barnes_hut(0.5) if method == "bh" else t.fit_sne()
        t.embedding()
        kl_p.append(t.kl_divergence())
        t.close()
        lat_p.append(time.perf_counter() - w0 - arrivals[i])
    plain_s = time.perf_counter() - w0
    gap = np.abs(np.array(kl_s) - np.array(kl_p)) / np.abs(np.array(kl_p))
    J = len(reqs)
    return {
        "workload": f"{J} requests, N log-uniform [1000, 300000] (total {sum(len(r[0]) for r in reqs)} points), "
                    f"input dim 50, 10-component mixtures, Barnes-Hut theta 0.5 / FIt-SNE 50:50 "
                    f"({sum(r[1] == 'bh' for r in reqs)} BH), perplexity 30, 2-D, {E} epochs, Poisson arrivals "
                    f"at {args.serve_rate}/s",
        "jobs_per_s": round(J / served_s, 3), "plain_jobs_per_s": round(J / plain_s, 3),
        "speedup_vs_plain": round(plain_s / served_s, 3),
        "latency_s": {"p50": round(float(np.percentile(lat_s, 50)), 3), "p99": round(float(np.percentile(lat_s, 99)), 3),
                      "plain_p50": round(float(np.percentile(lat_p, 50)), 3),
                      "plain_p99": round(float(np.percentile(lat_p, 99)), 3)},
        "peak_admitted_bytes": st["peak_bytes"], "budget_bytes": budget if budget else "90% of free device memory",
        "mean_batch_points": round(st["mean_batch_points"], 1),
        "fit_workers": args.serve_fit_workers,
        "server_busy_s": {k: round(st[k], 3) for k in ("round_s", "repack_s", "prepare_s", "fit_worker_s")},
        "kl_gap": {"mean": round(float(gap.mean()), 5), "p99": round(float(np.percentile(gap, 99)), 5),
                   "max": round(float(gap.max()), 5), "within_1pct": int((gap <= 0.01).sum())},
    }


def cpu_baseline_sample(aff, y0, epochs, count_at=None):
    """The oracle (C++/OpenMP restatement) on the same CSR for a bounded number
    of 1M-point epochs from y0, the embedding after the GPU's timed window, with
    the exaggeration over and the final momentum (the window's own settings).
    With count_at, also the work of one Barnes-Hut repulsion pass at that
    embedding (theta tests and accepted cells of the reference's walk),
    untimed."""
    from oracle import pyoracle as O
    n = y0.shape[0]
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    t = O.TSNE(n).epochs(epochs).stop_lying_epoch(0).momentum(0.8).initial_embedding(y0)
    t.with_affinities(aff.rows, aff.columns, aff.values, aff.perplexity)
    dummy = np.zeros((n, 1), np.float32)
    w0 = time.perf_counter()
    t.barnes_hut(0.5, dummy)
    s = time.perf_counter() - w0
    out = {"value": round(epochs / s, 4), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{epochs} Barnes-Hut epochs at N={n} on the same CSR from the embedding after the timed "
                     "window (oracle C++ restatement, OpenMP; includes its P normalisation)"}
    if count_at is not None:
        try:
            vis, inter = O.bh_interactions(np.ascontiguousarray(count_at, dtype=np.float32), 0.5)
            out["bh_work_per_epoch"] = {"theta_tests": int(vis), "interactions": int(inter)}
        except Exception as exc:  # a measurement aid: never fails the run
            out["bh_work_per_epoch_error"] = str(exc)[:200]
    return out


def run_reference(args):
    """The reference arm: the oracle (the reference's CPU path restated in C++,
    OpenMP on every host core) on the same workload, from the same initial
    embedding, through one continuous fit of burn-in + warm-up + steps epochs;
    the timed region is the window of `steps` epochs after the first
    burn-in + warm-up ones, timed inside the fit by the epoch callback."""
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import ctypes as C
    from oracle import pyoracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    n = args.n
    X, lab = make_workload(n, seed=args.seed)
    idx, dist = within_cluster_knn(X, lab, 90)
    del X
    first = args.burn_in + args.warmup
    total = first + args.steps
    stamps = {}

    def on_epoch(epoch, yptr, user):
        if epoch == first - 1 or epoch == total - 1:
            stamps[int(epoch)] = time.perf_counter()

    cb = O.EPOCH_CB(on_epoch)
    h = O.TSNE(n).perplexity(30.0).epochs(total).initial_embedding(initial_embedding(n))
    O.lib().orc_tsne_set_epoch_callback(h._h, C.cast(cb, C.c_void_p), None)
    w0 = time.perf_counter()
    h.barnes_hut_with_neighbors(0.5, idx, dist)
    fit_s = time.perf_counter() - w0
    s = stamps[total - 1] - stamps[first - 1]
    v = args.steps / s
    out = {"metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(1e3 * s / args.steps, 2), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
           "config": workload_config(args, 1),
           "nnz": int(h.affinities()[2].size),
           "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"epochs {first}-{total - 1} of one {total}-epoch Barnes-Hut fit at N={n} "
                                      "(oracle C++ restatement, OpenMP), timed by the epoch callback; "
                                      "affinities from a within-cluster kNN (untimed)",
                            "fit_s": round(fit_s, 2)},
           "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_fft_only(args):
    """FIt-SNE repulsion alone (spread, transforms, gather) for --n points
    spread uniformly over [-700, 700]^2: the 1000-box cap, 3000 nodes per
    axis, transforms of length 6144. --warmup untimed calls, then --steps
    timed ones."""
    import bhtsne_gb300 as bg
    ctx = bg.Context(0)
    y = np.random.default_rng(args.seed).uniform(-700, 700, size=(args.n, 2)).astype(np.float32)
    rows = np.zeros(args.n + 1, np.uint64)
    empty_c, empty_v = np.zeros(0, np.uint32), np.zeros(0, np.float32)
    for _ in range(args.warmup):
        bg.gradient(bg.METHOD_FIT_SNE, y, rows, empty_c, empty_v, ctx=ctx)
    w0 = time.perf_counter()
    for _ in range(args.steps):
        bg.gradient(bg.METHOD_FIT_SNE, y, rows, empty_c, empty_v, ctx=ctx)
    ms = 1e3 * (time.perf_counter() - w0) / args.steps
    print(json.dumps({"fft_only": {"n_points": args.n, "grid": "1000 boxes per axis, transforms of length 6144",
                                   "ms_per_call": round(ms, 3),
                                   "note": "host wall time per call, including the copies of y in and forces out"}}))


def run_fit_only(args):
    """The 1M FIt-SNE configuration alone (2-D, the bh2d workload's affinities at
    --n points, seeded start): --burn-in, --warmup and --steps epochs, then a
    profiled pass for the phase split, as in the configurations leg."""
    import bhtsne_gb300 as bg
    ctx = bg.Context(0)
    X, _ = make_workload(args.n, seed=args.seed)
    t0 = bg.TSNE(X, D=2, ctx=ctx).perplexity(30.0).epochs(0).initial_embedding(initial_embedding(args.n))
    t0.barnes_hut(0.5)
    aff = t0.affinities()
    t0.close()
    t = bg.TSNE(args.n, D=2, ctx=ctx).with_affinities(aff).epochs(0).initial_embedding(initial_embedding(args.n))
    t.fit_sne()
    eps, ph = timed_epochs(t, args)
    print(json.dumps({"fitsne2d": {"n_points": args.n, "epochs_per_s": eps, "phase_ms_per_epoch": ph,
                                   "burn_in_epochs": args.burn_in, "steps": args.steps}}))


def run_knn_only(args):
    """The affinity build's kNN alone on the 1M workload's distribution at --n
    points (k = 90): a 2,000-row warm-up call, then all rows, timed on the host."""
    import bhtsne_gb300 as bg
    from bhtsne_gb300 import _lib as L
    X, _ = make_workload(args.n, seed=args.seed)
    bg.knn_euclidean(X[:2000], 90)
    w0 = time.perf_counter()
    bg.knn_euclidean(X, 90)
    el = time.perf_counter() - w0
    staged = os.environ.get("BHTSNE_KNN_TC_STAGED", "0") not in ("", "0")
    print(json.dumps({"metric": "exact kNN seconds (k = 90)", "value": round(el, 4), "unit": "s",
                      "higher_is_better": False, "fallback_rows": L.default_context().knn_fallback_rows(),
                      "brute_rows": L.default_context().knn_brute_rows(),
                      "candidate_pass": "staged" if staged else "resident",
                      "config": {"n_points": args.n, "input_dim": 128, "k": 90}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--seed", type=int, default=1003)
    ap.add_argument("--cpu-epochs", type=int, default=3)
    ap.add_argument("--burn-in", type=int, default=250, help="untimed epochs before the warm-up")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the 1M-point parity checks")
    ap.add_argument("--e2e-reps", type=int, default=5, help="repetitions of the end-to-end leg (median reported)")
    ap.add_argument("--parity-rows", type=int, default=2000, help="kNN query rows checked against brute force")
    ap.add_argument("--batch-jobs", type=int, default=512, help="batched-fit comparison (0 to skip)")
    ap.add_argument("--batch-epochs", type=int, default=500)
    ap.add_argument("--serve-requests", type=int, default=48, help="serving comparison (0 to skip)")
    ap.add_argument("--serve-epochs", type=int, default=750)
    ap.add_argument("--serve-rate", type=float, default=64.0, help="Poisson arrivals per second")
    ap.add_argument("--serve-fit-workers", type=int, default=8, help="server streams for FIt-SNE requests")
    ap.add_argument("--serve-budget-gb", type=float, default=0.0,
                    help="server admission budget in GB (0: 90%% of free device memory)")
    ap.add_argument("--serve-only", action="store_true", help="run only the serving comparison")
    ap.add_argument("--batch-only", action="store_true", help="run only the batched arm of the batch comparison")
    ap.add_argument("--knn-only", action="store_true", help="time only the kNN of the workload at --n points")
    ap.add_argument("--fit-only", action="store_true",
                    help="time only the 2-D FIt-SNE configuration on the workload's affinities at --n points")
    ap.add_argument("--fft-only", action="store_true",
                    help="time only the FIt-SNE repulsion of --n points at the largest grid")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the other configurations (3-D, FIt-SNE, 70k, 5k accuracy)")
    args = ap.parse_args()
    if args.fft_only:
        return run_fft_only(args)
    if args.knn_only:
        run_knn_only(args)
        return
    if args.fit_only:
        run_fit_only(args)
        return
    if args.serve_only:
        import bhtsne_gb300 as bg
        print(json.dumps({"serving": run_serving(args, bg.Context(0))}))
        return
    if args.batch_only:
        import bhtsne_gb300 as bg
        print(json.dumps({"batched_arm": run_batched_only(args, bg.Context(0))}))
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        if args.steps > 30:
            args.steps = 30  # bounded CPU sample: each step is a full 1M-point epoch
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
