//! Raw declarations of the C ABI in `include/bhtsne_gpu.h`, one per function,
//! in the header's order. Every call returns a status (0 = BHTSNE_OK); the
//! message of a failed call is read with the matching `*_last_error`. Arrays
//! are host pointers owned by the caller unless a comment says otherwise.
//!
//! Not compiled here (no cargo or rustc on either machine); the safe builder
//! with the reference's names is the `bhtsne-gpu` crate next to this one.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const BHTSNE_OK: c_int = 0;
pub const BHTSNE_EIO: c_int = 5;
pub const BHTSNE_ENOMEM: c_int = 12;
pub const BHTSNE_EINVAL: c_int = 22;
pub const BHTSNE_ETIMEDOUT: c_int = 110;
pub const BHTSNE_ECUDA: c_int = 1001;
pub const BHTSNE_EINTERNAL: c_int = 1002;

pub const BHTSNE_F32: c_int = 0;
pub const BHTSNE_F64: c_int = 1;

pub const BHTSNE_METHOD_EXACT: i32 = 1;
pub const BHTSNE_METHOD_BARNES_HUT: i32 = 2;
pub const BHTSNE_METHOD_FIT_SNE: i32 = 3;

pub const BHTSNE_PHASE_TREE: usize = 0;
pub const BHTSNE_PHASE_REPULSION: usize = 1;
pub const BHTSNE_PHASE_ATTRACTIVE: usize = 2;
pub const BHTSNE_PHASE_UPDATE: usize = 3;
pub const BHTSNE_PHASES: usize = 4;

pub const BHTSNE_JOB_QUEUED: i32 = 0;
pub const BHTSNE_JOB_RUNNING: i32 = 1;
pub const BHTSNE_JOB_DONE: i32 = 2;
pub const BHTSNE_JOB_FAILED: i32 = 3;

#[repr(C)]
pub struct bhtsne_ctx {
    _p: [u8; 0],
}
#[repr(C)]
pub struct bhtsne_tsne {
    _p: [u8; 0],
}
#[repr(C)]
pub struct bhtsne_batch {
    _p: [u8; 0],
}
#[repr(C)]
pub struct bhtsne_server {
    _p: [u8; 0],
}

/// `EpochCallback` (src/lib.rs:95): epoch index and a host snapshot of n * D values.
pub type bhtsne_epoch_cb = Option<unsafe extern "C" fn(epoch: i64, embedding: *const c_void, user: *mut c_void)>;

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bhtsne_batch_params {
    pub perplexity: f64,
    pub epochs: i64,
    pub learning_rate: f64,
    pub momentum: f64,
    pub final_momentum: f64,
    pub momentum_switch_epoch: i64,
    pub stop_lying_epoch: i64,
    pub early_exaggeration: f64,
    pub theta: f64,
    pub seed: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bhtsne_server_params {
    pub perplexity: f64,
    pub theta: f64,
    pub hbm_budget_bytes: i64,
    pub round_epochs: i32,
    pub fit_workers: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct bhtsne_request {
    pub data: *const c_void,
    pub n: i64,
    pub dim: i32,
    pub method: i32,
    pub epochs: i64,
    pub seed: u64,
    pub want_kl: i32,
}

#[link(name = "bhtsne_gpu")]
extern "C" {
    // ---- context
    pub fn bhtsne_ctx_create(device: c_int, out: *mut *mut bhtsne_ctx) -> c_int;
    pub fn bhtsne_ctx_destroy(ctx: *mut bhtsne_ctx) -> c_int;
    pub fn bhtsne_ctx_last_error(ctx: *const bhtsne_ctx) -> *const c_char;
    pub fn bhtsne_version() -> *const c_char;
    pub fn bhtsne_ctx_knn_fallback_rows(ctx: *const bhtsne_ctx, rows: *mut i64) -> c_int;
    pub fn bhtsne_ctx_knn_brute_rows(ctx: *const bhtsne_ctx, rows: *mut i64) -> c_int;

    // ---- builder: tSNE::new (src/lib.rs:241-266) and its setters (:277-435)
    pub fn bhtsne_tsne_new(ctx: *mut bhtsne_ctx, dtype: c_int, embed_dim: i32, n_samples: i64,
                           out: *mut *mut bhtsne_tsne) -> c_int;
    pub fn bhtsne_tsne_free(t: *mut bhtsne_tsne) -> c_int;
    pub fn bhtsne_tsne_last_error(t: *const bhtsne_tsne) -> *const c_char;
    pub fn bhtsne_tsne_learning_rate(t: *mut bhtsne_tsne, learning_rate: f64) -> c_int;
    pub fn bhtsne_tsne_epochs(t: *mut bhtsne_tsne, epochs: i64) -> c_int;
    pub fn bhtsne_tsne_momentum(t: *mut bhtsne_tsne, momentum: f64) -> c_int;
    pub fn bhtsne_tsne_final_momentum(t: *mut bhtsne_tsne, final_momentum: f64) -> c_int;
    pub fn bhtsne_tsne_momentum_switch_epoch(t: *mut bhtsne_tsne, epoch: i64) -> c_int;
    pub fn bhtsne_tsne_stop_lying_epoch(t: *mut bhtsne_tsne, epoch: i64) -> c_int;
    pub fn bhtsne_tsne_early_exaggeration(t: *mut bhtsne_tsne, exaggeration: f64) -> c_int;
    pub fn bhtsne_tsne_perplexity(t: *mut bhtsne_tsne, perplexity: f64) -> c_int;
    pub fn bhtsne_tsne_epoch_callback(t: *mut bhtsne_tsne, cb: bhtsne_epoch_cb, user: *mut c_void) -> c_int;
    pub fn bhtsne_tsne_initial_embedding(t: *mut bhtsne_tsne, y: *const c_void, len: i64) -> c_int;
    pub fn bhtsne_tsne_random_seed(t: *mut bhtsne_tsne, seed: u64) -> c_int;

    // ---- finishers: exact (:489-646), barnes_hut (:701-772), fit_sne (:835-894)
    pub fn bhtsne_tsne_exact_euclidean(t: *mut bhtsne_tsne, data: *const c_void, dim: i32, squared: i32) -> c_int;
    pub fn bhtsne_tsne_exact_distances(t: *mut bhtsne_tsne, distances: *const c_void) -> c_int;
    pub fn bhtsne_tsne_barnes_hut_euclidean(t: *mut bhtsne_tsne, theta: f64, data: *const c_void, dim: i32) -> c_int;
    pub fn bhtsne_tsne_barnes_hut_with_neighbors(t: *mut bhtsne_tsne, theta: f64, indices: *const u64,
                                                 distances: *const c_void, rows: i64, k: i64) -> c_int;
    pub fn bhtsne_tsne_fit_sne_euclidean(t: *mut bhtsne_tsne, data: *const c_void, dim: i32) -> c_int;
    pub fn bhtsne_tsne_fit_sne_with_neighbors(t: *mut bhtsne_tsne, indices: *const u64, distances: *const c_void,
                                              rows: i64, k: i64) -> c_int;

    // ---- getters: embedding (:438-440), kl_divergence (:448-477), affinities (:1019-1051)
    pub fn bhtsne_tsne_embedding(t: *mut bhtsne_tsne, out: *mut c_void) -> c_int;
    pub fn bhtsne_tsne_kl_divergence(t: *mut bhtsne_tsne, quirk: i32, out: *mut f64, has_value: *mut i32) -> c_int;
    pub fn bhtsne_tsne_affinities(t: *mut bhtsne_tsne, rows: *mut u64, columns: *mut u32, values: *mut c_void,
                                  nnz: *mut i64, perplexity: *mut f64, has_value: *mut i32) -> c_int;
    pub fn bhtsne_tsne_with_affinities(t: *mut bhtsne_tsne, rows: *const u64, n_rows: i64, columns: *const u32,
                                       values: *const c_void, nnz: i64, perplexity: f64) -> c_int;

    // ---- no reference counterpart: continuation and measurement
    pub fn bhtsne_tsne_advance(t: *mut bhtsne_tsne, epochs: i64) -> c_int;
    pub fn bhtsne_tsne_timings(t: *const bhtsne_tsne, affinity_ms: *mut f64, loop_ms: *mut f64,
                               loop_epochs: *mut i64) -> c_int;
    pub fn bhtsne_tsne_profile(t: *mut bhtsne_tsne, enable: i32) -> c_int;
    pub fn bhtsne_tsne_phase_times(t: *const bhtsne_tsne, ms: *mut f64, epochs: *mut i64) -> c_int;
    pub fn bhtsne_tsne_relayout_times(t: *const bhtsne_tsne, ms: *mut f64, count: *mut i64) -> c_int;
    pub fn bhtsne_tsne_layout_info(t: *const bhtsne_tsne, component_layout: *mut i32, largest_component: *mut i64)
                                   -> c_int;
    pub fn bhtsne_launch_count() -> i64;

    // ---- stage entry points
    pub fn bhtsne_knn_euclidean(ctx: *mut bhtsne_ctx, dtype: c_int, data: *const c_void, n: i64, dim: i32, k: i32,
                                indices: *mut u32, distances: *mut c_void) -> c_int;
    pub fn bhtsne_conditional_p(ctx: *mut bhtsne_ctx, dtype: c_int, distances: *const c_void, n: i64, k: i32,
                                perplexity: f64, p: *mut c_void, iterations: *mut i32) -> c_int;
    pub fn bhtsne_symmetrize(ctx: *mut bhtsne_ctx, dtype: c_int, columns: *const u32, p: *const c_void, n: i64, k: i32,
                             rows_out: *mut u64, columns_out: *mut u32, values_out: *mut c_void, nnz: *mut i64) -> c_int;
    pub fn bhtsne_gradient(ctx: *mut bhtsne_ctx, dtype: c_int, method: i32, embed_dim: i32, y: *const c_void, n: i64,
                           rows: *const u64, columns: *const u32, values: *const c_void, nnz: i64, theta: f64,
                           pos: *mut c_void, neg: *mut c_void, z: *mut f64) -> c_int;
    /// Device pointers; `stream` is a cudaStream_t (null: the default stream).
    pub fn bhtsne_bh_repulsion_noalloc(y: *const f32, n: i64, theta: f64, neg: *mut f32, z: *mut f64,
                                       stream: *mut c_void) -> c_int;
    pub fn bhtsne_update(ctx: *mut bhtsne_ctx, dtype: c_int, embed_dim: i32, y: *mut c_void, pos: *const c_void,
                         neg: *const c_void, uy: *mut c_void, gains: *mut c_void, n: i64, learning_rate: f64,
                         momentum: f64, inverse_z: f64) -> c_int;

    // ---- autotuning
    pub fn bhtsne_tune(ctx: *mut bhtsne_ctx, dtype: c_int, embed_dim: i32, n: i64, k: i32, dim: i32) -> c_int;
    pub fn bhtsne_tune_config(dtype: c_int, embed_dim: i32, n: i64, json: *mut c_char, len: i64) -> c_int;
    pub fn bhtsne_tune_load(path: *const c_char) -> c_int;
    pub fn bhtsne_tune_save(path: *const c_char) -> c_int;

    // ---- CSV input and output (src/csv.rs:31-118); host only
    pub fn bhtsne_load_csv(path: *const c_char, has_headers: i32, skip: *const i64, n_skip: i64, dtype: c_int,
                           out: *mut c_void, count: *mut i64, records: *mut i64) -> c_int;
    pub fn bhtsne_tsne_write_csv(t: *mut bhtsne_tsne, path: *const c_char) -> c_int;
    pub fn bhtsne_write_csv(embedding: *const c_void, n: i64, embed_dim: i32, dtype: c_int, path: *const c_char) -> c_int;
    pub fn bhtsne_load_npz(path: *const c_char, name: *const c_char, dtype: c_int, out: *mut c_void,
                           count: *mut i64, ndim: *mut i32, shape: *mut i64) -> c_int;
    pub fn bhtsne_io_last_error() -> *const c_char;

    // ---- batches of independent fits
    pub fn bhtsne_batch_params_default(p: *mut bhtsne_batch_params);
    pub fn bhtsne_batch_new(ctx: *mut bhtsne_ctx, dtype: c_int, embed_dim: i32, p: *const bhtsne_batch_params,
                            out: *mut *mut bhtsne_batch) -> c_int;
    pub fn bhtsne_batch_free(b: *mut bhtsne_batch) -> c_int;
    pub fn bhtsne_batch_last_error(b: *const bhtsne_batch) -> *const c_char;
    pub fn bhtsne_batch_add_euclidean(b: *mut bhtsne_batch, data: *const c_void, n: i64, dim: i32,
                                      job: *mut i64) -> c_int;
    pub fn bhtsne_batch_add_with_neighbors(b: *mut bhtsne_batch, indices: *const u64, distances: *const c_void,
                                           n: i64, k: i64, job: *mut i64) -> c_int;
    pub fn bhtsne_batch_initial_embedding(b: *mut bhtsne_batch, job: i64, y: *const c_void) -> c_int;
    pub fn bhtsne_batch_fit(b: *mut bhtsne_batch) -> c_int;
    pub fn bhtsne_batch_jobs(b: *const bhtsne_batch) -> i64;
    pub fn bhtsne_batch_embedding(b: *mut bhtsne_batch, job: i64, out: *mut c_void) -> c_int;
    pub fn bhtsne_batch_kl_divergence(b: *mut bhtsne_batch, job: i64, quirk: i32, out: *mut f64) -> c_int;
    pub fn bhtsne_batch_timings(b: *const bhtsne_batch, affinity_ms: *mut f64, loop_ms: *mut f64) -> c_int;

    // ---- serving
    pub fn bhtsne_server_params_default(p: *mut bhtsne_server_params);
    pub fn bhtsne_server_new(ctx: *mut bhtsne_ctx, dtype: c_int, embed_dim: i32, p: *const bhtsne_server_params,
                             out: *mut *mut bhtsne_server) -> c_int;
    pub fn bhtsne_server_free(s: *mut bhtsne_server) -> c_int;
    pub fn bhtsne_server_last_error(s: *const bhtsne_server) -> *const c_char;
    pub fn bhtsne_server_submit(s: *mut bhtsne_server, r: *const bhtsne_request, id: *mut i64) -> c_int;
    pub fn bhtsne_server_poll(s: *mut bhtsne_server, id: i64, state: *mut i32) -> c_int;
    pub fn bhtsne_server_wait(s: *mut bhtsne_server, id: i64, timeout_s: f64) -> c_int;
    pub fn bhtsne_server_result(s: *mut bhtsne_server, id: i64, embedding: *mut c_void, kl: *mut f64,
                                latency_ms: *mut f64) -> c_int;
    pub fn bhtsne_server_stats(s: *mut bhtsne_server, done: *mut i64, in_flight: *mut i64, peak_bytes: *mut i64,
                               mean_batch_points: *mut f64) -> c_int;
    pub fn bhtsne_server_timings(s: *mut bhtsne_server, round_s: *mut f64, repack_s: *mut f64, prepare_s: *mut f64,
                                 fit_s: *mut f64) -> c_int;
}
