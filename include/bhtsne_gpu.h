/*
 * bhtsne_gpu.h - C ABI of the GB300 (sm_103a) t-SNE library.
 *
 * This is the drop-in boundary for the fitting path of the Rust crate bhtsne
 * 0.7.10. The reference has no FFI of its own; its public surface is the
 * `tSNE<'data, T, U, const D>` builder in src/lib.rs. Every entry point below
 * names the reference item it stands in for (path:line in the reference
 * crate), so that a thin Rust wrapper can re-export the builder with the
 * same method names, defaults and panic messages.
 *
 * Conventions
 *  - Every call returns an int status: BHTSNE_OK (0) or an error code. The
 *    reference's panics become BHTSNE_EINVAL with the reference's message
 *    text, readable through bhtsne_tsne_last_error / bhtsne_ctx_last_error.
 *  - All array arguments are HOST pointers owned by the caller; the library
 *    copies in and out. Device state (affinities, embedding, gains, velocity)
 *    lives in the handle until bhtsne_tsne_free.
 *  - A handle computes in one scalar type fixed at creation (the reference's
 *    T): BHTSNE_F32 or BHTSNE_F64. `const void*` / `void*` value buffers hold
 *    that type. Neighbour indices are uint64_t (the reference's usize),
 *    sparse columns uint32_t, sparse row offsets uint64_t.
 *  - A context owns one CUDA stream on one device and is single-threaded;
 *    separate contexts may be used from separate threads.
 */
#ifndef BHTSNE_GPU_H
#define BHTSNE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BHTSNE_OK 0
#define BHTSNE_EIO 5
#define BHTSNE_ENOMEM 12
#define BHTSNE_EINVAL 22
#define BHTSNE_ETIMEDOUT 110
#define BHTSNE_ECUDA 1001
#define BHTSNE_EINTERNAL 1002

#define BHTSNE_F32 0
#define BHTSNE_F64 1

/* Fitting routines, as recorded by the reference's `enum Fit` (src/lib.rs:99-103). */
#define BHTSNE_METHOD_EXACT 1
#define BHTSNE_METHOD_BARNES_HUT 2
#define BHTSNE_METHOD_FIT_SNE 3

typedef struct bhtsne_ctx bhtsne_ctx;
typedef struct bhtsne_tsne bhtsne_tsne;

/* Epoch callback: `EpochCallback` (src/lib.rs:95), invoked on the calling
 * thread after each epoch with a host snapshot of the embedding (n * D values
 * of the handle's type). */
typedef void (*bhtsne_epoch_cb)(int64_t epoch, const void* embedding, void* user);

/* ---- context ------------------------------------------------------------- */
/* No reference counterpart: owns the device, stream and scratch. */
int bhtsne_ctx_create(int device, bhtsne_ctx** out);
int bhtsne_ctx_destroy(bhtsne_ctx* ctx);
const char* bhtsne_ctx_last_error(const bhtsne_ctx* ctx);
const char* bhtsne_version(void);
/* No reference counterpart: the number of rows of the last Euclidean kNN run
 * on this context (bhtsne_knn_euclidean, or the affinity build of a dense
 * barnes_hut / fit_sne finisher) whose candidate list failed the exactness
 * certificate and were recomputed exactly: by a bounded re-scan (every
 * candidate within the row's error bound, re-ranked exactly) after the
 * tensor-core pass, else by brute force. */
int bhtsne_ctx_knn_fallback_rows(const bhtsne_ctx* ctx, int64_t* rows);
/* No reference counterpart: of those rows, the ones recomputed by exact brute
 * force (their bounded re-scan list overflowed, or no re-scan applied). */
int bhtsne_ctx_knn_brute_rows(const bhtsne_ctx* ctx, int64_t* rows);

/* ---- builder ------------------------------------------------------------- */
/* tSNE::new (src/lib.rs:241-266): defaults lr auto, 1000 epochs, momentum
 * 0.5 -> 0.8 at epoch 250, stop lying at 250, exaggeration 12, perplexity 20.
 * `embed_dim` is the const generic D: 2..7 for Barnes-Hut (the reference's
 * Morton<D> bound), 1..2 for FIt-SNE, 1..7 for exact. */
int bhtsne_tsne_new(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, int64_t n_samples, bhtsne_tsne** out);
int bhtsne_tsne_free(bhtsne_tsne* t);
const char* bhtsne_tsne_last_error(const bhtsne_tsne* t);

/* Setters: src/lib.rs:277-435. */
int bhtsne_tsne_learning_rate(bhtsne_tsne* t, double learning_rate);        /* :277 */
int bhtsne_tsne_epochs(bhtsne_tsne* t, int64_t epochs);                      /* :288 */
int bhtsne_tsne_momentum(bhtsne_tsne* t, double momentum);                   /* :299 */
int bhtsne_tsne_final_momentum(bhtsne_tsne* t, double final_momentum);       /* :310 */
int bhtsne_tsne_momentum_switch_epoch(bhtsne_tsne* t, int64_t epoch);        /* :322 */
int bhtsne_tsne_stop_lying_epoch(bhtsne_tsne* t, int64_t epoch);             /* :338 */
int bhtsne_tsne_early_exaggeration(bhtsne_tsne* t, double exaggeration);     /* :352 */
int bhtsne_tsne_perplexity(bhtsne_tsne* t, double perplexity);               /* :367 */
int bhtsne_tsne_epoch_callback(bhtsne_tsne* t, bhtsne_epoch_cb cb, void* user); /* :415 */
int bhtsne_tsne_initial_embedding(bhtsne_tsne* t, const void* y, int64_t len);  /* :431 */
/* No reference counterpart: the reference's random_init (src/tsne/mod.rs:142-147)
 * draws N(0, 1e-4) from an unseeded generator; here the draw is seeded. */
int bhtsne_tsne_random_seed(bhtsne_tsne* t, uint64_t seed);

/* Finishers. `data` is n_samples x dim, row-major, of the handle's type. */
/* exact (src/lib.rs:489-646) with the Euclidean distance (squared = 0) or the
 * squared Euclidean distance (squared = 1) as `distance_f`. */
int bhtsne_tsne_exact_euclidean(bhtsne_tsne* t, const void* data, int32_t dim, int32_t squared);
/* exact with an arbitrary `distance_f`, given as its n x n matrix (only the
 * strict upper triangle is read, as the reference evaluates it). */
int bhtsne_tsne_exact_distances(bhtsne_tsne* t, const void* distances);
/* barnes_hut (src/lib.rs:701-742) with the Euclidean metric. */
int bhtsne_tsne_barnes_hut_euclidean(bhtsne_tsne* t, double theta, const void* data, int32_t dim);
/* barnes_hut_with_neighbors (src/lib.rs:757-772): rows x k table of
 * Neighbor{index, distance} (src/lib.rs:108-111) split into two arrays. */
int bhtsne_tsne_barnes_hut_with_neighbors(bhtsne_tsne* t, double theta, const uint64_t* indices,
                                          const void* distances, int64_t rows, int64_t k);
/* fit_sne (src/lib.rs:835-871) with the Euclidean metric. */
int bhtsne_tsne_fit_sne_euclidean(bhtsne_tsne* t, const void* data, int32_t dim);
/* fit_sne_with_neighbors (src/lib.rs:884-894). */
int bhtsne_tsne_fit_sne_with_neighbors(bhtsne_tsne* t, const uint64_t* indices, const void* distances, int64_t rows,
                                       int64_t k);

/* Getters. */
/* embedding (src/lib.rs:438-440): n * D values. */
int bhtsne_tsne_embedding(bhtsne_tsne* t, void* out);
/* kl_divergence (src/lib.rs:448-477). *has_value = 0 before a fit. With
 * quirk = 1 the sparse cost reads the value array at the row index, exactly
 * as the reference does (src/tsne/mod.rs:768-770); quirk = 0 gives the
 * textbook sum over the CSR entries. The exact method ignores `quirk`. */
int bhtsne_tsne_kl_divergence(bhtsne_tsne* t, int32_t quirk, double* out, int32_t* has_value);
/* affinities (src/lib.rs:1019-1037): pristine (un-exaggerated) CSR. Pass NULL
 * arrays to query nnz first. *has_value = 0 when no sparse graph exists. */
int bhtsne_tsne_affinities(bhtsne_tsne* t, uint64_t* rows, uint32_t* columns, void* values, int64_t* nnz,
                           double* perplexity, int32_t* has_value);
/* with_affinities (src/lib.rs:1043-1051). rows has n_rows entries. */
int bhtsne_tsne_with_affinities(bhtsne_tsne* t, const uint64_t* rows, int64_t n_rows, const uint32_t* columns,
                                const void* values, int64_t nnz, double perplexity);

/* No reference counterpart: continues the last fit for `epochs` more epochs on
 * the device-resident state (same epoch numbering, exaggeration and momentum
 * schedule), so that fit(E1) followed by advance(E2) equals fit(E1 + E2). */
int bhtsne_tsne_advance(bhtsne_tsne* t, int64_t epochs);
/* No reference counterpart: device time of the last affinity build and of the
 * epochs run by the last finisher or advance call (CUDA events, ms). */
int bhtsne_tsne_timings(const bhtsne_tsne* t, double* affinity_ms, double* loop_ms, int64_t* loop_epochs);

/* No reference counterpart: per-phase device times of the epoch loop. With
 * profiling enabled, each epoch records CUDA events on the handle's stream
 * around the phases below; bhtsne_tsne_phase_times returns the summed ms and
 * the number of timed epochs of the last finisher or advance call. */
#define BHTSNE_PHASE_TREE 0       /* Morton codes, radix sort, tree build */
#define BHTSNE_PHASE_REPULSION 1  /* BH traversal, or FIt-SNE spread/convolution/gather, or exact gradient */
#define BHTSNE_PHASE_ATTRACTIVE 2 /* CSR attractive forces */
#define BHTSNE_PHASE_UPDATE 3     /* fused update + recentre + bounding box */
#define BHTSNE_PHASES 4
int bhtsne_tsne_profile(bhtsne_tsne* t, int32_t enable);
int bhtsne_tsne_phase_times(const bhtsne_tsne* t, double* ms, int64_t* epochs);
/* No reference counterpart: device time (CUDA events, ms, summed) and number of
 * the locality re-layouts run by the last finisher or advance call. The sparse
 * methods re-lay out y, the velocity, the gains and the CSR in the Morton
 * order of the current embedding every 50 epochs (epochs 50, 100, ...). */
int bhtsne_tsne_relayout_times(const bhtsne_tsne* t, double* ms, int64_t* count);
/* No reference counterpart: the layout of the last fit. *component_layout is
 * 1 when the points were grouped by connected component of P's graph, once,
 * at the first periodic re-layout point (epoch 50; Barnes-Hut fits of at least
 * 65,536 points whose graph splits into components of at most n / 4 points;
 * no Morton re-layout after it), 0 otherwise; *largest_component is the size
 * of P's largest component, 0 when it was not computed (fits shorter than a
 * re-layout period, or not eligible). BHTSNE_COMPONENT_LAYOUT=0 turns the
 * component layout off, =2 also applies it below 65,536 points. */
int bhtsne_tsne_layout_info(const bhtsne_tsne* t, int32_t* component_layout, int64_t* largest_component);
/* Number of CUDA kernel launches this library has issued since it was loaded. */
int64_t bhtsne_launch_count(void);

/* ---- stage entry points (parity and integration seams) -------------------- */
/* Exact kNN under the Euclidean metric, the result the VP-tree search
 * (src/tsne/vptree.rs:274-319) returns for `barnes_hut`: per row the k nearest
 * other rows by (distance, index). idx/dist are n x k. */
int bhtsne_knn_euclidean(bhtsne_ctx* ctx, int dtype, const void* data, int64_t n, int32_t dim, int32_t k,
                         uint32_t* indices, void* distances);
/* search_beta per row (src/tsne/mod.rs:201-275): conditional P (n x k) from
 * neighbour distances (n x k). iterations (optional, n) gets the bisection
 * count per row. */
int bhtsne_conditional_p(bhtsne_ctx* ctx, int dtype, const void* distances, int64_t n, int32_t k, double perplexity,
                         void* p, int32_t* iterations);
/* symmetrize_sparse_matrix (src/tsne/mod.rs:306-406): symmetric CSR from the
 * kNN table (n x k columns and conditional P). Call with NULL outputs to get
 * nnz, then with rows (n + 1), columns (nnz), values (nnz). */
int bhtsne_symmetrize(bhtsne_ctx* ctx, int dtype, const uint32_t* columns, const void* p, int64_t n, int32_t k,
                      uint64_t* rows_out, uint32_t* columns_out, void* values_out, int64_t* nnz);
/* Repulsion::step (src/repulsion.rs:31-54): attractive forces `pos`,
 * repulsive forces `neg` (n x D) and Z at a fixed embedding y, for
 * BHTSNE_METHOD_BARNES_HUT (theta) or BHTSNE_METHOD_FIT_SNE. For
 * BHTSNE_METHOD_EXACT, `values` is the dense n x n P, `pos` receives the
 * exact gradient dy (src/lib.rs:596-619) and `neg` is unused. */
int bhtsne_gradient(bhtsne_ctx* ctx, int dtype, int32_t method, int32_t embed_dim, const void* y, int64_t n,
                    const uint64_t* rows, const uint32_t* columns, const void* values, int64_t nnz, double theta,
                    void* pos, void* neg, double* z);
/* No counterpart in the reference. Barnes-Hut repulsion at a fixed embedding
 * for callers that cannot allocate device memory: code recording into a CUDA
 * stream capture (cudaMalloc may not run while a capture is open), hosts that
 * give the library a fixed device budget from their own pool, and loops where
 * an allocation could synchronise the device. y (n x 2), neg (n x 2) and z (one
 * double) are DEVICE pointers owned by the caller; `stream` is a cudaStream_t
 * (NULL for the default stream). The result equals the Barnes-Hut step of
 * bhtsne_gradient. f32 and D = 2 only, 2 <= n <= 32768 points; anything else
 * returns BHTSNE_EINVAL. Scratch is one fixed ~3.4 MB device array per GPU,
 * kept until the process exits and shared by all calls: calls that overlap on
 * the GPU race, so serialise them. The first call on a device looks up the
 * array's address for that device; make it before any stream capture. */
int bhtsne_bh_repulsion_noalloc(const float* y, int64_t n, double theta, float* neg, double* z, void* stream);

/* gradient_descent_step + zero_mean (src/tsne/mod.rs:470-516, :534-568) on
 * host arrays (n x D), in place. */
int bhtsne_update(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, void* y, const void* pos, const void* neg, void* uy,
                  void* gains, int64_t n, double learning_rate, double momentum, double inverse_z);

/* ---- autotuning (no reference counterpart) --------------------------------- */
/* Times the candidates of three launch-shape knobs on synthetic data of the
 * given shape (n points in embed_dim dimensions, k neighbours per row; dim > 0
 * also tunes the kNN candidate pass on a sample of dim-dimensional points):
 * the attractive pass's task length (64, 128, 256 entries), the Barnes-Hut
 * traversal's block size (128, 256, 512 threads) and the kNN candidate pass
 * (tensor cores or CUDA cores). The fastest of each is kept for this GPU, the
 * value type, embed_dim and the N bucket floor(log2 n); fits that start later
 * use them. The traversal block size and the kNN pass do not change results;
 * the task length changes the grouping of each row's attractive terms, so a
 * fit's forces move by rounding. The timings are left in
 * bhtsne_ctx_last_error. When BHTSNE_TUNE_FILE is set, contexts read that
 * JSON table when the first one is created, and bhtsne_tune rewrites it. */
int bhtsne_tune(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, int64_t n, int32_t k, int32_t dim);
/* The configuration a fit of (dtype, embed_dim, n) on the current device would
 * use, as JSON: {"key": ..., "knobs": {...}}. Host only. */
int bhtsne_tune_config(int dtype, int32_t embed_dim, int64_t n, char* json, int64_t len);
/* Adds the entries of a tuning table file / writes the table. Host only;
 * errors from bhtsne_io_last_error. */
int bhtsne_tune_load(const char* path);
int bhtsne_tune_save(const char* path);

/* ---- CSV input and output (host only; no GPU needed) ----------------------- */
/* load_csv (src/csv.rs:61-118) for numeric data: the fields of every record,
 * except the columns listed in skip (n_skip of them), parsed as the dtype's
 * float in file order; has_headers skips the first record. The reference
 * converts fields with a caller's closure; here they are parsed as Rust's
 * str::parse does. Call with out == NULL to get *count (values) and *records;
 * then with out holding *count values. Records must all have the first
 * record's field count. Errors: BHTSNE_EIO (file), BHTSNE_EINVAL (a field
 * that does not parse, a ragged record), with a message from
 * bhtsne_io_last_error (per thread). */
int bhtsne_load_csv(const char* path, int32_t has_headers, const int64_t* skip, int64_t n_skip, int dtype, void* out,
                    int64_t* count, int64_t* records);
/* write_csv (src/csv.rs:31-58) of a fitted handle's embedding: one point per
 * record, headers "x,y" (D = 2) or "x,y,z" (D = 3), values printed as Rust's
 * Display prints a float (shortest round-trip decimal, no exponent). */
int bhtsne_tsne_write_csv(bhtsne_tsne* t, const char* path);
/* No reference counterpart: write_csv of an embedding held by the caller
 * (n x embed_dim values of dtype), e.g. a batch or server result. */
int bhtsne_write_csv(const void* embedding, int64_t n, int32_t embed_dim, int dtype, const char* path);
/* The npz input of the reference's example (examples/mnist_pca_tsne.rs:39-44,
 * npyz 0.9 NpzArchive::open + by_name + into_vec): array `name` (without its
 * ".npy" suffix) of an .npz archive, entries stored or deflated, ZIP64
 * included, in C order (Fortran-order arrays are reordered) and converted to
 * the dtype's float. Element types: little-endian f4, f8, i1..i8, u1..u8, b1.
 * Call with out == NULL to get *count (values), *ndim and shape[0 .. min(ndim,
 * 8)) (ndim and shape may be NULL); then with out holding *count values.
 * Errors: BHTSNE_EIO (file), BHTSNE_EINVAL (not an npz archive, no such array,
 * unsupported type, corrupt or truncated data), with a message from
 * bhtsne_io_last_error (per thread). Host only. */
int bhtsne_load_npz(const char* path, const char* name, int dtype, void* out, int64_t* count, int32_t* ndim,
                    int64_t* shape);
const char* bhtsne_io_last_error(void);

/* ---- batches of independent fits (no reference counterpart) --------------- */
/* Many independent Barnes-Hut embeddings of uneven size, fitted together: every
 * stage of an epoch (box, Morton sort, tree, traversal, Z, attractive pass,
 * update) runs once for the whole batch. Each job follows the reference's
 * schedule (defaults of tSNE::new, src/lib.rs:241-266) with its own learning
 * rate max(n_j / exaggeration / 4, 50) and its own Z, mean and tree. */
typedef struct bhtsne_batch bhtsne_batch;
typedef struct bhtsne_batch_params {
  double perplexity;             /* 20 */
  int64_t epochs;                /* 1000 */
  double learning_rate;          /* <= 0: automatic per job */
  double momentum;               /* 0.5 */
  double final_momentum;         /* 0.8 */
  int64_t momentum_switch_epoch; /* 250 */
  int64_t stop_lying_epoch;      /* 250 */
  double early_exaggeration;     /* 12 */
  double theta;                  /* 0.5 */
  uint64_t seed;                 /* job j's random_init is seeded with seed + j */
} bhtsne_batch_params;
void bhtsne_batch_params_default(bhtsne_batch_params* p);
int bhtsne_batch_new(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, const bhtsne_batch_params* p, bhtsne_batch** out);
int bhtsne_batch_free(bhtsne_batch* b);
const char* bhtsne_batch_last_error(const bhtsne_batch* b);
/* Adds a job from dense data (Euclidean kNN on the device) or from a kNN table;
 * its affinities are built immediately. *job receives the job index. */
int bhtsne_batch_add_euclidean(bhtsne_batch* b, const void* data, int64_t n, int32_t dim, int64_t* job);
int bhtsne_batch_add_with_neighbors(bhtsne_batch* b, const uint64_t* indices, const void* distances, int64_t n,
                                    int64_t k, int64_t* job);
int bhtsne_batch_initial_embedding(bhtsne_batch* b, int64_t job, const void* y);
/* Runs params.epochs Barnes-Hut epochs for every job. */
int bhtsne_batch_fit(bhtsne_batch* b);
int64_t bhtsne_batch_jobs(const bhtsne_batch* b);
int bhtsne_batch_embedding(bhtsne_batch* b, int64_t job, void* out);
int bhtsne_batch_kl_divergence(bhtsne_batch* b, int64_t job, int32_t quirk, double* out);
int bhtsne_batch_timings(const bhtsne_batch* b, double* affinity_ms, double* loop_ms);

/* ---- serving: continuous batching of embedding requests ----------------
 * No reference counterpart (the reference fits one embedding per builder).
 * Requests are queued, admitted in order while their estimated device
 * footprint fits the byte budget, and fitted concurrently: Barnes-Hut
 * requests join one running batch (all in-flight jobs stepped together, each
 * with its own epoch count; jobs enter and leave every round_epochs epochs),
 * FIt-SNE requests run on fit_workers extra streams. Every request uses the
 * reference's defaults (early exaggeration 12 until epoch 250, momentum 0.5
 * then 0.8, learning rate max(n / 12 / 4, 50)) and the server's perplexity and
 * theta. A server owns host threads; its calls are thread-safe. */
typedef struct bhtsne_server bhtsne_server;
typedef struct bhtsne_server_params {
  double perplexity;        /* 30 (k = 3 * perplexity <= 224) */
  double theta;             /* 0.5, for Barnes-Hut requests */
  int64_t hbm_budget_bytes; /* admission budget; <= 0: 90% of the free device memory at creation */
  int32_t round_epochs;     /* epochs between batch changes (25) */
  int32_t fit_workers;      /* streams for FIt-SNE requests (2) */
} bhtsne_server_params;
typedef struct bhtsne_request {
  const void* data; /* n x dim row-major in the server's dtype; copied by submit */
  int64_t n;
  int32_t dim;
  int32_t method; /* BHTSNE_METHOD_BARNES_HUT or BHTSNE_METHOD_FIT_SNE */
  int64_t epochs;
  uint64_t seed;   /* random_init seed of this request */
  int32_t want_kl; /* nonzero: compute the reference-compatible KL of the result */
} bhtsne_request;
#define BHTSNE_JOB_QUEUED 0
#define BHTSNE_JOB_RUNNING 1
#define BHTSNE_JOB_DONE 2
#define BHTSNE_JOB_FAILED 3
void bhtsne_server_params_default(bhtsne_server_params* p);
/* embed_dim 2 or 3 (FIt-SNE requests need 2). */
int bhtsne_server_new(bhtsne_ctx* ctx, int dtype, int32_t embed_dim, const bhtsne_server_params* p,
                      bhtsne_server** out);
/* Stops the threads after the current round; unfinished requests fail. */
int bhtsne_server_free(bhtsne_server* s);
const char* bhtsne_server_last_error(const bhtsne_server* s);
int bhtsne_server_submit(bhtsne_server* s, const bhtsne_request* r, int64_t* id);
int bhtsne_server_poll(bhtsne_server* s, int64_t id, int32_t* state);
/* timeout_s < 0 waits without limit; BHTSNE_ETIMEDOUT when it runs out. */
int bhtsne_server_wait(bhtsne_server* s, int64_t id, double timeout_s);
/* Copies the n x embed_dim embedding (and KL, submit-to-done latency) of a
 * finished request and forgets it; a failed request returns its error. */
int bhtsne_server_result(bhtsne_server* s, int64_t id, void* embedding, double* kl, double* latency_ms);
int bhtsne_server_stats(bhtsne_server* s, int64_t* done, int64_t* in_flight, int64_t* peak_bytes,
                        double* mean_batch_points);
/* Host seconds spent so far: Barnes-Hut rounds, repacks, affinity preparation,
 * FIt-SNE requests (summed over workers). */
int bhtsne_server_timings(bhtsne_server* s, double* round_s, double* repack_s, double* prepare_s, double* fit_s);

#ifdef __cplusplus
}
#endif

#endif /* BHTSNE_GPU_H */
