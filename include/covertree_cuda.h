/*
 * covertree_cuda.h — C ABI of libcovertree_cuda.so, the GB300 (sm_103a) engine for
 * covertreex's residual-correlation cover tree.
 *
 * The library replaces the native surface of the reference's PyO3 module
 * `covertreex_backend` (src/lib.rs:941-952 of covertreex) on the hot path:
 *   ct_build_residual  <- build_pcct2_residual_tree(v_matrix, p_diag, coords, rbf_var,
 *                          rbf_ls, chunk_size, batch_order, ..., kernel_type)
 *                          src/lib.rs:1374-1564
 *   ct_knn_residual    <- CoverTreeWrapper.knn_query_residual(query_indices, node_to_dataset,
 *                          v_matrix, p_diag, coords, rbf_var, rbf_ls, k, kernel_type,
 *                          predecessor_mode, subtree_min_bounds)  src/lib.rs:370-507
 *                          (output contract of to_py_arrays, src/lib.rs:907-938)
 *   ct_tree_arrays     <- CoverTreeWrapper.get_parents / get_levels (src/lib.rs:840-900)
 *                          + compute_subtree_bounds_py (src/lib.rs:991-1006)
 *   ct_free            <- dropping the CoverTreeWrapper
 *   ct_last_error      <- the PyErr raised by the bindings (TypeError / RuntimeError)
 *
 * Conventions
 *   - Array arguments are DEVICE pointers unless marked "host".  Row-major, contiguous.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     asynchronous on that stream except where a comment says otherwise.
 *   - Every entry point returns CT_OK (0) or a CT_ERR_* code; ct_last_error() gives a
 *     one-line message for the calling thread's most recent failure.
 *   - Neighbour output: out_idx int64 [nq x k] dataset ids, out_dist f32 [nq x k],
 *     ascending by (distance, index); rows with fewer than k neighbours are padded
 *     with -1 / FLT_MAX (3.402823466e38).
 */
#ifndef COVERTREE_CUDA_H
#define COVERTREE_CUDA_H

#include <stdint.h>

#if defined(__GNUC__)
#define CT_API __attribute__((visibility("default")))
#else
#define CT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define CT_OK 0
#define CT_ERR_ARG 1
#define CT_ERR_CUDA 2
#define CT_ERR_STATE 3
#define CT_ERR_UNSUPPORTED 4
#define CT_ERR_TIMEOUT 5
#define CT_ERR_NOMEM 6

/* kernel_type: the reference's ResidualKernelType (src/metric.rs:44-57). */
#define CT_KERNEL_RBF 0
#define CT_KERNEL_MATERN52 1

/* order: batch order of the build (src/lib.rs:1398-1405 batch_order).
 *   CT_ORDER_HILBERT: the Python PCCT path's Hilbert curve (covertreex/algo/order/strategy.py:38-100)
 *   CT_ORDER_MORTON:  the Rust crate's `hilbert_like_order` (src/pcct.rs:27-67), a 3-D Morton code,
 *                     the identity for D != 3 */
#define CT_ORDER_NATURAL 0
#define CT_ORDER_HILBERT 1
#define CT_ORDER_MORTON 2

/* form: which search ct_knn_residual runs; all return the same neighbour contract. */
#define CT_FORM_DENSE 0     /* plain FP32, dense sweep, bit-exact reference f32 distances */
#define CT_FORM_TREE 1      /* plain FP32, cover-tree traversal                          */
#define CT_FORM_SCREENED 2  /* BF16 tcgen05 screening + compensated rescoring (FP64-grade) */

/* build flags */
#define CT_BUILD_METRIC_ONLY 1   /* skip the cover-tree build (dense / screened forms only) */
#define CT_BUILD_QUERY_SLAB 2    /* reserve 4096 rows for new points of the screened form (serving) */

typedef struct ct_tree ct_tree;

typedef struct {
    int64_t distance_evals;   /* residual distances evaluated exactly (reference `distance_evals`) */
    int64_t pairs_screened;   /* query x candidate pairs screened by the BF16 passes          */
    int64_t pairs_rescored;   /* pairs rescored exactly (compensated FP32 dot, double-float distance) */
    int64_t kernel_launches;  /* engine kernels launched by the call                          */
    double device_ms;         /* device time of the whole call (timing enabled, else 0)       */
    double screen_ms;         /* tensor-core screening sweep                                  */
    double threshold_ms;      /* setup before the sweep: query order, seeded thresholds, jobs  */
    double rescore_ms;        /* rescoring kernels                                            */
    int64_t screen_pairs_main;/* pairs screened by the main sweep                             */
    int64_t overflow_queries; /* query slots whose survivor list overflowed (rescored exhaustively) */
    int64_t pairs_exhaustive; /* of pairs_rescored, those of the exhaustive pass over overflowed slots */
} ct_stats;

/* Library version (major*10000 + minor*100 + patch). */
CT_API int ct_version(void);

/* Per-phase device timing for the calling thread (0 = off, default).  When on, each
 * ct_knn_residual records CUDA events around its kernels, synchronises its stream before
 * returning and fills the *_ms fields of ct_stats.  No counterpart in the reference. */
CT_API int ct_set_timing(int enable);

/* Cap (per calling thread) on the number of thread blocks of the FP64 kernel-matrix and
 * GEMM kernels of ct_vfactor_embed; 0 (the default) = no cap.  A serving loop sets it in
 * its build thread: with GB300's low FP64 rate a few blocks per SM already fill the FP64
 * pipe, and the SMs left free of build blocks stay available to query kernels (a
 * trade against build latency: the serving engine leaves it off by default). */
CT_API int ct_set_cta_budget(int32_t ctas);

/* Message of the calling thread's last failure ("" if none). */
CT_API const char* ct_last_error(void);

/*
 * Build the device-resident residual metric and cover tree.
 *   v [n x m], p [n], coords [n x d]: device, f32 (the reference casts to f32 too).
 *   lengthscale: HOST pointer to n_lengthscale floats (missing axes reuse entry 0,
 *   |l| < 1e-6 is clamped to 1e-6, src/metric.rs:93-101).
 *   variance: kernel variance (rbf_var).  kernel_type: CT_KERNEL_*.
 *   chunk: the reference's batch-insert chunk size, accepted for its signature; the
 *   device build inserts prefix-doubling groups instead (ct_build.cu).  order: CT_ORDER_*.
 *   seed: MIS seed.  flags: CT_BUILD_*.
 * The inputs are copied; the caller may free them after the call returns.
 * Synchronises `stream` once at the end of the build.
 */
CT_API int ct_build_residual(const float* v, const float* p, const float* coords, int64_t n, int32_t m, int32_t d,
                      float variance, const float* lengthscale, int32_t n_lengthscale, int32_t kernel_type,
                      int32_t chunk, int32_t order, uint64_t seed, int32_t flags, void* stream, ct_tree** out);

/*
 * k nearest neighbours of dataset rows q_ids[0..nq) (device int64).
 *   predecessor != 0: only neighbours j < q_id (Vecchia ordering).
 *   Ids outside [0, n) produce an all-padding row.
 *   stats may be NULL.
 */
CT_API int ct_knn_residual(ct_tree* tree, const int64_t* q_ids, int64_t nq, int32_t k, int32_t predecessor, int32_t form,
                    int64_t* out_idx, float* out_dist, ct_stats* stats, void* stream);

/*
 * Exact Euclidean kNN of `queries` [nq x d] against `points` [n x d] (device f32).
 * Replaces CoverTreeWrapper.insert + knn_query for the Euclidean metric
 * (src/lib.rs:207-223, 299-326; src/algo.rs:179-323).  predecessor != 0: query row i
 * only gets points j < i (src/algo.rs:193-195).  d <= 16, k <= 64.
 */
CT_API int ct_knn_euclidean(const float* points, int64_t n, int32_t d, const float* queries, int64_t nq, int32_t k,
                            int32_t predecessor, int64_t* out_idx, float* out_dist, void* stream);

/*
 * Allocation-free dense residual kNN.  No counterpart in the reference: for callers that
 * cannot allocate device memory (their framework owns all GPU memory through its own
 * pool, or their loop cannot afford the device synchronisation of cudaMalloc/cudaFree).
 * Same result as ct_build_residual + ct_knn_residual(..., CT_FORM_DENSE, ...), bit for
 * bit, from the caller's raw inputs (v [n x m], p [n], coords [n x d], q_ids [nq]; device)
 * into the caller's outputs (out_idx [nq x k] int64, out_dist [nq x k] f32; device).
 * lengthscale is a HOST pointer, as in ct_build_residual.
 * Scratch: one fixed __device__ array of CT_NOALLOC_SCRATCH_BYTES (64 MiB) inside the
 * library, held by every GPU (every CUDA context) that loads it until the process
 * exits.  A call needs the sum of five pieces, each rounded up to a multiple of 256
 * bytes: 4 n m + 4 n d + 4 n + 4 n + 256 (V, scaled coordinates, norms, p, inverse
 * lengthscales); beyond CT_NOALLOC_SCRATCH_BYTES it is rejected with CT_ERR_UNSUPPORTED
 * before any device work.  The first call in a CUDA context looks up the array's device
 * address (cudaGetSymbolAddress, kept for that context).  All calls in one context share
 * the array and it keeps the last call's contents (each call writes every byte it reads):
 * calls whose GPU work overlaps (different streams or threads) race and must be
 * serialised by the caller.  m must be a multiple of 16; k <= 128.  Allocates nothing.
 */
#define CT_NOALLOC_SCRATCH_BYTES (64ull << 20)
CT_API int ct_knn_residual_dense_noalloc(const float* v, const float* p, const float* coords, int64_t n, int32_t m,
                                         int32_t d, float variance, const float* lengthscale, int32_t n_lengthscale,
                                         int32_t kernel_type, const int64_t* q_ids, int64_t nq, int32_t k,
                                         int32_t predecessor, int64_t* out_idx, float* out_dist, void* stream);

/*
 * Batch order of points: out_perm[i] = row of `coords` [n x d] (device f32) at sorted
 * position i, stable (ties keep the lower row).  Replaces the PyO3 function
 * hilbert_order(coords) (src/lib.rs:954-962 -> src/pcct.rs:27-67, mode CT_ORDER_MORTON)
 * and the Python path's _hilbert_permutation (covertreex/algo/order/strategy.py:38-100,
 * mode CT_ORDER_HILBERT; keys quantised in FP64 from the f32 coordinates).
 * out_perm: device int64 [n].  Asynchronous except for the sort's small host copies.
 */
CT_API int ct_batch_order(const float* coords, int64_t n, int32_t d, int32_t mode, int64_t* out_perm, void* stream);

/*
 * Maximal independent set of a conflict graph in CSR form (indptr [n+1], indices
 * [nnz]; device int64; symmetric adjacency expected, as the reference builds it) into
 * out_sel (device int8 [n], 1 = selected).  Replaces run_mis_numba(indptr, indices,
 * seed) (covertreex/algo/_mis_numba.py:134-140): the greedy in index order when the
 * maximum degree is <= 8, else seeded Luby rounds with the reference's hash
 * priorities; *iterations (host, may be NULL) receives the reference's iteration count.
 * A malformed graph (indptr not starting at 0 or decreasing, an index outside [0, n))
 * is rejected with CT_ERR_ARG before any kernel reads it.  Synchronises `stream` once
 * per round.
 */
CT_API int ct_luby_mis(const int64_t* indptr, const int64_t* indices, int64_t n, uint64_t seed, int8_t* out_sel,
                       int32_t* iterations, void* stream);

/* Copy tree arrays to device buffers of n entries each (any may be NULL):
 * parents (node numbering), levels, si (cover radii), node_to_dataset, subtree_min. */
CT_API int ct_tree_arrays(const ct_tree* tree, int64_t* parents, int32_t* levels, float* si, int64_t* node_to_dataset,
                   int64_t* subtree_min, void* stream);

/* Diagnostic: the BF16 screening pass's raw FP32 dot products hi.hi + hi.lo + lo.hi for
 * the 128 x 256 block rows_a (128 device int32 dataset rows, -1 = zero row) x rows_b
 * (256 device int32 rows) into out (device f32 [128 x 256], row-major).  No counterpart
 * in the reference; exposed so the tensor-core path can be checked against FP64.
 * Synchronises `stream`. */
CT_API int ct_debug_screen_dots(ct_tree* tree, const int32_t* rows_a, const int32_t* rows_b, float* out,
                                void* stream);

/* Build the screened form's operands now instead of at the first screened query
 * (synchronises `stream`).  No counterpart in the reference. */
CT_API int ct_prepare_screened(ct_tree* tree, void* stream);

/* Device memory held by a tree handle, in bytes (host output). */
CT_API int ct_tree_device_bytes(const ct_tree* tree, int64_t* bytes);

/* Copy the tree's inputs (V [n x m] natural order, p [n], raw coords [n x d]; dataset
 * order; device f32; any may be NULL), e.g. to persist the tree.  No counterpart in
 * the reference, which has no tree persistence. */
CT_API int ct_tree_inputs(const ct_tree* tree, float* v, float* p, float* coords, void* stream);

/* Telemetry of the cover-tree build (host outputs; any may be NULL), the counterpart of
 * the reference's BatchInsertTelemetry (src/algo/batch/mod.rs): prefix-doubling groups
 * inserted, conflict-graph edges stored, points selected by the MIS, rows kept out of
 * the tree (tiny residual variance, scored by every query), roots, build milliseconds. */
CT_API int ct_tree_build_info(const ct_tree* tree, int64_t* groups, int64_t* conflict_edges, int64_t* selected,
                              int64_t* side_rows, int64_t* roots, double* build_ms);

/* n, m, d of a tree (host outputs; any may be NULL). */
CT_API int ct_tree_shape(const ct_tree* tree, int64_t* n, int32_t* m, int32_t* d);

/*
 * k nearest dataset rows of NEW points (no counterpart in the reference, whose
 * queries are dataset ids only).  Query row i is qv[i] [m] (natural column order,
 * as ct_vfactor_embed writes it), qp[i] and qcoords[i] [d] (unscaled); all device f32.
 * form CT_FORM_DENSE: each point is scaled, normalised and compared exactly like one
 * more dataset row would be (plain FP32, the dense form's arithmetic), k <= 128.
 * form CT_FORM_SCREENED: BF16 tcgen05 screening + FP64-grade rescoring (the screened
 * form's contract), k <= 64, d <= 8; the points pass through a per-tree query slab
 * (grown on demand, which synchronises the device), and calls on one tree take turns.
 * Either way a point's result does not depend on the other points of the call.
 */
CT_API int ct_knn_residual_points(ct_tree* tree, const float* qv, const float* qp, const float* qcoords, int64_t nq,
                                  int32_t k, int32_t form, int64_t* out_idx, float* out_dist, ct_stats* stats,
                                  void* stream);

/*
 * Batching form: many query sets against many resident trees in ONE persistent
 * kernel launch that drains a device work queue of (query set, query tile,
 * candidate chunk) items; with use_graph the launch (descriptor copy + kernel) is
 * replayed from a CUDA graph.  No counterpart in the reference, which runs one
 * tree's knn_query_residual per call (src/lib.rs:370-507).
 *   ct_batch_add_ids     a query set of dataset ids (same contract as ct_knn_residual,
 *                        CT_FORM_DENSE: bit-identical output)
 *   ct_batch_add_points  a query set of new points (same contract as ct_knn_residual_points)
 *   ct_batch_set_shape   fix the launch shape: qt (queries per CTA tile: 16/32/64),
 *                        ctas_per_sm (1/2), items_per_slot (candidate-split target); 0 = auto
 *   ct_batch_autotune    time the candidate shapes on the current batch (reps runs each,
 *                        synchronising `stream`) and keep the fastest
 *   ct_batch_run         launch every added query set; asynchronous on `stream`
 *   ct_batch_get_shape   shape, grid and work-item count of the last run
 *   ct_batch_reserve     size shared memory for at least (m, d, k), so that batches
 *                        of different mixes keep one launch shape and one graph
 * Added query sets keep pointers to the caller's device buffers, which must stay
 * valid until the run completes.  Results do not depend on the shape or on the
 * other query sets of the batch.  One batch object serves one stream at a time.
 */
typedef struct ct_batch ct_batch;
CT_API int ct_batch_create(ct_batch** out);
CT_API int ct_batch_clear(ct_batch* b);
CT_API int ct_batch_add_ids(ct_batch* b, ct_tree* tree, const int64_t* q_ids, int64_t nq, int32_t k,
                            int32_t predecessor, int64_t* out_idx, float* out_dist);
CT_API int ct_batch_add_points(ct_batch* b, ct_tree* tree, const float* qv, const float* qp, const float* qcoords,
                               int64_t nq, int32_t k, int64_t* out_idx, float* out_dist);
CT_API int ct_batch_set_shape(ct_batch* b, int32_t qt, int32_t ctas_per_sm, int32_t items_per_slot);
CT_API int ct_batch_autotune(ct_batch* b, int32_t reps, void* stream, int32_t* qt, int32_t* ctas_per_sm,
                             int32_t* items_per_slot);
CT_API int ct_batch_run(ct_batch* b, int32_t use_graph, ct_stats* stats, void* stream);
CT_API int ct_batch_get_shape(const ct_batch* b, int32_t* qt, int32_t* ctas_per_sm, int32_t* items_per_slot,
                              int32_t* grid, int64_t* items);
CT_API int ct_batch_reserve(ct_batch* b, int32_t m, int32_t d, int32_t k);
CT_API int ct_batch_free(ct_batch* b);

/*
 * Residual-backend factor, built on the GPU in FP64.  Replaces the dense algebra of
 * build_residual_backend (covertreex/metrics/residual/host_backend.py:202-219):
 *   ct_vfactor_create  <- k_mm = K(Z, Z) + 1e-6 variance I; l_mm = cholesky(k_mm)
 *                         (host_backend.py:207-212); also keeps l_mm^-1 on the device
 *   ct_vfactor_embed   <- v = solve(l_mm, K(X, Z)^T)^T, p = max(variance - |v|^2, 1e-9),
 *                         cast to f32 (host_backend.py:214-219 and 236-239); the same
 *                         call embeds new query points for serving
 *   ct_vfactor_chol    <- l_mm itself (m x m FP64, lower, zero upper triangle)
 * z [m x d] and x [n x d] are device FP64 (the reference's float64 points and
 * points[inducing_idx]); v_out [n x m] and p_out [n] device f32.  lengthscale is the
 * scalar the reference's builder takes; kernel_type CT_KERNEL_*.  ct_vfactor_create
 * synchronises `stream` and returns CT_ERR_ARG when k_mm is not positive definite
 * (numpy's LinAlgError).  The factor is read-only after creation: embeds may run
 * concurrently on different streams (each takes stream-ordered scratch of its own).
 */
typedef struct ct_vfactor ct_vfactor;
CT_API int ct_vfactor_create(const double* z, int32_t m, int32_t d, int32_t kernel_type, double variance,
                             double lengthscale, void* stream, ct_vfactor** out);
CT_API int ct_vfactor_embed(ct_vfactor* f, const double* x, int64_t n, float* v_out, float* p_out, void* stream);
CT_API int ct_vfactor_chol(const ct_vfactor* f, double* l_out, void* stream);
CT_API int ct_vfactor_free(ct_vfactor* f);

/* Release a tree and its device memory. */
/*
 * A new handle over the base handle's rows followed by n_new new rows (v [n_new x m],
 * p [n_new], coords [n_new x d]; device f32, the base's m, d and metric parameters):
 * the counterpart of CoverTree.insert / CoverTreeWrapper.insert_residual
 * (covertreex/api/pcct.py:171-197, src/lib.rs:254-321), whose trees are immutable, so
 * the base stays valid.  The base's rows and derived data are copied device to device;
 * when the base has a cover tree, its nodes keep their parents and levels and the new
 * rows are inserted as prefix-doubling groups.  New rows get dataset ids base_n ..
 * base_n + n_new - 1.  Every form answers exactly as a fresh build over all rows would.
 */
CT_API int ct_tree_extend(const ct_tree* base, const float* v, const float* p, const float* coords, int64_t n_new,
                          void* stream, ct_tree** out);

/*
 * A new handle over the base's rows `rows` (device int64, ascending, in [0, base n)),
 * renumbered 0 .. n_keep - 1: the counterpart of CoverTree.delete (covertreex/api/pcct.py:
 * 199-220, algo/batch_delete.py), immutable like it.  The rows are gathered on the device
 * and the handle (and its cover tree, when the base has one) is built from them.
 */
CT_API int ct_tree_subset(const ct_tree* base, const int64_t* rows, int64_t n_keep, void* stream, ct_tree** out);

CT_API int ct_free(ct_tree* tree);

#ifdef __cplusplus
}
#endif

#endif /* COVERTREE_CUDA_H */
