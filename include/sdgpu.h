/*
 * sdgpu.h -- C ABI of libsdgpu.so, the GB300 (sm_103a) implementation of the
 * blocked exact k-nearest-neighbour path of the R package sparseDist
 * (gambalab/sparseDist): the column-pair distance slabs, the per-column
 * top-k, the running per-row top-k, the SNN overlap weights and the SNN graph.
 *
 * Conventions
 *  - Every entry point is extern "C", never throws, and returns an int status
 *    (SDG_OK == 0).  sdg_last_error() returns the message of the calling
 *    thread's last failure; messages reproduce the reference's error text.
 *  - Sparse inputs are borrowed host pointers to the slots of an R dgCMatrix
 *    (sdg_csc): p has ncol+1 entries, i / x have p[ncol] entries, row indices
 *    ascending within each column.  Observations are the COLUMNS.
 *  - Outputs are caller-allocated, column-major (R's layout): an n x k matrix
 *    stores element (row r, column t) at [t * n + r].  Indices are 1-based.
 *    Empty slots hold NA: INT32_MIN for indices (R's NA_integer_) and the bit
 *    pattern 0x7FF00000000007A2 for values (R's NA_real_).
 *  - `ncores` and `block_size` are validated exactly as the reference does and
 *    never change a result; the GPU does not use them.
 *  - Methods: see sdg_method.  "jaccard" is the caller's alias of SDG_BINARY.
 *
 * Each function's comment names the reference interface it replaces.
 */
#ifndef SDGPU_H
#define SDGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define SDG_EXTERN extern "C"
#else
#define SDG_EXTERN extern
#endif
#define SDG_API SDG_EXTERN __attribute__((visibility("default")))

typedef enum {
  SDG_BINARY = 0,     /* Jaccard on the sparsity pattern */
  SDG_COSINE = 1,
  SDG_EUCLIDEAN = 2,
  SDG_MANHATTAN = 3,
  SDG_PEARSON = 4,
  SDG_JS = 5,         /* Jensen-Shannon distance sqrt(JSD) */
  SDG_COVARIANCE = 6  /* sample covariance (N - 1); a coefficient, kNN keeps the largest */
} sdg_method;

typedef enum {
  SDG_OK = 0,
  SDG_E_ARG = -1,          /* invalid argument (reference's validation text) */
  SDG_E_NONFINITE = -2,    /* cosine / js input not finite (or js negative) */
  SDG_E_ROWS = -3,         /* row dimensions differ */
  SDG_E_NOCAND = -4,       /* "No candidate neighbours available." */
  SDG_E_NOMEM = -5,        /* device or host allocation failed */
  SDG_E_INDEX = -6,        /* SNN index out of range */
  SDG_E_CUDA = -7,         /* CUDA runtime error */
  SDG_E_UNSUPPORTED = -8,  /* outside the library's limits (message says which) */
  SDG_E_CANCELLED = -9     /* sdg_ctx_cancel() was called */
} sdg_status;

/* Bits of *flags: the reference's k-clamp warnings ("k (K) exceeds the N
 * available neighbours; returning N."), reported instead of printed. */
enum { SDG_WARN_CLAMP_FWD = 1, SDG_WARN_CLAMP_REV = 2 };

typedef struct {
  int32_t nrow, ncol;
  const int32_t* p;   /* ncol + 1 */
  const int32_t* i;   /* p[ncol] */
  const double* x;    /* p[ncol] */
} sdg_csc;

typedef struct sdg_ctx sdg_ctx;

/* ---- context ------------------------------------------------------------ */

/* Library version as 10000*major + 100*minor + patch. */
SDG_API int sdg_version(void);

/* Copies the calling thread's last error message into buf (NUL-terminated,
 * truncated to len) and returns its full length. */
SDG_API int sdg_last_error(char* buf, size_t len);

/* One context per (thread, device): owns a CUDA stream and the device memory
 * of in-flight work.  device < 0 selects the current device. */
SDG_API int sdg_ctx_create(int device, sdg_ctx** out);
SDG_API int sdg_ctx_destroy(sdg_ctx* ctx);

/* Asks running work on ctx to stop at its next query tile; the call then
 * returns SDG_E_CANCELLED.  Safe to call from another thread (this is what
 * R_CheckUserInterrupt maps onto).  Cleared by sdg_ctx_reset_cancel(). */
SDG_API int sdg_ctx_cancel(sdg_ctx* ctx);
SDG_API int sdg_ctx_reset_cancel(sdg_ctx* ctx);

/* ---- the reference's .Call kernels, one for one --------------------------- */

/* Distance / similarity slab between the columns of m and m2:
 * D is ncol(m) x ncol(m2), D(i, j) = method(column i of m, column j of m2).
 * Replaces fastJacc2 / fastCosine2 / fastEuclidean2 / fastManhattan2 /
 * fastCorr2 / fastJS2 / fastCov2 (src/sparseDist.cpp:559, :967, :833, :734,
 * :403, :1074, :481; .Call stubs R/RcppExports.R:24-74).  dist selects
 * 1 - similarity for binary / cosine / pearson and is ignored by the other
 * methods' kernels, as the reference ignores it. */
SDG_API int sdg_dist_cross(sdg_ctx* ctx, int method, int dist, const sdg_csc* m,
                           const sdg_csc* m2, double* D);

/* Single-matrix form: D is the reference's dense ncol(m) x ncol(m) accumulator
 * (column-major) before its dense-or-sparse return, i.e. the pair (i, j),
 * i < j, at D(j, i) and, with full, also at D(i, j); the rest 0.  The
 * diagonal: 0 / 1 (dist / similarity) for binary, cosine and pearson; the
 * self pair for euclidean, manhattan and covariance with diag, else 0; 0 for
 * js.  Replaces fastJacc / fastCosine / fastEuclidean / fastManhattan /
 * fastCorr / fastJS / fastCov (src/sparseDist.cpp:620, :918, :786, :688,
 * :339, :1021, :450; .Call stubs R/RcppExports.R:20-70), called by
 * sparseDist(X) at R/sparseDist.R:162-171. */
SDG_API int sdg_dist(sdg_ctx* ctx, int method, int dist, const sdg_csc* m, int full, int diag,
                     double* D);

/* Per-column top-k of a dense block D (nrow x ncol, column-major).
 * idx / dist are ncol x k.  self_row[b] is 0 or the 1-based row excluded for
 * column b.  Replaces topKBlock (src/topK.cpp:66-149, R/RcppExports.R:77-79). */
SDG_API int sdg_topk_block(sdg_ctx* ctx, const double* D, int64_t nrow, int64_t ncol,
                           int k, int decreasing, const int32_t* self_row,
                           int32_t* idx, double* dist);

/* Folds block D (query columns col_offset .. col_offset+ncol-1, 0-based) into
 * the running per-row top-k best_idx / best_val (nrow x k, updated in place).
 * self_col[i] is 0 or the 1-based global query index excluded for row i.
 * Replaces topKRowsAccum (src/topKRows.cpp:103-248, R/RcppExports.R:81-83). */
SDG_API int sdg_topk_rows_accum(sdg_ctx* ctx, const double* D, int64_t nrow, int64_t ncol,
                                int k, int decreasing, int32_t* best_idx, double* best_val,
                                int32_t col_offset, const int32_t* self_col);

/* Jaccard overlap of kNN neighbour sets: w (n x k) aligned with idx (n x k,
 * 1-based, NA padded).  Replaces snnJaccard (src/snn.cpp:197-250,
 * R/RcppExports.R:13-15). */
SDG_API int sdg_snn_jaccard(sdg_ctx* ctx, const int32_t* idx, int32_t n, int32_t k,
                            int include_self, double* w);

/* sdg_snn_jaccard for callers that cannot allocate device memory on their
 * call path (a host framework that owns the GPU's memory through its own
 * allocator, or a thread that must not call cudaMalloc / cudaFree because
 * they synchronise the device).  No counterpart in the reference.
 *
 * idx (n x k int32, column-major, 1-based, NA = INT32_MIN) and w (n x k
 * double) are DEVICE pointers owned by the caller; stream is a cudaStream_t
 * (NULL = the legacy default stream).  The neighbour sets live in a fixed
 * 32 MiB array compiled into the library (held by every GPU that loads it,
 * until exit): a call is rejected with SDG_E_UNSUPPORTED unless
 * n * (k + 2) + 1 <= 8,388,608.  Nothing is allocated.  Every call looks up
 * the array's device address in the current context (so a device reset or
 * another context never leaves a stale address); the first call on a device
 * loads the library's device code (make it before any stream capture).  The
 * call synchronises `stream` once, to read the index check.
 * All calls share the array: calls whose work overlaps on the GPU race. */
SDG_API int sdg_snn_jaccard_noalloc(const int32_t* idx, int32_t n, int32_t k, int include_self,
                                    double* w, void* stream);

/* ---- the fused paths (the R block loops move onto the GPU) ----------------- */

/* sparseKNN(X, Y, k, method, dist, include_self, drop_degenerate, block_size):
 * Y == NULL is the self-search.  idx / dist must hold ncol(X) * k values; the
 * result is ncol(X) x k_eff with k_eff = *k_eff <= k after the reference's
 * clamp (SDG_WARN_CLAMP_FWD set in *flags when it applied).  Replaces the
 * block loop of R/sparseKNN.R:110-313 (slab .Call + topKBlock .Call per
 * block). */
SDG_API int sdg_knn(sdg_ctx* ctx, const sdg_csc* X, const sdg_csc* Y, int method, int dist,
                    int k, int include_self, int drop_degenerate, int block_size, int ncores,
                    int32_t* idx, double* dist_out, int* k_eff, int* flags);

/* sparseKNNCross(X, Y, k, ...): forward (ncol(X) x k_fwd, indices into Y) and
 * reverse (ncol(Y) x k_rev, indices into X), each clamped independently.
 * fwd_* hold ncol(X) * k and rev_* hold ncol(Y) * k values.  Replaces
 * R/sparseKNNCross.R:44-199 (slab + topKBlock + topKRowsAccum per block). */
SDG_API int sdg_knn_cross(sdg_ctx* ctx, const sdg_csc* X, const sdg_csc* Y, int method,
                          int dist, int k, int drop_degenerate, int block_size, int ncores,
                          int32_t* fwd_idx, double* fwd_dist, int32_t* rev_idx,
                          double* rev_dist, int* k_fwd, int* k_rev, int* flags);

/* Many independent sparseKNNCross problems in one call: problem p is
 * sparseKNNCross(X[p], Y[p], k[p], method[p], dist[p], drop_degenerate), with
 * its results written to fwd_idx[p] / fwd_dist[p] (ncol(X[p]) * k[p] values)
 * and rev_idx[p] / rev_dist[p] (ncol(Y[p]) * k[p]), clamped k in k_fwd[p] /
 * k_rev[p], warnings in flags[p] and the problem's own status in status[p] (a
 * failing problem leaves the others untouched; the call returns the first
 * failure's code and message, or SDG_OK).  An autotuner picks each search
 * direction's engine (exact FP64, FP32 sparse screen or tensor-core screen)
 * from the problem's shape, with corrections learned from measured times
 * and kept per shape class for the process; every exact-path search of the
 * call (up to a device-memory budget per wave of problems) runs in ONE
 * persistent launch over a work queue of (problem, direction, query column,
 * reference range) items sized by their merge-walk cost.  engines (optional,
 * 2 * nprob) receives the engine of each problem's forward and reverse
 * search (1 exact, 2 FP32 screen, 3 tensor-core screen) and engine_seconds
 * (optional, 3) the device time spent in each engine over the call.  Replaces a loop of R/sparseKNNCross.R:44-199 over the problems;
 * each problem's result equals sdg_knn_cross's. */
SDG_API int sdg_knn_cross_batch(sdg_ctx* ctx, int nprob, const sdg_csc* X, const sdg_csc* Y,
                                const int* method, const int* dist, const int* k, int drop_degenerate,
                                int32_t* const* fwd_idx, double* const* fwd_dist,
                                int32_t* const* rev_idx, double* const* rev_dist, int* k_fwd,
                                int* k_rev, int* flags, int* status, int* engines,
                                double* engine_seconds);

/* sparseSNN(idx, include_self, prune, symmetrise, edges = "knn") as the slots
 * of the n x n dgCMatrix.  Call once with p == NULL to learn *nnz, then with
 * p (n + 1), i and x (nnz each).  The size query keeps its graph on the
 * device and a fetch with the same arguments and idx contents copies it
 * instead of building it again (any other call on ctx drops it).  Replaces
 * snnJaccard plus the Matrix assembly of R/sparseSNN.R:221-250. */
SDG_API int sdg_snn_graph(sdg_ctx* ctx, const int32_t* idx, int32_t n, int32_t k,
                          int include_self, double prune, int symmetrise, int64_t* nnz,
                          int32_t* p, int32_t* i, double* x);

/* sparseSNN(idx, include_self, prune, edges = "shared") as the slots of the
 * symmetric n x n dgCMatrix: every pair (i, j), i != j, whose neighbour sets
 * intersect, weighted |N(i) n N(j)| / |N(i) u N(j)|, kept when the weight
 * exceeds prune (no diagonal).  Same two-call protocol as sdg_snn_graph.
 * Replaces snnJaccardShared (src/snn.cpp:252-447, R/RcppExports.R:16-18) plus the
 * Matrix assembly of R/sparseSNN.R:202-219. */
SDG_API int sdg_snn_graph_shared(sdg_ctx* ctx, const int32_t* idx, int32_t n, int32_t k,
                                 int include_self, double prune, int64_t* nnz, int32_t* p,
                                 int32_t* i, double* x);

/* ---- device-resident inputs (serving / batching) ---------------------------- */

/* A CSC matrix uploaded once and kept in device memory, with its per-column
 * data (norms, unit values, masks) computed on first use. */
typedef struct sdg_matrix sdg_matrix;
SDG_API int sdg_matrix_upload(sdg_ctx* ctx, const sdg_csc* M, sdg_matrix** out);
SDG_API int sdg_matrix_free(sdg_matrix* M);
/* As sdg_matrix_upload from dgCMatrix slots that already live in device
 * memory (int32 p / i, double x; copied device to device). */
SDG_API int sdg_matrix_upload_device(sdg_ctx* ctx, int32_t nrow, int32_t ncol, const int32_t* p,
                                     const int32_t* i, const double* x, sdg_matrix** out);

/* sdg_knn over resident matrices; results are written to host buffers. */
SDG_API int sdg_knn_resident(sdg_ctx* ctx, const sdg_matrix* X, const sdg_matrix* Y,
                             int method, int dist, int k, int include_self,
                             int drop_degenerate, int32_t* idx, double* dist_out,
                             int* k_eff, int* flags);

/* ---- dense embedding columns (BF16 tensor-core screen, exact FP64 re-rank) --
 * X is d x n FP32, column-major (host or device pointer), each column one
 * embedding.  sdg_dense_knn_block returns rows q0 .. q0+nq-1 of the
 * self-search sparseKNN(X, k, method) (include_self = FALSE,
 * drop_degenerate = TRUE) for cosine (dist) or euclidean.  mode 0: BF16
 * tensor-core screen with a rigorous bound, a second FP32 cut with a rigorous
 * bound, and exact FP64 values of the survivors (the reference's idx and
 * distances), the screen fused in one tcgen05 kernel (no slab in HBM, one
 * CTA per 128-query group) for k <= 64 and d <= 256, else as mode 2; mode 3: the fused screen on CTA pairs (clusters of two CTAs sharing
 * cta_group::2 UMMAs of 256 queries; the same results) when the block has
 * more than 128 queries; mode 2: the same screen through a cuBLAS BF16 GEMM slab; mode 1:
 * the plain FP32 path (FP32 GEMM, top-k on FP32 values, no re-rank).  k above
 * 1,024: every mode values every pair exactly.  No counterpart in the reference, whose
 * dense inputs are coerced to dgCMatrix (R/sparseKNN.R:194-200); the FP64
 * values are those sparseKNN computes on the same data. */
typedef struct sdg_dense sdg_dense;
SDG_API int sdg_dense_upload(sdg_ctx* ctx, const float* X, int32_t d, int64_t n, sdg_dense** out);
SDG_API int sdg_dense_free(sdg_dense* D);
SDG_API int sdg_dense_knn_block(sdg_ctx* ctx, const sdg_dense* D, int64_t q0, int64_t nq,
                                int method, int k, int mode, int32_t* idx, double* dist_out,
                                int device_out, int* k_eff, int* flags);

/* sparseKNN(Q, D, k, method) for new query embeddings: Q is d x nq FP32
 * (column-major, host or device pointer), searched against the resident D
 * (drop_degenerate = TRUE; no self-exclusion, as in the reference's
 * two-matrix form, R/sparseKNN.R:183-301 with Y given).  Same modes, outputs
 * and clamp as sdg_dense_knn_block; idx are 1-based columns of D.  The
 * queries' FP64 / unit / FP32 / BF16 forms are built on the context's stream
 * from its memory pool and released when the call returns.  A non-finite
 * query value fails the call with SDG_E_NONFINITE (the outputs' contents are
 * then unspecified). */
SDG_API int sdg_dense_knn_query(sdg_ctx* ctx, const sdg_dense* D, const float* Q, int32_t d, int64_t nq,
                                int method, int k, int mode, int32_t* idx, double* dist_out,
                                int device_out, int* k_eff, int* flags);

/* ---- serving: continuous batching against a resident reference -------------
 * A server keeps `ref` resident (with the per-column data of `methods`
 * prepared up front), admits submitted query matrices while one of max_slots
 * slots is free and their device-memory estimate (query, screen slab share,
 * candidate table, results) fits mem_budget bytes, packs admitted requests
 * that share (method, dist, drop_degenerate) into one engine pass, and runs
 * passes on `workers` threads, each with its own stream, so work from
 * requests arriving while others run overlaps on the device.  A request's
 * result is sparseKNN(Q, ref, ...) exactly, alone or in any mix.  No
 * counterpart in the reference (its serving path is this library's own). */
typedef struct sdg_server sdg_server;
SDG_API int sdg_server_create(sdg_ctx* ctx, const sdg_matrix* ref, int workers, int max_slots,
                              int64_t mem_budget, const int* methods, int nmethods,
                              sdg_server** out);
SDG_API int sdg_server_submit(sdg_server* server, const sdg_csc* Q, int method, int dist, int k,
                              int drop_degenerate, int64_t* request_id);
/* A server over a resident dense reference (sdg_dense_upload): requests are
 * d x nq FP32 query columns (column-major, host memory, copied at submit),
 * method cosine or euclidean, any k; admitted requests of one method are
 * packed column-wise into one fused BF16 tensor-core search with the exact
 * FP64 re-rank (sdg_dense_knn_query at the batch's largest k), so a
 * request's result is sparseKNN(Q, ref, k, method) exactly, alone or in any
 * mix.  sdg_server_wait / result / cancel / stats / destroy as above.  No
 * counterpart in the reference. */
SDG_API int sdg_server_create_dense(sdg_ctx* ctx, const sdg_dense* ref, int workers, int max_slots,
                                    int64_t mem_budget, sdg_server** out);
SDG_API int sdg_server_submit_dense(sdg_server* server, const float* Q, int32_t d, int32_t nq,
                                    int method, int k, int64_t* request_id);
/* 0 when the request finished, 1 on timeout (timeout_ms < 0 waits forever). */
SDG_API int sdg_server_wait(sdg_server* server, int64_t request_id, int timeout_ms);
/* Copies a finished request's ncol(Q) x k_eff result and releases it. */
SDG_API int sdg_server_result(sdg_server* server, int64_t request_id, int32_t* idx,
                              double* dist_out, int* k_eff, int* flags);
/* Cancels a request that has not started (0); 1 if it is already running. */
SDG_API int sdg_server_cancel(sdg_server* server, int64_t request_id);
/* out[0..8]: completed requests, completed columns, p50 / p99 / mean latency
 * (s, submit to completion), columns/s, batches, bytes admitted, requests
 * waiting for admission. */
SDG_API int sdg_server_stats(sdg_server* server, double* out, int n);
SDG_API int sdg_server_destroy(sdg_server* server);

/* Rows q0 .. q0+nq-1 of sparseKNN(X, Y, ...) over resident matrices: one
 * block of the reference's block loop (R/sparseKNN.R:248-294) with the
 * whole search's semantics -- self-exclusion by global column index and the
 * k clamp over the whole reference -- so that ranks or streams can each take
 * a share of the query columns.  idx / dist_out hold nq * k values (column-
 * major nq x k_eff); device_out selects device (1) or host (0) buffers. */
SDG_API int sdg_knn_block(sdg_ctx* ctx, const sdg_matrix* X, const sdg_matrix* Y, int64_t q0,
                          int64_t nq, int method, int dist, int k, int include_self,
                          int drop_degenerate, int32_t* idx, double* dist_out, int device_out,
                          int* k_eff, int* flags);

/* As sdg_knn_resident, with idx / dist_out in DEVICE memory (caller
 * allocated, ncol(X) * k each); nothing is copied back and the call returns
 * once the work is queued on the context's stream (stream order). */
SDG_API int sdg_knn_resident_device(sdg_ctx* ctx, const sdg_matrix* X, const sdg_matrix* Y,
                                    int method, int dist, int k, int include_self,
                                    int drop_degenerate, int32_t* idx, double* dist_out,
                                    int* k_eff, int* flags);

/* Makes ctx launch its work on the caller's CUDA stream (a cudaStream_t
 * passed as void*; NULL restores the context's own stream), so that a host
 * framework can order and time the library's kernels on its stream. */
SDG_API int sdg_ctx_set_stream(sdg_ctx* ctx, void* stream);

/* Statistics of the last sdg_knn* call on ctx (for profiling and tests):
 * out[0] = pairs screened, out[1] = pairs re-ranked exactly, out[2] = queries
 * whose candidate buffer overflowed (finished by the exact path), out[3] =
 * kernels launched, out[4] = screening kernel time in microseconds (device
 * events), out[5] = total device time in microseconds, out[6] = dense flops
 * of the tensor-core screen's GEMMs. */
SDG_API int sdg_last_stats(sdg_ctx* ctx, int64_t* out, int n);

/* Device time of the kernel that bounds the kNN path (the pair-value slab of
 * the exact engine, the screen of the screened engine), accumulated with
 * CUDA events on the context's stream over every sdg_knn* call since the
 * previous sdg_kernel_time call: *ms is the total, *launches the number of
 * launches.  Synchronises with the last recorded launch and resets. */
SDG_API int sdg_kernel_time(sdg_ctx* ctx, double* ms, int64_t* launches);

/* Selects the candidate-generation engine for subsequent calls on ctx:
 * 0 = automatic, 1 = exact FP64 slab for every pair, 2 = screened (FP32 /
 * integer sparse screen, exact FP64 re-rank), 3 = tensor-core screen
 * (binary / cosine / euclidean: FP16 GEMM over dense copies of the screen
 * values with a rigorous bound, exact FP64 re-rank; other methods, or values
 * beyond FP16's range, use 2).  Results are identical; only speed differs.
 * Used by tests to cross-check the engines. */
SDG_API int sdg_ctx_set_engine(sdg_ctx* ctx, int engine);

/* Failure-detection test hook: the next `launches` launches of the fused
 * tensor-core screens (the dense BF16 screen and the sparse FP16 screen) make
 * their MMA issuer wait on a pipeline phase that nothing completes.  Every
 * wait of those kernels is bounded (1 s); the one that runs out raises the
 * CTA's abort flag, the other roles leave their loops, issued copies and MMAs
 * are drained, TMEM is freed and the kernel returns, so the call fails with
 * SDG_E_CUDA ("... timed out") and the context stays usable.  0 clears it.
 * Process-wide; used by the tests only. */
SDG_API int sdg_debug_stall_tc(int launches);

#endif
