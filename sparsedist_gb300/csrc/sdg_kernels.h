// sdg_kernels.h -- host-side launchers of the CUDA kernels (implemented in the
// .cu files of this directory), called by the orchestration in sdg_api.cpp.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sdg_common.cuh"

struct sdg_ctx;
struct sdg_dense;
// Bracket one launch of the bounding kernel (sdg_kernel_time).
void sdg_time_begin(sdg_ctx* c);
void sdg_time_end(sdg_ctx* c);

namespace sdg {

// Sets the calling thread's error message (sdg_last_error); never allocates.
void set_error(const char* msg);

// Context accessors for the translation units outside sdg_api.cpp.
cudaStream_t ctx_stream(sdg_ctx* c);
int ctx_device(sdg_ctx* c);
void ctx_add_overflow(sdg_ctx* c, int64_t n);
// slot t of the per-call statistics (sdg_last_stats); reset clears all eight
void ctx_stats_add(sdg_ctx* c, int slot, int64_t n);
void ctx_stats_reset(sdg_ctx* c);

// ---- sdg_exact.cu: per-column preparation and exact FP64 pair values --------
void launch_col_empty(const DevCsc& M, uint8_t* empty, cudaStream_t s);
void launch_unit_csc(const DevCsc& M, double* uval, double* scale, int* err, cudaStream_t s);
// unit_csc of n dense columns of d values (column-major, zeros included and
// skipped by the recurrence): the same values as launch_unit_csc on the
// all-entries CSC view, bit for bit
void launch_unit_dense(int32_t d, int64_t n, const double* x, double* uval, double* scale, int* err,
                       cudaStream_t s);
void launch_moments(const DevCsc& M, double* sum, double* sumsq, cudaStream_t s);
void launch_check_js(const double* x, int64_t nnz, int* err, cudaStream_t s);
// xl[a] = xlogx(x[a]) for every stored value (js pair values reuse them)
void launch_xlogx_values(const double* x, int64_t nnz, double* xl, cudaStream_t s);

// Failure-detection test hook of the tcgen05 screens (sdg_sparse_tc.cu):
// tc_set_stall(n) makes the next n launches of k_dense_tc / k_sparse_tc wait
// on a phase that nothing completes, so that the bounded wait runs out and
// the launch returns its timeout status; tc_take_stall() consumes one.
void tc_set_stall(int n);
bool tc_take_stall();

// Exact values of every pair (ref column i, query column q0 + b) for
// b < nb into D (nb columns of length ref.ncol).  Masked reference columns
// (ref_mask[i] != 0) get NaN; with restore_self, the self position i == q0 + b
// gets self_value (R/sparseKNN.R:270-279).
void launch_exact_slab(int method, int dist, const DevCsc& ref, const ColAux& ra,
                       const DevCsc& qry, const ColAux& qa, int64_t q0, int64_t nb,
                       const uint8_t* ref_mask, int restore_self, double self_value,
                       double* D, cudaStream_t s);

// Single-matrix sparseDist: columns c0 .. c0 + nb - 1 of the n x n result
// into D (nb columns of length n); the upper triangle is computed only with
// `upper`, else written 0.
void launch_self_slab(int method, int dist, const DevCsc& m, const ColAux& a, int64_t c0,
                      int64_t nb, int upper, int diag, double* D, cudaStream_t s);
// Copies the strict lower triangle of the device n x n matrix D onto its
// upper triangle.
void launch_mirror_lower(double* D, int64_t n, cudaStream_t s);
// The match-only methods (binary, cosine, pearson, covariance; nrow <= 2^18)
// of the single-matrix form on the query-centric re-rank kernel: the strict
// upper triangle D(c, q) = value(column c, column q), c < q, and the
// diagonal; the lower triangle is left for launch_mirror_upper.
bool self_tri_supported(int method, int32_t nrow);
void launch_self_tri(int method, int dist, const DevCsc& m, const ColAux& a, int diag, double* D,
                     cudaStream_t s);
// Copies the strict upper triangle of D onto the lower one; with clear, the
// upper triangle is zeroed after it is read.
void launch_mirror_upper(double* D, int64_t n, int clear, cudaStream_t s);

// Exact values of listed pairs: out[t] = value(ref col ref_idx[t], query col
// qry_idx[t]).
void launch_exact_pairs(int method, int dist, const DevCsc& ref, const ColAux& ra,
                        const DevCsc& qry, const ColAux& qa, const int32_t* ref_idx,
                        const int32_t* qry_idx, int64_t npairs, double* out, cudaStream_t s);

// Candidate pairs (screened engine): slots with ref_idx < 0 are skipped; with
// restore_self the self pair takes self_value.
void launch_exact_pairs_sparse(int method, int dist, const DevCsc& ref, const ColAux& ra,
                               const DevCsc& qry, const ColAux& qa, const int32_t* ref_idx,
                               const int32_t* qry_idx, int64_t npairs, int restore_self,
                               double self_value, double* out, cudaStream_t s);

// Warp-cooperative exact values of a candidate table (cand[ql * cap + t] for
// t < count[ql]) for the match-only methods (binary, cosine, pearson).
bool rerank_warp_supported(int method);
void launch_rerank_warp(int method, int dist, const DevCsc& ref, const ColAux& ra,
                        const DevCsc& qry, const ColAux& qa, const int32_t* cand,
                        const int32_t* count, int cap, int64_t nq_local, int64_t q_begin,
                        int restore_self, double self_value, double* out, cudaStream_t s);

// ---- sdg_select.cu: exact top-k selection --------------------------------------

// One "segment" per output row: candidates are vals[seg*seg_stride +
// t*elem_stride] for t < len with global index idx_base + t.  Skipped: non-
// finite values, elem_mask[t] != 0, and the global index skip_base + seg when
// skip_base >= 0 or skip_arr[seg] (0-based global, < 0 = none) when given.
// Optional seeds (1-based idx / values, column-major with leading dim seed_ld,
// read up to the first NA) join the candidates.  The k best under
// (value asc|desc, index asc) are written best-first, NA padded, to
// out_idx / out_val at [t * out_ld + out_row0 + seg]; rows with
// seg_blank[out_row0 + seg] != 0 are written all-NA.
struct SelectArgs {
  const double* vals = nullptr;
  int64_t seg_stride = 0, elem_stride = 1, len = 0, nseg = 0;
  int64_t idx_base = 0;
  const uint8_t* elem_mask = nullptr;
  int64_t skip_base = -1;
  const int64_t* skip_arr = nullptr;
  const int32_t* seed_idx = nullptr;
  const double* seed_val = nullptr;
  int64_t seed_ld = 0;
  const uint8_t* seg_blank = nullptr;
  int32_t* out_idx = nullptr;
  double* out_val = nullptr;
  int64_t out_ld = 0, out_row0 = 0;
  int k = 1;
  int decreasing = 0;
  // Candidate lists: when cand is set, element t of segment seg has global
  // index cand[seg * cand_ld + t] and the segment's length is cand_count[seg]
  // (len is then ignored).
  const int32_t* cand = nullptr;
  const int32_t* cand_count = nullptr;
  int64_t cand_ld = 0;
};
constexpr int kMaxK = 1024;   // largest k whose selection lists sit in shared memory (and the screens' limit)

// ---- sdg_exact.cu: batched exact kNN of many independent problems -------------
// Problem p of a batch: the forward direction searches the columns of X among
// the columns of Y, the reverse one the columns of Y among those of X.
struct BatchProb {
  DevCsc X, Y;
  ColAux xa, ya;
  int method, dist, decreasing;
  int kf, kr;                              // clamped k of each direction
  const uint8_t* xmask;                    // dropped (degenerate) columns, or null
  const uint8_t* ymask;
  int32_t* fidx; double* fval;             // device results: ncol(X) x kf, column-major
  int32_t* ridx; double* rval;             // ncol(Y) x kr
};
// one unit of the persistent launch: query column q of direction dir against
// the reference columns [r0, r1); its top k goes to partial slot `part`
struct BatchItem {
  int32_t prob, dir, q, r0, r1, pad;
  int64_t part;
};
// one output row: its items' lists are the partial slots part0 .. + nparts
struct BatchRow {
  int32_t prob, dir, q, nparts;
  int64_t part0;
};
constexpr int kBatchMaxK = 256;          // largest k of the batched exact path
size_t batch_smem(int kmax);
// words of a query-column row lookup per warp for a problem of this method and
// row count (0: the problem's pairs use the merge walk)
int batch_lookup_words(int method, int32_t nrow);
void launch_batch_exact(const BatchProb* probs, const BatchItem* items, int64_t nitems, unsigned long long* counter,
                        int kmax, int lwords, uint64_t* pkey, int32_t* pidx, double* pval, int sms, cudaStream_t s);
void launch_batch_merge(const BatchProb* probs, const BatchRow* rows, int64_t nrows, int kmax, const uint64_t* pkey,
                        const int32_t* pidx, const double* pval, cudaStream_t s);
void launch_select(const SelectArgs& a, cudaStream_t s);

// ---- sdg_snn.cu: SNN weights and graph ------------------------------------------
void launch_snn_check(const int32_t* idx, int32_t n, int32_t k, int* err, cudaStream_t s);
// sets: n x (k+1) scratch, sizes: n
void launch_snn_sets(const int32_t* idx, int32_t n, int32_t k, int include_self,
                     int32_t* sets, int32_t* sizes, cudaStream_t s);
void launch_snn_weights(const int32_t* idx, int32_t n, int32_t k, const int32_t* sets,
                        const int32_t* sizes, double* w, cudaStream_t s);
// Graph assembly: returns nnz through *nnz_host (synchronises the stream).
// Buffers are allocated from the stream-ordered pool and returned; the caller
// frees them with cudaFreeAsync.
// sparseSNN(edges = "shared"): the symmetric graph of every pair sharing a
// neighbour with weight > prune, from the device neighbour sets (sets: n x
// (k + 1), sizes: n); outputs as snn_graph_build.
int snn_shared_build(const int32_t* d_sets, const int32_t* d_sizes, int32_t n, int32_t k, double prune,
                     int64_t* nnz_host, int32_t** d_p, int32_t** d_i, double** d_x, cudaStream_t s);
int snn_graph_build(const int32_t* d_idx, const double* d_w, int32_t n, int32_t k,
                    double prune, int symmetrise, int64_t* nnz_host, int32_t** d_p,
                    int32_t** d_i, double** d_x, cudaStream_t s);

// ---- sdg_dense.cu: resident dense embeddings (host-side view) ---------------------
// sparseKNN(Q, D, k, method) of nq new query columns Q (d x nq FP32, host or
// device) against the resident D; the body of sdg_dense_knn_query.
int dense_query(sdg_ctx* ctx, const sdg_dense* D, const float* Q, int32_t d, int64_t nq, int method, int k,
                int mode, int32_t* idx, double* dist_out, int device_out, int* k_eff, int* flags);
int32_t dense_rows(const sdg_dense* D);
int64_t dense_cols(const sdg_dense* D);
// device memory one dense_query of nq columns at k takes from the pool
int64_t dense_query_bytes(const sdg_dense* D, int64_t nq, int k);

}  // namespace sdg
