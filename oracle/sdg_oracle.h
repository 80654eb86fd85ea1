/*
 * sdg_oracle.h -- CPU oracle for the blocked exact-kNN path of sparseDist.
 *
 * TEST INFRASTRUCTURE ONLY.  This header and oracle/sdg_oracle.c restate, in
 * plain C, the reference's column-pair distance slabs, the per-column top-k,
 * the running per-row top-k, the SNN overlap weights and the R orchestration
 * around them.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs load it, as the oracle or as the timed
 * CPU baseline.  The product (libsdgpu.so) never links or calls it.
 *
 * Pinning: binary, cosine, euclidean, manhattan, topKBlock, topKRowsAccum and
 * snnJaccard are checked bit-for-bit against the reference's own unmodified
 * C++ (compiled by oracle/build.py (build_ref) against a project-written API shim into
 * oracle/_ref/) and against the literal fixtures of the reference's tests.
 * pearson and js take their arithmetic from Armadillo (arma::cor, arma::accu),
 * a third-party dependency that the reference does not vendor or pin; for
 * those two methods this oracle states one concrete formulation (see the
 * function comments) and parity with the real package is "parity unpinned".
 */
#ifndef SDG_ORACLE_H
#define SDG_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BINARY = 0, ORC_COSINE = 1, ORC_EUCLIDEAN = 2, ORC_MANHATTAN = 3,
       ORC_PEARSON = 4, ORC_JS = 5, ORC_COVARIANCE = 6 };

/* Status codes; a message is available from orc_last_error(). */
enum { ORC_OK = 0, ORC_E_ARG = -1, ORC_E_NONFINITE = -2, ORC_E_ROWS = -3,
       ORC_E_NOCAND = -4, ORC_E_NOMEM = -5, ORC_E_INDEX = -6 };

/* Bit flags returned through *flags by the orchestration functions. */
enum { ORC_WARN_CLAMP_FWD = 1, ORC_WARN_CLAMP_REV = 2 };

/* A dgCMatrix: p has ncol+1 entries, i/x have p[ncol] entries, rows ascending
 * within each column (R's invariant). */
typedef struct {
  int32_t nrow, ncol;
  const int32_t* p;
  const int32_t* i;
  const double*  x;
} orc_csc;

const char* orc_last_error(void);
void orc_set_threads(int n);         /* the reference's `ncores` */
double orc_na_real(void);           /* R's NA_real_ bit pattern */

/* fastXxx2 slab: D is ncol(m) x ncol(m2), column-major, D(i, j) relates
 * column i of m to column j of m2. */
int orc_slab(int method, int dist, const orc_csc* m, const orc_csc* m2, double* D);
/* single-matrix sparseDist(X, full, diag): n x n column-major into D */
int orc_dist(int method, int dist, const orc_csc* m, int full, int diag, double* D);

/* topKBlock: idx_out / dist_out are ncol x k column-major, 1-based, NA padded. */
int orc_topk_block(const double* D, int64_t nrow, int64_t ncol, int k, int decreasing,
                   const int32_t* self_row, int32_t* idx_out, double* dist_out);

/* topKRowsAccum: best_idx / best_val (nrow x k) are updated in place. */
int orc_topk_rows_accum(const double* D, int64_t nrow, int64_t ncol, int k,
                        int decreasing, int32_t* best_idx, double* best_val,
                        int32_t col_offset, const int32_t* self_col);

/* snnJaccard: w_out is n x k column-major, NA where idx is NA or a set is empty. */
int orc_snn_jaccard(const int32_t* idx, int32_t n, int32_t k, int include_self,
                    double* w_out);

/* sparseKNN: Y == NULL means self-search.  idx_out / dist_out must hold
 * ncol(X) x k; the effective k (after the clamp) is written to *k_eff and the
 * outputs are laid out ncol(X) x k_eff. */
int orc_knn(const orc_csc* X, const orc_csc* Y, int method, int dist, int k,
            int include_self, int drop_degenerate, int block_size,
            int32_t* idx_out, double* dist_out, int* k_eff, int* flags);

/* sparseKNNCross: forward (ncol(X) x k_fwd) and reverse (ncol(Y) x k_rev). */
int orc_knn_cross(const orc_csc* X, const orc_csc* Y, int method, int dist, int k,
                  int drop_degenerate, int block_size,
                  int32_t* fwd_idx, double* fwd_dist, int32_t* rev_idx, double* rev_dist,
                  int* k_fwd, int* k_rev, int* flags);

/* sparseSNN(edges = "knn") assembly.  Two calls: with out_p == NULL only the
 * number of stored entries is written to *nnz_out; then with buffers of that
 * size (out_p: n+1, out_i / out_x: nnz) the dgCMatrix slots are filled. */
int orc_snn_graph(const int32_t* idx, int32_t n, int32_t k, int include_self,
                  double prune, int symmetrise, int64_t* nnz_out,
                  int32_t* out_p, int32_t* out_i, double* out_x);

/* snnJaccardShared: the 1-based upper-triangle triplets (i < j) of every pair
 * sharing a neighbour with weight > prune, rows ascending, each row's pairs in
 * first-touch order.  Two calls: with ti == NULL only *m_out is written. */
int orc_snn_shared(const int32_t* idx, int32_t n, int32_t k, int include_self, double prune,
                   int64_t* m_out, int32_t* ti, int32_t* tj, double* tx);
typedef int (*orc_shared_fn)(const int32_t*, int32_t, int32_t, int, double, int64_t*, int32_t*,
                             int32_t*, double*);

/* sparseSNN(edges = "shared") assembly: the symmetric n x n dgCMatrix (both
 * triangles, no diagonal).  Same two-call protocol as orc_snn_graph. */
int orc_snn_graph_shared(const int32_t* idx, int32_t n, int32_t k, int include_self, double prune,
                         int64_t* nnz_out, int32_t* out_p, int32_t* out_i, double* out_x);
int orc_snn_graph_shared_with(orc_shared_fn f, const int32_t* idx, int32_t n, int32_t k,
                              int include_self, double prune, int64_t* nnz_out, int32_t* out_p,
                              int32_t* out_i, double* out_x);

/* Plug-in points so the same orchestration can drive the reference's own
 * kernels (oracle/_ref) instead of this file's restatement. */
typedef struct {
  int (*slab)(int method, int dist, const orc_csc* m, const orc_csc* m2, double* D);
  int (*topk_block)(const double*, int64_t, int64_t, int, int, const int32_t*,
                    int32_t*, double*);
  int (*topk_rows_accum)(const double*, int64_t, int64_t, int, int, int32_t*,
                         double*, int32_t, const int32_t*);
  int (*snn_jaccard)(const int32_t*, int32_t, int32_t, int, double*);
} orc_backend;

int orc_knn_with(const orc_backend* be, const orc_csc* X, const orc_csc* Y, int method,
                 int dist, int k, int include_self, int drop_degenerate, int block_size,
                 int32_t* idx_out, double* dist_out, int* k_eff, int* flags);
int orc_knn_cross_with(const orc_backend* be, const orc_csc* X, const orc_csc* Y,
                       int method, int dist, int k, int drop_degenerate, int block_size,
                       int32_t* fwd_idx, double* fwd_dist, int32_t* rev_idx,
                       double* rev_dist, int* k_fwd, int* k_rev, int* flags);
int orc_snn_graph_with(const orc_backend* be, const int32_t* idx, int32_t n, int32_t k,
                       int include_self, double prune, int symmetrise, int64_t* nnz_out,
                       int32_t* out_p, int32_t* out_i, double* out_x);

/* Degenerate-column mask: 1 where every stored value is +-0 (R's
 * colSums(abs(M)) == 0 with NA/NaN counting as non-empty). */
void orc_empty_columns(const orc_csc* M, uint8_t* out);

#ifdef __cplusplus
}
#endif
#endif
