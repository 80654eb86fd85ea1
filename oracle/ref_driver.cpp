// ref_driver.cpp -- C entry points over the reference's own, unmodified
// hot-path kernels (src/sparseDist.cpp, src/topK.cpp, src/topKRows.cpp,
// src/snn.cpp), compiled against oracle/shim/.  Built by oracle/build_ref.sh
// into oracle/_ref/libsdref.so.
//
// TEST INFRASTRUCTURE ONLY: it pins the oracle's restatement to the
// reference's own arithmetic and is the "reference" CPU baseline that
// bench.py times.  The product never loads it.
//
// The R orchestration (block loop, masks, clamps) is the oracle's C
// restatement (sdg_oracle.c), driven here through orc_backend with these
// kernels plugged in.
#include <RcppArmadillo.h>

#include <cstdio>
#include <string>

extern "C" {
#include "../sdg_oracle.h"
}

// Reference kernels (declared exactly as in src/*.cpp).
SEXP fastJacc2(const arma::sp_mat& m, const arma::sp_mat& m2, int ncores, bool verbose, bool dist);
SEXP fastCosine2(const arma::sp_mat& m, const arma::sp_mat& m2, int ncores, bool verbose, bool dist);
arma::mat fastEuclidean2(const arma::sp_mat& m, const arma::sp_mat& m2, int ncores, bool verbose);
arma::mat fastManhattan2(const arma::sp_mat& m, const arma::sp_mat& m2, int ncores, bool verbose);
SEXP fastCorr2(const arma::sp_mat& m, const arma::sp_mat& m2, int ncores, bool verbose, bool dist);
arma::mat fastJS2(const arma::mat& m, const arma::mat& m2, int ncores, bool verbose);
arma::sp_mat fastCov2(const arma::sp_mat& m, const arma::sp_mat& m2, int ncores, bool verbose);
SEXP fastJacc(const arma::sp_mat& m, int ncores, bool verbose, bool full, bool diag, bool dist);
SEXP fastCosine(const arma::sp_mat& m, int ncores, bool verbose, bool full, bool diag, bool dist);
arma::mat fastEuclidean(const arma::sp_mat& m, int ncores, bool verbose, bool full, bool diag);
arma::mat fastManhattan(const arma::sp_mat& m, int ncores, bool verbose, bool full, bool diag);
SEXP fastCorr(const arma::sp_mat& m, int ncores, bool verbose, bool full, bool diag, bool dist);
arma::mat fastJS(const arma::mat& m, int ncores, bool verbose, bool full, bool diag);
arma::sp_mat fastCov(const arma::sp_mat& m, int ncores, bool verbose, bool full, bool diag);
Rcpp::List topKBlock(const arma::mat& D, int k, bool decreasing,
                     const Rcpp::IntegerVector& self_row, int ncores);
void topKRowsAccum(const arma::mat& D, int k, bool decreasing, Rcpp::IntegerMatrix best_idx,
                   Rcpp::NumericMatrix best_val, int col_offset,
                   const Rcpp::IntegerVector& self_col, int ncores, int tile_rows);
Rcpp::NumericMatrix snnJaccard(const Rcpp::IntegerMatrix& idx, bool include_self, int ncores,
                               bool verbose);
Rcpp::List snnJaccardShared(const Rcpp::IntegerMatrix& idx, bool include_self, double prune,
                            int ncores, bool verbose);

namespace {

int g_threads = 1;
std::string g_msg;

int fail(const std::exception& e) { g_msg = e.what(); return ORC_E_ARG; }

void dense_out(const SEXP& s, double* D) {
  if (auto m = std::dynamic_pointer_cast<SdgRBox<arma::mat>>(s)) {
    std::memcpy(D, m->value.mem.data(), sizeof(double) * m->value.n_elem);
  } else if (auto sp = std::dynamic_pointer_cast<SdgRBox<arma::sp_mat>>(s)) {
    arma::mat d = sp->value.dense();
    std::memcpy(D, d.mem.data(), sizeof(double) * d.n_elem);
  } else {
    throw std::logic_error("unexpected slab type");
  }
}

int ref_slab(int method, int dist, const orc_csc* a, const orc_csc* b, double* D) {
  try {
    const arma::sp_mat m(a->nrow, a->ncol, a->p, a->i, a->x);
    const arma::sp_mat m2(b->nrow, b->ncol, b->p, b->i, b->x);
    switch (method) {
      case ORC_BINARY: dense_out(fastJacc2(m, m2, g_threads, false, dist != 0), D); break;
      case ORC_COSINE: dense_out(fastCosine2(m, m2, g_threads, false, dist != 0), D); break;
      case ORC_EUCLIDEAN: {
        arma::mat d = fastEuclidean2(m, m2, g_threads, false);
        std::memcpy(D, d.mem.data(), sizeof(double) * d.n_elem);
        break;
      }
      case ORC_MANHATTAN: {
        arma::mat d = fastManhattan2(m, m2, g_threads, false);
        std::memcpy(D, d.mem.data(), sizeof(double) * d.n_elem);
        break;
      }
      case ORC_PEARSON: dense_out(fastCorr2(m, m2, g_threads, false, dist != 0), D); break;
      case ORC_COVARIANCE: dense_out(Rcpp::wrap(fastCov2(m, m2, g_threads, false)), D); break;
      case ORC_JS: {
        // R/sparseKNN.R:194-196: js inputs are coerced with as.matrix.
        arma::mat d = fastJS2(m.dense(), m2.dense(), g_threads, false);
        std::memcpy(D, d.mem.data(), sizeof(double) * d.n_elem);
        break;
      }
      default: g_msg = "unknown method"; return ORC_E_ARG;
    }
    return ORC_OK;
  } catch (const std::exception& e) {
    g_msg = e.what();
    return (g_msg.find("Mismatched") != std::string::npos) ? ORC_E_ROWS : ORC_E_NONFINITE;
  }
}

// R/sparseDist.R:162-171: the single-matrix kernels
int ref_dist(int method, int dist, const orc_csc* a, int full, int diag, double* D) {
  try {
    const arma::sp_mat m(a->nrow, a->ncol, a->p, a->i, a->x);
    const bool f = full != 0, g = diag != 0, d = dist != 0;
    auto put = [&](const arma::mat& r) { std::memcpy(D, r.mem.data(), sizeof(double) * r.n_elem); };
    switch (method) {
      case ORC_BINARY: dense_out(fastJacc(m, g_threads, false, f, g, d), D); break;
      case ORC_COSINE: dense_out(fastCosine(m, g_threads, false, f, g, d), D); break;
      case ORC_EUCLIDEAN: put(fastEuclidean(m, g_threads, false, f, g)); break;
      case ORC_MANHATTAN: put(fastManhattan(m, g_threads, false, f, g)); break;
      case ORC_PEARSON: dense_out(fastCorr(m, g_threads, false, f, g, d), D); break;
      case ORC_COVARIANCE: dense_out(Rcpp::wrap(fastCov(m, g_threads, false, f, g)), D); break;
      case ORC_JS: put(fastJS(m.dense(), g_threads, false, f, g)); break;
      default: g_msg = "unknown method"; return ORC_E_ARG;
    }
    return ORC_OK;
  } catch (const std::exception& e) {
    g_msg = e.what();
    return ORC_E_NONFINITE;
  }
}

int ref_topk_block(const double* D, int64_t nrow, int64_t ncol, int k, int decreasing,
                   const int32_t* self_row, int32_t* idx_out, double* dist_out) {
  try {
    const arma::mat Dm(D, (arma::uword)nrow, (arma::uword)ncol);
    Rcpp::IntegerVector sr((size_t)ncol);
    for (int64_t b = 0; b < ncol; ++b) sr[(size_t)b] = self_row ? self_row[b] : 0;
    Rcpp::List r = topKBlock(Dm, k, decreasing != 0, sr, g_threads);
    Rcpp::IntegerMatrix idx = r.get<Rcpp::IntegerMatrix>("idx");
    Rcpp::NumericMatrix dst = r.get<Rcpp::NumericMatrix>("dist");
    std::memcpy(idx_out, idx.begin(), sizeof(int32_t) * idx.size());
    std::memcpy(dist_out, dst.begin(), sizeof(double) * dst.size());
    return ORC_OK;
  } catch (const std::exception& e) { return fail(e); }
}

int ref_topk_rows_accum(const double* D, int64_t nrow, int64_t ncol, int k, int decreasing,
                        int32_t* best_idx, double* best_val, int32_t col_offset,
                        const int32_t* self_col) {
  try {
    const arma::mat Dm(D, (arma::uword)nrow, (arma::uword)ncol);
    Rcpp::IntegerVector sc((size_t)nrow);
    for (int64_t i = 0; i < nrow; ++i) sc[(size_t)i] = self_col ? self_col[i] : 0;
    topKRowsAccum(Dm, k, decreasing != 0,
                  Rcpp::IntegerMatrix::view(best_idx, (int)nrow, k),
                  Rcpp::NumericMatrix::view(best_val, (int)nrow, k), col_offset, sc,
                  g_threads, 64);
    return ORC_OK;
  } catch (const std::exception& e) { return fail(e); }
}

int ref_snn_jaccard(const int32_t* idx, int32_t n, int32_t k, int include_self, double* w_out) {
  try {
    Rcpp::IntegerMatrix m = Rcpp::IntegerMatrix::view(const_cast<int32_t*>(idx), n, k);
    Rcpp::NumericMatrix w = snnJaccard(m, include_self != 0, g_threads, false);
    std::memcpy(w_out, w.begin(), sizeof(double) * w.size());
    return ORC_OK;
  } catch (const std::exception& e) {
    g_msg = e.what();
    return (g_msg.find("1-based") != std::string::npos) ? ORC_E_INDEX : ORC_E_ARG;
  }
}

const orc_backend g_ref_backend = {ref_slab, ref_topk_block, ref_topk_rows_accum, ref_snn_jaccard};

int ref_snn_shared(const int32_t* idx, int32_t n, int32_t k, int include_self, double prune,
                   int64_t* m_out, int32_t* ti, int32_t* tj, double* tx) {
  try {
    Rcpp::IntegerMatrix m = Rcpp::IntegerMatrix::view(const_cast<int32_t*>(idx), n, k);
    Rcpp::List L = snnJaccardShared(m, include_self != 0, prune, g_threads, false);
    Rcpp::IntegerVector I = L.get<Rcpp::IntegerVector>("i");
    Rcpp::IntegerVector J = L.get<Rcpp::IntegerVector>("j");
    Rcpp::NumericVector X = L.get<Rcpp::NumericVector>("x");
    *m_out = (int64_t)I.size();
    if (ti) {
      std::memcpy(ti, I.begin(), sizeof(int32_t) * I.size());
      std::memcpy(tj, J.begin(), sizeof(int32_t) * J.size());
      std::memcpy(tx, X.begin(), sizeof(double) * X.size());
    }
    return ORC_OK;
  } catch (const std::exception& e) {
    g_msg = e.what();
    return (g_msg.find("1-based") != std::string::npos) ? ORC_E_INDEX : ORC_E_ARG;
  }
}

}  // namespace

extern "C" {

void ref_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
const char* ref_last_error(void) { return g_msg.empty() ? orc_last_error() : g_msg.c_str(); }
void ref_clear_error(void) { g_msg.clear(); }

int ref_slab_c(int method, int dist, const orc_csc* m, const orc_csc* m2, double* D) {
  return ref_slab(method, dist, m, m2, D);
}
int ref_dist_c(int method, int dist, const orc_csc* m, int full, int diag, double* D) {
  g_msg.clear();
  return ref_dist(method, dist, m, full, diag, D);
}
int ref_topk_block_c(const double* D, int64_t nrow, int64_t ncol, int k, int decreasing,
                     const int32_t* self_row, int32_t* idx_out, double* dist_out) {
  return ref_topk_block(D, nrow, ncol, k, decreasing, self_row, idx_out, dist_out);
}
int ref_topk_rows_accum_c(const double* D, int64_t nrow, int64_t ncol, int k, int decreasing,
                          int32_t* best_idx, double* best_val, int32_t col_offset,
                          const int32_t* self_col) {
  return ref_topk_rows_accum(D, nrow, ncol, k, decreasing, best_idx, best_val, col_offset,
                             self_col);
}
int ref_snn_jaccard_c(const int32_t* idx, int32_t n, int32_t k, int include_self, double* w) {
  return ref_snn_jaccard(idx, n, k, include_self, w);
}
int ref_knn(const orc_csc* X, const orc_csc* Y, int method, int dist, int k, int include_self,
            int drop_degenerate, int block_size, int32_t* idx_out, double* dist_out, int* k_eff,
            int* flags) {
  g_msg.clear();
  return orc_knn_with(&g_ref_backend, X, Y, method, dist, k, include_self, drop_degenerate,
                      block_size, idx_out, dist_out, k_eff, flags);
}
int ref_knn_cross(const orc_csc* X, const orc_csc* Y, int method, int dist, int k,
                  int drop_degenerate, int block_size, int32_t* fwd_idx, double* fwd_dist,
                  int32_t* rev_idx, double* rev_dist, int* k_fwd, int* k_rev, int* flags) {
  g_msg.clear();
  return orc_knn_cross_with(&g_ref_backend, X, Y, method, dist, k, drop_degenerate, block_size,
                            fwd_idx, fwd_dist, rev_idx, rev_dist, k_fwd, k_rev, flags);
}
int ref_snn_graph(const int32_t* idx, int32_t n, int32_t k, int include_self, double prune,
                  int symmetrise, int64_t* nnz_out, int32_t* out_p, int32_t* out_i,
                  double* out_x) {
  g_msg.clear();
  return orc_snn_graph_with(&g_ref_backend, idx, n, k, include_self, prune, symmetrise, nnz_out,
                            out_p, out_i, out_x);
}

int ref_snn_shared_c(const int32_t* idx, int32_t n, int32_t k, int include_self, double prune,
                     int64_t* m_out, int32_t* ti, int32_t* tj, double* tx) {
  g_msg.clear();
  return ref_snn_shared(idx, n, k, include_self, prune, m_out, ti, tj, tx);
}
int ref_snn_graph_shared(const int32_t* idx, int32_t n, int32_t k, int include_self, double prune,
                         int64_t* nnz_out, int32_t* out_p, int32_t* out_i, double* out_x) {
  g_msg.clear();
  return orc_snn_graph_shared_with(ref_snn_shared, idx, n, k, include_self, prune, nnz_out, out_p,
                                   out_i, out_x);
}

}  // extern "C"
