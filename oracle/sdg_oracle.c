/*
 * sdg_oracle.c -- CPU oracle for the blocked exact-kNN path of sparseDist.
 *
 * TEST INFRASTRUCTURE ONLY: the results that the GPU library is compared
 * against, and the scalar CPU baseline ("port") that bench.py times.  It is
 * never linked into, or called by, libsdgpu.so.
 *
 * Each function restates the reference's algorithm and cites the file:line of
 * the reference (gambalab/sparseDist) that it follows.  Floating-point
 * expressions are written in the reference's evaluation order and the file is
 * compiled with -ffp-contract=off, so no multiply-add is fused: the results are
 * those of an IEEE double build of the reference (e.g. the usual x86-64 one).
 */
#include "sdg_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* errors and sentinels                                                       */
/* ------------------------------------------------------------------------- */

static char g_err[512];
static int g_threads = 1;

/* Threads used by the slab and top-k loops (the reference's `ncores`). */
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

static int fail(int code, const char* msg) {
  snprintf(g_err, sizeof g_err, "%s", msg);
  return code;
}

const char* orc_last_error(void) { return g_err; }

/* R_NaReal: a NaN whose low word is 1954 (R's arithmetic.c). */
double orc_na_real(void) {
  const uint64_t bits = 0x7FF00000000007A2ULL;
  double d;
  memcpy(&d, &bits, sizeof d);
  return d;
}

#define NA_INT INT_MIN

static int is_na_real(double v) { return isnan(v); }

/* ------------------------------------------------------------------------- */
/* degenerate columns: R/sparseKNN.R:214-220 (colSums(abs(M)) == 0, NA-safe)  */
/* ------------------------------------------------------------------------- */

void orc_empty_columns(const orc_csc* M, uint8_t* out) {
  for (int32_t j = 0; j < M->ncol; ++j) {
    int empty = 1;
    for (int32_t a = M->p[j]; a < M->p[j + 1]; ++a) {
      const double v = M->x[a];
      if (!(v == 0.0)) { empty = 0; break; }   /* non-zero or NaN */
    }
    out[j] = (uint8_t)empty;
  }
}

/* ------------------------------------------------------------------------- */
/* unit-normalised copy: src/sparseDist.cpp:246-284                           */
/* ------------------------------------------------------------------------- */

static int unit_csc(const orc_csc* m, double* uval, double* scale_out) {
  for (int32_t j = 0; j < m->ncol; ++j) {
    double scale = 0.0, ssq = 1.0;
    for (int32_t a = m->p[j]; a < m->p[j + 1]; ++a) {
      const double v = m->x[a];
      if (!isfinite(v))
        return fail(ORC_E_NONFINITE, "Cosine requires finite input (found NA, NaN or Inf).");
      if (v == 0.0) continue;
      const double av = fabs(v);
      if (scale < av) { const double r = scale / av; ssq = 1.0 + ssq * r * r; scale = av; }
      else            { const double r = av / scale; ssq += r * r; }
    }
    const double sq = sqrt(ssq);
    scale_out[j] = scale;
    for (int32_t a = m->p[j]; a < m->p[j + 1]; ++a)
      uval[a] = (scale == 0.0) ? 0.0 : ((m->x[a]) / scale) / sq;
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* per-pair kernels                                                           */
/* ------------------------------------------------------------------------- */

/* jacc_common + jacc_value: src/sparseDist.cpp:535-556 */
static double pair_binary(const orc_csc* A, int32_t i, const orc_csc* B, int32_t j, int dist) {
  int64_t a = A->p[i], ae = A->p[i + 1], b = B->p[j], be = B->p[j + 1];
  const double ni = (double)(ae - a), nj = (double)(be - b);
  double common = 0.0;
  while (a < ae && b < be) {
    const int32_t ra = A->i[a], rb = B->i[b];
    common += (double)(ra == rb);
    a += (ra <= rb);
    b += (rb <= ra);
  }
  const double denom = ni + nj - common;
  const double sim = (denom > 0.0) ? (common / denom) : 1.0;
  return dist ? (1.0 - sim) : sim;
}

/* unit_dot + unit_cosine: src/sparseDist.cpp:287-331; fastCosine2 :990-993 */
static double pair_cosine(const orc_csc* A, const double* ua, const double* sa, int32_t i,
                          const orc_csc* B, const double* ub, const double* sb, int32_t j,
                          int dist) {
  const int ea = (sa[i] == 0.0), eb = (sb[j] == 0.0);
  double c;
  if (ea || eb) {
    c = (ea && eb) ? 1.0 : 0.0;
  } else {
    int64_t a = A->p[i], ae = A->p[i + 1], b = B->p[j], be = B->p[j + 1];
    double s = 0.0;
    while (a < ae && b < be) {
      if (A->i[a] == B->i[b]) { s += ua[a] * ub[b]; ++a; ++b; }
      else if (A->i[a] < B->i[b]) { ++a; }
      else { ++b; }
    }
    c = s;
    if (!(c == c)) c = 0.0;
    else if (c > 1.0) c = 1.0;
    else if (c < -1.0) c = -1.0;
  }
  return dist ? (1.0 - c) : c;
}

/* fastEuclidean2 pair loop: src/sparseDist.cpp:855-871 */
static double pair_euclidean(const orc_csc* A, int32_t i, const orc_csc* B, int32_t j) {
  int64_t a = A->p[i], ae = A->p[i + 1], b = B->p[j], be = B->p[j + 1];
  double num = 0;
  while (a < ae && b < be) {
    if (A->i[a] == B->i[b]) {
      const double diff = A->x[a] - B->x[b]; num += diff * diff; ++a; ++b;
    } else if (A->i[a] < B->i[b]) {
      num += A->x[a] * A->x[a]; ++a;
    } else {
      num += B->x[b] * B->x[b]; ++b;
    }
  }
  for (; a < ae; ++a) num += A->x[a] * A->x[a];
  for (; b < be; ++b) num += B->x[b] * B->x[b];
  return sqrt(num);
}

/* fastManhattan2 pair loop: src/sparseDist.cpp:755-772 */
static double pair_manhattan(const orc_csc* A, int32_t i, const orc_csc* B, int32_t j) {
  int64_t a = A->p[i], ae = A->p[i + 1], b = B->p[j], be = B->p[j + 1];
  double num = 0;
  while (a < ae && b < be) {
    if (A->i[a] == B->i[b]) { num += fabs(A->x[a] - B->x[b]); ++a; ++b; }
    else if (A->i[a] < B->i[b]) { num += fabs(A->x[a]); ++a; }
    else { num += fabs(B->x[b]); ++b; }
  }
  for (; a < ae; ++a) num += fabs(A->x[a]);
  for (; b < be; ++b) num += fabs(B->x[b]);
  return num;
}

/*
 * pearson: fastCorr2, src/sparseDist.cpp:424-431, i.e.
 * as_scalar(arma::cor(li, vec(m2.col(j)), 0)), non-finite -> 0, clamp, 1 - c.
 *
 * arma::cor is Armadillo code (unvendored, version unpinned).  This oracle
 * fixes its vector-vector case as the single-pass form
 *     N = n_rows, norm = (N > 1 ? N - 1 : 1)
 *     cov = (sum(a*b) - (sum(a)*sum(b))/N) / norm
 *     var = (sum(a*a) - (sum(a)*sum(a))/N) / norm
 *     c   = cov / (sqrt(var_a) * sqrt(var_b))
 * with every sum accumulated sequentially in ascending row order.  Zero rows
 * add nothing to any sum, so the sums run over stored entries only.
 * Parity with the real package: unpinned (tolerance only).
 */
typedef struct { double s, ss; } col_moments;

static void moments(const orc_csc* M, col_moments* out) {
  for (int32_t j = 0; j < M->ncol; ++j) {
    double s = 0.0, ss = 0.0;
    for (int32_t a = M->p[j]; a < M->p[j + 1]; ++a) { s += M->x[a]; ss += M->x[a] * M->x[a]; }
    out[j].s = s; out[j].ss = ss;
  }
}

static double pair_pearson(const orc_csc* A, const col_moments* ma, int32_t i,
                           const orc_csc* B, const col_moments* mb, int32_t j, int dist) {
  int64_t a = A->p[i], ae = A->p[i + 1], b = B->p[j], be = B->p[j + 1];
  double sab = 0.0;
  while (a < ae && b < be) {
    if (A->i[a] == B->i[b]) { sab += A->x[a] * B->x[b]; ++a; ++b; }
    else if (A->i[a] < B->i[b]) { ++a; }
    else { ++b; }
  }
  const double N = (double)A->nrow;
  const double norm = (A->nrow > 1) ? (N - 1.0) : 1.0;
  const double cov = (sab - (ma[i].s * mb[j].s) / N) / norm;
  const double va = (ma[i].ss - (ma[i].s * ma[i].s) / N) / norm;
  const double vb = (mb[j].ss - (mb[j].s * mb[j].s) / N) / norm;
  double c = cov / (sqrt(va) * sqrt(vb));
  if (!isfinite(c)) c = 0.0;
  if (c > 1.0) c = 1.0;
  if (c < -1.0) c = -1.0;
  return dist ? (1.0 - c) : c;
}

/*
 * covariance: fastCov2, src/sparseDist.cpp:480-510, i.e.
 * as_scalar(arma::cov(li, vec(m2.col(j)))) with no clamp or non-finite fix:
 * the cov of the single-pass form stated for pearson above (same sums, same
 * order).  Parity with the real package: unpinned (tolerance only).
 */
static double pair_covariance(const orc_csc* A, const col_moments* ma, int32_t i,
                              const orc_csc* B, const col_moments* mb, int32_t j) {
  int64_t a = A->p[i], ae = A->p[i + 1], b = B->p[j], be = B->p[j + 1];
  double sab = 0.0;
  while (a < ae && b < be) {
    if (A->i[a] == B->i[b]) { sab += A->x[a] * B->x[b]; ++a; ++b; }
    else if (A->i[a] < B->i[b]) { ++a; }
    else { ++b; }
  }
  const double N = (double)A->nrow;
  const double norm = (A->nrow > 1) ? (N - 1.0) : 1.0;
  return (sab - (ma[i].s * mb[j].s) / N) / norm;
}

/*
 * js: fastJS2, src/sparseDist.cpp:1099-1108, with xlogx :206-210.
 * Per dense row r the summand is ((xlogx(P)+xlogx(Q)) - xlogx(P+Q)) + (P+Q)*log(2)
 * (Armadillo's element-wise evaluation order of the expression at :1104), and
 * arma::accu sums it with two accumulators, even rows into the first and odd
 * rows into the second, returning acc_even + acc_odd (Armadillo's
 * arrayops::accumulate; unvendored, version unpinned).  Rows where both P and
 * Q are zero give +0 and leave an accumulator unchanged, so the walk visits
 * the union of the stored rows only.  Parity with the real package: unpinned.
 */
static double xlogx(double x) {
  const double r = x * log(x);
  return isnan(r) ? 0.0 : r;
}

static double pair_js(const orc_csc* A, int32_t i, const orc_csc* B, int32_t j) {
  const double log2v = log(2.0);
  int64_t a = A->p[i], ae = A->p[i + 1], b = B->p[j], be = B->p[j + 1];
  double acc[2] = {0.0, 0.0};
  while (a < ae || b < be) {
    int32_t r;
    double P = 0.0, Q = 0.0;
    if (b >= be || (a < ae && A->i[a] < B->i[b])) { r = A->i[a]; P = A->x[a]; ++a; }
    else if (a >= ae || B->i[b] < A->i[a])        { r = B->i[b]; Q = B->x[b]; ++b; }
    else { r = A->i[a]; P = A->x[a]; Q = B->x[b]; ++a; ++b; }
    const double PQ = P + Q;
    const double t = ((xlogx(P) + xlogx(Q)) - xlogx(PQ)) + PQ * log2v;
    acc[r & 1] += t;
  }
  const double v = 0.5 * (acc[0] + acc[1]);
  return (v > 0.0) ? sqrt(v) : 0.0;
}

static int check_js_input_named(const orc_csc* m, const char* fn) {
  const int64_t nnz = m->p[m->ncol];
  for (int64_t a = 0; a < nnz; ++a) {
    const double v = m->x[a];
    if (!isfinite(v) || v < 0.0) {
      char buf[256];
      snprintf(buf, sizeof buf,
               "%s requires finite, non-negative input (columns should be "
               "normalised to sum to 1 for a true JS divergence).", fn);
      return fail(ORC_E_NONFINITE, buf);
    }
  }
  return ORC_OK;
}

static int check_js_input(const orc_csc* m) { return check_js_input_named(m, "fastJS2"); }

/* ------------------------------------------------------------------------- */
/* fastXxx2 slab dispatch: R/sparseDist.R:172-182 -> src/sparseDist.cpp       */
/* ------------------------------------------------------------------------- */

int orc_slab(int method, int dist, const orc_csc* m, const orc_csc* m2, double* D) {
  if (method == ORC_JS) {                       /* src/sparseDist.cpp:1077-1081 first */
    int st = check_js_input(m);
    if (st == ORC_OK) st = check_js_input(m2);
    if (st != ORC_OK) return st;
  }
  if (m->nrow != m2->nrow) {
    char buf[256];
    snprintf(buf, sizeof buf, "Mismatched row dimensions of m (%d) and m2 (%d).",
             (int)m->nrow, (int)m2->nrow);
    return fail(ORC_E_ROWS, buf);
  }
  const int64_t nc = m->ncol, nc2 = m2->ncol;
  double *ua = NULL, *ub = NULL, *sa = NULL, *sb = NULL;
  col_moments *ma = NULL, *mb = NULL;
  int st = ORC_OK;
  if (method == ORC_COSINE) {
    ua = malloc(sizeof(double) * ((size_t)m->p[nc] + 1));
    ub = malloc(sizeof(double) * ((size_t)m2->p[nc2] + 1));
    sa = malloc(sizeof(double) * ((size_t)nc + 1));
    sb = malloc(sizeof(double) * ((size_t)nc2 + 1));
    if (!ua || !ub || !sa || !sb) { st = fail(ORC_E_NOMEM, "out of memory"); goto done; }
    st = unit_csc(m, ua, sa);
    if (st == ORC_OK) st = unit_csc(m2, ub, sb);
    if (st != ORC_OK) goto done;
  } else if (method == ORC_PEARSON || method == ORC_COVARIANCE) {
    ma = malloc(sizeof(col_moments) * ((size_t)nc + 1));
    mb = malloc(sizeof(col_moments) * ((size_t)nc2 + 1));
    if (!ma || !mb) { st = fail(ORC_E_NOMEM, "out of memory"); goto done; }
    moments(m, ma);
    moments(m2, mb);
  } else if (method < 0 || method > ORC_COVARIANCE) {
    return fail(ORC_E_ARG, "unknown method");
  }
  /* parallel over the columns of m, as the reference's OpenMP loops are */
#pragma omp parallel for num_threads(g_threads) schedule(dynamic)
  for (int64_t i = 0; i < nc; ++i) {
    for (int64_t j = 0; j < nc2; ++j) {
      double v;
      switch (method) {
        case ORC_BINARY:    v = pair_binary(m, (int32_t)i, m2, (int32_t)j, dist); break;
        case ORC_COSINE:    v = pair_cosine(m, ua, sa, (int32_t)i, m2, ub, sb, (int32_t)j, dist); break;
        case ORC_EUCLIDEAN: v = pair_euclidean(m, (int32_t)i, m2, (int32_t)j); break;
        case ORC_MANHATTAN: v = pair_manhattan(m, (int32_t)i, m2, (int32_t)j); break;
        case ORC_PEARSON:   v = pair_pearson(m, ma, (int32_t)i, m2, mb, (int32_t)j, dist); break;
        case ORC_COVARIANCE: v = pair_covariance(m, ma, (int32_t)i, m2, mb, (int32_t)j); break;
        default:            v = pair_js(m, (int32_t)i, m2, (int32_t)j); break;
      }
      D[j * nc + i] = v;
    }
  }
done:
  free(ua); free(ub); free(sa); free(sb); free(ma); free(mb);
  return st;
}

/* ------------------------------------------------------------------------- */
/* single-matrix form: R/sparseDist.R:162-171 -> fastJacc (src/sparseDist.cpp: */
/* 620-680), fastCosine (:918-960), fastEuclidean (:786-830), fastManhattan    */
/* (:688-731), fastCorr (:339-398), fastCov (:450-478), fastJS (:1021-1071).   */
/* Column i is visited against j = i (diag) or i + 1 .. n-1; the value of the  */
/* pair (i, j) with i <= j goes to d(j, i) and, with full, to d(i, j) too.     */
/* ------------------------------------------------------------------------- */

int orc_dist(int method, int dist, const orc_csc* m, int full, int diag, double* D) {
  if (method < 0 || method > ORC_COVARIANCE) return fail(ORC_E_ARG, "unknown method");
  if (method == ORC_JS) {                       /* src/sparseDist.cpp:1024-1027 */
    int st = check_js_input_named(m, "fastJS");
    if (st != ORC_OK) return st;
  }
  const int64_t n = m->ncol;
  double *ua = NULL, *sa = NULL;
  col_moments* ma = NULL;
  int st = ORC_OK;
  memset(D, 0, sizeof(double) * (size_t)(n * n));
  if (method == ORC_COSINE) {
    ua = malloc(sizeof(double) * ((size_t)m->p[n] + 1));
    sa = malloc(sizeof(double) * ((size_t)n + 1));
    if (!ua || !sa) { st = fail(ORC_E_NOMEM, "out of memory"); goto done; }
    st = unit_csc(m, ua, sa);
    if (st != ORC_OK) goto done;
  } else if (method == ORC_PEARSON || method == ORC_COVARIANCE) {
    ma = malloc(sizeof(col_moments) * ((size_t)n + 1));
    if (!ma) { st = fail(ORC_E_NOMEM, "out of memory"); goto done; }
    moments(m, ma);
  }
#pragma omp parallel for num_threads(g_threads) schedule(dynamic)
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t j = diag ? i : i + 1; j < n; ++j) {
      double v;
      switch (method) {
        case ORC_BINARY:    v = pair_binary(m, (int32_t)i, m, (int32_t)j, dist); break;
        case ORC_COSINE:    /* :937-939: the self pair is exact */
          v = (i == j) ? (dist ? 0.0 : 1.0)
                       : pair_cosine(m, ua, sa, (int32_t)i, m, ua, sa, (int32_t)j, dist);
          break;
        case ORC_EUCLIDEAN: v = pair_euclidean(m, (int32_t)i, m, (int32_t)j); break;
        case ORC_MANHATTAN: v = pair_manhattan(m, (int32_t)i, m, (int32_t)j); break;
        case ORC_PEARSON:   /* :358-363 */
          v = (i == j) ? (dist ? 0.0 : 1.0)
                       : pair_pearson(m, ma, (int32_t)i, m, ma, (int32_t)j, dist);
          break;
        case ORC_COVARIANCE: v = pair_covariance(m, ma, (int32_t)i, m, ma, (int32_t)j); break;
        default:            /* :1045-1048: the self pair is skipped (stays 0) */
          v = (i == j) ? 0.0 : pair_js(m, (int32_t)i, m, (int32_t)j);
          break;
      }
      D[i * n + j] = v;
      if (full) D[j * n + i] = v;
    }
  }
  /* :393, :674, :957: the similarity forms carry a unit diagonal */
  if (!dist && (method == ORC_BINARY || method == ORC_COSINE || method == ORC_PEARSON))
    for (int64_t i = 0; i < n; ++i) D[i * n + i] = 1.0;
done:
  free(ua); free(sa); free(ma);
  return st;
}

/* ------------------------------------------------------------------------- */
/* bounded heap on (value, index): src/topK.cpp:38-50, src/topKRows.cpp:54-66 */
/* ------------------------------------------------------------------------- */

typedef struct { double v; int64_t i; } cand;

/* "a is a better neighbour than b" */
static int better(const cand* a, const cand* b, int decreasing) {
  if (a->v != b->v) return decreasing ? (a->v > b->v) : (a->v < b->v);
  return a->i < b->i;
}

/* max-heap under "better": the root is the WORST kept candidate */
static void sift_down(cand* h, int64_t n, int64_t at, int dec) {
  for (;;) {
    int64_t l = 2 * at + 1, r = l + 1, w = at;
    if (l < n && better(&h[w], &h[l], dec)) w = l;
    if (r < n && better(&h[w], &h[r], dec)) w = r;
    if (w == at) return;
    cand t = h[at]; h[at] = h[w]; h[w] = t; at = w;
  }
}

static void sift_up(cand* h, int64_t at, int dec) {
  while (at > 0) {
    int64_t par = (at - 1) / 2;
    if (!better(&h[par], &h[at], dec)) return;
    cand t = h[at]; h[at] = h[par]; h[par] = t; at = par;
  }
}

static void heap_offer(cand* h, int64_t* n, int64_t K, cand c, int dec) {
  if (*n < K) { h[*n] = c; sift_up(h, *n, dec); ++*n; }
  else if (better(&c, &h[0], dec)) { h[0] = c; sift_down(h, K, 0, dec); }
}

static int cmp_best_first_inc(const void* x, const void* y) {
  const cand* a = (const cand*)x; const cand* b = (const cand*)y;
  if (better(a, b, 0)) return -1;
  if (better(b, a, 0)) return 1;
  return 0;
}
static int cmp_best_first_dec(const void* x, const void* y) {
  const cand* a = (const cand*)x; const cand* b = (const cand*)y;
  if (better(a, b, 1)) return -1;
  if (better(b, a, 1)) return 1;
  return 0;
}

static void sort_best_first(cand* h, int64_t n, int dec) {
  qsort(h, (size_t)n, sizeof(cand), dec ? cmp_best_first_dec : cmp_best_first_inc);
}

/* topKBlock: src/topK.cpp:66-149 */
int orc_topk_block(const double* D, int64_t nrow, int64_t ncol, int k, int decreasing,
                   const int32_t* self_row, int32_t* idx_out, double* dist_out) {
  if (k < 1) return fail(ORC_E_ARG, "k must be >= 1.");
  for (int64_t b = 0; b < ncol; ++b) {
    const int32_t sr = self_row ? self_row[b] : 0;
    if (sr == NA_INT || sr < 0 || (int64_t)sr > nrow)
      return fail(ORC_E_ARG, "self_row entries must be 0 or valid 1-based rows of D.");
  }
  const double na = orc_na_real();
  int st = ORC_OK;
#pragma omp parallel num_threads(g_threads)
  {
  cand* h = malloc(sizeof(cand) * (size_t)k);
  if (!h) {
#pragma omp critical
    st = fail(ORC_E_NOMEM, "out of memory");
  }
#pragma omp for schedule(dynamic)
  for (int64_t b = 0; b < ncol; ++b) {
    if (!h) continue;
    const int32_t sr = self_row ? self_row[b] : 0;
    const int64_t skip = (sr > 0) ? (int64_t)(sr - 1) : nrow;
    int64_t n = 0;
    for (int64_t i = 0; i < nrow; ++i) {
      if (i == skip) continue;
      const double v = D[b * nrow + i];
      if (!isfinite(v)) continue;
      cand c = { v, i };
      heap_offer(h, &n, k, c, decreasing);
    }
    sort_best_first(h, n, decreasing);
    for (int64_t t = 0; t < k; ++t) {
      const int64_t at = t * ncol + b;
      if (t < n) { dist_out[at] = h[t].v; idx_out[at] = (int32_t)(h[t].i + 1); }
      else       { dist_out[at] = na;     idx_out[at] = NA_INT; }
    }
  }
  free(h);
  }
  return st;
}

/* topKRowsAccum: src/topKRows.cpp:103-248 */
int orc_topk_rows_accum(const double* D, int64_t nrow, int64_t ncol, int k,
                        int decreasing, int32_t* best_idx, double* best_val,
                        int32_t col_offset, const int32_t* self_col) {
  if (k < 1) return fail(ORC_E_ARG, "k must be >= 1.");
  if (col_offset < 0) return fail(ORC_E_ARG, "col_offset must be >= 0.");
  for (int64_t i = 0; i < nrow; ++i) {
    const int32_t sc = self_col ? self_col[i] : 0;
    if (sc == NA_INT || sc < 0)
      return fail(ORC_E_ARG, "self_col entries must be 0 or a positive 1-based query index.");
  }
  const double na = orc_na_real();
  cand* h = malloc(sizeof(cand) * (size_t)k);
  if (!h) return fail(ORC_E_NOMEM, "out of memory");
  for (int64_t i = 0; i < nrow; ++i) {
    int64_t n = 0;
    for (int64_t t = 0; t < k; ++t) {          /* seed from the carried state */
      const int32_t gi = best_idx[t * nrow + i];
      if (gi == NA_INT || gi <= 0) break;
      cand c = { best_val[t * nrow + i], (int64_t)gi - 1 };
      heap_offer(h, &n, k, c, decreasing);
    }
    const int32_t sc = self_col ? self_col[i] : 0;
    for (int64_t b = 0; b < ncol; ++b) {
      const int64_t g = (int64_t)col_offset + b;
      if ((int64_t)sc == g + 1) continue;
      const double v = D[b * nrow + i];
      if (!isfinite(v)) continue;
      cand c = { v, g };
      heap_offer(h, &n, k, c, decreasing);
    }
    sort_best_first(h, n, decreasing);
    for (int64_t t = 0; t < k; ++t) {
      const int64_t at = t * nrow + i;
      if (t < n) { best_val[at] = h[t].v; best_idx[at] = (int32_t)(h[t].i + 1); }
      else       { best_val[at] = na;     best_idx[at] = NA_INT; }
    }
  }
  free(h);
  return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* snnJaccard: src/snn.cpp:73-82 (inter_size), :94-108 (copy_indices),         */
/* :119-141 (build_sets), :179-181 (jaccard_from_counts), :197-250            */
/* ------------------------------------------------------------------------- */

static int cmp_int(const void* x, const void* y) {
  const int32_t a = *(const int32_t*)x, b = *(const int32_t*)y;
  return (a > b) - (a < b);
}

int orc_snn_jaccard(const int32_t* idx, int32_t n, int32_t k, int include_self,
                    double* w_out) {
  if (n < 1 || k < 1) return fail(ORC_E_ARG, "'idx' must have at least one row and column.");
  const int64_t N = n;
  for (int32_t t = 0; t < k; ++t)
    for (int32_t i = 0; i < n; ++i) {
      const int32_t v = idx[i + N * t];
      if (v != NA_INT && (v < 1 || v > n))
        return fail(ORC_E_INDEX,
                    "'idx' entries must be NA or 1-based row indices in [1, nrow(idx)].");
    }
  const int64_t S = (int64_t)k + 1;
  int32_t* sets = malloc(sizeof(int32_t) * (size_t)(N * S));
  int32_t* size = malloc(sizeof(int32_t) * (size_t)N);
  if (!sets || !size) { free(sets); free(size); return fail(ORC_E_NOMEM, "out of memory"); }
  for (int32_t i = 0; i < n; ++i) {
    int32_t* s = sets + (int64_t)i * S;
    int32_t c = 0;
    if (include_self) s[c++] = i;
    for (int32_t t = 0; t < k; ++t) {
      const int32_t v = idx[i + N * t];
      if (v == NA_INT) continue;
      if (v - 1 != i) s[c++] = v - 1;
    }
    qsort(s, (size_t)c, sizeof(int32_t), cmp_int);
    int32_t u = 0;
    for (int32_t a = 0; a < c; ++a)
      if (u == 0 || s[u - 1] != s[a]) s[u++] = s[a];
    size[i] = u;
  }
  const double na = orc_na_real();
  for (int64_t a = 0; a < N * k; ++a) w_out[a] = na;
  for (int32_t i = 0; i < n; ++i) {
    if (size[i] == 0) continue;
    const int32_t* si = sets + (int64_t)i * S;
    for (int32_t t = 0; t < k; ++t) {
      const int32_t v = idx[i + N * t];
      if (v == NA_INT) continue;
      const int32_t j = v - 1;
      if (size[j] == 0) continue;
      const int32_t* sj = sets + (int64_t)j * S;
      int64_t c = 0, ia = 0, ib = 0;
      while (ia < size[i] && ib < size[j]) {
        if (si[ia] < sj[ib]) ++ia;
        else if (sj[ib] < si[ia]) ++ib;
        else { ++c; ++ia; ++ib; }
      }
      w_out[i + N * t] = (double)c / (double)((int64_t)size[i] + size[j] - c);
    }
  }
  free(sets); free(size);
  return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* backends                                                                   */
/* ------------------------------------------------------------------------- */

static const orc_backend g_self_backend = {
  orc_slab, orc_topk_block, orc_topk_rows_accum, orc_snn_jaccard
};

static int decreasing_for(int method, int dist) {
  /* R/sparseKNN.R:172-181 */
  switch (method) {
    case ORC_BINARY: case ORC_COSINE: case ORC_PEARSON: return !dist;
    case ORC_COVARIANCE: return 1;               /* a coefficient: keep the largest */
    default: return 0;
  }
}

static int check_dist_form(int method, int dist) {
  /* R/sparseKNN.R:168-171 */
  if (method < 0 || method > ORC_COVARIANCE) return fail(ORC_E_ARG, "unknown method");
  if ((method == ORC_EUCLIDEAN || method == ORC_MANHATTAN || method == ORC_JS) && !dist) {
    static const char* names[] = {"binary", "cosine", "euclidean", "manhattan", "pearson", "js"};
    char buf[256];
    snprintf(buf, sizeof buf,
             "'dist = FALSE' is only meaningful for methods \"binary\", \"cosine\" and "
             "\"pearson\"; %s has no similarity form.", names[method]);
    return fail(ORC_E_ARG, buf);
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------- */
/* sparseKNN orchestration: R/sparseKNN.R:110-313                             */
/* ------------------------------------------------------------------------- */

int orc_knn_with(const orc_backend* be, const orc_csc* X, const orc_csc* Y, int method,
                 int dist, int k, int include_self, int drop_degenerate, int block_size,
                 int32_t* idx_out, double* dist_out, int* k_eff, int* flags) {
  *flags = 0;
  if (k < 1) return fail(ORC_E_ARG, "'k' must be a positive integer no larger than .Machine$integer.max.");
  if (block_size < 1)
    return fail(ORC_E_ARG, "'block_size' must be a positive integer no larger than .Machine$integer.max.");
  int st = check_dist_form(method, dist);
  if (st != ORC_OK) return st;
  const int decreasing = decreasing_for(method, dist);
  const int64_t nq = X->ncol;
  if (nq < 1) return fail(ORC_E_ARG, "'X' must have at least one column.");
  const int selfmode = (Y == NULL);
  if (!selfmode && X->nrow != Y->nrow)
    return fail(ORC_E_ROWS, "'X' and 'Y' must have the same number of rows.");
  const orc_csc* ref = selfmode ? X : Y;
  const int64_t nref = ref->ncol;

  uint8_t* deg_ref = calloc((size_t)nref + 1, 1);
  uint8_t* deg_q = calloc((size_t)nq + 1, 1);
  if (!deg_ref || !deg_q) { free(deg_ref); free(deg_q); return fail(ORC_E_NOMEM, "out of memory"); }
  if (drop_degenerate) orc_empty_columns(ref, deg_ref);
  if (selfmode) memcpy(deg_q, deg_ref, (size_t)nq);
  else if (drop_degenerate) orc_empty_columns(X, deg_q);

  int64_t avail = 0;
  for (int64_t j = 0; j < nref; ++j) avail += !deg_ref[j];
  if (selfmode && !include_self) avail -= 1;
  if (avail < 1) { free(deg_ref); free(deg_q); return fail(ORC_E_NOCAND, "No candidate neighbours available."); }
  if (k > avail) { *flags |= ORC_WARN_CLAMP_FWD; k = (int)avail; }
  *k_eff = k;

  const double na = orc_na_real();
  for (int64_t a = 0; a < nq * k; ++a) { idx_out[a] = NA_INT; dist_out[a] = na; }

  const int64_t B = block_size < nq ? block_size : nq;
  double* D = malloc(sizeof(double) * (size_t)(nref * B));
  int32_t* self_row = malloc(sizeof(int32_t) * (size_t)B);
  int32_t* pidx = malloc(sizeof(int32_t) * (size_t)(B * k));
  double* pdst = malloc(sizeof(double) * (size_t)(B * k));
  if (!D || !self_row || !pidx || !pdst) { st = fail(ORC_E_NOMEM, "out of memory"); goto out; }

  for (int64_t from = 0; from < nq; from += block_size) {
    const int64_t to = (from + block_size < nq) ? from + block_size : nq;
    const int64_t nb = to - from;
    orc_csc blk = { X->nrow, (int32_t)nb, X->p + from, X->i, X->x };
    st = be->slab(method, dist, ref, &blk, D);
    if (st != ORC_OK) goto out;
    for (int64_t b = 0; b < nb; ++b)
      self_row[b] = (selfmode && !include_self) ? (int32_t)(from + b + 1) : 0;
    /* R/sparseKNN.R:270-279; covariance keeps its computed self value (the variance) */
    if (selfmode && include_self && method != ORC_COVARIANCE) {
      const double sv = (method == ORC_BINARY || method == ORC_COSINE || method == ORC_PEARSON)
                            ? (dist ? 0.0 : 1.0) : 0.0;
      for (int64_t b = 0; b < nb; ++b) D[b * nref + (from + b)] = sv;
    }
    for (int64_t i = 0; i < nref; ++i)               /* R/sparseKNN.R:285 */
      if (deg_ref[i]) for (int64_t b = 0; b < nb; ++b) D[b * nref + i] = na;
    st = be->topk_block(D, nref, nb, k, decreasing, self_row, pidx, pdst);
    if (st != ORC_OK) goto out;
    for (int64_t t = 0; t < k; ++t)
      for (int64_t b = 0; b < nb; ++b) {
        idx_out[t * nq + from + b] = pidx[t * nb + b];
        dist_out[t * nq + from + b] = pdst[t * nb + b];
      }
  }
  for (int64_t q = 0; q < nq; ++q)                   /* R/sparseKNN.R:298-301 */
    if (deg_q[q]) for (int64_t t = 0; t < k; ++t) { idx_out[t * nq + q] = NA_INT; dist_out[t * nq + q] = na; }
out:
  free(D); free(self_row); free(pidx); free(pdst); free(deg_ref); free(deg_q);
  return st;
}

int orc_knn(const orc_csc* X, const orc_csc* Y, int method, int dist, int k,
            int include_self, int drop_degenerate, int block_size,
            int32_t* idx_out, double* dist_out, int* k_eff, int* flags) {
  return orc_knn_with(&g_self_backend, X, Y, method, dist, k, include_self, drop_degenerate,
                      block_size, idx_out, dist_out, k_eff, flags);
}

/* ------------------------------------------------------------------------- */
/* sparseKNNCross orchestration: R/sparseKNNCross.R:44-199                    */
/* ------------------------------------------------------------------------- */

int orc_knn_cross_with(const orc_backend* be, const orc_csc* X, const orc_csc* Y,
                       int method, int dist, int k, int drop_degenerate, int block_size,
                       int32_t* fwd_idx, double* fwd_dist, int32_t* rev_idx,
                       double* rev_dist, int* k_fwd, int* k_rev, int* flags) {
  *flags = 0;
  if (Y == NULL)
    return fail(ORC_E_ARG, "'Y' is required. For a single matrix use sparseKNN(), which already "
                           "exploits symmetry via the full/diag arguments.");
  if (k < 1) return fail(ORC_E_ARG, "'k' must be a positive integer no larger than .Machine$integer.max.");
  if (block_size < 1)
    return fail(ORC_E_ARG, "'block_size' must be a positive integer no larger than .Machine$integer.max.");
  int st = check_dist_form(method, dist);
  if (st != ORC_OK) return st;
  const int decreasing = decreasing_for(method, dist);
  if (X->nrow != Y->nrow) return fail(ORC_E_ROWS, "'X' and 'Y' must have the same number of rows.");
  const int64_t nq = X->ncol, nr = Y->ncol;
  if (nq < 1) return fail(ORC_E_ARG, "'X' must have at least one column.");
  if (nr < 1) return fail(ORC_E_ARG, "'Y' must have at least one column.");

  uint8_t* deg_q = calloc((size_t)nq + 1, 1);
  uint8_t* deg_r = calloc((size_t)nr + 1, 1);
  if (!deg_q || !deg_r) { free(deg_q); free(deg_r); return fail(ORC_E_NOMEM, "out of memory"); }
  if (drop_degenerate) { orc_empty_columns(X, deg_q); orc_empty_columns(Y, deg_r); }
  int64_t av_f = 0, av_r = 0;
  for (int64_t j = 0; j < nr; ++j) av_f += !deg_r[j];
  for (int64_t j = 0; j < nq; ++j) av_r += !deg_q[j];
  /* R/sparseKNNCross.R:117-127 */
  if (av_f < 1) { free(deg_q); free(deg_r); return fail(ORC_E_NOCAND, "No candidate neighbours available for the forward direction."); }
  int kf = k, kr = k;
  if (kf > av_f) { *flags |= ORC_WARN_CLAMP_FWD; kf = (int)av_f; }
  if (av_r < 1) { free(deg_q); free(deg_r); return fail(ORC_E_NOCAND, "No candidate neighbours available for the reverse direction."); }
  if (kr > av_r) { *flags |= ORC_WARN_CLAMP_REV; kr = (int)av_r; }
  *k_fwd = kf; *k_rev = kr;

  const double na = orc_na_real();
  for (int64_t a = 0; a < nq * kf; ++a) { fwd_idx[a] = NA_INT; fwd_dist[a] = na; }
  for (int64_t a = 0; a < nr * kr; ++a) { rev_idx[a] = NA_INT; rev_dist[a] = na; }

  const int64_t B = block_size < nq ? block_size : nq;
  double* D = malloc(sizeof(double) * (size_t)(nr * B));
  int32_t* zeros_b = calloc((size_t)B, sizeof(int32_t));
  int32_t* zeros_r = calloc((size_t)nr, sizeof(int32_t));
  int32_t* pidx = malloc(sizeof(int32_t) * (size_t)(B * kf));
  double* pdst = malloc(sizeof(double) * (size_t)(B * kf));
  if (!D || !zeros_b || !zeros_r || !pidx || !pdst) { st = fail(ORC_E_NOMEM, "out of memory"); goto out; }

  for (int64_t from = 0; from < nq; from += block_size) {
    const int64_t to = (from + block_size < nq) ? from + block_size : nq;
    const int64_t nb = to - from;
    orc_csc blk = { X->nrow, (int32_t)nb, X->p + from, X->i, X->x };
    st = be->slab(method, dist, Y, &blk, D);
    if (st != ORC_OK) goto out;
    for (int64_t i = 0; i < nr; ++i)                 /* R/sparseKNNCross.R:166-168 */
      if (deg_r[i]) for (int64_t b = 0; b < nb; ++b) D[b * nr + i] = na;
    for (int64_t b = 0; b < nb; ++b)
      if (deg_q[from + b]) for (int64_t i = 0; i < nr; ++i) D[b * nr + i] = na;
    st = be->topk_block(D, nr, nb, kf, decreasing, zeros_b, pidx, pdst);
    if (st != ORC_OK) goto out;
    for (int64_t t = 0; t < kf; ++t)
      for (int64_t b = 0; b < nb; ++b) {
        fwd_idx[t * nq + from + b] = pidx[t * nb + b];
        fwd_dist[t * nq + from + b] = pdst[t * nb + b];
      }
    st = be->topk_rows_accum(D, nr, nb, kr, decreasing, rev_idx, rev_dist, (int32_t)from, zeros_r);
    if (st != ORC_OK) goto out;
  }
  for (int64_t q = 0; q < nq; ++q)
    if (deg_q[q]) for (int64_t t = 0; t < kf; ++t) { fwd_idx[t * nq + q] = NA_INT; fwd_dist[t * nq + q] = na; }
  for (int64_t r = 0; r < nr; ++r)
    if (deg_r[r]) for (int64_t t = 0; t < kr; ++t) { rev_idx[t * nr + r] = NA_INT; rev_dist[t * nr + r] = na; }
out:
  free(D); free(zeros_b); free(zeros_r); free(pidx); free(pdst); free(deg_q); free(deg_r);
  return st;
}

int orc_knn_cross(const orc_csc* X, const orc_csc* Y, int method, int dist, int k,
                  int drop_degenerate, int block_size,
                  int32_t* fwd_idx, double* fwd_dist, int32_t* rev_idx, double* rev_dist,
                  int* k_fwd, int* k_rev, int* flags) {
  return orc_knn_cross_with(&g_self_backend, X, Y, method, dist, k, drop_degenerate,
                            block_size, fwd_idx, fwd_dist, rev_idx, rev_dist, k_fwd, k_rev,
                            flags);
}

/* ------------------------------------------------------------------------- */
/* sparseSNN(edges = "knn") assembly: R/sparseSNN.R:221-250                   */
/* ------------------------------------------------------------------------- */

typedef struct { int64_t key; int64_t ord; double x; } trip;

static int cmp_trip(const void* a, const void* b) {
  const trip* x = (const trip*)a; const trip* y = (const trip*)b;
  if (x->key != y->key) return (x->key > y->key) - (x->key < y->key);
  return (x->ord > y->ord) - (x->ord < y->ord);
}

/* binary search of a sorted, de-duplicated key array */
static int64_t find_key(const trip* t, int64_t n, int64_t key) {
  int64_t lo = 0, hi = n;
  while (lo < hi) { int64_t mid = (lo + hi) / 2; if (t[mid].key < key) lo = mid + 1; else hi = mid; }
  return (lo < n && t[lo].key == key) ? lo : -1;
}

int orc_snn_graph_with(const orc_backend* be, const int32_t* idx, int32_t n, int32_t k,
                       int include_self, double prune, int symmetrise, int64_t* nnz_out,
                       int32_t* out_p, int32_t* out_i, double* out_x) {
  const int64_t N = n;
  double* w = malloc(sizeof(double) * (size_t)(N * k + 1));
  if (!w) return fail(ORC_E_NOMEM, "out of memory");
  int st = be->snn_jaccard(idx, n, k, include_self, w);
  if (st != ORC_OK) { free(w); return st; }
  /* keep <- !is.na(w) & !is.na(idx) & (w > prune); triplets in column-major order */
  trip* g = malloc(sizeof(trip) * (size_t)(N * k + 1));
  if (!g) { free(w); return fail(ORC_E_NOMEM, "out of memory"); }
  int64_t m = 0;
  for (int64_t a = 0; a < N * k; ++a) {
    if (is_na_real(w[a]) || idx[a] == NA_INT || !(w[a] > prune)) continue;
    const int64_t i = a % N, j = (int64_t)idx[a] - 1;
    g[m].key = j * N + i; g[m].ord = a; g[m].x = w[a]; ++m;
  }
  free(w);
  /* sparseMatrix(use.last.ij = TRUE): the last triplet of each (i, j) wins */
  qsort(g, (size_t)m, sizeof(trip), cmp_trip);
  int64_t u = 0;
  for (int64_t a = 0; a < m; ++a) {
    if (u > 0 && g[u - 1].key == g[a].key) g[u - 1] = g[a];
    else g[u++] = g[a];
  }
  m = u;
  trip* out = g;
  int64_t nout = m;
  if (symmetrise) {
    /* g + t(g) - t(g) * (g > 0): the union of both patterns; where both hold
     * an entry the value is (g_ij + g_ji) - g_ji */
    out = malloc(sizeof(trip) * (size_t)(2 * m + 1));
    if (!out) { free(g); return fail(ORC_E_NOMEM, "out of memory"); }
    nout = 0;
    for (int64_t a = 0; a < m; ++a) {
      const int64_t j = g[a].key / N, i = g[a].key % N;
      const int64_t tk = i * N + j;                 /* (j, i) stored as column i, row j */
      const int64_t b = find_key(g, m, tk);
      out[nout].key = g[a].key; out[nout].ord = 0;
      out[nout].x = (b >= 0) ? ((g[a].x + g[b].x) - g[b].x) : g[a].x;
      ++nout;
      if (b < 0) {                                   /* mirror entry absent from g */
        out[nout].key = tk; out[nout].ord = 0; out[nout].x = g[a].x; ++nout;
      }
    }
    qsort(out, (size_t)nout, sizeof(trip), cmp_trip);
  }
  *nnz_out = nout;
  if (out_p) {
    for (int64_t c = 0; c <= N; ++c) out_p[c] = 0;
    for (int64_t a = 0; a < nout; ++a) out_p[out[a].key / N + 1] += 1;
    for (int64_t c = 0; c < N; ++c) out_p[c + 1] += out_p[c];
    for (int64_t a = 0; a < nout; ++a) { out_i[a] = (int32_t)(out[a].key % N); out_x[a] = out[a].x; }
  }
  if (out != g) free(out);
  free(g);
  return ORC_OK;
}

int orc_snn_graph(const int32_t* idx, int32_t n, int32_t k, int include_self,
                  double prune, int symmetrise, int64_t* nnz_out,
                  int32_t* out_p, int32_t* out_i, double* out_x) {
  return orc_snn_graph_with(&g_self_backend, idx, n, k, include_self, prune, symmetrise,
                            nnz_out, out_p, out_i, out_x);
}

/* ------------------------------------------------------------------------- */
/* sparseSNN(edges = "shared"): snnJaccardShared (src/snn.cpp:252-447) and    */
/* its assembly (R/sparseSNN.R:202-219)                                       */
/* ------------------------------------------------------------------------- */

/* Neighbour sets as in snnJaccard (copy_indices :94-108, build_sets :119-141):
 * NA dropped, self removed then added iff include_self, sorted, unique. */
static int shared_sets(const int32_t* idx, int32_t n, int32_t k, int include_self,
                       int32_t** sets_out, int32_t** size_out) {
  if (n < 1 || k < 1) return fail(ORC_E_ARG, "'idx' must have at least one row and column.");
  const int64_t N = n, S = (int64_t)k + 1;
  for (int32_t t = 0; t < k; ++t)
    for (int32_t i = 0; i < n; ++i) {
      const int32_t v = idx[i + N * t];
      if (v != NA_INT && (v < 1 || v > n))
        return fail(ORC_E_INDEX,
                    "'idx' entries must be NA or 1-based row indices in [1, nrow(idx)].");
    }
  int32_t* sets = malloc(sizeof(int32_t) * (size_t)(N * S));
  int32_t* size = malloc(sizeof(int32_t) * (size_t)N);
  if (!sets || !size) { free(sets); free(size); return fail(ORC_E_NOMEM, "out of memory"); }
  for (int32_t i = 0; i < n; ++i) {
    int32_t* s = sets + (int64_t)i * S;
    int32_t c = 0;
    if (include_self) s[c++] = i;
    for (int32_t t = 0; t < k; ++t) {
      const int32_t v = idx[i + N * t];
      if (v == NA_INT) continue;
      if (v - 1 != i) s[c++] = v - 1;
    }
    qsort(s, (size_t)c, sizeof(int32_t), cmp_int);
    int32_t u = 0;
    for (int32_t a = 0; a < c; ++a)
      if (u == 0 || s[u - 1] != s[a]) s[u++] = s[a];
    size[i] = u;
  }
  *sets_out = sets;
  *size_out = size;
  return ORC_OK;
}

int orc_snn_shared(const int32_t* idx, int32_t n, int32_t k, int include_self, double prune,
                   int64_t* m_out, int32_t* ti, int32_t* tj, double* tx) {
  int32_t *sets = NULL, *size = NULL;
  int st = shared_sets(idx, n, k, include_self, &sets, &size);
  if (st != ORC_OK) return st;
  const int64_t N = n, S = (int64_t)k + 1;
  /* inverted index R(m) = { i : m in N(i) } as CSR; filled in i order, so
   * every R(m) is ascending (:319-339) */
  int64_t* rp = calloc((size_t)N + 1, sizeof(int64_t));
  int64_t tot = 0;
  for (int32_t i = 0; i < n; ++i) tot += size[i];
  int32_t* ri = malloc(sizeof(int32_t) * (size_t)(tot + 1));
  int64_t* fill = malloc(sizeof(int64_t) * (size_t)(N + 1));
  int32_t* acc = calloc((size_t)N, sizeof(int32_t));
  int32_t* touched = malloc(sizeof(int32_t) * (size_t)N);
  if (!rp || !ri || !fill || !acc || !touched) {
    free(rp); free(ri); free(fill); free(acc); free(touched); free(sets); free(size);
    return fail(ORC_E_NOMEM, "out of memory");
  }
  for (int32_t i = 0; i < n; ++i)
    for (int32_t a = 0; a < size[i]; ++a) rp[sets[(int64_t)i * S + a] + 1] += 1;
  for (int64_t m = 0; m < N; ++m) rp[m + 1] += rp[m];
  for (int64_t m = 0; m < N; ++m) fill[m] = rp[m];
  for (int32_t i = 0; i < n; ++i)
    for (int32_t a = 0; a < size[i]; ++a) ri[fill[sets[(int64_t)i * S + a]]++] = i;
  /* rows in order; per row the pairs (i, j > i) in first-touch order
   * (accumulate_row :156-174), weights u / (ni + nj - u) (:179-181), kept
   * when w > prune, 1-based */
  int64_t m_count = 0;
  for (int32_t i = 0; i < n; ++i) {
    const int32_t* si = sets + (int64_t)i * S;
    if (size[i] == 0) continue;
    int64_t nt = 0;
    for (int32_t a = 0; a < size[i]; ++a) {
      const int32_t mm = si[a];
      int64_t lo = rp[mm], hi = rp[mm + 1];
      while (lo < hi) { const int64_t mid = (lo + hi) / 2; if (ri[mid] <= i) lo = mid + 1; else hi = mid; }
      for (int64_t q = lo; q < rp[mm + 1]; ++q) {
        const int32_t j = ri[q];
        if (acc[j]++ == 0) touched[nt++] = j;
      }
    }
    for (int64_t a = 0; a < nt; ++a) {
      const int32_t j = touched[a];
      const int64_t u = acc[j];
      const double w = (double)u / (double)((int64_t)size[i] + size[j] - u);
      if (w > prune) {
        if (ti) { ti[m_count] = i + 1; tj[m_count] = j + 1; tx[m_count] = w; }
        ++m_count;
      }
      acc[j] = 0;
    }
  }
  *m_out = m_count;
  free(rp); free(ri); free(fill); free(acc); free(touched); free(sets); free(size);
  return ORC_OK;
}

/* sparseMatrix(i, j, x, symmetric = TRUE) of the upper-triangle triplets,
 * then as(generalMatrix) / CsparseMatrix: every (i, j, w) stored at (i, j)
 * and (j, i); no pair repeats and i != j, so there are no duplicates. */
int orc_snn_graph_shared_with(orc_shared_fn f, const int32_t* idx, int32_t n, int32_t k,
                              int include_self, double prune, int64_t* nnz_out, int32_t* out_p,
                              int32_t* out_i, double* out_x) {
  int64_t m = 0;
  int st = f(idx, n, k, include_self, prune, &m, NULL, NULL, NULL);
  if (st != ORC_OK) return st;
  *nnz_out = 2 * m;
  if (!out_p) return ORC_OK;
  const int64_t N = n;
  int32_t* ti = malloc(sizeof(int32_t) * (size_t)(m + 1));
  int32_t* tj = malloc(sizeof(int32_t) * (size_t)(m + 1));
  double* tx = malloc(sizeof(double) * (size_t)(m + 1));
  trip* e = malloc(sizeof(trip) * (size_t)(2 * m + 1));
  if (!ti || !tj || !tx || !e) { free(ti); free(tj); free(tx); free(e); return fail(ORC_E_NOMEM, "out of memory"); }
  int64_t m2 = 0;
  st = f(idx, n, k, include_self, prune, &m2, ti, tj, tx);
  if (st != ORC_OK || m2 != m) { free(ti); free(tj); free(tx); free(e); return st != ORC_OK ? st : fail(ORC_E_ARG, "inconsistent edge count"); }
  for (int64_t a = 0; a < m; ++a) {
    const int64_t i = ti[a] - 1, j = tj[a] - 1;
    e[2 * a].key = j * N + i; e[2 * a].ord = 0; e[2 * a].x = tx[a];          /* (i, j): column j */
    e[2 * a + 1].key = i * N + j; e[2 * a + 1].ord = 0; e[2 * a + 1].x = tx[a];  /* (j, i): column i */
  }
  qsort(e, (size_t)(2 * m), sizeof(trip), cmp_trip);
  for (int64_t c = 0; c <= N; ++c) out_p[c] = 0;
  for (int64_t a = 0; a < 2 * m; ++a) out_p[e[a].key / N + 1] += 1;
  for (int64_t c = 0; c < N; ++c) out_p[c + 1] += out_p[c];
  for (int64_t a = 0; a < 2 * m; ++a) { out_i[a] = (int32_t)(e[a].key % N); out_x[a] = e[a].x; }
  free(ti); free(tj); free(tx); free(e);
  return ORC_OK;
}

int orc_snn_graph_shared(const int32_t* idx, int32_t n, int32_t k, int include_self, double prune,
                         int64_t* nnz_out, int32_t* out_p, int32_t* out_i, double* out_x) {
  return orc_snn_graph_shared_with(orc_snn_shared, idx, n, k, include_self, prune, nnz_out, out_p,
                                   out_i, out_x);
}
