// sdg_exact.cu -- exact FP64 column-pair values, in the reference's order.
//
// Compiled with -fmad=false and written with __dadd_rn / __dmul_rn: no
// multiply-add is ever fused, so each value is the IEEE double the reference
// computes (sequential sums in ascending row order).  These kernels produce
// every distance this library returns; the FP32 screen only decides which
// pairs need one.
#include <cmath>

#include "sdg_kernels.h"
#include "sdg_topk.cuh"

namespace sdg {
namespace {

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// ---- per-column preparation -------------------------------------------------

// R/sparseKNN.R:214-220: colSums(abs(M)) == 0 with NA treated as non-empty.
__global__ void k_col_empty(DevCsc M, uint8_t* empty) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= M.ncol) return;
  uint8_t e = 1;
  for (int64_t a = M.p[j]; a < M.p[j + 1]; ++a)
    if (!(M.x[a] == 0.0)) { e = 0; break; }
  empty[j] = e;
}

// unit_csc: src/sparseDist.cpp:246-284, the dnrm2-style recurrence
//   if (scale < a) { r = scale / a; ssq = 1 + ssq * r * r; scale = a; }
//   else           { r = a / scale; ssq += r * r; }
// over the non-zero entries, then u = (x / scale) / sqrt(ssq).  One warp per
// column: the running scale is a prefix maximum, so every ratio r (and its
// branch) is computed in parallel; only the sum-of-squares update is a serial
// chain, run by lane 0 in the reference's order and expression form, so the
// result is bit-identical to the reference's sequential loop.
__global__ void k_unit_csc_warp(DevCsc M, double* uval, double* scale_out, int* err) {
  __shared__ double s_r[8][32];
  __shared__ int s_f[8][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j = blockIdx.x * (int64_t)(blockDim.x >> 5) + warp;
  if (j >= M.ncol) return;
  const int64_t a0 = M.p[j], a1 = M.p[j + 1];
  double scale = 0.0, ssq = 1.0;
  bool bad = false;
  for (int64_t c0 = a0; c0 < a1; c0 += 32) {
    const int64_t a = c0 + lane;
    double av = 0.0;
    bool nz = false;
    if (a < a1) {
      const double v = M.x[a];
      if (!isfinite(v)) bad = true;
      nz = (v != 0.0);
      av = fabs(v);
    }
    // exclusive prefix max of the magnitudes (scale before this element)
    double incl = nz ? av : 0.0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl = fmax(incl, y);
    }
    double prev = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) prev = 0.0;
    prev = fmax(prev, scale);
    int flag = 0;                  // 0: skip (zero), 1: new maximum, 2: below maximum
    double r = 0.0;
    if (nz) {
      if (prev < av) { flag = 1; r = prev / av; }
      else { flag = 2; r = av / prev; }
    }
    s_r[warp][lane] = r;
    s_f[warp][lane] = flag;
    __syncwarp();
    if (lane == 0) {
      const int n = (int)((a1 - c0) < 32 ? (a1 - c0) : 32);
      for (int t = 0; t < n; ++t) {
        const int f = s_f[warp][t];
        const double rr = s_r[warp][t];
        if (f == 1) ssq = dadd(1.0, dmul(dmul(ssq, rr), rr));
        else if (f == 2) ssq = dadd(ssq, dmul(rr, rr));
      }
    }
    __syncwarp();
    scale = fmax(scale, __shfl_sync(0xffffffffu, incl, 31));
  }
  if (__any_sync(0xffffffffu, bad)) { if (lane == 0) atomicOr(err, 1); return; }
  ssq = __shfl_sync(0xffffffffu, ssq, 0);
  const double sq = sqrt(ssq);
  if (lane == 0) scale_out[j] = scale;
  for (int64_t a = a0 + lane; a < a1; a += 32)
    uval[a] = (scale == 0.0) ? 0.0 : ((M.x[a]) / scale) / sq;
}

// unit_csc of dense columns (d values each, zeros included and skipped as
// above): the same recurrence, ratios and branches, with the serial part
// spread over columns instead of run by one lane.  A warp owns 32 columns;
// for each 32-row chunk it computes every column's ratios and flags with the
// lanes over the rows (prefix maximum of the magnitudes on their bit
// patterns, which order non-negative doubles as integers), parks them in
// shared memory, and then lane c runs column c's sum-of-squares chain over
// the chunk in the reference's order.  The FP64 pipe issues one instruction
// for cpw columns' chain steps instead of one per step; cpw (columns per
// warp, <= 32) trades that against the number of warps for small n.
constexpr int UD_WARPS = 2;

__global__ void __launch_bounds__(UD_WARPS * 32) k_unit_dense(int32_t d, int64_t n, int cpw, const double* x,
                                                              double* uval, double* scale_out, int* err) {
  __shared__ double s_r[UD_WARPS][32][33];
  __shared__ uint8_t s_f[UD_WARPS][32][33];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t j0 = ((int64_t)blockIdx.x * UD_WARPS + warp) * cpw;
  if (j0 >= n) return;
  const int nc = (int)((n - j0) < cpw ? (n - j0) : cpw);
  long long scale_bits = 0;        // lane c: column c's running maximum magnitude (bits)
  double ssq = 1.0;                // lane c: column c's sum of squares
  bool bad = false;
  for (int32_t k0 = 0; k0 < d; k0 += 32) {
    const int kn = (d - k0) < 32 ? (d - k0) : 32;
    for (int c = 0; c < nc; ++c) {
      long long ab = 0;
      if (lane < kn) {
        const long long b = __double_as_longlong(x[(j0 + c) * d + k0 + lane]);
        ab = b & 0x7fffffffffffffffLL;
        if ((ab >> 52) == 0x7ff) bad = true;        // reported for the whole call below
      }
      long long incl = ab;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl = incl > y ? incl : y;
      }
      long long prev = __shfl_up_sync(0xffffffffu, incl, 1);
      if (lane == 0) prev = 0;
      const long long sc = __shfl_sync(0xffffffffu, scale_bits, c);
      prev = prev > sc ? prev : sc;
      uint8_t flag = 0;              // 0: skip (zero), 1: new maximum, 2: below maximum
      double r = 0.0;
      if (ab != 0) {
        const double av = __longlong_as_double(ab), pv = __longlong_as_double(prev);
        if (prev < ab) { flag = 1; r = pv / av; }
        else { flag = 2; r = av / pv; }
      }
      s_r[warp][lane][c] = r;
      s_f[warp][lane][c] = flag;
      const long long tot = __shfl_sync(0xffffffffu, incl, 31);
      if (lane == c && tot > scale_bits) scale_bits = tot;
    }
    __syncwarp();
    if (lane < nc) {
      for (int t = 0; t < kn; ++t) {
        const uint8_t f = s_f[warp][t][lane];
        const double rr = s_r[warp][t][lane];
        if (f == 1) ssq = dadd(1.0, dmul(dmul(ssq, rr), rr));
        else if (f == 2) ssq = dadd(ssq, dmul(rr, rr));
      }
    }
    __syncwarp();
  }
  if (__any_sync(0xffffffffu, bad)) { if (lane == 0) atomicOr(err, 1); return; }
  const double sq = sqrt(ssq);
  if (lane < nc) scale_out[j0 + lane] = __longlong_as_double(scale_bits);
  for (int c = 0; c < nc; ++c) {
    const double scale = __longlong_as_double(__shfl_sync(0xffffffffu, scale_bits, c));
    const double q = __shfl_sync(0xffffffffu, sq, c);
    for (int32_t a = lane; a < d; a += 32) {
      const int64_t at = (j0 + c) * d + a;
      uval[at] = (scale == 0.0) ? 0.0 : (x[at] / scale) / q;
    }
  }
}

__global__ void k_moments(DevCsc M, double* sum, double* sumsq) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= M.ncol) return;
  double s = 0.0, ss = 0.0;
  for (int64_t a = M.p[j]; a < M.p[j + 1]; ++a) {
    const double v = M.x[a];
    s = dadd(s, v);
    ss = dadd(ss, dmul(v, v));
  }
  sum[j] = s;
  sumsq[j] = ss;
}

// fastJS2 input check: src/sparseDist.cpp:1077-1081.
__global__ void k_check_js(const double* x, int64_t nnz, int* err) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nnz;
       a += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[a];
    if (!isfinite(v) || v < 0.0) { atomicOr(err, 1); return; }
  }
}

// ---- exact pair values ---------------------------------------------------------

// jacc_value from the two columns' stored counts and the common count
__device__ __forceinline__ double binary_finish(double ni, double nj, int64_t common, bool dist) {
  const double c = (double)common;
  const double denom = dsub(dadd(ni, nj), c);
  const double sim = (denom > 0.0) ? (c / denom) : 1.0;
  return dist ? dsub(1.0, sim) : sim;
}

// jacc_common / jacc_value: src/sparseDist.cpp:535-556
__device__ double pair_binary(const DevCsc& A, int32_t i, const DevCsc& B, int32_t j, bool dist) {
  int64_t a = A.p[i], ae = A.p[i + 1], b = B.p[j], be = B.p[j + 1];
  const double ni = (double)(ae - a), nj = (double)(be - b);
  int64_t common = 0;
  while (a < ae && b < be) {
    const int32_t ra = __ldg(A.i + a), rb = __ldg(B.i + b);
    common += (ra == rb);
    a += (ra <= rb);
    b += (rb <= ra);
  }
  return binary_finish(ni, nj, common, dist);
}

// unit_cosine's clamp of the unit dot product s (NaN -> 0)
__device__ __forceinline__ double cosine_finish(double s, bool dist) {
  double c = s;
  if (!(c == c)) c = 0.0;
  else if (c > 1.0) c = 1.0;
  else if (c < -1.0) c = -1.0;
  return dist ? dsub(1.0, c) : c;
}

// unit_dot / unit_cosine: src/sparseDist.cpp:287-331
__device__ double pair_cosine(const DevCsc& A, const ColAux& aa, int32_t i, const DevCsc& B,
                              const ColAux& ba, int32_t j, bool dist) {
  const bool ea = (aa.scale[i] == 0.0), eb = (ba.scale[j] == 0.0);
  if (ea || eb) {
    const double c = (ea && eb) ? 1.0 : 0.0;
    return dist ? dsub(1.0, c) : c;
  }
  int64_t a = A.p[i], ae = A.p[i + 1], b = B.p[j], be = B.p[j + 1];
  double s = 0.0;
  while (a < ae && b < be) {
    const int32_t ra = __ldg(A.i + a), rb = __ldg(B.i + b);
    if (ra == rb) { s = dadd(s, dmul(aa.uval[a], ba.uval[b])); ++a; ++b; }
    else if (ra < rb) { ++a; }
    else { ++b; }
  }
  return cosine_finish(s, dist);
}

// fastEuclidean2 pair loop: src/sparseDist.cpp:855-871
__device__ double pair_euclidean(const DevCsc& A, int32_t i, const DevCsc& B, int32_t j) {
  int64_t a = A.p[i], ae = A.p[i + 1], b = B.p[j], be = B.p[j + 1];
  double num = 0.0;
  while (a < ae && b < be) {
    const int32_t ra = __ldg(A.i + a), rb = __ldg(B.i + b);
    if (ra == rb) {
      const double diff = dsub(A.x[a], B.x[b]); num = dadd(num, dmul(diff, diff)); ++a; ++b;
    } else if (ra < rb) {
      num = dadd(num, dmul(A.x[a], A.x[a])); ++a;
    } else {
      num = dadd(num, dmul(B.x[b], B.x[b])); ++b;
    }
  }
  for (; a < ae; ++a) num = dadd(num, dmul(A.x[a], A.x[a]));
  for (; b < be; ++b) num = dadd(num, dmul(B.x[b], B.x[b]));
  return sqrt(num);
}

// fastManhattan2 pair loop: src/sparseDist.cpp:755-772
__device__ double pair_manhattan(const DevCsc& A, int32_t i, const DevCsc& B, int32_t j) {
  int64_t a = A.p[i], ae = A.p[i + 1], b = B.p[j], be = B.p[j + 1];
  double num = 0.0;
  while (a < ae && b < be) {
    const int32_t ra = __ldg(A.i + a), rb = __ldg(B.i + b);
    if (ra == rb) { num = dadd(num, fabs(dsub(A.x[a], B.x[b]))); ++a; ++b; }
    else if (ra < rb) { num = dadd(num, fabs(A.x[a])); ++a; }
    else { num = dadd(num, fabs(B.x[b])); ++b; }
  }
  for (; a < ae; ++a) num = dadd(num, fabs(A.x[a]));
  for (; b < be; ++b) num = dadd(num, fabs(B.x[b]));
  return num;
}

// arma::cor's single-pass form from the matched-product sum sab and the
// columns' moments
__device__ __forceinline__ double pearson_finish(double sab, int32_t nrow, const ColAux& aa, int32_t i,
                                                 const ColAux& ba, int32_t j, bool dist) {
  const double N = (double)nrow;
  const double norm = (nrow > 1) ? dsub(N, 1.0) : 1.0;
  const double cov = dsub(sab, dmul(aa.s[i], ba.s[j]) / N) / norm;
  const double va = dsub(aa.ss[i], dmul(aa.s[i], aa.s[i]) / N) / norm;
  const double vb = dsub(ba.ss[j], dmul(ba.s[j], ba.s[j]) / N) / norm;
  double c = cov / dmul(sqrt(va), sqrt(vb));
  if (!isfinite(c)) c = 0.0;
  if (c > 1.0) c = 1.0;
  if (c < -1.0) c = -1.0;
  return dist ? dsub(1.0, c) : c;
}

// fastCorr2 (src/sparseDist.cpp:424-431) with arma::cor in the single-pass
// vector form: sums in ascending row order over stored entries.
__device__ double pair_pearson(const DevCsc& A, const ColAux& aa, int32_t i, const DevCsc& B,
                               const ColAux& ba, int32_t j, bool dist) {
  int64_t a = A.p[i], ae = A.p[i + 1], b = B.p[j], be = B.p[j + 1];
  double sab = 0.0;
  while (a < ae && b < be) {
    const int32_t ra = __ldg(A.i + a), rb = __ldg(B.i + b);
    if (ra == rb) { sab = dadd(sab, dmul(A.x[a], B.x[b])); ++a; ++b; }
    else if (ra < rb) { ++a; }
    else { ++b; }
  }
  return pearson_finish(sab, A.nrow, aa, i, ba, j, dist);
}

// fastJS2 (src/sparseDist.cpp:1099-1108, xlogx :206-210): per row
// ((xlogx(P)+xlogx(Q)) - xlogx(P+Q)) + (P+Q)*log 2, summed into an even-row and
// an odd-row accumulator; rows where P and Q are both 0 add +0 and are skipped.
__device__ __forceinline__ double xlogx(double x) {
  const double r = dmul(x, log(x));
  return isnan(r) ? 0.0 : r;
}

__device__ __forceinline__ double covariance_finish(double sab, int32_t nrow, const ColAux& aa, int32_t i,
                                                    const ColAux& ba, int32_t j) {
  const double N = (double)nrow;
  const double norm = (nrow > 1) ? dsub(N, 1.0) : 1.0;
  return dsub(sab, dmul(aa.s[i], ba.s[j]) / N) / norm;
}

// covariance: fastCov2, src/sparseDist.cpp:480-510 -- arma::cov of the two
// columns in the single-pass form used for pearson: (sum(ab) - sum(a) sum(b)
// / N) / (N - 1), the matched products summed in ascending row order; no clamp
__device__ double pair_covariance(const DevCsc& A, const ColAux& aa, int32_t i, const DevCsc& B,
                                  const ColAux& ba, int32_t j) {
  int64_t a = A.p[i], ae = A.p[i + 1], b = B.p[j], be = B.p[j + 1];
  double sab = 0.0;
  while (a < ae && b < be) {
    const int32_t ra = __ldg(A.i + a), rb = __ldg(B.i + b);
    if (ra == rb) { sab = dadd(sab, dmul(A.x[a], B.x[b])); ++a; ++b; }
    else if (ra < rb) { ++a; }
    else { ++b; }
  }
  return covariance_finish(sab, A.nrow, aa, i, ba, j);
}

// A row stored in one column only (Q = 0) contributes exactly P log 2: xlogx(0)
// is 0, P + 0 is P, and (xlogx(P) + 0) - xlogx(P) is +0, so no logarithm is
// taken there; a shared row takes xlogx(P), xlogx(Q) from the columns'
// precomputed values (ColAux::xl, the same function of the same double) and
// one logarithm for xlogx(P + Q).  The terms and their order of summation
// are the formula's above: pair_js_walk evaluates every stored row.
__device__ double pair_js_walk(const DevCsc& A, const ColAux& aa, int32_t i, const DevCsc& B, const ColAux& ba,
                               int32_t j) {
  const double log2v = 0.69314718055994530942;   // log(2.0), correctly rounded
  int64_t a = A.p[i], ae = A.p[i + 1], b = B.p[j], be = B.p[j + 1];
  double acc0 = 0.0, acc1 = 0.0;
  while (a < ae || b < be) {
    const int32_t ra = (a < ae) ? __ldg(A.i + a) : INT32_MAX;
    const int32_t rb = (b < be) ? __ldg(B.i + b) : INT32_MAX;
    int32_t r;
    double t;
    if (ra < rb) {
      r = ra; t = dmul(A.x[a], log2v); ++a;
    } else if (rb < ra) {
      r = rb; t = dmul(B.x[b], log2v); ++b;
    } else {
      r = ra;
      const double P = A.x[a], Q = B.x[b];
      const double xp = aa.xl ? aa.xl[a] : xlogx(P), xq = ba.xl ? ba.xl[b] : xlogx(Q);
      const double PQ = dadd(P, Q);
      t = dadd(dsub(dadd(xp, xq), xlogx(PQ)), dmul(PQ, log2v));
      ++a; ++b;
    }
    if (r & 1) acc1 = dadd(acc1, t); else acc0 = dadd(acc0, t);
  }
  const double v = dmul(0.5, dadd(acc0, acc1));
  return (v > 0.0) ? sqrt(v) : 0.0;
}

// fastJS2's value with the rows stored in one column only summed in bulk.
// Every row's term is >= 0 (P log 2 for a one-sided row; (P + Q) log 2 minus
// g(P, Q) = xlogx(P + Q) - xlogx(P) - xlogx(Q) <= (P + Q) log 2 for a shared
// one), so the order of summation moves the result by a few units of 2^-53 of
// it.  The one-sided rows add log 2 times the columns' one-sided masses,
// S_P - (shared P) and S_Q - (shared Q) from the columns' sums: the walk
// touches only the shared rows' values.  The difference is taken only when
// each one-sided mass is at least half its column's sum (then its relative
// error is below ~2e-13); a pair sharing most of its mass is walked in full.
// The value is fastJS2's within 1e-12 relative (the reference sums with
// Armadillo's accu, whose order is not pinned either).
// The bulk form's value from the column sums SA, SB, the shared rows' value
// sums sp, sq and their terms' sum; false when a one-sided mass is below half
// its column's sum (the caller then walks the pair in full).
__device__ __forceinline__ bool js_bulk(double SA, double SB, double sp, double sq, double shared, double* out) {
  const double log2v = 0.69314718055994530942;
  const double oa = dsub(SA, sp), ob = dsub(SB, sq);
  if (!(oa >= 0.5 * SA) || !(ob >= 0.5 * SB)) return false;
  const double v = dmul(0.5, dadd(dmul(dadd(oa, ob), log2v), shared));
  *out = (v > 0.0) ? sqrt(v) : 0.0;
  return true;
}
// the term of a row stored in both columns (P, Q and their xlogx values)
__device__ __forceinline__ double js_shared_term(double P, double Q, double xp, double xq) {
  const double log2v = 0.69314718055994530942;
  const double PQ = dadd(P, Q);
  return dadd(dsub(dadd(xp, xq), xlogx(PQ)), dmul(PQ, log2v));
}

__device__ double pair_js(const DevCsc& A, const ColAux& aa, int32_t i, const DevCsc& B, const ColAux& ba,
                          int32_t j) {
  if (!aa.xsum || !ba.xsum || !aa.xl || !ba.xl) return pair_js_walk(A, aa, i, B, ba, j);
  int64_t a = A.p[i], ae = A.p[i + 1], b = B.p[j], be = B.p[j + 1];
  double shared = 0.0, sp = 0.0, sq = 0.0;
  while (a < ae && b < be) {
    const int32_t ra = __ldg(A.i + a), rb = __ldg(B.i + b);
    if (ra == rb) {
      const double P = A.x[a], Q = B.x[b];
      shared = dadd(shared, js_shared_term(P, Q, aa.xl[a], ba.xl[b]));
      sp = dadd(sp, P);
      sq = dadd(sq, Q);
      ++a; ++b;
    } else {
      a += (ra < rb);
      b += (rb < ra);
    }
  }
  double v;
  if (!js_bulk(aa.xsum[i], ba.xsum[j], sp, sq, shared, &v)) return pair_js_walk(A, aa, i, B, ba, j);
  return v;
}

// xlogx of each stored value (the per-entry half of pair_js's shared rows)
__global__ void k_xlogx_values(const double* x, int64_t nnz, double* xl) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nnz; a += (int64_t)gridDim.x * blockDim.x)
    xl[a] = xlogx(x[a]);
}

__device__ __forceinline__ double pair_value(int method, bool dist, const DevCsc& A,
                                             const ColAux& aa, int32_t i, const DevCsc& B,
                                             const ColAux& ba, int32_t j) {
  switch (method) {
    case BINARY: return pair_binary(A, i, B, j, dist);
    case COSINE: return pair_cosine(A, aa, i, B, ba, j, dist);
    case EUCLIDEAN: return pair_euclidean(A, i, B, j);
    case MANHATTAN: return pair_manhattan(A, i, B, j);
    case PEARSON: return pair_pearson(A, aa, i, B, ba, j, dist);
    case COVARIANCE: return pair_covariance(A, aa, i, B, ba, j);
    default: return pair_js(A, aa, i, B, ba, j);
  }
}

// ---- the query column as a row lookup -----------------------------------------
//
// For the match-only methods (binary, cosine, pearson, covariance) and js's
// bulk form, a pair's value needs only the rows stored in both columns, in
// ascending row order.  With the query column held in shared memory as a row
// lookup -- bit r % 32 of bits[r / 32] set when row r is stored, base[w] the
// position in the column of the first stored row of word w (read only for
// words that hold one) -- a thread walks its reference column alone: every
// stored row is tested with one shared-memory load, no load's address waits
// on a comparison (the merge walk's serial dependence), and the matched rows
// come in the same ascending order as in the merge walk, so every sum is the
// same sequence of operations and the values are the merge walk's bit for bit.
constexpr int32_t LOOKUP_MAX_ROWS = 32768;

__host__ __device__ __forceinline__ bool lookup_method(int method) {
  return method == BINARY || method == COSINE || method == PEARSON || method == COVARIANCE || method == JS;
}

// The lookup of column q, built by the threads t = 0 .. nt - 1 of the calling
// group (a warp or a block): first lookup_clear, then (after the group
// synchronises) lookup_fill, then the group synchronises again.
__device__ __forceinline__ void lookup_clear(uint32_t* bits, int32_t nrow, int t, int nt) {
  for (int32_t w = t; w < ((nrow + 31) >> 5); w += nt) bits[w] = 0u;
}
__device__ __forceinline__ void lookup_fill(const DevCsc& Q, int32_t q, uint32_t* bits, int32_t* base, int t,
                                            int nt) {
  const int64_t b0 = Q.p[q], b1 = Q.p[q + 1];
  for (int64_t b = b0 + t; b < b1; b += nt) {
    const int32_t row = __ldg(Q.i + b);
    atomicOr(bits + (row >> 5), 1u << (row & 31));
    if (b == b0 || (__ldg(Q.i + b - 1) >> 5) != (row >> 5)) base[row >> 5] = (int32_t)(b - b0);
  }
}

// pair_value(method, dist, R, ra, r, Q, qa, q) for a lookup method, with
// column q of Q given as its lookup.
__device__ double pair_value_lookup(int method, bool dist, const DevCsc& R, const ColAux& ra, int32_t r,
                                    const DevCsc& Q, const ColAux& qa, int32_t q, const uint32_t* bits,
                                    const int32_t* base) {
  const int64_t a0 = R.p[r], a1 = R.p[r + 1], qb = Q.p[q];
  switch (method) {
    case BINARY: {
      int64_t common = 0;
      for (int64_t a = a0; a < a1; ++a) {
        const int32_t row = __ldg(R.i + a);
        common += (bits[row >> 5] >> (row & 31)) & 1u;
      }
      return binary_finish((double)(a1 - a0), (double)(Q.p[q + 1] - qb), common, dist);
    }
    case COSINE: {
      const bool ea = (ra.scale[r] == 0.0), eb = (qa.scale[q] == 0.0);
      if (ea || eb) {
        const double c = (ea && eb) ? 1.0 : 0.0;
        return dist ? dsub(1.0, c) : c;
      }
      double sum = 0.0;
      for (int64_t a = a0; a < a1; ++a) {
        const int32_t row = __ldg(R.i + a);
        const uint32_t w = bits[row >> 5];
        if ((w >> (row & 31)) & 1u) {
          const int64_t b = qb + base[row >> 5] + __popc(w & ((1u << (row & 31)) - 1u));
          sum = dadd(sum, dmul(ra.uval[a], qa.uval[b]));
        }
      }
      return cosine_finish(sum, dist);
    }
    case PEARSON:
    case COVARIANCE: {
      double sab = 0.0;
      for (int64_t a = a0; a < a1; ++a) {
        const int32_t row = __ldg(R.i + a);
        const uint32_t w = bits[row >> 5];
        if ((w >> (row & 31)) & 1u) {
          const int64_t b = qb + base[row >> 5] + __popc(w & ((1u << (row & 31)) - 1u));
          sab = dadd(sab, dmul(R.x[a], Q.x[b]));
        }
      }
      return method == PEARSON ? pearson_finish(sab, R.nrow, ra, r, qa, q, dist)
                               : covariance_finish(sab, R.nrow, ra, r, qa, q);
    }
    case JS: {
      if (!ra.xsum || !qa.xsum || !ra.xl || !qa.xl) return pair_js_walk(R, ra, r, Q, qa, q);
      double shared = 0.0, sp = 0.0, sq = 0.0;
      for (int64_t a = a0; a < a1; ++a) {
        const int32_t row = __ldg(R.i + a);
        const uint32_t w = bits[row >> 5];
        if ((w >> (row & 31)) & 1u) {
          const int64_t b = qb + base[row >> 5] + __popc(w & ((1u << (row & 31)) - 1u));
          const double P = R.x[a], Qv = Q.x[b];
          shared = dadd(shared, js_shared_term(P, Qv, ra.xl[a], qa.xl[b]));
          sp = dadd(sp, P);
          sq = dadd(sq, Qv);
        }
      }
      double v;
      if (!js_bulk(ra.xsum[r], qa.xsum[q], sp, sq, shared, &v)) return pair_js_walk(R, ra, r, Q, qa, q);
      return v;
    }
    default:
      return pair_value(method, dist, R, ra, r, Q, qa, q);
  }
}

// One query column per blockIdx.y, one reference column per thread.  With
// `lookup` (a lookup method and nrow <= LOOKUP_MAX_ROWS) the block first holds
// its query column as a row lookup in dynamic shared memory.
__global__ void k_exact_slab(int method, int dist, DevCsc ref, ColAux ra, DevCsc qry, ColAux qa,
                             int64_t q0, const uint8_t* ref_mask, int restore_self,
                             double self_value, double* D, int lookup) {
  extern __shared__ uint32_t lk_bits[];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t b = blockIdx.y;
  const int64_t q = q0 + b;
  const int32_t words = (qry.nrow + 31) >> 5;
  int32_t* lk_base = reinterpret_cast<int32_t*>(lk_bits + words);
  if (lookup) {
    lookup_clear(lk_bits, qry.nrow, threadIdx.x, blockDim.x);
    __syncthreads();
    lookup_fill(qry, (int32_t)q, lk_bits, lk_base, threadIdx.x, blockDim.x);
    __syncthreads();
  }
  if (i >= ref.ncol) return;
  double v;
  if (ref_mask && ref_mask[i]) v = na_real();
  else if (restore_self && i == q) v = self_value;
  else if (lookup) v = pair_value_lookup(method, dist != 0, ref, ra, (int32_t)i, qry, qa, (int32_t)q, lk_bits, lk_base);
  else v = pair_value(method, dist != 0, ref, ra, (int32_t)i, qry, qa, (int32_t)q);
  D[b * (int64_t)ref.ncol + i] = v;
}

// Single-matrix form (src/sparseDist.cpp fastJacc :620-680, fastCosine
// :918-960, fastEuclidean :786-830, fastManhattan :688-731, fastCorr
// :339-398, fastCov :450-478, fastJS :1021-1071): entry (r, c) of the n x n
// result holds the pair (min(r, c), max(r, c)) in the reference's i <= j
// orientation.  The lower triangle (r > c) is always computed; the upper one
// only with `upper` (else it is written 0: unwritten, or mirrored later).
// The diagonal follows each kernel: a unit / zero self value for binary,
// cosine and pearson; the computed self pair for euclidean, manhattan and
// covariance only with `diag`; always 0 for js.
__global__ void k_self_slab(int method, int dist, DevCsc m, ColAux a, int64_t c0, int upper,
                            int diag, double* D) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t b = blockIdx.y;
  if (r >= m.ncol) return;
  const int64_t c = c0 + b;
  double v = 0.0;
  if (r == c) {
    if (method == BINARY || method == COSINE || method == PEARSON) v = dist ? 0.0 : 1.0;
    else if (diag && method != JS) v = pair_value(method, dist != 0, m, a, (int32_t)r, m, a, (int32_t)r);
  } else if (r > c) {
    v = pair_value(method, dist != 0, m, a, (int32_t)c, m, a, (int32_t)r);
  } else if (upper) {
    v = pair_value(method, dist != 0, m, a, (int32_t)r, m, a, (int32_t)c);
  }
  D[b * m.ncol + r] = v;
}

// D (n x n, column-major): copies the strict lower triangle onto the upper
// one through a 32 x 32 shared-memory tile, so both the reads and the writes
// are coalesced.  Block (tx, ty) with tx > ty owns the upper tile at rows
// ty*32.., columns tx*32..; it reads the lower tile at rows tx*32..,
// columns ty*32..  Diagonal tiles (tx == ty) mirror within themselves.
__global__ void k_mirror_lower(double* D, int64_t n) {
  __shared__ double t[32][33];
  const int64_t tx = blockIdx.x, ty = blockIdx.y;
  if (tx < ty) return;
  const int64_t r0 = tx * 32, c0 = ty * 32;          // source tile (lower)
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = r0 + threadIdx.x, c = c0 + k;
    t[k][threadIdx.x] = (r < n && c < n) ? D[c * n + r] : 0.0;
  }
  __syncthreads();
  // destination: row c0 + threadIdx.x, column r0 + k holds source (r0 + k, c0 + threadIdx.x)
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = c0 + threadIdx.x, c = r0 + k;
    if (r < n && c < n && r < c) D[c * n + r] = t[threadIdx.x][k];
  }
}

// D (n x n, column-major): copies the strict upper triangle onto the lower
// one (tile transpose through shared memory, as k_mirror_lower), and with
// `clear` zeroes the upper triangle once it has been read.  Block (tx, ty),
// tx >= ty, reads the upper tile at rows ty*32.., columns tx*32.. and writes
// the lower tile at rows tx*32.., columns ty*32..; each upper tile is read
// by one block only, so the clearing races with nothing.
__global__ void k_mirror_upper(double* D, int64_t n, int clear) {
  __shared__ double t[32][33];
  const int64_t tx = blockIdx.x, ty = blockIdx.y;
  if (tx < ty) return;
  const int64_t r0 = ty * 32, c0 = tx * 32;          // source tile (upper)
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = r0 + threadIdx.x, c = c0 + k;
    t[k][threadIdx.x] = (r < n && c < n) ? D[c * n + r] : 0.0;
  }
  __syncthreads();
  // destination (c0 + threadIdx.x, r0 + k) holds source (r0 + k, c0 + threadIdx.x)
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = c0 + threadIdx.x, c = r0 + k;
    if (r < n && c < n && r > c) D[c * n + r] = t[threadIdx.x][k];
  }
  if (clear) {
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
      const int64_t r = r0 + threadIdx.x, c = c0 + k;
      if (r < n && c < n && r < c) D[c * n + r] = 0.0;
    }
  }
}

// The diagonal of the single-matrix form (the rules of k_self_slab's r == c).
__global__ void k_self_diag(int method, int dist, DevCsc m, ColAux a, int diag, double* D) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= m.ncol) return;
  double v = 0.0;
  if (method == BINARY || method == COSINE || method == PEARSON) v = dist ? 0.0 : 1.0;
  else if (diag && method != JS) v = pair_value(method, dist != 0, m, a, (int32_t)r, m, a, (int32_t)r);
  D[r * m.ncol + r] = v;
}

__global__ void k_exact_pairs(int method, int dist, DevCsc ref, ColAux ra, DevCsc qry,
                              ColAux qa, const int32_t* ref_idx, const int32_t* qry_idx,
                              int64_t npairs, double* out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= npairs) return;
  out[t] = pair_value(method, dist != 0, ref, ra, ref_idx[t], qry, qa, qry_idx[t]);
}

// Candidate pairs of the screened engine: slots with ref_idx < 0 are unused;
// with restore_self the self pair (ref == query) takes self_value.
__global__ void k_exact_pairs_sparse(int method, int dist, DevCsc ref, ColAux ra, DevCsc qry,
                                     ColAux qa, const int32_t* ref_idx, const int32_t* qry_idx,
                                     int64_t npairs, int restore_self, double self_value,
                                     double* out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= npairs) return;
  const int32_t c = ref_idx[t], q = qry_idx[t];
  if (c < 0 || q < 0) return;
  out[t] = (restore_self && c == q) ? self_value
                                    : pair_value(method, dist != 0, ref, ra, c, qry, qa, q);
}

// The value of a match-only pair from the ascending-row sum of matched
// products (`sum`) and the matched-row count (`common`): Jaccard
// (jacc_value, src/sparseDist.cpp:549-556), cosine (unit_cosine's NaN / clamp,
// src/sparseDist.cpp:326-330) or pearson (arma::cor's formulation); A / i is
// the reference column, B / j the query column.
__device__ double match_finish(int method, bool dist, double sum, int64_t common, const DevCsc& A,
                               const ColAux& aa, int32_t i, const DevCsc& B, const ColAux& ba, int32_t j) {
  if (method == BINARY) {
    const double ni = (double)(A.p[i + 1] - A.p[i]), nj = (double)(B.p[j + 1] - B.p[j]), c = (double)common;
    const double denom = dsub(dadd(ni, nj), c);
    const double sim = (denom > 0.0) ? (c / denom) : 1.0;
    return dist ? dsub(1.0, sim) : sim;
  }
  if (method == COSINE) {
    double c = sum;
    if (!(c == c)) c = 0.0;
    else if (c > 1.0) c = 1.0;
    else if (c < -1.0) c = -1.0;
    return dist ? dsub(1.0, c) : c;
  }
  const double N = (double)A.nrow;
  const double norm = (A.nrow > 1) ? dsub(N, 1.0) : 1.0;
  if (method == COVARIANCE) return dsub(sum, dmul(aa.s[i], ba.s[j]) / N) / norm;
  // pearson
  const double cov = dsub(sum, dmul(aa.s[i], ba.s[j]) / N) / norm;
  const double va = dsub(aa.ss[i], dmul(aa.s[i], aa.s[i]) / N) / norm;
  const double vb = dsub(ba.ss[j], dmul(ba.s[j], ba.s[j]) / N) / norm;
  double c = cov / dmul(sqrt(va), sqrt(vb));
  if (!isfinite(c)) c = 0.0;
  if (c > 1.0) c = 1.0;
  if (c < -1.0) c = -1.0;
  return dist ? dsub(1.0, c) : c;
}

// Match-only methods (binary, cosine, pearson): the value depends on the rows
// both columns store, summed in ascending row order.  One warp per query row
// of the candidate table: for each candidate, lanes take 32 consecutive
// entries of the shorter column and binary-search them in the longer one; the
// matched products are then added by lane 0 in ascending row order, so the sum
// is the reference's sequential sum bit for bit.
__device__ double warp_match_value(int method, bool dist, const DevCsc& A, const ColAux& aa,
                                   int32_t i, const DevCsc& B, const ColAux& ba, int32_t j,
                                   int lane) {
  const int64_t ia0 = A.p[i], ia1 = A.p[i + 1], jb0 = B.p[j], jb1 = B.p[j + 1];
  if (method == COSINE) {
    const bool ea = (aa.scale[i] == 0.0), eb = (ba.scale[j] == 0.0);
    if (ea || eb) { const double c = (ea && eb) ? 1.0 : 0.0; return dist ? dsub(1.0, c) : c; }
  }
  const bool a_short = (ia1 - ia0) <= (jb1 - jb0);
  const int32_t* si = a_short ? A.i : B.i;
  const int32_t* li = a_short ? B.i : A.i;
  const int64_t s0 = a_short ? ia0 : jb0, s1 = a_short ? ia1 : jb1;
  int64_t l0 = a_short ? jb0 : ia0;
  const int64_t l1 = a_short ? jb1 : ia1;
  const double* av = (method == COSINE) ? aa.uval : A.x;
  const double* bv = (method == COSINE) ? ba.uval : B.x;
  double sum = 0.0;
  int64_t common = 0;
  for (int64_t c0 = s0; c0 < s1 && l0 < l1; c0 += 32) {
    const int64_t s = c0 + lane;
    bool hit = false;
    double prod = 0.0;
    int64_t lb = l1;
    if (s < s1) {
      const int32_t r = __ldg(si + s);
      int64_t lo = l0, hi = l1;                        // first index with row >= r
      while (lo < hi) { const int64_t mid = (lo + hi) >> 1; if (__ldg(li + mid) < r) lo = mid + 1; else hi = mid; }
      lb = lo;
      if (lo < l1 && __ldg(li + lo) == r) {
        hit = true;
        if (method != BINARY) {
          const int64_t ea_ = a_short ? s : lo, eb_ = a_short ? lo : s;
          prod = dmul(av[ea_], bv[eb_]);
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    common += __popc(m);
    if (method != BINARY) {
      for (int t = 0; t < 32; ++t) {
        const double p = __shfl_sync(0xffffffffu, prod, t);
        if ((m >> t) & 1u) sum = dadd(sum, p);
      }
    }
    l0 = __shfl_sync(0xffffffffu, lb, 31);
  }
  return match_finish(method, dist, sum, common, A, aa, i, B, ba, j);
}

__global__ void k_rerank_warp(int method, int dist, DevCsc ref, ColAux ra, DevCsc qry, ColAux qa,
                              const int32_t* cand, const int32_t* count, int cap, int64_t nq_local,
                              int64_t q_begin, int restore_self, double self_value, double* out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = blockIdx.x * (int64_t)(blockDim.x >> 5) + warp;
  if (ql >= nq_local) return;
  const int32_t q = (int32_t)(q_begin + ql);
  const int n = count[ql];
  for (int t = 0; t < n; ++t) {
    const int32_t c = cand[ql * cap + t];
    double v;
    if (restore_self && c == q) v = self_value;
    else v = warp_match_value(method, dist != 0, ref, ra, c, qry, qa, q, lane);
    if (lane == 0) out[ql * cap + t] = v;
  }
}

// Query-centric re-rank of the match-only methods, one CTA per query row of
// the candidate table.  The query column's rows go into a shared-memory
// bitmap (bit r % 32 of word r / 32) with, for each word holding a row, the
// index of its first entry, so a matched row r is entry
// first[r / 32] + popc(word & below(r)) of the query; the query's values sit
// in shared memory too (up to RQ_MAX_QV entries, else they are read from
// global memory).  The candidates are sorted by column length (bitonic, in
// shared memory) and dealt round-robin to the warps' lanes.
//
// GB300's FP64 pipe spends the same time on an FP64 warp instruction whatever
// the number of active lanes, so the sequential sum of a pair (one dadd per
// matched row, in ascending row order, as the reference adds them) runs one
// pair per LANE.  A warp works on its 32 candidates in passes: (scan) for
// each candidate in turn, the warp streams the column 32 entries a round
// (coalesced, four rounds' loads in flight), tests the rows against the
// bitmap, multiplies the matched values (dmul, the same product the
// reference forms) and appends the products, in row order, to that
// candidate's list of RM slots until it is full or the column ends; (sum)
// lane j then adds candidate j's list in order, all lanes at once, operands
// in shared memory.  Each lane's sum is the reference's sequential sum bit for
// bit.
//
// kTri (the single-matrix sparseDist): no candidate table; CTA (x, y) takes
// column q = x of m as the query and the reference columns c = y * 2048 ..
// of m below it (c < q) as its candidates, in the reference's orientation
// (first operand c, second q), and writes the strict upper triangle entry
// out[q * ncol + c].
constexpr int RQ_THREADS = 256;
constexpr int RQ_WARPS = RQ_THREADS / 32;
constexpr int32_t RQ_MAX_NROW = 1 << 18;
constexpr int RQ_MAX_QV = 2048;
constexpr int RQ_MAX_CAND = 2048;     // candidates sorted in shared memory
constexpr int RM = 32;                // list slots per candidate per pass

template <bool kTri>
__global__ void k_rerank_q(int method, int dist, DevCsc ref, ColAux ra, DevCsc qry, ColAux qa,
                           const int32_t* cand, const int32_t* count, int cap, int64_t q_begin,
                           int restore_self, double self_value, double* out) {
  extern __shared__ __align__(16) uint32_t rq_smem[];
  const int W = (qry.nrow + 31) >> 5;
  double* qvs = reinterpret_cast<double*>(rq_smem);                          // RQ_MAX_QV
  uint64_t* order = reinterpret_cast<uint64_t*>(rq_smem + 2 * RQ_MAX_QV);    // RQ_MAX_CAND
  double* lists = reinterpret_cast<double*>(order + RQ_MAX_CAND);           // [warp][32][RM]
  uint32_t* bits = reinterpret_cast<uint32_t*>(lists + RQ_WARPS * 32 * RM);
  int32_t* first = reinterpret_cast<int32_t*>(bits + W);
  const int64_t ql = blockIdx.x;
  const int32_t q = (int32_t)(q_begin + ql);
  const int32_t cbase = kTri ? (int32_t)blockIdx.y * RQ_MAX_CAND : 0;
  const int n = kTri ? max(0, min(q - cbase, RQ_MAX_CAND)) : min(count[ql], RQ_MAX_CAND);
  if (n == 0) return;
  for (int w = threadIdx.x; w < W; w += blockDim.x) bits[w] = 0u;
  // sort keys: (column length, position in the list), longest first
  int np2 = 1;
  while (np2 < n) np2 <<= 1;
  for (int t = threadIdx.x; t < np2; t += blockDim.x) {
    uint64_t key = 0;                       // padding sorts last
    if (t < n) {
      const int32_t c = kTri ? cbase + t : cand[ql * (int64_t)cap + t];
      const int64_t len64 = ref.p[c + 1] - ref.p[c];
      const uint32_t len = (uint32_t)(len64 < 0x7fffffff ? len64 : 0x7fffffff);
      key = ((uint64_t)(len + 1u) << 32) | (uint32_t)t;
    }
    order[t] = key;
  }
  __syncthreads();
  const int64_t q0 = qry.p[q], q1 = qry.p[q + 1];
  const double* qsrc = ((method == COSINE) ? qa.uval : qry.x) + q0;
  const bool qv_shared = (q1 - q0) <= RQ_MAX_QV;
  for (int64_t e = q0 + threadIdx.x; e < q1; e += blockDim.x) {
    const int32_t r = qry.i[e];
    atomicOr(&bits[r >> 5], 1u << (r & 31));
    if (e == q0 || (qry.i[e - 1] >> 5) != (r >> 5)) first[r >> 5] = (int32_t)(e - q0);
    if (qv_shared && method != BINARY) qvs[e - q0] = qsrc[e - q0];
  }
  for (int k2 = 2; k2 <= np2; k2 <<= 1) {             // bitonic sort, descending
    for (int j = k2 >> 1; j > 0; j >>= 1) {
      __syncthreads();
      for (int t = threadIdx.x; t < np2; t += blockDim.x) {
        const int u = t ^ j;
        if (u > t) {
          const uint64_t x = order[t], y = order[u];
          const bool desc = (t & k2) == 0;
          if (desc ? (x < y) : (x > y)) { order[t] = y; order[u] = x; }
        }
      }
    }
  }
  __syncthreads();
  const double* qv = qv_shared ? qvs : qsrc;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const double* rv = (method == COSINE) ? ra.uval : ref.x;
  const bool q_empty = (method == COSINE) && qa.scale[q] == 0.0;
  double* wl = lists + warp * 32 * RM;
  for (int g = 0; g < n; g += RQ_WARPS * 32) {
    // lane j of warp w owns sorted candidate g + 8 j + w: the candidates are
    // dealt round-robin, so every warp gets work even for short lists
    const int slot = g + lane * RQ_WARPS + warp;
    const int t = (slot < n) ? (int)(uint32_t)order[slot] : -1;
    int32_t c = -1;
    double v = 0.0;
    bool special = false;
    int64_t a = 0, a_end = 0, c0 = 0;
    if (t >= 0) {
      c = kTri ? cbase + t : cand[ql * (int64_t)cap + t];
      if (restore_self && c == q) {
        v = self_value;
        special = true;
      } else if (method == COSINE && (q_empty || ra.scale[c] == 0.0)) {
        const double cv = (q_empty && ra.scale[c] == 0.0) ? 1.0 : 0.0;
        v = dist ? dsub(1.0, cv) : cv;
        special = true;
      } else {
        c0 = a = ref.p[c];
        a_end = ref.p[c + 1];
      }
    }
    bool active = (t >= 0) && !special && a < a_end;
    double sum = 0.0;
    int64_t common = 0;
    while (__any_sync(0xffffffffu, active)) {
      int my_fill = 0;
      // scan: each active candidate in turn, the whole warp on its column
      for (int j = 0; j < 32; ++j) {
        if (!__shfl_sync(0xffffffffu, active, j)) continue;
        int64_t pos = __shfl_sync(0xffffffffu, a, j);
        const int64_t end = __shfl_sync(0xffffffffu, a_end, j);
        double* lj = wl + j * RM;
        int fill = 0;
        bool full = false;
        while (pos < end && !full) {
          int32_t r[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int64_t e = pos + 32 * u + lane;
            r[u] = (e < end) ? __ldg(ref.i + e) : -1;
          }
          int qe[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            qe[u] = -1;
            if (r[u] >= 0) {
              const uint32_t wd = bits[r[u] >> 5];
              const uint32_t bit = 1u << (r[u] & 31);
              if (wd & bit) qe[u] = first[r[u] >> 5] + __popc(wd & (bit - 1u));
            }
          }
          double pv[4];
          if (method != BINARY) {
#pragma unroll
            for (int u = 0; u < 4; ++u) pv[u] = (qe[u] >= 0) ? __ldg(rv + pos + 32 * u + lane) : 0.0;
#pragma unroll
            for (int u = 0; u < 4; ++u) if (qe[u] >= 0) pv[u] = dmul(pv[u], qv[qe[u]]);
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (full || pos >= end) break;
            const bool hit = qe[u] >= 0;
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            const int cnt = __popc(m);
            if (method != BINARY) {
              if (fill + cnt > RM) { full = true; break; }
              if (hit) lj[fill + __popc(m & below)] = pv[u];
            }
            fill += cnt;
            pos += 32;
          }
        }
        if (lane == j) {
          a = pos < end ? pos : end;
          active = pos < end;
          my_fill = fill;
        }
      }
      __syncwarp();
      common += my_fill;
      // sum: lane j runs candidate j's list in order
      if (method != BINARY) {
        const int mx = __reduce_max_sync(0xffffffffu, my_fill);
        const double* ll = wl + lane * RM;
        for (int s2 = 0; s2 < mx; ++s2)
          if (s2 < my_fill) sum = dadd(sum, ll[s2]);
      }
      __syncwarp();
    }
    if (t >= 0) {
      if (!special) v = match_finish(method, dist != 0, sum, common, ref, ra, c, qry, qa, q);
      if (kTri) out[(int64_t)q * ref.ncol + c] = v;
      else out[ql * (int64_t)cap + t] = v;
    }
  }
}

inline unsigned blocks_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

// ---- batched exact kNN of many independent problems ------------------------
//
// One persistent launch serves every (problem, direction, query column,
// reference range) item of a batch: a warp takes the next item from a global
// counter, computes the exact FP64 value of each pair of its range (one pair
// per lane, the reference's arithmetic through pair_value, reference column
// first as in the slab) and keeps the item's top k under the reference's
// comparator (topk::insert_batch); the item's list goes to its partial slot.
// k_batch_merge then takes each output row's top k over its items' lists:
// the top k of a union is the top k of the parts' top k, so the rows equal
// topKBlock / topKRowsAccum over whole slabs (src/topK.cpp:104-148,
// src/topKRows.cpp:201-248).
constexpr int BATCH_WARPS = 8;

__global__ void __launch_bounds__(BATCH_WARPS * 32) k_batch_exact(const BatchProb* probs, const BatchItem* items,
                                                                  int64_t nitems, unsigned long long* counter,
                                                                  int kmax, int lwords, uint64_t* pkey,
                                                                  int32_t* pidx, double* pval) {
  extern __shared__ unsigned char bsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* lk = reinterpret_cast<uint64_t*>(bsm) + (int64_t)warp * kmax;
  double* lv = reinterpret_cast<double*>(bsm) + (int64_t)BATCH_WARPS * kmax + (int64_t)warp * kmax;
  int32_t* li = reinterpret_cast<int32_t*>(reinterpret_cast<double*>(bsm) + 2 * (int64_t)BATCH_WARPS * kmax) +
                (int64_t)warp * kmax;
  // this warp's query-column lookup (lwords words of bits, then of bases)
  uint32_t* lbits = reinterpret_cast<uint32_t*>(bsm + (size_t)BATCH_WARPS * kmax * 20) + (int64_t)warp * 2 * lwords;
  int32_t* lbase = reinterpret_cast<int32_t*>(lbits + lwords);
  int32_t held_prob = -1, held_dir = -1, held_q = -1;        // the column the lookup holds
  for (;;) {
    unsigned long long it = 0;
    if (lane == 0) it = atomicAdd(counter, 1ull);
    it = __shfl_sync(topk::FULL, it, 0);
    if (it >= (unsigned long long)nitems) break;
    const BatchItem I = items[it];
    const BatchProb& P = probs[I.prob];
    const bool fwd = I.dir == 0;
    const DevCsc R = fwd ? P.Y : P.X, Q = fwd ? P.X : P.Y;
    const ColAux ra = fwd ? P.ya : P.xa, qa = fwd ? P.xa : P.ya;
    const uint8_t* rmask = fwd ? P.ymask : P.xmask;
    const int K = fwd ? P.kf : P.kr;
    const bool dec = P.decreasing != 0;
    const bool lookup = lookup_method(P.method) && Q.nrow <= lwords * 32;
    if (lookup && (held_prob != I.prob || held_dir != I.dir || held_q != I.q)) {
      lookup_clear(lbits, Q.nrow, lane, 32);
      __syncwarp();
      lookup_fill(Q, I.q, lbits, lbase, lane, 32);
      __syncwarp();
      held_prob = I.prob; held_dir = I.dir; held_q = I.q;
    }
    int n = 0;
    for (int32_t b = I.r0; b < I.r1; b += 32) {
      const int32_t r = b + lane;
      bool ok = r < I.r1 && !(rmask && rmask[r]);
      double v = 0.0;
      if (ok) {
        v = lookup ? pair_value_lookup(P.method, P.dist != 0, R, ra, r, Q, qa, I.q, lbits, lbase)
                   : pair_value(P.method, P.dist != 0, R, ra, r, Q, qa, I.q);
        ok = isfinite(v);
      }
      topk::insert_batch(ok, ok ? order_key(v, dec) : 0, r, v, lk, li, lv, n, K, lane);
    }
    const int64_t base = I.part * (int64_t)kmax;
    for (int t = lane; t < K; t += 32) {
      pkey[base + t] = (t < n) ? lk[t] : ~0ull;
      pidx[base + t] = (t < n) ? li[t] : 0;
      pval[base + t] = (t < n) ? lv[t] : 0.0;
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(BATCH_WARPS * 32) k_batch_merge(const BatchProb* probs, const BatchRow* rows,
                                                                  int64_t nrows, int kmax, const uint64_t* pkey,
                                                                  const int32_t* pidx, const double* pval) {
  extern __shared__ unsigned char bsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t rw = (int64_t)blockIdx.x * BATCH_WARPS + warp;
  if (rw >= nrows) return;
  uint64_t* lk = reinterpret_cast<uint64_t*>(bsm) + (int64_t)warp * kmax;
  double* lv = reinterpret_cast<double*>(bsm) + (int64_t)BATCH_WARPS * kmax + (int64_t)warp * kmax;
  int32_t* li = reinterpret_cast<int32_t*>(reinterpret_cast<double*>(bsm) + 2 * (int64_t)BATCH_WARPS * kmax) +
                (int64_t)warp * kmax;
  const BatchRow W = rows[rw];
  const BatchProb& P = probs[W.prob];
  const bool fwd = W.dir == 0;
  const int K = fwd ? P.kf : P.kr;
  const int64_t ld = fwd ? P.X.ncol : P.Y.ncol;
  int32_t* oi = fwd ? P.fidx : P.ridx;
  double* ov = fwd ? P.fval : P.rval;
  const uint8_t* qmask = fwd ? P.xmask : P.ymask;
  int n = 0;
  if (!(qmask && qmask[W.q])) {
    for (int64_t part = W.part0; part < W.part0 + W.nparts; ++part) {
      for (int t0 = 0; t0 < K; t0 += 32) {
        const int t = t0 + lane;
        const uint64_t key = (t < K) ? pkey[part * kmax + t] : ~0ull;
        const bool ok = key != ~0ull;
        topk::insert_batch(ok, key, ok ? pidx[part * kmax + t] : 0, ok ? pval[part * kmax + t] : 0.0, lk, li, lv, n,
                           K, lane);
      }
    }
  }
  for (int t = lane; t < K; t += 32) {
    const int64_t at = (int64_t)t * ld + W.q;
    if (t < n) { oi[at] = li[t] + 1; ov[at] = lv[t]; }
    else       { oi[at] = NA_INT;    ov[at] = na_real(); }
  }
}

}  // namespace

void launch_col_empty(const DevCsc& M, uint8_t* empty, cudaStream_t s) {
  if (M.ncol > 0) k_col_empty<<<blocks_for(M.ncol, 256), 256, 0, s>>>(M, empty);
}
void launch_unit_csc(const DevCsc& M, double* uval, double* scale, int* err, cudaStream_t s) {
  if (M.ncol > 0) k_unit_csc_warp<<<blocks_for(M.ncol, 8), 256, 0, s>>>(M, uval, scale, err);
}
void launch_unit_dense(int32_t d, int64_t n, const double* x, double* uval, double* scale, int* err,
                       cudaStream_t s) {
  if (n <= 0) return;
  const int cpw = (n >= (int64_t)152 * 64 * 32) ? 32 : 8;   // 32 once every SM has 64 warps' worth
  const int64_t per_block = (int64_t)cpw * UD_WARPS;
  k_unit_dense<<<(unsigned)((n + per_block - 1) / per_block), UD_WARPS * 32, 0, s>>>(d, n, cpw, x, uval, scale,
                                                                                    err);
}
void launch_moments(const DevCsc& M, double* sum, double* sumsq, cudaStream_t s) {
  if (M.ncol > 0) k_moments<<<blocks_for(M.ncol, 128), 128, 0, s>>>(M, sum, sumsq);
}
void launch_xlogx_values(const double* x, int64_t nnz, double* xl, cudaStream_t s) {
  if (nnz > 0) k_xlogx_values<<<(unsigned)std::min<int64_t>((nnz + 255) / 256, 152 * 32), 256, 0, s>>>(x, nnz, xl);
}

void launch_check_js(const double* x, int64_t nnz, int* err, cudaStream_t s) {
  if (nnz > 0) {
    unsigned g = blocks_for(nnz, 256);
    if (g > 152u * 16u) g = 152u * 16u;
    k_check_js<<<g, 256, 0, s>>>(x, nnz, err);
  }
}

void launch_exact_slab(int method, int dist, const DevCsc& ref, const ColAux& ra,
                       const DevCsc& qry, const ColAux& qa, int64_t q0, int64_t nb,
                       const uint8_t* ref_mask, int restore_self, double self_value,
                       double* D, cudaStream_t s) {
  if (ref.ncol == 0 || nb == 0) return;
  for (int64_t b0 = 0; b0 < nb; b0 += 65535) {            // gridDim.y limit
    const int64_t cnt = (nb - b0 < 65535) ? nb - b0 : 65535;
    dim3 grid(blocks_for(ref.ncol, 128), (unsigned)cnt);
    const bool lookup = lookup_method(method) && qry.nrow <= LOOKUP_MAX_ROWS;
    const size_t smem = lookup ? (size_t)((qry.nrow + 31) / 32) * 8 : 0;
    k_exact_slab<<<grid, 128, smem, s>>>(method, dist, ref, ra, qry, qa, q0 + b0, ref_mask,
                                         restore_self, self_value, D + b0 * (int64_t)ref.ncol, lookup ? 1 : 0);
  }
}

void launch_self_slab(int method, int dist, const DevCsc& m, const ColAux& a, int64_t c0,
                      int64_t nb, int upper, int diag, double* D, cudaStream_t s) {
  if (m.ncol == 0 || nb == 0) return;
  for (int64_t b0 = 0; b0 < nb; b0 += 65535) {            // gridDim.y limit
    const int64_t cnt = (nb - b0 < 65535) ? nb - b0 : 65535;
    dim3 grid(blocks_for(m.ncol, 128), (unsigned)cnt);
    k_self_slab<<<grid, 128, 0, s>>>(method, dist, m, a, c0 + b0, upper, diag, D + b0 * (int64_t)m.ncol);
  }
}

bool self_tri_supported(int method, int32_t nrow) {
  return (method == BINARY || method == COSINE || method == PEARSON || method == COVARIANCE) &&
         nrow <= RQ_MAX_NROW;
}

void launch_self_tri(int method, int dist, const DevCsc& m, const ColAux& a, int diag, double* D,
                     cudaStream_t s) {
  const int64_t n = m.ncol;
  if (n == 0) return;
  if (n > 1) {
    const size_t smem = (size_t)RQ_MAX_QV * 8 + (size_t)RQ_MAX_CAND * 8 + (size_t)RQ_WARPS * 32 * RM * 8 +
                        (size_t)((m.nrow + 31) / 32) * 8;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_rerank_q<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const unsigned chunks = (unsigned)((n - 1 + RQ_MAX_CAND - 1) / RQ_MAX_CAND);
    k_rerank_q<true><<<dim3((unsigned)n, chunks), RQ_THREADS, smem, s>>>(method, dist, m, a, m, a, nullptr,
                                                                        nullptr, 0, 0, 0, 0.0, D);
  }
  k_self_diag<<<blocks_for(n, 256), 256, 0, s>>>(method, dist, m, a, diag, D);
}

void launch_mirror_upper(double* D, int64_t n, int clear, cudaStream_t s) {
  if (n <= 1) return;
  const unsigned T = (unsigned)((n + 31) / 32);
  k_mirror_upper<<<dim3(T, T), dim3(32, 8), 0, s>>>(D, n, clear);
}

void launch_mirror_lower(double* D, int64_t n, cudaStream_t s) {
  // the caller holds n x n doubles on the device, so n / 32 is far below the
  // 65,535 limit of gridDim.y
  if (n <= 1) return;
  const unsigned T = (unsigned)((n + 31) / 32);
  k_mirror_lower<<<dim3(T, T), dim3(32, 8), 0, s>>>(D, n);
}

void launch_exact_pairs(int method, int dist, const DevCsc& ref, const ColAux& ra,
                        const DevCsc& qry, const ColAux& qa, const int32_t* ref_idx,
                        const int32_t* qry_idx, int64_t npairs, double* out, cudaStream_t s) {
  if (npairs > 0)
    k_exact_pairs<<<blocks_for(npairs, 128), 128, 0, s>>>(method, dist, ref, ra, qry, qa,
                                                           ref_idx, qry_idx, npairs, out);
}

bool rerank_warp_supported(int method) {
  return method == BINARY || method == COSINE || method == PEARSON;
}

void launch_rerank_warp(int method, int dist, const DevCsc& ref, const ColAux& ra,
                        const DevCsc& qry, const ColAux& qa, const int32_t* cand,
                        const int32_t* count, int cap, int64_t nq_local, int64_t q_begin,
                        int restore_self, double self_value, double* out, cudaStream_t s) {
  if (nq_local <= 0) return;
  if (qry.nrow <= RQ_MAX_NROW && cap <= RQ_MAX_CAND) {
    const size_t smem = (size_t)RQ_MAX_QV * 8 + (size_t)RQ_MAX_CAND * 8 + (size_t)RQ_WARPS * 32 * RM * 8 +
                        (size_t)((qry.nrow + 31) / 32) * 8;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_rerank_q<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_rerank_q<false><<<(unsigned)nq_local, RQ_THREADS, smem, s>>>(method, dist, ref, ra, qry, qa, cand, count, cap,
                                                           q_begin, restore_self, self_value, out);
  } else {
    k_rerank_warp<<<blocks_for(nq_local, 8), 256, 0, s>>>(method, dist, ref, ra, qry, qa, cand,
                                                          count, cap, nq_local, q_begin,
                                                          restore_self, self_value, out);
  }
}

void launch_exact_pairs_sparse(int method, int dist, const DevCsc& ref, const ColAux& ra,
                               const DevCsc& qry, const ColAux& qa, const int32_t* ref_idx,
                               const int32_t* qry_idx, int64_t npairs, int restore_self,
                               double self_value, double* out, cudaStream_t s) {
  if (npairs > 0)
    k_exact_pairs_sparse<<<blocks_for(npairs, 128), 128, 0, s>>>(
        method, dist, ref, ra, qry, qa, ref_idx, qry_idx, npairs, restore_self, self_value, out);
}

}  // namespace sdg

namespace sdg {

size_t batch_smem(int kmax) { return (size_t)BATCH_WARPS * kmax * 20; }

int batch_lookup_words(int method, int32_t nrow) {
  return (lookup_method(method) && nrow <= LOOKUP_MAX_ROWS) ? (nrow + 31) / 32 : 0;
}

void launch_batch_exact(const BatchProb* probs, const BatchItem* items, int64_t nitems, unsigned long long* counter,
                        int kmax, int lwords, uint64_t* pkey, int32_t* pidx, double* pval, int sms, cudaStream_t s) {
  if (nitems <= 0) return;
  const size_t smem = batch_smem(kmax) + (size_t)BATCH_WARPS * lwords * 8;
  if (smem > 48 * 1024) cudaFuncSetAttribute(k_batch_exact, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_exact, BATCH_WARPS * 32, smem);
  const int64_t grid = std::min<int64_t>((int64_t)std::max(1, per_sm) * std::max(1, sms),
                                         (nitems + BATCH_WARPS - 1) / BATCH_WARPS);
  k_batch_exact<<<(unsigned)grid, BATCH_WARPS * 32, smem, s>>>(probs, items, nitems, counter, kmax, lwords, pkey,
                                                                pidx, pval);
}

void launch_batch_merge(const BatchProb* probs, const BatchRow* rows, int64_t nrows, int kmax, const uint64_t* pkey,
                        const int32_t* pidx, const double* pval, cudaStream_t s) {
  if (nrows <= 0) return;
  const size_t smem = batch_smem(kmax);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k_batch_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_batch_merge<<<(unsigned)((nrows + BATCH_WARPS - 1) / BATCH_WARPS), BATCH_WARPS * 32, smem, s>>>(
      probs, rows, nrows, kmax, pkey, pidx, pval);
}

}  // namespace sdg
