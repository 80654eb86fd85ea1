// sdg_screen.cu -- the screened candidate engine (see sdg_screen.h).
//
// GB300 executes FP64 at roughly 1/70 of its FP32 rate, so evaluating every
// column pair exactly in FP64 (as the reference does on the CPU) is bound by
// the FP64 pipe.  This engine evaluates every pair in FP32 instead, with a
// rigorous per-pair error bound E, and re-ranks in exact FP64 only the pairs
// whose optimistic bound can still reach the k-th best pessimistic bound:
//
//   keep (q, c)  iff  key(q, c) + E(q, c) >= T_q - margin,
//   T_q = k-th largest of key(q, c') - E(q, c') over eligible c'.
//
// Every member of the exact top-k (ties included) satisfies the test, so the
// exact re-rank over the kept pairs returns exactly the reference's result.
// A query whose kept set exceeds the candidate capacity is finished by the
// exact slab engine instead.
//
// Screen kernel layout: one CTA of 512 threads holds a tile of up to 16 query
// columns in shared memory as a row-indexed table -- one 32-bit word per row,
// row[r] = (mask16 << 16) | off16 (mask16: which tile queries store row r;
// off16: where row r's values start in vals[]) -- and vals[] (the tile's
// values, row-major then by query).  Each lane then walks one reference column (reference
// columns are visited in descending-nnz order so the 32 lanes of a warp do
// similar work), looks each stored row up in the table and accumulates 16
// FP32 screen values in registers.  Work items (tile, reference part) are
// handed out part-major by an atomic counter, so the 152 SMs stream the same
// reference part at the same time and it is read from HBM about once.
#include <cub/device/device_radix_sort.cuh>
#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "sdg_kernels.h"
#include "sdg_screen.h"
#include "sdg_tc_bounds.cuh"

namespace sdg {
namespace {

constexpr int QT = 16;               // queries per tile
constexpr int SCREEN_THREADS = 512;
constexpr int SELECT_WARPS = 8;
// dynamic shared memory of the screen kernel: the 227 KB per-CTA maximum less
// room for its static shared memory
constexpr size_t kSmemMax = 227 * 1024 - 1024;
constexpr float U32 = 5.9604644775390625e-8f;   // 2^-24

inline unsigned blocks_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

// the failing call of the last screen error on this thread (for the message)
thread_local const char* g_screen_site = "";
#define SK_STR2(l) #l
#define SK_STR(l) SK_STR2(l)
#define SK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { g_screen_site = #x " at line " SK_STR(__LINE__); return (int)e_; } } while (0)
// a call of a function that records its own failing site
#define SKN(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return (int)e_; } while (0)

// ---------------------------------------------------------------------------
// validation used at upload
// ---------------------------------------------------------------------------
__global__ void k_check_rows(DevCsc M, int* err) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= M.ncol) return;
  int32_t prev = -1;
  for (int64_t a = M.p[j]; a < M.p[j + 1]; ++a) {
    const int32_t r = M.i[a];
    if (r <= prev || r >= M.nrow) { atomicOr(err, 1); return; }
    prev = r;
  }
}

// ---------------------------------------------------------------------------
// per-matrix screening data
// ---------------------------------------------------------------------------
// fval: the value the screen multiplies (unit value for cosine, raw value for
// euclidean / manhattan, 1 for binary); cnorm: sum of squares (euclidean) or
// of magnitudes (manhattan), accumulated in FP64 then rounded; nnz per column.
// One warp per column: the FP32 screen values (coalesced) and the column's
// norm term (a warp sum in FP64, rounded to FP32: the screen bounds allow for
// its rounding whatever the summation order).
// js: fval = the value, fxl = its x log x (from the FP64 values the exact path
// uses), cnorm = the column's sum of |x log x| + x rounded up, and *range_err
// set when a nonzero value lies outside [2^-100, 2^100]; pearson /
// covariance: fval = the value, *range_err when a nonzero |value| lies outside
// [2^-50, 2^50].
__global__ void k_screen_prep(DevCsc M, int method, const double* uval, const double* xl, float* fval,
                              float* fxl, float* cnorm, int32_t* nnz, int* range_err) {
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= M.ncol) return;
  double acc = 0.0;
  bool bad = false;
  const int64_t a0 = M.p[j], a1 = M.p[j + 1];
  for (int64_t a = a0 + lane; a < a1; a += 32) {
    const double v = M.x[a];
    float f;
    if (method == COSINE) f = (float)uval[a];
    else if (method == BINARY) f = 1.0f;
    else f = (float)v;
    fval[a] = f;
    if (method == EUCLIDEAN) acc += v * v;
    else if (method == MANHATTAN) acc += fabs(v);
    else if (method == JS) {
      fxl[a] = (float)xl[a];
      acc += fabs(xl[a]) + v;
      bad = bad || (v != 0.0 && !(v >= 0x1p-100 && v <= 0x1p100));
    } else if (method == PEARSON || method == COVARIANCE) {
      // FP32 products of values within 2^+-50 stay normal and their sums finite
      bad = bad || (v != 0.0 && !(fabs(v) >= 0x1p-50 && fabs(v) <= 0x1p50));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(range_err, 1);
  if (lane == 0) {
    cnorm[j] = (method == JS) ? __double2float_ru(acc * (1.0 + 1e-12)) : (float)acc;
    nnz[j] = (int32_t)(a1 - a0);
  }
}

__global__ void k_iota_neg_nnz(const int32_t* nnz, int64_t n, uint32_t* keys, int32_t* ids) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= n) return;
  keys[j] = 0x7fffffffu - (uint32_t)nnz[j];   // ascending key = descending nnz
  ids[j] = (int32_t)j;
}

// ---------------------------------------------------------------------------
// the screen kernel
// ---------------------------------------------------------------------------
struct ScreenArgs {
  int method;
  int32_t nrow;
  int groups;                 // ceil(nrow / 64)
  int vcap;                   // tile value capacity (floats)
  // reference
  const int64_t* rp; const int32_t* ri; const float* rv;
  const float* rxl;           // js: x log x of each reference value
  const int32_t* rperm;       // position -> reference column
  int64_t nr;
  // queries (columns of the query matrix)
  const int64_t* qp; const int32_t* qi; const float* qv;
  const float* qxl;           // js: x log x of each query value
  const int32_t* tile_q;      // first local query of each tile
  const int32_t* tile_n;      // queries in each tile
  int64_t q_begin;            // local query 0 = query column q_begin
  int ntiles, nparts;
  int64_t part_len;
  float* S;                   // S[qlocal * nr + pos]
  int* work;                  // work counter
};

__device__ __forceinline__ void accumulate(int method, float (&acc)[QT], uint32_t m, uint32_t base,
                                           float v, const float* __restrict__ vals) {
  if (method == MANHATTAN) {
#pragma unroll
    for (int j = 0; j < QT; ++j) {
      if (m & (1u << j)) {
        const float q = vals[base];
        acc[j] += (fabsf(v) + fabsf(q)) - fabsf(v - q);
        ++base;
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < QT; ++j) {
      if (m & (1u << j)) {
        acc[j] = fmaf(v, vals[base], acc[j]);
        ++base;
      }
    }
  }
}

__device__ __forceinline__ void accumulate_word(int method, float (&acc)[QT], uint32_t w, float v,
                                                const float* __restrict__ vals) {
  const uint32_t m = w >> 16;
  if (m) accumulate(method, acc, m, w & 0xffffu, v, vals);   // rows outside the tile: skip
}

// js: the shared row's g = S log S - P log P - Q log Q (S = P + Q) in FP32,
// every operation rounded on its own (no contraction), summed in order; the
// logarithm is the __logf intrinsic, taken to err by at most 2^-20.41
// absolute on [0.5, 2] and 6 ulp elsewhere (twice its documented accuracy;
// tests/test_gpu_logf_bound.py checks every FP32 input in [2^-100, 2^102)).
// The error analysis of js_key_and_bound below follows these steps.
__device__ __forceinline__ void accumulate_js(float (&acc)[QT], uint32_t w, float v, float vx,
                                              const float* __restrict__ vals, const float* __restrict__ vxl) {
  uint32_t m = w >> 16;
  uint32_t base = w & 0xffffu;
#pragma unroll
  for (int j = 0; j < QT; ++j) {
    if (m & (1u << j)) {
      const float q = vals[base], qx = vxl[base];
      const float S = __fadd_rn(v, q);
      const float g = __fsub_rn(__fsub_rn(__fmul_rn(S, __logf(S)), vx), qx);
      acc[j] = __fadd_rn(acc[j], g);
      ++base;
    }
  }
}

template <int METHOD_KIND>   // 0: product, 1: manhattan, 2: js
__global__ void __launch_bounds__(SCREEN_THREADS, 1) k_screen(ScreenArgs A) {
  extern __shared__ __align__(16) unsigned char smem[];
  // row[r] = (mask16 << 16) | offset of row r's first value in vals[]
  uint32_t* row = reinterpret_cast<uint32_t*>(smem);
  float* vals = reinterpret_cast<float*>(row + A.nrow);
  float* vxl = vals + A.vcap;                       // js: the values' x log x
  __shared__ int s_item;
  __shared__ uint32_t s_warp[SCREEN_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int method = METHOD_KIND == 1 ? (int)MANHATTAN : (int)COSINE;
  int cur_tile = -1;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(A.work, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= A.ntiles * A.nparts) break;
    const int part = item / A.ntiles, tile = item % A.ntiles;
    const int tq0 = A.tile_q[tile], tn = A.tile_n[tile];

    if (tile != cur_tile) {
      // -- build the tile's row table --------------------------------------
      for (int r = tid; r < A.nrow; r += SCREEN_THREADS) row[r] = 0u;
      __syncthreads();
      for (int j = 0; j < tn; ++j) {
        const int64_t q = A.q_begin + tq0 + j;
        const int64_t e0 = A.qp[q], e1 = A.qp[q + 1];
        for (int64_t e = e0 + tid; e < e1; e += SCREEN_THREADS)
          atomicOr(&row[A.qi[e]], 1u << (16 + j));
      }
      __syncthreads();
      // exclusive scan of popc(mask) over rows: contiguous row ranges per thread
      const int per = (A.nrow + SCREEN_THREADS - 1) / SCREEN_THREADS;
      const int r0 = tid * per, r1 = min(A.nrow, r0 + per);
      uint32_t sum = 0;
      for (int r = r0; r < r1; ++r) sum += __popc(row[r] >> 16);
      uint32_t x = sum;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
      }
      if (lane == 31) s_warp[warp] = x;
      __syncthreads();
      if (warp == 0) {
        const uint32_t v = (lane < SCREEN_THREADS / 32) ? s_warp[lane] : 0u;
        uint32_t t = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, t, d);
          if (lane >= d) t += y;
        }
        if (lane < SCREEN_THREADS / 32) s_warp[lane] = t - v;
      }
      __syncthreads();
      uint32_t run = s_warp[warp] + x - sum;
      for (int r = r0; r < r1; ++r) {
        const uint32_t w = row[r];
        row[r] = (w & 0xffff0000u) | (run & 0xffffu);
        run += __popc(w >> 16);
      }
      __syncthreads();
      for (int j = 0; j < tn; ++j) {
        const int64_t q = A.q_begin + tq0 + j;
        const int64_t e0 = A.qp[q], e1 = A.qp[q + 1];
        const uint32_t below = (1u << j) - 1u;
        for (int64_t e = e0 + tid; e < e1; e += SCREEN_THREADS) {
          const uint32_t w = row[A.qi[e]];
          const uint32_t pos = (w & 0xffffu) + __popc((w >> 16) & below);
          if (pos < (uint32_t)A.vcap) {
            vals[pos] = A.qv[e];
            if (METHOD_KIND == 2) vxl[pos] = A.qxl[e];
          }
        }
      }
      __syncthreads();
      cur_tile = tile;
    }

    // -- stream the part's reference columns: one column per lane ----------
    const int64_t p0 = (int64_t)part * A.part_len;
    const int64_t p1 = min(A.nr, p0 + A.part_len);
    for (int64_t pos = p0 + tid; pos < p1; pos += SCREEN_THREADS) {
      const int32_t c = A.rperm[pos];
      float acc[QT];
#pragma unroll
      for (int j = 0; j < QT; ++j) acc[j] = 0.f;
      int64_t e = A.rp[c];
      const int64_t e1 = A.rp[c + 1];
      if (METHOD_KIND == 2) {
        // four entries (rows, values, x log x) per vector load, the next four
        // prefetched, as the product walk below; the arrays share offsets
        for (; e < e1 && (e & 3); ++e) {
          const uint32_t w = row[__ldg(A.ri + e)];
          if (w >> 16) accumulate_js(acc, w, __ldg(A.rv + e), __ldg(A.rxl + e), vals, vxl);
        }
        if (e + 4 <= e1) {
          int4 rn = __ldg(reinterpret_cast<const int4*>(A.ri + e));
          float4 vn = __ldg(reinterpret_cast<const float4*>(A.rv + e));
          float4 xn = __ldg(reinterpret_cast<const float4*>(A.rxl + e));
          for (; e + 4 <= e1; e += 4) {
            const int4 r4 = rn;
            const float4 v4 = vn, x4 = xn;
            if (e + 8 <= e1) {
              rn = __ldg(reinterpret_cast<const int4*>(A.ri + e + 4));
              vn = __ldg(reinterpret_cast<const float4*>(A.rv + e + 4));
              xn = __ldg(reinterpret_cast<const float4*>(A.rxl + e + 4));
            }
            const uint32_t w0 = row[r4.x], w1 = row[r4.y], w2 = row[r4.z], w3 = row[r4.w];
            if (w0 >> 16) accumulate_js(acc, w0, v4.x, x4.x, vals, vxl);
            if (w1 >> 16) accumulate_js(acc, w1, v4.y, x4.y, vals, vxl);
            if (w2 >> 16) accumulate_js(acc, w2, v4.z, x4.z, vals, vxl);
            if (w3 >> 16) accumulate_js(acc, w3, v4.w, x4.w, vals, vxl);
          }
        }
        for (; e < e1; ++e) {
          const uint32_t w = row[__ldg(A.ri + e)];
          if (w >> 16) accumulate_js(acc, w, __ldg(A.rv + e), __ldg(A.rxl + e), vals, vxl);
        }
      }
      for (; e < e1 && (e & 3); ++e)
        accumulate_word(method, acc, row[__ldg(A.ri + e)], __ldg(A.rv + e), vals);
      if (e + 4 <= e1) {
        int4 rn = __ldg(reinterpret_cast<const int4*>(A.ri + e));
        float4 vn = __ldg(reinterpret_cast<const float4*>(A.rv + e));
        for (; e + 4 <= e1; e += 4) {
          const int4 r4 = rn;
          const float4 v4 = vn;
          if (e + 8 <= e1) {                            // prefetch the next group
            rn = __ldg(reinterpret_cast<const int4*>(A.ri + e + 4));
            vn = __ldg(reinterpret_cast<const float4*>(A.rv + e + 4));
          }
          const uint32_t w0 = row[r4.x], w1 = row[r4.y], w2 = row[r4.z], w3 = row[r4.w];
          accumulate_word(method, acc, w0, v4.x, vals);
          accumulate_word(method, acc, w1, v4.y, vals);
          accumulate_word(method, acc, w2, v4.z, vals);
          accumulate_word(method, acc, w3, v4.w, vals);
        }
      }
      for (; e < e1; ++e)
        accumulate_word(method, acc, row[__ldg(A.ri + e)], __ldg(A.rv + e), vals);
#pragma unroll
      for (int j = 0; j < QT; ++j)
        if (j < tn) A.S[(int64_t)(tq0 + j) * A.nr + pos] = acc[j];
    }
  }
}

// ---------------------------------------------------------------------------
// screen select: per query, the k-th pessimistic bound and the kept pairs
// ---------------------------------------------------------------------------
struct SelectScreenArgs {
  int method, k;
  const float* S;
  int64_t nr;
  const int32_t* rperm;
  const int32_t* rnnz; const float* rnorm;
  const int32_t* qnnz; const float* qnorm;   // indexed by query column
  const double* rsum;                        // js: reference column sums
  const double* qsum;                        // js: query column sums (indexed by query column)
  // pearson / covariance: the columns' FP64 sums and sums of squares, nrow
  const double *rs, *rss, *qs, *qss;
  int32_t nrow;
  const uint8_t* ref_mask;                   // eligible reference columns
  const uint8_t* qry_blank;                  // query rows written all-NA
  const uint8_t* qry_force_exact;            // queries the screen cannot bound
  int64_t q_begin, nq;                       // local queries of this chunk
  int selfmode, include_self;                // self search: query q == reference q
  int cap;
  int32_t* cand;                             // [qlocal * cap + t] reference column
  int32_t* count;                            // kept pairs per query (capped)
  int32_t* overflow;                         // 1 = finish with the exact engine
};

// Larger key = better.  E bounds |key_fp32 - key_exact| (see the file header
// and DESIGN notes of each method).
__device__ __forceinline__ void key_and_bound(int method, float s, int32_t nq_, float Nq, int32_t nc_,
                                              float Nc, float& key, float& err) {
  const float n = (float)min(nq_, nc_);
  if (method == COSINE) {
    key = s;
    err = (n + 40.f) * U32 * 1.01f + 1e-12f;
  } else if (method == EUCLIDEAN) {
    const float T = Nq + Nc;
    key = 2.f * s - T;
    err = ((n + 46.f) * U32 * 1.01f + 1e-12f) * T + 1e-30f;
  } else if (method == MANHATTAN) {
    const float T = Nq + Nc;
    key = s - T;
    err = ((n + 46.f) * U32 * 1.01f + 1e-12f) * T + 1e-30f;
  } else {                                   // BINARY: s is the exact count
    const float denom = (float)(nq_ + nc_) - s;
    key = (denom > 0.f) ? s / denom : 1.f;
    err = key * (4.f * U32) + 1e-30f;
  }
}

// js (fastJS2, src/sparseDist.cpp:1099-1108): the value is sqrt(0.5 t) with
// t = (S_P + S_Q) log 2 - G, G = sum over shared rows of g = S log S - P log P
// - Q log Q (every other row adds its value times log 2), so with the query
// fixed the order is that of key = G - S_P log 2 (larger = better).  Error of
// the FP32 G (values in [2^-100, 2^100], u = 2^-24): p, q, S rounded once
// (S~ = S (1 + t), |t| <= 2.0001 u); |__logf(S~) - ln S~| <= 12.06 u + 12 u
// |ln S~| (2^-20.41 absolute on [0.5, 2], 6 ulp <= 12 u relative elsewhere),
// so |L - ln S| <= 14.07 u + 12 u |ln S|; the product and the two differences
// each rounded once, x log x stored to FP32: |g~ - g| <= u (17.0001 |S log S|
// + 14.07 S + 3.0001 |P log P| + 2.0001 |Q log Q|) <= 31.1 u (|P log P| + |Q
// log Q| + S), using |S log S| <= |P log P| + |Q log Q| + S; summed over the
// shared rows <= 31.1 u (A_P + A_Q), A = a column's sum of |x log x| + x.
// The recursive FP32 sum of n <= min(nnz) terms adds <= n u / (1 - n u) times
// sum |g~| <= log 2 (C_P + C_Q) + 31.1 u (A_P + A_Q) (0 <= g <= S log 2, C =
// a column's sum).  With n u <= 1/16 (n is below the row table's 56 K rows)
// the two give E_G = u (33.5 (A_P + A_Q) + 0.75 n (C_P + C_Q)) 1.01; the key's
// own rounding (u |key|, the FP64 S_P log 2 rounded once) is added.
__device__ __forceinline__ void js_key_and_bound(float G, double SP, double SQ, float AP, float AQ,
                                                 int32_t n_, float& key, float& err) {
  const float n = (float)n_;
  key = (float)((double)G - SP * 0.69314718055994530942);
  const float C = (float)(SP + SQ);
  err = U32 * (33.5f * (AP + AQ) + 0.75f * n * C) * 1.01f + 2.f * U32 * fabsf(key) + 1e-30f;
}

// pearson / covariance (fastCorr2 / fastCov2 in the single-pass form of the
// exact path, pearson_finish / covariance_finish): the screen's s~ is the FP32
// FMA chain over the matched rows' FP32 values; with u = 2^-24 and n <= min(nnz)
// terms, |s~ - s| <= (n + 3) u (1 + n u 1.1) sum |ab| <= (n + 4) u 1.01 sqrt(SS_P
// SS_Q) (Cauchy-Schwarz over the full columns' sums of squares; the exact
// path's own FP64 sum is within n 2^-53 of s, inside the factor).  The key is
// the exact path's formula evaluated in FP64 on s~ with the same rounded
// operations, so the decisions that depend only on the moments (a zero or
// non-finite denominator, which makes the exact value 0) are the exact path's:
// cov = (s - S_P S_Q / N) / (N - 1), errs by E_s / (N - 1) plus 2^-50 of its
// terms; pearson c = cov / (sqrt(v_P) sqrt(v_Q)) by E_cov / den plus 2^-50 |c|,
// and both bounds are clamped to [-1, 1] as the exact value is.  A pearson
// denominator below 1e-200 could let cov / den overflow (exact value 0 then):
// the bounds are [-1, 1].  Larger key = better for both methods.
__device__ __forceinline__ void moment_key_and_bound(bool pearson, float s, int32_t n_, int32_t nrow, double SP,
                                                     double SSP, double SQ, double SSQ, float& key, float& err) {
  const double N = (double)nrow;
  const double norm = (nrow > 1) ? __dsub_rn(N, 1.0) : 1.0;
  const double sd = (double)s;
  const double Es = (((double)n_ + 4.0) * 5.9604644775390625e-8 * 1.01) * sqrt(SSP * SSQ) + 1e-300;
  const double m = __dmul_rn(SP, SQ) / N;
  const double cov = __dsub_rn(sd, m) / norm;
  const double Ecov = (Es + 0x1p-50 * (fabs(sd) + fabs(m))) / norm;
  double lo, hi;
  if (!pearson) {
    lo = cov - Ecov * 1.0001;
    hi = cov + Ecov * 1.0001;
  } else {
    const double vp = __dsub_rn(SSP, __dmul_rn(SP, SP) / N) / norm;
    const double vq = __dsub_rn(SSQ, __dmul_rn(SQ, SQ) / N) / norm;
    const double den = __dmul_rn(sqrt(vp), sqrt(vq));
    if (!(den > 0.0) || !isfinite(den)) { key = 0.f; err = 0.f; return; }   // the exact value is 0
    if (den < 1e-200) { key = 0.f; err = 1.0001f; return; }
    const double c = cov / den;
    const double e = (Ecov / den + 0x1p-50 * fabs(c)) * 1.0001;
    lo = fmin(1.0, fmax(-1.0, c - e));
    hi = fmin(1.0, fmax(-1.0, c + e));
  }
  key = (float)(0.5 * (lo + hi));
  err = (float)(0.5 * (hi - lo)) + 2.f * U32 * (fabsf(key) + 1.f) + 1e-30f;
}

__global__ void k_screen_select(SelectScreenArgs A) {
  extern __shared__ float lists[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = (int64_t)blockIdx.x * SELECT_WARPS + warp;
  if (ql >= A.nq) return;
  const int64_t q = A.q_begin + ql;
  float* lst = lists + warp * A.k;
  const int K = A.k;
  if ((A.qry_blank && A.qry_blank[q]) ) {
    if (lane == 0) { A.count[ql] = 0; A.overflow[ql] = 0; }
    return;
  }
  if (A.qry_force_exact && A.qry_force_exact[q]) {
    if (lane == 0) { A.count[ql] = 0; A.overflow[ql] = 1; }
    return;
  }
  const int32_t nq_ = A.qnnz[q];
  const float Nq = A.qnorm ? A.qnorm[q] : 0.f;
  const float* Srow = A.S + ql * A.nr;
  const int64_t self_c = A.selfmode ? q : -1;
  int n = 0;
  // pass 1: the k largest pessimistic keys
  for (int64_t p0 = 0; p0 < A.nr; p0 += 32) {
    const int64_t pos = p0 + lane;
    float lo = -INFINITY;
    bool ok = pos < A.nr;
    if (ok) {
      const int32_t c = A.rperm[pos];
      if (A.ref_mask && A.ref_mask[c]) ok = false;
      else if (c == self_c && !(A.include_self && A.method == COVARIANCE)) {
        // a restored self value (R/sparseKNN.R:270-279) is the best key; a
        // covariance self pair keeps its computed value and is an ordinary pair
        if (A.include_self) lo = INFINITY; else ok = false;
      } else {
        float key, err;
        if (A.method == JS)
          js_key_and_bound(Srow[pos], A.rsum[c], A.qsum[q], A.rnorm[c], Nq, min(nq_, A.rnnz[c]), key, err);
        else if (A.method == PEARSON || A.method == COVARIANCE)
          moment_key_and_bound(A.method == PEARSON, Srow[pos], min(nq_, A.rnnz[c]), A.nrow, A.rs[c], A.rss[c],
                               A.qs[q], A.qss[q], key, err);
        else
          key_and_bound(A.method, Srow[pos], nq_, Nq, A.rnnz[c], A.rnorm ? A.rnorm[c] : 0.f, key, err);
        lo = key - err;
      }
    }
    bool pass = ok && (n < K || lo > lst[K - 1]);
    unsigned m = __ballot_sync(0xffffffffu, pass);
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      const float v = __shfl_sync(0xffffffffu, lo, src);
      if (n == K && !(v > lst[K - 1])) continue;
      int lo_i = 0, hi_i = n;                       // first index with lst[i] < v
      while (lo_i < hi_i) { const int mid = (lo_i + hi_i) >> 1; if (lst[mid] >= v) lo_i = mid + 1; else hi_i = mid; }
      const int last = (n < K) ? n : K - 1;
      if (last > lo_i) {
        for (int cch = (last - 1) >> 5; cch >= (lo_i >> 5); --cch) {
          const int e = cch * 32 + lane;
          const bool mv = (e >= lo_i && e < last);
          float t = 0.f;
          if (mv) t = lst[e];
          __syncwarp();
          if (mv) lst[e + 1] = t;
          __syncwarp();
        }
      }
      if (lane == 0) lst[lo_i] = v;
      __syncwarp();
      if (n < K) ++n;
    }
  }
  const float T = (n == K) ? lst[K - 1] : -INFINITY;
  const float margin = (T == -INFINITY || T == INFINITY) ? 0.f : fabsf(T) * (8.f * U32) + 1e-30f;
  // pass 2: keep every pair whose optimistic key reaches T
  int cnt = 0;
  bool over = false;
  int32_t* out = A.cand + ql * (int64_t)A.cap;
  for (int64_t p0 = 0; p0 < A.nr && !over; p0 += 32) {
    const int64_t pos = p0 + lane;
    bool keep = false;
    int32_t c = -1;
    if (pos < A.nr) {
      c = A.rperm[pos];
      if (A.ref_mask && A.ref_mask[c]) keep = false;
      else if (c == self_c && !(A.include_self && A.method == COVARIANCE)) keep = A.include_self != 0;
      else {
        float key, err;
        if (A.method == JS)
          js_key_and_bound(Srow[pos], A.rsum[c], A.qsum[q], A.rnorm[c], Nq, min(nq_, A.rnnz[c]), key, err);
        else if (A.method == PEARSON || A.method == COVARIANCE)
          moment_key_and_bound(A.method == PEARSON, Srow[pos], min(nq_, A.rnnz[c]), A.nrow, A.rs[c], A.rss[c],
                               A.qs[q], A.qss[q], key, err);
        else
          key_and_bound(A.method, Srow[pos], nq_, Nq, A.rnnz[c], A.rnorm ? A.rnorm[c] : 0.f, key, err);
        keep = (key + err) >= T - margin;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int rank = __popc(m & ((1u << lane) - 1u));
    if (keep && cnt + rank < A.cap) out[cnt + rank] = c;
    cnt += __popc(m);
    if (cnt > A.cap) over = true;
  }
  if (lane == 0) {
    A.count[ql] = over ? 0 : cnt;
    A.overflow[ql] = over ? 1 : 0;
  }
}

__global__ void k_exact_candidates_prep(const int32_t* count, int64_t nq, int cap, int32_t* qidx,
                                        const int32_t* cand, int32_t* ridx, int64_t q_begin) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nq * cap) return;
  const int64_t ql = s / cap, t = s % cap;
  if (t < count[ql]) { qidx[s] = (int32_t)(q_begin + ql); ridx[s] = cand[s]; }
  else { qidx[s] = -1; ridx[s] = -1; }
}

// ---------------------------------------------------------------------------
// the tensor-core screen
//
// For cosine and euclidean the screen value of a pair is an inner product
// over the rows (binary: of the 0 / 1 patterns, the matched-row count), so a
// dense FP16 copy of the screen values of both matrices (TensorCache) turns a
// block of screens into one GEMM on the tensor cores: the fused tcgen05
// kernel of sdg_sparse_tc.cu (FP16 in, FP32 accumulate; FP16 runs at BF16's
// tensor rate and rounds 4x finer, 2^-11) with the selection in its
// epilogue.  The bound (tcb::tc_bounds, sdg_tc_bounds.cuh) is built from each
// column's exact rounding error ||v - h|| (FP64, v the exact values, h the
// FP16 copy), so it covers every way the copy differs: values below FP16's
// smallest normal are written as 0, never as FP16 subnormals, and a value
// above FP16's range makes the copy unusable (TensorCache::usable: the FP32
// screen runs).  The FP16 products are exact in FP32; the FP32 accumulation
// of at most n = min(nnz_q, nnz_c) nonzero products (zero products add no
// error) is allowed (n + 64) 2^-21 of sum |h_q h_c|.
// ---------------------------------------------------------------------------
constexpr float HALF_MAX = 65504.f;
constexpr float HALF_MIN_NORMAL = 6.103515625e-05f;   // 2^-14

// One warp per column: scatter the FP16 values into the dense column and
// compute ||v - b|| and ||b|| in FP64 (v: src, the exact values; b: the FP16
// values the GEMM multiplies), rounded up to FP32.
__global__ void k_tensor_fill(DevCsc M, const float* fval, const double* src, __half* dense, int64_t ld,
                              float* err_out, float* bn_out, int* bad) {
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= M.ncol) return;
  __half* col = dense + j * ld;
  double se = 0.0, sb = 0.0;
  for (int64_t a = M.p[j] + lane; a < M.p[j + 1]; a += 32) {
    const float f = fval[a];
    const float af = fabsf(f);
    if (!(af <= HALF_MAX)) atomicOr(bad, 1);          // beyond FP16, or not finite
    const __half hv = __float2half_rn(af < HALF_MIN_NORMAL ? 0.f : f);
    col[M.i[a]] = hv;
    const double b = (double)__half2float(hv);
    const double v = src ? src[a] : (double)f;
    se += (v - b) * (v - b);
    sb += b * b;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    se += __shfl_xor_sync(0xffffffffu, se, o);
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
  }
  if (lane == 0) {
    // FP64 sums and sqrt are within a few units of 2^-52; the factor and the
    // upward FP32 rounding cover them
    err_out[j] = __double2float_ru(sqrt(se) * (1.0 + 1e-12));
    bn_out[j] = __double2float_ru(sqrt(sb) * (1.0 + 1e-12));
  }
}

// Warp-cooperative insertion of the lanes flagged in m (value v on each lane)
// into lst[0..n), kept sorted descending and at most K long.
__device__ __forceinline__ void warp_insert_desc(float* lst, int K, int& n, unsigned m, float v, int lane) {
  while (m) {
    const int src = __ffs(m) - 1;
    m &= m - 1;
    const float x = __shfl_sync(0xffffffffu, v, src);
    if (n == K && !(x > lst[K - 1])) continue;
    int a = 0, b = n;
    while (a < b) { const int mid = (a + b) >> 1; if (lst[mid] >= x) a = mid + 1; else b = mid; }
    const int last = (n < K) ? n : K - 1;
    if (last > a) {
      for (int cch = (last - 1) >> 5; cch >= (a >> 5); --cch) {
        const int e = cch * 32 + lane;
        const bool mv = (e >= a && e < last);
        float t = 0.f;
        if (mv) t = lst[e];
        __syncwarp();
        if (mv) lst[e + 1] = t;
        __syncwarp();
      }
    }
    if (lane == 0) lst[a] = x;
    __syncwarp();
    if (n < K) ++n;
  }
}

// ---------------------------------------------------------------------------
// second screen of the tensor candidates: FP32 sparse dot products
//
// The FP16 bound keeps a few hundred candidates per query; the FP32 screen's
// bound (key_and_bound) is ~100x tighter.  One CTA per query holds the query
// column as a shared-memory bitmap (with each word's first entry, as in the
// exact re-rank) and its FP32 screen values; a warp per candidate streams the
// candidate column (coalesced, four rounds in flight), multiplies the matched
// FP32 values and reduces across the warp.  The FP32 bound holds for any
// summation order, so the reduction is a tree.  Then, per query, T2 = the
// k-th largest pessimistic key and the list keeps the candidates whose
// optimistic key reaches T2 - margin: the exact re-rank sees only those.
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_MAX_QV = 4096;
constexpr int32_t RS_MAX_NROW = 1 << 18;

struct RescreenArgs {
  int method, k;
  DevCsc ref, qry;
  const float* rf;           // ScreenCache values (unit values / values)
  const float* qf;
  const int32_t* rnnz; const float* rnorm;
  const int32_t* qnnz; const float* qnorm;
  int64_t q_begin, nq;
  int selfmode;
  int cap;
  int32_t* cand;
  int32_t* count;
  float* lo;                 // [ql * cap + t]
  float* hi;
};

__global__ void k_rescreen(RescreenArgs A) {
  extern __shared__ __align__(16) uint32_t rs_smem[];
  const int W = (A.qry.nrow + 31) >> 5;
  float* qvs = reinterpret_cast<float*>(rs_smem);             // RS_MAX_QV
  uint32_t* bits = rs_smem + RS_MAX_QV;
  int32_t* first = reinterpret_cast<int32_t*>(bits + W);
  const int64_t ql = blockIdx.x;
  const int64_t q = A.q_begin + ql;
  const int n = A.count[ql];
  if (n == 0) return;
  for (int w = threadIdx.x; w < W; w += blockDim.x) bits[w] = 0u;
  __syncthreads();
  const int64_t q0 = A.qry.p[q], q1 = A.qry.p[q + 1];
  const bool qv_shared = (q1 - q0) <= RS_MAX_QV;
  for (int64_t e = q0 + threadIdx.x; e < q1; e += blockDim.x) {
    const int32_t r = A.qry.i[e];
    atomicOr(&bits[r >> 5], 1u << (r & 31));
    if (e == q0 || (A.qry.i[e - 1] >> 5) != (r >> 5)) first[r >> 5] = (int32_t)(e - q0);
    if (qv_shared) qvs[e - q0] = A.qf[e];
  }
  __syncthreads();
  const float* qv = qv_shared ? qvs : A.qf + q0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int32_t nq_ = A.qnnz[q];
  const float Nq = A.qnorm ? A.qnorm[q] : 0.f;
  for (int t = warp; t < n; t += nw) {
    const int32_t c = A.cand[ql * (int64_t)A.cap + t];
    float lo, hi;
    if (A.selfmode && c == q) {
      lo = hi = INFINITY;                       // the restored self pair
    } else {
      float acc = 0.f;
      const int64_t c0 = A.ref.p[c], c1 = A.ref.p[c + 1];
      for (int64_t a0 = c0; a0 < c1; a0 += 128) {
        int32_t r[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int64_t e = a0 + 32 * u + lane;
          r[u] = (e < c1) ? __ldg(A.ref.i + e) : -1;
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
        float f[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) f[u] = (qe[u] >= 0) ? __ldg(A.rf + a0 + 32 * u + lane) : 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (qe[u] >= 0) acc = fmaf(f[u], qv[qe[u]], acc);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      float key, err;
      key_and_bound(A.method, acc, nq_, Nq, A.rnnz[c], A.rnorm ? A.rnorm[c] : 0.f, key, err);
      lo = key - err;
      hi = key + err;
      if (!(fabsf(key) <= FLT_MAX) || !(err <= FLT_MAX)) { lo = -INFINITY; hi = INFINITY; }
    }
    if (lane == 0) {
      A.lo[ql * (int64_t)A.cap + t] = lo;
      A.hi[ql * (int64_t)A.cap + t] = hi;
    }
  }
}

// per query: T2 = k-th largest pessimistic key; compact the list in place to
// the candidates whose optimistic key reaches T2 - margin
__global__ void k_rescreen_select(RescreenArgs A) {
  extern __shared__ float lists[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = (int64_t)blockIdx.x * SELECT_WARPS + warp;
  if (ql >= A.nq) return;
  const int n = A.count[ql];
  if (n == 0) return;
  const int K = A.k;
  float* lst = lists + warp * K;
  const float* lo = A.lo + ql * (int64_t)A.cap;
  const float* hi = A.hi + ql * (int64_t)A.cap;
  int m = 0;
  for (int p0 = 0; p0 < n; p0 += 32) {
    const float v = p0 + lane < n ? lo[p0 + lane] : -INFINITY;
    const unsigned b = __ballot_sync(0xffffffffu, v > -INFINITY && (m < K || v > lst[K - 1]));
    if (b) warp_insert_desc(lst, K, m, b, v, lane);
  }
  const float T = (m == K) ? lst[K - 1] : -INFINITY;
  const float cut = T - ((T == -INFINITY || T == INFINITY) ? 0.f : fabsf(T) * (8.f * U32) + 1e-30f);
  int32_t* cl = A.cand + ql * (int64_t)A.cap;
  int w = 0;
  for (int p0 = 0; p0 < n; p0 += 32) {
    const int p = p0 + lane;
    const bool keep = p < n && hi[p] >= cut;
    const int32_t cv = p < n ? cl[p] : 0;
    const unsigned b = __ballot_sync(0xffffffffu, keep);
    __syncwarp();
    if (keep) cl[w + __popc(b & ((1u << lane) - 1u))] = cv;
    w += __popc(b);
    __syncwarp();
  }
  if (lane == 0) A.count[ql] = w;
}

}  // namespace

bool tensor_supported(int method) { return method == BINARY || method == COSINE || method == EUCLIDEAN; }

static int64_t tensor_ld(int32_t nrow) { return ((int64_t)nrow + 63) / 64 * 64; }

size_t tensor_cache_bytes(int32_t nrow, int64_t ncol) {
  return (size_t)tensor_ld(nrow) * (size_t)ncol * 2;
}

void tensor_cache_free(TensorCache* c, cudaStream_t s) {
  if (c && c->dense) cudaFreeAsync(c->dense, s);
  if (c && c->err) cudaFreeAsync(c->err, s);
  if (c && c->bn) cudaFreeAsync(c->bn, s);
  if (c) *c = TensorCache();
}

// Builds (or reuses) the dense FP16 copy of M's screen values for `method`
// from its ScreenCache; an allocation failure leaves it unusable (the FP32
// screen then runs) rather than failing the call.
static int ensure_tensor(TensorCache* t, int method, const DevCsc& M, const ColAux& aux, const ScreenCache* sc,
                         cudaStream_t s) {
  if (t->method == method) return 0;
  tensor_cache_free(t, s);
  t->method = method;
  t->ld = tensor_ld(M.nrow);
  const size_t bytes = tensor_cache_bytes(M.nrow, M.ncol) + 256;
  cudaError_t e = cudaMallocAsync(&t->dense, bytes, s);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    t->dense = nullptr;
    t->usable = 0;
    return 0;
  }
  SK(e);
  const size_t nbytes = sizeof(float) * ((size_t)M.ncol + 4);
  SK(cudaMallocAsync(&t->err, nbytes, s));
  SK(cudaMallocAsync(&t->bn, nbytes, s));
  int* bad = nullptr;
  SK(cudaMallocAsync(&bad, sizeof(int), s));
  SK(cudaMemsetAsync(bad, 0, sizeof(int), s));
  SK(cudaMemsetAsync(t->dense, 0, bytes, s));
  if (M.ncol > 0)
    k_tensor_fill<<<blocks_for(M.ncol * 32, 256), 256, 0, s>>>(
        M, sc->fval, (method == COSINE) ? aux.uval : (method == EUCLIDEAN) ? M.x : nullptr,
        static_cast<__half*>(t->dense), t->ld, t->err, t->bn, bad);
  int hbad = 0;
  SK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  SK(cudaStreamSynchronize(s));
  SK(cudaFreeAsync(bad, s));
  t->usable = hbad ? 0 : 1;
  if (!t->usable) {
    SK(cudaFreeAsync(t->dense, s));
    t->dense = nullptr;
  }
  return 0;
}

void launch_check_rows(const DevCsc& M, int* err, cudaStream_t s) {
  if (M.ncol > 0) k_check_rows<<<blocks_for(M.ncol, 128), 128, 0, s>>>(M, err);
}

bool screen_supported(int method, int k) {
  return (method == BINARY || method == COSINE || method == EUCLIDEAN || method == MANHATTAN || method == JS ||
          method == PEARSON || method == COVARIANCE) &&
         k >= 1 && k <= 1024;
}

static size_t table_bytes(int32_t nrow) { return (size_t)nrow * 4 + 16; }

bool screen_fits(int32_t nrow) {
  return nrow < (1 << 24) && table_bytes(nrow) + 4096 * 4 <= kSmemMax;
}

static int ensure_cache(ScreenCache* c, int method, const DevCsc& M, const ColAux& aux,
                        cudaStream_t s) {
  const int family = method;
  if (c->method == family) return 0;
  if (method == JS && !aux.xl) {                 // the js values' x log x come first
    g_screen_site = "js x log x values missing";
    return (int)cudaErrorInvalidValue;
  }
  if (c->blob) { SK(cudaFreeAsync(c->blob, s)); *c = ScreenCache(); }
  const int64_t nnz = M.ncol > 0 ? -1 : 0;
  (void)nnz;
  int64_t h_nnz = 0;
  if (M.ncol > 0) SK(cudaMemcpyAsync(&h_nnz, M.p + M.ncol, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  SK(cudaStreamSynchronize(s));
  // each array starts on a 256-byte boundary (16-byte vector loads of cnorm / nnz)
  auto seg = [](size_t bytes) { return (bytes + 255) & ~(size_t)255; };
  const size_t b_fval = seg(sizeof(float) * ((size_t)h_nnz + 4));
  const size_t b_col = seg(sizeof(float) * ((size_t)M.ncol + 4));
  const bool js = method == JS;
  const size_t bytes = (js ? 2 : 1) * b_fval + 3 * b_col + 256;
  SK(cudaMallocAsync(&c->blob, bytes, s));
  char* b = static_cast<char*>(c->blob);
  c->fval = reinterpret_cast<float*>(b);
  b += b_fval;
  if (js) {
    c->fxl = reinterpret_cast<float*>(b);
    b += b_fval;
  }
  int* range_err = reinterpret_cast<int*>(static_cast<char*>(c->blob) + bytes - 256);
  c->cnorm = reinterpret_cast<float*>(b);
  b += b_col;
  c->nnz = reinterpret_cast<int32_t*>(b);
  b += b_col;
  c->perm = reinterpret_cast<int32_t*>(b);
  c->nnz_total = h_nnz;
  if (M.ncol > 0) {
    SK(cudaMemsetAsync(range_err, 0, sizeof(int), s));
    k_screen_prep<<<blocks_for(M.ncol * 32, 256), 256, 0, s>>>(M, method, aux.uval, aux.xl, c->fval, c->fxl,
                                                                c->cnorm, c->nnz, range_err);
    // descending-nnz order of the columns (radix sort on 32-bit keys)
    uint32_t *k_in = nullptr, *k_out = nullptr;
    int32_t* ids = nullptr;
    void* tmp = nullptr;
    size_t tb = 0;
    SK(cudaMallocAsync(&k_in, sizeof(uint32_t) * M.ncol, s));
    SK(cudaMallocAsync(&k_out, sizeof(uint32_t) * M.ncol, s));
    SK(cudaMallocAsync(&ids, sizeof(int32_t) * M.ncol, s));
    k_iota_neg_nnz<<<blocks_for(M.ncol, 256), 256, 0, s>>>(c->nnz, M.ncol, k_in, ids);
    SK(cub::DeviceRadixSort::SortPairs(nullptr, tb, k_in, k_out, ids, c->perm, (int)M.ncol, 0, 32, s));
    SK(cudaMallocAsync(&tmp, tb + 16, s));
    SK(cub::DeviceRadixSort::SortPairs(tmp, tb, k_in, k_out, ids, c->perm, (int)M.ncol, 0, 32, s));
    SK(cudaFreeAsync(tmp, s));
    SK(cudaFreeAsync(k_in, s));
    SK(cudaFreeAsync(k_out, s));
    SK(cudaFreeAsync(ids, s));
  }
  SK(cudaGetLastError());
  c->values_ok = true;
  if ((js || method == PEARSON || method == COVARIANCE) && M.ncol > 0) {
    int h_err = 0;
    SK(cudaMemcpyAsync(&h_err, range_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SK(cudaStreamSynchronize(s));
    c->values_ok = h_err == 0;
  }
  c->method = family;
  return 0;
}

int screen_knn(cudaStream_t s, const ScreenRun& r, const DevCsc& ref, const ColAux& ra,
               ScreenCache* rc, TensorCache* rt, const DevCsc& qry, const ColAux& qa, ScreenCache* qc,
               TensorCache* qt, int32_t* d_idx, double* d_val, int64_t* stats, const ScreenHooks& hooks) {
  SKN((cudaError_t)ensure_cache(rc, r.method, ref, ra, s));
  SKN((cudaError_t)ensure_cache(qc, r.method, qry, qa, s));
  if ((r.method == JS || r.method == PEARSON || r.method == COVARIANCE) && !(rc->values_ok && qc->values_ok)) {
    // values outside the range the method's FP32 bound covers: every query exactly
    const int64_t lo = r.q_lo, hi = (r.q_hi < 0) ? qry.ncol : r.q_hi;
    if (hi > lo) hooks.exact_range(lo, hi - lo);
    return 0;
  }
  bool use_t = r.tensor && rt && qt && tensor_supported(r.method) && stc_supported(r.k);
  if (use_t) {
    SKN((cudaError_t)ensure_tensor(rt, r.method, ref, ra, rc, s));
    if (qt != rt) SKN((cudaError_t)ensure_tensor(qt, r.method, qry, qa, qc, s));
    use_t = rt->usable && qt->usable && rt->ld == qt->ld;
  }
  const int64_t nr = ref.ncol, nq = qry.ncol;
  const int32_t nrow = ref.nrow;
  const size_t tbytes = table_bytes(nrow);
  // row offsets are 16-bit: a tile holds at most 65,535 values (js keeps each
  // value's x log x beside it)
  const size_t vbytes = (r.method == JS) ? 8 : 4;
  const int vcap = (int)std::min<size_t>((kSmemMax - tbytes - 256) / vbytes, 65535);
  const int groups = (nrow + 63) / 64;

  // host copy of the query column sizes (tile formation)
  std::vector<int32_t> hq_nnz((size_t)nq);
  SK(cudaMemcpyAsync(hq_nnz.data(), qc->nnz, sizeof(int32_t) * nq, cudaMemcpyDeviceToHost, s));
  SK(cudaStreamSynchronize(s));
  const int64_t q_lo = r.q_lo, q_hi = (r.q_hi < 0) ? nq : r.q_hi;
  const int64_t out_ld = (r.out_ld < 0) ? nq : r.out_ld;

  // queries per screen pass: the FP32 sparse screen's slab S is chunk x nr
  // floats; the fused tensor screen writes no slab and takes 4,096 queries
  // (16 query groups of 256, about one CTA per SM at ~10 reference ranges)
  const int64_t sbudget = (int64_t)4 << 30;
  const int64_t ldS = nr;
  const int64_t chunk = use_t ? std::min<int64_t>(std::max<int64_t>(q_hi - q_lo, 1), 4096)
                              : std::max<int64_t>(QT, std::min<int64_t>(std::max<int64_t>(q_hi - q_lo, 1),
                                                                         sbudget / (4 * std::max<int64_t>(ldS, 1))));
  // the FP16 bound is wider than the FP32 one: room for more candidates
  const int cap = use_t ? std::max(512, std::min(16384, 64 * r.k + 256))
                        : std::max(256, std::min(8192, 16 * r.k + 64));
  float *rlo = nullptr, *rhi = nullptr;
  if (use_t) {
    SK(cudaMallocAsync(&rlo, sizeof(float) * (size_t)(chunk * cap + 4), s));
    SK(cudaMallocAsync(&rhi, sizeof(float) * (size_t)(chunk * cap + 4), s));
  }

  float* S = nullptr;
  int32_t *cand = nullptr, *count = nullptr, *over = nullptr, *qidx = nullptr, *ridx = nullptr;
  int32_t *tile_q = nullptr, *tile_n = nullptr;
  int* work = nullptr;
  double* rvals = nullptr;
  uint8_t* force = nullptr;
  const int64_t cslots = chunk * (int64_t)cap;
  if (!use_t) SK(cudaMallocAsync(&S, sizeof(float) * (size_t)(chunk * ldS + 4), s));
  SK(cudaMallocAsync(&cand, sizeof(int32_t) * (size_t)cslots, s));
  SK(cudaMallocAsync(&count, sizeof(int32_t) * (size_t)chunk, s));
  SK(cudaMallocAsync(&over, sizeof(int32_t) * (size_t)chunk, s));
  SK(cudaMallocAsync(&qidx, sizeof(int32_t) * (size_t)cslots, s));
  SK(cudaMallocAsync(&ridx, sizeof(int32_t) * (size_t)cslots, s));
  SK(cudaMallocAsync(&rvals, sizeof(double) * (size_t)cslots, s));
  SK(cudaMallocAsync(&tile_q, sizeof(int32_t) * (size_t)(chunk + 1), s));
  SK(cudaMallocAsync(&tile_n, sizeof(int32_t) * (size_t)(chunk + 1), s));
  SK(cudaMallocAsync(&work, sizeof(int), s));
  // cosine cannot bound an all-zero query (its convention value is not a dot
  // product): such queries go to the exact engine.
  if (r.method == COSINE && r.qry_empty) force = const_cast<uint8_t*>(r.qry_empty);

  const size_t smem = tbytes + (size_t)vcap * vbytes + 64;
  // a function attribute is per device: set on every call (cheap, thread-safe),
  // never cached process-wide
  SK(cudaFuncSetAttribute(k_screen<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax));
  SK(cudaFuncSetAttribute(k_screen<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax));
  SK(cudaFuncSetAttribute(k_screen<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax));
  int nsm = 152;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }

  std::vector<int> overflow_queries;
  for (int64_t q0 = q_lo; q0 < q_hi; q0 += chunk) {
    hooks.check_cancel();
    const int64_t nb = std::min(chunk, q_hi - q0);
    if (use_t) {
      // the fused tcgen05 screen: FP16 GEMM tiles of the block against every
      // reference with the FP16-bound selection in the epilogue
      StcRun T;
      T.method = r.method; T.k = r.k; T.selfmode = r.selfmode; T.include_self = r.include_self;
      T.ld = rt->ld; T.nr = nr; T.q0 = q0; T.nq = nb;
      T.rdense = static_cast<const __half*>(rt->dense); T.qdense = static_cast<const __half*>(qt->dense);
      T.rnnz = rc->nnz; T.rnorm = (r.method == EUCLIDEAN) ? rc->cnorm : nullptr;
      T.rerr = rt->err; T.rbn = rt->bn; T.ref_mask = r.ref_mask;
      T.qnnz = qc->nnz; T.qnorm = (r.method == EUCLIDEAN) ? qc->cnorm : nullptr;
      T.qerr = qt->err; T.qbn = qt->bn;
      T.qry_blank = r.qry_blank; T.qry_force = force;
      const int64_t ld = rt->ld;
      SK((cudaError_t)stc_screen(T, s, cand, count, over, cap, hooks.time_begin, hooks.time_end));
      if (nrow <= RS_MAX_NROW) {
        RescreenArgs R;
        R.method = r.method; R.k = r.k; R.ref = ref; R.qry = qry; R.rf = rc->fval; R.qf = qc->fval;
        R.rnnz = rc->nnz; R.rnorm = (r.method == EUCLIDEAN) ? rc->cnorm : nullptr;
        R.qnnz = qc->nnz; R.qnorm = (r.method == EUCLIDEAN) ? qc->cnorm : nullptr;
        R.q_begin = q0; R.nq = nb; R.selfmode = r.selfmode; R.cap = cap; R.cand = cand; R.count = count;
        R.lo = rlo; R.hi = rhi;
        const size_t rsmem = (size_t)RS_MAX_QV * 4 + (size_t)((nrow + 31) / 32) * 8;
        if (rsmem > 48 * 1024)
          SK(cudaFuncSetAttribute(k_rescreen, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem));
        k_rescreen<<<(unsigned)nb, RS_THREADS, rsmem, s>>>(R);
        const size_t ssm = sizeof(float) * (size_t)SELECT_WARPS * r.k;
        if (ssm > 48 * 1024)
          SK(cudaFuncSetAttribute(k_rescreen_select, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
        k_rescreen_select<<<blocks_for(nb, SELECT_WARPS), SELECT_WARPS * 32, ssm, s>>>(R);
        SK(cudaGetLastError());
      }
      stats[6] += 2 * ld * nr * nb;
    } else {
    // tiles: up to QT consecutive queries whose values fit the table
    std::vector<int32_t> tq, tn;
    int64_t j = 0;
    while (j < nb) {
      int n = 0;
      int64_t vals = 0;
      while (j + n < nb && n < QT) {
        const int64_t add = hq_nnz[(size_t)(q0 + j + n)];
        if (n > 0 && vals + add > vcap) break;
        vals += add;
        ++n;
      }
      if (vals > vcap) {                        // a single query too large for the table
        overflow_queries.push_back((int)(q0 + j));
        // leave its S rows unused: it is finished by the exact engine
      }
      tq.push_back((int32_t)j);
      tn.push_back(vals > vcap ? 0 : n);
      j += n;
    }
    const int ntiles = (int)tq.size();
    SK(cudaMemcpyAsync(tile_q, tq.data(), sizeof(int32_t) * ntiles, cudaMemcpyHostToDevice, s));
    SK(cudaMemcpyAsync(tile_n, tn.data(), sizeof(int32_t) * ntiles, cudaMemcpyHostToDevice, s));
    SK(cudaMemsetAsync(work, 0, sizeof(int), s));
    // reference parts: a part's screen data should stay in L2 while all SMs read it
    const int64_t ref_bytes = (rc->nnz_total + 1) * 8;
    int nparts = (int)std::max<int64_t>(1, (ref_bytes + (96ll << 20) - 1) / (96ll << 20));
    nparts = std::max(nparts, (2 * nsm + ntiles - 1) / ntiles);
    nparts = (int)std::min<int64_t>(nparts, std::max<int64_t>(1, nr / 64));
    const int64_t part_len = (nr + nparts - 1) / nparts;

    ScreenArgs A;
    A.method = r.method; A.nrow = nrow; A.groups = groups; A.vcap = vcap;
    A.rp = ref.p; A.ri = ref.i; A.rv = rc->fval; A.rxl = rc->fxl; A.rperm = rc->perm; A.nr = nr;
    A.qp = qry.p; A.qi = qry.i; A.qv = qc->fval; A.qxl = qc->fxl;
    A.tile_q = tile_q; A.tile_n = tile_n; A.q_begin = q0; A.ntiles = ntiles; A.nparts = nparts;
    A.part_len = part_len; A.S = S; A.work = work;
    const int grid = std::min<int64_t>((int64_t)nsm, (int64_t)ntiles * nparts);
    hooks.time_begin();
    if (r.method == MANHATTAN) k_screen<1><<<grid, SCREEN_THREADS, smem, s>>>(A);
    else if (r.method == JS) k_screen<2><<<grid, SCREEN_THREADS, smem, s>>>(A);
    else k_screen<0><<<grid, SCREEN_THREADS, smem, s>>>(A);
    hooks.time_end();
    SK(cudaGetLastError());

    SelectScreenArgs B;
    B.method = r.method; B.k = r.k; B.S = S; B.nr = nr; B.rperm = rc->perm;
    const bool normed = r.method == EUCLIDEAN || r.method == MANHATTAN || r.method == JS;
    B.rnnz = rc->nnz; B.rnorm = normed ? rc->cnorm : nullptr;
    B.qnnz = qc->nnz; B.qnorm = normed ? qc->cnorm : nullptr;
    B.rsum = ra.xsum; B.qsum = qa.xsum;
    B.rs = ra.s; B.rss = ra.ss; B.qs = qa.s; B.qss = qa.ss; B.nrow = ref.nrow;
    B.ref_mask = r.ref_mask; B.qry_blank = r.qry_blank; B.qry_force_exact = force;
    B.q_begin = q0; B.nq = nb; B.selfmode = r.selfmode; B.include_self = r.include_self;
    B.cap = cap; B.cand = cand; B.count = count; B.overflow = over;
    const size_t ssmem = sizeof(float) * (size_t)SELECT_WARPS * r.k;
    if (ssmem > 48 * 1024)
      SK(cudaFuncSetAttribute(k_screen_select, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssmem));
    k_screen_select<<<blocks_for(nb, SELECT_WARPS), SELECT_WARPS * 32, ssmem, s>>>(B);
    SK(cudaGetLastError());
    }

    // exact FP64 values of the kept pairs, then the exact top-k
    if (rerank_warp_supported(r.method)) {
      launch_rerank_warp(r.method, r.dist, ref, ra, qry, qa, cand, count, cap, nb, q0,
                         r.selfmode && r.include_self && r.method != COVARIANCE, r.self_value, rvals, s);
    } else {
      k_exact_candidates_prep<<<blocks_for(nb * cap, 256), 256, 0, s>>>(count, nb, cap, qidx,
                                                                          cand, ridx, q0);
      launch_exact_pairs_sparse(r.method, r.dist, ref, ra, qry, qa, ridx, qidx, nb * cap,
                                r.selfmode && r.include_self && r.method != COVARIANCE, r.self_value, rvals, s);
    }
    SelectArgs sa;
    sa.vals = rvals; sa.seg_stride = cap; sa.elem_stride = 1; sa.nseg = nb;
    sa.cand = cand; sa.cand_count = count; sa.cand_ld = cap;
    sa.seg_blank = r.qry_blank ? r.qry_blank + r.out_first : nullptr;
    sa.out_idx = d_idx; sa.out_val = d_val; sa.out_ld = out_ld; sa.out_row0 = q0 - r.out_first;
    sa.k = r.k; sa.decreasing = r.decreasing;
    launch_select(sa, s);
    SK(cudaGetLastError());

    std::vector<int32_t> h_over((size_t)nb), h_count((size_t)nb);
    SK(cudaMemcpyAsync(h_over.data(), over, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, s));
    SK(cudaMemcpyAsync(h_count.data(), count, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, s));
    SK(cudaStreamSynchronize(s));
    for (int64_t t = 0; t < nb; ++t) {
      if (h_over[(size_t)t]) overflow_queries.push_back((int)(q0 + t));
      stats[1] += h_count[(size_t)t];
    }
    stats[0] += nb * nr;
    stats[3] += 5;
  }
  std::sort(overflow_queries.begin(), overflow_queries.end());
  overflow_queries.erase(std::unique(overflow_queries.begin(), overflow_queries.end()),
                         overflow_queries.end());
  stats[2] += (int64_t)overflow_queries.size();
  if (S) SK(cudaFreeAsync(S, s));
  SK(cudaFreeAsync(cand, s)); SK(cudaFreeAsync(count, s));
  SK(cudaFreeAsync(over, s)); SK(cudaFreeAsync(qidx, s)); SK(cudaFreeAsync(ridx, s));
  SK(cudaFreeAsync(rvals, s)); SK(cudaFreeAsync(tile_q, s)); SK(cudaFreeAsync(tile_n, s));
  SK(cudaFreeAsync(work, s));
  if (rlo) SK(cudaFreeAsync(rlo, s));
  if (rhi) SK(cudaFreeAsync(rhi, s));
  // queries the screen could not bound: the exact slab engine, run by runs
  size_t a = 0;
  while (a < overflow_queries.size()) {
    size_t b = a + 1;
    while (b < overflow_queries.size() && overflow_queries[b] == overflow_queries[b - 1] + 1) ++b;
    hooks.exact_range(overflow_queries[a], (int64_t)(b - a));
    a = b;
  }
  return 0;
}

void screen_cache_free(ScreenCache* c, cudaStream_t s) {
  if (c && c->blob) cudaFreeAsync(c->blob, s);
  if (c) *c = ScreenCache();
}

const char* screen_error_site() { return g_screen_site; }

}  // namespace sdg
