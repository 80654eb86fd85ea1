// sdg_sparse_tc.cu -- the tensor-core screen of the sparse path on tcgen05,
// with the bound-based selection fused into the epilogue (no slab in HBM).
//
// Operands are the dense FP16 copies of the screen values (TensorCache: one
// column of ld = nrow rounded up to 64 halves per matrix column, K-major).
// A CTA owns 256 query columns (two 128-row UMMA A tiles) and a range of
// reference tiles of 256 columns.  For every reference tile the K dimension
// (all ld rows) streams through a three-stage TMA ring of 64-row chunks
// (A: 2 x 128 x 64, B: 256 x 64 FP16, SWIZZLE_128B, 64 KB a stage); one
// thread issues tcgen05.mma.kind::f16 (M = 128, N = 256, K = 16, FP16 in,
// FP32 accumulate) into two TMEM accumulators of 128 lanes x 256 columns, all
// 512 columns.  The K loop of a tile is hundreds of chunks long at the sizes
// this screen is chosen for, so the epilogue's drain of a finished tile (the
// only time the tensor pipe waits) costs about 1 % and no second accumulator
// is kept.
//
// Epilogue: eight warps, one thread per query (warp w reads TMEM lanes
// 32 (w % 4) .. + 31 of query tile (w - 2) / 4).  A thread keeps the top k
// pessimistic keys of its reference range in registers and appends every
// reference whose optimistic key reaches its running cut tcb::tc_cut(T) to a
// per-(query, range) list.  The keys are tcb::tc_bounds of the GEMM value,
// the same FP32 arithmetic as the slab selection, and the running cut (the
// k-th best of a subset, tc_cut increasing in T) never exceeds the final one,
// so the union of the lists holds every reference the slab selection keeps;
// k_stc_merge applies the final cut per query.
//
// Hot test.  Before the exact bounds, a thread tests x = a s - b w[r] >= C
// with per-thread a, b, C derived from its running cut and from the largest
// per-column error terms of the tile (tile maxima of err, bn and sqrt(Nr)),
// so that hi >= cut implies the test passes; only references passing it (and
// the query's own column in a self-search) get their exact bounds:
//   cosine     x = s                       C = cut - E - slack
//   euclidean  x = 2 s - (1 - 2^-20) Nr    C = cut + (1 - 2^-20) Nq - E - slack
//   binary     x = alpha s - beta nr       C = beta nq - 1e-6 - slack
// (binary: beta = c' / (1 + c'), c' = (cut - 1e-30) / (1 + 2^-22) the Jaccard
// cut before its final rounding, alpha = 1 + 1.01 acc_q bounds the count's
// accumulation allowance; every test passes while cut <= 0).  The slack,
// 2^-12 of the terms' magnitudes, is far above the FP32 rounding of x, C and
// of the keys.  With usable FP16 copies every GEMM value is finite (|b| <=
// 65504 over at most 2^24 rows), so no key is NaN.
//
// Warp roles (320 threads): warp 0 TMA producer, warp 1 TMEM allocator + MMA
// issuer, warps 2..9 epilogue.  Every mbarrier wait is bounded (1 s of
// %globaltimer, sdg_tc_ptx.cuh); a wait that runs out sets *status, and the
// CTA drains its copies and MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>

#include "../../include/sdgpu.h"
#include "sdg_kernels.h"
#include "sdg_screen.h"
#include "sdg_tc_bounds.cuh"
#include "sdg_tc_ptx.cuh"

namespace sdg {
namespace {

using namespace tc;

constexpr int BM = 128;                 // queries per UMMA tile (TMEM lanes)
constexpr int BN = 256;                 // references per tile (UMMA N)
constexpr int BK = 64;                  // rows of a K chunk: 64 FP16 = one 128-byte swizzle row
constexpr int QT = 2;                   // query tiles per CTA
constexpr int STAGES = 3;
constexpr int THREADS = 320;
constexpr int KMAX = 64;                // largest k of the fused screen
constexpr int ECAP = 1024;              // appended references per (query, range)
constexpr uint32_t A_BYTES = BM * BK * 2;              // 16 KB
constexpr uint32_t B_BYTES = BN * BK * 2;              // 32 KB
constexpr uint32_t STAGE_BYTES = QT * A_BYTES + B_BYTES;
constexpr uint32_t TMEM_COLS = QT * BN;                // 512: both accumulators
// 1 KB alignment slack, the ring, barriers
constexpr size_t SMEM_BYTES = 1024 + (size_t)STAGES * STAGE_BYTES + 256;
constexpr uint32_t IDESC = idesc_f16(BM, BN, false);   // FP16 A and B
constexpr float SLACK = 2.44140625e-4f;                // 2^-12
constexpr float ONE_M20 = 0.99999904632568359375f;     // 1 - 2^-20

struct SArgs {
  int method, k, kch, nqg, nrr, tiles_per_range;
  int selfmode, include_self;
  int64_t nr, q0, nq, ntiles;              // q0: global index of the block's first query
  const int32_t* rnnz;
  const float* rnorm;                      // euclidean: sum of squares; else null
  const float* rerr;
  const float* rbn;
  const uint8_t* ref_mask;                 // excluded references (or null)
  const float* w;                          // [ntiles * BN]: hot-test weight, +inf past nr
  const float* tmax;                       // [ntiles][3]: max err, max bn, max sqrt(Nr)
  const int32_t* qnnz;
  const float* qnorm;
  const float* qerr;
  const float* qbn;
  const uint8_t* qskip;                    // [nq]: queries without a list (blank / forced exact)
  float* lists;                            // [nq][nrr][k]
  int32_t* ecount;                         // [nq][nrr]
  int32_t* eidx;                           // [nq][nrr][ECAP]
  float* ehi;
  int* status;
  int stall;                               // failure-detection test: the MMA issuer's first wait never completes
};

// Per-thread hot-test coefficients (x = a s - b w >= C) for running cut `cut`
// and the tile's error maxima.
struct Hot {
  float a, b, C;
};

__device__ __forceinline__ Hot hot_test(int method, float cut, float eq, float bq, float accq, float Nq, int32_t nq_,
                                        float ER, float BR, float SNR) {
  Hot h;
  if (cut == -INFINITY) { h.a = 1.f; h.b = 0.f; h.C = -INFINITY; return h; }
  if (method == COSINE) {
    const float E = (1.000001f * eq + bq * ER + accq * bq * BR) * 1.01f + 1e-12f;
    h.a = 1.f; h.b = 0.f;
    h.C = cut - E - SLACK * (fabsf(cut) + 1.f);
  } else if (method == EUCLIDEAN) {
    const float E = 2.f * (SNR * 1.000001f * eq + bq * ER + accq * bq * BR) * 1.01f + 1e-30f;
    h.a = 2.f; h.b = ONE_M20;
    h.C = cut + ONE_M20 * Nq - E - SLACK * (fabsf(cut) + 2.f * Nq + E);
  } else {
    const float cp = (cut - 1e-30f) / (1.f + 4.f * tcb::U32);
    if (!(cp > 0.f)) { h.a = 1.f; h.b = 0.f; h.C = -INFINITY; return h; }
    const float beta = cp / (1.f + cp);
    h.a = 1.f + 1.01f * accq; h.b = beta;
    h.C = beta * (float)nq_ - 1e-6f - SLACK * (2.f * beta * (float)nq_ + 1.f);
  }
  return h;
}

template <int KL>
__global__ void __launch_bounds__(THREADS, 1) k_sparse_tc(const __grid_constant__ CUtensorMap qmap,
                                                        const __grid_constant__ CUtensorMap rmap, SArgs P) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(base + (size_t)STAGES * STAGE_BYTES);
  uint64_t* full = bars;
  uint64_t* emptyb = bars + STAGES;
  uint64_t* acc_full = bars + 2 * STAGES;
  uint64_t* acc_empty = acc_full + 1;
  uint64_t* mma_done = acc_empty + 1;
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qg = blockIdx.x % P.nqg, rr = blockIdx.x / P.nqg;
  const int qbase = qg * (QT * BM);                 // local index of the CTA's first query
  const int64_t t0 = (int64_t)rr * P.tiles_per_range;
  const int64_t t1 = min(P.ntiles, t0 + (int64_t)P.tiles_per_range);
  const int ntile = (int)max((int64_t)0, t1 - t0);
  const int kch = P.kch;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) { mbar_init(full + s, 1); mbar_init(emptyb + s, 1); }
    mbar_init(acc_full, 1);
    mbar_init(acc_empty, 8);
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(tmem_slot, TMEM_COLS);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---- TMA producer ----
    if (lane == 0 && ntile > 0) {
      prefetch_map(&qmap);
      prefetch_map(&rmap);
      int it = 0;
      bool ok = true;
      for (int j = 0; j < ntile && ok; ++j) {
        const int rcol = (int)((t0 + j) * BN);
        for (int c = 0; c < kch; ++c, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
          if (!mbar_wait(emptyb + s, ph ^ 1u, abort_flag, P.status)) { ok = false; break; }
          uint8_t* st = base + (size_t)s * STAGE_BYTES;
          mbar_expect_tx(full + s, STAGE_BYTES);
          tma_load_2d(st, &qmap, full + s, c * BK, qbase);
          tma_load_2d(st + A_BYTES, &qmap, full + s, c * BK, qbase + BM);
          tma_load_2d(st + 2 * A_BYTES, &rmap, full + s, c * BK, rcol);
        }
      }
      // every issued copy lands before the CTA can exit
      for (int x = max(0, it - STAGES); x < it; ++x) mbar_drain(full + x % STAGES, (uint32_t)(x / STAGES) & 1u);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0 && ntile > 0) {
      int it = 0;
      bool ok = true;
      for (int j = 0; j < ntile && ok; ++j) {
        // the epilogue has drained tile j - 1
        // (with P.stall the first wait asks for the phase the epilogue has not
        // begun, so it runs out: the failure-detection test's path)
        const uint32_t flip = (P.stall && j == 0) ? 0u : 1u;
        if (!mbar_wait(acc_empty, ((uint32_t)j & 1u) ^ flip, abort_flag, P.status)) break;
        fence_after();
        for (int c = 0; c < kch; ++c, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
          if (!mbar_wait(full + s, ph, abort_flag, P.status)) { ok = false; break; }
          fence_after();
          const uint32_t a0 = smem_u32(base + (size_t)s * STAGE_BYTES);
          const uint32_t a1 = a0 + A_BYTES, b = a0 + 2 * A_BYTES;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            const uint64_t bd = sw128_desc(b + kk * 32);
            const uint32_t acc = (c | kk) != 0;
            umma_f16(tmem, sw128_desc(a0 + kk * 32), bd, IDESC, acc);
            umma_f16(tmem + BN, sw128_desc(a1 + kk * 32), bd, IDESC, acc);
          }
          umma_commit(emptyb + s);            // the stage is free once these MMAs have read it
        }
        if (!ok) break;
        umma_commit(acc_full);                // tile j's accumulators are complete
      }
      // all issued MMAs complete before TMEM is freed
      umma_commit(mma_done);
      mbar_drain(mma_done, 0);
    }
    __syncwarp();
  } else {
    // ---- epilogue: one thread per query ----
    const int qt = (warp - 2) >> 2, quarter = warp & 3;
    const int row = quarter * 32 + lane;
    const int64_t ql = (int64_t)qbase + qt * BM + row;
    const int64_t q = P.q0 + ql;
    const int K = P.k;
    bool active = ql < P.nq;
    if (active) active = !P.qskip[ql];
    float eq = 0.f, bq = 0.f, Nq = 0.f, accq = 0.f;
    int32_t nq_ = 0;
    if (active) {
      eq = P.qerr[q];
      bq = P.qbn[q];
      nq_ = P.qnnz[q];
      Nq = P.qnorm ? P.qnorm[q] : 0.f;
      accq = ((float)nq_ + 64.f) * tcb::ACC_ULP;
    }
    // this thread's top k pessimistic keys, sorted descending, in registers:
    // KL - k leading +inf sentinels, so that lst[KL - 1] is the k-th best
    float lst[KL];
#pragma unroll
    for (int i = 0; i < KL; ++i) lst[i] = (i < KL - K) ? INFINITY : -INFINITY;
    float T = -INFINITY, cut = -INFINITY;
    int cnt = 0;
    const int64_t slot = active ? (ql * P.nrr + rr) : 0;
    int32_t* my_idx = P.eidx + slot * ECAP;
    float* my_hi = P.ehi + slot * ECAP;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    const bool use_w = P.method != COSINE;
    for (int j = 0; j < ntile; ++j) {
      const bool ok = mbar_wait(acc_full, (uint32_t)j & 1u, abort_flag, P.status);
      if (!__all_sync(0xffffffffu, ok)) break;     // the warp leaves together (tcgen05.ld is .aligned)
      fence_after();
      const int64_t tt = t0 + j;
      float ER = 0.f, BR = 0.f, SNR = 0.f;
      if (active) { ER = P.tmax[3 * tt]; BR = P.tmax[3 * tt + 1]; SNR = P.tmax[3 * tt + 2]; }
      Hot h = hot_test(P.method, cut, eq, bq, accq, Nq, nq_, ER, BR, SNR);
#pragma unroll 1
      for (int hh = 0; hh < BN / 32; ++hh) {
        uint32_t v[32];
        tmem_ld32(tmem + lane_base + (uint32_t)(qt * BN + hh * 32), v);
        if (!active) continue;
        const int64_t r0 = tt * BN + hh * 32;
        uint32_t mask = 0;
        if (use_w) {
          const float4* w4 = reinterpret_cast<const float4*>(P.w + r0);
#pragma unroll
          for (int j4 = 0; j4 < 8; ++j4) {
            const float4 ww = __ldg(w4 + j4);
            const float wv[4] = {ww.x, ww.y, ww.z, ww.w};
#pragma unroll
            for (int t = 0; t < 4; ++t)
              if (fmaf(-h.b, wv[t], h.a * __uint_as_float(v[4 * j4 + t])) >= h.C) mask |= 1u << (4 * j4 + t);
          }
        } else {
#pragma unroll
          for (int t = 0; t < 32; ++t)
            if (__uint_as_float(v[t]) >= h.C) mask |= 1u << t;
        }
        // the query's own column always gets its exact bounds (the restored self pair)
        if (P.selfmode && q >= r0 && q < r0 + 32) mask |= 1u << (int)(q - r0);
        while (mask) {
          const int jj = __ffs(mask) - 1;
          mask &= mask - 1;
          const int64_t r = r0 + jj;
          if (r >= P.nr || (P.ref_mask && P.ref_mask[r])) continue;
          float lo, hi;
          if (P.selfmode && r == q) {
            if (!P.include_self) continue;
            lo = hi = INFINITY;
          } else {
            float s = 0.f;
#pragma unroll
            for (int t = 0; t < 32; ++t) s = (t == jj) ? __uint_as_float(v[t]) : s;
            tcb::tc_bounds(P.method, s, nq_, Nq, P.rnnz[r], P.rnorm ? P.rnorm[r] : 0.f, eq, bq, P.rerr[r], P.rbn[r],
                           lo, hi);
          }
          if (hi >= cut) {
            if (cnt < ECAP) { my_idx[cnt] = (int32_t)r; my_hi[cnt] = hi; }
            ++cnt;
          }
          if (lo > T) {
            // sorted insert: the new lst[i] is the median of lst[i - 1], lo, lst[i]
#pragma unroll
            for (int i = KL - 1; i > 0; --i) lst[i] = fmaxf(lst[i], fminf(lst[i - 1], lo));
            lst[0] = fmaxf(lst[0], lo);
            T = lst[KL - 1];
            cut = tcb::tc_cut(T);
            h = hot_test(P.method, cut, eq, bq, accq, Nq, nq_, ER, BR, SNR);
          }
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty);
    }
    if (active) {
      float* out = P.lists + slot * K;
#pragma unroll
      for (int i = 0; i < KL; ++i)
        if (i >= KL - K) out[i - (KL - K)] = lst[i];
      P.ecount[slot] = cnt;
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 1) tmem_dealloc(tmem, TMEM_COLS);
}

// Per reference tile: the largest err, bn and sqrt(Nr) of its columns (the
// hot test's error maxima), and the hot-test weight of each column (Nr for
// euclidean, nnz for binary, +inf past the last column).  One warp per tile.
__global__ void k_stc_prep(int method, int64_t nr, int64_t ntiles, const int32_t* rnnz, const float* rnorm,
                           const float* rerr, const float* rbn, float* w, float* tmax) {
  const int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= ntiles) return;
  float me = 0.f, mb = 0.f, mn = 0.f;
  for (int c = lane; c < BN; c += 32) {
    const int64_t r = t * BN + c;
    float wv = INFINITY;
    if (r < nr) {
      me = fmaxf(me, rerr[r]);
      mb = fmaxf(mb, rbn[r]);
      if (rnorm) mn = fmaxf(mn, sqrtf(rnorm[r]) * 1.000001f);
      wv = (method == EUCLIDEAN) ? rnorm[r] : (method == BINARY) ? (float)rnnz[r] : 0.f;
    }
    w[r] = wv;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    me = fmaxf(me, __shfl_xor_sync(0xffffffffu, me, o));
    mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    mn = fmaxf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  }
  if (lane == 0) { tmax[3 * t] = me; tmax[3 * t + 1] = mb; tmax[3 * t + 2] = mn; }
}

// qskip[ql] = 1 for the block's queries that get no list: blank rows (written
// all NA) and queries the exact engine finishes (forced)
__global__ void k_stc_skip(int64_t nb, int64_t q0, const uint8_t* blank, const uint8_t* force, uint8_t* qskip) {
  const int64_t ql = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (ql >= nb) return;
  const int64_t q = q0 + ql;
  qskip[ql] = ((blank && blank[q]) || (force && force[q])) ? 1 : 0;
}

// ---- merge: the final cut of each query over its ranges ---------------------
constexpr int MW = 8;   // warps per block

__device__ __forceinline__ void warp_insert_desc_m(float* lst, int K, int& n, unsigned m, float v, int lane) {
  while (m) {
    const int src = __ffs(m) - 1;
    m &= m - 1;
    const float x = __shfl_sync(0xffffffffu, v, src);
    if (n == K && !(x > lst[K - 1])) continue;
    int a = 0, b = n;
    while (a < b) { const int mid = (a + b) >> 1; if (lst[mid] >= x) a = mid + 1; else b = mid; }
    const int last = (n < K) ? n : K - 1;
    if (lane == 0) {                               // K <= 64: a serial shift is short
      for (int e = last; e > a; --e) lst[e] = lst[e - 1];
      lst[a] = x;
    }
    __syncwarp();
    if (n < K) ++n;
  }
}

// Per query: T = the k-th largest pessimistic key over the ranges' lists (the
// exact k-th over all references: the top k of a union is the top k of the
// parts' top k), cut = tc_cut(T); the candidates are the appended references
// with hi >= cut, in the slab selection's format (cand / count / over).
__global__ void k_stc_merge(int64_t q0, int64_t nq, int nrr, int K, const uint8_t* blank, const uint8_t* force,
                            const float* lists, const int32_t* ecount, const int32_t* eidx, const float* ehi, int cap,
                            int32_t* cand, int32_t* count, int32_t* over) {
  __shared__ float sl[MW][KMAX];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = (int64_t)blockIdx.x * MW + warp;
  if (ql >= nq) return;
  const int64_t q = q0 + ql;
  const bool is_blank = blank && blank[q], is_forced = force && force[q];
  if (is_blank || is_forced) {
    if (lane == 0) { count[ql] = 0; over[ql] = (is_forced && !is_blank) ? 1 : 0; }
    return;
  }
  float* lst = sl[warp];
  int n = 0;
  const float* in = lists + ql * nrr * (int64_t)K;
  const int64_t tot = (int64_t)nrr * K;
  for (int64_t p0 = 0; p0 < tot; p0 += 32) {
    const float v = p0 + lane < tot ? in[p0 + lane] : -INFINITY;
    const unsigned m = __ballot_sync(0xffffffffu, v > -INFINITY && (n < K || v > lst[K - 1]));
    if (m) warp_insert_desc_m(lst, K, n, m, v, lane);
  }
  const float cut = tcb::tc_cut((n == K) ? lst[K - 1] : -INFINITY);
  bool ovf = false;
  int total = 0;
  int32_t* out = cand + ql * (int64_t)cap;
  for (int r = 0; r < nrr && !ovf; ++r) {
    const int64_t slot = ql * nrr + r;
    const int c = ecount[slot];
    if (c > ECAP) { ovf = true; break; }
    for (int p0 = 0; p0 < c; p0 += 32) {
      const int p = p0 + lane;
      const bool keep = p < c && ehi[slot * ECAP + p] >= cut;
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      const int rank = __popc(m & ((1u << lane) - 1u));
      if (keep && total + rank < cap) out[total + rank] = eidx[slot * ECAP + p];
      total += __popc(m);
    }
    if (total > cap) ovf = true;
  }
  if (lane == 0) { count[ql] = ovf ? 0 : total; over[ql] = ovf ? 1 : 0; }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult qr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &qr) ==
            cudaSuccess &&
        qr == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

}  // namespace

bool stc_supported(int k) { return k >= 1 && k <= KMAX && encode_fn() != nullptr; }

int stc_screen(const StcRun& R, cudaStream_t s, int32_t* cand, int32_t* count, int32_t* over, int cap,
               const std::function<void()>& time_begin, const std::function<void()>& time_end) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) { set_error("cuTensorMapEncodeTiled is unavailable"); return (int)cudaErrorNotSupported; }
  const int64_t ld = R.ld, nr = R.nr, nb = R.nq;
  // one map per operand: K-major FP16 columns of ld rows (a multiple of 64);
  // boxes of 64 rows x 128 query columns / 256 reference columns; columns past
  // the end read as zero
  auto encode = [&](const __half* base_ptr, int64_t ncols, int box_cols, CUtensorMap* map) {
    const cuuint64_t gdim[2] = {(cuuint64_t)ld, (cuuint64_t)ncols};
    const cuuint64_t gstride[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_cols};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, (void*)base_ptr, gdim, gstride, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  CUtensorMap qmap, rmap;
  if (!encode(R.qdense + R.q0 * ld, nb, BM, &qmap) || !encode(R.rdense, nr, BN, &rmap)) {
    set_error("cuTensorMapEncodeTiled failed");
    return (int)cudaErrorInvalidValue;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) sms = 1;
  const int nqg = (int)((nb + QT * BM - 1) / (QT * BM));
  const int64_t ntiles = (nr + BN - 1) / BN;
  int nrr = std::max(1, sms / nqg);
  nrr = (int)std::min<int64_t>(nrr, ntiles);
  const int tpr = (int)((ntiles + nrr - 1) / nrr);
  nrr = (int)((ntiles + tpr - 1) / tpr);

  float *w = nullptr, *tmax = nullptr, *lists = nullptr, *ehi = nullptr;
  int32_t *ecount = nullptr, *eidx = nullptr;
  int* status = nullptr;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  chk(cudaMallocAsync(&w, sizeof(float) * (size_t)(ntiles * BN), s));
  chk(cudaMallocAsync(&tmax, sizeof(float) * (size_t)(ntiles * 3), s));
  chk(cudaMallocAsync(&lists, sizeof(float) * (size_t)(nb * nrr * R.k), s));
  chk(cudaMallocAsync(&ecount, sizeof(int32_t) * (size_t)(nb * nrr), s));
  chk(cudaMallocAsync(&eidx, sizeof(int32_t) * (size_t)(nb * nrr * ECAP), s));
  chk(cudaMallocAsync(&ehi, sizeof(float) * (size_t)(nb * nrr * ECAP), s));
  chk(cudaMallocAsync(&status, sizeof(int), s));
  uint8_t* qskip = nullptr;
  chk(cudaMallocAsync(&qskip, (size_t)nb + 16, s));
  int hstatus = 0;
  if (e == cudaSuccess) {
    chk(cudaMemsetAsync(status, 0, sizeof(int), s));
    chk(cudaMemsetAsync(ecount, 0, sizeof(int32_t) * (size_t)(nb * nrr), s));
    k_stc_prep<<<(unsigned)((ntiles * 32 + 255) / 256), 256, 0, s>>>(R.method, nr, ntiles, R.rnnz, R.rnorm, R.rerr,
                                                                      R.rbn, w, tmax);
    SArgs P;
    P.method = R.method; P.k = R.k; P.kch = (int)(ld / BK); P.nqg = nqg; P.nrr = nrr; P.tiles_per_range = tpr;
    P.selfmode = R.selfmode; P.include_self = R.include_self;
    P.nr = nr; P.q0 = R.q0; P.nq = nb; P.ntiles = ntiles;
    P.rnnz = R.rnnz; P.rnorm = R.rnorm; P.rerr = R.rerr; P.rbn = R.rbn; P.ref_mask = R.ref_mask;
    P.w = w; P.tmax = tmax;
    P.qnnz = R.qnnz; P.qnorm = R.qnorm; P.qerr = R.qerr; P.qbn = R.qbn;
    P.qskip = qskip;
    P.lists = lists; P.ecount = ecount; P.eidx = eidx; P.ehi = ehi; P.status = status;
    P.stall = tc_take_stall() ? 1 : 0;
    k_stc_skip<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(nb, R.q0, R.qry_blank, R.qry_force, qskip);
    const int k = R.k;
    auto kern = (k <= 16) ? k_sparse_tc<16> : (k <= 32) ? k_sparse_tc<32> : k_sparse_tc<64>;
    chk(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    if (e == cudaSuccess) {
      time_begin();
      kern<<<(unsigned)(nqg * nrr), THREADS, SMEM_BYTES, s>>>(qmap, rmap, P);
      time_end();
    }
    chk(cudaGetLastError());
    k_stc_merge<<<(unsigned)((nb + MW - 1) / MW), MW * 32, 0, s>>>(R.q0, nb, nrr, k, R.qry_blank, R.qry_force,
                                                                    lists, ecount, eidx, ehi, cap, cand, count,
                                                                    over);
    chk(cudaGetLastError());
    chk(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    chk(cudaStreamSynchronize(s));
  }
  for (void* p : {(void*)w, (void*)tmax, (void*)lists, (void*)ecount, (void*)eidx, (void*)ehi, (void*)status,
                  (void*)qskip})
    if (p) cudaFreeAsync(p, s);
  if (e != cudaSuccess) return (int)e;
  if (hstatus) {
    set_error("tensor-core screen: a pipeline wait timed out");
    return (int)cudaErrorLaunchTimeout;
  }
  return 0;
}

namespace {
std::atomic<int> g_stall{0};
}
void tc_set_stall(int n) { g_stall.store(n > 0 ? n : 0); }
bool tc_take_stall() {
  int v = g_stall.load();
  while (v > 0 && !g_stall.compare_exchange_weak(v, v - 1)) {}
  return v > 0;
}

}  // namespace sdg
