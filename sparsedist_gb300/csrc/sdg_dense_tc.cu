// sdg_dense_tc.cu -- the dense screen fused on the 5th-generation tensor cores.
//
// The BF16 screen of the dense path without a slab in HBM: each CTA owns 256
// query columns (two 128-row UMMA A tiles, resident in shared memory) and a
// range of reference columns, streamed by TMA in 128-column x 64-row K chunks
// (SWIZZLE_128B, five-stage ring).  One thread issues tcgen05.mma
// (M = 128 queries, N = 128 references, K = 16, BF16 in, FP32 accumulate) into
// TMEM: two query tiles x two accumulator buffers = 4 x 128 = 512 columns, so
// the MMAs of reference tile j + 1 run while eight epilogue warps read tile j
// back with tcgen05.ld.  An epilogue thread owns one query: it keeps the top k
// pessimistic keys of its reference range in shared memory and appends every
// reference whose optimistic key reaches its running cut to a per-(query,
// range) candidate list.  The running cut is the k-th best of a subset, never
// above the query's final cut, so the union of the lists holds every reference
// that the slab screen keeps; k_tc_merge applies the final cut (the k-th best
// over all ranges' lists) exactly as the slab screen does.
//
// Hot test.  An epilogue thread first tests x = a s - w[r] against one
// threshold e_thr per query (a = 1, w = 0 for cosine; a = 2,
// w = (1 - c) Nr for euclidean, c = rel + 2^-20; w = +inf for degenerate and
// padding references), and only references passing it get their exact key
// bounds.  For euclidean 2 rel sqrt(Nq Nr) <= rel (Nq + Nr), so
// hi <= 2 s - (1 - c)(Nq + Nr) + 1e-30 and hi >= cut implies
// x >= cut + (1 - c) Nq; for cosine hi = s + rel.  e_thr subtracts 2^-12
// (|cut| + Nq) (euclidean) or 2^-12 (|cut| + 1) (cosine) more, far above the
// FP32 rounding of x.
//
// Warp roles (320 threads): warp 0 TMA producer, warp 1 TMEM allocator + MMA
// issuer, warps 2..9 epilogue (warp w reads TMEM lanes 32 (w % 4) .. + 31, of
// query tile (w - 2) / 4).  Every mbarrier wait is bounded (1 s of
// %globaltimer); a wait that runs out sets *status, raises the CTA's abort
// flag, and the CTA drains its own copies and MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>
#include <cmath>

#include "../../include/sdgpu.h"
#include "sdg_dense.h"
#include "sdg_tc_ptx.cuh"

namespace sdg {
namespace {

constexpr int BM = 128;                 // queries per UMMA tile (TMEM lanes)
constexpr int BN = 128;                 // references per tile (UMMA N)
constexpr int BK = 64;                  // rows of a K chunk: 64 BF16 = one 128-byte swizzle row
constexpr int QT = 2;                   // query tiles per CTA
constexpr int STAGES = 5;               // reference chunk ring
constexpr int NB = 8;                   // buffered passing references per epilogue thread
constexpr int EPI_THREADS = 256;
constexpr int KT = 64;                  // largest k of the fused screen
constexpr int THREADS = 320;
constexpr uint32_t TILE_BYTES = BN * BK * 2;   // 16 KB (a 128 x 64 BF16 tile)
constexpr uint32_t TMEM_COLS = 512;
constexpr int MAX_DCH = 4;              // dpad <= 256
// 1 KB alignment slack, A tiles, B ring, barriers
constexpr size_t SMEM_BYTES = 1024 + (size_t)(QT * MAX_DCH + STAGES) * TILE_BYTES + (size_t)NB * EPI_THREADS * 8 + 256;

struct TcArgs {
  int method, k, dch, nqg, nrr, tiles_per_range, ecap;
  int self;                   // queries are columns of the reference (skip r == q)
  int32_t d;
  int64_t n, q0, nq, ntiles;
  float a;                    // x = a * s - w[r] (1 cosine, 2 euclidean)
  float one_minus_c;          // euclidean hot-test coefficient
  const float* w;             // [npad]: +inf for degenerate / padding references
  const float* norm2;         // [npad] reference sums of squares
  const float* qnorm2;        // query sums of squares
  const uint8_t* qempty;      // degenerate queries (no list)
  float* lists;               // [nq][nrr][k]
  int32_t* ecount;            // [nq][nrr]
  int32_t* eidx;              // [nq][nrr][ecap]
  float* ehi;                 // [nq][nrr][ecap]
  int* status;
};

using namespace tc;
constexpr uint32_t IDESC = idesc_f16(BM, BN, true);

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accum) {
  umma_f16(d_tmem, adesc, bdesc, IDESC, accum);
}

// ---- the fused screen ------------------------------------------------------
template <int KL>
__global__ void __launch_bounds__(THREADS, 1) k_dense_tc(const __grid_constant__ CUtensorMap qmap,
                                                       const __grid_constant__ CUtensorMap rmap, TcArgs P) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = base;                                    // QT * dch tiles
  uint8_t* sB = base + (size_t)QT * MAX_DCH * TILE_BYTES;  // STAGES tiles
  // per epilogue thread NB (reference, GEMM value) slots, slot-major so that a
  // warp's accesses to one slot are conflict-free
  int32_t* buf_r = (int32_t*)(sB + (size_t)STAGES * TILE_BYTES);
  float* buf_s = (float*)(buf_r + NB * EPI_THREADS);
  uint64_t* bars = (uint64_t*)(buf_s + NB * EPI_THREADS);
  uint64_t* full = bars;
  uint64_t* emptyb = bars + STAGES;
  uint64_t* acc_full = bars + 2 * STAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* a_full = acc_empty + 2;
  uint64_t* mma_done = a_full + 1;
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qg = blockIdx.x % P.nqg, rr = blockIdx.x / P.nqg;
  const int64_t qbase = P.q0 + (int64_t)qg * (QT * BM);
  const int64_t t0 = (int64_t)rr * P.tiles_per_range;
  const int64_t t1 = min(P.ntiles, t0 + (int64_t)P.tiles_per_range);
  const int ntile = (int)max((int64_t)0, t1 - t0);
  const int dch = P.dch;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) { mbar_init(full + s, 1); mbar_init(emptyb + s, 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(acc_full + b, 1); mbar_init(acc_empty + b, 8); }
    mbar_init(a_full, 1);
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(tmem_slot)), "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---- TMA producer ----
    if (lane == 0 && ntile > 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&qmap) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&rmap) : "memory");
      mbar_expect_tx(a_full, (uint32_t)(QT * dch) * TILE_BYTES);
      for (int qt = 0; qt < QT; ++qt)
        for (int c = 0; c < dch; ++c)
          tma_load_2d(sA + (size_t)(qt * MAX_DCH + c) * TILE_BYTES, &qmap, a_full, c * BK,
                      (int)(qbase + qt * BM));
      int it = 0;
      bool ok = true;
      for (int j = 0; j < ntile && ok; ++j) {
        for (int c = 0; c < dch; ++c, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
          if (!mbar_wait(emptyb + s, ph ^ 1u, abort_flag, P.status)) { ok = false; break; }
          mbar_expect_tx(full + s, TILE_BYTES);
          tma_load_2d(sB + (size_t)s * TILE_BYTES, &rmap, full + s, c * BK, (int)((t0 + j) * BN));
        }
      }
      // every issued copy lands before the CTA can exit
      for (int x = max(0, it - STAGES); x < it; ++x) mbar_drain(full + x % STAGES, (uint32_t)(x / STAGES) & 1u);
      mbar_drain(a_full, 0);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0 && ntile > 0) {
      bool ok = mbar_wait(a_full, 0, abort_flag, P.status);
      fence_after();
      int it = 0;
      for (int j = 0; j < ntile && ok; ++j) {
        const int buf = j & 1;
        const uint32_t aph = (uint32_t)(j >> 1) & 1u;
        if (!mbar_wait(acc_empty + buf, aph ^ 1u, abort_flag, P.status)) { ok = false; break; }
        fence_after();
        for (int c = 0; c < dch; ++c, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
          if (!mbar_wait(full + s, ph, abort_flag, P.status)) { ok = false; break; }
          fence_after();
          const uint32_t b_addr = smem_u32(sB + (size_t)s * TILE_BYTES);
          for (int qt = 0; qt < QT; ++qt) {
            const uint32_t a_addr = smem_u32(sA + (size_t)(qt * MAX_DCH + c) * TILE_BYTES);
            const uint32_t d_addr = tmem + (uint32_t)((buf * QT + qt) * BN);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk)
              umma_bf16(d_addr, sw128_desc(a_addr + kk * 32), sw128_desc(b_addr + kk * 32), (c | kk) != 0);
          }
          umma_commit(emptyb + s);            // the stage is free once these MMAs have read it
        }
        if (!ok) break;
        umma_commit(acc_full + buf);          // tile j's accumulators are complete
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
    const int64_t q = qbase + qt * BM + row;
    const int K = P.k;
    bool active = q < P.q0 + P.nq;
    float Nq = 0.f;
    if (active) {
      active = !P.qempty[q];                 // a degenerate query has no list
      Nq = P.qnorm2[q];
    }
    const int32_t d = P.d;
    const float rel = 0.0040f + (float)d * 2.384185791015625e-7f;
    const bool cosine = P.method == COSINE;
    // this thread's top k pessimistic keys, sorted descending, in registers:
    // KL - k leading +inf sentinels, so that lst[KL - 1] is the k-th best
    float lst[KL];
#pragma unroll
    for (int i = 0; i < KL; ++i) lst[i] = (i < KL - K) ? INFINITY : -INFINITY;
    float T = -INFINITY;                       // k-th best pessimistic key so far
    // hot-loop threshold on x; finite, so that x = -inf (degenerate or padding
    // references) never passes
    float e_thr = -FLT_MAX;
    int cnt = 0;
    const int64_t slot = active ? ((q - P.q0) * P.nrr + rr) : 0;
    int32_t* my_idx = P.eidx + slot * P.ecap;
    float* my_hi = P.ehi + slot * P.ecap;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;

    // The exact key bounds of one reference r with GEMM value s (the slow
    // path): append it if its optimistic key reaches the running cut, insert
    // its pessimistic key into the running top k and tighten the hot test.
    // Degenerate and padding references carry w = +inf and are skipped (their
    // GEMM value is exactly 0, so w is read only then).
    auto process = [&](int64_t r, float s) {
      if (P.self && r == q) return;
      if (s == 0.f && P.w[r] == INFINITY) return;
      const float Nr = cosine ? 0.f : P.norm2[r];
      float key, err;
      dense_key(P.method, 0, d, s, Nq, Nr, key, err);
      const float lo = key - err, hi = key + err;
      if (hi >= dense_cut(T)) {
        if (cnt < P.ecap) { my_idx[cnt] = (int32_t)r; my_hi[cnt] = hi; }
        ++cnt;
      }
      if (lo > T) {
        // sorted insert: the new lst[i] is the median of lst[i - 1], lo, lst[i]
#pragma unroll
        for (int i = KL - 1; i > 0; --i) lst[i] = fmaxf(lst[i], fminf(lst[i - 1], lo));
        lst[0] = fmaxf(lst[0], lo);
        T = lst[KL - 1];
        const float cut = dense_cut(T);
        // hi >= cut implies x >= e_thr (the hot-test bound in the file
        // header), with 2^-12 slack for the FP32 roundings of x and e_thr
        e_thr = cosine ? cut - rel - (2.44140625e-4f * (fabsf(cut) + 1.f) + 1e-30f)
                       : cut + P.one_minus_c * Nq - (2.44140625e-4f * (fabsf(cut) + Nq) + 1e-30f);
        e_thr = fmaxf(-FLT_MAX, e_thr);
      }
    };
    // Passing references wait in this thread's NB shared-memory slots and are
    // processed by the whole warp at once when some lane's slots run out (and
    // at the end), so that the slow path runs with most lanes active instead
    // of one lane at a time; a deferred reference is judged against the cut
    // current when it is processed, which only tightens the test.
    const int et = threadIdx.x - 64;                  // epilogue thread 0 .. 255
    int nbuf = 0;
    auto flush = [&]() {
      const int nmax = __reduce_max_sync(0xffffffffu, nbuf);
      for (int i = 0; i < nmax; ++i)
        if (i < nbuf) process(buf_r[i * EPI_THREADS + et], buf_s[i * EPI_THREADS + et]);
      nbuf = 0;
      __syncwarp();
    };
    // The hot test of one 32-reference chunk: x = s (cosine) or x = 2 s - w[r]
    // (euclidean), the maximum as a tree; the mask of the references with
    // x >= e_thr (0 for an inactive lane), built as a tree of ORs.  Trees keep
    // the dependent chains five instructions deep.
    auto hot_mask = [&](const uint32_t (&v)[32], int64_t r0) -> uint32_t {
      if (!active) return 0u;
      float x[32];
      if (cosine) {
#pragma unroll
        for (int t = 0; t < 32; ++t) x[t] = __uint_as_float(v[t]);
      } else {
        const float4* w4 = reinterpret_cast<const float4*>(P.w + r0);
#pragma unroll
        for (int j4 = 0; j4 < 8; ++j4) {
          const float4 ww = __ldg(w4 + j4);
          x[4 * j4 + 0] = fmaf(P.a, __uint_as_float(v[4 * j4 + 0]), -ww.x);
          x[4 * j4 + 1] = fmaf(P.a, __uint_as_float(v[4 * j4 + 1]), -ww.y);
          x[4 * j4 + 2] = fmaf(P.a, __uint_as_float(v[4 * j4 + 2]), -ww.z);
          x[4 * j4 + 3] = fmaf(P.a, __uint_as_float(v[4 * j4 + 3]), -ww.w);
        }
      }
      float m[16];
#pragma unroll
      for (int t = 0; t < 16; ++t) m[t] = fmaxf(x[2 * t], x[2 * t + 1]);
#pragma unroll
      for (int w = 8; w > 0; w >>= 1)
#pragma unroll
        for (int t = 0; t < w; ++t) m[t] = fmaxf(m[t], m[t + w]);
      if (!(m[0] >= e_thr)) return 0u;
      uint32_t b[16];
#pragma unroll
      for (int t = 0; t < 16; ++t)
        b[t] = (x[2 * t] >= e_thr ? 1u << (2 * t) : 0u) | (x[2 * t + 1] >= e_thr ? 2u << (2 * t) : 0u);
#pragma unroll
      for (int w = 8; w > 0; w >>= 1)
#pragma unroll
        for (int t = 0; t < w; ++t) b[t] |= b[t + w];
      return b[0];
    };
    // v[jj] as a five-level tree of selects on the bits of jj
    auto pick = [](const uint32_t (&v)[32], int jj) -> float {
      uint32_t a[16];
#pragma unroll
      for (int t = 0; t < 16; ++t) a[t] = (jj & 1) ? v[2 * t + 1] : v[2 * t];
#pragma unroll
      for (int lvl = 1, w = 8; w > 0; ++lvl, w >>= 1)
#pragma unroll
        for (int t = 0; t < w; ++t) a[t] = ((jj >> lvl) & 1) ? a[2 * t + 1] : a[2 * t];
      return __uint_as_float(a[0]);
    };
    // The passing references of one chunk into this lane's slots (lanes
    // converged): the warp flushes first if some lane's slots would overflow;
    // a lane with more than NB of them (only while its list is filling) takes
    // the slow path at once.
    auto take = [&](const uint32_t (&v)[32], uint32_t mask, int64_t r0) {
      const int nnew = __popc(mask);
      if (__any_sync(0xffffffffu, nbuf + nnew > NB)) flush();
      if (nnew > NB) {
        while (mask) {
          const int jj = __ffs(mask) - 1;
          mask &= mask - 1;
          process(r0 + jj, pick(v, jj));
        }
      } else {
        while (mask) {
          const int jj = __ffs(mask) - 1;
          mask &= mask - 1;
          buf_r[nbuf * EPI_THREADS + et] = (int32_t)(r0 + jj);
          buf_s[nbuf * EPI_THREADS + et] = pick(v, jj);
          ++nbuf;
        }
      }
      __syncwarp();
    };
    // two chunks at once: their hot tests are independent, so they overlap
    auto chunk2 = [&](const uint32_t (&va)[32], int64_t ra, const uint32_t (&vb)[32], int64_t rb) {
      const uint32_t ma = hot_mask(va, ra), mb = hot_mask(vb, rb);
      if (__any_sync(0xffffffffu, (ma | mb) != 0u)) {
        take(va, ma, ra);
        take(vb, mb, rb);
      }
    };

    for (int j = 0; j < ntile; ++j) {
      const int buf = j & 1;
      const uint32_t aph = (uint32_t)(j >> 1) & 1u;
      const bool ok = mbar_wait(acc_full + buf, aph, abort_flag, P.status);
      if (!__all_sync(0xffffffffu, ok)) break;     // the warp leaves together (tcgen05.ld is .aligned)
      fence_after();
      const int64_t rtile = (t0 + j) * BN;
      const uint32_t tb = tmem + lane_base + (uint32_t)((buf * QT + qt) * BN);
      static_assert(BN % 64 == 0, "pairs of 32-column chunks");
      if constexpr (KL <= 32) {
        // chunks in pairs (the TMEM loads take a few tens of cycles; the
        // pair's hot tests overlap)
#pragma unroll 1
        for (int hh = 0; hh < BN / 32; hh += 2) {
          uint32_t va[32], vb[32];
          tmem_ld32_issue(tb + hh * 32, va);
          tmem_ld32_issue(tb + hh * 32 + 32, vb);
          tmem_ld_wait(va);
          tmem_ld_wait(vb);
          chunk2(va, rtile + hh * 32, vb, rtile + hh * 32 + 32);
        }
      } else {
        // longer lists leave registers for one chunk at a time
#pragma unroll 1
        for (int hh = 0; hh < BN / 32; ++hh) {
          uint32_t va[32];
          tmem_ld32(tb + hh * 32, va);
          const uint32_t ma = hot_mask(va, rtile + hh * 32);
          if (__any_sync(0xffffffffu, ma != 0u)) take(va, ma, rtile + hh * 32);
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty + buf);
    }
    flush();
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
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ---- merge: the final cut of each query over its ranges ---------------------
constexpr int MW = 8;   // warps per block

__device__ __forceinline__ void warp_insert_desc_tc(float* lst, int K, int& n, unsigned m, float v, int lane) {
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

__global__ void k_tc_merge(int64_t q0, int64_t nq, int nrr, int K, int ecap, const uint8_t* empty,
                           const float* lists, const int32_t* ecount, const int32_t* eidx, const float* ehi,
                           int cap, int32_t* cand, int32_t* count, int32_t* over) {
  __shared__ float sl[MW][KT];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = (int64_t)blockIdx.x * MW + warp;
  if (ql >= nq) return;
  if (empty[q0 + ql]) {
    if (lane == 0) { count[ql] = 0; over[ql] = 0; }
    return;
  }
  float* lst = sl[warp];
  int n = 0;
  const float* in = lists + ql * nrr * (int64_t)K;
  const int64_t tot = (int64_t)nrr * K;
  for (int64_t p0 = 0; p0 < tot; p0 += 32) {
    const float v = p0 + lane < tot ? in[p0 + lane] : -INFINITY;
    const unsigned m = __ballot_sync(0xffffffffu, v > -INFINITY && (n < K || v > lst[K - 1]));
    if (m) warp_insert_desc_tc(lst, K, n, m, v, lane);
  }
  const float cut = dense_cut((n == K) ? lst[K - 1] : -INFINITY);
  bool ovf = false;
  int total = 0;
  int32_t* out = cand + ql * (int64_t)cap;
  for (int r = 0; r < nrr && !ovf; ++r) {
    const int64_t slot = ql * nrr + r;
    const int c = ecount[slot];
    if (c > ecap) { ovf = true; break; }
    for (int p0 = 0; p0 < c; p0 += 32) {
      const int p = p0 + lane;
      const bool keep = p < c && ehi[slot * ecap + p] >= cut;
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      const int rank = __popc(m & ((1u << lane) - 1u));
      if (keep && total + rank < cap) out[total + rank] = eidx[slot * ecap + p];
      total += __popc(m);
    }
    if (total > cap) ovf = true;
  }
  if (lane == 0) { count[ql] = ovf ? 0 : total; over[ql] = ovf ? 1 : 0; }
}

// w[r]: +inf for degenerate references and the padding; 0 (cosine) or
// (1 - c) Nr (euclidean) otherwise
__global__ void k_tc_weights(int method, int64_t n, int64_t npad, float one_minus_c, const float* norm2,
                             const uint8_t* empty, float* w) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= npad) return;
  float v = INFINITY;
  if (r < n && !empty[r]) v = (method == COSINE) ? 0.f : one_minus_c * norm2[r];
  w[r] = v;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

int fail(int code, const char* msg) { set_error(msg); return code; }

}  // namespace

bool tc_screen_supported(const sdg_dense* R, int method, int k) {
  return (method == COSINE || method == EUCLIDEAN) && k >= 1 && k <= KT && R->dpad <= MAX_DCH * BK &&
         R->n < (int64_t)1 << 30 && encode_fn() != nullptr;
}

int tc_screen(sdg_ctx* ctx, const sdg_dense* Q, const sdg_dense* D, bool self, int method, int k, int64_t q0,
              int64_t nq, int32_t* cand, int32_t* count, int32_t* over, int cap, cudaStream_t s) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(SDG_E_CUDA, "cuTensorMapEncodeTiled is unavailable");
  if (Q->dpad != D->dpad || Q->n >= (int64_t)1 << 30) return fail(SDG_E_ARG, "query and reference shapes differ");
  const int64_t n = D->n;
  const int dch = D->dpad / BK;
  // one map per operand: 64-row x 128-column boxes of the K-major BF16 copy
  // (rows padded to dpad with zeros; columns beyond the matrix read as zero)
  auto encode = [&](const sdg_dense* M, CUtensorMap* map) {
    const __nv_bfloat16* base = (method == COSINE) ? M->ubp : M->xbp;
    const cuuint64_t gdim[2] = {(cuuint64_t)M->dpad, (cuuint64_t)M->n};
    const cuuint64_t gstride[1] = {(cuuint64_t)M->dpad * 2};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)BN};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, gdim, gstride, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  CUtensorMap qmap, rmap;
  if (!encode(Q, &qmap) || !encode(D, &rmap)) return fail(SDG_E_CUDA, "cuTensorMapEncodeTiled failed");

  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device);
  if (sms < 1) sms = 1;
  const int nqg = (int)((nq + QT * BM - 1) / (QT * BM));
  const int64_t ntiles = (n + BN - 1) / BN;
  int nrr = std::max(1, sms / nqg);
  nrr = (int)std::min<int64_t>(nrr, ntiles);
  const int tpr = (int)((ntiles + nrr - 1) / nrr);
  nrr = (int)((ntiles + tpr - 1) / tpr);
  const int ecap = 768;
  const float rel = 0.0040f + (float)D->d * 2.384185791015625e-7f;
  const float omc = 1.f - (rel + 9.5367431640625e-7f);

  float *w = nullptr, *lists = nullptr, *ehi = nullptr;
  int32_t *ecount = nullptr, *eidx = nullptr;
  int* status = nullptr;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  chk(cudaMallocAsync(&w, sizeof(float) * (size_t)D->npad, s));
  chk(cudaMallocAsync(&lists, sizeof(float) * (size_t)(nq * nrr * k), s));
  chk(cudaMallocAsync(&ecount, sizeof(int32_t) * (size_t)(nq * nrr), s));
  chk(cudaMallocAsync(&eidx, sizeof(int32_t) * (size_t)(nq * nrr * ecap), s));
  chk(cudaMallocAsync(&ehi, sizeof(float) * (size_t)(nq * nrr * ecap), s));
  chk(cudaMallocAsync(&status, sizeof(int), s));
  if (e == cudaSuccess) {
    chk(cudaMemsetAsync(status, 0, sizeof(int), s));
    chk(cudaMemsetAsync(ecount, 0, sizeof(int32_t) * (size_t)(nq * nrr), s));
    k_tc_weights<<<(unsigned)((D->npad + 255) / 256), 256, 0, s>>>(method, n, D->npad, omc, D->norm2, D->empty, w);
    TcArgs P;
    P.method = method; P.k = k; P.dch = dch; P.nqg = nqg; P.nrr = nrr; P.tiles_per_range = tpr; P.ecap = ecap;
    P.self = self ? 1 : 0;
    P.d = D->d; P.n = n; P.q0 = q0; P.nq = nq; P.ntiles = ntiles;
    P.a = (method == COSINE) ? 1.f : 2.f; P.one_minus_c = omc;
    P.w = w; P.norm2 = D->norm2; P.qnorm2 = Q->norm2; P.qempty = Q->empty;
    P.lists = lists; P.ecount = ecount; P.eidx = eidx; P.ehi = ehi;
    P.status = status;
    // the list length: the smallest of 16 / 24 / 32 / 48 / 64 that holds k
    auto kern = (k <= 16) ? k_dense_tc<16> : (k <= 24) ? k_dense_tc<24> : (k <= 32) ? k_dense_tc<32>
              : (k <= 48) ? k_dense_tc<48> : k_dense_tc<64>;
    chk(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    sdg_time_begin(ctx);
    if (e == cudaSuccess) kern<<<(unsigned)(nqg * nrr), THREADS, SMEM_BYTES, s>>>(qmap, rmap, P);
    sdg_time_end(ctx);
    chk(cudaGetLastError());
    k_tc_merge<<<(unsigned)((nq + MW - 1) / MW), MW * 32, 0, s>>>(q0, nq, nrr, k, ecap, Q->empty, lists, ecount,
                                                                  eidx, ehi, cap, cand, count, over);
    chk(cudaGetLastError());
  }
  int hstatus = 0;
  if (e == cudaSuccess) chk(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (e == cudaSuccess) chk(cudaStreamSynchronize(s));
  for (void* p : {(void*)w, (void*)lists, (void*)ecount, (void*)eidx, (void*)ehi, (void*)status})
    if (p) cudaFreeAsync(p, s);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SDG_E_NOMEM : SDG_E_CUDA;
  }
  if (hstatus) return fail(SDG_E_CUDA, "tensor-core screen: a pipeline wait timed out");
  return SDG_OK;
}

}  // namespace sdg
