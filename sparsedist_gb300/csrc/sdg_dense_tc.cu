// sdg_dense_tc.cu -- the dense screen fused on the 5th-generation tensor cores.
//
// The BF16 screen of the dense path without a slab in HBM.  The work of a
// query block is the grid of (query group, reference tile) items: a query
// group is 128 query columns (one UMMA A tile, M = 128), a reference tile 256
// reference columns (UMMA N = 256).  The items, query-group-major, are split
// into equal contiguous spans, one per CTA (a persistent grid of at most one
// CTA per SM), so every SM gets the same work whatever the block size; a span
// usually covers the tail of one query group and the head of the next, and
// each (query group, CTA) piece of a span is a "segment".
//
// Per segment the query group's 128 x d BF16 columns are loaded into shared
// memory once (TMA, SWIZZLE_128B, K-major, 64-row chunks); reference tiles of
// 256 columns x 64 rows stream through a four-stage TMA ring.  One thread
// issues tcgen05.mma.cta_group::1.kind::f16 (M = 128 queries, N = 256
// references, K = 16, BF16 in, FP32 accumulate) into TMEM: two accumulator
// buffers of 256 columns fill all 512, so the MMAs of tile j + 1 run while
// the epilogue reads tile j back with tcgen05.ld.
//
// Epilogue: eight warps; warp w reads TMEM lanes 32 (w % 4) .. + 31 (its 32
// queries) and one half of the tile's 256 columns ((w - 2) / 4).  A thread
// owns one (query, column half): it keeps the top k pessimistic keys of its
// half of the segment's references in registers and appends every reference
// whose optimistic key reaches its running cut to a per-(query, segment,
// half) list.  The running cut is the k-th best of a subset, never above the
// query's final cut, so the union of the lists holds every reference that the
// slab screen keeps; k_tc_merge applies the final cut (the k-th best over all
// the query's lists) exactly as the slab screen does, then a second, tighter
// cut from per-pair bounds (the columns' BF16 rounding-error norms) on the
// candidates alone.
//
// Hot test.  An epilogue thread tests x = a s - w[r] against one threshold
// e_thr per query (a = 1, w = 0 for cosine; a = 2, w = (1 - c) Nr for
// euclidean, c = rel + 2^-20; w = +inf for degenerate and padding references),
// and only references passing it get their exact key bounds.  For euclidean
// 2 rel sqrt(Nq Nr) <= rel (Nq + Nr), so hi <= 2 s - (1 - c)(Nq + Nr) + 1e-30
// and hi >= cut implies x >= cut + (1 - c) Nq; for cosine hi = s + rel.
// e_thr subtracts 2^-12 (|cut| + Nq) (euclidean) or 2^-12 (|cut| + 1)
// (cosine) more, far above the FP32 rounding of x.  The test's maximum, the
// pass mask and the pick of a passing value are trees five levels deep, and
// two 32-column chunks are tested together.  Passing references wait in eight
// shared-memory slots per thread and are processed by the whole warp at once
// when some lane's slots run out, so the slow path (key bounds, append,
// sorted insert) runs with most lanes active.
//
// Warp roles (320 threads): warp 0 TMA producer, warp 1 TMEM allocator + MMA
// issuer, warps 2..9 epilogue.  Every mbarrier wait is bounded (1 s of
// %globaltimer, sdg_tc_ptx.cuh) and sleeps instead of spinning; a wait that
// runs out sets *status, raises the CTA's abort flag, and the CTA drains its
// own copies and MMAs, frees TMEM and returns.
//
// CTA pairs (PAIR = true, dense mode 3).  A cluster of two CTAs shares each
// UMMA: the even CTA issues tcgen05.mma.cta_group::2 with M = 256 (its 128
// queries in rows 0-127, the odd CTA's in 128-255) and N = 256, each CTA
// holding its own query tile and one 128-column half of every reference chunk
// (16 KB, an 8-stage ring).  Both CTAs' TMA loads (cta_group::2) count their
// bytes on the even CTA's barriers, whose commits multicast to both CTAs; the
// odd CTA's epilogue releases the even CTA's accumulator barrier remotely;
// TMEM is allocated and freed by a warp of each CTA, and a cluster barrier
// keeps either CTA from leaving while the other may still touch its memory.
// Measured on the 256 x 2,000,000 workload it is no faster than one CTA per
// group (3.55 against 3.41 ms): the loop is bound by the per-tile hand-off
// between the MMAs and the epilogue through the two TMEM buffers, not by the
// reference chunks' supply that the pairs halve.
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

using namespace tc;

constexpr int BM = 128;                 // queries per group (UMMA M, TMEM lanes)
constexpr int BN = 256;                 // references per tile (UMMA N)
constexpr int BK = 64;                  // rows of a K chunk: 64 BF16 = one 128-byte swizzle row
constexpr int NB = 8;                   // buffered passing references per epilogue thread
constexpr int EPI_THREADS = 256;
constexpr int KT = 64;                  // largest k of the fused screen
constexpr int THREADS = 320;
constexpr uint32_t A_BYTES = BM * BK * 2;      // 16 KB: a 128 x 64 BF16 query chunk
constexpr uint32_t RING_BYTES = 128 * 1024;    // the reference chunk ring
constexpr uint32_t TMEM_COLS = 2 * BN;         // two accumulator buffers
constexpr int MAX_DCH = 4;              // dpad <= 256
constexpr int MAX_STAGES = 8;
// 1 KB alignment slack, A chunks, B ring, candidate slots, barriers
constexpr size_t SMEM_BYTES = 1024 + (size_t)MAX_DCH * A_BYTES + RING_BYTES + (size_t)NB * EPI_THREADS * 8 + 256;

// One CTA (PAIR = false): a query group is 128 queries, the CTA loads whole
// 256-column reference chunks (32 KB, a 4-stage ring) and issues
// cta_group::1 MMAs (M = 128).  A CTA pair (PAIR = true, a cluster of two): a
// query group is 256 queries, 128 per CTA; each CTA loads its 128-column half
// of every reference chunk (16 KB, an 8-stage ring in the same bytes, so the
// ring covers twice the MMA time) and the even CTA issues cta_group::2 MMAs
// (M = 256, N = 256) over both CTAs' operands.
template <bool PAIR>
struct Cfg {
  static constexpr int GM = PAIR ? 2 * BM : BM;            // queries per group
  static constexpr int BNL = PAIR ? BN / 2 : BN;           // reference columns a CTA loads per chunk
  static constexpr uint32_t B_BYTES = BNL * BK * 2;
  static constexpr int STAGES = (int)(RING_BYTES / B_BYTES);
  static constexpr uint32_t IDESC = idesc_f16(GM, BN, true);
};
static_assert(Cfg<true>::STAGES <= MAX_STAGES && Cfg<false>::STAGES <= MAX_STAGES, "barrier space");

struct TcArgs {
  int method, k, dch, ecap;
  int self;                   // queries are columns of the reference (skip r == q)
  int32_t d;
  int64_t n, q0, nq;          // references; the block's first query (index in Q) and size
  int64_t ntiles, tiles_per_cta, nslots;   // reference tiles; items per CTA; list slots per query
  float a;                    // x = a * s - w[r] (1 cosine, 2 euclidean)
  float one_minus_c;          // euclidean hot-test coefficient
  const float* w;             // [ntiles * BN]: +inf for degenerate / padding references
  const float* norm2;         // reference sums of squares
  const float* qnorm2;        // query sums of squares (index in Q)
  const uint8_t* qempty;      // degenerate queries (no list)
  unsigned* tshared;          // [nq]: the best running k-th pessimistic key of any list (ordered bits)
  float* lists;               // [nq][nslots][k]
  int32_t* ecount;            // [nq][nslots]
  int32_t* eidx;              // [nq][nslots][ecap]
  float* es;                  // [nq][nslots][ecap]: the appended references' GEMM values
  int* status;
  int stall;                  // failure-detection test: the MMA issuer's first wait never completes
};

// Order-preserving map of a float onto uint32 (ascending value -> ascending
// key), so that atomicMax on the keys is a max on the floats.
__device__ __forceinline__ unsigned fkey(float f) {
  const unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_value(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
constexpr int SHARE_TILES = 8;          // tiles between exchanges of the shared running key

// the first and the last work unit (a CTA, or a CTA pair) whose span holds an
// item of query group g
__host__ __device__ __forceinline__ int64_t first_cta(int64_t g, int64_t ntiles, int64_t per) {
  return (g * ntiles) / per;
}
__host__ __device__ __forceinline__ int64_t last_cta(int64_t g, int64_t ntiles, int64_t per) {
  return ((g + 1) * ntiles - 1) / per;
}

template <int KL, bool PAIR>
__global__ void __launch_bounds__(THREADS, 1) k_dense_tc(const __grid_constant__ CUtensorMap qmap,
                                                       const __grid_constant__ CUtensorMap rmap, TcArgs P) {
  using C = Cfg<PAIR>;
  constexpr int STAGES = C::STAGES;
  constexpr uint32_t B_BYTES = C::B_BYTES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = base;                                     // MAX_DCH query chunks
  uint8_t* sB = base + (size_t)MAX_DCH * A_BYTES;          // STAGES reference chunks
  // per epilogue thread NB (reference, GEMM value) slots, slot-major so that a
  // warp's accesses to one slot are conflict-free
  int32_t* buf_r = (int32_t*)(sB + (size_t)RING_BYTES);
  float* buf_s = (float*)(buf_r + NB * EPI_THREADS);
  uint64_t* bars = (uint64_t*)(buf_s + NB * EPI_THREADS);
  uint64_t* full = bars;
  uint64_t* emptyb = bars + MAX_STAGES;
  uint64_t* acc_full = bars + 2 * MAX_STAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* a_full = acc_empty + 2;
  uint64_t* a_empty = a_full + 1;
  uint64_t* mma_done = a_empty + 1;
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // this CTA's rank in its pair (0: the MMA issuer) and its work unit
  const uint32_t crank = PAIR ? cluster_rank() : 0u;
  const bool leader = crank == 0;
  const int64_t unit = PAIR ? (int64_t)(blockIdx.x >> 1) : (int64_t)blockIdx.x;
  const int64_t per = P.tiles_per_cta, ntiles = P.ntiles;
  const int64_t f0 = unit * per;
  const int64_t f1 = min(f0 + per, ((P.nq + C::GM - 1) / C::GM) * ntiles);
  const int dch = P.dch;
  // the bounded waits (CTA-scope acquire: the pair's barriers are completed
  // by TMA transactions, tcgen05 commits and the other CTA's arrivals, each
  // ordered by the barrier itself)
  auto wait = [&](uint64_t* bar, uint32_t parity) -> bool { return mbar_wait(bar, parity, abort_flag, P.status); };
  auto drain = [&](uint64_t* bar, uint32_t parity) { mbar_drain(bar, parity); };

  if (threadIdx.x == 0) {
    // a pair's MMA waits on the even CTA's barriers: both CTAs' loads count
    // their bytes there, and both CTAs' epilogues release its buffers
    for (int s = 0; s < STAGES; ++s) { mbar_init(full + s, 1); mbar_init(emptyb + s, 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(acc_full + b, 1); mbar_init(acc_empty + b, PAIR ? 16 : 8); }
    mbar_init(a_full, 1);
    mbar_init(a_empty, 1);
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    if constexpr (PAIR) tmem_alloc_pair(tmem_slot, TMEM_COLS);
    else tmem_alloc(tmem_slot, TMEM_COLS);
  }
  fence_before();
  __syncthreads();
  if constexpr (PAIR) cluster_sync();            // both CTAs' barriers exist before any remote arrival
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---- TMA producer ----
    if (lane == 0 && f1 > f0) {
      prefetch_map(&qmap);
      prefetch_map(&rmap);
      int it = 0, seg = 0;
      bool ok = true;
      for (int64_t f = f0; f < f1 && ok; ++seg) {
        const int64_t g = f / ntiles;
        const int64_t fe = min(f1, (g + 1) * ntiles);
        // the previous segment's MMAs have finished reading the query chunks
        if (!wait(a_empty, ((uint32_t)seg & 1u) ^ 1u)) break;
        const int qy = (int)(P.q0 + g * C::GM + crank * BM);
        if constexpr (PAIR) {
          // both CTAs' query chunks are counted on the even CTA's barrier
          if (leader) mbar_expect_tx(a_full, 2u * (uint32_t)dch * A_BYTES);
          const uint32_t bar = cluster_addr(a_full, 0);
          for (int c = 0; c < dch; ++c) tma_load_2d_pair(sA + (size_t)c * A_BYTES, &qmap, bar, c * BK, qy);
        } else {
          mbar_expect_tx(a_full, (uint32_t)dch * A_BYTES);
          for (int c = 0; c < dch; ++c) tma_load_2d(sA + (size_t)c * A_BYTES, &qmap, a_full, c * BK, qy);
        }
        for (; f < fe && ok; ++f) {
          const int rcol = (int)((f - g * ntiles) * BN + crank * C::BNL);
          for (int c = 0; c < dch; ++c, ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
            if (!wait(emptyb + s, ph ^ 1u)) { ok = false; break; }
            if constexpr (PAIR) {
              if (leader) mbar_expect_tx(full + s, 2u * B_BYTES);
              tma_load_2d_pair(sB + (size_t)s * B_BYTES, &rmap, cluster_addr(full + s, 0), c * BK, rcol);
            } else {
              mbar_expect_tx(full + s, B_BYTES);
              tma_load_2d(sB + (size_t)s * B_BYTES, &rmap, full + s, c * BK, rcol);
            }
          }
        }
      }
      // every issued copy lands before the CTA can exit; a pair's copies are
      // counted on the even CTA's barriers, so the even CTA waits for both
      // CTAs' (the odd CTA leaves only after it, at the final cluster barrier)
      if (!PAIR || leader) {
        for (int x = max(0, it - STAGES); x < it; ++x) drain(full + x % STAGES, (uint32_t)(x / STAGES) & 1u);
        if (seg > 0) drain(a_full, (uint32_t)(seg - 1) & 1u);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (!PAIR || leader) {
      // ---- MMA issuer ----
      if (lane == 0 && f1 > f0) {
        int it = 0, seg = 0;
        int64_t j = 0;
        bool ok = true;
        for (int64_t f = f0; f < f1 && ok; ++seg) {
          const int64_t g = f / ntiles;
          const int64_t fe = min(f1, (g + 1) * ntiles);
          if (!wait(a_full, (uint32_t)seg & 1u)) break;
          fence_after();
          const uint32_t a0 = smem_u32(sA);
          for (; f < fe && ok; ++f, ++j) {
            const int buf = (int)(j & 1);
            // the epilogue has drained this buffer's previous tile
            // (with P.stall the first wait asks for the phase the epilogue has not
            // begun, so it runs out: the failure-detection test's path)
            const uint32_t flip = (P.stall && j == 0) ? 0u : 1u;
            if (!wait(acc_empty + buf, ((uint32_t)(j >> 1) & 1u) ^ flip)) {
              ok = false;
              break;
            }
            fence_after();
            const uint32_t d_addr = tmem + (uint32_t)(buf * BN);
            for (int c = 0; c < dch; ++c, ++it) {
              const int s = it % STAGES;
              const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
              if (!wait(full + s, ph)) { ok = false; break; }
              fence_after();
              const uint32_t b_addr = smem_u32(sB + (size_t)s * B_BYTES);
              const uint32_t a_addr = a0 + (uint32_t)c * A_BYTES;
#pragma unroll
              for (int kk = 0; kk < BK / 16; ++kk) {
                if constexpr (PAIR)
                  umma_f16_pair(d_addr, sw128_desc(a_addr + kk * 32), sw128_desc(b_addr + kk * 32), C::IDESC,
                                (c | kk) != 0);
                else
                  umma_f16(d_addr, sw128_desc(a_addr + kk * 32), sw128_desc(b_addr + kk * 32), C::IDESC,
                           (c | kk) != 0);
              }
              // the stage is free (in both CTAs of a pair) once these MMAs have read it
              if constexpr (PAIR) umma_commit_pair(emptyb + s, 3); else umma_commit(emptyb + s);
            }
            if (!ok) break;
            // the tile's accumulators are complete
            if constexpr (PAIR) umma_commit_pair(acc_full + buf, 3); else umma_commit(acc_full + buf);
          }
          // the query chunks are free once the segment's MMAs are done
          if constexpr (PAIR) umma_commit_pair(a_empty, 3); else umma_commit(a_empty);
        }
        // all issued MMAs complete before TMEM is freed
        if constexpr (PAIR) umma_commit_pair(mma_done, 3); else umma_commit(mma_done);
        drain(mma_done, 0);
      }
    } else if constexpr (PAIR) {
      // the odd CTA: the even CTA's last commit also arrives on this CTA's
      // barriers; it lands before they go away
      if (lane == 0 && f1 > f0) drain(mma_done, 0);
    }
    __syncwarp();
  } else {
    // ---- epilogue: one thread per (query, column half) ----
    const int quarter = warp & 3, half = (warp - 2) >> 2;
    const int row = quarter * 32 + lane;
    const int K = P.k;
    const int32_t d = P.d;
    const float rel = 0.0040f + (float)d * 2.384185791015625e-7f;
    const bool cosine = P.method == COSINE;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    const int et = threadIdx.x - 64;                  // epilogue thread 0 .. 255

    // per-segment state
    bool active = false;
    int64_t q = 0;
    float Nq = 0.f;
    // this thread's top k pessimistic keys, sorted descending, in registers:
    // KL - k leading +inf sentinels, so that lst[KL - 1] is the k-th best
    float lst[KL];
    float T = -INFINITY;                       // k-th best pessimistic key of this list so far
    // the best running k-th key of any of the query's lists (segments and
    // halves running on other warps and CTAs), exchanged every SHARE_TILES
    // tiles: each is the k-th best of a subset, so their maximum never
    // exceeds the query's final k-th best and may stand in for T in every test
    float Ts = -INFINITY;
    // hot-loop threshold on x; finite, so that x = -inf (degenerate or padding
    // references) never passes
    float e_thr = -FLT_MAX;
    int cnt = 0, nbuf = 0;
    int32_t* my_idx = P.eidx;
    float* my_s = P.es;

    // hi >= cut implies x >= e_thr (the hot-test bound in the file header),
    // with 2^-12 slack for the FP32 roundings of x and e_thr
    auto set_thr = [&]() {
      const float cut = dense_cut(fmaxf(T, Ts));
      e_thr = cosine ? cut - rel - (2.44140625e-4f * (fabsf(cut) + 1.f) + 1e-30f)
                     : cut + P.one_minus_c * Nq - (2.44140625e-4f * (fabsf(cut) + Nq) + 1e-30f);
      e_thr = fmaxf(-FLT_MAX, e_thr);
    };
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
      const float Te = fmaxf(T, Ts);
      if (hi >= dense_cut(Te)) {
        if (cnt < P.ecap) { my_idx[cnt] = (int32_t)r; my_s[cnt] = s; }
        ++cnt;
      }
      if (lo > Te) {
        // sorted insert: the new lst[i] is the median of lst[i - 1], lo, lst[i]
#pragma unroll
        for (int i = KL - 1; i > 0; --i) lst[i] = fmaxf(lst[i], fminf(lst[i - 1], lo));
        lst[0] = fmaxf(lst[0], lo);
        T = lst[KL - 1];
        set_thr();
      }
    };
    // Passing references wait in this thread's NB slots and are processed by
    // the whole warp at once when some lane's slots run out (and at the end of
    // a segment); a deferred reference is judged against the cut current when
    // it is processed, which is never above the final one.
    auto flush = [&]() {
      const int nmax = __reduce_max_sync(0xffffffffu, nbuf);
      for (int i = 0; i < nmax; ++i)
        if (i < nbuf) process(buf_r[i * EPI_THREADS + et], buf_s[i * EPI_THREADS + et]);
      nbuf = 0;
      __syncwarp();
    };
    // The hot test of one 32-reference chunk: the mask of the references with
    // x >= e_thr (0 for an inactive lane); maximum and mask as trees.
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
      for (int wdt = 8; wdt > 0; wdt >>= 1)
#pragma unroll
        for (int t = 0; t < wdt; ++t) m[t] = fmaxf(m[t], m[t + wdt]);
      if (!(m[0] >= e_thr)) return 0u;
      uint32_t b[16];
#pragma unroll
      for (int t = 0; t < 16; ++t)
        b[t] = (x[2 * t] >= e_thr ? 1u << (2 * t) : 0u) | (x[2 * t + 1] >= e_thr ? 2u << (2 * t) : 0u);
#pragma unroll
      for (int wdt = 8; wdt > 0; wdt >>= 1)
#pragma unroll
        for (int t = 0; t < wdt; ++t) b[t] |= b[t + wdt];
      return b[0];
    };
    // v[jj] as a five-level tree of selects on the bits of jj
    auto pick = [](const uint32_t (&v)[32], int jj) -> float {
      uint32_t a[16];
#pragma unroll
      for (int t = 0; t < 16; ++t) a[t] = (jj & 1) ? v[2 * t + 1] : v[2 * t];
#pragma unroll
      for (int lvl = 1, wdt = 8; wdt > 0; ++lvl, wdt >>= 1)
#pragma unroll
        for (int t = 0; t < wdt; ++t) a[t] = ((jj >> lvl) & 1) ? a[2 * t + 1] : a[2 * t];
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

    int64_t j = 0;                                    // tile counter (the MMA's order)
    bool ok = true;
    for (int64_t f = f0; f < f1 && ok;) {
      const int64_t g = f / ntiles;
      const int64_t fe = min(f1, (g + 1) * ntiles);
      const int64_t ql = g * C::GM + crank * BM + row;
      q = P.q0 + ql;
      active = ql < P.nq;
      if (active) active = !P.qempty[q];           // a degenerate query has no list
      Nq = active ? P.qnorm2[q] : 0.f;
#pragma unroll
      for (int i = 0; i < KL; ++i) lst[i] = (i < KL - K) ? INFINITY : -INFINITY;
      T = -INFINITY;
      Ts = active ? fkey_value(*(volatile unsigned*)(P.tshared + ql)) : -INFINITY;
      e_thr = -FLT_MAX;
      if (Ts > -INFINITY) set_thr();
      cnt = 0;
      nbuf = 0;
      const int64_t slot =
          active ? (ql * P.nslots + (unit - first_cta(g, ntiles, per)) * 2 + half) : 0;
      my_idx = P.eidx + slot * P.ecap;
      my_s = P.es + slot * P.ecap;
      for (; f < fe; ++f, ++j) {
        const int buf = (int)(j & 1);
        const bool got = wait(acc_full + buf, (uint32_t)(j >> 1) & 1u);
        if (!__all_sync(0xffffffffu, got)) { ok = false; break; }   // the warp leaves together
        fence_after();
        const int64_t r_half = (f - g * ntiles) * BN + half * (BN / 2);
        const uint32_t tb = tmem + lane_base + (uint32_t)(buf * BN + half * (BN / 2));
        // the buffer goes back to the MMAs as soon as its last TMEM reads are
        // done (the values being processed are in registers by then): the
        // hand-off to the next-but-one tile does not wait for the processing
        auto release = [&]() {
          fence_before();
          __syncwarp();
          if (lane == 0) {
            if constexpr (PAIR) mbar_arrive_remote(acc_empty + buf, 0);   // the even CTA's MMA waits on it
            else mbar_arrive(acc_empty + buf);
          }
        };
        if constexpr (KL <= 32) {
          // chunks in pairs (the TMEM loads take a few tens of cycles; the
          // pair's hot tests overlap)
#pragma unroll 1
          for (int hh = 0; hh < BN / 64; hh += 2) {
            uint32_t va[32], vb[32];
            tmem_ld32_issue(tb + hh * 32, va);
            tmem_ld32_issue(tb + hh * 32 + 32, vb);
            tmem_ld_wait(va);
            tmem_ld_wait(vb);
            if (hh == BN / 64 - 2) release();
            const uint32_t ma = hot_mask(va, r_half + hh * 32), mb = hot_mask(vb, r_half + hh * 32 + 32);
            if (__any_sync(0xffffffffu, (ma | mb) != 0u)) {
              take(va, ma, r_half + hh * 32);
              take(vb, mb, r_half + hh * 32 + 32);
            }
          }
        } else {
          // longer lists leave registers for one chunk at a time
#pragma unroll 1
          for (int hh = 0; hh < BN / 64; ++hh) {
            uint32_t va[32];
            tmem_ld32(tb + hh * 32, va);
            if (hh == BN / 64 - 1) release();
            const uint32_t ma = hot_mask(va, r_half + hh * 32);
            if (__any_sync(0xffffffffu, ma != 0u)) take(va, ma, r_half + hh * 32);
          }
        }
        if ((j & (SHARE_TILES - 1)) == SHARE_TILES - 1 && active) {
          // publish this list's running key and take the best one published
          const unsigned prev = atomicMax(P.tshared + ql, fkey(T));
          const float best = fmaxf(fkey_value(prev), T);
          if (best > Ts) { Ts = best; set_thr(); }
        }
      }
      flush();
      if (active) atomicMax(P.tshared + ql, fkey(T));
      if (active) {
        float* out = P.lists + slot * K;
#pragma unroll
        for (int i = 0; i < KL; ++i)
          if (i >= KL - K) out[i - (KL - K)] = lst[i];
        P.ecount[slot] = cnt;
      }
    }
  }
  fence_before();
  __syncthreads();
  // a pair's MMAs read both CTAs' shared memory and write both TMEMs: neither
  // CTA frees TMEM or exits before the other is done
  if constexpr (PAIR) cluster_sync();
  fence_after();
  if (warp == 1) {
    if constexpr (PAIR) tmem_dealloc_pair(tmem, TMEM_COLS);
    else tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ---- merge: the final cut of each query over its lists ---------------------
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

struct MergeArgs {
  int64_t q0, nq;
  int gm;                      // queries per group
  int64_t ntiles, per, nslots;
  int K, ecap, method;
  int32_t d;
  const uint8_t* qempty;
  const unsigned* tshared;
  const float* lists;
  const int32_t* ecount;
  const int32_t* eidx;
  const float* es;
  const float* norm2;          // reference sums of squares
  const float* qnorm2;         // query sums of squares (index in Q)
  const float *re, *rn;        // reference copies: rounding-error norm, norm (the method's copy)
  const float *qe, *qn;        // query copies (index in Q)
  int cap;
  int32_t* cand;
  float* cand_s;               // [nq][cap] the candidates' GEMM values
  int32_t* count;
  int32_t* over;
};

// The per-pair bound of one candidate from the columns' BF16 copies: with v
// the exact (unit) columns and b their BF16 copies, |sum v_q v_r - sum b_q b_r|
// <= e_q ||v_r|| + ||b_q|| e_r (Cauchy-Schwarz; e = ||v - b||, computed in
// FP64 and rounded up at upload), the BF16 products are exact in FP32 and the
// tensor cores' FP32 accumulation of d products is allowed (d + 64) 2^-21
// ||b_q|| ||b_r||; ||v_r|| is 1 (unit columns) or sqrt(Nr).  The key is the
// screen's (s for cosine, 2 s - Nq - Nr for euclidean) with the FP32 roundings
// of Nq, Nr and the key allowed 2^-20 of the terms.
__device__ __forceinline__ void tight_bounds(const MergeArgs& A, float s, int64_t r, float Nq, float qe, float qn,
                                             float& lo, float& hi) {
  const float acc = (float)(A.d + 64) * 4.76837158203125e-7f;     // 2^-21
  if (A.method == COSINE) {
    const float E = (1.000001f * qe * 1.000001f + qn * A.re[r] + acc * qn * A.rn[r]) * 1.01f + 1e-12f +
                    2.384185791015625e-7f * fabsf(s);               // 2^-22 |s|
    lo = s - E;
    hi = s + E;
  } else {
    const float Nr = A.norm2[r];
    const float Es = (qe * sqrtf(Nr) * 1.000001f + qn * A.re[r] + acc * qn * A.rn[r]) * 1.01f + 1e-30f;
    const float key = 2.f * s - (Nq + Nr);
    const float E = 2.f * Es + 9.5367431640625e-7f * (Nq + Nr + 2.f * fabsf(s)) + 1e-30f;
    lo = key - E;
    hi = key + E;
  }
}

// Per query: T = the k-th largest pessimistic key over the lists of every
// (segment, half) that covered it (the exact k-th over all references: the top
// k of a union is the top k of the parts' top k), cut = dense_cut(T); the
// candidates are the appended references with hi >= cut, hi the uniform bound
// of the screen.  A second, tighter cut follows on the candidates alone: T2 =
// the k-th largest per-pair lower bound (tight_bounds) among them is again at
// most the exact k-th best key (k candidates reach it), so every member of the
// exact top k (ties included) has its per-pair upper bound at or above
// dense_cut(max(T, T2)) and is kept.
__global__ void k_tc_merge(MergeArgs A) {
  __shared__ float sl[MW][KT];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = (int64_t)blockIdx.x * MW + warp;
  if (ql >= A.nq) return;
  const int K = A.K;
  if (A.qempty[A.q0 + ql]) {
    if (lane == 0) { A.count[ql] = 0; A.over[ql] = 0; }
    return;
  }
  const int64_t g = ql / A.gm;
  const int64_t used = 2 * (last_cta(g, A.ntiles, A.per) - first_cta(g, A.ntiles, A.per) + 1);
  float* lst = sl[warp];
  int n = 0;
  const float* in = A.lists + ql * A.nslots * (int64_t)K;
  const int64_t tot = used * K;
  for (int64_t p0 = 0; p0 < tot; p0 += 32) {
    const float v = p0 + lane < tot ? in[p0 + lane] : -INFINITY;
    const unsigned m = __ballot_sync(0xffffffffu, v > -INFINITY && (n < K || v > lst[K - 1]));
    if (m) warp_insert_desc_tc(lst, K, n, m, v, lane);
  }
  // A list keeps only keys above the shared key it saw, so when some list's
  // view of the shared key reached the final k-th best, fewer than k keys at
  // or above it may be listed; the shared key (the k-th best of a subset,
  // never above the final) then is the final k-th best.
  const float T = fmaxf((n == K) ? lst[K - 1] : -INFINITY, fkey_value(A.tshared[ql]));
  const float cut = dense_cut(T);
  const int64_t q = A.q0 + ql;
  const float Nq = A.qnorm2[q];
  bool ovf = false;
  int total = 0;
  int32_t* out = A.cand + ql * (int64_t)A.cap;
  float* out_s = A.cand_s + ql * (int64_t)A.cap;
  for (int64_t r = 0; r < used && !ovf; ++r) {
    const int64_t slot = ql * A.nslots + r;
    const int c = A.ecount[slot];
    if (c > A.ecap) { ovf = true; break; }
    for (int p0 = 0; p0 < c; p0 += 32) {
      const int p = p0 + lane;
      bool keep = false;
      int32_t ref = 0;
      float sv = 0.f;
      if (p < c) {
        ref = A.eidx[slot * A.ecap + p];
        sv = A.es[slot * A.ecap + p];
        float key, err;
        dense_key(A.method, 0, A.d, sv, Nq, A.norm2[ref], key, err);
        keep = key + err >= cut;
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      const int rank = __popc(m & ((1u << lane) - 1u));
      if (keep && total + rank < A.cap) { out[total + rank] = ref; out_s[total + rank] = sv; }
      total += __popc(m);
    }
    if (total > A.cap) ovf = true;
  }
  if (!ovf && total > K) {
    const float qe = A.qe[q], qn = A.qn[q];
    n = 0;
    __syncwarp();
    for (int p0 = 0; p0 < total; p0 += 32) {
      const int p = p0 + lane;
      float lo = -INFINITY, hi;
      if (p < total) tight_bounds(A, out_s[p], out[p], Nq, qe, qn, lo, hi);
      const unsigned m = __ballot_sync(0xffffffffu, p < total && (n < K || lo > lst[K - 1]));
      if (m) warp_insert_desc_tc(lst, K, n, m, lo, lane);
    }
    const float T2 = (n == K) ? lst[K - 1] : -INFINITY;
    const float cut2 = dense_cut(fmaxf(T, T2));
    int kept = 0;
    for (int p0 = 0; p0 < total; p0 += 32) {
      const int p = p0 + lane;
      bool keep = false;
      int32_t ref = 0;
      float sv = 0.f;
      if (p < total) {
        ref = out[p];
        sv = out_s[p];
        float lo, hi;
        tight_bounds(A, sv, ref, Nq, qe, qn, lo, hi);
        keep = hi >= cut2;
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);   // every lane has read slot p first
      const int rank = __popc(m & ((1u << lane) - 1u));
      if (keep) { out[kept + rank] = ref; out_s[kept + rank] = sv; }
      kept += __popc(m);
      __syncwarp();
    }
    total = kept;
  }
  if (lane == 0) { A.count[ql] = ovf ? 0 : total; A.over[ql] = ovf ? 1 : 0; }
}

__global__ void k_tc_key_init(int64_t nq, unsigned* keys) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nq) keys[i] = fkey(-INFINITY);
}

// w[r]: +inf for degenerate references and the padding; 0 (cosine) or
// (1 - c) Nr (euclidean) otherwise
__global__ void k_tc_weights(int method, int64_t n, int64_t nw, float one_minus_c, const float* norm2,
                             const uint8_t* empty, float* w) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nw) return;
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
              int64_t nq, int32_t* cand, int32_t* count, int32_t* over, int cap, cudaStream_t s, bool allow_pairs,
              int* status) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return fail(SDG_E_CUDA, "cuTensorMapEncodeTiled is unavailable");
  if (Q->dpad != D->dpad || Q->n >= (int64_t)1 << 30) return fail(SDG_E_ARG, "query and reference shapes differ");
  const int64_t n = D->n;
  const int dch = D->dpad / BK;
  // one map per operand: 64-row x 128-column (query) / 256-column (reference)
  // boxes of the K-major BF16 copy (rows padded to dpad with zeros; columns
  // beyond the matrix read as zero)
  auto encode = [&](const sdg_dense* M, int box_cols, CUtensorMap* map) {
    const __nv_bfloat16* base_ptr = (method == COSINE) ? M->ubp : M->xbp;
    const cuuint64_t gdim[2] = {(cuuint64_t)M->dpad, (cuuint64_t)M->n};
    const cuuint64_t gstride[1] = {(cuuint64_t)M->dpad * 2};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_cols};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base_ptr, gdim, gstride, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  };
  // the list length: the smallest of 16 / 24 / 32 / 48 / 64 that holds k
  auto pick_kernel = [&](bool pair) {
    if (pair)
      return (k <= 16) ? k_dense_tc<16, true> : (k <= 24) ? k_dense_tc<24, true> : (k <= 32) ? k_dense_tc<32, true>
           : (k <= 48) ? k_dense_tc<48, true> : k_dense_tc<64, true>;
    return (k <= 16) ? k_dense_tc<16, false> : (k <= 24) ? k_dense_tc<24, false> : (k <= 32) ? k_dense_tc<32, false>
         : (k <= 48) ? k_dense_tc<48, false> : k_dense_tc<64, false>;
  };
  // CTA pairs (clusters of two) where the block has more than one 128-query
  // group and the device can hold such clusters; the work unit is then a pair
  int64_t units = 0;
  bool pair = false;
  if (allow_pairs && nq > BM) {
    auto kp = pick_kernel(true);
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2; attr[0].val.clusterDim.y = 1; attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(2, 1, 1); cfg.blockDim = dim3(THREADS, 1, 1); cfg.dynamicSmemBytes = SMEM_BYTES;
    cfg.attrs = attr; cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaFuncSetAttribute(kp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES) == cudaSuccess &&
        cudaOccupancyMaxActiveClusters(&clusters, kp, &cfg) == cudaSuccess && clusters > 0) {
      pair = true;
      units = clusters;
    }
    cudaGetLastError();
  }
  if (!pair) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device);
    units = std::max(sms, 1);
  }
  const int GM = pair ? Cfg<true>::GM : Cfg<false>::GM;
  CUtensorMap qmap, rmap;
  if (!encode(Q, BM, &qmap) || !encode(D, pair ? Cfg<true>::BNL : Cfg<false>::BNL, &rmap))
    return fail(SDG_E_CUDA, "cuTensorMapEncodeTiled failed");

  // (query group, reference tile) items in equal contiguous spans, one per unit
  const int64_t G = (nq + GM - 1) / GM;
  const int64_t ntiles = (n + BN - 1) / BN;
  const int64_t items = G * ntiles;
  int64_t grid = std::min<int64_t>(units, items);
  const int64_t per = (items + grid - 1) / grid;
  grid = (items + per - 1) / per;
  // list slots per query: two halves per CTA whose span meets its group
  int64_t maxc = 1;
  for (int64_t g = 0; g < G; ++g)
    maxc = std::max<int64_t>(maxc, last_cta(g, ntiles, per) - first_cta(g, ntiles, per) + 1);
  const int64_t nslots = 2 * maxc;
  const int ecap = 768;
  const float rel = 0.0040f + (float)D->d * 2.384185791015625e-7f;
  const float omc = 1.f - (rel + 9.5367431640625e-7f);

  float *w = nullptr, *lists = nullptr, *es = nullptr, *cand_s = nullptr;
  int32_t *ecount = nullptr, *eidx = nullptr;
  unsigned* tshared = nullptr;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  const int64_t nw = ntiles * BN;
  chk(cudaMallocAsync(&w, sizeof(float) * (size_t)nw, s));
  chk(cudaMallocAsync(&lists, sizeof(float) * (size_t)(nq * nslots * k), s));
  chk(cudaMallocAsync(&ecount, sizeof(int32_t) * (size_t)(nq * nslots), s));
  chk(cudaMallocAsync(&eidx, sizeof(int32_t) * (size_t)(nq * nslots * ecap), s));
  chk(cudaMallocAsync(&es, sizeof(float) * (size_t)(nq * nslots * ecap), s));
  chk(cudaMallocAsync(&cand_s, sizeof(float) * (size_t)(nq * cap), s));
  chk(cudaMallocAsync(&tshared, sizeof(unsigned) * (size_t)nq, s));
  if (e == cudaSuccess) {
    // every query's shared key starts at fkey(-inf)
    k_tc_key_init<<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(nq, tshared);
    chk(cudaMemsetAsync(ecount, 0, sizeof(int32_t) * (size_t)(nq * nslots), s));
    k_tc_weights<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(method, n, nw, omc, D->norm2, D->empty, w);
    TcArgs P;
    P.method = method; P.k = k; P.dch = dch; P.ecap = ecap;
    P.self = self ? 1 : 0;
    P.d = D->d; P.n = n; P.q0 = q0; P.nq = nq;
    P.ntiles = ntiles; P.tiles_per_cta = per; P.nslots = nslots;
    P.a = (method == COSINE) ? 1.f : 2.f; P.one_minus_c = omc;
    P.w = w; P.norm2 = D->norm2; P.qnorm2 = Q->norm2; P.qempty = Q->empty;
    P.tshared = tshared;
    P.lists = lists; P.ecount = ecount; P.eidx = eidx; P.es = es;
    P.status = status;
    P.stall = tc_take_stall() ? 1 : 0;
    auto kern = pick_kernel(pair);
    chk(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
    sdg_time_begin(ctx);
    if (e == cudaSuccess) {
      if (pair) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2; attr[0].val.clusterDim.y = 1; attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)(2 * grid), 1, 1); cfg.blockDim = dim3(THREADS, 1, 1);
        cfg.dynamicSmemBytes = SMEM_BYTES; cfg.stream = s;
        cfg.attrs = attr; cfg.numAttrs = 1;
        chk(cudaLaunchKernelEx(&cfg, kern, qmap, rmap, P));
      } else {
        kern<<<(unsigned)grid, THREADS, SMEM_BYTES, s>>>(qmap, rmap, P);
      }
    }
    sdg_time_end(ctx);
    chk(cudaGetLastError());
    MergeArgs M;
    M.q0 = q0; M.nq = nq; M.gm = GM; M.ntiles = ntiles; M.per = per; M.nslots = nslots;
    M.K = k; M.ecap = ecap; M.method = method; M.d = D->d;
    M.qempty = Q->empty; M.tshared = tshared; M.lists = lists; M.ecount = ecount; M.eidx = eidx; M.es = es;
    M.norm2 = D->norm2; M.qnorm2 = Q->norm2;
    M.re = (method == COSINE) ? D->ue : D->xe; M.rn = (method == COSINE) ? D->un : D->xn;
    M.qe = (method == COSINE) ? Q->ue : Q->xe; M.qn = (method == COSINE) ? Q->un : Q->xn;
    M.cap = cap; M.cand = cand; M.cand_s = cand_s; M.count = count; M.over = over;
    k_tc_merge<<<(unsigned)((nq + MW - 1) / MW), MW * 32, 0, s>>>(M);
    chk(cudaGetLastError());
  }
  // stream-ordered frees: the caller reads *status with its own results
  for (void* p : {(void*)w, (void*)lists, (void*)ecount, (void*)eidx, (void*)es, (void*)cand_s, (void*)tshared})
    if (p) cudaFreeAsync(p, s);
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SDG_E_NOMEM : SDG_E_CUDA;
  }
  return SDG_OK;
}

}  // namespace sdg
