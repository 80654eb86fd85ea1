// sdg_select.cu -- exact top-k selection under the reference's comparator.
//
// One warp owns one output row ("segment") and keeps its k best candidates in
// shared memory as a list sorted best-first on the key (order_key(value),
// index), with each candidate's own value beside it: order_key maps -0 and +0
// onto one key (IEEE equality, as the reference's comparator), and the value
// written out is the candidate's, bit for bit, as topKBlock writes D's.  The comparator is a strict total order, so the result is the top-k
// of the candidate set whatever order candidates arrive in: it equals the
// bounded-heap results of topKBlock (src/topK.cpp:104-131) and of
// topKRowsAccum's strictly-better replacement (src/topKRows.cpp:201-228).
#include <algorithm>

#include "sdg_kernels.h"
#include "sdg_topk.cuh"

namespace sdg {
namespace {

using namespace topk;

// Selects output row seg of the call into the list (lk, li, lv) of k slots.
__device__ void select_row(const SelectArgs& a, int64_t seg, uint64_t* lk, double* lv, int32_t* li, int lane) {
  const int K = a.k;
  const bool dec = a.decreasing != 0;
  const int64_t row = a.out_row0 + seg;
  int n = 0;

  const bool blank = a.seg_blank && a.seg_blank[row];
  if (!blank) {
    if (a.seed_idx) {
      // Carried state: slots fill left to right, read up to the first NA.
      for (int t0 = 0; t0 < K; t0 += 32) {
        const int t = t0 + lane;
        int32_t gi = NA_INT;
        double v = 0.0;
        if (t < K) { gi = a.seed_idx[(int64_t)t * a.seed_ld + row]; v = a.seed_val[(int64_t)t * a.seed_ld + row]; }
        const bool bad = (t < K) && (gi == NA_INT || gi <= 0);
        const unsigned bm = __ballot_sync(FULL, bad);
        const int lim = bm ? (__ffs(bm) - 1) : 32;
        const bool ok = (lane < lim) && (t < K);
        insert_batch(ok, ok ? order_key(v, dec) : 0, ok ? gi - 1 : 0, v, lk, li, lv, n, K, lane);
        if (bm) break;
      }
    }
    const int64_t skip = (a.skip_base >= 0) ? a.skip_base + seg
                         : (a.skip_arr ? a.skip_arr[seg] : (int64_t)-1);
    const double* base = a.vals + seg * a.seg_stride;
    const int64_t len = a.cand ? (int64_t)a.cand_count[seg] : a.len;
    const int32_t* cidx = a.cand ? a.cand + seg * a.cand_ld : nullptr;
    for (int64_t t0 = 0; t0 < len; t0 += 32) {
      const int64_t t = t0 + lane;
      bool ok = t < len;
      uint64_t key = 0;
      int32_t g = 0;
      double v = 0.0;
      if (ok) {
        v = base[t * a.elem_stride];
        const int64_t gg = cidx ? (int64_t)cidx[t] : a.idx_base + t;
        ok = isfinite(v) && gg != skip && !(a.elem_mask && a.elem_mask[t]);
        key = order_key(v, dec);
        g = (int32_t)gg;
      }
      insert_batch(ok, key, g, v, lk, li, lv, n, K, lane);
    }
  }
  for (int t = lane; t < K; t += 32) {
    const int64_t at = (int64_t)t * a.out_ld + row;
    if (t < n) { a.out_idx[at] = li[t] + 1; a.out_val[at] = lv[t]; }
    else       { a.out_idx[at] = NA_INT;    a.out_val[at] = na_real(); }
  }
}

// k <= kMaxK: a warp's list in shared memory, one row per warp.
__global__ void k_select(SelectArgs a) {
  extern __shared__ unsigned char smem[];
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t seg = (int64_t)blockIdx.x * warps + warp;
  if (seg >= a.nseg) return;                         // uniform per warp
  const int K = a.k;
  uint64_t* lk = reinterpret_cast<uint64_t*>(smem) + (int64_t)warp * K;
  double* lv = reinterpret_cast<double*>(smem) + (int64_t)warps * K + (int64_t)warp * K;
  int32_t* li = reinterpret_cast<int32_t*>(reinterpret_cast<uint64_t*>(smem) + 2 * (int64_t)warps * K) +
                (int64_t)warp * K;
  select_row(a, seg, lk, lv, li, lane);
}

// Bytes of one warp's list in device scratch: k keys (8 B), values (8 B) and
// indices (4 B), rounded up to 16 so that every warp's keys stay 8-byte aligned.
__host__ __device__ __forceinline__ int64_t wide_list_bytes(int64_t k) { return (k * 20 + 15) / 16 * 16; }

// Any k: each warp owns wide_list_bytes(k) of device scratch and takes rows
// warp, warp + (all warps), ...  The list's operations are the same, in
// global memory (a row's list is private to its warp; L1 holds its tail).
__global__ void k_select_wide(SelectArgs a, unsigned char* scratch) {
  const int warps = blockDim.x >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * warps + (threadIdx.x >> 5);
  const int64_t stride = (int64_t)gridDim.x * warps;
  const int64_t K = a.k;
  unsigned char* base = scratch + w * wide_list_bytes(K);
  uint64_t* lk = reinterpret_cast<uint64_t*>(base);
  double* lv = reinterpret_cast<double*>(base + K * 8);
  int32_t* li = reinterpret_cast<int32_t*>(base + K * 16);
  for (int64_t seg = w; seg < a.nseg; seg += stride) {
    select_row(a, seg, lk, lv, li, lane);
    __syncwarp();
  }
}

}  // namespace

void launch_select(const SelectArgs& a, cudaStream_t s) {
  if (a.nseg <= 0) return;
  if (a.k <= kMaxK) {
    int warps = 8;
    while (warps > 1 && (size_t)warps * a.k * 20 > 48 * 1024) warps >>= 1;
    const size_t smem = (size_t)warps * a.k * 20;
    const int64_t blocks = (a.nseg + warps - 1) / warps;
    k_select<<<(unsigned)blocks, warps * 32, smem, s>>>(a);
    return;
  }
  // Lists in device scratch: at most 256 MiB of them and 64 warps per SM.
  const int warps = 8;
  const int64_t per = wide_list_bytes(a.k);
  int64_t nw = std::min<int64_t>(a.nseg, std::max<int64_t>(1, ((int64_t)256 << 20) / per));
  nw = std::min<int64_t>(nw, 152 * 64);
  const int64_t blocks = (nw + warps - 1) / warps;
  unsigned char* scratch = nullptr;
  // a failed allocation is left as the thread's last error for the caller's check
  if (cudaMallocAsync(reinterpret_cast<void**>(&scratch), (size_t)(blocks * warps * per), s) != cudaSuccess) return;
  k_select_wide<<<(unsigned)blocks, warps * 32, 0, s>>>(a, scratch);
  cudaFreeAsync(scratch, s);
}

}  // namespace sdg
