// sdg_topk.cuh -- the warp-level top-k list under the reference's comparator
// (order_key(value), then the lower index; src/topK.cpp:38-50), shared by the
// selection kernel (sdg_select.cu) and the batched exact kNN (sdg_exact.cu).
// A list lives in shared memory sorted best-first, each entry's own value
// beside its key.
#pragma once

#include "sdg_common.cuh"

namespace sdg {
namespace topk {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ bool less_key(uint64_t ka, int32_t ia, uint64_t kb, int32_t ib) {
  return ka < kb || (ka == kb && ia < ib);
}

// Warp-cooperative insertion of the lanes' candidates into the sorted list.
__device__ __forceinline__ void insert_batch(bool valid, uint64_t key, int32_t gidx, double val,
                                             uint64_t* lk, int32_t* li, double* lv, int& n, int K,
                                             int lane) {
  bool pass = valid;
  if (n == K) pass = pass && less_key(key, gidx, lk[K - 1], li[K - 1]);
  unsigned m = __ballot_sync(FULL, pass);
  while (m) {
    const int src = __ffs(m) - 1;
    m &= m - 1;
    const uint64_t kk = __shfl_sync(FULL, key, src);
    const int32_t ii = __shfl_sync(FULL, gidx, src);
    const double vv = __shfl_sync(FULL, val, src);
    if (n == K && !less_key(kk, ii, lk[K - 1], li[K - 1])) continue;
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (less_key(lk[mid], li[mid], kk, ii)) lo = mid + 1; else hi = mid;
    }
    const int last = (n < K) ? n : K - 1;            // [lo, last) moves right by one
    if (last > lo) {
      for (int c = (last - 1) >> 5; c >= (lo >> 5); --c) {
        const int e = c * 32 + lane;
        const bool mv = (e >= lo && e < last);
        uint64_t tk = 0;
        int32_t ti = 0;
        double tv = 0.0;
        if (mv) { tk = lk[e]; ti = li[e]; tv = lv[e]; }
        __syncwarp();
        if (mv) { lk[e + 1] = tk; li[e + 1] = ti; lv[e + 1] = tv; }
        __syncwarp();
      }
    }
    if (lane == 0) { lk[lo] = kk; li[lo] = ii; lv[lo] = vv; }
    __syncwarp();
    if (n < K) ++n;
  }
}

}  // namespace topk
}  // namespace sdg
