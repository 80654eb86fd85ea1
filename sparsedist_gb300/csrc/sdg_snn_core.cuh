// sdg_snn_core.cuh -- device-side steps of snnJaccard (src/snn.cpp), shared by
// the kernels that compute SNN weights.
#pragma once

#include "sdg_common.cuh"

namespace sdg {

// copy_indices range check: src/snn.cpp:94-108
__device__ __forceinline__ bool snn_index_bad(int32_t v, int32_t n) {
  return v != NA_INT && (v < 1 || v > n);
}

// build_sets for row i: src/snn.cpp:119-141.  S has room for k + 1 entries.
__device__ __forceinline__ int32_t snn_build_set(const int32_t* idx, int32_t n, int32_t k,
                                                 int include_self, int64_t i, int32_t* S) {
  int c = 0;
  if (include_self) S[c++] = (int32_t)i;
  for (int32_t t = 0; t < k; ++t) {
    const int32_t v = idx[(int64_t)t * n + i];
    if (v == NA_INT) continue;
    if (v - 1 != i) S[c++] = v - 1;
  }
  for (int a = 1; a < c; ++a) {                       // insertion sort (c <= k + 1)
    const int32_t x = S[a];
    int b = a - 1;
    while (b >= 0 && S[b] > x) { S[b + 1] = S[b]; --b; }
    S[b + 1] = x;
  }
  int u = 0;
  for (int a = 0; a < c; ++a)
    if (u == 0 || S[u - 1] != S[a]) S[u++] = S[a];
  return u;
}

// weight of slot a = (i, t): src/snn.cpp:224-242, inter_size :73-82,
// jaccard_from_counts :179-181; NA where idx is NA or a set is empty.
__device__ __forceinline__ double snn_weight(const int32_t* idx, int32_t n, int32_t k,
                                             const int32_t* sets, const int32_t* sizes,
                                             int64_t a) {
  const int64_t i = a % n;
  const int32_t v = idx[a];
  const int32_t ni = sizes[i];
  if (v == NA_INT || ni == 0) return na_real();
  const int64_t j = v - 1;
  const int32_t nj = sizes[j];
  if (nj == 0) return na_real();
  const int32_t* Si = sets + i * (int64_t)(k + 1);
  const int32_t* Sj = sets + j * (int64_t)(k + 1);
  int64_t c = 0, x = 0, y = 0;
  while (x < ni && y < nj) {
    const int32_t p = Si[x], q = Sj[y];
    if (p < q) ++x;
    else if (q < p) ++y;
    else { ++c; ++x; ++y; }
  }
  return (double)c / (double)((int64_t)ni + nj - c);
}

}  // namespace sdg
