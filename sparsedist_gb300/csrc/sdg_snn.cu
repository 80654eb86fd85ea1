// sdg_snn.cu -- shared-nearest-neighbour weights and the SNN graph.
//
// snnJaccard (src/snn.cpp:197-250): each row's neighbour set is built once
// (NA dropped, self removed and re-added iff include_self, sorted,
// de-duplicated), then w(i, t) = |N(i) n N(j)| / |N(i) u N(j)| from integer
// counts and one IEEE division, so the weights are bit-identical to the
// reference.  The graph (R/sparseSNN.R:221-250) is assembled on the device:
// kept triplets -> (column, row) keys -> radix sort -> unique -> CSC.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include "sdg_kernels.h"
#include "sdg_snn_core.cuh"

namespace sdg {
namespace {

inline unsigned blocks_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

__global__ void k_snn_check(const int32_t* idx, int64_t total, int32_t n, int* err) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < total;
       a += (int64_t)gridDim.x * blockDim.x) {
    if (snn_index_bad(idx[a], n)) { atomicOr(err, 1); return; }
  }
}

__global__ void k_snn_sets(const int32_t* idx, int32_t n, int32_t k, int include_self,
                           int32_t* sets, int32_t* sizes) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  sizes[i] = snn_build_set(idx, n, k, include_self, i, sets + i * (int64_t)(k + 1));
}

__global__ void k_snn_weights(const int32_t* idx, int32_t n, int32_t k, const int32_t* sets,
                              const int32_t* sizes, double* w) {
  const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= (int64_t)n * k) return;
  w[a] = snn_weight(idx, n, k, sets, sizes, a);
}

// keep <- !is.na(w) & !is.na(idx) & (w > prune)  (R/sparseSNN.R:226); each kept
// slot emits key col * n + row (and the mirrored key when symmetrising).
__global__ void k_snn_triplets(const int32_t* idx, const double* w, int32_t n, int32_t k,
                               double prune, int symmetrise, uint64_t* keys, double* vals,
                               unsigned long long* count) {
  const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= (int64_t)n * k) return;
  const int32_t v = idx[a];
  const double x = w[a];
  if (v == NA_INT || isnan(x) || !(x > prune)) return;
  const uint64_t i = (uint64_t)(a % n), j = (uint64_t)(v - 1);
  const unsigned long long at = atomicAdd(count, symmetrise ? 2ull : 1ull);
  keys[at] = j * (uint64_t)n + i;
  vals[at] = x;
  if (symmetrise) { keys[at + 1] = i * (uint64_t)n + j; vals[at + 1] = x; }
}

// p[c] = first position whose key >= c * n
__global__ void k_snn_colptr(const uint64_t* keys, int64_t m, int32_t n, int32_t* p) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c > n) return;
  const uint64_t target = (uint64_t)c * (uint64_t)n;
  int64_t lo = 0, hi = m;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < target) lo = mid + 1; else hi = mid;
  }
  p[c] = (int32_t)lo;
}

__global__ void k_snn_rows(const uint64_t* keys, int64_t m, int32_t n, int32_t* rows) {
  const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a < m) rows[a] = (int32_t)(keys[a] % (uint64_t)n);
}

int key_bits(int32_t n) {
  const uint64_t maxkey = (uint64_t)n * (uint64_t)n;
  int b = 1;
  while (b < 64 && (maxkey >> b) != 0) ++b;
  return b;
}

}  // namespace

void launch_snn_check(const int32_t* idx, int32_t n, int32_t k, int* err, cudaStream_t s) {
  const int64_t total = (int64_t)n * k;
  unsigned g = blocks_for(total, 256);
  if (g > 152u * 16u) g = 152u * 16u;
  if (total > 0) k_snn_check<<<g, 256, 0, s>>>(idx, total, n, err);
}

void launch_snn_sets(const int32_t* idx, int32_t n, int32_t k, int include_self,
                     int32_t* sets, int32_t* sizes, cudaStream_t s) {
  if (n > 0) k_snn_sets<<<blocks_for(n, 128), 128, 0, s>>>(idx, n, k, include_self, sets, sizes);
}

void launch_snn_weights(const int32_t* idx, int32_t n, int32_t k, const int32_t* sets,
                        const int32_t* sizes, double* w, cudaStream_t s) {
  const int64_t total = (int64_t)n * k;
  if (total > 0) k_snn_weights<<<blocks_for(total, 256), 256, 0, s>>>(idx, n, k, sets, sizes, w);
}

#define SDG_TRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return (int)e_; } while (0)

int snn_graph_build(const int32_t* d_idx, const double* d_w, int32_t n, int32_t k,
                    double prune, int symmetrise, int64_t* nnz_host, int32_t** d_p,
                    int32_t** d_i, double** d_x, cudaStream_t s) {
  const int64_t slots = (int64_t)n * k;
  const int64_t cap = slots * (symmetrise ? 2 : 1) + 1;
  uint64_t *keys = nullptr, *keys2 = nullptr, *ukeys = nullptr;
  double *vals = nullptr, *vals2 = nullptr, *uvals = nullptr;
  unsigned long long* count = nullptr;
  int64_t* nsel = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0, tmp2 = 0;
  SDG_TRY(cudaMallocAsync(&keys, cap * sizeof(uint64_t), s));
  SDG_TRY(cudaMallocAsync(&keys2, cap * sizeof(uint64_t), s));
  SDG_TRY(cudaMallocAsync(&vals, cap * sizeof(double), s));
  SDG_TRY(cudaMallocAsync(&vals2, cap * sizeof(double), s));
  SDG_TRY(cudaMallocAsync(&count, sizeof(unsigned long long) + sizeof(int64_t), s));
  nsel = reinterpret_cast<int64_t*>(count + 1);
  SDG_TRY(cudaMemsetAsync(count, 0, sizeof(unsigned long long), s));
  if (slots > 0)
    k_snn_triplets<<<blocks_for(slots, 256), 256, 0, s>>>(d_idx, d_w, n, k, prune, symmetrise,
                                                          keys, vals, count);
  unsigned long long m_host = 0;
  SDG_TRY(cudaMemcpyAsync(&m_host, count, sizeof m_host, cudaMemcpyDeviceToHost, s));
  SDG_TRY(cudaStreamSynchronize(s));
  const int64_t m = (int64_t)m_host;
  const int bits = key_bits(n);
  SDG_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, vals, vals2, (int)m,
                                          0, bits, s));
  SDG_TRY(cub::DeviceSelect::UniqueByKey(nullptr, tmp2, keys2, vals2, keys, vals, nsel, (int)m, s));
  if (tmp2 > tmp_bytes) tmp_bytes = tmp2;
  SDG_TRY(cudaMallocAsync(&tmp, tmp_bytes + 16, s));
  if (m > 0) {
    SDG_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, vals, vals2, (int)m, 0,
                                            bits, s));
    SDG_TRY(cub::DeviceSelect::UniqueByKey(tmp, tmp_bytes, keys2, vals2, keys, vals, nsel,
                                           (int)m, s));
  } else {
    SDG_TRY(cudaMemsetAsync(nsel, 0, sizeof(int64_t), s));
  }
  int64_t u = 0;
  SDG_TRY(cudaMemcpyAsync(&u, nsel, sizeof u, cudaMemcpyDeviceToHost, s));
  SDG_TRY(cudaStreamSynchronize(s));
  ukeys = keys;
  uvals = vals;
  int32_t* p = nullptr;
  int32_t* rows = nullptr;
  SDG_TRY(cudaMallocAsync(&p, sizeof(int32_t) * ((size_t)n + 1), s));
  SDG_TRY(cudaMallocAsync(&rows, sizeof(int32_t) * ((size_t)u + 1), s));
  k_snn_colptr<<<blocks_for((int64_t)n + 1, 256), 256, 0, s>>>(ukeys, u, n, p);
  if (u > 0) k_snn_rows<<<blocks_for(u, 256), 256, 0, s>>>(ukeys, u, n, rows);
  SDG_TRY(cudaGetLastError());
  SDG_TRY(cudaFreeAsync(keys2, s));
  SDG_TRY(cudaFreeAsync(vals2, s));
  SDG_TRY(cudaFreeAsync(count, s));
  SDG_TRY(cudaFreeAsync(tmp, s));
  SDG_TRY(cudaFreeAsync(ukeys, s));
  *nnz_host = u;
  *d_p = p;
  *d_i = rows;
  *d_x = uvals;   // values already compacted in key order
  return 0;
}

}  // namespace sdg
