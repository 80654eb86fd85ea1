// sdg_snn.cu -- shared-nearest-neighbour weights and the SNN graph.
//
// snnJaccard (src/snn.cpp:197-250): each row's neighbour set is built once
// (NA dropped, self removed and re-added iff include_self, sorted,
// de-duplicated), then w(i, t) = |N(i) n N(j)| / |N(i) u N(j)| from integer
// counts and one IEEE division, so the weights are bit-identical to the
// reference.  The graph (R/sparseSNN.R:221-250) is assembled on the device:
// kept triplets -> (column, row) keys -> radix sort -> unique -> CSC.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>
#include <cstdlib>
#include <utility>
#include <vector>

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

// ---- sparseSNN(edges = "shared"): snnJaccardShared (src/snn.cpp:252-447) ---
//
// The pairs (i, j), i < j, sharing a neighbour are the nonzeros of the upper
// triangle of A A^T (A the n x n neighbourhood-membership matrix); their
// overlap counts u are found by sorting instead of a per-row accumulator:
// every (i, m in N(i), j in R(m), j > i) emits the key i n + j, a radix sort
// brings equal keys together and a run-length encode counts them.  R(m) =
// {i : m in N(i)} comes from a stable sort of the (m, i) pairs, so it is
// ascending and j > i is a binary search.  Weights u / (|N(i)| + |N(j)| - u)
// are the reference's integer counts and one IEEE division.

// (m, i) for every member m of every set N(i), in (i, position) order
__global__ void k_shared_pairs(const int32_t* sets, const int32_t* sizes, const int64_t* off, int32_t n,
                               int32_t k, uint32_t* mkeys, int32_t* ivals) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t* S = sets + i * (int64_t)(k + 1);
  const int64_t o = off[i];
  for (int32_t a = 0; a < sizes[i]; ++a) { mkeys[o + a] = (uint32_t)S[a]; ivals[o + a] = (int32_t)i; }
}

// rev_ptr[m] = first position of key m in the sorted member keys
__global__ void k_shared_revptr(const uint32_t* keys, int64_t t, int32_t n, int64_t* rp) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m > n) return;
  int64_t lo = 0, hi = t;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < (uint32_t)m) lo = mid + 1; else hi = mid;
  }
  rp[m] = lo;
}

// first position in R(m) holding a row > i
__device__ __forceinline__ int64_t shared_after(const int32_t* rev, int64_t lo, int64_t hi, int32_t i) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (rev[mid] <= i) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// per (i, member slot): how many j > i share that member
__global__ void k_shared_count(const int32_t* mk_by_i, const int32_t* iv_by_i, int64_t t, const int64_t* rp,
                               const int32_t* rev, int64_t* cnt) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= t) return;
  const int32_t m = mk_by_i[e], i = iv_by_i[e];
  cnt[e] = rp[m + 1] - shared_after(rev, rp[m], rp[m + 1], i);
}

// the keys of members t0 .. t1 - 1 (whole rows), at pos[e] - base
__global__ void k_shared_emit(const int32_t* mk_by_i, const int32_t* iv_by_i, int64_t t0, int64_t t1,
                              const int64_t* rp, const int32_t* rev, const int64_t* pos, int64_t base,
                              int32_t n, uint64_t* keys) {
  const int64_t e = t0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= t1) return;
  const int32_t m = mk_by_i[e], i = iv_by_i[e];
  const int64_t q0 = shared_after(rev, rp[m], rp[m + 1], i);
  uint64_t* out = keys + (pos[e] - base);
  for (int64_t q = q0; q < rp[m + 1]; ++q) out[q - q0] = (uint64_t)i * (uint64_t)n + (uint64_t)rev[q];
}

// rowpos[i] = number of keys before row i's first member (members are in
// row order; a row without members starts where the next one does)
__global__ void k_shared_rowpos(const int64_t* off, const int64_t* pos, const int64_t* cnt, int64_t t,
                                int32_t n, int64_t* rowpos) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i > n) return;
  const int64_t o = off[i];
  rowpos[i] = (o < t) ? pos[o] : (t > 0 ? pos[t - 1] + cnt[t - 1] : 0);
}

// one run = one pair (i, j) with its overlap count: weight, prune, and both
// triangle entries as (column, row) keys
__global__ void k_shared_weights(const uint64_t* ukeys, const int32_t* counts, const int64_t* nruns,
                                 const int32_t* sizes, int32_t n, double prune, uint64_t* okeys,
                                 double* ovals, unsigned long long* kept) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= *nruns) return;
  const uint64_t key = ukeys[r];
  const uint64_t i = key / (uint64_t)n, j = key % (uint64_t)n;
  const int64_t u = counts[r];
  const double w = (double)u / (double)((int64_t)sizes[i] + sizes[j] - u);
  if (!(w > prune)) return;
  const unsigned long long at = atomicAdd(kept, 2ull);
  okeys[at] = j * (uint64_t)n + i;        // (row i, column j)
  ovals[at] = w;
  okeys[at + 1] = i * (uint64_t)n + j;    // (row j, column i)
  ovals[at + 1] = w;
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

// Device buffers of one build, released on every return path (stream
// ordered); release() hands a buffer to the caller instead.
struct AsyncBufs {
  cudaStream_t s;
  std::vector<void*> held;
  explicit AsyncBufs(cudaStream_t st) : s(st) {}
  ~AsyncBufs() { for (void* q : held) if (q) cudaFreeAsync(q, s); }
  template <class T> cudaError_t alloc(T** out, size_t count) {
    *out = nullptr;
    const cudaError_t e = cudaMallocAsync((void**)out, sizeof(T) * (count ? count : 1), s);
    if (e == cudaSuccess) held.push_back((void*)*out);
    return e;
  }
  void drop(void* q) {
    for (auto& h : held) if (h == q) { cudaFreeAsync(h, s); h = nullptr; }
  }
  void release(void* q) {
    for (auto& h : held) if (h == q) h = nullptr;
  }
};

int snn_shared_build(const int32_t* d_sets, const int32_t* d_sizes, int32_t n, int32_t k, double prune,
                     int64_t* nnz_host, int32_t** d_p, int32_t** d_i, double** d_x, cudaStream_t s) {
  AsyncBufs B(s);
  size_t tb = 0, tb2 = 0;
  void* tmp = nullptr;
  // set sizes -> offsets of the (m, i) member pairs
  int64_t *off = nullptr, *sz64 = nullptr;
  SDG_TRY(B.alloc(&off, (size_t)n + 1));
  SDG_TRY(B.alloc(&sz64, (size_t)n + 1));
  // exclusive sum of the set sizes, widened to int64 (a strided copy into the
  // low words of a zeroed int64 array; sizes are non-negative)
  SDG_TRY(cudaMemsetAsync(sz64, 0, sizeof(int64_t) * ((size_t)n + 1), s));
  SDG_TRY(cudaMemcpy2DAsync(sz64, sizeof(int64_t), d_sizes, sizeof(int32_t), sizeof(int32_t), (size_t)n,
                            cudaMemcpyDeviceToDevice, s));
  SDG_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tb, sz64, off, (int)n + 1, s));
  SDG_TRY(B.alloc((char**)&tmp, tb + 16));
  SDG_TRY(cub::DeviceScan::ExclusiveSum(tmp, tb, sz64, off, (int)n + 1, s));
  B.drop(tmp);
  B.drop(sz64);
  int64_t t = 0;
  SDG_TRY(cudaMemcpyAsync(&t, off + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  SDG_TRY(cudaStreamSynchronize(s));
  uint32_t *mk = nullptr, *mk2 = nullptr;
  int32_t *iv = nullptr, *rev = nullptr;
  int64_t *rp = nullptr, *cnt = nullptr, *pos = nullptr;
  SDG_TRY(B.alloc(&mk, (size_t)t + 1));
  SDG_TRY(B.alloc(&mk2, (size_t)t + 1));
  SDG_TRY(B.alloc(&iv, (size_t)t + 1));
  SDG_TRY(B.alloc(&rev, (size_t)t + 1));
  SDG_TRY(B.alloc(&rp, (size_t)n + 1));
  SDG_TRY(B.alloc(&cnt, (size_t)t + 1));
  SDG_TRY(B.alloc(&pos, (size_t)t + 1));
  k_shared_pairs<<<blocks_for(n, 128), 128, 0, s>>>(d_sets, d_sizes, off, n, k, mk, iv);
  // R(m): a stable sort by m keeps each R(m) in ascending i
  int mbits = 1;
  while (mbits < 32 && ((uint64_t)n >> mbits) != 0) ++mbits;
  SDG_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, mk, mk2, iv, rev, (int)t, 0, mbits, s));
  SDG_TRY(B.alloc((char**)&tmp, tb + 16));
  if (t > 0) SDG_TRY(cub::DeviceRadixSort::SortPairs(tmp, tb, mk, mk2, iv, rev, (int)t, 0, mbits, s));
  B.drop(tmp);
  k_shared_revptr<<<blocks_for((int64_t)n + 1, 256), 256, 0, s>>>(mk2, t, n, rp);
  // the members in (i, position) order again (mk / iv were sort inputs, unchanged)
  if (t > 0) {
    k_shared_count<<<blocks_for(t, 256), 256, 0, s>>>(reinterpret_cast<const int32_t*>(mk), iv, t, rp, rev, cnt);
    SDG_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt, pos, (int)t, s));
    SDG_TRY(B.alloc((char**)&tmp, tb + 16));
    SDG_TRY(cub::DeviceScan::ExclusiveSum(tmp, tb, cnt, pos, (int)t, s));
    B.drop(tmp);
  }
  // key count before each row's first member: chunks of whole rows, so that
  // every pair (i, j), whose keys all come from row i's members, is counted
  // within one chunk
  int64_t* rowpos = nullptr;
  SDG_TRY(B.alloc(&rowpos, (size_t)n + 1));
  k_shared_rowpos<<<blocks_for((int64_t)n + 1, 256), 256, 0, s>>>(off, pos, cnt, t, n, rowpos);
  std::vector<int64_t> h_rowpos((size_t)n + 1), h_off((size_t)n + 1);
  SDG_TRY(cudaMemcpyAsync(h_rowpos.data(), rowpos, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
  SDG_TRY(cudaMemcpyAsync(h_off.data(), off, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
  SDG_TRY(cudaStreamSynchronize(s));
  // one row emits at most (k + 1) n keys; a chunk holds at least one row.
  // 2^28 keys (2 GiB of keys, about 7 GiB with the sort's buffers) unless
  // SDG_SNN_CHUNK_KEYS asks for less
  int64_t want = (int64_t)1 << 28;
  if (const char* ev = std::getenv("SDG_SNN_CHUNK_KEYS")) {
    const long long v = std::atoll(ev);
    if (v > 0) want = std::min<int64_t>(want, (int64_t)v);
  }
  const int64_t chunk_cap = std::max<int64_t>(want, (int64_t)(k + 1) * n);
  std::vector<std::pair<int32_t, int32_t>> chunks;
  int64_t max_chunk = 0;
  for (int32_t i0 = 0; i0 < n;) {
    int32_t i1 = i0 + 1;
    while (i1 < n && h_rowpos[(size_t)i1 + 1] - h_rowpos[(size_t)i0] <= chunk_cap) ++i1;
    const int64_t e = h_rowpos[(size_t)i1] - h_rowpos[(size_t)i0];
    if (e > 0) {
      chunks.emplace_back(i0, i1);
      max_chunk = std::max(max_chunk, e);
    }
    i0 = i1;
  }
  if (max_chunk >= ((int64_t)1 << 31)) return (int)cudaErrorInvalidValue;
  const int bits = key_bits(n);
  uint64_t *keys = nullptr, *keys2 = nullptr, *okeys = nullptr;
  int32_t* counts = nullptr;
  double* ovals = nullptr;
  int64_t* nruns = nullptr;
  unsigned long long* kept = nullptr;
  SDG_TRY(B.alloc(&keys, (size_t)max_chunk + 1));
  SDG_TRY(B.alloc(&keys2, (size_t)max_chunk + 1));
  SDG_TRY(B.alloc(&counts, (size_t)max_chunk + 1));
  SDG_TRY(B.alloc(&nruns, 1));
  SDG_TRY(B.alloc(&kept, 1));
  SDG_TRY(cudaMemsetAsync(kept, 0, sizeof(unsigned long long), s));
  if (max_chunk > 0) {
    SDG_TRY(cub::DeviceRadixSort::SortKeys(nullptr, tb, keys, keys2, (int)max_chunk, 0, bits, s));
    SDG_TRY(cub::DeviceRunLengthEncode::Encode(nullptr, tb2, keys2, keys, counts, nruns, (int)max_chunk, s));
    if (tb2 > tb) tb = tb2;
    SDG_TRY(B.alloc((char**)&tmp, tb + 16));
  }
  int64_t out_cap = 0, kept_total = 0;
  for (const auto& ch : chunks) {
    const int64_t base = h_rowpos[(size_t)ch.first];
    const int64_t e = h_rowpos[(size_t)ch.second] - base;
    const int64_t t0 = h_off[(size_t)ch.first], t1 = h_off[(size_t)ch.second];
    k_shared_emit<<<blocks_for(t1 - t0, 256), 256, 0, s>>>(reinterpret_cast<const int32_t*>(mk), iv, t0, t1, rp,
                                                           rev, pos, base, n, keys);
    size_t tbs = tb;
    SDG_TRY(cub::DeviceRadixSort::SortKeys(tmp, tbs, keys, keys2, (int)e, 0, bits, s));
    tbs = tb;
    SDG_TRY(cub::DeviceRunLengthEncode::Encode(tmp, tbs, keys2, keys, counts, nruns, (int)e, s));
    int64_t runs = 0;
    SDG_TRY(cudaMemcpyAsync(&runs, nruns, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    SDG_TRY(cudaStreamSynchronize(s));
    if (kept_total + 2 * runs > out_cap) {            // grow the kept (key, weight) lists
      const int64_t cap = std::max<int64_t>(2 * out_cap, kept_total + 2 * runs);
      uint64_t* nk = nullptr;
      double* nv = nullptr;
      SDG_TRY(B.alloc(&nk, (size_t)cap));
      SDG_TRY(B.alloc(&nv, (size_t)cap));
      if (kept_total > 0) {
        SDG_TRY(cudaMemcpyAsync(nk, okeys, sizeof(uint64_t) * (size_t)kept_total, cudaMemcpyDeviceToDevice, s));
        SDG_TRY(cudaMemcpyAsync(nv, ovals, sizeof(double) * (size_t)kept_total, cudaMemcpyDeviceToDevice, s));
      }
      if (okeys) B.drop(okeys);
      if (ovals) B.drop(ovals);
      okeys = nk;
      ovals = nv;
      out_cap = cap;
    }
    if (runs > 0)
      k_shared_weights<<<blocks_for(runs, 256), 256, 0, s>>>(keys, counts, nruns, d_sizes, n, prune, okeys, ovals,
                                                            kept);
    unsigned long long m_host = 0;
    SDG_TRY(cudaMemcpyAsync(&m_host, kept, sizeof m_host, cudaMemcpyDeviceToHost, s));
    SDG_TRY(cudaStreamSynchronize(s));
    kept_total = (int64_t)m_host;
  }
  const int64_t m = kept_total;
  if (m >= ((int64_t)1 << 31)) return (int)cudaErrorInvalidValue;   // beyond a dgCMatrix
  uint64_t* okeys2 = nullptr;
  double* ovals2 = nullptr;
  SDG_TRY(B.alloc(&okeys2, (size_t)m + 1));
  SDG_TRY(B.alloc(&ovals2, (size_t)m + 1));
  if (m > 0) {
    size_t tbo = 0;
    SDG_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tbo, okeys, okeys2, ovals, ovals2, (int)m, 0, bits, s));
    void* tmp2 = nullptr;
    SDG_TRY(B.alloc((char**)&tmp2, tbo + 16));
    SDG_TRY(cub::DeviceRadixSort::SortPairs(tmp2, tbo, okeys, okeys2, ovals, ovals2, (int)m, 0, bits, s));
  }
  int32_t* p = nullptr;
  int32_t* rows = nullptr;
  SDG_TRY(B.alloc(&p, (size_t)n + 1));
  SDG_TRY(B.alloc(&rows, (size_t)m + 1));
  k_snn_colptr<<<blocks_for((int64_t)n + 1, 256), 256, 0, s>>>(okeys2, m, n, p);
  if (m > 0) k_snn_rows<<<blocks_for(m, 256), 256, 0, s>>>(okeys2, m, n, rows);
  SDG_TRY(cudaGetLastError());
  B.release(p);
  B.release(rows);
  B.release(ovals2);
  *nnz_host = m;
  *d_p = p;
  *d_i = rows;
  *d_x = ovals2;
  return 0;
}

}  // namespace sdg
