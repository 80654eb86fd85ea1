// sdg_noalloc.cu -- SNN overlap weights without any device allocation.
//
// sdg_snn_jaccard needs scratch memory for the per-row neighbour sets and
// takes it from the CUDA memory pool on every call.  Some callers cannot let
// a library allocate device memory on their call path: a host framework that
// owns all device memory through its own allocator (and reserves nearly all
// of the GPU for it), a process that forbids cudaMalloc / cudaFree because
// they synchronise the device, or a latency-critical serving thread that must
// not touch the allocator at all.  For them sdg_snn_jaccard_noalloc takes
// device pointers for its input and output and keeps its scratch in one
// fixed array compiled into this library, g_noalloc_scratch, which every GPU
// that loads the library holds until the process exits.
//
// The array holds kNoallocScratchInts 32-bit integers (32 MiB): the sets need
// n * (k + 1), the set sizes n, and an error flag 1, so a call is accepted
// when n * (k + 2) + 1 <= kNoallocScratchInts.  All calls share the array and
// it keeps the last call's contents, so each call clears the error flag
// before use; two calls whose work overlaps on the GPU (different streams,
// or the same array reached from two threads) race on it.
#include "../../include/sdgpu.h"
#include "sdg_kernels.h"
#include "sdg_snn_core.cuh"

namespace sdg {
namespace {

constexpr int64_t kNoallocScratchInts = (int64_t)8 << 20;   // 32 MiB per device

static __device__ __align__(256) int32_t g_noalloc_scratch[kNoallocScratchInts];

// Host code may not use g_noalloc_scratch as an address: on the host the name
// is a stand-in for the device symbol.  Its device address is looked up on
// every call, in the calling thread's current context: an address cached
// across calls would go stale when the module is loaded again at another
// address (after cudaDeviceReset, or in another context of the same device).
// The lookup allocates nothing; the first one on a device loads the module,
// which is why the first call should come before any stream capture.

inline unsigned blocks_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

__global__ void k_na_check(const int32_t* idx, int64_t total, int32_t n, int32_t* flag) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < total;
       a += (int64_t)gridDim.x * blockDim.x) {
    if (snn_index_bad(idx[a], n)) { atomicOr(flag, 1); return; }
  }
}

__global__ void k_na_sets(const int32_t* idx, int32_t n, int32_t k, int include_self,
                          int32_t* sets, int32_t* sizes) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  sizes[i] = snn_build_set(idx, n, k, include_self, i, sets + i * (int64_t)(k + 1));
}

__global__ void k_na_weights(const int32_t* idx, int32_t n, int32_t k, const int32_t* sets,
                             const int32_t* sizes, double* w) {
  const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= (int64_t)n * k) return;
  w[a] = snn_weight(idx, n, k, sets, sizes, a);
}

int fail_with(int code, const char* msg) {
  set_error(msg);
  return code;
}

int cuda_fail(cudaError_t e) {
  set_error(cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? SDG_E_NOMEM : SDG_E_CUDA;
}

}  // namespace
}  // namespace sdg

using namespace sdg;

SDG_API int sdg_snn_jaccard_noalloc(const int32_t* d_idx, int32_t n, int32_t k,
                                               int include_self, double* d_w, void* stream) {
  if (n < 1 || k < 1)
    return fail_with(SDG_E_ARG, "'idx' must have at least one row and column.");
  if (!d_idx || !d_w) return fail_with(SDG_E_ARG, "d_idx and d_w must be device pointers.");
  const int64_t need = (int64_t)n * ((int64_t)k + 2) + 1;
  if (need > kNoallocScratchInts)
    return fail_with(SDG_E_UNSUPPORTED,
                     "sdg_snn_jaccard_noalloc: n * (k + 2) + 1 exceeds the fixed scratch of "
                     "8388608 integers; use sdg_snn_jaccard for this size.");
  void* sym = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&sym, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e);
  int32_t* scratch = static_cast<int32_t*>(sym);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int32_t* sets = scratch;
  int32_t* sizes = sets + (int64_t)n * (k + 1);
  int32_t* flag = sizes + n;
  const int64_t total = (int64_t)n * k;
  if ((e = cudaMemsetAsync(flag, 0, sizeof(int32_t), s)) != cudaSuccess) return cuda_fail(e);
  unsigned g = blocks_for(total, 256);
  if (g > 152u * 16u) g = 152u * 16u;
  k_na_check<<<g, 256, 0, s>>>(d_idx, total, n, flag);
  int32_t bad = 0;
  if ((e = cudaMemcpyAsync(&bad, flag, sizeof bad, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_fail(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e);
  if (bad)
    return fail_with(SDG_E_INDEX,
                     "'idx' entries must be NA or 1-based row indices in [1, nrow(idx)].");
  k_na_sets<<<blocks_for(n, 128), 128, 0, s>>>(d_idx, n, k, include_self, sets, sizes);
  k_na_weights<<<blocks_for(total, 256), 256, 0, s>>>(d_idx, n, k, sets, sizes, d_w);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
  return SDG_OK;
}
