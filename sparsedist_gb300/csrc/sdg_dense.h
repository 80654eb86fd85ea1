// sdg_dense.h -- the resident dense-embedding matrix and what the two screens
// of the dense path (sdg_dense.cu: cuBLAS slab; sdg_dense_tc.cu: fused
// tcgen05 kernel) share.
#pragma once

#include <cstdint>
#include <mutex>
#include <cublas_v2.h>
#include <cuda_bf16.h>

#include "sdg_kernels.h"

struct sdg_dense {
  int device = 0;
  int32_t d = 0;
  int64_t n = 0;
  int64_t npad = 0;               // n rounded up to 128 (padding of norm2 / empty)
  double* x64 = nullptr;          // d x n column-major
  double* u64 = nullptr;          // unit columns (unit_csc on the dense column)
  float* x32 = nullptr;
  float* u32 = nullptr;
  __nv_bfloat16* xb = nullptr;    // d x n
  __nv_bfloat16* ub = nullptr;
  int32_t dpad = 0;               // d rounded up to 64: rows of 128-byte multiples
  __nv_bfloat16* xbp = nullptr;   // dpad x n, zero rows below d (aliases xb when dpad == d)
  __nv_bfloat16* ubp = nullptr;
  float* norm2 = nullptr;         // sum of squares (FP64, rounded), padded to npad with 0
  // per column, for the fused screen's per-pair bound: the exact norm of each
  // BF16 copy's rounding error and of the copy (FP64, rounded up), unit
  // columns (cosine) and columns (euclidean); [npad], 0 past n
  float* ue = nullptr;
  float* un = nullptr;
  float* xe = nullptr;
  float* xn = nullptr;
  double* scale = nullptr;        // unit_csc scale (0 = empty column)
  uint8_t* empty = nullptr;       // padded to npad with 1
  int64_t n_empty = 0;
  cublasHandle_t blas = nullptr;  // slab (mode 2) and plain (mode 1) GEMMs; resident references only
  std::mutex blas_mu;             // one caller at a time on `blas` (it is bound to a stream)
  bool async = false;             // buffers from the stream-ordered pool of `stream`
  cudaStream_t stream = nullptr;
};

namespace sdg {

// Screen key of one pair from its FP32 inner product s (of unit columns for
// cosine, of the columns for euclidean) and the bound err on |key - exact|:
//   cosine     key = s                  err = rel
//   euclidean  key = 2 s - (Nq + Nr)    err = 2 rel sqrt(Nq Nr) + 2^-20 (Nq + Nr)
// with rel = 0.0040 + d 2^-22 for BF16 operands and err = 0 in the plain
// FP32 mode.  Larger keys are nearer.
__device__ __forceinline__ void dense_key(int method, int mode, int32_t d, float s, float Nq, float Nr,
                                          float& key, float& err) {
  const float rel = 0.0040f + (float)d * 2.384185791015625e-7f;   // 2^-22
  if (method == COSINE) {
    key = s;
    err = mode == 0 ? rel : 0.f;
  } else {
    key = 2.f * s - (Nq + Nr);
    err = mode == 0 ? 2.f * rel * sqrtf(Nq * Nr) + 9.5367431640625e-7f * (Nq + Nr) + 1e-30f : 0.f;
  }
}

// cut = T - margin(T): the FP32 allowance under the k-th pessimistic key T
__device__ __forceinline__ float dense_cut(float T) {
  return (T == -INFINITY) ? -INFINITY : T - (fabsf(T) * 4.76837158203125e-7f + 1e-30f);
}

// Fused tensor-core screen (sdg_dense_tc.cu).  Supported for cosine and
// euclidean with k <= 64 and dpad <= 256.  Fills, for the nq queries q0.., the
// candidate lists cand[ql * cap + t] (t < count[ql]) with every reference
// whose optimistic key reaches the query's cut, or sets over[ql] (count 0)
// when a list does not fit; degenerate queries get count 0.
// Queries are columns q0.. of Q, references the columns of D (self: Q is D
// and each query's own column is skipped).
bool tc_screen_supported(const sdg_dense* D, int method, int k);
// allow_pairs: run CTA pairs (cta_group::2, M = 256) where the block has more
// than one 128-query group; otherwise one CTA per query group.  status: a
// device int that a pipeline wait which ran out sets to 1; the call returns
// without synchronising and the caller reads it with the results.
int tc_screen(sdg_ctx* ctx, const sdg_dense* Q, const sdg_dense* D, bool self, int method, int k, int64_t q0,
              int64_t nq, int32_t* cand, int32_t* count, int32_t* over, int cap, cudaStream_t s,
              bool allow_pairs, int* status);

}  // namespace sdg
