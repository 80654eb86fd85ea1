// sdg_common.cuh -- device-side types and helpers shared by the kernels of
// libsdgpu.so.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sdg {

enum Method { BINARY = 0, COSINE = 1, EUCLIDEAN = 2, MANHATTAN = 3, PEARSON = 4, JS = 5, COVARIANCE = 6 };
constexpr int kMethodCount = 7;

constexpr int32_t NA_INT = INT32_MIN;
constexpr uint64_t NA_REAL_BITS = 0x7FF00000000007A2ULL;   // R's NA_real_

// A CSC matrix in device memory.  Column offsets are 64-bit so that address
// arithmetic never overflows; row indices are int32 as in a dgCMatrix.
struct DevCsc {
  int32_t nrow = 0, ncol = 0;
  const int64_t* p = nullptr;
  const int32_t* i = nullptr;
  const double* x = nullptr;
};

// Per-column data derived once per matrix (and per method family).
struct ColAux {
  const uint8_t* empty = nullptr;   // every stored value is +-0
  const double* uval = nullptr;     // cosine: unit-normalised values (nnz)
  const double* scale = nullptr;    // cosine: largest |value| (0 = empty column)
  const double* s = nullptr;        // pearson: sum of values
  const double* ss = nullptr;       // pearson: sum of squares
  const float* fval = nullptr;      // screening: float copy of the values the
                                    // screen multiplies (unit values for cosine)
  const float* norm = nullptr;      // screening: per-column norm term (method-specific)
  const double* xl = nullptr;       // js: xlogx of each stored value (nnz), or null
  const double* xsum = nullptr;     // js: sum of each column's values, or null
};

__host__ __device__ inline double na_real() {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)NA_REAL_BITS);
#else
  union { uint64_t u; double d; } c{NA_REAL_BITS};
  return c.d;
#endif
}

#ifdef __CUDACC__
// Order-preserving map of a finite double onto uint64 (ascending value ->
// ascending key), flipped for "larger is better".  -0 maps like +0, so the
// comparison agrees with IEEE equality, which is what the reference's
// comparator (value, index) uses; the value itself is carried beside the key.
__device__ __forceinline__ uint64_t order_key(double v, bool decreasing) {
  if (v == 0.0) v = 0.0;
  uint64_t b = (uint64_t)__double_as_longlong(v);
  b = (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
  return decreasing ? ~b : b;
}

#endif

}  // namespace sdg
