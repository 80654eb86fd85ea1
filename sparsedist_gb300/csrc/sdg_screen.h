// sdg_screen.h -- the screened candidate engine: an FP32 / integer screen over
// every (query, reference) pair with a rigorous error bound, a candidate list
// per query column, and an exact FP64 re-rank of the candidates (sdg_exact.cu)
// followed by the exact top-k (sdg_select.cu).
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <functional>

#include "sdg_common.cuh"

namespace sdg {

// Screening data derived from one matrix for one method, kept with the
// matrix so that a resident reference pays for it once.
struct ScreenCache {
  int method = -1;
  void* blob = nullptr;      // one device allocation holding the arrays below
  float* fval = nullptr;     // per stored entry: value the screen multiplies
  float* fxl = nullptr;      // js: per stored entry, x log x of the value (FP32)
  float* cnorm = nullptr;    // per column: norm term of the method (js: sum of |x log x| + x, rounded up)
  int32_t* nnz = nullptr;    // per column: stored entries
  int32_t* perm = nullptr;   // columns in descending-nnz order
  int64_t nnz_total = 0;
  // js / pearson / covariance: every nonzero stored value lies in the range
  // the method's FP32 bound is derived for ([2^-100, 2^100] for js, |value| in
  // [2^-50, 2^50] for the moment methods); else the searches of this matrix
  // with that method are exact
  bool values_ok = true;
};

// Dense FP16 copy of one matrix's screen values for the tensor-core screen
// (cosine: the unit values; euclidean: the values; binary: 1), one column of
// ld rows (nrow rounded up to 64, zero below nrow) per matrix column; values
// below FP16's smallest normal are stored as 0.  usable = 0 when a value is
// not finite or beyond FP16's range: the FP32 screen is used instead.
struct TensorCache {
  int method = -1;
  int usable = 0;
  void* dense = nullptr;     // __half[ncol * ld]
  int64_t ld = 0;
  // per column, rounded up to FP32: err = ||v - h(v)||_2 and bn = ||h(v)||_2,
  // v the exact values the key is defined on (FP64 unit values for cosine,
  // the values for euclidean)
  float* err = nullptr;
  float* bn = nullptr;
};

struct ScreenRun {
  int method = 0, dist = 1, k = 1;
  // the tensor-core screen (the fused tcgen05 FP16 screen, sdg_sparse_tc.cu)
  // instead of the FP32 sparse screen, when tensor_supported(method),
  // stc_supported(k) and both matrices' TensorCache are usable
  bool tensor = false;
  bool decreasing = false, selfmode = false, include_self = false;
  double self_value = 0.0;                 // restored self value (include_self)
  const uint8_t* ref_mask = nullptr;       // excluded reference columns
  const uint8_t* qry_blank = nullptr;      // query rows written all-NA
  const uint8_t* qry_empty = nullptr;      // all-zero query columns
  // query columns [q_lo, q_hi) of the query matrix (q_hi < 0: all); result
  // row of query q is q - out_first in an output with leading dimension
  // out_ld (< 0: the query count)
  int64_t q_lo = 0, q_hi = -1, out_first = 0, out_ld = -1;
};

struct ScreenHooks {
  std::function<void()> check_cancel;
  std::function<void()> time_begin, time_end;        // bracket the screen kernel
  std::function<void(int64_t, int64_t)> exact_range;  // finish queries [q0, q0+n) exactly
};

// The fused tcgen05 screen of the tensor engine (sdg_sparse_tc.cu): the FP16
// GEMM of the query block against every reference column with the
// selection of the slab path in its epilogue.  Fills cand / count / over (as
// the slab selection does) for queries q0 .. q0 + nq - 1 of the query matrix.
struct StcRun {
  int method = 0, k = 1;
  int selfmode = 0, include_self = 0;
  int64_t ld = 0;                          // rows of the dense copies (multiple of 64)
  int64_t nr = 0, q0 = 0, nq = 0;
  const __half* rdense = nullptr;          // TensorCache of the reference
  const __half* qdense = nullptr;          // TensorCache of the query matrix
  const int32_t* rnnz = nullptr; const float* rnorm = nullptr;
  const float* rerr = nullptr; const float* rbn = nullptr;
  const uint8_t* ref_mask = nullptr;
  const int32_t* qnnz = nullptr; const float* qnorm = nullptr;
  const float* qerr = nullptr; const float* qbn = nullptr;
  const uint8_t* qry_blank = nullptr;      // global query index
  const uint8_t* qry_force = nullptr;
};
bool stc_supported(int k);
// the call that failed in the last screen_knn error on this thread
const char* screen_error_site();
// 0 or a cudaError_t value (the message is set)
int stc_screen(const StcRun& r, cudaStream_t s, int32_t* cand, int32_t* count, int32_t* over, int cap,
               const std::function<void()>& time_begin, const std::function<void()>& time_end);

bool screen_supported(int method, int k);
bool screen_fits(int32_t nrow);
bool tensor_supported(int method);
// bytes of the TensorCache of an nrow x ncol matrix
size_t tensor_cache_bytes(int32_t nrow, int64_t ncol);

// Returns 0 or a cudaError_t value; exceptions thrown by the hooks propagate.
// stats: see sdg_last_stats in include/sdgpu.h.
// rt / qt: the TensorCaches of ref / qry (the same object for a self-search).
int screen_knn(cudaStream_t s, const ScreenRun& r, const DevCsc& ref, const ColAux& ra,
               ScreenCache* rc, TensorCache* rt, const DevCsc& qry, const ColAux& qa, ScreenCache* qc,
               TensorCache* qt, int32_t* d_idx, double* d_val, int64_t* stats, const ScreenHooks& hooks);

void screen_cache_free(ScreenCache* c, cudaStream_t s);
void tensor_cache_free(TensorCache* c, cudaStream_t s);

// Device check used at upload: rows in [0, nrow) and strictly ascending.
void launch_check_rows(const DevCsc& M, int* err, cudaStream_t s);

}  // namespace sdg
