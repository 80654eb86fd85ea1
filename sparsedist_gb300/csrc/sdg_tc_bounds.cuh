// sdg_tc_bounds.cuh -- the rigorous bound of the tensor-core screen of the
// sparse path, shared by the slab selection (sdg_screen.cu) and the fused
// tcgen05 screen (sdg_sparse_tc.cu), so that both compute the same FP32 keys.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>

#include "sdg_common.cuh"

namespace sdg {
namespace tcb {

constexpr float U32 = 5.9604644775390625e-8f;       // 2^-24
constexpr float ACC_ULP = 4.76837158203125e-7f;     // 2^-21

// The tensor-screen bounds of one eligible pair from its GEMM value s (a key
// that is not finite, or a bound that is not, keeps the pair unconditionally).
// With v the exact values and b their FP16 copies (per column eq, er = ||v - b||
// and bq, br = ||b||), Cauchy-Schwarz gives
//   |sum v_q v_r - sum b_q b_r| <= eq ||v_r|| + bq er,
// ||v_r|| = 1 for unit columns and sqrt(Nr) otherwise; the FP32 accumulation
// of at most n = min(nnz_q, nnz_r) nonzero products is allowed
// (n + 64) 2^-21 sum |b_q b_r| <= (n + 64) 2^-21 bq br.
// Binary: s estimates the matched-row count c (0 / 1 factors are exact in
// FP16); with the accumulation allowance c lies in [c_lo, c_hi] and the
// Jaccard key c / (nq + nc - c) increases with c.
__device__ __forceinline__ void tc_bounds(int method, float s, int32_t nq_, float Nq, int32_t nc_, float Nc,
                                            float eq, float bq, float er, float br, float& lo, float& hi) {
  const float nmin = (float)min(nq_, nc_);
  const float acc = (nmin + 64.f) * ACC_ULP;
  float key, err;
  if (method == BINARY) {
    const float e = acc * 1.01f * fabsf(s) + 1e-6f;
    const float clo = fmaxf(0.f, s - e), chi = fminf(nmin, s + e);
    const float N = (float)nq_ + (float)nc_;
    lo = (N - clo > 0.f) ? clo / (N - clo) : 1.f;
    hi = (N - chi > 0.f) ? chi / (N - chi) : 1.f;
    lo = lo * (1.f - 4.f * U32);
    hi = hi * (1.f + 4.f * U32) + 1e-30f;
    if (!(fabsf(s) <= FLT_MAX)) { lo = -INFINITY; hi = INFINITY; }
    return;
  }
  if (method == COSINE) {
    key = s;
    err = (1.000001f * eq + bq * er + acc * bq * br) * 1.01f + 1e-12f;
  } else {
    const float T = Nq + Nc;
    key = 2.f * s - T;
    err = 2.f * (sqrtf(Nc) * 1.000001f * eq + bq * er + acc * bq * br) * 1.01f + 9.5367431640625e-7f * T + 1e-30f;
  }
  if (!(fabsf(key) <= FLT_MAX) || !(err <= FLT_MAX)) { lo = -INFINITY; hi = INFINITY; return; }
  lo = key - err;
  hi = key + err;
}

// cut = T - margin(T): the FP32 allowance under the k-th pessimistic key T
// (increasing in T, so a running cut over a subset never exceeds the final one)
__device__ __forceinline__ float tc_cut(float T) {
  return T - ((T == -INFINITY || T == INFINITY) ? 0.f : fabsf(T) * (8.f * U32) + 1e-30f);
}

}  // namespace tcb
}  // namespace sdg
