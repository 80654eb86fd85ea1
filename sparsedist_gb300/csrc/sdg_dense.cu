// sdg_dense.cu -- kNN over dense embedding columns (FP32 embeddings, d x n).
//
// Columns are dense (d values each).  A cosine / euclidean slab between
// dense columns is a true contraction, so the screen runs on the tensor
// cores: the fused tcgen05 kernel of sdg_dense_tc.cu (modes 0 and 3), or
// BF16 GEMM tiles with FP32 accumulation (cuBLAS GemmEx, mode 2) that write
// the screen slab S[q][r] = <col q, col r> for the segmented selection here.
// Either keeps every reference whose optimistic bound reaches the k-th
// pessimistic bound (the BF16 rounding bound below); an FP32 cut with a
// rigorous bound (k_dense_refine_*) leaves about k of them per query, and
// those are valued in exact FP64 with the reference's arithmetic (unit_csc
// normalisation and a sequential dot for cosine, a sequential sum of squared
// differences for euclidean), so the returned idx and distances are those of
// sparseKNN on the same data.
//
// The plain path (mode 1) is the FP32 baseline: an FP32 SGEMM on the CUDA
// cores and the top-k taken directly on the FP32 values (no re-rank).
//
// BF16 bound: every input is rounded to BF16 (relative error <= 2^-9), so a
// product has relative error <= 2^-8 + 2^-18, and the FP32 accumulation of d
// products adds at most d * 2^-22 relative (a conservative allowance for the
// tensor cores' accumulation); with S|x_i y_i| <= |x| |y|:
//   cosine    (unit vectors):  |S - S_exact| <= 0.0040 + d * 2^-22
//   euclidean (2S - Nq - Nr):  2 (0.0040 + d * 2^-22) sqrt(Nq Nr) + 2^-20 (Nq + Nr)
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/sdgpu.h"
#include "sdg_dense.h"

namespace sdg {
namespace {

constexpr int DSEL_WARPS = 8;

inline unsigned blocks_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

// One warp per column (coalesced rows): the FP64 copy, the sum of squares
// (FP64, any order: it only feeds the screens' bounds and the plain mode),
// the empty flag and the finiteness check.
__global__ void k_dense_prep(int32_t d, int64_t n, const float* x32, double* x64, float* norm2,
                             uint8_t* empty, int* err) {
  const int lane = threadIdx.x & 31;
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  double s = 0.0;
  bool nz = false, bad = false;
  for (int32_t r = lane; r < d; r += 32) {
    const float v = x32[j * d + r];
    bad |= !isfinite(v);
    nz |= (v != 0.f);
    const double dv = (double)v;
    x64[j * d + r] = dv;
    s += dv * dv;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  nz = __any_sync(0xffffffffu, nz);
  bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) {
    norm2[j] = (float)s;
    empty[j] = nz ? 0 : 1;
    if (bad) atomicOr(err, 1);
  }
}

__global__ void k_dense_cast(int64_t total, const double* u64, const float* x32, float* u32,
                             __nv_bfloat16* ub, __nv_bfloat16* xb) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < total;
       a += (int64_t)gridDim.x * blockDim.x) {
    const float u = (float)u64[a];
    u32[a] = u;
    ub[a] = __float2bfloat16_rn(u);
    xb[a] = __float2bfloat16_rn(x32[a]);
  }
}

// Per column: ||v - bf16(v)|| and ||bf16(v)|| of the unit column and of the
// column, in FP64 from the copies the screen multiplies (one warp per column;
// the FP64 sums' rounding, under d 2^-53 relative, is inside the 1e-12
// allowance), rounded up to FP32.
__global__ void k_dense_errnorm(int32_t d, int64_t n, const double* u64, const double* x64,
                                const __nv_bfloat16* ub, const __nv_bfloat16* xb, float* ue, float* un, float* xe,
                                float* xn) {
  const int lane = threadIdx.x & 31;
  const int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (j >= n) return;
  double eu = 0.0, nu = 0.0, ex = 0.0, nx = 0.0;
  for (int32_t r = lane; r < d; r += 32) {
    const int64_t a = j * d + r;
    const double bu = (double)__bfloat162float(ub[a]), bx = (double)__bfloat162float(xb[a]);
    const double du = u64[a] - bu, dx = x64[a] - bx;
    eu += du * du; nu += bu * bu; ex += dx * dx; nx += bx * bx;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    eu += __shfl_xor_sync(0xffffffffu, eu, o);
    nu += __shfl_xor_sync(0xffffffffu, nu, o);
    ex += __shfl_xor_sync(0xffffffffu, ex, o);
    nx += __shfl_xor_sync(0xffffffffu, nx, o);
  }
  if (lane == 0) {
    ue[j] = __double2float_ru(sqrt(eu) * (1.0 + 1e-12));
    un[j] = __double2float_ru(sqrt(nu) * (1.0 + 1e-12));
    xe[j] = __double2float_ru(sqrt(ex) * (1.0 + 1e-12));
    xn[j] = __double2float_ru(sqrt(nx) * (1.0 + 1e-12));
  }
}

// A query's scan over the n references is split into segments of DSEG
// references, one warp per (query, segment), so that the slab is streamed at
// full bandwidth: (1) each warp keeps the top k of its segment's pessimistic
// keys (key - err); (2) one warp per query merges the segments' lists into
// the exact k-th largest pessimistic key T (the top k of a union is the top k
// of the parts' top k); (3) each warp keeps every reference of its segment
// whose optimistic key reaches T - margin, appended to the query's candidate
// list with one atomic per 32 x 4 references.
constexpr int DSEG = 32768;

struct DenseSelArgs {
  int method, k, mode;           // mode 0: BF16 bound, 1: plain FP32 (no bound)
  const float* S;                // S[ql * ldS + r]
  int64_t ldS;                   // multiple of 4 (float4 rows)
  int64_t n, q0, nq;
  int32_t d;
  int self;                      // queries are columns of the reference: skip r == q
  const float* norm2;            // padded to ldS entries
  const uint8_t* empty;          // padded to ldS entries (padding = 1)
  const float* qnorm2;           // query sums of squares
  const uint8_t* qempty;         // degenerate queries
  int nseg;
  float* segtop;                 // [ql][seg][k], best first, -inf padded
  float* cut;                    // [ql]: T - margin
  int cap;
  int32_t* cand;
  int32_t* count;
  int32_t* overflow;
};

// Warp-cooperative insertion of the lanes flagged in m (value v on each lane)
// into lst[0..n), kept sorted descending and at most K long.
__device__ __forceinline__ void warp_insert_desc(float* lst, int K, int& n, unsigned m, float v, int lane) {
  while (m) {
    const int src = __ffs(m) - 1;
    m &= m - 1;
    const float x = __shfl_sync(0xffffffffu, v, src);
    if (n == K && !(x > lst[K - 1])) continue;
    int a = 0, b = n;
    while (a < b) { const int mid = (a + b) >> 1; if (lst[mid] >= x) a = mid + 1; else b = mid; }
    const int last = (n < K) ? n : K - 1;
    if (last > a) {
      for (int c = (last - 1) >> 5; c >= (a >> 5); --c) {
        const int e = c * 32 + lane;
        const bool mv = (e >= a && e < last);
        float t = 0.f;
        if (mv) t = lst[e];
        __syncwarp();
        if (mv) lst[e + 1] = t;
        __syncwarp();
      }
    }
    if (lane == 0) lst[a] = x;
    __syncwarp();
    if (n < K) ++n;
  }
}

// The four references r0..r0+3 of one lane: their pessimistic (lo) and
// optimistic (hi) keys, -inf where the reference is not a candidate.
__device__ __forceinline__ void dense_keys4(const DenseSelArgs& A, int64_t q, float Nq, const float* Srow,
                                            int64_t r0, float lo[4], float hi[4]) {
  const float4 s4 = *reinterpret_cast<const float4*>(Srow + r0);
  const uchar4 e4 = *reinterpret_cast<const uchar4*>(A.empty + r0);
  float4 n4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (A.method != COSINE) n4 = *reinterpret_cast<const float4*>(A.norm2 + r0);
  const float sv[4] = {s4.x, s4.y, s4.z, s4.w};
  const float nv[4] = {n4.x, n4.y, n4.z, n4.w};
  const uint8_t ev[4] = {e4.x, e4.y, e4.z, e4.w};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int64_t r = r0 + j;
    lo[j] = hi[j] = -INFINITY;
    if (r < A.n && !(A.self && r == q) && !ev[j]) {
      float key, err;
      dense_key(A.method, A.mode, A.d, sv[j], Nq, nv[j], key, err);
      lo[j] = key - err;
      hi[j] = key + err;
    }
  }
}

// (1) top k of each (query, segment)'s pessimistic keys
__global__ void k_dense_segtop(DenseSelArgs A) {
  extern __shared__ float lists[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = (int64_t)blockIdx.x * DSEL_WARPS + warp;
  const int seg = blockIdx.y;
  if (ql >= A.nq) return;
  const int64_t q = A.q0 + ql;
  const int K = A.k;
  float* lst = lists + warp * K;
  int n = 0;
  if (!A.qempty[q]) {
    const float Nq = A.qnorm2[q];
    const float* Srow = A.S + ql * A.ldS;
    const int64_t r_end = min(A.n, (int64_t)(seg + 1) * DSEG);
    float thr = -INFINITY;                       // lst[K - 1] once the list is full
    for (int64_t p0 = (int64_t)seg * DSEG; p0 < r_end; p0 += 128) {
      float lo[4], hi[4];
      dense_keys4(A, q, Nq, Srow, p0 + 4 * lane, lo, hi);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const unsigned m = __ballot_sync(0xffffffffu, lo[j] > -INFINITY && (n < K || lo[j] > thr));
        if (m) {
          warp_insert_desc(lst, K, n, m, lo[j], lane);
          if (n == K) thr = lst[K - 1];
        }
      }
    }
  }
  float* out = A.segtop + (ql * A.nseg + seg) * (int64_t)K;
  for (int t = lane; t < K; t += 32) out[t] = t < n ? lst[t] : -INFINITY;
}

// (2) per query: T = k-th largest pessimistic key over all segments
__global__ void k_dense_thresh(DenseSelArgs A) {
  extern __shared__ float lists[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = (int64_t)blockIdx.x * DSEL_WARPS + warp;
  if (ql >= A.nq) return;
  const int K = A.k;
  float* lst = lists + warp * K;
  const float* in = A.segtop + ql * A.nseg * (int64_t)K;
  const int64_t tot = (int64_t)A.nseg * K;
  int n = 0;
  for (int64_t p0 = 0; p0 < tot; p0 += 32) {
    const float v = p0 + lane < tot ? in[p0 + lane] : -INFINITY;
    const unsigned m = __ballot_sync(0xffffffffu, v > -INFINITY && (n < K || v > lst[K - 1]));
    if (m) warp_insert_desc(lst, K, n, m, v, lane);
  }
  if (lane == 0) {
    A.cut[ql] = dense_cut((n == K) ? lst[K - 1] : -INFINITY);
    A.count[ql] = 0;
  }
}

// (3) keep every reference of the segment whose optimistic key reaches the cut
__global__ void k_dense_keep(DenseSelArgs A) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = (int64_t)blockIdx.x * DSEL_WARPS + warp;
  const int seg = blockIdx.y;
  if (ql >= A.nq) return;
  const int64_t q = A.q0 + ql;
  if (A.qempty[q]) return;
  const float Nq = A.qnorm2[q];
  const float cut = A.cut[ql];
  const float* Srow = A.S + ql * A.ldS;
  int32_t* out = A.cand + ql * (int64_t)A.cap;
  const int64_t r_end = min(A.n, (int64_t)(seg + 1) * DSEG);
  for (int64_t p0 = (int64_t)seg * DSEG; p0 < r_end; p0 += 128) {
    float lo[4], hi[4];
    dense_keys4(A, q, Nq, Srow, p0 + 4 * lane, lo, hi);
    int mine = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) mine += (hi[j] > -INFINITY && hi[j] >= cut);
    int incl = mine;                              // warp inclusive scan of the lanes' counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0) continue;
    int base = 0;
    if (lane == 31) base = atomicAdd(A.count + ql, total);
    base = __shfl_sync(0xffffffffu, base, 31) + incl - mine;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (hi[j] > -INFINITY && hi[j] >= cut) {
        if (base < A.cap) out[base] = (int32_t)(p0 + 4 * lane + j);
        ++base;
      }
    }
  }
}

// overflowing queries drop their list (they are finished by the exact row path)
__global__ void k_dense_overflow(int64_t nq, int cap, int32_t* count, int32_t* overflow) {
  const int64_t ql = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (ql >= nq) return;
  const bool over = count[ql] > cap;
  overflow[ql] = over ? 1 : 0;
  if (over) count[ql] = 0;
}

// Exact FP64 value of each kept pair, in the reference's arithmetic; in the
// plain mode the FP32 value of the slab instead.
// Third cut, on the candidates of the BF16 screens: FP32 inner products of
// the FP32 copies with a rigorous bound on their distance from the FP64 value
// that k_dense_values_flat computes.  A warp values up to 8 candidates of one
// query at a time: each lane accumulates its share of the elements with FMA
// (at most J roundings per product: J = 4 ceil(d / 128) when d is a multiple
// of 4 and lane l takes the float4s l, l + 32, ...; else J = ceil(d / 32),
// lane l taking elements l, l + 32, ...), and a five-level xor butterfly adds
// the lanes (five more, the same sum on every lane).  With u = 2^-24 and
// g(m) = m u / (1 - m u) (Higham's gamma; g53 the same for u = 2^-53):
//   cosine:    s = fl32(sum u32_q u32_r) of the FP32 copies (|u32 - u| <= u |u|),
//              |s - c| <= [g(J + 5) (1 + u)^2 + 2u + u^2 + g53(d + 1)] Nq Nr,
//              c the FP64 sequential dot, N = ||b|| + ||u - b|| >= ||u|| (the
//              BF16 copy's norm and error norm, both rounded up);
//   euclidean: m = fl32(sum fl32(x_r - x_q)^2) of the FP32 inputs; every term is
//              >= 0, so |m - num| <= (g(J + 7) + g53(d + 2)) / (1 - g(J + 7)) m.
// Key = s (cosine) or -m (euclidean), larger is nearer.  The allowances get a
// factor 1.01 and absolute terms (1e-15 cosine, 1e-36 euclidean) covering FP32
// underflow and the keys that the FP64 distance rounds into a tie (1 - c: one
// ulp of a value <= 2, at most 2^-52; sqrt(num): 2^-51 num relative, inside
// the 1 % slack); lo and hi are formed with directed rounding.  T3 = the k-th
// largest lo among the candidates is at most the k-th best exact key (k
// candidates reach it), so every member of the exact top k, ties included,
// has hi >= dense_cut(T3) and is kept.  A non-finite m keeps its pair.
//
// Candidate counts are very uneven (a query inside a cluster of near
// duplicates has hundreds), so the products run over a flat list of items,
// ceil(count / 8) per query that needs the cut (k_dense_refine_scan: their
// exclusive offsets), dealt round-robin to a persistent grid of warps
// (k_dense_refine_dot); a warp per query then makes the cut from the stored
// values (k_dense_refine_cut).
constexpr int RW = 8;        // warps per block of the cut
constexpr int RG = 8;        // candidates per item of the products

struct RefineArgs {
  int method, k;
  int32_t d;
  int J;                       // FMA roundings per product in a lane (see above)
  const float* rv;             // reference FP32 copies, d x n (u32 cosine, x32 euclidean)
  const float* qv;             // query FP32 copies, column q0 + ql
  const float *rn, *re;        // reference BF16 copy norm / error norm (unit columns)
  const float *qn, *qe;        // query
  int64_t q0, nq;
  int cap;
  int32_t* cand;               // [nq][cap], compacted in place
  int32_t* count;              // [nq], updated
  float* sv;                   // [nq][cap] scratch: the FP32 values
  int64_t* off;                // [nq + 1] exclusive offsets of the items (0 for queries without the cut)
  int unit;                    // k_dense_refine_scan: RG (the cut's items) or 1 (every candidate)
};

inline int refine_lane_terms(int32_t d) { return (d % 4 == 0) ? 4 * ((d + 127) / 128) : (d + 31) / 32; }

__device__ __forceinline__ double gam(int m, double u) { return m * u / (1.0 - m * u); }

__device__ __forceinline__ void refine_bounds(const RefineArgs& A, float s, int32_t r, float Nq, float C, float& lo,
                                              float& hi) {
  if (A.method == COSINE) {
    const float Nr = __fadd_ru(A.rn[r], A.re[r]);
    const float E = __fmaf_ru(C, __fmul_ru(Nq, Nr), 1e-15f);
    lo = __fsub_rd(s, E);
    hi = __fadd_ru(s, E);
  } else if (isfinite(s)) {
    const float E = __fmaf_ru(C, s, 1e-36f);
    lo = __fsub_rd(-s, E);
    hi = __fadd_ru(-s, E);
  } else {
    lo = -INFINITY;
    hi = INFINITY;
  }
}

__device__ __forceinline__ int refine_items(int c, int k, int unit) {
  return unit == 1 ? c : (c > k ? (c + unit - 1) / unit : 0);
}

// One block of 1024 threads: off[ql] = the items of the queries before ql,
// off[nq] = the total (unit RG: ceil(count / RG) items for each query with
// more than k candidates; unit 1: every candidate).
__global__ void k_dense_refine_scan(RefineArgs A) {
  __shared__ int64_t wsum[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t per = (A.nq + blockDim.x - 1) / blockDim.x;
  const int64_t b = tid * per, e = (b + per < A.nq) ? b + per : A.nq;
  int64_t own = 0;
  for (int64_t i = b; i < e; ++i) own += refine_items(A.count[i], A.k, A.unit);
  int64_t incl = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int64_t w = (lane < (int)(blockDim.x >> 5)) ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;                                  // inclusive over warps
  }
  __syncthreads();
  int64_t run = incl - own + (warp ? wsum[warp - 1] : 0);
  for (int64_t i = b; i < e; ++i) {
    A.off[i] = run;
    run += refine_items(A.count[i], A.k, A.unit);
  }
  if (tid == (int)blockDim.x - 1) A.off[A.nq] = run;
}

__device__ __forceinline__ void refine_fma(bool cosine, float a, float b, float& acc) {
  if (cosine) {
    acc = __fmaf_rn(a, b, acc);
  } else {
    const float df = __fsub_rn(a, b);
    acc = __fmaf_rn(df, df, acc);
  }
}

__global__ void __launch_bounds__(128) k_dense_refine_dot(RefineArgs A) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t items = A.off[A.nq];
  const int32_t d = A.d;
  const bool cosine = (A.method == COSINE);
  const bool vec = (d % 4 == 0);
  for (int64_t it = w; it < items; it += warps) {
    int64_t lo = 0, hi = A.nq;                       // off[lo] <= it < off[hi]
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (__ldg(A.off + mid) <= it) lo = mid;
      else hi = mid;
    }
    const int64_t ql = lo;
    const int t0 = (int)(it - __ldg(A.off + ql)) * RG;
    const int n = min(RG, A.count[ql] - t0);
    const int32_t* cp = A.cand + ql * A.cap + t0;
    const int32_t mine = lane < n ? cp[lane] : 0;
    const float* qv = A.qv + (A.q0 + ql) * d;
    const float* row[RG];
#pragma unroll
    for (int j = 0; j < RG; ++j) row[j] = A.rv + (int64_t)__shfl_sync(0xffffffffu, mine, j < n ? j : n - 1) * d;
    float acc[RG];
#pragma unroll
    for (int j = 0; j < RG; ++j) acc[j] = 0.f;
    if (vec) {
      const int32_t d4 = d >> 2;
      for (int32_t f0 = 0; f0 < d4; f0 += 64) {
        float4 qa[2], ra[2][RG];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int32_t f = f0 + lane + 32 * h;
          if (f < d4) {
            qa[h] = __ldg(reinterpret_cast<const float4*>(qv) + f);
#pragma unroll
            for (int j = 0; j < RG; ++j) ra[h][j] = __ldg(reinterpret_cast<const float4*>(row[j]) + f);
          }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (f0 + lane + 32 * h < d4) {
#pragma unroll
            for (int j = 0; j < RG; ++j) {
              refine_fma(cosine, ra[h][j].x, qa[h].x, acc[j]);
              refine_fma(cosine, ra[h][j].y, qa[h].y, acc[j]);
              refine_fma(cosine, ra[h][j].z, qa[h].z, acc[j]);
              refine_fma(cosine, ra[h][j].w, qa[h].w, acc[j]);
            }
          }
        }
      }
    } else {
      for (int32_t e = lane; e < d; e += 32) {
        const float b = __ldg(qv + e);
#pragma unroll
        for (int j = 0; j < RG; ++j) refine_fma(cosine, __ldg(row[j] + e), b, acc[j]);
      }
    }
    float out = 0.f;
#pragma unroll
    for (int j = 0; j < RG; ++j) {
#pragma unroll
      for (int o = 16; o; o >>= 1) acc[j] = __fadd_rn(acc[j], __shfl_xor_sync(0xffffffffu, acc[j], o));
      if (lane == j) out = acc[j];
    }
    if (lane < n) A.sv[ql * A.cap + t0 + lane] = out;
  }
}

__global__ void k_dense_refine_cut(RefineArgs A) {
  extern __shared__ float rl[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ql = blockIdx.x * (int64_t)RW + warp;
  if (ql >= A.nq) return;
  const int c = A.count[ql], K = A.k;
  if (c <= K) return;
  const int64_t q = A.q0 + ql;
  const int32_t d = A.d;
  int32_t* cand = A.cand + ql * (int64_t)A.cap;
  const float* sv = A.sv + ql * (int64_t)A.cap;
  float* lst = rl + warp * K;
  const int J = A.J;
  const double u = 5.9604644775390625e-8;             // 2^-24
  const double u53 = 1.1102230246251565e-16;          // 2^-53
  double Cd;
  if (A.method == COSINE) Cd = gam(J + 5, u) * (1.0 + u) * (1.0 + u) + 2.0 * u + u * u + gam(d + 1, u53);
  else Cd = (gam(J + 7, u) + gam(d + 2, u53)) / (1.0 - gam(J + 7, u));
  const float C = __double2float_ru(Cd * 1.01 * (1.0 + 1e-12));
  const float Nq = (A.method == COSINE) ? __fadd_ru(A.qn[q], A.qe[q]) : 0.f;
  int n = 0;
  for (int t0 = 0; t0 < c; t0 += 32) {
    const int t = t0 + lane;
    float lo = -INFINITY, hi;
    if (t < c) refine_bounds(A, sv[t], cand[t], Nq, C, lo, hi);
    const unsigned m = __ballot_sync(0xffffffffu, t < c && (n < K || lo > lst[K - 1]));
    if (m) warp_insert_desc(lst, K, n, m, lo, lane);
  }
  const float cut = dense_cut((n == K) ? lst[K - 1] : -INFINITY);
  int kept = 0;
  for (int t0 = 0; t0 < c; t0 += 32) {
    const int t = t0 + lane;
    bool keep = false;
    int32_t r = 0;
    if (t < c) {
      r = cand[t];
      float lo, hi;
      refine_bounds(A, sv[t], r, Nq, C, lo, hi);
      keep = hi >= cut;
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);    // every lane has read slot t first
    if (keep) cand[kept + __popc(m & ((1u << lane) - 1u))] = r;
    kept += __popc(m);
    __syncwarp();
  }
  if (lane == 0) A.count[ql] = kept;
}

// Exact values of the candidates after the FP32 cut, over the flat list of
// every candidate (k_dense_refine_scan with unit 1): lane l of a warp values
// candidate base + l with the reference's sequential FP64 loop, so every lane
// of the FP64 pipe works whatever the queries' counts.  The rows are read 32
// elements at a time, coalesced, through a shared-memory tile.
constexpr int VW = 4;        // warps per block

__global__ void __launch_bounds__(VW * 32) k_dense_values_flat(int method, int32_t d, const double* rv,
                                                               const double* qv, const int32_t* cand,
                                                               int cap, int64_t q0, int64_t nq,
                                                               const int64_t* off, double* out) {
  __shared__ double tile[VW][32][33];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * VW;
  const int64_t total = off[nq];
  const bool cosine = (method == COSINE);
  for (int64_t base = ((int64_t)blockIdx.x * VW + warp) * 32; base < total; base += warps * 32) {
    const int64_t f = base + lane;
    const int nv = (int)((total - base) < 32 ? (total - base) : 32);
    int64_t ql = 0, slot = 0;
    int32_t r = 0;
    if (lane < nv) {
      int64_t lo = 0, hi = nq;                       // off[lo] <= f < off[hi]
      while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= f) lo = mid;
        else hi = mid;
      }
      ql = lo;
      slot = ql * cap + (f - __ldg(off + ql));
      r = cand[slot];
    }
    const double* b = qv + (q0 + ql) * d;
    double acc = 0.0;
    for (int32_t k0 = 0; k0 < d; k0 += 32) {
      const int kn = (d - k0) < 32 ? (d - k0) : 32;
#pragma unroll 8
      for (int j = 0; j < nv; ++j) {
        const int32_t rj = __shfl_sync(0xffffffffu, r, j);
        if (lane < kn) tile[warp][j][lane] = rv[(int64_t)rj * d + k0 + lane];
      }
      __syncwarp();
      if (lane < nv) {
        // unit_dot (src/sparseDist.cpp:287-331) / fastEuclidean2's pair loop
        // (src/sparseDist.cpp:855-871), reference column first, ascending rows
        for (int t = 0; t < kn; ++t) {
          const double a = tile[warp][lane][t], bv = b[k0 + t];
          if (cosine) {
            acc = __dadd_rn(acc, __dmul_rn(a, bv));
          } else {
            const double diff = __dsub_rn(a, bv);
            acc = __dadd_rn(acc, __dmul_rn(diff, diff));
          }
        }
      }
      __syncwarp();
    }
    if (lane < nv) {
      if (cosine) {
        double c = acc;
        if (!(c == c)) c = 0.0;
        else if (c > 1.0) c = 1.0;
        else if (c < -1.0) c = -1.0;
        out[slot] = __dsub_rn(1.0, c);
      } else {
        out[slot] = sqrt(acc);
      }
    }
  }
}

// The plain mode's values (no exact re-rank): the FP32 slab values as
// distances, one warp per query.
__global__ void k_dense_values_plain(int method, const float* S, int64_t ldS, const float* norm2,
                                     const float* qnorm2, const int32_t* cand, const int32_t* count, int cap,
                                     int64_t q0, int64_t nq, double* out) {
  const int64_t ql = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
  if (ql >= nq) return;
  const int lane = threadIdx.x & 31;
  const int c = count[ql];
  const int64_t q = q0 + ql;
  for (int t = lane; t < c; t += 32) {
    const int64_t s = ql * cap + t, r = cand[s];
    const float sv = S[ql * ldS + r];
    out[s] = (method == COSINE) ? (double)(1.f - fminf(1.f, fmaxf(-1.f, sv)))
                                : (double)sqrtf(fmaxf(0.f, qnorm2[q] + norm2[r] - 2.f * sv));
  }
}

// exact FP64 values of one query against every reference (overflow fallback)
__global__ void k_dense_exact_row(int method, int32_t d, const double* x64, const double* u64,
                                  const double* qx64, const double* qu64, const uint8_t* empty, int64_t n,
                                  int64_t q, int self, double* out) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  if ((self && r == q) || empty[r]) { out[r] = na_real(); return; }
  double acc = 0.0;
  if (method == COSINE) {
    for (int32_t k = 0; k < d; ++k) acc = __dadd_rn(acc, __dmul_rn(u64[r * d + k], qu64[q * d + k]));
    double c = acc;
    if (!(c == c)) c = 0.0; else if (c > 1.0) c = 1.0; else if (c < -1.0) c = -1.0;
    out[r] = __dsub_rn(1.0, c);
  } else {
    for (int32_t k = 0; k < d; ++k) {
      const double diff = __dsub_rn(x64[r * d + k], qx64[q * d + k]);
      acc = __dadd_rn(acc, __dmul_rn(diff, diff));
    }
    out[r] = sqrt(acc);
  }
}

int fail_with(int code, const char* msg) { set_error(msg); return code; }
int cuda_fail(cudaError_t e) {
  set_error(cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? SDG_E_NOMEM : SDG_E_CUDA;
}
#define DK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return cuda_fail(e_); } while (0)
#define DB(x) do { cublasStatus_t b_ = (x); if (b_ != CUBLAS_STATUS_SUCCESS) return fail_with(SDG_E_CUDA, "cuBLAS call failed"); } while (0)

}  // namespace
}  // namespace sdg

using namespace sdg;

namespace {

// Builds the resident form of d x n FP32 columns X (host or device memory):
// FP64 values and unit columns (unit_csc on each dense column), their FP32
// and BF16 copies (rows padded to a multiple of 64 with zeros), sums of
// squares and degenerate flags.  `async` takes the buffers from the stream's
// pool (a per-request query matrix) instead of cudaMalloc (a resident
// reference); `blas` creates the cuBLAS handle of the slab and plain modes.
// keep_err (stream-ordered builds only): instead of reading the finiteness
// flag back (a stream synchronisation), hand the device flag to the caller,
// who reads it with its own results and frees it; n_empty is then not counted
// (a query block needs only the device flags).
int dense_build(sdg_ctx* ctx, const float* X, int32_t d, int64_t n, bool async, bool blas, sdg_dense** out,
                int** keep_err = nullptr) {
  cudaStream_t s = ctx_stream(ctx);
  DK(cudaSetDevice(ctx_device(ctx)));
  auto D = new sdg_dense();
  D->device = ctx_device(ctx);
  D->d = d;
  D->n = n;
  D->async = async;
  D->stream = s;
  auto alloc = [&](auto** p, size_t bytes) {
    return async ? cudaMallocAsync((void**)p, bytes, s) : cudaMalloc((void**)p, bytes);
  };
  const size_t tot = (size_t)d * (size_t)n;
  int* err = nullptr;
  const int64_t npad = (n + 127) / 128 * 128;       // float4 / uchar4 reads past n stay in bounds
  D->npad = npad;
  D->dpad = (d + 63) / 64 * 64;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  chk(alloc(&D->x64, tot * 8)); chk(alloc(&D->u64, tot * 8));
  chk(alloc(&D->x32, tot * 4)); chk(alloc(&D->u32, tot * 4));
  chk(alloc(&D->xb, tot * 2)); chk(alloc(&D->ub, tot * 2));
  chk(alloc(&D->norm2, npad * 4)); chk(alloc(&D->scale, n * 8));
  chk(alloc(&D->empty, npad));
  chk(alloc(&D->ue, npad * 4)); chk(alloc(&D->un, npad * 4));
  chk(alloc(&D->xe, npad * 4)); chk(alloc(&D->xn, npad * 4));
  chk(alloc(&err, sizeof(int)));
  if (D->dpad != d) {
    const size_t ptot = (size_t)D->dpad * (size_t)n;
    chk(alloc(&D->ubp, ptot * 2)); chk(alloc(&D->xbp, ptot * 2));
  }
  if (e != cudaSuccess) { sdg_dense_free(D); return cuda_fail(e); }
  chk(cudaMemsetAsync(D->norm2, 0, npad * 4, s));
  chk(cudaMemsetAsync(D->empty, 1, npad, s));
  for (float* p : {D->ue, D->un, D->xe, D->xn}) chk(cudaMemsetAsync(p, 0, npad * 4, s));
  chk(cudaMemsetAsync(err, 0, sizeof(int), s));
  chk(cudaMemcpyAsync(D->x32, X, tot * 4, cudaMemcpyDefault, s));
  if (e == cudaSuccess) {
    k_dense_prep<<<blocks_for(n * 32, 256), 256, 0, s>>>(d, n, D->x32, D->x64, D->norm2, D->empty, err);
    launch_unit_dense(d, n, D->x64, D->u64, D->scale, err, s);
    k_dense_cast<<<152 * 16, 256, 0, s>>>((int64_t)tot, D->u64, D->x32, D->u32, D->ub, D->xb);
    k_dense_errnorm<<<blocks_for(n * 32, 256), 256, 0, s>>>(d, n, D->u64, D->x64, D->ub, D->xb, D->ue, D->un,
                                                            D->xe, D->xn);
  }
  if (D->dpad == d) {
    D->ubp = D->ub;
    D->xbp = D->xb;
  } else if (e == cudaSuccess) {                    // rows d..dpad-1 of the padded copies are zero
    chk(cudaMemset2DAsync(D->ubp, (size_t)D->dpad * 2, 0, (size_t)D->dpad * 2, (size_t)n, s));
    chk(cudaMemset2DAsync(D->xbp, (size_t)D->dpad * 2, 0, (size_t)D->dpad * 2, (size_t)n, s));
    chk(cudaMemcpy2DAsync(D->ubp, (size_t)D->dpad * 2, D->ub, (size_t)d * 2, (size_t)d * 2, (size_t)n,
                          cudaMemcpyDeviceToDevice, s));
    chk(cudaMemcpy2DAsync(D->xbp, (size_t)D->dpad * 2, D->xb, (size_t)d * 2, (size_t)d * 2, (size_t)n,
                          cudaMemcpyDeviceToDevice, s));
  }
  chk(cudaGetLastError());
  if (keep_err && async) {
    if (e != cudaSuccess) { cudaFreeAsync(err, s); sdg_dense_free(D); return cuda_fail(e); }
    *keep_err = err;
    *out = D;
    return SDG_OK;
  }
  int herr = 0;
  std::vector<uint8_t> he((size_t)n);
  chk(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  chk(cudaMemcpyAsync(he.data(), D->empty, (size_t)n, cudaMemcpyDeviceToHost, s));
  if (async) chk(cudaFreeAsync(err, s));
  chk(cudaStreamSynchronize(s));
  if (!async) cudaFree(err);
  if (e != cudaSuccess) { sdg_dense_free(D); return cuda_fail(e); }
  for (uint8_t v : he) D->n_empty += v;
  if (herr) { sdg_dense_free(D); return fail_with(SDG_E_NONFINITE, "Cosine requires finite input (found NA, NaN or Inf)."); }
  if (blas && cublasCreate(&D->blas) != CUBLAS_STATUS_SUCCESS) {
    sdg_dense_free(D);
    return fail_with(SDG_E_CUDA, "cublasCreate failed");
  }
  *out = D;
  return SDG_OK;
}

// Rows q0 .. q0+nq-1 (query columns of Q) of sparseKNN(Q, R, k, method) with
// drop_degenerate = TRUE: the self-search with include_self = FALSE when self
// (Q is R), else the two-matrix search.  See sdg_dense_knn_block for modes.
// build_err: the query build's device finiteness flag (dense_build's
// keep_err), read back with the first chunk's counts; NULL when the queries
// were checked already.
int dense_search(sdg_ctx* ctx, const sdg_dense* Q, int64_t q0, int64_t nq, const sdg_dense* D, bool self,
                 int method, int k, int mode, int32_t* idx, double* dist_out, int device_out, int* k_eff,
                 int* flags, const int* build_err = nullptr) {
  if (!ctx || !Q || !D || !idx || !dist_out || !k_eff || !flags) return fail_with(SDG_E_ARG, "NULL argument");
  if (method != COSINE && method != EUCLIDEAN) return fail_with(SDG_E_UNSUPPORTED, "dense kNN supports cosine and euclidean");
  if (mode < 0 || mode > 3)
    return fail_with(SDG_E_ARG,
                     "mode must be 0 (BF16 screen), 1 (plain FP32), 2 (BF16 slab screen) or 3 (BF16 screen on "
                     "CTA pairs)");
  if (k < 1) return fail_with(SDG_E_ARG, "'k' must be a positive integer no larger than .Machine$integer.max.");
  if (q0 < 0 || nq < 1 || q0 + nq > Q->n) return fail_with(SDG_E_ARG, "invalid query column range");
  if (Q->d != D->d) return fail_with(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
  if ((mode == 1 || mode == 2) && !D->blas)
    return fail_with(SDG_E_ARG, "modes 1 and 2 need the reference's cuBLAS handle");
  DK(cudaSetDevice(D->device));
  cudaStream_t s = ctx_stream(ctx);
  *flags = 0;
  const int64_t avail = D->n - D->n_empty - (self ? 1 : 0);   // include_self = FALSE
  if (avail < 1) return fail_with(SDG_E_NOCAND, "No candidate neighbours available.");
  if (k > avail) { k = (int)avail; *flags |= SDG_WARN_CLAMP_FWD; }
  *k_eff = k;
  const int64_t n = D->n;
  if (k > kMaxK) {
    // more neighbours than the screens' lists hold: every query is valued
    // exactly against every reference and selected with lists in device
    // scratch (the same kernels as the screens' overflow path)
    int32_t* o_idx = idx;
    double *o_val = dist_out, *row = nullptr;
    if (!device_out) {
      DK(cudaMallocAsync(&o_idx, sizeof(int32_t) * (size_t)(nq * k), s));
      DK(cudaMallocAsync(&o_val, sizeof(double) * (size_t)(nq * k), s));
    }
    DK(cudaMallocAsync(&row, sizeof(double) * (size_t)n, s));
    ctx_stats_reset(ctx);
    for (int64_t q = q0; q < q0 + nq; ++q) {
      k_dense_exact_row<<<blocks_for(n, 256), 256, 0, s>>>(method, D->d, D->x64, D->u64, Q->x64, Q->u64,
                                                            D->empty, n, q, self ? 1 : 0, row);
      SelectArgs sa;
      sa.vals = row; sa.seg_stride = 0; sa.elem_stride = 1; sa.len = n; sa.nseg = 1;
      sa.seg_blank = Q->empty + q0;
      sa.out_idx = o_idx; sa.out_val = o_val; sa.out_ld = nq; sa.out_row0 = q - q0;
      sa.k = k; sa.decreasing = 0;
      launch_select(sa, s);
    }
    DK(cudaGetLastError());
    if (!device_out) {
      DK(cudaMemcpyAsync(idx, o_idx, sizeof(int32_t) * (size_t)(nq * k), cudaMemcpyDeviceToHost, s));
      DK(cudaMemcpyAsync(dist_out, o_val, sizeof(double) * (size_t)(nq * k), cudaMemcpyDeviceToHost, s));
      DK(cudaFreeAsync(o_idx, s));
      DK(cudaFreeAsync(o_val, s));
    }
    DK(cudaFreeAsync(row, s));
    int h_build = 0;
    if (build_err) DK(cudaMemcpyAsync(&h_build, build_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    DK(cudaStreamSynchronize(s));
    if (h_build) return fail_with(SDG_E_NONFINITE, "Cosine requires finite input (found NA, NaN or Inf).");
    ctx_stats_add(ctx, 1, n * nq);
    ctx_stats_add(ctx, 3, 2 * nq);
    return SDG_OK;
  }
  const int cap = std::max(512, std::min(16384, 64 * k + 256));
  // modes 0 and 3 run the fused tensor-core screen where it applies (no slab
  // in HBM; mode 0 one CTA per query group, mode 3 on CTA pairs), else the
  // BF16 slab screen of mode 2; smode is the bound in force
  const bool fused = (mode == 0 || mode == 3) && tc_screen_supported(D, method, k);
  const int smode = (mode == 1) ? 1 : 0;
  const int64_t ldS = (n + 127) / 128 * 128;
  const int nseg = (int)((n + DSEG - 1) / DSEG);
  const int64_t chunk = fused ? std::min<int64_t>(nq, 65536)
                              : std::max<int64_t>(1, std::min<int64_t>(nq, ((int64_t)8 << 30) / (4 * ldS)));
  float* S = nullptr;
  float *segtop = nullptr, *cut = nullptr;
  int32_t *cand = nullptr, *count = nullptr, *over = nullptr, *o_idx = idx;
  int64_t* off = nullptr;
  int* tc_status = nullptr;                            // the fused screen's wait status (0 = ok)
  double *vals = nullptr, *o_val = dist_out, *row = nullptr;
  if (!fused) {
    DK(cudaMallocAsync(&S, sizeof(float) * (size_t)(chunk * ldS), s));
    DK(cudaMallocAsync(&segtop, sizeof(float) * (size_t)(chunk * nseg * k), s));
    DK(cudaMallocAsync(&cut, sizeof(float) * (size_t)chunk, s));
  }
  DK(cudaMallocAsync(&cand, sizeof(int32_t) * (size_t)(chunk * cap), s));
  DK(cudaMallocAsync(&count, sizeof(int32_t) * (size_t)chunk, s));
  DK(cudaMallocAsync(&over, sizeof(int32_t) * (size_t)chunk, s));
  DK(cudaMallocAsync(&vals, sizeof(double) * (size_t)(chunk * cap), s));
  if (smode == 0) DK(cudaMallocAsync(&off, sizeof(int64_t) * (size_t)(chunk + 1), s));
  if (fused) {
    DK(cudaMallocAsync(&tc_status, sizeof(int), s));
    DK(cudaMemsetAsync(tc_status, 0, sizeof(int), s));
  }
  if (!device_out) {
    DK(cudaMallocAsync(&o_idx, sizeof(int32_t) * (size_t)(nq * k), s));
    DK(cudaMallocAsync(&o_val, sizeof(double) * (size_t)(nq * k), s));
  }
  // the slab and plain modes share the reference's cuBLAS handle: one caller at a time
  std::unique_lock<std::mutex> blas_lock(const_cast<sdg_dense*>(D)->blas_mu, std::defer_lock);
  if (!fused) {
    blas_lock.lock();
    DB(cublasSetStream(D->blas, s));
  }
  // stream-ordered frees of this call's buffers (the error returns below)
  auto release_all = [&]() {
    for (void* p : {(void*)S, (void*)segtop, (void*)cut, (void*)cand, (void*)count, (void*)over, (void*)vals,
                    (void*)off, (void*)tc_status, (void*)(device_out ? nullptr : o_idx),
                    (void*)(device_out ? nullptr : o_val)})
      if (p) cudaFreeAsync(p, s);
  };
  const float one = 1.f, zero = 0.f;
  std::vector<int64_t> overflow;
  ctx_stats_reset(ctx);
  ctx_stats_add(ctx, 0, n * nq);                      // pairs screened
  for (int64_t c0 = q0; c0 < q0 + nq; c0 += chunk) {
    const int64_t nb = std::min(chunk, q0 + nq - c0);
    if (fused) {
      const int st = tc_screen(ctx, Q, D, self, method, k, c0, nb, cand, count, over, cap, s, mode == 3, tc_status);
      if (st != SDG_OK) { release_all(); return st; }
      ctx_stats_add(ctx, 6, 2 * (int64_t)D->dpad * n * nb);
    } else {
    // S (n x nb, column-major, leading dimension ldS) = R^T Q:
    // S[ql * ldS + r] = <col r, col c0 + ql>
    sdg_time_begin(ctx);
    if (smode == 0) {
      const __nv_bfloat16* M = (method == COSINE) ? D->ub : D->xb;
      const __nv_bfloat16* QM = (method == COSINE) ? Q->ub : Q->xb;
      DB(cublasGemmEx(D->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)n, (int)nb, D->d, &one, M,
                      CUDA_R_16BF, D->d, QM + (size_t)c0 * D->d, CUDA_R_16BF, D->d, &zero, S,
                      CUDA_R_32F, (int)ldS, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT));
    } else {
      const float* M = (method == COSINE) ? D->u32 : D->x32;
      const float* QM = (method == COSINE) ? Q->u32 : Q->x32;
      DB(cublasSgemm(D->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)n, (int)nb, D->d, &one, M, D->d,
                     QM + (size_t)c0 * D->d, D->d, &zero, S, (int)ldS));
    }
    sdg_time_end(ctx);
    ctx_stats_add(ctx, 6, 2 * (int64_t)D->d * n * nb);
    DenseSelArgs A;
    A.method = method; A.k = k; A.mode = smode; A.S = S; A.ldS = ldS; A.n = n; A.q0 = c0; A.nq = nb;
    A.d = D->d; A.self = self ? 1 : 0; A.norm2 = D->norm2; A.empty = D->empty;
    A.qnorm2 = Q->norm2; A.qempty = Q->empty;
    A.nseg = nseg; A.segtop = segtop; A.cut = cut;
    A.cap = cap; A.cand = cand; A.count = count; A.overflow = over;
    const size_t smem = sizeof(float) * (size_t)DSEL_WARPS * k;     // <= 32 KB (k <= kMaxK here)
    const dim3 grid(blocks_for(nb, DSEL_WARPS), (unsigned)nseg);
    k_dense_segtop<<<grid, DSEL_WARPS * 32, smem, s>>>(A);
    k_dense_thresh<<<blocks_for(nb, DSEL_WARPS), DSEL_WARPS * 32, smem, s>>>(A);
    k_dense_keep<<<grid, DSEL_WARPS * 32, 0, s>>>(A);
    k_dense_overflow<<<blocks_for(nb, 256), 256, 0, s>>>(nb, cap, count, over);
    }
    if (smode == 0) {
      RefineArgs R;
      R.method = method; R.k = k; R.d = D->d; R.J = refine_lane_terms(D->d);
      R.rv = (method == COSINE) ? D->u32 : D->x32;
      R.qv = (method == COSINE) ? Q->u32 : Q->x32;
      R.rn = D->un; R.re = D->ue; R.qn = Q->un; R.qe = Q->ue;
      R.q0 = c0; R.nq = nb; R.cap = cap; R.cand = cand; R.count = count;
      R.sv = reinterpret_cast<float*>(vals);          // free until the exact values are written
      R.off = off;
      R.unit = RG;
      k_dense_refine_scan<<<1, 1024, 0, s>>>(R);
      // persistent grids: every block resident at once on this device (asked
      // per call: a host-side query, no state shared between threads)
      int sms = 0, per_sm = 0;
      DK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device));
      DK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dense_refine_dot, 128, 0));
      k_dense_refine_dot<<<std::max(1, per_sm * sms), 128, 0, s>>>(R);
      const size_t rsm = sizeof(float) * (size_t)RW * k;   // <= 32 KB (k <= kMaxK here)
      k_dense_refine_cut<<<blocks_for(nb, RW), RW * 32, rsm, s>>>(R);
      R.unit = 1;
      k_dense_refine_scan<<<1, 1024, 0, s>>>(R);
      DK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dense_values_flat, VW * 32, 0));
      const bool cos = (method == COSINE);
      k_dense_values_flat<<<std::max(1, per_sm * sms), VW * 32, 0, s>>>(
          method, D->d, cos ? D->u64 : D->x64, cos ? Q->u64 : Q->x64, cand, cap, c0, nb, off, vals);
    } else {
      k_dense_values_plain<<<blocks_for(nb, 8), 256, 0, s>>>(method, S, ldS, D->norm2, Q->norm2, cand, count, cap,
                                                             c0, nb, vals);
    }
    SelectArgs sa;
    sa.vals = vals; sa.seg_stride = cap; sa.elem_stride = 1; sa.nseg = nb;
    sa.cand = cand; sa.cand_count = count; sa.cand_ld = cap;
    sa.seg_blank = Q->empty + q0;          // rows are relative to q0
    sa.out_idx = o_idx; sa.out_val = o_val; sa.out_ld = nq; sa.out_row0 = c0 - q0;
    sa.k = k; sa.decreasing = 0;
    launch_select(sa, s);
    DK(cudaGetLastError());
    std::vector<int32_t> h_over((size_t)nb), h_count((size_t)nb);
    int h_status = 0, h_build = 0;
    DK(cudaMemcpyAsync(h_over.data(), over, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, s));
    DK(cudaMemcpyAsync(h_count.data(), count, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, s));
    if (tc_status) DK(cudaMemcpyAsync(&h_status, tc_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (build_err) DK(cudaMemcpyAsync(&h_build, build_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    DK(cudaStreamSynchronize(s));
    if (h_build || h_status) {
      // the flags were raised before this chunk's kernels ran on the results;
      // nothing is returned
      release_all();
      cudaStreamSynchronize(s);
      if (h_build) return fail_with(SDG_E_NONFINITE, "Cosine requires finite input (found NA, NaN or Inf).");
      return fail_with(SDG_E_CUDA, "tensor-core screen: a pipeline wait timed out");
    }
    for (int64_t t = 0; t < nb; ++t) {
      if (h_over[(size_t)t]) overflow.push_back(c0 + t);
      ctx_stats_add(ctx, 1, h_over[(size_t)t] ? n : h_count[(size_t)t]);   // pairs valued exactly
    }
  }
  if (!overflow.empty()) {
    DK(cudaMallocAsync(&row, sizeof(double) * (size_t)n, s));
    for (int64_t q : overflow) {
      k_dense_exact_row<<<blocks_for(n, 256), 256, 0, s>>>(method, D->d, D->x64, D->u64, Q->x64, Q->u64,
                                                            D->empty, n, q, self ? 1 : 0, row);
      SelectArgs sa;
      sa.vals = row; sa.seg_stride = 0; sa.elem_stride = 1; sa.len = n; sa.nseg = 1;
      sa.seg_blank = Q->empty + q0;
      sa.out_idx = o_idx; sa.out_val = o_val; sa.out_ld = nq; sa.out_row0 = q - q0;
      sa.k = k; sa.decreasing = 0;
      launch_select(sa, s);
    }
    DK(cudaGetLastError());
  }
  if (!device_out) {
    DK(cudaMemcpyAsync(idx, o_idx, sizeof(int32_t) * (size_t)(nq * k), cudaMemcpyDeviceToHost, s));
    DK(cudaMemcpyAsync(dist_out, o_val, sizeof(double) * (size_t)(nq * k), cudaMemcpyDeviceToHost, s));
  }
  if (S) DK(cudaFreeAsync(S, s));
  if (segtop) DK(cudaFreeAsync(segtop, s));
  if (cut) DK(cudaFreeAsync(cut, s));
  DK(cudaFreeAsync(cand, s)); DK(cudaFreeAsync(count, s));
  DK(cudaFreeAsync(over, s)); DK(cudaFreeAsync(vals, s));
  if (off) DK(cudaFreeAsync(off, s));
  if (tc_status) DK(cudaFreeAsync(tc_status, s));
  if (row) DK(cudaFreeAsync(row, s));
  if (!device_out) { DK(cudaFreeAsync(o_idx, s)); DK(cudaFreeAsync(o_val, s)); }
  DK(cudaStreamSynchronize(s));
  ctx_add_overflow(ctx, (int64_t)overflow.size());
  // kernels per chunk: the screen (fused: key init, weights, k_dense_tc, merge;
  // slab: the GEMM, segtop, thresh, keep, overflow), the FP32 cut (scan, dot,
  // cut) and the scan of the exact values, the exact values and the
  // selection; two more per overflowing query
  const int64_t chunks = (nq + chunk - 1) / chunk;
  ctx_stats_add(ctx, 3, chunks * ((fused ? 4 : 5) + (smode == 0 ? 4 : 0) + 2) + 2 * (int64_t)overflow.size());
  return SDG_OK;
}

}  // namespace

namespace sdg {
int32_t dense_rows(const sdg_dense* D) { return D->d; }
int64_t dense_cols(const sdg_dense* D) { return D->n; }
int64_t dense_query_bytes(const sdg_dense* D, int64_t nq, int k) {
  const int64_t cap = std::max(512, std::min(16384, 64 * k + 256));
  // the query's forms (FP64 x2, FP32 x2, BF16 x2 + padded), candidates and
  // exact values, results, and the fused screen's per-(query, range) lists
  // (at most 152 ranges for a single query tile, ~9 for full tiles)
  const int64_t ranges = std::max<int64_t>(9, 152 / std::max<int64_t>(1, (nq + 255) / 256));
  return nq * (36 * (int64_t)D->dpad + cap * 12 + (int64_t)k * 12 + ranges * (768 * 8 + (int64_t)k * 4 + 4)) +
         ((int64_t)1 << 20);
}
int dense_query(sdg_ctx* ctx, const sdg_dense* D, const float* Q, int32_t d, int64_t nq, int method, int k,
                int mode, int32_t* idx, double* dist_out, int device_out, int* k_eff, int* flags) {
  if (!ctx || !D || !Q) return fail_with(SDG_E_ARG, "NULL argument");
  if (d != D->d) return fail_with(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
  if (nq < 1) return fail_with(SDG_E_ARG, "'X' must have at least one column.");
  sdg_dense* QD = nullptr;
  int* berr = nullptr;
  int st = dense_build(ctx, Q, d, nq, true, false, &QD, &berr);
  if (st != SDG_OK) return st;
  st = dense_search(ctx, QD, 0, nq, D, false, method, k, mode, idx, dist_out, device_out, k_eff, flags, berr);
  if (st == SDG_OK) ctx_stats_add(ctx, 3, 4);        // the query block's prep, unit columns, cast, error norms
  if (st != SDG_OK && st != SDG_E_NONFINITE) {
    // an argument error found before the flag was read: non-finite input
    // still takes precedence, as when the build checked it at once
    int h = 0;
    if (cudaMemcpyAsync(&h, berr, sizeof(int), cudaMemcpyDeviceToHost, QD->stream) == cudaSuccess &&
        cudaStreamSynchronize(QD->stream) == cudaSuccess && h)
      st = fail_with(SDG_E_NONFINITE, "Cosine requires finite input (found NA, NaN or Inf).");
  }
  cudaFreeAsync(berr, QD->stream);
  sdg_dense_free(QD);
  return st;
}
}  // namespace sdg

extern "C" {

SDG_API int sdg_dense_upload(sdg_ctx* ctx, const float* X, int32_t d, int64_t n, sdg_dense** out) {
  if (!ctx || !X || !out || d < 1 || n < 1) return fail_with(SDG_E_ARG, "invalid dense upload arguments");
  return dense_build(ctx, X, d, n, false, true, out);
}

SDG_API int sdg_dense_free(sdg_dense* D) {
  if (!D) return SDG_OK;
  cudaSetDevice(D->device);
  void* bufs[] = {(void*)D->x64, (void*)D->u64, (void*)D->x32, (void*)D->u32, (void*)D->xb, (void*)D->ub,
                  (void*)D->norm2, (void*)D->scale, (void*)D->empty,
                  (void*)D->ue, (void*)D->un, (void*)D->xe, (void*)D->xn,
                  (void*)(D->ubp != D->ub ? D->ubp : nullptr), (void*)(D->xbp != D->xb ? D->xbp : nullptr)};
  if (D->async) {
    // a per-request matrix: stream-ordered frees after the work queued on its stream
    for (void* p : bufs)
      if (p) cudaFreeAsync(p, D->stream);
  } else {
    cudaDeviceSynchronize();
    for (void* p : bufs)
      if (p) cudaFree(p);
  }
  if (D->blas) cublasDestroy(D->blas);
  delete D;
  return SDG_OK;
}

SDG_API int sdg_dense_knn_block(sdg_ctx* ctx, const sdg_dense* D, int64_t q0, int64_t nq,
                                int method, int k, int mode, int32_t* idx, double* dist_out,
                                int device_out, int* k_eff, int* flags) {
  return dense_search(ctx, D, q0, nq, D, true, method, k, mode, idx, dist_out, device_out, k_eff, flags);
}

SDG_API int sdg_dense_knn_query(sdg_ctx* ctx, const sdg_dense* D, const float* Q, int32_t d, int64_t nq,
                                int method, int k, int mode, int32_t* idx, double* dist_out,
                                int device_out, int* k_eff, int* flags) {
  return dense_query(ctx, D, Q, d, nq, method, k, mode, idx, dist_out, device_out, k_eff, flags);
}

}  // extern "C"
