// sdg_api.cpp -- the C ABI of libsdgpu.so (include/sdgpu.h) and the host-side
// orchestration of the blocked kNN path: argument checks with the reference's
// messages, uploads, per-column preparation, the k clamp, and the
// candidate-generation engines (exact slab, or screen + exact re-rank).
//
// Reference behaviour restated here: R/sparseKNN.R:110-313 (sparseKNN),
// R/sparseKNNCross.R:44-199 (sparseKNNCross), R/sparseSNN.R:120-250
// (sparseSNN, edges = "knn") and the kernels' own checks in src/*.cpp.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <new>
#include <string>
#include <vector>

#include "../../include/sdgpu.h"
#include "sdg_kernels.h"
#include "sdg_screen.h"

using namespace sdg;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
namespace {

// The calling thread's last error message, in a fixed buffer so that setting
// it never allocates.
struct ErrBuf {
  char text[1024] = {0};
  size_t len = 0;
  void set(const char* s, size_t n) {
    n = std::min(n, sizeof(text) - 1);
    std::memcpy(text, s, n);
    text[n] = '\0';
    len = n;
  }
  ErrBuf& operator=(const std::string& s) { set(s.data(), s.size()); return *this; }
  ErrBuf& operator=(const char* s) { set(s, std::strlen(s)); return *this; }
  size_t size() const { return len; }
  const char* data() const { return text; }
};
thread_local ErrBuf g_err;

}  // namespace

namespace sdg {
void set_error(const char* msg) { g_err = msg; }
}  // namespace sdg

namespace {

struct Fail {
  int code;
};

[[noreturn]] void fail(int code, const std::string& msg) {
  g_err = msg;
  throw Fail{code};
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fail(e == cudaErrorMemoryAllocation ? SDG_E_NOMEM : SDG_E_CUDA,
         std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
  }
}
#define CK(x) cuda_check((x), #x)

const char* kMsgK = "'k' must be a positive integer no larger than .Machine$integer.max.";
const char* kMsgBlock = "'block_size' must be a positive integer no larger than .Machine$integer.max.";
const char* kMsgNcores = "'ncores' must be a non-negative integer no larger than .Machine$integer.max.";
const char* kMsgCosine = "Cosine requires finite input (found NA, NaN or Inf).";
const char* kMsgJS =
    "fastJS2 requires finite, non-negative input (columns should be normalised to sum to 1 "
    "for a true JS divergence).";

const char* method_name(int m) {
  static const char* names[] = {"binary", "cosine", "euclidean", "manhattan", "pearson", "js", "covariance"};
  return (m >= 0 && m <= 6) ? names[m] : "?";
}

void check_method(int method, int dist) {
  if (method < 0 || method > 6) fail(SDG_E_ARG, "unknown method");
  if ((method == EUCLIDEAN || method == MANHATTAN || method == JS) && !dist) {
    // R/sparseKNN.R:168-171
    fail(SDG_E_ARG, std::string("'dist = FALSE' is only meaningful for methods \"binary\", "
                                "\"cosine\" and \"pearson\"; ") +
                        method_name(method) + " has no similarity form.");
  }
}

// R/sparseKNN.R:172-181 (covariance is a coefficient: always the largest)
bool decreasing_for(int method, int dist) {
  if (method == COVARIANCE) return true;
  return (method == BINARY || method == COSINE || method == PEARSON) ? !dist : false;
}

template <typename T>
T* dalloc(size_t n, cudaStream_t s) {
  void* p = nullptr;
  CK(cudaMallocAsync(&p, std::max<size_t>(n, 1) * sizeof(T), s));
  return static_cast<T*>(p);
}

// RAII holder for stream-ordered device allocations.
struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  DevBuf() {}
  DevBuf(size_t bytes, cudaStream_t st) : s(st) { CK(cudaMallocAsync(&p, std::max<size_t>(bytes, 1), st)); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), s(o.s) { o.p = nullptr; }
  DevBuf& operator=(DevBuf&& o) noexcept { release(); p = o.p; s = o.s; o.p = nullptr; return *this; }
  ~DevBuf() { release(); }
  // Buffers owned by a resident matrix outlive any one stream: they are
  // released with the synchronous cudaFree (which also frees pool memory).
  void detach() { s = nullptr; }
  void release() {
    if (p) { if (s) cudaFreeAsync(p, s); else cudaFree(p); }
    p = nullptr;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

// The SNN graph a size query (p == NULL) built, kept on the device for the
// call that fetches the slots, so that the two-call protocol computes the
// graph once.  Matched on every argument and on a copy of idx's contents.
struct GraphCache {
  int kind = 0;                        // 1: edges = "knn", 2: edges = "shared"
  int32_t n = 0, k = 0;
  int include_self = 0, symmetrise = 0;
  double prune = 0.0;
  std::vector<int32_t> idx;
  int64_t m = 0;
  DevBuf p, i, x;
  bool matches(int kind_, const int32_t* idx_, int32_t n_, int32_t k_, int inc, int sym, double prune_) const {
    return kind == kind_ && n == n_ && k == k_ && include_self == inc && symmetrise == sym && prune == prune_ &&
           std::memcmp(idx.data(), idx_, sizeof(int32_t) * (size_t)n_ * (size_t)k_) == 0;
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// context and resident matrices
// ---------------------------------------------------------------------------
struct sdg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;       // where work is launched
  cudaStream_t own_stream = nullptr;   // the context's own stream
  std::atomic<int> cancel{0};
  int engine = 0;
  int64_t stats[8] = {0};
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // event pairs bracketing the bounding kernel's launches (sdg_kernel_time)
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> tev;
  size_t tev_used = 0;
  double tev_folded_ms = 0.0;
  int64_t tev_launches = 0;
  // false: choose the tensor-core screen only where the reference's dense
  // copy already exists (serving workers share the reference and must not
  // build it concurrently)
  bool tensor_lazy = true;
  std::unique_ptr<GraphCache> graph;   // see GraphCache
};

namespace {

void fold_kernel_times(sdg_ctx* c) {
  if (c->tev_used == 0) return;
  CK(cudaEventSynchronize(c->tev[c->tev_used - 1].second));
  for (size_t t = 0; t < c->tev_used; ++t) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->tev[t].first, c->tev[t].second));
    c->tev_folded_ms += ms;
  }
  c->tev_used = 0;
}

}  // namespace

namespace sdg {
cudaStream_t ctx_stream(sdg_ctx* c) { return c->stream; }
int ctx_device(sdg_ctx* c) { return c->device; }
void ctx_add_overflow(sdg_ctx* c, int64_t n) { c->stats[2] += n; }
void ctx_stats_add(sdg_ctx* c, int slot, int64_t n) { if (slot >= 0 && slot < 8) c->stats[slot] += n; }
void ctx_stats_reset(sdg_ctx* c) { std::memset(c->stats, 0, sizeof c->stats); }
}  // namespace sdg

// Brackets one launch of the bounding kernel (see sdg_kernel_time).
void sdg_time_begin(sdg_ctx* c) {
  if (c->tev_used == c->tev.size()) {
    if (c->tev.size() >= 1024) fold_kernel_times(c);
    else {
      cudaEvent_t a, b;
      CK(cudaEventCreate(&a));
      CK(cudaEventCreate(&b));
      c->tev.emplace_back(a, b);
    }
  }
  CK(cudaEventRecord(c->tev[c->tev_used].first, c->stream));
}
void sdg_time_end(sdg_ctx* c) {
  CK(cudaEventRecord(c->tev[c->tev_used].second, c->stream));
  ++c->tev_used;
  ++c->tev_launches;
}

struct sdg_matrix {
  sdg_ctx* ctx = nullptr;
  int32_t nrow = 0, ncol = 0;
  int64_t nnz = 0;
  DevBuf p, i, x;
  DevBuf empty;                 // uint8 per column
  int64_t n_empty = -1;
  DevBuf uval, scale;           // cosine
  int cos_status = 1;           // 1 = not computed, 0 = ok, <0 = error code
  DevBuf s1, s2;                // pearson moments
  bool have_moments = false;
  int js_status = 1;
  DevBuf xl;                    // js: xlogx of each stored value
  DevBuf xsum;                  // js: column sums
  ScreenCache screen[kMethodCount];   // screening data per method (sdg_screen.h)
  TensorCache tensor[kMethodCount];   // dense FP16 screen values per method (tensor-core screen)

  ~sdg_matrix() {
    if (ctx) {
      for (auto& sc : screen) screen_cache_free(&sc, ctx->stream);
      for (auto& tc : tensor) tensor_cache_free(&tc, ctx->stream);
      cudaStreamSynchronize(ctx->stream);
    }
    for (DevBuf* b : {&p, &i, &x, &empty, &uval, &scale, &s1, &s2, &xl, &xsum}) b->detach();
  }

  DevCsc dev() const {
    DevCsc d;
    d.nrow = nrow; d.ncol = ncol;
    d.p = p.as<int64_t>(); d.i = i.as<int32_t>(); d.x = x.as<double>();
    return d;
  }
};

namespace {

void check_csc_host(const sdg_csc* M, const char* name) {
  if (!M) fail(SDG_E_ARG, std::string("'") + name + "' must be provided.");
  if (M->nrow < 0 || M->ncol < 0) fail(SDG_E_ARG, std::string("invalid dimensions of '") + name + "'.");
  if (M->ncol > 0 && !M->p) fail(SDG_E_ARG, std::string("invalid dgCMatrix '") + name + "': no column pointers.");
  if (M->ncol > 0) {
    if (M->p[0] != 0) fail(SDG_E_ARG, std::string("invalid dgCMatrix '") + name + "': p[0] != 0.");
    for (int32_t j = 0; j < M->ncol; ++j)
      if (M->p[j + 1] < M->p[j])
        fail(SDG_E_ARG, std::string("invalid dgCMatrix '") + name + "': column pointers decrease.");
  }
}

__attribute__((unused)) void sync(sdg_ctx* c) { CK(cudaStreamSynchronize(c->stream)); }

// Row indices in range and strictly ascending within each column: checked on
// the device before any kernel indexes by row.
std::unique_ptr<sdg_matrix> upload(sdg_ctx* c, const sdg_csc* M, const char* name) {
  check_csc_host(M, name);
  auto m = std::make_unique<sdg_matrix>();
  m->ctx = c;
  m->nrow = M->nrow;
  m->ncol = M->ncol;
  m->nnz = M->ncol > 0 ? M->p[M->ncol] : 0;
  cudaStream_t s = c->stream;
  std::vector<int64_t> p64((size_t)m->ncol + 1, 0);
  for (int32_t j = 0; j <= m->ncol && m->ncol > 0; ++j) p64[j] = M->p[j];
  m->p = DevBuf(sizeof(int64_t) * p64.size(), s);
  m->i = DevBuf(sizeof(int32_t) * (size_t)m->nnz, s);
  m->x = DevBuf(sizeof(double) * (size_t)m->nnz, s);
  CK(cudaMemcpyAsync(m->p.p, p64.data(), sizeof(int64_t) * p64.size(), cudaMemcpyHostToDevice, s));
  if (m->nnz > 0) {
    CK(cudaMemcpyAsync(m->i.p, M->i, sizeof(int32_t) * (size_t)m->nnz, cudaMemcpyDefault, s));
    CK(cudaMemcpyAsync(m->x.p, M->x, sizeof(double) * (size_t)m->nnz, cudaMemcpyDefault, s));
  }
  DevBuf err(sizeof(int), s);
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  launch_check_rows(m->dev(), err.as<int>(), s);
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (herr)
    fail(SDG_E_ARG, std::string("invalid dgCMatrix '") + name +
                        "': row indices must lie in [0, nrow) and ascend within each column.");
  return m;
}

void ensure_empty(sdg_matrix* m) {
  if (m->n_empty >= 0) return;
  cudaStream_t s = m->ctx->stream;
  m->empty = DevBuf((size_t)m->ncol, s);
  launch_col_empty(m->dev(), m->empty.as<uint8_t>(), s);
  std::vector<uint8_t> h((size_t)m->ncol);
  if (m->ncol > 0)
    CK(cudaMemcpyAsync(h.data(), m->empty.p, (size_t)m->ncol, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int64_t n = 0;
  for (uint8_t v : h) n += v;
  m->n_empty = n;
}

void ensure_cosine(sdg_matrix* m) {
  if (m->cos_status == 0) return;
  if (m->cos_status < 0) fail(SDG_E_NONFINITE, kMsgCosine);
  cudaStream_t s = m->ctx->stream;
  m->uval = DevBuf(sizeof(double) * (size_t)m->nnz, s);
  m->scale = DevBuf(sizeof(double) * (size_t)m->ncol, s);
  DevBuf err(sizeof(int), s);
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  launch_unit_csc(m->dev(), m->uval.as<double>(), m->scale.as<double>(), err.as<int>(), s);
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  m->cos_status = herr ? SDG_E_NONFINITE : 0;
  if (herr) fail(SDG_E_NONFINITE, kMsgCosine);
}

void ensure_moments(sdg_matrix* m) {
  if (m->have_moments) return;
  cudaStream_t s = m->ctx->stream;
  m->s1 = DevBuf(sizeof(double) * (size_t)m->ncol, s);
  m->s2 = DevBuf(sizeof(double) * (size_t)m->ncol, s);
  launch_moments(m->dev(), m->s1.as<double>(), m->s2.as<double>(), s);
  m->have_moments = true;
}

void ensure_js(sdg_matrix* m, const char* msg = kMsgJS) {
  if (m->js_status == 0) return;
  if (m->js_status < 0) fail(SDG_E_NONFINITE, msg);
  cudaStream_t s = m->ctx->stream;
  DevBuf err(sizeof(int), s);
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  launch_check_js(m->x.as<double>(), m->nnz, err.as<int>(), s);
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  m->js_status = herr ? SDG_E_NONFINITE : 0;
  if (herr) fail(SDG_E_NONFINITE, msg);
  m->xl = DevBuf(sizeof(double) * (size_t)std::max<int64_t>(m->nnz, 1), s);
  launch_xlogx_values(m->x.as<double>(), m->nnz, m->xl.as<double>(), s);
  // column sums in row order (the moments' sums; the squares are not needed)
  m->xsum = DevBuf(sizeof(double) * (size_t)std::max<int64_t>(m->ncol, 1), s);
  DevBuf sq(sizeof(double) * (size_t)std::max<int64_t>(m->ncol, 1), s);
  launch_moments(m->dev(), m->xsum.as<double>(), sq.as<double>(), s);
}

// Method-specific preparation of the reference-side (m) and query-side (m2)
// matrices, in the order the reference raises its errors.
void prepare(int method, sdg_matrix* ref, sdg_matrix* qry) {
  if (method == COSINE) { ensure_cosine(ref); if (qry != ref) ensure_cosine(qry); }
  else if (method == PEARSON || method == COVARIANCE) { ensure_moments(ref); if (qry != ref) ensure_moments(qry); }
  else if (method == JS) { ensure_js(ref); if (qry != ref) ensure_js(qry); }
}

ColAux aux_of(const sdg_matrix* m) {
  ColAux a;
  a.empty = m->empty.as<uint8_t>();
  a.uval = m->uval.as<double>();
  a.scale = m->scale.as<double>();
  a.s = m->s1.as<double>();
  a.ss = m->s2.as<double>();
  a.xl = m->xl.as<double>();
  a.xsum = m->xsum.as<double>();
  return a;
}

void check_cancel(sdg_ctx* c) {
  if (c->cancel.load(std::memory_order_relaxed)) fail(SDG_E_CANCELLED, "Computation interrupted by the user.");
}

// ---------------------------------------------------------------------------
// forward kNN on the device: result d_idx / d_val (nq x k, column-major)
// ---------------------------------------------------------------------------
struct KnnPlan {
  int method = 0, dist = 1, k = 1;
  bool decreasing = false;
  bool selfmode = false, include_self = false;
  const uint8_t* ref_mask = nullptr;   // degenerate reference columns (or null)
  const uint8_t* qry_blank = nullptr;  // degenerate query columns (or null)
  // result row of query column q: q - out_first, leading dimension out_ld
  int64_t out_first = 0, out_ld = 0;
};

double self_value_for(const KnnPlan& P) {
  // R/sparseKNN.R:270-279
  return (P.method == BINARY || P.method == COSINE || P.method == PEARSON) ? (P.dist ? 0.0 : 1.0)
                                                                           : 0.0;
}

// Exact FP64 slab + exact top-k for query columns [q_lo, q_hi).
void exact_engine(sdg_ctx* c, const KnnPlan& P, sdg_matrix* ref, sdg_matrix* qry,
                  int32_t* d_idx, double* d_val, int64_t q_lo, int64_t q_hi) {
  cudaStream_t s = c->stream;
  const int64_t nr = ref->ncol, nq = qry->ncol;
  const int64_t budget = (int64_t)1 << 30;                 // slab bytes per chunk
  int64_t B = std::max<int64_t>(1, std::min<int64_t>(q_hi - q_lo, budget / std::max<int64_t>(1, nr * 8)));
  DevBuf D(sizeof(double) * (size_t)(nr * B), s);
  const ColAux ra = aux_of(ref), qa = aux_of(qry);
  const double self_value = self_value_for(P);
  for (int64_t q0 = q_lo; q0 < q_hi; q0 += B) {
    check_cancel(c);
    const int64_t nb = std::min(B, q_hi - q0);
    sdg_time_begin(c);
    // R/sparseKNN.R:270-279; covariance keeps its computed self value (the variance)
    launch_exact_slab(P.method, P.dist, ref->dev(), ra, qry->dev(), qa, q0, nb, P.ref_mask,
                      P.selfmode && P.include_self && P.method != COVARIANCE, self_value, D.as<double>(), s);
    sdg_time_end(c);
    SelectArgs a;
    a.vals = D.as<double>();
    a.seg_stride = nr; a.elem_stride = 1; a.len = nr; a.nseg = nb;
    a.idx_base = 0;
    a.skip_base = (P.selfmode && !P.include_self) ? q0 : -1;
    a.seg_blank = P.qry_blank ? P.qry_blank + P.out_first : nullptr;
    a.out_idx = d_idx; a.out_val = d_val; a.out_ld = P.out_ld; a.out_row0 = q0 - P.out_first;
    a.k = P.k; a.decreasing = P.decreasing;
    launch_select(a, s);
    c->stats[1] += nr * nb;
    c->stats[3] += 2;
  }
  CK(cudaGetLastError());
}

// 1: exact FP64 slab; 2: FP32 sparse screen; 3: BF16 tensor-core screen
// (cosine / euclidean; falls back to 2 inside screen_knn when a matrix's
// values do not admit the BF16 bound or its dense copy does not fit).
int pick_engine(sdg_ctx* c, const KnnPlan& P, const sdg_matrix* ref, const sdg_matrix* X, int64_t nq) {
  const int32_t nrow = ref->nrow;
  const int64_t nr = ref->ncol;
  if (c->engine == 1) return 1;
  if (!screen_supported(P.method, P.k) || !screen_fits(nrow)) return 1;
  if (c->engine == 2) return 2;
  if (c->engine == 3) return (tensor_supported(P.method) && stc_supported(P.k)) ? 3 : 2;
  // Small problems: the exact slab is already latency-bound.
  if (nr * nq <= (int64_t)1 << 22) return 1;
  // The tensor screen does 2 nrow nr nq dense flops where the FP32 screen
  // visits nq / 16 * nnz(ref) stored entries: it wins from ~0.5 % density
  // on, if the dense copies fit in half of the free device memory.
  if (tensor_supported(P.method) && stc_supported(P.k) && nrow > 0 && nr > 0 &&
      (c->tensor_lazy || (ref->tensor[P.method].method == P.method && ref->tensor[P.method].usable))) {
    const double density = (double)ref->nnz / ((double)nrow * (double)nr);
    size_t bytes = tensor_cache_bytes(nrow, nr);
    if (X != ref) bytes += tensor_cache_bytes(nrow, X->ncol);
    size_t fr = 0, tot = 0;
    if (ref->tensor[P.method].method == P.method && ref->tensor[P.method].usable) bytes = 0;   // already resident
    if (density >= 0.005 && cudaMemGetInfo(&fr, &tot) == cudaSuccess && bytes <= fr / 2) return 3;
    cudaGetLastError();
  }
  return 2;
}

// sparseKNN core (R/sparseKNN.R:183-301) after argument checks.
// Computes rows [q_lo, q_hi) (q_hi < 0: all) of the result, laid out as a
// (q_hi - q_lo) x k column-major matrix.
void knn_device(sdg_ctx* c, sdg_matrix* X, sdg_matrix* Y, int method, int dist, int k,
                int include_self, int drop_degenerate, bool cross_side, int side,
                int32_t* d_idx_out, double* d_val_out, int* k_eff, int* flags,
                DevBuf* hold_idx, DevBuf* hold_val, int64_t q_lo = 0, int64_t q_hi = -1) {
  const bool selfmode = (Y == nullptr);
  sdg_matrix* ref = selfmode ? X : Y;
  ensure_empty(ref);
  ensure_empty(X);
  int64_t avail = drop_degenerate ? (ref->ncol - ref->n_empty) : ref->ncol;
  if (selfmode && !include_self) avail -= 1;
  if (avail < 1) {
    if (cross_side)
      fail(SDG_E_NOCAND, std::string("No candidate neighbours available for the ") +
                             (side == 0 ? "forward" : "reverse") + " direction.");
    fail(SDG_E_NOCAND, "No candidate neighbours available.");
  }
  if (k > avail) {
    *flags |= (side == 0) ? SDG_WARN_CLAMP_FWD : SDG_WARN_CLAMP_REV;
    k = (int)avail;
  }
  *k_eff = k;
  prepare(method, ref, X);

  KnnPlan P;
  P.method = method; P.dist = dist; P.k = k; P.decreasing = decreasing_for(method, dist);
  P.selfmode = selfmode; P.include_self = include_self != 0;
  P.ref_mask = drop_degenerate ? ref->empty.as<uint8_t>() : nullptr;
  P.qry_blank = drop_degenerate ? X->empty.as<uint8_t>() : nullptr;

  cudaStream_t s = c->stream;
  const int64_t nq_all = X->ncol;
  if (q_hi < 0) q_hi = nq_all;
  if (q_lo < 0 || q_hi > nq_all || q_lo >= q_hi) fail(SDG_E_ARG, "invalid query column range");
  const int64_t nq = q_hi - q_lo;
  P.out_first = q_lo;
  P.out_ld = nq;
  int32_t* d_idx = d_idx_out;
  double* d_val = d_val_out;
  if (!d_idx) {
    *hold_idx = DevBuf(sizeof(int32_t) * (size_t)(nq * k), s);
    *hold_val = DevBuf(sizeof(double) * (size_t)(nq * k), s);
    d_idx = hold_idx->as<int32_t>();
    d_val = hold_val->as<double>();
  }
  const int eng = pick_engine(c, P, ref, X, nq);
  if (eng == 2 || eng == 3) {
    ScreenRun r;
    r.method = method; r.dist = dist; r.k = k; r.decreasing = P.decreasing;
    r.selfmode = selfmode; r.include_self = P.include_self;
    r.self_value = self_value_for(P);
    r.ref_mask = P.ref_mask; r.qry_blank = P.qry_blank;
    r.qry_empty = X->empty.as<uint8_t>();
    r.q_lo = q_lo; r.q_hi = q_hi; r.out_first = q_lo; r.out_ld = nq;
    if (eng == 3) {
      r.tensor = true;
    }
    ScreenHooks h;
    h.check_cancel = [c]() { check_cancel(c); };
    h.time_begin = [c]() { sdg_time_begin(c); };
    h.time_end = [c]() { sdg_time_end(c); };
    h.exact_range = [&](int64_t q0, int64_t n) { exact_engine(c, P, ref, X, d_idx, d_val, q0, q0 + n); };
    const int st = screen_knn(c->stream, r, ref->dev(), aux_of(ref), &ref->screen[method], &ref->tensor[method],
                              X->dev(), aux_of(X), &X->screen[method], &X->tensor[method], d_idx, d_val, c->stats, h);
    if (st) cuda_check((cudaError_t)st, (std::string("screen_knn (") + screen_error_site() + ")").c_str());
  } else {
    exact_engine(c, P, ref, X, d_idx, d_val, q_lo, q_hi);
  }
}

template <typename F>
int guarded(F&& f) {
  try {
    f();
    return SDG_OK;
  } catch (const Fail& e) {
    return e.code;
  } catch (const std::bad_alloc&) {
    g_err = "out of host memory";
    return SDG_E_NOMEM;
  } catch (const std::exception& e) {
    g_err = e.what();
    return SDG_E_CUDA;
  } catch (...) {
    g_err = "unknown failure";
    return SDG_E_CUDA;
  }
}

void check_counts(int k, int block_size, int ncores) {
  if (k < 1) fail(SDG_E_ARG, kMsgK);
  if (block_size < 1) fail(SDG_E_ARG, kMsgBlock);
  if (ncores < 0) fail(SDG_E_ARG, kMsgNcores);
}

void begin_stats(sdg_ctx* c) {
  std::memset(c->stats, 0, sizeof c->stats);
  CK(cudaEventRecord(c->ev[0], c->stream));
}
void end_stats(sdg_ctx* c) {
  CK(cudaEventRecord(c->ev[1], c->stream));
  CK(cudaEventSynchronize(c->ev[1]));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  c->stats[5] = (int64_t)(ms * 1000.0f);
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

SDG_API int sdg_version(void) { return 10000; }

SDG_API int sdg_last_error(char* buf, size_t len) {
  if (buf && len > 0) {
    const size_t n = std::min(len - 1, g_err.size());
    std::memcpy(buf, g_err.data(), n);
    buf[n] = '\0';
  }
  return (int)g_err.size();
}

SDG_API int sdg_ctx_create(int device, sdg_ctx** out) {
  return guarded([&] {
    if (!out) fail(SDG_E_ARG, "out must not be NULL");
    auto c = std::make_unique<sdg_ctx>();
    if (device < 0) CK(cudaGetDevice(&device));
    c->device = device;
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    c->stream = c->own_stream;
    // Keep freed pool memory mapped: the per-call slabs (up to a few GB) are
    // re-allocated on every call and would otherwise be unmapped and mapped
    // again at each synchronisation.
    cudaMemPool_t pool;
    CK(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = UINT64_MAX;
    CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    for (auto& e : c->ev) CK(cudaEventCreate(&e));
    *out = c.release();
  });
}

SDG_API int sdg_ctx_destroy(sdg_ctx* c) {
  if (!c) return SDG_OK;
  cudaStreamSynchronize(c->stream);
  c->graph.reset();
  for (auto& e : c->ev) if (e) cudaEventDestroy(e);
  for (auto& pr : c->tev) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
  cudaStreamDestroy(c->own_stream);
  delete c;
  return SDG_OK;
}

SDG_API int sdg_ctx_cancel(sdg_ctx* c) {
  if (!c) return SDG_E_ARG;
  c->cancel.store(1);
  return SDG_OK;
}

SDG_API int sdg_ctx_reset_cancel(sdg_ctx* c) {
  if (!c) return SDG_E_ARG;
  c->cancel.store(0);
  return SDG_OK;
}

SDG_API int sdg_ctx_set_stream(sdg_ctx* c, void* stream) {
  return guarded([&] {
    if (!c) fail(SDG_E_ARG, "ctx must not be NULL");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  });
}

SDG_API int sdg_ctx_set_engine(sdg_ctx* c, int engine) {
  if (!c || engine < 0 || engine > 3) { g_err = "invalid engine"; return SDG_E_ARG; }
  c->engine = engine;
  return SDG_OK;
}

SDG_API int sdg_debug_stall_tc(int launches) {
  if (launches < 0) { g_err = "launches must be >= 0"; return SDG_E_ARG; }
  tc_set_stall(launches);
  return SDG_OK;
}

SDG_API int sdg_kernel_time(sdg_ctx* c, double* ms, int64_t* launches) {
  return guarded([&] {
    if (!c || !ms || !launches) fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    fold_kernel_times(c);
    *ms = c->tev_folded_ms;
    *launches = c->tev_launches;
    c->tev_folded_ms = 0.0;
    c->tev_launches = 0;
  });
}

SDG_API int sdg_last_stats(sdg_ctx* c, int64_t* out, int n) {
  if (!c || !out) return SDG_E_ARG;
  for (int t = 0; t < n && t < 8; ++t) out[t] = c->stats[t];
  return SDG_OK;
}

SDG_API int sdg_dist_cross(sdg_ctx* c, int method, int dist, const sdg_csc* m, const sdg_csc* m2,
                           double* D) {
  return guarded([&] {
    if (!c) fail(SDG_E_ARG, "ctx must not be NULL");
    CK(cudaSetDevice(c->device));
    if (method < 0 || method > 6) fail(SDG_E_ARG, "unknown method");
    check_csc_host(m, "m");
    check_csc_host(m2, "m2");
    if (method == JS) {                              // src/sparseDist.cpp:1077-1081 first
      auto a = upload(c, m, "m");
      auto b = upload(c, m2, "m2");
      ensure_js(a.get());
      ensure_js(b.get());
    }
    if (m->nrow != m2->nrow)
      fail(SDG_E_ROWS, "Mismatched row dimensions of m (" + std::to_string(m->nrow) +
                           ") and m2 (" + std::to_string(m2->nrow) + ").");
    auto a = upload(c, m, "m");
    auto b = upload(c, m2, "m2");
    prepare(method, a.get(), b.get());
    cudaStream_t s = c->stream;
    const int64_t nc = a->ncol, nc2 = b->ncol;
    const int64_t budget = (int64_t)1 << 30;
    const int64_t B = std::max<int64_t>(1, std::min<int64_t>(std::max<int64_t>(nc2, 1),
                                                             budget / std::max<int64_t>(1, nc * 8)));
    DevBuf Dd(sizeof(double) * (size_t)(nc * B), s);
    for (int64_t q0 = 0; q0 < nc2; q0 += B) {
      const int64_t nb = std::min(B, nc2 - q0);
      launch_exact_slab(method, dist, a->dev(), aux_of(a.get()), b->dev(), aux_of(b.get()), q0,
                        nb, nullptr, 0, 0.0, Dd.as<double>(), s);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(D + q0 * nc, Dd.p, sizeof(double) * (size_t)(nc * nb),
                         cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
  });
}

// mean stored entries per column from which the single-matrix form of the
// match-only methods runs on the query-centric kernel
constexpr double kSelfTriMinNnz = 256.0;

SDG_API int sdg_dist(sdg_ctx* c, int method, int dist, const sdg_csc* m, int full, int diag,
                     double* D) {
  return guarded([&] {
    if (!c) fail(SDG_E_ARG, "ctx must not be NULL");
    CK(cudaSetDevice(c->device));
    if (method < 0 || method > 6) fail(SDG_E_ARG, "unknown method");
    check_csc_host(m, "m");
    auto a = upload(c, m, "m");
    if (method == JS)                                // src/sparseDist.cpp:1024-1027
      ensure_js(a.get(), "fastJS requires finite, non-negative input (columns should be "
                         "normalised to sum to 1 for a true JS divergence).");
    prepare(method, a.get(), a.get());
    cudaStream_t s = c->stream;
    const int64_t n = a->ncol;
    if (n == 0) return;
    if ((uint64_t)n > ((uint64_t)1 << 30))                  // n^2 doubles would overflow size_t
      fail(SDG_E_NOMEM, "the ncol x ncol result does not fit in memory");
    const size_t whole = sizeof(double) * (size_t)n * (size_t)n;
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    // device bytes the result may hold: half the free memory, or less where
    // SDG_DIST_RESIDENT_BYTES says so (a tuning knob; it also reaches the
    // streamed path on small inputs)
    size_t cap = free_b / 2;
    if (const char* e = std::getenv("SDG_DIST_RESIDENT_BYTES"))
      cap = std::min<size_t>(cap, (size_t)std::strtoull(e, nullptr, 10));
    if (whole <= cap) {
      // resident: the lower triangle once, mirrored on the device with full
      DevBuf Dd(whole, s);
      // match-only methods with long columns: the upper triangle on the
      // query-centric kernel (one pair per lane), then moved to the lower
      // one; short columns merge faster one pair per thread.  Engine 1 forces
      // the per-thread kernel, 2 / 3 the query-centric one where supported.
      const double mean_nnz = (double)a->nnz / (double)n;
      const bool tri = self_tri_supported(method, a->nrow) &&
                       (c->engine == 2 || c->engine == 3 || (c->engine == 0 && mean_nnz >= kSelfTriMinNnz));
      if (tri) {
        sdg_time_begin(c);
        launch_self_tri(method, dist, a->dev(), aux_of(a.get()), diag, Dd.as<double>(), s);
        sdg_time_end(c);
        CK(cudaGetLastError());
        launch_mirror_upper(Dd.as<double>(), n, full ? 0 : 1, s);
        CK(cudaGetLastError());
      } else {
        sdg_time_begin(c);
        launch_self_slab(method, dist, a->dev(), aux_of(a.get()), 0, n, 0, diag, Dd.as<double>(), s);
        sdg_time_end(c);
        CK(cudaGetLastError());
        if (full) {
          launch_mirror_lower(Dd.as<double>(), n, s);
          CK(cudaGetLastError());
        }
      }
      CK(cudaMemcpyAsync(D, Dd.p, whole, cudaMemcpyDeviceToHost, s));
    } else {
      // streamed in column blocks of about 1 GiB; with full both triangles
      // are computed, as no earlier block stays on the device to mirror
      const int64_t budget = std::min<int64_t>((int64_t)1 << 30, (int64_t)cap);
      const int64_t B = std::max<int64_t>(1, std::min<int64_t>(n, budget / (n * 8)));
      DevBuf Dd(sizeof(double) * (size_t)(n * B), s);
      for (int64_t c0 = 0; c0 < n; c0 += B) {
        const int64_t nb = std::min(B, n - c0);
        sdg_time_begin(c);
        launch_self_slab(method, dist, a->dev(), aux_of(a.get()), c0, nb, full, diag,
                         Dd.as<double>(), s);
        sdg_time_end(c);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(D + c0 * n, Dd.p, sizeof(double) * (size_t)(n * nb),
                           cudaMemcpyDeviceToHost, s));
      }
    }
    CK(cudaStreamSynchronize(s));
  });
}

SDG_API int sdg_topk_block(sdg_ctx* c, const double* D, int64_t nrow, int64_t ncol, int k,
                           int decreasing, const int32_t* self_row, int32_t* idx, double* dist) {
  return guarded([&] {
    if (!c) fail(SDG_E_ARG, "ctx must not be NULL");
    CK(cudaSetDevice(c->device));
    if (k < 1) fail(SDG_E_ARG, "k must be >= 1.");
    if (nrow < 0 || ncol < 0) fail(SDG_E_ARG, "invalid dimensions of D.");
    std::vector<int64_t> skip((size_t)std::max<int64_t>(ncol, 1), -1);
    for (int64_t b = 0; b < ncol; ++b) {
      const int32_t sr = self_row ? self_row[b] : 0;
      if (sr == NA_INT || sr < 0 || (int64_t)sr > nrow)
        fail(SDG_E_ARG, "self_row entries must be 0 or valid 1-based rows of D.");
      skip[(size_t)b] = sr > 0 ? sr - 1 : -1;
    }
    if (ncol == 0) return;
    cudaStream_t s = c->stream;
    DevBuf dD(sizeof(double) * (size_t)(nrow * ncol), s), dskip(sizeof(int64_t) * (size_t)ncol, s);
    DevBuf di(sizeof(int32_t) * (size_t)(ncol * k), s), dv(sizeof(double) * (size_t)(ncol * k), s);
    if (nrow > 0) CK(cudaMemcpyAsync(dD.p, D, sizeof(double) * (size_t)(nrow * ncol), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dskip.p, skip.data(), sizeof(int64_t) * (size_t)ncol, cudaMemcpyHostToDevice, s));
    SelectArgs a;
    a.vals = dD.as<double>(); a.seg_stride = nrow; a.elem_stride = 1; a.len = nrow; a.nseg = ncol;
    a.skip_arr = dskip.as<int64_t>();
    a.out_idx = di.as<int32_t>(); a.out_val = dv.as<double>(); a.out_ld = ncol; a.out_row0 = 0;
    a.k = k; a.decreasing = decreasing != 0;
    launch_select(a, s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(idx, di.p, sizeof(int32_t) * (size_t)(ncol * k), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(dist, dv.p, sizeof(double) * (size_t)(ncol * k), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  });
}

SDG_API int sdg_topk_rows_accum(sdg_ctx* c, const double* D, int64_t nrow, int64_t ncol, int k,
                                int decreasing, int32_t* best_idx, double* best_val,
                                int32_t col_offset, const int32_t* self_col) {
  return guarded([&] {
    if (!c) fail(SDG_E_ARG, "ctx must not be NULL");
    CK(cudaSetDevice(c->device));
    if (k < 1) fail(SDG_E_ARG, "k must be >= 1.");
    if (col_offset < 0) fail(SDG_E_ARG, "col_offset must be >= 0.");
    if (nrow < 0 || ncol < 0) fail(SDG_E_ARG, "invalid dimensions of D.");
    std::vector<int64_t> skip((size_t)std::max<int64_t>(nrow, 1), -1);
    for (int64_t r = 0; r < nrow; ++r) {
      const int32_t sc = self_col ? self_col[r] : 0;
      if (sc == NA_INT || sc < 0)
        fail(SDG_E_ARG, "self_col entries must be 0 or a positive 1-based query index.");
      skip[(size_t)r] = sc > 0 ? (int64_t)sc - 1 : -1;
    }
    if (nrow == 0) return;
    cudaStream_t s = c->stream;
    DevBuf dD(sizeof(double) * (size_t)std::max<int64_t>(nrow * ncol, 1), s);
    DevBuf dskip(sizeof(int64_t) * (size_t)nrow, s);
    DevBuf di(sizeof(int32_t) * (size_t)(nrow * k), s), dv(sizeof(double) * (size_t)(nrow * k), s);
    if (ncol > 0) CK(cudaMemcpyAsync(dD.p, D, sizeof(double) * (size_t)(nrow * ncol), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dskip.p, skip.data(), sizeof(int64_t) * (size_t)nrow, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(di.p, best_idx, sizeof(int32_t) * (size_t)(nrow * k), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dv.p, best_val, sizeof(double) * (size_t)(nrow * k), cudaMemcpyHostToDevice, s));
    SelectArgs a;
    a.vals = dD.as<double>(); a.seg_stride = 1; a.elem_stride = nrow; a.len = ncol; a.nseg = nrow;
    a.idx_base = col_offset;
    a.skip_arr = dskip.as<int64_t>();
    a.seed_idx = di.as<int32_t>(); a.seed_val = dv.as<double>(); a.seed_ld = nrow;
    a.out_idx = di.as<int32_t>(); a.out_val = dv.as<double>(); a.out_ld = nrow; a.out_row0 = 0;
    a.k = k; a.decreasing = decreasing != 0;
    launch_select(a, s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(best_idx, di.p, sizeof(int32_t) * (size_t)(nrow * k), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(best_val, dv.p, sizeof(double) * (size_t)(nrow * k), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  });
}

namespace {
void snn_weights_device(sdg_ctx* c, const int32_t* idx, int32_t n, int32_t k, int include_self,
                        DevBuf* d_idx, DevBuf* d_w) {
  if (n < 1 || k < 1) fail(SDG_E_ARG, "'idx' must have at least one row and column.");
  cudaStream_t s = c->stream;
  const int64_t total = (int64_t)n * k;
  *d_idx = DevBuf(sizeof(int32_t) * (size_t)total, s);
  *d_w = DevBuf(sizeof(double) * (size_t)total, s);
  CK(cudaMemcpyAsync(d_idx->p, idx, sizeof(int32_t) * (size_t)total, cudaMemcpyHostToDevice, s));
  DevBuf err(sizeof(int), s);
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  launch_snn_check(d_idx->as<int32_t>(), n, k, err.as<int>(), s);
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (herr)
    fail(SDG_E_INDEX, "'idx' entries must be NA or 1-based row indices in [1, nrow(idx)].");
  DevBuf sets(sizeof(int32_t) * (size_t)n * ((size_t)k + 1), s), sizes(sizeof(int32_t) * (size_t)n, s);
  launch_snn_sets(d_idx->as<int32_t>(), n, k, include_self, sets.as<int32_t>(), sizes.as<int32_t>(), s);
  launch_snn_weights(d_idx->as<int32_t>(), n, k, sets.as<int32_t>(), sizes.as<int32_t>(),
                     d_w->as<double>(), s);
  CK(cudaGetLastError());
}
}  // namespace

SDG_API int sdg_snn_jaccard(sdg_ctx* c, const int32_t* idx, int32_t n, int32_t k, int include_self,
                            double* w) {
  return guarded([&] {
    if (!c) fail(SDG_E_ARG, "ctx must not be NULL");
    CK(cudaSetDevice(c->device));
    DevBuf di, dw;
    snn_weights_device(c, idx, n, k, include_self, &di, &dw);
    CK(cudaMemcpyAsync(w, dw.p, sizeof(double) * (size_t)n * k, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  });
}

namespace {

// Copies a graph's slots to the host (p, i, x non-NULL).
void graph_to_host(sdg_ctx* c, int32_t n, int64_t m, const void* dp, const void* drow, const void* dx,
                   int32_t* p, int32_t* i, double* x) {
  CK(cudaMemcpyAsync(p, dp, sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost, c->stream));
  if (m > 0) {
    CK(cudaMemcpyAsync(i, drow, sizeof(int32_t) * (size_t)m, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(x, dx, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
}

// A fetch (p != NULL) that a size query with the same arguments prepared:
// copies the kept graph and drops it.
bool graph_from_cache(sdg_ctx* c, int kind, const int32_t* idx, int32_t n, int32_t k, int inc, int sym,
                      double prune, int64_t* nnz, int32_t* p, int32_t* i, double* x) {
  GraphCache* g = c->graph.get();
  if (!p || !g || !idx || !g->matches(kind, idx, n, k, inc, sym, prune)) return false;
  *nnz = g->m;
  graph_to_host(c, n, g->m, g->p.p, g->i.p, g->x.p, p, i, x);
  c->graph.reset();
  return true;
}

// After a build: a size query keeps the graph for the fetch; a fetch copies it.
void graph_finish(sdg_ctx* c, int kind, const int32_t* idx, int32_t n, int32_t k, int inc, int sym, double prune,
                  int64_t m, DevBuf& hp, DevBuf& hi, DevBuf& hx, int64_t* nnz, int32_t* p, int32_t* i,
                  double* x) {
  *nnz = m;
  if (p) {
    graph_to_host(c, n, m, hp.p, hi.p, hx.p, p, i, x);
    return;
  }
  CK(cudaStreamSynchronize(c->stream));
  auto g = std::make_unique<GraphCache>();
  g->kind = kind;
  g->n = n;
  g->k = k;
  g->include_self = inc;
  g->symmetrise = sym;
  g->prune = prune;
  g->idx.assign(idx, idx + (size_t)n * (size_t)k);
  g->m = m;
  g->p = std::move(hp);
  g->i = std::move(hi);
  g->x = std::move(hx);
  g->p.detach();                          // freed synchronously, whatever stream is current then
  g->i.detach();
  g->x.detach();
  c->graph = std::move(g);
}

}  // namespace

SDG_API int sdg_snn_graph(sdg_ctx* c, const int32_t* idx, int32_t n, int32_t k, int include_self,
                          double prune, int symmetrise, int64_t* nnz, int32_t* p, int32_t* i,
                          double* x) {
  return guarded([&] {
    if (!c) fail(SDG_E_ARG, "ctx must not be NULL");
    if (!nnz || !idx) fail(SDG_E_ARG, "idx and nnz must not be NULL");
    CK(cudaSetDevice(c->device));
    if (!(prune >= 0.0 && prune <= 1.0))
      fail(SDG_E_ARG, "'prune' must be a finite number between 0 and 1.");
    if (graph_from_cache(c, 1, idx, n, k, include_self, symmetrise, prune, nnz, p, i, x)) return;
    c->graph.reset();
    DevBuf di, dw;
    snn_weights_device(c, idx, n, k, include_self, &di, &dw);
    int32_t *dp = nullptr, *drow = nullptr;
    double* dx = nullptr;
    int64_t m = 0;
    const int st = snn_graph_build(di.as<int32_t>(), dw.as<double>(), n, k, prune, symmetrise, &m,
                                   &dp, &drow, &dx, c->stream);
    if (st) cuda_check((cudaError_t)st, "snn_graph_build");
    DevBuf hp, hi, hx;
    hp.p = dp; hp.s = c->stream;
    hi.p = drow; hi.s = c->stream;
    hx.p = dx; hx.s = c->stream;
    graph_finish(c, 1, idx, n, k, include_self, symmetrise, prune, m, hp, hi, hx, nnz, p, i, x);
  });
}

SDG_API int sdg_snn_graph_shared(sdg_ctx* c, const int32_t* idx, int32_t n, int32_t k, int include_self,
                                 double prune, int64_t* nnz, int32_t* p, int32_t* i, double* x) {
  return guarded([&] {
    if (!c) fail(SDG_E_ARG, "ctx must not be NULL");
    if (!nnz || !idx) fail(SDG_E_ARG, "idx and nnz must not be NULL");
    CK(cudaSetDevice(c->device));
    if (!(prune >= 0.0 && prune <= 1.0))
      fail(SDG_E_ARG, "'prune' must be a finite number between 0 and 1.");
    if (n < 1 || k < 1) fail(SDG_E_ARG, "'idx' must have at least one row and column.");
    if (graph_from_cache(c, 2, idx, n, k, include_self, 1, prune, nnz, p, i, x)) return;
    c->graph.reset();
    cudaStream_t s = c->stream;
    const int64_t total = (int64_t)n * k;
    DevBuf di(sizeof(int32_t) * (size_t)total, s);
    CK(cudaMemcpyAsync(di.p, idx, sizeof(int32_t) * (size_t)total, cudaMemcpyHostToDevice, s));
    DevBuf err(sizeof(int), s);
    CK(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    launch_snn_check(di.as<int32_t>(), n, k, err.as<int>(), s);
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (herr)
      fail(SDG_E_INDEX, "'idx' entries must be NA or 1-based row indices in [1, nrow(idx)].");
    DevBuf sets(sizeof(int32_t) * (size_t)n * ((size_t)k + 1), s), sizes(sizeof(int32_t) * (size_t)n, s);
    launch_snn_sets(di.as<int32_t>(), n, k, include_self, sets.as<int32_t>(), sizes.as<int32_t>(), s);
    int32_t *dp = nullptr, *drow = nullptr;
    double* dx = nullptr;
    int64_t m = 0;
    const int st = snn_shared_build(sets.as<int32_t>(), sizes.as<int32_t>(), n, k, prune, &m, &dp, &drow, &dx, s);
    if (st) cuda_check((cudaError_t)st, "snn_shared_build");
    DevBuf hp, hi, hx;
    hp.p = dp; hp.s = s;
    hi.p = drow; hi.s = s;
    hx.p = dx; hx.s = s;
    graph_finish(c, 2, idx, n, k, include_self, 1, prune, m, hp, hi, hx, nnz, p, i, x);
  });
}

SDG_API int sdg_knn(sdg_ctx* c, const sdg_csc* X, const sdg_csc* Y, int method, int dist, int k,
                    int include_self, int drop_degenerate, int block_size, int ncores,
                    int32_t* idx, double* dist_out, int* k_eff, int* flags) {
  return guarded([&] {
    if (!c || !idx || !dist_out || !k_eff || !flags) fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    *flags = 0;
    check_counts(k, block_size, ncores);
    check_method(method, dist);
    check_csc_host(X, "X");
    if (X->ncol < 1) fail(SDG_E_ARG, "'X' must have at least one column.");
    if (Y) {
      check_csc_host(Y, "Y");
      if (X->nrow != Y->nrow) fail(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
    }
    begin_stats(c);
    auto xm = upload(c, X, "X");
    std::unique_ptr<sdg_matrix> ym;
    if (Y) ym = upload(c, Y, "Y");
    DevBuf hi, hv;
    knn_device(c, xm.get(), ym.get(), method, dist, k, include_self, drop_degenerate, false, 0,
               nullptr, nullptr, k_eff, flags, &hi, &hv);
    const size_t cnt = (size_t)xm->ncol * (size_t)*k_eff;
    CK(cudaMemcpyAsync(idx, hi.p, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(dist_out, hv.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost, c->stream));
    end_stats(c);
  });
}

SDG_API int sdg_knn_block(sdg_ctx* c, const sdg_matrix* X, const sdg_matrix* Y, int64_t q0,
                          int64_t nq, int method, int dist, int k, int include_self,
                          int drop_degenerate, int32_t* idx, double* dist_out, int device_out,
                          int* k_eff, int* flags) {
  return guarded([&] {
    if (!c || !X || !idx || !dist_out || !k_eff || !flags) fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    *flags = 0;
    if (k < 1) fail(SDG_E_ARG, kMsgK);
    check_method(method, dist);
    if (Y && X->nrow != Y->nrow) fail(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
    if (q0 < 0 || nq < 1 || q0 + nq > X->ncol) fail(SDG_E_ARG, "invalid query column range");
    std::memset(c->stats, 0, sizeof c->stats);
    DevBuf hi, hv;
    knn_device(c, const_cast<sdg_matrix*>(X), const_cast<sdg_matrix*>(Y), method, dist, k,
               include_self, drop_degenerate, false, 0, device_out ? idx : nullptr,
               device_out ? dist_out : nullptr, k_eff, flags, &hi, &hv, q0, q0 + nq);
    if (!device_out) {
      const size_t cnt = (size_t)nq * (size_t)*k_eff;
      CK(cudaMemcpyAsync(idx, hi.p, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, c->stream));
      CK(cudaMemcpyAsync(dist_out, hv.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
    }
  });
}

SDG_API int sdg_knn_cross(sdg_ctx* c, const sdg_csc* X, const sdg_csc* Y, int method, int dist,
                          int k, int drop_degenerate, int block_size, int ncores,
                          int32_t* fwd_idx, double* fwd_dist, int32_t* rev_idx, double* rev_dist,
                          int* k_fwd, int* k_rev, int* flags) {
  return guarded([&] {
    if (!c || !fwd_idx || !fwd_dist || !rev_idx || !rev_dist || !k_fwd || !k_rev || !flags)
      fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    *flags = 0;
    if (!Y)
      fail(SDG_E_ARG, "'Y' is required. For a single matrix use sparseKNN(), which already "
                      "exploits symmetry via the full/diag arguments.");
    check_counts(k, block_size, ncores);
    check_method(method, dist);
    check_csc_host(X, "X");
    check_csc_host(Y, "Y");
    if (X->nrow != Y->nrow) fail(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
    if (X->ncol < 1) fail(SDG_E_ARG, "'X' must have at least one column.");
    if (Y->ncol < 1) fail(SDG_E_ARG, "'Y' must have at least one column.");
    begin_stats(c);
    auto xm = upload(c, X, "X");
    auto ym = upload(c, Y, "Y");
    // Both clamps are decided before any work (R/sparseKNNCross.R:117-127).
    ensure_empty(xm.get());
    ensure_empty(ym.get());
    const int64_t av_f = drop_degenerate ? ym->ncol - ym->n_empty : ym->ncol;
    const int64_t av_r = drop_degenerate ? xm->ncol - xm->n_empty : xm->ncol;
    if (av_f < 1) fail(SDG_E_NOCAND, "No candidate neighbours available for the forward direction.");
    if (av_r < 1) fail(SDG_E_NOCAND, "No candidate neighbours available for the reverse direction.");
    // forward == sparseKNN(X, Y); reverse == sparseKNN(Y, X): every kernel is
    // bit-for-bit symmetric in its two columns (R/sparseKNNCross.R:33-40).
    DevBuf fi, fv, ri, rv;
    knn_device(c, xm.get(), ym.get(), method, dist, k, 0, drop_degenerate, true, 0, nullptr,
               nullptr, k_fwd, flags, &fi, &fv);
    knn_device(c, ym.get(), xm.get(), method, dist, k, 0, drop_degenerate, true, 1, nullptr,
               nullptr, k_rev, flags, &ri, &rv);
    const size_t cf = (size_t)xm->ncol * (size_t)*k_fwd, cr = (size_t)ym->ncol * (size_t)*k_rev;
    CK(cudaMemcpyAsync(fwd_idx, fi.p, sizeof(int32_t) * cf, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(fwd_dist, fv.p, sizeof(double) * cf, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(rev_idx, ri.p, sizeof(int32_t) * cr, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(rev_dist, rv.p, sizeof(double) * cr, cudaMemcpyDeviceToHost, c->stream));
    end_stats(c);
  });
}

SDG_API int sdg_matrix_upload(sdg_ctx* c, const sdg_csc* M, sdg_matrix** out) {
  return guarded([&] {
    if (!c || !out) fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    auto m = upload(c, M, "M");
    ensure_empty(m.get());
    *out = m.release();
  });
}

SDG_API int sdg_matrix_upload_device(sdg_ctx* c, int32_t nrow, int32_t ncol, const int32_t* d_p,
                                     const int32_t* d_i, const double* d_x, sdg_matrix** out) {
  return guarded([&] {
    if (!c || !out || ncol < 0 || (ncol > 0 && !d_p)) fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    std::vector<int32_t> hp((size_t)ncol + 1, 0);
    if (ncol > 0)
      CK(cudaMemcpy(hp.data(), d_p, sizeof(int32_t) * hp.size(), cudaMemcpyDefault));
    sdg_csc M{nrow, ncol, hp.data(), d_i, d_x};
    auto m = upload(c, &M, "M");
    ensure_empty(m.get());
    *out = m.release();
  });
}

SDG_API int sdg_matrix_free(sdg_matrix* M) {
  if (!M) return SDG_OK;
  cudaSetDevice(M->ctx->device);
  cudaStream_t s = M->ctx->stream;
  cudaStreamSynchronize(s);
  for (auto& sc : M->screen) screen_cache_free(&sc, s);
  cudaStreamSynchronize(s);
  delete M;
  return SDG_OK;
}

SDG_API int sdg_knn_resident_device(sdg_ctx* c, const sdg_matrix* X, const sdg_matrix* Y,
                                    int method, int dist, int k, int include_self,
                                    int drop_degenerate, int32_t* idx, double* dist_out,
                                    int* k_eff, int* flags) {
  return guarded([&] {
    if (!c || !X || !idx || !dist_out || !k_eff || !flags) fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    *flags = 0;
    if (k < 1) fail(SDG_E_ARG, kMsgK);
    check_method(method, dist);
    if (X->ncol < 1) fail(SDG_E_ARG, "'X' must have at least one column.");
    if (Y && X->nrow != Y->nrow) fail(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
    std::memset(c->stats, 0, sizeof c->stats);
    knn_device(c, const_cast<sdg_matrix*>(X), const_cast<sdg_matrix*>(Y), method, dist, k,
               include_self, drop_degenerate, false, 0, idx, dist_out, k_eff, flags, nullptr,
               nullptr);
  });
}

SDG_API int sdg_knn_resident(sdg_ctx* c, const sdg_matrix* X, const sdg_matrix* Y, int method,
                             int dist, int k, int include_self, int drop_degenerate, int32_t* idx,
                             double* dist_out, int* k_eff, int* flags) {
  return guarded([&] {
    if (!c || !X || !idx || !dist_out || !k_eff || !flags) fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    *flags = 0;
    if (k < 1) fail(SDG_E_ARG, kMsgK);
    check_method(method, dist);
    if (X->ncol < 1) fail(SDG_E_ARG, "'X' must have at least one column.");
    if (Y && X->nrow != Y->nrow) fail(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
    begin_stats(c);
    DevBuf hi, hv;
    knn_device(c, const_cast<sdg_matrix*>(X), const_cast<sdg_matrix*>(Y), method, dist, k,
               include_self, drop_degenerate, false, 0, nullptr, nullptr, k_eff, flags, &hi, &hv);
    const size_t cnt = (size_t)X->ncol * (size_t)*k_eff;
    CK(cudaMemcpyAsync(idx, hi.p, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(dist_out, hv.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost, c->stream));
    end_stats(c);
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// batched sparseKNNCross: many independent problems, an autotuned engine per
// search direction, one persistent launch for every exact-path search
// ---------------------------------------------------------------------------
namespace {

// The features that decide an engine, bucketed on a log2 scale: searches of
// one shape class take the same engine and share the learned corrections.
struct ShapeClass {
  int method, lq, lr, ln, lk;
  bool operator<(const ShapeClass& o) const {
    return std::tie(method, lq, lr, ln, lk) < std::tie(o.method, o.lq, o.lr, o.ln, o.lk);
  }
};

int ilog2(double v) { return v < 1.0 ? 0 : (int)std::floor(std::log2(v)); }

// One search direction of one problem: nq query columns against nr reference
// columns of nrow rows.
struct SearchShape {
  int method = 0, k = 1;
  int64_t nq = 0, nr = 0, nnz_q = 0, nnz_r = 0;
  int32_t nrow = 0;
  ShapeClass cls() const {
    const double per_col = nr > 0 ? (double)nnz_r / (double)nr : 0.0;
    return ShapeClass{method, ilog2((double)nq), ilog2((double)nr), ilog2(per_col), ilog2((double)k)};
  }
};

// Engine choice per search direction.  A cost model predicts each engine's
// time from the shape (merge steps of the exact walk at the measured exact
// rate; screened stored entries and slab bytes of the FP32 screen; dense flops
// and copy bytes of the tensor screen), corrected per (shape class, engine) by
// the ratio of measured to predicted time (exponential average, learned from
// every timed search and kept for the process); an engine a class has not
// tried yet is tried once when its prediction is within 2x of the best.  The
// persistent exact launch's work-item size (merge steps per item) is tuned the
// same way over {2^20, 2^22, 2^24}.
struct Autotuner {
  std::mutex mu;
  std::map<std::pair<ShapeClass, int>, std::pair<double, int>> corr;   // (ratio, samples)
  double exact_rate = 2.0e11;            // merge steps per second, batched exact kernel
  std::map<int, std::pair<double, int>> item_rate;                      // log2 size -> (steps/s, samples)

  static double predict(int engine, const SearchShape& sh) {
    const double nq = (double)sh.nq, nr = (double)sh.nr;
    if (engine == 1) return 0.0;                                        // scaled by exact_rate
    if (engine == 2) return nq / 16.0 * (double)sh.nnz_r / 1.1e11 + nq * nr * 8.0 / 4.0e12 + 2e-3;
    const double ld = std::ceil((double)sh.nrow / 64.0) * 64.0;
    return 2.0 * ld * nq * nr / 1.9e15 + ld * (nq + nr) * 2.0 / 3.0e12 + 3e-3;
  }
  double predict_exact(const SearchShape& sh) const {
    return ((double)sh.nr * (double)sh.nnz_q + (double)sh.nq * (double)sh.nnz_r) / exact_rate;
  }
  double cost(int engine, const SearchShape& sh) {
    const double base = engine == 1 ? predict_exact(sh) : predict(engine, sh);
    auto it = corr.find({sh.cls(), engine});
    return base * (it == corr.end() ? 1.0 : it->second.first);
  }
  int choose(const SearchShape& sh, const std::vector<int>& engines) {
    std::lock_guard<std::mutex> lock(mu);
    int best = engines.front();
    double bc = cost(best, sh);
    for (int e : engines) {
      const double c = cost(e, sh);
      if (c < bc) { bc = c; best = e; }
    }
    for (int e : engines)
      if (e != best && corr.find({sh.cls(), e}) == corr.end() && cost(e, sh) <= 2.0 * bc) return e;
    return best;
  }
  void learn(int engine, const SearchShape& sh, double seconds) {
    std::lock_guard<std::mutex> lock(mu);
    const double pred = engine == 1 ? predict_exact(sh) : predict(engine, sh);
    if (!(pred > 0.0) || !(seconds > 0.0)) return;
    auto& c = corr[{sh.cls(), engine}];
    const double r = seconds / pred;
    c.first = c.second == 0 ? r : 0.7 * c.first + 0.3 * r;
    ++c.second;
  }
  int item_log2() {
    std::lock_guard<std::mutex> lock(mu);
    for (int l : {22, 20, 24})
      if (item_rate.find(l) == item_rate.end()) return l;
    int best = 22;
    double br = 0.0;
    for (auto& kv : item_rate)
      if (kv.second.first > br) { br = kv.second.first; best = kv.first; }
    return best;
  }
  void learn_exact(int l, double steps, double seconds) {
    std::lock_guard<std::mutex> lock(mu);
    if (!(steps > 0.0) || !(seconds > 0.0)) return;
    const double rate = steps / seconds;
    auto& r = item_rate[l];
    r.first = r.second == 0 ? rate : 0.7 * r.first + 0.3 * rate;
    ++r.second;
    exact_rate = 0.7 * exact_rate + 0.3 * rate;
  }
};

Autotuner& autotuner() {
  static Autotuner t;
  return t;
}

// engines that can run a search: 1 (exact) always where k fits the batched
// launch, 2 and 3 where the method and k admit the screens
std::vector<int> candidate_engines(const SearchShape& sh, bool drop) {
  (void)drop;
  std::vector<int> e;
  if (sh.k <= kBatchMaxK) e.push_back(1);
  if (screen_supported(sh.method, sh.k) && screen_fits(sh.nrow)) {
    e.push_back(2);
    const double density = (sh.nrow > 0 && sh.nr > 0) ? (double)sh.nnz_r / ((double)sh.nrow * (double)sh.nr) : 0.0;
    if (tensor_supported(sh.method) && stc_supported(sh.k) && density >= 0.005) {
      const size_t bytes = tensor_cache_bytes(sh.nrow, sh.nr) + tensor_cache_bytes(sh.nrow, sh.nq);
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && bytes <= fr / 2) e.push_back(3);
      cudaGetLastError();
    }
  }
  // no batched exact item and no screen: the problem's own search, whose
  // engine choice falls back to the exact slab (engine 2 = "run it alone")
  if (e.empty()) e.push_back(2);
  return e;
}

double elapsed_s(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  CK(cudaEventSynchronize(b));
  CK(cudaEventElapsedTime(&ms, a, b));
  return ms / 1000.0;
}

}  // namespace

extern "C" {

SDG_API int sdg_knn_cross_batch(sdg_ctx* c, int nprob, const sdg_csc* X, const sdg_csc* Y, const int* method,
                                const int* dist, const int* k, int drop_degenerate, int32_t* const* fwd_idx,
                                double* const* fwd_dist, int32_t* const* rev_idx, double* const* rev_dist,
                                int* k_fwd, int* k_rev, int* flags, int* status, int* engines,
                                double* engine_seconds) {
  return guarded([&] {
    if (engine_seconds) for (int e = 0; e < 3; ++e) engine_seconds[e] = 0.0;
    if (!c || nprob < 0 || (nprob > 0 && (!X || !Y || !method || !dist || !k || !fwd_idx || !fwd_dist ||
                                          !rev_idx || !rev_dist || !k_fwd || !k_rev || !flags || !status)))
      fail(SDG_E_ARG, "NULL argument");
    CK(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    // per-problem validation on the host, in the reference's order
    // (R/sparseKNNCross.R:44-127); a failing problem keeps its own status
    std::string first_err;
    int first_code = SDG_OK;
    auto record = [&](int p, int code) {
      status[p] = code;
      if (code != SDG_OK && first_code == SDG_OK) { first_code = code; first_err.assign(g_err.data(), g_err.size()); }
    };
    std::vector<int> ok_probs;
    for (int p = 0; p < nprob; ++p) {
      flags[p] = 0; k_fwd[p] = 0; k_rev[p] = 0;
      if (engines) engines[2 * p] = engines[2 * p + 1] = 0;
      record(p, guarded([&] {
        check_counts(k[p], 1, 0);
        check_method(method[p], dist[p]);
        check_csc_host(&X[p], "X");
        check_csc_host(&Y[p], "Y");
        if (X[p].nrow != Y[p].nrow) fail(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
        if (X[p].ncol < 1) fail(SDG_E_ARG, "'X' must have at least one column.");
        if (Y[p].ncol < 1) fail(SDG_E_ARG, "'Y' must have at least one column.");
      }));
      if (status[p] == SDG_OK) ok_probs.push_back(p);
    }
    // waves of problems within a device-memory budget
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    const int64_t budget = std::max<int64_t>((int64_t)1 << 30, std::min<int64_t>((int64_t)fr / 2, (int64_t)64 << 30));
    size_t w0 = 0;
    Autotuner& T = autotuner();
    while (w0 < ok_probs.size()) {
      std::vector<int> wave;
      int64_t used = 0;
      for (size_t w = w0; w < ok_probs.size(); ++w) {
        const int p = ok_probs[w];
        const int64_t nnz = (int64_t)X[p].p[X[p].ncol] + Y[p].p[Y[p].ncol];
        const int64_t need = nnz * 32 + ((int64_t)X[p].ncol + Y[p].ncol) * (16 + 12 * (int64_t)k[p]);
        if (!wave.empty() && used + need > budget) break;
        wave.push_back(p);
        used += need;
      }
      w0 += wave.size();
      struct Held {
        int p;
        std::unique_ptr<sdg_matrix> xm, ym;
        DevBuf fi, fv, ri, rv;
        int ef = 0, er = 0;
        SearchShape fs, rs;
        std::vector<uint8_t> xe, ye;
      };
      std::vector<Held> held;
      held.reserve(wave.size());
      std::vector<BatchProb> probs;
      std::vector<int> prob_of;                       // index into held of each BatchProb
      cudaEvent_t e0 = c->ev[2], e1 = c->ev[3];
      for (int p : wave) {
        Held h;
        h.p = p;
        const int st = guarded([&] {
          h.xm = upload(c, &X[p], "X");
          h.ym = upload(c, &Y[p], "Y");
          ensure_empty(h.xm.get());
          ensure_empty(h.ym.get());
          const bool drop = drop_degenerate != 0;
          const int64_t av_f = drop ? h.ym->ncol - h.ym->n_empty : h.ym->ncol;
          const int64_t av_r = drop ? h.xm->ncol - h.xm->n_empty : h.xm->ncol;
          if (av_f < 1) fail(SDG_E_NOCAND, "No candidate neighbours available for the forward direction.");
          if (av_r < 1) fail(SDG_E_NOCAND, "No candidate neighbours available for the reverse direction.");
          prepare(method[p], h.ym.get(), h.xm.get());
          int kf = k[p], kr = k[p];
          if (kf > av_f) { kf = (int)av_f; flags[p] |= SDG_WARN_CLAMP_FWD; }
          if (kr > av_r) { kr = (int)av_r; flags[p] |= SDG_WARN_CLAMP_REV; }
          k_fwd[p] = kf; k_rev[p] = kr;
          const int64_t nx = h.xm->ncol, ny = h.ym->ncol;
          h.fs = SearchShape{method[p], kf, nx, ny, h.xm->nnz, h.ym->nnz, h.xm->nrow};
          h.rs = SearchShape{method[p], kr, ny, nx, h.ym->nnz, h.xm->nnz, h.xm->nrow};
          h.ef = T.choose(h.fs, candidate_engines(h.fs, drop));
          h.er = T.choose(h.rs, candidate_engines(h.rs, drop));
          if (engines) { engines[2 * p] = h.ef; engines[2 * p + 1] = h.er; }
          h.fi = DevBuf(sizeof(int32_t) * (size_t)(nx * kf), s);
          h.fv = DevBuf(sizeof(double) * (size_t)(nx * kf), s);
          h.ri = DevBuf(sizeof(int32_t) * (size_t)(ny * kr), s);
          h.rv = DevBuf(sizeof(double) * (size_t)(ny * kr), s);
          // the screened searches run now, one at a time (each fills the GPU)
          const int saved = c->engine;
          for (int dir = 0; dir < 2; ++dir) {
            const int eng = dir == 0 ? h.ef : h.er;
            if (eng == 1) continue;
            c->engine = eng;
            int ke = 0, fl = 0;
            DevBuf hi_, hv_;
            CK(cudaEventRecord(e0, s));
            if (dir == 0)
              knn_device(c, h.xm.get(), h.ym.get(), method[p], dist[p], k[p], 0, drop_degenerate, true, 0,
                         h.fi.as<int32_t>(), h.fv.as<double>(), &ke, &fl, &hi_, &hv_);
            else
              knn_device(c, h.ym.get(), h.xm.get(), method[p], dist[p], k[p], 0, drop_degenerate, true, 1,
                         h.ri.as<int32_t>(), h.rv.as<double>(), &ke, &fl, &hi_, &hv_);
            CK(cudaEventRecord(e1, s));
            c->engine = saved;
            const double secs = elapsed_s(e0, e1);
            T.learn(eng, dir == 0 ? h.fs : h.rs, secs);
            if (engine_seconds) engine_seconds[eng - 1] += secs;
          }
          if (h.ef == 1 || h.er == 1) {
            h.xe.resize((size_t)nx);
            h.ye.resize((size_t)ny);
            CK(cudaMemcpyAsync(h.xe.data(), h.xm->empty.p, (size_t)nx, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(h.ye.data(), h.ym->empty.p, (size_t)ny, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            BatchProb b;
            b.X = h.xm->dev(); b.Y = h.ym->dev();
            b.xa = aux_of(h.xm.get()); b.ya = aux_of(h.ym.get());
            b.method = method[p]; b.dist = dist[p]; b.decreasing = decreasing_for(method[p], dist[p]) ? 1 : 0;
            b.kf = kf; b.kr = kr;
            b.xmask = drop ? h.xm->empty.as<uint8_t>() : nullptr;
            b.ymask = drop ? h.ym->empty.as<uint8_t>() : nullptr;
            b.fidx = h.fi.as<int32_t>(); b.fval = h.fv.as<double>();
            b.ridx = h.ri.as<int32_t>(); b.rval = h.rv.as<double>();
            probs.push_back(b);
            prob_of.push_back((int)held.size());
          }
        });
        record(p, st);
        if (st == SDG_OK) held.push_back(std::move(h));
      }
      // the exact-path searches of the wave: one persistent launch
      if (!probs.empty()) {
        const int lg = T.item_log2();
        std::vector<BatchItem> items;
        std::vector<BatchRow> rows;
        double total_steps = 0.0;
        int kmax = 1, lwords = 0;
        for (size_t b = 0; b < probs.size(); ++b) {
          Held& h = held[(size_t)prob_of[b]];
          for (int dir = 0; dir < 2; ++dir) {
            if ((dir == 0 ? h.ef : h.er) != 1) continue;
            lwords = std::max(lwords, batch_lookup_words(probs[b].method, probs[b].X.nrow));
            const sdg_csc& Qc = dir == 0 ? X[h.p] : Y[h.p];
            const sdg_csc& Rc = dir == 0 ? Y[h.p] : X[h.p];
            const std::vector<uint8_t>& qe = dir == 0 ? h.xe : h.ye;
            const int kk = dir == 0 ? probs[b].kf : probs[b].kr;
            kmax = std::max(kmax, kk);
            const int64_t nnz_r = Rc.p[Rc.ncol];
            for (int32_t q = 0; q < Qc.ncol; ++q) {
              BatchRow rw;
              rw.prob = (int32_t)b; rw.dir = dir; rw.q = q; rw.nparts = 0; rw.part0 = (int64_t)items.size();
              if (!(drop_degenerate && qe[(size_t)q])) {
                const double steps = (double)Rc.ncol * (double)(Qc.p[q + 1] - Qc.p[q]) + (double)nnz_r;
                total_steps += steps;
                const int64_t parts = std::max<int64_t>(
                    1, std::min<int64_t>((Rc.ncol + 31) / 32, (int64_t)std::ceil(steps / std::ldexp(1.0, lg))));
                for (int64_t t = 0; t < parts; ++t) {
                  BatchItem it;
                  it.prob = (int32_t)b; it.dir = dir; it.q = q; it.pad = 0;
                  it.r0 = (int32_t)(Rc.ncol * t / parts);
                  it.r1 = (int32_t)(Rc.ncol * (t + 1) / parts);
                  it.part = (int64_t)items.size();
                  items.push_back(it);
                }
                rw.nparts = (int32_t)parts;
              }
              rows.push_back(rw);
            }
          }
        }
        DevBuf dp(sizeof(BatchProb) * probs.size(), s), di(sizeof(BatchItem) * std::max<size_t>(1, items.size()), s);
        DevBuf dr(sizeof(BatchRow) * rows.size(), s), dc(sizeof(unsigned long long), s);
        const size_t slots = std::max<size_t>(1, items.size()) * (size_t)kmax;
        DevBuf pk(slots * 8, s), pi(slots * 4, s), pv(slots * 8, s);
        CK(cudaMemcpyAsync(dp.p, probs.data(), sizeof(BatchProb) * probs.size(), cudaMemcpyHostToDevice, s));
        if (!items.empty())
          CK(cudaMemcpyAsync(di.p, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(dr.p, rows.data(), sizeof(BatchRow) * rows.size(), cudaMemcpyHostToDevice, s));
        CK(cudaMemsetAsync(dc.p, 0, sizeof(unsigned long long), s));
        CK(cudaEventRecord(e0, s));
        launch_batch_exact(dp.as<BatchProb>(), di.as<BatchItem>(), (int64_t)items.size(), dc.as<unsigned long long>(),
                           kmax, lwords, pk.as<uint64_t>(), pi.as<int32_t>(), pv.as<double>(), sms, s);
        CK(cudaEventRecord(e1, s));
        launch_batch_merge(dp.as<BatchProb>(), dr.as<BatchRow>(), (int64_t)rows.size(), kmax, pk.as<uint64_t>(),
                           pi.as<int32_t>(), pv.as<double>(), s);
        CK(cudaGetLastError());
        const double secs = elapsed_s(e0, e1);
        T.learn_exact(lg, total_steps, secs);
        if (engine_seconds) engine_seconds[0] += secs;
        c->stats[1] += (int64_t)total_steps;
        c->stats[3] += 2;
      }
      // results to the caller's host buffers
      for (Held& h : held) {
        const int p = h.p;
        const size_t cf = (size_t)h.xm->ncol * (size_t)k_fwd[p], cr = (size_t)h.ym->ncol * (size_t)k_rev[p];
        CK(cudaMemcpyAsync(fwd_idx[p], h.fi.p, sizeof(int32_t) * cf, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(fwd_dist[p], h.fv.p, sizeof(double) * cf, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(rev_idx[p], h.ri.p, sizeof(int32_t) * cr, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(rev_dist[p], h.rv.p, sizeof(double) * cr, cudaMemcpyDeviceToHost, s));
      }
      CK(cudaStreamSynchronize(s));
    }
    if (first_code != SDG_OK) fail(first_code, first_err);
  });
}

}  // extern "C"

// ===========================================================================
// Serving: a resident reference, continuous batching, memory-budget admission
// ===========================================================================
//
// Requests (query matrices of any column count, method, dist and k) are
// admitted while a slot is free and their device-memory estimate fits the
// budget; admitted requests that share (method, dist, drop_degenerate) are
// packed column-wise into one query matrix and searched in one pass of the
// engine at the largest k among them (the top-k at k_max, cut to each
// request's k, IS its top-k under the reference's total order).  Several
// worker threads, each with its own context and stream, run batches
// concurrently, so a request that arrives while others run is admitted and
// packed into the next batch as soon as memory and a slot free up.  Every
// query column's result depends only on that column and the reference, so a
// request's result is the same alone and in any mix.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int64_t id = 0;
  int method = 0, dist = 1, k = 1, drop = 1;
  int32_t nrow = 0, ncol = 0;
  std::vector<int32_t> p, i;
  std::vector<double> x;
  std::vector<float> q;           // dense queries: nrow x ncol FP32, column-major
  std::vector<int32_t> idx;
  std::vector<double> val;
  int k_eff = 0, flags = 0, status = SDG_OK;
  std::string err;
  int64_t mem = 0;
  double t_submit = 0, t_start = 0, t_done = 0;
  enum State { PENDING, ADMITTED, RUNNING, DONE, CANCELLED } state = PENDING;
};

}  // namespace

struct sdg_server {
  sdg_matrix* ref = nullptr;
  const sdg_dense* dref = nullptr;        // a dense reference instead (sdg_server_create_dense)
  int device = 0;
  int64_t budget = 0, in_use = 0;
  int max_slots = 1, active = 0;
  int64_t max_batch_cols = 8192;
  // methods whose reference-side data sdg_server_create prepared (bit m for
  // method m): the workers only read the shared reference, so submit refuses
  // any other method rather than let two workers prepare it concurrently
  uint32_t methods_ready = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> pending, admitted;
  std::unordered_map<int64_t, std::unique_ptr<Request>> reqs;
  int64_t next_id = 1;
  bool stop = false;
  std::vector<std::thread> workers;
  std::vector<sdg_ctx*> ctxs;
  std::vector<double> latencies;          // completed requests, seconds
  int64_t done_cols = 0, batches = 0;
  double t_first = 0, t_last = 0;
};

namespace {

// Device memory a request needs while it runs: its query CSC, its share of
// the FP32 screen slab (capped by the engine's per-pass slab), the candidate
// table and exact values, and the result buffers; where the reference holds
// the method's tensor-screen copy, the query block's own FP16 copy too (the
// tensor screen builds one for the queries: ld x ncol halves plus per-column
// bounds).
int64_t request_mem(const sdg_server* S, int method, int64_t ncol, int64_t nnz, int k) {
  if (S->dref) return dense_query_bytes(S->dref, ncol, k);
  const int64_t nr = S->ref->ncol;
  const int64_t slab_cols = std::min<int64_t>(ncol, std::max<int64_t>(16, ((int64_t)4 << 30) / (4 * std::max<int64_t>(nr, 1))));
  const int64_t cap = std::max(256, std::min(8192, 16 * k + 64));
  int64_t bytes = nnz * 12 + (ncol + 1) * 8 + slab_cols * nr * 4 + ncol * cap * 24 + ncol * (int64_t)k * 12;
  constexpr int kTensorSlots = (int)(sizeof(sdg_matrix::tensor) / sizeof(sdg_matrix::tensor[0]));
  if (method >= 0 && method < kTensorSlots && S->ref->tensor[method].method == method &&
      S->ref->tensor[method].usable)
    bytes += (int64_t)tensor_cache_bytes(S->ref->nrow, ncol);
  return bytes;
}

void admit_locked(sdg_server* S) {
  while (!S->pending.empty()) {
    Request* r = S->pending.front();
    if (r->state == Request::CANCELLED) { S->pending.pop_front(); continue; }
    if (S->active >= S->max_slots) break;
    if (S->in_use + r->mem > S->budget && S->active > 0) break;   // always admit one
    S->pending.pop_front();
    r->state = Request::ADMITTED;
    S->in_use += r->mem;
    ++S->active;
    S->admitted.push_back(r);
  }
}

// Copies the packed result (ncol_total x k_eff, column-major) into each
// request's own ncol x min(k, k_eff) matrix.
void split_results(std::vector<Request*>& batch, int64_t ncol_total, int k_eff, const std::vector<int32_t>& idx,
                   const std::vector<double>& val) {
  int64_t col0 = 0;
  for (Request* r : batch) {
    const int ke = std::min(r->k, k_eff);
    r->k_eff = ke;
    r->flags = (r->k > ke) ? SDG_WARN_CLAMP_FWD : 0;
    r->idx.resize((size_t)r->ncol * ke);
    r->val.resize((size_t)r->ncol * ke);
    for (int t = 0; t < ke; ++t)
      for (int32_t j = 0; j < r->ncol; ++j) {
        r->idx[(size_t)t * r->ncol + j] = idx[(size_t)t * ncol_total + col0 + j];
        r->val[(size_t)t * r->ncol + j] = val[(size_t)t * ncol_total + col0 + j];
      }
    col0 += r->ncol;
  }
}

void finish_batch(sdg_server* S, std::vector<Request*>& batch, int st);

// A batch against a dense reference: the requests' query columns packed into
// one d x ncol FP32 matrix, one fused tensor-core search at the largest k.
void run_dense_batch(sdg_server* S, sdg_ctx* c, std::vector<Request*>& batch) {
  const int32_t d = dense_rows(S->dref);
  std::vector<float> q;
  int64_t ncol = 0;
  int kmax = 1;
  for (Request* r : batch) {
    q.insert(q.end(), r->q.begin(), r->q.end());
    ncol += r->ncol;
    kmax = std::max(kmax, r->k);
  }
  const int st = guarded([&] {
    std::vector<int32_t> idx((size_t)ncol * kmax);
    std::vector<double> val((size_t)ncol * kmax);
    int k_eff = 0, flags = 0;
    const int rc = dense_query(c, S->dref, q.data(), d, ncol, batch.front()->method, kmax, 0, idx.data(),
                               val.data(), 0, &k_eff, &flags);
    if (rc != SDG_OK) throw Fail{rc};
    split_results(batch, ncol, k_eff, idx, val);
  });
  finish_batch(S, batch, st);
}

void run_batch(sdg_server* S, sdg_ctx* c, std::vector<Request*>& batch) {
  if (S->dref) {
    run_dense_batch(S, c, batch);
    return;
  }
  // pack the requests' columns into one dgCMatrix
  sdg_csc Q;
  std::vector<int32_t> p(1, 0), i;
  std::vector<double> x;
  int kmax = 1;
  for (Request* r : batch) {
    const int32_t base = p.back();
    for (int32_t j = 0; j < r->ncol; ++j) p.push_back(base + r->p[j + 1]);
    i.insert(i.end(), r->i.begin(), r->i.end());
    x.insert(x.end(), r->x.begin(), r->x.end());
    kmax = std::max(kmax, r->k);
  }
  Q.nrow = S->ref->nrow;
  Q.ncol = (int32_t)(p.size() - 1);
  Q.p = p.data(); Q.i = i.data(); Q.x = x.data();
  const Request* r0 = batch.front();
  int st = guarded([&] {
    auto qm = upload(c, &Q, "X");
    DevBuf hi, hv;
    int k_eff = 0, flags = 0;
    knn_device(c, qm.get(), S->ref, r0->method, r0->dist, kmax, 0, r0->drop, false, 0, nullptr,
               nullptr, &k_eff, &flags, &hi, &hv);
    std::vector<int32_t> idx((size_t)Q.ncol * k_eff);
    std::vector<double> val((size_t)Q.ncol * k_eff);
    CK(cudaMemcpyAsync(idx.data(), hi.p, sizeof(int32_t) * idx.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(val.data(), hv.p, sizeof(double) * val.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // k_eff here is min(kmax, available); each request keeps min(k, available)
    split_results(batch, Q.ncol, k_eff, idx, val);
  });
  finish_batch(S, batch, st);
}

void finish_batch(sdg_server* S, std::vector<Request*>& batch, int st) {
  const std::string err = st == SDG_OK ? std::string() : std::string(g_err.data(), g_err.size());
  const double t = now_s();
  std::lock_guard<std::mutex> lock(S->mu);
  for (Request* r : batch) {
    r->status = st;
    r->err = err;
    r->t_done = t;
    r->state = Request::DONE;
    S->in_use -= r->mem;
    --S->active;
    S->latencies.push_back(r->t_done - r->t_submit);
    S->done_cols += r->ncol;
  }
  ++S->batches;
  S->t_last = t;
  admit_locked(S);
  S->cv_done.notify_all();
  S->cv_work.notify_all();
}

void worker_main(sdg_server* S, sdg_ctx* c) {
  cudaSetDevice(S->device);
  for (;;) {
    std::vector<Request*> batch;
    {
      std::unique_lock<std::mutex> lock(S->mu);
      S->cv_work.wait(lock, [&] { return S->stop || !S->admitted.empty(); });
      if (S->stop && S->admitted.empty()) return;
      // the oldest admitted request decides the group; take every admitted
      // request of that group, oldest first, up to the batch column limit
      Request* head = S->admitted.front();
      int64_t cols = 0, nnz = 0;
      for (auto it = S->admitted.begin(); it != S->admitted.end();) {
        Request* r = *it;
        if (r->state == Request::CANCELLED) { it = S->admitted.erase(it); continue; }
        const bool same = r->method == head->method && r->dist == head->dist && r->drop == head->drop;
        // the packed query is a dgCMatrix: int32 column pointers
        const int64_t rn = (int64_t)r->i.size();
        if (same && (batch.empty() || (cols + r->ncol <= S->max_batch_cols && nnz + rn <= INT32_MAX))) {
          batch.push_back(r);
          cols += r->ncol;
          nnz += rn;
          r->state = Request::RUNNING;
          r->t_start = now_s();
          it = S->admitted.erase(it);
        } else {
          ++it;
        }
      }
    }
    if (!batch.empty()) run_batch(S, c, batch);
  }
}

}  // namespace

extern "C" {

SDG_API int sdg_server_create(sdg_ctx* ctx, const sdg_matrix* ref, int workers, int max_slots,
                              int64_t mem_budget, const int* methods, int nmethods,
                              sdg_server** out) {
  return guarded([&] {
    if (!ctx || !ref || !out || workers < 1 || max_slots < 1 || mem_budget <= 0)
      fail(SDG_E_ARG, "invalid server arguments");
    CK(cudaSetDevice(ctx->device));
    auto S = std::make_unique<sdg_server>();
    S->ref = const_cast<sdg_matrix*>(ref);
    S->device = ctx->device;
    S->budget = mem_budget;
    S->max_slots = max_slots;
    // Prepare everything the served methods read from the reference now, so
    // that the workers only ever read it: masks, unit values, screen data.
    ensure_empty(S->ref);
    const int saved_engine = ctx->engine;
    for (int t = 0; t < nmethods; ++t) {
      const int m = methods[t];
      check_method(m, 1);
      sdg_csc one;
      std::vector<int64_t> hp(2);
      CK(cudaMemcpy(hp.data(), S->ref->p.p, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost));
      std::vector<int32_t> pi = {0, (int32_t)(hp[1] - hp[0])}, ii((size_t)std::max<int64_t>(1, hp[1] - hp[0]));
      std::vector<double> xx(ii.size(), 1.0);
      if (hp[1] > hp[0]) {
        CK(cudaMemcpy(ii.data(), S->ref->i.as<int32_t>() + hp[0], sizeof(int32_t) * (hp[1] - hp[0]), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(xx.data(), S->ref->x.as<double>() + hp[0], sizeof(double) * (hp[1] - hp[0]), cudaMemcpyDeviceToHost));
      }
      one.nrow = S->ref->nrow; one.ncol = 1; one.p = pi.data(); one.i = ii.data(); one.x = xx.data();
      auto q = upload(ctx, &one, "X");
      DevBuf hi, hv;
      int ke = 0, fl = 0;
      ctx->engine = screen_supported(m, 1) ? 2 : 1;
      knn_device(ctx, q.get(), S->ref, m, 1, 1, 0, 1, false, 0, nullptr, nullptr, &ke, &fl, &hi, &hv);
      CK(cudaStreamSynchronize(ctx->stream));
      S->methods_ready |= 1u << m;
    }
    // The tensor-core screen's dense copy of the reference is built here too,
    // per served method that can use it while a copy fits in half the free
    // device memory (the automatic choice's test) and leaves the admission
    // budget free; workers never build one.
    if (saved_engine == 0) {
      for (int t = 0; t < nmethods; ++t) {
        const int m = methods[t];
        if (!tensor_supported(m) || !screen_fits(S->ref->nrow) || S->ref->ncol < 1) continue;
        const double density = (double)S->ref->nnz / ((double)S->ref->nrow * (double)S->ref->ncol);
        size_t fr = 0, tot = 0;
        const size_t bytes = tensor_cache_bytes(S->ref->nrow, S->ref->ncol);
        // the copy must leave the admission budget free for the requests
        if (density < 0.005 || cudaMemGetInfo(&fr, &tot) != cudaSuccess || bytes > fr / 2 ||
            (int64_t)(bytes + (size_t)mem_budget) > (int64_t)fr) {
          cudaGetLastError();
          continue;
        }
        sdg_csc one;
        std::vector<int32_t> pi = {0, 0}, ii(1, 0);
        std::vector<double> xx(1, 1.0);
        one.nrow = S->ref->nrow; one.ncol = 1; one.p = pi.data(); one.i = ii.data(); one.x = xx.data();
        auto q = upload(ctx, &one, "X");
        DevBuf hi, hv;
        int ke = 0, fl = 0;
        ctx->engine = 3;
        knn_device(ctx, q.get(), S->ref, m, 1, 1, 0, 0, false, 0, nullptr, nullptr, &ke, &fl, &hi, &hv);
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->engine = saved_engine;
      }
    }
    ctx->engine = saved_engine;
    for (int w = 0; w < workers; ++w) {
      sdg_ctx* c = nullptr;
      const int st = sdg_ctx_create(S->device, &c);
      if (st != SDG_OK) fail(st, std::string(g_err.data(), g_err.size()));
      c->engine = saved_engine;
      c->tensor_lazy = false;
      S->ctxs.push_back(c);
    }
    S->t_first = now_s();
    sdg_server* raw = S.get();
    for (sdg_ctx* c : S->ctxs) S->workers.emplace_back(worker_main, raw, c);
    *out = S.release();
  });
}

SDG_API int sdg_server_create_dense(sdg_ctx* ctx, const sdg_dense* ref, int workers, int max_slots,
                                    int64_t mem_budget, sdg_server** out) {
  return guarded([&] {
    if (!ctx || !ref || !out || workers < 1 || max_slots < 1 || mem_budget <= 0)
      fail(SDG_E_ARG, "invalid server arguments");
    CK(cudaSetDevice(ctx->device));
    auto S = std::make_unique<sdg_server>();
    S->dref = ref;
    S->device = ctx->device;
    S->budget = mem_budget;
    S->max_slots = max_slots;
    // a dense reference holds every form both methods read (sdg_dense_upload)
    S->methods_ready = (1u << COSINE) | (1u << EUCLIDEAN);
    for (int w = 0; w < workers; ++w) {
      sdg_ctx* c = nullptr;
      const int st = sdg_ctx_create(S->device, &c);
      if (st != SDG_OK) fail(st, std::string(g_err.data(), g_err.size()));
      S->ctxs.push_back(c);
    }
    S->t_first = now_s();
    sdg_server* raw = S.get();
    for (sdg_ctx* c : S->ctxs) S->workers.emplace_back(worker_main, raw, c);
    *out = S.release();
  });
}

SDG_API int sdg_server_submit_dense(sdg_server* S, const float* Q, int32_t d, int32_t nq, int method, int k,
                                    int64_t* id) {
  return guarded([&] {
    if (!S || !id || !Q) fail(SDG_E_ARG, "NULL argument");
    if (!S->dref) fail(SDG_E_ARG, "the server's reference is sparse: submit a dgCMatrix (sdg_server_submit)");
    if (k < 1) fail(SDG_E_ARG, kMsgK);
    check_method(method, 1);
    if (!(S->methods_ready & (1u << method))) fail(SDG_E_UNSUPPORTED, "dense kNN supports cosine and euclidean");
    if (nq < 1) fail(SDG_E_ARG, "'X' must have at least one column.");
    if (d != dense_rows(S->dref)) fail(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
    auto r = std::make_unique<Request>();
    r->method = method; r->dist = 1; r->k = k; r->drop = 1;
    r->nrow = d; r->ncol = nq;
    r->q.assign(Q, Q + (size_t)d * (size_t)nq);
    r->mem = request_mem(S, method, nq, 0, k);
    r->t_submit = now_s();
    std::lock_guard<std::mutex> lock(S->mu);
    r->id = S->next_id++;
    *id = r->id;
    S->pending.push_back(r.get());
    S->reqs.emplace(r->id, std::move(r));
    admit_locked(S);
    S->cv_work.notify_all();
  });
}

SDG_API int sdg_server_submit(sdg_server* S, const sdg_csc* Q, int method, int dist, int k,
                              int drop_degenerate, int64_t* id) {
  return guarded([&] {
    if (!S || !id) fail(SDG_E_ARG, "NULL argument");
    if (S->dref) fail(SDG_E_ARG, "the server's reference is dense: submit FP32 columns (sdg_server_submit_dense)");
    if (k < 1) fail(SDG_E_ARG, kMsgK);
    check_method(method, dist);
    if (!(S->methods_ready & (1u << method)))
      fail(SDG_E_ARG, "method " + std::to_string(method) +
                          " was not prepared by sdg_server_create (pass it in `methods`).");
    check_csc_host(Q, "X");
    if (Q->ncol < 1) fail(SDG_E_ARG, "'X' must have at least one column.");
    if (Q->nrow != S->ref->nrow) fail(SDG_E_ROWS, "'X' and 'Y' must have the same number of rows.");
    auto r = std::make_unique<Request>();
    r->method = method; r->dist = dist; r->k = k; r->drop = drop_degenerate ? 1 : 0;
    r->nrow = Q->nrow; r->ncol = Q->ncol;
    r->p.assign(Q->p, Q->p + Q->ncol + 1);
    r->i.assign(Q->i, Q->i + Q->p[Q->ncol]);
    r->x.assign(Q->x, Q->x + Q->p[Q->ncol]);
    r->mem = request_mem(S, method, Q->ncol, Q->p[Q->ncol], k);
    r->t_submit = now_s();
    std::lock_guard<std::mutex> lock(S->mu);
    r->id = S->next_id++;
    *id = r->id;
    S->pending.push_back(r.get());
    S->reqs.emplace(r->id, std::move(r));
    admit_locked(S);
    S->cv_work.notify_all();
  });
}

SDG_API int sdg_server_wait(sdg_server* S, int64_t id, int timeout_ms) {
  if (!S) return SDG_E_ARG;
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) { g_err = "unknown request"; return SDG_E_ARG; }
  Request* r = it->second.get();
  auto done = [&] { return r->state == Request::DONE || r->state == Request::CANCELLED; };
  if (timeout_ms < 0) S->cv_done.wait(lock, done);
  else if (!S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), done)) return 1;
  return SDG_OK;
}

SDG_API int sdg_server_result(sdg_server* S, int64_t id, int32_t* idx, double* dist_out,
                              int* k_eff, int* flags) {
  if (!S || !k_eff || !flags) return SDG_E_ARG;
  std::unique_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) { g_err = "unknown request"; return SDG_E_ARG; }
    const auto st = it->second->state;
    if (st != Request::DONE && st != Request::CANCELLED) { g_err = "request not finished"; return SDG_E_ARG; }
    r = std::move(it->second);
    S->reqs.erase(it);
  }
  if (r->status != SDG_OK) { g_err = r->err; return r->status; }
  *k_eff = r->k_eff;
  *flags = r->flags;
  if (idx) std::memcpy(idx, r->idx.data(), sizeof(int32_t) * r->idx.size());
  if (dist_out) std::memcpy(dist_out, r->val.data(), sizeof(double) * r->val.size());
  return SDG_OK;
}

SDG_API int sdg_server_cancel(sdg_server* S, int64_t id) {
  if (!S) return SDG_E_ARG;
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) { g_err = "unknown request"; return SDG_E_ARG; }
  Request* r = it->second.get();
  if (r->state == Request::PENDING || r->state == Request::ADMITTED) {
    if (r->state == Request::ADMITTED) { S->in_use -= r->mem; --S->active; }
    // out of the queues now, so that sdg_server_result may release it
    for (auto* q : {&S->pending, &S->admitted}) q->erase(std::remove(q->begin(), q->end(), r), q->end());
    r->state = Request::CANCELLED;
    r->status = SDG_E_CANCELLED;
    r->err = "Computation interrupted by the user.";
    admit_locked(S);
    S->cv_done.notify_all();
    S->cv_work.notify_all();
    return SDG_OK;
  }
  return 1;   // already running or finished: the result will be delivered
}

// out[0] completed requests, [1] completed columns, [2] p50 latency (s),
// [3] p99 latency (s), [4] mean latency (s), [5] columns/s since creation,
// [6] batches run, [7] bytes admitted now, [8] requests waiting for admission.
SDG_API int sdg_server_stats(sdg_server* S, double* out, int n) {
  if (!S || !out) return SDG_E_ARG;
  std::lock_guard<std::mutex> lock(S->mu);
  std::vector<double> l = S->latencies;
  std::sort(l.begin(), l.end());
  auto pct = [&](double q) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
  double mean = 0;
  for (double v : l) mean += v;
  mean = l.empty() ? 0 : mean / l.size();
  const double span = std::max(1e-9, S->t_last - S->t_first);
  const double vals[9] = {(double)l.size(), (double)S->done_cols, pct(0.5), pct(0.99), mean,
                          S->done_cols / span, (double)S->batches, (double)S->in_use,
                          (double)S->pending.size()};
  for (int t = 0; t < n && t < 9; ++t) out[t] = vals[t];
  return SDG_OK;
}

SDG_API int sdg_server_destroy(sdg_server* S) {
  if (!S) return SDG_OK;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto& t : S->workers) t.join();
  for (sdg_ctx* c : S->ctxs) sdg_ctx_destroy(c);
  delete S;
  return SDG_OK;
}

}  // extern "C"
