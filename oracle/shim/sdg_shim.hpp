// sdg_shim.hpp -- a minimal, project-written stand-in for the parts of the
// Rcpp, RcppArmadillo and RcppProgress APIs that the reference's hot-path
// sources (src/sparseDist.cpp, src/topK.cpp, src/topKRows.cpp, src/snn.cpp)
// use, so that those files compile unmodified with g++ into oracle/_ref/.
//
// TEST INFRASTRUCTURE ONLY.  It implements the API surface, not the libraries:
// storage is plain std::vector, errors are C++ exceptions, and there is no R.
// The arithmetic of the reference's own loops is untouched.  Where a
// reference kernel delegates arithmetic to Armadillo (arma::cor for pearson,
// arma::accu for js), the shim implements the same formulation as the oracle's
// restatement (oracle/sdg_oracle.c), so those two methods stay "parity
// unpinned" with respect to the real Armadillo.
#ifndef SDG_SHIM_HPP
#define SDG_SHIM_HPP

#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

// ---------------------------------------------------------------------------
// SEXP: a type-erased, reference-counted R object
// ---------------------------------------------------------------------------
struct SdgRObject { virtual ~SdgRObject() {} };
template <typename T> struct SdgRBox : SdgRObject { T value; explicit SdgRBox(const T& v) : value(v) {} };
typedef std::shared_ptr<SdgRObject> SEXP;

inline double sdg_shim_na_real() {
  const uint64_t bits = 0x7FF00000000007A2ULL;
  double d;
  std::memcpy(&d, &bits, sizeof d);
  return d;
}
#define NA_INTEGER (INT_MIN)
#define NA_REAL (sdg_shim_na_real())

// ---------------------------------------------------------------------------
// RcppProgress
// ---------------------------------------------------------------------------
class Progress {
 public:
  Progress(unsigned long, bool = true) {}
  void increment(unsigned long = 1) {}
  static bool check_abort() { return false; }
  bool is_aborted() const { return false; }
};

// ---------------------------------------------------------------------------
// Armadillo subset
// ---------------------------------------------------------------------------
namespace arma {

#ifdef ARMA_64BIT_WORD
typedef unsigned long long uword;
#else
typedef unsigned int uword;
#endif

namespace fill { struct fill_zeros_t {}; static const fill_zeros_t zeros = {}; }
namespace datum { static const double nan = std::numeric_limits<double>::quiet_NaN(); }

class SpMat;
class Col;

struct DiagView {
  double* base; uword n_rows, n;
  void ones() { for (uword k = 0; k < n; ++k) base[k * n_rows + k] = 1.0; }
};

class Mat {
 public:
  uword n_rows = 0, n_cols = 0, n_elem = 0;
  std::vector<double> mem;
  Mat() {}
  Mat(uword r, uword c) : n_rows(r), n_cols(c), n_elem(r * c), mem(r * c, 0.0) {}
  Mat(uword r, uword c, fill::fill_zeros_t) : Mat(r, c) {}
  Mat(const double* src, uword r, uword c) : n_rows(r), n_cols(c), n_elem(r * c), mem(src, src + r * c) {}
  double& operator()(uword i, uword j) { return mem[j * n_rows + i]; }
  double operator()(uword i, uword j) const { return mem[j * n_rows + i]; }
  double& operator[](uword k) { return mem[k]; }
  double operator[](uword k) const { return mem[k]; }
  double* colptr(uword j) { return mem.data() + j * n_rows; }
  const double* colptr(uword j) const { return mem.data() + j * n_rows; }
  const double* memptr() const { return mem.data(); }
  DiagView diag() { return DiagView{mem.data(), n_rows, n_rows < n_cols ? n_rows : n_cols}; }
  bool is_empty() const { return n_elem == 0; }
  bool is_finite() const { for (double v : mem) if (!std::isfinite(v)) return false; return true; }
  double min() const {
    if (mem.empty()) throw std::logic_error("min(): object has no elements");
    double m = mem[0];
    for (double v : mem) if (v < m) m = v;
    return m;
  }
  inline Col col(uword j) const;
};

typedef Mat mat;

class Col : public Mat {
 public:
  Col() {}
  explicit Col(uword n) : Mat(n, 1) {}
  Col(const Mat& m) : Mat(m) {}
  inline Col(const struct SpCol& c);
  Col& replace(double old_val, double new_val) {
    const bool nan_old = std::isnan(old_val);
    for (double& v : mem) if (nan_old ? std::isnan(v) : (v == old_val)) v = new_val;
    return *this;
  }
};
typedef Col vec;

inline Col Mat::col(uword j) const {
  Col c(n_rows);
  for (uword i = 0; i < n_rows; ++i) c.mem[i] = mem[j * n_rows + i];
  return c;
}

// Element-wise operators, evaluated eagerly.  Each element sees the same
// sequence of IEEE operations as Armadillo's delayed evaluation of the same
// expression tree, so the results are identical element by element.
#define SDG_EW(OP)                                                          \
  inline Col operator OP(const Col& a, const Col& b) {                      \
    Col r(a.n_elem);                                                        \
    for (uword k = 0; k < a.n_elem; ++k) r.mem[k] = a.mem[k] OP b.mem[k];   \
    return r;                                                               \
  }
SDG_EW(+)
SDG_EW(-)
#undef SDG_EW
inline Col operator%(const Col& a, const Col& b) {
  Col r(a.n_elem);
  for (uword k = 0; k < a.n_elem; ++k) r.mem[k] = a.mem[k] * b.mem[k];
  return r;
}
inline Col operator*(const Col& a, double s) {
  Col r(a.n_elem);
  for (uword k = 0; k < a.n_elem; ++k) r.mem[k] = a.mem[k] * s;
  return r;
}
inline Col log(const Col& a) {
  Col r(a.n_elem);
  for (uword k = 0; k < a.n_elem; ++k) r.mem[k] = std::log(a.mem[k]);
  return r;
}

// accu: two interleaved accumulators, even then odd elements (the
// formulation the oracle states for arma::accu).
inline double accu(const Mat& X) {
  const double* s = X.mem.data();
  const uword n = X.n_elem;
  double acc1 = 0.0, acc2 = 0.0;
  uword i, j;
  for (i = 0, j = 1; j < n; i += 2, j += 2) { acc1 += s[i]; acc2 += s[j]; }
  if (i < n) acc1 += s[i];
  return acc1 + acc2;
}

inline double as_scalar(const Mat& m) { return m.mem.at(0); }

// cor / cov of two vectors: the single-pass form the oracle states
// (sequential sums in element order).
inline Mat cor(const Col& A, const Col& B, uword norm_type = 0) {
  const uword N = A.n_elem;
  double sa = 0.0, sb = 0.0, saa = 0.0, sbb = 0.0, sab = 0.0;
  for (uword k = 0; k < N; ++k) {
    const double a = A.mem[k], b = B.mem[k];
    sa += a; saa += a * a; sb += b; sbb += b * b; sab += a * b;
  }
  const double Nd = (double)N;
  const double norm = (norm_type == 0) ? ((N > 1) ? (Nd - 1.0) : 1.0) : Nd;
  const double cov = (sab - (sa * sb) / Nd) / norm;
  const double va = (saa - (sa * sa) / Nd) / norm;
  const double vb = (sbb - (sb * sb) / Nd) / norm;
  Mat r(1, 1);
  r.mem[0] = cov / (std::sqrt(va) * std::sqrt(vb));
  return r;
}
inline Mat cov(const Col& A, const Col& B, uword norm_type = 0) {
  const uword N = A.n_elem;
  double sa = 0.0, sb = 0.0, sab = 0.0;
  for (uword k = 0; k < N; ++k) { sa += A.mem[k]; sb += B.mem[k]; sab += A.mem[k] * B.mem[k]; }
  const double Nd = (double)N;
  const double norm = (norm_type == 0) ? ((N > 1) ? (Nd - 1.0) : 1.0) : Nd;
  Mat r(1, 1);
  r.mem[0] = (sab - (sa * sb) / Nd) / norm;
  return r;
}

struct SpCol { const SpMat* m; uword j; };

class SpMat {
 public:
  uword n_rows = 0, n_cols = 0, n_nonzero = 0;
  std::vector<uword> rows_v, cptr_v;
  std::vector<double> vals_v;
  const uword* row_indices = nullptr;
  const uword* col_ptrs = nullptr;
  const double* values = nullptr;

  SpMat() { relink(); }
  SpMat(const SpMat& o) : n_rows(o.n_rows), n_cols(o.n_cols), n_nonzero(o.n_nonzero),
                          rows_v(o.rows_v), cptr_v(o.cptr_v), vals_v(o.vals_v) { relink(); }
  SpMat& operator=(const SpMat& o) {
    n_rows = o.n_rows; n_cols = o.n_cols; n_nonzero = o.n_nonzero;
    rows_v = o.rows_v; cptr_v = o.cptr_v; vals_v = o.vals_v; relink(); return *this;
  }
  // From dgCMatrix slots (int32 p/i, double x): copied, explicit zeros kept,
  // as RcppArmadillo's conversion of a dgCMatrix does.
  SpMat(int32_t nrow, int32_t ncol, const int32_t* p, const int32_t* i, const double* x)
      : n_rows((uword)nrow), n_cols((uword)ncol) {
    const int64_t base = p[0];
    n_nonzero = (uword)(p[ncol] - base);
    cptr_v.resize((size_t)ncol + 1);
    for (int32_t c = 0; c <= ncol; ++c) cptr_v[c] = (uword)(p[c] - base);
    rows_v.resize(n_nonzero + 1);
    vals_v.resize(n_nonzero + 1);
    for (uword a = 0; a < n_nonzero; ++a) { rows_v[a] = (uword)i[base + a]; vals_v[a] = x[base + a]; }
    relink();
  }
  explicit SpMat(const Mat& d) : n_rows(d.n_rows), n_cols(d.n_cols) {
    cptr_v.assign(n_cols + 1, 0);
    for (uword c = 0; c < n_cols; ++c) {
      for (uword r = 0; r < n_rows; ++r) {
        const double v = d(r, c);
        if (v != 0.0) { rows_v.push_back(r); vals_v.push_back(v); }
      }
      cptr_v[c + 1] = rows_v.size();
    }
    n_nonzero = rows_v.size();
    rows_v.push_back(0); vals_v.push_back(0.0);
    relink();
  }
  void relink() {
    if (cptr_v.empty()) cptr_v.assign(n_cols + 1, 0);
    if (rows_v.empty()) rows_v.push_back(0);
    if (vals_v.empty()) vals_v.push_back(0.0);
    row_indices = rows_v.data(); col_ptrs = cptr_v.data(); values = vals_v.data();
  }
  void sync() const {}

  class const_col_iterator {
   public:
    const SpMat* m; uword pos;
    uword row() const { return m->row_indices[pos]; }
    double operator*() const { return m->values[pos]; }
    const_col_iterator& operator++() { ++pos; return *this; }
    bool operator!=(const const_col_iterator& o) const { return pos != o.pos; }
    bool operator==(const const_col_iterator& o) const { return pos == o.pos; }
  };
  const_col_iterator begin_col(uword j) const { return const_col_iterator{this, col_ptrs[j]}; }
  const_col_iterator end_col(uword j) const { return const_col_iterator{this, col_ptrs[j + 1]}; }
  SpCol col(uword j) const { return SpCol{this, j}; }

  Mat dense() const {
    Mat d(n_rows, n_cols);
    for (uword c = 0; c < n_cols; ++c)
      for (uword a = col_ptrs[c]; a < col_ptrs[c + 1]; ++a) d(row_indices[a], c) = values[a];
    return d;
  }
};
typedef SpMat sp_mat;

inline Col::Col(const SpCol& c) : Mat(c.m->n_rows, 1) {
  for (uword a = c.m->col_ptrs[c.j]; a < c.m->col_ptrs[c.j + 1]; ++a)
    mem[c.m->row_indices[a]] = c.m->values[a];
}

}  // namespace arma

// ---------------------------------------------------------------------------
// Rcpp subset
// ---------------------------------------------------------------------------
namespace Rcpp {

inline void stop(const std::string& msg) { throw std::runtime_error(msg); }

template <typename T>
class Matrix {
 public:
  std::shared_ptr<std::vector<T>> own;
  T* data = nullptr;
  int nr = 0, nc = 0;
  Matrix() {}
  Matrix(size_t r, size_t c)
      : own(std::make_shared<std::vector<T>>(r * c + 1, T())), data(own->data()),
        nr((int)r), nc((int)c) {}
  // A view over caller-owned storage (R's matrices are passed by reference).
  static Matrix view(T* p, int r, int c) { Matrix m; m.data = p; m.nr = r; m.nc = c; return m; }
  int nrow() const { return nr; }
  int ncol() const { return nc; }
  T& operator()(int i, int j) { return data[(size_t)j * nr + i]; }
  const T& operator()(int i, int j) const { return data[(size_t)j * nr + i]; }
  T& operator[](size_t k) { return data[k]; }
  const T& operator[](size_t k) const { return data[k]; }
  T* begin() { return data; }
  T* end() { return data + (size_t)nr * nc; }
  size_t size() const { return (size_t)nr * nc; }
};
typedef Matrix<int> IntegerMatrix;
typedef Matrix<double> NumericMatrix;

template <typename T>
class Vector {
 public:
  std::shared_ptr<std::vector<T>> own;
  T* data = nullptr;
  size_t n = 0;
  Vector() {}
  explicit Vector(size_t len)
      : own(std::make_shared<std::vector<T>>(len + 1, T())), data(own->data()), n(len) {}
  static Vector view(T* p, size_t len) { Vector v; v.data = p; v.n = len; return v; }
  size_t size() const { return n; }
  T& operator[](size_t k) { return data[k]; }
  const T& operator[](size_t k) const { return data[k]; }
  T* begin() { return data; }
  T* end() { return data + n; }
};
typedef Vector<int> IntegerVector;
typedef Vector<double> NumericVector;

template <typename T> inline SEXP wrap(const T& v) { return std::make_shared<SdgRBox<T>>(v); }

struct NamedArg { std::string name; SEXP value; };
struct Named {
  std::string name;
  explicit Named(const std::string& n) : name(n) {}
  template <typename T> NamedArg operator=(const T& v) const { return NamedArg{name, wrap(v)}; }
};

class List {
 public:
  std::vector<NamedArg> items;
  static List create(std::initializer_list<NamedArg> a) { List l; l.items.assign(a.begin(), a.end()); return l; }
  template <typename... A> static List create(const A&... a) { return create({a...}); }
  template <typename T> T get(const std::string& name) const {
    for (const NamedArg& it : items)
      if (it.name == name) {
        auto b = std::dynamic_pointer_cast<SdgRBox<T>>(it.value);
        if (!b) throw std::logic_error("shim List: type mismatch for " + name);
        return b->value;
      }
    throw std::logic_error("shim List: no element " + name);
  }
};

}  // namespace Rcpp

#define RcppExport extern "C"

#endif
