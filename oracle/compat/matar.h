// Host-only stand-in for the MATAR / Kokkos API subset that Fierro's
// Explicit-Lagrange-Kokkos/SGH_solver sources use, so those sources compile
// UNMODIFIED with g++ -fopenmp as the CPU oracle (test infrastructure only;
// nothing in the shipped library includes this file).
//
// Written from the usage surface of the SGH solver, not from MATAR (which is
// not available here).  Semantics honoured, matching Kokkos-OpenMP:
//   * every owning allocation is zero-initialised (Kokkos View semantics; the
//     SGH code relies on it, e.g. mesh.h:295 DynamicRagged stride counters,
//     setup.cpp:625 num_bdy_nodes_in_set);
//   * host and "device" alias the same memory, so update_host/update_device and
//     Kokkos::fence are no-ops;
//   * owning containers are shallow, reference-counted handles (a mesh_t passed
//     by value, momentum.cpp:222, shares its arrays);
//   * FOR_ALL is an OpenMP static-schedule loop (Kokkos RangePolicy default on
//     the OpenMP backend); short ranges (the 8-wide per-element loops at
//     mesh.h:191,219) run inline;
//   * RUN is serial; REDUCE_{SUM,MIN,MAX} are OpenMP reductions with the
//     reducer identity as the initial thread-local value.
#ifndef FIERRO_ORACLE_MATAR_COMPAT_H
#define FIERRO_ORACLE_MATAR_COMPAT_H

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <limits>
#include <memory>
#include <algorithm>

typedef double real_t;

#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline

namespace Kokkos {
inline void initialize() {}
inline void initialize(int&, char**) {}
inline void finalize() {}
inline void fence() {}
}  // namespace Kokkos

namespace matar_compat {

// Row-major index arithmetic shared by every array flavour.  Dims beyond the
// array's rank are 1, so an index tuple shorter than the rank addresses the
// leading sub-array (only reached from dead code paths of the solver).
struct Shape {
  size_t d[4] = {1, 1, 1, 1};
  size_t rank = 0;
  size_t size() const { return d[0] * d[1] * d[2] * d[3]; }
  size_t at(size_t i) const { return i; }
  size_t at(size_t i, size_t j) const { return i * d[1] + j; }
  size_t at(size_t i, size_t j, size_t k) const { return (i * d[1] + j) * d[2] + k; }
  size_t at(size_t i, size_t j, size_t k, size_t l) const {
    return ((i * d[1] + j) * d[2] + k) * d[3] + l;
  }
};

inline Shape make_shape(size_t a) { Shape s; s.d[0] = a; s.rank = 1; return s; }
inline Shape make_shape(size_t a, size_t b) { Shape s; s.d[0] = a; s.d[1] = b; s.rank = 2; return s; }
inline Shape make_shape(size_t a, size_t b, size_t c) {
  Shape s; s.d[0] = a; s.d[1] = b; s.d[2] = c; s.rank = 3; return s;
}
inline Shape make_shape(size_t a, size_t b, size_t c, size_t e) {
  Shape s; s.d[0] = a; s.d[1] = b; s.d[2] = c; s.d[3] = e; s.rank = 4; return s;
}

// Owning, zero-initialised, shallow-copy array (CArray, CArrayKokkos,
// DCArrayKokkos all map here).
template <typename T>
class OwnedArray {
 public:
  OwnedArray() = default;
  template <typename... D>
  explicit OwnedArray(D... dims) : shape_(make_shape(static_cast<size_t>(dims)...)) {
    size_t n = shape_.size();
    store_ = std::shared_ptr<T>(new T[n ? n : 1](), std::default_delete<T[]>());
    ptr_ = store_.get();
  }
  template <typename... I>
  T& operator()(I... idx) const { return ptr_[shape_.at(static_cast<size_t>(idx)...)]; }
  template <typename... I>
  T& host(I... idx) const { return ptr_[shape_.at(static_cast<size_t>(idx)...)]; }
  size_t size() const { return shape_.size(); }
  size_t extent() const { return shape_.size(); }
  size_t dims(size_t i) const { return shape_.d[i]; }
  size_t order() const { return shape_.rank; }
  T* pointer() const { return ptr_; }
  void update_host() const {}
  void update_device() const {}

 private:
  Shape shape_;
  std::shared_ptr<T> store_;
  T* ptr_ = nullptr;
};

// Non-owning view over caller memory (ViewCArrayKokkos, DViewCArrayKokkos).
template <typename T>
class View {
 public:
  View() = default;
  template <typename... D>
  View(T* p, D... dims) : shape_(make_shape(static_cast<size_t>(dims)...)), ptr_(p) {}
  template <typename... I>
  T& operator()(I... idx) const { return ptr_[shape_.at(static_cast<size_t>(idx)...)]; }
  template <typename... I>
  T& host(I... idx) const { return ptr_[shape_.at(static_cast<size_t>(idx)...)]; }
  size_t size() const { return shape_.size(); }
  size_t extent() const { return shape_.size(); }
  size_t dims(size_t i) const { return shape_.d[i]; }
  size_t order() const { return shape_.rank; }
  T* pointer() const { return ptr_; }
  void update_host() const {}
  void update_device() const {}

 private:
  Shape shape_;
  T* ptr_ = nullptr;
};

// 1-based non-owning matrix view (ViewCMatrixKokkos, user_mat.cpp:151).
template <typename T>
class MatrixView {
 public:
  MatrixView() = default;
  template <typename... D>
  MatrixView(T* p, D... dims) : shape_(make_shape(static_cast<size_t>(dims)...)), ptr_(p) {}
  template <typename... I>
  T& operator()(I... idx) const { return ptr_[shape_.at((static_cast<size_t>(idx) - 1)...)]; }
  size_t dims(size_t i) const { return shape_.d[i]; }

 private:
  Shape shape_;
  T* ptr_ = nullptr;
};

// Ragged rows whose lengths are fixed at construction from a stride array
// (RaggedRightArrayKokkos built from num_corners_in_node, mesh.h:204).
template <typename T>
class Ragged {
 public:
  Ragged() = default;
  template <typename S>
  explicit Ragged(const S& strides) {
    rows_ = strides.size();
    start_ = std::shared_ptr<size_t>(new size_t[rows_ + 1](), std::default_delete<size_t[]>());
    size_t* st = start_.get();
    for (size_t i = 0; i < rows_; ++i) st[i + 1] = st[i] + static_cast<size_t>(strides(i));
    size_t n = st[rows_];
    store_ = std::shared_ptr<T>(new T[n ? n : 1](), std::default_delete<T[]>());
  }
  T& operator()(size_t i, size_t j) const { return store_.get()[start_.get()[i] + j]; }
  size_t stride(size_t i) const { return start_.get()[i + 1] - start_.get()[i]; }

 private:
  size_t rows_ = 0;
  std::shared_ptr<size_t> start_;
  std::shared_ptr<T> store_;
};

// Rows of fixed capacity with a mutable per-row length
// (DynamicRaggedRightArrayKokkos, mesh.h:265, mesh.h:307 `.stride(i)++`).
template <typename T>
class DynamicRagged {
 public:
  DynamicRagged() = default;
  DynamicRagged(size_t rows, size_t cap) : rows_(rows), cap_(cap) {
    strides_ = std::shared_ptr<size_t>(new size_t[rows ? rows : 1](), std::default_delete<size_t[]>());
    size_t n = rows * cap;
    store_ = std::shared_ptr<T>(new T[n ? n : 1](), std::default_delete<T[]>());
  }
  T& operator()(size_t i, size_t j) const { return store_.get()[i * cap_ + j]; }
  size_t& stride(size_t i) const { return strides_.get()[i]; }

 private:
  size_t rows_ = 0, cap_ = 0;
  std::shared_ptr<size_t> strides_;
  std::shared_ptr<T> store_;
};

}  // namespace matar_compat

template <typename T> using CArray = matar_compat::OwnedArray<T>;
template <typename T> using CArrayKokkos = matar_compat::OwnedArray<T>;
template <typename T> using DCArrayKokkos = matar_compat::OwnedArray<T>;
template <typename T> using ViewCArrayKokkos = matar_compat::View<T>;
template <typename T> using DViewCArrayKokkos = matar_compat::View<T>;
template <typename T> using ViewCMatrixKokkos = matar_compat::MatrixView<T>;
template <typename T> using RaggedRightArrayKokkos = matar_compat::Ragged<T>;
template <typename T> using DynamicRaggedRightArrayKokkos = matar_compat::DynamicRagged<T>;

// Ranges shorter than this run inline instead of opening a parallel region.
#ifndef MATAR_COMPAT_PAR_MIN
#define MATAR_COMPAT_PAR_MIN 4096
#endif

#define MATAR_COMPAT_PRAGMA(x) _Pragma(#x)

#define FOR_ALL(i, x0, x1, ...)                                                        \
  do {                                                                                 \
    const long long matar_lo_ = static_cast<long long>(x0);                           \
    const long long matar_hi_ = static_cast<long long>(x1);                           \
    MATAR_COMPAT_PRAGMA(omp parallel for schedule(static) if (matar_hi_ - matar_lo_ >= MATAR_COMPAT_PAR_MIN)) \
    for (long long i = matar_lo_; i < matar_hi_; ++i) __VA_ARGS__                      \
  } while (0)

#define FOR_ALL_CLASS(i, x0, x1, ...) FOR_ALL(i, x0, x1, __VA_ARGS__)

#define RUN(...) do __VA_ARGS__ while (0)
#define RUN_CLASS(...) RUN(__VA_ARGS__)

#define MATAR_COMPAT_REDUCE(i, x0, x1, loc, body, result, ident, combine)              \
  do {                                                                                 \
    typedef decltype(result) matar_t_;                                                \
    matar_t_ matar_acc_ = (ident);                                                     \
    const long long matar_lo_ = static_cast<long long>(x0);                           \
    const long long matar_hi_ = static_cast<long long>(x1);                           \
    MATAR_COMPAT_PRAGMA(omp parallel if (matar_hi_ - matar_lo_ >= MATAR_COMPAT_PAR_MIN)) \
    {                                                                                  \
      matar_t_ loc = (ident);                                                          \
      MATAR_COMPAT_PRAGMA(omp for schedule(static))                                    \
      for (long long i = matar_lo_; i < matar_hi_; ++i) body                           \
      MATAR_COMPAT_PRAGMA(omp critical(matar_compat_reduce))                           \
      { combine; }                                                                     \
    }                                                                                  \
    result = matar_acc_;                                                               \
  } while (0)

#define REDUCE_SUM(i, x0, x1, loc, body, result) \
  MATAR_COMPAT_REDUCE(i, x0, x1, loc, body, result, matar_t_(0), matar_acc_ += loc)
#define REDUCE_MIN(i, x0, x1, loc, body, result)                                          \
  MATAR_COMPAT_REDUCE(i, x0, x1, loc, body, result, std::numeric_limits<matar_t_>::max(), \
                      if (loc < matar_acc_) matar_acc_ = loc)
#define REDUCE_MAX(i, x0, x1, loc, body, result)                                             \
  MATAR_COMPAT_REDUCE(i, x0, x1, loc, body, result, std::numeric_limits<matar_t_>::lowest(), \
                      if (loc > matar_acc_) matar_acc_ = loc)
#define REDUCE_SUM_CLASS(...) REDUCE_SUM(__VA_ARGS__)
#define REDUCE_MIN_CLASS(...) REDUCE_MIN(__VA_ARGS__)
#define REDUCE_MAX_CLASS(...) REDUCE_MAX(__VA_ARGS__)

#endif  // FIERRO_ORACLE_MATAR_COMPAT_H
