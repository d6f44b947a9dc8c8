// Stand-in for the part of the Kokkos 2.x API that the reference miniAero
// sources use, so that those sources compile unmodified into the oracle's
// reference build (test infrastructure only; nothing in the product links it).
//
// Written for this project from the documented behaviour of the calls, not
// from Kokkos itself. Two host back ends, chosen at compile time:
//   * Serial (default): every parallel_for is a loop in index order and the
//     atomics are plain read-modify-writes, which is the order the reference's
//     Kokkos Serial build runs in and the order its golden files come from.
//   * OpenMP (-DMINIAERO_SHIM_OPENMP -fopenmp): static-schedule loops and real
//     atomics, like the Kokkos OpenMP back end the reference's Makefile
//     selects (KOKKOS_DEVICES=OpenMP); results then depend on the thread count.
//
// Views are reference-counted host allocations, zero-filled on construction,
// with LayoutRight strides (a subview may carry other strides). A view whose
// label was registered with Kokkos::shim::capture() keeps its allocation alive
// after the reference code drops it, so a driver can read the solver's final
// state after Solve() returns.
#ifndef MINIAERO_KOKKOS_SHIM_CORE_HPP
#define MINIAERO_KOKKOS_SHIM_CORE_HPP

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]

namespace Kokkos {

struct HostSpace {
  typedef HostSpace memory_space;
};

struct Serial {
  typedef Serial execution_space;
  typedef HostSpace memory_space;
  typedef Serial device_type;
  typedef int size_type;
  static void fence() {}
};

struct OpenMP {
  typedef OpenMP execution_space;
  typedef HostSpace memory_space;
  typedef OpenMP device_type;
  typedef int size_type;
  static void fence() {}
};

#ifdef MINIAERO_SHIM_OPENMP
typedef OpenMP DefaultExecutionSpace;
#else
typedef Serial DefaultExecutionSpace;
#endif
typedef DefaultExecutionSpace DefaultHostExecutionSpace;

struct LayoutRight {};
struct LayoutLeft {};
struct LayoutStride {};

enum MemoryTraitsFlags { Unmanaged = 0x01, RandomAccess = 0x02, Atomic = 0x04 };
template <unsigned Flags>
struct MemoryTraits {};

// Kokkos::ALL() as a subview argument: the whole extent.
struct ALL {};

template <class... Args>
inline void initialize(Args&&...) {}
inline void finalize() {}

namespace shim {

// One allocation of a captured view: its label, element size and extents.
struct Captured {
  std::string label;
  std::shared_ptr<void> storage;
  const void* data;
  size_t elem_size;
  bool is_int;
  std::vector<size_t> extents;
};

inline std::set<std::string>& capture_labels() {
  static std::set<std::string> s;
  return s;
}

inline std::vector<Captured>& captured() {
  static std::vector<Captured> v;
  return v;
}

// Every view allocated from now on under this label is kept (in allocation
// order) until the process ends or clear_captured() is called.
inline void capture(const std::string& label) { capture_labels().insert(label); }
inline void clear_captured() { captured().clear(); }

}  // namespace shim

namespace Impl {

// Pointer levels of a Kokkos data type ("double**" has two runtime extents).
template <class D>
struct RuntimeDims {
  typedef D scalar;
  static const int count = 0;
};
template <class D>
struct RuntimeDims<D*> {
  typedef typename RuntimeDims<D>::scalar scalar;
  static const int count = RuntimeDims<D>::count + 1;
};

// "double *[5][3]" in a View means one runtime extent followed by the
// compile-time extents 5 and 3: C++ reads it as an array of arrays of
// pointers, so the array extents come off first and the pointers after.
template <class DataType>
struct Shape {
  typedef typename std::remove_all_extents<DataType>::type pointer_part;
  typedef typename RuntimeDims<pointer_part>::scalar value_type;
  static const int runtime_rank = RuntimeDims<pointer_part>::count;
  static const int static_rank = static_cast<int>(std::rank<DataType>::value);
  static const int rank = runtime_rank + static_rank;
};

template <class D, int K, int N>
struct StaticExtents {
  static void fill(size_t* e) {
    e[K] = std::extent<D, K>::value;
    StaticExtents<D, K + 1, N>::fill(e);
  }
};
template <class D, int N>
struct StaticExtents<D, N, N> {
  static void fill(size_t*) {}
};

// The same data type with const removed from the element type.
template <class D>
struct NonConstData {
  typedef typename std::remove_const<D>::type type;
};
template <class D>
struct NonConstData<D*> {
  typedef typename NonConstData<D>::type* type;
};
template <class D, size_t N>
struct NonConstData<D[N]> {
  typedef typename NonConstData<D>::type type[N];
};

}  // namespace Impl

template <class DataType, class Arg1 = void, class Arg2 = void, class Arg3 = void>
class View {
 public:
  typedef Impl::Shape<DataType> shape_type;
  typedef DataType data_type;
  typedef typename shape_type::value_type value_type;
  typedef typename std::remove_const<value_type>::type non_const_value_type;
  typedef typename Impl::NonConstData<DataType>::type non_const_data_type;
  typedef View<non_const_data_type> HostMirror;
  typedef size_t size_type;
  typedef DefaultExecutionSpace execution_space;
  typedef HostSpace memory_space;
  enum { Rank = shape_type::rank };

  View() : ptr_(nullptr) { clear_shape(); }

  // View(label, n0[, n1 ...]): the arguments give the runtime extents only.
  explicit View(const std::string& label, size_t n0 = 0, size_t n1 = 0, size_t n2 = 0, size_t n3 = 0,
                size_t n4 = 0, size_t n5 = 0, size_t n6 = 0, size_t n7 = 0)
      : ptr_(nullptr) {
    const size_t given[8] = {n0, n1, n2, n3, n4, n5, n6, n7};
    allocate(label, given);
  }

  // Shallow copy between views of the same element type (const may be added,
  // layout and memory traits may differ): both share one allocation.
  template <class D2, class B1, class B2, class B3>
  View(const View<D2, B1, B2, B3>& other)
      : track_(other.track_), ptr_(other.ptr_), label_(other.label_) {
    static_assert(static_cast<int>(View<D2, B1, B2, B3>::Rank) == static_cast<int>(Rank), "view rank mismatch");
    static_assert(std::is_same<non_const_value_type,
                               typename View<D2, B1, B2, B3>::non_const_value_type>::value,
                  "view element type mismatch");
    for (int k = 0; k < 8; ++k) {
      ext_[k] = other.ext_[k];
      str_[k] = other.str_[k];
    }
  }

  template <class I0>
  value_type& operator()(const I0& i0) const {
    return ptr_[static_cast<ptrdiff_t>(i0) * str_[0]];
  }
  template <class I0, class I1>
  value_type& operator()(const I0& i0, const I1& i1) const {
    return ptr_[static_cast<ptrdiff_t>(i0) * str_[0] + static_cast<ptrdiff_t>(i1) * str_[1]];
  }
  template <class I0, class I1, class I2>
  value_type& operator()(const I0& i0, const I1& i1, const I2& i2) const {
    return ptr_[static_cast<ptrdiff_t>(i0) * str_[0] + static_cast<ptrdiff_t>(i1) * str_[1] +
                static_cast<ptrdiff_t>(i2) * str_[2]];
  }
  template <class I0, class I1, class I2, class I3>
  value_type& operator()(const I0& i0, const I1& i1, const I2& i2, const I3& i3) const {
    return ptr_[static_cast<ptrdiff_t>(i0) * str_[0] + static_cast<ptrdiff_t>(i1) * str_[1] +
                static_cast<ptrdiff_t>(i2) * str_[2] + static_cast<ptrdiff_t>(i3) * str_[3]];
  }

  size_t dimension(int k) const { return ext_[k]; }
  size_t dimension_0() const { return ext_[0]; }
  size_t dimension_1() const { return ext_[1]; }
  size_t dimension_2() const { return ext_[2]; }
  size_t dimension_3() const { return ext_[3]; }
  size_t extent(int k) const { return ext_[k]; }
  size_t size() const {
    size_t n = 1;
    for (int k = 0; k < Rank; ++k) n *= ext_[k];
    return Rank == 0 ? 0 : n;
  }
  ptrdiff_t stride(int k) const { return str_[k]; }
  value_type* ptr_on_device() const { return ptr_; }
  value_type* data() const { return ptr_; }
  const std::string& label() const { return label_; }
  // LayoutRight strides over the whole extent (what memcpy-style copies need).
  bool contiguous() const {
    ptrdiff_t s = 1;
    for (int k = Rank - 1; k >= 0; --k) {
      if (ext_[k] > 1 && str_[k] != s) return false;
      s *= static_cast<ptrdiff_t>(ext_[k]);
    }
    return true;
  }

  // Allocates a zero-filled LayoutRight array. runtime_extents: the runtime
  // extents first (only those are read); compile-time extents come from the
  // data type.
  void allocate(const std::string& label, const size_t* runtime_extents) {
    clear_shape();
    label_ = label;
    for (int k = 0; k < shape_type::runtime_rank; ++k) ext_[k] = runtime_extents[k];
    Impl::StaticExtents<DataType, 0, shape_type::static_rank>::fill(ext_ + shape_type::runtime_rank);
    size_t n = 1;
    for (int k = Rank - 1; k >= 0; --k) {
      str_[k] = static_cast<ptrdiff_t>(n);
      n *= ext_[k];
    }
    non_const_value_type* p = new non_const_value_type[n > 0 ? n : 1]();
    track_ = std::shared_ptr<void>(p, [](void* q) { delete[] static_cast<non_const_value_type*>(q); });
    ptr_ = p;
    if (shim::capture_labels().count(label)) {
      shim::Captured c;
      c.label = label;
      c.storage = track_;
      c.data = p;
      c.elem_size = sizeof(non_const_value_type);
      c.is_int = std::is_integral<non_const_value_type>::value;
      c.extents.assign(ext_, ext_ + Rank);
      shim::captured().push_back(c);
    }
  }

  // Internals are public so that views of other template arguments, the
  // mirrors and subviews can share them.
  std::shared_ptr<void> track_;
  value_type* ptr_;
  size_t ext_[8];
  ptrdiff_t str_[8];
  std::string label_;

 private:
  void clear_shape() {
    for (int k = 0; k < 8; ++k) {
      ext_[k] = 0;
      str_[k] = 0;
    }
  }
};

// A new host allocation with the extents of v (contents zero, not copied).
template <class D, class A1, class A2, class A3>
typename View<D, A1, A2, A3>::HostMirror create_mirror(const View<D, A1, A2, A3>& v) {
  typename View<D, A1, A2, A3>::HostMirror m;
  m.allocate(v.label() + "_mirror", v.ext_);
  return m;
}

// Host views are their own host mirrors.
template <class D, class A1, class A2, class A3>
typename View<D, A1, A2, A3>::HostMirror create_mirror_view(const View<D, A1, A2, A3>& v) {
  return typename View<D, A1, A2, A3>::HostMirror(v);
}

template <class DD, class D1, class D2, class D3, class SD, class S1, class S2, class S3>
void deep_copy(const View<DD, D1, D2, D3>& dst, const View<SD, S1, S2, S3>& src) {
  typedef View<DD, D1, D2, D3> dst_type;
  static_assert(static_cast<int>(dst_type::Rank) == static_cast<int>(View<SD, S1, S2, S3>::Rank),
                "deep_copy rank mismatch");
  const int rank = dst_type::Rank;
  for (int k = 0; k < rank; ++k) {
    if (dst.ext_[k] != src.ext_[k]) {
      std::fprintf(stderr, "deep_copy: extent mismatch (%s <- %s)\n", dst.label().c_str(), src.label().c_str());
      std::abort();
    }
  }
  const size_t n = dst.size();
  if (n == 0 || static_cast<const void*>(dst.ptr_) == static_cast<const void*>(src.ptr_)) return;
  if (dst.contiguous() && src.contiguous()) {
    std::memcpy(const_cast<typename dst_type::non_const_value_type*>(dst.ptr_), src.ptr_,
                n * sizeof(typename dst_type::non_const_value_type));
    return;
  }
  // General strides: walk the index space in LayoutRight order.
  size_t idx[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (size_t e = 0; e < n; ++e) {
    ptrdiff_t od = 0, os = 0;
    for (int k = 0; k < rank; ++k) {
      od += static_cast<ptrdiff_t>(idx[k]) * dst.str_[k];
      os += static_cast<ptrdiff_t>(idx[k]) * src.str_[k];
    }
    const_cast<typename dst_type::non_const_value_type*>(dst.ptr_)[od] = src.ptr_[os];
    for (int k = rank - 1; k >= 0; --k) {
      if (++idx[k] < dst.ext_[k]) break;
      idx[k] = 0;
    }
  }
}

// subview(v, ALL(), j) of a rank-2 view: column j as a strided rank-1 view.
template <class D, class A1, class A2, class A3>
View<typename View<D, A1, A2, A3>::value_type*, LayoutStride> subview(const View<D, A1, A2, A3>& v, ALL,
                                                                        size_t j) {
  static_assert(static_cast<int>(View<D, A1, A2, A3>::Rank) == 2, "subview(v, ALL, j) needs a rank-2 view");
  View<typename View<D, A1, A2, A3>::value_type*, LayoutStride> s;
  s.track_ = v.track_;
  s.ptr_ = v.ptr_ + static_cast<ptrdiff_t>(j) * v.str_[1];
  s.ext_[0] = v.ext_[0];
  s.str_[0] = v.str_[0];
  s.label_ = v.label_;
  return s;
}

template <class F>
inline void parallel_for(const size_t n, const F& f) {
#ifdef MINIAERO_SHIM_OPENMP
  const long long count = static_cast<long long>(n);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < count; ++i) f(static_cast<int>(i));
#else
  for (size_t i = 0; i < n; ++i) f(static_cast<int>(i));
#endif
}

// parallel_reduce with a reducer: setup-time only in the reference (the face
// sort's key range), so it runs serially in both back ends.
template <class F, class Reducer>
inline void parallel_reduce(const size_t n, const F& f, const Reducer& r) {
  typename Reducer::value_type acc;
  r.init(acc);
  for (size_t i = 0; i < n; ++i) {
    const int ii = static_cast<int>(i);
    f(ii, acc);
  }
  r.reference() = acc;
}

namespace Experimental {

template <class Scalar>
struct MinMaxScalar {
  Scalar min_val;
  Scalar max_val;
};

template <class Scalar, class Space = void>
struct MinMax {
  typedef MinMaxScalar<typename std::remove_cv<Scalar>::type> value_type;
  value_type& value_;
  explicit MinMax(value_type& v) : value_(v) {}
  void init(value_type& v) const {
    v.min_val = std::numeric_limits<typename std::remove_cv<Scalar>::type>::max();
    v.max_val = std::numeric_limits<typename std::remove_cv<Scalar>::type>::lowest();
  }
  void join(value_type& dst, const value_type& src) const {
    if (src.min_val < dst.min_val) dst.min_val = src.min_val;
    if (src.max_val > dst.max_val) dst.max_val = src.max_val;
  }
  value_type& reference() const { return value_; }
};

}  // namespace Experimental

// ---- atomics on host memory ----------------------------------------------
// Serial: plain read-modify-write (what a single thread's atomic does).
// OpenMP: compare-and-swap on the value's bits.

// Compares bit patterns, not values (so -0.0 and +0.0 differ), and returns
// the value *p held before the call. The memory is only ever accessed as T:
// reading it through an integer pointer would break C++ aliasing rules, and
// at -O3 the compiler then keeps the reference's re-read of *p in a register
// and its compare-and-swap retry loops never end.
template <class T>
inline T atomic_compare_exchange(volatile T* p, const T comparand, const T value) {
  static_assert(sizeof(T) == 8 || sizeof(T) == 4, "atomic_compare_exchange: 4- or 8-byte types only");
  T* q = const_cast<T*>(p);
#ifdef MINIAERO_SHIM_OPENMP
  T expected = comparand;
  T desired = value;
  __atomic_compare_exchange(q, &expected, &desired, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return expected;
#else
  const T current = *q;
  if (std::memcmp(&current, &comparand, sizeof(T)) == 0) *q = value;
  return current;
#endif
}

template <class T, class U>
inline T atomic_fetch_add(volatile T* p, const U v) {
#ifdef MINIAERO_SHIM_OPENMP
  T old = *const_cast<T*>(p);
  for (;;) {
    const T next = static_cast<T>(old + v);
    const T seen = atomic_compare_exchange(p, old, next);
    if (std::memcmp(&seen, &old, sizeof(T)) == 0) return old;
    old = seen;
  }
#else
  T* q = const_cast<T*>(p);
  const T old = *q;
  *q = static_cast<T>(old + v);
  return old;
#endif
}

template <class T, class U>
inline void atomic_add(volatile T* p, const U v) {
  atomic_fetch_add(p, v);
}

namespace Impl {

class Timer {
 public:
  Timer() { reset(); }
  void reset() { start_ = std::chrono::steady_clock::now(); }
  double seconds() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - start_).count();
  }

 private:
  std::chrono::steady_clock::time_point start_;
};

}  // namespace Impl

typedef Impl::Timer Timer;

}  // namespace Kokkos

#endif
