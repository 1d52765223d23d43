/*
 * A minimal stand-in for the few RAJA and camp names that Kripke's sources use, written for
 * this project so that the reference's own C++ (generator, kernels, solvers, DataStore) compiles
 * and runs here on one host thread.  TEST INFRASTRUCTURE ONLY: it builds the reference into
 * oracle/_ref/ to pin the oracle; nothing in the product includes it.
 *
 * RAJA and camp are empty submodules in the reference tree, so nothing here comes from them.
 * What each name has to do follows from how the reference uses it:
 *   - RAJA::kernel with KernelPolicy<For<arg, exec, ...>, Lambda<0>> nests one loop per For in
 *     the policy's order, each walking its segment in the segment's own order, and calls the
 *     lambda with the current value of every segment in tuple order; Collapse<exec,
 *     ArgList<a, b, ...>, body> is the same nest over a, b, ... in that order.  Kripke's
 *     Sequential policies are built only of For, Collapse and Lambda (src/Kripke/Arch/*.h).
 *   - TypedRangeStrideSegment(begin, end, stride) visits begin, begin+stride, ... up to but not
 *     including end, in either direction (the upwind walk, Kernel/SweepSubdomain.cpp:70-82).
 *   - Layout(s0, s1, ...) is row-major over the dimensions whose size is non-zero; a zero-size
 *     dimension has stride 0 and takes no part in the product (the projections of
 *     Core/PartitionSpace.cpp:90-98 rely on that).  make_permuted_layout(sizes, perm) gives
 *     stride 1 to perm's last dimension, perm listing dimensions from slowest to fastest
 *     (Core/VarLayout.h:96-170 builds perm that way).  toIndices is the inverse.
 *   - Views index their pointer through the layout; typed indices are unwrapped with operator*.
 *   - ReduceSum copies share one accumulator (reducers are captured by value in
 *     Generate/Space.cpp:274-313 and updated from a non-mutable lambda).
 */
#ifndef KGB_REFSHIM_RAJA_HPP
#define KGB_REFSHIM_RAJA_HPP

#include <algorithm>
#include <array>
#include <cfloat>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>
#include <cstddef>
#include <memory>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>

#define RAJA_INLINE inline
#define RAJA_HOST_DEVICE
#define RAJA_HOST
#define RAJA_DEVICE

namespace camp {

using idx_t = std::ptrdiff_t;

template <typename... T>
struct list {};

template <typename L>
struct size;
template <typename... T>
struct size<list<T...>> {
  static constexpr idx_t value = sizeof...(T);
};

template <typename L, idx_t I>
struct at_impl;
template <typename... T, idx_t I>
struct at_impl<list<T...>, I> {
  using type = typename std::tuple_element<(size_t)I, std::tuple<T...>>::type;
};
template <typename L, idx_t I>
using at_v = typename at_impl<L, I>::type;

template <idx_t... I>
struct idx_seq {
  static std::array<idx_t, sizeof...(I)> array() { return {{I...}}; }
};

namespace detail {
template <typename S>
struct to_idx_seq;
template <idx_t... I>
struct to_idx_seq<std::integer_sequence<idx_t, I...>> {
  using type = idx_seq<I...>;
};
}  // namespace detail

template <idx_t N>
using make_idx_seq_t = typename detail::to_idx_seq<std::make_integer_sequence<idx_t, N>>::type;
template <idx_t N>
struct make_idx_seq {
  using type = make_idx_seq_t<N>;
};

template <typename... T>
using tuple = std::tuple<T...>;
using std::get;
using std::make_tuple;

}  // namespace camp

namespace RAJA {

using Index_type = std::ptrdiff_t;

/* ---- strongly typed indices (RAJA_INDEX_VALUE) ------------------------------------------ */

struct IndexValueTag {};

template <typename TYPE, typename VALUE = Index_type>
class IndexValue : public IndexValueTag {
 public:
  using value_type = VALUE;
  constexpr IndexValue() : v_(0) {}
  constexpr explicit IndexValue(VALUE v) : v_(v) {}
  template <typename T, typename = typename std::enable_if<std::is_integral<T>::value>::type>
  constexpr explicit IndexValue(T v) : v_((VALUE)v) {}

  VALUE &operator*() { return v_; }
  const VALUE &operator*() const { return v_; }

  TYPE &operator++() { ++v_; return self(); }
  TYPE operator++(int) { TYPE t(v_); ++v_; return t; }
  TYPE &operator--() { --v_; return self(); }
  TYPE operator--(int) { TYPE t(v_); --v_; return t; }

  TYPE operator+(VALUE a) const { return TYPE(v_ + a); }
  TYPE operator+(TYPE a) const { return TYPE(v_ + *a); }
  TYPE operator-(VALUE a) const { return TYPE(v_ - a); }
  TYPE operator-(TYPE a) const { return TYPE(v_ - *a); }
  TYPE operator*(VALUE a) const { return TYPE(v_ * a); }
  TYPE operator/(VALUE a) const { return TYPE(v_ / a); }
  TYPE &operator+=(VALUE a) { v_ += a; return self(); }
  TYPE &operator+=(TYPE a) { v_ += *a; return self(); }
  TYPE &operator-=(VALUE a) { v_ -= a; return self(); }
  TYPE &operator-=(TYPE a) { v_ -= *a; return self(); }

  bool operator<(VALUE a) const { return v_ < a; }
  bool operator<(TYPE a) const { return v_ < *a; }
  bool operator<=(VALUE a) const { return v_ <= a; }
  bool operator<=(TYPE a) const { return v_ <= *a; }
  bool operator>(VALUE a) const { return v_ > a; }
  bool operator>(TYPE a) const { return v_ > *a; }
  bool operator>=(VALUE a) const { return v_ >= a; }
  bool operator>=(TYPE a) const { return v_ >= *a; }
  bool operator==(VALUE a) const { return v_ == a; }
  bool operator==(TYPE a) const { return v_ == *a; }
  bool operator!=(VALUE a) const { return v_ != a; }
  bool operator!=(TYPE a) const { return v_ != *a; }

 private:
  TYPE &self() { return *static_cast<TYPE *>(this); }
  VALUE v_;
};

#define RAJA_INDEX_VALUE(TYPE, NAME)                              \
  class TYPE : public ::RAJA::IndexValue<TYPE> {                  \
    using parent = ::RAJA::IndexValue<TYPE>;                      \
                                                                  \
   public:                                                        \
    using parent::parent;                                         \
    constexpr TYPE() : parent() {}                                \
    static inline std::string getName() { return NAME; }          \
  };

template <typename T>
inline Index_type stripIndexType(T const &v, typename std::enable_if<std::is_base_of<IndexValueTag, T>::value>::type * = nullptr) {
  return (Index_type)*v;
}
template <typename T>
inline Index_type stripIndexType(T const &v, typename std::enable_if<!std::is_base_of<IndexValueTag, T>::value>::type * = nullptr) {
  return (Index_type)v;
}

template <typename T>
inline T makeIndex(Index_type v, typename std::enable_if<std::is_base_of<IndexValueTag, T>::value>::type * = nullptr) {
  return T(v);
}
template <typename T>
inline T makeIndex(Index_type v, typename std::enable_if<!std::is_base_of<IndexValueTag, T>::value>::type * = nullptr) {
  return (T)v;
}

/* ---- segments ---------------------------------------------------------------------------- */

template <typename T>
struct TypedRangeStrideSegment {
  using value_type = T;
  TypedRangeStrideSegment(Index_type begin, Index_type end, Index_type stride) : b(begin), e(end), s(stride) {}
  Index_type count() const {
    if (s > 0) return e > b ? (e - b + s - 1) / s : 0;
    if (s < 0) return b > e ? (b - e + (-s) - 1) / (-s) : 0;
    return 0;
  }
  struct iterator {
    Index_type v, s;
    T operator*() const { return makeIndex<T>(v); }
    iterator &operator++() { v += s; return *this; }
    bool operator!=(iterator const &o) const { return v != o.v; }
  };
  iterator begin() const { return iterator{b, s}; }
  iterator end() const { return iterator{b + count() * s, s}; }
  Index_type size() const { return count(); }
  Index_type b, e, s;
};

template <typename T>
struct TypedRangeSegment : TypedRangeStrideSegment<T> {
  TypedRangeSegment(Index_type begin, Index_type end) : TypedRangeStrideSegment<T>(begin, end, 1) {}
};

using RangeSegment = TypedRangeSegment<Index_type>;
using RangeStrideSegment = TypedRangeStrideSegment<Index_type>;

/* ---- execution and reduction policies (names only: everything runs in order, on this thread) */

struct loop_exec {};
struct seq_exec {};
struct simd_exec {};
struct seq_reduce {};
struct auto_atomic {};
struct seq_atomic {};
template <size_t N>
struct tile_fixed {};
template <camp::idx_t... I>
struct ArgList {};

template <typename ExecPolicy, typename Segment, typename Body>
inline void forall(Segment const &seg, Body const &body) {
  for (auto v : seg) body(v);
}

/* ---- RAJA::kernel over For / Lambda statements --------------------------------------------- */

template <typename... Stmts>
struct KernelPolicy {};

namespace statement {
template <camp::idx_t ArgN, typename ExecPolicy, typename... Body>
struct For {};
template <camp::idx_t LambdaN, typename... Args>
struct Lambda {};
template <typename... T>
struct Collapse {};
template <typename... T>
struct If {};
template <camp::idx_t N>
struct Param {};
template <typename T>
struct Not {};
template <typename... T>
struct Hyperplane {};
template <typename... T>
struct Tile {};
}  // namespace statement

namespace detail {

template <typename Segs, typename Idx, typename Bodies>
struct KernelData {
  Segs const &segs;
  Idx idx;
  Bodies bodies;
};

template <typename Stmt>
struct Exec;

template <camp::idx_t ArgN, typename EP, typename... Body>
struct Exec<statement::For<ArgN, EP, Body...>> {
  template <typename Data>
  static void run(Data &d) {
    for (auto v : std::get<ArgN>(d.segs)) {
      std::get<ArgN>(d.idx) = v;
      int dummy[] = {0, (Exec<Body>::run(d), 0)...};
      (void)dummy;
    }
  }
};

template <typename ArgL, typename... Body>
struct CollapseExec;
template <typename... Body>
struct CollapseExec<ArgList<>, Body...> {
  template <typename Data>
  static void run(Data &d) {
    int dummy[] = {0, (Exec<Body>::run(d), 0)...};
    (void)dummy;
  }
};
template <camp::idx_t A, camp::idx_t... Rest, typename... Body>
struct CollapseExec<ArgList<A, Rest...>, Body...> {
  template <typename Data>
  static void run(Data &d) {
    for (auto v : std::get<A>(d.segs)) {
      std::get<A>(d.idx) = v;
      CollapseExec<ArgList<Rest...>, Body...>::run(d);
    }
  }
};

template <typename EP, camp::idx_t... Args, typename... Body>
struct Exec<statement::Collapse<EP, ArgList<Args...>, Body...>> {
  template <typename Data>
  static void run(Data &d) {
    CollapseExec<ArgList<Args...>, Body...>::run(d);
  }
};

template <camp::idx_t L, typename... Args>
struct Exec<statement::Lambda<L, Args...>> {
  template <typename Data>
  static void run(Data &d) {
    std::apply(std::get<L>(d.bodies), d.idx);
  }
};

template <typename Seg>
using seg_value_t = typename std::decay<Seg>::type::value_type;

}  // namespace detail

namespace detail {
template <typename P>
struct PolicyStmts;
template <typename... S>
struct PolicyStmts<KernelPolicy<S...>> {
  template <typename Data>
  static void run(Data &d) {
    int dummy[] = {0, (Exec<S>::run(d), 0)...};
    (void)dummy;
  }
};
template <typename Tuple>
struct IdxTuple;
template <typename... Segs>
struct IdxTuple<std::tuple<Segs...>> {
  using type = std::tuple<seg_value_t<Segs>...>;
};
}  // namespace detail

template <typename Policy, typename SegTuple, typename... Bodies>
inline void kernel(SegTuple const &segs, Bodies const &... bodies) {
  using Segs = typename std::decay<SegTuple>::type;
  using Idx = typename detail::IdxTuple<Segs>::type;
  using BodyTuple = std::tuple<Bodies const &...>;
  detail::KernelData<Segs, Idx, BodyTuple> d{segs, Idx{}, BodyTuple(bodies...)};
  detail::PolicyStmts<Policy>::run(d);
}

/* ---- reductions ------------------------------------------------------------------------------ */

template <typename ReducePolicy, typename T>
class ReduceSum {
 public:
  ReduceSum() : v_(std::make_shared<T>(T())) {}
  explicit ReduceSum(T init) : v_(std::make_shared<T>(init)) {}
  ReduceSum const &operator+=(T x) const {
    *v_ = *v_ + x;
    return *this;
  }
  T get() const { return *v_; }
  operator T() const { return *v_; }
  void reset(T init) { *v_ = init; }

 private:
  std::shared_ptr<T> v_;
};

/* ---- layouts and views ----------------------------------------------------------------------- */

template <size_t N, typename IdxLin = Index_type, camp::idx_t StrideOne = -1>
struct Layout {
  static constexpr size_t n_dims = N;
  std::array<IdxLin, N> sizes{};
  std::array<IdxLin, N> strides{};

  Layout() = default;

  template <typename... S, typename = typename std::enable_if<sizeof...(S) == N && N != 0>::type>
  explicit Layout(S... s) {
    std::array<IdxLin, N> sz{{(IdxLin)s...}};
    std::array<IdxLin, N> perm;
    for (size_t i = 0; i < N; ++i) perm[i] = (IdxLin)i;
    init(sz, perm);
  }

  template <camp::idx_t S2>
  Layout(Layout<N, IdxLin, S2> const &o) : sizes(o.sizes), strides(o.strides) {}

  template <typename Sz, typename Pm>
  void init(std::array<Sz, N> const &sz, std::array<Pm, N> const &perm) {
    for (size_t i = 0; i < N; ++i) sizes[i] = (IdxLin)sz[i];
    IdxLin run = 1;
    for (size_t p = N; p-- > 0;) {
      size_t dim = (size_t)perm[p];
      strides[dim] = sizes[dim] ? run : 0;
      run *= sizes[dim] ? sizes[dim] : 1;
    }
  }

  template <typename... I>
  IdxLin operator()(I const &... idx) const {
    static_assert(sizeof...(I) == N, "layout index count");
    std::array<IdxLin, N> v{{(IdxLin)stripIndexType(idx)...}};
    IdxLin lin = 0;
    for (size_t i = 0; i < N; ++i) lin += v[i] * strides[i];
    return lin;
  }

  template <typename... I>
  void toIndices(IdxLin lin, I &... idx) const {
    static_assert(sizeof...(I) == N, "layout index count");
    std::array<IdxLin, N> out;
    for (size_t i = 0; i < N; ++i) out[i] = (strides[i] && sizes[i]) ? (lin / strides[i]) % sizes[i] : 0;
    size_t k = 0;
    int dummy[] = {0, (idx = (typename std::decay<I>::type)out[k++], 0)...};
    (void)dummy;
  }

  IdxLin size() const {
    IdxLin s = 1;
    for (size_t i = 0; i < N; ++i) s *= sizes[i] ? sizes[i] : 1;
    return s;
  }
};

template <size_t N, typename IdxLin = Index_type, typename Sz, typename Pm>
inline Layout<N, IdxLin> make_permuted_layout(std::array<Sz, N> const &sizes, std::array<Pm, N> const &perm) {
  Layout<N, IdxLin> l;
  l.init(sizes, perm);
  return l;
}

template <camp::idx_t S, size_t N, typename IdxLin, camp::idx_t S0>
inline Layout<N, IdxLin, S> make_stride_one(Layout<N, IdxLin, S0> const &l) {
  return Layout<N, IdxLin, S>(l);
}

template <typename IdxLin, typename IdxTuple, camp::idx_t StrideOne = -1>
struct TypedLayout;

template <typename IdxLin, typename... IdxTypes, camp::idx_t StrideOne>
struct TypedLayout<IdxLin, std::tuple<IdxTypes...>, StrideOne>
    : Layout<sizeof...(IdxTypes), IdxLin, StrideOne> {
  using Base = Layout<sizeof...(IdxTypes), IdxLin, StrideOne>;
  TypedLayout() = default;
  template <camp::idx_t S2>
  TypedLayout(Layout<sizeof...(IdxTypes), IdxLin, S2> const &o) : Base(o) {}
  template <typename... S, typename = typename std::enable_if<sizeof...(S) == sizeof...(IdxTypes) &&
                                                              (std::is_integral<S>::value && ...)>::type>
  explicit TypedLayout(S... s) : Base(s...) {}
};

template <typename PERM>
struct as_array;
template <camp::idx_t... I>
struct as_array<camp::idx_seq<I...>> {
  static std::array<Index_type, sizeof...(I)> get() { return {{(Index_type)I...}}; }
};
template <size_t N>
using MakePerm = camp::make_idx_seq_t<(camp::idx_t)N>;

namespace internal {
template <typename T, typename PtrT, typename LayoutT>
struct ViewBase {
  using value_type = T;
  PtrT data{};
  LayoutT layout{};
  ViewBase() = default;
  ViewBase(PtrT p, LayoutT const &l) : data(p), layout(l) {}
  template <typename... I>
  T &operator()(I const &... idx) const {
    return data[layout(idx...)];
  }
};
}  // namespace internal

template <typename T, typename LayoutT, typename PtrT = T *>
struct View : internal::ViewBase<T, PtrT, LayoutT> {
  using internal::ViewBase<T, PtrT, LayoutT>::ViewBase;
};

/* ---- timer ----------------------------------------------------------------------------------- */

class Timer {
 public:
  void start(const char * = nullptr) { t0_ = clock::now(); running_ = true; }
  void stop(const char * = nullptr) {
    if (running_) {
      acc_ += std::chrono::duration<double>(clock::now() - t0_).count();
      running_ = false;
    }
  }
  void reset() { acc_ = 0.0; running_ = false; }
  double elapsed() const { return acc_; }

 private:
  using clock = std::chrono::steady_clock;
  clock::time_point t0_{};
  double acc_ = 0.0;
  bool running_ = false;
};

}  // namespace RAJA

#endif
