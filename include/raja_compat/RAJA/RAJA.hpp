// raja_compat -- a minimal RAJA-API front-end (namespace RAJA) for builds
// where RAJA itself is not available.
//
// RAJA's own headers need its camp library and a CMake-generated config,
// which an application may not have.  This header restates the small part
// of RAJA's front-end that the data-parallel primitive path uses, with the
// reference's semantics (its host policies reproduce RAJA's own seq / omp
// results bit for bit on the shared fixtures):
//
//   forall / forall with expt params       pattern/forall.hpp:323-652
//   Reduce{Sum,Min,Max,MinLoc,MaxLoc,
//          BitOr,BitAnd}<seq_reduce|omp_reduce>   pattern/reduce.hpp,
//                                          pattern/detail/reduce.hpp:212-358
//   expt::Reduce / ReduceLoc / ValOp /
//          ValLoc / KernelName             pattern/params/*.hpp
//   inclusive/exclusive_scan[_inplace]     pattern/scan.hpp:49-441
//   sort / stable_sort / sort_pairs /
//          stable_sort_pairs               pattern/sort.hpp:59-451
//   WorkPool / WorkGroup / WorkSite        pattern/WorkGroup.hpp:117-530
//   segments                               index/RangeSegment.hpp,
//                                          index/ListSegment.hpp
//
// Back-ends plug in exactly as in RAJA: the front-end calls unqualified
// implementation functions (forall_impl, impl::scan::*, impl::sort::*,
// reducer specialisations) that are overloaded on the policy type.  This
// header provides seq_exec / omp_parallel_for_exec and seq_reduce /
// omp_reduce; include/raja_b200/RAJA_b200.hpp adds the b200 family.
#pragma once

// Marks this front-end for back-end headers that also build against an
// installed RAJA (include/raja_b200/RAJA_b200.hpp).
#define RAJA_COMPAT_FRONTEND 1

#include <algorithm>
#include <array>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iterator>
#include <limits>
#include <memory>
#include <stdexcept>
#include <tuple>
#include <type_traits>
#include <utility>
#include <variant>
#include <vector>

#if defined(_OPENMP)
#include <omp.h>
#endif

#if defined(__CUDACC__)
#define RAJA_HOST_DEVICE __host__ __device__
#define RAJA_DEVICE __device__
#define RAJA_HOST __host__
#else
#define RAJA_HOST_DEVICE
#define RAJA_DEVICE
#define RAJA_HOST
#endif
#define RAJA_INLINE inline
// Team-shared arrays in RAJA::launch bodies (shared memory on the device).
#if defined(__CUDA_ARCH__)
#define RAJA_TEAM_SHARED __shared__
#else
#define RAJA_TEAM_SHARED
#endif

namespace RAJA {

using Index_type = std::ptrdiff_t;

// ------------------------------------------------------------ operators
// util/Operators.hpp: limits (:248-333), plus (:363-372), minimum /
// maximum keep the first of equal values (:555-591).
namespace operators {

template <typename T, typename Enable = void>
struct limits;
template <typename T>
struct limits<T, typename std::enable_if<std::is_integral<T>::value>::type> {
  RAJA_HOST_DEVICE static constexpr T min() { return std::numeric_limits<T>::lowest(); }
  RAJA_HOST_DEVICE static constexpr T max() { return std::numeric_limits<T>::max(); }
};
template <typename T>
struct limits<T, typename std::enable_if<std::is_floating_point<T>::value>::type> {
  RAJA_HOST_DEVICE static constexpr T min() { return -std::numeric_limits<T>::max(); }
  RAJA_HOST_DEVICE static constexpr T max() { return std::numeric_limits<T>::max(); }
};

template <typename Ret, typename Arg1 = Ret, typename Arg2 = Arg1>
struct plus {
  using result_type = Ret;
  RAJA_HOST_DEVICE constexpr Ret operator()(const Arg1& lhs, const Arg2& rhs) const { return lhs + rhs; }
  RAJA_HOST_DEVICE static constexpr Ret identity() { return Ret(0); }
};
template <typename Ret, typename Arg1 = Ret, typename Arg2 = Arg1>
struct minimum {
  using result_type = Ret;
  RAJA_HOST_DEVICE constexpr Ret operator()(const Arg1& lhs, const Arg2& rhs) const {
    return (rhs < lhs) ? rhs : lhs;
  }
  RAJA_HOST_DEVICE static constexpr Ret identity() { return limits<Ret>::max(); }
};
template <typename Ret, typename Arg1 = Ret, typename Arg2 = Arg1>
struct maximum {
  using result_type = Ret;
  RAJA_HOST_DEVICE constexpr Ret operator()(const Arg1& lhs, const Arg2& rhs) const {
    return (lhs < rhs) ? rhs : lhs;
  }
  RAJA_HOST_DEVICE static constexpr Ret identity() { return limits<Ret>::min(); }
};
template <typename Ret, typename Arg1 = Ret, typename Arg2 = Arg1>
struct bit_or {
  using result_type = Ret;
  RAJA_HOST_DEVICE constexpr Ret operator()(const Arg1& lhs, const Arg2& rhs) const { return lhs | rhs; }
  RAJA_HOST_DEVICE static constexpr Ret identity() { return Ret(0); }
};
template <typename Ret, typename Arg1 = Ret, typename Arg2 = Arg1>
struct bit_and {
  using result_type = Ret;
  RAJA_HOST_DEVICE constexpr Ret operator()(const Arg1& lhs, const Arg2& rhs) const { return lhs & rhs; }
  RAJA_HOST_DEVICE static constexpr Ret identity() { return Ret(~Ret(0)); }
};
template <typename T>
struct less {
  RAJA_HOST_DEVICE constexpr bool operator()(const T& a, const T& b) const { return a < b; }
};
template <typename T>
struct greater {
  RAJA_HOST_DEVICE constexpr bool operator()(const T& a, const T& b) const { return b < a; }
};

}  // namespace operators

// ---------------------------------------------------- strongly typed indices
// IndexValue<TYPE, VALUE> (index/IndexValue.hpp:34-415): an index wrapped in
// its own type, so that indices of different spaces do not mix.  TYPE is
// the derived class that RAJA_INDEX_VALUE / RAJA_INDEX_VALUE_T declare; the
// arithmetic and comparisons take another TYPE or a raw VALUE and return
// TYPE; *x and stripIndexType(x) give the raw value (there is no implicit
// conversion to an integer).
template <typename TYPE, typename VALUE = Index_type>
class IndexValue {
 public:
  using value_type = VALUE;
  RAJA_HOST_DEVICE constexpr IndexValue() : value(0) {}
  RAJA_HOST_DEVICE constexpr explicit IndexValue(VALUE v) : value(v) {}
  RAJA_HOST_DEVICE VALUE& operator*() { return value; }
  RAJA_HOST_DEVICE constexpr const VALUE& operator*() const { return value; }

  RAJA_HOST_DEVICE TYPE& operator++() { ++value; return self(); }
  RAJA_HOST_DEVICE TYPE operator++(int) { TYPE t = self(); ++value; return t; }
  RAJA_HOST_DEVICE TYPE& operator--() { --value; return self(); }
  RAJA_HOST_DEVICE TYPE operator--(int) { TYPE t = self(); --value; return t; }

#define RAJA_COMPAT_INDEX_ARITH(OP)                                                              \
  RAJA_HOST_DEVICE TYPE operator OP(VALUE a) const { return TYPE(VALUE(value OP a)); }           \
  RAJA_HOST_DEVICE TYPE operator OP(TYPE a) const { return TYPE(VALUE(value OP a.value)); }      \
  RAJA_HOST_DEVICE TYPE& operator OP##=(VALUE a) { value = VALUE(value OP a); return self(); }    \
  RAJA_HOST_DEVICE TYPE& operator OP##=(TYPE a) { value = VALUE(value OP a.value); return self(); }
  RAJA_COMPAT_INDEX_ARITH(+)
  RAJA_COMPAT_INDEX_ARITH(-)
  RAJA_COMPAT_INDEX_ARITH(*)
  RAJA_COMPAT_INDEX_ARITH(/)
#undef RAJA_COMPAT_INDEX_ARITH
  RAJA_HOST_DEVICE TYPE operator%(VALUE a) const { return TYPE(VALUE(value % a)); }
  RAJA_HOST_DEVICE TYPE operator%(TYPE a) const { return TYPE(VALUE(value % a.value)); }

#define RAJA_COMPAT_INDEX_CMP(OP)                                                 \
  RAJA_HOST_DEVICE bool operator OP(VALUE a) const { return value OP a; }         \
  RAJA_HOST_DEVICE bool operator OP(TYPE a) const { return value OP a.value; }
  RAJA_COMPAT_INDEX_CMP(<)
  RAJA_COMPAT_INDEX_CMP(<=)
  RAJA_COMPAT_INDEX_CMP(>)
  RAJA_COMPAT_INDEX_CMP(>=)
  RAJA_COMPAT_INDEX_CMP(==)
  RAJA_COMPAT_INDEX_CMP(!=)
#undef RAJA_COMPAT_INDEX_CMP

 protected:
  VALUE value;

 private:
  RAJA_HOST_DEVICE TYPE& self() { return static_cast<TYPE&>(*this); }
  RAJA_HOST_DEVICE const TYPE& self() const { return static_cast<const TYPE&>(*this); }
};

namespace detail {
template <typename T, typename = void>
struct is_index_value : std::false_type {};
template <typename T>
struct is_index_value<T, std::void_t<typename T::IndexValueType>> : std::true_type {};
template <typename T, bool = is_index_value<T>::value>
struct strip_index {
  using type = T;
};
template <typename T>
struct strip_index<T, true> {
  using type = typename T::value_type;
};
}  // namespace detail
// The raw value of an index (the value itself for integer indices).
template <typename T>
using strip_index_type_t = typename detail::strip_index<T>::type;
template <typename T>
RAJA_HOST_DEVICE constexpr strip_index_type_t<T> stripIndexType(const T& v) {
  if constexpr (detail::is_index_value<T>::value) return *v;
  else return v;
}
// convertIndex<TO>(from): the raw value of `from` as index type TO.
template <typename TO, typename FROM>
RAJA_HOST_DEVICE constexpr TO convertIndex(const FROM& v) {
  return TO(static_cast<strip_index_type_t<TO>>(stripIndexType(v)));
}

}  // namespace RAJA

// Declare a strongly typed index TYPE over Index_type (or over IDXT).
#define RAJA_INDEX_VALUE(TYPE, NAME)                                                  \
  class TYPE : public ::RAJA::IndexValue<TYPE> {                                      \
   public:                                                                            \
    using IndexValueType = TYPE;                                                      \
    RAJA_HOST_DEVICE TYPE() : ::RAJA::IndexValue<TYPE>() {}                           \
    RAJA_HOST_DEVICE explicit TYPE(::RAJA::Index_type v) : ::RAJA::IndexValue<TYPE>(v) {} \
    static inline std::string getName() { return NAME; }                             \
  }
#define RAJA_INDEX_VALUE_T(TYPE, IDXT, NAME)                                          \
  class TYPE : public ::RAJA::IndexValue<TYPE, IDXT> {                                \
   public:                                                                            \
    using IndexValueType = TYPE;                                                      \
    RAJA_HOST_DEVICE TYPE() : ::RAJA::IndexValue<TYPE, IDXT>() {}                     \
    RAJA_HOST_DEVICE explicit TYPE(IDXT v) : ::RAJA::IndexValue<TYPE, IDXT>(v) {}    \
    static inline std::string getName() { return NAME; }                             \
  }

namespace RAJA {

// ------------------------------------------------------------- segments
// Random-access iterator over the values start, start + step, ... (the role
// of Iterators::numeric_iterator / strided_numeric_iterator,
// index/RangeSegment.hpp, index/RangeStrideSegment.hpp).
template <typename T>
struct NumericIterator {
  using iterator_category = std::random_access_iterator_tag;
  using value_type = T;
  using difference_type = Index_type;
  using pointer = const T*;
  using reference = T;
  T v, step;
  RAJA_HOST_DEVICE T operator*() const { return v; }
  RAJA_HOST_DEVICE T operator[](difference_type k) const { return T(v + T(k) * step); }
  RAJA_HOST_DEVICE NumericIterator& operator++() { v += step; return *this; }
  RAJA_HOST_DEVICE NumericIterator operator++(int) { NumericIterator t = *this; v += step; return t; }
  RAJA_HOST_DEVICE NumericIterator& operator--() { v -= step; return *this; }
  RAJA_HOST_DEVICE NumericIterator& operator+=(difference_type k) { v += T(k) * step; return *this; }
  RAJA_HOST_DEVICE NumericIterator& operator-=(difference_type k) { v -= T(k) * step; return *this; }
  RAJA_HOST_DEVICE NumericIterator operator+(difference_type k) const { return {T(v + T(k) * step), step}; }
  RAJA_HOST_DEVICE NumericIterator operator-(difference_type k) const { return {T(v - T(k) * step), step}; }
  RAJA_HOST_DEVICE difference_type operator-(const NumericIterator& o) const {
    return difference_type(stripIndexType((v - o.v) / step));
  }
  RAJA_HOST_DEVICE bool operator==(const NumericIterator& o) const { return v == o.v; }
  RAJA_HOST_DEVICE bool operator!=(const NumericIterator& o) const { return v != o.v; }
  RAJA_HOST_DEVICE bool operator<(const NumericIterator& o) const { return (o - *this) > 0; }
};

template <typename T>
struct TypedRangeSegment {
  using value_type = T;
  using iterator = NumericIterator<T>;
  T b, e;
  RAJA_HOST_DEVICE TypedRangeSegment(T begin, T end) : b(begin), e(end < begin ? begin : end) {}
  RAJA_HOST_DEVICE T size() const { return e - b; }
  RAJA_HOST_DEVICE iterator begin() const { return {b, T(1)}; }
  RAJA_HOST_DEVICE iterator end() const { return {e, T(1)}; }
  // the sub-range [begin + off, begin + off + len), clipped to this one
  RAJA_HOST_DEVICE TypedRangeSegment slice(T off, T len) const {
    const T lo = b + off < e ? T(b + off) : e;
    const T hi = lo + len < e ? T(lo + len) : e;
    return TypedRangeSegment(lo, hi);
  }
  RAJA_HOST_DEVICE bool operator==(const TypedRangeSegment& o) const { return b == o.b && e == o.e; }
};
using RangeSegment = TypedRangeSegment<Index_type>;

template <typename T>
struct TypedRangeStrideSegment {
  using value_type = T;
  using iterator = NumericIterator<T>;
  T b, e, s;
  RAJA_HOST_DEVICE TypedRangeStrideSegment(T begin, T end, T stride) : b(begin), e(end), s(stride) {}
  RAJA_HOST_DEVICE T size() const {
    if (s > 0) return e > b ? (e - b + s - 1) / s : 0;
    return b > e ? (b - e + (-s) - 1) / (-s) : 0;
  }
  RAJA_HOST_DEVICE iterator begin() const { return {b, s}; }
  RAJA_HOST_DEVICE iterator end() const { return {T(b + size() * s), s}; }
};
using RangeStrideSegment = TypedRangeStrideSegment<Index_type>;

// A list of indices.  `data` must be readable where the loop runs (host
// memory for host policies, device or managed memory for b200 policies).
template <typename T>
struct TypedListSegment {
  using value_type = T;
  const T* data;
  Index_type len;
  RAJA_HOST_DEVICE TypedListSegment(const T* d, Index_type n) : data(d), len(n) {}
  RAJA_HOST_DEVICE Index_type size() const { return len; }
  RAJA_HOST_DEVICE const T* begin() const { return data; }
  RAJA_HOST_DEVICE const T* end() const { return data + len; }
};
using ListSegment = TypedListSegment<Index_type>;

// IndexSet (index/IndexSet.hpp:50-630): an ordered list of segments of the
// listed types (range, strided, list) over one index type, e.g.
// TypedIndexSet<RangeSegment, ListSegment>.  forall runs the segments in
// order; forall_Icount numbers the indices across them.
template <typename S, typename... Ts>
struct one_of : std::bool_constant<(std::is_same<S, Ts>::value || ...)> {};
template <typename... SegmentTypes>
class TypedIndexSet {
  static_assert(sizeof...(SegmentTypes) >= 1, "an IndexSet lists its segment types");
  using first_segment = std::tuple_element_t<0, std::tuple<SegmentTypes...>>;

 public:
  using value_type = typename first_segment::value_type;
  using segment_variant = std::variant<SegmentTypes...>;
  template <typename S>
  void push_back(const S& seg) {
    static_assert(one_of<S, SegmentTypes...>::value, "segment type not listed in the IndexSet");
    segs_.emplace_back(seg);
  }
  template <typename S>
  void push_front(const S& seg) {
    static_assert(one_of<S, SegmentTypes...>::value, "segment type not listed in the IndexSet");
    segs_.insert(segs_.begin(), segment_variant(seg));
  }
  size_t getNumSegments() const { return segs_.size(); }
  // total number of indices
  size_t getLength() const {
    size_t n = 0;
    for (const auto& v : segs_)
      n += size_t(std::visit([](const auto& g) { return Index_type(stripIndexType(g.size())); }, v));
    return n;
  }
  // position of segment i's first index in the whole traversal
  Index_type getStartingIcount(size_t i) const {
    Index_type n = 0;
    for (size_t k = 0; k < i && k < segs_.size(); ++k)
      n += std::visit([](const auto& g) { return Index_type(stripIndexType(g.size())); }, segs_[k]);
    return n;
  }
  template <typename S>
  const S& getSegment(size_t i) const {
    return std::get<S>(segs_.at(i));
  }
  const std::vector<segment_variant>& segments() const { return segs_; }

 private:
  std::vector<segment_variant> segs_;
};
using IndexSet = TypedIndexSet<RangeSegment, ListSegment, RangeStrideSegment>;

// Element k of a segment, and its length (loop executors, forall params).
namespace detail {
template <typename T>
RAJA_HOST_DEVICE Index_type seg_len(const TypedRangeSegment<T>& s) { return Index_type(stripIndexType(s.e - s.b)); }
template <typename T>
RAJA_HOST_DEVICE T seg_at(const TypedRangeSegment<T>& s, Index_type k) { return T(s.b + T(k)); }
template <typename T>
RAJA_HOST_DEVICE Index_type seg_len(const TypedRangeStrideSegment<T>& s) { return Index_type(stripIndexType(s.size())); }
template <typename T>
RAJA_HOST_DEVICE T seg_at(const TypedRangeStrideSegment<T>& s, Index_type k) { return T(s.b + T(k) * s.s); }
template <typename T>
RAJA_HOST_DEVICE Index_type seg_len(const TypedListSegment<T>& s) { return s.len; }
template <typename T>
RAJA_HOST_DEVICE T seg_at(const TypedListSegment<T>& s, Index_type k) { return s.data[k]; }
// Tile t of size `ts` of a range segment (the last one may be short).
template <typename T>
RAJA_HOST_DEVICE TypedRangeSegment<T> seg_tile(const TypedRangeSegment<T>& s, Index_type ts, Index_type t) {
  const Index_type lo = t * ts, n = seg_len(s);
  return TypedRangeSegment<T>(T(s.b + T(lo)), T(s.b + T(lo + ts < n ? lo + ts : n)));
}
}  // namespace detail

// ---------------------------------------------------------------- spans
template <typename T>
struct Span {
  T* ptr;
  Index_type n;
  T* begin() const { return ptr; }
  T* end() const { return ptr + n; }
  Index_type size() const { return n; }
};
template <typename T>
Span<T> make_span(T* p, Index_type n) { return Span<T>{p, n}; }

// ------------------------------------------------------------ policies
struct seq_exec {};
struct simd_exec {};  // policy/simd/policy.hpp:41: the sequential loop, vectorised by the compiler
struct omp_parallel_for_exec {};
// OpenMP loop schedules (policy/openmp/policy.hpp:238-252); a chunk size of
// 0 leaves it to the runtime
enum class omp_schedule { static_, dynamic_, guided_ };
template <omp_schedule S, int Chunk>
struct omp_parallel_for_schedule_exec {};
template <int Chunk = 0>
using omp_parallel_for_static_exec = omp_parallel_for_schedule_exec<omp_schedule::static_, Chunk>;
template <int Chunk = 0>
using omp_parallel_for_dynamic_exec = omp_parallel_for_schedule_exec<omp_schedule::dynamic_, Chunk>;
template <int Chunk = 0>
using omp_parallel_for_guided_exec = omp_parallel_for_schedule_exec<omp_schedule::guided_, Chunk>;
struct seq_reduce {};
struct omp_reduce {};
struct seq_multi_reduce {};
struct seq_atomic {};
// IndexSet execution (policy/sequential/policy.hpp, policy/openmp/policy.hpp,
// index/IndexSet.hpp): ExecPolicy<SegIt, SegExec> walks an IndexSet's
// segments with SegIt (in order: seq_segit; spread over OpenMP threads:
// omp_parallel_segit) and runs each segment with SegExec.
struct seq_segit {};
struct omp_parallel_segit {};
template <typename SEG_IT, typename SEG_EXEC>
struct ExecPolicy {
  using seg_it = SEG_IT;
  using seg_exec = SEG_EXEC;
};
struct omp_atomic {};

// ------------------------------------------------------------ resources
// RAJA::resources (util/resource.hpp:37-64) re-exports camp's resources
// (the camp submodule, github.com/llnl/camp, not vendored in the reference
// tree).  This restates the part the primitive path uses, following its
// call sites in pattern/forall.hpp:545-627, pattern/scan.hpp:49-441,
// pattern/sort.hpp:54-451 and the resource unit tests
// (test/unit/resource/tests/*.hpp):
//   - a concrete resource (Host here; back-ends add theirs) allocates,
//     copies and sets memory in its own order, hands out events, waits
//     for its own work (wait) or for an event (wait_for);
//   - Resource and Event erase the concrete types; copies share the same
//     underlying resource or event;
//   - every forall / scan / sort returns EventProxy<Res>, which becomes an
//     Event (recorded on the resource at that point) when converted.
// A back-end is told which resource a call runs on through
// bind_resource(res): the returned guard keeps the binding for the call.
namespace resources {

enum class Platform { undefined = 0, host = 1, cuda = 2 };
enum class MemoryAccess { Unknown, Device, Pinned, Managed };

struct EventProxyBase {};

struct HostEvent {
  bool check() const { return true; }
  void wait() const {}
};

class Event {
  struct Concept {
    virtual ~Concept() = default;
    virtual bool check() const = 0;
    virtual void wait() const = 0;
  };
  template <typename E>
  struct Model final : Concept {
    explicit Model(E e) : ev(std::move(e)) {}
    bool check() const override { return ev.check(); }
    void wait() const override { ev.wait(); }
    E ev;
  };
  std::shared_ptr<Concept> m_;

 public:
  Event() = default;  // an event that has already happened
  template <typename E, typename std::enable_if<!std::is_same<std::decay_t<E>, Event>::value &&
                                                    !std::is_base_of<EventProxyBase, std::decay_t<E>>::value,
                                                int>::type = 0>
  Event(E e) : m_(std::make_shared<Model<std::decay_t<E>>>(std::move(e))) {}
  bool check() const { return !m_ || m_->check(); }
  void wait() const {
    if (m_) m_->wait();
  }
  template <typename E>
  const E* try_get() const {
    auto* m = dynamic_cast<const Model<E>*>(m_.get());
    return m ? &m->ev : nullptr;
  }
  template <typename E>
  E get() const {
    const E* e = try_get<E>();
    if (!e) throw std::runtime_error("resources::Event::get: the event is of another type");
    return *e;
  }
};

class Host {
 public:
  static Host get_default() { return Host{}; }
  Platform get_platform() const { return Platform::host; }
  template <typename T>
  T* allocate(size_t n, MemoryAccess = MemoryAccess::Device) {
    return static_cast<T*>(std::malloc(n * sizeof(T)));
  }
  void* calloc(size_t bytes, MemoryAccess = MemoryAccess::Device) { return std::calloc(1, bytes); }
  void deallocate(void* p, MemoryAccess = MemoryAccess::Device) { std::free(p); }
  void memcpy(void* dst, const void* src, size_t bytes) {
    if (bytes) std::memcpy(dst, src, bytes);
  }
  void memset(void* p, int v, size_t bytes) {
    if (bytes) std::memset(p, v, bytes);
  }
  HostEvent get_event() { return {}; }
  Event get_event_erased() { return Event{HostEvent{}}; }
  void wait() {}
  void wait_for(Event* e) { e->wait(); }
};

// Host work binds nothing.
struct NoBinding {};
inline NoBinding bind_resource(Host&) { return {}; }

class Resource {
  struct Concept {
    virtual ~Concept() = default;
    virtual Platform platform() const = 0;
    virtual void* alloc(size_t bytes, MemoryAccess ma) = 0;
    virtual void* zalloc(size_t bytes, MemoryAccess ma) = 0;
    virtual void dealloc(void* p, MemoryAccess ma) = 0;
    virtual void copy(void* dst, const void* src, size_t bytes) = 0;
    virtual void set(void* p, int v, size_t bytes) = 0;
    virtual Event event() = 0;
    virtual void wait() = 0;
    virtual void wait_for(Event* e) = 0;
    virtual std::shared_ptr<void> bind() = 0;
  };
  template <typename R>
  struct Model final : Concept {
    explicit Model(R res) : r(std::move(res)) {}
    Platform platform() const override { return r.get_platform(); }
    void* alloc(size_t bytes, MemoryAccess ma) override { return r.template allocate<char>(bytes, ma); }
    void* zalloc(size_t bytes, MemoryAccess ma) override { return r.calloc(bytes, ma); }
    void dealloc(void* p, MemoryAccess ma) override { r.deallocate(p, ma); }
    void copy(void* dst, const void* src, size_t bytes) override { r.memcpy(dst, src, bytes); }
    void set(void* p, int v, size_t bytes) override { r.memset(p, v, bytes); }
    Event event() override { return r.get_event_erased(); }
    void wait() override { r.wait(); }
    void wait_for(Event* e) override { r.wait_for(e); }
    std::shared_ptr<void> bind() override {
      using G = decltype(bind_resource(r));
      return std::make_shared<G>(bind_resource(r));
    }
    R r;
  };
  std::shared_ptr<Concept> m_;

 public:
  template <typename R, typename std::enable_if<!std::is_same<std::decay_t<R>, Resource>::value, int>::type = 0>
  Resource(R r) : m_(std::make_shared<Model<std::decay_t<R>>>(std::move(r))) {}
  Platform get_platform() const { return m_->platform(); }
  template <typename T>
  T* allocate(size_t n, MemoryAccess ma = MemoryAccess::Device) {
    return static_cast<T*>(m_->alloc(n * sizeof(T), ma));
  }
  void* calloc(size_t bytes, MemoryAccess ma = MemoryAccess::Device) { return m_->zalloc(bytes, ma); }
  void deallocate(void* p, MemoryAccess ma = MemoryAccess::Device) { m_->dealloc(p, ma); }
  void memcpy(void* dst, const void* src, size_t bytes) { m_->copy(dst, src, bytes); }
  void memset(void* p, int v, size_t bytes) { m_->set(p, v, bytes); }
  Event get_event() { return m_->event(); }
  Event get_event_erased() { return m_->event(); }
  void wait() { m_->wait(); }
  void wait_for(Event* e) { m_->wait_for(e); }
  template <typename R>
  R* try_get() {
    auto* m = dynamic_cast<Model<R>*>(m_.get());
    return m ? &m->r : nullptr;
  }
  template <typename R>
  R get() {
    R* r = try_get<R>();
    if (!r) throw std::runtime_error("resources::Resource::get: the resource is of another type");
    return *r;
  }
  friend std::shared_ptr<void> bind_resource(Resource& r) { return r.m_->bind(); }
};

// EventProxy<Res>: what an asynchronous call returns.  Converting it to an
// Event (or to the resource's own event type) records an event on the
// resource at that point; get() does the same.
template <typename Res>
class EventProxy : public EventProxyBase {
  using native_event = decltype(std::declval<Res&>().get_event());

 public:
  explicit EventProxy(Res r) : r_(std::move(r)) {}
  Event get() const { return r_.get_event_erased(); }
  operator Event() const { return get(); }
  template <typename E, typename std::enable_if<std::is_same<E, native_event>::value &&
                                                    !std::is_same<E, Event>::value,
                                                int>::type = 0>
  operator E() const {
    return r_.get_event();
  }
  Res resource() const { return r_; }

 private:
  mutable Res r_;
};

template <typename T>
struct is_resource : std::false_type {};
template <>
struct is_resource<Host> : std::true_type {};
template <>
struct is_resource<Resource> : std::true_type {};

// Resource type of an execution policy (util/resource.hpp:44-58); host
// policies run on Host, back-ends specialise for theirs.
template <typename Pol>
struct get_resource {
  using type = Host;
};
// an IndexSet policy runs on its segment policy's resource
template <typename SEG_IT, typename SEG_EXEC>
struct get_resource<ExecPolicy<SEG_IT, SEG_EXEC>> {
  using type = typename get_resource<SEG_EXEC>::type;
};
template <typename Pol>
typename get_resource<Pol>::type get_default_resource() {
  return get_resource<Pol>::type::get_default();
}

}  // namespace resources

namespace detail {
template <typename T>
using enable_if_resource = typename std::enable_if<resources::is_resource<std::decay_t<T>>::value, int>::type;
template <typename T>
using enable_if_not_resource =
    typename std::enable_if<!resources::is_resource<std::decay_t<T>>::value, int>::type;
}  // namespace detail

namespace expt {
// ---- ValLoc / ValOp / KernelName (pattern/params/params_base.hpp:10-253)
template <typename T, typename IndexType = Index_type>
struct ValLoc {
  using value_type = T;
  using index_type = IndexType;
  T val;
  IndexType loc;
  RAJA_HOST_DEVICE constexpr ValLoc() : val(T()), loc(IndexType(-1)) {}
  RAJA_HOST_DEVICE constexpr ValLoc(T v) : val(v), loc(IndexType(-1)) {}
  RAJA_HOST_DEVICE constexpr ValLoc(T v, IndexType l) : val(v), loc(l) {}
  RAJA_HOST_DEVICE bool operator<(const ValLoc& o) const { return val < o.val; }
  RAJA_HOST_DEVICE bool operator>(const ValLoc& o) const { return val > o.val; }
  RAJA_HOST_DEVICE T getVal() const { return val; }
  RAJA_HOST_DEVICE IndexType getLoc() const { return loc; }
};

template <typename T, template <typename, typename, typename> class Op>
struct ValOp {
  using value_type = T;
  using op_type = Op<T, T, T>;
  T val;
  RAJA_HOST_DEVICE constexpr ValOp() : val(op_type::identity()) {}
  RAJA_HOST_DEVICE constexpr explicit ValOp(T v) : val(v) {}
  RAJA_HOST_DEVICE ValOp& operator+=(const T& r) { val += r; return *this; }
  RAJA_HOST_DEVICE ValOp& operator|=(const T& r) { val |= r; return *this; }
  RAJA_HOST_DEVICE ValOp& operator&=(const T& r) { val &= r; return *this; }
  RAJA_HOST_DEVICE ValOp& min(const T& v) { if (v < val) val = v; return *this; }
  RAJA_HOST_DEVICE ValOp& max(const T& v) { if (val < v) val = v; return *this; }
  RAJA_HOST_DEVICE T get() const { return val; }
};
// ValOp over ValLoc: minloc / maxloc keep the first extreme
template <typename T, typename I, template <typename, typename, typename> class Op>
struct ValOp<ValLoc<T, I>, Op> {
  using value_type = ValLoc<T, I>;
  using op_type = Op<value_type, value_type, value_type>;
  value_type val;
  RAJA_HOST_DEVICE constexpr ValOp() : val(op_type::identity()) {}
  RAJA_HOST_DEVICE ValOp& minloc(const T& v, I l) { if (v < val.val) val = value_type(v, l); return *this; }
  RAJA_HOST_DEVICE ValOp& maxloc(const T& v, I l) { if (val.val < v) val = value_type(v, l); return *this; }
  RAJA_HOST_DEVICE ValOp& min(value_type v) { if (v.val < val.val) val = v; return *this; }
  RAJA_HOST_DEVICE ValOp& max(value_type v) { if (val.val < v.val) val = v; return *this; }
  RAJA_HOST_DEVICE T getVal() const { return val.val; }
  RAJA_HOST_DEVICE I getLoc() const { return val.loc; }
};

// ValLocOp<T, I, Op>: the lambda argument type of a ReduceLoc param
// (pattern/params/params_base.hpp:253)
template <typename T, typename I, template <typename, typename, typename> class Op>
using ValLocOp = ValOp<ValLoc<T, I>, Op>;

// A kernel name param (pattern/params/kernel_name.hpp:11-22: RAJA::Name
// returns one); expt::Name is kept as a second spelling.
struct KernelName {
  const char* name;
};
inline KernelName Name(const char* n) { return KernelName{n}; }

namespace detail {
template <typename Op, typename T, typename VOp>
struct Reducer {
  using op = Op;
  using value_type = T;
  using valop_type = VOp;
  T* target;
  Reducer(T* t) : target(t) {}
  void combineTarget(T in) const { *target = Op{}(*target, in); }
};
template <typename T, typename I, typename Op, typename VOp>
struct ReducerLoc {
  using op = Op;
  using value_type = ValLoc<T, I>;
  using valop_type = VOp;
  T* target;
  I* index;
  ReducerLoc(T* t, I* i) : target(t), index(i) {}
  void combineTarget(value_type in) const {
    value_type cur(*target, *index);
    value_type r = Op{}(cur, in);
    *target = r.val;
    *index = r.loc;
  }
};
template <typename X>
struct is_reducer : std::false_type {};
template <typename Op, typename T, typename VOp>
struct is_reducer<Reducer<Op, T, VOp>> : std::true_type {};
template <typename T, typename I, typename Op, typename VOp>
struct is_reducer<ReducerLoc<T, I, Op, VOp>> : std::true_type {};
}  // namespace detail

// pattern/params/reducer.hpp:220-248
template <template <typename, typename, typename> class Op, typename T>
detail::Reducer<Op<T, T, T>, T, ValOp<T, Op>> Reduce(T* target) {
  return detail::Reducer<Op<T, T, T>, T, ValOp<T, Op>>(target);
}
template <template <typename, typename, typename> class Op, typename T, typename I>
detail::ReducerLoc<T, I, Op<ValLoc<T, I>, ValLoc<T, I>, ValLoc<T, I>>, ValOp<ValLoc<T, I>, Op>>
ReduceLoc(T* target, I* index) {
  return {target, index};
}
}  // namespace expt

inline expt::KernelName Name(const char* n) { return expt::KernelName{n}; }

// operators::limits for ValLoc identities (pattern/detail/reduce.hpp:185-203)
namespace operators {
template <typename T, typename I>
struct limits<expt::ValLoc<T, I>, void> {
  RAJA_HOST_DEVICE static constexpr expt::ValLoc<T, I> min() { return expt::ValLoc<T, I>(limits<T>::min()); }
  RAJA_HOST_DEVICE static constexpr expt::ValLoc<T, I> max() { return expt::ValLoc<T, I>(limits<T>::max()); }
};
}  // namespace operators

// ------------------------------------------------------------- reducers
// Reducer class templates; each policy specialises them.
template <typename POL, typename T> class ReduceSum;
template <typename POL, typename T> class ReduceMin;
template <typename POL, typename T> class ReduceMax;
template <typename POL, typename T, typename I = Index_type> class ReduceMinLoc;
template <typename POL, typename T, typename I = Index_type> class ReduceMaxLoc;
template <typename POL, typename T> class ReduceBitOr;
template <typename POL, typename T> class ReduceBitAnd;

namespace detail {
// BaseCombinable semantics (pattern/detail/reduce.hpp:287-358): a copy
// starts at the identity and folds into its parent when destroyed; the
// parent holds init.  Host policies only.
template <typename T, typename Op>
class HostCombinable {
 protected:
  const HostCombinable* parent = nullptr;
  T identity;
  mutable T my;
  mutable std::shared_ptr<std::vector<T>> omp_parts;  // omp: thread partials

 public:
  HostCombinable(T init, T ident) : identity(ident), my(init) {}
  HostCombinable(const HostCombinable& o)
      : parent(o.parent ? o.parent : &o), identity(o.identity), my(o.identity) {}
  ~HostCombinable() {
    if (parent) {
#if defined(_OPENMP)
#pragma omp critical(raja_compat_reduce)
#endif
      parent->my = Op{}(parent->my, my);
    }
  }
  void combine(const T& v) const { my = Op{}(my, v); }
  T get() const { return my; }
  void reset(T init, T ident) {
    my = init;
    identity = ident;
  }
};
}  // namespace detail

#define RAJA_COMPAT_HOST_REDUCERS(POL)                                                           \
  template <typename T>                                                                          \
  class ReduceSum<POL, T> : public detail::HostCombinable<T, operators::plus<T>> {               \
    using B = detail::HostCombinable<T, operators::plus<T>>;                                     \
                                                                                                 \
   public:                                                                                       \
    explicit ReduceSum(T init = T(0)) : B(init, T(0)) {}                                         \
    const ReduceSum& operator+=(T v) const { this->combine(v); return *this; }                   \
    T get() const { return B::get(); }                                                           \
    operator T() const { return get(); }                                                         \
    void reset(T v) { B::reset(v, T(0)); }                                                       \
  };                                                                                             \
  template <typename T>                                                                          \
  class ReduceMin<POL, T> : public detail::HostCombinable<T, operators::minimum<T>> {            \
    using B = detail::HostCombinable<T, operators::minimum<T>>;                                  \
                                                                                                 \
   public:                                                                                       \
    explicit ReduceMin(T init = operators::limits<T>::max()) : B(init, operators::limits<T>::max()) {} \
    const ReduceMin& min(T v) const { this->combine(v); return *this; }                          \
    T get() const { return B::get(); }                                                           \
    operator T() const { return get(); }                                                         \
  };                                                                                             \
  template <typename T>                                                                          \
  class ReduceMax<POL, T> : public detail::HostCombinable<T, operators::maximum<T>> {            \
    using B = detail::HostCombinable<T, operators::maximum<T>>;                                  \
                                                                                                 \
   public:                                                                                       \
    explicit ReduceMax(T init = operators::limits<T>::min()) : B(init, operators::limits<T>::min()) {} \
    const ReduceMax& max(T v) const { this->combine(v); return *this; }                          \
    T get() const { return B::get(); }                                                           \
    operator T() const { return get(); }                                                         \
  };                                                                                             \
  template <typename T, typename I>                                                              \
  class ReduceMinLoc<POL, T, I>                                                                  \
      : public detail::HostCombinable<expt::ValLoc<T, I>, operators::minimum<expt::ValLoc<T, I>>> { \
    using VL = expt::ValLoc<T, I>;                                                               \
    using B = detail::HostCombinable<VL, operators::minimum<VL>>;                                \
                                                                                                 \
   public:                                                                                       \
    ReduceMinLoc(T init, I idx) : B(VL(init, idx), VL(operators::limits<T>::max(), I(-1))) {}    \
    const ReduceMinLoc& minloc(T v, I l) const { this->combine(VL(v, l)); return *this; }        \
    T get() const { return B::get().val; }                                                       \
    I getLoc() const { return B::get().loc; }                                                    \
    operator T() const { return get(); }                                                         \
    void reset(T v, I l) { B::reset(VL(v, l), VL(operators::limits<T>::max(), I(-1))); }         \
  };                                                                                             \
  template <typename T, typename I>                                                              \
  class ReduceMaxLoc<POL, T, I>                                                                  \
      : public detail::HostCombinable<expt::ValLoc<T, I>, operators::maximum<expt::ValLoc<T, I>>> { \
    using VL = expt::ValLoc<T, I>;                                                               \
    using B = detail::HostCombinable<VL, operators::maximum<VL>>;                                \
                                                                                                 \
   public:                                                                                       \
    ReduceMaxLoc(T init, I idx) : B(VL(init, idx), VL(operators::limits<T>::min(), I(-1))) {}    \
    const ReduceMaxLoc& maxloc(T v, I l) const { this->combine(VL(v, l)); return *this; }        \
    T get() const { return B::get().val; }                                                       \
    I getLoc() const { return B::get().loc; }                                                    \
    operator T() const { return get(); }                                                         \
    void reset(T v, I l) { B::reset(VL(v, l), VL(operators::limits<T>::min(), I(-1))); }         \
  };                                                                                             \
  template <typename T>                                                                          \
  class ReduceBitOr<POL, T> : public detail::HostCombinable<T, operators::bit_or<T>> {           \
    using B = detail::HostCombinable<T, operators::bit_or<T>>;                                   \
                                                                                                 \
   public:                                                                                       \
    explicit ReduceBitOr(T init = T(0)) : B(init, T(0)) {}                                       \
    const ReduceBitOr& operator|=(T v) const { this->combine(v); return *this; }                 \
    T get() const { return B::get(); }                                                           \
    operator T() const { return get(); }                                                         \
  };                                                                                             \
  template <typename T>                                                                          \
  class ReduceBitAnd<POL, T> : public detail::HostCombinable<T, operators::bit_and<T>> {         \
    using B = detail::HostCombinable<T, operators::bit_and<T>>;                                  \
                                                                                                 \
   public:                                                                                       \
    explicit ReduceBitAnd(T init = T(~T(0))) : B(init, T(~T(0))) {}                              \
    const ReduceBitAnd& operator&=(T v) const { this->combine(v); return *this; }                \
    T get() const { return B::get(); }                                                           \
    operator T() const { return get(); }                                                         \
  };

RAJA_COMPAT_HOST_REDUCERS(seq_reduce)
RAJA_COMPAT_HOST_REDUCERS(omp_reduce)
#undef RAJA_COMPAT_HOST_REDUCERS

// ---------------------------------------------------------- multi reduce
// MultiReduce{Sum,Min,Max,BitOr,BitAnd}<POL, T> (pattern/multi_reduce.hpp:
// 68-190, pattern/detail/multi_reduce.hpp:60-402): num_bins values, each
// starting at init; mr[bin] += v / .min(v) / .max(v) / |= v / &= v combine
// with the op's rule (min: `if (v < val) val = v`, max: `if (val < v) val =
// v`); get(bin), get_all(container), reset(), size().  Copies (the loop
// body's capture) combine into the same bins.
template <typename POL, typename T> class MultiReduceSum;
template <typename POL, typename T> class MultiReduceMin;
template <typename POL, typename T> class MultiReduceMax;
template <typename POL, typename T> class MultiReduceBitOr;
template <typename POL, typename T> class MultiReduceBitAnd;

namespace detail {
template <typename T> struct MrSum { static T ident() { return T(0); } void operator()(T& a, T v) const { a += v; } };
template <typename T> struct MrMin { static T ident() { return operators::limits<T>::max(); } void operator()(T& a, T v) const { if (v < a) a = v; } };
template <typename T> struct MrMax { static T ident() { return operators::limits<T>::min(); } void operator()(T& a, T v) const { if (a < v) a = v; } };
template <typename T> struct MrOr { static T ident() { return T(0); } void operator()(T& a, T v) const { a |= v; } };
template <typename T> struct MrAnd { static T ident() { return T(~T(0)); } void operator()(T& a, T v) const { a &= v; } };

template <typename T, typename Op>
class HostMultiReduce {
 public:
  using value_type = T;
  HostMultiReduce(size_t num_bins, T init) : data_(std::make_shared<std::vector<T>>(num_bins, init)) {}
  explicit HostMultiReduce(size_t num_bins) : HostMultiReduce(num_bins, Op::ident()) {}
  template <typename Container, typename = decltype(std::declval<const Container&>().begin())>
  explicit HostMultiReduce(const Container& c)
      : data_(std::make_shared<std::vector<T>>(c.begin(), c.end())) {}
  size_t size() const { return data_->size(); }
  T get(size_t bin) const { return (*data_)[bin]; }
  template <typename Container>
  void get_all(Container& c) const {
    size_t b = 0;
    for (auto& v : c) v = get(b++);
  }
  void reset() { std::fill(data_->begin(), data_->end(), Op::ident()); }
  void reset(size_t num_bins, T init = Op::ident()) { data_->assign(num_bins, init); }
  void combine(size_t bin, T v) const { Op{}((*data_)[bin], v); }

 private:
  std::shared_ptr<std::vector<T>> data_;
};
}  // namespace detail

#define RAJA_COMPAT_HOST_MULTI_REDUCER(CLS, OPK, METHOD, RET)                                  \
  template <typename T>                                                                        \
  class CLS<seq_multi_reduce, T> : public detail::HostMultiReduce<T, detail::OPK<T>> {           \
    using B = detail::HostMultiReduce<T, detail::OPK<T>>;                                      \
                                                                                               \
   public:                                                                                     \
    using B::B;                                                                                \
    struct reference {                                                                         \
      const B* mr;                                                                             \
      size_t bin;                                                                              \
      RET METHOD(T v) const { mr->combine(bin, v); return *this; }                              \
      T get() const { return mr->get(bin); }                                                   \
    };                                                                                         \
    reference operator[](size_t bin) const { return reference{this, bin}; }                    \
  };
RAJA_COMPAT_HOST_MULTI_REDUCER(MultiReduceSum, MrSum, operator+=, const reference&)
RAJA_COMPAT_HOST_MULTI_REDUCER(MultiReduceMin, MrMin, min, const reference&)
RAJA_COMPAT_HOST_MULTI_REDUCER(MultiReduceMax, MrMax, max, const reference&)
RAJA_COMPAT_HOST_MULTI_REDUCER(MultiReduceBitOr, MrOr, operator|=, const reference&)
RAJA_COMPAT_HOST_MULTI_REDUCER(MultiReduceBitAnd, MrAnd, operator&=, const reference&)
#undef RAJA_COMPAT_HOST_MULTI_REDUCER

// --------------------------------------------------------------- atomics
// RAJA::atomicX<Policy>(acc, ...) dispatches to atomicX(Policy{}, acc, ...)
// (pattern/atomic.hpp:90-286); seq_atomic is plain read-modify-write
// (policy/sequential/atomic.hpp:37-170).  Each returns the value before the
// operation.
template <typename T> RAJA_HOST_DEVICE T atomicLoad(seq_atomic, T* acc) { return *acc; }
template <typename T> RAJA_HOST_DEVICE void atomicStore(seq_atomic, T* acc, T v) { *acc = v; }
template <typename T> RAJA_HOST_DEVICE T atomicAdd(seq_atomic, T* acc, T v) { T o = *acc; *acc = o + v; return o; }
template <typename T> RAJA_HOST_DEVICE T atomicSub(seq_atomic, T* acc, T v) { T o = *acc; *acc = o - v; return o; }
template <typename T> RAJA_HOST_DEVICE T atomicMin(seq_atomic, T* acc, T v) { T o = *acc; if (v < o) *acc = v; return o; }
template <typename T> RAJA_HOST_DEVICE T atomicMax(seq_atomic, T* acc, T v) { T o = *acc; if (o < v) *acc = v; return o; }
template <typename T> RAJA_HOST_DEVICE T atomicInc(seq_atomic, T* acc) { T o = *acc; *acc = o + T(1); return o; }
template <typename T> RAJA_HOST_DEVICE T atomicInc(seq_atomic, T* acc, T val) { T o = *acc; *acc = val <= o ? T(0) : o + T(1); return o; }
template <typename T> RAJA_HOST_DEVICE T atomicDec(seq_atomic, T* acc) { T o = *acc; *acc = o - T(1); return o; }
template <typename T> RAJA_HOST_DEVICE T atomicDec(seq_atomic, T* acc, T val) { T o = *acc; *acc = (o == T(0) || val < o) ? val : o - T(1); return o; }
template <typename T> RAJA_HOST_DEVICE T atomicAnd(seq_atomic, T* acc, T v) { T o = *acc; *acc = o & v; return o; }
template <typename T> RAJA_HOST_DEVICE T atomicOr(seq_atomic, T* acc, T v) { T o = *acc; *acc = o | v; return o; }
template <typename T> RAJA_HOST_DEVICE T atomicXor(seq_atomic, T* acc, T v) { T o = *acc; *acc = o ^ v; return o; }
template <typename T> RAJA_HOST_DEVICE T atomicExchange(seq_atomic, T* acc, T v) { T o = *acc; *acc = v; return o; }
template <typename T> RAJA_HOST_DEVICE T atomicCAS(seq_atomic, T* acc, T compare, T v) { T o = *acc; if (o == compare) *acc = v; return o; }

// omp_atomic (policy/openmp/atomic.hpp:37-93): host atomics, safe under
// omp_parallel_for_exec.  Every operation is a compare-exchange loop on the
// value's bits with the compiler's __atomic builtins, so it covers
// floating-point types too.  Host code only.
namespace detail {
template <typename T, typename F>
inline T host_atomic_update(T* acc, F next) {
  T old;
  __atomic_load(acc, &old, __ATOMIC_RELAXED);
  T want = next(old);
  while (!__atomic_compare_exchange(acc, &old, &want, true, __ATOMIC_SEQ_CST, __ATOMIC_RELAXED)) want = next(old);
  return old;
}
}  // namespace detail
template <typename T> inline T atomicLoad(omp_atomic, T* acc) { T v; __atomic_load(acc, &v, __ATOMIC_SEQ_CST); return v; }
template <typename T> inline void atomicStore(omp_atomic, T* acc, T v) { __atomic_store(acc, &v, __ATOMIC_SEQ_CST); }
template <typename T> inline T atomicAdd(omp_atomic, T* acc, T v) { return detail::host_atomic_update(acc, [v](T o) { return T(o + v); }); }
template <typename T> inline T atomicSub(omp_atomic, T* acc, T v) { return detail::host_atomic_update(acc, [v](T o) { return T(o - v); }); }
template <typename T> inline T atomicMin(omp_atomic, T* acc, T v) { return detail::host_atomic_update(acc, [v](T o) { return v < o ? v : o; }); }
template <typename T> inline T atomicMax(omp_atomic, T* acc, T v) { return detail::host_atomic_update(acc, [v](T o) { return o < v ? v : o; }); }
template <typename T> inline T atomicInc(omp_atomic, T* acc) { return detail::host_atomic_update(acc, [](T o) { return T(o + T(1)); }); }
template <typename T> inline T atomicInc(omp_atomic, T* acc, T val) { return detail::host_atomic_update(acc, [val](T o) { return val <= o ? T(0) : T(o + T(1)); }); }
template <typename T> inline T atomicDec(omp_atomic, T* acc) { return detail::host_atomic_update(acc, [](T o) { return T(o - T(1)); }); }
template <typename T> inline T atomicDec(omp_atomic, T* acc, T val) { return detail::host_atomic_update(acc, [val](T o) { return (o == T(0) || val < o) ? val : T(o - T(1)); }); }
template <typename T> inline T atomicAnd(omp_atomic, T* acc, T v) { return detail::host_atomic_update(acc, [v](T o) { return T(o & v); }); }
template <typename T> inline T atomicOr(omp_atomic, T* acc, T v) { return detail::host_atomic_update(acc, [v](T o) { return T(o | v); }); }
template <typename T> inline T atomicXor(omp_atomic, T* acc, T v) { return detail::host_atomic_update(acc, [v](T o) { return T(o ^ v); }); }
template <typename T> inline T atomicExchange(omp_atomic, T* acc, T v) { T o; __atomic_exchange(acc, &v, &o, __ATOMIC_SEQ_CST); return o; }
template <typename T> inline T atomicCAS(omp_atomic, T* acc, T compare, T v) {
  __atomic_compare_exchange(acc, &compare, &v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return compare;  // the value found: equal to the old compare when the swap happened
}

template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicLoad(T* acc) { return atomicLoad(Policy{}, acc); }
template <typename Policy, typename T> RAJA_HOST_DEVICE void atomicStore(T* acc, T v) { atomicStore(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicAdd(T* acc, T v) { return atomicAdd(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicSub(T* acc, T v) { return atomicSub(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicMin(T* acc, T v) { return atomicMin(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicMax(T* acc, T v) { return atomicMax(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicInc(T* acc) { return atomicInc(Policy{}, acc); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicInc(T* acc, T val) { return atomicInc(Policy{}, acc, val); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicDec(T* acc) { return atomicDec(Policy{}, acc); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicDec(T* acc, T val) { return atomicDec(Policy{}, acc, val); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicAnd(T* acc, T v) { return atomicAnd(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicOr(T* acc, T v) { return atomicOr(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicXor(T* acc, T v) { return atomicXor(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicExchange(T* acc, T v) { return atomicExchange(Policy{}, acc, v); }
template <typename Policy, typename T> RAJA_HOST_DEVICE T atomicCAS(T* acc, T compare, T v) { return atomicCAS(Policy{}, acc, compare, v); }

// AtomicRef<T, Policy> (pattern/atomic.hpp:299-): a pointer with atomic
// member operations; fetch_* return the previous value, the operators the
// new one.
template <typename T, typename Policy = seq_atomic>
class AtomicRef {
 public:
  using value_type = T;
  RAJA_HOST_DEVICE explicit AtomicRef(T* p) : p_(p) {}
  RAJA_HOST_DEVICE T* getPointer() const { return p_; }
  RAJA_HOST_DEVICE void store(T v) const { atomicStore(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T load() const { return atomicLoad(Policy{}, p_); }
  RAJA_HOST_DEVICE operator T() const { return load(); }
  RAJA_HOST_DEVICE T operator=(T v) const { store(v); return v; }
  RAJA_HOST_DEVICE T exchange(T v) const { return atomicExchange(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T CAS(T compare, T v) const { return atomicCAS(Policy{}, p_, compare, v); }
  RAJA_HOST_DEVICE bool compare_exchange_strong(T& expect, T v) const {
    const T o = atomicCAS(Policy{}, p_, expect, v);
    const bool ok = o == expect;
    expect = o;
    return ok;
  }
  RAJA_HOST_DEVICE T fetch_add(T v) const { return atomicAdd(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T fetch_sub(T v) const { return atomicSub(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T fetch_min(T v) const { return atomicMin(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T fetch_max(T v) const { return atomicMax(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T fetch_and(T v) const { return atomicAnd(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T fetch_or(T v) const { return atomicOr(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T fetch_xor(T v) const { return atomicXor(Policy{}, p_, v); }
  RAJA_HOST_DEVICE T operator++() const { return atomicInc(Policy{}, p_) + T(1); }
  RAJA_HOST_DEVICE T operator++(int) const { return atomicInc(Policy{}, p_); }
  RAJA_HOST_DEVICE T operator--() const { return atomicDec(Policy{}, p_) - T(1); }
  RAJA_HOST_DEVICE T operator--(int) const { return atomicDec(Policy{}, p_); }
  RAJA_HOST_DEVICE T operator+=(T v) const { return atomicAdd(Policy{}, p_, v) + v; }
  RAJA_HOST_DEVICE T operator-=(T v) const { return atomicSub(Policy{}, p_, v) - v; }
  RAJA_HOST_DEVICE T operator&=(T v) const { return atomicAnd(Policy{}, p_, v) & v; }
  RAJA_HOST_DEVICE T operator|=(T v) const { return atomicOr(Policy{}, p_, v) | v; }
  RAJA_HOST_DEVICE T operator^=(T v) const { return atomicXor(Policy{}, p_, v) ^ v; }
  RAJA_HOST_DEVICE T min(T v) const { const T o = atomicMin(Policy{}, p_, v); return v < o ? v : o; }
  RAJA_HOST_DEVICE T max(T v) const { const T o = atomicMax(Policy{}, p_, v); return o < v ? v : o; }

 private:
  T* p_;
};

// ---------------------------------------------------------------- forall
// Host implementations (policy/sequential/forall.hpp:58-102,
// policy/openmp/forall.hpp:129-260).  The loop body is copied once per
// thread, like thread_privatize, so captured reducers fold on destruction.
template <typename Body, typename T>
void forall_impl(seq_exec, const TypedRangeSegment<T>& r, Body&& body) {
  auto b = body;
  for (T i = r.b; i < r.e; ++i) b(i);
}
template <typename Body, typename T>
void forall_impl(seq_exec, const TypedRangeStrideSegment<T>& r, Body&& body) {
  auto b = body;
  const Index_type n = r.size();
  for (Index_type k = 0; k < n; ++k) b(T(r.b + k * r.s));
}
template <typename Body, typename T>
void forall_impl(seq_exec, const TypedListSegment<T>& l, Body&& body) {
  auto b = body;
  for (Index_type k = 0; k < l.len; ++k) b(l.data[k]);
}
template <typename Body, typename T>
void forall_impl(omp_parallel_for_exec, const TypedRangeSegment<T>& r, Body&& body) {
#if defined(_OPENMP)
#pragma omp parallel
  {
    auto b = body;
    const Index_type n = detail::seg_len(r);  // an integer loop: T may be a strongly typed index
#pragma omp for schedule(static)
    for (Index_type k = 0; k < n; ++k) b(detail::seg_at(r, k));
  }
#else
  forall_impl(seq_exec{}, r, body);
#endif
}
// omp_parallel_for_exec over list and strided segments (range segments
// have their own overload above)
template <typename Seg, typename Body, typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_impl(omp_parallel_for_exec, const Seg& seg, Body&& body) {
  const Index_type n = detail::seg_len(seg);
#if defined(_OPENMP)
#pragma omp parallel
  {
    auto b = body;
#pragma omp for schedule(static)
    for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
  }
#else
  auto b = body;
  for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
#endif
}
// simd_exec: the sequential loop (any segment kind)
template <typename Seg, typename Body, typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_impl(simd_exec, const Seg& seg, Body&& body) {
  auto b = body;
  const Index_type n = detail::seg_len(seg);
#if defined(_OPENMP)
#pragma omp simd
#endif
  for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
}
// scheduled OpenMP loops over any segment kind; the body is copied once per
// thread, as for omp_parallel_for_exec
template <omp_schedule S, int Chunk, typename Seg, typename Body,
          typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_impl(omp_parallel_for_schedule_exec<S, Chunk>, const Seg& seg, Body&& body) {
  const Index_type n = detail::seg_len(seg);
#if defined(_OPENMP)
#pragma omp parallel
  {
    auto b = body;
    if (S == omp_schedule::static_) {
      if (Chunk > 0) {
#pragma omp for schedule(static, Chunk > 0 ? Chunk : 1)
        for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
      } else {
#pragma omp for schedule(static)
        for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
      }
    } else if (S == omp_schedule::dynamic_) {
#pragma omp for schedule(dynamic, Chunk > 0 ? Chunk : 1)
      for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
    } else {
#pragma omp for schedule(guided, Chunk > 0 ? Chunk : 1)
      for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
    }
  }
#else
  auto b = body;
  for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
#endif
}

// Work-sharing loops for use inside RAJA::region<omp_parallel_region>
// (policy/openmp/policy.hpp: omp_for_exec, omp_for_static_exec,
// omp_for_nowait_static_exec): an `omp for` with no parallel region of its
// own, so the threads of the enclosing region share the iterations.
// Outside a region the calling thread runs them all.
struct omp_for_exec {};
template <int Chunk = 0>
struct omp_for_static_exec {};
template <int Chunk = 0>
struct omp_for_nowait_static_exec {};
namespace detail {
template <bool NOWAIT, int Chunk, typename Seg, typename Body>
void omp_for_loop(const Seg& seg, const Body& body) {
  const Index_type n = detail::seg_len(seg);
  auto b = body;
#if defined(_OPENMP)
  if (NOWAIT) {
#pragma omp for schedule(static, Chunk > 0 ? Chunk : 1) nowait
    for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
  } else if (Chunk > 0) {
#pragma omp for schedule(static, Chunk > 0 ? Chunk : 1)
    for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
  } else {
#pragma omp for schedule(static)
    for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
  }
#else
  for (Index_type k = 0; k < n; ++k) b(detail::seg_at(seg, k));
#endif
}
}  // namespace detail
template <typename Seg, typename Body, typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_impl(omp_for_exec, const Seg& seg, Body&& body) {
  detail::omp_for_loop<false, 0>(seg, body);
}
template <int Chunk, typename Seg, typename Body, typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_impl(omp_for_static_exec<Chunk>, const Seg& seg, Body&& body) {
  detail::omp_for_loop<false, Chunk>(seg, body);
}
template <int Chunk, typename Seg, typename Body, typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_impl(omp_for_nowait_static_exec<Chunk>, const Seg& seg, Body&& body) {
  detail::omp_for_loop<true, Chunk>(seg, body);
}

// RAJA::region<Pol>(body) (pattern/region.hpp, policy/sequential/region.hpp,
// policy/openmp/region.hpp): seq_region runs body once; omp_parallel_region
// runs it on every thread of one OpenMP parallel region, where the omp_for
// loops above share out their iterations.
struct seq_region {};
struct omp_parallel_region {};
template <typename Pol, typename Body>
void region(Body&& body) {
  if constexpr (std::is_same<Pol, omp_parallel_region>::value) {
#if defined(_OPENMP)
#pragma omp parallel
    {
      body();
    }
#else
    body();
#endif
  } else {
    static_assert(std::is_same<Pol, seq_region>::value, "region policy: seq_region or omp_parallel_region");
    body();
  }
}

template <typename Pol, typename Body, typename... Segs>
void forall_impl(Pol p, const TypedIndexSet<Segs...>& is, Body&& body) {
  for (const auto& s : is.segments()) std::visit([&](const auto& seg) { forall_impl(p, seg, body); }, s);
}
// A single segment under an IndexSet policy runs with the segment policy.
template <typename IT, typename E, typename Seg, typename Body,
          typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_impl(ExecPolicy<IT, E>, const Seg& seg, Body&& body) {
  forall_impl(E{}, seg, std::forward<Body>(body));
}
// ExecPolicy<seq_segit, E>: the segment policy's own IndexSet loop (a
// back-end may fuse the segments into one launch).
template <typename E, typename Body, typename... Segs>
void forall_impl(ExecPolicy<seq_segit, E>, const TypedIndexSet<Segs...>& is, Body&& body) {
  forall_impl(E{}, is, std::forward<Body>(body));
}
// ExecPolicy<omp_parallel_segit, E>: the segments are shared among OpenMP
// threads, each run with E (host policies; the loop body must be safe to
// run for several segments at once).
template <typename E, typename Body, typename... Segs>
void forall_impl(ExecPolicy<omp_parallel_segit, E>, const TypedIndexSet<Segs...>& is, Body&& body) {
  const auto& segs = is.segments();
  const Index_type n = Index_type(segs.size());
#if defined(_OPENMP)
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (Index_type k = 0; k < n; ++k) std::visit([&](const auto& seg) { forall_impl(E{}, seg, body); }, segs[k]);
}

// expt params under an IndexSet policy: each segment runs the segment
// policy's params loop, which folds its result into the targets, so the
// targets end up reduced over every segment.
template <typename IT, typename E, typename Seg, typename Body, typename... Red,
          typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_params_impl(ExecPolicy<IT, E>, const Seg& seg, Body&& body, Red&... reds) {
  forall_params_impl(E{}, seg, body, reds...);
}
template <typename IT, typename E, typename Body, typename... Segs, typename... Red>
void forall_params_impl(ExecPolicy<IT, E>, const TypedIndexSet<Segs...>& is, Body&& body, Red&... reds) {
  for (const auto& s : is.segments())
    std::visit([&](const auto& seg) { forall_params_impl(E{}, seg, body, reds...); }, s);
}

// getIndices / getIndicesConditional (index/IndexSetUtils.hpp:47-120): the
// indices of a segment or IndexSet, in order, into a container with
// push_back (only those for which `conditional(index)` holds).
template <typename CONTAINER_T, typename SEGMENT_T, typename CONDITIONAL>
void getIndicesConditional(CONTAINER_T& con, const SEGMENT_T& seg, CONDITIONAL conditional) {
  CONTAINER_T tcon;
  auto take = [&](typename CONTAINER_T::value_type idx) {
    if (conditional(idx)) tcon.push_back(idx);
  };
  forall_impl(seq_exec{}, seg, take);
  con = tcon;
}
template <typename CONTAINER_T, typename SEGMENT_T>
void getIndices(CONTAINER_T& con, const SEGMENT_T& seg) {
  getIndicesConditional(con, seg, [](const typename CONTAINER_T::value_type&) { return true; });
}

// forall with expt params on host: each param gets a ValOp local starting
// at its identity; after the loop the target is combined (param_resolve,
// policy/sequential/params/reduce.hpp:42-46).
template <typename Seg, typename Body, typename... Red,
          typename = decltype(detail::seg_len(std::declval<const Seg&>()))>
void forall_params_impl(seq_exec, const Seg& r, Body&& body, Red&... reds) {
  std::tuple<typename Red::valop_type...> vals;
  const Index_type n = detail::seg_len(r);
  std::apply([&](auto&... v) {
    for (Index_type k = 0; k < n; ++k) body(detail::seg_at(r, k), v...);
  }, vals);
  std::apply([&](auto&... v) { (reds.combineTarget(v.val), ...); }, vals);
}

// Kernel names (RAJA::Name) bracket the loop they name.  The front-end
// finds the first name among the params and asks the policy for a scope
// (kernel_name_scope, found by argument-dependent lookup): host policies
// take none, as in the reference, whose CUDA back-end pushes an NVTX range
// (policy/cuda/params/kernel_name.hpp:33-70).
struct NoNameScope {};
template <typename Pol>
NoNameScope kernel_name_scope(const Pol&, const char*) {
  return {};
}
namespace detail {
inline const char* find_name() { return nullptr; }
template <typename P0, typename... Ps>
const char* find_name(const P0& p0, const Ps&... ps) {
  if constexpr (std::is_same<std::decay_t<P0>, expt::KernelName>::value) return p0.name;
  else return find_name(ps...);
}
}  // namespace detail

// ------------------------------------------------------------- plugins
// Launch hooks (util/PluginStrategy.hpp:20-37, util/PluginContext.hpp,
// util/plugins.hpp:34-64, util/Registry.hpp): plugins registered with
//   static RAJA::util::PluginRegistry::add<MyPlugin> P("name", "description");
// see preCapture / postCapture around the front-end's copy of the loop body
// and preLaunch / postLaunch around the launch, in registration order, with
// the policy's platform and the kernel name (pattern/forall.hpp:567-582).
// With no plugin registered the front-end skips the hooks and the copy.
using Platform = resources::Platform;
namespace util {
struct PluginOptions {
  std::string str;
};
struct PluginContext {
  PluginContext(Platform p, std::string name) : platform(p), kernel_name(std::move(name)) {}
  Platform platform;
  std::string kernel_name;
};
class PluginStrategy {
 public:
  virtual ~PluginStrategy() = default;
  virtual void init(const PluginOptions&) {}
  virtual void preCapture(const PluginContext&) {}
  virtual void postCapture(const PluginContext&) {}
  virtual void preLaunch(const PluginContext&) {}
  virtual void postLaunch(const PluginContext&) {}
  virtual void finalize() {}
};
// A process-wide list of named objects of type T, filled by static
// registration objects (add<U>) before main runs.
template <typename T>
class Registry {
 public:
  class entry {
   public:
    entry(std::string n, std::string d, std::shared_ptr<T> p) : name_(std::move(n)), desc_(std::move(d)), p_(std::move(p)) {}
    const std::string& getName() const { return name_; }
    const std::string& getDesc() const { return desc_; }
    T* get() const { return p_.get(); }

   private:
    std::string name_, desc_;
    std::shared_ptr<T> p_;
  };
  using iterator = typename std::vector<entry>::const_iterator;
  template <typename U>
  struct add {
    add(const char* name, const char* desc) { entries().emplace_back(name, desc, std::make_shared<U>()); }
  };
  static iterator begin() { return entries().cbegin(); }
  static iterator end() { return entries().cend(); }
  static bool empty() { return entries().empty(); }

 private:
  static std::vector<entry>& entries() {
    static std::vector<entry> v;
    return v;
  }
};
using PluginRegistry = Registry<PluginStrategy>;

template <typename Policy>
PluginContext make_context(std::string name) {
  return PluginContext(resources::get_resource<Policy>::type::get_default().get_platform(), std::move(name));
}
// The front-end's copy of the loop body, between the capture hooks.
template <typename T>
std::remove_reference_t<T> trigger_updates_before(T&& item) {
  return item;
}
inline void callPreCapturePlugins(const PluginContext& p) {
  for (auto it = PluginRegistry::begin(); it != PluginRegistry::end(); ++it) it->get()->preCapture(p);
}
inline void callPostCapturePlugins(const PluginContext& p) {
  for (auto it = PluginRegistry::begin(); it != PluginRegistry::end(); ++it) it->get()->postCapture(p);
}
inline void callPreLaunchPlugins(const PluginContext& p) {
  for (auto it = PluginRegistry::begin(); it != PluginRegistry::end(); ++it) it->get()->preLaunch(p);
}
inline void callPostLaunchPlugins(const PluginContext& p) {
  for (auto it = PluginRegistry::begin(); it != PluginRegistry::end(); ++it) it->get()->postLaunch(p);
}
}  // namespace util

namespace detail {
// Dispatch of forall(seg, params..., body): the kernel name (RAJA::Name)
// opens the policy's name scope and labels the plugin context; reducer
// params are collected, in order, for forall_params_impl.
template <typename Pol, typename Seg, typename Body, typename... Red>
void forall_collect(Pol p, Seg&& seg, Body&& body, std::tuple<Red&...> reds);
template <typename Pol, typename Seg, typename Body, typename... Red, typename... Rest>
void forall_collect(Pol p, Seg&& seg, Body&& body, std::tuple<Red&...> reds, expt::KernelName,
                    Rest&&... rest);
template <typename Pol, typename Seg, typename Body, typename... Red, typename R0, typename... Rest,
          typename std::enable_if<expt::detail::is_reducer<std::decay_t<R0>>::value, int>::type = 0>
void forall_collect(Pol p, Seg&& seg, Body&& body, std::tuple<Red&...> reds, R0& r0,
                    Rest&&... rest);

template <typename Pol, typename Seg, typename Body, typename... Red>
void forall_collect(Pol p, Seg&& seg, Body&& body, std::tuple<Red&...> reds) {
  std::apply([&](auto&... r) {
    forall_params_impl(p, std::forward<Seg>(seg), std::forward<Body>(body), r...);
  }, reds);
}
template <typename Pol, typename Seg, typename Body, typename... Red, typename... Rest>
void forall_collect(Pol p, Seg&& seg, Body&& body, std::tuple<Red&...> reds, expt::KernelName,
                    Rest&&... rest) {
  forall_collect(p, std::forward<Seg>(seg), std::forward<Body>(body), reds,
                 std::forward<Rest>(rest)...);
}
template <typename Pol, typename Seg, typename Body, typename... Red, typename R0, typename... Rest,
          typename std::enable_if<expt::detail::is_reducer<std::decay_t<R0>>::value, int>::type>
void forall_collect(Pol p, Seg&& seg, Body&& body, std::tuple<Red&...> reds, R0& r0,
                    Rest&&... rest) {
  forall_collect(p, std::forward<Seg>(seg), std::forward<Body>(body),
                 std::tuple_cat(reds, std::tie(r0)), std::forward<Rest>(rest)...);
}

template <typename Pol, typename Seg, typename Body, typename... Params>
void forall_dispatch(Pol p, Seg&& seg, Body&& body, Params&&... params) {
  if constexpr ((expt::detail::is_reducer<std::decay_t<Params>>::value || ... || false)) {
    forall_collect(p, std::forward<Seg>(seg), std::forward<Body>(body), std::tuple<>(), params...);
  } else {
    forall_impl(p, std::forward<Seg>(seg), std::forward<Body>(body));
  }
}
template <typename Pol, typename Seg, typename Body, typename... Params>
void forall_with(Pol p, Seg&& seg, Body&& body, Params&&... params) {
  const char* name = find_name(params...);
  auto named = kernel_name_scope(p, name);
  (void)named;
  if (util::PluginRegistry::empty()) {
    forall_dispatch(p, std::forward<Seg>(seg), std::forward<Body>(body), params...);
    return;
  }
  const util::PluginContext ctx = util::make_context<Pol>(name ? name : "");
  util::callPreCapturePlugins(ctx);
  auto captured = util::trigger_updates_before(body);
  util::callPostCapturePlugins(ctx);
  util::callPreLaunchPlugins(ctx);
  forall_dispatch(p, std::forward<Seg>(seg), captured, params...);
  util::callPostLaunchPlugins(ctx);
}
template <typename Pol, typename Seg, typename Tup, size_t... I>
void forall_split(Seg&& seg, Tup&& tup, std::index_sequence<I...>) {
  constexpr size_t N = std::tuple_size<std::decay_t<Tup>>::value;
  forall_with(Pol{}, std::forward<Seg>(seg), std::get<N - 1>(tup), std::get<I>(tup)...);
}
}  // namespace detail

// RAJA::forall<POLICY>([resource,] segment, [params...,] body)
// (pattern/forall.hpp:545-627).  Without a resource the policy's default
// resource is used.  The call runs with the resource bound and returns an
// EventProxy on it.
template <typename Pol, typename Res, typename Seg, typename... Args, detail::enable_if_resource<Res> = 0>
resources::EventProxy<std::decay_t<Res>> forall(Res&& r, Seg&& seg, Args&&... args) {
  static_assert(sizeof...(Args) >= 1, "forall needs a loop body");
  std::decay_t<Res> res = r;
  {
    auto bound = bind_resource(res);
    (void)bound;
    detail::forall_split<Pol>(std::forward<Seg>(seg), std::forward_as_tuple(std::forward<Args>(args)...),
                              std::make_index_sequence<sizeof...(Args) - 1>{});
  }
  return resources::EventProxy<std::decay_t<Res>>(res);
}
template <typename Pol, typename Seg, typename... Args, detail::enable_if_not_resource<Seg> = 0>
resources::EventProxy<typename resources::get_resource<Pol>::type> forall(Seg&& seg, Args&&... args) {
  return forall<Pol>(resources::get_resource<Pol>::type::get_default(), std::forward<Seg>(seg),
                     std::forward<Args>(args)...);
}

}  // namespace RAJA

// The policy list of RAJA::dynamic_forall (camp::list in the reference;
// only the list itself is needed here).
namespace camp {
template <typename... Ts>
struct list {};
}  // namespace camp

namespace RAJA {

// RAJA::dynamic_forall<camp::list<P0, P1, ...>>([resource,] pol, segment,
// [params...,] body) runs forall<P_pol> (pattern/forall.hpp:704-825, an
// experimental interface there).  A `pol` outside the list throws, as
// RAJA_ABORT_OR_THROW does with exceptions enabled.  The resource form
// passes resource.get<resource type of P_pol>() and returns an EventProxy
// on the type-erased resource.
namespace detail {
template <typename List>
struct policy_list;
template <typename... Pols>
struct policy_list<camp::list<Pols...>> {
  static constexpr int size = int(sizeof...(Pols));
  template <typename F>
  static void pick(int pol, F&& f) {
    int idx = 0;
    bool ran = false;
    (void)std::initializer_list<int>{
        ((idx++ == pol && !ran) ? (f(static_cast<Pols*>(nullptr)), ran = true, 0) : 0)...};
  }
};
}  // namespace detail

template <typename POLICY_LIST, typename Seg, typename... Args>
void dynamic_forall(const int pol, Seg&& seg, Args&&... args) {
  using L = detail::policy_list<POLICY_LIST>;
  static_assert(L::size > 0, "RAJA policy list must not be empty");
  if (pol < 0 || pol >= L::size) throw std::runtime_error("RAJA::dynamic_forall: policy enum not supported");
  L::pick(pol, [&](auto* p) {
    using P = std::remove_pointer_t<decltype(p)>;
    forall<P>(seg, args...);
  });
}
template <typename POLICY_LIST, typename Seg, typename... Args>
resources::EventProxy<resources::Resource> dynamic_forall(resources::Resource r, const int pol, Seg&& seg,
                                                          Args&&... args) {
  using L = detail::policy_list<POLICY_LIST>;
  static_assert(L::size > 0, "RAJA policy list must not be empty");
  if (pol < 0 || pol >= L::size) throw std::runtime_error("RAJA::dynamic_forall: policy value out of range");
  L::pick(pol, [&](auto* p) {
    using P = std::remove_pointer_t<decltype(p)>;
    forall<P>(r.template get<typename resources::get_resource<P>::type>(), seg, args...);
  });
  return resources::EventProxy<resources::Resource>(r);
}

// ---------------------------------------------------------------- launch
// RAJA::launch (pattern/launch/launch_core.hpp:45-675): a kernel of
// Teams x Threads with a LaunchContext for dynamic shared memory and
// team barriers; loop / loop_icount / tile / tile_tcount map segments onto
// the team and thread indices through loop policies.  LaunchPolicy and
// LoopPolicy pair a host policy with a device one; a loop body compiled
// for the device uses the device policy (launch_core.hpp:454-459).
enum struct ExecPlace : int { HOST, DEVICE, NUM_PLACES };

template <typename HOST_POLICY, typename DEVICE_POLICY = HOST_POLICY>
struct LoopPolicy {
  using host_policy_t = HOST_POLICY;
  using device_policy_t = DEVICE_POLICY;
};
template <typename HOST_POLICY, typename DEVICE_POLICY = HOST_POLICY>
struct LaunchPolicy {
  using host_policy_t = HOST_POLICY;
  using device_policy_t = DEVICE_POLICY;
};

struct Teams {
  int value[3];
  RAJA_HOST_DEVICE constexpr Teams() : value{1, 1, 1} {}
  RAJA_HOST_DEVICE constexpr Teams(int i) : value{i, 1, 1} {}
  RAJA_HOST_DEVICE constexpr Teams(int i, int j) : value{i, j, 1} {}
  RAJA_HOST_DEVICE constexpr Teams(int i, int j, int k) : value{i, j, k} {}
};
struct Threads {
  int value[3];
  RAJA_HOST_DEVICE constexpr Threads() : value{1, 1, 1} {}
  RAJA_HOST_DEVICE constexpr Threads(int i) : value{i, 1, 1} {}
  RAJA_HOST_DEVICE constexpr Threads(int i, int j) : value{i, j, 1} {}
  RAJA_HOST_DEVICE constexpr Threads(int i, int j, int k) : value{i, j, k} {}
};
struct Lanes {
  int value;
  RAJA_HOST_DEVICE constexpr Lanes() : value(0) {}
  RAJA_HOST_DEVICE constexpr Lanes(int i) : value(i) {}
};

struct LaunchParams {
  Teams teams;
  Threads threads;
  size_t shared_mem_size = 0;
  LaunchParams() = default;
  LaunchParams(Teams t, Threads th, size_t shmem = 0) : teams(t), threads(th), shared_mem_size(shmem) {}
};

// Bytes a launch reserves beyond LaunchParams::shared_mem_size, for the
// alignment padding getSharedMemory adds between requests.
constexpr size_t kLaunchSharedSlack = 256;

class LaunchContext {
 public:
  size_t shared_mem_offset = 0;
  void* shared_mem_ptr = nullptr;
  RAJA_HOST_DEVICE LaunchContext() {}
  // Bump allocation of `n` elements from the launch's dynamic shared
  // memory, each request aligned to its type.
  template <typename T>
  RAJA_HOST_DEVICE T* getSharedMemory(size_t n) {
    const size_t a = alignof(T);
    shared_mem_offset = (shared_mem_offset + a - 1) / a * a;
    T* p = reinterpret_cast<T*>(static_cast<char*>(shared_mem_ptr) + shared_mem_offset);
    shared_mem_offset += n * sizeof(T);
    return p;
  }
  RAJA_HOST_DEVICE void releaseSharedMemory() { shared_mem_offset = 0; }
  RAJA_HOST_DEVICE void teamSync() {
#if defined(__CUDA_ARCH__)
    __syncthreads();
#endif
  }
};

#if defined(__CUDA_ARCH__)
template <typename POLICY_LIST>
using loop_policy = typename POLICY_LIST::device_policy_t;
#else
template <typename POLICY_LIST>
using loop_policy = typename POLICY_LIST::host_policy_t;
#endif


// Loop executors, specialised per loop policy (launch_core.hpp:461-465,
// 560-564).  seq_exec runs every index in order on the calling thread.
template <typename POLICY, typename SEGMENT>
struct LoopExecute;
template <typename POLICY, typename SEGMENT>
struct LoopICountExecute;
template <typename POLICY, typename SEGMENT>
struct TileExecute;
template <typename POLICY, typename SEGMENT>
struct TileTCountExecute;

template <typename SEGMENT>
struct LoopExecute<seq_exec, SEGMENT> {
  template <typename BODY>
  RAJA_HOST_DEVICE static void exec(const LaunchContext&, const SEGMENT& seg, const BODY& body) {
    const Index_type n = detail::seg_len(seg);
    for (Index_type k = 0; k < n; ++k) body(detail::seg_at(seg, k));
  }
};
template <typename SEGMENT>
struct LoopICountExecute<seq_exec, SEGMENT> {
  template <typename BODY>
  RAJA_HOST_DEVICE static void exec(const LaunchContext&, const SEGMENT& seg, const BODY& body) {
    using I = std::decay_t<decltype(detail::seg_at(seg, 0))>;
    const Index_type n = detail::seg_len(seg);
    for (Index_type k = 0; k < n; ++k) body(detail::seg_at(seg, k), I(k));
  }
};
template <typename SEGMENT>
struct TileExecute<seq_exec, SEGMENT> {
  template <typename TILE_T, typename BODY>
  RAJA_HOST_DEVICE static void exec(const LaunchContext&, TILE_T ts, const SEGMENT& seg, const BODY& body) {
    const Index_type n = detail::seg_len(seg), t = Index_type(ts);
    for (Index_type k = 0; k * t < n; ++k) body(detail::seg_tile(seg, t, k));
  }
};
template <typename SEGMENT>
struct TileTCountExecute<seq_exec, SEGMENT> {
  template <typename TILE_T, typename BODY>
  RAJA_HOST_DEVICE static void exec(const LaunchContext&, TILE_T ts, const SEGMENT& seg, const BODY& body) {
    using I = std::decay_t<decltype(detail::seg_at(seg, 0))>;
    const Index_type n = detail::seg_len(seg), t = Index_type(ts);
    for (Index_type k = 0; k * t < n; ++k) body(detail::seg_tile(seg, t, k), I(k));
  }
};

template <typename POLICY_LIST, typename CONTEXT, typename SEGMENT, typename BODY>
RAJA_HOST_DEVICE void loop(const CONTEXT& ctx, const SEGMENT& seg, const BODY& body) {
  LoopExecute<loop_policy<POLICY_LIST>, SEGMENT>::exec(ctx, seg, body);
}
template <typename POLICY_LIST, typename CONTEXT, typename SEGMENT, typename BODY>
RAJA_HOST_DEVICE void loop_icount(const CONTEXT& ctx, const SEGMENT& seg, const BODY& body) {
  LoopICountExecute<loop_policy<POLICY_LIST>, SEGMENT>::exec(ctx, seg, body);
}
template <typename POLICY_LIST, typename CONTEXT, typename TILE_T, typename SEGMENT, typename BODY>
RAJA_HOST_DEVICE void tile(const CONTEXT& ctx, TILE_T tile_size, const SEGMENT& seg, const BODY& body) {
  TileExecute<loop_policy<POLICY_LIST>, SEGMENT>::exec(ctx, tile_size, seg, body);
}
template <typename POLICY_LIST, typename CONTEXT, typename TILE_T, typename SEGMENT, typename BODY>
RAJA_HOST_DEVICE void tile_tcount(const CONTEXT& ctx, TILE_T tile_size, const SEGMENT& seg, const BODY& body) {
  TileTCountExecute<loop_policy<POLICY_LIST>, SEGMENT>::exec(ctx, tile_size, seg, body);
}

// Launch executors, specialised per launch policy.  exec(res, params,
// body) runs the body with no reducer params; exec_params(res, params,
// body, reds...) passes one ValOp per expt reducer and combines them into
// the targets afterwards.
template <typename LAUNCH_POLICY>
struct LaunchExecute;

struct seq_launch_t {};

template <>
struct LaunchExecute<seq_launch_t> {
  template <typename Res, typename Body>
  static void exec(Res, const LaunchParams& p, const Body& body) {
    std::vector<std::max_align_t> shm((p.shared_mem_size + kLaunchSharedSlack) / sizeof(std::max_align_t) + 1);
    LaunchContext ctx;
    ctx.shared_mem_ptr = shm.data();
    body(ctx);
  }
  template <typename Res, typename Body, typename... Red>
  static void exec_params(Res, const LaunchParams& p, const Body& body, Red&... reds) {
    std::vector<std::max_align_t> shm((p.shared_mem_size + kLaunchSharedSlack) / sizeof(std::max_align_t) + 1);
    LaunchContext ctx;
    ctx.shared_mem_ptr = shm.data();
    std::tuple<typename Red::valop_type...> vals;
    std::apply([&](auto&... v) { body(ctx, v...); }, vals);
    std::apply([&](auto&... v) { (reds.combineTarget(v.val), ...); }, vals);
  }
};

namespace resources {
template <>
struct get_resource<seq_launch_t> {
  using type = Host;
};
}  // namespace resources

namespace detail {
// launch(res, params, [names / reducers ...,] body): names are dropped,
// reducers collected in order (as for forall).
template <typename LP, typename Res, typename Body, typename... Red>
void launch_collect(Res& r, const LaunchParams& p, const Body& body, std::tuple<Red&...> reds) {
  if constexpr (sizeof...(Red) == 0) {
    LaunchExecute<LP>::exec(r, p, body);
  } else {
    std::apply([&](auto&... rd) { LaunchExecute<LP>::exec_params(r, p, body, rd...); }, reds);
  }
}
template <typename LP, typename Res, typename Body, typename... Red, typename R0, typename... Rest>
void launch_collect(Res& r, const LaunchParams& p, const Body& body, std::tuple<Red&...> reds, R0& r0,
                    Rest&... rest) {
  if constexpr (expt::detail::is_reducer<std::decay_t<R0>>::value) {
    launch_collect<LP>(r, p, body, std::tuple_cat(reds, std::tie(r0)), rest...);
  } else {
    static_assert(std::is_same<std::decay_t<R0>, expt::KernelName>::value,
                  "launch arguments between the params and the body are reducers or names");
    launch_collect<LP>(r, p, body, reds, rest...);
  }
}
template <typename LP, typename Res, typename Tup, size_t... I>
void launch_split(Res& r, const LaunchParams& p, Tup&& tup, std::index_sequence<I...>) {
  constexpr size_t N = std::tuple_size<std::decay_t<Tup>>::value;
  launch_collect<LP>(r, p, std::get<N - 1>(tup), std::tuple<>(), std::get<I>(tup)...);
}
template <typename LP, typename Res, typename Body, typename Tup, size_t... I>
void launch_split_body(Res& r, const LaunchParams& p, const Body& body, Tup&& tup, std::index_sequence<I...>) {
  launch_collect<LP>(r, p, body, std::tuple<>(), std::get<I>(tup)...);
}
// With plugins registered, the capture hooks bracket a copy of the body and
// the launch hooks bracket the launch (launch_core.hpp:264-286).
template <typename LP, typename Res, typename... Args>
void launch_on(Res r, const LaunchParams& p, Args&&... args) {
  static_assert(sizeof...(Args) >= 1, "launch needs a body");
  auto bound = bind_resource(r);
  (void)bound;
  const char* name = find_name(args...);
  auto named = kernel_name_scope(LP{}, name);
  (void)named;
  auto tup = std::forward_as_tuple(args...);
  constexpr size_t N = sizeof...(Args);
  if (util::PluginRegistry::empty()) {
    launch_split<LP>(r, p, tup, std::make_index_sequence<N - 1>{});
    return;
  }
  const util::PluginContext ctx = util::make_context<LP>(name ? name : "");
  util::callPreCapturePlugins(ctx);
  auto captured = util::trigger_updates_before(std::get<N - 1>(tup));
  util::callPostCapturePlugins(ctx);
  util::callPreLaunchPlugins(ctx);
  launch_split_body<LP>(r, p, captured, tup, std::make_index_sequence<N - 1>{});
  util::callPostLaunchPlugins(ctx);
}
}  // namespace detail

// launch<POLICY>(params, [names / reducers ...,] body): runs the launch
// policy's first (host_policy_t) entry on its default resource
// (launch_core.hpp:249-289).
template <typename POLICY_LIST, typename... Args>
void launch(const LaunchParams& p, Args&&... args) {
  using LP = typename POLICY_LIST::host_policy_t;
  detail::launch_on<LP>(resources::get_resource<LP>::type::get_default(), p, std::forward<Args>(args)...);
}
// launch<POLICY>(place, params, ...): host or device policy chosen at run
// time (launch_core.hpp:291-337).
template <typename POLICY_LIST, typename... Args>
void launch(ExecPlace place, const LaunchParams& p, Args&&... args) {
  if (place == ExecPlace::HOST) {
    using LP = typename POLICY_LIST::host_policy_t;
    detail::launch_on<LP>(resources::get_resource<LP>::type::get_default(), p, std::forward<Args>(args)...);
  } else if (place == ExecPlace::DEVICE) {
    using LP = typename POLICY_LIST::device_policy_t;
    detail::launch_on<LP>(resources::get_resource<LP>::type::get_default(), p, std::forward<Args>(args)...);
  } else {
    throw std::runtime_error("launch: unknown ExecPlace");
  }
}
// launch<POLICY>(resource, params, ...): the resource's platform picks the
// host or the device policy (launch_core.hpp:370-452).
template <typename POLICY_LIST, typename... Args>
resources::EventProxy<resources::Resource> launch(resources::Resource res, const LaunchParams& p,
                                                  Args&&... args) {
  if (res.get_platform() == resources::Platform::host) {
    using LP = typename POLICY_LIST::host_policy_t;
    detail::launch_on<LP>(res, p, std::forward<Args>(args)...);
  } else {
    using LP = typename POLICY_LIST::device_policy_t;
    detail::launch_on<LP>(res, p, std::forward<Args>(args)...);
  }
  return resources::EventProxy<resources::Resource>(res);
}

// Resource for a run-time place (launch_core.hpp:339-369).
template <typename T, typename U>
resources::Resource Get_Runtime_Resource(T host_res, U device_res, ExecPlace place) {
  if (place == ExecPlace::DEVICE) return resources::Resource(device_res);
  return resources::Resource(host_res);
}
template <typename T>
resources::Resource Get_Host_Resource(T host_res, ExecPlace place) {
  if (place == ExecPlace::DEVICE) throw std::runtime_error("Get_Host_Resource: device is not enabled");
  return resources::Resource(host_res);
}

// ------------------------------------------------------------ View/Layout
// Layouts and views (util/View.hpp, util/Layout.hpp, util/PermutedLayout.hpp).
// A layout holds the extent and stride of every dimension.  By default the
// last index has stride one (row-major); make_permuted_layout orders the
// strides by a permutation whose last entry is the stride-one dimension.
// StrideOne names that dimension for the reader (-1: not stated), as in
// RAJA; the strides themselves are kept at run time.

// Permutations of the dimensions (util/Permutations.hpp), as index
// sequences.
using PERM_I = std::index_sequence<0>;
using PERM_IJ = std::index_sequence<0, 1>;
using PERM_JI = std::index_sequence<1, 0>;
using PERM_IJK = std::index_sequence<0, 1, 2>;
using PERM_IKJ = std::index_sequence<0, 2, 1>;
using PERM_JIK = std::index_sequence<1, 0, 2>;
using PERM_JKI = std::index_sequence<1, 2, 0>;
using PERM_KIJ = std::index_sequence<2, 0, 1>;
using PERM_KJI = std::index_sequence<2, 1, 0>;
// as_array<Perm>::get(): the permutation as an array.
template <typename Perm>
struct as_array;
template <size_t... P>
struct as_array<std::index_sequence<P...>> {
  static std::array<Index_type, sizeof...(P)> get() { return {{Index_type(P)...}}; }
};

template <size_t DIM, typename IdxT = Index_type, ptrdiff_t StrideOne = -1>
struct Layout {
  static_assert(StrideOne >= -1 && StrideOne < ptrdiff_t(DIM), "stride-one dimension out of range");
  Index_type sizes[DIM];
  Index_type strides[DIM];
  template <typename... Ns, typename std::enable_if<sizeof...(Ns) == DIM &&
                                                        (std::is_integral<Ns>::value && ...),
                                                    int>::type = 0>
  RAJA_HOST_DEVICE Layout(Ns... ns) : sizes{Index_type(ns)...} {
    set_strides();
  }
  explicit Layout(const std::array<Index_type, DIM>& s) {
    for (size_t d = 0; d < DIM; ++d) sizes[d] = s[d];
    set_strides();
  }
  // Strides in the order of `perm`: perm[DIM-1] has stride one.
  Layout(const std::array<Index_type, DIM>& s, const std::array<Index_type, DIM>& perm) {
    for (size_t d = 0; d < DIM; ++d) sizes[d] = s[d];
    Index_type st = 1;
    for (size_t k = DIM; k-- > 0;) {
      strides[perm[k]] = st;
      st *= sizes[perm[k]];
    }
  }
  RAJA_HOST_DEVICE void set_strides() {
    Index_type st = 1;
    for (size_t d = DIM; d-- > 0;) {
      strides[d] = st;
      st *= sizes[d];
    }
  }
  template <typename... Is>
  RAJA_HOST_DEVICE Index_type operator()(Is... is) const {
    static_assert(sizeof...(Is) == DIM, "one index per dimension");
    const Index_type idx[DIM] = {Index_type(is)...};
    Index_type off = 0;
    for (size_t d = 0; d < DIM; ++d) off += idx[d] * strides[d];
    return off;
  }
  // The indices of a linear offset (the inverse of operator()).
  template <typename... Is>
  RAJA_HOST_DEVICE void toIndices(Index_type linear, Is&... is) const {
    static_assert(sizeof...(Is) == DIM, "one index per dimension");
    size_t d = 0;
    ((is = static_cast<std::decay_t<Is>>(sizes[d] ? (linear / strides[d]) % sizes[d] : 0), ++d), ...);
  }
  RAJA_HOST_DEVICE Index_type size() const {
    Index_type n = 1;
    for (size_t d = 0; d < DIM; ++d) n *= sizes[d];
    return n;
  }
  RAJA_HOST_DEVICE Index_type size_noproj() const { return size(); }
};
template <size_t DIM, typename IdxT = Index_type>
Layout<DIM, IdxT> make_permuted_layout(const std::array<Index_type, DIM>& sizes,
                                       const std::array<Index_type, DIM>& perm) {
  return Layout<DIM, IdxT>(sizes, perm);
}
// Offset layouts (util/OffsetLayout.hpp:40-244): dimension d runs over
// [begin[d], end[d]), stored row-major from begin.
template <size_t DIM, typename IdxT = Index_type>
struct OffsetLayout {
  Layout<DIM, IdxT> base;
  Index_type offsets[DIM];
  OffsetLayout(const std::array<Index_type, DIM>& begin, const std::array<Index_type, DIM>& end)
      : base(sizes_of(begin, end)) {
    for (size_t d = 0; d < DIM; ++d) offsets[d] = begin[d];
  }
  template <typename... Is>
  RAJA_HOST_DEVICE Index_type operator()(Is... is) const {
    static_assert(sizeof...(Is) == DIM, "one index per dimension");
    const Index_type idx[DIM] = {Index_type(is)...};
    Index_type off = 0;
    for (size_t d = 0; d < DIM; ++d) off += (idx[d] - offsets[d]) * base.strides[d];
    return off;
  }
  RAJA_HOST_DEVICE Index_type size() const { return base.size(); }

 private:
  static std::array<Index_type, DIM> sizes_of(const std::array<Index_type, DIM>& b,
                                               const std::array<Index_type, DIM>& e) {
    std::array<Index_type, DIM> s{};
    for (size_t d = 0; d < DIM; ++d) s[d] = e[d] - b[d];
    return s;
  }
};
template <size_t DIM, typename IdxT = Index_type>
OffsetLayout<DIM, IdxT> make_offset_layout(const std::array<Index_type, DIM>& begin,
                                           const std::array<Index_type, DIM>& end) {
  return OffsetLayout<DIM, IdxT>(begin, end);
}

template <typename T, typename LayoutT>
struct View {
  using value_type = T;
  using pointer_type = T*;
  using layout_type = LayoutT;
  T* data;
  LayoutT layout;
  template <typename... Ns,
            typename std::enable_if<(sizeof...(Ns) > 0) && (std::is_integral<Ns>::value && ...), int>::type = 0>
  RAJA_HOST_DEVICE View(T* p, Ns... ns) : data(p), layout(ns...) {}
  RAJA_HOST_DEVICE View(T* p, const LayoutT& l) : data(p), layout(l) {}
  template <typename... Is>
  RAJA_HOST_DEVICE T& operator()(Is... is) const {
    return data[layout(is...)];
  }
  RAJA_HOST_DEVICE void set_data(T* p) { data = p; }
};

// Index layouts (util/IndexLayout.hpp:28-230, util/View.hpp:58-72): each
// dimension maps its index through DirectIndex (as is), IndexList
// (index_list[i]) or ConditionalIndexList (index_list[i], or i when the list
// is null) before the row-major strides apply.
template <typename IdxLin = Index_type>
struct DirectIndex {
  RAJA_HOST_DEVICE constexpr IdxLin operator()(IdxLin i) const { return i; }
};
template <typename IdxLin = Index_type>
struct IndexList {
  IdxLin* index_list = nullptr;
  RAJA_HOST_DEVICE constexpr IdxLin operator()(IdxLin i) const { return index_list[i]; }
};
template <typename IdxLin = Index_type>
struct ConditionalIndexList {
  IdxLin* index_list = nullptr;
  RAJA_HOST_DEVICE constexpr IdxLin operator()(IdxLin i) const { return index_list ? index_list[i] : i; }
};
template <size_t DIM = 1, typename IdxLin = Index_type, typename... IndexTypes>
struct IndexLayout {
  static_assert(sizeof...(IndexTypes) == DIM, "one index map per dimension");
  Layout<DIM, IdxLin> base;
  std::tuple<IndexTypes...> maps;
  template <typename... Ns>
  IndexLayout(const std::tuple<IndexTypes...>& m, Ns... ns) : base(ns...), maps(m) {}
  template <typename... Is>
  RAJA_HOST_DEVICE IdxLin operator()(Is... is) const {
    static_assert(sizeof...(Is) == DIM, "one index per dimension");
    return apply(std::index_sequence_for<IndexTypes...>{}, is...);
  }
  RAJA_HOST_DEVICE Index_type size() const { return base.size(); }
  RAJA_HOST_DEVICE Index_type size_noproj() const { return base.size(); }

 private:
  template <size_t... D, typename... Is>
  RAJA_HOST_DEVICE IdxLin apply(std::index_sequence<D...>, Is... is) const {
    return IdxLin((Index_type(0) + ... + (base.strides[D] * Index_type(std::get<D>(maps)(IdxLin(is))))));
  }
};
template <typename... IndexTypes>
std::tuple<IndexTypes...> make_index_tuple(IndexTypes... it) {
  return std::tuple<IndexTypes...>(it...);
}
template <typename IdxLin = Index_type, typename... IndexTypes, typename... Ns>
IndexLayout<sizeof...(Ns), IdxLin, IndexTypes...> make_index_layout(const std::tuple<IndexTypes...>& maps, Ns... ns) {
  return IndexLayout<sizeof...(Ns), IdxLin, IndexTypes...>(maps, ns...);
}
template <size_t DIM, typename IdxLin, typename T, typename... IndexTypes>
View<T, IndexLayout<DIM, IdxLin, IndexTypes...>> make_index_view(T* ptr,
                                                                 const IndexLayout<DIM, IdxLin, IndexTypes...>& layout) {
  return View<T, IndexLayout<DIM, IdxLin, IndexTypes...>>(ptr, layout);
}

// make_permuted_view<meta_layout>(ptr, extents...) (util/View.hpp:328-417):
// layout_right is row-major (the last index has stride one), layout_left
// column-major (the first index has stride one), and an index sequence
// gives the stride order (its last entry has stride one).
struct layout_left {};
struct layout_right {};
template <typename meta_layout, typename IndexType = Index_type, typename T, typename... Extents>
View<T, Layout<sizeof...(Extents), IndexType>> make_permuted_view(T* ptr, Extents... extents) {
  constexpr size_t N = sizeof...(Extents);
  const std::array<Index_type, N> sizes{{Index_type(extents)...}};
  std::array<Index_type, N> order{};
  for (size_t d = 0; d < N; ++d) order[d] = Index_type(d);
  if constexpr (std::is_same<meta_layout, layout_left>::value) {
    for (size_t d = 0; d < N; ++d) order[d] = Index_type(N - 1 - d);
  } else if constexpr (!std::is_same<meta_layout, layout_right>::value) {
    order = as_array<meta_layout>::get();
  }
  return View<T, Layout<N, IndexType>>(ptr, Layout<N, IndexType>(sizes, order));
}

// Integer helpers (util/math.hpp:36-105): floor(log2(n)) (0 for n <= 0),
// the smallest power of two >= n and the largest <= n (0 for n <= 0), and
// lhs mod rhs for a power-of-two rhs.
template <typename T, std::enable_if_t<std::is_integral<T>::value, int> = 0>
RAJA_HOST_DEVICE constexpr T log2(T n) noexcept {
  T r = 0;
  while (n > 1) {
    n = T(n >> 1);
    ++r;
  }
  return r;
}
template <typename T, std::enable_if_t<std::is_integral<T>::value, int> = 0>
RAJA_HOST_DEVICE constexpr T next_pow2(T n) noexcept {
  if (n <= 0) return 0;
  T p = 1;
  while (p < n) {
    if (p > std::numeric_limits<T>::max() / 2) return 0;  // no larger power fits in T
    p = T(p << 1);
  }
  return p;
}
template <typename T, std::enable_if_t<std::is_integral<T>::value, int> = 0>
RAJA_HOST_DEVICE constexpr T prev_pow2(T n) noexcept {
  if (n <= 0) return 0;
  T p = 1;
  while (p <= n / 2) p = T(p << 1);
  return p;
}
template <typename L, typename R,
          std::enable_if_t<std::is_integral<L>::value && std::is_integral<R>::value, int> = 0>
RAJA_HOST_DEVICE constexpr auto power_of_2_mod(L lhs, R rhs) noexcept {
  return lhs & (rhs - R(1));
}

// for_each over a container's elements, a type list or a tuple
// (util/for_each.hpp:36-125); each returns the function object.
template <typename Container, typename UnaryFunc>
UnaryFunc for_each(Container&& c, UnaryFunc func) {
  for (auto&& x : c) func(x);
  return func;
}
template <typename... Ts, typename UnaryFunc>
UnaryFunc for_each_type(const camp::list<Ts...>&, UnaryFunc func) {
  (func(Ts{}), ...);
  return func;
}
template <typename Tuple, typename UnaryFunc>
UnaryFunc for_each_tuple(Tuple&& t, UnaryFunc func) {
  std::apply([&](auto&&... x) { (func(x), ...); }, std::forward<Tuple>(t));
  return func;
}

// TypedView<T, Layout, IndexTypes...> (util/View.hpp:55-57,
// util/TypedViewBase.hpp): a view whose operator() takes exactly one index of
// each listed type, so strongly typed indices of different spaces cannot be
// swapped; the layout sees their raw values.
template <typename T, typename LayoutT, typename... IndexTypes>
struct TypedView : View<T, LayoutT> {
  using View<T, LayoutT>::View;
  RAJA_HOST_DEVICE T& operator()(IndexTypes... is) const {
    return this->data[this->layout(stripIndexType(is)...)];
  }
};

// Views whose elements are AtomicRefs (util/View.hpp:272-326):
// make_atomic_view<Policy>(view)(i, j) += v is an atomic update.  With
// seq_atomic the element reference is returned as it is.
template <typename ViewType, typename AtomicPolicy>
struct AtomicViewWrapper {
  using base_type = ViewType;
  using pointer_type = typename ViewType::pointer_type;
  using value_type = typename ViewType::value_type;
  using atomic_type = AtomicRef<value_type, AtomicPolicy>;
  base_type base_;
  explicit AtomicViewWrapper(const ViewType& v) : base_(v) {}
  void set_data(pointer_type p) { base_.set_data(p); }
  template <typename... Is>
  RAJA_HOST_DEVICE atomic_type operator()(Is... is) const {
    return atomic_type(&base_(is...));
  }
};
template <typename ViewType>
struct AtomicViewWrapper<ViewType, seq_atomic> {
  using base_type = ViewType;
  using pointer_type = typename ViewType::pointer_type;
  using value_type = typename ViewType::value_type;
  base_type base_;
  explicit AtomicViewWrapper(const ViewType& v) : base_(v) {}
  void set_data(pointer_type p) { base_.set_data(p); }
  template <typename... Is>
  RAJA_HOST_DEVICE value_type& operator()(Is... is) const {
    return base_(is...);
  }
};
template <typename AtomicPolicy, typename ViewType>
AtomicViewWrapper<ViewType, AtomicPolicy> make_atomic_view(const ViewType& view) {
  return AtomicViewWrapper<ViewType, AtomicPolicy>(view);
}

// ------------------------------------------------------- CombiningAdapter
// A lambda of D indices run as a 1-D loop (util/CombiningAdapter.hpp:80-275):
// linear index k maps through the layout to offsets within each range, and
// the body receives begin_d + offset_d for every dimension:
//   auto ad = make_CombiningAdapter(body, irange, jrange);
//   forall<pol>(ad.getRange(), ad);
// The layout is row-major (the last range fastest) or, for
// make_PermutedCombiningAdapter<Perm>, ordered by Perm.
template <typename Lambda, typename IdxLin, typename... IdxTs>
struct CombiningAdapter {
  static constexpr size_t D = sizeof...(IdxTs);
  using RangeLinear = TypedRangeSegment<IdxLin>;
  Lambda m_lambda;
  Layout<D, IdxLin> m_layout;
  Index_type m_begin[D];

  CombiningAdapter(Lambda l, const Layout<D, IdxLin>& layout, const std::array<Index_type, D>& begin)
      : m_lambda(std::move(l)), m_layout(layout) {
    for (size_t d = 0; d < D; ++d) m_begin[d] = begin[d];
  }
  RAJA_HOST_DEVICE auto operator()(IdxLin linear) const { return call(linear, std::index_sequence_for<IdxTs...>{}); }
  RAJA_HOST_DEVICE IdxLin size() const { return static_cast<IdxLin>(m_layout.size_noproj()); }
  RAJA_HOST_DEVICE RangeLinear getRange() const { return RangeLinear(static_cast<IdxLin>(0), size()); }

 private:
  template <size_t... I>
  RAJA_HOST_DEVICE auto call(IdxLin linear, std::index_sequence<I...>) const {
    Index_type idx[D];
    m_layout.toIndices(static_cast<Index_type>(linear), idx[I]...);
    return m_lambda(static_cast<IdxTs>(m_begin[I] + idx[I])...);
  }
};

namespace detail {
template <typename Lambda, typename... IdxTs>
auto combining_adapter(Lambda&& lambda, const std::array<Index_type, sizeof...(IdxTs)>* perm,
                       const TypedRangeSegment<IdxTs>&... segs) {
  using IdxLin = typename std::common_type<IdxTs...>::type;
  constexpr size_t D = sizeof...(IdxTs);
  const std::array<Index_type, D> sizes{{Index_type(segs.size())...}};
  const std::array<Index_type, D> begin{{(segs.size() ? Index_type(*segs.begin()) : Index_type(0))...}};
  Layout<D, IdxLin> layout = perm ? Layout<D, IdxLin>(sizes, *perm) : Layout<D, IdxLin>(sizes);
  return CombiningAdapter<std::decay_t<Lambda>, IdxLin, IdxTs...>(std::forward<Lambda>(lambda), layout, begin);
}
}  // namespace detail

template <typename Lambda, typename... IdxTs>
auto make_CombiningAdapter(Lambda&& lambda, const TypedRangeSegment<IdxTs>&... segs) {
  return detail::combining_adapter(std::forward<Lambda>(lambda), nullptr, segs...);
}
template <typename Perm, typename Lambda, typename... IdxTs>
auto make_PermutedCombiningAdapter(Lambda&& lambda, const TypedRangeSegment<IdxTs>&... segs) {
  const auto perm = as_array<Perm>::get();
  static_assert(std::tuple_size<decltype(perm)>::value == sizeof...(IdxTs), "one permutation entry per range");
  return detail::combining_adapter(std::forward<Lambda>(lambda), &perm, segs...);
}

// ------------------------------------------------------ IndexSet builders
// buildIndexSetAligned (index/IndexSetBuilders.hpp:56-62, algorithm in
// src/AlignedRangeIndexSetBuilders.cpp): splits an index array into range
// segments and list segments.  Walking the array, a range starts at a value
// v with v % range_align == 0 whose successor is v + 1, and runs while the
// indices stay consecutive; the indices between ranges form list segments.
// The split is kept only if its encoded size (2 per range, 1 + length per
// list, 1 to terminate) is below length * (range_align - 1) / range_align;
// otherwise, and whenever length <= range_min_length, the whole array is one
// list segment.  The list segments point into indices_in, which must stay
// alive and readable where the loops run (the reference copies them into
// work_res's memory).
inline void buildIndexSetAligned(TypedIndexSet<RangeSegment, ListSegment>& iset, resources::Resource work_res,
                                 const Index_type* const indices_in, Index_type length, Index_type range_min_length,
                                 Index_type range_align) {
  (void)work_res;
  if (length <= 0) return;
  if (length <= range_min_length) {
    iset.push_back(ListSegment(indices_in, length));
    return;
  }
  struct Piece {
    bool range;
    Index_type first;  // range: first value; list: first position in indices_in
    Index_type len;
  };
  std::vector<Piece> pieces;
  if (length == 1) {
    pieces.push_back({false, 0, 1});
  } else {
    const Index_type* x = indices_in;
    bool in_range = x[1] == x[0] + 1 && x[0] % range_align == 0;
    Index_type first = in_range ? x[0] : 0, count = 0;
    for (Index_type ii = 1; ii < length; ++ii) {
      const Index_type prev = x[ii - 1];
      if (x[ii] == prev + 1) {
        if (!in_range && prev % range_align == 0) {   // a list ends where an aligned run starts
          if (count != 0) pieces.push_back({false, first, count});
          in_range = true;
          first = prev;
          count = 0;
        }
        ++count;
      } else if (in_range) {                          // the run ends with prev
        pieces.push_back({true, first, count + 1});
        in_range = false;
        first = ii;
        count = 0;
      } else {
        ++count;
      }
    }
    pieces.push_back({in_range, first, count + 1});
  }
  Index_type cost = 1;
  for (const Piece& p : pieces) cost += p.range ? 2 : 1 + p.len;
  if (cost < (length * (range_align - 1)) / range_align) {
    for (const Piece& p : pieces) {
      if (p.range) iset.push_back(RangeSegment(p.first, p.first + p.len));
      else iset.push_back(ListSegment(indices_in + p.first, p.len));
    }
  } else {
    iset.push_back(ListSegment(indices_in, length));
  }
}

// ---------------------------------------------------------- forall_Icount
// forall_Icount<POLICY>(segment, icount, body): body(icount + k, seg[k])
// for k in [0, len) (pattern/forall.hpp:102-124, 227-276); over an
// IndexSet the count runs on across the segments, one forall per segment.
namespace detail {
template <typename Seg, typename Body>
struct IcountAdapter {
  Seg seg;
  Body body;
  Index_type icount;
  template <typename I>
  RAJA_HOST_DEVICE void operator()(I k) const {
    body(Index_type(icount + Index_type(k)), seg_at(seg, Index_type(k)));
  }
};
}  // namespace detail
template <typename Pol, typename Seg, typename Body,
          typename = decltype(detail::seg_len(std::declval<const std::decay_t<Seg>&>()))>
void forall_Icount(Seg&& seg, Index_type icount, Body&& body) {
  detail::IcountAdapter<std::decay_t<Seg>, std::decay_t<Body>> ad{seg, body, icount};
  forall<Pol>(TypedRangeSegment<Index_type>(0, detail::seg_len(seg)), ad);
}
template <typename Pol, typename... Segs, typename Body>
void forall_Icount(const TypedIndexSet<Segs...>& is, Body&& body) {
  Index_type ic = 0;
  for (const auto& s : is.segments())
    std::visit([&](const auto& seg) {
      forall_Icount<Pol>(seg, ic, body);
      ic += detail::seg_len(seg);
    }, s);
}

// ----------------------------------------------------------------- scans
// pattern/scan.hpp front-ends.  Back-ends overload scan_inclusive /
// scan_exclusive in namespace RAJA on their policy type; the front-end
// calls them unqualified so argument-dependent lookup finds overloads
// declared after this header (the role of impl::scan::* in
// policy/*/scan.hpp).  Host implementations follow
// policy/sequential/scan.hpp:43-153.
template <typename T, typename F>
void scan_inclusive(seq_exec, const T* b, const T* e, T* out, F f) {
  if (b == e) return;
  T agg = *b;
  *out++ = agg;
  for (const T* i = b + 1; i != e; ++i) {
    agg = f(agg, *i);
    *out++ = agg;
  }
}
template <typename T, typename F>
void scan_exclusive(seq_exec, const T* b, const T* e, T* out, F f, T v) {
  const Index_type n = e - b;
  T agg = v;
  for (Index_type i = 0; i < n; ++i) {
    const T t = b[i];
    out[i] = agg;
    agg = f(agg, t);
  }
}

// Each front-end has a form that takes the resource first
// (pattern/scan.hpp:336-441) and returns an EventProxy on it; the form
// without one uses the policy's default resource.
#define RAJA_COMPAT_DEFAULT_RES(Pol) resources::get_resource<Pol>::type::get_default()
#define RAJA_COMPAT_RES_T(Pol) resources::EventProxy<typename resources::get_resource<Pol>::type>

template <typename Pol, typename Res, typename T, typename F = operators::plus<std::remove_const_t<T>>,
          detail::enable_if_resource<Res> = 0>
resources::EventProxy<Res> inclusive_scan(Res r, Span<T> in, Span<std::remove_const_t<T>> out, F f = F{}) {
  auto bound = bind_resource(r);
  (void)bound;
  if (in.size() != 0)
    scan_inclusive(Pol{}, static_cast<const std::remove_const_t<T>*>(in.begin()),
                   static_cast<const std::remove_const_t<T>*>(in.end()), out.begin(), f);
  return resources::EventProxy<Res>(r);
}
template <typename Pol, typename Res, typename T, typename F = operators::plus<std::remove_const_t<T>>,
          detail::enable_if_resource<Res> = 0>
resources::EventProxy<Res> exclusive_scan(Res r, Span<T> in, Span<std::remove_const_t<T>> out, F f = F{},
                                          std::remove_const_t<T> v = F::identity()) {
  auto bound = bind_resource(r);
  (void)bound;
  if (in.size() != 0)
    scan_exclusive(Pol{}, static_cast<const std::remove_const_t<T>*>(in.begin()),
                   static_cast<const std::remove_const_t<T>*>(in.end()), out.begin(), f, v);
  return resources::EventProxy<Res>(r);
}
template <typename Pol, typename Res, typename T, typename F = operators::plus<T>,
          detail::enable_if_resource<Res> = 0>
resources::EventProxy<Res> inclusive_scan_inplace(Res r, Span<T> io, F f = F{}) {
  auto bound = bind_resource(r);
  (void)bound;
  if (io.size() != 0)
    scan_inclusive(Pol{}, static_cast<const T*>(io.begin()), static_cast<const T*>(io.end()), io.begin(), f);
  return resources::EventProxy<Res>(r);
}
template <typename Pol, typename Res, typename T, typename F = operators::plus<T>,
          detail::enable_if_resource<Res> = 0>
resources::EventProxy<Res> exclusive_scan_inplace(Res r, Span<T> io, F f = F{}, T v = F::identity()) {
  auto bound = bind_resource(r);
  (void)bound;
  if (io.size() != 0)
    scan_exclusive(Pol{}, static_cast<const T*>(io.begin()), static_cast<const T*>(io.end()), io.begin(), f, v);
  return resources::EventProxy<Res>(r);
}

template <typename Pol, typename T, typename F = operators::plus<std::remove_const_t<T>>>
RAJA_COMPAT_RES_T(Pol) inclusive_scan(Span<T> in, Span<std::remove_const_t<T>> out, F f = F{}) {
  return inclusive_scan<Pol>(RAJA_COMPAT_DEFAULT_RES(Pol), in, out, f);
}
template <typename Pol, typename T, typename F = operators::plus<std::remove_const_t<T>>>
RAJA_COMPAT_RES_T(Pol) exclusive_scan(Span<T> in, Span<std::remove_const_t<T>> out, F f = F{},
                                      std::remove_const_t<T> v = F::identity()) {
  return exclusive_scan<Pol>(RAJA_COMPAT_DEFAULT_RES(Pol), in, out, f, v);
}
template <typename Pol, typename T, typename F = operators::plus<T>>
RAJA_COMPAT_RES_T(Pol) inclusive_scan_inplace(Span<T> io, F f = F{}) {
  return inclusive_scan_inplace<Pol>(RAJA_COMPAT_DEFAULT_RES(Pol), io, f);
}
template <typename Pol, typename T, typename F = operators::plus<T>>
RAJA_COMPAT_RES_T(Pol) exclusive_scan_inplace(Span<T> io, F f = F{}, T v = F::identity()) {
  return exclusive_scan_inplace<Pol>(RAJA_COMPAT_DEFAULT_RES(Pol), io, f, v);
}

// ----------------------------------------------------------------- sorts
// pattern/sort.hpp; back-ends overload sort_stable / sort_unstable /
// sort_stable_pairs / sort_unstable_pairs in namespace RAJA (found by ADL,
// as above).  Host: stable merge sort (util/sort.hpp:577).
template <typename T, typename C>
void sort_stable(seq_exec, T* b, T* e, C c) { std::stable_sort(b, e, c); }
template <typename T, typename C>
void sort_unstable(seq_exec, T* b, T* e, C c) { std::stable_sort(b, e, c); }
template <typename K, typename V, typename C>
void sort_stable_pairs(seq_exec, K* kb, K* ke, V* vb, C c) {
  const Index_type n = ke - kb;
  std::vector<std::pair<K, V>> z(static_cast<size_t>(n));
  for (Index_type i = 0; i < n; ++i) z[i] = {kb[i], vb[i]};
  std::stable_sort(z.begin(), z.end(), [&](const std::pair<K, V>& a, const std::pair<K, V>& b) {
    return c(a.first, b.first);
  });
  for (Index_type i = 0; i < n; ++i) {
    kb[i] = z[i].first;
    vb[i] = z[i].second;
  }
}
template <typename K, typename V, typename C>
void sort_unstable_pairs(seq_exec p, K* kb, K* ke, V* vb, C c) { sort_stable_pairs(p, kb, ke, vb, c); }

// Resource-first forms as for the scans (pattern/sort.hpp:54-451).
template <typename Pol, typename Res, typename T, typename C = operators::less<T>,
          detail::enable_if_resource<Res> = 0>
resources::EventProxy<Res> sort(Res r, Span<T> s, C c = C{}) {
  auto bound = bind_resource(r);
  (void)bound;
  if (s.size() > 1) sort_unstable(Pol{}, s.begin(), s.end(), c);
  return resources::EventProxy<Res>(r);
}
template <typename Pol, typename Res, typename T, typename C = operators::less<T>,
          detail::enable_if_resource<Res> = 0>
resources::EventProxy<Res> stable_sort(Res r, Span<T> s, C c = C{}) {
  auto bound = bind_resource(r);
  (void)bound;
  if (s.size() > 1) sort_stable(Pol{}, s.begin(), s.end(), c);
  return resources::EventProxy<Res>(r);
}
template <typename Pol, typename Res, typename K, typename V, typename C = operators::less<K>,
          detail::enable_if_resource<Res> = 0>
resources::EventProxy<Res> sort_pairs(Res r, Span<K> k, Span<V> v, C c = C{}) {
  auto bound = bind_resource(r);
  (void)bound;
  if (k.size() > 1) sort_unstable_pairs(Pol{}, k.begin(), k.end(), v.begin(), c);
  return resources::EventProxy<Res>(r);
}
template <typename Pol, typename Res, typename K, typename V, typename C = operators::less<K>,
          detail::enable_if_resource<Res> = 0>
resources::EventProxy<Res> stable_sort_pairs(Res r, Span<K> k, Span<V> v, C c = C{}) {
  auto bound = bind_resource(r);
  (void)bound;
  if (k.size() > 1) sort_stable_pairs(Pol{}, k.begin(), k.end(), v.begin(), c);
  return resources::EventProxy<Res>(r);
}

template <typename Pol, typename T, typename C = operators::less<T>>
RAJA_COMPAT_RES_T(Pol) sort(Span<T> s, C c = C{}) {
  return sort<Pol>(RAJA_COMPAT_DEFAULT_RES(Pol), s, c);
}
template <typename Pol, typename T, typename C = operators::less<T>>
RAJA_COMPAT_RES_T(Pol) stable_sort(Span<T> s, C c = C{}) {
  return stable_sort<Pol>(RAJA_COMPAT_DEFAULT_RES(Pol), s, c);
}
template <typename Pol, typename K, typename V, typename C = operators::less<K>>
RAJA_COMPAT_RES_T(Pol) sort_pairs(Span<K> k, Span<V> v, C c = C{}) {
  return sort_pairs<Pol>(RAJA_COMPAT_DEFAULT_RES(Pol), k, v, c);
}
template <typename Pol, typename K, typename V, typename C = operators::less<K>>
RAJA_COMPAT_RES_T(Pol) stable_sort_pairs(Span<K> k, Span<V> v, C c = C{}) {
  return stable_sort_pairs<Pol>(RAJA_COMPAT_DEFAULT_RES(Pol), k, v, c);
}
#undef RAJA_COMPAT_DEFAULT_RES
#undef RAJA_COMPAT_RES_T

// ------------------------------------------------------------- WorkGroup
// pattern/WorkGroup.hpp:117-530.  Host runners execute the loops in
// enqueue order (ordered) like the reference's WorkRunnerForallOrdered.
// WorkGroup execution policies (policy/sequential/policy.hpp:86,
// policy/openmp/policy.hpp:295): the host runners execute the loops with
// the matching forall policy
using seq_work = seq_exec;
using omp_work = omp_parallel_for_exec;
struct ordered {};
struct reverse_ordered {};
struct unordered {};
struct array_of_pointers {};
struct ragged_array_of_objects {};
struct constant_stride_array_of_objects {};
// dispatch policies (policy/WorkGroup.hpp): how a runner calls the stored
// loops; every b200 and host runner here calls them directly, so the
// choice is accepted and has no effect
struct indirect_function_call_dispatch {};
struct indirect_virtual_function_dispatch {};
template <typename... Callables>
struct direct_dispatch {};
template <typename EXEC, typename ORDER = ordered, typename STORAGE = ragged_array_of_objects,
          typename DISPATCH = indirect_function_call_dispatch>
struct WorkGroupPolicy {
  using exec_policy = EXEC;
  using order_policy = ORDER;
};
template <typename... Args>
struct xargs {};

template <typename POL, typename Index, typename XArgs = xargs<>, typename Alloc = void>
class WorkPool;
template <typename POL, typename Index, typename XArgs = xargs<>, typename Alloc = void>
class WorkGroup;
template <typename POL, typename Index, typename XArgs = xargs<>, typename Alloc = void>
class WorkSite {
 public:
  using resource_type = typename resources::get_resource<typename POL::exec_policy>::type;
  WorkSite() : m_resource(resource_type::get_default()) {}
  explicit WorkSite(resource_type r) : m_resource(r) {}
  resource_type get_resource() const { return m_resource; }
  void clear() {}

 private:
  resource_type m_resource;
};

namespace detail {
// Host runner: type-erased loops kept in enqueue order.
template <typename Index>
struct HostLoops {
  std::vector<std::function<void()>> loops;
};
}  // namespace detail

template <typename EXEC, typename ORDER, typename STORAGE, typename DISPATCH, typename Index, typename Alloc>
class WorkPool<WorkGroupPolicy<EXEC, ORDER, STORAGE, DISPATCH>, Index, xargs<>, Alloc> {
 public:
  using policy = WorkGroupPolicy<EXEC, ORDER, STORAGE, DISPATCH>;
  WorkPool() = default;
  template <typename A>
  explicit WorkPool(const A&) {}  // the allocator (pattern/WorkGroup.hpp:272-300); host loops need none
  // The loops run through forall_impl at run(), inside the group's launch
  // hooks; with plugins registered, each enqueue brackets the body copy with
  // the capture hooks (pattern/WorkGroup.hpp:287-296).
  template <typename Seg, typename Body>
  void enqueue(Seg seg, Body body) {
    if (util::PluginRegistry::empty()) {
      m_loops.push_back([seg, body]() { forall_impl(EXEC{}, seg, body); });
      return;
    }
    const util::PluginContext ctx = util::make_context<EXEC>(std::string());
    util::callPreCapturePlugins(ctx);
    auto captured = util::trigger_updates_before(body);
    m_loops.push_back([seg, captured]() { forall_impl(EXEC{}, seg, captured); });
    util::callPostCapturePlugins(ctx);
  }
  void reserve(size_t n, size_t) { m_loops.reserve(n); }
  size_t num_loops() const { return m_loops.size(); }
  WorkGroup<policy, Index, xargs<>, Alloc> instantiate() {
    WorkGroup<policy, Index, xargs<>, Alloc> g;
    g.m_loops = std::move(m_loops);
    m_loops.clear();
    return g;
  }

 private:
  std::vector<std::function<void()>> m_loops;
};

template <typename EXEC, typename ORDER, typename STORAGE, typename DISPATCH, typename Index, typename Alloc>
class WorkGroup<WorkGroupPolicy<EXEC, ORDER, STORAGE, DISPATCH>, Index, xargs<>, Alloc> {
 public:
  using policy = WorkGroupPolicy<EXEC, ORDER, STORAGE, DISPATCH>;
  using resource_type = typename resources::get_resource<EXEC>::type;
  // run([resource]) (pattern/WorkGroup.hpp:357-370): the loops run on the
  // resource, the policy's default one when none is given.
  // With plugins registered, the launch hooks bracket the whole run
  // (pattern/WorkGroup.hpp:515-528).
  WorkSite<policy, Index, xargs<>, Alloc> run(resource_type r) {
    auto bound = bind_resource(r);
    (void)bound;
    const bool hooks = !util::PluginRegistry::empty();
    const util::PluginContext ctx = util::make_context<EXEC>(std::string());
    if (hooks) util::callPreLaunchPlugins(ctx);
    if (std::is_same<ORDER, reverse_ordered>::value) {
      for (auto it = m_loops.rbegin(); it != m_loops.rend(); ++it) (*it)();
    } else {
      for (auto& f : m_loops) f();
    }
    if (hooks) util::callPostLaunchPlugins(ctx);
    return WorkSite<policy, Index, xargs<>, Alloc>(r);
  }
  WorkSite<policy, Index, xargs<>, Alloc> run() { return run(resource_type::get_default()); }
  void clear() { m_loops.clear(); }
  std::vector<std::function<void()>> m_loops;
};

template <typename Pol>
void synchronize() {}

}  // namespace RAJA
