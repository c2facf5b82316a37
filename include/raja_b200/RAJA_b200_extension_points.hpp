// RAJA_b200_extension_points.hpp -- the b200 policies on an installed RAJA.
//
// Included by RAJA_b200.hpp when the front-end is RAJA itself rather than
// raja_compat.  Each overload below has the shape of the extension point
// that the reference's CUDA back-end provides, so RAJA's unchanged
// front-ends (RAJA::forall, the scans, the sorts) reach the b200 kernels
// when an application switches its policy alias:
//
//   forall_impl(resources::Cuda, b200_exec<B, A> const&, Iterable&&,
//               LoopBody&&, ForallParam) -> resources::EventProxy<Cuda>
//                                    policy/cuda/forall.hpp:554-573
//   forall_impl(resources::Cuda, ExecPolicy<seq_segit, b200_exec<B, A>>,
//               const TypedIndexSet<...>&, LoopBody&&)
//                                    policy/cuda/forall.hpp:675-692
//   wrap::forall(Res, ExecPolicy<seq_segit, b200_exec<B, A>>,
//               const TypedIndexSet<...>&, LoopBody, ForallParams)
//               (the front-end's IndexSet dispatch, pattern/forall.hpp:
//               279-299): one launch over every segment
//   impl::scan::{inclusive_inplace, exclusive_inplace, inclusive, exclusive}
//               (resources::Cuda, b200_exec<B, A>, ...)
//                                    policy/cuda/scan.hpp:45-235
//   impl::sort::{stable, unstable, stable_pairs, unstable_pairs}
//               (resources::Cuda, b200_exec<B, A>, ...)
//                                    policy/cuda/sort.hpp:92-653
//   param_init / param_combine / param_resolve for expt::Reduce and
//               expt::ReduceLoc params on b200_exec
//                                    policy/cuda/params/reduce.hpp:21-62
//   detail::WorkRunner<b200_work<B, A>, order, dispatch, allocator, index>
//               (enqueue / run / clear, behind RAJA's unchanged WorkPool,
//               WorkGroup and WorkSite)
//                                    policy/cuda/WorkGroup/WorkRunner.hpp:38-407
//
// The resource is camp's CUDA resource (camp::resources::Cuda, present in
// a RAJA installed with CUDA).  The reducer classes ReduceSum<b200_reduce,
// T> and the others are specialisations of RAJA's own class templates and
// come from RAJA_b200.hpp unchanged.
#pragma once

namespace RAJA {

namespace resources {
template <int BLOCK, bool Async>
struct get_resource<b200_exec<BLOCK, Async>> {
  using type = camp::resources::Cuda;
};
template <int BLOCK, bool Async>
struct get_resource<ExecPolicy<seq_segit, b200_exec<BLOCK, Async>>> {
  using type = camp::resources::Cuda;
};
}  // namespace resources

#if !defined(RAJA_CUDA_ACTIVE)
// RAJA marks camp's CUDA resource a resource only with its own CUDA
// back-end compiled in; the b200 policies use it either way.
namespace type_traits {
template <>
struct is_resource<camp::resources::Cuda> : std::true_type {};
}  // namespace type_traits
#endif

namespace b200 {
namespace detail {

// The b200 stream for the duration of one call is the resource's stream.
class ResourceStream {
 public:
  explicit ResourceStream(cudaStream_t s) : prev_(stream()) { stream() = s; }
  ~ResourceStream() { stream() = prev_; }
  ResourceStream(const ResourceStream&) = delete;
  ResourceStream& operator=(const ResourceStream&) = delete;

 private:
  cudaStream_t prev_;
};

}  // namespace detail
}  // namespace b200

// ---- scans (policy/cuda/scan.hpp:45-235): libb200prims' single-pass scan
namespace impl {
namespace scan {

template <int BLOCK, bool Async, typename Iter, typename Function>
RAJA_INLINE resources::EventProxy<resources::Cuda> inclusive_inplace(resources::Cuda cuda_res,
                                                                      b200_exec<BLOCK, Async>, Iter begin,
                                                                      Iter end, Function) {
  using T = std::remove_cv_t<std::remove_reference_t<decltype(*begin)>>;
  static_assert(std::is_pointer<Iter>::value, "b200 scans take contiguous arrays (pointers)");
  constexpr int op = b200::detail::scan_op<Function, T>();
  static_assert(op >= 0, "b200 scans take operators::plus / minimum / maximum");
  b200::detail::ResourceStream bound(cuda_res.get_stream());
  b200::check(b200::detail::scan_incl<T>(begin, begin, size_t(end - begin), op, b200::stream()),
              "b200 inclusive_scan_inplace");
  if (!Async) b200::wait();
  return resources::EventProxy<resources::Cuda>(cuda_res);
}

template <int BLOCK, bool Async, typename Iter, typename Function, typename TT>
RAJA_INLINE resources::EventProxy<resources::Cuda> exclusive_inplace(resources::Cuda cuda_res,
                                                                      b200_exec<BLOCK, Async>, Iter begin,
                                                                      Iter end, Function, TT init) {
  using T = std::remove_cv_t<std::remove_reference_t<decltype(*begin)>>;
  static_assert(std::is_pointer<Iter>::value, "b200 scans take contiguous arrays (pointers)");
  constexpr int op = b200::detail::scan_op<Function, T>();
  static_assert(op >= 0, "b200 scans take operators::plus / minimum / maximum");
  b200::detail::ResourceStream bound(cuda_res.get_stream());
  b200::check(b200::detail::scan_excl<T>(begin, begin, size_t(end - begin), op, T(init), b200::stream()),
              "b200 exclusive_scan_inplace");
  if (!Async) b200::wait();
  return resources::EventProxy<resources::Cuda>(cuda_res);
}

template <int BLOCK, bool Async, typename InputIter, typename OutputIter, typename Function>
RAJA_INLINE resources::EventProxy<resources::Cuda> inclusive(resources::Cuda cuda_res,
                                                              b200_exec<BLOCK, Async>, InputIter begin,
                                                              InputIter end, OutputIter out, Function) {
  using T = std::remove_cv_t<std::remove_reference_t<decltype(*out)>>;
  static_assert(std::is_pointer<InputIter>::value && std::is_pointer<OutputIter>::value,
                "b200 scans take contiguous arrays (pointers)");
  constexpr int op = b200::detail::scan_op<Function, T>();
  static_assert(op >= 0, "b200 scans take operators::plus / minimum / maximum");
  b200::detail::ResourceStream bound(cuda_res.get_stream());
  b200::check(b200::detail::scan_incl<T>(begin, out, size_t(end - begin), op, b200::stream()),
              "b200 inclusive_scan");
  if (!Async) b200::wait();
  return resources::EventProxy<resources::Cuda>(cuda_res);
}

template <int BLOCK, bool Async, typename InputIter, typename OutputIter, typename Function,
          typename TT>
RAJA_INLINE resources::EventProxy<resources::Cuda> exclusive(resources::Cuda cuda_res,
                                                              b200_exec<BLOCK, Async>, InputIter begin,
                                                              InputIter end, OutputIter out, Function,
                                                              TT init) {
  using T = std::remove_cv_t<std::remove_reference_t<decltype(*out)>>;
  static_assert(std::is_pointer<InputIter>::value && std::is_pointer<OutputIter>::value,
                "b200 scans take contiguous arrays (pointers)");
  constexpr int op = b200::detail::scan_op<Function, T>();
  static_assert(op >= 0, "b200 scans take operators::plus / minimum / maximum");
  b200::detail::ResourceStream bound(cuda_res.get_stream());
  b200::check(b200::detail::scan_excl<T>(begin, out, size_t(end - begin), op, T(init), b200::stream()),
              "b200 exclusive_scan");
  if (!Async) b200::wait();
  return resources::EventProxy<resources::Cuda>(cuda_res);
}

}  // namespace scan

// ---- sorts (policy/cuda/sort.hpp:92-653): libb200prims' stable radix
// sort; the unstable forms give the stable result
namespace sort {

template <int BLOCK, bool Async, typename Iter, typename Compare>
RAJA_INLINE resources::EventProxy<resources::Cuda> stable(resources::Cuda cuda_res,
                                                           b200_exec<BLOCK, Async>, Iter begin, Iter end,
                                                           Compare) {
  using K = std::remove_cv_t<std::remove_reference_t<decltype(*begin)>>;
  static_assert(std::is_pointer<Iter>::value, "b200 sorts take contiguous arrays (pointers)");
  b200::detail::ResourceStream bound(cuda_res.get_stream());
  b200::check(b200d::keys<K>(begin, size_t(end - begin), b200d::desc_of<Compare, K>(), b200::stream()),
              "b200 sort");
  if (!Async) b200::wait();
  return resources::EventProxy<resources::Cuda>(cuda_res);
}
template <int BLOCK, bool Async, typename Iter, typename Compare>
RAJA_INLINE resources::EventProxy<resources::Cuda> unstable(resources::Cuda cuda_res,
                                                             b200_exec<BLOCK, Async> p, Iter begin, Iter end,
                                                             Compare c) {
  return stable(cuda_res, p, begin, end, c);
}
template <int BLOCK, bool Async, typename KeyIter, typename ValIter, typename Compare>
RAJA_INLINE resources::EventProxy<resources::Cuda> stable_pairs(resources::Cuda cuda_res,
                                                                 b200_exec<BLOCK, Async>, KeyIter keys_begin,
                                                                 KeyIter keys_end, ValIter vals_begin,
                                                                 Compare) {
  using K = std::remove_cv_t<std::remove_reference_t<decltype(*keys_begin)>>;
  using V = std::remove_cv_t<std::remove_reference_t<decltype(*vals_begin)>>;
  static_assert(std::is_pointer<KeyIter>::value && std::is_pointer<ValIter>::value,
                "b200 sorts take contiguous arrays (pointers)");
  b200::detail::ResourceStream bound(cuda_res.get_stream());
  b200::check(b200d::pairs<K, V>(keys_begin, vals_begin, size_t(keys_end - keys_begin),
                                 b200d::desc_of<Compare, K>(), b200::stream()),
              "b200 sort_pairs");
  if (!Async) b200::wait();
  return resources::EventProxy<resources::Cuda>(cuda_res);
}
template <int BLOCK, bool Async, typename KeyIter, typename ValIter, typename Compare>
RAJA_INLINE resources::EventProxy<resources::Cuda> unstable_pairs(resources::Cuda cuda_res,
                                                                   b200_exec<BLOCK, Async> p,
                                                                   KeyIter keys_begin, KeyIter keys_end,
                                                                   ValIter vals_begin, Compare c) {
  return stable_pairs(cuda_res, p, keys_begin, keys_end, vals_begin, c);
}

}  // namespace sort
}  // namespace impl

}  // namespace RAJA

// ---- forall over an IndexSet.  RAJA's front-end hands IndexSet policies
// to wrap::forall by qualified name (pattern/forall.hpp:383-417), whose
// generic form runs one forall per segment (pattern/forall.hpp:279-299), as
// the CUDA back-end's IndexSet forall_impl does (policy/cuda/forall.hpp:
// 675-706).  This more specialised overload, declared before RAJA's
// front-end, runs every range, strided and list segment in one launch; it
// is defined at the end of this header.
#include "RAJA/index/IndexSet.hpp"
#include "RAJA/policy/sequential/policy.hpp"

namespace RAJA {
namespace wrap {
template <typename Res, int BLOCK, bool Async, typename... SegmentTypes, typename LoopBody, typename ForallParams>
resources::EventProxy<Res> forall(Res r, ExecPolicy<seq_segit, b200_exec<BLOCK, Async>>,
                                  const TypedIndexSet<SegmentTypes...>& iset, LoopBody loop_body,
                                  ForallParams f_params);
}  // namespace wrap
}  // namespace RAJA

// ---------------------------------------------------------------------------
// RAJA itself, then the overloads that need its front-end types.
#include "RAJA/RAJA.hpp"

namespace RAJA {

namespace b200 {
namespace detail {

// forall over any random-access iterable: element i is begin[i].
template <int BLOCK, class Body, class Iter>
__global__ void __launch_bounds__(BLOCK) forall_iter_kernel(Body body_in, Iter begin, long long len) {
  Body body(body_in);  // per-thread copy: captured b200 reducers privatise here
  const long long stride = (long long)gridDim.x * BLOCK;
  for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < len; i += stride)
    body(begin[i]);
}

// The combine kind of an expt reducer param of RAJA (Reducer<Op, T, VOp>,
// pattern/params/reducer.hpp:68-215), from its operator and value type.
template <class R>
struct RefParamKind;
template <template <class, class, class> class Op, class T, class VOp>
struct RefParamKind<expt::detail::Reducer<Op<T, T, T>, T, VOp>> {
  using type = typename std::conditional<
      std::is_same<Op<T, T, T>, operators::plus<T, T, T>>::value, SumK<T>,
      typename std::conditional<
          std::is_same<Op<T, T, T>, operators::minimum<T, T, T>>::value, MinK<T>,
          typename std::conditional<
              std::is_same<Op<T, T, T>, operators::maximum<T, T, T>>::value, MaxK<T>,
              typename std::conditional<std::is_same<Op<T, T, T>, operators::bit_or<T, T, T>>::value,
                                        OrK<T>, AndK<T>>::type>::type>::type>::type;
  using valop = VOp;
  static T to_target(typename type::V v) { return v; }
  static B200_HOST_DEVICE typename type::V from_valop(const VOp& v) { return v.val; }
};
template <template <class, class, class> class Op, class T, class I, class VOp>
struct RefParamKind<expt::detail::Reducer<Op<expt::ValLoc<T, I>, expt::ValLoc<T, I>, expt::ValLoc<T, I>>,
                                          expt::ValLoc<T, I>, VOp>> {
  using VL = expt::ValLoc<T, I>;
  static constexpr bool is_min = std::is_same<Op<VL, VL, VL>, operators::minimum<VL, VL, VL>>::value;
  using type = LocK<T, I, is_min>;
  using valop = VOp;
  static VL to_target(typename type::V v) { return VL(v.val, v.loc); }
  static B200_HOST_DEVICE typename type::V from_valop(const VOp& v) { return {v.val.val, v.val.loc}; }
};

template <class R>
using RefSlot = DevSlot<typename RefParamKind<R>::type::V>;

template <class R>
__device__ inline void ref_combine_param(const RefSlot<R>& slot, const typename RefParamKind<R>::valop& v) {
  using K = typename RefParamKind<R>::type;
  grid_combine(slot, RefParamKind<R>::from_valop(v), [](typename K::V a, typename K::V b) { return K::merge(a, b); });
}

// Each thread runs the loop with its own ValOps (identities), in parameter
// order, then every parameter is combined across the grid.
template <int BLOCK, class Body, class Iter, class... R, size_t... I>
__device__ inline void ref_params_body(Body& body, Iter begin, long long len,
                                       const DTuple<RefSlot<R>...>& slots, std::index_sequence<I...>) {
  DTuple<typename RefParamKind<R>::valop...> vals{};
  const long long stride = (long long)gridDim.x * BLOCK;
  for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < len; i += stride)
    body(begin[i], dget<I>(vals)...);
  (ref_combine_param<R>(dget<I>(slots), dget<I>(vals)), ...);
}

template <int BLOCK, class Body, class Iter, class... R>
__global__ void __launch_bounds__(BLOCK)
forall_ref_params_kernel(Body body, Iter begin, long long len, DTuple<RefSlot<R>...> slots) {
  ref_params_body<BLOCK, Body, Iter, R...>(body, begin, len, slots, std::index_sequence_for<R...>{});
}

// What param_init hands the kernel and param_resolve reads back: one slot
// (partials, ticket, result cell) per reducer parameter.
template <size_t N>
struct ParamLaunchInfo {
  unsigned grid = 1;
  cudaStream_t stream = nullptr;
  SlotMem mem[N + 1];
  size_t next = 0;
};

template <class R, class Info>
inline RefSlot<R> param_slot(Info& info) {
  return alloc_slot<typename RefParamKind<R>::type::V>(info.grid, info.stream, &info.mem[info.next++]);
}

}  // namespace detail
}  // namespace b200

// ---- expt params on b200_exec (policy/cuda/params/reduce.hpp:21-62): the
// launch's device slot for one reducer, the in-kernel combine, and the
// fold of the result into the user's target after the launch.
template <int BLOCK, bool Async, class Op, class T, class VOp, class Info>
b200::detail::RefSlot<expt::detail::Reducer<Op, T, VOp>> param_init(
    const b200_exec<BLOCK, Async>&, expt::detail::Reducer<Op, T, VOp>&, Info& info) {
  return b200::detail::param_slot<expt::detail::Reducer<Op, T, VOp>>(info);
}
template <int BLOCK, bool Async, class Op, class T, class VOp>
__device__ void param_combine(const b200_exec<BLOCK, Async>&,
                              const b200::detail::RefSlot<expt::detail::Reducer<Op, T, VOp>>& slot,
                              const VOp& v) {
  b200::detail::ref_combine_param<expt::detail::Reducer<Op, T, VOp>>(slot, v);
}
template <int BLOCK, bool Async, class Op, class T, class VOp>
void param_resolve(const b200_exec<BLOCK, Async>&, expt::detail::Reducer<Op, T, VOp>& red,
                   const b200::detail::SlotMem& mem) {
  using RK = b200::detail::RefParamKind<expt::detail::Reducer<Op, T, VOp>>;
  red.combineTarget(RK::to_target(b200::detail::read_cell<typename RK::type::V>(mem.cell)));
}

namespace b200 {
namespace detail {

template <int BLOCK, bool Async, class Iter, class Body, class... R, size_t... I>
void forall_ref_params(const b200_exec<BLOCK, Async>& pol, Iter begin, long long len, Body&& body,
                       std::index_sequence<I...>, R&... reds) {
  using B = std::decay_t<Body>;
  ParamLaunchInfo<sizeof...(R)> info;
  info.stream = stream();
  tune::shaped_launch<BLOCK, tune::Tag<5, B, Iter, R...>>(
      "forall params", len > 0 ? len : 1, info.stream, [&](auto NB, int items) {
        auto k = forall_ref_params_kernel<NB(), B, Iter, R...>;
        info.grid = grid_for<forall_ref_params_kernel<NB(), B, Iter, R...>>(NB(), len > 0 ? len : 1, items);
        DTuple<RefSlot<R>...> slots{param_init(pol, reds, info)...};
        k<<<info.grid, NB(), 0, info.stream>>>(body, begin, len, slots);
      });
  check_cuda(cudaGetLastError(), "b200 forall params");
  // param_resolve waits for the launch, as the reference's does
  const uint32_t* status = nullptr;
  check(b200_status_word_address(&status), "b200 status word");
  check_cuda(cudaStreamSynchronize(info.stream), "b200 forall params");
  const bool ok = __atomic_load_n(status, __ATOMIC_ACQUIRE) == 0;
  if (ok) (param_resolve(pol, reds, info.mem[I]), ...);
  for (size_t i = 0; i < sizeof...(R); ++i) {
    release_cell(info.mem[i].cell);
    if (info.mem[i].block) cudaFreeAsync(info.mem[i].block, info.stream);
  }
  if (!ok) wait();  // reports the device status and throws
}

template <class T>
struct is_expt_reducer : std::false_type {};
template <class Op, class T, class VOp>
struct is_expt_reducer<expt::detail::Reducer<Op, T, VOp>> : std::true_type {};

template <int BLOCK, bool Async, class Iter, class Body, class Reds, size_t... J>
void forall_ref_unpack(const b200_exec<BLOCK, Async>& pol, Iter begin, long long len, Body&& body,
                       Reds& reds, std::index_sequence<J...>) {
  forall_ref_params(pol, begin, len, std::forward<Body>(body), std::index_sequence<J...>{},
                    camp::get<J>(reds)...);
}


// The reducer parameters of a ForallParamPack, in order (kernel names and
// other non-reducer params carry no lambda argument).
template <int BLOCK, bool Async, class Iter, class Body, class Tup, size_t... I>
void forall_ref_dispatch_params(const b200_exec<BLOCK, Async>& pol, Iter begin, long long len,
                                Body&& body, Tup& params, std::index_sequence<I...>) {
  auto reds = ::RAJA::expt::detail::filter_reducers(params);
  constexpr size_t nred = camp::tuple_size<decltype(reds)>::value;
  forall_ref_unpack(pol, begin, len, std::forward<Body>(body), reds, std::make_index_sequence<nred>{});
}
}  // namespace detail
}  // namespace b200

// ---- forall over an iterable (policy/cuda/forall.hpp:554-573)
template <typename Iterable, typename LoopBody, int BLOCK, bool Async, typename ForallParam>
RAJA_INLINE concepts::enable_if_t<resources::EventProxy<resources::Cuda>,
                                  expt::type_traits::is_ForallParamPack<ForallParam>>
forall_impl(resources::Cuda cuda_res, b200_exec<BLOCK, Async> const& pol, Iterable&& iter,
            LoopBody&& loop_body, ForallParam f_params) {
  using Iterator = camp::decay<decltype(std::begin(iter))>;
  using B = camp::decay<LoopBody>;
  Iterator begin = std::begin(iter);
  const long long len = (long long)std::distance(begin, std::end(iter));
  b200::detail::ResourceStream bound(cuda_res.get_stream());
  if (len > 0) {
    if constexpr (expt::type_traits::is_ForallParamPack_empty<ForallParam>::value) {
      cudaStream_t s = b200::stream();
      b200::tune::shaped_launch<BLOCK, b200::tune::Tag<6, B, Iterator>>("forall", len, s, [&](auto NB, int items) {
        auto k = b200::detail::forall_iter_kernel<NB(), B, Iterator>;
        const unsigned g =
            b200::detail::grid_for<b200::detail::forall_iter_kernel<NB(), B, Iterator>>(NB(), len, items);
        B lb = b200::detail::LaunchCopy<B>::make(loop_body, g, s);
        k<<<g, NB(), 0, s>>>(lb, begin, len);
      });
      b200::detail::finish<Async>("b200 forall");
    } else {
      b200::detail::forall_ref_dispatch_params(pol, begin, len, std::forward<LoopBody>(loop_body),
                                               f_params.param_tup,
                                               std::make_index_sequence<0>{});
    }
  }
  return resources::EventProxy<resources::Cuda>(cuda_res);
}

// ---- IndexSet segments in one launch
namespace b200 {
namespace detail {

// Parameters of one segment of RAJA's (range, strided, list) for the
// one-launch table; *ok = false for another segment type.  RANGES: the
// IndexSet holds range segments only, and the table keeps their bases.
template <class T, bool RANGES>
struct RefSegDesc {
  template <class Seg>
  void operator()(const Seg& g, unsigned char* descs, size_t i, long long* len, bool* ok) const {
    using G = std::decay_t<Seg>;
    *len = (long long)g.size();
    if constexpr (RANGES) {
      reinterpret_cast<long long*>(descs)[i] = (long long)*g.begin();
    } else {
      SegDesc& d = reinterpret_cast<SegDesc*>(descs)[i];
      if constexpr (std::is_same<G, TypedRangeSegment<T>>::value) {
        d = SegDesc{(long long)*g.begin(), 1};
      } else if constexpr (std::is_same<G, TypedRangeStrideSegment<T>>::value) {
        d = SegDesc{(long long)*g.begin(), *len > 1 ? (long long)(*(g.begin() + 1) - *g.begin()) : 1};
      } else if constexpr (std::is_same<G, TypedListSegment<T>>::value) {
        d = SegDesc{(long long)reinterpret_cast<intptr_t>(g.begin()), kListStep};
      } else {
        *ok = false;
      }
    }
  }
};

// Whether a ForallParamPack holds reducers (a kernel name alone does not).
template <class FP>
constexpr bool has_reducer_params() {
  if constexpr (expt::type_traits::is_ForallParamPack_empty<FP>::value) {
    return false;
  } else {
    using R = decltype(::RAJA::expt::detail::filter_reducers(std::declval<FP&>().param_tup));
    return camp::tuple_size<std::decay_t<R>>::value > 0;
  }
}

template <class Res>
inline cudaStream_t res_stream(Res& r) {
  if constexpr (std::is_same<std::decay_t<Res>, camp::resources::Cuda>::value) return r.get_stream();
  else return stream();
}

// Every segment in one launch on the resource's stream; IndexSets with
// another segment type, or with reducer params, run per segment.
template <int BLOCK, bool Async, class Res, class LoopBody, class ForallParams, class... SegmentTypes>
void ref_indexset_forall(Res& r, const TypedIndexSet<SegmentTypes...>& iset, LoopBody&& loop_body,
                         ForallParams f_params) {
  using T = typename TypedIndexSet<SegmentTypes...>::value_type;
  const int nseg = int(iset.getNumSegments());
  ResourceStream bound(res_stream(r));
  bool ok = !has_reducer_params<ForallParams>();
  if (ok && nseg > 0) {
    constexpr bool kRanges = (std::is_same<SegmentTypes, TypedRangeSegment<T>>::value && ...);
    size_t db = 0;
    const size_t bytes = seg_table_bytes<kRanges>(nseg, &db);
    unsigned char* h = pinned_stage().get(bytes);
    long long* prefix = reinterpret_cast<long long*>(h + db);
    long long acc = 0;
    prefix[0] = 0;
    for (int i = 0; i < nseg && ok; ++i) {
      long long len = 0;
      iset.segmentCall(size_t(i), RefSegDesc<T, kRanges>{}, h, size_t(i), &len, &ok);
      acc += len;
      prefix[size_t(i) + 1] = acc;
    }
    if (ok) {
      indexset_launch<BLOCK, Async, kRanges, T>(h, nseg, db, bytes, acc, std::forward<LoopBody>(loop_body));
      return;
    }
  } else if (ok) {
    return;  // no segments
  }
  for (int i = 0; i < nseg; ++i)
    iset.segmentCall(size_t(i), ::RAJA::detail::CallForall{}, b200_exec<BLOCK, true>(), loop_body, r, f_params);
  if (!Async) wait();
}

}  // namespace detail
}  // namespace b200

// the CUDA back-end's extension point (policy/cuda/forall.hpp:675-692)
template <typename LoopBody, int BLOCK, bool Async, typename... SegmentTypes>
RAJA_INLINE resources::EventProxy<resources::Cuda> forall_impl(
    resources::Cuda r, ExecPolicy<seq_segit, b200_exec<BLOCK, Async>>,
    const TypedIndexSet<SegmentTypes...>& iset, LoopBody&& loop_body) {
  b200::detail::ref_indexset_forall<BLOCK, Async>(r, iset, std::forward<LoopBody>(loop_body),
                                                  expt::ForallParamPack<>());
  return resources::EventProxy<resources::Cuda>(r);
}

// ---- WorkGroup (pattern/WorkGroup.hpp:207-530): RAJA's WorkPool /
// WorkGroup / WorkSite stay unchanged and call their runner,
// detail::WorkRunner<exec, order, dispatch, allocator, index, args...>
// (policy/cuda/WorkGroup/WorkRunner.hpp:38-407 for cuda_work).  The b200
// runner keeps the loops itself (RAJA's work storage stays empty): its
// enqueue captures the range and the body, its run launches every loop
// in one persistent launch (b200_unordered) or one launch per loop
// (ordered, reverse_ordered), with captured b200_reduce reducers combined
// inside the launch.
namespace detail {
template <int BLOCK, bool Async, typename ORDER, typename DISPATCH, typename ALLOC, typename INDEX>
struct WorkRunner<b200_work<BLOCK, Async>, ORDER, DISPATCH, ALLOC, INDEX> {
  static_assert(std::is_same<ORDER, b200_unordered>::value || std::is_same<ORDER, ordered>::value ||
                    std::is_same<ORDER, reverse_ordered>::value,
                "b200_work runs b200_unordered, ordered or reverse_ordered WorkGroups");
  using exec_policy = b200_work<BLOCK, Async>;
  using order_policy = ORDER;
  using dispatch_policy = DISPATCH;
  using Allocator = ALLOC;
  using index_type = INDEX;
  using resource_type = resources::Cuda;
  // RAJA's WorkStorage is typed by a dispatcher; the b200 runner stores
  // nothing there, so the sequential runner's dispatcher serves.
  using dispatcher_type = typename WorkRunner<seq_work, ordered, DISPATCH, ALLOC, INDEX>::dispatcher_type;

  WorkRunner() = default;
  WorkRunner(const WorkRunner&) = delete;
  WorkRunner& operator=(const WorkRunner&) = delete;
  WorkRunner(WorkRunner&&) noexcept = default;
  WorkRunner& operator=(WorkRunner&&) noexcept = default;

  template <typename WorkContainer, typename Iterable, typename LoopBody>
  void enqueue(WorkContainer&, Iterable&& iter, LoopBody&& loop_body) {
    using Seg = camp::decay<Iterable>;
    static_assert(std::is_same<Seg, TypedRangeSegment<typename Seg::value_type>>::value,
                  "b200_work loops take range segments");
    const long long begin = (long long)*std::begin(iter);
    const long long len = (long long)std::distance(std::begin(iter), std::end(iter));
    if (len > 0) core_.enqueue(begin, len, loop_body);
  }

  using per_run_storage = int;

  template <typename WorkContainer>
  per_run_storage run(WorkContainer const&, resource_type r) {
    b200::detail::ResourceStream bound(r.get_stream());
    constexpr b200::detail::WgOrder o =
        std::is_same<ORDER, b200_unordered>::value
            ? b200::detail::kWgUnordered
            : (std::is_same<ORDER, reverse_ordered>::value ? b200::detail::kWgReverse : b200::detail::kWgOrdered);
    core_.run(b200::stream(), o);
    if (!Async) b200::wait();
    return 0;
  }

  void clear() { core_.clear(); }

  // the tuner's state for b200_work<0>
  b200::tune::Report tuning() const { return core_.tuning(); }

 private:
  b200::detail::WgCore<BLOCK> core_;
};
}  // namespace detail

// the front-end's IndexSet dispatch (declared before RAJA/RAJA.hpp)
namespace wrap {
template <typename Res, int BLOCK, bool Async, typename... SegmentTypes, typename LoopBody, typename ForallParams>
resources::EventProxy<Res> forall(Res r, ExecPolicy<seq_segit, b200_exec<BLOCK, Async>>,
                                  const TypedIndexSet<SegmentTypes...>& iset, LoopBody loop_body,
                                  ForallParams f_params) {
  b200::detail::ref_indexset_forall<BLOCK, Async>(r, iset, std::move(loop_body), f_params);
  return resources::EventProxy<Res>(r);
}
}  // namespace wrap

}  // namespace RAJA
