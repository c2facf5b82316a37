// Clean-room subset of the camp metaprogramming library, written from
// RAJA's call sites (the camp sources are not part of the RAJA tree) so
// that RAJA's own host policy headers compile for the oracle's reference
// build.  Test infrastructure only: nothing in the product includes it.
//
// defines.hpp: basic macros and the index type.
#ifndef CAMP_SUBSET_DEFINES_HPP
#define CAMP_SUBSET_DEFINES_HPP

#include <cstddef>
#include <initializer_list>
#include <type_traits>
#include <utility>

#if defined(__CUDACC__)
#define CAMP_HOST_DEVICE __host__ __device__
#define CAMP_DEVICE __device__
#define CAMP_HOST __host__
#define CAMP_SUPPRESS_HD_WARN _Pragma("nv_exec_check_disable")
#else
#define CAMP_HOST_DEVICE
#define CAMP_DEVICE
#define CAMP_HOST
#define CAMP_SUPPRESS_HD_WARN
#endif
#define CAMP_INLINE inline
#define CAMP_CONSTEXPR14 constexpr

// Evaluate an expression that contains an unexpanded parameter pack once
// per pack element, left to right.
#define CAMP_EXPAND(...) \
  ((void)::std::initializer_list<int>{0, ((void)(__VA_ARGS__), 0)...})

namespace camp
{
using idx_t = std::ptrdiff_t;
using nullptr_t = decltype(nullptr);

// swallow any arguments (used to expand packs for their side effects)
template <typename... Ts>
CAMP_HOST_DEVICE constexpr void sink(Ts const&...)
{
}
}  // namespace camp

#endif
