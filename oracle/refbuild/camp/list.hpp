// Clean-room camp subset (test infrastructure): type lists.
#ifndef CAMP_SUBSET_LIST_HPP
#define CAMP_SUBSET_LIST_HPP

#include "camp/number.hpp"

namespace camp
{
template <typename... Ts>
struct list {
  using type = list;
};

struct nil {
};

template <typename L>
struct size;
template <typename... Ts>
struct size<list<Ts...>> : num<idx_t(sizeof...(Ts))> {
};
template <typename T, T... Vs>
struct size<int_seq<T, Vs...>> : num<idx_t(sizeof...(Vs))> {
};

// at<List, Index>: the element at a position (an integral constant or an
// index value); at_v / at_t name its type directly
namespace detail
{
template <idx_t I, typename... Ts>
struct at_impl;
template <typename T, typename... Ts>
struct at_impl<0, T, Ts...> {
  using type = T;
};
template <idx_t I, typename T, typename... Ts>
struct at_impl<I, T, Ts...> : at_impl<I - 1, Ts...> {
};
}  // namespace detail
template <typename L, typename I>
struct at;
template <typename... Ts, typename I>
struct at<list<Ts...>, I> : detail::at_impl<idx_t(I::value), Ts...> {
};
template <typename L, typename I>
using at_t = typename at<L, I>::type;
template <typename L, idx_t I>
using at_v = typename at<L, num<I>>::type;
template <typename L, idx_t I>
struct at_key_impl;

template <typename L>
using first = at_v<L, 0>;

template <typename L, typename T>
struct append;
template <typename... Ts, typename T>
struct append<list<Ts...>, T> {
  using type = list<Ts..., T>;
};
template <typename L, typename T>
struct prepend;
template <typename... Ts, typename T>
struct prepend<list<Ts...>, T> {
  using type = list<T, Ts...>;
};

template <typename... Ls>
struct extend;
template <typename... As, typename... Bs>
struct extend<list<As...>, list<Bs...>> {
  using type = list<As..., Bs...>;
};

// flatten nested lists into one
template <typename L>
struct flatten;
template <>
struct flatten<list<>> {
  using type = list<>;
};
template <typename T, typename... Ts>
struct flatten<list<T, Ts...>> {
  using type = typename extend<list<T>, typename flatten<list<Ts...>>::type>::type;
};
template <typename... Is, typename... Ts>
struct flatten<list<list<Is...>, Ts...>> {
  using type = typename extend<typename flatten<list<Is...>>::type,
                               typename flatten<list<Ts...>>::type>::type;
};

// transform<Op, list<Ts...>> = list<Op<Ts>...>
template <template <typename...> class Op, typename L>
struct transform;
template <template <typename...> class Op, typename... Ts>
struct transform<Op, list<Ts...>> {
  using type = list<typename Op<Ts>::type...>;
};

// lambda<Template> and apply_l<Lambda, list<Ts...>> = Template<Ts...>
template <template <typename...> class T>
struct lambda {
  template <typename... Ts>
  struct expr {
    using type = T<Ts...>;
  };
};
template <typename Lambda, typename L>
struct apply_l;
template <typename Lambda, typename... Ts>
struct apply_l<Lambda, list<Ts...>> {
  using type = typename Lambda::template expr<Ts...>::type;
};

// index of the first element satisfying Cond, or nil
template <template <typename> class Cond, typename L>
struct find_if;
template <template <typename> class Cond>
struct find_if<Cond, list<>> {
  using type = nil;
};
template <template <typename> class Cond, typename T, typename... Ts>
struct find_if<Cond, list<T, Ts...>> {
  using type = typename std::conditional<Cond<T>::value, T,
                                         typename find_if<Cond, list<Ts...>>::type>::type;
};
}  // namespace camp

#endif
