// Clean-room camp subset (test infrastructure): a tuple with index and
// type access, built on one storage leaf per element.
#ifndef CAMP_SUBSET_TUPLE_HPP
#define CAMP_SUBSET_TUPLE_HPP

#include <type_traits>
#include <utility>

#include "camp/helpers.hpp"
#include "camp/list.hpp"
#include "camp/number.hpp"

namespace camp
{
template <typename... Ts>
struct tuple;

namespace detail
{
template <idx_t I, typename T>
struct tuple_leaf {
  T value;
  CAMP_HOST_DEVICE constexpr tuple_leaf() : value() {}
  template <typename U>
  CAMP_HOST_DEVICE constexpr explicit tuple_leaf(U&& u) : value(static_cast<U&&>(u))
  {
  }
};

template <typename Seq, typename... Ts>
struct tuple_storage;
template <idx_t... Is, typename... Ts>
struct tuple_storage<idx_seq<Is...>, Ts...> : tuple_leaf<Is, Ts>... {
  CAMP_HOST_DEVICE constexpr tuple_storage() = default;
  template <typename... Us>
  CAMP_HOST_DEVICE constexpr explicit tuple_storage(int, Us&&... us)
      : tuple_leaf<Is, Ts>(static_cast<Us&&>(us))...
  {
  }
};

template <typename T>
struct is_tuple : std::false_type {
};
template <typename... Ts>
struct is_tuple<tuple<Ts...>> : std::true_type {
};
}  // namespace detail

template <typename... Ts>
struct tuple : detail::tuple_storage<idx_seq_for_t<Ts...>, Ts...> {
  using TList = list<Ts...>;
  using type = tuple;
  using Base = detail::tuple_storage<idx_seq_for_t<Ts...>, Ts...>;

  CAMP_HOST_DEVICE constexpr tuple() = default;
  CAMP_HOST_DEVICE constexpr tuple(tuple const&) = default;
  CAMP_HOST_DEVICE constexpr tuple(tuple&&) = default;
  CAMP_HOST_DEVICE tuple& operator=(tuple const&) = default;
  CAMP_HOST_DEVICE tuple& operator=(tuple&&) = default;

  // element-wise construction (not for a single argument that is itself a
  // tuple, which copies or moves instead)
  template <typename... Us,
            typename = typename std::enable_if<
                sizeof...(Us) == sizeof...(Ts) && (sizeof...(Us) > 0) &&
                !(sizeof...(Us) == 1 && (detail::is_tuple<decay<Us>>::value && ...))>::type>
  CAMP_HOST_DEVICE constexpr tuple(Us&&... us) : Base(0, static_cast<Us&&>(us)...)
  {
  }

  // element-wise conversion from another tuple of the same length
  template <typename... Us,
            typename = typename std::enable_if<sizeof...(Us) == sizeof...(Ts) &&
                                               !std::is_same<tuple<Us...>, tuple>::value>::type>
  CAMP_HOST_DEVICE constexpr tuple(tuple<Us...>&& o)
      : tuple(static_cast<tuple<Us...>&&>(o), idx_seq_for_t<Us...>())
  {
  }
  template <typename... Us,
            typename = typename std::enable_if<sizeof...(Us) == sizeof...(Ts) &&
                                               !std::is_same<tuple<Us...>, tuple>::value>::type>
  CAMP_HOST_DEVICE constexpr tuple(tuple<Us...> const& o) : tuple(o, idx_seq_for_t<Us...>())
  {
  }

private:
  template <typename O, idx_t... Is>
  CAMP_HOST_DEVICE constexpr tuple(O&& o, idx_seq<Is...>);
};

template <typename T>
struct tuple_size;
template <typename... Ts>
struct tuple_size<tuple<Ts...>> : num<idx_t(sizeof...(Ts))> {
};
template <typename T>
struct tuple_size<const T> : tuple_size<T> {
};
template <typename T>
struct tuple_size<T&> : tuple_size<T> {
};
template <typename T>
struct tuple_size<T&&> : tuple_size<T> {
};

template <idx_t I, typename T>
struct tuple_element;
template <idx_t I, typename... Ts>
struct tuple_element<I, tuple<Ts...>> {
  using type = at_v<list<Ts...>, I>;
};
template <idx_t I, typename T>
struct tuple_element<I, const T> : tuple_element<I, T> {
};
template <idx_t I, typename T>
using tuple_element_t = typename tuple_element<I, T>::type;

// get<I>: element I (an lvalue for lvalue tuples, forwarded for rvalues);
// a reference element stays a reference of its own type
template <idx_t I, typename... Ts>
CAMP_HOST_DEVICE constexpr decltype(auto) get(tuple<Ts...>& t) noexcept
{
  using T = at_v<list<Ts...>, I>;
  return (static_cast<detail::tuple_leaf<I, T>&>(t).value);
}
template <idx_t I, typename... Ts>
CAMP_HOST_DEVICE constexpr decltype(auto) get(tuple<Ts...> const& t) noexcept
{
  using T = at_v<list<Ts...>, I>;
  return (static_cast<detail::tuple_leaf<I, T> const&>(t).value);
}
template <idx_t I, typename... Ts>
CAMP_HOST_DEVICE constexpr at_v<list<Ts...>, I>&& get(tuple<Ts...>&& t) noexcept
{
  using T = at_v<list<Ts...>, I>;
  return static_cast<T&&>(static_cast<detail::tuple_leaf<I, T>&>(t).value);
}

template <typename... Ts>
template <typename O, idx_t... Is>
CAMP_HOST_DEVICE constexpr tuple<Ts...>::tuple(O&& o, idx_seq<Is...>)
    : Base(0, get<Is>(static_cast<O&&>(o))...)
{
}

// get<T>: the element of type T (exactly one must exist)
namespace detail
{
template <typename T, typename L, idx_t I = 0>
struct index_of;
template <typename T, idx_t I>
struct index_of<T, list<>, I> : num<-1> {
};
template <typename T, typename U, typename... Us, idx_t I>
struct index_of<T, list<U, Us...>, I>
    : std::conditional<std::is_same<T, U>::value, num<I>, index_of<T, list<Us...>, I + 1>>::type {
};
}  // namespace detail
template <typename T, typename... Ts>
CAMP_HOST_DEVICE constexpr decltype(auto) get(tuple<Ts...>& t) noexcept
{
  return get<detail::index_of<T, list<Ts...>>::value>(t);
}
template <typename T, typename... Ts>
CAMP_HOST_DEVICE constexpr decltype(auto) get(tuple<Ts...> const& t) noexcept
{
  return get<detail::index_of<T, list<Ts...>>::value>(t);
}

template <typename... Args>
CAMP_HOST_DEVICE constexpr tuple<decay<Args>...> make_tuple(Args&&... args)
{
  return tuple<decay<Args>...>(static_cast<Args&&>(args)...);
}
CAMP_HOST_DEVICE constexpr tuple<> make_tuple() { return tuple<>(); }

template <typename... Args>
CAMP_HOST_DEVICE constexpr tuple<Args&&...> forward_as_tuple(Args&&... args) noexcept
{
  return tuple<Args&&...>(static_cast<Args&&>(args)...);
}

template <typename... Args>
CAMP_HOST_DEVICE constexpr tuple<Args&...> tie(Args&... args) noexcept
{
  return tuple<Args&...>(args...);
}

// concatenation of two tuples (elements copied or moved)
namespace detail
{
template <typename A, typename B, idx_t... Ia, idx_t... Ib>
CAMP_HOST_DEVICE constexpr auto cat_pair(A&& a, B&& b, idx_seq<Ia...>, idx_seq<Ib...>)
{
  using TA = decay<A>;
  using TB = decay<B>;
  return tuple<tuple_element_t<Ia, TA>..., tuple_element_t<Ib, TB>...>(
      get<Ia>(static_cast<A&&>(a))..., get<Ib>(static_cast<B&&>(b))...);
}
}  // namespace detail
template <typename A, typename B>
CAMP_HOST_DEVICE constexpr auto tuple_cat_pair(A&& a, B&& b)
{
  return detail::cat_pair(static_cast<A&&>(a), static_cast<B&&>(b),
                          make_idx_seq_t<tuple_size<decay<A>>::value>(),
                          make_idx_seq_t<tuple_size<decay<B>>::value>());
}

// references to the elements whose type satisfies Trait, as a tuple of
// references, in order
namespace detail
{
template <template <typename> class Trait, typename Tup, typename Sel, idx_t I, typename... Ts>
struct select_by_trait;
template <template <typename> class Trait, typename Tup, idx_t... Sel, idx_t I>
struct select_by_trait<Trait, Tup, idx_seq<Sel...>, I> {
  using type = idx_seq<Sel...>;
};
template <template <typename> class Trait, typename Tup, idx_t... Sel, idx_t I, typename T, typename... Ts>
struct select_by_trait<Trait, Tup, idx_seq<Sel...>, I, T, Ts...>
    : select_by_trait<Trait, Tup,
                      typename std::conditional<Trait<T>::value, idx_seq<Sel..., I>,
                                                idx_seq<Sel...>>::type,
                      I + 1, Ts...> {
};
template <typename... Ts, idx_t... Sel>
CAMP_HOST_DEVICE constexpr auto refs_at(tuple<Ts...>& t, idx_seq<Sel...>)
{
  return tuple<at_v<list<Ts...>, Sel>&...>(get<Sel>(t)...);
}
}  // namespace detail
template <template <typename> class Trait, typename... Ts>
CAMP_HOST_DEVICE constexpr auto get_refs_to_elements_by_type_trait(tuple<Ts...>& t)
{
  using sel = typename detail::select_by_trait<Trait, tuple<Ts...>, idx_seq<>, 0, Ts...>::type;
  return detail::refs_at(t, sel());
}

// invoke f with the tuple's elements as arguments
namespace detail
{
template <typename Fn, typename Tup, idx_t... Is>
CAMP_HOST_DEVICE constexpr decltype(auto) apply_impl(Fn&& f, Tup&& t, idx_seq<Is...>)
{
  return static_cast<Fn&&>(f)(get<Is>(static_cast<Tup&&>(t))...);
}
}  // namespace detail
template <typename Fn, typename Tup>
CAMP_HOST_DEVICE constexpr decltype(auto) apply(Fn&& f, Tup&& t)
{
  return detail::apply_impl(static_cast<Fn&&>(f), static_cast<Tup&&>(t),
                            make_idx_seq_t<tuple_size<decay<Tup>>::value>());
}
template <typename Fn, typename Tup>
CAMP_HOST_DEVICE constexpr decltype(auto) invoke(Tup&& t, Fn&& f)
{
  return apply(static_cast<Fn&&>(f), static_cast<Tup&&>(t));
}
}  // namespace camp

#endif
