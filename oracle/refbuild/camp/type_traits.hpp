// Clean-room camp subset (test infrastructure): type traits that RAJA
// reaches through camp::type_traits.
#ifndef CAMP_SUBSET_TYPE_TRAITS_HPP
#define CAMP_SUBSET_TYPE_TRAITS_HPP

#include <iterator>
#include <type_traits>

#include "camp/helpers.hpp"
#include "camp/list.hpp"

namespace camp
{
namespace type_traits
{
namespace detail
{
template <typename...>
using void_t = void;

template <typename T, typename = void>
struct has_begin_end : std::false_type {
};
template <typename T>
struct has_begin_end<T, void_t<decltype(std::begin(val<T&>())), decltype(std::end(val<T&>()))>>
    : std::true_type {
};

template <typename T, typename = void>
struct iter_category {
  using type = void;
};
template <typename T>
struct iter_category<T, void_t<typename std::iterator_traits<T>::iterator_category>> {
  using type = typename std::iterator_traits<T>::iterator_category;
};
template <typename T, typename = void>
struct range_iter {
  using type = void;
};
template <typename T>
struct range_iter<T, void_t<decltype(std::begin(val<T&>()))>> {
  using type = decltype(std::begin(val<T&>()));
};
}  // namespace detail

template <typename T>
struct is_iterator
    : bool_<!std::is_same<typename detail::iter_category<decay<T>>::type, void>::value> {
};
template <typename T>
struct is_random_access_iterator
    : bool_<std::is_base_of<std::random_access_iterator_tag,
                            typename detail::iter_category<decay<T>>::type>::value> {
};
template <typename T>
struct is_range : detail::has_begin_end<decay<T>> {
};
template <typename T>
struct is_random_access_range
    : bool_<is_range<T>::value &&
            is_random_access_iterator<typename detail::range_iter<decay<T>>::type>::value> {
};

template <typename T>
using is_integral = std::is_integral<T>;
template <typename T>
using is_signed = std::is_signed<T>;
template <typename T>
using is_arithmetic = std::is_arithmetic<T>;
template <typename T>
using is_floating_point = std::is_floating_point<T>;

// SpecializationOf<Template, T>: T is Template<Args...>
template <template <typename...> class Template, typename T>
struct SpecializationOf : std::false_type {
};
template <template <typename...> class Template, typename... Args>
struct SpecializationOf<Template, Template<Args...>> : std::true_type {
};

template <typename T>
struct IterableValue {
  using type = decay<decltype(*std::begin(val<T&>()))>;
};
template <typename T>
using iterable_value_t = typename IterableValue<T>::type;
}  // namespace type_traits
}  // namespace camp

#endif
