// Clean-room camp subset (test infrastructure): small helpers.
#ifndef CAMP_SUBSET_HELPERS_HPP
#define CAMP_SUBSET_HELPERS_HPP

#include <iterator>
#include <utility>

#include "camp/defines.hpp"

namespace camp
{
template <typename T>
using decay = typename std::decay<T>::type;

template <typename T, typename U>
using is_same = std::is_same<T, U>;
template <typename T, typename U>
using is_same_t = typename std::is_same<T, U>::type;

// a value of type T for unevaluated expressions
template <typename T>
T&& val() noexcept;

template <typename T>
CAMP_HOST_DEVICE constexpr T&& forward(typename std::remove_reference<T>::type& t) noexcept
{
  return static_cast<T&&>(t);
}
template <typename T>
CAMP_HOST_DEVICE constexpr T&& forward(typename std::remove_reference<T>::type&& t) noexcept
{
  return static_cast<T&&>(t);
}
template <typename T>
CAMP_HOST_DEVICE constexpr typename std::remove_reference<T>::type&& move(T&& t) noexcept
{
  return static_cast<typename std::remove_reference<T>::type&&>(t);
}

template <typename T>
CAMP_HOST_DEVICE void safe_swap(T& a, T& b)
{
  T tmp = static_cast<T&&>(a);
  a = static_cast<T&&>(b);
  b = static_cast<T&&>(tmp);
}

// iterator type of a range
template <typename T>
using iterator_from = decltype(std::begin(val<T&>()));

namespace type
{
namespace ref
{
template <typename T>
using rem = typename std::remove_reference<T>::type;
template <typename T>
using add = typename std::add_lvalue_reference<T>::type;
}  // namespace ref
namespace rvref
{
template <typename T>
using add = typename std::add_rvalue_reference<T>::type;
}
namespace ptr
{
template <typename T>
using add = typename std::add_pointer<T>::type;
template <typename T>
using rem = typename std::remove_pointer<T>::type;
}  // namespace ptr
namespace c
{
template <typename T>
using add = typename std::add_const<T>::type;
template <typename T>
using rem = typename std::remove_const<T>::type;
}  // namespace c
namespace v
{
template <typename T>
using add = typename std::add_volatile<T>::type;
template <typename T>
using rem = typename std::remove_volatile<T>::type;
}  // namespace v
namespace cv
{
template <typename T>
using add = typename std::add_cv<T>::type;
template <typename T>
using rem = typename std::remove_cv<T>::type;
}  // namespace cv
}  // namespace type
}  // namespace camp

#endif
