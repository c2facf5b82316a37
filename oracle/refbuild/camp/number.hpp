// Clean-room camp subset (test infrastructure): integral constants and
// integer sequences.
#ifndef CAMP_SUBSET_NUMBER_HPP
#define CAMP_SUBSET_NUMBER_HPP

#include "camp/defines.hpp"

namespace camp
{
template <typename T, T V>
using integral_constant = std::integral_constant<T, V>;
template <bool B>
using bool_ = std::integral_constant<bool, B>;
using true_type = std::true_type;
using false_type = std::false_type;
using t = true_type;
using f = false_type;

template <idx_t N>
using num = integral_constant<idx_t, N>;

template <typename T, T... Vs>
struct int_seq {
  using type = int_seq;
  using value_type = T;
  static constexpr std::size_t size() { return sizeof...(Vs); }
};
template <idx_t... Is>
using idx_seq = int_seq<idx_t, Is...>;

namespace detail
{
template <typename T, typename S>
struct to_int_seq;
template <typename T, T... Vs>
struct to_int_seq<T, std::integer_sequence<T, Vs...>> {
  using type = int_seq<T, Vs...>;
};
}  // namespace detail

template <typename T, T N>
struct make_int_seq : detail::to_int_seq<T, std::make_integer_sequence<T, N>> {
};
template <typename T, T N>
using make_int_seq_t = typename make_int_seq<T, N>::type;
template <idx_t N>
struct make_idx_seq : make_int_seq<idx_t, N> {
};
template <idx_t N>
using make_idx_seq_t = typename make_idx_seq<N>::type;
template <typename... Ts>
using idx_seq_for_t = make_idx_seq_t<idx_t(sizeof...(Ts))>;

template <typename T>
struct idx_seq_from;

// element Idx of an int_seq, as an integral constant
template <idx_t Idx, typename Seq>
struct seq_at;
template <idx_t Idx, typename T, T First, T... Rest>
struct seq_at<Idx, int_seq<T, First, Rest...>>
    : seq_at<Idx - 1, int_seq<T, Rest...>> {
};
template <typename T, T First, T... Rest>
struct seq_at<0, int_seq<T, First, Rest...>> : integral_constant<T, First> {
};

template <typename T>
struct value : T {
};
}  // namespace camp

#endif
