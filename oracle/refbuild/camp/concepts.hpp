// Clean-room camp subset (test infrastructure): the concept emulation that
// RAJA's headers use -- boolean combinators over traits, enable_if forms
// for SFINAE, and concepts written as structs over expressions.
//
// A concept is written `template <...> struct C : DefineConcept(exprs...) {}`
// and derives from true_type or false_type.  The has_type / convertible_to
// checks report false instead of failing, so concepts made of them are
// usable in overload selection; any other expression in a concept must be
// well formed where RAJA evaluates it (in the headers the oracle compiles
// those are static_asserts and explicitly given execution policies).
#ifndef CAMP_SUBSET_CONCEPTS_HPP
#define CAMP_SUBSET_CONCEPTS_HPP

#include <type_traits>

#include "camp/helpers.hpp"
#include "camp/list.hpp"
#include "camp/number.hpp"
#include "camp/type_traits.hpp"

namespace camp
{
namespace concepts
{
namespace metalib
{
template <typename T, typename U>
using is_same = std::is_same<T, U>;
}

template <typename... Conds>
struct all_of : bool_<(true && ... && bool(Conds::value))> {
};
template <typename... Conds>
struct any_of : bool_<(false || ... || bool(Conds::value))> {
};
template <typename Cond>
struct negate : bool_<!bool(Cond::value)> {
};

template <typename... Conds>
using enable_if = typename std::enable_if<all_of<Conds...>::value>::type;
template <typename Ret, typename... Conds>
using enable_if_t = typename std::enable_if<all_of<Conds...>::value, Ret>::type;

// Expression checks usable inside DefineConcept.  They never fail to
// compile: each yields true_type or false_type, and a concept models when
// none of its checks yields false_type.  Other expressions in a concept
// must be well formed for the types it is used on.  Declarations only:
// they appear in unevaluated operands.
template <typename T, typename U>
auto has_type(U&&) -> bool_<std::is_same<decay<U>, T>::value>;
template <typename T, typename U>
auto convertible_to(U&&) -> bool_<std::is_convertible<U, T>::value>;

namespace detail
{
template <typename... Ts>
auto valid_expressions(Ts&&...)
    -> bool_<(true && ... && !std::is_same<decay<Ts>, std::false_type>::value)>;
}  // namespace detail

template <template <typename...> class Concept, typename... Args>
struct requires_ : bool_<bool(Concept<Args...>::value)> {
};
}  // namespace concepts
}  // namespace camp

#define DefineConcept(...) decltype(::camp::concepts::detail::valid_expressions(__VA_ARGS__))

#define DefineTypeTraitFromConcept(TTName, ConceptName) \
  template <typename... Args>                           \
  struct TTName : ::camp::concepts::requires_<ConceptName, Args...> {                  \
  }

#endif
