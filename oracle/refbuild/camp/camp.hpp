// Clean-room camp subset (test infrastructure): everything.
#ifndef CAMP_SUBSET_CAMP_HPP
#define CAMP_SUBSET_CAMP_HPP
#include "camp/defines.hpp"
#include "camp/number.hpp"
#include "camp/list.hpp"
#include "camp/helpers.hpp"
#include "camp/type_traits.hpp"
#include "camp/concepts.hpp"
#include "camp/tuple.hpp"
#include "camp/resource.hpp"
#endif
