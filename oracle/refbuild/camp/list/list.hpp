// Clean-room camp subset (test infrastructure).
#include "camp/list.hpp"
