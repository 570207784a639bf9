// portableRT.hpp (compat) - umbrella header, as portableRT's include/portableRT/portableRT.hpp.
#pragma once

#include "backend.hpp"
#include "intersect_b200.hpp"
#include "nearest_hits_impl.hpp"
