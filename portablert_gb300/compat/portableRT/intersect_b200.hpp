// Forwards to the backend header kept in the repository's include/ directory.
#pragma once
#include "../../../include/portableRT/intersect_b200.hpp"
