// core.hpp (compat) - the ray and triangle types of portableRT (core.hpp:19-25 there),
// restated: a ray is origin then direction (6 floats), a triangle is v0, v1, v2 (9 floats).
#pragma once

#include <array>
#include <vector>

#include "hitreg.hpp"

namespace portableRT {

struct Ray {
	std::array<float, 3> origin;
	std::array<float, 3> direction;
};

using Tri = std::array<float, 9>;
using Tris = std::vector<Tri>;

} // namespace portableRT
