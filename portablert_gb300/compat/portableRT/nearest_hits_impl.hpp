// nearest_hits_impl.hpp (compat) - the free nearest_hits<Tags...> dispatch of portableRT
// (nearest_hits_impl.hpp:28-36 there): visit the selected backend, throw on none.
#pragma once

#include <stdexcept>

#include "backend.hpp"
#include "intersect_b200.hpp"

namespace portableRT {

template <class... Tags> std::vector<HitReg<Tags...>> nearest_hits(const std::vector<Ray> &rays) {
	return std::visit(
	    [&](auto *b) -> std::vector<HitReg<Tags...>> {
		    if (!b)
			    throw std::runtime_error("Unknown backend");
		    return b->template nearest_hits<Tags...>(rays);
	    },
	    var_selected);
}

} // namespace portableRT
