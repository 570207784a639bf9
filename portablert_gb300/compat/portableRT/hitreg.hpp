// hitreg.hpp (compat) - portableRT's filter-tagged hit record, restated for building the
// B200 backend without the portableRT tree.  Same names, same member order and the same
// one-byte placeholder for absent fields, so the layout (and therefore the bytes the
// B200 kernels write) is identical to portableRT's include/portableRT/hitreg.hpp:16-61.
#pragma once

#include <cstdint>
#include <type_traits>

namespace portableRT {

// Stand-in for an absent field: one byte, writes are discarded, reads do not compile.
struct Empty {
	template <class T> constexpr Empty &operator=(T &&) noexcept { return *this; }
	template <class T> constexpr operator T() const = delete;
};

namespace filter {
struct uv {};
struct t {};
struct primitive_id {};
struct p {};
struct valid {};
} // namespace filter

template <typename T, typename... List> constexpr bool has_tag = (std::is_same_v<T, List> || ...);

template <bool UV, bool T, bool PID, bool P, bool VALID> struct HitRegImpl {
	using has_uv = std::bool_constant<UV>;
	using has_t = std::bool_constant<T>;
	using has_primitive_id = std::bool_constant<PID>;
	using has_p = std::bool_constant<P>;
	using has_valid = std::bool_constant<VALID>;

	std::conditional_t<UV, float, Empty> u;
	std::conditional_t<UV, float, Empty> v;
	std::conditional_t<T, float, Empty> t;
	std::conditional_t<PID, uint32_t, Empty> primitive_id;
	std::conditional_t<VALID, bool, Empty> valid;
	std::conditional_t<P, float, Empty> px;
	std::conditional_t<P, float, Empty> py;
	std::conditional_t<P, float, Empty> pz;
};

template <class... Tags>
using HitReg = HitRegImpl<has_tag<filter::uv, Tags...>, has_tag<filter::t, Tags...>,
                          has_tag<filter::primitive_id, Tags...>, has_tag<filter::p, Tags...>,
                          has_tag<filter::valid, Tags...>>;

using FullHitReg =
    HitReg<filter::uv, filter::t, filter::primitive_id, filter::p, filter::valid>;

} // namespace portableRT
