// intersect_b200.hpp - GB300 (sm_103a) backend for portableRT.
//
// Drops into portableRT's include/portableRT/ beside intersect_cpu.hpp and registers
// itself exactly like the CPU backend does (intersect_cpu.hpp:10,55 in portableRT): a
// static instance whose constructor runs RegisterBackend.  nearest_hits<Tags...> is
// defined here so that every tag list, in any order, instantiates (std::visit in
// nearest_hits_impl.hpp instantiates it for each backend of the variant); it computes
// the record layout of HitReg<Tags...> with offsetof and hands it to the C ABI, which
// writes those bytes directly into the returned vector.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../prt_b200.h"
#include "backend.hpp"
#include "core.hpp"

namespace portableRT {

namespace b200_detail {

template <class R> struct RecordLayout {
	uint32_t mask = 0;
	uint8_t off[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	RecordLayout() {
		if constexpr (R::has_uv::value)
			mask |= PRT_FIELD_UV;
		if constexpr (R::has_t::value)
			mask |= PRT_FIELD_T;
		if constexpr (R::has_primitive_id::value)
			mask |= PRT_FIELD_PRIMITIVE_ID;
		if constexpr (R::has_p::value)
			mask |= PRT_FIELD_P;
		if constexpr (R::has_valid::value)
			mask |= PRT_FIELD_VALID;
		off[PRT_OFF_U] = static_cast<uint8_t>(offsetof(R, u));
		off[PRT_OFF_V] = static_cast<uint8_t>(offsetof(R, v));
		off[PRT_OFF_T] = static_cast<uint8_t>(offsetof(R, t));
		off[PRT_OFF_PID] = static_cast<uint8_t>(offsetof(R, primitive_id));
		off[PRT_OFF_VALID] = static_cast<uint8_t>(offsetof(R, valid));
		off[PRT_OFF_PX] = static_cast<uint8_t>(offsetof(R, px));
		off[PRT_OFF_PY] = static_cast<uint8_t>(offsetof(R, py));
		off[PRT_OFF_PZ] = static_cast<uint8_t>(offsetof(R, pz));
	}
};

} // namespace b200_detail

class B200Backend : public InvokableBackend<B200Backend> {
  public:
	B200Backend() : InvokableBackend("B200") { static RegisterBackend reg(*this); }

	template <class... Tags>
	std::vector<HitReg<Tags...>> nearest_hits(const std::vector<Ray> &rays) {
		using R = HitReg<Tags...>;
		static_assert(sizeof(Ray) == 6 * sizeof(float), "Ray must be 6 packed floats");
		static_assert(sizeof(R) <= 32 && sizeof(R) % 4 == 0, "unexpected HitReg layout");
		static const b200_detail::RecordLayout<R> lay;
		std::vector<R> hits(rays.size());
		if (!ctx_)
			throw std::runtime_error("B200 backend is not initialised");
		int rc = prt_b200_nearest_hits(ctx_, reinterpret_cast<const float *>(rays.data()),
		                               rays.size(), lay.mask, sizeof(R), lay.off, hits.data());
		if (rc != PRT_OK)
			throw std::runtime_error(std::string("B200: ") + prt_b200_last_error(ctx_));
		return hits;
	}

	bool is_available() const override;
	void init() override;
	void shutdown() override;
	void set_tris(const Tris &tris) override;
	std::string device_name() const override;

	// Backend-specific tuning (see prt_b200_set_option); applies from the next call.
	void set_option(const char *key, int64_t value);
	prt_b200_ctx *context() const { return ctx_; }

  private:
	prt_b200_ctx *ctx_ = nullptr;
};

static B200Backend b200_backend;

} // namespace portableRT
