// intersect_b200.cpp - non-template members of portableRT::B200Backend.
//
// Drops into portableRT's src/ beside intersect_cpu.cpp (the counterpart of
// src/intersect_cpu.cpp:9-27 there).  Every member forwards to the C ABI of
// libprt_b200.so; failures become std::runtime_error except in is_available, which
// static registration calls before main and which must not throw.
#include <portableRT/intersect_b200.hpp>

#include <stdexcept>
#include <string>

namespace portableRT {

namespace {

void throw_if(int rc, const prt_b200_ctx *ctx) {
	if (rc != PRT_OK)
		throw std::runtime_error(std::string("B200: ") + prt_b200_last_error(ctx));
}

} // namespace

bool B200Backend::is_available() const { return prt_b200_available() == 1; }

void B200Backend::init() {
	if (ctx_)
		return;
	prt_b200_ctx *c = nullptr;
	throw_if(prt_b200_create(0, &c), nullptr);
	ctx_ = c;
}

void B200Backend::shutdown() {
	prt_b200_destroy(ctx_);
	ctx_ = nullptr;
}

void B200Backend::set_tris(const Tris &tris) {
	if (!ctx_)
		init();
	static_assert(sizeof(Tri) == 9 * sizeof(float), "Tri must be 9 packed floats");
	throw_if(prt_b200_set_tris(ctx_, reinterpret_cast<const float *>(tris.data()), tris.size()),
	         ctx_);
}

std::string B200Backend::device_name() const {
	if (!ctx_)
		return "unsupported";
	char buf[256];
	if (prt_b200_device_name(ctx_, buf, sizeof buf) != PRT_OK)
		return "unsupported";
	return buf;
}

void B200Backend::set_option(const char *key, int64_t value) {
	if (!ctx_)
		init();
	throw_if(prt_b200_set_option(ctx_, key, value), ctx_);
}

} // namespace portableRT
