// backend.hpp (compat) - portableRT's backend registry, restated with only the B200
// backend in the variant, for building and testing the backend without the portableRT
// tree.  Names and behaviour follow portableRT's include/portableRT/backend.hpp:12-95:
// RegisterBackend selects the first available backend, select_backend shuts the old one
// down and initialises the new one, nearest_hits() without tags means all five.
#pragma once

#include <string>
#include <variant>
#include <vector>

#include "core.hpp"

namespace portableRT {

class Backend {
  public:
	Backend(std::string name, void *self_ptr) : self_{self_ptr}, name_{std::move(name)} {}
	virtual ~Backend() = default;

	const std::string &name() const { return name_; }

	virtual void set_tris(const Tris &tris) = 0;
	virtual bool is_available() const = 0;
	virtual void init() = 0;
	virtual void shutdown() = 0;
	virtual std::string device_name() const = 0;

	void *self_;

  private:
	std::string name_;
};

template <class Derived> class InvokableBackend : public Backend {
  public:
	explicit InvokableBackend(std::string name)
	    : Backend{std::move(name), static_cast<void *>(this)} {}
};

inline Backend *selected_backend = nullptr;
inline std::vector<Backend *> all_backends_;
inline std::vector<Backend *> available_backends_;
inline const std::vector<Backend *> &all_backends() { return all_backends_; }
inline const std::vector<Backend *> &available_backends() { return available_backends_; }

class B200Backend;
using BackendVar = std::variant<B200Backend *>;
inline BackendVar var_selected{static_cast<B200Backend *>(nullptr)};

template <class... Tags> std::vector<HitReg<Tags...>> nearest_hits(const std::vector<Ray> &rays);

inline std::vector<FullHitReg> nearest_hits(const std::vector<Ray> &rays) {
	return nearest_hits<filter::uv, filter::t, filter::primitive_id, filter::p, filter::valid>(
	    rays);
}

BackendVar to_variant(Backend *backend);
void select_backend(Backend *backend);

struct RegisterBackend {
	explicit RegisterBackend(Backend &b) {
		if (b.is_available()) {
			if (selected_backend == nullptr)
				select_backend(&b);
			available_backends_.push_back(&b);
		}
		all_backends_.push_back(&b);
	}
};

} // namespace portableRT
