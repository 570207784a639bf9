// backend.cpp (compat) - to_variant and select_backend for the compat registry
// (portableRT src/backend.cpp:24-56): shut the previous backend down, switch the
// variant, initialise the new one.
#include <stdexcept>

#include <portableRT/portableRT.hpp>

namespace portableRT {

BackendVar to_variant(Backend *backend) {
	if (auto *q = dynamic_cast<B200Backend *>(backend))
		return q;
	throw std::runtime_error("Unknown backend");
}

void select_backend(Backend *backend) {
	if (selected_backend)
		selected_backend->shutdown();
	selected_backend = backend;
	var_selected = to_variant(backend);
	backend->init();
}

} // namespace portableRT
