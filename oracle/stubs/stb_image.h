// Stand-in for stb_image's loader (TEST INFRASTRUCTURE, for the oracle's examples
// harness): there is no image to load, so it reports none.
#pragma once

#include <cstdlib>

static inline unsigned char *stbi_load(const char *, int *w, int *h, int *c, int) {
	*w = *h = *c = 0;
	return nullptr;
}
static inline void stbi_image_free(void *p) { std::free(p); }
