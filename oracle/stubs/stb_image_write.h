// Stand-in for stb_image_write's PNG writer (TEST INFRASTRUCTURE, for the oracle's
// examples harness): the pixels are written raw, row after row, to the file named by
// PRT_STUB_IMAGE (nothing is written when it is unset).
#pragma once

#include <cstdio>
#include <cstdlib>

static inline int stbi_write_png(const char *, int w, int h, int comp, const void *data,
                                 int stride) {
	const char *out = std::getenv("PRT_STUB_IMAGE");
	if (!out)
		return 1;
	FILE *f = std::fopen(out, "wb");
	if (!f)
		return 0;
	for (int y = 0; y < h; ++y)
		std::fwrite(static_cast<const unsigned char *>(data) + (size_t)y * stride, 1,
		            (size_t)w * comp, f);
	std::fclose(f);
	return 1;
}
