// Runs portableRT's own example programs (TEST INFRASTRUCTURE): their sources are
// compiled unchanged from the reference tree (oracle/Makefile, target "examples"), with
// oracle/stubs/ standing in for tinyobjloader and stb, which are not installed.
//
//   PRT_EXAMPLE_VALIDATION: examples/validation/main.cpp.  Its rays -- the 1024 x 1024
//     pinhole sensor camera it builds at start-up (main.cpp:170-198) -- are written to
//     the file named by argv[1] (6 floats per ray, in its order).
//   PRT_EXAMPLE_BUNNY: examples/bunny/main.cpp, run as is (it reads the backend index on
//     standard input); the valid mask it writes as its PNG (one byte per pixel of its
//     4096 x 4096 camera) goes to PRT_STUB_IMAGE, its mesh comes from PRT_STUB_OBJ.
#include <cstdio>

#if defined(PRT_EXAMPLE_VALIDATION)
#define main validation_example_main
#include "examples/validation/main.cpp"
#undef main

int main(int argc, char **argv) {
	if (argc < 2)
		return 2;
	FILE *f = std::fopen(argv[1], "wb");
	if (!f)
		return 1;
	for (const portableRT::Ray &r : rays) {
		std::fwrite(r.origin.data(), sizeof(float), 3, f);
		std::fwrite(r.direction.data(), sizeof(float), 3, f);
	}
	std::fclose(f);
	return 0;
}
#elif defined(PRT_EXAMPLE_BUNNY)
#include "examples/bunny/main.cpp"
#else
#error "define PRT_EXAMPLE_VALIDATION or PRT_EXAMPLE_BUNNY"
#endif
