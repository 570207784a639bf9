// ref_harness.cpp - drives the reference's own CPU backend (TEST INFRASTRUCTURE).
//
// oracle/Makefile compiles this file together with the reference's unmodified
// src/backend.cpp and src/intersect_cpu.cpp, read where they lie in the reference
// tree, into oracle/_ref/ref_oracle.  It is the ground truth the C restatement in
// prt_oracle.c is pinned against, and the source of the committed golden vectors.
//
// usage: ref_oracle <tris.f32> <rays.f32> <out_dir> [--combos] [--repeat N]
//   <tris.f32>: n x 9 float32 (v0, v1, v2), <rays.f32>: m x 6 float32 (origin, dir)
//   writes <out_dir>/full.bin       raw FullHitReg records (32 B each)
//          <out_dir>/<combo>.bin    with --combos: raw HitReg<combo> records for all 31
//                                   TAG_COMBOS, named by hitreg_name<>()
//          <out_dir>/nodes.bin      the BVH2 node count (uint64)
//   prints one JSON line: build seconds, median query seconds, thread count.
#include <portableRT/portableRT.hpp>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

namespace {

std::vector<float> read_f32(const char *path) {
	std::ifstream f(path, std::ios::binary | std::ios::ate);
	if (!f) {
		std::fprintf(stderr, "cannot open %s\n", path);
		std::exit(2);
	}
	std::streamsize n = f.tellg();
	f.seekg(0);
	std::vector<float> v(static_cast<size_t>(n) / sizeof(float));
	f.read(reinterpret_cast<char *>(v.data()), static_cast<std::streamsize>(v.size() * 4));
	return v;
}

template <class T> void write_raw(const std::string &path, const std::vector<T> &v) {
	std::ofstream f(path, std::ios::binary);
	f.write(reinterpret_cast<const char *>(v.data()),
	        static_cast<std::streamsize>(v.size() * sizeof(T)));
}

template <class... Tags>
void dump_combo(const std::vector<portableRT::Ray> &rays, const std::string &dir) {
	auto hits = portableRT::nearest_hits<Tags...>(rays);
	write_raw(dir + "/" + portableRT::hitreg_name<Tags...>() + ".bin", hits);
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
	return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

} // namespace

int main(int argc, char **argv) {
	if (argc < 4) {
		std::fprintf(stderr, "usage: %s tris.f32 rays.f32 out_dir [--combos] [--repeat N]\n",
		             argv[0]);
		return 2;
	}
	bool combos = false;
	int repeat = 1;
	for (int i = 4; i < argc; ++i) {
		if (!std::strcmp(argv[i], "--combos"))
			combos = true;
		else if (!std::strcmp(argv[i], "--repeat") && i + 1 < argc)
			repeat = std::max(1, std::atoi(argv[++i]));
	}
	const std::string out_dir = argv[3];

	std::vector<float> tf = read_f32(argv[1]);
	std::vector<float> rf = read_f32(argv[2]);
	portableRT::Tris tris(tf.size() / 9);
	for (size_t i = 0; i < tris.size(); ++i)
		std::copy(tf.begin() + 9 * i, tf.begin() + 9 * i + 9, tris[i].begin());
	std::vector<portableRT::Ray> rays(rf.size() / 6);
	for (size_t i = 0; i < rays.size(); ++i) {
		for (int k = 0; k < 3; ++k) {
			rays[i].origin[k] = rf[6 * i + k];
			rays[i].direction[k] = rf[6 * i + 3 + k];
		}
	}

	for (auto *b : portableRT::available_backends())
		if (b->name() == "CPU")
			portableRT::select_backend(b);
	if (!portableRT::selected_backend || portableRT::selected_backend->name() != "CPU") {
		std::fprintf(stderr, "CPU backend not available\n");
		return 3;
	}

	auto t0 = std::chrono::steady_clock::now();
	portableRT::selected_backend->set_tris(tris);
	double build_s = seconds_since(t0);

	std::vector<portableRT::FullHitReg> hits;
	std::vector<double> q;
	for (int r = 0; r < repeat; ++r) {
		auto t1 = std::chrono::steady_clock::now();
		hits = portableRT::nearest_hits(rays);
		q.push_back(seconds_since(t1));
	}
	std::sort(q.begin(), q.end());
	write_raw(out_dir + "/full.bin", hits);

	if (combos) {
#define X(...) dump_combo<ADD_FILTER(__VA_ARGS__)>(rays, out_dir);
		TAG_COMBOS
#undef X
	}

	std::printf("{\"n_tris\": %zu, \"n_rays\": %zu, \"build_s\": %.6f, \"query_s\": %.6f, "
	            "\"threads\": %u}\n",
	            tris.size(), rays.size(), build_s, q[q.size() / 2],
	            std::thread::hardware_concurrency());
	return 0;
}
