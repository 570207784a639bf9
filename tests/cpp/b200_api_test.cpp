// b200_api_test.cpp - drives B200Backend through the portableRT C++ API.
//
//   b200_api_test kat
//       The single-triangle known answers of portableRT's validation example
//       (examples/validation/main.cpp:66-111): one JSON line with every field.
//   b200_api_test dump <tris.f32> <rays.f32> <out_dir>
//       set_tris + nearest_hits<Tags...> for all 31 tag combinations, each written raw
//       to <out_dir>/<tags joined by '_'>.bin, plus tag lists in a non-canonical order.
#include <portableRT/portableRT.hpp>

#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

using namespace portableRT;
using namespace portableRT::filter;

namespace {

std::vector<float> read_f32(const char *path) {
	std::ifstream f(path, std::ios::binary | std::ios::ate);
	std::vector<float> v(static_cast<size_t>(f.tellg()) / 4);
	f.seekg(0);
	f.read(reinterpret_cast<char *>(v.data()), static_cast<std::streamsize>(v.size() * 4));
	return v;
}

template <class... Tags> void dump(const std::vector<Ray> &rays, const std::string &path) {
	auto hits = portableRT::nearest_hits<Tags...>(rays);
	std::ofstream f(path, std::ios::binary);
	f.write(reinterpret_cast<const char *>(hits.data()),
	        static_cast<std::streamsize>(hits.size() * sizeof(HitReg<Tags...>)));
}

int kat() {
	Tri tri = {-1, -1, 0, 1, -1, 0, 0, 1, 0};
	Ray hit{{0.1f, 0.0f, -1.0f}, {0.0f, 0.0f, 1.0f}};
	Ray miss{{-2.0f, 0.0f, -1.0f}, {0.0f, 0.0f, 1.0f}};
	if (available_backends().empty()) {
		std::printf("{\"error\": \"no backend available\"}\n");
		return 3;
	}
	select_backend(available_backends()[0]);
	selected_backend->set_tris({tri});
	auto h = portableRT::nearest_hits({hit});
	auto m = portableRT::nearest_hits({miss});
	auto hv = portableRT::nearest_hits<valid>({hit});
	auto mv = portableRT::nearest_hits<valid>({miss});
	std::printf("{\"backend\": \"%s\", \"device\": \"%s\", \"hit\": {\"valid\": %d, \"t\": %.9g, "
	            "\"u\": %.9g, \"v\": %.9g, \"primitive_id\": %u, \"px\": %.9g, \"py\": %.9g, "
	            "\"pz\": %.9g}, \"miss_valid\": %d, \"filtered_hit_valid\": %d, "
	            "\"filtered_miss_valid\": %d}\n",
	            selected_backend->name().c_str(), selected_backend->device_name().c_str(),
	            (int)h[0].valid, h[0].t, h[0].u, h[0].v, h[0].primitive_id, h[0].px, h[0].py,
	            h[0].pz, (int)m[0].valid, (int)hv[0].valid, (int)mv[0].valid);
	return 0;
}

int dump_all(const char *tp, const char *rp, const std::string &dir) {
	std::vector<float> tf = read_f32(tp), rf = read_f32(rp);
	Tris tris(tf.size() / 9);
	for (size_t i = 0; i < tris.size(); ++i)
		for (int k = 0; k < 9; ++k)
			tris[i][k] = tf[9 * i + k];
	std::vector<Ray> rays(rf.size() / 6);
	for (size_t i = 0; i < rays.size(); ++i)
		for (int k = 0; k < 3; ++k) {
			rays[i].origin[k] = rf[6 * i + k];
			rays[i].direction[k] = rf[6 * i + 3 + k];
		}
	select_backend(available_backends().at(0));
	selected_backend->set_tris(tris);
	const std::string d = dir + "/";
	dump<uv>(rays, d + "uv.bin");
	dump<t>(rays, d + "t.bin");
	dump<primitive_id>(rays, d + "primitive_id.bin");
	dump<p>(rays, d + "p.bin");
	dump<valid>(rays, d + "valid.bin");
	dump<uv, t>(rays, d + "uv_t.bin");
	dump<uv, primitive_id>(rays, d + "uv_primitive_id.bin");
	dump<uv, p>(rays, d + "uv_p.bin");
	dump<uv, valid>(rays, d + "uv_valid.bin");
	dump<t, primitive_id>(rays, d + "t_primitive_id.bin");
	dump<t, p>(rays, d + "t_p.bin");
	dump<t, valid>(rays, d + "t_valid.bin");
	dump<primitive_id, p>(rays, d + "primitive_id_p.bin");
	dump<primitive_id, valid>(rays, d + "primitive_id_valid.bin");
	dump<p, valid>(rays, d + "p_valid.bin");
	dump<uv, t, primitive_id>(rays, d + "uv_t_primitive_id.bin");
	dump<uv, t, p>(rays, d + "uv_t_p.bin");
	dump<uv, t, valid>(rays, d + "uv_t_valid.bin");
	dump<uv, primitive_id, p>(rays, d + "uv_primitive_id_p.bin");
	dump<uv, primitive_id, valid>(rays, d + "uv_primitive_id_valid.bin");
	dump<uv, p, valid>(rays, d + "uv_p_valid.bin");
	dump<t, primitive_id, p>(rays, d + "t_primitive_id_p.bin");
	dump<t, primitive_id, valid>(rays, d + "t_primitive_id_valid.bin");
	dump<t, p, valid>(rays, d + "t_p_valid.bin");
	dump<primitive_id, p, valid>(rays, d + "primitive_id_p_valid.bin");
	dump<uv, t, primitive_id, p>(rays, d + "uv_t_primitive_id_p.bin");
	dump<uv, t, primitive_id, valid>(rays, d + "uv_t_primitive_id_valid.bin");
	dump<uv, t, p, valid>(rays, d + "uv_t_p_valid.bin");
	dump<uv, primitive_id, p, valid>(rays, d + "uv_primitive_id_p_valid.bin");
	dump<t, primitive_id, p, valid>(rays, d + "t_primitive_id_p_valid.bin");
	dump<uv, t, primitive_id, p, valid>(rays, d + "uv_t_primitive_id_p_valid.bin");
	// Tag lists in the orders the README and the spec use: same type, same bytes.
	dump<t, primitive_id, uv, p, valid>(rays, d + "order_t_primitive_id_uv_p_valid.bin");
	dump<t, uv, primitive_id, p, valid>(rays, d + "order_t_uv_primitive_id_p_valid.bin");
	dump<valid, t>(rays, d + "order_valid_t.bin");
	std::printf("{\"n_tris\": %zu, \"n_rays\": %zu, \"files\": 34}\n", tris.size(), rays.size());
	return 0;
}

} // namespace

int main(int argc, char **argv) {
	try {
		if (argc >= 2 && std::string(argv[1]) == "kat")
			return kat();
		if (argc >= 5 && std::string(argv[1]) == "dump")
			return dump_all(argv[2], argv[3], argv[4]);
		std::fprintf(stderr, "usage: %s kat | dump tris.f32 rays.f32 out_dir\n", argv[0]);
		return 2;
	} catch (const std::exception &e) {
		std::printf("{\"error\": \"%s\"}\n", e.what());
		return 4;
	}
}
