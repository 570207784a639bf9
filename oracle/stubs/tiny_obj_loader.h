// Stand-in for the slice of tinyobjloader's interface that portableRT's examples call
// (TEST INFRASTRUCTURE: used only to compile the examples' own sources in the
// oracle's examples harness).  The parser reads vertex positions and triangle faces
// ("v x y z", "f a b c" with a, a/t, a//n or a/t/n references); the examples keep only
// those.  When PRT_STUB_OBJ is set in the environment it names the file read instead
// of the one the example asks for.
#pragma once

// The examples call sqrt without including <cmath>; the real header includes it.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace tinyobj {

typedef float real_t;

struct index_t {
	int vertex_index = -1, normal_index = -1, texcoord_index = -1;
};
struct mesh_t {
	std::vector<index_t> indices;
	std::vector<unsigned int> num_face_vertices;
};
struct shape_t {
	std::string name;
	mesh_t mesh;
};
struct attrib_t {
	std::vector<real_t> vertices;
};
struct material_t {};
struct ObjReaderConfig {
	std::string mtl_search_path;
	bool triangulate = true;
};

class ObjReader {
  public:
	bool ParseFromFile(const std::string &path, const ObjReaderConfig & = ObjReaderConfig()) {
		const char *over = std::getenv("PRT_STUB_OBJ");
		std::ifstream in(over ? over : path.c_str());
		if (!in) {
			err_ = "cannot open " + std::string(over ? over : path);
			return false;
		}
		shapes_.assign(1, shape_t());
		std::string line;
		while (std::getline(in, line)) {
			std::istringstream ls(line);
			std::string tag;
			ls >> tag;
			if (tag == "v") {
				double x, y, z;
				ls >> x >> y >> z;
				attrib_.vertices.insert(attrib_.vertices.end(), {(real_t)x, (real_t)y, (real_t)z});
			} else if (tag == "f") {
				std::string ref;
				unsigned int n = 0;
				while (ls >> ref) {
					index_t idx;
					const long v = std::strtol(ref.c_str(), nullptr, 10);
					idx.vertex_index = (int)(v > 0 ? v - 1 : (long)(attrib_.vertices.size() / 3) + v);
					shapes_[0].mesh.indices.push_back(idx);
					++n;
				}
				shapes_[0].mesh.num_face_vertices.push_back(n);
			}
		}
		return true;
	}
	const std::string &Error() const { return err_; }
	const std::string &Warning() const { return warn_; }
	const attrib_t &GetAttrib() const { return attrib_; }
	const std::vector<shape_t> &GetShapes() const { return shapes_; }
	const std::vector<material_t> &GetMaterials() const { return materials_; }

  private:
	std::string err_, warn_;
	attrib_t attrib_;
	std::vector<shape_t> shapes_;
	std::vector<material_t> materials_;
};

} // namespace tinyobj
