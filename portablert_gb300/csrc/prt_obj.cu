// prt_obj.cu - Wavefront OBJ triangles for set_tris (host code only).
//
// The examples read their meshes with tinyobjloader and keep only triangles
// (examples/bunny/main.cpp:22-73: vertex positions of each 3-vertex face, in file order,
// as std::array<float, 9>).  This reader gives the same triangle soup for such files:
//   v x y z [w]            position (w and any trailing colour values ignored)
//   f a b c ...            vertex references a, a/t, a//n or a/t/n; 1-based, negative
//                          = relative to the vertices read so far
// Faces of n > 3 vertices are split as a fan (a, b_k, b_k+1) (tinyobjloader triangulates
// too; its own split of polygons is not restated, the examples' meshes are triangle
// meshes).  Every other line (vt, vn, o, g, s, usemtl, mtllib, comments) is skipped.
// Numbers are parsed as double (independent of the C locale) and rounded to float, as
// tinyobjloader does.
#include <stdint.h>

#include <algorithm>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/prt_b200.h"

namespace prt {
void set_global_error(const std::string &msg);
}

namespace {

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r'; }

const char *skip_space(const char *p, const char *e) {
	while (p < e && is_space(*p))
		++p;
	return p;
}

// A decimal number in [p, e) (optional sign, digits, fraction, exponent, or inf/nan),
// correctly rounded to double whatever the process's locale; the end of the number, or
// null when none starts at p.
const char *parse_number(const char *p, const char *e, double &out) {
	const bool neg = p < e && *p == '-';
	const char *q = (p < e && (*p == '+' || *p == '-')) ? p + 1 : p;
	if (q < e && (*q == '+' || *q == '-'))
		return nullptr;
	const std::from_chars_result r = std::from_chars(q, e, out);
	if (r.ec == std::errc::invalid_argument || r.ptr == q)
		return nullptr;
	if (r.ec == std::errc::result_out_of_range) {
		// Beyond double's range: the nearest double, as the C library's strtod gives.
		const char *x = q;
		while (x < r.ptr && *x != 'e' && *x != 'E')
			++x;
		const bool tiny = x < r.ptr && x + 1 < r.ptr && x[1] == '-';
		out = tiny ? 0.0 : HUGE_VAL;
	}
	if (neg)
		out = -out;
	return r.ptr;
}

// One vertex reference of an `f` line: the position index before any '/'.
bool parse_ref(const char *&p, const char *e, long long n_verts, uint32_t &out) {
	char *end = nullptr;
	errno = 0;
	const long long v = std::strtoll(p, &end, 10);
	if (end == p || errno)
		return false;
	p = end;
	while (p < e && !is_space(*p)) // texture / normal indices
		++p;
	const long long idx = v > 0 ? v - 1 : n_verts + v;
	if (v == 0 || idx < 0 || idx >= n_verts)
		return false;
	out = (uint32_t)idx;
	return true;
}

int parse(const std::vector<char> &buf, std::vector<float> &tris, std::string &err) {
	std::vector<float> verts;
	// buf ends with a NUL that is not part of the text (it stops strtoll).
	const char *p = buf.data(), *end = buf.data() + buf.size() - 1;
	uint64_t line = 0;
	std::vector<uint32_t> face;
	while (p < end) {
		const char *le = static_cast<const char *>(std::memchr(p, '\n', end - p));
		if (!le)
			le = end;
		++line;
		const char *q = skip_space(p, le);
		if (q + 1 < le && q[0] == 'v' && is_space(q[1])) {
			q += 2;
			for (int k = 0; k < 3; ++k) {
				q = skip_space(q, le);
				double d = 0.0;
				const char *ne = parse_number(q, le, d);
				if (!ne) {
					err = "obj line " + std::to_string(line) + ": bad vertex";
					return PRT_ERR_ARG;
				}
				verts.push_back((float)d);
				q = ne;
			}
		} else if (q + 1 < le && q[0] == 'f' && is_space(q[1])) {
			q += 2;
			face.clear();
			const long long nv = (long long)(verts.size() / 3);
			for (;;) {
				q = skip_space(q, le);
				if (q >= le)
					break;
				uint32_t idx;
				if (!parse_ref(q, le, nv, idx)) {
					err = "obj line " + std::to_string(line) + ": bad face vertex reference";
					return PRT_ERR_ARG;
				}
				face.push_back(idx);
			}
			if (face.size() < 3) {
				err = "obj line " + std::to_string(line) + ": face with fewer than 3 vertices";
				return PRT_ERR_ARG;
			}
			for (size_t k = 1; k + 1 < face.size(); ++k)
				for (uint32_t v : {face[0], face[k], face[k + 1]})
					tris.insert(tris.end(), verts.begin() + 3 * (size_t)v,
					            verts.begin() + 3 * (size_t)v + 3);
		}
		p = le + 1;
	}
	return PRT_OK;
}

} // namespace

extern "C" {

int prt_b200_obj_load(const char *path, float **tris9, uint64_t *n_tris) {
	if (!path || !tris9 || !n_tris) {
		prt::set_global_error("obj_load: null argument");
		return PRT_ERR_ARG;
	}
	*tris9 = nullptr;
	*n_tris = 0;
	FILE *f = std::fopen(path, "rb");
	if (!f) {
		prt::set_global_error(std::string("obj_load: cannot open ") + path);
		return PRT_ERR_ARG;
	}
	// The file and the soup are held in host vectors: a file too large for host memory
	// is an error status, not an exception through the C boundary.
	std::vector<float> tris;
	try {
		std::vector<char> buf;
		char chunk[1 << 16];
		size_t got;
		while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0)
			buf.insert(buf.end(), chunk, chunk + got);
		std::fclose(f);
		f = nullptr;
		buf.push_back('\0');
		std::string err;
		const int rc = parse(buf, tris, err);
		if (rc != PRT_OK) {
			prt::set_global_error(err);
			return rc;
		}
	} catch (const std::bad_alloc &) {
		if (f)
			std::fclose(f);
		prt::set_global_error("obj_load: out of host memory");
		return PRT_ERR_OOM;
	}
	float *out = static_cast<float *>(std::malloc(std::max<size_t>(tris.size(), 1) * sizeof(float)));
	if (!out) {
		prt::set_global_error("obj_load: out of host memory");
		return PRT_ERR_OOM;
	}
	if (!tris.empty())
		std::memcpy(out, tris.data(), tris.size() * sizeof(float));
	*tris9 = out;
	*n_tris = tris.size() / 9;
	return PRT_OK;
}

void prt_b200_free(void *p) { std::free(p); }

} // extern "C"
