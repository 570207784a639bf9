// prt_gltf.cu - glTF 2.0 triangles for set_tris (host code only).
//
// The sponza example reads its scene with cgltf and keeps the triangles of every mesh
// (examples/sponza/main.cpp:35-101): for each mesh in the file's `meshes` array, each
// primitive of mode TRIANGLES that has both a POSITION accessor and an index accessor
// (others are skipped), the triangles (idx[i], idx[i+1], idx[i+2]) for i = 0, 3, ...
// while i + 2 < count, each vertex the float3 position at that index, in mesh space (no
// node transforms), indices read as u8, u16 or u32.  This reader gives the same soup.
// It differs only where the example reads out of bounds or ignores the format: it
// follows a bufferView's byteStride (the example assumes tightly packed positions, which
// is what it reads whenever byteStride is absent or 12), and it reports as errors what
// the example would read past a buffer for (an index beyond the position count, an
// accessor beyond its view), a position accessor that is not float VEC3, sparse
// accessors and required extensions (compressed geometry).
//
// Containers: a .gltf JSON file whose buffers are files beside it (relative URIs,
// %-escapes decoded) or base64 data: URIs, or a binary .glb (12-byte header, a JSON
// chunk, an optional BIN chunk that a buffer without a URI refers to).  The JSON parser
// is a small recursive-descent one of our own, bounded in nesting depth.
#include <stdint.h>

#include <algorithm>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/prt_b200.h"

namespace prt {
void set_global_error(const std::string &msg);
}

namespace {

// ---------------------------------------------------------------------------------------
// JSON
// ---------------------------------------------------------------------------------------

struct Json {
	enum Kind : uint8_t { Null, Bool, Num, Str, Arr, Obj };
	Kind kind = Null;
	bool b = false;
	double num = 0.0;
	std::string str;
	std::vector<Json> arr;
	std::vector<std::pair<std::string, Json>> obj;

	// The member named key of an object (the last one if repeated), or null.
	const Json *get(const char *key) const {
		if (kind != Obj)
			return nullptr;
		const Json *found = nullptr;
		for (const auto &kv : obj)
			if (kv.first == key)
				found = &kv.second;
		return found;
	}
};

constexpr int kMaxDepth = 64;

int hex_digit(char c) {
	if (c >= '0' && c <= '9')
		return c - '0';
	if (c >= 'a' && c <= 'f')
		return c - 'a' + 10;
	if (c >= 'A' && c <= 'F')
		return c - 'A' + 10;
	return -1;
}

class JsonParser {
  public:
	JsonParser(const char *p, const char *e) : p_(p), e_(e) {}

	// Parses one value spanning the whole text (white space around it allowed).
	bool parse(Json &out, std::string &err) {
		ws();
		if (!value(out, 0))
			return fail_out(err);
		ws();
		if (p_ != e_) {
			err_ = "trailing characters";
			return fail_out(err);
		}
		return true;
	}

  private:
	bool fail_out(std::string &err) {
		err = "JSON: " + (err_.empty() ? std::string("syntax error") : err_);
		return false;
	}

	bool fail(const char *msg) {
		if (err_.empty())
			err_ = msg;
		return false;
	}

	void ws() {
		while (p_ < e_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r'))
			++p_;
	}

	bool literal(const char *word) {
		const size_t n = std::strlen(word);
		if ((size_t)(e_ - p_) < n || std::memcmp(p_, word, n) != 0)
			return fail("unknown literal");
		p_ += n;
		return true;
	}

	bool value(Json &v, int depth) {
		if (depth > kMaxDepth)
			return fail("nested too deeply");
		if (p_ >= e_)
			return fail("unexpected end");
		switch (*p_) {
		case '{':
			return object(v, depth);
		case '[':
			return array(v, depth);
		case '"':
			v.kind = Json::Str;
			return string(v.str);
		case 't':
			v.kind = Json::Bool;
			v.b = true;
			return literal("true");
		case 'f':
			v.kind = Json::Bool;
			v.b = false;
			return literal("false");
		case 'n':
			v.kind = Json::Null;
			return literal("null");
		default:
			v.kind = Json::Num;
			return number(v.num);
		}
	}

	bool object(Json &v, int depth) {
		v.kind = Json::Obj;
		++p_; // '{'
		ws();
		if (p_ < e_ && *p_ == '}') {
			++p_;
			return true;
		}
		for (;;) {
			ws();
			if (p_ >= e_ || *p_ != '"')
				return fail("expected a member name");
			v.obj.emplace_back();
			if (!string(v.obj.back().first))
				return false;
			ws();
			if (p_ >= e_ || *p_ != ':')
				return fail("expected ':'");
			++p_;
			ws();
			if (!value(v.obj.back().second, depth + 1))
				return false;
			ws();
			if (p_ < e_ && *p_ == ',') {
				++p_;
				continue;
			}
			if (p_ < e_ && *p_ == '}') {
				++p_;
				return true;
			}
			return fail("expected ',' or '}'");
		}
	}

	bool array(Json &v, int depth) {
		v.kind = Json::Arr;
		++p_; // '['
		ws();
		if (p_ < e_ && *p_ == ']') {
			++p_;
			return true;
		}
		for (;;) {
			ws();
			v.arr.emplace_back();
			if (!value(v.arr.back(), depth + 1))
				return false;
			ws();
			if (p_ < e_ && *p_ == ',') {
				++p_;
				continue;
			}
			if (p_ < e_ && *p_ == ']') {
				++p_;
				return true;
			}
			return fail("expected ',' or ']'");
		}
	}

	bool hex4(uint32_t &u) {
		if (e_ - p_ < 4)
			return fail("short \\u escape");
		u = 0;
		for (int k = 0; k < 4; ++k) {
			const int h = hex_digit(p_[k]);
			if (h < 0)
				return fail("bad \\u escape");
			u = (u << 4) | (uint32_t)h;
		}
		p_ += 4;
		return true;
	}

	static void utf8(uint32_t c, std::string &s) {
		if (c < 0x80) {
			s += (char)c;
		} else if (c < 0x800) {
			s += (char)(0xC0 | (c >> 6));
			s += (char)(0x80 | (c & 0x3F));
		} else if (c < 0x10000) {
			s += (char)(0xE0 | (c >> 12));
			s += (char)(0x80 | ((c >> 6) & 0x3F));
			s += (char)(0x80 | (c & 0x3F));
		} else {
			s += (char)(0xF0 | (c >> 18));
			s += (char)(0x80 | ((c >> 12) & 0x3F));
			s += (char)(0x80 | ((c >> 6) & 0x3F));
			s += (char)(0x80 | (c & 0x3F));
		}
	}

	bool string(std::string &s) {
		++p_; // opening quote
		for (;;) {
			if (p_ >= e_)
				return fail("unterminated string");
			const unsigned char c = (unsigned char)*p_++;
			if (c == '"')
				return true;
			if (c < 0x20)
				return fail("control character in a string");
			if (c != '\\') {
				s += (char)c;
				continue;
			}
			if (p_ >= e_)
				return fail("unterminated escape");
			const char x = *p_++;
			switch (x) {
			case '"':
			case '\\':
			case '/':
				s += x;
				break;
			case 'b':
				s += '\b';
				break;
			case 'f':
				s += '\f';
				break;
			case 'n':
				s += '\n';
				break;
			case 'r':
				s += '\r';
				break;
			case 't':
				s += '\t';
				break;
			case 'u': {
				uint32_t u = 0;
				if (!hex4(u))
					return false;
				if (u >= 0xD800 && u < 0xDC00) { // high surrogate: a low one must follow
					uint32_t lo = 0;
					if (e_ - p_ < 2 || p_[0] != '\\' || p_[1] != 'u')
						return fail("unpaired surrogate");
					p_ += 2;
					if (!hex4(lo) || lo < 0xDC00 || lo >= 0xE000)
						return fail("unpaired surrogate");
					u = 0x10000 + ((u - 0xD800) << 10) + (lo - 0xDC00);
				} else if (u >= 0xDC00 && u < 0xE000) {
					return fail("unpaired surrogate");
				}
				utf8(u, s);
				break;
			}
			default:
				return fail("bad escape");
			}
		}
	}

	// -?(0|[1-9][0-9]*)(.[0-9]+)?([eE][+-]?[0-9]+)?, correctly rounded to double.
	bool number(double &d) {
		const char *s = p_, *q = p_;
		auto digits = [&]() {
			const char *b = q;
			while (q < e_ && *q >= '0' && *q <= '9')
				++q;
			return q > b;
		};
		if (q < e_ && *q == '-')
			++q;
		if (q < e_ && *q == '0')
			++q;
		else if (!digits())
			return fail("bad number");
		if (q < e_ && *q == '.') {
			++q;
			if (!digits())
				return fail("bad number");
		}
		if (q < e_ && (*q == 'e' || *q == 'E')) {
			++q;
			if (q < e_ && (*q == '+' || *q == '-'))
				++q;
			if (!digits())
				return fail("bad number");
		}
		const std::from_chars_result r = std::from_chars(s, q, d);
		if (r.ec == std::errc::invalid_argument || r.ptr != q)
			return fail("bad number");
		if (r.ec == std::errc::result_out_of_range) {
			// Beyond double's range (only possible in fields this reader does not use):
			// 0 or infinity with the number's sign, as strtod gives.
			const char *x = s;
			while (x < q && *x != 'e' && *x != 'E')
				++x;
			const bool tiny = x + 1 < q && x[1] == '-';
			d = tiny ? 0.0 : __builtin_huge_val();
			if (*s == '-')
				d = -d;
		}
		p_ = q;
		return true;
	}

	const char *p_, *e_;
	std::string err_;
};

// ---------------------------------------------------------------------------------------
// Files, containers and buffers
// ---------------------------------------------------------------------------------------

bool read_file(const std::string &path, std::vector<uint8_t> &out, std::string &err) {
	FILE *f = std::fopen(path.c_str(), "rb");
	if (!f) {
		err = "cannot open " + path;
		return false;
	}
	uint8_t chunk[1 << 16];
	size_t got;
	try {
		while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0)
			out.insert(out.end(), chunk, chunk + got);
	} catch (...) {
		std::fclose(f);
		throw;
	}
	const bool bad = std::ferror(f) != 0;
	std::fclose(f);
	if (bad)
		err = "cannot read " + path;
	return !bad;
}

uint32_t le32(const uint8_t *p) {
	return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

constexpr uint32_t kGlbMagic = 0x46546C67u; // "glTF"
constexpr uint32_t kChunkJson = 0x4E4F534Au; // "JSON"
constexpr uint32_t kChunkBin = 0x004E4942u;  // "BIN\0"

// Splits a .glb into its JSON text and its BIN chunk (empty if none).
bool split_glb(const std::vector<uint8_t> &f, const uint8_t *&json, uint64_t &json_len,
               const uint8_t *&bin, uint64_t &bin_len, std::string &err) {
	if (f.size() < 20 || le32(f.data()) != kGlbMagic) {
		err = "GLB: bad header";
		return false;
	}
	if (le32(f.data() + 4) != 2) {
		err = "GLB: only version 2 is supported";
		return false;
	}
	const uint64_t total = std::min<uint64_t>(le32(f.data() + 8), f.size());
	json = bin = nullptr;
	json_len = bin_len = 0;
	uint64_t at = 12;
	for (int k = 0; at + 8 <= total; ++k) {
		const uint64_t len = le32(f.data() + at), type = le32(f.data() + at + 4);
		if (at + 8 + len > total) {
			err = "GLB: chunk runs past the end of the file";
			return false;
		}
		const uint8_t *data = f.data() + at + 8;
		if (k == 0) {
			if (type != kChunkJson) {
				err = "GLB: the first chunk is not JSON";
				return false;
			}
			json = data;
			json_len = len;
		} else if (k == 1 && type == kChunkBin) {
			bin = data;
			bin_len = len;
		}
		at += 8 + ((len + 3) & ~3ull);
	}
	if (!json) {
		err = "GLB: no JSON chunk";
		return false;
	}
	return true;
}

int b64(unsigned char c) {
	if (c >= 'A' && c <= 'Z')
		return c - 'A';
	if (c >= 'a' && c <= 'z')
		return c - 'a' + 26;
	if (c >= '0' && c <= '9')
		return c - '0' + 52;
	if (c == '+' || c == '-')
		return 62;
	if (c == '/' || c == '_')
		return 63;
	return -1;
}

// Standard base64 (RFC 4648, padding optional, URL-safe letters accepted).
bool decode_base64(const char *p, const char *e, std::vector<uint8_t> &out, std::string &err) {
	uint32_t acc = 0;
	int bits = 0;
	for (; p < e; ++p) {
		if (*p == '=')
			break;
		const int v = b64((unsigned char)*p);
		if (v < 0) {
			err = "data URI: bad base64";
			return false;
		}
		acc = (acc << 6) | (uint32_t)v;
		bits += 6;
		if (bits >= 8) {
			bits -= 8;
			out.push_back((uint8_t)(acc >> bits));
		}
	}
	for (; p < e; ++p)
		if (*p != '=') {
			err = "data URI: characters after the padding";
			return false;
		}
	return true;
}

// The bytes a buffer URI names: base64 data: URIs, or a file relative to `dir`.
bool load_uri(const std::string &uri, const std::string &dir, std::vector<uint8_t> &out,
              std::string &err) {
	if (uri.compare(0, 5, "data:") == 0) {
		const size_t comma = uri.find(',');
		if (comma == std::string::npos || comma < 7 || uri.compare(comma - 7, 7, ";base64") != 0) {
			err = "data URI: only base64 data is supported";
			return false;
		}
		return decode_base64(uri.data() + comma + 1, uri.data() + uri.size(), out, err);
	}
	const size_t colon = uri.find(':'), slash = uri.find('/');
	if (colon != std::string::npos && (slash == std::string::npos || colon < slash)) {
		err = "buffer URI " + uri + ": only relative file names and data: URIs are supported";
		return false;
	}
	std::string path;
	for (size_t i = 0; i < uri.size(); ++i) { // %XX escapes
		const int h1 = i + 2 < uri.size() ? hex_digit(uri[i + 1]) : -1;
		const int h2 = i + 2 < uri.size() ? hex_digit(uri[i + 2]) : -1;
		if (uri[i] == '%' && h1 >= 0 && h2 >= 0) {
			path += (char)(h1 * 16 + h2);
			i += 2;
		} else {
			path += uri[i];
		}
	}
	return read_file(dir + path, out, err);
}

// A non-negative integer member (default `def` when absent).
bool get_uint(const Json &o, const char *key, uint64_t def, uint64_t &v, std::string &err,
              const char *what) {
	const Json *m = o.get(key);
	if (!m) {
		v = def;
		return true;
	}
	if (m->kind != Json::Num || !(m->num >= 0.0) || m->num > 9007199254740992.0 ||
	    m->num != (double)(uint64_t)m->num) {
		err = std::string(what) + ": " + key + " must be a non-negative integer";
		return false;
	}
	v = (uint64_t)m->num;
	return true;
}

// One typed element array in a buffer: count elements of `size` bytes, `stride` apart.
struct Elements {
	const uint8_t *p = nullptr; // null: every element is zero (an accessor without view)
	uint64_t count = 0, stride = 0, size = 0;
};

struct Document {
	Json root;
	std::vector<std::vector<uint8_t>> buffers;
	const uint8_t *bin = nullptr; // the GLB's BIN chunk
	uint64_t bin_len = 0;

	// The bytes of buffer i.
	bool buffer(uint64_t i, const uint8_t *&p, uint64_t &len, std::string &err) const {
		if (i >= buffers.size()) {
			err = "bufferView refers to a missing buffer";
			return false;
		}
		const Json &b = root.get("buffers")->arr[i];
		if (i == 0 && !b.get("uri") && bin) { // a GLB's BIN chunk is its buffer 0
			p = bin;
			len = bin_len;
		} else {
			p = buffers[i].data();
			len = buffers[i].size();
		}
		return true;
	}

	// Accessor `index` as elements of `size` bytes; components must be of `ctypes` (a
	// list of allowed componentType values) and its type `type`.
	bool accessor(uint64_t index, const char *type, std::initializer_list<uint64_t> ctypes,
	              Elements &el, uint64_t *ctype_out, std::string &err) const {
		const Json *accs = root.get("accessors");
		if (!accs || accs->kind != Json::Arr || index >= accs->arr.size()) {
			err = "primitive refers to a missing accessor";
			return false;
		}
		const Json &a = accs->arr[index];
		const std::string what = "accessor " + std::to_string(index);
		if (a.get("sparse")) {
			err = what + ": sparse accessors are not supported";
			return false;
		}
		const Json *t = a.get("type");
		if (!t || t->kind != Json::Str || t->str != type) {
			err = what + ": type must be " + type;
			return false;
		}
		uint64_t ct = 0, count = 0, off = 0, view = 0;
		if (!get_uint(a, "componentType", 0, ct, err, what.c_str()) ||
		    !get_uint(a, "count", 0, count, err, what.c_str()) ||
		    !get_uint(a, "byteOffset", 0, off, err, what.c_str()))
			return false;
		bool ok = false;
		for (uint64_t c : ctypes)
			ok = ok || c == ct;
		if (!ok) {
			err = what + ": unsupported componentType " + std::to_string(ct);
			return false;
		}
		const uint64_t csize = ct == 5121 ? 1 : ct == 5123 ? 2 : 4;
		const uint64_t size = csize * (std::strcmp(type, "VEC3") == 0 ? 3 : 1);
		if (ctype_out)
			*ctype_out = ct;
		el.count = count;
		el.size = size;
		el.stride = size;
		el.p = nullptr;
		if (!a.get("bufferView"))
			return true; // all zeros (glTF 2.0, accessors without a bufferView)
		if (!get_uint(a, "bufferView", 0, view, err, what.c_str()))
			return false;
		const Json *views = root.get("bufferViews");
		if (!views || views->kind != Json::Arr || view >= views->arr.size()) {
			err = what + ": missing bufferView";
			return false;
		}
		const Json &v = views->arr[view];
		const std::string vwhat = "bufferView " + std::to_string(view);
		uint64_t buf = 0, voff = 0, vlen = 0, stride = 0;
		if (!get_uint(v, "buffer", 0, buf, err, vwhat.c_str()) ||
		    !get_uint(v, "byteOffset", 0, voff, err, vwhat.c_str()) ||
		    !get_uint(v, "byteLength", 0, vlen, err, vwhat.c_str()) ||
		    !get_uint(v, "byteStride", 0, stride, err, vwhat.c_str()))
			return false;
		if (stride && (stride < size || stride > 255)) {
			err = vwhat + ": byteStride smaller than the element or above 255";
			return false;
		}
		el.stride = stride ? stride : size;
		const uint8_t *bp = nullptr;
		uint64_t blen = 0;
		if (!buffer(buf, bp, blen, err))
			return false;
		if (voff > blen || vlen > blen - voff) {
			err = vwhat + ": runs past the end of its buffer";
			return false;
		}
		const uint64_t need = count ? off + el.stride * (count - 1) + size : off;
		if (count > (1ull << 40) || need > vlen) {
			err = what + ": runs past the end of its bufferView";
			return false;
		}
		el.p = bp + voff + off;
		return true;
	}
};

// Reads the file at `path` (.gltf or .glb) with every buffer it names.
bool load_document(const std::string &path, Document &doc, std::vector<uint8_t> &file,
                   std::string &err) {
	if (!read_file(path, file, err))
		return false;
	const uint8_t *json = file.data();
	uint64_t json_len = file.size();
	if (file.size() >= 4 && le32(file.data()) == kGlbMagic &&
	    !split_glb(file, json, json_len, doc.bin, doc.bin_len, err))
		return false;
	JsonParser jp(reinterpret_cast<const char *>(json),
	              reinterpret_cast<const char *>(json) + json_len);
	if (!jp.parse(doc.root, err))
		return false;
	if (doc.root.kind != Json::Obj) {
		err = "the document is not a JSON object";
		return false;
	}
	if (const Json *req = doc.root.get("extensionsRequired")) {
		if (req->kind == Json::Arr && !req->arr.empty()) {
			err = "unsupported required extension";
			if (req->arr[0].kind == Json::Str)
				err += " " + req->arr[0].str;
			return false;
		}
	}
	const size_t slash = path.find_last_of('/');
	const std::string dir = slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
	const Json *bufs = doc.root.get("buffers");
	if (!bufs)
		return true;
	if (bufs->kind != Json::Arr) {
		err = "buffers is not an array";
		return false;
	}
	doc.buffers.resize(bufs->arr.size());
	for (size_t i = 0; i < bufs->arr.size(); ++i) {
		const Json &b = bufs->arr[i];
		const std::string what = "buffer " + std::to_string(i);
		uint64_t len = 0;
		if (!get_uint(b, "byteLength", 0, len, err, what.c_str()))
			return false;
		const Json *uri = b.get("uri");
		uint64_t have = 0;
		if (uri) {
			if (uri->kind != Json::Str) {
				err = what + ": uri is not a string";
				return false;
			}
			if (!load_uri(uri->str, dir, doc.buffers[i], err)) {
				err = what + ": " + err;
				return false;
			}
			have = doc.buffers[i].size();
		} else if (i == 0 && doc.bin) {
			have = doc.bin_len;
		}
		if (have < len) {
			err = what + ": shorter than its byteLength";
			return false;
		}
	}
	return true;
}

uint32_t read_index(const Elements &el, uint64_t ctype, uint64_t i) {
	if (!el.p)
		return 0;
	const uint8_t *p = el.p + el.stride * i;
	if (ctype == 5121)
		return p[0];
	if (ctype == 5123)
		return (uint32_t)p[0] | ((uint32_t)p[1] << 8);
	return le32(p);
}

void read_position(const Elements &el, uint64_t i, float *out) {
	if (!el.p) {
		out[0] = out[1] = out[2] = 0.0f;
		return;
	}
	std::memcpy(out, el.p + el.stride * i, 12); // little-endian IEEE floats, as stored
}

// The triangle soup of every mesh, in the example's order (see the file comment).
bool triangles(const Document &doc, std::vector<float> &tris, std::string &err) {
	const Json *meshes = doc.root.get("meshes");
	if (!meshes)
		return true;
	if (meshes->kind != Json::Arr) {
		err = "meshes is not an array";
		return false;
	}
	for (size_t m = 0; m < meshes->arr.size(); ++m) {
		const Json *prims = meshes->arr[m].get("primitives");
		if (!prims || prims->kind != Json::Arr)
			continue;
		for (size_t pi = 0; pi < prims->arr.size(); ++pi) {
			const Json &pr = prims->arr[pi];
			const std::string what =
			    "mesh " + std::to_string(m) + " primitive " + std::to_string(pi);
			uint64_t mode = 4, pos = 0, idx = 0;
			if (!get_uint(pr, "mode", 4, mode, err, what.c_str()))
				return false;
			if (mode != 4)
				continue; // not TRIANGLES
			const Json *attrs = pr.get("attributes");
			const Json *pa = attrs ? attrs->get("POSITION") : nullptr;
			if (!pa || !pr.get("indices"))
				continue; // the example needs both
			if (!get_uint(*attrs, "POSITION", 0, pos, err, what.c_str()) ||
			    !get_uint(pr, "indices", 0, idx, err, what.c_str()))
				return false;
			Elements P, I;
			uint64_t ictype = 0;
			if (!doc.accessor(pos, "VEC3", {5126}, P, nullptr, err) ||
			    !doc.accessor(idx, "SCALAR", {5121, 5123, 5125}, I, &ictype, err)) {
				err = what + ": " + err;
				return false;
			}
			const uint64_t n_tri = I.count / 3;
			tris.reserve(tris.size() + 9 * n_tri);
			for (uint64_t t = 0; t < n_tri; ++t)
				for (int k = 0; k < 3; ++k) {
					const uint32_t v = read_index(I, ictype, 3 * t + k);
					if (v >= P.count) {
						err = what + ": index " + std::to_string(v) + " beyond " +
						      std::to_string(P.count) + " positions";
						return false;
					}
					float xyz[3];
					read_position(P, v, xyz);
					tris.insert(tris.end(), xyz, xyz + 3);
				}
		}
	}
	return true;
}

} // namespace

extern "C" int prt_b200_gltf_load(const char *path, float **tris9, uint64_t *n_tris) {
	if (!path || !tris9 || !n_tris) {
		prt::set_global_error("gltf_load: null argument");
		return PRT_ERR_ARG;
	}
	*tris9 = nullptr;
	*n_tris = 0;
	std::vector<float> tris;
	try {
		Document doc;
		std::vector<uint8_t> file;
		std::string err;
		if (!load_document(path, doc, file, err) || !triangles(doc, tris, err)) {
			prt::set_global_error("gltf_load: " + err);
			return PRT_ERR_ARG;
		}
	} catch (const std::bad_alloc &) {
		prt::set_global_error("gltf_load: out of host memory");
		return PRT_ERR_OOM;
	}
	float *out = static_cast<float *>(std::malloc(std::max<size_t>(tris.size(), 1) * sizeof(float)));
	if (!out) {
		prt::set_global_error("gltf_load: out of host memory");
		return PRT_ERR_OOM;
	}
	if (!tris.empty())
		std::memcpy(out, tris.data(), tris.size() * sizeof(float));
	*tris9 = out;
	*n_tris = tris.size() / 9;
	return PRT_OK;
}
