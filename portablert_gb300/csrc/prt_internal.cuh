// prt_internal.cuh - shared definitions of the GB300 ray-query backend.
//
// Data layout in HBM for one scene (n triangles):
//   tri4   float4[3n]  triangle records in leaf order: (v0.xyz, primitive id bits),
//                      (v1.xyz, 0), (v2.xyz, 0); 48 B per triangle.
//   nodes  Node8[]     8-wide nodes, 256 B each (eight 32-B child records: box and
//                      reference), root at index 0.
//   cnodes CNode8[]    the same tree with 8-bit child boxes, 96 B each (optional).
//
// A child reference is 32 bits: 0xFFFFFFFF = empty slot; bit 31 clear = index of a
// child node; bit 31 set = leaf holding triangles [first, first + count) of tri4 with
// first in bits 0..27 and count - 1 in bits 28..30.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace prt {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kFirstMask = 0x0FFFFFFFu;
constexpr int kMaxLeaf = 8;
// Triangles per scene: the traversal packs (ray slot, node or triangle index) into 32
// bits with 27 bits for the index.
constexpr uint64_t kMaxTris = (1ull << 27) - 1;
constexpr uint32_t kIndexBits = 27;
constexpr uint32_t kIndexMask = (1u << kIndexBits) - 1u;

// Bits of the device error word.
enum : uint32_t {
	kErrStack = 1u,    // traversal stack overflow (ray abandoned)
	kErrLookback = 2u, // radix-sort look-back gave up waiting
	kErrCollapse = 4u, // 8-wide collapse ran out of node slots
	kErrSah = 8u,      // SAH build: a range, node id or task list check failed
};

// One child of an 8-wide FP32 node: its box and its reference, 32 B, so the lane that
// tests child c reads it with one 32-byte load and a node's 8 children are 256
// contiguous bytes.
struct alignas(16) Child8 {
	float lo_x, lo_y, lo_z;
	uint32_t ref;
	float hi_x, hi_y, hi_z;
	uint32_t pad;
};
struct alignas(16) Node8 {
	Child8 c[8];
};
static_assert(sizeof(Node8) == 256, "Node8 layout");

// A decoded compressed bound, origin + q * scale with one rounding (a fused multiply-add:
// q <= 255 times a power of two is exact, so this is o + q * s correctly rounded, even
// where q * s alone would overflow).  The builder verifies every bound with this
// function and the traversal decodes with it, so the two agree bit for bit.
__device__ __forceinline__ float cdec_f(float o, float q, float s) { return __fmaf_rn(q, s, o); }

// Compressed 8-wide node (96 B = 37.5 % of Node8), the same tree as Node8.  Child box
// k, per axis a: lo = origin_a + q_lo * 2^(e_a - 127), hi = origin_a + q_hi * 2^(e_a - 127),
// evaluated in FP32 exactly as the traversal does (cdec_f); the builder chooses each q so
// that the decoded box contains the child's FP32 box (rounded outward), which keeps
// every box test conservative.  Child k is an inner node when bit k of imask is set, at
// index child_base + (number of inner children before k); otherwise, when count > 0,
// a leaf of `count` triangles starting at tri_base + first.
struct alignas(8) CChild8 {
	uint8_t qlo_x, qhi_x, qlo_y, qhi_y, qlo_z, qhi_z;
	uint8_t count; // leaf triangles (0 = inner child or empty slot)
	uint8_t first; // leaf: first triangle relative to tri_base
};
struct alignas(16) CNode8 {
	float ox, oy, oz;       // frame origin (the node's lower corner)
	uint8_t ex, ey, ez;     // scale exponents, IEEE-biased
	uint8_t imask;          // inner-node children
	uint32_t child_base;    // first inner child
	uint32_t tri_base;      // first triangle of the node's leaf children
	uint32_t pad[2];
	CChild8 c[8];
};
static_assert(sizeof(CChild8) == 8, "CChild8 layout");
static_assert(sizeof(CNode8) == 96, "CNode8 layout");

// Decodes one quantised bound.  2^(e-127) * q is exact (q < 256, e in [1, 254]); the
// sum is rounded once, and the builder verified the rounded value, so this exact
// expression must be used on both sides.
__host__ __device__ inline float cscale(uint8_t e) {
	union { uint32_t u; float f; } s;
	s.u = (uint32_t)e << 23;
	return s.f;
}

__host__ __device__ inline uint32_t make_leaf(uint32_t first, uint32_t count) {
	return kLeafBit | ((count - 1u) << 28) | first;
}
__host__ __device__ inline bool ref_is_leaf(uint32_t r) { return (r & kLeafBit) != 0; }
__host__ __device__ inline uint32_t leaf_first(uint32_t r) { return r & kFirstMask; }
__host__ __device__ inline uint32_t leaf_count(uint32_t r) { return ((r >> 28) & 7u) + 1u; }

// std::min / std::max as portableRT calls them: select on operator<, so a NaN in the
// first argument survives and a NaN in the second is dropped.
__device__ __forceinline__ float rmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float rmax(float a, float b) { return (a < b) ? b : a; }

// Order-preserving float <-> uint32 map for atomicMin / atomicMax on floats.
__device__ __forceinline__ uint32_t f2ord(float f) {
	uint32_t u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
	return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Per-ray constants.  `kind` selects the box test used on inner nodes:
//   0 regular: all three reciprocals finite; the plain slab test is exact and safe.
//   1 axis:    some reciprocal is infinite (a zero or denormal direction component);
//              inner nodes use conservative_box below.
//   2 all:     a non-finite component or all reciprocals infinite: every inner box
//              passes and only the exact per-triangle test decides.
struct RayC {
	float ox, oy, oz, dx, dy, dz, fx, fy, fz;
	int kind;
};

__device__ __forceinline__ RayC make_ray(float ox, float oy, float oz, float dx, float dy,
                                         float dz) {
	RayC r;
	r.ox = ox; r.oy = oy; r.oz = oz;
	r.dx = dx; r.dy = dy; r.dz = dz;
	// IEEE reciprocal, identical to portableRT's 1.0f / direction (bvh.hpp:199-201).
	r.fx = __frcp_rn(dx);
	r.fy = __frcp_rn(dy);
	r.fz = __frcp_rn(dz);
	bool fin = isfinite(ox) && isfinite(oy) && isfinite(oz) && isfinite(dx) && isfinite(dy) &&
	           isfinite(dz);
	int n_inf = (int)isinf(r.fx) + (int)isinf(r.fy) + (int)isinf(r.fz);
	r.kind = (!fin || n_inf == 3) ? 2 : (n_inf ? 1 : 0);
	return r;
}

// Slab test of portableRT's ray_box_intersect (bvh.hpp:195-222), bit for bit: each
// t is (bound - origin) * reciprocal in round-to-nearest, combined with the select
// min/max in the reference's nesting.  Used on every triangle's own bounding box.
__device__ __forceinline__ bool ref_slab(const RayC &r, float lx, float ly, float lz, float hx,
                                         float hy, float hz) {
	float t1 = __fmul_rn(__fsub_rn(lx, r.ox), r.fx);
	float t2 = __fmul_rn(__fsub_rn(hx, r.ox), r.fx);
	float t3 = __fmul_rn(__fsub_rn(ly, r.oy), r.fy);
	float t4 = __fmul_rn(__fsub_rn(hy, r.oy), r.fy);
	float t5 = __fmul_rn(__fsub_rn(lz, r.oz), r.fz);
	float t6 = __fmul_rn(__fsub_rn(hz, r.oz), r.fz);
	float tmin = rmax(rmax(rmin(t1, t2), rmin(t3, t4)), rmin(t5, t6));
	float tmax = rmin(rmin(rmax(t1, t2), rmax(t3, t4)), rmax(t5, t6));
	if (tmax < 0.0f)
		return false;
	if (tmin > tmax)
		return false;
	return true;
}

// Inner-node test for regular rays.  Same (bound - origin) * reciprocal rounding as
// ref_slab; an inner box contains every triangle box below it and that expression is
// monotone in the bound, so whatever ref_slab accepts below, this accepts here.  No
// NaN can arise (finite bounds or +-inf, finite non-zero reciprocal).
__device__ __forceinline__ bool regular_box(const RayC &r, float lx, float hx, float ly, float hy,
                                            float lz, float hz) {
	float t1 = (lx - r.ox) * r.fx, t2 = (hx - r.ox) * r.fx;
	float t3 = (ly - r.oy) * r.fy, t4 = (hy - r.oy) * r.fy;
	float t5 = (lz - r.oz) * r.fz, t6 = (hz - r.oz) * r.fz;
	float tmin = fmaxf(fmaxf(fminf(t1, t2), fminf(t3, t4)), fminf(t5, t6));
	float tmax = fminf(fminf(fmaxf(t1, t2), fmaxf(t3, t4)), fmaxf(t5, t6));
	return tmax >= 0.0f && tmin <= tmax;
}

// One axis of the conservative test for a ray with an infinite reciprocal on it.
// A triangle box on this axis yields, per ref_slab: origin below the box -> both t's
// +inf (reciprocal +inf) or -inf; origin above -> the opposite; strictly inside ->
// (-inf, +inf); origin exactly on the lower face -> NaN, which on the x axis makes the
// whole reference test pass and on y or z removes that axis from it.  For an inner box
// the same below/above answer holds for every box under it; otherwise the axis is
// treated as unconstrained (y, z) or the box passes outright (x).
__device__ __forceinline__ bool inf_axis(float o, float lo, float hi, float f, bool is_x, float &m,
                                         float &M) {
	if (o < lo) {
		m = M = (f > 0.0f) ? INFINITY : -INFINITY;
	} else if (o > hi) {
		m = M = (f > 0.0f) ? -INFINITY : INFINITY;
	} else {
		if (is_x)
			return true;
		m = -INFINITY;
		M = INFINITY;
	}
	return false;
}

__device__ __forceinline__ bool conservative_box(const RayC &r, float lx, float hx, float ly,
                                                 float hy, float lz, float hz) {
	if (r.kind == 2)
		return true;
	float m0, M0, m1, M1, m2, M2;
	if (isinf(r.fx)) {
		if (inf_axis(r.ox, lx, hx, r.fx, true, m0, M0))
			return true;
	} else {
		float a = (lx - r.ox) * r.fx, b = (hx - r.ox) * r.fx;
		m0 = fminf(a, b);
		M0 = fmaxf(a, b);
	}
	if (isinf(r.fy)) {
		inf_axis(r.oy, ly, hy, r.fy, false, m1, M1);
	} else {
		float a = (ly - r.oy) * r.fy, b = (hy - r.oy) * r.fy;
		m1 = fminf(a, b);
		M1 = fmaxf(a, b);
	}
	if (isinf(r.fz)) {
		inf_axis(r.oz, lz, hz, r.fz, false, m2, M2);
	} else {
		float a = (lz - r.oz) * r.fz, b = (hz - r.oz) * r.fz;
		m2 = fminf(a, b);
		M2 = fmaxf(a, b);
	}
	float tmin = fmaxf(fmaxf(m0, m1), m2);
	float tmax = fminf(fminf(M0, M1), M2);
	return tmax >= 0.0f && tmin <= tmax;
}

// Moller-Trumbore in portableRT's operation order (core.hpp:27-65): every product and
// sum rounded separately (no FMA), sums left to right, IEEE reciprocal of det.
__device__ __forceinline__ bool ref_mt(const RayC &r, float v0x, float v0y, float v0z, float v1x,
                                       float v1y, float v1z, float v2x, float v2y, float v2z,
                                       float &t, float &u, float &v) {
	float e1x = __fsub_rn(v1x, v0x), e1y = __fsub_rn(v1y, v0y), e1z = __fsub_rn(v1z, v0z);
	float e2x = __fsub_rn(v2x, v0x), e2y = __fsub_rn(v2y, v0y), e2z = __fsub_rn(v2z, v0z);
	float px = __fsub_rn(__fmul_rn(r.dy, e2z), __fmul_rn(r.dz, e2y));
	float py = __fsub_rn(__fmul_rn(r.dz, e2x), __fmul_rn(r.dx, e2z));
	float pz = __fsub_rn(__fmul_rn(r.dx, e2y), __fmul_rn(r.dy, e2x));
	float det = __fadd_rn(__fadd_rn(__fmul_rn(e1x, px), __fmul_rn(e1y, py)), __fmul_rn(e1z, pz));
	if (det == 0.0f)
		return false;
	float inv = __frcp_rn(det);
	float tx = __fsub_rn(r.ox, v0x), ty = __fsub_rn(r.oy, v0y), tz = __fsub_rn(r.oz, v0z);
	u = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(tx, px), __fmul_rn(ty, py)), __fmul_rn(tz, pz)),
	              inv);
	if (u < 0.0f || u > 1.0f)
		return false;
	float qx = __fsub_rn(__fmul_rn(ty, e1z), __fmul_rn(tz, e1y));
	float qy = __fsub_rn(__fmul_rn(tz, e1x), __fmul_rn(tx, e1z));
	float qz = __fsub_rn(__fmul_rn(tx, e1y), __fmul_rn(ty, e1x));
	v = __fmul_rn(
	    __fadd_rn(__fadd_rn(__fmul_rn(r.dx, qx), __fmul_rn(r.dy, qy)), __fmul_rn(r.dz, qz)), inv);
	if (v < 0.0f || __fadd_rn(u, v) > 1.0f)
		return false;
	t = __fmul_rn(
	    __fadd_rn(__fadd_rn(__fmul_rn(e2x, qx), __fmul_rn(e2y, qy)), __fmul_rn(e2z, qz)), inv);
	return true;
}

// The closest hit so far.  Ties in t go to the smaller primitive id, so the answer
// does not depend on traversal order; a t of +inf or NaN is never recorded (the
// reference keeps a hit only when t < t_near, t_near starting at +inf).
struct Best {
	float t, u, v;
	uint32_t pid;
};

__device__ __forceinline__ void best_init(Best &b) {
	b.t = INFINITY;
	b.u = 0.0f;
	b.v = 0.0f;
	b.pid = kNone;
}

// The box half of tri_test for a ray with finite origin, direction and reciprocals (kind
// 0) and a triangle whose nine coordinates are finite (its record's flag word is 0):
// then no value is NaN, the select min/max of the reference agree with fminf / fmaxf
// (three-input where they nest; a zero's sign can differ, and no comparison sees it),
// and the answer is ref_slab's with fewer instructions.
__device__ __forceinline__ bool tri_box_finite(const RayC &r, const float4 a, const float4 b,
                                               const float4 c) {
	const float lx = fminf(a.x, fminf(b.x, c.x)), ly = fminf(a.y, fminf(b.y, c.y)),
	            lz = fminf(a.z, fminf(b.z, c.z));
	const float hx = fmaxf(a.x, fmaxf(b.x, c.x)), hy = fmaxf(a.y, fmaxf(b.y, c.y)),
	            hz = fmaxf(a.z, fmaxf(b.z, c.z));
	return regular_box(r, lx, hx, ly, hy, lz, hz);
}

// A triangle record's flag word (the second float4's w): 0 when every coordinate is
// finite, 1 otherwise.
__device__ __forceinline__ bool tri_record_finite(const float4 &b) { return b.w == 0.0f; }

// Exact per-triangle test: the reference slab test on the triangle's own bounding
// box (make_aabb, bvh.hpp:28-37, select semantics) and then Moller-Trumbore.  True
// when the reference would accept the triangle (its t may still be +inf or NaN, which
// the reference never records).
// finite: the ray is of kind 0 and the triangle's record flags no non-finite coordinate
// (tri_box_finite then decides the box test, with the same answer).
__device__ __forceinline__ bool tri_test(const RayC &r, const float4 a, const float4 b,
                                         const float4 c, float &t, float &u, float &v,
                                         bool finite = false) {
	bool pass;
	if (finite) {
		pass = tri_box_finite(r, a, b, c);
	} else {
		float lx = rmin(a.x, rmin(b.x, c.x)), ly = rmin(a.y, rmin(b.y, c.y)),
		      lz = rmin(a.z, rmin(b.z, c.z));
		float hx = rmax(a.x, rmax(b.x, c.x)), hy = rmax(a.y, rmax(b.y, c.y)),
		      hz = rmax(a.z, rmax(b.z, c.z));
		pass = ref_slab(r, lx, ly, lz, hx, hy, hz);
	}
	if (!pass)
		return false;
	return ref_mt(r, a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z, t, u, v);
}

// The closest hit as one 64-bit key: order-preserving bits of t above the primitive
// id, so the minimum key is the smallest t and, among equal t, the smallest id (ties in
// t go to the smaller id).  -0 and +0 compare equal as floats, so both map to +0's key
// (the traversal keeps the winner's own zero sign, u and v beside the key, or tests the
// winner again).  kNoHit: nothing recorded.
constexpr unsigned long long kNoHit = ~0ull;

__device__ __forceinline__ unsigned long long hit_key(float t, uint32_t pid) {
	float tc = (t == 0.0f) ? 0.0f : t;
	return ((unsigned long long)f2ord(tc) << 32) | pid;
}

} // namespace prt
