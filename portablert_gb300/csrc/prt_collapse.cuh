// prt_collapse.cuh - what the builders share about the 8-wide collapse: the level
// counters the host reads, and the least-expected-cost model that decides which binary
// subtrees become 8-wide nodes and which become leaves (prt_build.cu, prt_build_small.cu).
#pragma once

#include <cfloat>
#include <stdint.h>

#include "prt_internal.cuh"

namespace prt {

constexpr int kMaxLevels = 32;     // 8-wide levels (the traversal's depth limit)
constexpr int kLevelsPerCheck = 4; // collapse launches between host checks
// counters layout: [0, kMaxLevels] frontier size per level, then nodes used, triangles placed
constexpr int kCtrNodes = kMaxLevels + 1;
constexpr int kCtrTris = kMaxLevels + 2;
constexpr int kCtrWords = kMaxLevels + 3;

// Surface area (up to a constant) of a box; FLT_MAX when it overflows.
__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
	float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
	float a = dx * dy + dx * dz + dy * dz;
	return isfinite(a) ? a : FLT_MAX;
}

// Cost-optimal collapse.  Without culling by t, a ray tests the children of every 8-wide
// node whose box it passes and every triangle of every leaf box it passes, so the
// expected work per ray is proportional to the sum of area x cost over those boxes: 1
// per 8-wide node, kTriCost per triangle of a leaf.  A bottom-up pass computes for each
// binary node the least cost of its subtree in a single child slot (c1: as a leaf, or
// as an 8-wide node whose 8 slots are shared out below it) and in i = 2..8 slots when
// the node itself is opened (cd), with the split of the slots between its children; the
// collapse then opens exactly what the optimum opens.  (The dynamic programme of Ylitie,
// Karras and Laine 2017 for compressed wide BVHs, restated for this traversal's costs.)
// Costs are stored in units of the node's own surface area (expected work once a ray
// passes its box), so they stay in float range whatever the scene's scale; a child
// enters its parent's sums weighted by the ratio of the two areas, both computed from
// half extents divided by the parent's largest one (values in [0, 1]: no overflow for
// [-FLT_MAX, FLT_MAX] boxes, no underflow for tiny scenes).
constexpr float kTriCost = 0.25f; // a triangle test against a node visit (measured)

struct CostNode {
	float c1;
	float cd[7];   // slots 2..8
	uint32_t bits; // 3 bits per slot count i = 2..8: (left share - 1); bit 31: leaf is best
};

__device__ __forceinline__ float3 half_extent(float4 lo, float4 hi) {
	return make_float3(fmaxf(hi.x * 0.5f - lo.x * 0.5f, 0.0f),
	                   fmaxf(hi.y * 0.5f - lo.y * 0.5f, 0.0f),
	                   fmaxf(hi.z * 0.5f - lo.z * 0.5f, 0.0f));
}

// Surface area (up to a constant) of a box of half extents e, in units of unit^2.
__device__ __forceinline__ float scaled_area(float3 e, float unit) {
	if (!(unit > 0.0f))
		return 0.0f;
	const float x = fminf(e.x / unit, 1.0f), y = fminf(e.y / unit, 1.0f),
	            z = fminf(e.z / unit, 1.0f);
	return x * y + x * z + y * z;
}

// The left child's share of i slots.
__device__ __forceinline__ uint32_t split_of(uint32_t bits, uint32_t i) {
	const uint32_t a = ((bits >> (3u * (i - 2u))) & 7u) + 1u;
	return min(max(a, 1u), i - 1u);
}

// Costs of a child in j = 1..7 slots (cs[j]), in units of its own area: a single
// triangle costs kTriCost in any number of slots; a binary node its c1, or less when
// opening it into j slots is cheaper.
__device__ __forceinline__ void leaf_costs(float cs[8]) {
#pragma unroll
	for (int j = 1; j < 8; ++j)
		cs[j] = kTriCost;
}
__device__ __forceinline__ void node_costs(const CostNode &c, float cs[8]) {
	cs[1] = c.c1;
#pragma unroll
	for (int j = 2; j < 8; ++j)
		cs[j] = fminf(c.c1, c.cd[j - 2]);
}

// Surface area of a box of half extents e in units of unit^2, given 1 / unit (0 when
// unit is not positive): multiplications instead of divisions, rounded differently.
__device__ __forceinline__ float scaled_area_rcp(float3 e, float rcp) {
	const float x = fminf(e.x * rcp, 1.0f), y = fminf(e.y * rcp, 1.0f), z = fminf(e.z * rcp, 1.0f);
	return x * y + x * z + y * z;
}

// The cost record of a binary node of `count` triangles from its children's costs (cl,
// cr: in units of each child's own area) and the half extents of the three boxes.
// kRcp: the area ratios from two reciprocals instead of eleven divisions (the one-block
// build, whose merges are a chain of dependent work on one SM); the decisions may then
// differ from the divided ones where two costs differ in the last bits.
template <bool kRcp = false>
__device__ __forceinline__ CostNode merge_costs(float cl[8], float cr[8], float3 el, float3 er,
                                                float3 ep, uint32_t count, uint32_t leaf_size) {
	const float unit = fmaxf(ep.x, fmaxf(ep.y, ep.z));
	float ap, rl, rr;
	if (kRcp) {
		const float ru = unit > 0.0f ? 1.0f / unit : 0.0f;
		ap = scaled_area_rcp(ep, ru);
		const float ra = ap > 0.0f ? 1.0f / ap : 0.0f;
		rl = fminf(scaled_area_rcp(el, ru) * ra, 1.0f);
		rr = fminf(scaled_area_rcp(er, ru) * ra, 1.0f);
	} else {
		ap = scaled_area(ep, unit);
		rl = ap > 0.0f ? fminf(scaled_area(el, unit) / ap, 1.0f) : 0.0f;
		rr = ap > 0.0f ? fminf(scaled_area(er, unit) / ap, 1.0f) : 0.0f;
	}
#pragma unroll
	for (int j = 1; j < 8; ++j) {
		cl[j] *= rl;
		cr[j] *= rr;
	}
	CostNode c;
	c.bits = 0;
#pragma unroll
	for (uint32_t s = 2; s <= 8; ++s) {
		float best = INFINITY;
		uint32_t ba = 1;
#pragma unroll
		for (uint32_t a = 1; a < s; ++a) {
			const float v = cl[a] + cr[s - a];
			if (v < best) {
				best = v;
				ba = a;
			}
		}
		c.cd[s - 2] = best;
		c.bits |= (ba - 1u) << (3u * (s - 2u));
	}
	const float as_node = 1.0f + c.cd[6];
	const bool may_leaf = count <= leaf_size;
	const float as_leaf = kTriCost * (float)count;
	c.c1 = may_leaf ? fminf(as_node, as_leaf) : as_node;
	if (may_leaf && as_leaf <= as_node)
		c.bits |= 0x80000000u;
	return c;
}

} // namespace prt
