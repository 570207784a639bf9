// prt_build.cu - LBVH build of 8-wide trees on the GPU, for one scene or many at once,
// and the stages every build shares (collapse, re-layout, compression).
//
// Replaces the single-threaded binned-SAH build of portableRT (bvh.hpp:58-193).  The
// tree's shape does not affect the answers (every triangle whose own box passes the
// reference slab test is examined; see prt_traverse.cu), only how many boxes a ray
// passes: set_tris, batch builds and servers build their binary trees with binned SAH
// by default (prt_sah.cu, steps 1-5 replaced); graph-captured batch builds and the
// option build_sah = 0 use this LBVH, about 3x faster to build.  Several scenes are
// built in the same launches: scene s owns the input triangles [tri_off[s],
// tri_off[s+1]), its sort key carries the scene index above the Morton code, its binary
// nodes are the range [int_off[s], int_off[s+1]) and its 8-wide root is node s.
//   1. centroid bounds per scene  (k_centroid_bounds; warp reduce + ordered-int atomics)
//   2. 30-bit Morton codes        (k_morton; 10 bits per axis, centroids normalised)
//   3. onesweep radix sort        (prt_sort.cu; 4 digit passes, +1 or 2 for the scene)
//   4. Karras hierarchy           (k_karras; Karras 2012 within each scene's range)
//   5. bottom-up refit            (k_leaf_boxes + k_refit; atomic arrival counters)
//   6. collapse to 8-wide nodes   (k_collapse_cost: bottom-up least expected cost per
//                                  ray, which subtrees become nodes and which leaves;
//                                  then k_collapse, one launch per level, per-level
//                                  counters, so the host checks progress every few levels)
//   7. triangle re-layout         (k_relayout; each node's leaf triangles contiguous)
//   8. optional 8-bit encoding    (k_compress; outward-rounded child boxes)
// A triangle with a non-finite vertex gets the box [-FLT_MAX, FLT_MAX]^3 in the tree,
// which every finite ray passes, so the exact per-triangle test still sees it.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <cstring>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"
#include "prt_collapse.cuh"
#include "prt_sah.cuh"

namespace prt {

namespace {
std::atomic<int64_t> g_alloc_failure{0}; // growths left before the injected failure
} // namespace

void arm_alloc_failure(int64_t n) { g_alloc_failure.store(n > 0 ? n : 0); }

bool alloc_failure_due() {
	int64_t v = g_alloc_failure.load(std::memory_order_relaxed);
	while (v > 0)
		if (g_alloc_failure.compare_exchange_weak(v, v - 1))
			return v == 1;
	return false;
}

void BuildScratch::release() {
	DevBuf *all[] = {&keys,        &vals,     &keys2,      &vals2,    &scene_of,   &int_off,
	                 &left,        &right,    &parent_int, &parent_leaf, &rfirst,  &rlast,
	                 &ibox,        &lbox,     &flags,      &items_a,  &items_b,    &counters,
	                 &perm,        &sort_hist, &sort_tiles, &sort_status, &bounds,
	                 &sah,         &roots,    &cost};
	for (DevBuf *b : all)
		b->release();
	if (h_counters)
		cudaFreeHost(h_counters);
	h_counters = nullptr;
	h_sah = nullptr;
}

namespace {

struct Item {
	uint32_t ref;  // binary-tree reference (bit 31 = leaf); kNone = empty scene
	uint32_t slot; // index of the 8-wide node it becomes
};

__device__ __forceinline__ bool tri_finite(const float *t) {
	bool ok = true;
#pragma unroll
	for (int k = 0; k < 9; ++k)
		ok = ok && isfinite(t[k]);
	return ok;
}

__device__ __forceinline__ float centroid(const float *t, int k) {
	return t[k] * (1.0f / 3.0f) + t[k + 3] * (1.0f / 3.0f) + t[k + 6] * (1.0f / 3.0f);
}

__device__ __forceinline__ uint32_t scene_at(const uint32_t *scene_of, uint32_t i) {
	return scene_of ? scene_of[i] : 0u;
}

// scene_of[i] = s for every triangle of scene s (one block per scene, grid-stride).
__global__ void k_scene_of(const uint32_t *tri_off, uint32_t n_scenes, uint32_t *scene_of) {
	for (uint32_t s = blockIdx.x; s < n_scenes; s += gridDim.x)
		for (uint32_t i = tri_off[s] + threadIdx.x; i < tri_off[s + 1]; i += blockDim.x)
			scene_of[i] = s;
}

__global__ void k_bounds_init(uint32_t *gb, uint32_t n_scenes) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 6 * n_scenes;
	     i += gridDim.x * blockDim.x)
		gb[i] = (i % 6) < 3 ? 0xFFFFFFFFu : 0u;
}

// Per-scene centroid bounds as ordered words: a warp whose triangles all belong to one
// scene reduces first; otherwise each lane updates its own scene.
__global__ void k_centroid_bounds(const float *__restrict__ tris, uint32_t n,
                                  const uint32_t *__restrict__ scene_of, uint32_t *gb) {
	const int lane = threadIdx.x & 31;
	if (!scene_of) {
		// One scene: each thread folds its grid-stride share, then the block reduces and
		// one thread updates the six words (so the same-address atomics stay few).
		float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
		for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
		     i += gridDim.x * blockDim.x) {
			const float *t = tris + 9 * (size_t)i;
			if (tri_finite(t)) {
#pragma unroll
				for (int k = 0; k < 3; ++k) {
					const float c = centroid(t, k);
					mn[k] = fminf(mn[k], c);
					mx[k] = fmaxf(mx[k], c);
				}
			}
		}
		__shared__ float red[32][6];
#pragma unroll
		for (int k = 0; k < 3; ++k)
			for (int o = 16; o > 0; o >>= 1) {
				mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
				mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
			}
		const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
		if (lane == 0)
			for (int k = 0; k < 3; ++k) {
				red[w][k] = mn[k];
				red[w][3 + k] = mx[k];
			}
		__syncthreads();
		if (threadIdx.x == 0) {
			for (int v = 1; v < nw; ++v)
				for (int k = 0; k < 3; ++k) {
					mn[k] = fminf(mn[k], red[v][k]);
					mx[k] = fmaxf(mx[k], red[v][3 + k]);
				}
			if (mn[0] <= mx[0])
				for (int k = 0; k < 3; ++k) {
					atomicMin(&gb[k], f2ord(mn[k]));
					atomicMax(&gb[3 + k], f2ord(mx[k]));
				}
		}
		return;
	}
	for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
		const uint32_t i = base + threadIdx.x;
		float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
		uint32_t s = 0;
		if (i < n) {
			const float *t = tris + 9 * (size_t)i;
			s = scene_at(scene_of, i);
			if (tri_finite(t)) {
#pragma unroll
				for (int k = 0; k < 3; ++k)
					mn[k] = mx[k] = centroid(t, k);
			}
		}
		// Lanes past the end hold empty bounds, so they never change a reduction.
		const uint32_t s0 = __shfl_sync(0xFFFFFFFFu, s, 0);
		const bool same = __all_sync(0xFFFFFFFFu, s == s0 || i >= n);
		if (same) {
#pragma unroll
			for (int k = 0; k < 3; ++k) {
				for (int o = 16; o > 0; o >>= 1) {
					mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
					mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
				}
			}
			if (lane == 0 && mn[0] <= mx[0]) {
#pragma unroll
				for (int k = 0; k < 3; ++k) {
					atomicMin(&gb[6 * s0 + k], f2ord(mn[k]));
					atomicMax(&gb[6 * s0 + 3 + k], f2ord(mx[k]));
				}
			}
		} else if (i < n && mn[0] <= mx[0]) {
#pragma unroll
			for (int k = 0; k < 3; ++k) {
				atomicMin(&gb[6 * s + k], f2ord(mn[k]));
				atomicMax(&gb[6 * s + 3 + k], f2ord(mx[k]));
			}
		}
	}
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
	x &= 1023u;
	x = (x | (x << 16)) & 0x030000FFu;
	x = (x | (x << 8)) & 0x0300F00Fu;
	x = (x | (x << 4)) & 0x030C30C3u;
	x = (x | (x << 2)) & 0x09249249u;
	return x;
}

// Key = Morton code of the centroid in its scene's centroid box; with several scenes
// (64-bit keys) the scene index sits above it.
template <typename K>
__global__ void k_morton(const float *__restrict__ tris, uint32_t n,
                         const uint32_t *__restrict__ scene_of, const uint32_t *gb, K *keys,
                         uint32_t *vals) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const float *t = tris + 9 * (size_t)i;
	const uint32_t s = scene_at(scene_of, i);
	const uint32_t *b = gb + 6 * s;
	uint32_t code = 0;
	if (tri_finite(t) && ord2f(b[0]) <= ord2f(b[3])) {
		uint32_t q[3];
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			const float lo = ord2f(b[k]), hi = ord2f(b[3 + k]);
			const float ext = hi - lo;
			const float sc = ext > 0.0f ? 1024.0f / ext : 0.0f;
			const float qf = fminf(fmaxf((centroid(t, k) - lo) * sc, 0.0f), 1023.0f);
			q[k] = (uint32_t)qf;
		}
		code = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
	}
	if (sizeof(K) == 8)
		keys[i] = (K)(((uint64_t)s << 32) | code);
	else
		keys[i] = (K)code;
	vals[i] = i;
}

// Common-prefix length of the Morton codes of leaves i and j of one scene, with the
// index appended to break ties between equal codes; -1 outside [0, n).
template <typename K>
__device__ __forceinline__ int kdelta(const K *__restrict__ k, int n, int i, int j) {
	if (j < 0 || j >= n)
		return -1;
	const uint32_t a = (uint32_t)k[i], b = (uint32_t)k[j];
	return (a != b) ? __clz(a ^ b) : 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

// Binary node gi: find its scene (int_off is non-decreasing), then Karras's
// construction on that scene's sorted leaves.  References are global: leaf positions
// are tri_off[s] + local, binary nodes int_off[s] + local.
template <typename K>
__global__ void k_karras(const K *__restrict__ keys, uint32_t n_int, const uint32_t *tri_off,
                         const uint32_t *int_off, uint32_t n_scenes, uint32_t *left,
                         uint32_t *right, uint32_t *parent_int, uint32_t *parent_leaf,
                         uint32_t *rfirst, uint32_t *rlast) {
	const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
	if (gi >= n_int)
		return;
	uint32_t lo_s = 0, hi_s = n_scenes; // last s with int_off[s] <= gi
	while (hi_s - lo_s > 1) {
		const uint32_t mid = (lo_s + hi_s) >> 1;
		if (int_off[mid] <= gi)
			lo_s = mid;
		else
			hi_s = mid;
	}
	const uint32_t s = lo_s;
	const uint32_t first = tri_off[s], ibase = int_off[s];
	const int n = (int)(tri_off[s + 1] - first);
	const int i = (int)(gi - ibase);
	const K *k = keys + first;
	const int d = kdelta(k, n, i, i + 1) > kdelta(k, n, i, i - 1) ? 1 : -1;
	const int dmin = kdelta(k, n, i, i - d);
	int lmax = 2;
	while (kdelta(k, n, i, i + lmax * d) > dmin)
		lmax <<= 1;
	int l = 0;
	for (int t = lmax >> 1; t >= 1; t >>= 1)
		if (kdelta(k, n, i, i + (l + t) * d) > dmin)
			l += t;
	const int j = i + l * d;
	const int dnode = kdelta(k, n, i, j);
	int sp = 0;
	for (int div = 2;; div <<= 1) {
		const int t = (l + div - 1) / div;
		if (kdelta(k, n, i, i + (sp + t) * d) > dnode)
			sp += t;
		if (t <= 1)
			break;
	}
	const int gamma = i + sp * d + min(d, 0);
	const int lo = min(i, j), hi = max(i, j);
	const bool lleaf = lo == gamma, rleaf = hi == gamma + 1;
	const uint32_t lc = lleaf ? (kLeafBit | (first + gamma)) : (ibase + gamma);
	const uint32_t rc = rleaf ? (kLeafBit | (first + gamma + 1)) : (ibase + gamma + 1);
	left[gi] = lc;
	right[gi] = rc;
	if (lleaf)
		parent_leaf[first + gamma] = gi;
	else
		parent_int[ibase + gamma] = gi;
	if (rleaf)
		parent_leaf[first + gamma + 1] = gi;
	else
		parent_int[ibase + gamma + 1] = gi;
	rfirst[gi] = first + lo;
	rlast[gi] = first + hi;
	if (i == 0)
		parent_int[gi] = kNone;
}

__global__ void k_leaf_boxes(const float *__restrict__ tris, const uint32_t *__restrict__ vals,
                             uint32_t n, float4 *lbox) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const float *t = tris + 9 * (size_t)vals[i];
	float4 lo, hi;
	if (tri_finite(t)) {
		lo = make_float4(fminf(t[0], fminf(t[3], t[6])), fminf(t[1], fminf(t[4], t[7])),
		                 fminf(t[2], fminf(t[5], t[8])), 0.0f);
		hi = make_float4(fmaxf(t[0], fmaxf(t[3], t[6])), fmaxf(t[1], fmaxf(t[4], t[7])),
		                 fmaxf(t[2], fmaxf(t[5], t[8])), 0.0f);
	} else {
		lo = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
		hi = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f);
	}
	lbox[2 * i] = lo;
	lbox[2 * i + 1] = hi;
}

// atomicAdd(p, 1) with acquire-release ordering at device scope.
__device__ __forceinline__ uint32_t arrive_acq_rel(uint32_t *p) {
	uint32_t old;
	asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
	return old;
}

__device__ __forceinline__ void child_box(uint32_t ref, const float4 *ibox, const float4 *lbox,
                                          float4 &lo, float4 &hi) {
	if (ref & kLeafBit) {
		uint32_t k = ref & ~kLeafBit;
		lo = __ldcg(&lbox[2 * k]);
		hi = __ldcg(&lbox[2 * k + 1]);
	} else {
		lo = __ldcg(&ibox[2 * ref]);
		hi = __ldcg(&ibox[2 * ref + 1]);
	}
}

// One thread per leaf walks towards its scene's root; at each binary node the first
// thread to arrive stops and the second, which then sees both children's boxes, writes
// the union and continues.  No thread waits on another.  A scene of one triangle has
// no binary node (parent_leaf stays kNone).  The unused w slots of a node's box carry
// the surface areas of its two children (-1 for a leaf child), which the collapse
// reads together with the child indices when it opens the node.
__global__ void k_refit(uint32_t n, uint32_t n_int, const uint32_t *__restrict__ parent_leaf,
                        const uint32_t *__restrict__ parent_int, const uint32_t *__restrict__ left,
                        const uint32_t *__restrict__ right, const float4 *lbox, float4 *ibox,
                        uint32_t *flags, uint32_t *err) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	uint32_t p = parent_leaf[i];
	// A path to the root passes each binary node once; a longer walk (or an index out
	// of range) means corrupt parents, reported instead of followed.
	for (uint32_t steps = 0; p != kNone; ++steps) {
		if (p >= n_int || steps >= n_int) {
			atomicOr(err, kErrCollapse);
			return;
		}
		// Release: the union this thread wrote one level down is visible before its
		// arrival counts.  Acquire: the sibling's union is read after its arrival.
		if (arrive_acq_rel(&flags[p]) == 0u)
			return;
		float4 alo, ahi, blo, bhi;
		const uint32_t l = left[p], r = right[p];
		child_box(l, ibox, lbox, alo, ahi);
		child_box(r, ibox, lbox, blo, bhi);
		const float al = (l & kLeafBit) ? -1.0f : half_area(alo, ahi);
		const float ar = (r & kLeafBit) ? -1.0f : half_area(blo, bhi);
		__stcg(&ibox[2 * p], make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y),
		                                 fminf(alo.z, blo.z), al));
		__stcg(&ibox[2 * p + 1], make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y),
		                                     fmaxf(ahi.z, bhi.z), ar));
		p = parent_int[p];
	}
}

// Costs of child `y` in j = 1..7 slots (cs[j]), in units of its own area; returns its
// half extents.
__device__ __forceinline__ float3 child_costs(uint32_t y, const CostNode *cost,
                                              const float4 *ibox, const float4 *lbox,
                                              float cs[8]) {
	if (y & kLeafBit) {
		const uint32_t k = y & ~kLeafBit;
		leaf_costs(cs);
		return half_extent(__ldcg(&lbox[2 * k]), __ldcg(&lbox[2 * k + 1]));
	}
	CostNode c;
	c.c1 = __ldcg(&cost[y].c1);
#pragma unroll
	for (int j = 0; j < 7; ++j)
		c.cd[j] = __ldcg(&cost[y].cd[j]);
	node_costs(c, cs);
	return half_extent(__ldcg(&ibox[2 * y]), __ldcg(&ibox[2 * y + 1]));
}

// One thread per leaf walks towards the root like k_refit; the second thread to arrive
// at a binary node computes its costs from both children's.
__global__ void k_collapse_cost(uint32_t n, uint32_t n_ids, const uint32_t *__restrict__ parent_leaf,
                                const uint32_t *__restrict__ parent_int,
                                const uint32_t *__restrict__ left, const uint32_t *__restrict__ right,
                                const uint32_t *__restrict__ rfirst,
                                const uint32_t *__restrict__ rlast, const float4 *__restrict__ ibox,
                                const float4 *__restrict__ lbox, uint32_t *flags, CostNode *cost,
                                uint32_t leaf_size, uint32_t *err) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	uint32_t p = parent_leaf[i];
	for (uint32_t steps = 0; p != kNone; ++steps) {
		if (p >= n_ids || steps >= n_ids) {
			atomicOr(err, kErrCollapse);
			return;
		}
		if (arrive_acq_rel(&flags[p]) == 0u)
			return;
		float cl[8], cr[8];
		const float3 el = child_costs(left[p], cost, ibox, lbox, cl);
		const float3 er = child_costs(right[p], cost, ibox, lbox, cr);
		const float3 ep = half_extent(__ldcg(&ibox[2 * p]), __ldcg(&ibox[2 * p + 1]));
		const CostNode c =
		    merge_costs(cl, cr, el, er, ep, rlast[p] - rfirst[p] + 1u, leaf_size);
		__stcg(&cost[p].c1, c.c1);
#pragma unroll
		for (int k = 0; k < 7; ++k)
			__stcg(&cost[p].cd[k], c.cd[k]);
		__stcg(&cost[p].bits, c.bits);
		p = parent_int[p];
	}
}

// Child slot `r` of an 8-wide node becomes an 8-wide node of its own (else a leaf).
__device__ __forceinline__ bool is_inner(uint32_t r, uint32_t count, uint32_t leaf_size,
                                         const CostNode *cost) {
	if (r & kLeafBit)
		return false;
	if (count > leaf_size)
		return true;
	return cost ? (__ldg(&cost[r].bits) >> 31) == 0u : false;
}

// Level-0 frontier: the root of every scene becomes 8-wide node s; the node counter
// starts after the roots.
__global__ void k_collapse_roots(const uint32_t *tri_off, const uint32_t *int_off,
                                 uint32_t n_scenes, Item *items, uint32_t *ctr) {
	const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
	if (s == 0) {
		ctr[0] = n_scenes;
		ctr[kCtrNodes] = n_scenes;
	}
	if (s >= n_scenes)
		return;
	const uint32_t n = tri_off[s + 1] - tri_off[s];
	const uint32_t ref = n == 0 ? kNone : (n == 1 ? (kLeafBit | tri_off[s]) : int_off[s]);
	items[s] = Item{ref, s};
}

__device__ __forceinline__ uint32_t bcount(uint32_t ref, const uint32_t *rfirst,
                                           const uint32_t *rlast) {
	return (ref & kLeafBit) ? 1u : (rlast[ref] - rfirst[ref] + 1u);
}

__device__ __forceinline__ uint32_t bfirst(uint32_t ref, const uint32_t *rfirst) {
	return (ref & kLeafBit) ? (ref & ~kLeafBit) : rfirst[ref];
}


__device__ __forceinline__ float open_area(uint32_t r, const float4 *__restrict__ ibox) {
	return (r & kLeafBit) ? -1.0f : half_area(ibox[2 * r], ibox[2 * r + 1]);
}

// Compare-exchange of two children by first leaf (registers only).
__device__ __forceinline__ void cx(uint32_t &ca, uint32_t &fa, uint32_t &na, uint32_t &cb,
                                   uint32_t &fb, uint32_t &nb) {
	if (fa > fb) {
		uint32_t t = ca; ca = cb; cb = t;
		t = fa; fa = fb; fb = t;
		t = na; na = nb; nb = t;
	}
}

// One level: each frontier item becomes an 8-wide node.  A warp takes 32 items; the
// node slots, triangle ranges and next-level items it needs are reserved with one
// atomic per counter per warp.
__global__ void __launch_bounds__(128)
    k_collapse(const Item *__restrict__ in, const uint32_t *in_count, Item *out,
               uint32_t *out_count, uint32_t *node_counter, uint32_t node_cap,
               uint32_t *tri_counter, Node8 *nodes, uint32_t *perm,
               const uint32_t *__restrict__ left, const uint32_t *__restrict__ right,
               const uint32_t *__restrict__ rfirst, const uint32_t *__restrict__ rlast,
               const float4 *__restrict__ ibox, const float4 *__restrict__ lbox,
               uint32_t leaf_size, uint32_t n_tris, const CostNode *__restrict__ cost,
               uint32_t *err) {
	const uint32_t n_in = *in_count;
	const uint32_t lane = threadIdx.x & 31u;
	for (uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < n_in;
	     w0 += gridDim.x * blockDim.x) {
		const uint32_t w = w0 + lane;
		const bool live = w < n_in;
		const Item it = live ? in[w] : Item{kNone, 0u};
		const bool empty_scene = live && it.ref == kNone;
		// Open the binary child of largest surface area until 8 children: any binary
		// node can be opened, so nodes fill up and small subtrees end as single
		// triangles (whose box is then tested exactly like the reference's leaf box).
		uint32_t C[8], F[8], N[8];
		float A[8];
#pragma unroll
		for (int c = 0; c < 8; ++c) {
			C[c] = kNone;
			A[c] = -1.0f;
		}
		int nc = 0;
		if (live && !empty_scene && cost && !(it.ref & kLeafBit)) {
			// Share out the 8 slots as the cost pass decided: a pending (subtree, slots)
			// entry is opened when splitting it is cheaper than keeping it whole.  The
			// shares of the pending entries add up to 8, so there are at most 8.
			uint32_t py[8], pi[8];
			const uint32_t a0 = split_of(cost[it.ref].bits, 8u);
			py[0] = right[it.ref];
			pi[0] = 8u - a0;
			py[1] = left[it.ref];
			pi[1] = a0;
			int top = 2;
			while (top > 0) {
				--top;
				const uint32_t y = py[top], i = pi[top];
				bool open = false;
				uint32_t a = 1;
				if (!(y & kLeafBit) && i > 1u) {
					open = cost[y].cd[i - 2u] < cost[y].c1;
					a = split_of(cost[y].bits, i);
				}
				if (open && top <= 6) {
					py[top] = right[y];
					pi[top] = i - a;
					py[top + 1] = left[y];
					pi[top + 1] = a;
					top += 2;
				} else {
#pragma unroll
					for (int c = 0; c < 8; ++c)
						if (c == nc)
							C[c] = y;
					nc = min(nc + 1, 8);
				}
			}
		} else if (live && !empty_scene) {
			C[0] = it.ref;
			A[0] = open_area(it.ref, ibox);
			nc = 1;
			while (nc < 8) {
				int best = -1;
				float best_area = -1.0f;
#pragma unroll
				for (int c = 0; c < 8; ++c)
					if (c < nc && A[c] > best_area) {
						best_area = A[c];
						best = c;
					}
				if (best < 0)
					break;
				uint32_t x = 0;
#pragma unroll
				for (int c = 0; c < 8; ++c)
					if (c == best)
						x = C[c];
				// Children and their areas (stored by the refit) in one round of loads.
				const uint32_t l = left[x], r = right[x];
				const float al = ibox[2 * x].w, ar = ibox[2 * x + 1].w;
#pragma unroll
				for (int c = 0; c < 8; ++c) {
					if (c == best) {
						C[c] = l;
						A[c] = al;
					}
					if (c == nc) {
						C[c] = r;
						A[c] = ar;
					}
				}
				++nc;
			}
		}
		// First leaf and triangle count of each child; unused slots sort last.  Children
		// are ordered by first leaf, so a node's leaf triangles keep the Morton order
		// (first leaves of distinct children differ, so the order is unique).
		uint32_t n_inner = 0, n_leaf_tris = 0;
#pragma unroll
		for (int c = 0; c < 8; ++c) {
			if (c < nc) {
				F[c] = bfirst(C[c], rfirst);
				N[c] = bcount(C[c], rfirst, rlast);
				if (is_inner(C[c], N[c], leaf_size, cost))
					++n_inner;
				else
					n_leaf_tris += N[c];
			} else {
				F[c] = 0xFFFFFFFFu;
				N[c] = 0;
			}
		}
		cx(C[0], F[0], N[0], C[2], F[2], N[2]);
		cx(C[1], F[1], N[1], C[3], F[3], N[3]);
		cx(C[4], F[4], N[4], C[6], F[6], N[6]);
		cx(C[5], F[5], N[5], C[7], F[7], N[7]);
		cx(C[0], F[0], N[0], C[4], F[4], N[4]);
		cx(C[1], F[1], N[1], C[5], F[5], N[5]);
		cx(C[2], F[2], N[2], C[6], F[6], N[6]);
		cx(C[3], F[3], N[3], C[7], F[7], N[7]);
		cx(C[0], F[0], N[0], C[1], F[1], N[1]);
		cx(C[2], F[2], N[2], C[3], F[3], N[3]);
		cx(C[4], F[4], N[4], C[5], F[5], N[5]);
		cx(C[6], F[6], N[6], C[7], F[7], N[7]);
		cx(C[2], F[2], N[2], C[4], F[4], N[4]);
		cx(C[3], F[3], N[3], C[5], F[5], N[5]);
		cx(C[1], F[1], N[1], C[4], F[4], N[4]);
		cx(C[3], F[3], N[3], C[6], F[6], N[6]);
		cx(C[1], F[1], N[1], C[2], F[2], N[2]);
		cx(C[3], F[3], N[3], C[4], F[4], N[4]);
		cx(C[5], F[5], N[5], C[6], F[6], N[6]);
		// Warp-wide reservation: exclusive prefix sums of the lanes' needs.
		uint32_t inc_i = n_inner, inc_t = n_leaf_tris;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t vi = __shfl_up_sync(0xFFFFFFFFu, inc_i, o);
			const uint32_t vt = __shfl_up_sync(0xFFFFFFFFu, inc_t, o);
			if (lane >= (uint32_t)o) {
				inc_i += vi;
				inc_t += vt;
			}
		}
		const uint32_t tot_i = __shfl_sync(0xFFFFFFFFu, inc_i, 31);
		const uint32_t tot_t = __shfl_sync(0xFFFFFFFFu, inc_t, 31);
		uint32_t nb = 0, tb = 0, ob = 0;
		if (lane == 31) {
			nb = tot_i ? atomicAdd(node_counter, tot_i) : 0u;
			tb = tot_t ? atomicAdd(tri_counter, tot_t) : 0u;
			ob = tot_i ? atomicAdd(out_count, tot_i) : 0u;
		}
		nb = __shfl_sync(0xFFFFFFFFu, nb, 31);
		tb = __shfl_sync(0xFFFFFFFFu, tb, 31);
		ob = __shfl_sync(0xFFFFFFFFu, ob, 31);
		if (nb + tot_i > node_cap || tb + tot_t > n_tris) {
			if (lane == 0)
				atomicOr(err, kErrCollapse);
			continue;
		}
		if (!live)
			continue;
		Node8 *nd = nodes + it.slot;
		if (empty_scene) { // a node without children
			for (int c = 0; c < 8; ++c) {
				Child8 ch;
				ch.lo_x = ch.lo_y = ch.lo_z = __int_as_float(0x7FC00000);
				ch.hi_x = ch.hi_y = ch.hi_z = __int_as_float(0x7FC00000);
				ch.ref = kNone;
				ch.pad = 0u;
				nd->c[c] = ch;
			}
			continue;
		}
		const uint32_t base = nb + inc_i - n_inner, obase = ob + inc_i - n_inner;
		uint32_t dst = tb + inc_t - n_leaf_tris;
		uint32_t k_inner = 0;
#pragma unroll
		for (int c = 0; c < 8; ++c) {
			// An unused slot gets a NaN box: no slab test passes it.
			float4 lo = make_float4(__int_as_float(0x7FC00000), __int_as_float(0x7FC00000),
			                        __int_as_float(0x7FC00000), 0.f),
			       hi = lo;
			uint32_t ref = kNone;
			if (c < nc) {
				const uint32_t r = C[c];
				if (r & kLeafBit) {
					const uint32_t k = r & ~kLeafBit;
					lo = lbox[2 * k];
					hi = lbox[2 * k + 1];
				} else {
					lo = ibox[2 * r];
					hi = ibox[2 * r + 1];
				}
				if (is_inner(r, N[c], leaf_size, cost)) {
					ref = base + k_inner;
					out[obase + k_inner] = Item{r, ref};
					++k_inner;
				} else {
					for (uint32_t k = 0; k < N[c]; ++k)
						perm[dst + k] = F[c] + k;
					ref = make_leaf(dst, N[c]);
					dst += N[c];
				}
			}
			Child8 ch;
			ch.lo_x = lo.x;
			ch.lo_y = lo.y;
			ch.lo_z = lo.z;
			ch.ref = ref;
			ch.hi_x = hi.x;
			ch.hi_y = hi.y;
			ch.hi_z = hi.z;
			ch.pad = 0u;
			nd->c[c] = ch;
		}
	}
}

// Triangle records in leaf order; tri4.w holds the per-scene primitive id and inv maps
// a global input index to its leaf-order position.
__global__ void k_relayout(const float *__restrict__ tris, const uint32_t *__restrict__ vals,
                           const uint32_t *__restrict__ perm, const uint32_t *__restrict__ scene_of,
                           const uint32_t *__restrict__ tri_off, uint32_t n, float4 *tri4,
                           uint32_t *inv) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const uint32_t g = vals[perm[i]];
	const uint32_t pid = g - tri_off[scene_at(scene_of, g)];
	inv[g] = i;
	const float *t = tris + 9 * (size_t)g;
	tri4[3 * (size_t)i] = make_float4(t[0], t[1], t[2], __uint_as_float(pid));
	tri4[3 * (size_t)i + 1] = make_float4(t[3], t[4], t[5], tri_finite(t) ? 0.0f : 1.0f);
	tri4[3 * (size_t)i + 2] = make_float4(t[6], t[7], t[8], 0.0f);
}

__device__ __forceinline__ float cdec(float o, uint32_t q, float s) { return cdec_f(o, (float)q, s); }

// Largest q in [0, 255] whose decoded value is <= v (decoding is monotone in q and
// q = 0 decodes to the origin, which is <= every child bound).  The estimate comes from
// a directed-rounding FP32 quotient; the loops make the answer exact, so it does not
// depend on the estimate.
__device__ uint32_t quant_lo(float o, float s, float v) {
	const float g = floorf(__fdiv_rd(__fsub_rd(v, o), s));
	uint32_t q = (uint32_t)fminf(fmaxf(g, 0.0f), 255.0f);
	while (q > 0 && cdec(o, q, s) > v)
		--q;
	while (q < 255 && cdec(o, q + 1, s) <= v)
		++q;
	return q;
}

// Smallest q in [0, 255] whose decoded value is >= v (the exponent was chosen so that
// q = 255 qualifies).
__device__ uint32_t quant_hi(float o, float s, float v) {
	const float g = ceilf(__fdiv_ru(__fsub_ru(v, o), s));
	uint32_t q = (uint32_t)fminf(fmaxf(g, 0.0f), 255.0f);
	while (q < 255 && cdec(o, q, s) < v)
		++q;
	while (q > 0 && cdec(o, q - 1, s) >= v)
		--q;
	return q;
}

// Smallest biased exponent e in [1, 254] with o + 255 * 2^(e-127) >= mx in FP32 (254
// when none is; the traversal then still tests the children exactly at the leaves).
// The start is at most the answer: the FP32 range rounded up, over 255 rounded up, has
// an exponent at least that of the answer's scale less two.
__device__ uint32_t scale_exponent(float mn, float mx) {
	const float r = __fdiv_ru(__fsub_ru(mx, mn), 255.0f);
	int e = 254;
	if (isfinite(r)) {
		const uint32_t bits = __float_as_uint(r);
		const int e0 = (int)((bits >> 23) & 0xFFu) + ((bits & 0x7FFFFFu) ? 1 : 0);
		e = max(1, min(254, e0 - 2));
	}
	while (e < 254 && cdec(mn, 255u, cscale((uint8_t)e)) < mx)
		++e;
	return (uint32_t)e;
}

// Eight lanes per node, lane k on child k: reads and writes are contiguous per node.
// n_nodes_dev (when not null) holds the node count on the device: a build queued
// without host round-trips launches this kernel over the node capacity.
__global__ void __launch_bounds__(256)
    k_compress(const Node8 *__restrict__ nodes, uint32_t n_nodes, const uint32_t *n_nodes_dev,
               CNode8 *cn) {
	const uint32_t k = threadIdx.x & 7u;
	const uint32_t i = blockIdx.x * (blockDim.x / 8u) + threadIdx.x / 8u;
	const uint32_t n = n_nodes_dev ? *n_nodes_dev : n_nodes;
	const bool live = i < n;
	// Groups of 8 lanes never straddle the node range, but the warp does: every lane
	// takes part in the shuffles, idle ones with an empty child.
	const unsigned gmask = 0xFFu << (threadIdx.x & 24u);
	Child8 ch;
	if (live) {
		const float4 *src = reinterpret_cast<const float4 *>(&nodes[i].c[k]);
		const float4 a = __ldg(src), b = __ldg(src + 1);
		ch.lo_x = a.x;
		ch.lo_y = a.y;
		ch.lo_z = a.z;
		ch.ref = __float_as_uint(a.w);
		ch.hi_x = b.x;
		ch.hi_y = b.y;
		ch.hi_z = b.z;
	} else {
		ch.ref = kNone;
		ch.lo_x = ch.lo_y = ch.lo_z = ch.hi_x = ch.hi_y = ch.hi_z = 0.0f;
	}
	const uint32_t r = ch.ref;
	const bool used = r != kNone;
	const bool leaf = used && (r & kLeafBit);
	uint32_t cb = (used && !leaf) ? r : kNone;
	uint32_t tb = leaf ? leaf_first(r) : kNone;
	float lo[3] = {ch.lo_x, ch.lo_y, ch.lo_z}, hi[3] = {ch.hi_x, ch.hi_y, ch.hi_z};
	float mn[3], mx[3];
	for (int a = 0; a < 3; ++a) {
		mn[a] = used ? lo[a] : INFINITY;
		mx[a] = used ? hi[a] : -INFINITY;
	}
	for (int o = 4; o > 0; o >>= 1) {
		cb = min(cb, __shfl_xor_sync(gmask, cb, o, 8));
		tb = min(tb, __shfl_xor_sync(gmask, tb, o, 8));
		for (int a = 0; a < 3; ++a) {
			mn[a] = fminf(mn[a], __shfl_xor_sync(gmask, mn[a], o, 8));
			mx[a] = fmaxf(mx[a], __shfl_xor_sync(gmask, mx[a], o, 8));
		}
	}
	const uint32_t imask = (__ballot_sync(gmask, used && !leaf) >> (threadIdx.x & 24u)) & 0xFFu;
	if (!live)
		return;
	float org[3];
	uint32_t ex[3];
	for (int a = 0; a < 3; ++a) {
		if (!(mn[a] <= mx[a])) { // no children: an empty frame at the origin
			mn[a] = 0.0f;
			mx[a] = 0.0f;
		}
		org[a] = mn[a];
		ex[a] = scale_exponent(mn[a], mx[a]);
	}
	const uint32_t tri_base = tb == kNone ? 0u : tb;
	CChild8 c;
	c.qlo_x = c.qhi_x = c.qlo_y = c.qhi_y = c.qlo_z = c.qhi_z = 0;
	c.count = 0;
	c.first = 0;
	if (used) {
		uint8_t q[6];
		for (int a = 0; a < 3; ++a) {
			const float sc = cscale((uint8_t)ex[a]);
			q[2 * a] = (uint8_t)quant_lo(org[a], sc, lo[a]);
			q[2 * a + 1] = (uint8_t)quant_hi(org[a], sc, hi[a]);
		}
		c.qlo_x = q[0];
		c.qhi_x = q[1];
		c.qlo_y = q[2];
		c.qhi_y = q[3];
		c.qlo_z = q[4];
		c.qhi_z = q[5];
		if (leaf) {
			c.count = (uint8_t)leaf_count(r);
			c.first = (uint8_t)(leaf_first(r) - tri_base);
		}
	}
	cn[i].c[k] = c;
	if (k == 0) { // the 32-byte header as two 16-byte stores (ex, ey, ez, imask: bytes 12-15)
		uint4 *h = reinterpret_cast<uint4 *>(&cn[i]);
		h[0] = make_uint4(__float_as_uint(org[0]), __float_as_uint(org[1]),
		                  __float_as_uint(org[2]),
		                  ex[0] | (ex[1] << 8) | (ex[2] << 16) | (imask << 24));
		h[1] = make_uint4(cb == kNone ? 0u : cb, tri_base, 0u, 0u);
	}
}
static_assert(offsetof(CNode8, ex) == 12 && offsetof(CNode8, imask) == 15 &&
                  offsetof(CNode8, child_base) == 16 && offsetof(CNode8, tri_base) == 20 &&
                  offsetof(CNode8, c) == 32,
              "CNode8 header layout");

#define BUILD_TRY(call)                                                                        \
	do {                                                                                       \
		cudaError_t e_ = (call);                                                               \
		if (e_ != cudaSuccess) {                                                               \
			msg = std::string("CUDA error in build: ") + cudaGetErrorString(e_) + " (" #call ")"; \
			return e_ == cudaErrorMemoryAllocation ? PRT_ERR_OOM : PRT_ERR_CUDA;              \
		}                                                                                      \
	} while (0)

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

} // namespace

int build_plan(const uint64_t *tri_off64, uint32_t S, int leaf_size, bool compressed,
               SceneGPU &sc, BuildScratch &ws, cudaStream_t st, BuildPlan &plan,
               std::string &msg, bool sah, bool collapse_cost, bool one_block) {
	if (leaf_size < 1 || leaf_size > kMaxLeaf) {
		msg = "leaf_size must be in [1, 8]";
		return PRT_ERR_ARG;
	}
	if (S == 0 || !tri_off64 || tri_off64[0] != 0) {
		msg = "build: at least one scene, offsets starting at 0";
		return PRT_ERR_ARG;
	}
	for (uint32_t s = 0; s < S; ++s) {
		if (tri_off64[s + 1] < tri_off64[s]) {
			msg = "build: triangle offsets must not decrease";
			return PRT_ERR_ARG;
		}
	}
	const uint64_t n64 = tri_off64[S];
	if (n64 > kMaxTris) {
		msg = "set_tris: at most 134217727 triangles per scene";
		return PRT_ERR_LIMIT;
	}
	plan.S = S;
	plan.n = (uint32_t)n64;
	plan.leaf_size = leaf_size;
	plan.compressed = compressed;
	plan.multi = S > 1;
	plan.sah = sah;
	plan.collapse_cost = collapse_cost;
	plan.small = one_block && sah && S == 1 && n64 >= 1 && n64 <= small_build_max();
	plan.toff.resize(S + 1);
	plan.ioff.resize(S + 1);
	for (uint32_t s = 0; s <= S; ++s)
		plan.toff[s] = (uint32_t)tri_off64[s];
	plan.n_int = 0;
	for (uint32_t s = 0; s <= S; ++s) {
		plan.ioff[s] = plan.n_int;
		if (s < S) {
			const uint32_t ns = plan.toff[s + 1] - plan.toff[s];
			plan.n_int += ns > 1 ? ns - 1 : 0;
		}
	}
	if (plan.n_int >= std::max<uint32_t>(plan.toff[S], 1u)) {
		msg = "build: inconsistent scene offsets";
		return PRT_ERR_ARG;
	}
	plan.scene_digits = 0;
	for (uint32_t v = S - 1; v; v >>= 8)
		++plan.scene_digits;
	const uint32_t n = plan.n;
	plan.node_cap = n + S;

	sc.n_scenes = S;
	sc.n_tris = n;
	sc.leaf_size = leaf_size;
	sc.n_nodes = 0;
	sc.depth = 0;
	sc.has_cnodes = false;
	sc.built_small = false;
	sc.h_tri_off.assign(tri_off64, tri_off64 + S + 1);

	const size_t key_bytes = plan.multi ? 8 : 4;
	// SAH node ids run up to n_int + S (scene s's root is node s).
	const size_t ni = std::max<size_t>((size_t)plan.n_int + (sah ? S : 0u), 1);
	const size_t nn = std::max<uint32_t>(n, 1);
	BUILD_TRY(sc.tri_off.reserve(4ull * (S + 1)));
	BUILD_TRY(ws.keys.reserve(key_bytes * nn));
	BUILD_TRY(ws.keys2.reserve(key_bytes * nn));
	BUILD_TRY(ws.vals.reserve(4 * nn));
	BUILD_TRY(ws.vals2.reserve(4 * nn));
	if (plan.multi)
		BUILD_TRY(ws.scene_of.reserve(4 * nn));
	BUILD_TRY(ws.int_off.reserve(4ull * (S + 1)));
	BUILD_TRY(ws.left.reserve(4 * ni));
	BUILD_TRY(ws.right.reserve(4 * ni));
	BUILD_TRY(ws.parent_int.reserve(4 * ni));
	BUILD_TRY(ws.parent_leaf.reserve(4 * nn));
	BUILD_TRY(ws.rfirst.reserve(4 * ni));
	BUILD_TRY(ws.rlast.reserve(4 * ni));
	BUILD_TRY(ws.flags.reserve(4 * ni));
	BUILD_TRY(ws.ibox.reserve(32 * ni));
	BUILD_TRY(ws.lbox.reserve(32 * nn));
	BUILD_TRY(ws.items_a.reserve(8ull * plan.node_cap));
	BUILD_TRY(ws.items_b.reserve(8ull * plan.node_cap));
	BUILD_TRY(ws.counters.reserve(4 * kCtrWords));
	BUILD_TRY(ws.perm.reserve(4 * nn));
	BUILD_TRY(ws.sort_hist.reserve(8 * 256 * 4));
	BUILD_TRY(ws.sort_tiles.reserve(8 * 4));
	BUILD_TRY(ws.sort_status.reserve(4 * sort_status_words(n)));
	BUILD_TRY(ws.bounds.reserve(24ull * S));
	if (sah && !plan.small) {
		BUILD_TRY(ws.sah.reserve(sah_scratch_bytes(n, S)));
		BUILD_TRY(ws.roots.reserve(4ull * S));
	}
	if (collapse_cost)
		BUILD_TRY(ws.cost.reserve(sizeof(CostNode) * ni));
	BUILD_TRY(sc.tri4.reserve(48 * nn));
	BUILD_TRY(sc.inv.reserve(4 * nn));
	// One node past the capacity: the empty node the traversal pads partial steps with.
	BUILD_TRY(sc.nodes.reserve(sizeof(Node8) * ((size_t)plan.node_cap + 1)));
	if (compressed)
		BUILD_TRY(sc.cnodes.reserve(sizeof(CNode8) * ((size_t)plan.node_cap + 1)));
	// Work items hold 27-bit node indices; a tree's nodes stay below n - 1 < 2^27 - 1.
	sc.dead = std::min<uint32_t>(plan.node_cap, kIndexMask);
	if (!ws.h_counters)
		BUILD_TRY(cudaMallocHost(&ws.h_counters, 4 * (kCtrWords + kHostSahWords)));
	ws.h_sah = ws.h_counters + kCtrWords;
	if (plan.small)
		return PRT_OK; // the one-block build reads no offset table
	BUILD_TRY(cudaMemcpyAsync(sc.tri_off.p, plan.toff.data(), 4ull * (S + 1),
	                          cudaMemcpyHostToDevice, st));
	BUILD_TRY(cudaMemcpyAsync(ws.int_off.p, plan.ioff.data(), 4ull * (S + 1),
	                          cudaMemcpyHostToDevice, st));
	return PRT_OK;
}

// Morton codes, radix sort, Karras hierarchy and refit: the binary trees of the LBVH
// path, with svals set to the sorted triangle order.
static int lbvh_enqueue(const float *d_tris, const BuildPlan &plan, BuildScratch &ws,
                        const uint32_t *d_toff, const uint32_t *d_ioff, const uint32_t *scene_of,
                        cudaStream_t st, uint32_t *d_err, const uint32_t *&svals, std::string &msg) {
	const uint32_t S = plan.S, n = plan.n, n_int = plan.n_int;
	const size_t ni = std::max<uint32_t>(n_int, 1);
	const size_t nn = std::max<uint32_t>(n, 1);
	uint32_t *gb = ws.bounds.as<uint32_t>();
	svals = ws.vals.as<uint32_t>();
	k_bounds_init<<<blocks_for(6ull * S, 256), 256, 0, st>>>(gb, S);
	if (n)
		k_centroid_bounds<<<std::min(blocks_for(n, 256), 2048u), 256, 0, st>>>(d_tris, n, scene_of,
		                                                                        gb);
	SortScratch ss{ws.sort_hist.as<uint32_t>(), ws.sort_tiles.as<uint32_t>(),
	               ws.sort_status.as<uint32_t>()};
	const void *skeys = ws.keys.p;
	if (n && !plan.multi) {
		k_morton<uint32_t><<<blocks_for(n, 256), 256, 0, st>>>(d_tris, n, nullptr, gb,
		                                                       ws.keys.as<uint32_t>(),
		                                                       ws.vals.as<uint32_t>());
		int where = sort_pairs_u32(ws.keys.as<uint32_t>(), ws.vals.as<uint32_t>(),
		                           ws.keys2.as<uint32_t>(), ws.vals2.as<uint32_t>(), n, 4, ss, st,
		                           d_err);
		skeys = where ? ws.keys2.p : ws.keys.p;
		svals = where ? ws.vals2.as<uint32_t>() : ws.vals.as<uint32_t>();
	} else if (n) {
		k_morton<uint64_t><<<blocks_for(n, 256), 256, 0, st>>>(d_tris, n, scene_of, gb,
		                                                       ws.keys.as<uint64_t>(),
		                                                       ws.vals.as<uint32_t>());
		int where = sort_pairs_u64(ws.keys.as<uint64_t>(), ws.vals.as<uint32_t>(),
		                           ws.keys2.as<uint64_t>(), ws.vals2.as<uint32_t>(), n,
		                           4 + plan.scene_digits, ss, st, d_err);
		skeys = where ? ws.keys2.p : ws.keys.p;
		svals = where ? ws.vals2.as<uint32_t>() : ws.vals.as<uint32_t>();
	}

	BUILD_TRY(cudaMemsetAsync(ws.parent_leaf.p, 0xFF, 4 * nn, st));
	if (n_int) {
		if (plan.multi)
			k_karras<uint64_t><<<blocks_for(n_int, 256), 256, 0, st>>>(
			    static_cast<const uint64_t *>(skeys), n_int, d_toff, d_ioff, S,
			    ws.left.as<uint32_t>(), ws.right.as<uint32_t>(), ws.parent_int.as<uint32_t>(),
			    ws.parent_leaf.as<uint32_t>(), ws.rfirst.as<uint32_t>(), ws.rlast.as<uint32_t>());
		else
			k_karras<uint32_t><<<blocks_for(n_int, 256), 256, 0, st>>>(
			    static_cast<const uint32_t *>(skeys), n_int, d_toff, d_ioff, S,
			    ws.left.as<uint32_t>(), ws.right.as<uint32_t>(), ws.parent_int.as<uint32_t>(),
			    ws.parent_leaf.as<uint32_t>(), ws.rfirst.as<uint32_t>(), ws.rlast.as<uint32_t>());
		BUILD_TRY(cudaMemsetAsync(ws.flags.p, 0, 4 * ni, st));
	}
	if (n) {
		k_leaf_boxes<<<blocks_for(n, 256), 256, 0, st>>>(d_tris, svals, n, ws.lbox.as<float4>());
		if (n_int)
			k_refit<<<blocks_for(n, 256), 256, 0, st>>>(
			    n, n_int, ws.parent_leaf.as<uint32_t>(), ws.parent_int.as<uint32_t>(),
			    ws.left.as<uint32_t>(), ws.right.as<uint32_t>(), ws.lbox.as<float4>(),
			    ws.ibox.as<float4>(), ws.flags.as<uint32_t>(), d_err);
	}
	return PRT_OK;
}

// The empty node at index sc.dead (node_cap, past every built node): eight NaN boxes with no reference (no slab test
// passes them, and the general test skips a child without reference); compressed, a
// node with no inner mask and no leaf counts.  Queued on the build's stream, so a batch
// graph captures it with the build.
static cudaError_t write_dead_node(const BuildPlan &plan, SceneGPU &sc, cudaStream_t st) {
	cudaError_t e = cudaMemsetAsync(static_cast<char *>(sc.nodes.p) +
	                                    sizeof(Node8) * (size_t)sc.dead,
	                                0xFF, sizeof(Node8), st);
	if (e == cudaSuccess && plan.compressed)
		e = cudaMemsetAsync(static_cast<char *>(sc.cnodes.p) + sizeof(CNode8) * (size_t)sc.dead,
		                    0, sizeof(CNode8), st);
	return e;
}

int build_enqueue(const float *d_tris, const BuildPlan &plan, SceneGPU &sc, BuildScratch &ws,
                  cudaStream_t st, uint32_t *d_err, bool host_checks, std::string &msg) {
	const uint32_t S = plan.S, n = plan.n, n_int = plan.n_int;
	if (plan.sah && !host_checks) {
		msg = "the SAH build reads its level counters on the host";
		return PRT_ERR_ARG;
	}
	if (plan.small) {
		// One block: PLOC, collapse and re-layout in one launch, which also zeroes the
		// counters, writes the empty node and leaves the counters in the pinned host
		// buffer; the compression reads the node count on the device, so the host only
		// waits, once, at the end.
		uint32_t *ctr = ws.counters.as<uint32_t>();
		BUILD_TRY(launch_build_small(d_tris, n, (uint32_t)plan.leaf_size, plan.collapse_cost,
		                             plan.compressed, ws, sc, plan.node_cap, ctr, ws.h_counters,
		                             d_err, st));
		sc.built_small = true;
		if (plan.compressed) {
			k_compress<<<blocks_for(8ull * plan.node_cap, 256), 256, 0, st>>>(
			    sc.nodes.as<Node8>(), plan.node_cap, ctr + kCtrNodes, sc.cnodes.as<CNode8>());
			sc.has_cnodes = true;
		}
		BUILD_TRY(cudaGetLastError());
		return host_checks ? build_finish(sc, ws, st, msg, true) : PRT_OK;
	}
	BUILD_TRY(write_dead_node(plan, sc, st));
	uint32_t *d_toff = sc.tri_off.as<uint32_t>();
	uint32_t *d_ioff = ws.int_off.as<uint32_t>();
	uint32_t *scene_of = plan.multi ? ws.scene_of.as<uint32_t>() : nullptr;
	if (plan.multi)
		k_scene_of<<<std::min(S, 4096u), 256, 0, st>>>(d_toff, S, scene_of);
	const uint32_t *svals = ws.vals.as<uint32_t>();
	const uint32_t *roots = d_ioff;
	if (plan.sah) {
		int rc = sah_build_enqueue(d_tris, plan, ws, d_toff, scene_of, st, d_err, msg);
		if (rc != PRT_OK)
			return rc;
		roots = ws.roots.as<uint32_t>();
	} else {
		int rc = lbvh_enqueue(d_tris, plan, ws, d_toff, d_ioff, scene_of, st, d_err, svals, msg);
		if (rc != PRT_OK)
			return rc;
	}
	// Binary node ids run up to n_int (LBVH) or n_int + S (SAH: scene s's root is s).
	const uint32_t n_ids = n_int + (plan.sah ? S : 0u);
	const CostNode *cost = nullptr;
	if (plan.collapse_cost && n_int) {
		BUILD_TRY(cudaMemsetAsync(ws.flags.p, 0, 4ull * n_ids, st));
		k_collapse_cost<<<blocks_for(n, 256), 256, 0, st>>>(
		    n, n_ids, ws.parent_leaf.as<uint32_t>(), ws.parent_int.as<uint32_t>(),
		    ws.left.as<uint32_t>(), ws.right.as<uint32_t>(), ws.rfirst.as<uint32_t>(),
		    ws.rlast.as<uint32_t>(), ws.ibox.as<float4>(), ws.lbox.as<float4>(),
		    ws.flags.as<uint32_t>(), ws.cost.as<CostNode>(), (uint32_t)plan.leaf_size, d_err);
		cost = ws.cost.as<CostNode>();
	}

	uint32_t *ctr = ws.counters.as<uint32_t>();
	BUILD_TRY(cudaMemsetAsync(ctr, 0, 4 * kCtrWords, st));
	Item *items[2] = {ws.items_a.as<Item>(), ws.items_b.as<Item>()};
	k_collapse_roots<<<blocks_for(S, 128), 128, 0, st>>>(d_toff, roots, S, items[0], ctr);
	int level = 0;
	for (;;) {
		for (int k = 0; (host_checks ? k < kLevelsPerCheck : true) && level < kMaxLevels;
		     ++k, ++level)
			k_collapse<<<1216, 128, 0, st>>>(
			    items[level & 1], ctr + level, items[(level + 1) & 1], ctr + level + 1,
			    ctr + kCtrNodes, plan.node_cap, ctr + kCtrTris, sc.nodes.as<Node8>(),
			    ws.perm.as<uint32_t>(), ws.left.as<uint32_t>(), ws.right.as<uint32_t>(),
			    ws.rfirst.as<uint32_t>(), ws.rlast.as<uint32_t>(), ws.ibox.as<float4>(),
			    ws.lbox.as<float4>(), (uint32_t)plan.leaf_size, n, cost, d_err);
		if (!host_checks)
			break;
		BUILD_TRY(cudaMemcpyAsync(ws.h_counters, ctr, 4 * kCtrWords, cudaMemcpyDeviceToHost, st));
		BUILD_TRY(cudaStreamSynchronize(st));
		if (ws.h_counters[level] == 0)
			break;
		if (level >= kMaxLevels) {
			msg = "tree deeper than " + std::to_string(kMaxLevels) + " levels";
			return PRT_ERR_LIMIT;
		}
	}
	if (n)
		k_relayout<<<blocks_for(n, 256), 256, 0, st>>>(d_tris, svals, ws.perm.as<uint32_t>(),
		                                               scene_of, d_toff, n, sc.tri4.as<float4>(),
		                                               sc.inv.as<uint32_t>());
	if (host_checks) {
		int rc = build_finish(sc, ws, st, msg);
		if (rc != PRT_OK)
			return rc;
	}
	if (plan.compressed) {
		if (host_checks)
			k_compress<<<blocks_for(8ull * sc.n_nodes, 256), 256, 0, st>>>(
			    sc.nodes.as<Node8>(), sc.n_nodes, nullptr, sc.cnodes.as<CNode8>());
		else
			k_compress<<<blocks_for(8ull * plan.node_cap, 256), 256, 0, st>>>(
			    sc.nodes.as<Node8>(), plan.node_cap, ctr + kCtrNodes, sc.cnodes.as<CNode8>());
		sc.has_cnodes = true;
	}
	BUILD_TRY(cudaGetLastError());
	if (host_checks)
		BUILD_TRY(cudaStreamSynchronize(st));
	return PRT_OK;
}

int build_finish(SceneGPU &sc, BuildScratch &ws, cudaStream_t st, std::string &msg,
                 bool on_host) {
	if (!on_host)
		BUILD_TRY(cudaMemcpyAsync(ws.h_counters, ws.counters.p, 4 * kCtrWords,
		                          cudaMemcpyDeviceToHost, st));
	BUILD_TRY(cudaStreamSynchronize(st));
	uint32_t depth = 0;
	while (depth < (uint32_t)kMaxLevels && ws.h_counters[depth])
		++depth;
	if (depth == (uint32_t)kMaxLevels && ws.h_counters[kMaxLevels]) {
		msg = "tree deeper than " + std::to_string(kMaxLevels) + " levels";
		return PRT_ERR_LIMIT;
	}
	sc.n_nodes = ws.h_counters[kCtrNodes];
	sc.depth = depth;
	if (ws.h_counters[kCtrTris] != sc.n_tris) {
		msg = "collapse placed " + std::to_string(ws.h_counters[kCtrTris]) + " of " +
		      std::to_string(sc.n_tris) + " triangles";
		return PRT_ERR_DEVICE;
	}
	return PRT_OK;
}

int build_scenes(const float *d_tris, const uint64_t *tri_off, uint32_t n_scenes, int leaf_size,
                 bool compressed, SceneGPU &sc, BuildScratch &ws, cudaStream_t st,
                 uint32_t *d_err, std::string &msg, bool sah, bool collapse_cost,
                 bool one_block) {
	BuildPlan plan;
	int rc = build_plan(tri_off, n_scenes, leaf_size, compressed, sc, ws, st, plan, msg, sah,
	                    collapse_cost, one_block);
	if (rc != PRT_OK)
		return rc;
	return build_enqueue(d_tris, plan, sc, ws, st, d_err, true, msg);
}

int build_scene(const float *d_tris, uint64_t n, int leaf_size, bool compressed, SceneGPU &sc,
                BuildScratch &ws, cudaStream_t st, uint32_t *d_err, std::string &msg, bool sah,
                bool collapse_cost, bool one_block) {
	const uint64_t off[2] = {0, n};
	return build_scenes(d_tris, off, 1, leaf_size, compressed, sc, ws, st, d_err, msg, sah,
	                    collapse_cost, one_block);
}

} // namespace prt
