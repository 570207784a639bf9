// prt_build_small.cu - a scene of at most 4,096 triangles built by one thread block.
//
// Replaces, for small scenes, the chain of about 57 dependent launches of the binned-SAH
// build (each level's kernels wait on global memory; at this size the build is latency,
// not work) with one launch whose dependencies go through shared memory:
//   1. one pass over the triangles (boxes into shared memory and to the leaf-box array,
//      centroid bounds), 30-bit Morton codes (as k_morton makes them), a bitonic sort of
//      (code, index) in shared memory;
//   2. PLOC (Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding
//      Volume Hierarchy Construction", 2018): the clusters in Morton order each find
//      the cluster within kRadius (3) positions whose union with it has the least surface
//      area; mutual nearest neighbours merge into a binary node; the survivors are
//      compacted in order (staged in free rows); repeated until one cluster is left.
//      Candidates are ordered by (area, distance in Morton order, parity of the lower
//      position, lower position): a total order on pairs, so the least pair of an
//      iteration is mutual and every iteration merges at least one; equal clusters pair
//      up as (2k, 2k + 1) instead of one pair at a time.  After kPlocRounds iterations
//      (scenes whose clusters keep choosing one neighbour, such as exponentially spaced
//      triangles) positions 2k and 2k + 1 merge regardless, which bounds the iterations
//      and the depth by kPlocRounds + log2(n).  An iteration's merges are numbered in
//      position order (a block scan) and dealt out one per thread; each computes the new
//      node's least-expected-cost record from its children's (merge_costs, the model of
//      prt_collapse.cuh), kept in shared memory, so no bottom-up pass follows;
//   3. the 8-wide collapse, level by level from shared-memory copies of the binary
//      nodes' children, counts and cost records (or areas, for the largest-child-first
//      collapse), eight lanes per frontier node (lane c writes child c), positions from
//      block scans: a node's inner children are consecutive in slot order and its leaf
//      triangles contiguous, as k_collapse lays them out; each leaf's triangles go to a
//      shared-memory permutation;
//   4. the triangles re-laid out in leaf order (as k_relayout): copied into shared
//      memory with coalesced loads, then written out in permutation order.
// The counters end as the multi-launch build leaves them, and in the host's pinned copy
// (build_finish reads that after its wait).
// No thread waits on another except at __syncthreads; every loop is bounded.
#include <atomic>
#include <cfloat>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"
#include "prt_collapse.cuh"

namespace prt {

namespace {

constexpr uint32_t kSmallMax = 4096; // triangles: four positions per thread
constexpr int kThreads = 1024;
#ifndef PRT_PLOC_RADIUS
#define PRT_PLOC_RADIUS 3 // 3 / 4 / 6 / 8 / 12 measured: 3 fastest, and no worse a tree
#endif
constexpr int kRadius = PRT_PLOC_RADIUS; // PLOC's search radius in Morton order
constexpr uint32_t kPlocRounds = 48; // PLOC iterations before neighbours pair regardless
// 16-bit node references: a binary node's index, or the leaf flag | triangle index.
constexpr uint32_t kLeaf16 = 0x8000u;
// A cluster's word: its reference, its nearest neighbour's position (12 bits) and its
// triangle count, saturating at 15 (exact up to the largest leaf, which is all a count
// above leaf_size is used for).
constexpr uint32_t kNnShift = 16, kNnMask = 0xFFFu, kCntShift = 28, kCntMax = 15u;
static_assert(kSmallMax - 1u <= kNnMask, "neighbour positions take 12 bits");
static_assert((uint32_t)kMaxLeaf < kCntMax, "saturated counts must exceed every leaf size");

// Shared memory, in rows of one word per triangle.  PLOC: the clusters' boxes (six rows,
// structure of arrays), their words, and seven rows of the binary nodes' costs in 1..7
// child slots (row k - 1 for k slots; row 0 holds the area for the largest-child-first
// collapse).  Before PLOC the sort's keys and per-warp digit counts take the box rows
// and the triangles' boxes in input order the cost rows; within an iteration, row 6 of
// the nodes it is about to make lists its merges, and the rows of the nodes after those
// stage its survivors.  Collapse, over the box and word rows: the leaf permutation, the
// binary nodes' children, slot splits and counts, two frontiers and the groups' exchange
// words (the cost rows stay).  Re-layout: the permutation, then the triangles as
// loaded.  The block-scan words last.
constexpr uint32_t kRow = 4u * kSmallMax;
constexpr uint32_t kOffBox = 0;
constexpr uint32_t kOffWord = 6u * kRow;
constexpr uint32_t kOffCost = 7u * kRow;
constexpr uint32_t kOffScan = 14u * kRow;
constexpr uint32_t kSmemBytes = kOffScan + 4u * 64u;
constexpr uint32_t kOffPerm = 0;                         // leaf order -> triangle (16 bits)
constexpr uint32_t kOffLr = kOffPerm + 2u * kSmallMax;    // children (16 + 16 bits)
constexpr uint32_t kOffBits = kOffLr + kRow;              // slot splits (CostNode::bits)
constexpr uint32_t kOffCnt = kOffBits + kRow;             // counts (16 bits)
constexpr uint32_t kOffFr0 = kOffCnt + 2u * kSmallMax;    // frontier: ref | slot << 16
constexpr uint32_t kOffFr1 = kOffFr0 + kRow;
constexpr uint32_t kOffXch = kOffFr1 + kRow;             // one word per thread
constexpr uint32_t kOffStage = kOffPerm + 2u * kSmallMax; // 9 words per triangle
static_assert(kOffXch + 4u * kThreads <= kOffCost, "collapse tables overlap the cost rows");
static_assert(kOffStage + 36u * kSmallMax <= kOffScan, "staged triangles overlap the scan words");
static_assert(kSmemBytes <= 232448u, "more shared memory than a block can have");
static_assert(8u * kSmallMax + 4u * 32u * 257u <= kOffWord, "sort keys and counts overlap the words");
constexpr int kPer = (int)(kSmallMax / kThreads); // positions per thread

struct Box {
	float lx, ly, lz, hx, hy, hz;
};

__device__ __forceinline__ Box load_box(const float *b, uint32_t i) {
	return Box{b[i], b[kSmallMax + i], b[2 * kSmallMax + i], b[3 * kSmallMax + i],
	           b[4 * kSmallMax + i], b[5 * kSmallMax + i]};
}
__device__ __forceinline__ void store_box(float *b, uint32_t i, const Box &x) {
	b[i] = x.lx;
	b[kSmallMax + i] = x.ly;
	b[2 * kSmallMax + i] = x.lz;
	b[3 * kSmallMax + i] = x.hx;
	b[4 * kSmallMax + i] = x.hy;
	b[5 * kSmallMax + i] = x.hz;
}
__device__ __forceinline__ Box join(const Box &a, const Box &b) {
	return Box{fminf(a.lx, b.lx), fminf(a.ly, b.ly), fminf(a.lz, b.lz),
	           fmaxf(a.hx, b.hx), fmaxf(a.hy, b.hy), fmaxf(a.hz, b.hz)};
}
__device__ __forceinline__ float4 box_lo(const Box &b) { return make_float4(b.lx, b.ly, b.lz, 0.0f); }
__device__ __forceinline__ float4 box_hi(const Box &b) { return make_float4(b.hx, b.hy, b.hz, 0.0f); }

// Surface area (up to a constant) of the union of two boxes, the same value whichever
// is first; an overflow (or an infinite extent times a zero one) reads as FLT_MAX.
__device__ __forceinline__ float union_area(const Box &a, const Box &b) {
	const float dx = fmaxf(a.hx, b.hx) - fminf(a.lx, b.lx);
	const float dy = fmaxf(a.hy, b.hy) - fminf(a.ly, b.ly);
	const float dz = fmaxf(a.hz, b.hz) - fminf(a.lz, b.lz);
	return fminf(dx * dy + dz * (dx + dy), FLT_MAX);
}

// The box of a triangle as the other builders make it (k_leaf_boxes): [-FLT_MAX,
// FLT_MAX]^3 for a non-finite vertex.
__device__ __forceinline__ Box tri_box(const float t[9], bool fin) {
	if (!fin)
		return Box{-FLT_MAX, -FLT_MAX, -FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX};
	return Box{fminf(t[0], fminf(t[3], t[6])), fminf(t[1], fminf(t[4], t[7])),
	           fminf(t[2], fminf(t[5], t[8])), fmaxf(t[0], fmaxf(t[3], t[6])),
	           fmaxf(t[1], fmaxf(t[4], t[7])), fmaxf(t[2], fmaxf(t[5], t[8]))};
}

// A child's costs in 1..7 slots (cs[1..7], in units of its own area): a triangle's from
// the model, a binary node's from its cost rows (node_costs' values, stored that way).
__device__ __forceinline__ void row_costs(uint32_t y, const float *crow, float cs[8]) {
	if (y & kLeaf16) {
		leaf_costs(cs);
		return;
	}
#pragma unroll
	for (int j = 1; j < 8; ++j)
		cs[j] = crow[(uint32_t)(j - 1) * kSmallMax + y];
}

__device__ __forceinline__ float tri_centroid(const float t[9], int k) {
	return t[k] * (1.0f / 3.0f) + t[k + 3] * (1.0f / 3.0f) + t[k + 6] * (1.0f / 3.0f);
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
	x &= 1023u;
	x = (x | (x << 16)) & 0x030000FFu;
	x = (x | (x << 8)) & 0x0300F00Fu;
	x = (x | (x << 4)) & 0x030C30C3u;
	x = (x | (x << 2)) & 0x09249249u;
	return x;
}

// Exclusive prefix sum of one word per thread over the block; `total` gets the sum.
// The caller separates two calls with a __syncthreads (the scan words are reused).
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t *words, uint32_t &total) {
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	uint32_t x = v;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
		if (lane >= (uint32_t)o)
			x += y;
	}
	if (lane == 31u)
		words[warp] = x;
	__syncthreads();
	if (warp == 0) {
		uint32_t w = words[lane];
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
			if (lane >= (uint32_t)o)
				w += y;
		}
		words[32 + lane] = w;
	}
	__syncthreads();
	total = words[63];
	return (warp ? words[32 + warp - 1] : 0u) + x - v;
}

// An 8-wide node's child record (an empty slot: NaN bounds and kNone).
__device__ __forceinline__ Child8 make_child(float4 lo, float4 hi, uint32_t ref) {
	Child8 ch;
	ch.lo_x = lo.x;
	ch.lo_y = lo.y;
	ch.lo_z = lo.z;
	ch.ref = ref;
	ch.hi_x = hi.x;
	ch.hi_y = hi.y;
	ch.hi_z = hi.z;
	ch.pad = 0u;
	return ch;
}

// Position i's nearest neighbour within kRadius positions among m clusters: the least
// pair in the order (union area, distance, parity of the lower position, lower position;
// the last three as fields of 4, 1 and 12 bits), a total order, so the loop's order does
// not matter; unrolled, so the neighbours' boxes load together.
__device__ __forceinline__ uint32_t nearest(const float *box, uint32_t i, uint32_t m) {
	const Box bi = load_box(box, i);
	float best = INFINITY;
	uint32_t best_tb = 0xFFFFFFFFu, bj = i;
#pragma unroll
	for (int o = -kRadius; o <= kRadius; ++o) {
		const int jj = (int)i + o;
		if (o == 0 || jj < 0 || jj >= (int)m)
			continue;
		const uint32_t j = (uint32_t)jj, low = min(i, j);
		const float d = union_area(bi, load_box(box, j));
		const uint32_t tb = ((uint32_t)(o < 0 ? -o : o) << 13) | ((low & 1u) << 12) | low;
		if (d < best || (d == best && tb < best_tb)) {
			best = d;
			best_tb = tb;
			bj = j;
		}
	}
	return bj;
}

// Binary node `node` over clusters (bi, wi) and (bj, wj): its cost rows (row 0: its area
// for the largest-child-first collapse), slot splits, children, box and count.  Returns
// the node's cluster word; u gets its box.
__device__ __forceinline__ uint32_t make_node(uint32_t node, const Box &bi, const Box &bj,
                                              uint32_t wi, uint32_t wj, int use_cost,
                                              uint32_t leaf_size, float *crow, CostNode *cost,
                                              uint32_t *lr, float4 *ibox, Box &u) {
	u = join(bi, bj);
	const uint32_t a = wi & 0xFFFFu, c = wj & 0xFFFFu;
	const uint32_t count = min((wi >> kCntShift) + (wj >> kCntShift), kCntMax);
	const float area = half_area(box_lo(u), box_hi(u));
	if (use_cost) {
		float cl[8], cr[8];
		row_costs(a, crow, cl);
		row_costs(c, crow, cr);
		const CostNode cn = merge_costs<true>(cl, cr, half_extent(box_lo(bi), box_hi(bi)),
		                                      half_extent(box_lo(bj), box_hi(bj)),
		                                      half_extent(box_lo(u), box_hi(u)), count, leaf_size);
		crow[node] = cn.c1;
#pragma unroll
		for (uint32_t s = 2; s < 8; ++s)
			crow[(s - 1u) * kSmallMax + node] = fminf(cn.c1, cn.cd[s - 2u]);
		cost[node].bits = cn.bits;
	} else {
		crow[node] = area;
	}
	lr[node] = a | (c << 16);
	ibox[2 * node] = make_float4(u.lx, u.ly, u.lz, area);
	ibox[2 * node + 1] = make_float4(u.hx, u.hy, u.hz, __uint_as_float(count));
	return node | (count << kCntShift);
}

// Exclusive prefix over the warps of one value per warp (lane 0's), and the total, with
// one barrier.  The caller separates two calls with a __syncthreads.
static_assert(kThreads == 32 * 32, "one scan word per warp, one warp of them");
__device__ __forceinline__ uint32_t warp_totals_scan(uint32_t v, uint32_t *words, uint32_t &total) {
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	if (lane == 0u)
		words[warp] = v;
	__syncthreads();
	const uint32_t own = words[lane];
	uint32_t x = own;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
		if (lane >= (uint32_t)o)
			x += y;
	}
	total = __shfl_sync(0xFFFFFFFFu, x, 31);
	return __shfl_sync(0xFFFFFFFFu, x - own, warp);
}

// Whether child y (16-bit reference) of an 8-wide node becomes a node of its own.
__device__ __forceinline__ bool child_inner(uint32_t y, uint32_t count, uint32_t leaf_size,
                                            int use_cost, const uint32_t *bits) {
	return !(y & kLeaf16) && (count > leaf_size || (use_cost && (bits[y] >> 31) == 0u));
}

__global__ void __launch_bounds__(kThreads, 1)
    k_build_small(const float *__restrict__ tris, uint32_t n, uint32_t leaf_size, int use_cost,
                  float4 *__restrict__ ibox, float4 *__restrict__ lbox, uint32_t *__restrict__ lr,
                  CostNode *__restrict__ cost, Node8 *__restrict__ nodes, uint32_t node_cap,
                  float4 *__restrict__ tri4, uint32_t *__restrict__ inv, uint32_t *__restrict__ ctr,
                  uint32_t *__restrict__ hctr, Node8 *__restrict__ dead, CNode8 *__restrict__ cdead,
                  uint32_t *__restrict__ err) {
	extern __shared__ __align__(16) unsigned char sm[];
	uint32_t *scan = reinterpret_cast<uint32_t *>(sm + kOffScan);
	const uint32_t tid = threadIdx.x;
	float *box = reinterpret_cast<float *>(sm + kOffBox);
	uint32_t *word = reinterpret_cast<uint32_t *>(sm + kOffWord);
	float *crow = reinterpret_cast<float *>(sm + kOffCost);
	// The counters (on the device, and the host's copy in mapped pinned memory) start at
	// zero; the empty node (NaN boxes, no references; compressed: no masks, no counts) is
	// written here rather than by separate copies.
	if (tid < (uint32_t)kCtrWords) {
		ctr[tid] = 0u;
		hctr[tid] = 0u;
	}
	if (tid < sizeof(Node8) / 4u)
		reinterpret_cast<uint32_t *>(dead)[tid] = 0xFFFFFFFFu;
	if (cdead && tid < sizeof(CNode8) / 4u)
		reinterpret_cast<uint32_t *>(cdead)[tid] = 0u;

	// 1. One pass over the triangles: boxes (input order, into the cost rows, and to the
	// leaf-box array for the collapse), centroids kept for the keys; centroid bounds of
	// the finite triangles; Morton keys; bitonic sort.
	float cen[kPer][3];
	bool cfin[kPer];
	{
		float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = tid + (uint32_t)k * kThreads;
			cfin[k] = false;
			if (i < n) {
				float t[9];
#pragma unroll
				for (int q = 0; q < 9; ++q)
					t[q] = __ldg(tris + 9 * (size_t)i + q);
				bool fin = true;
#pragma unroll
				for (int q = 0; q < 9; ++q)
					fin = fin && isfinite(t[q]);
				const Box b = tri_box(t, fin);
				store_box(crow, i, b);
				lbox[2 * i] = box_lo(b);
				lbox[2 * i + 1] = box_hi(b);
				cfin[k] = fin;
#pragma unroll
				for (int q = 0; q < 3; ++q) {
					cen[k][q] = tri_centroid(t, q);
					if (fin) {
						mn[q] = fminf(mn[q], cen[k][q]);
						mx[q] = fmaxf(mx[q], cen[k][q]);
					}
				}
			}
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1)
#pragma unroll
			for (int q = 0; q < 3; ++q) {
				mn[q] = fminf(mn[q], __shfl_xor_sync(0xFFFFFFFFu, mn[q], o));
				mx[q] = fmaxf(mx[q], __shfl_xor_sync(0xFFFFFFFFu, mx[q], o));
			}
		float *red = reinterpret_cast<float *>(word); // 32 x 6 words
		if ((tid & 31u) == 0)
			for (int q = 0; q < 3; ++q) {
				red[6 * (tid >> 5) + q] = mn[q];
				red[6 * (tid >> 5) + 3 + q] = mx[q];
			}
		__syncthreads();
		if (tid < 32) {
#pragma unroll
			for (int q = 0; q < 3; ++q) {
				mn[q] = red[6 * tid + q];
				mx[q] = red[6 * tid + 3 + q];
			}
#pragma unroll
			for (int o = 16; o > 0; o >>= 1)
#pragma unroll
				for (int q = 0; q < 3; ++q) {
					mn[q] = fminf(mn[q], __shfl_xor_sync(0xFFFFFFFFu, mn[q], o));
					mx[q] = fmaxf(mx[q], __shfl_xor_sync(0xFFFFFFFFu, mx[q], o));
				}
			if (tid == 0)
				for (int q = 0; q < 3; ++q) {
					scan[q] = __float_as_uint(mn[q]);
					scan[3 + q] = __float_as_uint(mx[q]);
				}
		}
		__syncthreads();
	}
	unsigned long long *keys = reinterpret_cast<unsigned long long *>(sm + kOffBox);
	{
		float lo[3], sc[3];
		const bool any = __uint_as_float(scan[0]) <= __uint_as_float(scan[3]);
#pragma unroll
		for (int q = 0; q < 3; ++q) {
			lo[q] = __uint_as_float(scan[q]);
			const float ext = __uint_as_float(scan[3 + q]) - lo[q];
			sc[q] = ext > 0.0f ? 1024.0f / ext : 0.0f;
		}
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = tid + (uint32_t)k * kThreads;
			if (i < n) {
				uint32_t code = 0;
				if (cfin[k] && any) {
					uint32_t qv[3];
#pragma unroll
					for (int q = 0; q < 3; ++q)
						qv[q] = (uint32_t)fminf(fmaxf((cen[k][q] - lo[q]) * sc[q], 0.0f), 1023.0f);
					code = (spread10(qv[0]) << 2) | (spread10(qv[1]) << 1) | spread10(qv[2]);
				}
				keys[i] = ((unsigned long long)code << 32) | i;
			}
		}
	}
	__syncthreads();
	// LSD radix sort of the keys by code, 8 bits a pass; each pass is stable, so equal
	// codes keep index order (the order of the keys' low words).  Warp w holds positions
	// 128w .. 128w + 127, round r at 128w + 32r + lane: a key's rank among the warp's keys
	// of its digit comes from ballots, round by round; the digit's start for the warp
	// from one scan over the counts in (digit, warp) order.
	{
		// Warp w's count of digit d at hist[w * 257 + d]: a warp's 32 lanes, on different
		// digits, and a scan thread's 8 warps, on one digit, fall in different banks.
		uint32_t *hist = reinterpret_cast<uint32_t *>(sm + kOffBox) + 2u * kSmallMax;
		const uint32_t warp = tid >> 5, lane = tid & 31u, below = (1u << lane) - 1u;
		unsigned long long kv[kPer];
#pragma unroll
		for (int r = 0; r < kPer; ++r) {
			const uint32_t p = 128u * warp + 32u * (uint32_t)r + lane;
			kv[r] = p < n ? keys[p] : 0ull;
		}
		for (uint32_t shift = 32; shift < 62; shift += 8) {
			for (uint32_t j = tid; j < 32u * 257u; j += kThreads)
				hist[j] = 0u;
			__syncthreads();
			uint32_t dg[kPer], rank[kPer];
#pragma unroll
			for (int r = 0; r < kPer; ++r) {
				const bool valid = 128u * warp + 32u * (uint32_t)r + lane < n;
				dg[r] = valid ? (uint32_t)(kv[r] >> shift) & 255u : 256u;
				// The lanes whose digit equals this lane's, one ballot per digit bit.
				uint32_t same = 0xFFFFFFFFu;
#pragma unroll
				for (int b = 0; b < 9; ++b) {
					const uint32_t v = __ballot_sync(0xFFFFFFFFu, (dg[r] >> b) & 1u);
					same &= ((dg[r] >> b) & 1u) ? v : ~v;
				}
				const uint32_t base = valid ? hist[257u * warp + dg[r]] : 0u;
				__syncwarp();
				if (valid && (same & below) == 0u) // the lowest lane of its digit
					hist[257u * warp + dg[r]] = base + __popc(same);
				__syncwarp();
				rank[r] = base + __popc(same & below);
			}
			__syncthreads();
			// Counts in (digit, warp) order: thread t has digit t / 4, warps 8 (t % 4) + j.
			const uint32_t sd = tid >> 2, sw = 8u * (tid & 3u);
			uint32_t c[8], sum = 0, total;
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				c[j] = hist[257u * (sw + (uint32_t)j) + sd];
				sum += c[j];
			}
			uint32_t run = block_scan(sum, scan, total); // every count read before the writes
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				hist[257u * (sw + (uint32_t)j) + sd] = run;
				run += c[j];
			}
			__syncthreads();
#pragma unroll
			for (int r = 0; r < kPer; ++r)
				if (dg[r] < 256u)
					keys[hist[257u * warp + dg[r]] + rank[r]] = kv[r];
			__syncthreads();
#pragma unroll
			for (int r = 0; r < kPer; ++r) {
				const uint32_t p = 128u * warp + 32u * (uint32_t)r + lane;
				kv[r] = p < n ? keys[p] : 0ull;
			}
		}
	}

	// 2. Leaves in Morton order (boxes gathered from the cost rows), then PLOC.
	{
		uint32_t prim[kPer];
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = tid + (uint32_t)k * kThreads;
			prim[k] = i < n ? (uint32_t)(keys[i] & 0xFFFFFFFFull) : 0u;
			if (prim[k] >= n) { // cannot happen: the keys of [0, n) sort first
				atomicOr(err, kErrCollapse);
				prim[k] = 0;
			}
		}
		__syncthreads(); // every key read before the box rows are overwritten
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = tid + (uint32_t)k * kThreads;
			if (i < n) {
				store_box(box, i, load_box(crow, prim[k]));
				word[i] = kLeaf16 | prim[k] | (1u << kCntShift);
			}
		}
	}
	__syncthreads();
	uint32_t *list = reinterpret_cast<uint32_t *>(crow + 6u * kSmallMax);
	uint32_t m = n, made = 0;
	uint32_t iter = 0;
	for (; m > 32u; ++iter) { // the last 32 clusters merge in one warp (below)
		// (a) Each cluster's nearest neighbour, into its word.
		for (uint32_t i = tid; i < m; i += kThreads) {
			const uint32_t bj = iter >= kPlocRounds ? ((i ^ 1u) < m ? (i ^ 1u) : i) // odd m: last stays
			                                        : nearest(box, i, m);
			word[i] = (word[i] & ~(kNnMask << kNnShift)) | (bj << kNnShift);
		}
		__syncthreads();
		// (b) Survivors and merges.  Warp w takes positions 128w .. 128w + 127, round k at
		// 128w + 32k + lane; ballots give each position's rank within its warp, one scan
		// of the warps' totals (kept | merges << 16) the warps' starts.  Survivor r is
		// staged at index made + merged + r of the cost rows (boxes in rows 0-5, words in
		// row 6: nodes not made yet, and kept <= n - made - merged of them are free); a
		// merge's position and rank are listed in row 6 of the node it makes.
		const uint32_t wp = tid >> 5, ln = tid & 31u, below = (1u << ln) - 1u;
		uint32_t bk[kPer], bm[kPer], wsum = 0;
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = 128u * wp + 32u * (uint32_t)k + ln;
			bool keep = false, merge = false;
			if (i < m) {
				const uint32_t j = (word[i] >> kNnShift) & kNnMask;
				const bool mutual = ((word[j] >> kNnShift) & kNnMask) == i;
				keep = !(mutual && i > j);
				merge = mutual && i < j;
			}
			bk[k] = __ballot_sync(0xFFFFFFFFu, keep);
			bm[k] = __ballot_sync(0xFFFFFFFFu, merge);
			wsum += (uint32_t)__popc(bk[k]) | ((uint32_t)__popc(bm[k]) << 16);
		}
		uint32_t total;
		const uint32_t wpre = warp_totals_scan(wsum, scan, total);
		const uint32_t kept = total & 0xFFFFu, merged = total >> 16;
		uint32_t *stage_w = list; // row 6
		const uint32_t tbase = made + merged;
		{
			uint32_t pos0 = wpre & 0xFFFFu, q0 = made + (wpre >> 16);
#pragma unroll
			for (int k = 0; k < kPer; ++k) {
				const uint32_t i = 128u * wp + 32u * (uint32_t)k + ln;
				if ((bk[k] >> ln) & 1u) {
					const uint32_t pos = pos0 + __popc(bk[k] & below);
					if ((bm[k] >> ln) & 1u) {
						list[q0 + __popc(bm[k] & below)] = i | (pos << 16);
					} else {
						store_box(crow, tbase + pos, load_box(box, i));
						stage_w[tbase + pos] = word[i];
					}
				}
				pos0 += __popc(bk[k]);
				q0 += __popc(bm[k]);
			}
		}
		__syncthreads();
		// (c) The merges, one per thread: node made + q joins the clusters at its listed
		// position i and at i's neighbour j, and is staged at its survivor rank.  Each
		// position belongs to one pair, and nothing writes the clusters until (d).
		for (uint32_t q = tid; q < merged; q += kThreads) {
			const uint32_t node = made + q;
			const uint32_t e = list[node], i = e & 0xFFFFu, pos = e >> 16; // before row 6 is written
			const uint32_t wi = word[i], j = (wi >> kNnShift) & kNnMask, wj = word[j];
			Box u;
			const uint32_t w = make_node(node, load_box(box, i), load_box(box, j), wi, wj, use_cost,
			                             leaf_size, crow, cost, lr, ibox, u);
			store_box(crow, tbase + pos, u);
			stage_w[tbase + pos] = w;
		}
		__syncthreads();
		// (d) The staged survivors become clusters 0 .. kept - 1.
		for (uint32_t r = tid; r < kept; r += kThreads) {
			store_box(box, r, load_box(crow, tbase + r));
			word[r] = stage_w[tbase + r];
		}
		made += merged;
		m = kept;
		if (merged == 0u || iter >= n) { // cannot happen (see above); reported, not looped
			if (tid == 0)
				atomicOr(err, kErrCollapse);
			return;
		}
		__syncthreads();
	}
	// The last clusters (at most 32: about the last ten iterations) in warp 0, one per
	// lane, with warp barriers: each merging lane makes its node, every survivor moves
	// to its rank once all have read.  The other warps wait at the barrier after.
	if (m > 1u) {
		if (tid < 32u) {
			const uint32_t i = tid, below = (1u << i) - 1u;
			uint32_t failed = 0;
			for (; m > 1u; ++iter) {
				const bool act = i < m;
				if (act) {
					const uint32_t bj = iter >= kPlocRounds ? ((i ^ 1u) < m ? (i ^ 1u) : i)
					                                        : nearest(box, i, m);
					word[i] = (word[i] & ~(kNnMask << kNnShift)) | (bj << kNnShift);
				}
				__syncwarp();
				bool keep = false, merge = false;
				uint32_t j = i, wi = 0;
				if (act) {
					wi = word[i];
					j = (wi >> kNnShift) & kNnMask;
					const bool mutual = ((word[j] >> kNnShift) & kNnMask) == i;
					keep = !(mutual && i > j);
					merge = mutual && i < j;
				}
				const uint32_t bk = __ballot_sync(0xFFFFFFFFu, keep);
				const uint32_t bm = __ballot_sync(0xFFFFFFFFu, merge);
				Box ub;
				uint32_t uw = wi;
				if (merge)
					uw = make_node(made + __popc(bm & below), load_box(box, i), load_box(box, j), wi,
					               word[j], use_cost, leaf_size, crow, cost, lr, ibox, ub);
				else if (keep)
					ub = load_box(box, i);
				__syncwarp(); // every cluster read before any moves
				if (keep) {
					const uint32_t pos = __popc(bk & below);
					store_box(box, pos, ub);
					word[pos] = uw;
				}
				__syncwarp();
				made += (uint32_t)__popc(bm);
				m = (uint32_t)__popc(bk);
				if (bm == 0u || iter >= n) { // cannot happen (see above); reported, not looped
					failed = 1u;
					break;
				}
			}
			if (i == 0u) {
				scan[0] = made;
				scan[1] = failed;
				if (failed)
					atomicOr(err, kErrCollapse);
			}
		}
		__syncthreads();
		made = scan[0];
		if (scan[1])
			return;
	}

	// 3. The 8-wide collapse from shared-memory copies of the binary nodes: eight lanes
	// per frontier node, lane c on child c.
	const uint32_t root = word[0] & 0xFFFFu;
	__syncthreads(); // everything of PLOC read before its space is reused
	uint16_t *perm = reinterpret_cast<uint16_t *>(sm + kOffPerm);
	uint32_t *lr_s = reinterpret_cast<uint32_t *>(sm + kOffLr);
	uint32_t *bits_s = reinterpret_cast<uint32_t *>(sm + kOffBits);
	uint16_t *cnt_s = reinterpret_cast<uint16_t *>(sm + kOffCnt);
	uint32_t *fr[2] = {reinterpret_cast<uint32_t *>(sm + kOffFr0),
	                   reinterpret_cast<uint32_t *>(sm + kOffFr1)};
	uint32_t *xch = reinterpret_cast<uint32_t *>(sm + kOffXch);
	{
		// All of a thread's loads before its stores (one wait, not one per node).
		uint32_t w[kPer], cn[kPer], bt[kPer];
#pragma unroll
		for (int u = 0; u < kPer; ++u) {
			const uint32_t k = tid + (uint32_t)u * kThreads;
			if (k < made) {
				w[u] = __ldcg(&lr[k]);
				cn[u] = __float_as_uint(__ldcg(&ibox[2 * k + 1].w));
				bt[u] = use_cost ? __ldcg(&cost[k].bits) : 0u;
			}
		}
#pragma unroll
		for (int u = 0; u < kPer; ++u) {
			const uint32_t k = tid + (uint32_t)u * kThreads;
			if (k < made) {
				lr_s[k] = w[u];
				cnt_s[k] = (uint16_t)cn[u];
				bits_s[k] = bt[u];
			}
		}
	}
	if (tid == 0)
		fr[0][0] = root; // slot 0
	__syncthreads();
	const uint32_t c8 = tid & 7u;            // this lane's child
	const uint32_t lane = tid & 31u;
	uint32_t n_items = 1, n_nodes = 1, n_placed = 0;
	int level = 0;
	for (;; ++level) {
		if (tid == 0)
			ctr[level] = n_items;
		if (level == kMaxLevels)
			break; // deeper than the traversal allows: build_finish reports it
		const uint32_t *fin = fr[level & 1];
		uint32_t *fout = fr[(level + 1) & 1];
		uint32_t next_items = 0;
		for (uint32_t b0 = 0; b0 < n_items; b0 += kThreads / 8u) {
			const uint32_t it = b0 + tid / 8u;
			const bool live = it < n_items;
			uint32_t slot = 0, y = 0, k = c8;
			bool has = false;
			const uint32_t r = live ? fin[it] & 0xFFFFu : 0u;
			if (live)
				slot = fin[it] >> 16;
			if (use_cost) {
				// The node's children as slot ranges: lane c8 holds the subtree covering
				// slots [c8, c8 + span).  A subtree opened into its span (the root always;
				// another when its cost in `span` slots, row span - 1, is below its cost
				// in one, row 0) splits it: the left child keeps the first split_of(span)
				// slots, the right child goes to the lane after them.  Every subtree
				// splits at once, at most 7 rounds; the ranges end in the order of the
				// depth-first opening (left subtrees first), which is the slot order.
				uint32_t span = (live && c8 == 0u) ? 8u : 0u;
				y = r;
				uint32_t *x = xch + (tid & ~7u);
				for (int round = 0; round < 8; ++round) {
					uint32_t give = 0, a = 0;
					if (span > 1u && !(y & kLeaf16) &&
					    (round == 0 || crow[(span - 1u) * kSmallMax + y] < crow[y])) {
						a = split_of(bits_s[y], span);
						const uint32_t w = lr_s[y];
						give = (w >> 16) | ((span - a) << 16); // nonzero: span - a >= 1
						y = w & 0xFFFFu;
						span = a;
					}
					if (!__any_sync(0xFFFFFFFFu, give != 0u))
						break;
					x[c8] = 0u; // only this lane reads its word (below)
					__syncwarp();
					if (give)
						x[c8 + a] = give; // inside the giver's range: no other holder there
					__syncwarp();
					const uint32_t got = x[c8];
					if (got) {
						y = got & 0xFFFFu;
						span = got >> 16;
					}
				}
				has = span > 0u;
				const uint32_t held = (__ballot_sync(0xFFFFFFFFu, has) >> (lane & 24u)) & 0xFFu;
				k = __popc(held & ((1u << c8) - 1u));
			} else if (live) {
				// Largest child first (the group's lanes all compute the same list).
				uint32_t C[8];
				int nc = 1;
				C[0] = r;
				while (nc < 8) {
					int best = -1;
					float best_area = -1.0f;
					for (int c = 0; c < nc; ++c) {
						const float ac = (C[c] & kLeaf16) ? -1.0f : crow[C[c]];
						if (ac > best_area) {
							best_area = ac;
							best = c;
						}
					}
					if (best < 0)
						break;
					const uint32_t x = C[best];
					C[best] = lr_s[x] & 0xFFFFu;
					C[nc++] = lr_s[x] >> 16;
				}
				has = (int)c8 < nc;
				for (int c = 0; c < 8; ++c)
					if ((uint32_t)c == c8 && has)
						y = C[c];
			}
			// This lane's child (slot k): its count, whether it becomes a node, and its box
			// (loaded now: the wait overlaps the scan).  A binary node's box comes from its
			// record, a single triangle's from the leaf-box array.
			uint32_t nz = 0;
			bool in = false;
			const float4 none = make_float4(__int_as_float(0x7FC00000), __int_as_float(0x7FC00000),
			                                __int_as_float(0x7FC00000), 0.f);
			float4 lo = none, hi = none;
			if (has) {
				nz = (y & kLeaf16) ? 1u : cnt_s[y];
				in = child_inner(y, nz, leaf_size, use_cost, bits_s);
				const float4 *src = (y & kLeaf16) ? lbox + 2 * (y & ~kLeaf16) : ibox + 2 * y;
				lo = __ldcg(src);
				hi = __ldcg(src + 1);
			}
			// Inner children and triangles before this one, and the group's totals (lane
			// order is child order).
			const uint32_t gsh = lane & 24u;
			const uint32_t nc = __popc((__ballot_sync(0xFFFFFFFFu, has) >> gsh) & 0xFFu);
			const uint32_t inm = (__ballot_sync(0xFFFFFFFFu, has && in) >> gsh) & 0xFFu;
			const uint32_t my_inner = __popc(inm & ((1u << c8) - 1u)), n_inner = __popc(inm);
			const uint32_t mine_t = (has && !in) ? nz : 0u;
			uint32_t tsum = mine_t;
#pragma unroll
			for (uint32_t o = 1; o < 8u; o <<= 1) {
				const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, tsum, o, 8);
				if (c8 >= o)
					tsum += v;
			}
			const uint32_t n_tris = __shfl_sync(0xFFFFFFFFu, tsum, gsh | 7u);
			const uint32_t my_tris = tsum - mine_t;
			uint32_t total;
			const uint32_t pre = block_scan(c8 == 0u ? (n_inner | (n_tris << 16)) : 0u, scan, total);
			const uint32_t pg = __shfl_sync(0xFFFFFFFFu, pre, gsh); // the group's lane 0
			const uint32_t nb = n_nodes + (pg & 0xFFFFu), ob = next_items + (pg & 0xFFFFu);
			const uint32_t tb = n_placed + (pg >> 16);
			const bool fits = nb + n_inner <= node_cap && ob + n_inner <= kSmallMax &&
			                  tb + n_tris <= n;
			if (live && !fits && c8 == 0u)
				atomicOr(err, kErrCollapse);
			if (live && fits) {
				if (has) {
					uint32_t ref;
					if (in) {
						ref = nb + my_inner;
						fout[ob + my_inner] = y | (ref << 16);
					} else {
						// A leaf: its triangles' positions in subtree order (at most
						// leaf_size <= 8) go to the permutation; the triangles are copied
						// after the last level, all at once.
						uint32_t dst = tb + my_tris;
						ref = make_leaf(dst, nz);
						uint32_t stack[8];
						int sp = 0;
						stack[sp++] = y;
						while (sp > 0) {
							const uint32_t z = stack[--sp];
							if (z & kLeaf16) {
								perm[dst++] = (uint16_t)(z & ~kLeaf16);
							} else if (sp <= 6) {
								stack[sp++] = lr_s[z] >> 16;
								stack[sp++] = lr_s[z] & 0xFFFFu;
							} else {
								atomicOr(err, kErrCollapse); // more than 8 leaves: not a leaf
							}
						}
					}
					nodes[slot].c[k] = make_child(lo, hi, ref);
				}
				if (c8 >= nc) // the slots after the last child
					nodes[slot].c[c8] = make_child(none, none, kNone);
			}
			n_nodes += total & 0xFFFFu;
			next_items += total & 0xFFFFu;
			n_placed += total >> 16;
			__syncthreads();
		}
		n_items = next_items;
		if (n_items == 0u) {
			if (tid == 0 && level + 1 <= kMaxLevels)
				ctr[level + 1] = 0u;
			break;
		}
	}
	if (tid == 0) {
		ctr[kCtrNodes] = n_nodes;
		ctr[kCtrTris] = n_placed;
	}
	// 4. The triangles in leaf order (as k_relayout; the second word's w flags a
	// non-finite vertex): copied into shared memory by consecutive words, every load of a
	// batch issued before its stores, then written out in permutation order.
	__syncthreads();
	float *stage = reinterpret_cast<float *>(sm + kOffStage);
	const uint32_t words = 9u * n;
	constexpr uint32_t kBatch = 12;
	for (uint32_t base = 0; base < words; base += kBatch * kThreads) {
		float v[kBatch];
#pragma unroll
		for (uint32_t u = 0; u < kBatch; ++u) {
			const uint32_t w = base + u * kThreads + tid;
			v[u] = w < words ? __ldg(tris + w) : 0.0f;
		}
#pragma unroll
		for (uint32_t u = 0; u < kBatch; ++u) {
			const uint32_t w = base + u * kThreads + tid;
			if (w < words)
				stage[w] = v[u];
		}
	}
	__syncthreads();
	const uint32_t placed = min(n_placed, n);
#pragma unroll
	for (int k = 0; k < kPer; ++k) {
		const uint32_t d = tid + (uint32_t)k * kThreads;
		const uint32_t p = d < placed ? perm[d] : 0xFFFFu;
		if (p >= n)
			continue;
		float t[9];
		bool fin = true;
#pragma unroll
		for (int q = 0; q < 9; ++q) {
			t[q] = stage[9u * p + q];
			fin = fin && isfinite(t[q]);
		}
		tri4[3 * (size_t)d] = make_float4(t[0], t[1], t[2], __uint_as_float(p));
		tri4[3 * (size_t)d + 1] = make_float4(t[3], t[4], t[5], fin ? 0.0f : 1.0f);
		tri4[3 * (size_t)d + 2] = make_float4(t[6], t[7], t[8], 0.0f);
		inv[p] = d;
	}
	// The counters' host copy, which the host reads after its wait without a copy of its
	// own (thread 0 wrote the device counters before the barriers above).
	if (tid < (uint32_t)kCtrWords)
		hctr[tid] = __ldcg(&ctr[tid]);
}

} // namespace

uint32_t small_build_max() { return kSmallMax; }

cudaError_t launch_build_small(const float *d_tris, uint32_t n, uint32_t leaf_size, bool use_cost,
                               bool compressed, BuildScratch &ws, SceneGPU &sc, uint32_t node_cap,
                               uint32_t *ctr, uint32_t *h_ctr, uint32_t *d_err, cudaStream_t st) {
	// The shared-memory limit is a per-device attribute: set once per device.
	static std::atomic<uint32_t> attr_set{0};
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess)
		return e;
	// The host's pinned counters, as the device addresses them.
	uint32_t *h_dev = nullptr;
	e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&h_dev), h_ctr, 0);
	if (e != cudaSuccess)
		return e;
	const uint32_t bit = (dev >= 0 && dev < 32) ? (1u << dev) : 0u;
	if (!bit || !(attr_set.load() & bit)) {
		e = cudaFuncSetAttribute(k_build_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                         (int)kSmemBytes);
		if (e != cudaSuccess)
			return e;
		attr_set.fetch_or(bit);
	}
	k_build_small<<<1, kThreads, kSmemBytes, st>>>(
	    d_tris, n, leaf_size, use_cost ? 1 : 0, ws.ibox.as<float4>(), ws.lbox.as<float4>(),
	    ws.left.as<uint32_t>(), use_cost ? ws.cost.as<CostNode>() : nullptr,
	    sc.nodes.as<Node8>(), node_cap, sc.tri4.as<float4>(), sc.inv.as<uint32_t>(), ctr, h_dev,
	    sc.nodes.as<Node8>() + sc.dead, compressed ? sc.cnodes.as<CNode8>() + sc.dead : nullptr,
	    d_err);
	return cudaGetLastError();
}

} // namespace prt
