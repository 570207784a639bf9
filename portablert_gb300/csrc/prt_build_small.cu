// prt_build_small.cu - a scene of at most 4,096 triangles built by one thread block.
//
// Replaces, for small scenes, the chain of about 57 dependent launches of the binned-SAH
// build (each level's kernels wait on global memory; at this size the build is latency,
// not work) with one launch whose dependencies go through shared memory:
//   1. one pass over the triangles (boxes into shared memory, centroid bounds), 30-bit
//      Morton codes (as k_morton makes them), a bitonic sort of (code, index) in shared
//      memory;
//   2. PLOC (Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding
//      Volume Hierarchy Construction", 2018): the clusters in Morton order each find
//      the cluster within kRadius (3) positions whose union with it has the least surface
//      area; mutual nearest neighbours merge into a binary node; the survivors are
//      compacted in order; repeated until one cluster is left.  Candidates are ordered
//      by (area, distance in Morton order, parity of the lower position, lower
//      position): a total order on pairs, so the least pair of an iteration is mutual
//      and every iteration merges at least one; equal clusters pair up as (2k, 2k + 1)
//      instead of one pair at a time.  After kPlocRounds iterations (scenes whose
//      clusters keep choosing one neighbour, such as exponentially spaced triangles)
//      positions 2k and 2k + 1 merge regardless, which bounds the iterations and the
//      depth by kPlocRounds + log2(n).  Each merge computes the new node's
//      least-expected-cost record from its children's (merge_costs, the model of
//      prt_collapse.cuh), so no bottom-up pass follows;
//   3. the 8-wide collapse, level by level from shared-memory copies of the binary
//      nodes' children, counts and cost records (or areas, for the largest-child-first
//      collapse), eight lanes per frontier node (lane c writes child c), positions from
//      block scans: a node's inner children are consecutive in slot order and its leaf
//      triangles contiguous, as k_collapse lays them out; the triangles are re-laid out
//      in leaf order in the same pass (as k_relayout).
// The counters end as the multi-launch build leaves them (build_finish reads them).
// No thread waits on another except at __syncthreads; every loop is bounded.
#include <atomic>
#include <cfloat>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"
#include "prt_collapse.cuh"

namespace prt {

namespace {

constexpr uint32_t kSmallMax = 4096; // triangles; a power of two (the sort's size)
constexpr int kThreads = 1024;
#ifndef PRT_PLOC_RADIUS
#define PRT_PLOC_RADIUS 3 // 3 / 4 / 6 / 8 / 12 measured: 3 fastest, and no worse a tree
#endif
constexpr int kRadius = PRT_PLOC_RADIUS; // PLOC's search radius in Morton order
constexpr uint32_t kPlocRounds = 48; // PLOC iterations before neighbours pair regardless
// 16-bit node references: a binary node's index, or the leaf flag | triangle index.
constexpr uint32_t kLeaf16 = 0x8000u;

// Shared memory (bytes).  PLOC: two cluster buffers, each six box arrays and one word
// per cluster (16-bit reference | triangle count << 16); the nearest neighbours of an
// iteration sit in the buffer the iteration writes (read into registers before it is
// written).  Before PLOC the triangles' boxes, in input order, fill buffer 1 and the
// sort's keys buffer 0.  Collapse: the binary nodes' cost records (or areas), children
// and counts, and two frontiers.  The block-scan words last.
constexpr uint32_t kBoxBytes = 6u * 4u * kSmallMax;
constexpr uint32_t kOffBox0 = 0, kOffBox1 = kBoxBytes;
constexpr uint32_t kOffId0 = 2u * kBoxBytes, kOffId1 = kOffId0 + 4u * kSmallMax;
constexpr uint32_t kOffScan = kOffId1 + 4u * kSmallMax;
constexpr uint32_t kOffCost = 0;
constexpr uint32_t kOffLr = kOffCost + (uint32_t)sizeof(CostNode) * kSmallMax;
constexpr uint32_t kOffCnt = kOffLr + 4u * kSmallMax;
constexpr uint32_t kOffFr0 = kOffCnt + 2u * kSmallMax;
constexpr uint32_t kOffFr1 = kOffFr0 + 4u * kSmallMax;
constexpr uint32_t kSmemBytes = kOffScan + 4u * 64u;
static_assert(kOffFr1 + 4u * kSmallMax <= kOffScan, "collapse tables overlap the scan words");
static_assert(kSmemBytes <= 232448u, "more shared memory than a block can have");
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

__device__ __forceinline__ CostNode load_cost(const CostNode *p) {
	CostNode c;
	c.c1 = __ldcg(&p->c1);
#pragma unroll
	for (int k = 0; k < 7; ++k)
		c.cd[k] = __ldcg(&p->cd[k]);
	c.bits = __ldcg(&p->bits);
	return c;
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

// Whether child y (16-bit reference) of an 8-wide node becomes a node of its own.
__device__ __forceinline__ bool child_inner(uint32_t y, uint32_t count, uint32_t leaf_size,
                                            int use_cost, const CostNode *cs) {
	return !(y & kLeaf16) && (count > leaf_size || (use_cost && (cs[y].bits >> 31) == 0u));
}

__global__ void __launch_bounds__(kThreads, 1)
    k_build_small(const float *__restrict__ tris, uint32_t n, uint32_t leaf_size, int use_cost,
                  float4 *__restrict__ ibox, uint32_t *__restrict__ lr,
                  CostNode *__restrict__ cost, Node8 *__restrict__ nodes, uint32_t node_cap,
                  float4 *__restrict__ tri4, uint32_t *__restrict__ inv, uint32_t *__restrict__ ctr,
                  uint32_t *__restrict__ err) {
	extern __shared__ __align__(16) unsigned char sm[];
	uint32_t *scan = reinterpret_cast<uint32_t *>(sm + kOffScan);
	const uint32_t tid = threadIdx.x;
	float *box[2] = {reinterpret_cast<float *>(sm + kOffBox0), reinterpret_cast<float *>(sm + kOffBox1)};
	uint32_t *ids[2] = {reinterpret_cast<uint32_t *>(sm + kOffId0),
	                    reinterpret_cast<uint32_t *>(sm + kOffId1)};

	// 1. One pass over the triangles: boxes (input order, buffer 1), centroids kept for
	// the keys; centroid bounds of the finite triangles; Morton keys; bitonic sort.
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
				store_box(box[1], i, tri_box(t, fin));
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
		float *red = reinterpret_cast<float *>(sm + kOffId0); // 32 x 6 words
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
	uint32_t P = 2;
	while (P < n)
		P <<= 1;
	unsigned long long *keys = reinterpret_cast<unsigned long long *>(sm + kOffBox0);
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
			if (i >= P)
				continue;
			unsigned long long key = ~0ull;
			if (i < n) {
				uint32_t code = 0;
				if (cfin[k] && any) {
					uint32_t qv[3];
#pragma unroll
					for (int q = 0; q < 3; ++q)
						qv[q] = (uint32_t)fminf(fmaxf((cen[k][q] - lo[q]) * sc[q], 0.0f), 1023.0f);
					code = (spread10(qv[0]) << 2) | (spread10(qv[1]) << 1) | spread10(qv[2]);
				}
				key = ((unsigned long long)code << 32) | i;
			}
			keys[i] = key;
		}
	}
	__syncthreads();
	for (uint32_t size = 2; size <= P; size <<= 1)
		for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
			for (uint32_t t = tid; t < P / 2; t += kThreads) {
				const uint32_t i = (t / stride) * 2u * stride + (t % stride), j = i + stride;
				const unsigned long long a = keys[i], b = keys[j];
				if ((a > b) == ((i & size) == 0u)) {
					keys[i] = b;
					keys[j] = a;
				}
			}
			__syncthreads();
		}

	// 2. Leaves in Morton order (boxes gathered from buffer 1), then PLOC.
	{
		uint32_t prim[kPer];
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = tid + (uint32_t)k * kThreads;
			prim[k] = i < n ? (uint32_t)(keys[i] & 0xFFFFFFFFull) : 0u;
		}
		__syncthreads(); // every key read before buffer 0 is overwritten
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = tid + (uint32_t)k * kThreads;
			if (i < n) {
				store_box(box[0], i, load_box(box[1], prim[k]));
				ids[0][i] = kLeaf16 | prim[k] | (1u << 16);
			}
		}
	}
	__syncthreads();
	uint32_t m = n, made = 0;
	int cur = 0;
	for (uint32_t iter = 0; m > 1; ++iter) {
		const float *bc = box[cur];
		uint16_t *nn = reinterpret_cast<uint16_t *>(ids[cur ^ 1]); // free until the writes
		for (uint32_t i = tid; i < m; i += kThreads) {
			if (iter >= kPlocRounds) {
				nn[i] = (uint16_t)((i ^ 1u) < m ? (i ^ 1u) : i); // the last of odd m stays
				continue;
			}
			const Box bi = load_box(bc, i);
			const uint32_t lo = i > (uint32_t)kRadius ? i - kRadius : 0u;
			const uint32_t hi = min(m - 1u, i + (uint32_t)kRadius);
			float best = INFINITY;
			uint32_t best_tb = 0xFFFFFFFFu, bj = i;
			for (uint32_t j = lo; j <= hi; ++j) {
				if (j == i)
					continue;
				const float d = union_area(bi, load_box(bc, j));
				// Tie-break of the pair {i, j}: distance, parity of the lower position,
				// lower position (fields of 4, 1 and 12 bits).
				const uint32_t low = min(i, j);
				const uint32_t tb = ((j > i ? j - i : i - j) << 13) | ((low & 1u) << 12) | low;
				if (d < best || (d == best && tb < best_tb)) {
					best = d;
					best_tb = tb;
					bj = j;
				}
			}
			nn[i] = (uint16_t)bj;
		}
		__syncthreads();
		// Survivors and merges over contiguous chunks of kPer positions per thread,
		// packed (kept | merges << 16) for one scan; the partners read before the scan's
		// barriers, after which the neighbour words are overwritten.
		uint32_t flag[kPer], part[kPer], local = 0;
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = tid * (uint32_t)kPer + (uint32_t)k;
			uint32_t f = 0, j = 0;
			if (i < m) {
				j = nn[i];
				const bool mutual = nn[j] == i;
				f = (mutual && i > j) ? 0u : (1u | ((mutual && i < j) ? 0x10000u : 0u));
			}
			flag[k] = f;
			part[k] = j;
			local += f;
		}
		uint32_t total;
		uint32_t pre = block_scan(local, scan, total);
		const uint32_t kept = total & 0xFFFFu, merged = total >> 16;
		const float *bs = box[cur];
		float *bd = box[cur ^ 1];
		const uint32_t *is = ids[cur];
		uint32_t *id_out = ids[cur ^ 1];
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t i = tid * (uint32_t)kPer + (uint32_t)k;
			const uint32_t f = flag[k];
			if (f) {
				const uint32_t pos = pre & 0xFFFFu;
				Box b = load_box(bs, i);
				uint32_t word = is[i];
				if (f >> 16) {
					const uint32_t j = part[k];
					const Box bj = load_box(bs, j);
					const uint32_t node = made + (pre >> 16);
					const uint32_t wa = word, wc = is[j];
					const uint32_t a = wa & 0xFFFFu, c = wc & 0xFFFFu;
					const uint32_t count = (wa >> 16) + (wc >> 16);
					const Box u = join(b, bj);
					if (use_cost) {
						float cl[8], cr[8];
						if (a & kLeaf16) {
							leaf_costs(cl);
						} else {
							const CostNode ca = load_cost(cost + a);
							node_costs(ca, cl);
						}
						if (c & kLeaf16) {
							leaf_costs(cr);
						} else {
							const CostNode cc = load_cost(cost + c);
							node_costs(cc, cr);
						}
						cost[node] = merge_costs(cl, cr, half_extent(box_lo(b), box_hi(b)),
						                         half_extent(box_lo(bj), box_hi(bj)),
						                         half_extent(box_lo(u), box_hi(u)), count,
						                         leaf_size);
					}
					lr[node] = a | (c << 16);
					ibox[2 * node] = make_float4(u.lx, u.ly, u.lz, half_area(box_lo(u), box_hi(u)));
					ibox[2 * node + 1] = make_float4(u.hx, u.hy, u.hz, __uint_as_float(count));
					b = u;
					word = node | (count << 16);
				}
				store_box(bd, pos, b);
				id_out[pos] = word;
			}
			pre += f;
		}
		made += merged;
		m = kept;
		cur ^= 1;
		if (merged == 0u || iter >= n) { // cannot happen (see above); reported, not looped
			if (tid == 0)
				atomicOr(err, kErrCollapse);
			return;
		}
		__syncthreads();
	}

	// 3. The 8-wide collapse from shared-memory copies of the binary nodes: eight lanes
	// per frontier node, lane c on child c.
	const uint32_t root = ids[cur][0] & 0xFFFFu;
	__syncthreads(); // everything of PLOC read before its space is reused
	CostNode *cs = reinterpret_cast<CostNode *>(sm + kOffCost);
	float *area = reinterpret_cast<float *>(sm + kOffCost);
	uint32_t *lr_s = reinterpret_cast<uint32_t *>(sm + kOffLr);
	uint16_t *cnt_s = reinterpret_cast<uint16_t *>(sm + kOffCnt);
	uint32_t *fr[2] = {reinterpret_cast<uint32_t *>(sm + kOffFr0),
	                   reinterpret_cast<uint32_t *>(sm + kOffFr1)};
	for (uint32_t k = tid; k < made; k += kThreads) {
		lr_s[k] = __ldcg(&lr[k]);
		const float4 lo = __ldcg(&ibox[2 * k]);
		cnt_s[k] = (uint16_t)__float_as_uint(__ldcg(&ibox[2 * k + 1].w));
		if (use_cost)
			cs[k] = load_cost(cost + k);
		else
			area[k] = lo.w;
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
			// Every lane of the group computes the node's children (same smem reads).
			uint32_t C[8];
			int nc = 0;
			uint32_t slot = 0;
			if (live) {
				const uint32_t r = fin[it] & 0xFFFFu;
				slot = fin[it] >> 16;
				if (r & kLeaf16) {
					C[0] = r;
					nc = 1;
				} else if (use_cost) {
					uint32_t py[8], pi[8];
					const uint32_t a0 = split_of(cs[r].bits, 8u);
					py[0] = lr_s[r] >> 16;
					pi[0] = 8u - a0;
					py[1] = lr_s[r] & 0xFFFFu;
					pi[1] = a0;
					int top = 2;
					while (top > 0) {
						--top;
						const uint32_t y = py[top], i = pi[top];
						bool open = false;
						uint32_t a = 1;
						if (!(y & kLeaf16) && i > 1u) {
							open = cs[y].cd[i - 2u] < cs[y].c1;
							a = split_of(cs[y].bits, i);
						}
						if (open && top <= 6) {
							py[top] = lr_s[y] >> 16;
							pi[top] = i - a;
							py[top + 1] = lr_s[y] & 0xFFFFu;
							pi[top + 1] = a;
							top += 2;
						} else if (nc < 8) {
							C[nc++] = y;
						}
					}
				} else {
					C[0] = r;
					nc = 1;
					while (nc < 8) {
						int best = -1;
						float best_area = -1.0f;
						for (int c = 0; c < nc; ++c) {
							const float ac = (C[c] & kLeaf16) ? -1.0f : area[C[c]];
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
				}
			}
			// This lane's child: inner children before it, triangles before it.
			uint32_t n_inner = 0, n_tris = 0, my_inner = 0, my_tris = 0, y = 0, cnt_y = 0;
			bool mine = false, inner_y = false;
			for (int c = 0; c < nc; ++c) {
				const uint32_t z = C[c];
				const uint32_t nz = (z & kLeaf16) ? 1u : cnt_s[z];
				const bool in = child_inner(z, nz, leaf_size, use_cost, cs);
				if ((uint32_t)c == c8) {
					my_inner = n_inner;
					my_tris = n_tris;
					y = z;
					cnt_y = nz;
					inner_y = in;
					mine = true;
				}
				n_inner += in ? 1u : 0u;
				n_tris += in ? 0u : nz;
			}
			uint32_t total;
			const uint32_t pre = block_scan(c8 == 0u ? (n_inner | (n_tris << 16)) : 0u, scan, total);
			const uint32_t pg = __shfl_sync(0xFFFFFFFFu, pre, lane & 24u); // the group's lane 0
			const uint32_t nb = n_nodes + (pg & 0xFFFFu), ob = next_items + (pg & 0xFFFFu);
			const uint32_t tb = n_placed + (pg >> 16);
			const bool fits = nb + n_inner <= node_cap && ob + n_inner <= kSmallMax &&
			                  tb + n_tris <= n;
			if (live && !fits && c8 == 0u)
				atomicOr(err, kErrCollapse);
			if (live && fits) {
				float4 lo = make_float4(__int_as_float(0x7FC00000), __int_as_float(0x7FC00000),
				                        __int_as_float(0x7FC00000), 0.f),
				       hi = lo;
				uint32_t ref = kNone;
				if (mine) {
					if (inner_y) {
						ref = nb + my_inner;
						fout[ob + my_inner] = y | (ref << 16);
						lo = __ldcg(&ibox[2 * y]);
						hi = __ldcg(&ibox[2 * y + 1]);
					} else {
						// A leaf: its triangles in subtree order (at most leaf_size <= 8),
						// re-laid out here; a single triangle's box comes from the triangle.
						uint32_t dst = tb + my_tris;
						ref = make_leaf(dst, cnt_y);
						if (!(y & kLeaf16)) {
							lo = __ldcg(&ibox[2 * y]);
							hi = __ldcg(&ibox[2 * y + 1]);
						}
						uint32_t stack[8];
						int sp = 0;
						stack[sp++] = y;
						while (sp > 0) {
							const uint32_t z = stack[--sp];
							if (z & kLeaf16) {
								const uint32_t p = z & ~kLeaf16;
								float t[9];
#pragma unroll
								for (int q = 0; q < 9; ++q)
									t[q] = __ldg(tris + 9 * (size_t)p + q);
								bool fin = true;
#pragma unroll
								for (int q = 0; q < 9; ++q)
									fin = fin && isfinite(t[q]);
								if (y & kLeaf16) {
									const Box tb9 = tri_box(t, fin);
									lo = box_lo(tb9);
									hi = box_hi(tb9);
								}
								// As k_relayout: the second word's w flags a non-finite vertex.
								tri4[3 * (size_t)dst] = make_float4(t[0], t[1], t[2], __uint_as_float(p));
								tri4[3 * (size_t)dst + 1] = make_float4(t[3], t[4], t[5], fin ? 0.0f : 1.0f);
								tri4[3 * (size_t)dst + 2] = make_float4(t[6], t[7], t[8], 0.0f);
								inv[p] = dst;
								++dst;
							} else if (sp <= 6) {
								stack[sp++] = lr_s[z] >> 16;
								stack[sp++] = lr_s[z] & 0xFFFFu;
							} else {
								atomicOr(err, kErrCollapse); // more than 8 leaves: not a leaf
							}
						}
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
				nodes[slot].c[c8] = ch;
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
}

} // namespace

uint32_t small_build_max() { return kSmallMax; }

cudaError_t launch_build_small(const float *d_tris, uint32_t n, uint32_t leaf_size, bool use_cost,
                               BuildScratch &ws, SceneGPU &sc, uint32_t node_cap, uint32_t *ctr,
                               uint32_t *d_err, cudaStream_t st) {
	// The shared-memory limit is a per-device attribute: set once per device.
	static std::atomic<uint32_t> attr_set{0};
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
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
	    d_tris, n, leaf_size, use_cost ? 1 : 0, ws.ibox.as<float4>(), ws.left.as<uint32_t>(),
	    use_cost ? ws.cost.as<CostNode>() : nullptr, sc.nodes.as<Node8>(), node_cap,
	    sc.tri4.as<float4>(), sc.inv.as<uint32_t>(), ctr, d_err);
	return cudaGetLastError();
}

} // namespace prt
