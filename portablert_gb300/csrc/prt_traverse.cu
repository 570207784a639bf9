// prt_traverse.cu - persistent nearest-hit traversal of the 8-wide tree.
//
// Replaces BVH2::nearest_tri (portableRT bvh.hpp:224-265) and the std::thread loop of
// CPUBackend::nearest_hits (intersect_cpu.hpp:20-43).
//
// Answer (identical to the reference's on finite inputs): the smallest t over the
// triangles whose own bounding box passes the reference slab test and which
// Moller-Trumbore accepts; t may be negative, there is no t-min and no culling by t,
// exactly as in the reference.  Inner nodes only prune with tests that are
// conservative for that set (prt_internal.cuh), so neither the tree's shape nor the
// visit order changes the answer; ties in t go to the smaller primitive id.
//
// Execution: one warp = 8 groups of 4 lanes; all state for 32 rays is in shared memory.
//  * A warp takes up to 32 consecutive rays from a global counter ("slots": 32 per
//    batch, or 8 or 16 when one small run would leave most warps idle): origin,
//    direction, reciprocal and best-hit key per slot live in shared memory.
//  * Work items (slot, node) sit in a warp-local LIFO pool.  Each step every group
//    pops one item and each of its 4 lanes loads and slab-tests 2 of the node's 8
//    children: lane s takes children s and s + 4, so each of the two 256-bit loads of a
//    group reads one 128-byte line of the node (children 2s and 2s + 1 would spread each
//    load over two lines and double the L1 wavefronts: 15 % slower).  Hit inner children
//    are pushed back as items and hit leaf triangles are appended to a triangle queue,
//    at positions from ballots and popc, child-major (all lanes' first children, then
//    all second children: no position depends on the lane's previous child; the step
//    issues 16 % fewer ALU-pipe instructions than in lane order, and the half-rate ALU
//    pipe is what bounds it).  Roots of new rays are admitted whenever fewer than 8
//    items are left.  Unused child slots hold NaN boxes, which no plain slab test
//    passes.
//  * A query of ray buffers is two launches: a regular pass over the batches whose 32
//    rays all have finite reciprocals (the plain slab test only), which counts and skips
//    the others, and a deferred pass over those with the conservative test for zero
//    direction components (it returns at once when there are none).  Camera queries and
//    counting runs are one general launch.  A request server's serving launch (pass 3)
//    takes its batches from device queues that the host extends while it runs
//    (claim_batch) and picks the plain or the general test per batch.
//  * When 32 triangles are queued, the 32 lanes test one each with the exact reference
//    test and fold (t, primitive id) into the slot's 64-bit key with a shared atomicMin;
//    with FP32 nodes the lane whose key the slot kept records its u, v (and a zero t's
//    sign) beside it, with compressed nodes the winner is tested again at the end.
//  * When the pool and the queue are empty the warp writes the 32 records in the
//    caller's HitReg<Tags...> layout to shared memory and stores them as 16-byte words.
//  * The pool holds at most 7 K (D - 1) + K items for K = 8 items per step and a tree of
//    depth D (each step's pushes leave at most 7 K items behind per level); it is sized
//    per launch as 7 K (D - 1) + 2 K; a push that would not fit, or a batch that takes
//    more steps than a tree can need, is reported as an error and ends the batch.
//
// Algorithmic bytes per ray: 24 (ray) + R (record) + node bytes visited + 48 per
// triangle tested; the counting variant (COUNT) measures the visits.
#include <algorithm>
#include <mutex>

#include "../../include/prt_b200.h"
#include "prt_camera.cuh"
#include "prt_traverse.cuh"

namespace prt {

namespace {

constexpr int kWarpsPerBlock = 4;
// Lanes that test one node together (each takes 8 / kLanesPerNode children); a warp
// step visits 32 / kLanesPerNode nodes.
#ifndef PRT_TRAVERSE_LANES_PER_NODE
#define PRT_TRAVERSE_LANES_PER_NODE 4
#endif
constexpr int kLanesPerNode = PRT_TRAVERSE_LANES_PER_NODE;
constexpr int kItems = 32 / kLanesPerNode;       // items per step (K)
constexpr int kChildPerLane = 8 / kLanesPerNode;
constexpr int kMaxDepth = 32;

struct TravArgs {
	const SceneDesc *scenes; // scene table (n_segs > 0)
	const SegDesc *segs;     // segment table sorted by vbegin (n_segs > 0)
	uint32_t n_segs;         // 0: one run, described by seg0 / scene0
	uint32_t n_virtual;      // padded ray count
	SceneDesc scene0;
	SegDesc seg0;
	uint32_t n_nodes;        // largest node array (bounds the steps of a batch)
	uint32_t dead;           // index of a node of eight empty children in every scene's
	                         // node array (pads a step that has fewer than K items)
	uint32_t pool_cap;       // entries of the pool (>= 256, it also holds the staged records)
	uint32_t queue_cap;      // entries of the triangle queue
	uint32_t warp_bytes;     // shared memory per warp
	uint32_t max_leaf;       // most triangles in a leaf of any scene of the launch
	uint32_t max_batches;    // batches per warp before it exits (0 = no bound)
	uint32_t batch;          // rays a warp takes at a time: 32, or 16 / 8 for one small
	                         // run (more warps busy, shorter chains per warp)
	uint32_t *counter;
	uint32_t *deferred;      // [0] batches the regular pass left to the general one,
	                         // [1] the deferred pass's batch counter
	uint32_t *err;
	unsigned long long *visits;
	uint32_t use_cam;        // 1: rays of the single run come from `cam`, not seg0.rays
	prt_b200_camera cam;
	ServeQueues serve;       // PASS 3 only
};

// Per-warp shared memory: fixed part, then the queue and the pool (sizes per launch).
// alignas(16): the queue follows this part and the pool after it doubles as the staging
// area of the output records, which is read with 16-byte vector loads.
struct alignas(16) WarpFixed {
	unsigned long long key[32]; // best (t, primitive id) per slot
	float4 ro[32];              // origin and kind (int bits) per slot
	float4 rf[32];              // reciprocals per slot
	float4 rd[32];              // direction per slot
	// rf[s].w and rd[s].w: u and v of slot s's winning hit (its key holds t exactly, up
	// to the sign of a zero, which bit s of negzero keeps); no array of their own, so
	// shared memory does not grow (a deep tree's pool already brings nine blocks close
	// to the SM's limit, and the L1 cache gets what shared memory leaves).
	SegDesc seg;                // the run the current 32 rays belong to
	uint32_t batches;           // batches this warp has taken (kept here, not in a register)
	// Serving launches: tickets past the published end per queue, and the queue whose
	// run `seg` holds (kept here, not in registers).
	uint32_t held[kServeQueues];
	uint32_t cached_q;
	uint32_t negzero; // bit s: slot s's winning t is -0 (read only when its key's t is 0)
	uint32_t pad_[(16 - (4 + 4 * kServeQueues + 4 + 4) % 16) % 16 / 4];
};
static_assert(sizeof(WarpFixed) % 16 == 0, "queue and pool must start 16-byte aligned");

__host__ __device__ inline uint32_t warp_smem_bytes(uint32_t pool_cap, uint32_t queue_cap) {
	return (uint32_t)sizeof(WarpFixed) + 4u * (queue_cap + pool_cap);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
	uint32_t m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

// One 32-byte read-only load (sm_100 and later; p 32-byte aligned): a whole child
// record, or a compressed node's header, in one instruction and one L1 sector.
__device__ __forceinline__ void ld_nc_256(const void *p, float4 &a, float4 &b) {
	asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
	    : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
	    : "l"(p));
}

// Three-input minimum and maximum (sm_100 and later; NaN operands ignored, as fminf and
// fmaxf ignore them).
__device__ __forceinline__ float max3f(float a, float b, float c) {
	float r;
	asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
	return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
	float r;
	asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
	return r;
}

// regular_box with its two comparisons folded into one: tmax >= 0 and tmin <= tmax hold
// exactly when max(tmin, 0) <= tmax, and the 0 joins the last axis' minimum.  Same
// products, same answer (an unused slot's NaN box: max(NaN, 0) = 0, and 0 <= NaN fails);
// one ALU instruction fewer per child, which the half-rate ALU pipe of FP32-node steps
// turns into 1 % more rays (compressed nodes measured 1 % slower with it, so they keep
// regular_box).
__device__ __forceinline__ bool regular_box_folded(const RayC &r, float lx, float hx, float ly,
                                                   float hy, float lz, float hz) {
	const float t1 = (lx - r.ox) * r.fx, t2 = (hx - r.ox) * r.fx;
	const float t3 = (ly - r.oy) * r.fy, t4 = (hy - r.oy) * r.fy;
	const float t5 = (lz - r.oz) * r.fz, t6 = (hz - r.oz) * r.fz;
	const float tmin = max3f(fminf(t1, t2), fminf(t3, t4), fmaxf(fminf(t5, t6), 0.0f));
	const float tmax = min3f(fmaxf(t1, t2), fmaxf(t3, t4), fmaxf(t5, t6));
	return tmin <= tmax;
}

template <bool REGULAR, bool FOLDED = false>
__device__ __forceinline__ bool box_test(const RayC &r, float lx, float hx, float ly, float hy,
                                         float lz, float hz) {
	if (REGULAR || r.kind == 0)
		return FOLDED ? regular_box_folded(r, lx, hx, ly, hy, lz, hz)
		              : regular_box(r, lx, hx, ly, hy, lz, hz);
	return conservative_box(r, lx, hx, ly, hy, lz, hz);
}

__device__ __forceinline__ uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xFFu; }

// float(byte k of w), exactly: the byte placed in the mantissa of 2^23 (one byte
// permute), minus 2^23 -- full-rate instructions instead of an integer conversion.
__device__ __forceinline__ float byte_as_float(uint32_t w, int k) {
	return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (uint32_t)k)),
	                 8388608.0f);
}

__device__ __forceinline__ RayC slot_ray(const WarpFixed &S, uint32_t s) {
	RayC r;
	// Two 16-byte shared loads for the slab test (the direction is dead there).
	const float4 o = S.ro[s], f = S.rf[s], d = S.rd[s];
	r.ox = o.x;
	r.oy = o.y;
	r.oz = o.z;
	r.dx = d.x;
	r.dy = d.y;
	r.dz = d.z;
	r.fx = f.x;
	r.fy = f.y;
	r.fz = f.z;
	r.kind = __float_as_int(o.w);
	return r;
}

// Tests queue entries [lo, lo + n) (n <= 32), one per lane.  KEEP: the lane whose hit a
// slot keeps also records its u, v (and the sign of a zero t) for the records.
template <bool COUNT, bool KEEP>
__device__ __forceinline__ void test_queued(const float4 *__restrict__ tri4, WarpFixed &S,
                                            const uint32_t *queue, uint32_t lo, uint32_t n,
                                            int lane, uint32_t &n_tests) {
	unsigned long long mykey = kNoHit;
	uint32_t my_slot = 0;
	float mt = 0.0f, mu = 0.0f, mv = 0.0f;
	if ((uint32_t)lane < n) {
		const uint32_t e = queue[lo + lane];
		const uint32_t slot = e >> kIndexBits;
		const RayC r = slot_ray(S, slot);
		const float4 *p = tri4 + 3 * (size_t)(e & kIndexMask);
		const float4 A = __ldg(p), B = __ldg(p + 1), C = __ldg(p + 2);
		float t, u, v;
		// Finite ray and triangle (nearly always): the box test with plain min/max.
		if (tri_test(r, A, B, C, t, u, v, r.kind == 0 && tri_record_finite(B)) && t < INFINITY) {
			mykey = hit_key(t, __float_as_uint(A.w));
			atomicMin(&S.key[slot], mykey);
			my_slot = slot;
			mt = t;
			mu = u;
			mv = v;
		}
		if (COUNT)
			++n_tests;
	}
	// The lane whose key the slot kept (keys are unique: they hold the primitive id)
	// records its u and v, so the records need no second test of the winner.
	if (!KEEP)
		return;
	__syncwarp();
	if (mykey != kNoHit && S.key[my_slot] == mykey) {
		S.rf[my_slot].w = mu;
		S.rd[my_slot].w = mv;
		if (mt == 0.0f) { // the key holds +0 for both zeros
			if (signbit(mt))
				atomicOr(&S.negzero, 1u << my_slot);
			else
				atomicAnd(&S.negzero, ~(1u << my_slot));
		}
	}
}

// Child `k` of `node`: slab test and what it refers to.
template <int FMT, bool REGULAR>
__device__ __forceinline__ void test_child(const void *__restrict__ nodes, const RayC &r,
                                           uint32_t node, int k, bool &hit, bool &inner,
                                           uint32_t &child, uint32_t &leaf_n) {
	hit = false;
	inner = false;
	child = 0;
	leaf_n = 0;
	if (FMT == PRT_NODES_FP32) {
		float4 lo, hi;
		ld_nc_256(&(static_cast<const Node8 *>(nodes) + node)->c[k], lo, hi);
		const uint32_t ref = __float_as_uint(lo.w);
		// An unused slot has a NaN box, which the plain slab test never passes; the
		// conservative test would, so only the general pass checks the reference.
		if (REGULAR || ref != kNone) {
			inner = !ref_is_leaf(ref);
			hit = box_test<REGULAR, true>(r, lo.x, hi.x, lo.y, hi.y, lo.z, hi.z);
			// A node index, or a leaf's first triangle: both below 2^27, under the
			// leaf flag and count bits.
			child = ref & kIndexMask;
			leaf_n = inner ? 0u : leaf_count(ref);
		}
	} else {
		const CNode8 *cn = static_cast<const CNode8 *>(nodes) + node;
		float4 h0, h1;
		ld_nc_256(cn, h0, h1); // the 32-byte header (96-byte nodes keep it 32-byte aligned)
		const uint4 w0 = make_uint4(__float_as_uint(h0.x), __float_as_uint(h0.y),
		                            __float_as_uint(h0.z), __float_as_uint(h0.w));
		const uint2 w1 = make_uint2(__float_as_uint(h1.x), __float_as_uint(h1.y));
		const uint2 ck = __ldg(reinterpret_cast<const uint2 *>(&cn->c[k]));
		const uint32_t imask = byte_of(w0.w, 3);
		const uint32_t m = byte_of(ck.y, 2);
		inner = (imask >> k) & 1u;
		if (inner || m) {
			const float sx = cscale((uint8_t)byte_of(w0.w, 0));
			const float sy = cscale((uint8_t)byte_of(w0.w, 1));
			const float sz = cscale((uint8_t)byte_of(w0.w, 2));
			const float ox = __uint_as_float(w0.x), oy = __uint_as_float(w0.y),
			            oz = __uint_as_float(w0.z);
			const float lx = cdec_f(ox, byte_as_float(ck.x, 0), sx);
			const float hx = cdec_f(ox, byte_as_float(ck.x, 1), sx);
			const float ly = cdec_f(oy, byte_as_float(ck.x, 2), sy);
			const float hy = cdec_f(oy, byte_as_float(ck.x, 3), sy);
			const float lz = cdec_f(oz, byte_as_float(ck.y, 0), sz);
			const float hz = cdec_f(oz, byte_as_float(ck.y, 1), sz);
			hit = box_test<REGULAR>(r, lx, hx, ly, hy, lz, hz);
			if (inner) {
				child = w1.x + __popc(imask & ((1u << k) - 1u));
			} else {
				child = w1.y + byte_of(ck.y, 3);
				leaf_n = m;
			}
		}
	}
}

// Resident blocks per SM the register budget is set for, per node format (measured on
// the 1M-triangle heightfield: 9 blocks of 4 warps = 56 registers, with a few spilled
// words, is fastest for both formats).
#ifndef PRT_TRAVERSE_MIN_BLOCKS_FP32
#define PRT_TRAVERSE_MIN_BLOCKS_FP32 9
#endif
#ifndef PRT_TRAVERSE_MIN_BLOCKS_COMPRESSED
#define PRT_TRAVERSE_MIN_BLOCKS_COMPRESSED 9
#endif

// The traversal of one batch of up to 32 rays (slots 0..nb-1 of S) through scene sd.
// REGULAR: every ray of the batch has finite reciprocals, so inner boxes take the plain
// slab test only (no branch to the conservative test per child).
template <int FMT, bool COUNT, bool LEAF1, bool REGULAR>
__device__ __forceinline__ void trace_batch(const TravArgs &a, WarpFixed &S, uint32_t *queue,
                                            uint32_t *pool, const SceneDesc &sd, uint32_t nb,
                                            int lane, int g, int s, uint32_t lt,
                                            uint32_t step_limit, uint32_t &n_visits,
                                            uint32_t &n_tests, bool &fault) {
	const float4 *__restrict__ tri4 = sd.tri4;
	const void *__restrict__ nodes = sd.nodes;
	uint32_t top = 0;  // items in the pool (warp-uniform)
	uint32_t q = 0;    // queued triangles (warp-uniform)
	uint32_t next = 0; // next slot whose root is not yet in the pool
	uint32_t steps = 0;
	for (;;) {
		// Admit new rays while fewer than K items are pending (a branch the common step
		// skips with one test).
		if (top < (uint32_t)kItems) {
			if (next < nb) {
				const uint32_t add = min((uint32_t)kItems - top, nb - next);
				if ((uint32_t)lane < add)
					pool[top + lane] = ((next + lane) << kIndexBits) | sd.root;
				top += add;
				next += add;
				__syncwarp();
			}
			if (top == 0u)
				break;
			// Fewer than K items left: the empty node (slot 0's ray) fills the step, so
			// every step takes K items and no group needs a "has an item" test.  A
			// counting run keeps the test (it counts visits of real items only).
			if (!COUNT && top < (uint32_t)kItems) {
				if ((uint32_t)lane >= top && lane < kItems)
					pool[lane] = a.dead;
				top = kItems;
				__syncwarp();
			}
		}
		const uint32_t take = COUNT ? min(top, (uint32_t)kItems) : (uint32_t)kItems;
		top -= take;
		// (Counting runs: groups without an item repeat the first one and drop what they
		// find.)
		const bool work = !COUNT || (uint32_t)g < take;
		const uint32_t item = pool[top + (COUNT ? (work ? g : 0) : g)];
		__syncwarp(); // the pops above are read before the pushes below overwrite them
		const uint32_t slot = item >> kIndexBits, node = item & kIndexMask;
		const RayC r = slot_ray(S, slot);
		if (COUNT && work && s == 0)
			++n_visits;

		bool hit[kChildPerLane], inner[kChildPerLane];
		uint32_t child[kChildPerLane], leaf_n[kChildPerLane];
#pragma unroll
		for (int j = 0; j < kChildPerLane; ++j) {
			test_child<FMT, REGULAR>(nodes, r, node, s + kLanesPerNode * j, hit[j], inner[j],
			                         child[j], leaf_n[j]);
			hit[j] = hit[j] && work;
		}
		// Every hit leaf of the step holds one triangle: always with single-triangle leaves
		// (predicates only on that path: the half-rate ALU pipe bounds the step).
		bool one_each = true;
		if (!LEAF1) {
			bool single = true;
#pragma unroll
			for (int j = 0; j < kChildPerLane; ++j)
				single = single && (!hit[j] || inner[j] || leaf_n[j] <= 1u);
			one_each = __all_sync(0xFFFFFFFFu, single);
		}

		// Positions, child-major: every lane's child j before any lane's child j + 1, so
		// no position waits on the lane's previous child.  Pushed inner children go to
		// the pool; with at most one triangle per hit leaf the queue positions come from
		// the same ballots.
		uint32_t pp[kChildPerLane], pq[kChildPerLane];
		uint32_t ptop = top, qtop = q;
#pragma unroll
		for (int j = 0; j < kChildPerLane; ++j) {
			const uint32_t bp = __ballot_sync(0xFFFFFFFFu, hit[j] && inner[j]);
			pp[j] = ptop + __popc(bp & lt);
			ptop += __popc(bp);
			if (one_each) {
				const uint32_t bl = __ballot_sync(0xFFFFFFFFu, hit[j] && !inner[j]);
				pq[j] = qtop + __popc(bl & lt);
				qtop += __popc(bl);
			}
		}
		// The pool holds every push of a well-formed tree and a well-formed tree ends
		// within step_limit steps; anything else is reported and ends the batch.
		++steps;
		if (ptop > a.pool_cap || steps > step_limit) {
			if (lane == 0)
				atomicOr(a.err, kErrStack);
			fault = true;
			break;
		}
		const uint32_t hi = slot << kIndexBits;
		if (one_each) {
#pragma unroll
			for (int j = 0; j < kChildPerLane; ++j) {
				if (hit[j] && inner[j])
					pool[pp[j]] = hi | child[j];
				if (hit[j] && !inner[j])
					queue[pq[j]] = hi | child[j];
			}
		} else {
#pragma unroll
			for (int j = 0; j < kChildPerLane; ++j)
				if (hit[j] && inner[j])
					pool[pp[j]] = hi | child[j];
			// Leaves of several triangles: positions from a scan of the per-lane counts.
			uint32_t cnt[kChildPerLane], all_cnt = 0;
#pragma unroll
			for (int j = 0; j < kChildPerLane; ++j) {
				cnt[j] = (hit[j] && !inner[j]) ? leaf_n[j] : 0u;
				all_cnt += cnt[j];
			}
			uint32_t incl = all_cnt;
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
				if (lane >= o)
					incl += y;
			}
			uint32_t pos = q + incl - all_cnt;
#pragma unroll
			for (int j = 0; j < kChildPerLane; ++j)
				for (uint32_t k = 0; k < cnt[j]; ++k)
					queue[pos++] = hi | (child[j] + k);
			qtop = q + __shfl_sync(0xFFFFFFFFu, incl, 31);
		}
		top = ptop;
		q = qtop;
		__syncwarp();
		while (q >= 32u) {
			q -= 32u;
			test_queued<COUNT, FMT == PRT_NODES_FP32>(tri4, S, queue, q, 32u, lane, n_tests);
			__syncwarp();
		}
	}
	while (q > 0u) {
		const uint32_t n = min(q, 32u);
		q -= n;
		test_queued<COUNT, FMT == PRT_NODES_FP32>(tri4, S, queue, q, n, lane, n_tests);
		__syncwarp();
	}
}

// A copy of a run descriptor that bypasses L1 (a serving launch reads descriptors that the
// host's copies write while it runs).
__device__ __forceinline__ SegDesc load_seg_cg(const SegDesc *p) {
	static_assert(sizeof(SegDesc) % 8 == 0, "descriptor copied as 8-byte words");
	SegDesc d;
	const unsigned long long *src = reinterpret_cast<const unsigned long long *>(p);
	unsigned long long *dst = reinterpret_cast<unsigned long long *>(&d);
#pragma unroll
	for (int k = 0; k < (int)(sizeof(SegDesc) / 8); ++k)
		dst[k] = __ldcg(src + k);
	return d;
}

// Serving launches (PASS 3): lane 0 takes the next batch, queues in priority order.  Batches
// are tickets drawn with atomicAdd on the queue's `next` (a compare-and-swap retried by
// thousands of warps on one word serialises them); a warp draws only when it saw a
// published batch, and a ticket that lands past the published end (another warp took
// the last one meanwhile) is kept in `held` until the host publishes that batch, while
// the warp serves the other queues.  The host stops a launch only when every published
// batch is finished, so tickets still held then are past all work.  Returns false when
// the warp should leave: stop set, or idle for idle_limit polls (an idle warp sleeps 0.25
// to 4 us between polls).  A warp that still holds a ticket after 16 x idle_limit polls
// without stop sets the error flag and leaves: every wait is bounded.
__device__ __forceinline__ bool claim_batch(const ServeQueues &q, uint32_t held[kServeQueues],
                                            uint32_t &qsel, uint32_t &batch) {
	uint32_t sleep_ns = 250;
	for (uint32_t idle = 0;; ++idle) {
		bool holding = false;
#pragma unroll
		for (uint32_t k = 0; k < (uint32_t)kServeQueues; ++k) {
			ServeQueueState *st = q.state[k];
			const uint32_t pub = *reinterpret_cast<volatile const uint32_t *>(&st->published);
			if (held[k] != kNone) {
				if (held[k] < pub) {
					qsel = k;
					batch = held[k];
					held[k] = kNone;
					return true;
				}
				holding = true;
				continue;
			}
			if (*reinterpret_cast<volatile const uint32_t *>(&st->next) < pub) {
				const uint32_t t = atomicAdd(&st->next, 1u);
				if (t < pub) {
					qsel = k;
					batch = t;
					return true;
				}
				held[k] = t; // past the end: served once published
				holding = true;
			}
		}
		if (*reinterpret_cast<volatile const uint32_t *>(q.stop))
			return false;
		if (idle >= (holding ? 16u * q.idle_limit : q.idle_limit)) {
			if (holding)
				*reinterpret_cast<volatile uint32_t *>(q.err_flag) = 1u;
			return false;
		}
		__nanosleep(sleep_ns);
		sleep_ns = min(sleep_ns * 2u, 4000u);
	}
}

// LEAF1: every leaf holds one triangle (leaf size 1), so a hit leaf queues exactly one.
// BOUNDED: a warp takes at most a.max_batches batches (a separate instantiation, so the
// unbounded kernels keep their register allocation).
// PASS: 0 = every batch with the general box test (the counting runs); 1 = batches whose
// rays all have finite reciprocals, with the plain slab test only (no conservative code
// in the kernel at all: 8 % faster), the others counted in a.deferred and skipped; 2 =
// the skipped batches with the general test (returns at once when there are none); 3 =
// a serving launch: batches claimed from the serving queues (claim_batch), the plain or
// the general test chosen per batch, descriptors and rays read around L1.
template <int FMT, bool COUNT, bool LEAF1, bool BOUNDED, int PASS>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, FMT == PRT_NODES_FP32
                                                           ? PRT_TRAVERSE_MIN_BLOCKS_FP32
                                                           : PRT_TRAVERSE_MIN_BLOCKS_COMPRESSED)
    k_trace8(TravArgs a) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	unsigned char *wbase = smem_raw + (size_t)(threadIdx.x >> 5) * a.warp_bytes;
	WarpFixed &S = *reinterpret_cast<WarpFixed *>(wbase);
	uint32_t *queue = reinterpret_cast<uint32_t *>(wbase + sizeof(WarpFixed));
	uint32_t *pool = queue + a.queue_cap; // also the staging area of the output records
	const int lane = threadIdx.x & 31, g = lane / kLanesPerNode, s = lane % kLanesPerNode;
	const uint32_t lt = lanemask_lt();
	uint32_t n_visits = 0, n_tests = 0;
	// A tree is visited at most once per ray; more steps than this means a malformed
	// tree, which is reported instead of looping.
	const uint32_t step_limit = (uint32_t)min(32ull * a.n_nodes + 64ull, 0xFFFFFFFFull);
	if (PASS == 2 && *(volatile const uint32_t *)a.deferred == 0u)
		return; // the regular pass took every batch (it ran before, on the same stream)

	if (BOUNDED && lane == 0)
		S.batches = 0;
	if (PASS == 3 && lane == 0) {
		for (int k = 0; k < kServeQueues; ++k)
			S.held[k] = kNone;
		S.cached_q = kNone;
	}
	__syncwarp();
	for (;;) {
		if (BOUNDED) {
			if (S.batches == a.max_batches)
				break;
			__syncwarp();
			if (lane == 0)
				++S.batches;
		}
		// Batches are taken in order from a counter (the deferred pass has its own, so
		// the few batches it works on spread over all warps); a serving launch claims
		// them from its queues.
		uint32_t base = 0;
		const SegDesc *segs = a.segs;
		if (PASS == 3) {
			uint32_t qsel = 0, batch = 0;
			const bool got = lane == 0 ? claim_batch(a.serve, S.held, qsel, batch) : false;
			if (!__shfl_sync(0xFFFFFFFFu, got, 0))
				break;
			qsel = __shfl_sync(0xFFFFFFFFu, qsel, 0);
			base = 32u * __shfl_sync(0xFFFFFFFFu, batch, 0);
			segs = a.serve.segs[qsel];
			// The run of this batch: the warp's last one when it still covers it (a large
			// request's batches mostly go to the same warps in turn), else a binary search
			// of the table (around L1: the host writes it while the launch runs).
			if (lane == 0 && !(S.cached_q == qsel && base >= (uint32_t)S.seg.vbegin &&
			                   base - (uint32_t)S.seg.vbegin < S.seg.n_rays)) {
				// Published after the table: covers every claimed batch.
				const uint32_t n_segs = *reinterpret_cast<volatile const uint32_t *>(
				    &a.serve.state[qsel]->n_segs);
				uint32_t lo_s = 0, hi_s = n_segs;
				while (hi_s - lo_s > 1) {
					const uint32_t mid = (lo_s + hi_s) >> 1;
					if (__ldcg(&segs[mid].vbegin) <= base)
						lo_s = mid;
					else
						hi_s = mid;
				}
				S.seg = load_seg_cg(segs + lo_s);
				S.cached_q = qsel;
			}
		} else {
			if (lane == 0)
				base = atomicAdd(PASS == 2 ? a.deferred + 1 : a.counter, a.batch);
			base = __shfl_sync(0xFFFFFFFFu, base, 0);
			if (base >= a.n_virtual)
				break;
			// The run these rays belong to (runs are padded to whole warps of 32, and
			// a batch of fewer rays never straddles one).
			uint32_t si = 0;
			if (a.n_segs) {
				if (lane == 0) {
					uint32_t lo_s = 0, hi_s = a.n_segs;
					while (hi_s - lo_s > 1) {
						const uint32_t mid = (lo_s + hi_s) >> 1;
						if (a.segs[mid].vbegin <= base)
							lo_s = mid;
						else
							hi_s = mid;
					}
					si = lo_s;
				}
				si = __shfl_sync(0xFFFFFFFFu, si, 0);
			}
			if (lane == 0)
				S.seg = a.n_segs ? a.segs[si] : a.seg0;
		}
		__syncwarp();
		const uint32_t local = base - (uint32_t)S.seg.vbegin;
		const uint32_t run_rays = S.seg.n_rays;
		if (local >= run_rays)
			continue; // padding of the run
		const uint32_t nb = min(PASS == 3 ? 32u : a.batch, run_rays - local);
		const SceneDesc sd = (PASS == 3 || a.n_segs) ? a.scenes[S.seg.scene] : a.scene0;
		const float4 *__restrict__ tri4 = sd.tri4;

		if ((uint32_t)lane < nb) {
			RayC r;
			if (a.use_cam) {
				float o[3], d[3];
				camera_ray(a.cam, local + lane, o, d);
				r = make_ray(o[0], o[1], o[2], d[0], d[1], d[2]);
			} else {
				const float2 *rp =
				    reinterpret_cast<const float2 *>(S.seg.rays + 6 * (size_t)(local + lane));
				float2 p0, p1, p2;
				if (PASS == 3) {
					p0 = __ldcg(rp);
					p1 = __ldcg(rp + 1);
					p2 = __ldcg(rp + 2);
				} else {
					p0 = __ldcs(rp);
					p1 = __ldcs(rp + 1);
					p2 = __ldcs(rp + 2);
				}
				r = make_ray(p0.x, p0.y, p1.x, p1.y, p2.x, p2.y);
			}
			S.ro[lane] = make_float4(r.ox, r.oy, r.oz, __int_as_float(r.kind));
			S.rf[lane] = make_float4(r.fx, r.fy, r.fz, 0.0f);
			S.rd[lane] = make_float4(r.dx, r.dy, r.dz, 0.0f);
		}
		S.key[lane] = kNoHit;
		__syncwarp();

		bool fault = false; // the batch's traversal reported an error (warp-uniform)
		if (sd.n_tris) {
			// Nearly every batch has only rays with finite reciprocals.
			const bool regular =
			    __all_sync(0xFFFFFFFFu, (uint32_t)lane >= nb || __float_as_int(S.ro[lane].w) == 0);
			if (PASS == 1 && !regular) {
				if (lane == 0)
					atomicAdd(a.deferred, 1u);
				continue; // left to the deferred pass
			}
			if (PASS == 2 && regular)
				continue; // done by the regular pass
			if (PASS == 3 && regular)
				trace_batch<FMT, COUNT, LEAF1, true>(a, S, queue, pool, sd, nb, lane, g, s, lt,
				                                     step_limit, n_visits, n_tests, fault);
			else
				trace_batch<FMT, COUNT, LEAF1, PASS == 1>(a, S, queue, pool, sd, nb, lane, g, s,
				                                          lt, step_limit, n_visits, n_tests, fault);
		} else if (PASS == 2) {
			continue; // the regular pass wrote this empty scene's misses
		}
		__syncwarp();

		// Finalise: stage each slot's record (its winner's t, u, v as its test found them)
		// in the run's HitReg<Tags...> layout.
		uint32_t *stage = pool;
		const uint32_t rec = S.seg.rec_size, fmask = S.seg.mask;
		const uint32_t rw = rec >> 2;
		// 32 records of rw words: rw * 8 16-byte words (record sizes are multiples of 4).
		for (uint32_t k = lane; k < rw * 8u; k += 32u)
			reinterpret_cast<uint4 *>(stage)[k] = make_uint4(0u, 0u, 0u, 0u);
		__syncwarp();
		if ((uint32_t)lane < nb) {
			const RayC r = slot_ray(S, lane);
			Best best;
			best_init(best);
			const unsigned long long key = S.key[lane];
			if (key != kNoHit && FMT == PRT_NODES_FP32) {
				const float tk = ord2f((uint32_t)(key >> 32));
				best.t = tk != 0.0f ? tk : (((S.negzero >> lane) & 1u) ? -0.0f : 0.0f);
				best.u = S.rf[lane].w;
				best.v = S.rd[lane].w;
				best.pid = (uint32_t)key;
			} else if (key != kNoHit) {
				// Compressed nodes (measured 1 % faster this way): the winner's test again.
				const uint32_t pid = (uint32_t)key;
				const float4 *p = tri4 + 3 * (size_t)__ldg(&sd.inv[pid]);
				const float4 A = __ldg(p), B = __ldg(p + 1), C = __ldg(p + 2);
				float t, u, v;
				if (tri_test(r, A, B, C, t, u, v, r.kind == 0 && tri_record_finite(B))) {
					best.t = t;
					best.u = u;
					best.v = v;
					best.pid = pid;
				}
			}
			const uint8_t *off = S.seg.off;
			uint8_t *rb = reinterpret_cast<uint8_t *>(stage) + lane * rec;
			if (fmask & PRT_FIELD_UV) {
				*reinterpret_cast<float *>(rb + off[PRT_OFF_U]) = best.u;
				*reinterpret_cast<float *>(rb + off[PRT_OFF_V]) = best.v;
			}
			if (fmask & PRT_FIELD_T)
				*reinterpret_cast<float *>(rb + off[PRT_OFF_T]) = best.t;
			if (fmask & PRT_FIELD_PRIMITIVE_ID)
				*reinterpret_cast<uint32_t *>(rb + off[PRT_OFF_PID]) = best.pid;
			if (fmask & PRT_FIELD_VALID)
				rb[off[PRT_OFF_VALID]] = best.t < INFINITY ? 1 : 0;
			if (fmask & PRT_FIELD_P) {
				// bvh.hpp:261-263: p = origin + t * direction, per component.
				*reinterpret_cast<float *>(rb + off[PRT_OFF_PX]) =
				    __fadd_rn(r.ox, __fmul_rn(best.t, r.dx));
				*reinterpret_cast<float *>(rb + off[PRT_OFF_PY]) =
				    __fadd_rn(r.oy, __fmul_rn(best.t, r.dy));
				*reinterpret_cast<float *>(rb + off[PRT_OFF_PZ]) =
				    __fadd_rn(r.oz, __fmul_rn(best.t, r.dz));
			}
		}
		__syncwarp();
		uint8_t *dst = S.seg.out + (size_t)local * rec;
		const uint32_t bytes = nb * rec;
		const uint32_t mode = S.seg.store_mode;
		if (mode == 0 && (bytes & 15u) == 0u) { // local is a multiple of 8: 16-byte aligned
			uint4 *d4 = reinterpret_cast<uint4 *>(dst);
			const uint4 *s4 = reinterpret_cast<const uint4 *>(stage);
			for (uint32_t k = lane; k < bytes / 16u; k += 32u)
				__stcs(d4 + k, s4[k]);
		} else if (mode <= 1) {
			uint32_t *d1 = reinterpret_cast<uint32_t *>(dst);
			for (uint32_t k = lane; k < bytes / 4u; k += 32u)
				d1[k] = stage[k];
		} else {
			const uint8_t *sb = reinterpret_cast<const uint8_t *>(stage);
			for (uint32_t k = lane; k < bytes; k += 32u)
				dst[k] = sb[k];
		}
		if (S.seg.done_ctr) {
			// The run's completion count (SegDesc): every lane's record stores are made
			// visible system-wide before lane 0 counts the batch; the batch that finishes
			// the run raises the host flag after another system fence.
			__threadfence_system();
			__syncwarp();
			if (lane == 0 && !fault) {
				const uint32_t before = atomicAdd(S.seg.done_ctr, nb);
				if (before + nb == run_rays) {
					__threadfence_system();
					*reinterpret_cast<volatile uint32_t *>(S.seg.done_flag) = 1u;
				}
			}
		}
		if (PASS == 3 && fault && lane == 0) {
			// The host learns of the fault at once (the run will never complete).
			__threadfence_system();
			*reinterpret_cast<volatile uint32_t *>(a.serve.err_flag) = 1u;
		}
		__syncwarp();
	}
	if (COUNT) {
		unsigned long long a0 = n_visits, a1 = n_tests;
		for (int o = 16; o > 0; o >>= 1) {
			a0 += __shfl_xor_sync(0xFFFFFFFFu, a0, o);
			a1 += __shfl_xor_sync(0xFFFFFFFFu, a1, o);
		}
		if (lane == 0) {
			atomicAdd(&a.visits[0], a0);
			atomicAdd(&a.visits[1], a1);
		}
	}
}

// Resident blocks per SM for `warps` warps of `warp_bytes` shared memory each, on the
// current device.  The kernel's dynamic shared-memory limit is a per-device attribute
// that only grows (under a lock), so a launch that another thread sized earlier still
// fits when this one needs less.
constexpr int kCachedDevices = 16;
template <int FMT, bool COUNT, bool LEAF1, bool BOUNDED, int PASS>
int blocks_per_sm(int warps, uint32_t warp_bytes) {
	struct Cache {
		int warps = -1;
		uint32_t bytes = 0;
		int blocks = 1;
		size_t limit = 0;
	};
	static std::mutex mu;
	static Cache cache[kCachedDevices];
	int dev = 0;
	cudaGetDevice(&dev);
	const size_t smem = (size_t)warp_bytes * warps;
	std::lock_guard<std::mutex> lk(mu);
	Cache uncached;
	Cache &c = (dev >= 0 && dev < kCachedDevices) ? cache[dev] : uncached;
	if (smem > c.limit &&
	    cudaFuncSetAttribute(k_trace8<FMT, COUNT, LEAF1, BOUNDED, PASS>,
	                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess)
		c.limit = smem;
	if (c.warps != warps || c.bytes != warp_bytes) {
		int b = 0;
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_trace8<FMT, COUNT, LEAF1, BOUNDED, PASS>,
		                                              32 * warps, smem);
		c.blocks = b > 0 ? b : 1;
		c.warps = warps;
		c.bytes = warp_bytes;
	}
	return c.blocks;
}

template <int FMT, bool COUNT, bool LEAF1, bool BOUNDED, int PASS>
void launch_t(const TravArgs &a, int warps, int sm_count, cudaStream_t st) {
	const int bps = blocks_per_sm<FMT, COUNT, LEAF1, BOUNDED, PASS>(warps, a.warp_bytes);
	const uint64_t batches = (a.n_virtual + a.batch - 1ull) / a.batch;
	// Unbounded warps: at most one block per resident slot (persistent).  Bounded: enough
	// blocks that every batch has a warp even if each warp takes its maximum.
	const uint64_t per_block = (uint64_t)warps * (BOUNDED ? a.max_batches : 1u);
	const uint64_t need = (batches + per_block - 1) / per_block;
	const uint64_t grid = BOUNDED ? need : std::min<uint64_t>((uint64_t)sm_count * bps, need);
	k_trace8<FMT, COUNT, LEAF1, BOUNDED, PASS>
	    <<<(unsigned)grid, 32 * warps, (size_t)a.warp_bytes * warps, st>>>(a);
}

template <int FMT, bool LEAF1>
void launch_passes(const TravArgs &a, int warps, int sm_count, cudaStream_t st) {
	if (a.max_batches > 0)
		launch_t<FMT, false, LEAF1, true, 1>(a, warps, sm_count, st);
	else
		launch_t<FMT, false, LEAF1, false, 1>(a, warps, sm_count, st);
	launch_t<FMT, false, LEAF1, false, 2>(a, warps, sm_count, st);
}

template <int FMT, bool COUNT>
void launch(const TravArgs &a, int warps, int sm_count, cudaStream_t st) {
	// A counting run is one general pass over all the work (no bounded warps).  So are
	// camera rays: the examples' cameras put a zero direction component in one batch of
	// every row, and finding those batches again costs the deferred pass a recomputation
	// of every ray.
	if (COUNT || a.use_cam) {
		if (a.max_leaf <= 1u)
			launch_t<FMT, COUNT, true, false, 0>(a, warps, sm_count, st);
		else
			launch_t<FMT, COUNT, false, false, 0>(a, warps, sm_count, st);
	} else if (a.max_leaf <= 1u) {
		launch_passes<FMT, true>(a, warps, sm_count, st);
	} else {
		launch_passes<FMT, false>(a, warps, sm_count, st);
	}
}

void size_smem(TravArgs &a, uint32_t depth, int leaf_size) {
	depth = std::max<uint32_t>(depth, 1u);
	a.pool_cap = std::max<uint32_t>(256u, 7u * kItems * (depth - 1u) + 2u * kItems);
	a.queue_cap = 32u + (uint32_t)kItems * 8u * (uint32_t)std::max(leaf_size, 1);
	a.max_leaf = (uint32_t)std::max(leaf_size, 1);
	a.max_batches = 0;
	a.warp_bytes = (warp_smem_bytes(a.pool_cap, a.queue_cap) + 15u) & ~15u;
}

// Rays per warp batch for one run of m rays: 32 when the launch holds at least two
// batches for every resident warp (about 36 per SM), else 16, else 8: a small query
// then spreads over all warps instead of leaving most of them idle while a few walk 32
// rays each (bounded waves keep 32: their batch count per warp is the caller's).
uint32_t batch_rays(uint64_t m, int sm_count, uint32_t max_batches) {
	const uint64_t wave = (uint64_t)std::max(sm_count, 1) * 36u * 32u;
	if (max_batches > 0 || m >= 2 * wave)
		return 32;
	return m >= wave ? 16 : 8;
}

int warps_for(const TravConfig &cfg) {
	return (cfg.block >= 32 && cfg.block <= 32 * kWarpsPerBlock && cfg.block % 32 == 0)
	           ? cfg.block / 32
	           : kWarpsPerBlock;
}

cudaError_t dispatch(const TravArgs &a, const TravConfig &cfg, int sm_count, cudaStream_t st) {
	cudaError_t e = cudaMemsetAsync(a.counter, 0, 4, st);
	if (e == cudaSuccess)
		e = cudaMemsetAsync(a.deferred, 0, 8, st);
	if (e != cudaSuccess)
		return e;
	const int warps = warps_for(cfg);
	if (cfg.format == PRT_NODES_COMPRESSED) {
		if (cfg.count)
			launch<PRT_NODES_COMPRESSED, true>(a, warps, sm_count, st);
		else
			launch<PRT_NODES_COMPRESSED, false>(a, warps, sm_count, st);
	} else {
		if (cfg.count)
			launch<PRT_NODES_FP32, true>(a, warps, sm_count, st);
		else
			launch<PRT_NODES_FP32, false>(a, warps, sm_count, st);
	}
	return cudaGetLastError();
}

} // namespace

int traversal_stack_depth() { return kMaxDepth; }

cudaError_t launch_nearest_hits(const SceneGPU &sc, const float *d_rays, uint64_t n,
                                const OutLayout &lay, void *d_out, const TravConfig &cfg,
                                uint32_t *d_work, unsigned long long *d_visits, uint32_t *d_err,
                                cudaStream_t st, int sm_count, const prt_b200_camera *cam) {
	if (cfg.count)
		cudaMemsetAsync(d_visits, 0, 2 * sizeof(unsigned long long), st);
	const uint64_t chunk = 1ull << 31;
	if (cam && n > chunk)
		return cudaErrorInvalidValue; // camera rays are numbered within one launch
	for (uint64_t s = 0; s < n; s += chunk) {
		const uint64_t m = std::min(chunk, n - s);
		TravArgs a;
		a.use_cam = cam ? 1u : 0u;
		if (cam)
			a.cam = *cam;
		a.scenes = nullptr;
		a.segs = nullptr;
		a.n_segs = 0;
		a.n_virtual = (uint32_t)m;
		a.scene0.tri4 = sc.tri4.as<float4>();
		a.scene0.inv = sc.inv.as<uint32_t>();
		a.scene0.nodes = cfg.format == PRT_NODES_COMPRESSED ? sc.cnodes.p : sc.nodes.p;
		a.scene0.root = 0;
		a.scene0.n_tris = (uint32_t)sc.n_tris;
		a.seg0.vbegin = 0;
		a.seg0.rays = cam ? nullptr : d_rays + 6 * s;
		a.seg0.out = static_cast<uint8_t *>(d_out) + s * lay.rec_size;
		a.seg0.n_rays = (uint32_t)m;
		a.seg0.scene = 0;
		a.seg0.mask = lay.mask;
		a.seg0.rec_size = lay.rec_size;
		for (int k = 0; k < 8; ++k)
			a.seg0.off[k] = lay.off[k];
		a.seg0.store_mode = store_mode_for(a.seg0.out);
		a.seg0.pad = 0;
		a.n_nodes = sc.n_nodes;
		a.dead = sc.dead;
		size_smem(a, cfg.pool_depth ? (uint32_t)cfg.pool_depth : sc.depth, sc.leaf_size);
		a.max_batches = cfg.max_batches;
		a.batch = batch_rays(m, sm_count, cfg.max_batches);
		a.counter = d_work;
		a.deferred = d_work + 2;
		a.err = d_err;
		a.visits = d_visits;
		cudaError_t e = dispatch(a, cfg, sm_count, st);
		if (e != cudaSuccess)
			return e;
	}
	return cudaSuccess;
}

cudaError_t launch_nearest_hits_segments(const SceneDesc *d_scenes, const SegDesc *d_segs,
                                         uint32_t n_segs, unsigned long long n_virtual,
                                         uint32_t depth, int leaf_size, uint32_t n_nodes,
                                         uint32_t dead, const TravConfig &cfg,
                                         uint32_t *d_work, unsigned long long *d_visits,
                                         uint32_t *d_err, cudaStream_t st, int sm_count) {
	if (cfg.count)
		cudaMemsetAsync(d_visits, 0, 2 * sizeof(unsigned long long), st);
	if (n_segs == 0 || n_virtual == 0)
		return cudaSuccess;
	if (n_virtual > (1ull << 31))
		return cudaErrorInvalidValue;
	TravArgs a;
	memset(&a, 0, sizeof a);
	a.scenes = d_scenes;
	a.segs = d_segs;
	a.n_segs = n_segs;
	a.n_virtual = (uint32_t)n_virtual;
	a.n_nodes = n_nodes;
	a.dead = dead;
	size_smem(a, cfg.pool_depth ? (uint32_t)cfg.pool_depth : depth, leaf_size);
	a.max_batches = cfg.max_batches;
	a.batch = 32; // runs are padded to whole warps of 32
	a.counter = d_work;
	a.deferred = d_work + 2;
	a.err = d_err;
	a.visits = d_visits;
	return dispatch(a, cfg, sm_count, st);
}

namespace {

template <int FMT, bool LEAF1>
void launch_serving_t(const TravArgs &a, int sm_count, cudaStream_t st) {
	const int bps = blocks_per_sm<FMT, false, LEAF1, false, 3>(kWarpsPerBlock, a.warp_bytes);
	k_trace8<FMT, false, LEAF1, false, 3>
	    <<<(unsigned)(sm_count * bps), 32 * kWarpsPerBlock, (size_t)a.warp_bytes * kWarpsPerBlock,
	       st>>>(a);
}

} // namespace

cudaError_t launch_serving(const SceneDesc *d_scenes, const ServeQueues &q, uint32_t depth,
                           int leaf_size, uint32_t n_nodes, uint32_t dead, int format,
                           uint32_t *d_err, cudaStream_t st, int sm_count) {
	TravArgs a;
	memset(&a, 0, sizeof a);
	a.scenes = d_scenes;
	a.serve = q;
	a.n_nodes = n_nodes;
	a.dead = dead;
	size_smem(a, depth, leaf_size);
	a.batch = 32; // one ticket = 32 rays
	a.err = d_err;
	// Every resident slot: the warps poll for work, none waits for another, so the
	// launch needs no co-residency (blocks that do not fit start as others leave).
	if (format == PRT_NODES_COMPRESSED) {
		if (a.max_leaf <= 1u)
			launch_serving_t<PRT_NODES_COMPRESSED, true>(a, sm_count, st);
		else
			launch_serving_t<PRT_NODES_COMPRESSED, false>(a, sm_count, st);
	} else {
		if (a.max_leaf <= 1u)
			launch_serving_t<PRT_NODES_FP32, true>(a, sm_count, st);
		else
			launch_serving_t<PRT_NODES_FP32, false>(a, sm_count, st);
	}
	return cudaGetLastError();
}

} // namespace prt
