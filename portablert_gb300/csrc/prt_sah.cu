// prt_sah.cu - binned-SAH construction of the binary tree, the alternative to the
// Morton/Karras hierarchy of prt_build.cu for a scene that is built once and queried
// many times.
//
// portableRT's own build (bvh.hpp:58-193) splits each node top-down at the best of a
// few binned surface-area-heuristic planes; this is the same kind of tree, built
// breadth-first on the GPU.  Every node is a contiguous range of a permutation of the
// scene's triangles, so the outputs are exactly what the LBVH path hands the collapse:
// the final order (vals), leaf boxes in that order, children, leaf ranges and node
// boxes with the children's surface areas in the w slots.  The answers do not depend on
// the tree (the traversal examines every triangle whose box the ray passes); only the
// number of boxes a ray passes does, which is what the heuristic minimises.
//
// Tasks are ranges still to be split, in three tiers by size:
//   large (> 512 triangles): per level, blocks bin chunks of 2048 triangles into the
//         task's 3 x 32 global bins (k_sah_bin), one warp per task picks the plane
//         (k_sah_split), blocks scatter the triangles to the other buffer (k_sah_part);
//   mid   (33-512): one warp per task per level does all three in shared memory with a
//         stable ballot partition (k_sah_mid);
//   small (<= 32): one warp builds the whole subtree, one triangle per lane, with an
//         exact sweep over the sorted centres of each axis (k_sah_small).
// Binning uses box centres; a task deeper than 48 levels, or one whose centres all fall
// into one bin on every axis, is split into halves instead.  All positions, node ids and
// list slots are checked before they are written; a failed check sets kErrSah.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"
#include "prt_sah.cuh"

namespace prt {
namespace {

constexpr int kBins = 32;
constexpr uint32_t kLarge = 512;    // larger tasks are binned by many blocks (512 / 1,024
                                    // / 4,096: heightfield build 3.05 / 3.16 / 3.83 ms)
constexpr uint32_t kSmall = 32;     // tasks up to this size go to one warp each
constexpr uint32_t kChunk = 2048;   // triangles per binning / partition block
constexpr uint32_t kDepthGuard = 48;
constexpr int kMaxLevels = 96;
constexpr int kLevelsPerCheck = 4;
constexpr int kBinWords = 3 * kBins * 7; // per axis and bin: lo xyz, hi xyz (ordered), count
constexpr uint32_t kOrdPosInf = 0xFF800000u; // f2ord(+inf)
constexpr uint32_t kOrdNegInf = 0x007FFFFFu; // f2ord(-inf)
constexpr uint32_t kHalves = 3;              // split "axis" meaning: first half / second half

// Counter words.
enum : int {
	kCtrLarge = 0, // [0], [1]: large tasks per list parity
	kCtrMid = 2,   // [2], [3]: mid tasks per list parity
	kCtrSmall = 4,
	kCtrNodes = 5,
	kCtrChunks = 6,
	kCtrWordsSah = 8
};
static_assert(kCtrWordsSah + 1 <= kHostSahWords, "the SAH counters' pinned words");

struct alignas(16) SahTask {
	uint32_t begin, count, node, parent; // parent = (node << 1 | side), kNone at a root
	uint32_t meta;                       // bit 0: buffer holding the range; bits 8-15: depth
	uint32_t axis, split, n_left;        // the split chosen (large tasks)
	float lo[3];
	uint32_t cur_l;                      // partition cursors (large tasks)
	float scale[3];
	uint32_t cur_r;
};
static_assert(sizeof(SahTask) == 64, "task layout");

struct alignas(16) SmallTask {
	uint32_t begin, meta, node, parent;  // meta: count | buffer << 8 | depth << 16
};

struct SahArgs {
	float4 *rec[2];         // (lo, id) (hi, 0) per triangle, two buffers
	SahTask *large[2];
	uint32_t *bins[2];      // kBinWords per large task
	SahTask *mid[2];
	SmallTask *small;
	uint32_t *chunk_off;    // per large task of the level: first chunk
	uint32_t *ctr;
	uint32_t *vals;         // out: position -> triangle index
	float4 *lbox;           // out: leaf boxes by position
	uint32_t *left, *right, *rfirst, *rlast;
	float4 *ibox;
	uint32_t *parent_int, *parent_leaf; // for the bottom-up cost pass of the collapse
	uint32_t node_cap, max_large, max_mid, max_small;
	uint32_t n;             // triangles (records per buffer)
	uint32_t *err;
};

// Task counts clamped to the list capacities (a list that overflowed was flagged).
__device__ __forceinline__ uint32_t n_large(const SahArgs &A, int par) {
	return min(A.ctr[kCtrLarge + par], A.max_large);
}
__device__ __forceinline__ uint32_t n_mid(const SahArgs &A, int par) {
	return min(A.ctr[kCtrMid + par], A.max_mid);
}

__device__ __forceinline__ bool range_ok(const SahArgs &A, uint32_t begin, uint32_t count) {
	return begin <= A.n && count <= A.n - begin && count >= 2;
}

__device__ __forceinline__ float centre(float lo, float hi) {
	return __fadd_rn(__fmul_rn(lo, 0.5f), __fmul_rn(hi, 0.5f));
}

__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
	const float t = __fmul_rn(__fsub_rn(c, lo), scale);
	return (int)fminf(fmaxf(t, 0.0f), (float)(kBins - 1)); // NaN -> 0
}

__device__ __forceinline__ float frame_scale(float lo, float hi) {
	const float e = hi - lo;
	return (e > 0.0f && isfinite(e)) ? (float)kBins / e : 0.0f;
}

__device__ __forceinline__ float area3(float lx, float ly, float lz, float hx, float hy,
                                       float hz) {
	const float dx = hx - lx, dy = hy - ly, dz = hz - lz;
	const float a = dx * dy + dx * dz + dy * dz;
	return isfinite(a) ? a : FLT_MAX;
}

__device__ __forceinline__ float rec_c(const float4 &lo, const float4 &hi, int k) {
	return k == 0 ? centre(lo.x, hi.x) : (k == 1 ? centre(lo.y, hi.y) : centre(lo.z, hi.z));
}

__device__ __forceinline__ void flag(uint32_t *err) { atomicOr(err, kErrSah); }

__device__ __forceinline__ void bins_init(uint32_t *b, int lane) {
	for (int k = lane; k < kBinWords; k += 32) {
		const int w = k % 7;
		b[k] = w < 3 ? kOrdPosInf : (w < 6 ? kOrdNegInf : 0u);
	}
}

// Adds each valid lane's triangle to the bins of all three axes (shared or global
// words).  Counts go in once per group of lanes with the same bin; bounds only when
// they improve what is there.
__device__ __forceinline__ void bins_add(uint32_t *b, bool valid, const float4 &lo,
                                         const float4 &hi, const float *flo, const float *fsc,
                                         int lane) {
#pragma unroll
	for (int a = 0; a < 3; ++a) {
		const int bin = valid ? bin_of(rec_c(lo, hi, a), flo[a], fsc[a]) : -1;
		const uint32_t g = __match_any_sync(0xFFFFFFFFu, bin);
		if (!valid)
			continue;
		uint32_t *w = b + (a * kBins + bin) * 7;
		if (lane == __ffs(g) - 1)
			atomicAdd(&w[6], (uint32_t)__popc(g));
		const uint32_t v[6] = {f2ord(lo.x), f2ord(lo.y), f2ord(lo.z),
		                       f2ord(hi.x), f2ord(hi.y), f2ord(hi.z)};
#pragma unroll
		for (int k = 0; k < 3; ++k)
			if (v[k] < *(volatile uint32_t *)&w[k])
				atomicMin(&w[k], v[k]);
#pragma unroll
		for (int k = 3; k < 6; ++k)
			if (v[k] > *(volatile uint32_t *)&w[k])
				atomicMax(&w[k], v[k]);
	}
}

struct Box6 {
	float lx, ly, lz, hx, hy, hz;
};

__device__ __forceinline__ Box6 box_union(const Box6 &a, const Box6 &b) {
	return Box6{fminf(a.lx, b.lx), fminf(a.ly, b.ly), fminf(a.lz, b.lz),
	            fmaxf(a.hx, b.hx), fmaxf(a.hy, b.hy), fmaxf(a.hz, b.hz)};
}

__device__ __forceinline__ Box6 shfl_box(const Box6 &b, int src) {
	return Box6{__shfl_sync(0xFFFFFFFFu, b.lx, src), __shfl_sync(0xFFFFFFFFu, b.ly, src),
	            __shfl_sync(0xFFFFFFFFu, b.lz, src), __shfl_sync(0xFFFFFFFFu, b.hx, src),
	            __shfl_sync(0xFFFFFFFFu, b.hy, src), __shfl_sync(0xFFFFFFFFu, b.hz, src)};
}

__device__ __forceinline__ Box6 empty_box() {
	return Box6{INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
}

__device__ __forceinline__ float box_area(const Box6 &b) {
	return area3(b.lx, b.ly, b.lz, b.hx, b.hy, b.hz);
}

// Union over the lanes in [a, b) of the warp (every lane calls).
__device__ __forceinline__ Box6 range_box(const Box6 &mine, int lane, int a, int b) {
	Box6 x = (lane >= a && lane < b) ? mine : empty_box();
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		Box6 y{__shfl_xor_sync(0xFFFFFFFFu, x.lx, o), __shfl_xor_sync(0xFFFFFFFFu, x.ly, o),
		       __shfl_xor_sync(0xFFFFFFFFu, x.lz, o), __shfl_xor_sync(0xFFFFFFFFu, x.hx, o),
		       __shfl_xor_sync(0xFFFFFFFFu, x.hy, o), __shfl_xor_sync(0xFFFFFFFFu, x.hz, o)};
		x = box_union(x, y);
	}
	return x;
}

struct Split {
	uint32_t axis, bin, n_left; // axis kHalves: no plane
	Box6 node, left, right;     // left / right valid for a binned split
};

// The best plane over the three axes' bins (lane = bin).  Ties go to the lower axis,
// then the lower bin.  Every lane returns the same result.
__device__ Split choose_split(const uint32_t *b, const float *fsc, uint32_t count, int lane) {
	Split s;
	s.axis = kHalves;
	s.bin = 0;
	s.n_left = count / 2;
	uint64_t best = ~0ull;
	for (int a = 0; a < 3; ++a) {
		const uint32_t *w = b + (a * kBins + lane) * 7;
		Box6 p{ord2f(w[0]), ord2f(w[1]), ord2f(w[2]), ord2f(w[3]), ord2f(w[4]), ord2f(w[5])};
		uint32_t pc = w[6];
		Box6 q = p;
		uint32_t qc = pc;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const Box6 pu = shfl_box(p, max(lane - o, 0));
			const uint32_t pcu = __shfl_up_sync(0xFFFFFFFFu, pc, o);
			const Box6 qd = shfl_box(q, min(lane + o, 31));
			const uint32_t qcd = __shfl_down_sync(0xFFFFFFFFu, qc, o);
			if (lane >= o) {
				p = box_union(p, pu);
				pc += pcu;
			}
			if (lane + o < 32) {
				q = box_union(q, qd);
				qc += qcd;
			}
		}
		if (a == 0)
			s.node = shfl_box(p, 31);
		const Box6 r = shfl_box(q, min(lane + 1, 31));
		const uint32_t rc = __shfl_down_sync(0xFFFFFFFFu, qc, 1);
		// The least cost on this axis, then the lowest plane with it (two redux.sync
		// minima).
		uint32_t c32 = 0xFFFFFFFFu;
		if (fsc[a] > 0.0f && lane < 31 && pc > 0 && rc > 0)
			c32 = f2ord(box_area(p) * (float)pc + box_area(r) * (float)rc);
		const uint32_t cmin = __reduce_min_sync(0xFFFFFFFFu, c32);
		const uint32_t plane = __reduce_min_sync(
		    0xFFFFFFFFu, (c32 == cmin && c32 != 0xFFFFFFFFu) ? (uint32_t)lane : 0xFFu);
		const uint64_t key =
		    cmin == 0xFFFFFFFFu ? ~0ull : (((uint64_t)cmin << 32) | ((uint32_t)a << 8) | plane);
		if (key < best) {
			best = key;
			const int src = (int)(key & 0xFF);
			s.axis = (uint32_t)a;
			s.bin = (uint32_t)src;
			s.n_left = __shfl_sync(0xFFFFFFFFu, pc, src);
			s.left = shfl_box(p, src);
			s.right = shfl_box(r, src);
		}
	}
	return s;
}

__device__ __forceinline__ void write_node_box(const SahArgs &A, uint32_t node, const Box6 &b,
                                               float wl, float wr) {
	A.ibox[2 * (size_t)node] = make_float4(b.lx, b.ly, b.lz, wl);
	A.ibox[2 * (size_t)node + 1] = make_float4(b.hx, b.hy, b.hz, wr);
}

__device__ __forceinline__ void write_parent_area(const SahArgs &A, uint32_t parent, float a) {
	if (parent != kNone)
		reinterpret_cast<float *>(&A.ibox[2 * (size_t)(parent >> 1) + (parent & 1u)])[3] = a;
}

__device__ __forceinline__ uint32_t new_node(const SahArgs &A, uint32_t k) {
	const uint32_t id = atomicAdd(&A.ctr[kCtrNodes], k);
	if (id + k > A.node_cap) {
		flag(A.err);
		return kNone;
	}
	return id;
}

// Files a child range as a task of the right tier (called by one lane).  `frame` gives
// the binning frame of a large child.  Returns the list slot of a large child, whose
// bins the calling warp then clears (init_new_bins), else kNone.
__device__ uint32_t add_child(const SahArgs &A, int out_par, uint32_t begin, uint32_t count,
                              uint32_t node, uint32_t parent, uint32_t buf, uint32_t depth,
                              const Box6 *frame, const float *pflo, const float *pfsc) {
	if (count > kLarge) {
		const uint32_t i = atomicAdd(&A.ctr[kCtrLarge + out_par], 1u);
		if (i >= A.max_large) {
			flag(A.err);
			return kNone;
		}
		SahTask t;
		t.begin = begin;
		t.count = count;
		t.node = node;
		t.parent = parent;
		t.meta = buf | (depth << 8);
		t.axis = kHalves;
		t.split = 0;
		t.n_left = 0;
		if (frame) {
			t.lo[0] = frame->lx;
			t.lo[1] = frame->ly;
			t.lo[2] = frame->lz;
			t.scale[0] = frame_scale(frame->lx, frame->hx);
			t.scale[1] = frame_scale(frame->ly, frame->hy);
			t.scale[2] = frame_scale(frame->lz, frame->hz);
		} else {
			for (int k = 0; k < 3; ++k) {
				t.lo[k] = pflo[k];
				t.scale[k] = pfsc[k];
			}
		}
		t.cur_l = t.cur_r = 0;
		A.large[out_par][i] = t;
		return i;
	} else if (count > kSmall) {
		const uint32_t i = atomicAdd(&A.ctr[kCtrMid + out_par], 1u);
		if (i >= A.max_mid) {
			flag(A.err);
			return kNone;
		}
		SahTask t;
		memset(&t, 0, sizeof(t));
		t.begin = begin;
		t.count = count;
		t.node = node;
		t.parent = parent;
		t.meta = buf | (depth << 8);
		A.mid[out_par][i] = t;
	} else {
		const uint32_t i = atomicAdd(&A.ctr[kCtrSmall], 1u);
		if (i >= A.max_small) {
			flag(A.err);
			return kNone;
		}
		A.small[i] = SmallTask{begin, count | (buf << 8) | (depth << 16), node, parent};
	}
	return kNone;
}

// Clears the bins of the large tasks that lane `from_lane`'s add_child calls filed
// (their slots); the whole warp calls this, 21 words per lane and task.  A single lane
// clearing the 672 words of two children took most of k_sah_split's time.
__device__ __forceinline__ void init_new_bins(const SahArgs &A, int out_par, uint32_t slot_a,
                                              uint32_t slot_b, int from_lane, int lane) {
	slot_a = __shfl_sync(0xFFFFFFFFu, slot_a, from_lane);
	slot_b = __shfl_sync(0xFFFFFFFFu, slot_b, from_lane);
	if (slot_a != kNone)
		bins_init(A.bins[out_par] + (size_t)slot_a * kBinWords, lane);
	if (slot_b != kNone)
		bins_init(A.bins[out_par] + (size_t)slot_b * kBinWords, lane);
}

// Writes node `t.node` (box, children, range) for split `s` and files both children
// (lane 0 only).  Children whose range holds one triangle are leaves.  slots[] receive
// the list slots of children filed as large tasks (kNone otherwise).
__device__ void emit_split(const SahArgs &A, const SahTask &t, const Split &s, int out_par,
                           const float *flo, const float *fsc, uint32_t slots[2]) {
	const uint32_t buf = (t.meta & 1u) ^ 1u, depth = ((t.meta >> 8) & 0xFFu) + 1u;
	const uint32_t nl = s.n_left, nr = t.count - s.n_left;
	slots[0] = slots[1] = kNone;
	if (nl == 0 || nl >= t.count || t.node == kNone || t.node >= A.node_cap) {
		flag(A.err);
		return;
	}
	const bool binned = s.axis != kHalves;
	uint32_t ids[2] = {kNone, kNone};
	const uint32_t need = (nl > 1) + (nr > 1);
	if (need) {
		const uint32_t id = new_node(A, need);
		if (id == kNone)
			return;
		uint32_t k = 0;
		if (nl > 1)
			ids[0] = id + k++;
		if (nr > 1)
			ids[1] = id + k;
	}
	const uint32_t rl = nl > 1 ? ids[0] : (kLeafBit | t.begin);
	const uint32_t rr = nr > 1 ? ids[1] : (kLeafBit | (t.begin + nl));
	A.left[t.node] = rl;
	A.right[t.node] = rr;
	A.rfirst[t.node] = t.begin;
	A.rlast[t.node] = t.begin + t.count - 1u;
	if (nl > 1)
		A.parent_int[ids[0]] = t.node;
	else
		A.parent_leaf[t.begin] = t.node;
	if (nr > 1)
		A.parent_int[ids[1]] = t.node;
	else
		A.parent_leaf[t.begin + nl] = t.node;
	// Children's areas: known now for a binned split (leaves keep -1); after halves each
	// child writes its own when it is split.
	write_node_box(A, t.node, s.node, (binned && nl > 1) ? box_area(s.left) : -1.0f,
	               (binned && nr > 1) ? box_area(s.right) : -1.0f);
	const uint32_t pl = binned ? kNone : (t.node << 1), pr = binned ? kNone : ((t.node << 1) | 1u);
	slots[0] = add_child(A, out_par, t.begin, nl, ids[0], pl, buf, depth,
	                     binned ? &s.left : nullptr, flo, fsc);
	slots[1] = add_child(A, out_par, t.begin + nl, nr, ids[1], pr, buf, depth,
	                     binned ? &s.right : nullptr, flo, fsc);
}

// ---------------------------------------------------------------------------------------
// Set-up: records, per-scene centre bounds, root tasks.

__global__ void k_sah_records(const float *__restrict__ tris, uint32_t n,
                              const uint32_t *__restrict__ scene_of, float4 *rec, uint32_t *gb) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	const int lane = threadIdx.x & 31;
	const bool live = i < n;
	float4 lo = make_float4(0, 0, 0, 0), hi = lo;
	uint32_t s = 0;
	if (live) {
		const float *t = tris + 9 * (size_t)i;
		bool fin = true;
#pragma unroll
		for (int k = 0; k < 9; ++k)
			fin = fin && isfinite(t[k]);
		if (fin) {
			lo = make_float4(fminf(t[0], fminf(t[3], t[6])), fminf(t[1], fminf(t[4], t[7])),
			                 fminf(t[2], fminf(t[5], t[8])), __uint_as_float(i));
			hi = make_float4(fmaxf(t[0], fmaxf(t[3], t[6])), fmaxf(t[1], fmaxf(t[4], t[7])),
			                 fmaxf(t[2], fmaxf(t[5], t[8])), 0.0f);
		} else {
			lo = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, __uint_as_float(i));
			hi = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f);
		}
		rec[2 * (size_t)i] = lo;
		rec[2 * (size_t)i + 1] = hi;
		s = scene_of ? scene_of[i] : 0u;
	}
	float mn[3], mx[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		const float c = rec_c(lo, hi, k);
		mn[k] = live ? c : INFINITY;
		mx[k] = live ? c : -INFINITY;
	}
	if (!scene_of) {
		// One scene: warps reduce, then the block, and one thread updates the six words
		// (one set of same-address atomics per block instead of per warp: with 32k warps
		// on a 1M-triangle scene those atomics were most of this kernel's time).
		__shared__ float red[32][6];
#pragma unroll
		for (int k = 0; k < 3; ++k)
			for (int o = 16; o > 0; o >>= 1) {
				mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
				mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
			}
		const int w = threadIdx.x >> 5;
		if (lane == 0)
			for (int k = 0; k < 3; ++k) {
				red[w][k] = mn[k];
				red[w][3 + k] = mx[k];
			}
		__syncthreads();
		if (threadIdx.x < 6) {
			const int k = threadIdx.x;
			float v = red[0][k];
			for (int j = 1; j < (int)(blockDim.x >> 5); ++j)
				v = k < 3 ? fminf(v, red[j][k]) : fmaxf(v, red[j][k]);
			if (k < 3 && v != INFINITY)
				atomicMin(&gb[k], f2ord(v));
			else if (k >= 3 && v != -INFINITY)
				atomicMax(&gb[k], f2ord(v));
		}
		return;
	}
	const uint32_t s0 = __shfl_sync(0xFFFFFFFFu, s, 0);
	if (__all_sync(0xFFFFFFFFu, !live || s == s0)) {
#pragma unroll
		for (int k = 0; k < 3; ++k)
			for (int o = 16; o > 0; o >>= 1) {
				mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
				mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
			}
		if (lane == 0 && mn[0] <= mx[0])
			for (int k = 0; k < 3; ++k) {
				atomicMin(&gb[6 * s0 + k], f2ord(mn[k]));
				atomicMax(&gb[6 * s0 + 3 + k], f2ord(mx[k]));
			}
	} else if (live) {
		for (int k = 0; k < 3; ++k) {
			atomicMin(&gb[6 * s + k], f2ord(mn[k]));
			atomicMax(&gb[6 * s + 3 + k], f2ord(mx[k]));
		}
	}
}

__global__ void k_sah_first_id(uint32_t *ctr, uint32_t S) { ctr[kCtrNodes] = S; }

// One warp per scene: lane 0 files the root task, the warp clears a large root's bins.
__global__ void k_sah_roots(SahArgs A, const uint32_t *__restrict__ tri_off, uint32_t n_scenes,
                            const uint32_t *__restrict__ gb, uint32_t *roots) {
	const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int lane = threadIdx.x & 31;
	if (s >= n_scenes)
		return;
	const uint32_t b = tri_off[s], n = tri_off[s + 1] - b;
	uint32_t slot = kNone;
	if (lane == 0) {
		roots[s] = s;
		if (n) {
			float flo[3], fsc[3];
			for (int k = 0; k < 3; ++k) {
				flo[k] = ord2f(gb[6 * s + k]);
				fsc[k] = frame_scale(flo[k], ord2f(gb[6 * s + 3 + k]));
			}
			slot = add_child(A, 0, b, n, n > 1 ? s : kNone, kNone, 0u, 0u, nullptr, flo, fsc);
		}
	}
	init_new_bins(A, 0, slot, kNone, 0, lane);
}

// ---------------------------------------------------------------------------------------
// Large tasks.

// First chunk of each large task of the level and the chunk total; clears the lists
// the level fills.  One block.
__global__ void __launch_bounds__(1024) k_sah_chunks(SahArgs A, int par) {
	__shared__ uint32_t warp_sum[32];
	__shared__ uint32_t carry;
	const uint32_t n = n_large(A, par);
	if (threadIdx.x == 0) {
		carry = 0;
		A.ctr[kCtrLarge + (par ^ 1)] = 0;
		A.ctr[kCtrMid + (par ^ 1)] = 0;
	}
	__syncthreads();
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	for (uint32_t base = 0; base < n; base += blockDim.x) {
		const uint32_t i = base + threadIdx.x;
		uint32_t c = 0;
		if (i < n) {
			const SahTask &t = A.large[par][i];
			c = range_ok(A, t.begin, t.count) ? (t.count + kChunk - 1) / kChunk : 0u;
		}
		uint32_t x = c;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
			if (lane >= o)
				x += y;
		}
		if (lane == 31)
			warp_sum[w] = x;
		__syncthreads();
		if (w == 0) {
			uint32_t v = lane < (int)(blockDim.x >> 5) ? warp_sum[lane] : 0u;
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
				if (lane >= o)
					v += y;
			}
			warp_sum[lane] = v;
		}
		__syncthreads();
		const uint32_t before = (w ? warp_sum[w - 1] : 0u) + x - c;
		if (i < n)
			A.chunk_off[i] = carry + before;
		__syncthreads();
		if (threadIdx.x == 0)
			carry += warp_sum[(blockDim.x >> 5) - 1];
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		A.chunk_off[n] = carry;
		A.ctr[kCtrChunks] = carry;
	}
}

__device__ __forceinline__ uint32_t task_of_chunk(const uint32_t *off, uint32_t n, uint32_t c) {
	uint32_t lo = 0, hi = n; // off[lo] <= c < off[hi]
	while (hi - lo > 1) {
		const uint32_t m = (lo + hi) >> 1;
		if (off[m] <= c)
			lo = m;
		else
			hi = m;
	}
	return lo;
}

__global__ void __launch_bounds__(256) k_sah_bin(SahArgs A, int par) {
	__shared__ uint32_t sb[kBinWords];
	const uint32_t n_tasks = n_large(A, par), n_chunks = A.ctr[kCtrChunks];
	const int lane = threadIdx.x & 31;
	for (uint32_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
		const uint32_t ti = task_of_chunk(A.chunk_off, n_tasks, c);
		const SahTask &t = A.large[par][ti];
		const uint32_t lo_i = t.begin + (c - A.chunk_off[ti]) * kChunk;
		const uint32_t hi_i = min(lo_i + kChunk, t.begin + t.count);
		const float4 *src = A.rec[t.meta & 1u];
		float flo[3], fsc[3];
		for (int k = 0; k < 3; ++k) {
			flo[k] = t.lo[k];
			fsc[k] = t.scale[k];
		}
		for (int k = threadIdx.x; k < kBinWords; k += blockDim.x) {
			const int w = k % 7;
			sb[k] = w < 3 ? kOrdPosInf : (w < 6 ? kOrdNegInf : 0u);
		}
		__syncthreads();
		for (uint32_t i0 = lo_i + (threadIdx.x & ~31u); i0 < hi_i; i0 += blockDim.x) {
			const uint32_t i = i0 + lane;
			const bool v = i < hi_i;
			float4 lo = make_float4(0, 0, 0, 0), hi = lo;
			if (v) {
				lo = src[2 * (size_t)i];
				hi = src[2 * (size_t)i + 1];
			}
			bins_add(sb, v, lo, hi, flo, fsc, lane);
		}
		__syncthreads();
		uint32_t *gbins = A.bins[par] + (size_t)ti * kBinWords;
		for (int k = threadIdx.x; k < kBinWords; k += blockDim.x) {
			const int w = k % 7;
			const uint32_t cnt = sb[k - w + 6];
			if (cnt == 0)
				continue;
			if (w < 3)
				atomicMin(&gbins[k], sb[k]);
			else if (w < 6)
				atomicMax(&gbins[k], sb[k]);
			else
				atomicAdd(&gbins[k], cnt);
		}
		__syncthreads();
	}
}

// One warp per large task: the plane, the node and the child tasks.
__global__ void __launch_bounds__(128) k_sah_split(SahArgs A, int par) {
	const uint32_t n_tasks = n_large(A, par);
	const int lane = threadIdx.x & 31;
	for (uint32_t ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; ti < n_tasks;
	     ti += (gridDim.x * blockDim.x) >> 5) {
		SahTask &tr = A.large[par][ti];
		const SahTask t = tr;
		if (!range_ok(A, t.begin, t.count)) {
			if (lane == 0)
				flag(A.err);
			continue;
		}
		const uint32_t *b = A.bins[par] + (size_t)ti * kBinWords;
		float flo[3], fsc[3];
		for (int k = 0; k < 3; ++k) {
			flo[k] = t.lo[k];
			fsc[k] = t.scale[k];
		}
		Split s = choose_split(b, fsc, t.count, lane);
		uint32_t slots[2] = {kNone, kNone};
		uint32_t total = b[lane * 7 + 6]; // the axis-0 bins hold every triangle once
		for (int o = 16; o > 0; o >>= 1)
			total += __shfl_xor_sync(0xFFFFFFFFu, total, o);
		if (((t.meta >> 8) & 0xFFu) >= kDepthGuard) {
			s.axis = kHalves;
			s.n_left = t.count / 2;
		}
		if (lane == 0 && total != t.count) {
			// Nothing placed: the partition then writes no triangle of this task.
			flag(A.err);
			tr.axis = kHalves;
			tr.n_left = 0;
			tr.cur_l = tr.cur_r = A.n;
		} else if (lane == 0) {
			write_parent_area(A, t.parent, box_area(s.node));
			tr.axis = s.axis;
			tr.split = s.bin;
			tr.n_left = s.n_left;
			tr.cur_l = t.begin;
			tr.cur_r = t.begin + s.n_left;
			emit_split(A, t, s, par ^ 1, flo, fsc, slots);
		}
		init_new_bins(A, par ^ 1, slots[0], slots[1], 0, lane);
	}
}

// Scatters the triangles of the large tasks to the other buffer, left side first.
__global__ void __launch_bounds__(256) k_sah_part(SahArgs A, int par) {
	const uint32_t n_tasks = n_large(A, par), n_chunks = A.ctr[kCtrChunks];
	const int lane = threadIdx.x & 31;
	const uint32_t lt = (1u << lane) - 1u;
	for (uint32_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
		const uint32_t ti = task_of_chunk(A.chunk_off, n_tasks, c);
		SahTask &t = A.large[par][ti];
		const uint32_t begin = t.begin, count = t.count, nl = t.n_left, axis = t.axis,
		               split = t.split, buf = t.meta & 1u;
		const uint32_t lo_i = begin + (c - A.chunk_off[ti]) * kChunk;
		const uint32_t hi_i = min(lo_i + kChunk, begin + count);
		const float4 *src = A.rec[buf];
		float4 *dst = A.rec[buf ^ 1u];
		const float flo = axis < 3 ? t.lo[axis] : 0.0f, fsc = axis < 3 ? t.scale[axis] : 0.0f;
		for (uint32_t i0 = lo_i + (threadIdx.x & ~31u); i0 < hi_i; i0 += blockDim.x) {
			const uint32_t i = i0 + lane;
			const bool v = i < hi_i;
			float4 lo = make_float4(0, 0, 0, 0), hi = lo;
			bool right = false;
			if (v) {
				lo = src[2 * (size_t)i];
				hi = src[2 * (size_t)i + 1];
				right = axis == kHalves ? (i - begin >= nl)
				                        : (bin_of(rec_c(lo, hi, (int)axis), flo, fsc) > (int)split);
			}
			const uint32_t bl = __ballot_sync(0xFFFFFFFFu, v && !right);
			const uint32_t br = __ballot_sync(0xFFFFFFFFu, v && right);
			uint32_t base_l = 0, base_r = 0;
			if (lane == 0) {
				if (bl)
					base_l = atomicAdd(&t.cur_l, (uint32_t)__popc(bl));
				if (br)
					base_r = atomicAdd(&t.cur_r, (uint32_t)__popc(br));
			}
			base_l = __shfl_sync(0xFFFFFFFFu, base_l, 0);
			base_r = __shfl_sync(0xFFFFFFFFu, base_r, 0);
			if (v) {
				const uint32_t pos = right ? base_r + __popc(br & lt) : base_l + __popc(bl & lt);
				const bool ok = right ? (pos >= begin + nl && pos < begin + count)
				                      : (pos >= begin && pos < begin + nl);
				if (ok) {
					dst[2 * (size_t)pos] = lo;
					dst[2 * (size_t)pos + 1] = hi;
				} else {
					flag(A.err);
				}
			}
		}
	}
}

// ---------------------------------------------------------------------------------------
// Mid tasks: one warp each, bins in shared memory, stable partition.

__global__ void __launch_bounds__(128) k_sah_mid(SahArgs A, int par) {
	__shared__ uint32_t sb_all[4][kBinWords];
	const uint32_t n_tasks = n_mid(A, par);
	const int lane = threadIdx.x & 31;
	const uint32_t lt = (1u << lane) - 1u;
	uint32_t *sb = sb_all[threadIdx.x >> 5];
	for (uint32_t ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; ti < n_tasks;
	     ti += (gridDim.x * blockDim.x) >> 5) {
		const SahTask t = A.mid[par][ti];
		if (!range_ok(A, t.begin, t.count) || t.count > kLarge) {
			if (lane == 0)
				flag(A.err);
			continue;
		}
		const uint32_t buf = t.meta & 1u;
		const float4 *src = A.rec[buf];
		float4 *dst = A.rec[buf ^ 1u];
		// Exact centre bounds of the range: the binning frame.
		float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
		for (uint32_t i = t.begin + lane; i < t.begin + t.count; i += 32) {
			const float4 lo = src[2 * (size_t)i], hi = src[2 * (size_t)i + 1];
#pragma unroll
			for (int k = 0; k < 3; ++k) {
				const float c = rec_c(lo, hi, k);
				mn[k] = fminf(mn[k], c);
				mx[k] = fmaxf(mx[k], c);
			}
		}
		float flo[3], fsc[3];
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			for (int o = 16; o > 0; o >>= 1) {
				mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
				mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
			}
			flo[k] = mn[k];
			fsc[k] = frame_scale(mn[k], mx[k]);
		}
		bins_init(sb, lane);
		__syncwarp();
		for (uint32_t i0 = t.begin; i0 < t.begin + t.count; i0 += 32) {
			const uint32_t i = i0 + lane;
			const bool v = i < t.begin + t.count;
			float4 lo = make_float4(0, 0, 0, 0), hi = lo;
			if (v) {
				lo = src[2 * (size_t)i];
				hi = src[2 * (size_t)i + 1];
			}
			bins_add(sb, v, lo, hi, flo, fsc, lane);
		}
		__syncwarp();
		Split s = choose_split(sb, fsc, t.count, lane);
		if (((t.meta >> 8) & 0xFFu) >= kDepthGuard) {
			s.axis = kHalves;
			s.n_left = t.count / 2;
		}
		// Stable partition into the other buffer.
		uint32_t nl_seen = 0, nr_seen = 0;
		for (uint32_t i0 = t.begin; i0 < t.begin + t.count; i0 += 32) {
			const uint32_t i = i0 + lane;
			const bool v = i < t.begin + t.count;
			float4 lo = make_float4(0, 0, 0, 0), hi = lo;
			bool right = false;
			if (v) {
				lo = src[2 * (size_t)i];
				hi = src[2 * (size_t)i + 1];
				right = s.axis == kHalves
				            ? (i - t.begin >= s.n_left)
				            : (bin_of(rec_c(lo, hi, (int)s.axis), flo[s.axis], fsc[s.axis]) >
				               (int)s.bin);
			}
			const uint32_t bl = __ballot_sync(0xFFFFFFFFu, v && !right);
			const uint32_t br = __ballot_sync(0xFFFFFFFFu, v && right);
			if (v) {
				const uint32_t pos = right ? t.begin + s.n_left + nr_seen + __popc(br & lt)
				                           : t.begin + nl_seen + __popc(bl & lt);
				const bool ok = right ? (pos < t.begin + t.count) : (pos < t.begin + s.n_left);
				if (ok) {
					dst[2 * (size_t)pos] = lo;
					dst[2 * (size_t)pos + 1] = hi;
				} else {
					flag(A.err);
				}
			}
			nl_seen += __popc(bl);
			nr_seen += __popc(br);
		}
		uint32_t slots[2] = {kNone, kNone}; // children of mid tasks are never large
		if (lane == 0) {
			if (nl_seen != s.n_left)
				flag(A.err);
			write_parent_area(A, t.parent, box_area(s.node));
			emit_split(A, t, s, par ^ 1, flo, fsc, slots);
		}
		__syncwarp();
	}
}

// ---------------------------------------------------------------------------------------
// Small tasks: one warp builds the subtree of up to 32 triangles, one per lane.  The
// triangles are ranked once per axis by (centre, index); each node orders its lanes on
// each axis from those ranks (one OR of rank bits and a population count), sweeps prefix
// and suffix boxes and reorders its lanes by the best axis; the children are the two
// parts.

__global__ void __launch_bounds__(128) k_sah_small(SahArgs A) {
	__shared__ float4 stage_all[4][2 * 32];
	const uint32_t n_tasks = min(A.ctr[kCtrSmall], A.max_small);
	const int lane = threadIdx.x & 31;
	float4 *stage = stage_all[threadIdx.x >> 5];
	for (uint32_t ti = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; ti < n_tasks;
	     ti += (gridDim.x * blockDim.x) >> 5) {
		const SmallTask st = A.small[ti];
		const uint32_t m = st.meta & 0xFFu, buf = (st.meta >> 8) & 1u, depth0 = st.meta >> 16;
		if (m == 0 || m > kSmall || st.begin > A.n || m > A.n - st.begin) {
			if (lane == 0)
				flag(A.err);
			continue;
		}
		const float4 *src = A.rec[buf];
		float4 lo = make_float4(0, 0, 0, 0), hi = lo;
		if ((uint32_t)lane < m) {
			lo = src[2 * (size_t)(st.begin + lane)];
			hi = src[2 * (size_t)(st.begin + lane) + 1];
		}
		if (m >= 3) {
			// Each triangle's rank among the task's on each axis, by (centre, index),
			// packed 5 bits per axis into the unused w of its box (it moves with the
			// triangle when lanes are reordered).  A node's own order on an axis is then
			// one OR over its lanes' rank bits and a population count.
			uint32_t gr = 0;
#pragma unroll
			for (int a = 0; a < 3; ++a) {
				const uint64_t key = (uint32_t)lane < m
				                         ? (((uint64_t)f2ord(rec_c(lo, hi, a)) << 32) |
				                            __float_as_uint(lo.w))
				                         : ~0ull;
				uint32_t rank = 0;
				for (uint32_t j = 0; j < m; ++j)
					rank += __shfl_sync(0xFFFFFFFFu, key, (int)j) < key;
				gr |= min(rank, 31u) << (5 * a);
			}
			hi.w = __uint_as_float(gr);
		}
		if (m >= 2) {
			uint32_t base = 0;
			if (lane == 0 && m > 2)
				base = new_node(A, m - 2);
			base = __shfl_sync(0xFFFFFFFFu, base, 0);
			if (base == kNone || st.node == kNone || st.node >= A.node_cap) {
				if (lane == 0 && base != kNone)
					flag(A.err);
				continue;
			}
			uint32_t next = 0;
			// Warp-distributed stack: lane j holds entry j (first | count << 8 | depth << 16,
			// node).
			uint32_t stk_a = 0, stk_n = 0;
			int top = 0;
			if (lane == 0) {
				stk_a = 0u | (m << 8) | (depth0 << 16);
				stk_n = st.node;
			}
			top = 1;
			bool root = true;
			while (top > 0) {
				--top;
				const uint32_t ea = __shfl_sync(0xFFFFFFFFu, stk_a, top);
				const uint32_t node = __shfl_sync(0xFFFFFFFFu, stk_n, top);
				const int f = (int)(ea & 0xFFu), cnt = (int)((ea >> 8) & 0xFFu);
				const uint32_t dep = ea >> 16;
				if (cnt < 2 || f + cnt > (int)m || node >= A.node_cap || top >= 31) {
					if (lane == 0)
						flag(A.err);
					break;
				}
				const bool in = lane >= f && lane < f + cnt;
				int k_best = cnt / 2 - 1; // last lane (relative) of the left part
				int axis_best = -1;
				Box6 nb, lb, rb;
				if (cnt > 2 && dep < kDepthGuard) {
					uint64_t best = ~0ull;
					uint32_t rank_best = 0;
					for (int a = 0; a < 3; ++a) {
						const uint32_t ga = (__float_as_uint(hi.w) >> (5 * a)) & 31u;
						const uint32_t members =
						    __reduce_or_sync(0xFFFFFFFFu, in ? (1u << ga) : 0u);
						const uint32_t rank = __popc(members & ((1u << ga) - 1u));
						// Boxes in sorted order: lane f + r holds the box of rank r.
						if (in)
							stage[f + rank] = make_float4(lo.x, lo.y, lo.z, hi.x);
						if (in)
							stage[32 + f + rank] = make_float4(hi.y, hi.z, 0.0f, 0.0f);
						__syncwarp();
						Box6 sb = empty_box();
						if (in) {
							const float4 s0 = stage[lane], s1 = stage[32 + lane];
							sb = Box6{s0.x, s0.y, s0.z, s0.w, s1.x, s1.y};
						}
						__syncwarp();
						Box6 p = sb, q = sb;
						for (int o = 1; o < cnt; o <<= 1) {
							const Box6 pu = shfl_box(p, max(lane - o, 0));
							const Box6 qd = shfl_box(q, min(lane + o, 31));
							if (in && lane - o >= f)
								p = box_union(p, pu);
							if (in && lane + o < f + cnt)
								q = box_union(q, qd);
						}
						const Box6 r = shfl_box(q, min(lane + 1, 31));
						// The least cost on this axis and, among its lanes, the lowest
						// position: two 32-bit warp minima (redux.sync) instead of five
						// shuffle rounds of a 64-bit key.
						uint32_t c32 = 0xFFFFFFFFu;
						if (in && lane < f + cnt - 1) {
							const int nl = lane - f + 1, nr = cnt - nl;
							c32 = f2ord(box_area(p) * (float)nl + box_area(r) * (float)nr);
						}
						const uint32_t cmin = __reduce_min_sync(0xFFFFFFFFu, c32);
						const uint32_t pos = __reduce_min_sync(
						    0xFFFFFFFFu, (c32 == cmin && c32 != 0xFFFFFFFFu) ? (uint32_t)(lane - f) : 0xFFu);
						const uint64_t ck = cmin == 0xFFFFFFFFu
						                        ? ~0ull
						                        : (((uint64_t)cmin << 32) | ((uint32_t)a << 8) | pos);
						if (ck < best) {
							best = ck;
							axis_best = a;
							k_best = (int)(ck & 0xFF);
							rank_best = rank;
							lb = shfl_box(p, f + k_best);
							rb = shfl_box(r, f + k_best);
						}
						if (a == 0)
							nb = shfl_box(p, f + cnt - 1);
					}
					if (axis_best >= 0) {
						// Reorder the node's lanes by the best axis.
						if (in) {
							stage[f + rank_best] = lo;
							stage[32 + f + rank_best] = hi;
						}
						__syncwarp();
						if (in) {
							lo = stage[lane];
							hi = stage[32 + lane];
						}
						__syncwarp();
					}
				}
				if (axis_best < 0) {
					k_best = cnt / 2 - 1;
					const Box6 me2{lo.x, lo.y, lo.z, hi.x, hi.y, hi.z};
					lb = range_box(me2, lane, f, f + k_best + 1);
					rb = range_box(me2, lane, f + k_best + 1, f + cnt);
					nb = box_union(lb, rb);
				}
				const int nl = k_best + 1, nr = cnt - nl;
				// Node ids of the children (warp-uniform: nl, nr and next are).
				uint32_t ids[2] = {kNone, kNone};
				if (nl > 1)
					ids[0] = base + next++;
				if (nr > 1)
					ids[1] = base + next++;
				if (lane == 0) {
					const uint32_t rl = nl > 1 ? ids[0] : (kLeafBit | (st.begin + f));
					const uint32_t rr = nr > 1 ? ids[1] : (kLeafBit | (st.begin + f + nl));
					A.left[node] = rl;
					A.right[node] = rr;
					A.rfirst[node] = st.begin + f;
					A.rlast[node] = st.begin + f + cnt - 1;
					if (nl > 1)
						A.parent_int[ids[0]] = node;
					else
						A.parent_leaf[st.begin + f] = node;
					if (nr > 1)
						A.parent_int[ids[1]] = node;
					else
						A.parent_leaf[st.begin + f + nl] = node;
					write_node_box(A, node, nb, nl > 1 ? box_area(lb) : -1.0f,
					               nr > 1 ? box_area(rb) : -1.0f);
					if (root)
						write_parent_area(A, st.parent, box_area(nb));
				}
				// Push the children (right first, so the left is taken next).
				if (nr > 1) {
					if (lane == top) {
						stk_a = (uint32_t)(f + nl) | ((uint32_t)nr << 8) | ((dep + 1u) << 16);
						stk_n = ids[1];
					}
					++top;
				}
				if (nl > 1) {
					if (lane == top) {
						stk_a = (uint32_t)f | ((uint32_t)nl << 8) | ((dep + 1u) << 16);
						stk_n = ids[0];
					}
					++top;
				}
				root = false;
			}
		}
		if ((uint32_t)lane < m) {
			const uint32_t pos = st.begin + lane;
			A.vals[pos] = __float_as_uint(lo.w);
			A.lbox[2 * (size_t)pos] = make_float4(lo.x, lo.y, lo.z, 0.0f);
			A.lbox[2 * (size_t)pos + 1] = make_float4(hi.x, hi.y, hi.z, 0.0f);
		}
	}
}

__global__ void k_sah_bounds_init(uint32_t *gb, uint32_t n_scenes) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < 6 * n_scenes;
	     i += gridDim.x * blockDim.x)
		gb[i] = (i % 6) < 3 ? 0xFFFFFFFFu : 0u;
}

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

struct Layout {
	size_t max_large, max_mid, max_small;
	size_t off[12];
	size_t total;
};

// Regions of the scratch, 256-byte aligned: records x2, then per parity large tasks,
// bins and mid tasks, then small tasks, chunk offsets and counters.
Layout layout(uint32_t n, uint32_t S) {
	Layout L;
	L.max_large = n / (kLarge + 1) + S + 1;
	L.max_mid = n / (kSmall + 1) + S + 1;
	L.max_small = (size_t)n + S + 1;
	const size_t sz[12] = {32ull * n,
	                       32ull * n,
	                       64 * L.max_large,
	                       4ull * kBinWords * L.max_large,
	                       64 * L.max_mid,
	                       64 * L.max_large,
	                       4ull * kBinWords * L.max_large,
	                       64 * L.max_mid,
	                       16 * L.max_small,
	                       4 * (L.max_large + 1),
	                       4 * kCtrWordsSah,
	                       0};
	size_t at = 0;
	for (int k = 0; k < 12; ++k) {
		L.off[k] = at;
		at += (sz[k] + 255) & ~size_t(255);
	}
	L.total = at;
	return L;
}

} // namespace

size_t sah_scratch_bytes(uint32_t n, uint32_t S) { return layout(n, S).total; }

int sah_build_enqueue(const float *d_tris, const BuildPlan &plan, BuildScratch &ws,
                      const uint32_t *d_toff, const uint32_t *scene_of, cudaStream_t st,
                      uint32_t *d_err, std::string &msg) {
	const uint32_t n = plan.n, S = plan.S;
	const Layout L = layout(n, S);
	if (ws.sah.bytes < L.total || ws.roots.bytes < 4ull * S) {
		msg = "sah build: scratch not reserved";
		return PRT_ERR_DEVICE;
	}
	char *p = ws.sah.as<char>();
	SahArgs A;
	A.rec[0] = reinterpret_cast<float4 *>(p + L.off[0]);
	A.rec[1] = reinterpret_cast<float4 *>(p + L.off[1]);
	for (int k = 0; k < 2; ++k) {
		A.large[k] = reinterpret_cast<SahTask *>(p + L.off[2 + 3 * k]);
		A.bins[k] = reinterpret_cast<uint32_t *>(p + L.off[3 + 3 * k]);
		A.mid[k] = reinterpret_cast<SahTask *>(p + L.off[4 + 3 * k]);
	}
	A.small = reinterpret_cast<SmallTask *>(p + L.off[8]);
	A.chunk_off = reinterpret_cast<uint32_t *>(p + L.off[9]);
	A.ctr = reinterpret_cast<uint32_t *>(p + L.off[10]);
	A.vals = ws.vals.as<uint32_t>();
	A.lbox = ws.lbox.as<float4>();
	A.left = ws.left.as<uint32_t>();
	A.right = ws.right.as<uint32_t>();
	A.rfirst = ws.rfirst.as<uint32_t>();
	A.rlast = ws.rlast.as<uint32_t>();
	A.ibox = ws.ibox.as<float4>();
	A.parent_int = ws.parent_int.as<uint32_t>();
	A.parent_leaf = ws.parent_leaf.as<uint32_t>();
	A.node_cap = plan.n_int + S;
	A.max_large = (uint32_t)L.max_large;
	A.max_mid = (uint32_t)L.max_mid;
	A.max_small = (uint32_t)L.max_small;
	A.n = n;
	A.err = d_err;

	uint32_t *gb = ws.bounds.as<uint32_t>();
	cudaMemsetAsync(A.ctr, 0, 4 * kCtrWordsSah, st);
	// No parent: the roots and the triangles of one-triangle scenes keep these.
	cudaMemsetAsync(A.parent_int, 0xFF, 4ull * A.node_cap, st);
	cudaMemsetAsync(A.parent_leaf, 0xFF, 4ull * n, st);
	k_sah_bounds_init<<<blocks_for(6ull * S, 256), 256, 0, st>>>(gb, S);
	if (n)
		k_sah_records<<<blocks_for(n, 256), 256, 0, st>>>(d_tris, n, scene_of, A.rec[0], gb);
	k_sah_first_id<<<1, 1, 0, st>>>(A.ctr, S);
	k_sah_roots<<<blocks_for(32ull * S, 128), 128, 0, st>>>(A, d_toff, S, gb,
	                                                        ws.roots.as<uint32_t>());
	int level = 0;
	bool large_left = true; // children are smaller than their parent: once no large task
	                        // is left, none comes back, and its four kernels are skipped
	// Before the first look at the level counters (a host wait each): as many levels as
	// halving splits need to bring the largest scene under the large-task size, since a
	// split leaves at least one triangle on each side and most leave about half.
	// For scenes of at most 64 Ki triangles the mid levels too (down to the small-task
	// size): their empty large-tier launches cost less than the wait they save.
	int ahead = 1;
	{
		uint32_t biggest = 0;
		for (uint32_t sc = 0; sc < S; ++sc)
			biggest = std::max(biggest, plan.toff[sc + 1] - plan.toff[sc]);
		const uint32_t floor = biggest <= 65536u ? kSmall : kLarge;
		for (uint64_t c = biggest; c > floor; c = (c + 1) / 2)
			++ahead;
		ahead = std::max(ahead, kLevelsPerCheck);
	}
	for (;;) {
		for (int k = 0; k < ahead && level < kMaxLevels; ++k, ++level) {
			const int par = level & 1;
			// Grids no larger than the work the level can hold: each task has at most two
			// children, so level L has at most S * 2^L tasks of a tier (a small scene's
			// levels are then a few blocks each instead of 1216 idle ones).
			const uint64_t tasks = (uint64_t)S << std::min(level, 40);
			const unsigned g_chunk =
			    (unsigned)std::min<uint64_t>(1216, n / kChunk + std::min<uint64_t>(tasks, L.max_large));
			const unsigned g_split = (unsigned)std::min<uint64_t>(152, (tasks + 3) / 4);
			const unsigned g_mid =
			    (unsigned)std::min<uint64_t>(1216, (std::min<uint64_t>(tasks, L.max_mid) + 3) / 4);
			if (large_left) {
				k_sah_chunks<<<1, 1024, 0, st>>>(A, par);
				k_sah_bin<<<g_chunk, 256, 0, st>>>(A, par);
				k_sah_split<<<g_split, 128, 0, st>>>(A, par);
				k_sah_part<<<g_chunk, 256, 0, st>>>(A, par);
			} else {
				// What k_sah_chunks does besides: clear the lists this level fills.
				cudaMemsetAsync(A.ctr + kCtrLarge + (par ^ 1), 0, 4, st);
				cudaMemsetAsync(A.ctr + kCtrMid + (par ^ 1), 0, 4, st);
			}
			k_sah_mid<<<g_mid, 128, 0, st>>>(A, par);
		}
		uint32_t *h = ws.h_sah;
		cudaError_t e = cudaMemcpyAsync(h, A.ctr, 4 * kCtrWordsSah, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(st);
		if (e != cudaSuccess) {
			msg = std::string("sah build: ") + cudaGetErrorString(e);
			return PRT_ERR_CUDA;
		}
		const int par = level & 1;
		if (h[kCtrLarge + par] == 0 && h[kCtrMid + par] == 0)
			break;
		if (h[kCtrLarge + par] == 0)
			large_left = false;
		if (level >= kMaxLevels) {
			msg = "sah build: more than " + std::to_string(kMaxLevels) + " levels";
			return PRT_ERR_LIMIT;
		}
		ahead = kLevelsPerCheck;
	}
	k_sah_small<<<2432, 128, 0, st>>>(A);
	// Every node id handed out must have been written before the collapse follows the
	// children: check the error word and the node count first.
	uint64_t want = S;
	for (uint32_t s = 0; s < S; ++s) {
		const uint32_t ns = plan.toff[s + 1] - plan.toff[s];
		want += ns >= 2 ? ns - 2 : 0;
	}
	uint32_t *h = ws.h_sah, *h_errw = h + kCtrWordsSah;
	cudaError_t e = cudaMemcpyAsync(h, A.ctr, 4 * kCtrWordsSah, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(h_errw, d_err, 4, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(st);
	const uint32_t h_err = *h_errw;
	if (e != cudaSuccess) {
		msg = std::string("sah build: ") + cudaGetErrorString(e);
		return PRT_ERR_CUDA;
	}
	if ((h_err & kErrSah) || h[kCtrNodes] != want) {
		cudaMemsetAsync(d_err, 0, 4, st);
		cudaStreamSynchronize(st);
		msg = "sah build: internal check failed (nodes " + std::to_string(h[kCtrNodes]) +
		      " of " + std::to_string(want) + ")";
		return PRT_ERR_DEVICE;
	}
	return PRT_OK;
}

} // namespace prt
