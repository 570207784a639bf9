// prt_build.cu - LBVH build of the 8-wide tree on the GPU.
//
// Replaces the single-threaded binned-SAH build of portableRT (bvh.hpp:58-193).  The
// tree's shape does not affect the answers (every triangle whose own box passes the
// reference slab test is examined; see prt_traverse.cu), so a fast parallel build is
// used instead:
//   1. centroid bounds            (k_centroid_bounds)
//   2. 30-bit Morton codes        (k_morton; 10 bits per axis, centroids normalised)
//   3. onesweep radix sort        (prt_sort.cu; 4 digit passes, stable)
//   4. Karras hierarchy           (k_karras; Karras 2012, ties broken by index)
//   5. bottom-up refit            (k_leaf_boxes + k_refit; atomic arrival counters)
//   6. collapse to 8-wide nodes   (k_collapse, one launch per level; the child of
//                                  largest surface area is opened until 8 children)
//   7. triangle re-layout         (k_relayout; each node's leaf triangles contiguous)
//   8. optional 8-bit encoding    (k_compress; outward-rounded child boxes)
// A triangle with a non-finite vertex gets the box [-FLT_MAX, FLT_MAX]^3 in the tree,
// which every finite ray passes, so the exact per-triangle test still sees it.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"

namespace prt {

void BuildScratch::release() {
	DevBuf *all[] = {&keys,       &vals,       &keys2,  &vals2,       &left,       &right,
	                 &parent_int, &parent_leaf, &rfirst, &rlast,       &ibox,       &lbox,
	                 &flags,      &items_a,    &items_b, &counters,   &perm,       &sort_hist,
	                 &sort_tiles, &sort_status, &bounds};
	for (DevBuf *b : all)
		b->release();
	if (h_counters)
		cudaFreeHost(h_counters);
	h_counters = nullptr;
}

namespace {

struct Item {
	uint32_t ref;  // binary-tree reference (bit 31 = leaf)
	uint32_t slot; // index of the 8-wide node it becomes
};

__device__ __forceinline__ bool tri_finite(const float *t) {
	bool ok = true;
#pragma unroll
	for (int k = 0; k < 9; ++k)
		ok = ok && isfinite(t[k]);
	return ok;
}

__global__ void k_centroid_bounds(const float *__restrict__ tris, uint32_t n, uint32_t *gb) {
	float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float *t = tris + 9 * (size_t)i;
		if (!tri_finite(t))
			continue;
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			float c = t[k] * (1.0f / 3.0f) + t[k + 3] * (1.0f / 3.0f) + t[k + 6] * (1.0f / 3.0f);
			mn[k] = fminf(mn[k], c);
			mx[k] = fmaxf(mx[k], c);
		}
	}
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		for (int o = 16; o > 0; o >>= 1) {
			mn[k] = fminf(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
			mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
		}
	}
	if ((threadIdx.x & 31) == 0 && mn[0] <= mx[0]) {
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			atomicMin(&gb[k], f2ord(mn[k]));
			atomicMax(&gb[3 + k], f2ord(mx[k]));
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

__global__ void k_morton(const float *__restrict__ tris, uint32_t n, const uint32_t *gb,
                         uint32_t *keys, uint32_t *vals) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const float *t = tris + 9 * (size_t)i;
	uint32_t code = 0;
	float lo0 = ord2f(gb[0]), hi0 = ord2f(gb[3]);
	if (tri_finite(t) && lo0 <= hi0) {
		uint32_t q[3];
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			float lo = ord2f(gb[k]), hi = ord2f(gb[3 + k]);
			float ext = hi - lo;
			float s = ext > 0.0f ? 1024.0f / ext : 0.0f;
			float c = t[k] * (1.0f / 3.0f) + t[k + 3] * (1.0f / 3.0f) + t[k + 6] * (1.0f / 3.0f);
			float qf = fminf(fmaxf((c - lo) * s, 0.0f), 1023.0f);
			q[k] = (uint32_t)qf;
		}
		code = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
	}
	keys[i] = code;
	vals[i] = i;
}

// Length of the common prefix of keys i and j, with the index appended to break ties
// between equal keys; -1 outside [0, n).
__device__ __forceinline__ int kdelta(const uint32_t *__restrict__ k, int n, int i, int j) {
	if (j < 0 || j >= n)
		return -1;
	uint32_t a = k[i], b = k[j];
	return (a != b) ? __clz(a ^ b) : 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void k_karras(const uint32_t *__restrict__ keys, int n, uint32_t *left,
                         uint32_t *right, uint32_t *parent_int, uint32_t *parent_leaf,
                         uint32_t *rfirst, uint32_t *rlast) {
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n - 1)
		return;
	const int d = kdelta(keys, n, i, i + 1) > kdelta(keys, n, i, i - 1) ? 1 : -1;
	const int dmin = kdelta(keys, n, i, i - d);
	int lmax = 2;
	while (kdelta(keys, n, i, i + lmax * d) > dmin)
		lmax <<= 1;
	int l = 0;
	for (int t = lmax >> 1; t >= 1; t >>= 1)
		if (kdelta(keys, n, i, i + (l + t) * d) > dmin)
			l += t;
	const int j = i + l * d;
	const int dnode = kdelta(keys, n, i, j);
	int s = 0;
	for (int div = 2;; div <<= 1) {
		int t = (l + div - 1) / div;
		if (kdelta(keys, n, i, i + (s + t) * d) > dnode)
			s += t;
		if (t <= 1)
			break;
	}
	const int gamma = i + s * d + min(d, 0);
	const int lo = min(i, j), hi = max(i, j);
	uint32_t lc = (lo == gamma) ? (kLeafBit | (uint32_t)gamma) : (uint32_t)gamma;
	uint32_t rc = (hi == gamma + 1) ? (kLeafBit | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
	left[i] = lc;
	right[i] = rc;
	if (lc & kLeafBit)
		parent_leaf[gamma] = i;
	else
		parent_int[gamma] = i;
	if (rc & kLeafBit)
		parent_leaf[gamma + 1] = i;
	else
		parent_int[gamma + 1] = i;
	rfirst[i] = lo;
	rlast[i] = hi;
	if (i == 0)
		parent_int[0] = kNone;
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

// One thread per leaf walks towards the root; at each binary node the first thread to
// arrive stops and the second, which then sees both children's boxes, writes the
// union and continues.  No thread waits on another.
__global__ void k_refit(uint32_t n, const uint32_t *__restrict__ parent_leaf,
                        const uint32_t *__restrict__ parent_int, const uint32_t *__restrict__ left,
                        const uint32_t *__restrict__ right, const float4 *lbox, float4 *ibox,
                        uint32_t *flags) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n || n < 2)
		return;
	uint32_t p = parent_leaf[i];
	while (p != kNone) {
		__threadfence();
		if (atomicAdd(&flags[p], 1u) == 0u)
			return;
		__threadfence();
		float4 alo, ahi, blo, bhi;
		child_box(left[p], ibox, lbox, alo, ahi);
		child_box(right[p], ibox, lbox, blo, bhi);
		__stcg(&ibox[2 * p], make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y),
		                                 fminf(alo.z, blo.z), 0.0f));
		__stcg(&ibox[2 * p + 1], make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y),
		                                     fmaxf(ahi.z, bhi.z), 0.0f));
		p = parent_int[p];
	}
}

__device__ __forceinline__ uint32_t bcount(uint32_t ref, const uint32_t *rfirst,
                                           const uint32_t *rlast) {
	return (ref & kLeafBit) ? 1u : (rlast[ref] - rfirst[ref] + 1u);
}

__device__ __forceinline__ uint32_t bfirst(uint32_t ref, const uint32_t *rfirst) {
	return (ref & kLeafBit) ? (ref & ~kLeafBit) : rfirst[ref];
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
	float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
	float a = dx * dy + dx * dz + dy * dz;
	return isfinite(a) ? a : FLT_MAX;
}

__global__ void __launch_bounds__(128)
    k_collapse(const Item *__restrict__ in, const uint32_t *in_count, Item *out,
               uint32_t *out_count, uint32_t *node_counter, uint32_t node_cap,
               uint32_t *tri_counter, Node8 *nodes, uint32_t *perm,
               const uint32_t *__restrict__ left, const uint32_t *__restrict__ right,
               const uint32_t *__restrict__ rfirst, const uint32_t *__restrict__ rlast,
               const float4 *__restrict__ ibox, const float4 *__restrict__ lbox,
               uint32_t leaf_size, uint32_t n_tris, uint32_t *err) {
	const uint32_t n_in = *in_count;
	for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < n_in;
	     w += gridDim.x * blockDim.x) {
		const Item it = in[w];
		uint32_t C[8];
		int nc = 1;
		C[0] = it.ref;
		// Open the binary child of largest surface area until 8 children: any binary
		// node can be opened, so nodes fill up and small subtrees end as single
		// triangles (whose box is then tested exactly like the reference's leaf box).
		while (nc < 8) {
			int best = -1;
			float best_area = -1.0f;
			for (int c = 0; c < nc; ++c) {
				uint32_t r = C[c];
				if (!(r & kLeafBit)) {
					float a = half_area(ibox[2 * r], ibox[2 * r + 1]);
					if (a > best_area) {
						best_area = a;
						best = c;
					}
				}
			}
			if (best < 0)
				break;
			uint32_t x = C[best];
			C[best] = left[x];
			C[nc++] = right[x];
		}
		// Children in order of their first leaf, so a node's leaf triangles keep the
		// Morton order.
		for (int a = 1; a < nc; ++a) {
			uint32_t v = C[a];
			uint32_t fv = bfirst(v, rfirst);
			int b = a - 1;
			while (b >= 0 && bfirst(C[b], rfirst) > fv) {
				C[b + 1] = C[b];
				--b;
			}
			C[b + 1] = v;
		}
		uint32_t n_inner = 0, n_leaf_tris = 0;
		for (int c = 0; c < nc; ++c) {
			uint32_t cnt = bcount(C[c], rfirst, rlast);
			if (!(C[c] & kLeafBit) && cnt > leaf_size)
				++n_inner;
			else
				n_leaf_tris += cnt;
		}
		uint32_t base = n_inner ? atomicAdd(node_counter, n_inner) : 0u;
		if (base + n_inner > node_cap) {
			atomicOr(err, kErrCollapse);
			continue;
		}
		uint32_t tbase = n_leaf_tris ? atomicAdd(tri_counter, n_leaf_tris) : 0u;
		if (tbase + n_leaf_tris > n_tris) {
			atomicOr(err, kErrCollapse);
			continue;
		}
		Node8 *nd = nodes + it.slot;
		uint32_t k_inner = 0, toff = 0;
		for (int c = 0; c < 8; ++c) {
			float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
			uint32_t ref = kNone;
			if (c < nc) {
				uint32_t r = C[c];
				uint32_t cnt = bcount(r, rfirst, rlast);
				if (r & kLeafBit) {
					uint32_t k = r & ~kLeafBit;
					lo = lbox[2 * k];
					hi = lbox[2 * k + 1];
				} else {
					lo = ibox[2 * r];
					hi = ibox[2 * r + 1];
				}
				if (!(r & kLeafBit) && cnt > leaf_size) {
					ref = base + k_inner++;
					out[atomicAdd(out_count, 1u)] = Item{r, ref};
				} else {
					uint32_t first = bfirst(r, rfirst);
					uint32_t dst = tbase + toff;
					toff += cnt;
					for (uint32_t k = 0; k < cnt; ++k)
						perm[dst + k] = first + k;
					ref = make_leaf(dst, cnt);
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

__global__ void k_relayout(const float *__restrict__ tris, const uint32_t *__restrict__ vals,
                           const uint32_t *__restrict__ perm, uint32_t n, float4 *tri4,
                           uint32_t *inv) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	uint32_t pid = vals[perm[i]];
	inv[pid] = i;
	const float *t = tris + 9 * (size_t)pid;
	tri4[3 * (size_t)i] = make_float4(t[0], t[1], t[2], __uint_as_float(pid));
	tri4[3 * (size_t)i + 1] = make_float4(t[3], t[4], t[5], 0.0f);
	tri4[3 * (size_t)i + 2] = make_float4(t[6], t[7], t[8], 0.0f);
}

__device__ __forceinline__ float cdec(float o, uint32_t q, float s) {
	return __fadd_rn(o, __fmul_rn((float)q, s));
}

// Largest q in [0, 255] whose decoded value is <= v (decoding is monotone in q and
// q = 0 decodes to the origin, which is <= every child bound).
__device__ uint32_t quant_lo(float o, float s, float v) {
	double g = floor(((double)v - (double)o) / (double)s);
	uint32_t q = (uint32_t)fmin(fmax(g, 0.0), 255.0);
	while (q > 0 && cdec(o, q, s) > v)
		--q;
	while (q < 255 && cdec(o, q + 1, s) <= v)
		++q;
	return q;
}

// Smallest q in [0, 255] whose decoded value is >= v (the exponent was chosen so that
// q = 255 qualifies).
__device__ uint32_t quant_hi(float o, float s, float v) {
	double g = ceil(((double)v - (double)o) / (double)s);
	uint32_t q = (uint32_t)fmin(fmax(g, 0.0), 255.0);
	while (q < 255 && cdec(o, q, s) < v)
		++q;
	while (q > 0 && cdec(o, q - 1, s) >= v)
		--q;
	return q;
}

__global__ void k_compress(const Node8 *__restrict__ nodes, uint32_t n_nodes, CNode8 *cn) {
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n_nodes)
		return;
	const Node8 &nd = nodes[i];
	float lo[3][8], hi[3][8];
	uint32_t ref[8];
	for (int k = 0; k < 8; ++k) {
		const Child8 &ch = nd.c[k];
		lo[0][k] = ch.lo_x;
		lo[1][k] = ch.lo_y;
		lo[2][k] = ch.lo_z;
		hi[0][k] = ch.hi_x;
		hi[1][k] = ch.hi_y;
		hi[2][k] = ch.hi_z;
		ref[k] = ch.ref;
	}
	CNode8 c;
	memset(&c, 0, sizeof c);
	uint32_t child_base = kNone, tri_base = kNone;
	for (int k = 0; k < 8; ++k) {
		const uint32_t r = ref[k];
		if (r == kNone)
			continue;
		if (r & kLeafBit)
			tri_base = min(tri_base, leaf_first(r));
		else {
			c.imask |= (uint8_t)(1u << k);
			child_base = min(child_base, r);
		}
	}
	c.child_base = child_base == kNone ? 0u : child_base;
	c.tri_base = tri_base == kNone ? 0u : tri_base;
	for (int k = 0; k < 8; ++k) {
		const uint32_t r = ref[k];
		if (r != kNone && (r & kLeafBit)) {
			c.c[k].count = (uint8_t)leaf_count(r);
			c.c[k].first = (uint8_t)(leaf_first(r) - c.tri_base);
		}
	}
	float org[3];
	uint8_t ex[3];
	for (int a = 0; a < 3; ++a) {
		float mn = INFINITY, mx = -INFINITY;
		for (int k = 0; k < 8; ++k) {
			if (ref[k] == kNone)
				continue;
			mn = fminf(mn, lo[a][k]);
			mx = fmaxf(mx, hi[a][k]);
		}
		if (!(mn <= mx)) {
			mn = 0.0f;
			mx = 0.0f;
		}
		org[a] = mn;
		double range = (double)mx - (double)mn;
		int e = 1;
		if (range > 0.0) {
			int est = (int)ceil(log2(range / 255.0)) + 127;
			e = max(1, min(254, est - 1));
		}
		while (e < 254 && cdec(mn, 255u, cscale((uint8_t)e)) < mx)
			++e;
		ex[a] = (uint8_t)e;
	}
	c.ox = org[0];
	c.oy = org[1];
	c.oz = org[2];
	c.ex = ex[0];
	c.ey = ex[1];
	c.ez = ex[2];
	for (int a = 0; a < 3; ++a) {
		float s = cscale(ex[a]);
		for (int k = 0; k < 8; ++k) {
			if (ref[k] == kNone)
				continue;
			uint8_t *qk = &c.c[k].qlo_x;
			qk[2 * a] = (uint8_t)quant_lo(org[a], s, lo[a][k]);
			qk[2 * a + 1] = (uint8_t)quant_hi(org[a], s, hi[a][k]);
		}
	}
	cn[i] = c;
}

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

int build_scene(const float *d_tris, uint64_t n64, int leaf_size, bool compressed, SceneGPU &sc,
                BuildScratch &ws, cudaStream_t st, uint32_t *d_err, std::string &msg) {
	if (n64 > kMaxTris) {
		msg = "set_tris: at most 134217727 triangles per scene";
		return PRT_ERR_LIMIT;
	}
	if (leaf_size < 1 || leaf_size > kMaxLeaf) {
		msg = "leaf_size must be in [1, 8]";
		return PRT_ERR_ARG;
	}
	const uint32_t n = (uint32_t)n64;
	sc.n_tris = n;
	sc.leaf_size = leaf_size;
	sc.n_nodes = 0;
	sc.depth = 0;
	sc.has_cnodes = false;
	if (n == 0)
		return PRT_OK;

	const size_t ni = std::max<uint32_t>(n - 1, 1);
	const uint32_t node_cap = n;
	BUILD_TRY(ws.keys.reserve(4ull * n));
	BUILD_TRY(ws.vals.reserve(4ull * n));
	BUILD_TRY(ws.keys2.reserve(4ull * n));
	BUILD_TRY(ws.vals2.reserve(4ull * n));
	BUILD_TRY(ws.left.reserve(4 * ni));
	BUILD_TRY(ws.right.reserve(4 * ni));
	BUILD_TRY(ws.parent_int.reserve(4 * ni));
	BUILD_TRY(ws.parent_leaf.reserve(4ull * n));
	BUILD_TRY(ws.rfirst.reserve(4 * ni));
	BUILD_TRY(ws.rlast.reserve(4 * ni));
	BUILD_TRY(ws.flags.reserve(4 * ni));
	BUILD_TRY(ws.ibox.reserve(32 * ni));
	BUILD_TRY(ws.lbox.reserve(32ull * n));
	BUILD_TRY(ws.items_a.reserve(8ull * n));
	BUILD_TRY(ws.items_b.reserve(8ull * n));
	BUILD_TRY(ws.counters.reserve(64));
	BUILD_TRY(ws.perm.reserve(4ull * n));
	BUILD_TRY(ws.sort_hist.reserve(8 * 256 * 4));
	BUILD_TRY(ws.sort_tiles.reserve(8 * 4));
	BUILD_TRY(ws.sort_status.reserve(4 * sort_status_words(n)));
	BUILD_TRY(ws.bounds.reserve(32));
	BUILD_TRY(sc.tri4.reserve(48ull * n));
	BUILD_TRY(sc.inv.reserve(4ull * n));
	BUILD_TRY(sc.nodes.reserve(sizeof(Node8) * (size_t)node_cap));
	if (!ws.h_counters)
		BUILD_TRY(cudaMallocHost(&ws.h_counters, 64));

	uint32_t *gb = ws.bounds.as<uint32_t>();
	BUILD_TRY(cudaMemsetAsync(gb, 0xFF, 12, st));
	BUILD_TRY(cudaMemsetAsync(gb + 3, 0x00, 12, st));
	k_centroid_bounds<<<std::min(blocks_for(n, 256), 1024u), 256, 0, st>>>(d_tris, n, gb);
	k_morton<<<blocks_for(n, 256), 256, 0, st>>>(d_tris, n, gb, ws.keys.as<uint32_t>(),
	                                             ws.vals.as<uint32_t>());
	SortScratch ss{ws.sort_hist.as<uint32_t>(), ws.sort_tiles.as<uint32_t>(),
	               ws.sort_status.as<uint32_t>()};
	int where = sort_pairs_u32(ws.keys.as<uint32_t>(), ws.vals.as<uint32_t>(),
	                           ws.keys2.as<uint32_t>(), ws.vals2.as<uint32_t>(), n, 4, ss, st, d_err);
	const uint32_t *skeys = where ? ws.keys2.as<uint32_t>() : ws.keys.as<uint32_t>();
	const uint32_t *svals = where ? ws.vals2.as<uint32_t>() : ws.vals.as<uint32_t>();

	if (n >= 2) {
		k_karras<<<blocks_for(n - 1, 256), 256, 0, st>>>(
		    skeys, (int)n, ws.left.as<uint32_t>(), ws.right.as<uint32_t>(),
		    ws.parent_int.as<uint32_t>(), ws.parent_leaf.as<uint32_t>(), ws.rfirst.as<uint32_t>(),
		    ws.rlast.as<uint32_t>());
		BUILD_TRY(cudaMemsetAsync(ws.flags.p, 0, 4 * ni, st));
	}
	k_leaf_boxes<<<blocks_for(n, 256), 256, 0, st>>>(d_tris, svals, n, ws.lbox.as<float4>());
	if (n >= 2)
		k_refit<<<blocks_for(n, 256), 256, 0, st>>>(
		    n, ws.parent_leaf.as<uint32_t>(), ws.parent_int.as<uint32_t>(), ws.left.as<uint32_t>(),
		    ws.right.as<uint32_t>(), ws.lbox.as<float4>(), ws.ibox.as<float4>(),
		    ws.flags.as<uint32_t>());

	// counters: [0], [1] frontier sizes, [2] nodes used, [3] triangles placed
	uint32_t init[4] = {1u, 0u, 1u, 0u};
	uint32_t *ctr = ws.counters.as<uint32_t>();
	BUILD_TRY(cudaMemcpyAsync(ctr, init, sizeof init, cudaMemcpyHostToDevice, st));
	Item root{n == 1 ? (kLeafBit | 0u) : 0u, 0u};
	BUILD_TRY(cudaMemcpyAsync(ws.items_a.p, &root, sizeof root, cudaMemcpyHostToDevice, st));
	Item *cur = ws.items_a.as<Item>(), *nxt = ws.items_b.as<Item>();
	int ci = 0;
	uint32_t level = 0;
	for (;;) {
		BUILD_TRY(cudaMemsetAsync(ctr + (ci ^ 1), 0, 4, st));
		k_collapse<<<1216, 128, 0, st>>>(cur, ctr + ci, nxt, ctr + (ci ^ 1), ctr + 2, node_cap,
		                                 ctr + 3, sc.nodes.as<Node8>(), ws.perm.as<uint32_t>(),
		                                 ws.left.as<uint32_t>(), ws.right.as<uint32_t>(),
		                                 ws.rfirst.as<uint32_t>(), ws.rlast.as<uint32_t>(),
		                                 ws.ibox.as<float4>(), ws.lbox.as<float4>(),
		                                 (uint32_t)leaf_size, n, d_err);
		++level;
		BUILD_TRY(cudaMemcpyAsync(ws.h_counters, ctr, 16, cudaMemcpyDeviceToHost, st));
		BUILD_TRY(cudaStreamSynchronize(st));
		if (ws.h_counters[ci ^ 1] == 0)
			break;
		std::swap(cur, nxt);
		ci ^= 1;
		if (level > 4096) {
			msg = "collapse did not terminate";
			return PRT_ERR_DEVICE;
		}
	}
	sc.n_nodes = ws.h_counters[2];
	sc.depth = level;
	if (ws.h_counters[3] != n) {
		msg = "collapse placed " + std::to_string(ws.h_counters[3]) + " of " + std::to_string(n) +
		      " triangles";
		return PRT_ERR_DEVICE;
	}
	k_relayout<<<blocks_for(n, 256), 256, 0, st>>>(d_tris, svals, ws.perm.as<uint32_t>(), n,
	                                               sc.tri4.as<float4>(), sc.inv.as<uint32_t>());
	if (compressed) {
		BUILD_TRY(sc.cnodes.reserve(sizeof(CNode8) * (size_t)sc.n_nodes));
		k_compress<<<blocks_for(sc.n_nodes, 128), 128, 0, st>>>(sc.nodes.as<Node8>(), sc.n_nodes,
		                                                        sc.cnodes.as<CNode8>());
		sc.has_cnodes = true;
	}
	BUILD_TRY(cudaGetLastError());
	BUILD_TRY(cudaStreamSynchronize(st));
	return PRT_OK;
}

} // namespace prt
