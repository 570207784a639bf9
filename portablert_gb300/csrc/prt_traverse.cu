// prt_traverse.cu - persistent nearest-hit traversal of the 8-wide tree.
//
// Replaces BVH2::nearest_tri (portableRT bvh.hpp:224-265) and the std::thread loop of
// CPUBackend::nearest_hits (intersect_cpu.hpp:20-43).
//
// Answer (identical to the reference's on finite inputs): the smallest t over the
// triangles whose own bounding box passes the reference slab test and which
// Moller-Trumbore accepts; t may be negative, there is no t-min and no culling by t,
// exactly as in the reference.  Inner nodes only prune with tests that are
// conservative for that set (prt_internal.cuh), so the tree's shape and the visit
// order do not change the answer; ties in t go to the smaller primitive id.
//
// Execution: a persistent grid (resident blocks on every SM); each warp takes 32
// consecutive rays at a time from a global counter, one ray per thread, with a
// per-thread stack of child references.  Hit records are assembled in shared memory
// in the caller's HitReg<Tags...> layout and the warp writes its 32 records (a
// contiguous, 128-B aligned run) with 16-byte stores.
//
// Algorithmic bytes per ray: 24 (ray) + R (record) + node bytes visited + 48 per
// triangle tested; the counting variant (COUNT) measures the visits.
#include <algorithm>

#include "../../include/prt_b200.h"
#include "prt_traverse.cuh"

namespace prt {

namespace {

constexpr int kStack = 192;

struct TravArgs {
	const float4 *tri4;
	const void *nodes;
	const float *rays;
	uint8_t *out;
	uint32_t n_tris;
	uint32_t n_rays;
	uint32_t rec_size;
	uint32_t mask;
	uint32_t off[8];
	uint32_t store_mode; // 0: 16-B stores, 1: 4-B stores, 2: byte stores
	uint32_t *counter;
	uint32_t *err;
	unsigned long long *visits;
};

__device__ __forceinline__ bool box_test(const RayC &r, float lx, float hx, float ly, float hy,
                                         float lz, float hz) {
	return r.kind == 0 ? regular_box(r, lx, hx, ly, hy, lz, hz)
	                   : conservative_box(r, lx, hx, ly, hy, lz, hz);
}

__device__ __forceinline__ uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xFFu; }

template <int FMT, bool COUNT>
__device__ __forceinline__ bool trace(const TravArgs &a, const RayC &r, Best &best,
                                      uint32_t &n_nodes, uint32_t &n_tris) {
	uint32_t stack[kStack];
	int sp = 0;
	stack[sp++] = 0u;
	while (sp > 0) {
		const uint32_t ref = stack[--sp];
		if (ref_is_leaf(ref)) {
			const uint32_t cnt = leaf_count(ref);
			const float4 *p = a.tri4 + 3 * (size_t)leaf_first(ref);
			for (uint32_t k = 0; k < cnt; ++k) {
				float4 A = __ldg(p + 3 * k), B = __ldg(p + 3 * k + 1), C = __ldg(p + 3 * k + 2);
				test_triangle(r, A, B, C, best);
			}
			if (COUNT)
				n_tris += cnt;
			continue;
		}
		if (COUNT)
			++n_nodes;
		if (FMT == PRT_NODES_FP32) {
			const float4 *np = reinterpret_cast<const float4 *>(
			    static_cast<const Node8 *>(a.nodes) + ref);
			float4 q[12];
#pragma unroll
			for (int i = 0; i < 12; ++i)
				q[i] = __ldg(np + i);
			const uint4 r0 = __ldg(reinterpret_cast<const uint4 *>(np) + 12);
			const uint4 r1 = __ldg(reinterpret_cast<const uint4 *>(np) + 13);
			const float lx[8] = {q[0].x, q[0].y, q[0].z, q[0].w, q[1].x, q[1].y, q[1].z, q[1].w};
			const float hx[8] = {q[2].x, q[2].y, q[2].z, q[2].w, q[3].x, q[3].y, q[3].z, q[3].w};
			const float ly[8] = {q[4].x, q[4].y, q[4].z, q[4].w, q[5].x, q[5].y, q[5].z, q[5].w};
			const float hy[8] = {q[6].x, q[6].y, q[6].z, q[6].w, q[7].x, q[7].y, q[7].z, q[7].w};
			const float lz[8] = {q[8].x, q[8].y, q[8].z, q[8].w, q[9].x, q[9].y, q[9].z, q[9].w};
			const float hz[8] = {q[10].x, q[10].y, q[10].z, q[10].w,
			                     q[11].x, q[11].y, q[11].z, q[11].w};
			const uint32_t rf[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
#pragma unroll
			for (int c = 0; c < 8; ++c) {
				if (rf[c] == kNone)
					continue;
				if (box_test(r, lx[c], hx[c], ly[c], hy[c], lz[c], hz[c])) {
					if (sp >= kStack)
						return false;
					stack[sp++] = rf[c];
				}
			}
		} else {
			const uint4 *np = reinterpret_cast<const uint4 *>(
			    static_cast<const CNode8 *>(a.nodes) + ref);
			const uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3),
			            w4 = __ldg(np + 4);
			const float ox = __uint_as_float(w0.x), oy = __uint_as_float(w0.y),
			            oz = __uint_as_float(w0.z);
			const float sx = cscale((uint8_t)byte_of(w0.w, 0)), sy = cscale((uint8_t)byte_of(w0.w, 1)),
			            sz = cscale((uint8_t)byte_of(w0.w, 2));
			const uint32_t imask = byte_of(w0.w, 3);
			const uint32_t child_base = w1.x, tri_base = w1.y;
			const uint32_t meta[2] = {w1.z, w1.w};
			// q rows: lo_x = w2.x,w2.y  hi_x = w2.z,w2.w  lo_y = w3.x,w3.y  hi_y = w3.z,w3.w
			//         lo_z = w4.x,w4.y  hi_z = w4.z,w4.w
			uint32_t inner_rank = 0, toff = 0;
#pragma unroll
			for (int c = 0; c < 8; ++c) {
				const int h = c >> 2, b = c & 3;
				const uint32_t m = byte_of(meta[h], b);
				const bool inner = (imask >> c) & 1u;
				uint32_t child;
				if (inner)
					child = child_base + inner_rank++;
				else if (m)
					child = make_leaf(tri_base + toff, m);
				else
					continue;
				toff += m;
				const float lxc = __fadd_rn(ox, __fmul_rn((float)byte_of(h ? w2.y : w2.x, b), sx));
				const float hxc = __fadd_rn(ox, __fmul_rn((float)byte_of(h ? w2.w : w2.z, b), sx));
				const float lyc = __fadd_rn(oy, __fmul_rn((float)byte_of(h ? w3.y : w3.x, b), sy));
				const float hyc = __fadd_rn(oy, __fmul_rn((float)byte_of(h ? w3.w : w3.z, b), sy));
				const float lzc = __fadd_rn(oz, __fmul_rn((float)byte_of(h ? w4.y : w4.x, b), sz));
				const float hzc = __fadd_rn(oz, __fmul_rn((float)byte_of(h ? w4.w : w4.z, b), sz));
				if (box_test(r, lxc, hxc, lyc, hyc, lzc, hzc)) {
					if (sp >= kStack)
						return false;
					stack[sp++] = child;
				}
			}
		}
	}
	return true;
}

template <int FMT, bool COUNT>
__global__ void __launch_bounds__(128) k_nearest(TravArgs a) {
	extern __shared__ __align__(16) uint32_t stage_all[];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint32_t *stage = stage_all + warp * 256; // 32 records x 32 B
	uint8_t *stage_b = reinterpret_cast<uint8_t *>(stage);
	const uint32_t rw = a.rec_size >> 2;
	uint32_t n_nodes = 0, n_tris = 0;
	for (;;) {
		uint32_t base = 0;
		if (lane == 0)
			base = atomicAdd(a.counter, 32u);
		base = __shfl_sync(0xFFFFFFFFu, base, 0);
		if (base >= a.n_rays)
			break;
		const uint32_t i = base + lane;
		const bool active = i < a.n_rays;
		Best best;
		best_init(best);
		RayC r;
		if (active) {
			const float2 *rp = reinterpret_cast<const float2 *>(a.rays + 6 * (size_t)i);
			const float2 p0 = __ldg(rp), p1 = __ldg(rp + 1), p2 = __ldg(rp + 2);
			r = make_ray(p0.x, p0.y, p1.x, p1.y, p2.x, p2.y);
			if (a.n_tris && !trace<FMT, COUNT>(a, r, best, n_nodes, n_tris))
				atomicOr(a.err, kErrStack);
		}
		for (uint32_t w = 0; w < rw; ++w)
			stage[lane * rw + w] = 0u;
		__syncwarp();
		if (active) {
			uint8_t *rb = stage_b + lane * a.rec_size;
			if (a.mask & PRT_FIELD_UV) {
				*reinterpret_cast<float *>(rb + a.off[PRT_OFF_U]) = best.u;
				*reinterpret_cast<float *>(rb + a.off[PRT_OFF_V]) = best.v;
			}
			if (a.mask & PRT_FIELD_T)
				*reinterpret_cast<float *>(rb + a.off[PRT_OFF_T]) = best.t;
			if (a.mask & PRT_FIELD_PRIMITIVE_ID)
				*reinterpret_cast<uint32_t *>(rb + a.off[PRT_OFF_PID]) = best.pid;
			if (a.mask & PRT_FIELD_VALID)
				rb[a.off[PRT_OFF_VALID]] = best.t < INFINITY ? 1 : 0;
			if (a.mask & PRT_FIELD_P) {
				// bvh.hpp:261-263: p = origin + t * direction, per component.
				*reinterpret_cast<float *>(rb + a.off[PRT_OFF_PX]) =
				    __fadd_rn(r.ox, __fmul_rn(best.t, r.dx));
				*reinterpret_cast<float *>(rb + a.off[PRT_OFF_PY]) =
				    __fadd_rn(r.oy, __fmul_rn(best.t, r.dy));
				*reinterpret_cast<float *>(rb + a.off[PRT_OFF_PZ]) =
				    __fadd_rn(r.oz, __fmul_rn(best.t, r.dz));
			}
		}
		__syncwarp();
		const uint32_t nrec = min(32u, a.n_rays - base);
		uint8_t *dst = a.out + (size_t)base * a.rec_size;
		const uint32_t bytes = nrec * a.rec_size;
		if (a.store_mode == 0 && nrec == 32u) {
			uint4 *d4 = reinterpret_cast<uint4 *>(dst);
			const uint4 *s4 = reinterpret_cast<const uint4 *>(stage);
			for (uint32_t c = lane; c < bytes / 16u; c += 32u)
				d4[c] = s4[c];
		} else if (a.store_mode <= 1) {
			uint32_t *d1 = reinterpret_cast<uint32_t *>(dst);
			for (uint32_t c = lane; c < bytes / 4u; c += 32u)
				d1[c] = stage[c];
		} else {
			for (uint32_t c = lane; c < bytes; c += 32u)
				dst[c] = stage_b[c];
		}
		__syncwarp();
	}
	if (COUNT) {
		unsigned long long a0 = n_nodes, a1 = n_tris;
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

template <int FMT, bool COUNT> int blocks_per_sm(int block) {
	static int cached_block = -1, cached = 0;
	if (cached_block != block) {
		int b = 0;
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_nearest<FMT, COUNT>, block,
		                                              (block / 32) * 1024);
		cached = b > 0 ? b : 1;
		cached_block = block;
	}
	return cached;
}

template <int FMT, bool COUNT>
void launch(const TravArgs &a, int block, int sm_count, cudaStream_t st) {
	const int bps = blocks_per_sm<FMT, COUNT>(block);
	uint64_t need = (a.n_rays + (uint64_t)block - 1) / block;
	uint64_t grid = std::min<uint64_t>((uint64_t)sm_count * bps, need);
	k_nearest<FMT, COUNT><<<(unsigned)grid, block, (block / 32) * 1024, st>>>(a);
}

} // namespace

cudaError_t launch_nearest_hits(const SceneGPU &sc, const float *d_rays, uint64_t n,
                                const OutLayout &lay, void *d_out, const TravConfig &cfg,
                                uint32_t *d_work, unsigned long long *d_visits, uint32_t *d_err,
                                cudaStream_t st, int sm_count) {
	if (cfg.count)
		cudaMemsetAsync(d_visits, 0, 2 * sizeof(unsigned long long), st);
	const uint64_t chunk = 1ull << 31;
	const int block = (cfg.block >= 32 && cfg.block <= 128 && cfg.block % 32 == 0) ? cfg.block : 128;
	for (uint64_t s = 0; s < n; s += chunk) {
		const uint64_t m = std::min(chunk, n - s);
		TravArgs a;
		a.tri4 = sc.tri4.as<float4>();
		a.nodes = cfg.format == PRT_NODES_COMPRESSED ? sc.cnodes.p : sc.nodes.p;
		a.rays = d_rays + 6 * s;
		a.out = static_cast<uint8_t *>(d_out) + s * lay.rec_size;
		a.n_tris = (uint32_t)sc.n_tris;
		a.n_rays = (uint32_t)m;
		a.rec_size = lay.rec_size;
		a.mask = lay.mask;
		for (int k = 0; k < 8; ++k)
			a.off[k] = lay.off[k];
		uintptr_t addr = reinterpret_cast<uintptr_t>(a.out);
		a.store_mode = (addr % 16 == 0) ? 0u : ((addr % 4 == 0) ? 1u : 2u);
		a.counter = d_work;
		a.err = d_err;
		a.visits = d_visits;
		cudaError_t e = cudaMemsetAsync(d_work, 0, 4, st);
		if (e != cudaSuccess)
			return e;
		if (cfg.format == PRT_NODES_COMPRESSED) {
			if (cfg.count)
				launch<PRT_NODES_COMPRESSED, true>(a, block, sm_count, st);
			else
				launch<PRT_NODES_COMPRESSED, false>(a, block, sm_count, st);
		} else {
			if (cfg.count)
				launch<PRT_NODES_FP32, true>(a, block, sm_count, st);
			else
				launch<PRT_NODES_FP32, false>(a, block, sm_count, st);
		}
		e = cudaGetLastError();
		if (e != cudaSuccess)
			return e;
	}
	return cudaSuccess;
}

} // namespace prt
