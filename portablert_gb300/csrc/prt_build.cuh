// prt_build.cuh - device scenes and the build pipelines (binned SAH or LBVH, then the
// shared collapse, re-layout and compression: prt_sah.cu, prt_build.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "prt_internal.cuh"
#include "prt_sort.cuh"

namespace prt {

// Grow-only device allocation.
// Host-side fault injection for tests (option "fail_alloc_after"): after
// arm_alloc_failure(n), the n-th device buffer growth from then on, in any context,
// fails with cudaErrorMemoryAllocation without calling the allocator, as a device out of
// memory would; n = 0 disarms.  Nothing reaches the GPU: every caller checks the status
// before it launches anything.
void arm_alloc_failure(int64_t n);
bool alloc_failure_due();

struct DevBuf {
	void *p = nullptr;
	size_t bytes = 0;
	cudaError_t reserve(size_t b) {
		if (b <= bytes)
			return cudaSuccess;
		if (p)
			cudaFree(p);
		p = nullptr;
		bytes = 0;
		if (alloc_failure_due())
			return cudaErrorMemoryAllocation;
		cudaError_t e = cudaMalloc(&p, b);
		if (e == cudaSuccess)
			bytes = b;
		return e;
	}
	void release() {
		if (p)
			cudaFree(p);
		p = nullptr;
		bytes = 0;
	}
	template <class T> T *as() const { return static_cast<T *>(p); }
};

// One or more scenes built together into shared arrays ("arena").  Scene s owns the
// triangles [tri_off[s], tri_off[s+1]) of the input, its root is node s, its triangle
// records sit anywhere in tri4, and inv + tri_off[s] maps its primitive ids (0-based,
// per scene, as in the reference) to positions in tri4.
struct SceneGPU {
	uint32_t n_scenes = 0;
	uint64_t n_tris = 0; // all scenes
	uint32_t n_nodes = 0;
	uint32_t depth = 0;  // levels of the deepest tree
	int leaf_size = 1;
	bool has_cnodes = false;
	bool built_small = false; // the last build was the one-block build (prt_build_small.cu)
	uint32_t dead = 0;   // a node of eight empty children (past every built node): the
	                     // traversal pads a partial step with it
	DevBuf tri4;         // float4[3 n]
	DevBuf inv;          // uint32[n]
	DevBuf nodes;        // Node8[n_nodes], and the empty node at `dead`
	DevBuf cnodes;       // CNode8[n_nodes], likewise
	DevBuf tri_off;      // uint32[n_scenes + 1] (device copy)
	std::vector<uint64_t> h_tri_off;
	void release() {
		tri4.release();
		inv.release();
		nodes.release();
		cnodes.release();
		tri_off.release();
		h_tri_off.clear();
		n_scenes = 0;
		n_tris = 0;
		n_nodes = 0;
		depth = 0;
		has_cnodes = false;
	}
};

// Pinned words after the collapse's counter mirror: the SAH tiers' counters and error
// word as the host reads them between levels (a copy into pageable memory is staged).
constexpr int kHostSahWords = 16;

// Scratch reused across builds (grow-only).
struct BuildScratch {
	DevBuf keys, vals, keys2, vals2;  // Morton keys (u32 or u64) and triangle indices
	DevBuf scene_of;                  // scene of each input triangle (several scenes)
	DevBuf int_off;                   // first binary node of each scene
	DevBuf left, right;               // children of the binary nodes (bit 31 = leaf)
	DevBuf parent_int, parent_leaf;   // parents of binary nodes and of leaves
	DevBuf rfirst, rlast;             // leaf range of each binary node
	DevBuf ibox, lbox;                // boxes of binary nodes and of leaves (2 float4 each)
	DevBuf flags;                     // refit arrival counters
	DevBuf items_a, items_b;          // collapse frontiers
	DevBuf counters;                  // per-level frontier sizes, node / triangle counters
	DevBuf perm;                      // leaf-order slot -> sorted index
	DevBuf sort_hist, sort_tiles, sort_status;
	DevBuf bounds;                    // centroid bounds, 6 ordered words per scene
	DevBuf sah;                       // SAH build: records, task lists, bins, counters
	DevBuf roots;                     // SAH build: root binary node of each scene
	DevBuf cost;                      // cost-optimal collapse: 36 B per binary node
	uint32_t *h_counters = nullptr;   // pinned mirror of `counters`
	uint32_t *h_sah = nullptr;        // pinned, kHostSahWords (in the same allocation)
	void release();
};

// Host-side tables of one build (kept alive until its uploads have been queued).
struct BuildPlan {
	uint32_t S = 0, n = 0, n_int = 0, node_cap = 0;
	int leaf_size = 1, scene_digits = 0;
	bool compressed = false, multi = false;
	bool sah = false;                 // binned-SAH binary trees instead of LBVH
	bool collapse_cost = true;        // cost-optimal 8-wide collapse (else largest area first)
	bool small = false;               // one scene of 1..small_build_max() triangles, with the
	                                  // quality build requested: one block builds it (PLOC)
	std::vector<uint32_t> toff, ioff; // triangle and binary-node offsets per scene
};

// Validates the offsets, reserves every buffer of the build and queues the uploads of
// the offset tables on `st`.  Nothing after it allocates.
// sah: build the binary trees top-down with binned SAH (prt_sah.cu) instead of the
// Morton/Karras hierarchy; needs host checks.  collapse_cost: collapse to 8-wide nodes
// by the least expected cost (a bottom-up pass over the binary tree) instead of opening
// the largest child first.
// one_block: a single scene of at most small_build_max() triangles with sah set is built
// by one thread block (prt_build_small.cu) instead.
int build_plan(const uint64_t *tri_off, uint32_t n_scenes, int leaf_size, bool compressed,
               SceneGPU &sc, BuildScratch &ws, cudaStream_t st, BuildPlan &plan,
               std::string &msg, bool sah = false, bool collapse_cost = true,
               bool one_block = false);

// Queues the build kernels.  host_checks: read the level counters every few levels and
// finish with build_finish (synchronises).  Without host checks nothing synchronises:
// all 32 collapse levels are queued (empty ones return at once) and the compression
// kernel reads the node count on the device, so the whole build can be captured in a
// CUDA graph; call build_finish after it ran to learn the node count and depth.
int build_enqueue(const float *d_tris, const BuildPlan &plan, SceneGPU &sc, BuildScratch &ws,
                  cudaStream_t st, uint32_t *d_err, bool host_checks, std::string &msg);

// Reads the build's counters (synchronises `st`): node count, depth, placement check.
// on_host: the build wrote them to the pinned host buffer itself (no copy is queued).
int build_finish(SceneGPU &sc, BuildScratch &ws, cudaStream_t st, std::string &msg,
                 bool on_host = false);

// Builds the 8-wide trees of the scenes [tri_off[s], tri_off[s+1]) of the triangles at
// d_tris (n x 9 floats, device memory) into `sc`.  tri_off is host memory with
// n_scenes + 1 entries (tri_off[0] = 0).  compressed: also encode CNode8.
// Synchronises `st` (a few times, never per tree level).  Returns PRT_* status.
int build_scenes(const float *d_tris, const uint64_t *tri_off, uint32_t n_scenes, int leaf_size,
                 bool compressed, SceneGPU &sc, BuildScratch &ws, cudaStream_t st,
                 uint32_t *d_err, std::string &msg, bool sah = false,
                 bool collapse_cost = true, bool one_block = false);

// One scene: build_scenes with tri_off = {0, n}.
int build_scene(const float *d_tris, uint64_t n, int leaf_size, bool compressed, SceneGPU &sc,
                BuildScratch &ws, cudaStream_t st, uint32_t *d_err, std::string &msg,
                bool sah = false, bool collapse_cost = true, bool one_block = false);

// The one-block build (prt_build_small.cu): the largest scene it takes, and its launch
// (PLOC binary tree, collapse, triangle re-layout; the level counters at `ctr` end as
// the multi-launch build leaves them, and are copied to the pinned host buffer h_ctr;
// it also writes the empty node at sc.dead, in cnodes too when `compressed`).
uint32_t small_build_max();
cudaError_t launch_build_small(const float *d_tris, uint32_t n, uint32_t leaf_size, bool use_cost,
                               bool compressed, BuildScratch &ws, SceneGPU &sc, uint32_t node_cap,
                               uint32_t *ctr, uint32_t *h_ctr, uint32_t *d_err, cudaStream_t st);

} // namespace prt
