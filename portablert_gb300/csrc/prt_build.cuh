// prt_build.cuh - device scene and the LBVH build pipeline (prt_build.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "prt_internal.cuh"
#include "prt_sort.cuh"

namespace prt {

// Grow-only device allocation.
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

struct SceneGPU {
	uint64_t n_tris = 0;
	uint32_t n_nodes = 0;
	uint32_t depth = 0;
	int leaf_size = 4;
	bool has_cnodes = false;
	DevBuf tri4;   // float4[3 n]
	DevBuf inv;    // uint32[n]: primitive id -> position in tri4
	DevBuf nodes;  // Node8[n_nodes]
	DevBuf cnodes; // CNode8[n_nodes]
	void release() {
		tri4.release();
		inv.release();
		nodes.release();
		cnodes.release();
		n_tris = 0;
		n_nodes = 0;
		depth = 0;
		has_cnodes = false;
	}
};

// Scratch reused across builds (grow-only).
struct BuildScratch {
	DevBuf keys, vals, keys2, vals2;  // Morton codes and triangle indices (sort ping-pong)
	DevBuf left, right;               // children of the n-1 binary nodes (bit 31 = leaf)
	DevBuf parent_int, parent_leaf;   // parents of binary nodes and of leaves
	DevBuf rfirst, rlast;             // leaf range of each binary node
	DevBuf ibox, lbox;                // boxes of binary nodes and of leaves (2 float4 each)
	DevBuf flags;                     // refit arrival counters
	DevBuf items_a, items_b;          // collapse frontiers
	DevBuf counters;                  // small device counters
	DevBuf perm;                      // leaf-order slot -> sorted index
	DevBuf sort_hist, sort_tiles, sort_status;
	DevBuf bounds;                    // centroid bounds (6 ordered words)
	uint32_t *h_counters = nullptr;   // pinned mirror of `counters`
	void release();
};

// Builds the 8-wide tree for n triangles at d_tris (n x 9 floats, device memory) into
// `sc`.  compressed: also encode CNode8.  Synchronises `st`.  Returns PRT_* status;
// on error `msg` says why.
int build_scene(const float *d_tris, uint64_t n, int leaf_size, bool compressed, SceneGPU &sc,
                BuildScratch &ws, cudaStream_t st, uint32_t *d_err, std::string &msg);

} // namespace prt
