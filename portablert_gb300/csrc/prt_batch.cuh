// prt_batch.cuh - the batch behind the prt_b200_batch handle (prt_batch.cu), shared
// with the request server (prt_serve.cu), which keeps its scenes in a batch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"
#include "prt_ctx.cuh"
#include "prt_traverse.cuh"

namespace prt {

constexpr int kSlots = 8; // launches that may be in flight on one batch

struct BatchSlot {
	DevBuf segs;  // SegDesc table of the launch
	DevBuf work;  // [0] ray counter, [1] error word, [16..31] visit counters
	cudaEvent_t done = nullptr;
	bool pending = false;
};

} // namespace prt

struct prt_b200_batch {
	prt_b200_ctx *ctx = nullptr;
	prt::SceneGPU arena;
	// The batch's own build scratch: a captured graph reads tables uploaded before the
	// capture, so nothing outside the batch may overwrite them between replays.
	prt::BuildScratch ws;
	bool built = false;
	prt::DevBuf scenes_fp32, scenes_comp; // SceneDesc[S] for each node format
	prt::BatchSlot slots[prt::kSlots];
	int next_slot = 0;
	double build_ms = 0.0;
	bool built_sah = false; // the resident trees are SAH trees (set_tris_dev)
	unsigned long long visits[2] = {0, 0};
	uint32_t *h_words = nullptr; // pinned: error word and visit counters read back
	// CUDA graph of build + query
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t gexec = nullptr;
	std::string graph_key;
	prt::BatchSlot gslot;
	prt::BuildPlan gplan;
	bool graph_dirty = false;   // arena stats not read back since the last replay
};

