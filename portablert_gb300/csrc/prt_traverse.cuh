// prt_traverse.cuh - host entry of the nearest-hit traversal (prt_traverse.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"

namespace prt {

struct OutLayout {
	uint32_t mask;      // PRT_FIELD_* bits
	uint32_t rec_size;  // bytes per record, 4..32
	uint8_t off[8];     // u, v, t, primitive_id, valid, px, py, pz
};

struct TravConfig {
	int format = 0;       // PRT_NODES_FP32 / PRT_NODES_COMPRESSED
	int block = 128;      // threads per block
	bool count = false;   // accumulate visit counters into d_visits[0..1]
	int pool_depth = 0;   // size the pool for this depth instead of the scene's (0 = scene)
	// Batches of 32 rays a warp takes before it exits (0 = until the work runs out).  With
	// a bound the grid covers all batches and blocks retire as they finish, so the block
	// scheduler can interleave other launches (of higher-priority streams) meanwhile.
	uint32_t max_batches = 0;
};

// One scene as the traversal sees it: its arrays, root node and triangle count.
struct SceneDesc {
	const float4 *tri4;
	const uint32_t *inv; // primitive id -> tri4 position for this scene
	const void *nodes;   // Node8 or CNode8 array holding the scene's tree
	uint32_t root;
	uint32_t n_tris;
};

// A run of rays of one scene and where their records go.  vbegin (a multiple of 32) is
// the first index of the run in the launch's "virtual" ray numbering, in which every
// run is padded to whole warps, so a warp's 32 rays never mix runs.
struct SegDesc {
	unsigned long long vbegin;
	const float *rays;   // n_rays x 6 floats, device memory
	uint8_t *out;        // n_rays records of rec_size bytes, device memory
	uint32_t n_rays;
	uint32_t scene;      // index into the scene table
	uint32_t mask;
	uint32_t rec_size;
	uint8_t off[8];
	uint32_t store_mode; // 0: 16-B stores, 1: 4-B stores, 2: byte stores
	uint32_t pad;
	// Completion of the run (request servers; null: not tracked).  Each batch of the run
	// adds its rays to *done_ctr (device memory) once its records are stored and fenced
	// system-wide; the batch that completes the count then sets *done_flag (host memory
	// the device reaches) to 1, so a host thread sees the run's records finished without
	// waiting for the rest of the launch.  A batch whose traversal reported an error does
	// not count, so its run never completes early.
	uint32_t *done_ctr = nullptr;
	uint32_t *done_flag = nullptr;
};

// The state of one serving queue (device memory): the host appends runs to its segment
// table and then publishes their batches; warps of a running serving launch claim
// batches one at a time with a compare-and-swap on `next`.
struct ServeQueueState {
	uint32_t published; // batches of 32 rays published (the host's copies)
	uint32_t n_segs;    // runs in the table (copied by the host before `published`)
	uint32_t next;      // batches claimed
	uint32_t pad;
};

// A serving launch: kServeQueues queues in priority order (small requests' first).  The
// launch's warps claim batches while any is published; an idle warp polls with a
// growing sleep and leaves when *stop is set or after idle_limit polls, so the launch
// ends by itself.
constexpr int kServeQueues = 3;
struct ServeQueues {
	ServeQueueState *state[kServeQueues];
	const SegDesc *segs[kServeQueues];
	const uint32_t *stop;  // device memory, set by the host
	uint32_t *err_flag;    // host memory the device reaches: set to 1 when a batch faults
	uint32_t idle_limit;   // polls of an idle warp before it leaves
	uint32_t pad;
};

// Levels of the 8-wide tree the traversal can walk.
int traversal_stack_depth();

// Queues one nearest-hit pass over n rays of one scene (device memory, 6 floats each,
// or when cam is not null the camera's rays 0..n-1, n <= 2^31) on `st`.  d_work:
// device scratch of at least 4 words: [0] the ray counter, [2] the count of batches left
// to the general pass, [3] that pass's batch counter ([1] is not touched: callers keep
// their error word there);
// d_visits: 2 uint64 counters (node visits, triangle tests), used when cfg.count.
cudaError_t launch_nearest_hits(const SceneGPU &sc, const float *d_rays, uint64_t n,
                                const OutLayout &lay, void *d_out, const TravConfig &cfg,
                                uint32_t *d_work, unsigned long long *d_visits, uint32_t *d_err,
                                cudaStream_t st, int sm_count,
                                const prt_b200_camera *cam = nullptr);

// One persistent launch over several runs of rays, each against its own scene and with
// its own output layout.  d_scenes / d_segs: device copies of the tables (segments
// sorted by vbegin); n_virtual: the padded ray count (end of the last run).  depth and
// leaf_size: the largest over the scenes (they size the shared-memory pool and queue);
// n_nodes: the largest node array (bounds the steps of a batch); dead: the index of the
// empty node (SceneGPU::dead) in the node array every scene's `nodes` points into.
// d_work as above.
cudaError_t launch_nearest_hits_segments(const SceneDesc *d_scenes, const SegDesc *d_segs,
                                         uint32_t n_segs, unsigned long long n_virtual,
                                         uint32_t depth, int leaf_size, uint32_t n_nodes,
                                         uint32_t dead, const TravConfig &cfg,
                                         uint32_t *d_work, unsigned long long *d_visits,
                                         uint32_t *d_err, cudaStream_t st, int sm_count);

// Queues one serving launch over the queues `q` on `st` (resident warps only; it runs
// until it is stopped or idle).  Scenes as for launch_nearest_hits_segments.
cudaError_t launch_serving(const SceneDesc *d_scenes, const ServeQueues &q, uint32_t depth,
                           int leaf_size, uint32_t n_nodes, uint32_t dead, int format,
                           uint32_t *d_err, cudaStream_t st, int sm_count);

// Store mode for an output pointer (16-byte, 4-byte or byte stores).
inline uint32_t store_mode_for(const void *p) {
	const uintptr_t a = reinterpret_cast<uintptr_t>(p);
	return (a % 16 == 0) ? 0u : ((a % 4 == 0) ? 1u : 2u);
}

} // namespace prt
