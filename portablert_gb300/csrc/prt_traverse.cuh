// prt_traverse.cuh - host entry of the nearest-hit traversal (prt_traverse.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "prt_build.cuh"

namespace prt {

struct OutLayout {
	uint32_t mask;      // PRT_FIELD_* bits
	uint32_t rec_size;  // bytes per record, 1..32
	uint8_t off[8];     // u, v, t, primitive_id, valid, px, py, pz
};

struct TravConfig {
	int format = 0;       // PRT_NODES_FP32 / PRT_NODES_COMPRESSED
	int block = 128;      // threads per block
	bool count = false;   // accumulate visit counters into d_visits[0..1]
};

// Levels of the 8-wide tree the traversal stack can hold.
int traversal_stack_depth();

// Queues one nearest-hit pass over n rays (device memory, 6 floats each) on `st`.
// d_work: 16 bytes of device scratch (ray counter); d_visits: 2 uint64 counters
// (node visits, triangle tests), used when cfg.count.
cudaError_t launch_nearest_hits(const SceneGPU &sc, const float *d_rays, uint64_t n,
                                const OutLayout &lay, void *d_out, const TravConfig &cfg,
                                uint32_t *d_work, unsigned long long *d_visits, uint32_t *d_err,
                                cudaStream_t st, int sm_count);

} // namespace prt
