// prt_sah.cuh - binned-SAH construction of the binary tree (prt_sah.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "prt_build.cuh"

namespace prt {

// Device scratch the SAH build of n triangles in S scenes needs (ws.sah).
size_t sah_scratch_bytes(uint32_t n, uint32_t S);

// Builds the binary trees of the plan's scenes top-down with binned SAH and writes what
// the collapse reads: ws.vals (position -> triangle), ws.lbox (by position), ws.left,
// ws.right, ws.rfirst, ws.rlast, ws.ibox (node ids up to n_int + S) and ws.roots
// (scene s -> its root node).  d_toff: the device triangle offsets; scene_of: the scene
// of each triangle (several scenes) or null.  Synchronises `st` every few levels.
int sah_build_enqueue(const float *d_tris, const BuildPlan &plan, BuildScratch &ws,
                      const uint32_t *d_toff, const uint32_t *scene_of, cudaStream_t st,
                      uint32_t *d_err, std::string &msg);

} // namespace prt
