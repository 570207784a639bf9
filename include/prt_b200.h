/*
 * prt_b200.h - C ABI of the GB300 (sm_103a) ray-query backend for portableRT.
 *
 * The C++ backend class (include/portableRT/intersect_b200.hpp) and any FFI caller
 * reach the CUDA kernels only through these functions: plain pointers and sizes, no
 * CUDA or torch types.  Every function returns 0 on success and a PRT_ERR_* code
 * otherwise; the message is kept per context (prt_b200_last_error).  Nothing aborts.
 *
 * Ownership: input arrays are borrowed for the duration of a call; the scene built by
 * prt_b200_set_tris lives in device memory owned by the context until the next
 * set_tris or prt_b200_destroy; output buffers belong to the caller.
 *
 * Threading: calls on one context are serialised by a mutex inside the context.
 * Different contexts are independent.
 */
#ifndef PRT_B200_H
#define PRT_B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct prt_b200_ctx prt_b200_ctx;

enum {
	PRT_OK = 0,
	PRT_ERR_ARG = 1,          /* bad argument (null pointer, bad layout, size) */
	PRT_ERR_CUDA = 2,         /* a CUDA runtime call failed */
	PRT_ERR_NO_DEVICE = 3,    /* no sm_103 device */
	PRT_ERR_NO_SCENE = 4,     /* nearest_hits before set_tris */
	PRT_ERR_DEVICE = 5,       /* a kernel reported an error (see last_error) */
	PRT_ERR_OOM = 6,          /* device or host allocation failed (or a thread did not start) */
	PRT_ERR_LIMIT = 7         /* a documented size limit was exceeded */
};

/* Field bits of the hit record, one per portableRT filter tag. */
#define PRT_FIELD_UV 1u
#define PRT_FIELD_T 2u
#define PRT_FIELD_PRIMITIVE_ID 4u
#define PRT_FIELD_P 8u
#define PRT_FIELD_VALID 16u

/* Byte offsets inside one HitReg<Tags...> record, in this order:
 * u, v, t, primitive_id, valid, px, py, pz.  Offsets of absent fields are ignored. */
#define PRT_OFF_U 0
#define PRT_OFF_V 1
#define PRT_OFF_T 2
#define PRT_OFF_PID 3
#define PRT_OFF_VALID 4
#define PRT_OFF_PX 5
#define PRT_OFF_PY 6
#define PRT_OFF_PZ 7

/* Acceleration-structure node formats (option "node_format"). */
#define PRT_NODES_FP32 0       /* 8-wide nodes, FP32 child boxes (256 B) */
#define PRT_NODES_COMPRESSED 1 /* 8-wide nodes, 8-bit child boxes rounded outward (96 B) */

/* Replaces CPUBackend::is_available (portableRT src/intersect_cpu.cpp:9) for this
 * backend: 1 when a device of compute capability 10.3 is visible.  Cheap, no context. */
int prt_b200_available(void);

/* Replaces Backend::init (include/portableRT/backend.hpp:21): creates the per-backend
 * state (stream, error word) on `device`. */
int prt_b200_create(int device, prt_b200_ctx **out);

/* Replaces Backend::shutdown (backend.hpp:22): frees every device and host resource. */
void prt_b200_destroy(prt_b200_ctx *ctx);

/* Message of the last failing call on ctx ("" if none).  With ctx == NULL: the last
 * failure of prt_b200_create, prt_b200_obj_load or prt_b200_gltf_load in this thread.  The string is the
 * calling thread's copy, valid until its next call of this function. */
const char *prt_b200_last_error(const prt_b200_ctx *ctx);

/* Replaces Backend::device_name (backend.hpp:23). */
int prt_b200_device_name(prt_b200_ctx *ctx, char *buf, size_t len);

/* Replaces Backend::set_tris -> BVH2::build (backend.hpp:19, src/intersect_cpu.cpp:12,
 * include/portableRT/bvh.hpp:158-193).  tris9: n x 9 floats (v0, v1, v2), host memory.
 * Builds an 8-wide LBVH on the device; primitive_id of triangle i is i. */
int prt_b200_set_tris(prt_b200_ctx *ctx, const float *tris9, uint64_t n);

/* As prt_b200_set_tris with tris9 already in device memory (read on the context's
 * stream; the build is complete when the call returns). */
int prt_b200_set_tris_dev(prt_b200_ctx *ctx, const float *d_tris9, uint64_t n);

/* Replaces CPUBackend::nearest_hits<Tags...> (include/portableRT/intersect_cpu.hpp:20-43)
 * and BVH2::nearest_tri (bvh.hpp:224-265).  rays6: n x 6 floats (origin, direction) in
 * host memory; out_host: n records of rec_size bytes laid out by `offs` (see
 * PRT_OFF_*), written only for the fields in field_mask.  Synchronous. */
int prt_b200_nearest_hits(prt_b200_ctx *ctx, const float *rays6, uint64_t n,
                          uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                          void *out_host);

/* Device-resident variant: d_rays6 and d_out are device pointers (d_rays6 8-byte
 * aligned, else PRT_ERR_ARG; d_out any alignment); the work is queued on `stream` (a
 * cudaStream_t, NULL = the context's stream) and the call returns without waiting.
 * prt_b200_sync waits and reports kernel-side errors. */
int prt_b200_nearest_hits_dev(prt_b200_ctx *ctx, const float *d_rays6, uint64_t n,
                              uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                              void *d_out, void *stream);

/* Waits for the context's queued work and reports errors the kernels flagged. */
int prt_b200_sync(prt_b200_ctx *ctx);

/* No counterpart in the reference.  prt_b200_nearest_hits for programs that must not
 * allocate device memory once running (for example a renderer that reserves its memory
 * at start-up and forbids allocation in its frame loop: cudaMalloc can synchronise the
 * device and can fail under a fixed budget).  Same arguments and results as
 * prt_b200_nearest_hits, but the call allocates nothing: rays, records, the ray counter
 * and the error word are staged in one fixed device array of the library (3.5 MiB on
 * each device that loads it, kept until the process exits).  At most 65536 rays per
 * call; more returns PRT_ERR_LIMIT.  The first call on a device looks the array's
 * address up (cudaGetSymbolAddress), so make that first call before any stream capture.
 * All calls share the array: they are synchronous and serialised by a process-wide
 * lock; GPU work of two calls that overlapped would race.  The context and the scene
 * must already exist (prt_b200_create, prt_b200_set_tris allocate).  Kernel errors are
 * reported as prt_b200_nearest_hits reports them: this call's own, and any that earlier
 * asynchronous calls on the context (the _dev calls) left pending. */
int prt_b200_nearest_hits_noalloc(prt_b200_ctx *ctx, const float *rays6, uint64_t n,
                                  uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                                  void *out_host);

/* ---- Batches: many scenes on the device at once --------------------------------------
 * No counterpart in the reference, which holds one scene per backend (Backend::set_tris,
 * backend.hpp:19).  A batch builds S scenes in one pass and answers any number of
 * queries against them with one persistent launch; each answer equals what
 * nearest_hits<Tags...> gives for that scene alone.  A batch uses its context's device,
 * options and scratch; calls on it are serialised with the context's. */
typedef struct prt_b200_batch prt_b200_batch;

/* One query: rays of one scene of the batch and where their records go (device memory,
 * layout as in prt_b200_nearest_hits). */
typedef struct {
	uint32_t scene;      /* index of the scene in the batch */
	uint32_t field_mask; /* PRT_FIELD_* */
	const float *rays;   /* n_rays x 6 floats, device memory, 8-byte aligned */
	uint64_t n_rays;
	void *out;           /* n_rays records of rec_size bytes, device memory */
	uint32_t rec_size;
	uint8_t offs[8];     /* PRT_OFF_* */
} prt_b200_query;

int prt_b200_batch_create(prt_b200_ctx *ctx, prt_b200_batch **out);
void prt_b200_batch_destroy(prt_b200_batch *batch);

/* Builds every scene: scene s is d_tris[tri_off[s] .. tri_off[s+1]) (triangles of 9
 * floats in device memory; tri_off is host memory with n_scenes + 1 entries, starting at
 * 0).  Primitive ids are per scene, from 0.  Synchronous. */
int prt_b200_batch_set_tris_dev(prt_b200_batch *batch, const float *d_tris,
                                const uint64_t *tri_off, uint32_t n_scenes);

/* Answers all queries with one launch queued on `stream` (NULL = the context's).  Up to
 * 8 launches per batch may be in flight; prt_b200_batch_sync waits for them. */
int prt_b200_batch_query_dev(prt_b200_batch *batch, const prt_b200_query *queries,
                             uint32_t n_queries, void *stream);

/* Build + query as one CUDA graph: the first call with these arguments (device pointers,
 * offsets, queries and the context's options) captures the whole build and the query
 * launch and instantiates the graph; later calls with the same arguments replay it on
 * `stream`.  Inputs are read when the graph runs. */
int prt_b200_batch_run_graph(prt_b200_batch *batch, const float *d_tris,
                             const uint64_t *tri_off, uint32_t n_scenes,
                             const prt_b200_query *queries, uint32_t n_queries, void *stream);

/* Waits for the batch's launches and reports kernel-side errors. */
int prt_b200_batch_sync(prt_b200_batch *batch);

/* "n_scenes", "n_tris", "n_nodes", "depth", "build_ms", "build_sah" (1 = set_tris_dev
 * built SAH trees), "visits_nodes", "visits_tris". */
int prt_b200_batch_stat(prt_b200_batch *batch, const char *key, double *value);

/* Tuning and statistics.  Options (take effect at the next set_tris unless noted):
 *   "leaf_size"    1..8  most triangles per leaf of the 8-wide tree (default 1)
 *   "node_format"  PRT_NODES_FP32 or PRT_NODES_COMPRESSED (default FP32; applies to the
 *                  next nearest_hits when both formats have been built)
 *   "block"        threads per block of the traversal kernel (default 128)
 *   "count_visits" 1 = the traversal also accumulates node / triangle visit counts
 *   "pool_depth"   0..32: tree depth the traversal's shared-memory pool is sized for in
 *                  a batch graph, where the depth is not known when the graph is
 *                  captured (0 = 32, always enough; a smaller value raises occupancy,
 *                  and a tree it does not fit makes the query fail with
 *                  PRT_ERR_DEVICE, never a wrong answer)
 *   "build_compressed" 1 = set_tris also builds the compressed nodes (default 1)
 *   "build_sah"    1 = set_tris builds the binary tree top-down with binned SAH, as
 *                  portableRT's own build does (default 1: about 5x the build time of
 *                  0 = Morton LBVH, for about 10 % fewer node visits per ray); an SAH
 *                  tree too deep for the traversal falls back to the LBVH.  Also
 *                  batch_set_tris_dev and request servers; batch graphs always build
 *                  LBVH trees.
 *   "collapse_cost" 1 = the binary tree is collapsed to 8-wide nodes by the least
 *                  expected cost per ray (a bottom-up pass chooses which subtrees become
 *                  nodes and leaves), 0 = by opening the largest child first (default 1)
 *   "build_small"  1 = with build_sah, set_tris builds a scene of at most 4,096 triangles
 *                  in one thread block: Morton order, PLOC clustering (radius 3) into a
 *                  binary tree whose least-cost records are computed as it merges, the
 *                  collapse and the triangle re-layout in one launch (default 1; 0 = the
 *                  binned-SAH build at every size)
 *   "host_direct"  1 = a host-buffer nearest_hits whose buffers the device can reach in
 *                  place (pinned memory; pageable memory where the device reads it
 *                  through the host's page tables, as on Grace) traverses them there:
 *                  rays read and records written over the host link, no staging copies
 *                  (default 1; rays not 8-byte aligned are copied); 0 = always the
 *                  chunked copy pipeline below
 *   "fail_alloc_after" test hook: n > 0 makes the n-th device buffer growth from now
 *                  on (in any context of the process) fail as if the device were out of
 *                  memory, once; the call that meets it returns PRT_ERR_OOM and the
 *                  context stays usable.  0 disarms (default 0).  Only this call sets
 *                  it; it has no environment override
 *   "fail_serve_after" test hook: n > 0 makes persistent request servers created
 *                  afterwards treat their n-th publication as if one of its batches had
 *                  faulted: the request never completes and the fault flag rises from the
 *                  host.  The server stops its launch once the rest of the published work
 *                  is done, fails that request with PRT_ERR_DEVICE, resets its queues and
 *                  serves again.  0 = off (default 0).  Only this call sets it
 *   "pipe_chunks"  1..16: chunks a host-buffer nearest_hits splits its rays into, so
 *                  copies and traversals overlap (default 8)
 *   "pipe_min_rays" fewest rays per chunk, a multiple of 32 (default 2^15)
 *   "serve_batches_per_warp" request servers created afterwards launch waves whose
 *                  warps take at most this many batches of 32 rays (0 = until the
 *                  work runs out; default 1): lower lets an express wave start sooner
 *   "serve_persistent" request servers created afterwards: 1 = admitted requests are
 *                  folded into one running launch whose warps take their batches from
 *                  three device queues by request size (up to 64 Ki rays, up to 512 Ki,
 *                  larger; smaller first) while the host appends to them; the launch stops after 5 ms without work and starts again
 *                  with the next request (default 1); 0 = each group of admitted
 *                  requests is a wave, one launch on one of the server's lanes
 *   "pipe_ramp"    1 = chunk sizes ramp up and down (1, 2, 4, 8, ..., 8, 4, 2, 1), so
 *                  the unoverlapped first copy-in and last copy-out are short (default 1)
 * Statistics: "n_tris", "n_nodes", "depth", "build_ms", "build_sah" (1 = the scene's tree
 *   is from the quality build: binned SAH, or the one-block build), "build_small" (1 = the
 *   one-block build made it), "in_place" (1 = the last host-buffer nearest_hits traversed the
 *   caller's buffers in place), "node_bytes", "tri_bytes",
 *   "visits_nodes", "visits_tris" (totals of the last counted nearest_hits), "sms".
 * Every option but the test hook can also be set for each new context from the
 * environment:
 *   PRT_B200_<OPTION> (the name in upper case), e.g. PRT_B200_LEAF_SIZE=4 or
 *   PRT_B200_BUILD_SAH=0, so programs that use the backend through portableRT's API are
 *   tuned without a change.  A value that is not a decimal integer makes
 *   prt_b200_create fail with PRT_ERR_ARG; one out of range, with the option's error. */
int prt_b200_set_option(prt_b200_ctx *ctx, const char *key, int64_t value);
int prt_b200_get_stat(prt_b200_ctx *ctx, const char *key, double *value);

/* Request server (no counterpart in portableRT): S scenes (device triangles and
 * offsets as for prt_b200_batch_set_tris_dev) are built once and stay resident; requests
 * (scene, host rays, record layout, host output) are admitted in arrival order while
 * their device buffers (24 B per ray rounded up to 256 B, plus the records) fit in a
 * region of budget_bytes reserved at creation, and each group of admitted requests
 * (a wave) runs as one launch on one of n_lanes streams, so up to n_lanes waves overlap.
 * With several lanes, lane 0 is an express lane of the highest stream priority that
 * carries only requests of at most 65,536 rays, taken ahead of larger ones; a wave's
 * warps take a bounded number of batches of 32 rays (option "serve_batches_per_warp"),
 * so a large wave's blocks retire as they finish and an express wave's blocks start
 * meanwhile.  Each request's records equal nearest_hits on its scene alone.  The
 * node format is the context's at creation.  Host buffers should be pinned: a copy
 * to or from pageable memory makes the scheduler wait for it.  Buffers belong to the
 * caller until prt_b200_server_wait returns for the ticket. */
typedef struct prt_b200_server prt_b200_server;
int prt_b200_server_create(prt_b200_ctx *ctx, const float *d_tris, const uint64_t *tri_off,
                           uint32_t n_scenes, uint64_t budget_bytes, uint32_t n_lanes,
                           prt_b200_server **server);
void prt_b200_server_destroy(prt_b200_server *server);
/* Queues a request (any thread); PRT_ERR_LIMIT if it can never fit the budget. */
int prt_b200_server_submit(prt_b200_server *server, uint32_t scene, const float *rays6,
                           uint64_t n_rays, uint32_t field_mask, uint32_t rec_size,
                           const uint8_t offs[8], void *out_host, uint64_t *ticket);
/* Blocks until the request is answered; latency_ms = submit to records in host memory.
 * Returns the request's status; the ticket is then forgotten. */
int prt_b200_server_wait(prt_b200_server *server, uint64_t ticket, double *latency_ms);
/* "waves", "express_waves", "max_in_flight_waves", "max_wave_requests", "completed",
 * "rays", "waiting",
 * "bytes_in_use", "peak_bytes", "budget_bytes", "n_scenes", "n_tris". */
int prt_b200_server_stat(prt_b200_server *server, const char *key, double *value);
const char *prt_b200_server_last_error(prt_b200_server *server);

/* Pinhole sensor camera of portableRT's examples, generated on the device (no ray
 * buffer, no ray copy).  Ray i is pixel x = i % width of row y = height - 1 - i / width
 * (the examples' loop order), with origin pos and, per form:
 *   PRT_CAMERA_PLANE (examples/bunny/main.cpp:101-124): sensor point (sx, sy, sensor_z),
 *     direction = (sensor - pos) / |sensor - pos|;
 *   PRT_CAMERA_PLANE_SENSOR_NORM (examples/validation/main.cpp:170-198): the same
 *     direction divided by |sensor| instead;
 *   PRT_CAMERA_ROTATED (examples/sponza/main.cpp:193-218): sensor point pos +
 *     (cos_a sx + sin_a sensor_dist, sy, -sin_a sx + cos_a sensor_dist), direction
 *     normalised by its length;
 * where sx = sensor_size * (float(x) / width - 0.5) with the subtraction in double
 * (likewise sy), all else in FP32 as the examples compute it: the rays are
 * bit-identical to the examples'. */
#define PRT_CAMERA_PLANE 0
#define PRT_CAMERA_PLANE_SENSOR_NORM 1
#define PRT_CAMERA_ROTATED 2
typedef struct prt_b200_camera {
	uint32_t width, height, form, pad;
	float pos[3];
	float sensor_size, sensor_dist, sensor_z, cos_a, sin_a;
} prt_b200_camera;

/* nearest_hits over the camera's width x height rays, records to device memory. */
int prt_b200_nearest_hits_camera(prt_b200_ctx *ctx, const prt_b200_camera *camera,
                                 uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                                 void *d_out, void *stream);
/* The camera's rays written to device memory (6 floats each). */
int prt_b200_camera_rays(prt_b200_ctx *ctx, const prt_b200_camera *camera, float *d_rays6,
                         void *stream);
/* Headless Lambert shading of examples/sponza/main.cpp:11-32,228-243 into RGBA8 (one
 * grey byte in R, G and B, alpha 255): grey = 255 * clamp(N . -d, 0, 1) truncated, N the
 * unit geometric normal of the hit triangle of the context's scene, black for a miss
 * (t = inf).  Rays come from `camera` when it is not NULL, else from d_rays6; records
 * (device) need the t and primitive_id fields. */
int prt_b200_shade_lambert(prt_b200_ctx *ctx, const prt_b200_camera *camera,
                           const float *d_rays6, uint64_t n, const void *d_records,
                           uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                           uint8_t *d_rgba, void *stream);

/* Triangles of a Wavefront OBJ file (positions of every face, polygons split as fans),
 * in file order, as the examples read meshes for set_tris (examples/bunny/main.cpp:22-73).
 * *tris9 is allocated by the library (free it with prt_b200_free); errors are reported
 * by prt_b200_last_error(NULL).  Host only: needs no device. */
int prt_b200_obj_load(const char *path, float **tris9, uint64_t *n_tris);

/* Triangles of a glTF 2.0 file (.gltf with file or base64 data: buffers, or .glb), as
 * the sponza example reads its scene for set_tris (examples/sponza/main.cpp:35-101):
 * every mesh in order, each TRIANGLES primitive with POSITION and indices (others
 * skipped), triangles of consecutive index triples, mesh-space positions.  byteStride
 * is followed; an index or accessor out of range, a non-float VEC3 position, sparse
 * accessors and required extensions are errors.  Allocation, errors and freeing as
 * prt_b200_obj_load.  Host only: needs no device. */
int prt_b200_gltf_load(const char *path, float **tris9, uint64_t *n_tris);
void prt_b200_free(void *p);

/* Seeded synthetic workloads written straight into device memory (no counterpart in
 * portableRT, whose examples read meshes from files).  SplitMix64 streams; the same
 * generators as portablert_gb300/workloads.py (values that pass through log/cos may
 * differ from the host's in the last bit).  n items of 9 floats (triangles) or 6 floats
 * (rays) are written to d_out on `stream` (NULL = the context's). */
#define PRT_GEN_SOUP_TRIS 0    /* centres in [-1,1]^3, vertex offsets in [-0.05,0.05]^3 */
#define PRT_GEN_SOUP_RAYS 1    /* origins on the radius-3 sphere, aimed into [-0.5,0.5]^3 */
#define PRT_GEN_CLUSTER_TRIS 2 /* param = cluster count: Gaussian clusters in [-10,10]^3 */
#define PRT_GEN_RANDOM_RAYS 3  /* param = extent e: origins in [-e,e]^3, uniform directions */
int prt_b200_generate(prt_b200_ctx *ctx, int kind, uint64_t seed, uint64_t n, double param,
                      void *d_out, void *stream);

/* Measurement helper (no counterpart in the reference): *ms = device time of `passes`
 * read passes over the device buffer d_buf (bytes, 32-byte aligned, >= 128 KiB) with the
 * traversal's own 32-byte read-only loads, after one untimed pass; each pass a block
 * reads a different slice than before, so L1 does not serve it.  A buffer under the
 * L2 capacity gives the L2 -> SM read bandwidth (bytes x passes / time), a larger one
 * HBM's.  Synchronous, on the context's stream. */
int prt_b200_probe_read(prt_b200_ctx *ctx, const void *d_buf, uint64_t bytes, int passes,
                        float *ms);

/* FP64 scorer of t (no counterpart in portableRT; measurement only).  For every valid
 * record of a nearest_hits result (device buffers; the records need t, primitive_id and
 * valid), recomputes t by the Möller-Trumbore formula of core.hpp:27-65 in double on the
 * triangle the record names (d_tris9, the AoS array set_tris was given) and reports
 * result[0] max |t - t64|, [1] max |t - t64| / |t64|, [2] mean |t - t64|, [3] records
 * scored, [4] records whose t equals t64 rounded to FP32, [5] valid records that could
 * not be scored (primitive id out of range, t64 not finite).  Synchronous. */
int prt_b200_t_error(prt_b200_ctx *ctx, const float *d_tris9, uint64_t n_tris,
                     const float *d_rays6, uint64_t n_rays, const void *d_records,
                     uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                     double result[6]);

#ifdef __cplusplus
}
#endif
#endif /* PRT_B200_H */
