// prt_capi.cu - the extern "C" boundary of the GB300 ray-query backend.
//
// Each entry point validates its arguments, takes the context's mutex, runs on the
// context's device and stream, and turns every CUDA or kernel-reported failure into a
// PRT_ERR_* status plus a message (prt_b200_last_error); nothing aborts or throws
// across the boundary.  The reference reports errors by printing and carrying on
// (portableRT include/portableRT/intersect_optix.hpp:34-50); here the C++ wrapper
// turns a status into std::runtime_error, the reference's exception type for an
// unusable backend (include/portableRT/nearest_hits_impl.hpp:31-32).
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"
#include "prt_camera.cuh"
#include "prt_ctx.cuh"
#include "prt_traverse.cuh"

namespace {

thread_local std::string g_create_error;

using prt::layout_ok;

int fail(prt_b200_ctx *ctx, int code, const std::string &msg) {
	if (ctx)
		ctx->err = msg;
	return code;
}

int cuda_fail(prt_b200_ctx *ctx, cudaError_t e, const char *what) {
	return fail(ctx, e == cudaErrorMemoryAllocation ? PRT_ERR_OOM : PRT_ERR_CUDA,
	            std::string(what) + ": " + cudaGetErrorString(e));
}

#define CAPI_TRY(ctx, call)                                                                    \
	do {                                                                                       \
		cudaError_t e_ = (call);                                                               \
		if (e_ != cudaSuccess)                                                                 \
			return cuda_fail((ctx), e_, #call);                                                \
	} while (0)

bool cc_ok(int dev) {
	int major = 0, minor = 0;
	if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess)
		return false;
	if (cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
		return false;
	return major == 10 && minor == 3;
}

int check_device_errors(prt_b200_ctx *ctx) {
	CAPI_TRY(ctx, cudaMemcpyAsync(ctx->h_err, ctx->d_err(), 4, cudaMemcpyDeviceToHost,
	                              ctx->stream));
	CAPI_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	uint32_t e = *ctx->h_err;
	if (e) {
		cudaMemsetAsync(ctx->d_err(), 0, 4, ctx->stream);
		cudaStreamSynchronize(ctx->stream);
		std::string m = "kernel reported:";
		if (e & prt::kErrStack)
			m += " traversal stack overflow;";
		if (e & prt::kErrLookback)
			m += " radix-sort look-back timed out;";
		if (e & prt::kErrCollapse)
			m += " collapse exceeded the node budget;";
		if (e & prt::kErrSah)
			m += " SAH build failed a range check;";
		return fail(ctx, PRT_ERR_DEVICE, m);
	}
	return PRT_OK;
}

// Every tuning option prt_b200_set_option accepts.  PRT_B200_<KEY> in the environment
// (the name in upper case, e.g. PRT_B200_LEAF_SIZE=4) sets option <key> of each new
// context, so programs that use the backend through portableRT's API can be tuned
// unchanged.  The test hooks "fail_alloc_after" and "fail_serve_after" are deliberately
// not among them: they inject failures, which no environment variable of a production
// program should be able to reach.
const char *const kOptionKeys[] = {"leaf_size",        "node_format",   "block",
                                   "pipe_chunks",      "pipe_ramp",     "pipe_min_rays",
                                   "serve_batches_per_warp", "pool_depth", "count_visits",
                                   "build_compressed", "build_sah",     "collapse_cost",
                                   "build_small",      "host_direct",   "serve_persistent"};

// The overrides set in the environment, as (key, value); false with a message when a
// value is not a decimal integer.
bool env_overrides(std::vector<std::pair<const char *, int64_t>> &out, std::string &err) {
	for (const char *key : kOptionKeys) {
		std::string name = "PRT_B200_";
		for (const char *c = key; *c; ++c)
			name += (char)std::toupper((unsigned char)*c);
		const char *text = std::getenv(name.c_str());
		if (!text)
			continue;
		char *end = nullptr;
		errno = 0;
		const long long v = std::strtoll(text, &end, 10);
		if (end == text || *end != '\0' || errno) {
			err = name + "=" + text + ": not a decimal integer";
			return false;
		}
		out.emplace_back(key, (int64_t)v);
	}
	return true;
}

// The record layout of a call, and the traversal settings of the context's options.
prt::OutLayout out_layout(uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8]) {
	prt::OutLayout lay;
	lay.mask = field_mask;
	lay.rec_size = rec_size;
	std::memcpy(lay.off, offs, 8);
	return lay;
}

prt::TravConfig trav_config(const prt_b200_ctx *ctx) {
	prt::TravConfig cfg;
	cfg.format = ctx->node_format;
	cfg.block = ctx->block;
	cfg.count = ctx->count;
	return cfg;
}

int do_build(prt_b200_ctx *ctx, const float *d_tris, uint64_t n) {
	// Queries still reading the old scene on callers' streams finish before the
	// rebuild overwrites its arrays.
	for (auto &q : ctx->query_streams)
		CAPI_TRY(ctx, cudaStreamWaitEvent(ctx->stream, q.ev, 0));
	prt::EventPair ev;
	CAPI_TRY(ctx, ev.create());
	cudaEventRecord(ev.a, ctx->stream);
	std::string msg;
	bool sah = ctx->build_sah;
	int rc = prt::build_scene(d_tris, n, ctx->leaf_size, ctx->build_compressed, ctx->scene,
	                          ctx->ws, ctx->stream, ctx->d_err(), msg, sah, ctx->collapse_cost,
	                          ctx->build_small);
	if (sah && rc == PRT_ERR_LIMIT) {
		// An SAH tree deeper than the collapse's 32 levels: the LBVH's depth is bounded.
		sah = false;
		msg.clear();
		rc = prt::build_scene(d_tris, n, ctx->leaf_size, ctx->build_compressed, ctx->scene,
		                      ctx->ws, ctx->stream, ctx->d_err(), msg, false, ctx->collapse_cost);
	}
	ctx->last_build_sah = sah;
	ctx->last_build_small = ctx->scene.built_small;
	cudaEventRecord(ev.b, ctx->stream);
	ctx->build_ms = ev.elapsed_ms();
	ctx->scene_set = false;
	if (rc != PRT_OK)
		return fail(ctx, rc, msg);
	rc = check_device_errors(ctx);
	if (rc != PRT_OK)
		return rc;
	if ((int)ctx->scene.depth > prt::traversal_stack_depth())
		return fail(ctx, PRT_ERR_LIMIT, "tree too deep for the traversal stack");
	ctx->scene_set = true;
	return PRT_OK;
}

} // namespace

namespace prt {

// The message prt_b200_last_error(NULL) returns on this thread.
void set_global_error(const std::string &msg) { g_create_error = msg; }

// The bookkeeping of a caller's stream (created at its first query).
int query_stream(prt_b200_ctx *ctx, cudaStream_t st, prt_b200_ctx::QueryStream **out) {
	for (auto &q : ctx->query_streams)
		if (q.st == st) {
			*out = &q;
			return PRT_OK;
		}
	// Room first: a failed host allocation then leaves no event or counter behind.
	ctx->query_streams.reserve(ctx->query_streams.size() + 1);
	prt_b200_ctx::QueryStream q{st, nullptr, nullptr};
	CAPI_TRY(ctx, cudaEventCreateWithFlags(&q.ev, cudaEventDisableTiming));
	cudaError_t e = cudaMalloc(&q.counter, 64);
	if (e != cudaSuccess) {
		cudaEventDestroy(q.ev);
		return cuda_fail(ctx, e, "nearest_hits_dev: stream counter");
	}
	ctx->query_streams.push_back(q);
	*out = &ctx->query_streams.back();
	return PRT_OK;
}

} // namespace prt

extern "C" {

int prt_b200_available(void) {
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	for (int d = 0; d < n; ++d)
		if (cc_ok(d))
			return 1;
	return 0;
}

int prt_b200_create(int device, prt_b200_ctx **out) {
	if (!out) {
		g_create_error = "out pointer is null";
		return PRT_ERR_ARG;
	}
	*out = nullptr;
	// Environment overrides are read first, so a malformed one is reported on any machine.
	std::vector<std::pair<const char *, int64_t>> env;
	std::string env_err;
	if (!env_overrides(env, env_err)) {
		g_create_error = env_err;
		return PRT_ERR_ARG;
	}
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n || !cc_ok(device)) {
		cudaGetLastError();
		g_create_error = "no compute capability 10.3 device at this index";
		return PRT_ERR_NO_DEVICE;
	}
	prt_b200_ctx *ctx = new (std::nothrow) prt_b200_ctx();
	if (!ctx) {
		g_create_error = "out of host memory";
		return PRT_ERR_OOM;
	}
	ctx->device = device;
	cudaError_t e = cudaSetDevice(device);
	if (e == cudaSuccess)
		e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess)
		e = ctx->work.reserve(64);
	if (e == cudaSuccess)
		e = cudaMemset(ctx->work.p, 0, 64);
	if (e == cudaSuccess)
		e = cudaMallocHost(&ctx->h_err, 16);
	if (e == cudaSuccess)
		e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
	if (e == cudaSuccess)
		e = cudaDeviceGetAttribute(&ctx->pageable_access, cudaDevAttrPageableMemoryAccess,
		                           device);
	for (cudaStream_t *s : {&ctx->s_in, &ctx->s_out, &ctx->s_k2})
		if (e == cudaSuccess)
			e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
	for (int i = 0; i < prt_b200_ctx::kPipe && e == cudaSuccess; ++i) {
		e = cudaEventCreateWithFlags(&ctx->ev_in[i], cudaEventDisableTiming);
		if (e == cudaSuccess)
			e = cudaEventCreateWithFlags(&ctx->ev_k[i], cudaEventDisableTiming);
	}
	if (e != cudaSuccess) {
		g_create_error = std::string("create: ") + cudaGetErrorString(e);
		prt_b200_destroy(ctx);
		return e == cudaErrorMemoryAllocation ? PRT_ERR_OOM : PRT_ERR_CUDA;
	}
	for (const auto &kv : env) {
		const int rc = prt_b200_set_option(ctx, kv.first, kv.second);
		if (rc != PRT_OK) {
			g_create_error = "environment override: " + ctx->err.get();
			prt_b200_destroy(ctx);
			return rc;
		}
	}
	*out = ctx;
	return PRT_OK;
}

void prt_b200_destroy(prt_b200_ctx *ctx) {
	if (!ctx)
		return;
	cudaSetDevice(ctx->device);
	for (cudaStream_t s : {ctx->stream, ctx->s_in, ctx->s_out, ctx->s_k2})
		if (s)
			cudaStreamSynchronize(s);
	for (auto &q : ctx->query_streams)
		cudaEventSynchronize(q.ev);
	ctx->scene.release();
	ctx->ws.release();
	ctx->tris_in.release();
	ctx->rays_buf.release();
	ctx->out_buf.release();
	ctx->work.release();
	if (ctx->h_err)
		cudaFreeHost(ctx->h_err);
	for (auto &q : ctx->query_streams) {
		cudaEventDestroy(q.ev);
		cudaFree(q.counter);
	}
	for (int i = 0; i < prt_b200_ctx::kPipe; ++i) {
		if (ctx->ev_in[i])
			cudaEventDestroy(ctx->ev_in[i]);
		if (ctx->ev_k[i])
			cudaEventDestroy(ctx->ev_k[i]);
	}
	for (cudaStream_t s : {ctx->s_in, ctx->s_out, ctx->s_k2, ctx->stream})
		if (s) {
			cudaStreamSynchronize(s);
			cudaStreamDestroy(s);
		}
	delete ctx;
}

// The calling thread's copy of the message, valid until its next call here.
const char *prt_b200_last_error(const prt_b200_ctx *ctx) {
	thread_local std::string copy;
	copy = ctx ? ctx->err.get() : g_create_error;
	return copy.c_str();
}

int prt_b200_device_name(prt_b200_ctx *ctx, char *buf, size_t len) {
	if (!ctx || !buf || len == 0)
		return fail(ctx, PRT_ERR_ARG, "device_name: bad argument");
	cudaDeviceProp p;
	CAPI_TRY(ctx, cudaGetDeviceProperties(&p, ctx->device));
	std::snprintf(buf, len, "%s", p.name);
	return PRT_OK;
}

int prt_b200_set_tris(prt_b200_ctx *ctx, const float *tris9, uint64_t n) {
	if (!ctx)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "set_tris", [&]() -> int {
		if (!tris9 && n)
			return fail(ctx, PRT_ERR_ARG, "set_tris: null triangle pointer");
		if (n > prt::kMaxTris)
			return fail(ctx, PRT_ERR_LIMIT, "set_tris: at most 134217727 triangles per scene");
		std::lock_guard<std::mutex> lk(ctx->mu);
		CAPI_TRY(ctx, cudaSetDevice(ctx->device));
		if (n) {
			CAPI_TRY(ctx, ctx->tris_in.reserve(36ull * n));
			CAPI_TRY(ctx, cudaMemcpyAsync(ctx->tris_in.p, tris9, 36ull * n, cudaMemcpyHostToDevice,
			                              ctx->stream));
		}
		return do_build(ctx, ctx->tris_in.as<float>(), n);
	});
}

int prt_b200_set_tris_dev(prt_b200_ctx *ctx, const float *d_tris9, uint64_t n) {
	if (!ctx)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "set_tris_dev", [&]() -> int {
		if (!d_tris9 && n)
			return fail(ctx, PRT_ERR_ARG, "set_tris_dev: null triangle pointer");
		if (n > prt::kMaxTris)
			return fail(ctx, PRT_ERR_LIMIT, "set_tris: at most 134217727 triangles per scene");
		std::lock_guard<std::mutex> lk(ctx->mu);
		CAPI_TRY(ctx, cudaSetDevice(ctx->device));
		return do_build(ctx, d_tris9, n);
	});
}

} // extern "C"

namespace {

// One query of the context's scene on `stream` (NULL = the context's stream): rays from
// d_rays6 or, when cam is not null, from the camera.  Caller holds the context's lock.
int queue_query(prt_b200_ctx *ctx, const float *d_rays6, uint64_t n, uint32_t field_mask,
                uint32_t rec_size, const uint8_t offs[8], void *d_out, void *stream,
                const prt_b200_camera *cam) {
	if (!ctx->scene_set)
		return fail(ctx, PRT_ERR_NO_SCENE, "nearest_hits: set_tris has not succeeded");
	if (ctx->node_format == PRT_NODES_COMPRESSED && !ctx->scene.has_cnodes && ctx->scene.n_tris)
		return fail(ctx, PRT_ERR_ARG, "nearest_hits: compressed nodes were not built");
	CAPI_TRY(ctx, cudaSetDevice(ctx->device));
	if (n == 0)
		return PRT_OK;
	const prt::OutLayout lay = out_layout(field_mask, rec_size, offs);
	const prt::TravConfig cfg = trav_config(ctx);
	cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
	prt_b200_ctx::QueryStream *qs = nullptr;
	if (st != ctx->stream) {
		int rc = prt::query_stream(ctx, st, &qs);
		if (rc != PRT_OK)
			return rc;
	}
	CAPI_TRY(ctx, prt::launch_nearest_hits(ctx->scene, d_rays6, n, lay, d_out, cfg,
	                                       qs ? qs->counter : ctx->d_work(), ctx->d_visits(),
	                                       ctx->d_err(), st, ctx->sms, cam));
	if (qs)
		CAPI_TRY(ctx, cudaEventRecord(qs->ev, st));
	return PRT_OK;
}

} // namespace

extern "C" {

int prt_b200_nearest_hits_dev(prt_b200_ctx *ctx, const float *d_rays6, uint64_t n,
                              uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                              void *d_out, void *stream) {
	if (!ctx)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "nearest_hits_dev", [&]() -> int {
		std::string why;
		if (!layout_ok(field_mask, rec_size, offs, why))
			return fail(ctx, PRT_ERR_ARG, "nearest_hits: " + why);
		if (n && (!d_rays6 || !d_out))
			return fail(ctx, PRT_ERR_ARG, "nearest_hits: null buffer");
		if (reinterpret_cast<uintptr_t>(d_rays6) % 8 != 0)
			return fail(ctx, PRT_ERR_ARG, "nearest_hits: rays must be 8-byte aligned");
		std::lock_guard<std::mutex> lk(ctx->mu);
		return queue_query(ctx, d_rays6, n, field_mask, rec_size, offs, d_out, stream, nullptr);
	});
}

int prt_b200_nearest_hits_camera(prt_b200_ctx *ctx, const prt_b200_camera *camera,
                                 uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                                 void *d_out, void *stream) {
	if (!ctx)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "nearest_hits_camera", [&]() -> int {
		std::string why;
		if (!prt::camera_ok(camera, why) || !layout_ok(field_mask, rec_size, offs, why))
			return fail(ctx, PRT_ERR_ARG, "nearest_hits_camera: " + why);
		if (!d_out)
			return fail(ctx, PRT_ERR_ARG, "nearest_hits_camera: null output");
		std::lock_guard<std::mutex> lk(ctx->mu);
		const prt_b200_camera cam = *camera;
		return queue_query(ctx, nullptr, (uint64_t)cam.width * cam.height, field_mask, rec_size,
		                   offs, d_out, stream, &cam);
	});
}

int prt_b200_sync(prt_b200_ctx *ctx) {
	if (!ctx)
		return PRT_ERR_ARG;
	std::lock_guard<std::mutex> lk(ctx->mu);
	CAPI_TRY(ctx, cudaSetDevice(ctx->device));
	CAPI_TRY(ctx, cudaDeviceSynchronize());
	if (ctx->count) {
		CAPI_TRY(ctx, cudaMemcpy(ctx->visits, ctx->d_visits(), 16, cudaMemcpyDeviceToHost));
	}
	return check_device_errors(ctx);
}

int prt_b200_nearest_hits(prt_b200_ctx *ctx, const float *rays6, uint64_t n, uint32_t field_mask,
                          uint32_t rec_size, const uint8_t offs[8], void *out_host) {
	if (!ctx)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "nearest_hits", [&]() -> int {
		std::string why;
		if (!layout_ok(field_mask, rec_size, offs, why))
			return fail(ctx, PRT_ERR_ARG, "nearest_hits: " + why);
		if (n && (!rays6 || !out_host))
			return fail(ctx, PRT_ERR_ARG, "nearest_hits: null buffer");
		std::lock_guard<std::mutex> lk(ctx->mu);
		if (!ctx->scene_set)
			return fail(ctx, PRT_ERR_NO_SCENE, "nearest_hits: set_tris has not succeeded");
		if (ctx->node_format == PRT_NODES_COMPRESSED && !ctx->scene.has_cnodes && ctx->scene.n_tris)
			return fail(ctx, PRT_ERR_ARG, "nearest_hits: compressed nodes were not built");
		if (n == 0)
			return PRT_OK;
		CAPI_TRY(ctx, cudaSetDevice(ctx->device));
		const prt::OutLayout lay = out_layout(field_mask, rec_size, offs);
		const prt::TravConfig cfg = trav_config(ctx);
		// In place when the device can reach both buffers: the traversal reads each ray from
		// host memory once and writes each record there once, over the host link, with no
		// staging buffers and nothing to overlap.  The traversal reads rays as 8-byte pairs,
		// so rays that are only 4-byte aligned (a float array at an odd index) are copied
		// into the aligned staging buffer instead; records may have any alignment.
		if (ctx->host_direct) {
			const void *d_in = prt::device_alias(ctx, rays6);
			if (reinterpret_cast<uintptr_t>(d_in) % 8 != 0)
				d_in = nullptr;
			void *d_out = d_in ? prt::device_alias(ctx, out_host) : nullptr;
			ctx->last_in_place = d_in && d_out;
			if (d_in && d_out) {
				CAPI_TRY(ctx, prt::launch_nearest_hits(ctx->scene, static_cast<const float *>(d_in),
				                                       n, lay, d_out, cfg, ctx->d_work(),
				                                       ctx->d_visits(), ctx->d_err(), ctx->stream,
				                                       ctx->sms));
				if (ctx->count)
					CAPI_TRY(ctx, cudaMemcpyAsync(ctx->visits, ctx->d_visits(), 16,
					                              cudaMemcpyDeviceToHost, ctx->stream));
				// One wait: the error word's copy is queued after the traversal.
				return check_device_errors(ctx);
			}
		}
		ctx->last_in_place = false;
		CAPI_TRY(ctx, ctx->rays_buf.reserve(24ull * n));
		CAPI_TRY(ctx, ctx->out_buf.reserve((uint64_t)rec_size * n));
		// Chunks: pipe_chunks of them (fewer when a chunk would hold under pipe_min_rays), one
		// when the visit counters are on (each launch would reset them).  With pipe_ramp the
		// sizes ramp up and down (weights 1, 2, 4, 8, ..., 8, 4, 2, 1), so the copy-in of the
		// first chunk and the copy-out of the last, which nothing overlaps, are short.  Chunk
		// c is copied in on s_in, traversed on stream c % 2 (so a chunk's last blocks overlap
		// the next chunk's first) and copied out on s_out.  Every chunk has its own rays,
		// records and events; the two compute streams have their own ray counters.
		int nc = ctx->count ? 1 : ctx->pipe_chunks;
		if (nc > 1 && n / (uint64_t)nc < ctx->pipe_min_rays)
			nc = (int)std::max<uint64_t>(1, n / ctx->pipe_min_rays);
		uint64_t bnd[prt_b200_ctx::kPipe + 1];
		{
			uint32_t w[prt_b200_ctx::kPipe], total = 0;
			for (int i = 0; i < nc; ++i) {
				w[i] = ctx->pipe_ramp ? 1u << std::min(std::min(i, nc - 1 - i), 3) : 1u;
				total += w[i];
			}
			bnd[0] = 0;
			uint64_t cum = 0;
			for (int i = 0; i < nc; ++i) {
				cum += w[i];
				bnd[i + 1] = (i + 1 == nc) ? n : ((unsigned __int128)n * cum / total) & ~31ull;
			}
		}
		cudaStream_t ks[2] = {ctx->stream, ctx->s_k2};
		uint32_t *ctr[2] = {ctx->d_work(), ctx->d_work() + 8};
		// Earlier work of the context's stream (a _dev call) finishes before the chunks start.
		CAPI_TRY(ctx, cudaEventRecord(ctx->ev_k[0], ctx->stream));
		for (cudaStream_t st : {ctx->s_in, ctx->s_out, ctx->s_k2})
			CAPI_TRY(ctx, cudaStreamWaitEvent(st, ctx->ev_k[0], 0));
		const uint8_t *rin = reinterpret_cast<const uint8_t *>(rays6);
		uint8_t *rout = static_cast<uint8_t *>(out_host);
		for (int c = 0; c <= nc; ++c) {
			if (c < nc) {
				const uint64_t b = bnd[c], m = bnd[c + 1] - bnd[c];
				CAPI_TRY(ctx, cudaMemcpyAsync(ctx->rays_buf.as<uint8_t>() + 24 * b, rin + 24 * b,
				                              24 * m, cudaMemcpyHostToDevice, ctx->s_in));
				CAPI_TRY(ctx, cudaEventRecord(ctx->ev_in[c], ctx->s_in));
				cudaStream_t st = ks[c & 1];
				CAPI_TRY(ctx, cudaStreamWaitEvent(st, ctx->ev_in[c], 0));
				CAPI_TRY(ctx, prt::launch_nearest_hits(
				                  ctx->scene, ctx->rays_buf.as<float>() + 6 * b, m, lay,
				                  ctx->out_buf.as<uint8_t>() + (uint64_t)rec_size * b, cfg, ctr[c & 1],
				                  ctx->d_visits(), ctx->d_err(), st, ctx->sms));
				CAPI_TRY(ctx, cudaEventRecord(ctx->ev_k[c], st));
			}
			// The copy-out of the chunk before is queued after this chunk's copy-in, so that
			// with pageable host memory (where the copy calls return only when done) the
			// copy-in still overlaps the traversal.
			if (c > 0) {
				const uint64_t b = bnd[c - 1], m = bnd[c] - bnd[c - 1];
				CAPI_TRY(ctx, cudaStreamWaitEvent(ctx->s_out, ctx->ev_k[c - 1], 0));
				CAPI_TRY(ctx, cudaMemcpyAsync(rout + (uint64_t)rec_size * b,
				                              ctx->out_buf.as<uint8_t>() + (uint64_t)rec_size * b,
				                              (uint64_t)rec_size * m, cudaMemcpyDeviceToHost,
				                              ctx->s_out));
			}
		}
		// s_out waited for every chunk's traversal; the context's stream waits for s_out.
		CAPI_TRY(ctx, cudaEventRecord(ctx->ev_in[0], ctx->s_out));
		CAPI_TRY(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_in[0], 0));
		CAPI_TRY(ctx, cudaStreamSynchronize(ctx->s_out));
		if (ctx->count)
			CAPI_TRY(ctx, cudaMemcpy(ctx->visits, ctx->d_visits(), 16, cudaMemcpyDeviceToHost));
		return check_device_errors(ctx);
	});
}

int prt_b200_set_option(prt_b200_ctx *ctx, const char *key, int64_t v) {
	if (!ctx || !key)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "set_option", [&]() -> int {
		std::lock_guard<std::mutex> lk(ctx->mu);
		std::string k(key);
		if (k == "leaf_size") {
			if (v < 1 || v > prt::kMaxLeaf)
				return fail(ctx, PRT_ERR_ARG, "leaf_size must be in [1, 8]");
			ctx->leaf_size = (int)v;
		} else if (k == "node_format") {
			if (v != PRT_NODES_FP32 && v != PRT_NODES_COMPRESSED)
				return fail(ctx, PRT_ERR_ARG, "node_format must be 0 or 1");
			ctx->node_format = (int)v;
		} else if (k == "block") {
			if (v < 32 || v > 128 || v % 32)
				return fail(ctx, PRT_ERR_ARG, "block must be 32, 64, 96 or 128");
			ctx->block = (int)v;
		} else if (k == "pipe_chunks") {
			if (v < 1 || v > prt_b200_ctx::kPipe)
				return fail(ctx, PRT_ERR_ARG, "pipe_chunks must be in [1, 16]");
			ctx->pipe_chunks = (int)v;
		} else if (k == "pipe_ramp") {
			ctx->pipe_ramp = v != 0;
		} else if (k == "pipe_min_rays") {
			if (v < 32 || v > (1ll << 30) || v % 32)
				return fail(ctx, PRT_ERR_ARG, "pipe_min_rays must be a multiple of 32 in [32, 2^30]");
			ctx->pipe_min_rays = (uint32_t)v;
		} else if (k == "serve_batches_per_warp") {
			if (v < 0 || v > (1 << 20))
				return fail(ctx, PRT_ERR_ARG, "serve_batches_per_warp must be in [0, 2^20]");
			ctx->serve_batches_per_warp = (int)v;
		} else if (k == "pool_depth") {
			if (v < 0 || v > prt::traversal_stack_depth())
				return fail(ctx, PRT_ERR_ARG, "pool_depth must be in [0, 32]");
			ctx->pool_depth = (int)v;
		} else if (k == "count_visits") {
			ctx->count = v != 0;
		} else if (k == "build_compressed") {
			ctx->build_compressed = v != 0;
		} else if (k == "build_sah") {
			ctx->build_sah = v != 0;
		} else if (k == "collapse_cost") {
			ctx->collapse_cost = v != 0;
		} else if (k == "build_small") {
			ctx->build_small = v != 0;
		} else if (k == "host_direct") {
			ctx->host_direct = v != 0;
		} else if (k == "serve_persistent") {
			ctx->serve_persistent = v != 0;
		} else if (k == "fail_serve_after") {
			if (v < 0)
				return fail(ctx, PRT_ERR_ARG, "fail_serve_after must be >= 0");
			ctx->fail_serve_after = v;
		} else if (k == "fail_alloc_after") {
			if (v < 0)
				return fail(ctx, PRT_ERR_ARG, "fail_alloc_after must be >= 0");
			prt::arm_alloc_failure(v);
		} else {
			return fail(ctx, PRT_ERR_ARG, "unknown option " + k);
		}
		return PRT_OK;
	});
}

int prt_b200_get_stat(prt_b200_ctx *ctx, const char *key, double *value) {
	if (!ctx || !key || !value)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "get_stat", [&]() -> int {
		std::lock_guard<std::mutex> lk(ctx->mu);
		std::string k(key);
		const prt::SceneGPU &s = ctx->scene;
		if (k == "n_tris")
			*value = (double)s.n_tris;
		else if (k == "n_nodes")
			*value = s.n_nodes;
		else if (k == "depth")
			*value = s.depth;
		else if (k == "build_ms")
			*value = ctx->build_ms;
		else if (k == "build_sah")
			*value = ctx->last_build_sah ? 1.0 : 0.0;
		else if (k == "build_small")
			*value = ctx->last_build_small ? 1.0 : 0.0;
		else if (k == "in_place")
			*value = ctx->last_in_place ? 1.0 : 0.0;
		else if (k == "node_bytes")
			*value = (double)s.n_nodes *
			         (ctx->node_format == PRT_NODES_COMPRESSED ? sizeof(prt::CNode8) : sizeof(prt::Node8));
		else if (k == "node_size")
			*value = (double)(ctx->node_format == PRT_NODES_COMPRESSED ? sizeof(prt::CNode8)
			                                                            : sizeof(prt::Node8));
		else if (k == "tri_bytes")
			*value = 48.0 * (double)s.n_tris;
		else if (k == "visits_nodes")
			*value = (double)ctx->visits[0];
		else if (k == "visits_tris")
			*value = (double)ctx->visits[1];
		else if (k == "sms")
			*value = ctx->sms;
		else if (k == "leaf_size")
			*value = s.leaf_size;
		else
			return fail(ctx, PRT_ERR_ARG, "unknown statistic " + k);
		return PRT_OK;
	});
}

} // extern "C"

// ---------------------------------------------------------------------------------------
// Nearest hits without any device allocation.
//
// Who needs it: programs that must not allocate device memory once they are running,
// e.g. a renderer that reserves its whole memory budget at start-up and forbids
// allocation inside its frame loop, because cudaMalloc can synchronise the device and
// can fail when the budget is fixed.  prt_b200_nearest_hits grows its device buffers on
// demand; this variant instead stages rays and records, and keeps the traversal's ray
// counter and error word, in one file-scope device array of fixed size, so a call never
// allocates.  The context and the scene are still created and built beforehand (at
// start-up, where allocation is allowed).
//
// The array is kNoallocBytes (3.5 MiB) on every device that loads the library, held
// until the process exits, and limits one call to kNoallocMaxRays rays.  Every call
// shares it and it keeps the last call's contents: each call clears the counter, the
// error word and the visit counters it uses.  Calls whose GPU work overlaps would race
// on the array; calls are synchronous and serialised by a process-wide mutex, so this
// only matters if the array is reached some other way.
// ---------------------------------------------------------------------------------------
namespace {

constexpr uint64_t kNoallocMaxRays = 65536;
constexpr size_t kNoallocWork = 256;                      // counter, error word, visits
constexpr size_t kNoallocRayBytes = 24 * kNoallocMaxRays; // 6 floats per ray
constexpr size_t kNoallocRecBytes = 32 * kNoallocMaxRays; // largest HitReg<Tags...>
constexpr size_t kNoallocBytes = kNoallocWork + kNoallocRayBytes + kNoallocRecBytes;
constexpr int kNoallocMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kNoallocMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (which must be current).  In host code
// the array's name is only a host-side stand-in, so its device address is looked up
// once per device with cudaGetSymbolAddress.  Caller holds g_noalloc_mu.
int noalloc_scratch(prt_b200_ctx *ctx, int device, unsigned char **out) {
	if (device < 0 || device >= kNoallocMaxDevices)
		return fail(ctx, PRT_ERR_ARG, "nearest_hits_noalloc: device index out of range");
	if (!g_noalloc_ptr[device]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess || !p)
			return cuda_fail(ctx, e, "nearest_hits_noalloc: cudaGetSymbolAddress");
		g_noalloc_ptr[device] = p;
	}
	*out = static_cast<unsigned char *>(g_noalloc_ptr[device]);
	return PRT_OK;
}

} // namespace

extern "C" int prt_b200_nearest_hits_noalloc(prt_b200_ctx *ctx, const float *rays6, uint64_t n,
                                             uint32_t field_mask, uint32_t rec_size,
                                             const uint8_t offs[8], void *out_host) {
	if (!ctx)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "nearest_hits_noalloc", [&]() -> int {
		std::string why;
		if (!layout_ok(field_mask, rec_size, offs, why))
			return fail(ctx, PRT_ERR_ARG, "nearest_hits_noalloc: " + why);
		if (n > kNoallocMaxRays)
			return fail(ctx, PRT_ERR_LIMIT,
			            "nearest_hits_noalloc: at most 65536 rays per call (" + std::to_string(n) +
			                " given); split the batch or use prt_b200_nearest_hits");
		if (n && (!rays6 || !out_host))
			return fail(ctx, PRT_ERR_ARG, "nearest_hits_noalloc: null buffer");
		std::lock_guard<std::mutex> glk(g_noalloc_mu);
		std::lock_guard<std::mutex> lk(ctx->mu);
		if (!ctx->scene_set)
			return fail(ctx, PRT_ERR_NO_SCENE, "nearest_hits_noalloc: set_tris has not succeeded");
		if (ctx->node_format == PRT_NODES_COMPRESSED && !ctx->scene.has_cnodes && ctx->scene.n_tris)
			return fail(ctx, PRT_ERR_ARG, "nearest_hits_noalloc: compressed nodes were not built");
		if (n == 0)
			return PRT_OK;
		CAPI_TRY(ctx, cudaSetDevice(ctx->device));
		unsigned char *scratch = nullptr;
		int rc = noalloc_scratch(ctx, ctx->device, &scratch);
		if (rc != PRT_OK)
			return rc;
		uint32_t *d_work = reinterpret_cast<uint32_t *>(scratch);
		uint32_t *d_err = d_work + 1;
		unsigned long long *d_visits = reinterpret_cast<unsigned long long *>(scratch + 16);
		float *d_rays = reinterpret_cast<float *>(scratch + kNoallocWork);
		void *d_out = scratch + kNoallocWork + kNoallocRayBytes;
		cudaStream_t st = ctx->stream;
		CAPI_TRY(ctx, cudaMemsetAsync(scratch, 0, kNoallocWork, st));
		CAPI_TRY(ctx, cudaMemcpyAsync(d_rays, rays6, 24ull * n, cudaMemcpyHostToDevice, st));
		const prt::OutLayout lay = out_layout(field_mask, rec_size, offs);
		const prt::TravConfig cfg = trav_config(ctx);
		CAPI_TRY(ctx, prt::launch_nearest_hits(ctx->scene, d_rays, n, lay, d_out, cfg, d_work,
		                                       d_visits, d_err, st, ctx->sms));
		CAPI_TRY(ctx, cudaMemcpyAsync(out_host, d_out, (uint64_t)rec_size * n, cudaMemcpyDeviceToHost,
		                              st));
		uint32_t err_word = 0;
		CAPI_TRY(ctx, cudaMemcpyAsync(&err_word, d_err, 4, cudaMemcpyDeviceToHost, st));
		CAPI_TRY(ctx, cudaStreamSynchronize(st));
		if (ctx->count)
			CAPI_TRY(ctx, cudaMemcpy(ctx->visits, d_visits, 16, cudaMemcpyDeviceToHost));
		if (err_word)
			return fail(ctx, PRT_ERR_DEVICE, "nearest_hits_noalloc: kernel reported an error");
		// Errors that earlier asynchronous calls on this context (the _dev calls) left in the
		// context's own error word are reported here too, as prt_b200_nearest_hits reports
		// them; reading it copies 4 bytes into the context's pinned word, no allocation.
		return check_device_errors(ctx);
	});
}
