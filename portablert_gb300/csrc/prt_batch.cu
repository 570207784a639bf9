// prt_batch.cu - many scenes built together and queried by one persistent launch.
//
// A batch holds S scenes in one arena (built by the same kernels as one scene: binned
// SAH, prt_sah.cu, by default; the LBVH of prt_build.cu inside a captured graph) and
// answers a list of queries (scene, rays, output, record layout) with one launch of the
// traversal kernel over all their rays (prt_traverse.cu, segment tables).  The build
// and the query can be captured together in a CUDA graph and replayed.
//
// No counterpart in the reference: portableRT holds one scene per backend
// (Backend::set_tris, backend.hpp:19); a batch is what the batching and serving
// workloads need, and each of its answers is the one nearest_hits<Tags...> gives for
// that scene alone (tested).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/prt_b200.h"
#include "prt_batch.cuh"
#include "prt_build.cuh"
#include "prt_ctx.cuh"
#include "prt_traverse.cuh"

namespace {

using prt::kSlots;
using Slot = prt::BatchSlot;

int bfail(prt_b200_ctx *ctx, int code, const std::string &msg) {
	ctx->err = msg;
	return code;
}

int bcuda(prt_b200_ctx *ctx, cudaError_t e, const char *what) {
	return bfail(ctx, e == cudaErrorMemoryAllocation ? PRT_ERR_OOM : PRT_ERR_CUDA,
	             std::string(what) + ": " + cudaGetErrorString(e));
}

#define B_TRY(ctx, call)                                                                       \
	do {                                                                                       \
		cudaError_t e_ = (call);                                                               \
		if (e_ != cudaSuccess)                                                                 \
			return bcuda((ctx), e_, #call);                                                    \
	} while (0)

} // namespace

namespace {

int check_slot(prt_b200_batch *b, Slot &s) {
	prt_b200_ctx *ctx = b->ctx;
	if (!s.pending)
		return PRT_OK;
	B_TRY(ctx, cudaEventSynchronize(s.done));
	s.pending = false;
	B_TRY(ctx, cudaMemcpy(b->h_words, s.work.p, 32, cudaMemcpyDeviceToHost));
	if (ctx->count) {
		b->visits[0] = reinterpret_cast<unsigned long long *>(b->h_words)[2];
		b->visits[1] = reinterpret_cast<unsigned long long *>(b->h_words)[3];
	}
	if (b->h_words[1]) {
		cudaMemset(s.work.p, 0, 32);
		return bfail(ctx, PRT_ERR_DEVICE, "batch query: kernel reported an error");
	}
	return PRT_OK;
}

int scene_tables(prt_b200_batch *b) {
	prt_b200_ctx *ctx = b->ctx;
	const prt::SceneGPU &a = b->arena;
	const uint32_t S = a.n_scenes;
	std::vector<prt::SceneDesc> f(S), c(S);
	for (uint32_t s = 0; s < S; ++s) {
		prt::SceneDesc d;
		d.tri4 = a.tri4.as<float4>();
		d.inv = a.inv.as<uint32_t>() + a.h_tri_off[s];
		d.nodes = a.nodes.p;
		d.root = s;
		d.n_tris = (uint32_t)(a.h_tri_off[s + 1] - a.h_tri_off[s]);
		f[s] = d;
		d.nodes = a.cnodes.p;
		c[s] = d;
	}
	B_TRY(ctx, b->scenes_fp32.reserve(sizeof(prt::SceneDesc) * S));
	B_TRY(ctx, b->scenes_comp.reserve(sizeof(prt::SceneDesc) * S));
	B_TRY(ctx, cudaMemcpy(b->scenes_fp32.p, f.data(), sizeof(prt::SceneDesc) * S,
	                      cudaMemcpyHostToDevice));
	B_TRY(ctx, cudaMemcpy(b->scenes_comp.p, c.data(), sizeof(prt::SceneDesc) * S,
	                      cudaMemcpyHostToDevice));
	return PRT_OK;
}

// SegDesc table for a query list; n_virtual = padded ray count.
int segments(prt_b200_batch *b, const prt_b200_query *q, uint32_t nq,
             std::vector<prt::SegDesc> &segs, unsigned long long &n_virtual) {
	prt_b200_ctx *ctx = b->ctx;
	segs.clear();
	n_virtual = 0;
	for (uint32_t i = 0; i < nq; ++i) {
		std::string why;
		if (q[i].scene >= b->arena.n_scenes)
			return bfail(ctx, PRT_ERR_ARG, "batch query " + std::to_string(i) + ": no such scene");
		if (!prt::layout_ok(q[i].field_mask, q[i].rec_size, q[i].offs, why))
			return bfail(ctx, PRT_ERR_ARG, "batch query " + std::to_string(i) + ": " + why);
		if (q[i].n_rays == 0)
			continue;
		if (!q[i].rays || !q[i].out)
			return bfail(ctx, PRT_ERR_ARG, "batch query " + std::to_string(i) + ": null buffer");
		if (reinterpret_cast<uintptr_t>(q[i].rays) % 8 != 0)
			return bfail(ctx, PRT_ERR_ARG, "batch query: rays must be 8-byte aligned");
		prt::SegDesc d;
		d.vbegin = n_virtual;
		d.rays = q[i].rays;
		d.out = static_cast<uint8_t *>(q[i].out);
		d.n_rays = (uint32_t)q[i].n_rays;
		d.scene = q[i].scene;
		d.mask = q[i].field_mask;
		d.rec_size = q[i].rec_size;
		std::memcpy(d.off, q[i].offs, 8);
		d.store_mode = prt::store_mode_for(d.out);
		d.pad = 0;
		if (q[i].n_rays > (1ull << 31))
			return bfail(ctx, PRT_ERR_LIMIT, "batch query: at most 2^31 rays per query");
		segs.push_back(d);
		n_virtual += (q[i].n_rays + 31ull) & ~31ull;
		if (n_virtual > (1ull << 31))
			return bfail(ctx, PRT_ERR_LIMIT, "batch query: at most 2^31 rays per launch");
	}
	return PRT_OK;
}

int launch_query(prt_b200_batch *b, Slot &s, const std::vector<prt::SegDesc> &segs,
                 unsigned long long n_virtual, int pool_depth, uint32_t n_nodes,
                 cudaStream_t st) {
	prt_b200_ctx *ctx = b->ctx;
	prt::TravConfig cfg;
	cfg.format = ctx->node_format;
	cfg.block = ctx->block;
	cfg.count = ctx->count;
	cfg.pool_depth = pool_depth;
	const prt::SceneDesc *tab = ctx->node_format == PRT_NODES_COMPRESSED
	                                ? b->scenes_comp.as<prt::SceneDesc>()
	                                : b->scenes_fp32.as<prt::SceneDesc>();
	uint32_t *w = s.work.as<uint32_t>();
	B_TRY(ctx, prt::launch_nearest_hits_segments(
	               tab, s.segs.as<prt::SegDesc>(), (uint32_t)segs.size(), n_virtual,
	               b->arena.depth, b->arena.leaf_size, n_nodes, b->arena.dead, cfg, w,
	               reinterpret_cast<unsigned long long *>(w + 4), w + 1, st, ctx->sms));
	return PRT_OK;
}

// Everything a captured graph bakes in (pointers, scene offsets, queries, options),
// compared in full so that a replay never runs a graph made for other buffers.
std::string graph_key(const float *d_tris, const uint64_t *tri_off, uint32_t S,
                      const prt_b200_query *q, uint32_t nq, const prt_b200_ctx *ctx) {
	std::string k(reinterpret_cast<const char *>(&d_tris), sizeof d_tris);
	k.append(reinterpret_cast<const char *>(tri_off), sizeof(uint64_t) * (S + 1));
	k.append(reinterpret_cast<const char *>(q), sizeof(prt_b200_query) * nq);
	const int opts[7] = {ctx->leaf_size,      ctx->node_format,       ctx->block,
	                     (int)ctx->count,     ctx->pool_depth,        (int)ctx->build_compressed,
	                     (int)ctx->collapse_cost};
	k.append(reinterpret_cast<const char *>(opts), sizeof opts);
	return k;
}

void drop_graph(prt_b200_batch *b) {
	if (b->gexec)
		cudaGraphExecDestroy(b->gexec);
	if (b->graph)
		cudaGraphDestroy(b->graph);
	b->gexec = nullptr;
	b->graph = nullptr;
	b->graph_key.clear();
}

// Frees every device and host resource of a batch (its work is finished; the caller
// holds the context's lock).
void release_batch(prt_b200_batch *b) {
	drop_graph(b);
	for (Slot *s : {&b->gslot}) {
		s->segs.release();
		s->work.release();
		if (s->done)
			cudaEventDestroy(s->done);
		s->done = nullptr;
	}
	for (int i = 0; i < kSlots; ++i) {
		b->slots[i].segs.release();
		b->slots[i].work.release();
		if (b->slots[i].done)
			cudaEventDestroy(b->slots[i].done);
		b->slots[i].done = nullptr;
	}
	b->arena.release();
	b->ws.release();
	b->scenes_fp32.release();
	b->scenes_comp.release();
	if (b->h_words)
		cudaFreeHost(b->h_words);
	b->h_words = nullptr;
}

} // namespace

extern "C" {

int prt_b200_batch_create(prt_b200_ctx *ctx, prt_b200_batch **out) {
	if (!ctx || !out)
		return PRT_ERR_ARG;
	*out = nullptr;
	std::lock_guard<std::mutex> lk(ctx->mu);
	B_TRY(ctx, cudaSetDevice(ctx->device));
	prt_b200_batch *b = new (std::nothrow) prt_b200_batch();
	if (!b)
		return bfail(ctx, PRT_ERR_OOM, "batch: out of host memory");
	b->ctx = ctx;
	cudaError_t e = cudaMallocHost(&b->h_words, 64);
	for (int i = 0; i < kSlots && e == cudaSuccess; ++i) {
		e = b->slots[i].work.reserve(64);
		if (e == cudaSuccess)
			e = cudaMemset(b->slots[i].work.p, 0, 64);
		if (e == cudaSuccess)
			e = cudaEventCreateWithFlags(&b->slots[i].done, cudaEventDisableTiming);
	}
	if (e == cudaSuccess)
		e = b->gslot.work.reserve(64);
	if (e == cudaSuccess)
		e = cudaMemset(b->gslot.work.p, 0, 64);
	if (e == cudaSuccess)
		e = cudaEventCreateWithFlags(&b->gslot.done, cudaEventDisableTiming);
	if (e != cudaSuccess) {
		// Whatever was created before the failure is freed (the lock is held here).
		int rc = bcuda(ctx, e, "batch create");
		release_batch(b);
		delete b;
		return rc;
	}
	*out = b;
	return PRT_OK;
}

void prt_b200_batch_destroy(prt_b200_batch *b) {
	if (!b)
		return;
	if (b->ctx) {
		std::lock_guard<std::mutex> lk(b->ctx->mu);
		cudaSetDevice(b->ctx->device);
		cudaDeviceSynchronize();
		release_batch(b);
	}
	delete b;
}

int prt_b200_batch_set_tris_dev(prt_b200_batch *b, const float *d_tris, const uint64_t *tri_off,
                                uint32_t n_scenes) {
	if (!b)
		return PRT_ERR_ARG;
	prt_b200_ctx *ctx = b->ctx;
	return prt::guarded(&ctx->err, "batch set_tris", [&]() -> int {
		if (n_scenes == 0 || !tri_off || (tri_off[n_scenes] && !d_tris))
			return bfail(ctx, PRT_ERR_ARG, "batch set_tris: need scenes, offsets and triangles");
		std::lock_guard<std::mutex> lk(ctx->mu);
		B_TRY(ctx, cudaSetDevice(ctx->device));
		for (int i = 0; i < kSlots; ++i) {
			int rc = check_slot(b, b->slots[i]);
			if (rc != PRT_OK)
				return rc;
		}
		drop_graph(b);
		b->built = false;
		prt::EventPair ev;
		B_TRY(ctx, ev.create());
		cudaEventRecord(ev.a, ctx->stream);
		std::string msg;
		// Binned-SAH trees as set_tris builds them (option build_sah); a tree too deep for
		// the collapse falls back to the LBVH.  Graph builds (run_graph) are always LBVH.
		bool sah = ctx->build_sah;
		int rc = prt::build_scenes(d_tris, tri_off, n_scenes, ctx->leaf_size, ctx->build_compressed,
		                           b->arena, b->ws, ctx->stream, ctx->d_err(), msg, sah,
		                           ctx->collapse_cost);
		if (sah && rc == PRT_ERR_LIMIT) {
			sah = false;
			msg.clear();
			rc = prt::build_scenes(d_tris, tri_off, n_scenes, ctx->leaf_size, ctx->build_compressed,
			                       b->arena, b->ws, ctx->stream, ctx->d_err(), msg, false,
			                       ctx->collapse_cost);
		}
		b->built_sah = sah;
		cudaEventRecord(ev.b, ctx->stream);
		b->build_ms = ev.elapsed_ms();
		if (rc != PRT_OK)
			return bfail(ctx, rc, msg);
		uint32_t err_word = 0;
		B_TRY(ctx, cudaMemcpy(&err_word, ctx->d_err(), 4, cudaMemcpyDeviceToHost));
		if (err_word) {
			cudaMemset(ctx->d_err(), 0, 4);
			return bfail(ctx, PRT_ERR_DEVICE, "batch build: kernel reported an error");
		}
		if ((int)b->arena.depth > prt::traversal_stack_depth())
			return bfail(ctx, PRT_ERR_LIMIT, "batch build: tree too deep for the traversal");
		rc = scene_tables(b);
		if (rc != PRT_OK)
			return rc;
		b->built = true;
		return PRT_OK;
	});
}

int prt_b200_batch_query_dev(prt_b200_batch *b, const prt_b200_query *queries, uint32_t n_queries,
                             void *stream) {
	if (!b || (n_queries && !queries))
		return b ? bfail(b->ctx, PRT_ERR_ARG, "batch query: null query list") : PRT_ERR_ARG;
	prt_b200_ctx *ctx = b->ctx;
	return prt::guarded(&ctx->err, "batch query", [&]() -> int {
		std::lock_guard<std::mutex> lk(ctx->mu);
		if (!b->built)
			return bfail(ctx, PRT_ERR_NO_SCENE, "batch query: batch_set_tris has not succeeded");
		if (ctx->node_format == PRT_NODES_COMPRESSED && !b->arena.has_cnodes)
			return bfail(ctx, PRT_ERR_ARG, "batch query: compressed nodes were not built");
		B_TRY(ctx, cudaSetDevice(ctx->device));
		std::vector<prt::SegDesc> segs;
		unsigned long long n_virtual = 0;
		int rc = segments(b, queries, n_queries, segs, n_virtual);
		if (rc != PRT_OK || segs.empty())
			return rc;
		Slot &s = b->slots[b->next_slot];
		b->next_slot = (b->next_slot + 1) % kSlots;
		rc = check_slot(b, s);
		if (rc != PRT_OK)
			return rc;
		cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
		B_TRY(ctx, s.segs.reserve(sizeof(prt::SegDesc) * segs.size()));
		B_TRY(ctx, cudaMemcpyAsync(s.segs.p, segs.data(), sizeof(prt::SegDesc) * segs.size(),
		                           cudaMemcpyHostToDevice, st));
		rc = launch_query(b, s, segs, n_virtual, 0, b->arena.n_nodes, st);
		if (rc != PRT_OK)
			return rc;
		B_TRY(ctx, cudaEventRecord(s.done, st));
		s.pending = true;
		return PRT_OK;
	});
}

int prt_b200_batch_run_graph(prt_b200_batch *b, const float *d_tris, const uint64_t *tri_off,
                             uint32_t n_scenes, const prt_b200_query *queries,
                             uint32_t n_queries, void *stream) {
	if (!b)
		return PRT_ERR_ARG;
	prt_b200_ctx *ctx = b->ctx;
	return prt::guarded(&ctx->err, "batch run_graph", [&]() -> int {
		if (n_scenes == 0 || !tri_off || (n_queries && !queries))
			return bfail(ctx, PRT_ERR_ARG, "batch run_graph: bad arguments");
		std::lock_guard<std::mutex> lk(ctx->mu);
		B_TRY(ctx, cudaSetDevice(ctx->device));
		cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
		std::string key = graph_key(d_tris, tri_off, n_scenes, queries, n_queries, ctx);
		if (!b->gexec || key != b->graph_key) {
			drop_graph(b);
			b->built = false;
			int rc = check_slot(b, b->gslot);
			if (rc != PRT_OK)
				return rc;
			std::string msg;
			// Plan: reserve everything and upload the offset tables outside the graph.
			rc = prt::build_plan(tri_off, n_scenes, ctx->leaf_size, ctx->build_compressed, b->arena,
			                     b->ws, ctx->stream, b->gplan, msg, false, ctx->collapse_cost);
			if (rc != PRT_OK)
				return bfail(ctx, rc, msg);
			b->arena.has_cnodes = ctx->build_compressed;
			b->arena.depth = (uint32_t)prt::traversal_stack_depth();
			b->arena.n_nodes = b->gplan.node_cap;
			rc = scene_tables(b);
			if (rc != PRT_OK)
				return rc;
			std::vector<prt::SegDesc> segs;
			unsigned long long n_virtual = 0;
			rc = segments(b, queries, n_queries, segs, n_virtual);
			if (rc != PRT_OK)
				return rc;
			B_TRY(ctx, b->gslot.segs.reserve(sizeof(prt::SegDesc) * std::max<size_t>(segs.size(), 1)));
			if (!segs.empty())
				B_TRY(ctx, cudaMemcpy(b->gslot.segs.p, segs.data(), sizeof(prt::SegDesc) * segs.size(),
				                      cudaMemcpyHostToDevice));
			B_TRY(ctx, cudaStreamSynchronize(ctx->stream));
			// Capture: the whole build (no host round-trips) and the query launch.
			B_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
			rc = prt::build_enqueue(d_tris, b->gplan, b->arena, b->ws, ctx->stream, ctx->d_err(),
			                        false, msg);
			if (rc == PRT_OK && !segs.empty())
				rc = launch_query(b, b->gslot, segs, n_virtual,
				                  ctx->pool_depth ? ctx->pool_depth : prt::traversal_stack_depth(),
				                  b->gplan.node_cap, ctx->stream);
			cudaGraph_t g = nullptr;
			cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
			if (rc != PRT_OK) {
				if (g)
					cudaGraphDestroy(g);
				return rc == PRT_ERR_CUDA ? rc : bfail(ctx, rc, msg.empty() ? ctx->err.get() : msg);
			}
			if (ce != cudaSuccess)
				return bcuda(ctx, ce, "batch run_graph: capture");
			b->graph = g;
			cudaError_t ie = cudaGraphInstantiate(&b->gexec, g, 0);
			if (ie != cudaSuccess) {
				drop_graph(b);
				return bcuda(ctx, ie, "batch run_graph: instantiate");
			}
			b->graph_key = std::move(key);
		} else {
			int rc = check_slot(b, b->gslot);
			if (rc != PRT_OK)
				return rc;
		}
		B_TRY(ctx, cudaGraphLaunch(b->gexec, st));
		B_TRY(ctx, cudaEventRecord(b->gslot.done, st));
		b->gslot.pending = true;
		b->graph_dirty = true;
		b->built = true;
		return PRT_OK;
	}, ctx->stream);
}

int prt_b200_batch_sync(prt_b200_batch *b) {
	if (!b)
		return PRT_ERR_ARG;
	prt_b200_ctx *ctx = b->ctx;
	std::lock_guard<std::mutex> lk(ctx->mu);
	B_TRY(ctx, cudaSetDevice(ctx->device));
	for (int i = 0; i < kSlots; ++i) {
		int rc = check_slot(b, b->slots[i]);
		if (rc != PRT_OK)
			return rc;
	}
	int rc = check_slot(b, b->gslot);
	if (rc != PRT_OK)
		return rc;
	if (b->graph_dirty) {
		std::string msg;
		rc = prt::build_finish(b->arena, b->ws, ctx->stream, msg);
		if (rc != PRT_OK)
			return bfail(ctx, rc, msg);
		uint32_t err_word = 0;
		B_TRY(ctx, cudaMemcpy(&err_word, ctx->d_err(), 4, cudaMemcpyDeviceToHost));
		if (err_word) {
			cudaMemset(ctx->d_err(), 0, 4);
			return bfail(ctx, PRT_ERR_DEVICE, "batch build: kernel reported an error");
		}
		b->graph_dirty = false;
	}
	return PRT_OK;
}

int prt_b200_batch_stat(prt_b200_batch *b, const char *key, double *value) {
	if (!b || !key || !value)
		return PRT_ERR_ARG;
	std::lock_guard<std::mutex> lk(b->ctx->mu);
	const std::string k(key);
	const prt::SceneGPU &a = b->arena;
	if (k == "n_scenes")
		*value = a.n_scenes;
	else if (k == "n_tris")
		*value = (double)a.n_tris;
	else if (k == "n_nodes")
		*value = a.n_nodes;
	else if (k == "depth")
		*value = a.depth;
	else if (k == "build_ms")
		*value = b->build_ms;
	else if (k == "build_sah")
		*value = b->built_sah ? 1.0 : 0.0;
	else if (k == "visits_nodes")
		*value = (double)b->visits[0];
	else if (k == "visits_tris")
		*value = (double)b->visits[1];
	else
		return bfail(b->ctx, PRT_ERR_ARG, "unknown batch statistic " + k);
	return PRT_OK;
}

} // extern "C"
