// prt_serve.cu - a request server over resident scenes (continuous batching).
//
// The server keeps S built scenes resident in HBM (a batch, prt_batch.cu) and answers
// nearest-hit requests (scene, host rays, record layout, host output) as they arrive:
//
//   submit  -> FIFO queue (any thread)
//   admit   -> the scheduler thread takes requests from the head of the queue while
//              their rays and records fit in the device memory budget (one region
//              reserved at start-up, carved by a first-fit range allocator) and a
//              lane is free; the admitted requests form one wave.  With several lanes,
//              lane 0 is an express lane (highest stream priority) that takes only
//              small requests, passing over larger ones queued before them
//   run     -> per wave, on the lane's stream: rays copied in, ONE launch of the
//              segment traversal over every request of the wave, smallest requests
//              first (each warp takes at most a few batches, so the blocks of a long
//              wave retire steadily and a higher-priority wave's blocks are scheduled
//              in between); up to n_lanes waves are in flight at once, so requests
//              that arrive while others run are admitted into the next wave as soon
//              as memory and a lane are free, and their work overlaps on the device
//   finish  -> per request: where the device reaches the request's output buffer
//              (pinned memory; pageable memory on a Grace host) the traversal writes
//              the records there and raises the request's completion flag when its
//              last batch is stored; the lane's completer thread polls the flags and
//              finishes each such request at once (finish time, memory returned,
//              waiters woken), while the rest of the wave still runs
//   retire  -> when the wave's launch ends the completer copies out the records of
//              requests whose buffers the device cannot reach, finishes them and frees
//              the lane
//
// That is wave mode (option serve_persistent 0).  In persistent mode (the default) there
// are no waves: the scheduler appends each admitted request to one of three device
// queues by size while one serving launch runs, the launch's warps take the queues'
// batches smallest-request-first, and the completer finishes requests from their
// completion flags, stops the launch when the server is idle and starts it again when
// work is outstanding (see the persistent-mode section below).
//
// A request's records are exactly nearest_hits<Tags...> on its scene alone: the launch
// gives each request its own segment (rays padded to whole warps), and the traversal of
// a ray depends only on the ray, its scene and the record layout.
//
// No counterpart in the reference (portableRT answers one synchronous call at a time,
// include/portableRT/nearest_hits_impl.hpp:28-36).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <exception>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/prt_b200.h"
#include "prt_batch.cuh"
#include "prt_range_alloc.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint32_t kMaxWaveRequests = 1024;
constexpr uint64_t kMaxRequestRays = 1ull << 31;
// Requests of at most this many rays may take the express lane (lane 0 of a server
// with several lanes: its stream has the highest priority and it carries small waves
// only), ahead of larger requests that arrived before them.
constexpr uint64_t kExpressRays = 65536;


struct Request {
	uint64_t id = 0;
	uint32_t scene = 0, mask = 0, rec = 0;
	uint8_t offs[8] = {};
	const float *rays = nullptr;
	uint64_t n = 0;
	void *out = nullptr;
	void *dev_out = nullptr; // the device's address of `out` (records written in place), or null
	uint64_t off = 0, ray_bytes = 0, bytes = 0; // range in the budget region
	Clock::time_point t_submit, t_launch, t_done;
	int status = PRT_OK;
	bool done = false;
};

struct Lane {
	cudaStream_t st = nullptr;
	cudaEvent_t ev = nullptr;
	prt::DevBuf segs;                // SegDesc table of the wave
	prt::DevBuf work;                // [0] ray counter, [1] error word, [4..7] visits
	prt::DevBuf seg_ctr;             // per request of the wave: rays stored (device)
	uint32_t *h_done = nullptr;      // per request: completion flag (pinned, mapped)
	uint32_t *d_done = nullptr;      // the device's address of h_done
	prt::SegDesc *h_segs = nullptr;  // pinned staging of the table
	uint32_t *h_err = nullptr;       // pinned copy of the error word
	std::vector<Request *> wave;     // requests in flight on this lane
	// Per request of the wave: written in place (1) or copied out; finished early (1).  A
	// request finished early may be deleted by its waiter at once, so after that only
	// these flags are read, never the request.
	std::vector<uint8_t> in_place, fin;
	bool launched = false;           // the wave's work (and event) has been queued
	std::thread completer;
	std::condition_variable cv;
};

// A persistent serving launch: the host appends each admitted request to one of three
// queues by size (at most kExpressRays rays; at most kMediumRays; larger) while the
// launch runs, and its warps claim the queues' batches in that order (ServeQueues), so a
// request never waits behind a larger one's batches.
constexpr uint64_t kMediumRays = 524288;
constexpr uint32_t kQueueSegs = 4096;        // requests per queue between resets
constexpr uint64_t kQueueBatches = 1ull << 26; // 2^31 rays in batches of 32
constexpr auto kIdleStop = std::chrono::milliseconds(5); // stop the launch after this idle time
constexpr uint32_t kIdlePolls = 1u << 18;    // an idle warp's polls before it leaves (~1 s)

struct PQueue {
	prt::DevBuf segs;                       // SegDesc[kQueueSegs] (device)
	prt::DevBuf done_ctr;                   // rays stored per request (device)
	prt::SegDesc *h_segs = nullptr;         // pinned staging of the descriptors
	uint32_t *h_words = nullptr;            // pinned staging of (n_segs, published) per request
	uint32_t *h_done = nullptr;             // completion flags (pinned, mapped)
	uint32_t *d_done = nullptr;             // the device's address of h_done
	std::vector<Request *> reqs;            // per request slot
	std::vector<uint8_t> fin;               // finished
	uint32_t n_segs = 0, first_open = 0;
	uint64_t n_batches = 0;
};

struct Persist {
	cudaStream_t st = nullptr;  // the serving launch
	cudaStream_t ctl = nullptr; // resets, ray copies, descriptors, publication, stop flag
	cudaStream_t out = nullptr; // copy-out of staged records
	cudaEvent_t ev = nullptr;   // recorded after the serving launch
	cudaEvent_t ev_ctl = nullptr;
	prt::DevBuf state;          // ServeQueueState[kServeQueues]
	prt::DevBuf stop;           // stop flag of the launch
	prt::DevBuf work;           // the launch's error word
	uint32_t *h_const = nullptr;             // pinned {0, 1}
	uint32_t *h_err = nullptr, *d_err = nullptr; // fault flag (pinned, mapped)
	PQueue q[prt::kServeQueues];
	bool running = false, stopping = false, faulted = false, full = false;
	uint64_t outstanding = 0;   // published, not finished
	uint64_t fail_after = 0;    // test hook: raise the fault flag after this publication
	uint64_t published = 0;     // publications so far
	Clock::time_point last_activity;
	std::thread completer;
};

} // namespace

struct prt_b200_server {
	prt_b200_ctx *ctx = nullptr;
	prt_b200_batch *batch = nullptr;
	int format = PRT_NODES_FP32;
	prt::DevBuf region;
	prt::RangeAllocator alloc;
	std::vector<std::unique_ptr<Lane>> lanes;
	std::thread sched;
	std::mutex mu;
	std::condition_variable cv_sched, cv_done;
	std::deque<Request *> waiting;
	std::unordered_map<uint64_t, Request *> reqs;
	uint64_t next_id = 1;
	bool stop = false;
	std::string err;
	// statistics
	uint64_t waves = 0, in_flight = 0, max_in_flight = 0, max_wave_requests = 0;
	uint64_t express_waves = 0;
	// Batches of 32 rays a warp of a wave's launch takes before it exits (0 = until the
	// wave's work runs out): blocks of a long wave retire as they finish, so the block
	// scheduler can start an express wave's blocks meanwhile.
	uint32_t batches_per_warp = 1;
	// Records go straight to a request's host buffer when the device reaches it (the
	// context's "host_direct" option when the server was created); else they are staged.
	bool host_direct = true;
	uint64_t completed = 0, rays_done = 0;
	// Persistent mode (the context's "serve_persistent" option when created): requests
	// are folded into one running launch instead of launched as waves.
	bool persistent = true;
	std::unique_ptr<Persist> P;
};

namespace {

// Records an error message; the caller holds the server's lock.
int sfail(prt_b200_server *s, int code, const std::string &msg) {
	s->err = msg;
	return code;
}

int sfail_unlocked(prt_b200_server *s, int code, const std::string &msg) {
	std::lock_guard<std::mutex> lk(s->mu);
	return sfail(s, code, msg);
}

uint64_t round256(uint64_t b) { return (b + 255) & ~255ull; }

// Moves waiting requests into L's wave while their buffers fit: in arrival order, up to
// the first that does not fit, or (express) only those of at most kExpressRays rays,
// passing over larger ones.  Caller holds the lock.
void fill_wave(prt_b200_server *s, Lane &L, bool express) {
	unsigned long long nv = 0;
	for (auto it = s->waiting.begin();
	     it != s->waiting.end() && L.wave.size() < kMaxWaveRequests;) {
		Request *r = *it;
		if (express && r->n > kExpressRays) {
			++it;
			continue;
		}
		const unsigned long long pad = (r->n + 31ull) & ~31ull;
		if (nv + pad > (1ull << 31))
			break;
		const uint64_t off = s->alloc.alloc(r->bytes);
		if (off == prt::RangeAllocator::kFail)
			break; // later requests wait behind this one
		r->off = off;
		r->t_launch = Clock::now();
		nv += pad;
		it = s->waiting.erase(it);
		L.wave.push_back(r);
	}
}

// A lane with a new wave, or null.  The express lane takes small requests first; the
// other lanes take requests in arrival order.
Lane *admit(prt_b200_server *s) {
	const size_t n = s->lanes.size();
	if (n > 1 && s->lanes[0]->wave.empty()) {
		fill_wave(s, *s->lanes[0], true);
		if (!s->lanes[0]->wave.empty()) {
			++s->express_waves;
			return s->lanes[0].get();
		}
	}
	for (size_t i = n > 1 ? 1 : 0; i < n; ++i) {
		Lane &L = *s->lanes[i];
		if (!L.wave.empty())
			continue;
		fill_wave(s, L, false);
		return L.wave.empty() ? nullptr : &L;
	}
	return nullptr;
}

// Queues the wave's copies, launch and event on the lane's stream (no lock held).  The
// wave's requests are ordered by size, smallest first: warps take batches in segment
// order, so a small request's batches are not queued behind a large one's.
cudaError_t launch_wave(prt_b200_server *s, Lane &L) {
	prt_b200_batch *b = s->batch;
	uint8_t *base = s->region.as<uint8_t>();
	unsigned long long nv = 0;
	std::stable_sort(L.wave.begin(), L.wave.end(),
	                 [](const Request *x, const Request *y) { return x->n < y->n; });
	const uint32_t k = (uint32_t)L.wave.size();
	L.fin.assign(k, 0); // capacity reserved at creation: no allocation
	L.in_place.assign(k, 0);
	for (uint32_t i = 0; i < k; ++i)
		L.in_place[i] = L.wave[i]->dev_out ? 1 : 0;
	// No launch of this lane is in flight (its last wave retired): the flags can be
	// cleared from the host.
	std::memset(L.h_done, 0, 4 * (size_t)k);
	cudaError_t e0 = cudaMemsetAsync(L.seg_ctr.p, 0, 4 * (size_t)k, L.st);
	if (e0 != cudaSuccess)
		return e0;
	for (uint32_t i = 0; i < k; ++i) {
		Request *r = L.wave[i];
		prt::SegDesc &d = L.h_segs[i];
		d = prt::SegDesc{};
		d.vbegin = nv;
		d.rays = reinterpret_cast<const float *>(base + r->off);
		d.out = r->dev_out ? static_cast<uint8_t *>(r->dev_out) : base + r->off + r->ray_bytes;
		d.n_rays = (uint32_t)r->n;
		d.scene = r->scene;
		d.mask = r->mask;
		d.rec_size = r->rec;
		std::memcpy(d.off, r->offs, 8);
		d.store_mode = prt::store_mode_for(d.out);
		d.pad = 0;
		d.done_ctr = L.seg_ctr.as<uint32_t>() + i;
		d.done_flag = L.d_done + i;
		nv += (r->n + 31ull) & ~31ull;
		cudaError_t e = cudaMemcpyAsync(base + r->off, r->rays, 24 * r->n,
		                                cudaMemcpyHostToDevice, L.st);
		if (e != cudaSuccess)
			return e;
	}
	cudaError_t e = cudaMemcpyAsync(L.segs.p, L.h_segs, sizeof(prt::SegDesc) * k,
	                                cudaMemcpyHostToDevice, L.st);
	if (e == cudaSuccess)
		e = cudaMemsetAsync(L.work.as<uint32_t>() + 1, 0, 4, L.st);
	if (e != cudaSuccess)
		return e;
	prt::TravConfig cfg;
	cfg.format = s->format;
	cfg.block = s->ctx->block;
	cfg.max_batches = s->batches_per_warp;
	const prt::SceneDesc *tab = s->format == PRT_NODES_COMPRESSED
	                                ? b->scenes_comp.as<prt::SceneDesc>()
	                                : b->scenes_fp32.as<prt::SceneDesc>();
	uint32_t *w = L.work.as<uint32_t>();
	e = prt::launch_nearest_hits_segments(tab, L.segs.as<prt::SegDesc>(), k, nv, b->arena.depth,
	                                      b->arena.leaf_size, b->arena.n_nodes, b->arena.dead,
	                                      cfg, w,
	                                      reinterpret_cast<unsigned long long *>(w + 4), w + 1,
	                                      L.st, s->ctx->sms);
	if (e != cudaSuccess)
		return e;
	e = cudaMemcpyAsync(L.h_err, w + 1, 4, cudaMemcpyDeviceToHost, L.st);
	if (e == cudaSuccess)
		e = cudaEventRecord(L.ev, L.st);
	return e;
}

// Copies the wave's records to the requests' host buffers, after its traversal (run by
// the lane's completer, so a copy to pageable memory, which returns only when done,
// never holds up the scheduler).
cudaError_t copy_out(prt_b200_server *s, Lane &L) {
	uint8_t *base = s->region.as<uint8_t>();
	for (size_t i = 0; i < L.wave.size(); ++i) {
		if (L.in_place[i])
			continue; // written in place by the traversal
		Request *r = L.wave[i];
		const cudaError_t e = cudaMemcpyAsync(r->out, base + r->off + r->ray_bytes,
		                                      (uint64_t)r->rec * r->n, cudaMemcpyDeviceToHost,
		                                      L.st);
		if (e != cudaSuccess)
			return e;
	}
	return cudaStreamSynchronize(L.st);
}

// Finishes one request (caller holds the lock): its memory returns to the budget.
void finish(prt_b200_server *s, Request *r, int status, Clock::time_point t) {
	r->t_done = t;
	r->status = status;
	r->done = true;
	s->alloc.release(r->off, r->bytes);
	++s->completed;
	s->rays_done += r->n;
}

// Finishes the requests of a lane's wave that are not finished yet and frees the lane
// (caller holds the lock).
void retire(prt_b200_server *s, Lane &L, int status, Clock::time_point t) {
	for (size_t i = 0; i < L.wave.size(); ++i)
		if (i >= L.fin.size() || !L.fin[i])
			finish(s, L.wave[i], status, t);
	L.wave.clear();
	L.launched = false;
	--s->in_flight;
	s->cv_done.notify_all();
	s->cv_sched.notify_one();
}

void scheduler(prt_b200_server *s) {
	cudaSetDevice(s->ctx->device);
	std::unique_lock<std::mutex> lk(s->mu);
	while (!s->stop) {
		Lane *L = s->waiting.empty() ? nullptr : admit(s);
		if (!L) {
			s->cv_sched.wait(lk); // a submit, a retired wave or stop
			continue;
		}
		++s->waves;
		++s->in_flight;
		s->max_in_flight = std::max(s->max_in_flight, s->in_flight);
		s->max_wave_requests = std::max<uint64_t>(s->max_wave_requests, L->wave.size());
		lk.unlock();
		const cudaError_t e = launch_wave(s, *L);
		lk.lock();
		if (e != cudaSuccess) {
			// Nothing of a failed wave is waited for: wait for its stream so that no
			// copy still uses the memory, then fail its requests.
			lk.unlock();
			cudaStreamSynchronize(L->st);
			lk.lock();
			s->err = std::string("server wave: ") + cudaGetErrorString(e);
			retire(s, *L, PRT_ERR_CUDA, Clock::now());
			continue;
		}
		L->launched = true;
		L->cv.notify_one();
	}
	// Stopping: requests that were never admitted fail.
	for (Request *r : s->waiting) {
		r->status = PRT_ERR_ARG;
		r->t_done = Clock::now();
		r->done = true;
	}
	s->waiting.clear();
	s->cv_done.notify_all();
}

void completer(prt_b200_server *s, Lane *L) {
	cudaSetDevice(s->ctx->device);
	std::unique_lock<std::mutex> lk(s->mu);
	for (;;) {
		L->cv.wait(lk, [&] { return L->launched || (s->stop && L->wave.empty()); });
		if (!L->launched)
			return;
		lk.unlock();
		// Requests whose records the traversal writes in place finish as soon as their
		// completion flag is up; the rest of the wave finishes when its launch has ended.
		// The wave's kernels end by themselves (bounded traversal steps), so this loop
		// ends too.
		const size_t k = L->wave.size();
		size_t open = 0;
		for (size_t i = 0; i < k; ++i)
			open += L->in_place[i];
		cudaError_t e = cudaSuccess;
		for (;;) {
			const cudaError_t q = cudaEventQuery(L->ev);
			const bool ended = q != cudaErrorNotReady;
			if (open) {
				const Clock::time_point t = Clock::now();
				bool any = false;
				for (size_t i = 0; i < k; ++i) {
					if (L->in_place[i] && !L->fin[i] &&
					    reinterpret_cast<volatile const uint32_t *>(L->h_done)[i]) {
						if (!any)
							lk.lock();
						any = true;
						finish(s, L->wave[i], PRT_OK, t);
						L->fin[i] = 1;
						--open;
					}
				}
				if (any) {
					s->cv_done.notify_all();
					s->cv_sched.notify_one();
					lk.unlock();
				}
			}
			if (ended) {
				if (q != cudaSuccess)
					e = q;
				break;
			}
			std::this_thread::sleep_for(std::chrono::microseconds(20));
		}
		if (e == cudaSuccess && !*L->h_err)
			e = copy_out(s, *L);
		const Clock::time_point t = Clock::now();
		lk.lock();
		int status = PRT_OK;
		if (e != cudaSuccess) {
			status = PRT_ERR_CUDA;
			s->err = std::string("server wave: ") + cudaGetErrorString(e);
		} else if (*L->h_err) {
			status = PRT_ERR_DEVICE;
			s->err = "server wave: kernel reported an error";
		}
		retire(s, *L, status, t);
	}
}

// Frees a lane's stream, event and buffers (its threads have stopped).
void release_lane(Lane &L) {
	if (L.st)
		cudaStreamSynchronize(L.st);
	L.segs.release();
	L.work.release();
	L.seg_ctr.release();
	if (L.h_done)
		cudaFreeHost(L.h_done);
	L.h_done = nullptr;
	L.d_done = nullptr;
	if (L.h_segs)
		cudaFreeHost(L.h_segs);
	if (L.h_err)
		cudaFreeHost(L.h_err);
	if (L.ev)
		cudaEventDestroy(L.ev);
	if (L.st)
		cudaStreamDestroy(L.st);
	L.h_segs = nullptr;
	L.h_err = nullptr;
	L.ev = nullptr;
	L.st = nullptr;
}

// ---------------------------------------------------------------------------------------
// Persistent mode.

// The serving launch's queue arguments (device addresses).
prt::ServeQueues p_queues(prt_b200_server *s) {
	Persist &P = *s->P;
	prt::ServeQueues q;
	for (int k = 0; k < prt::kServeQueues; ++k) {
		q.state[k] = P.state.as<prt::ServeQueueState>() + k;
		q.segs[k] = P.q[k].segs.as<prt::SegDesc>();
	}
	q.stop = P.stop.as<uint32_t>();
	q.err_flag = P.d_err;
	q.idle_limit = kIdlePolls;
	q.pad = 0;
	return q;
}

// Empties both queues for the next launch (caller holds the lock; no launch runs and
// no request is outstanding).  Queued on ctl, before any later publication.
cudaError_t p_reset(prt_b200_server *s) {
	Persist &P = *s->P;
	cudaError_t e = cudaMemsetAsync(P.state.p, 0, prt::kServeQueues * sizeof(prt::ServeQueueState),
	                                P.ctl);
	for (int k = 0; k < prt::kServeQueues && e == cudaSuccess; ++k) {
		PQueue &Q = P.q[k];
		e = cudaMemsetAsync(Q.done_ctr.p, 0, 4 * (size_t)kQueueSegs, P.ctl);
		std::memset(Q.h_done, 0, 4 * (size_t)kQueueSegs);
		Q.n_segs = Q.first_open = 0;
		Q.n_batches = 0;
	}
	*reinterpret_cast<volatile uint32_t *>(P.h_err) = 0;
	P.faulted = P.full = false;
	return e;
}

// Starts the serving launch on st after everything queued on ctl so far (the reset and
// the publications up to now); the stop flag is cleared first.  Caller holds the lock.
cudaError_t p_launch(prt_b200_server *s) {
	Persist &P = *s->P;
	prt_b200_batch *b = s->batch;
	cudaError_t e = cudaMemcpyAsync(P.stop.p, P.h_const, 4, cudaMemcpyHostToDevice, P.ctl);
	if (e == cudaSuccess)
		e = cudaEventRecord(P.ev_ctl, P.ctl);
	if (e == cudaSuccess)
		e = cudaStreamWaitEvent(P.st, P.ev_ctl, 0);
	if (e != cudaSuccess)
		return e;
	const prt::SceneDesc *tab = s->format == PRT_NODES_COMPRESSED
	                                ? b->scenes_comp.as<prt::SceneDesc>()
	                                : b->scenes_fp32.as<prt::SceneDesc>();
	e = prt::launch_serving(tab, p_queues(s), b->arena.depth, b->arena.leaf_size,
	                        b->arena.n_nodes, b->arena.dead, s->format, P.work.as<uint32_t>(),
	                        P.st, s->ctx->sms);
	if (e == cudaSuccess)
		e = cudaEventRecord(P.ev, P.st);
	if (e == cudaSuccess) {
		P.running = true;
		P.stopping = false;
		++s->waves;
	}
	return e;
}

// Tells the running launch to end once no batch is left to claim (caller holds the lock).
void p_stop(prt_b200_server *s) {
	Persist &P = *s->P;
	if (cudaMemcpyAsync(P.stop.p, P.h_const + 1, 4, cudaMemcpyHostToDevice, P.ctl) == cudaSuccess)
		P.stopping = true;
}

// Appends request r to queue qi and publishes its batches: its rays copied into its
// budget range, its descriptor into the table, the table size and then the batch count
// into the queue state, all in order on ctl, so a warp that sees the batches sees the
// rest.  Caller holds the lock.
cudaError_t p_publish(prt_b200_server *s, int qi, Request *r) {
	Persist &P = *s->P;
	PQueue &Q = P.q[qi];
	uint8_t *base = s->region.as<uint8_t>();
	const uint32_t i = Q.n_segs;
	prt::SegDesc d{};
	d.vbegin = 32ull * Q.n_batches;
	d.rays = reinterpret_cast<const float *>(base + r->off);
	d.out = r->dev_out ? static_cast<uint8_t *>(r->dev_out) : base + r->off + r->ray_bytes;
	d.n_rays = (uint32_t)r->n;
	d.scene = r->scene;
	d.mask = r->mask;
	d.rec_size = r->rec;
	std::memcpy(d.off, r->offs, 8);
	d.store_mode = prt::store_mode_for(d.out);
	d.pad = 0;
	d.done_ctr = Q.done_ctr.as<uint32_t>() + i;
	d.done_flag = Q.d_done + i;
	// Test hook: this publication behaves as if one of its batches faulted -- its run is
	// not counted, so the request never completes -- and the fault flag rises.
	const bool inject = P.fail_after && ++P.published == P.fail_after;
	if (inject)
		d.done_ctr = d.done_flag = nullptr;
	Q.h_segs[i] = d;
	Q.reqs[i] = r;
	Q.fin[i] = 0;
	cudaError_t e = cudaMemcpyAsync(base + r->off, r->rays, 24 * r->n, cudaMemcpyHostToDevice, P.ctl);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(Q.segs.as<prt::SegDesc>() + i, Q.h_segs + i, sizeof(prt::SegDesc),
		                    cudaMemcpyHostToDevice, P.ctl);
	Q.n_segs = i + 1;
	Q.n_batches += (r->n + 31) / 32;
	Q.h_words[2 * i] = Q.n_segs;
	Q.h_words[2 * i + 1] = (uint32_t)Q.n_batches;
	prt::ServeQueueState *st = P.state.as<prt::ServeQueueState>() + qi;
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(&st->n_segs, Q.h_words + 2 * i, 4, cudaMemcpyHostToDevice, P.ctl);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(&st->published, Q.h_words + 2 * i + 1, 4, cudaMemcpyHostToDevice, P.ctl);
	++P.outstanding;
	s->max_in_flight = std::max<uint64_t>(s->max_in_flight, P.outstanding);
	if (inject)
		*reinterpret_cast<volatile uint32_t *>(P.h_err) = 1u; // as the faulted batch would
	if (qi == 0)
		++s->express_waves;
	return e;
}

void scheduler_p(prt_b200_server *s) {
	cudaSetDevice(s->ctx->device);
	Persist &P = *s->P;
	std::unique_lock<std::mutex> lk(s->mu);
	while (!s->stop) {
		bool admitted = false, large_blocked = false;
		if (!P.stopping && !P.faulted && !P.full) {
			// Arrival order; a small request may pass larger ones that wait for memory.
			for (auto it = s->waiting.begin(); it != s->waiting.end();) {
				Request *r = *it;
				const int qi = r->n <= kExpressRays ? 0 : (r->n <= kMediumRays ? 1 : 2);
				if (qi > 0 && large_blocked) {
					++it;
					continue;
				}
				PQueue &Q = P.q[qi];
				if (Q.n_segs == kQueueSegs || Q.n_batches + (r->n + 31) / 32 > kQueueBatches) {
					P.full = true; // admitted again after the next reset
					break;
				}
				const uint64_t off = s->alloc.alloc(r->bytes);
				if (off == prt::RangeAllocator::kFail) {
					if (qi == 0)
						break;
					large_blocked = true;
					++it;
					continue;
				}
				r->off = off;
				r->t_launch = Clock::now();
				it = s->waiting.erase(it);
				const cudaError_t e = p_publish(s, qi, r);
				if (e != cudaSuccess) {
					s->err = std::string("server publish: ") + cudaGetErrorString(e);
					P.faulted = true; // what reached the queue is finished as failed
					break;
				}
				admitted = true;
			}
		}
		if (admitted) {
			P.last_activity = Clock::now();
			if (!P.running) {
				const cudaError_t e = p_launch(s);
				if (e != cudaSuccess) {
					s->err = std::string("server launch: ") + cudaGetErrorString(e);
					P.faulted = true;
				}
			}
		}
		s->cv_sched.wait_for(lk, std::chrono::milliseconds(1));
	}
	for (Request *r : s->waiting) {
		r->status = PRT_ERR_ARG;
		r->t_done = Clock::now();
		r->done = true;
	}
	s->waiting.clear();
	s->cv_done.notify_all();
}

// Finishes queue slot i of Q (caller holds the lock): records copied out first where they
// were staged.
void p_finish_slot(prt_b200_server *s, PQueue &Q, uint32_t i, int status,
                   std::unique_lock<std::mutex> &lk) {
	Persist &P = *s->P;
	Request *r = Q.reqs[i];
	if (status == PRT_OK && !r->dev_out) {
		uint8_t *src = s->region.as<uint8_t>() + r->off + r->ray_bytes;
		void *dst = r->out;
		const uint64_t bytes = (uint64_t)r->rec * r->n;
		lk.unlock();
		cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, P.out);
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(P.out);
		lk.lock();
		if (e != cudaSuccess) {
			status = PRT_ERR_CUDA;
			s->err = std::string("server copy-out: ") + cudaGetErrorString(e);
		}
	}
	finish(s, r, status, Clock::now());
	Q.fin[i] = 1;
	--P.outstanding;
}

void completer_p(prt_b200_server *s) {
	cudaSetDevice(s->ctx->device);
	Persist &P = *s->P;
	std::unique_lock<std::mutex> lk(s->mu);
	for (;;) {
		if (s->stop && s->waiting.empty() && P.outstanding == 0 && !P.running)
			break;
		lk.unlock();
		std::this_thread::sleep_for(std::chrono::microseconds(20));
		lk.lock();
		// Requests whose last batch is stored.  (A request's slot is read only while it is
		// unfinished: a finished request may be deleted by its waiter.)
		bool any = false;
		for (int k = 0; k < prt::kServeQueues; ++k) {
			PQueue &Q = P.q[k];
			for (uint32_t i = Q.first_open; i < Q.n_segs; ++i)
				if (!Q.fin[i] && reinterpret_cast<volatile const uint32_t *>(Q.h_done)[i]) {
					p_finish_slot(s, Q, i, PRT_OK, lk);
					any = true;
				}
			while (Q.first_open < Q.n_segs && Q.fin[Q.first_open])
				++Q.first_open;
		}
		if (any) {
			P.last_activity = Clock::now();
			s->cv_done.notify_all();
			s->cv_sched.notify_one();
		}
		// A batch that faulted: its request never completes.  Stop the launch; what is
		// unfinished fails once the launch has ended (until then it may still write).
		if (!P.faulted && *reinterpret_cast<volatile const uint32_t *>(P.h_err)) {
			P.faulted = true;
			s->err = "server: the traversal reported an error";
		}
		if (P.running && !P.stopping &&
		    (P.faulted || (P.outstanding == 0 &&
		                   (s->stop || P.full ||
		                    (s->waiting.empty() && Clock::now() - P.last_activity > kIdleStop)))))
			p_stop(s);
		// The launch has ended (stopped, or every warp left idle), or nothing runs after a
		// failure: fail what a fault left unfinished, then reset or go on.
		const cudaError_t q = P.running ? cudaEventQuery(P.ev) : cudaSuccess;
		if ((P.running && q != cudaErrorNotReady) || (!P.running && P.faulted && P.outstanding)) {
			if (P.running && q != cudaSuccess && !P.faulted) {
				P.faulted = true;
				s->err = std::string("server: the serving launch failed: ") + cudaGetErrorString(q);
			}
			P.running = false;
			P.stopping = false;
			if (P.faulted) {
				for (int k = 0; k < prt::kServeQueues; ++k) {
					PQueue &Q = P.q[k];
					for (uint32_t i = Q.first_open; i < Q.n_segs; ++i)
						if (!Q.fin[i])
							p_finish_slot(s, Q, i, PRT_ERR_DEVICE, lk);
					Q.first_open = Q.n_segs;
				}
				s->cv_done.notify_all();
			}
			if (P.outstanding == 0) {
				const cudaError_t e = p_reset(s);
				if (e != cudaSuccess) {
					s->err = std::string("server reset: ") + cudaGetErrorString(e);
					P.faulted = true;
				}
			} else {
				// Every warp left while work was still published (idle limit): go on.
				const cudaError_t e = p_launch(s);
				if (e != cudaSuccess) {
					s->err = std::string("server launch: ") + cudaGetErrorString(e);
					P.faulted = true;
				}
			}
			s->cv_sched.notify_one();
		}
	}
}

void p_release(Persist &P) {
	for (cudaStream_t st : {P.st, P.ctl, P.out})
		if (st)
			cudaStreamSynchronize(st);
	for (int k = 0; k < prt::kServeQueues; ++k) {
		PQueue &Q = P.q[k];
		Q.segs.release();
		Q.done_ctr.release();
		for (void *h : {(void *)Q.h_segs, (void *)Q.h_words, (void *)Q.h_done})
			if (h)
				cudaFreeHost(h);
		Q.h_segs = nullptr;
		Q.h_words = Q.h_done = Q.d_done = nullptr;
	}
	P.state.release();
	P.stop.release();
	P.work.release();
	for (void *h : {(void *)P.h_const, (void *)P.h_err})
		if (h)
			cudaFreeHost(h);
	P.h_const = P.h_err = P.d_err = nullptr;
	for (cudaEvent_t ev : {P.ev, P.ev_ctl})
		if (ev)
			cudaEventDestroy(ev);
	for (cudaStream_t st : {P.st, P.ctl, P.out})
		if (st)
			cudaStreamDestroy(st);
	P.ev = P.ev_ctl = nullptr;
	P.st = P.ctl = P.out = nullptr;
}

// Streams, buffers and the empty queues of persistent mode.
cudaError_t p_create(prt_b200_server *s) {
	Persist &P = *s->P;
	cudaError_t e = cudaSuccess;
	for (cudaStream_t *st : {&P.st, &P.ctl, &P.out})
		if (e == cudaSuccess)
			e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
	if (e == cudaSuccess)
		e = cudaEventCreateWithFlags(&P.ev, cudaEventDisableTiming);
	if (e == cudaSuccess)
		e = cudaEventCreateWithFlags(&P.ev_ctl, cudaEventDisableTiming);
	if (e == cudaSuccess)
		e = P.state.reserve(prt::kServeQueues * sizeof(prt::ServeQueueState));
	if (e == cudaSuccess)
		e = P.stop.reserve(16);
	if (e == cudaSuccess)
		e = P.work.reserve(16);
	if (e == cudaSuccess)
		e = cudaMemset(P.work.p, 0, 16);
	if (e == cudaSuccess)
		e = cudaMallocHost(&P.h_const, 8);
	if (e == cudaSuccess) {
		P.h_const[0] = 0;
		P.h_const[1] = 1;
		e = cudaHostAlloc(&P.h_err, 16, cudaHostAllocMapped);
	}
	if (e == cudaSuccess)
		e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&P.d_err), P.h_err, 0);
	for (int k = 0; k < prt::kServeQueues && e == cudaSuccess; ++k) {
		PQueue &Q = P.q[k];
		e = Q.segs.reserve(sizeof(prt::SegDesc) * kQueueSegs);
		if (e == cudaSuccess)
			e = Q.done_ctr.reserve(4 * (size_t)kQueueSegs);
		if (e == cudaSuccess)
			e = cudaMallocHost(&Q.h_segs, sizeof(prt::SegDesc) * kQueueSegs);
		if (e == cudaSuccess)
			e = cudaMallocHost(&Q.h_words, 8 * (size_t)kQueueSegs);
		if (e == cudaSuccess)
			e = cudaHostAlloc(&Q.h_done, 4 * (size_t)kQueueSegs, cudaHostAllocMapped);
		if (e == cudaSuccess)
			e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&Q.d_done), Q.h_done, 0);
		if (e == cudaSuccess) {
			try {
				Q.reqs.assign(kQueueSegs, nullptr);
				Q.fin.assign(kQueueSegs, 1);
			} catch (const std::bad_alloc &) {
				e = cudaErrorMemoryAllocation;
			}
		}
	}
	if (e == cudaSuccess)
		e = p_reset(s);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(P.ctl);
	P.last_activity = Clock::now();
	return e;
}

void shutdown(prt_b200_server *s) {
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	s->cv_sched.notify_all();
	if (s->sched.joinable())
		s->sched.join();
	if (s->P && s->P->completer.joinable())
		s->P->completer.join(); // it finishes what is outstanding and stops the launch
	for (auto &l : s->lanes) {
		{
			std::lock_guard<std::mutex> lk(s->mu);
			l->cv.notify_all();
		}
		if (l->completer.joinable())
			l->completer.join();
	}
}

} // namespace

extern "C" {

int prt_b200_server_create(prt_b200_ctx *ctx, const float *d_tris, const uint64_t *tri_off,
                           uint32_t n_scenes, uint64_t budget_bytes, uint32_t n_lanes,
                           prt_b200_server **out) {
	if (!ctx || !out)
		return PRT_ERR_ARG;
	*out = nullptr;
	if (n_lanes < 1 || n_lanes > 16 || budget_bytes < 4096) {
		ctx->err = "server: n_lanes must be in [1, 16] and the budget at least 4 KiB";
		return PRT_ERR_ARG;
	}
	std::unique_ptr<prt_b200_server> s(new (std::nothrow) prt_b200_server());
	if (!s)
		return PRT_ERR_OOM;
	s->ctx = ctx;
	int rc = prt_b200_batch_create(ctx, &s->batch);
	if (rc != PRT_OK)
		return rc;
	rc = prt_b200_batch_set_tris_dev(s->batch, d_tris, tri_off, n_scenes);
	if (rc != PRT_OK) {
		prt_b200_batch_destroy(s->batch);
		return rc;
	}
	uint64_t fail_serve_after = 0;
	{
		std::lock_guard<std::mutex> lk(ctx->mu);
		s->format = ctx->node_format;
		s->batches_per_warp = (uint32_t)ctx->serve_batches_per_warp;
		s->host_direct = ctx->host_direct;
		s->persistent = ctx->serve_persistent;
		fail_serve_after = (uint64_t)ctx->fail_serve_after;
	}
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e == cudaSuccess)
		e = s->region.reserve(budget_bytes);
	s->alloc.reset(budget_bytes, 256);
	if (e == cudaSuccess && s->persistent) {
		s->P.reset(new (std::nothrow) Persist());
		e = s->P ? p_create(s.get()) : cudaErrorMemoryAllocation;
		if (s->P)
			s->P->fail_after = fail_serve_after;
	}
	int least = 0, greatest = 0;
	if (e == cudaSuccess)
		e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
	for (uint32_t i = 0; i < n_lanes && e == cudaSuccess && !s->persistent; ++i) {
		std::unique_ptr<Lane> L(new (std::nothrow) Lane());
		if (!L) {
			e = cudaErrorMemoryAllocation;
			break;
		}
		// Lane 0 of several is the express lane: the highest stream priority.
		e = cudaStreamCreateWithPriority(&L->st, cudaStreamNonBlocking,
		                                 (i == 0 && n_lanes > 1) ? greatest : least);
		if (e == cudaSuccess)
			e = cudaEventCreateWithFlags(&L->ev, cudaEventDisableTiming);
		if (e == cudaSuccess)
			e = L->segs.reserve(sizeof(prt::SegDesc) * kMaxWaveRequests);
		if (e == cudaSuccess)
			e = L->work.reserve(64);
		if (e == cudaSuccess)
			e = cudaMemset(L->work.p, 0, 64);
		if (e == cudaSuccess)
			e = cudaMallocHost(&L->h_segs, sizeof(prt::SegDesc) * kMaxWaveRequests);
		if (e == cudaSuccess)
			e = cudaMallocHost(&L->h_err, 16);
		if (e == cudaSuccess)
			e = L->seg_ctr.reserve(4 * kMaxWaveRequests);
		if (e == cudaSuccess)
			e = cudaHostAlloc(&L->h_done, 4 * kMaxWaveRequests, cudaHostAllocMapped);
		if (e == cudaSuccess)
			e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&L->d_done), L->h_done, 0);
		// A wave holds at most kMaxWaveRequests requests: with the room reserved here the
		// scheduler thread never allocates to fill one.
		try {
			L->wave.reserve(kMaxWaveRequests);
			L->in_place.reserve(kMaxWaveRequests);
			L->fin.reserve(kMaxWaveRequests);
			s->lanes.push_back(std::move(L));
		} catch (const std::bad_alloc &) {
			if (L) // not yet owned by the server: free what it holds
				release_lane(*L);
			e = cudaErrorMemoryAllocation;
		}
	}
	if (e != cudaSuccess) {
		// No lock is held here: destroying the server destroys its batch, which takes the
		// context's lock (ctx->err has a lock of its own).
		ctx->err = std::string("server create: ") + cudaGetErrorString(e);
		prt_b200_server_destroy(s.release());
		return e == cudaErrorMemoryAllocation ? PRT_ERR_OOM : PRT_ERR_CUDA;
	}
	prt_b200_server *sp = s.get();
	try {
		if (sp->persistent) {
			sp->P->completer = std::thread(completer_p, sp);
			sp->sched = std::thread(scheduler_p, sp);
		} else {
			for (auto &l : sp->lanes)
				l->completer = std::thread(completer, sp, l.get());
			sp->sched = std::thread(scheduler, sp);
		}
	} catch (const std::exception &ex) {
		// A thread that could not start: stop those that did and free everything.
		ctx->err = std::string("server create: ") + ex.what();
		prt_b200_server_destroy(s.release());
		return PRT_ERR_OOM;
	}
	*out = s.release();
	return PRT_OK;
}

void prt_b200_server_destroy(prt_b200_server *s) {
	if (!s)
		return;
	shutdown(s);
	cudaSetDevice(s->ctx->device);
	for (auto &l : s->lanes)
		release_lane(*l);
	if (s->P)
		p_release(*s->P);
	for (auto &kv : s->reqs)
		delete kv.second;
	s->region.release();
	if (s->batch)
		prt_b200_batch_destroy(s->batch);
	delete s;
}

int prt_b200_server_submit(prt_b200_server *s, uint32_t scene, const float *rays6, uint64_t n,
                           uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                           void *out_host, uint64_t *ticket) {
	if (!s || !ticket)
		return PRT_ERR_ARG;
	std::string why;
	if (!prt::layout_ok(field_mask, rec_size, offs, why))
		return sfail_unlocked(s, PRT_ERR_ARG, "server submit: " + why);
	if (scene >= s->batch->arena.n_scenes)
		return sfail_unlocked(s, PRT_ERR_ARG, "server submit: no such scene");
	if (n && (!rays6 || !out_host))
		return sfail_unlocked(s, PRT_ERR_ARG, "server submit: null buffer");
	if (n > kMaxRequestRays)
		return sfail_unlocked(s, PRT_ERR_LIMIT, "server submit: at most 2^31 rays per request");
	std::unique_ptr<Request> r(new (std::nothrow) Request());
	if (!r)
		return PRT_ERR_OOM;
	r->scene = scene;
	r->mask = field_mask;
	r->rec = rec_size;
	std::memcpy(r->offs, offs, 8);
	r->rays = rays6;
	r->n = n;
	r->out = out_host;
	r->ray_bytes = round256(24 * n);
	// Records go straight to out_host when the device reaches it; otherwise they are
	// staged in the budget region and copied out when the wave's launch has ended.
	if (n && s->host_direct)
		r->dev_out = prt::device_alias(s->ctx, out_host);
	r->bytes = r->ray_bytes + (r->dev_out ? 0 : (uint64_t)rec_size * n);
	std::lock_guard<std::mutex> lk(s->mu);
	if (s->stop)
		return sfail(s, PRT_ERR_ARG, "server submit: server is stopping");
	if (n && !s->alloc.fits_ever(r->bytes))
		return sfail(s, PRT_ERR_LIMIT, "server submit: request larger than the memory budget");
	// Host memory for the ticket table or the queue may run out: the request is then
	// neither queued nor given a ticket, and the call returns PRT_ERR_OOM.
	r->id = s->next_id;
	r->t_submit = Clock::now();
	try {
		auto ins = s->reqs.emplace(r->id, r.get());
		if (n) {
			try {
				s->waiting.push_back(r.get());
			} catch (...) {
				s->reqs.erase(ins.first);
				throw;
			}
		}
	} catch (const std::bad_alloc &) {
		return sfail(s, PRT_ERR_OOM, "server submit: out of host memory");
	}
	++s->next_id;
	*ticket = r->id;
	Request *rp = r.release();
	if (n == 0) {
		rp->t_done = rp->t_submit;
		rp->done = true;
	} else {
		s->cv_sched.notify_one();
	}
	return PRT_OK;
}

int prt_b200_server_wait(prt_b200_server *s, uint64_t ticket, double *latency_ms) {
	if (!s)
		return PRT_ERR_ARG;
	std::unique_lock<std::mutex> lk(s->mu);
	auto it = s->reqs.find(ticket);
	if (it == s->reqs.end())
		return sfail(s, PRT_ERR_ARG, "server wait: unknown ticket");
	Request *r = it->second;
	s->cv_done.wait(lk, [&] { return r->done; });
	if (latency_ms)
		*latency_ms =
		    std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
	const int status = r->status;
	s->reqs.erase(it);
	delete r;
	return status;
}

int prt_b200_server_stat(prt_b200_server *s, const char *key, double *value) {
	if (!s || !key || !value)
		return PRT_ERR_ARG;
	std::lock_guard<std::mutex> lk(s->mu);
	const std::string k(key);
	if (k == "waves")
		*value = (double)s->waves;
	else if (k == "max_in_flight_waves")
		*value = (double)s->max_in_flight;
	else if (k == "express_waves")
		*value = (double)s->express_waves;
	else if (k == "max_wave_requests")
		*value = (double)s->max_wave_requests;
	else if (k == "completed")
		*value = (double)s->completed;
	else if (k == "rays")
		*value = (double)s->rays_done;
	else if (k == "waiting")
		*value = (double)s->waiting.size();
	else if (k == "bytes_in_use")
		*value = (double)s->alloc.used();
	else if (k == "peak_bytes")
		*value = (double)s->alloc.peak();
	else if (k == "budget_bytes")
		*value = (double)s->alloc.capacity();
	else if (k == "n_scenes")
		*value = (double)s->batch->arena.n_scenes;
	else if (k == "n_tris")
		*value = (double)s->batch->arena.n_tris;
	else
		return sfail(s, PRT_ERR_ARG, "unknown server statistic " + k);
	return PRT_OK;
}

// The calling thread's copy of the message, valid until its next call here.
const char *prt_b200_server_last_error(prt_b200_server *s) {
	if (!s)
		return "null server";
	thread_local std::string copy;
	std::lock_guard<std::mutex> lk(s->mu);
	copy = s->err;
	return copy.c_str();
}

} // extern "C"
