// prt_ctx.cuh - the context behind the C ABI handle, shared by the C ABI sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <exception>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/prt_b200.h"
#include "prt_build.cuh"

namespace prt {

// The message of a context's last failure.  Any thread may set it (argument checks run
// before the context's lock is taken), so it has a lock of its own; readers get a copy.
class ErrorText {
  public:
	ErrorText &operator=(const std::string &m) {
		std::lock_guard<std::mutex> lk(mu_);
		s_ = m;
		return *this;
	}
	std::string get() const {
		std::lock_guard<std::mutex> lk(mu_);
		return s_;
	}

  private:
	mutable std::mutex mu_;
	std::string s_;
};

} // namespace prt

struct prt_b200_ctx {
	int device = 0;
	int sms = 0;
	int pageable_access = 0; // the device reads pageable host memory in place
	cudaStream_t stream = nullptr;
	std::mutex mu;
	prt::ErrorText err;
	prt::SceneGPU scene;
	bool scene_set = false;
	prt::BuildScratch ws;
	prt::DevBuf tris_in;
	prt::DevBuf rays_buf, out_buf;
	prt::DevBuf work; // [0..3] ray counter, [4..7] error word, [8..15] deferred-pass
	                  // words, [16..31] visit counters, [32..47] ray counter and deferred
	                  // words of the second compute stream, [48..51] the read probe's sink
	// The host-buffer call splits large batches into chunks and overlaps the copy-in of a
	// chunk, the traversal of the one before and the copy-out of the one before that.
	static constexpr int kPipe = 16; // most chunks of one call
	int pipe_chunks = 8;             // chunks a call aims for ("pipe_chunks")
	uint32_t pipe_min_rays = 1u << 15; // fewest rays in a chunk ("pipe_min_rays")
	bool pipe_ramp = true;           // chunk sizes ramp up and down ("pipe_ramp")
	cudaStream_t s_in = nullptr, s_out = nullptr, s_k2 = nullptr;
	cudaEvent_t ev_in[kPipe] = {}, ev_k[kPipe] = {};
	// Callers' streams that nearest_hits_dev has queued queries on.  Each has its own
	// ray counter (so queries on different streams may run at once) and an event
	// recorded after its last query, which set_tris waits for before it rebuilds.
	struct QueryStream {
		cudaStream_t st;
		cudaEvent_t ev;
		uint32_t *counter;
	};
	std::vector<QueryStream> query_streams;
	uint32_t *h_err = nullptr;
	int leaf_size = 1;
	int node_format = PRT_NODES_FP32;
	int block = 128;
	int pool_depth = 0; // tree depth a batch graph's traversal pool is sized for (0 = 32)
	int serve_batches_per_warp = 1; // request servers created later ("serve_batches_per_warp")
	int64_t fail_serve_after = 0;   // test hook: a new persistent server's n-th publication
	                                // raises its fault flag ("fail_serve_after"; 0 = off)
	bool serve_persistent = true;   // request servers created later fold requests into one
	                                // running launch ("serve_persistent"; 0 = waves)
	bool count = false;
	bool build_compressed = true;
	bool build_sah = true;       // set_tris builds binned-SAH trees ("build_sah"; 0 = LBVH)
	bool collapse_cost = true;   // cost-optimal 8-wide collapse ("collapse_cost")
	bool build_small = true;     // one block builds scenes of <= 4,096 tris ("build_small")
	bool host_direct = true;     // host-buffer calls traverse in place when they can
	bool last_in_place = false;  // the last host-buffer call did
	bool last_build_sah = false; // the scene's tree is from the quality build
	bool last_build_small = false; // ... made by the one-block build
	double build_ms = 0.0;
	unsigned long long visits[2] = {0, 0};

	uint32_t *d_work() { return work.as<uint32_t>(); }
	uint32_t *d_err() { return work.as<uint32_t>() + 1; }
	unsigned long long *d_visits() {
		return reinterpret_cast<unsigned long long *>(work.as<uint8_t>() + 16);
	}
};

namespace prt {

// The bookkeeping of a caller's stream that reads the context's scene (created at its
// first use): record ->ev on the stream after the work, and set_tris waits for it.
// Caller holds the context's lock.
int query_stream(prt_b200_ctx *ctx, cudaStream_t st, prt_b200_ctx::QueryStream **out);

// Two timing events around work queued on a stream, destroyed however the scope ends.
struct EventPair {
	cudaEvent_t a = nullptr, b = nullptr;
	cudaError_t create() {
		cudaError_t e = cudaEventCreate(&a);
		return e == cudaSuccess ? cudaEventCreate(&b) : e;
	}
	// Milliseconds between the two (after b has been recorded), 0 if unavailable.
	float elapsed_ms() const {
		float ms = 0.0f;
		if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
			ms = 0.0f;
		return ms;
	}
	EventPair() = default;
	EventPair(const EventPair &) = delete;
	EventPair &operator=(const EventPair &) = delete;
	~EventPair() {
		if (a)
			cudaEventDestroy(a);
		if (b)
			cudaEventDestroy(b);
	}
};

// Runs the body of a C entry point and turns a C++ exception (host memory exhausted, a
// thread that could not start) into PRT_ERR_OOM with a message in *err, so that no
// exception crosses the C boundary.  When `capture` is a stream the body left
// capturing, the capture is ended and its graph dropped, so the stream stays usable.
template <class F>
int guarded(ErrorText *err, const char *what, F &&body, cudaStream_t capture = nullptr) noexcept {
	const char *why = "out of host memory";
	try {
		return body();
	} catch (const std::bad_alloc &) {
	} catch (const std::exception &ex) {
		why = ex.what();
	} catch (...) {
		why = "unexpected exception";
	}
	if (capture) {
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		if (cudaStreamIsCapturing(capture, &cs) == cudaSuccess &&
		    cs != cudaStreamCaptureStatusNone) {
			cudaGraph_t g = nullptr;
			if (cudaStreamEndCapture(capture, &g) == cudaSuccess && g)
				cudaGraphDestroy(g);
		}
		cudaGetLastError();
	}
	try {
		if (err)
			*err = std::string(what) + ": " + why;
	} catch (...) {
	}
	return PRT_ERR_OOM;
}

// The address under which the device reaches host buffer p in place, or null: pinned
// (page-locked, registered) memory through its device alias, pageable memory when the
// device reads it through the host's page tables (Grace: NVLink-C2C with address
// translation), managed and device memory as they are.
inline void *device_alias(const prt_b200_ctx *ctx, const void *p) {
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return nullptr;
	}
	switch (a.type) {
	case cudaMemoryTypeHost:
		return a.devicePointer;
	case cudaMemoryTypeDevice:
	case cudaMemoryTypeManaged:
		return a.device == ctx->device ? const_cast<void *>(p) : nullptr;
	case cudaMemoryTypeUnregistered:
		return ctx->pageable_access ? const_cast<void *>(p) : nullptr;
	default:
		return nullptr;
	}
}

// Validates a HitReg layout descriptor.
inline bool layout_ok(uint32_t mask, uint32_t rec, const uint8_t *off, std::string &why) {
	if (mask == 0 || mask > 31u) {
		why = "field_mask must be a non-empty subset of PRT_FIELD_*";
		return false;
	}
	if (rec < 4 || rec > 32 || rec % 4 != 0) {
		why = "rec_size must be a multiple of 4 in [4, 32]";
		return false;
	}
	if (!off) {
		why = "offsets pointer is null";
		return false;
	}
	struct F {
		uint32_t bit;
		int idx;
		uint32_t size;
	} fields[] = {{PRT_FIELD_UV, PRT_OFF_U, 4},      {PRT_FIELD_UV, PRT_OFF_V, 4},
	              {PRT_FIELD_T, PRT_OFF_T, 4},       {PRT_FIELD_PRIMITIVE_ID, PRT_OFF_PID, 4},
	              {PRT_FIELD_VALID, PRT_OFF_VALID, 1}, {PRT_FIELD_P, PRT_OFF_PX, 4},
	              {PRT_FIELD_P, PRT_OFF_PY, 4},      {PRT_FIELD_P, PRT_OFF_PZ, 4}};
	for (const F &f : fields) {
		if (!(mask & f.bit))
			continue;
		uint32_t o = off[f.idx];
		if (o + f.size > rec || (f.size == 4 && o % 4 != 0)) {
			why = "field offset out of range or misaligned";
			return false;
		}
	}
	return true;
}

} // namespace prt
