// prt_score.cu - the FP64 scorer of nearest-hit t values.
//
// For every valid record it recomputes t with the Möller–Trumbore formula of
// portableRT's intersect_tri (include/portableRT/core.hpp:27-65) in double, on the
// triangle the record names (its primitive_id, in the caller's AoS triangle array), and
// accumulates |t - t64|.  Every product and sum is rounded separately (no fused
// multiply-add), like the CPU oracle's orc_intersect_tri_f64, so the two agree bit for
// bit.  This is the only FP64 arithmetic on the GPU, and nothing on the query path
// calls it: it measures the FP32 answer's error, it does not produce answers.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/prt_b200.h"
#include "prt_ctx.cuh"

namespace {

// Accumulators: [0] max abs error bits, [1] max relative error bits, [2] sum of abs
// errors (double), [3] hits scored, [4] hits whose t equals t64 rounded to FP32,
// [5] hits that could not be scored (primitive id out of range or t64 not finite).
struct ScoreAcc {
	unsigned long long max_abs, max_rel;
	double sum_abs;
	unsigned long long scored, exact, unscored;
};

__device__ __forceinline__ double dot3(const double *a, const double *b) {
	return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}

__device__ __forceinline__ void cross3(const double *a, const double *b, double *c) {
	c[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
	c[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
	c[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
}

// t of ray r against triangle t9 in double (NaN when det == 0).
__device__ double mt_t64(const float *t9, const float *r) {
	double v0[3], e1[3], e2[3], o[3], d[3];
	for (int k = 0; k < 3; ++k) {
		v0[k] = t9[k];
		e1[k] = __dsub_rn((double)t9[3 + k], v0[k]);
		e2[k] = __dsub_rn((double)t9[6 + k], v0[k]);
		o[k] = r[k];
		d[k] = r[3 + k];
	}
	double p[3], q[3], tv[3];
	cross3(d, e2, p);
	const double det = dot3(e1, p);
	if (det == 0.0)
		return nan("");
	const double inv = __drcp_rn(det);
	for (int k = 0; k < 3; ++k)
		tv[k] = __dsub_rn(o[k], v0[k]);
	cross3(tv, e1, q);
	return __dmul_rn(dot3(e2, q), inv);
}

__device__ __forceinline__ double warp_max(double v) {
	for (int o = 16; o; o >>= 1)
		v = fmax(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
	return v;
}

__device__ __forceinline__ double warp_sum(double v) {
	for (int o = 16; o; o >>= 1)
		v = __dadd_rn(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
	return v;
}

__device__ __forceinline__ unsigned long long warp_count(bool b) {
	return (unsigned long long)__popc(__ballot_sync(0xFFFFFFFFu, b));
}

__global__ void k_t_error(const float *tris, uint64_t n_tris, const float *rays, uint64_t n,
                          const uint8_t *rec, uint32_t rec_size, uint32_t off_t, uint32_t off_pid,
                          uint32_t off_valid, ScoreAcc *acc) {
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint64_t start = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	// Whole warps iterate together (the shuffles need every lane).
	const uint64_t rounds = (n + stride - 1) / stride;
	double mabs = 0.0, mrel = 0.0, sabs = 0.0;
	unsigned long long scored = 0, exact = 0, unscored = 0;
	for (uint64_t k = 0; k < rounds; ++k) {
		const uint64_t i = start + k * stride;
		bool s_ok = false, s_exact = false, s_bad = false;
		if (i < n) {
			const uint8_t *r = rec + i * rec_size;
			if (r[off_valid]) {
				uint32_t pid;
				float t32;
				memcpy(&pid, r + off_pid, 4);
				memcpy(&t32, r + off_t, 4);
				const double t64 = pid < n_tris ? mt_t64(tris + 9ull * pid, rays + 6 * i) : nan("");
				if (isfinite(t64) && isfinite(t32)) {
					const double e = fabs(__dsub_rn((double)t32, t64));
					mabs = fmax(mabs, e);
					if (t64 != 0.0)
						mrel = fmax(mrel, e / fabs(t64));
					sabs = __dadd_rn(sabs, e);
					s_ok = true;
					s_exact = t32 == __double2float_rn(t64);
				} else {
					s_bad = true;
				}
			}
		}
		scored += warp_count(s_ok);
		exact += warp_count(s_exact);
		unscored += warp_count(s_bad);
	}
	mabs = warp_max(mabs);
	mrel = warp_max(mrel);
	sabs = warp_sum(sabs);
	if ((threadIdx.x & 31) == 0) {
		atomicMax(&acc->max_abs, (unsigned long long)__double_as_longlong(mabs));
		atomicMax(&acc->max_rel, (unsigned long long)__double_as_longlong(mrel));
		atomicAdd(&acc->sum_abs, sabs);
		atomicAdd(&acc->scored, scored);
		atomicAdd(&acc->exact, exact);
		atomicAdd(&acc->unscored, unscored);
	}
}

} // namespace

extern "C" int prt_b200_t_error(prt_b200_ctx *ctx, const float *d_tris9, uint64_t n_tris,
                                const float *d_rays6, uint64_t n_rays, const void *d_records,
                                uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                                double result[6]) {
	if (!ctx)
		return PRT_ERR_ARG;
	std::string why;
	if (!result || !prt::layout_ok(field_mask, rec_size, offs, why)) {
		ctx->err = "t_error: " + (why.empty() ? std::string("null result") : why);
		return PRT_ERR_ARG;
	}
	const uint32_t need = PRT_FIELD_T | PRT_FIELD_PRIMITIVE_ID | PRT_FIELD_VALID;
	if ((field_mask & need) != need) {
		ctx->err = "t_error: records need the t, primitive_id and valid fields";
		return PRT_ERR_ARG;
	}
	if (n_rays && (!d_tris9 || !d_rays6 || !d_records)) {
		ctx->err = "t_error: null buffer";
		return PRT_ERR_ARG;
	}
	std::lock_guard<std::mutex> lk(ctx->mu);
	auto cuda_err = [&](cudaError_t e) {
		ctx->err = std::string("t_error: ") + cudaGetErrorString(e);
		return e == cudaErrorMemoryAllocation ? PRT_ERR_OOM : PRT_ERR_CUDA;
	};
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return cuda_err(e);
	ScoreAcc h{};
	if (n_rays) {
		ScoreAcc *d = nullptr;
		e = cudaMallocAsync(&d, sizeof(ScoreAcc), ctx->stream);
		if (e != cudaSuccess)
			return cuda_err(e);
		cudaMemsetAsync(d, 0, sizeof(ScoreAcc), ctx->stream);
		const unsigned grid = (unsigned)std::min<uint64_t>((n_rays + 255) / 256, 16ull * ctx->sms);
		k_t_error<<<grid, 256, 0, ctx->stream>>>(d_tris9, n_tris, d_rays6, n_rays,
		                                         static_cast<const uint8_t *>(d_records), rec_size,
		                                         offs[PRT_OFF_T], offs[PRT_OFF_PID],
		                                         offs[PRT_OFF_VALID], d);
		e = cudaGetLastError();
		if (e == cudaSuccess)
			e = cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, ctx->stream);
		cudaFreeAsync(d, ctx->stream);
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(ctx->stream);
		if (e != cudaSuccess)
			return cuda_err(e);
	}
	double mabs, mrel;
	std::memcpy(&mabs, &h.max_abs, 8);
	std::memcpy(&mrel, &h.max_rel, 8);
	result[0] = mabs;
	result[1] = mrel;
	result[2] = h.scored ? h.sum_abs / (double)h.scored : 0.0;
	result[3] = (double)h.scored;
	result[4] = (double)h.exact;
	result[5] = (double)h.unscored;
	return PRT_OK;
}
