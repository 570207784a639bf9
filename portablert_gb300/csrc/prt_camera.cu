// prt_camera.cu - the steps either side of the nearest-hit path in portableRT's examples,
// on the device: the pinhole sensor camera (rays built inside the traversal, or written
// out) and the headless Lambert shading of the hits into an RGBA8 buffer.
//
// The reference computes these on the host around each nearest_hits call
// (examples/bunny/main.cpp:101-124, examples/validation/main.cpp:170-198,
// examples/sponza/main.cpp:11-32,193-243) and shows the image in an SDL window; here the
// image stays a device buffer (no window exists on this machine).
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/prt_b200.h"
#include "prt_camera.cuh"
#include "prt_ctx.cuh"
#include "prt_traverse.cuh"

namespace {

int cfail(prt_b200_ctx *ctx, int code, const std::string &msg) {
	ctx->err = msg;
	return code;
}

int cuda_fail(prt_b200_ctx *ctx, cudaError_t e, const char *what) {
	return cfail(ctx, e == cudaErrorMemoryAllocation ? PRT_ERR_OOM : PRT_ERR_CUDA,
	             std::string(what) + ": " + cudaGetErrorString(e));
}

} // namespace

namespace prt {

bool camera_ok(const prt_b200_camera *c, std::string &why) {
	if (!c) {
		why = "null camera";
		return false;
	}
	if (c->width == 0 || c->height == 0 || (uint64_t)c->width * c->height > (1ull << 31)) {
		why = "camera: width and height must be positive, width x height <= 2^31";
		return false;
	}
	if (c->form > PRT_CAMERA_ROTATED) {
		why = "camera: unknown form";
		return false;
	}
	return true;
}

} // namespace prt

namespace {

using prt::camera_ok;

__global__ void k_camera_rays(prt_b200_camera cam, uint64_t n, float *rays) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
	     i += (uint64_t)gridDim.x * blockDim.x) {
		float o[3], d[3];
		prt::camera_ray(cam, (uint32_t)i, o, d);
		float *r = rays + 6 * i;
		for (int k = 0; k < 3; ++k) {
			r[k] = o[k];
			r[3 + k] = d[k];
		}
	}
}

// examples/sponza/main.cpp:11-32: clamp(N . -d, 0, 1) with N the geometric normal
// (e1 x e2 from the first vertex), normalised when its length exceeds 0.001.
__device__ __forceinline__ float lambert(const float4 &A, const float4 &B, const float4 &C,
                                         const float d[3]) {
	const float e1[3] = {__fsub_rn(B.x, A.x), __fsub_rn(B.y, A.y), __fsub_rn(B.z, A.z)};
	const float e2[3] = {__fsub_rn(C.x, A.x), __fsub_rn(C.y, A.y), __fsub_rn(C.z, A.z)};
	float N[3] = {__fsub_rn(__fmul_rn(e1[1], e2[2]), __fmul_rn(e1[2], e2[1])),
	              __fsub_rn(__fmul_rn(e1[2], e2[0]), __fmul_rn(e1[0], e2[2])),
	              __fsub_rn(__fmul_rn(e1[0], e2[1]), __fmul_rn(e1[1], e2[0]))};
	const float len = __fsqrt_rn(
	    __fadd_rn(__fadd_rn(__fmul_rn(N[0], N[0]), __fmul_rn(N[1], N[1])), __fmul_rn(N[2], N[2])));
	if ((double)fabsf(len) > 0.001) {
		N[0] = __fdiv_rn(N[0], len);
		N[1] = __fdiv_rn(N[1], len);
		N[2] = __fdiv_rn(N[2], len);
	}
	const float dot = __fadd_rn(__fadd_rn(__fmul_rn(N[0], -d[0]), __fmul_rn(N[1], -d[1])),
	                            __fmul_rn(N[2], -d[2]));
	const float m = (1.0f < dot) ? 1.0f : dot; // std::min(dot, 1.0f)
	return (0.0f < m) ? m : 0.0f;               // std::max(0.0f, m)
}

// examples/sponza/main.cpp:228-243: grey = 255 * shade for t != inf, else black.
__global__ void k_lambert(const float4 *__restrict__ tri4, const uint32_t *__restrict__ inv,
                          uint64_t n_tris, prt_b200_camera cam, uint32_t use_cam,
                          const float *__restrict__ rays, uint64_t n,
                          const uint8_t *__restrict__ rec, uint32_t rec_size, uint32_t off_t,
                          uint32_t off_pid, uchar4 *rgba) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
	     i += (uint64_t)gridDim.x * blockDim.x) {
		const uint8_t *r = rec + i * rec_size;
		float t;
		uint32_t pid;
		memcpy(&t, r + off_t, 4);
		memcpy(&pid, r + off_pid, 4);
		uint8_t g = 0;
		if (t != INFINITY && pid < n_tris) {
			float d[3];
			if (use_cam) {
				float o[3];
				prt::camera_ray(cam, (uint32_t)i, o, d);
			} else {
				for (int k = 0; k < 3; ++k)
					d[k] = rays[6 * i + 3 + k];
			}
			const float4 *p = tri4 + 3 * (size_t)inv[pid];
			const float shade = lambert(p[0], p[1], p[2], d);
			g = (uint8_t)__float2uint_rz(__fmul_rn(255.0f, shade));
		}
		rgba[i] = make_uchar4(g, g, g, 255);
	}
}

unsigned grid_for(uint64_t n, int sms) {
	return (unsigned)std::min<uint64_t>((n + 255) / 256, 32ull * (uint64_t)sms);
}

} // namespace

extern "C" {

int prt_b200_camera_rays(prt_b200_ctx *ctx, const prt_b200_camera *camera, float *d_rays6,
                         void *stream) {
	if (!ctx)
		return PRT_ERR_ARG;
	std::string why;
	if (!camera_ok(camera, why))
		return cfail(ctx, PRT_ERR_ARG, "camera_rays: " + why);
	if (!d_rays6)
		return cfail(ctx, PRT_ERR_ARG, "camera_rays: null output");
	std::lock_guard<std::mutex> lk(ctx->mu);
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess)
		return cuda_fail(ctx, e, "camera_rays");
	cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
	const uint64_t n = (uint64_t)camera->width * camera->height;
	k_camera_rays<<<grid_for(n, ctx->sms), 256, 0, st>>>(*camera, n, d_rays6);
	e = cudaGetLastError();
	return e == cudaSuccess ? PRT_OK : cuda_fail(ctx, e, "camera_rays");
}

int prt_b200_shade_lambert(prt_b200_ctx *ctx, const prt_b200_camera *camera,
                           const float *d_rays6, uint64_t n, const void *d_records,
                           uint32_t field_mask, uint32_t rec_size, const uint8_t offs[8],
                           uint8_t *d_rgba, void *stream) {
	if (!ctx)
		return PRT_ERR_ARG;
	return prt::guarded(&ctx->err, "shade_lambert", [&]() -> int {
		std::string why;
		if (!prt::layout_ok(field_mask, rec_size, offs, why))
			return cfail(ctx, PRT_ERR_ARG, "shade_lambert: " + why);
		if ((field_mask & (PRT_FIELD_T | PRT_FIELD_PRIMITIVE_ID)) !=
		    (PRT_FIELD_T | PRT_FIELD_PRIMITIVE_ID))
			return cfail(ctx, PRT_ERR_ARG, "shade_lambert: records need t and primitive_id");
		if (camera) {
			if (!camera_ok(camera, why))
				return cfail(ctx, PRT_ERR_ARG, "shade_lambert: " + why);
			n = (uint64_t)camera->width * camera->height;
		} else if (n && !d_rays6) {
			return cfail(ctx, PRT_ERR_ARG, "shade_lambert: no camera and no rays");
		}
		if (n && (!d_records || !d_rgba))
			return cfail(ctx, PRT_ERR_ARG, "shade_lambert: null buffer");
		if (reinterpret_cast<uintptr_t>(d_rgba) % 4 != 0 ||
		    reinterpret_cast<uintptr_t>(d_records) % 4 != 0)
			return cfail(ctx, PRT_ERR_ARG, "shade_lambert: buffers must be 4-byte aligned");
		std::lock_guard<std::mutex> lk(ctx->mu);
		if (!ctx->scene_set)
			return cfail(ctx, PRT_ERR_NO_SCENE, "shade_lambert: set_tris has not succeeded");
		cudaError_t e = cudaSetDevice(ctx->device);
		if (e != cudaSuccess || n == 0)
			return e == cudaSuccess ? PRT_OK : cuda_fail(ctx, e, "shade_lambert");
		cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
		prt_b200_camera c{};
		if (camera)
			c = *camera;
		const prt::SceneGPU &sc = ctx->scene;
		k_lambert<<<grid_for(n, ctx->sms), 256, 0, st>>>(
		    sc.tri4.as<float4>(), sc.inv.as<uint32_t>(), sc.n_tris, c, camera ? 1u : 0u, d_rays6, n,
		    static_cast<const uint8_t *>(d_records), rec_size, offs[PRT_OFF_T], offs[PRT_OFF_PID],
		    reinterpret_cast<uchar4 *>(d_rgba));
		e = cudaGetLastError();
		if (e != cudaSuccess)
			return cuda_fail(ctx, e, "shade_lambert");
		if (st != ctx->stream) { // a rebuild waits for this read of the scene
			prt_b200_ctx::QueryStream *qs = nullptr;
			const int rc = prt::query_stream(ctx, st, &qs);
			if (rc != PRT_OK)
				return rc;
			e = cudaEventRecord(qs->ev, st);
			if (e != cudaSuccess)
				return cuda_fail(ctx, e, "shade_lambert");
		}
		return PRT_OK;
	});
}

} // extern "C"
