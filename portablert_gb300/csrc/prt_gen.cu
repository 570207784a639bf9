// prt_gen.cu - the seeded synthetic workloads, generated in device memory.
//
// The same generators as portablert_gb300/workloads.py, so the large configurations
// (millions of triangles, hundreds of millions of rays) need no host generation or
// copy.  Randomness: SplitMix64 (Steele, Lea, Flood 2014).  A stream (seed, id) starts
// at state0 = mix(seed | id << 32) and its k-th output (k = 1, 2, ...) is
// mix(state0 + k * 0x9E3779B97F4A7C15); each array a generator draws takes the next
// run of outputs in row-major order.  FP32 values use round-to-nearest operations in
// the order numpy evaluates them (no contraction); Gaussians are Box-Muller in double
// and rounded to FP32.  Integer draws are bit-identical to numpy's; a value that goes
// through log/cos can differ in its last bit where the device and host math libraries
// round a double differently (the tests bound this).
//
// No counterpart in the reference, which reads meshes from files (examples/bunny).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "../../include/prt_b200.h"
#include "prt_ctx.cuh"

namespace {

constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
	z ^= z >> 30;
	z *= 0xBF58476D1CE4E5B9ull;
	z ^= z >> 27;
	z *= 0x94D049BB133111EBull;
	z ^= z >> 31;
	return z;
}

uint64_t stream_state(uint64_t seed, uint32_t sid) {
	return mix64((seed & 0xFFFFFFFFull) | ((uint64_t)sid << 32));
}

// Output k (1-based) of the stream whose state is s.
__device__ __forceinline__ uint64_t draw(uint64_t s, uint64_t k) { return mix64(s + kGamma * k); }

__device__ __forceinline__ float u01(uint64_t x) {
	return __fmul_rn((float)(uint32_t)(x >> 40), 5.9604644775390625e-8f); // 2^-24
}

__device__ __forceinline__ float uniform(float a, float b, uint64_t x) {
	return __fadd_rn(a, __fmul_rn(__fsub_rn(b, a), u01(x)));
}

__device__ __forceinline__ double u01_f64(uint64_t x) {
	return __dmul_rn((double)(x >> 11), 1.1102230246251565e-16); // 2^-53
}

// Box-Muller from two outputs, as sqrt(-2 log(1 - u1)) * cos(2 pi u2) in double.
__device__ __forceinline__ float gauss(uint64_t x1, uint64_t x2) {
	const double u1 = __dsub_rn(1.0, u01_f64(x1));
	const double u2 = u01_f64(x2);
	const double two_pi = 6.283185307179586; // 2.0 * pi rounded to double
	const double r = __dsqrt_rn(__dmul_rn(-2.0, log(u1)));
	return __double2float_rn(__dmul_rn(r, cos(__dmul_rn(two_pi, u2))));
}

__device__ __forceinline__ void normalize3(float &x, float &y, float &z) {
	const float n = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)),
	                                     __fmul_rn(z, z)));
	x = __fdiv_rn(x, n);
	y = __fdiv_rn(y, n);
	z = __fdiv_rn(z, n);
}

// soup triangles: centre uniform in [-1,1]^3 (3n outputs), vertex offsets uniform in
// [-0.05,0.05]^3 (9n outputs), vertex = centre + offset.
__global__ void k_soup_tris(uint64_t s, uint64_t n, float *out) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
	     i += (uint64_t)gridDim.x * blockDim.x) {
		float c[3];
		for (int k = 0; k < 3; ++k)
			c[k] = uniform(-1.0f, 1.0f, draw(s, 1 + 3 * i + k));
		for (int v = 0; v < 3; ++v)
			for (int k = 0; k < 3; ++k) {
				const float o = uniform(-0.05f, 0.05f, draw(s, 1 + 3 * n + 9 * i + 3 * v + k));
				out[9 * i + 3 * v + k] = __fadd_rn(c[k], o);
			}
	}
}

// soup rays: origin = 3 * normalize(3 Gaussians) (u1: 3n outputs, u2: 3n outputs),
// target uniform in [-0.5,0.5]^3 (3n outputs), direction = normalize(target - origin).
__global__ void k_soup_rays(uint64_t s, uint64_t n, float *out) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
	     i += (uint64_t)gridDim.x * blockDim.x) {
		float o[3], d[3];
		for (int k = 0; k < 3; ++k)
			o[k] = gauss(draw(s, 1 + 3 * i + k), draw(s, 1 + 3 * n + 3 * i + k));
		normalize3(o[0], o[1], o[2]);
		for (int k = 0; k < 3; ++k) {
			o[k] = __fmul_rn(3.0f, o[k]);
			d[k] = __fsub_rn(uniform(-0.5f, 0.5f, draw(s, 1 + 6 * n + 3 * i + k)), o[k]);
		}
		normalize3(d[0], d[1], d[2]);
		for (int k = 0; k < 3; ++k) {
			out[6 * i + k] = o[k];
			out[6 * i + 3 + k] = d[k];
		}
	}
}

// clustered soup: C centres uniform in [-10,10]^3 (3C), sigmas uniform in [0.1,1] (C),
// cluster index floor(u * C) (n), v0 = centre + sigma * Gaussian (u1: 3n, u2: 3n),
// v1 and v2 = v0 + uniform in [-0.02,0.02]^3 (3n each).
__global__ void k_cluster_tris(uint64_t s, uint64_t n, uint32_t C, float *out) {
	const uint64_t b_cid = 1 + 4ull * C, b_g = b_cid + n, b_v1 = b_g + 6 * n, b_v2 = b_v1 + 3 * n;
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
	     i += (uint64_t)gridDim.x * blockDim.x) {
		const float f = __fmul_rn(u01(draw(s, b_cid + i)), (float)C);
		const uint32_t cid = min((uint32_t)f, C - 1);
		const float sigma = uniform(0.1f, 1.0f, draw(s, 1 + 3ull * C + cid));
		float v0[3];
		for (int k = 0; k < 3; ++k) {
			const float c = uniform(-10.0f, 10.0f, draw(s, 1 + 3ull * cid + k));
			const float g = gauss(draw(s, b_g + 3 * i + k), draw(s, b_g + 3 * n + 3 * i + k));
			v0[k] = __fadd_rn(c, __fmul_rn(sigma, g));
		}
		for (int k = 0; k < 3; ++k) {
			out[9 * i + k] = v0[k];
			out[9 * i + 3 + k] = __fadd_rn(v0[k], uniform(-0.02f, 0.02f, draw(s, b_v1 + 3 * i + k)));
			out[9 * i + 6 + k] = __fadd_rn(v0[k], uniform(-0.02f, 0.02f, draw(s, b_v2 + 3 * i + k)));
		}
	}
}

// random rays: origin uniform in [-e,e]^3 (3n), direction = normalize(3 Gaussians)
// (u1: 3n, u2: 3n).
__global__ void k_random_rays(uint64_t s, uint64_t n, float e, float *out) {
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
	     i += (uint64_t)gridDim.x * blockDim.x) {
		float d[3];
		for (int k = 0; k < 3; ++k) {
			out[6 * i + k] = uniform(-e, e, draw(s, 1 + 3 * i + k));
			d[k] = gauss(draw(s, 1 + 3 * n + 3 * i + k), draw(s, 1 + 6 * n + 3 * i + k));
		}
		normalize3(d[0], d[1], d[2]);
		for (int k = 0; k < 3; ++k)
			out[6 * i + 3 + k] = d[k];
	}
}

} // namespace

extern "C" int prt_b200_generate(prt_b200_ctx *ctx, int kind, uint64_t seed, uint64_t n,
                                 double param, void *d_out, void *stream) {
	if (!ctx)
		return PRT_ERR_ARG;
	if (n && !d_out) {
		ctx->err = "generate: null output";
		return PRT_ERR_ARG;
	}
	if (n > (1ull << 40)) {
		ctx->err = "generate: count too large";
		return PRT_ERR_LIMIT;
	}
	std::lock_guard<std::mutex> lk(ctx->mu);
	cudaError_t e = cudaSetDevice(ctx->device);
	if (e != cudaSuccess || n == 0) {
		if (e != cudaSuccess)
			ctx->err = std::string("generate: ") + cudaGetErrorString(e);
		return e == cudaSuccess ? PRT_OK : PRT_ERR_CUDA;
	}
	cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
	const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, 64ull * ctx->sms);
	float *out = static_cast<float *>(d_out);
	switch (kind) {
	case PRT_GEN_SOUP_TRIS:
		k_soup_tris<<<grid, 256, 0, st>>>(stream_state(seed, 1), n, out);
		break;
	case PRT_GEN_SOUP_RAYS:
		k_soup_rays<<<grid, 256, 0, st>>>(stream_state(seed, 2), n, out);
		break;
	case PRT_GEN_CLUSTER_TRIS: {
		if (!(param >= 1.0 && param <= 65536.0)) {
			ctx->err = "generate: cluster count must be in [1, 65536]";
			return PRT_ERR_ARG;
		}
		k_cluster_tris<<<grid, 256, 0, st>>>(stream_state(seed, 1), n, (uint32_t)param, out);
		break;
	}
	case PRT_GEN_RANDOM_RAYS:
		if (!(param > 0.0)) {
			ctx->err = "generate: extent must be positive";
			return PRT_ERR_ARG;
		}
		k_random_rays<<<grid, 256, 0, st>>>(stream_state(seed, 2), n, (float)param, out);
		break;
	default:
		ctx->err = "generate: unknown kind";
		return PRT_ERR_ARG;
	}
	e = cudaGetLastError();
	if (e != cudaSuccess) {
		ctx->err = std::string("generate: ") + cudaGetErrorString(e);
		return PRT_ERR_CUDA;
	}
	return PRT_OK;
}
