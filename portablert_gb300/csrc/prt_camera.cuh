// prt_camera.cuh - the examples' pinhole sensor camera as a device function (shared by
// the fused camera traversal, the ray writer and the shading kernel).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/prt_b200.h"

namespace prt {

// sensor_size * (float(k) / extent - 0.5): the float quotient widened to double by the
// 0.5 literal, the product rounded to float (examples/bunny/main.cpp:103-104).
__device__ __forceinline__ float sensor_coord(float size, uint32_t k, uint32_t extent) {
	const float q = __fdiv_rn((float)k, (float)extent);
	return __double2float_rn(__dmul_rn((double)size, __dsub_rn((double)q, 0.5)));
}

// Ray i of the camera (examples/bunny/main.cpp:101-124, validation/main.cpp:170-198,
// sponza/main.cpp:193-218), FP32 operation for operation, no contraction.
__device__ __forceinline__ void camera_ray(const prt_b200_camera &c, uint32_t i, float o[3],
                                           float d[3]) {
	const uint32_t x = i % c.width;
	const uint32_t y = c.height - 1u - i / c.width;
	const float sx = sensor_coord(c.sensor_size, x, c.width);
	const float sy = sensor_coord(c.sensor_size, y, c.height);
	float sp[3];
	if (c.form == PRT_CAMERA_ROTATED) {
		const float dx = __fadd_rn(__fmul_rn(c.cos_a, sx), __fmul_rn(c.sin_a, c.sensor_dist));
		const float dz = __fadd_rn(__fmul_rn(-c.sin_a, sx), __fmul_rn(c.cos_a, c.sensor_dist));
		sp[0] = __fadd_rn(c.pos[0], dx);
		sp[1] = __fadd_rn(c.pos[1], sy);
		sp[2] = __fadd_rn(c.pos[2], dz);
	} else {
		sp[0] = sx;
		sp[1] = sy;
		sp[2] = c.sensor_z;
	}
	for (int k = 0; k < 3; ++k) {
		o[k] = c.pos[k];
		d[k] = __fsub_rn(sp[k], c.pos[k]);
	}
	const float *l = c.form == PRT_CAMERA_PLANE_SENSOR_NORM ? sp : d;
	const float len = __fsqrt_rn(
	    __fadd_rn(__fadd_rn(__fmul_rn(l[0], l[0]), __fmul_rn(l[1], l[1])), __fmul_rn(l[2], l[2])));
	for (int k = 0; k < 3; ++k)
		d[k] = __fdiv_rn(d[k], len);
}

// Validates a camera (non-empty, at most 2^31 rays, a known form).
bool camera_ok(const prt_b200_camera *c, std::string &why);

} // namespace prt
