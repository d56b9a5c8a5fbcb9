// Camera-ray helpers shared by the primary-ray kernel and the fused wavefront kernels.
#pragma once

#include "common.cuh"

namespace phe_gb300 {

// getRayIdx (CudaDeviceHelpers.cuh:49-62) for 8x8 tiles when order == 1, row-major otherwise.
__device__ __forceinline__ uint32_t ray_index(uint32_t x, uint32_t y, uint32_t resX, int order)
{
	if (order == 0) return y * resX + x;
	uint32_t pixBlockIdx = (y >> 3) * (resX >> 3) + (x >> 3);
	return pixBlockIdx * 64u + (y & 7u) * 8u + (x & 7u);
}

// calculatePrimaryRayDir (RayCastKernel.cu:891-897) at pixel (x + jx, y + jy):
// normalize(dir + dX * c.x + dY * c.y), c = loc / res * 2 - 1.
__device__ __forceinline__ f3 primary_dir(const phe_camera_def& cam, uint32_t x, uint32_t y, uint32_t resX, uint32_t resY,
                                          float jx, float jy)
{
	float lx = __fadd_rn((float)x, jx), ly = __fadd_rn((float)y, jy);
	float nx = __fdiv_rn(lx, (float)resX), ny = __fdiv_rn(ly, (float)resY);
	float cx = __fsub_rn(__fmul_rn(nx, 2.0f), 1.0f), cy = __fsub_rn(__fmul_rn(ny, 2.0f), 1.0f);
	f3 dir = mk3(cam.dir[0], cam.dir[1], cam.dir[2]);
	f3 dX = mk3(cam.dX[0], cam.dX[1], cam.dX[2]);
	f3 dY = mk3(cam.dY[0], cam.dY[1], cam.dY[2]);
	return normalize3(add3(add3(dir, muls3(dX, cx)), muls3(dY, cy)));
}

} // namespace phe_gb300
