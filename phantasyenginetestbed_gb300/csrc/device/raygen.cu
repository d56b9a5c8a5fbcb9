// Primary-ray generation (genPrimaryRaysKernel + calculatePrimaryRayDir,
// cuda_ray_tracer/kernels/RayCastKernel.cu:891-919) with a sub-pixel jitter offset added to the
// pixel location, as the TAA camera offset does (screens/GameScreen.cpp:187-203).

#include "raygen.cuh"
#include "runtime.cuh"

namespace phe_gb300 {

__global__ void gen_primary_kernel(phe_ray_in* __restrict__ rays, phe_camera_def cam, uint32_t resX, uint32_t resY,
                                   float jx, float jy, int order)
{
	uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= resX || y >= resY) return;
	f3 d = primary_dir(cam, x, y, resX, resY, jx, jy);
	uint32_t id = ray_index(x, y, resX, order);
	float4* p = reinterpret_cast<float4*>(rays + id);
	p[0] = make_float4(cam.origin[0], cam.origin[1], cam.origin[2], 0.0001f);
	p[1] = make_float4(d.x, d.y, d.z, 3.402823466e+38f);
}

} // namespace phe_gb300

using namespace phe_gb300;

extern "C" phe_status phe_gen_primary_rays(phe_ray_in* rays, const phe_camera_def* cam, uint32_t resX, uint32_t resY,
                                           float jitterX, float jitterY, int order, void* stream)
{
	if (!rays || !cam) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_gen_primary_rays: null argument");
	if (order != 0 && order != 1) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_gen_primary_rays: order must be 0 or 1");
	if (order == 1 && ((resX % 8u) != 0 || (resY % 8u) != 0))
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_gen_primary_rays: 8x8 order needs a resolution multiple of 8");
	if ((uint64_t)resX * resY > 0xFFFFFFFFull) return fail(PHE_ERR_TOO_LARGE, "phe_gen_primary_rays: too many pixels");
	if (resX == 0 || resY == 0) return PHE_OK;
	dim3 block(8, 8);
	dim3 grid((resX + 7) / 8, (resY + 7) / 8);
	gen_primary_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(rays, *cam, resX, resY, jitterX, jitterY, order);
	PHE_CUDA_TRY(cudaGetLastError(), "gen_primary_kernel launch");
	return PHE_OK;
}
