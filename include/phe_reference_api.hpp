// phe_reference_api.hpp - the reference's kernel launch API, backed by libphe_gb300.
//
// Declares, with the reference's names, argument meaning and semantics, the launch functions of
// source/cuda_ray_tracer/kernels/RayCastKernel.hpp:47-74:
//   launchRayCastKernel, launchRayCastNoPersistenceKernel, launchShadowRayCastKernel,
//   launchGenPrimaryRaysKernel.
// Like the reference they are noexcept, synchronous (results are ready on return, the reference
// calls cudaDeviceSynchronize, RayCastKernel.cu:831-832), run on the legacy default stream, print
// CUDA errors and continue (CudaHelpers.hpp:13-25). The texture objects of RayCastKernelInput must
// wrap linear device memory (CudaTextureBuffer.hpp:45-69 creates them that way); they are resolved
// to device pointers and the scene is re-laid out once per distinct (nodes, triangles) pair.
//
// The structs below are layout-identical to the reference's (RayIn 32 B, RayHit 16 B, CameraDef of
// four vec3). A build that has the reference headers compiles phe_reference_api.cu with
// -DPHE_WITH_REFERENCE_HEADERS instead and uses the reference's own declarations; the symbols are
// then the ones the reference's callers (CudaTracerRenderer.cpp:501-503, 643, 676, 708) link
// against.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace phe {

struct ApiVec2i { int32_t x, y; };
struct ApiVec3 { float x, y, z; };

// RayCastKernel.hpp:22-37: data1 = (origin.xyz, minDist), data2 = (dir.xyz, maxDist).
struct RayIn final {
	float data1[4];
	float data2[4];
};
static_assert(sizeof(RayIn) == 32, "RayIn is padded");

// RayCastKernel.hpp:39-45.
struct RayHit final {
	uint32_t triangleIndex;
	float t;
	float u, v;
};
static_assert(sizeof(RayHit) == 16, "RayHit is padded");

// RayCastKernel.hpp:50-55.
struct RayCastKernelInput final {
	cudaTextureObject_t bvhNodes;
	cudaTextureObject_t triangleVerts;
	uint32_t numRays;
	const RayIn* rays;
};

// GenerateRays.hpp:14-24.
struct CameraDef final {
	ApiVec3 origin;
	ApiVec3 dir;
	ApiVec3 dX;
	ApiVec3 dY;
};

void launchRayCastKernel(const RayCastKernelInput& input, RayHit* __restrict__ rayResults,
                         const cudaDeviceProp& deviceProperties) noexcept;

void launchRayCastNoPersistenceKernel(const RayCastKernelInput& input, RayHit* __restrict__ rayResults,
                                      const cudaDeviceProp& deviceProperties) noexcept;

void launchShadowRayCastKernel(const RayCastKernelInput& input, bool* __restrict__ inLight,
                               const cudaDeviceProp& deviceProperties) noexcept;

void launchGenPrimaryRaysKernel(RayIn* rays, const CameraDef& cam, ApiVec2i res) noexcept;

// Drops the cached device re-layouts (call after freeing or rewriting scene buffers that were
// passed through texture objects).
void invalidateSceneCache() noexcept;

} // namespace phe
