// The reference's kernel launch functions (cuda_ray_tracer/kernels/RayCastKernel.hpp:57-74)
// implemented on top of the C ABI. See include/phe_reference_api.hpp.

#include <cstdio>
#include <map>
#include <mutex>
#include <tuple>

#ifdef PHE_WITH_REFERENCE_HEADERS
#include "kernels/RayCastKernel.hpp"
namespace phe {
using ShimVec2i = sfz::vec2i;
void invalidateSceneCache() noexcept;
}
#else
#include "phe_reference_api.hpp"
namespace phe {
using ShimVec2i = ApiVec2i;
}
#endif

#include "phe_gb300.h"

namespace phe {
namespace {

// CHECK_CUDA_ERROR behaviour (CudaHelpers.hpp:13-25): report and continue.
void report(const char* what, phe_status st, int line)
{
	std::fprintf(stderr, "%s:%d: %s failed (status %d): %s\n", __FILE__, line, what, st, phe_last_error());
}

void reportCuda(cudaError_t e, int line)
{
	if (e != cudaSuccess) std::fprintf(stderr, "%s:%d: CUDA error: %s\n", __FILE__, line, cudaGetErrorString(e));
}

struct LinearTex {
	void* ptr = nullptr;
	size_t bytes = 0;
};

bool resolve(cudaTextureObject_t tex, LinearTex& out)
{
	cudaResourceDesc desc;
	cudaError_t e = cudaGetTextureObjectResourceDesc(&desc, tex);
	if (e != cudaSuccess) {
		reportCuda(e, __LINE__);
		return false;
	}
	if (desc.resType != cudaResourceTypeLinear) {
		std::fprintf(stderr, "%s:%d: texture object is not over linear memory\n", __FILE__, __LINE__);
		return false;
	}
	out.ptr = desc.res.linear.devPtr;
	out.bytes = desc.res.linear.sizeInBytes;
	return true;
}

using Key = std::tuple<void*, size_t, void*, size_t>;
std::mutex g_cacheMutex;
std::map<Key, phe_scene*> g_cache;

// The device scene for a (nodes, triangles) texture pair, created on first use.
phe_scene* sceneFor(const RayCastKernelInput& input)
{
	LinearTex n, t;
	if (!resolve(input.bvhNodes, n) || !resolve(input.triangleVerts, t)) return nullptr;
	Key key{n.ptr, n.bytes, t.ptr, t.bytes};
	std::lock_guard<std::mutex> lock(g_cacheMutex);
	auto it = g_cache.find(key);
	if (it != g_cache.end()) return it->second;
	phe_scene* s = nullptr;
	phe_status st = phe_scene_create((const phe_bvh_node*)n.ptr, (uint32_t)(n.bytes / sizeof(phe_bvh_node)),
	                                 (const phe_triangle_vertices*)t.ptr,
	                                 nullptr, (uint32_t)(t.bytes / sizeof(phe_triangle_vertices)), nullptr, 0,
	                                 PHE_PTR_DEVICE, &s);
	if (st != PHE_OK) {
		report("phe_scene_create", st, __LINE__);
		return nullptr;
	}
	g_cache[key] = s;
	return s;
}

} // namespace

void launchRayCastKernel(const RayCastKernelInput& input, RayHit* __restrict__ rayResults,
                         const cudaDeviceProp& deviceProperties) noexcept
{
	(void)deviceProperties;
	phe_scene* s = sceneFor(input);
	if (!s) return;
	phe_status st = phe_cast_closest(s, (const phe_ray_in*)input.rays, (phe_ray_hit*)rayResults, input.numRays, nullptr);
	if (st != PHE_OK) report("phe_cast_closest", st, __LINE__);
	reportCuda(cudaDeviceSynchronize(), __LINE__);
}

void launchRayCastNoPersistenceKernel(const RayCastKernelInput& input, RayHit* __restrict__ rayResults,
                                      const cudaDeviceProp& deviceProperties) noexcept
{
	(void)deviceProperties;
	phe_scene* s = sceneFor(input);
	if (!s) return;
	phe_status st =
	    phe_cast_closest_plain(s, (const phe_ray_in*)input.rays, (phe_ray_hit*)rayResults, input.numRays, nullptr);
	if (st != PHE_OK) report("phe_cast_closest_plain", st, __LINE__);
	reportCuda(cudaDeviceSynchronize(), __LINE__);
}

void launchShadowRayCastKernel(const RayCastKernelInput& input, bool* __restrict__ inLight,
                               const cudaDeviceProp& deviceProperties) noexcept
{
	static_assert(sizeof(bool) == 1, "inLight is one byte per ray");
	(void)deviceProperties;
	phe_scene* s = sceneFor(input);
	if (!s) return;
	phe_status st = phe_cast_any(s, (const phe_ray_in*)input.rays, (uint8_t*)inLight, input.numRays, nullptr, nullptr);
	if (st != PHE_OK) report("phe_cast_any", st, __LINE__);
	reportCuda(cudaDeviceSynchronize(), __LINE__);
}

void launchGenPrimaryRaysKernel(RayIn* rays, const CameraDef& cam, ShimVec2i res) noexcept
{
	phe_camera_def c;
	c.origin[0] = cam.origin.x; c.origin[1] = cam.origin.y; c.origin[2] = cam.origin.z;
	c.dir[0] = cam.dir.x; c.dir[1] = cam.dir.y; c.dir[2] = cam.dir.z;
	c.dX[0] = cam.dX.x; c.dX[1] = cam.dX.y; c.dX[2] = cam.dX.z;
	c.dY[0] = cam.dY.x; c.dY[1] = cam.dY.y; c.dY[2] = cam.dY.z;
	// The reference writes rays in 8x8-tile order (getRayIdx with 8x8 blocks, RayCastKernel.cu:915-917).
	int order = ((res.x % 8) == 0 && (res.y % 8) == 0) ? 1 : 0;
	phe_status st = phe_gen_primary_rays((phe_ray_in*)rays, &c, (uint32_t)res.x, (uint32_t)res.y, 0.0f, 0.0f, order,
	                                     nullptr);
	if (st != PHE_OK) report("phe_gen_primary_rays", st, __LINE__);
	reportCuda(cudaDeviceSynchronize(), __LINE__);
}

void invalidateSceneCache() noexcept
{
	std::lock_guard<std::mutex> lock(g_cacheMutex);
	for (auto& kv : g_cache) phe_scene_destroy(kv.second);
	g_cache.clear();
}

} // namespace phe
