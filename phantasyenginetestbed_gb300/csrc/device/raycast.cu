// Ray-cast kernels and their C-ABI launchers: closest hit (plain and persistent) and any hit.
// Replaces rayCastKernel / rayCastNoPersistenceKernel / shadowRayCastKernel and their launchers
// (cuda_ray_tracer/kernels/RayCastKernel.cu:179-886).
//
// Differences in the launch model: every launch is asynchronous on the caller's stream (the
// reference synchronises the whole device after each launch, RayCastKernel.cu:831-832), and the
// persistent kernels take their work counter from a per-launch slot zeroed on the same stream
// instead of a file-static global reset by a second kernel (RayCastKernel.cu:172-177), so launches
// on different streams do not share state.

#include <atomic>

#include "runtime.cuh"
#include "traverse.cuh"

namespace phe_gb300 {

constexpr int kPlainBlock = 128;
constexpr int kPersistentBlock = 128;

template <bool WIDE>
__global__ void __launch_bounds__(kPlainBlock) closest_plain_kernel(DeviceScene s, const phe_ray_in* __restrict__ rays,
                                                                    phe_ray_hit* __restrict__ hits, uint32_t n,
                                                                    uint32_t* __restrict__ status)
{
	uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	RayState r = load_ray(rays, i);
	HitRecord h = empty_hit(r);
	uint32_t err = trace<false, WIDE>(s, r, h);
	if (err) atomicOr(status, err);
	store_hit(hits, i, r, h);
}

// Persistent warps: each warp takes 32 consecutive rays per atomic fetch (one atomic per warp,
// lane 0 fetches and broadcasts) until the batch is exhausted.
template <bool WIDE>
__global__ void __launch_bounds__(kPersistentBlock) closest_persistent_kernel(DeviceScene s,
                                                                              const phe_ray_in* __restrict__ rays,
                                                                              phe_ray_hit* __restrict__ hits, uint32_t n,
                                                                              uint32_t* __restrict__ counter,
                                                                              uint32_t* __restrict__ status)
{
	const uint32_t lane = threadIdx.x & 31u;
	for (;;) {
		uint32_t base = 0;
		if (lane == 0) base = atomicAdd(counter, 32u);
		base = __shfl_sync(0xffffffffu, base, 0);
		if (base >= n) break;
		uint32_t i = base + lane;
		if (i < n) {
			RayState r = load_ray(rays, i);
			HitRecord h = empty_hit(r);
			uint32_t err = trace<false, WIDE>(s, r, h);
			if (err) atomicOr(status, err);
			store_hit(hits, i, r, h);
		}
		__syncwarp();
	}
}

template <bool WIDE>
__global__ void __launch_bounds__(kPersistentBlock) any_persistent_kernel(DeviceScene s,
                                                                          const phe_ray_in* __restrict__ rays,
                                                                          uint8_t* __restrict__ inLight,
                                                                          const uint32_t* __restrict__ scatter, uint32_t n,
                                                                          uint32_t* __restrict__ counter,
                                                                          uint32_t* __restrict__ status)
{
	const uint32_t lane = threadIdx.x & 31u;
	for (;;) {
		uint32_t base = 0;
		if (lane == 0) base = atomicAdd(counter, 32u);
		base = __shfl_sync(0xffffffffu, base, 0);
		if (base >= n) break;
		uint32_t i = base + lane;
		if (i < n) {
			RayState r = load_ray(rays, i);
			HitRecord h = empty_hit(r);
			uint32_t err = trace<true, WIDE>(s, r, h);
			if (err) atomicOr(status, err);
			uint32_t o = scatter ? __ldg(scatter + i) : i;
			inLight[o] = h.slot == ~0u ? 1 : 0;
		}
		__syncwarp();
	}
}

// [closest, any] x [binary, wide]; filled on first use (threads that race store the same value)
static std::atomic<int> g_persistentBlocksPerSM[4] = {};

static phe_status persistent_grid(int which, const void* kernel, int* grid)
{
	DeviceInfo* d = nullptr;
	phe_status st = device_info(&d);
	if (st) return st;
	int blocks = g_persistentBlocksPerSM[which].load(std::memory_order_relaxed);
	if (blocks == 0) {
		int b = 0;
		PHE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, kPersistentBlock,
		                                                           stack_smem_bytes(kPersistentBlock)), "occupancy");
		blocks = b > 0 ? b : 1;
		g_persistentBlocksPerSM[which].store(blocks, std::memory_order_relaxed);
	}
	*grid = blocks * d->numSMs;
	return PHE_OK;
}

static phe_status check_cast_args(const phe_scene* scene, const void* rays, const void* out)
{
	if (!scene) return fail(PHE_ERR_INVALID_ARGUMENT, "scene is null");
	if (!rays || !out) return fail(PHE_ERR_INVALID_ARGUMENT, "ray or result buffer is null");
	if (((uintptr_t)rays & 15u) != 0) return fail(PHE_ERR_INVALID_ARGUMENT, "ray buffer must be 16-byte aligned");
	return PHE_OK;
}

} // namespace phe_gb300

using namespace phe_gb300;

extern "C" phe_status phe_cast_closest_plain(const phe_scene* scene, const phe_ray_in* rays, phe_ray_hit* hits, uint32_t n,
                                             void* stream)
{
	phe_status st = check_cast_args(scene, rays, hits);
	if (st) return st;
	if (((uintptr_t)hits & 15u) != 0) return fail(PHE_ERR_INVALID_ARGUMENT, "hit buffer must be 16-byte aligned");
	if (n == 0) return PHE_OK;
	uint32_t grid = (n + kPlainBlock - 1) / kPlainBlock;
	auto kernel = (scene->dev.nodes4 || scene->dev.nodes8) ? closest_plain_kernel<true> : closest_plain_kernel<false>;
	kernel<<<grid, kPlainBlock, stack_smem_bytes(kPlainBlock), (cudaStream_t)stream>>>(scene->dev, rays, hits, n,
	                                                                                   scene->status);
	PHE_CUDA_TRY(cudaGetLastError(), "closest_plain_kernel launch");
	return PHE_OK;
}

extern "C" phe_status phe_cast_closest(const phe_scene* scene, const phe_ray_in* rays, phe_ray_hit* hits, uint32_t n,
                                       void* stream)
{
	phe_status st = check_cast_args(scene, rays, hits);
	if (st) return st;
	if (((uintptr_t)hits & 15u) != 0) return fail(PHE_ERR_INVALID_ARGUMENT, "hit buffer must be 16-byte aligned");
	if (n == 0) return PHE_OK;
	if (n > kMaxPersistentRays) return fail(PHE_ERR_TOO_LARGE, "phe_cast_closest: at most %u rays per launch", kMaxPersistentRays);
	const bool wide = scene->dev.nodes4 || scene->dev.nodes8;
	auto kernel = wide ? closest_persistent_kernel<true> : closest_persistent_kernel<false>;
	int grid = 0;
	if ((st = persistent_grid(wide ? 2 : 0, (const void*)kernel, &grid))) return st;
	uint32_t maxGrid = (n + kPersistentBlock - 1) / kPersistentBlock;
	if ((uint32_t)grid > maxGrid) grid = (int)maxGrid;
	uint32_t* counter = nullptr;
	if ((st = acquire_counter((cudaStream_t)stream, &counter))) return st;
	kernel<<<grid, kPersistentBlock, stack_smem_bytes(kPersistentBlock), (cudaStream_t)stream>>>(scene->dev, rays, hits,
	                                                                                             n, counter,
	                                                                                             scene->status);
	PHE_CUDA_TRY(cudaGetLastError(), "closest_persistent_kernel launch");
	return PHE_OK;
}

extern "C" phe_status phe_cast_any(const phe_scene* scene, const phe_ray_in* rays, uint8_t* inLight, uint32_t n,
                                   const uint32_t* scatter, void* stream)
{
	phe_status st = check_cast_args(scene, rays, inLight);
	if (st) return st;
	if (n == 0) return PHE_OK;
	if (n > kMaxPersistentRays) return fail(PHE_ERR_TOO_LARGE, "phe_cast_any: at most %u rays per launch", kMaxPersistentRays);
	const bool wide = scene->dev.nodes4 || scene->dev.nodes8;
	auto kernel = wide ? any_persistent_kernel<true> : any_persistent_kernel<false>;
	int grid = 0;
	if ((st = persistent_grid(wide ? 3 : 1, (const void*)kernel, &grid))) return st;
	uint32_t maxGrid = (n + kPersistentBlock - 1) / kPersistentBlock;
	if ((uint32_t)grid > maxGrid) grid = (int)maxGrid;
	uint32_t* counter = nullptr;
	if ((st = acquire_counter((cudaStream_t)stream, &counter))) return st;
	kernel<<<grid, kPersistentBlock, stack_smem_bytes(kPersistentBlock), (cudaStream_t)stream>>>(scene->dev, rays,
	                                                                                             inLight, scatter, n,
	                                                                                             counter,
	                                                        scene->status);
	PHE_CUDA_TRY(cudaGetLastError(), "any_persistent_kernel launch");
	return PHE_OK;
}
