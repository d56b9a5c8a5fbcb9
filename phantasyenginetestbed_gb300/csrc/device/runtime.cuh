// Per-device runtime state of the library: device properties, kernel occupancy and the pool of
// per-launch work counters used by the persistent kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../host/common.hpp"
#include "common.cuh"

struct phe_scene {
	phe_gb300::DeviceScene dev;         // dev.nodes4 / dev.nodes8 are set only while that layout is selected
	const float4* nodes4 = nullptr;     // 4-wide nodes, when the tree allows them (else null)
	const uint4* nodes8 = nullptr;      // 8-wide compressed nodes and their leaf records, when the tree
	const float4* leaves8 = nullptr;    // allows them (else null)
	uint32_t numNodes8 = 0, numLeaves8 = 0, maxDepth8 = 0;
	void* allocation = nullptr;   // one cudaMalloc holding nodes, 4-wide nodes, tris, datas, status
	void* shading = nullptr;      // one cudaMalloc holding materials, texture table, sRGB table, texels
	uint64_t bytes = 0, shadingBytes = 0;
	uint64_t generation = 0;      // bumped whenever `dev` changes (layout, materials): graphs re-capture
	int64_t maxMaterialIndex = -1; // largest materialIndex of the triangle data (-1 without data)
	uint32_t* status = nullptr;   // device word: OR of error bits raised by kernels on this scene
	uint32_t maxDepth = 0, maxDepth4 = 0;   // deepest leaf level of the binary and 4-wide trees
	int device = 0;               // ordinal of the device holding the scene
};

namespace phe_gb300 {

struct DeviceInfo {
	int device = -1;
	int numSMs = 0;
	int maxThreadsPerSM = 0;
	uint32_t* counterPool = nullptr; // kCounterPool words
};

constexpr uint32_t kCounterPool = 4096;
// Largest ray count of one persistent launch. Every resident warp fetches 32 rays past the end before
// it stops, so the 32-bit work counter needs headroom above the count (2^26 covers 2M resident warps).
constexpr uint32_t kMaxPersistentRays = PHE_MAX_PERSISTENT_RAYS;

// Returns the runtime state of the current device, initialising it on first use.
phe_status device_info(DeviceInfo** out);
// A zeroed work counter for one persistent launch on `stream` (a memset is queued on the stream).
phe_status acquire_counter(cudaStream_t stream, uint32_t** counter);

inline phe_status cuda_fail(cudaError_t e, const char* what)
{
	return fail(e == cudaErrorMemoryAllocation ? PHE_ERR_OUT_OF_MEMORY : PHE_ERR_CUDA, "%s: %s", what,
	            cudaGetErrorString(e));
}

#define PHE_CUDA_TRY(call, what)                                  \
	do {                                                          \
		cudaError_t e_ = (call);                                  \
		if (e_ != cudaSuccess) return ::phe_gb300::cuda_fail(e_, what); \
	} while (0)

// Set-up uploads (cudaMemcpy from pageable host memory, cudaMemset of device memory) run on the legacy
// default stream and may return before the bytes reach the device, and launches on streams created
// non-blocking are not ordered after that stream. Waiting for it makes such uploads complete before the
// call that made them returns, so the next launch on any stream reads them.
inline phe_status finish_uploads(const char* what)
{
	cudaError_t e = cudaStreamSynchronize(cudaStreamLegacy);
	return e == cudaSuccess ? PHE_OK : cuda_fail(e, what);
}

} // namespace phe_gb300
