// Batched multi-scene launch shared by the batch object (batch.cu) and the serving loop (serve.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace phe_gb300 {

// One batch of a batched launch: rays [base, base + count) of the global index space (base is a
// multiple of 32), cast against scene `scene` of the scene table; kind 0 = closest (out is
// phe_ray_hit[count]), 1 = any (out is uint8_t[count]).
struct BatchItemDev {
	uint32_t scene, kind, count, base;
	const phe_ray_in* rays;
	void* out;
};
static_assert(sizeof(BatchItemDev) == 32, "BatchItemDev is 32 bytes");

// Launches the batched persistent kernel over `numItems` device-resident items covering
// `totalPadded` global ray indices. `counter` must be zero when the kernel starts (the caller
// clears it on `stream`). blockSize 64/128/256; blocksPerSM 0 = occupancy limit. `wide` must be set
// when some scene of the table has its 4-wide layout selected (DeviceScene::nodes4 non-null).
// Traversal errors go to each item's scene status word (DeviceScene::status).
phe_status launch_batch_table(const BatchItemDev* items, uint32_t numItems, uint32_t totalPadded,
                              const DeviceScene* scenes, uint32_t* counter, int blockSize, int blocksPerSM,
                              cudaStream_t stream, bool wide);

} // namespace phe_gb300
