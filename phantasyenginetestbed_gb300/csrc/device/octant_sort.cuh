// Stable counting sort of a window of rays by direction octant (the sign bits of dir.xyz), done by one
// block of kOctantBlock threads: thread t handles the entries [t * per, (t + 1) * per) of the window.
// Used to group rays of similar direction before tracing them (the bounce queue of a frame, the rays
// of a batch). Deterministic: equal keys keep their window order.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace phe_gb300 {

constexpr int kOctantBlock = 256;
constexpr int kMaxOctantWindow = 4096;   // entries per window: a multiple of kOctantBlock up to this

__device__ __forceinline__ uint8_t octant_key(float4 dir)
{
	return (uint8_t)((dir.x < 0.0f ? 1 : 0) | (dir.y < 0.0f ? 2 : 0) | (dir.z < 0.0f ? 4 : 0));
}

// keys[k] (0xFF = no entry) of this thread's `per` entries in; rank[8] out: this thread's first output
// position for each key. Every thread of the block calls it (it synchronises the block).
__device__ __forceinline__ void octant_ranks(const uint8_t* keys, int per, uint32_t (&cnt)[8][kOctantBlock],
                                             uint32_t (&bucketBase)[8], uint32_t rank[8])
{
	const int t = threadIdx.x;
	uint32_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	for (int k = 0; k < per; k++)
		if (keys[k] != 0xFF) c[keys[k]]++;
	for (int b = 0; b < 8; b++) cnt[b][t] = c[b];
	__syncthreads();
	// Exclusive scan of each bucket's per-thread counts: warp b scans bucket b (8 warps).
	const int warp = t >> 5, lane = t & 31;
	if (warp < 8) {
		uint32_t local[kOctantBlock / 32];
		uint32_t sum = 0;
		for (int j = 0; j < kOctantBlock / 32; j++) {
			local[j] = sum;
			sum += cnt[warp][lane * (kOctantBlock / 32) + j];
		}
		uint32_t incl = sum;
		for (int o = 1; o < 32; o <<= 1) {
			uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
			if (lane >= o) incl += v;
		}
		uint32_t excl = incl - sum;
		for (int j = 0; j < kOctantBlock / 32; j++) cnt[warp][lane * (kOctantBlock / 32) + j] = excl + local[j];
		if (lane == 31) bucketBase[warp] = incl;   // bucket total for now
	}
	__syncthreads();
	if (t == 0) {
		uint32_t acc = 0;
		for (int b = 0; b < 8; b++) {
			uint32_t tot = bucketBase[b];
			bucketBase[b] = acc;
			acc += tot;
		}
	}
	__syncthreads();
	for (int b = 0; b < 8; b++) rank[b] = bucketBase[b] + cnt[b][t];
	__syncthreads();   // cnt and bucketBase may be reused by the caller's next window
}

} // namespace phe_gb300
