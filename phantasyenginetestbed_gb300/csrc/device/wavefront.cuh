// Frame state shared by the wavefront kernels (wavefront.cu) and the renderer object (renderer.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

struct phe_scene;

namespace phe_gb300 {

constexpr uint32_t kMaxLights = 8;

// Counters in device memory, cleared at the start of every frame.
enum : uint32_t {
	kCtrShadow0 = 0,  // primary shadow-queue length
	kCtrBounce = 1,   // bounce-queue length
	kCtrShadow1 = 2,  // bounce shadow-queue length
	kCtrWork0 = 3,    // persistent work counters of the four traversal kernels
	kCtrWork1 = 4,
	kCtrWork2 = 5,
	kCtrWork3 = 6,
	kNumCounters = 8,
};

// Per-frame parameters, read by the kernels from device memory (so a captured graph replays
// with new values after one small copy).
struct FrameParamsDev {
	phe_camera_def cam;      // jitter is applied in ray generation
	float jitter[2];
	float camPos[3];
	uint32_t resX, resY, numPixels, numLights;
	uint32_t frame, parity;  // frame index (random streams) and history ping-pong side
	uint64_t seed;
	phe_sphere_light lights[kMaxLights];
	// Camera motion for TAA (velocity_gen.frag): the previous frame's camera (no jitter), this frame's
	// velocity output (null while the camera stands still: velocity 0 everywhere) and the previous
	// frame's velocity (null when it was 0 everywhere).
	phe_camera_def prevCam;
	float2* velocity;
	const float2* prevVelocity;
	// A frame split into `parts` parts (phe_renderer_set_frame_parts): this part covers the tile rows r
	// with r % parts == part, partPixels pixels; numPixels stays the whole frame (the stride of the
	// per-pixel buffers the parts share).
	uint32_t part, parts, partPixels, pad;
};

struct FrameBuffers {
	float4* contrib;          // [2][L][P] light contributions (primary lights, then bounce lights)
	uint8_t* inLight;         // [2][L][P] visibility of each contribution
	phe_ray_in* shadowRays;   // [2][L*P] compacted shadow queues
	uint32_t* shadowSlots;    // [2][L*P] visibility slot of each queued shadow ray
	phe_ray_in* bounceRays;   // [P] compacted bounce queue
	uint32_t* bouncePixel;    // [P]
	float4* bounceThroughput; // [P]
	float* roughness;         // [P] roughness at the primary hit (0 on a miss), read by TAA
	float4* rawColor;         // [P] resolved colour before TAA
	float4* history[2];       // [P] TAA history ping-pong (rgb + effective sample count)
	float4* color[2];         // [P] TAA output ping-pong (same side as the history it was blended into)
	uint32_t* counters;       // [kNumCounters]
	uint32_t capacityLP;      // L * P
	phe_ray_hit* primaryHits; // [P] closest hits of the primary rays, in 8x8-tile ray order
	phe_ray_hit* bounceHits;  // [P] closest hits of the bounce queue
	unsigned long long* rayTotals; // [4] rays cast per pass, summed over frames until reset
	uint32_t* bouncePerm;     // [P] bounce-queue order after binning by direction octant
	int refill;               // lane-refill threshold of the persistent traversal kernels
	int sortWindow;           // bounce rays are binned by direction octant within windows of this
	                          // many queue entries (0 = queue order)
};

// Allocates a renderer's frame buffers for up to `pixels` pixels and `lights` lights at once, so that
// later resolutions within that capacity reuse them (no allocation per request).
phe_status renderer_reserve(phe_renderer* r, uint64_t pixels, uint32_t lights);

// Resolves launch shapes (occupancy queries); call before capturing a frame into a graph.
phe_status prepare_frame();
// Kernels of one frame: primary trace, primary shade, primary any-hit, bounce binning, bounce trace,
// bounce shade, bounce any-hit, resolve + TAA (kFrameKernels); the fused pipeline has six (primary
// and bounce trace+shade fused), five with the merged shadow schedule. The binning kernel is launched
// only when sortWindow > 0, so the frame has one kernel less without binning.
constexpr int kFrameKernels = 8;
constexpr int kFusedFrameKernels = 6;
inline int frame_kernels(bool fused, int schedule, int sortWindow)
{
	int k = fused ? (schedule == PHE_SHADOWS_MERGED ? kFusedFrameKernels - 1 : kFusedFrameKernels) : kFrameKernels;
	return sortWindow > 0 ? k : k - 1;
}
// `events` (optional, kernels + 1 entries) are recorded on `stream` around each kernel. `fused`
// selects the pipeline with traversal and shading in one kernel; `schedule` (PHE_SHADOWS_*) the
// placement of its shadow passes. BESIDE_BOUNCE needs `streams` (a second stream and fork/join
// events) and runs in order while `events` are recorded.
struct FrameStreams {
	cudaStream_t side = nullptr;
	cudaEvent_t fork = nullptr, join = nullptr;
};
// `parts` selects the traversal kernels (counter reset, primary, bounce, shadow passes), the resolve +
// TAA kernel, or both: a renderer with two frames in flight launches them on different streams.
enum { kFrameTraversal = 1, kFrameResolve = 2, kFrameAll = 3 };
// `partPixels` (0 = the whole frame) sizes the grids of one part of a split frame.
phe_status launch_frame(const phe_scene* scene, const FrameParamsDev* dParams, const FrameBuffers& fb, uint32_t resX,
                        uint32_t resY, cudaStream_t stream, cudaEvent_t* events, bool fused, int schedule,
                        const FrameStreams* streams, int parts = kFrameAll, uint32_t partPixels = 0);

} // namespace phe_gb300
