// The renderer object behind the C ABI: the headless counterpart of CudaTracerRenderer
// (cuda_ray_tracer/CudaTracerRenderer.{hpp,cpp}) and the BaseRenderer entry points it implements
// (phantasy_engine/rendering/BaseRenderer.hpp:56-90): setStaticScene, setTargetResolution,
// updateCamera, render. RenderResult's GL textures become device pointers.
//
// Buffers are (re)allocated in set_target_resolution, as targetResolutionUpdated does
// (CudaTracerRenderer.cpp:735-793). A frame is either launched directly or replayed from a CUDA
// graph captured on first use; per-frame values travel in one small parameter copy.

#include <cmath>
#include <cstring>

#include "runtime.cuh"
#include "wavefront.cuh"

using namespace phe_gb300;

struct phe_renderer {
	const phe_scene* scene = nullptr;
	uint32_t resX = 0, resY = 0, numLights = 0;
	FrameBuffers fb{};
	void* allocation = nullptr;
	FrameParamsDev* dParams = nullptr;
	FrameParamsDev* hParams = nullptr;   // pinned staging ring of kParamSlots
	cudaEvent_t paramEvents[8] = {};     // last copy out of each staging slot
	uint32_t paramSlot = 0;
	size_t capacityP = 0, capacityL = 0; // frame buffers are kept while a resolution fits
	phe_camera_def cam{};
	float camPos[3] = {0, 0, 0};
	float jitter[2] = {0, 0};
	uint64_t seed = 1;
	uint32_t frame = 0;
	uint32_t parity = 0;
	int useGraph = 0;
	cudaGraphExec_t graphExec = nullptr;
	uint64_t graphGeneration = 0;          // scene generation the graph was captured with
	cudaStream_t graphStream = nullptr;  // stream the graph was captured for (graphs relaunch on any stream)
	bool cameraSet = false;
	bool fused = true;                     // traversal and shading fused in one kernel per bounce
	int refill = 28;                       // lane-refill threshold of the persistent traversal kernels
	int sortWindow = 0;                    // bounce-ray binning window (0 = off)
	bool timing = false;                   // record events around each kernel (direct launches only)
	cudaEvent_t events[kFrameKernels + 1] = {};
	double kernelMs[kFrameKernels] = {};   // accumulated since timing was enabled
	int timedKernels = 0;
	uint32_t timedFrames = 0;
	bool pendingTimes = false;
	FrameStreams streams;                  // second stream for PHE_SHADOWS_BESIDE_BOUNCE
	int shadowSchedule = PHE_SHADOWS_MERGED;
	// Asynchronous read-back: two device staging slots copied to the host on copyStream.
	// Camera motion (TAA velocity): the last rendered camera and which velocity sides are all zero.
	phe_camera_def prevCam{};
	bool hasPrevCam = false;
	bool velocityZero[2] = {true, true};
	cudaStream_t copyStream = nullptr;
	void* staging[2] = {nullptr, nullptr};
	size_t stagingBytes = 0;
	cudaEvent_t snapEvents[2] = {}, doneEvents[2] = {};
	bool readPending[2] = {false, false};
	uint32_t readSlot = 0;
	// Results kept per side of the frame parity (TAA colour, history, velocity) are copied out directly:
	// sideDone[s] follows the last copy from side s, and the next frame that writes side s (the one
	// after next) waits for it (sideGuard[s]).
	cudaEvent_t readyEvent = nullptr;
	cudaEvent_t sideDone[2] = {};
	bool sideGuard[2] = {false, false};
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
static const uint32_t kParamSlots = 8;

static void free_buffers(phe_renderer* r)
{
	// in-place read-backs may still be copying out of these buffers
	for (int i = 0; i < 2; i++) {
		if (r->sideDone[i]) cudaEventSynchronize(r->sideDone[i]);
		r->sideGuard[i] = false;
	}
	if (r->graphExec) cudaGraphExecDestroy(r->graphExec);
	r->graphExec = nullptr;
	if (r->allocation) cudaFree(r->allocation);
	r->allocation = nullptr;
	std::memset(&r->fb, 0, sizeof(r->fb));
	r->capacityP = r->capacityL = 0;
}

static phe_status allocate(phe_renderer* r, uint32_t resX, uint32_t resY, uint32_t numLights)
{
	const size_t P = (size_t)resX * resY;
	const size_t L = numLights ? numLights : 1;
	if (resX != r->resX || resY != r->resY) {   // velocities of another resolution do not carry over
		r->hasPrevCam = false;
		r->velocityZero[0] = r->velocityZero[1] = true;
	}
	if (r->allocation && P <= r->capacityP && L <= r->capacityL) {
		// Keep the buffers: every stride is computed from the current resolution at launch time. A
		// captured graph holds launch shapes for the old resolution, so it is rebuilt.
		if ((resX != r->resX || resY != r->resY) && r->graphExec) {
			cudaGraphExecDestroy(r->graphExec);
			r->graphExec = nullptr;
		}
		r->resX = resX;
		r->resY = resY;
		r->numLights = (uint32_t)L;
		return PHE_OK;
	}
	free_buffers(r);
	const size_t LP = P * L;
	size_t sizes[] = {
		2 * LP * sizeof(float4),      // contrib
		2 * LP,                       // inLight
		2 * LP * sizeof(phe_ray_in),  // shadowRays
		2 * LP * sizeof(uint32_t),    // shadowSlots
		P * sizeof(phe_ray_in),       // bounceRays
		P * sizeof(uint32_t),         // bouncePixel
		P * sizeof(float4),           // bounceThroughput
		P * sizeof(float),            // roughness
		P * sizeof(float4),           // rawColor
		P * sizeof(float4),           // history[0]
		P * sizeof(float4),           // history[1]
		P * sizeof(float4),           // color[0]
		kNumCounters * sizeof(uint32_t),
		P * sizeof(phe_ray_hit),      // primaryHits
		P * sizeof(phe_ray_hit),      // bounceHits
		4 * sizeof(unsigned long long), // rayTotals
		P * sizeof(uint32_t),         // bouncePerm
		P * sizeof(float2),           // velocity[0]
		P * sizeof(float2),           // velocity[1]
		P * sizeof(float4),           // color[1]
	};
	size_t total = 0;
	for (size_t s : sizes) total += align256(s);
	char* base = nullptr;
	cudaError_t e = cudaMalloc(&base, total);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(frame buffers)");
	char* p = base;
	auto take = [&](size_t i) { char* q = p; p += align256(sizes[i]); return q; };
	FrameBuffers& fb = r->fb;
	fb.contrib = (float4*)take(0);
	fb.inLight = (uint8_t*)take(1);
	fb.shadowRays = (phe_ray_in*)take(2);
	fb.shadowSlots = (uint32_t*)take(3);
	fb.bounceRays = (phe_ray_in*)take(4);
	fb.bouncePixel = (uint32_t*)take(5);
	fb.bounceThroughput = (float4*)take(6);
	fb.roughness = (float*)take(7);
	fb.rawColor = (float4*)take(8);
	fb.history[0] = (float4*)take(9);
	fb.history[1] = (float4*)take(10);
	fb.color[0] = (float4*)take(11);
	fb.counters = (uint32_t*)take(12);
	fb.primaryHits = (phe_ray_hit*)take(13);
	fb.bounceHits = (phe_ray_hit*)take(14);
	fb.rayTotals = (unsigned long long*)take(15);
	fb.bouncePerm = (uint32_t*)take(16);
	fb.velocity[0] = (float2*)take(17);
	fb.velocity[1] = (float2*)take(18);
	fb.color[1] = (float4*)take(19);
	fb.sortWindow = r->sortWindow;
	fb.capacityLP = (uint32_t)LP;
	fb.refill = r->refill;
	r->capacityP = P;
	r->capacityL = L;
	r->allocation = base;
	r->resX = resX;
	r->resY = resY;
	r->numLights = numLights;
	if ((e = cudaMemset(base, 0, total)) != cudaSuccess) return cuda_fail(e, "clear frame buffers");
	r->parity = 0;
	return PHE_OK;
}

// Adds the elapsed times of the last timed frame (waits for its last event).
static phe_status collect_times(phe_renderer* r)
{
	if (!r->pendingTimes) return PHE_OK;
	PHE_CUDA_TRY(cudaEventSynchronize(r->events[r->timedKernels]), "wait for timed frame");
	for (int i = 0; i < r->timedKernels; i++) {
		float ms = 0.0f;
		PHE_CUDA_TRY(cudaEventElapsedTime(&ms, r->events[i], r->events[i + 1]), "kernel time");
		r->kernelMs[i] += ms;
	}
	r->timedFrames++;
	r->pendingTimes = false;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_kernel_timing(phe_renderer* r, int enable)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_kernel_timing: null renderer");
	if (enable && !r->events[0])
		for (int i = 0; i <= kFrameKernels; i++) PHE_CUDA_TRY(cudaEventCreate(&r->events[i]), "cudaEventCreate");
	r->timing = enable != 0;
	r->pendingTimes = false;
	r->timedFrames = 0;
	for (int i = 0; i < kFrameKernels; i++) r->kernelMs[i] = 0.0;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_kernel_times(phe_renderer* r, double msTotal[8], uint32_t* numKernels, uint32_t* frames)
{
	if (!r || !msTotal || !frames || !numKernels)
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_kernel_times: null argument");
	phe_status st = collect_times(r);
	if (st) return st;
	for (int i = 0; i < 8; i++) msTotal[i] = i < kFrameKernels ? r->kernelMs[i] : 0.0;
	*numKernels = (uint32_t)frame_kernels(r->fused, r->shadowSchedule, r->sortWindow);
	*frames = r->timedFrames;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_pipeline(phe_renderer* r, int fused, int refill, int sortWindow)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_pipeline: null renderer");
	if (refill < 0 || refill > 32) return fail(PHE_ERR_INVALID_ARGUMENT, "refill threshold must be in [0, 32]");
	if (sortWindow != 0 && (sortWindow < 256 || sortWindow > 4096 || sortWindow % 256))
		return fail(PHE_ERR_INVALID_ARGUMENT, "sort window must be 0 or a multiple of 256 in [256, 4096]");
	r->fused = fused != 0;
	r->refill = refill;
	r->fb.refill = refill;
	r->sortWindow = sortWindow;
	r->fb.sortWindow = sortWindow;
	if (r->graphExec) {
		cudaGraphExecDestroy(r->graphExec);
		r->graphExec = nullptr;
	}
	r->pendingTimes = false;
	r->timedFrames = 0;
	for (int i = 0; i < kFrameKernels; i++) r->kernelMs[i] = 0.0;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_shadow_schedule(phe_renderer* r, int schedule)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_shadow_schedule: null renderer");
	if (schedule != PHE_SHADOWS_IN_ORDER && schedule != PHE_SHADOWS_BESIDE_BOUNCE && schedule != PHE_SHADOWS_MERGED)
		return fail(PHE_ERR_INVALID_ARGUMENT, "unknown shadow schedule %d", schedule);
	if (schedule != r->shadowSchedule && r->graphExec) {
		cudaGraphExecDestroy(r->graphExec);
		r->graphExec = nullptr;
	}
	r->shadowSchedule = schedule;
	r->pendingTimes = false;
	r->timedFrames = 0;
	for (int i = 0; i < kFrameKernels; i++) r->kernelMs[i] = 0.0;
	return PHE_OK;
}

namespace phe_gb300 {
phe_status renderer_reserve(phe_renderer* r, uint64_t pixels, uint32_t lights)
{
	if (!r || pixels == 0) return fail(PHE_ERR_INVALID_ARGUMENT, "renderer_reserve: bad arguments");
	if (pixels * kMaxLights * 2 >= 0xFFFFFFFFull) return fail(PHE_ERR_TOO_LARGE, "renderer_reserve: too many pixels");
	if (r->allocation && pixels <= r->capacityP && lights <= r->capacityL) return PHE_OK;
	// A 8-pixel-wide frame of the requested size: allocate() only uses the pixel and light counts.
	uint32_t resY = (uint32_t)((pixels + 7) / 8);
	phe_status st = allocate(r, 8, resY, lights);
	if (st) return st;
	r->resX = r->resY = 0;   // no target resolution chosen yet
	return PHE_OK;
}
} // namespace phe_gb300

extern "C" phe_status phe_renderer_create(phe_renderer** out)
{
	if (!out) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_create: out is null");
	*out = nullptr;
	DeviceInfo* d = nullptr;
	phe_status st = device_info(&d);
	if (st) return st;
	phe_renderer* r = new phe_renderer();
	cudaError_t e = cudaMalloc(&r->dParams, sizeof(FrameParamsDev));
	if (e == cudaSuccess) e = cudaMallocHost(&r->hParams, sizeof(FrameParamsDev) * kParamSlots);
	for (uint32_t i = 0; i < kParamSlots && e == cudaSuccess; i++)
		e = cudaEventCreateWithFlags(&r->paramEvents[i], cudaEventDisableTiming);
	if (e != cudaSuccess) {
		if (r->dParams) cudaFree(r->dParams);
		if (r->hParams) cudaFreeHost(r->hParams);
		delete r;
		return cuda_fail(e, "allocate frame parameters");
	}
	std::memset(r->hParams, 0, sizeof(FrameParamsDev) * kParamSlots);
	if (cudaStreamCreateWithFlags(&r->streams.side, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaEventCreateWithFlags(&r->streams.fork, cudaEventDisableTiming) != cudaSuccess ||
	    cudaEventCreateWithFlags(&r->streams.join, cudaEventDisableTiming) != cudaSuccess) {
		cudaError_t e2 = cudaGetLastError();
		phe_renderer_destroy(r);
		return cuda_fail(e2, "create renderer streams");
	}
	*out = r;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_destroy(phe_renderer* r)
{
	if (!r) return PHE_OK;
	cudaDeviceSynchronize();
	free_buffers(r);   // first: it waits on the read-back events destroyed below
	for (int i = 0; i <= kFrameKernels; i++)
		if (r->events[i]) cudaEventDestroy(r->events[i]);
	for (uint32_t i = 0; i < kParamSlots; i++)
		if (r->paramEvents[i]) cudaEventDestroy(r->paramEvents[i]);
	for (int i = 0; i < 2; i++) {
		if (r->staging[i]) cudaFree(r->staging[i]);
		if (r->snapEvents[i]) cudaEventDestroy(r->snapEvents[i]);
		if (r->doneEvents[i]) cudaEventDestroy(r->doneEvents[i]);
		if (r->sideDone[i]) cudaEventDestroy(r->sideDone[i]);
		r->sideDone[i] = nullptr;
	}
	if (r->readyEvent) cudaEventDestroy(r->readyEvent);
	if (r->copyStream) cudaStreamDestroy(r->copyStream);
	if (r->streams.side) cudaStreamDestroy(r->streams.side);
	if (r->streams.fork) cudaEventDestroy(r->streams.fork);
	if (r->streams.join) cudaEventDestroy(r->streams.join);
	cudaFree(r->dParams);
	cudaFreeHost(r->hParams);
	delete r;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_static_scene(phe_renderer* r, const phe_scene* scene)
{
	if (!r || !scene) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_static_scene: null argument");
	if (!scene->dev.datas)
		return fail(PHE_ERR_INVALID_SCENE, "rendering needs a scene created with triangle data");
	r->scene = scene;
	if (r->graphExec) cudaGraphExecDestroy(r->graphExec);
	r->graphExec = nullptr;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_target_resolution(phe_renderer* r, uint32_t resX, uint32_t resY)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_target_resolution: null renderer");
	if (resX == 0 || resY == 0 || (resX % 8u) || (resY % 8u))
		return fail(PHE_ERR_INVALID_ARGUMENT, "target resolution must be a non-zero multiple of 8 (CudaTracerRenderer.cpp:470-471)");
	if ((uint64_t)resX * resY * kMaxLights * 2 >= 0xFFFFFFFFull)
		return fail(PHE_ERR_TOO_LARGE, "target resolution too large");
	return allocate(r, resX, resY, r->numLights ? r->numLights : 1);
}

extern "C" phe_status phe_renderer_update_camera(phe_renderer* r, const float pos[3], const float dir[3], const float up[3],
                                                 float vertFovDeg, float pixelOffsetX, float pixelOffsetY)
{
	if (!r || !pos || !dir || !up) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_update_camera: null argument");
	if (!r->resX) return fail(PHE_ERR_INVALID_ARGUMENT, "set the target resolution before the camera");
	phe_generate_camera_def(pos, dir, up, vertFovDeg * 0.017453292519943295f, (float)r->resX, (float)r->resY, &r->cam);
	std::memcpy(r->camPos, pos, sizeof(r->camPos));
	r->jitter[0] = pixelOffsetX;
	r->jitter[1] = pixelOffsetY;
	r->cameraSet = true;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_camera_def(phe_renderer* r, const phe_camera_def* cam, const float camPos[3],
                                                  float pixelOffsetX, float pixelOffsetY)
{
	if (!r || !cam || !camPos) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_camera_def: null argument");
	r->cam = *cam;
	std::memcpy(r->camPos, camPos, sizeof(r->camPos));
	r->jitter[0] = pixelOffsetX;
	r->jitter[1] = pixelOffsetY;
	r->cameraSet = true;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_seed(phe_renderer* r, uint64_t seed, uint32_t frame)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_seed: null renderer");
	r->seed = seed;
	r->frame = frame;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_graph(phe_renderer* r, int enable)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_graph: null renderer");
	r->useGraph = enable ? 1 : 0;
	if (!enable && r->graphExec) {
		cudaGraphExecDestroy(r->graphExec);
		r->graphExec = nullptr;
	}
	return PHE_OK;
}

// Orders work on `s` that rewrites side `side` of the parity buffers after the asynchronous copies
// still reading it.
static phe_status guard_side(phe_renderer* r, uint32_t side, cudaStream_t s)
{
	if (!r->sideGuard[side]) return PHE_OK;
	PHE_CUDA_TRY(cudaStreamWaitEvent(s, r->sideDone[side], 0), "wait for read-back of the side");
	r->sideGuard[side] = false;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_reset_taa(phe_renderer* r, void* stream)
{
	if (!r || !r->allocation) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_reset_taa: no frame buffers");
	size_t P = (size_t)r->resX * r->resY;
	for (uint32_t side = 0; side < 2; side++) {
		phe_status st = guard_side(r, side, (cudaStream_t)stream);
		if (st) return st;
	}
	PHE_CUDA_TRY(cudaMemsetAsync(r->fb.history[0], 0, P * sizeof(float4), (cudaStream_t)stream), "reset TAA");
	PHE_CUDA_TRY(cudaMemsetAsync(r->fb.history[1], 0, P * sizeof(float4), (cudaStream_t)stream), "reset TAA");
	r->hasPrevCam = false;
	r->velocityZero[0] = r->velocityZero[1] = true;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_reset_ray_totals(phe_renderer* r, void* stream)
{
	if (!r || !r->allocation) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_reset_ray_totals: no frame buffers");
	PHE_CUDA_TRY(cudaMemsetAsync(r->fb.rayTotals, 0, 4 * sizeof(unsigned long long), (cudaStream_t)stream),
	             "reset ray totals");
	return PHE_OK;
}

extern "C" phe_status phe_renderer_ray_totals_async(const phe_renderer* r, uint64_t* hostTotals4, void* stream)
{
	if (!r || !r->allocation || !hostTotals4) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_ray_totals_async: no frame");
	PHE_CUDA_TRY(cudaMemcpyAsync(hostTotals4, r->fb.rayTotals, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost,
	                             (cudaStream_t)stream), "read ray totals");
	return PHE_OK;
}

extern "C" phe_status phe_renderer_render(phe_renderer* r, const phe_sphere_light* lights, uint32_t numLights, void* stream)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_render: null renderer");
	if (!r->scene) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_render: no static scene");
	if (!r->resX) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_render: no target resolution");
	if (!r->cameraSet) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_render: no camera");
	NvtxRange range("phe_renderer_render");
	if (!r->scene->dev.materials)
		return fail(PHE_ERR_INVALID_SCENE, "phe_renderer_render: the scene has no materials");
	if (numLights > kMaxLights) return fail(PHE_ERR_TOO_LARGE, "at most %u lights", kMaxLights);
	if (numLights && !lights) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_render: lights is null");
	cudaStream_t s = (cudaStream_t)stream;
	uint32_t L = numLights ? numLights : 1;
	if (L != r->numLights) {
		// Contribution and queue buffers scale with the light count.
		cudaStreamSynchronize(s);
		phe_status st = allocate(r, r->resX, r->resY, L);
		if (st) return st;
	}
	// Pinned staging ring: a slot is rewritten only after its previous copy has been consumed.
	uint32_t slot = r->paramSlot;
	r->paramSlot = (slot + 1) % kParamSlots;
	PHE_CUDA_TRY(cudaEventSynchronize(r->paramEvents[slot]), "wait for a free parameter slot");
	FrameParamsDev& fp = r->hParams[slot];
	// Camera motion: this frame writes the velocity on the side of its output history, the previous
	// frame's velocity is on the other side; a camera equal to the previous one has velocity 0.
	const uint32_t outSide = r->parity ^ 1u, inSide = r->parity;
	const bool moving = r->hasPrevCam && std::memcmp(&r->prevCam, &r->cam, sizeof(phe_camera_def)) != 0;
	fp.prevCam = r->hasPrevCam ? r->prevCam : r->cam;
	fp.velocity = moving ? r->fb.velocity[outSide] : nullptr;
	fp.prevVelocity = r->velocityZero[inSide] ? nullptr : r->fb.velocity[inSide];
	fp.cam = r->cam;
	fp.jitter[0] = r->jitter[0];
	fp.jitter[1] = r->jitter[1];
	std::memcpy(fp.camPos, r->camPos, sizeof(fp.camPos));
	fp.resX = r->resX;
	fp.resY = r->resY;
	fp.numPixels = r->resX * r->resY;
	fp.numLights = numLights;
	fp.frame = r->frame;
	fp.parity = r->parity;
	fp.seed = r->seed;
	std::memset(fp.lights, 0, sizeof(fp.lights));
	if (numLights) std::memcpy(fp.lights, lights, sizeof(phe_sphere_light) * numLights);
	{
		phe_status gst = guard_side(r, outSide, s);   // this frame rewrites side outSide
		if (gst) return gst;
	}
	PHE_CUDA_TRY(cudaMemcpyAsync(r->dParams, &fp, sizeof(FrameParamsDev), cudaMemcpyHostToDevice, s),
	             "upload frame parameters");
	PHE_CUDA_TRY(cudaEventRecord(r->paramEvents[slot], s), "record parameter slot");
	if (r->useGraph) {
		if (r->graphExec && r->graphGeneration != r->scene->generation) {   // scene arrays or layout changed
			cudaGraphExecDestroy(r->graphExec);
			r->graphExec = nullptr;
		}
		if (!r->graphExec) {
			phe_status pst = prepare_frame();
			if (pst) return pst;
			cudaStream_t cap = nullptr;
			PHE_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "create capture stream");
			cudaGraph_t g = nullptr;
			cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
			phe_status st = PHE_OK;
			if (e == cudaSuccess) {
				st = launch_frame(r->scene, r->dParams, r->fb, r->resX, r->resY, cap, nullptr, r->fused,
				                  r->shadowSchedule, &r->streams);
				e = cudaStreamEndCapture(cap, &g);
			}
			cudaStreamDestroy(cap);
			if (st) { if (g) cudaGraphDestroy(g); return st; }
			if (e != cudaSuccess) return cuda_fail(e, "capture frame graph");
			e = cudaGraphInstantiate(&r->graphExec, g, 0);
			cudaGraphDestroy(g);
			if (e != cudaSuccess) return cuda_fail(e, "instantiate frame graph");
			r->graphGeneration = r->scene->generation;
		}
		PHE_CUDA_TRY(cudaGraphLaunch(r->graphExec, s), "launch frame graph");
	} else {
		phe_status st;
		if (r->timing) {
			if ((st = collect_times(r))) return st;
			r->timedKernels = frame_kernels(r->fused, r->shadowSchedule, r->sortWindow);
			st = launch_frame(r->scene, r->dParams, r->fb, r->resX, r->resY, s, r->events, r->fused, r->shadowSchedule,
			                  nullptr);
			r->pendingTimes = true;
		} else {
			st = launch_frame(r->scene, r->dParams, r->fb, r->resX, r->resY, s, nullptr, r->fused,
			                  r->shadowSchedule, &r->streams);
		}
		if (st) return st;
	}
	r->velocityZero[outSide] = !moving;
	r->prevCam = r->cam;
	r->hasPrevCam = true;
	r->frame++;
	r->parity ^= 1u;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_result(const phe_renderer* r, phe_render_result* out)
{
	if (!r || !out) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_result: null argument");
	out->resX = r->resX;
	out->resY = r->resY;
	out->color = (const float*)r->fb.color[r->parity];   // written by the last frame
	out->history = (const float*)r->fb.history[r->parity];   // written by the last frame
	out->rawColor = (const float*)r->fb.rawColor;
	out->roughness = r->fb.roughness;
	out->velocity = r->velocityZero[r->parity] ? nullptr : (const float*)r->fb.velocity[r->parity];
	return PHE_OK;
}

extern "C" phe_status phe_renderer_ray_counts(const phe_renderer* r, uint64_t counts[4], void* stream)
{
	if (!r || !counts || !r->fb.counters) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_ray_counts: no frame");
	uint32_t c[kNumCounters];
	PHE_CUDA_TRY(cudaMemcpyAsync(c, r->fb.counters, sizeof(c), cudaMemcpyDeviceToHost, (cudaStream_t)stream), "read counters");
	PHE_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream), "read counters");
	counts[0] = (uint64_t)r->resX * r->resY;
	counts[1] = c[kCtrShadow0];
	counts[2] = c[kCtrBounce];
	counts[3] = c[kCtrShadow1];
	return PHE_OK;
}

static phe_status read_source(const phe_renderer* r, int which, const void** src, size_t* bytes)
{
	size_t P = (size_t)r->resX * r->resY;
	*bytes = P * sizeof(float4);
	switch (which) {
	case 0: *src = r->fb.color[r->parity]; break;
	case 1: *src = r->fb.history[r->parity]; break;
	case 2: *src = r->fb.rawColor; break;
	case 3: *src = r->fb.roughness; *bytes = P * sizeof(float); break;
	case 4: *src = r->velocityZero[r->parity] ? nullptr : r->fb.velocity[r->parity]; *bytes = P * sizeof(float2); break;
	default: return fail(PHE_ERR_INVALID_ARGUMENT, "renderer read: which must be 0..4");
	}
	return PHE_OK;
}

extern "C" phe_status phe_renderer_read(const phe_renderer* r, int which, void* hostDst, void* stream)
{
	if (!r || !hostDst || !r->allocation) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_read: no frame");
	const void* src = nullptr;
	size_t bytes = 0;
	phe_status st = read_source(r, which, &src, &bytes);
	if (st) return st;
	if (!src) {   // a velocity that is 0 everywhere is not stored
		PHE_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream), "read result");
		std::memset(hostDst, 0, bytes);
		return PHE_OK;
	}
	PHE_CUDA_TRY(cudaMemcpyAsync(hostDst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream), "read result");
	PHE_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream), "read result");
	return PHE_OK;
}

extern "C" phe_status phe_renderer_read_async(phe_renderer* r, int which, void* hostDst, void* stream)
{
	if (!r || !hostDst || !r->allocation) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_read_async: no frame");
	const void* src = nullptr;
	size_t bytes = 0;
	phe_status st = read_source(r, which, &src, &bytes);
	if (st) return st;
	cudaStream_t s = (cudaStream_t)stream;
	if (!r->copyStream) {
		PHE_CUDA_TRY(cudaStreamCreateWithFlags(&r->copyStream, cudaStreamNonBlocking), "create copy stream");
		for (int i = 0; i < 2; i++) {
			PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->snapEvents[i], cudaEventDisableTiming), "create read event");
			PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->doneEvents[i], cudaEventDisableTiming), "create read event");
			PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->sideDone[i], cudaEventDisableTiming), "create read event");
		}
		PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->readyEvent, cudaEventDisableTiming), "create read event");
	}
	// TAA colour, history and a stored velocity live on the side the last frame wrote; the next frame
	// only reads that side, so the copy reads it in place and the frame after next waits for the copy.
	if (src && (which == 0 || which == 1 || which == 4)) {
		const uint32_t side = r->parity;
		PHE_CUDA_TRY(cudaEventRecord(r->readyEvent, s), "record frame end");
		PHE_CUDA_TRY(cudaStreamWaitEvent(r->copyStream, r->readyEvent, 0), "order read-back");
		PHE_CUDA_TRY(cudaMemcpyAsync(hostDst, src, bytes, cudaMemcpyDeviceToHost, r->copyStream), "read result");
		PHE_CUDA_TRY(cudaEventRecord(r->sideDone[side], r->copyStream), "record read-back");
		r->sideGuard[side] = true;
		return PHE_OK;
	}
	if (bytes > r->stagingBytes) {   // grow both slots once no copy uses them
		if ((st = phe_renderer_read_wait(r))) return st;
		for (int i = 0; i < 2; i++) {
			if (r->staging[i]) cudaFree(r->staging[i]);
			r->staging[i] = nullptr;
		}
		r->stagingBytes = 0;
		for (int i = 0; i < 2; i++) PHE_CUDA_TRY(cudaMalloc(&r->staging[i], bytes), "allocate read-back staging");
		r->stagingBytes = bytes;
	}
	const uint32_t k = r->readSlot;
	r->readSlot ^= 1u;
	if (r->readPending[k]) PHE_CUDA_TRY(cudaStreamWaitEvent(s, r->doneEvents[k], 0), "wait for staging slot");
	if (src) PHE_CUDA_TRY(cudaMemcpyAsync(r->staging[k], src, bytes, cudaMemcpyDeviceToDevice, s), "snapshot result");
	else PHE_CUDA_TRY(cudaMemsetAsync(r->staging[k], 0, bytes, s), "snapshot zero velocity");
	PHE_CUDA_TRY(cudaEventRecord(r->snapEvents[k], s), "record snapshot");
	PHE_CUDA_TRY(cudaStreamWaitEvent(r->copyStream, r->snapEvents[k], 0), "order read-back");
	PHE_CUDA_TRY(cudaMemcpyAsync(hostDst, r->staging[k], bytes, cudaMemcpyDeviceToHost, r->copyStream), "read result");
	PHE_CUDA_TRY(cudaEventRecord(r->doneEvents[k], r->copyStream), "record read-back");
	r->readPending[k] = true;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_read_wait(phe_renderer* r)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_read_wait: null renderer");
	for (int i = 0; i < 2; i++)
		if (r->readPending[i]) {
			PHE_CUDA_TRY(cudaEventSynchronize(r->doneEvents[i]), "wait for read-back");
			r->readPending[i] = false;
		}
	for (int i = 0; i < 2; i++)   // an event never recorded counts as complete
		if (r->sideDone[i]) PHE_CUDA_TRY(cudaEventSynchronize(r->sideDone[i]), "wait for read-back");
	return PHE_OK;
}

extern "C" uint32_t phe_renderer_frame_param_bytes(void) { return (uint32_t)sizeof(FrameParamsDev); }
