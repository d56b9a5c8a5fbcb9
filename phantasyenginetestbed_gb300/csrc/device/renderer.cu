// The renderer object behind the C ABI: the headless counterpart of CudaTracerRenderer
// (cuda_ray_tracer/CudaTracerRenderer.{hpp,cpp}) and the BaseRenderer entry points it implements
// (phantasy_engine/rendering/BaseRenderer.hpp:56-90): setStaticScene, setTargetResolution,
// updateCamera, render. RenderResult's GL textures become device pointers.
//
// Buffers are (re)allocated in set_target_resolution, as targetResolutionUpdated does
// (CudaTracerRenderer.cpp:735-793). A frame is either launched directly or replayed from a CUDA
// graph captured on first use; per-frame values travel in one small parameter copy.
//
// Two frames in flight (phe_renderer_set_frames_in_flight): frame k's traversal kernels run on the
// renderer's traversal stream k % 2 with their own per-frame buffers (slot k % 2: queues,
// contributions, visibility, roughness, counters, parameters), after the caller's work enqueued before
// the call and after the resolve that last read that slot; its resolve + TAA runs on the renderer's
// resolve stream, after the previous frame's. Consecutive frames thus overlap on the GPU while the TAA
// chain keeps its order, and every frame computes exactly what it computes alone. The caller's stream
// is not made to wait (that would serialise the next frame): reads wait for the frame themselves, and
// phe_renderer_join orders a stream after the last frame.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "runtime.cuh"
#include "wavefront.cuh"

using namespace phe_gb300;

constexpr int kMaxFrameParts = 4;

struct phe_renderer {
	const phe_scene* scene = nullptr;
	uint32_t resX = 0, resY = 0, numLights = 0;
	FrameBuffers fb{};                   // slot 0 per-frame buffers + the shared ones
	void* allocation = nullptr;
	FrameBuffers fb1{};                  // slot 1: fb with its per-frame buffers replaced
	void* allocation1 = nullptr;
	int inFlight = 1;
	FrameParamsDev* dParams1 = nullptr;  // parameters of slot 1
	cudaStream_t travStream[2] = {}, resolveStream = nullptr;
	cudaEvent_t callEvent = nullptr;     // the caller's work before a render
	cudaEvent_t travDone[2] = {}, resolveDone[2] = {};
	bool slotUsed[2] = {false, false};   // resolveDone[slot] marks the last frame that used the slot
	uint32_t nextSlot = 0, lastSlot = 0;
	bool framePending = false;           // a frame in flight that no caller stream has been ordered after
	// A frame split into parts (phe_renderer_set_frame_parts): part j (tile rows r with r % parts == j)
	// runs on partStream[j] beside part 0 on the caller's stream, with queues and counters of its own
	// (part 1: fb1's, parts 2..: partFb's) over the per-pixel buffers of fb; the caller's stream joins
	// every part at the end of the frame.
	int frameParts = 1;
	uint32_t lastParts = 1;              // parts the last frame ran as
	cudaStream_t partStream[kMaxFrameParts] = {};
	cudaEvent_t partFork = nullptr, partJoin[kMaxFrameParts] = {};
	void* partAlloc[kMaxFrameParts] = {};
	FrameBuffers partFb[kMaxFrameParts] = {};
	FrameParamsDev* partParams[kMaxFrameParts] = {};   // parameters of parts 2.. (part 1: dParams1)
	// Latency recording of frames in flight: (start, end) event pairs, drained by frame_latencies.
	bool recordLatency = false;
	std::vector<cudaEvent_t> latencyPool;
	std::vector<std::pair<cudaEvent_t, cudaEvent_t>> latencyPending;
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
	// Camera motion (TAA velocity): the last rendered camera and a ring of three velocity buffers
	// (frame k writes entry velNext, its resolve reads the previous frame's entry velLast; with two
	// frames in flight, frame k+1 must not overwrite what frame k's resolve still reads).
	phe_camera_def prevCam{};
	bool hasPrevCam = false;
	float2* vel[3] = {};
	bool velZero[3] = {true, true, true};
	uint32_t velLast = 0, velNext = 1;
	cudaEvent_t velDone[3] = {};         // last asynchronous copy out of each velocity buffer
	bool velGuard[3] = {false, false, false};
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

// Buffers and parameters of part j of a split frame (part 0: the renderer's own).
static const FrameBuffers& part_fb(const phe_renderer* r, uint32_t j) { return j == 0 ? r->fb : j == 1 ? r->fb1 : r->partFb[j]; }
static FrameParamsDev* part_params(const phe_renderer* r, uint32_t j)
{
	return j == 0 ? r->dParams : j == 1 ? r->dParams1 : r->partParams[j];
}
static const uint32_t kParamSlots = 8;

// Waits for the frames in flight on the renderer's own streams (none in sequential mode).
static void drain_streams(phe_renderer* r)
{
	for (int j = 0; j < 2; j++)
		if (r->travStream[j]) cudaStreamSynchronize(r->travStream[j]);
	if (r->resolveStream) cudaStreamSynchronize(r->resolveStream);
}

static void free_buffers(phe_renderer* r)
{
	// Frames on any stream may still use the buffers: the caller's, the part streams of split frames and
	// the renderer's own frame streams.
	cudaDeviceSynchronize();
	// in-place read-backs may still be copying out of these buffers
	for (int i = 0; i < 2; i++) {
		if (r->sideDone[i]) cudaEventSynchronize(r->sideDone[i]);
		r->sideGuard[i] = false;
	}
	for (int i = 0; i < 3; i++) {
		if (r->velDone[i]) cudaEventSynchronize(r->velDone[i]);
		r->velGuard[i] = false;
	}
	if (r->graphExec) cudaGraphExecDestroy(r->graphExec);
	r->graphExec = nullptr;
	if (r->allocation) cudaFree(r->allocation);
	if (r->allocation1) cudaFree(r->allocation1);
	r->allocation = r->allocation1 = nullptr;
	for (int j = 2; j < kMaxFrameParts; j++) {
		if (r->partAlloc[j]) cudaFree(r->partAlloc[j]);
		r->partAlloc[j] = nullptr;
	}
	std::memset(&r->fb, 0, sizeof(r->fb));
	std::memset(&r->fb1, 0, sizeof(r->fb1));
	for (int i = 0; i < 3; i++) r->vel[i] = nullptr;
	r->slotUsed[0] = r->slotUsed[1] = false;
	r->framePending = false;
	r->capacityP = r->capacityL = 0;
}

// Per-frame buffers of one slot: everything a frame's traversal writes and its resolve reads. Sizes
// for P pixels and L lights, in carving order.
static const int kPerFrameParts = 12;
static void per_frame_sizes(size_t P, size_t L, size_t sizes[kPerFrameParts])
{
	const size_t LP = P * L;
	const size_t v[kPerFrameParts] = {
		2 * LP * sizeof(float4),          // contrib
		2 * LP,                           // inLight
		2 * LP * sizeof(phe_ray_in),      // shadowRays
		2 * LP * sizeof(uint32_t),        // shadowSlots
		P * sizeof(phe_ray_in),           // bounceRays
		P * sizeof(uint32_t),             // bouncePixel
		P * sizeof(float4),               // bounceThroughput
		P * sizeof(float),                // roughness
		kNumCounters * sizeof(uint32_t),  // counters
		P * sizeof(phe_ray_hit),          // primaryHits
		P * sizeof(phe_ray_hit),          // bounceHits
		P * sizeof(uint32_t),             // bouncePerm
	};
	for (int i = 0; i < kPerFrameParts; i++) sizes[i] = v[i];
}

static size_t per_frame_bytes(size_t P, size_t L)
{
	size_t sizes[kPerFrameParts], total = 0;
	per_frame_sizes(P, L, sizes);
	for (size_t x : sizes) total += align256(x);
	return total;
}

// Points fb's per-frame buffers into `base` (per_frame_bytes(P, L) bytes); returns the end.
static char* carve_per_frame(char* base, size_t P, size_t L, FrameBuffers& fb)
{
	size_t sizes[kPerFrameParts];
	per_frame_sizes(P, L, sizes);
	char* p = base;
	auto take = [&](int i) { char* q = p; p += align256(sizes[i]); return q; };
	fb.contrib = (float4*)take(0);
	fb.inLight = (uint8_t*)take(1);
	fb.shadowRays = (phe_ray_in*)take(2);
	fb.shadowSlots = (uint32_t*)take(3);
	fb.bounceRays = (phe_ray_in*)take(4);
	fb.bouncePixel = (uint32_t*)take(5);
	fb.bounceThroughput = (float4*)take(6);
	fb.roughness = (float*)take(7);
	fb.counters = (uint32_t*)take(8);
	fb.primaryHits = (phe_ray_hit*)take(9);
	fb.bounceHits = (phe_ray_hit*)take(10);
	fb.bouncePerm = (uint32_t*)take(11);
	return p;
}

static void share_pixels(const phe_renderer* r, FrameBuffers& f)
{
	f.contrib = r->fb.contrib;
	f.inLight = r->fb.inLight;
	f.roughness = r->fb.roughness;
}

// Slot 1 shares everything with slot 0 but its per-frame buffers; as part 1 of a split frame it also
// shares the per-pixel ones (the parts write disjoint pixels) and keeps only its queues and counters,
// as parts 2.. do.
static void make_fb1(phe_renderer* r)
{
	if (r->allocation1) {
		r->fb1 = r->fb;
		carve_per_frame((char*)r->allocation1, r->capacityP, r->capacityL, r->fb1);
		if (r->frameParts >= 2) share_pixels(r, r->fb1);
	}
	for (int j = 2; j < kMaxFrameParts; j++)
		if (r->partAlloc[j]) {
			r->partFb[j] = r->fb;
			carve_per_frame((char*)r->partAlloc[j], r->capacityP, r->capacityL, r->partFb[j]);
			share_pixels(r, r->partFb[j]);
		}
}

// Zeroes newly allocated frame buffers before any frame, on whichever stream, can use them.
static phe_status clear_new(void* p, size_t bytes)
{
	cudaError_t e = cudaMemset(p, 0, bytes);
	if (e != cudaSuccess) return cuda_fail(e, "clear frame buffers");
	return finish_uploads("clear frame buffers");
}

static phe_status allocate_slot1(phe_renderer* r)
{
	if (r->allocation1 || !r->allocation) return PHE_OK;
	const size_t bytes = per_frame_bytes(r->capacityP, r->capacityL);
	cudaError_t e = cudaMalloc(&r->allocation1, bytes);
	if (e != cudaSuccess) {
		r->allocation1 = nullptr;
		return cuda_fail(e, "cudaMalloc(frame buffers of the second frame in flight)");
	}
	make_fb1(r);
	return clear_new(r->allocation1, bytes);
}

// Queue buffers of parts 2.. of a split frame.
static phe_status allocate_parts(phe_renderer* r)
{
	if (!r->allocation) return PHE_OK;
	const size_t bytes = per_frame_bytes(r->capacityP, r->capacityL);
	for (int j = 2; j < r->frameParts; j++) {
		if (r->partAlloc[j]) continue;
		cudaError_t e = cudaMalloc(&r->partAlloc[j], bytes);
		if (e != cudaSuccess) {
			r->partAlloc[j] = nullptr;
			return cuda_fail(e, "cudaMalloc(ray queues of a frame part)");
		}
		make_fb1(r);
		if (phe_status st = clear_new(r->partAlloc[j], bytes)) return st;
	}
	return PHE_OK;
}

// Streams, events and slot-1 buffers of two frames in flight. Each is made once; a call after one that
// failed part way makes the rest, and with everything present it only checks.
static phe_status prepare_flight(phe_renderer* r)
{
	if (!r->resolveStream) {   // made last: present means the streams and events before it are too
		for (int j = 0; j < 2; j++) {
			if (!r->travStream[j])
				PHE_CUDA_TRY(cudaStreamCreateWithFlags(&r->travStream[j], cudaStreamNonBlocking), "create frame stream");
			if (!r->travDone[j])
				PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->travDone[j], cudaEventDisableTiming), "create frame event");
			if (!r->resolveDone[j])
				PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->resolveDone[j], cudaEventDisableTiming), "create frame event");
		}
		if (!r->callEvent)
			PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->callEvent, cudaEventDisableTiming), "create frame event");
		PHE_CUDA_TRY(cudaStreamCreateWithFlags(&r->resolveStream, cudaStreamNonBlocking), "create frame stream");
	}
	return allocate_slot1(r);
}

// Streams, events, parameters and queue buffers of a frame split into `parts` parts, made the same way.
static phe_status prepare_parts(phe_renderer* r, int parts)
{
	if (!r->partFork) PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->partFork, cudaEventDisableTiming), "create part event");
	for (int j = 1; j < parts; j++) {
		if (!r->partStream[j])
			PHE_CUDA_TRY(cudaStreamCreateWithFlags(&r->partStream[j], cudaStreamNonBlocking), "create part stream");
		if (!r->partJoin[j])
			PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->partJoin[j], cudaEventDisableTiming), "create part event");
		if (j >= 2 && !r->partParams[j])
			PHE_CUDA_TRY(cudaMalloc(&r->partParams[j], sizeof(FrameParamsDev)), "allocate part parameters");
	}
	phe_status st = allocate_slot1(r);
	if (!st) st = allocate_parts(r);
	return st;
}

static phe_status allocate(phe_renderer* r, uint32_t resX, uint32_t resY, uint32_t numLights)
{
	const size_t P = (size_t)resX * resY;
	const size_t L = numLights ? numLights : 1;
	if (resX != r->resX || resY != r->resY) {   // velocities of another resolution do not carry over
		r->hasPrevCam = false;
		r->velZero[0] = r->velZero[1] = r->velZero[2] = true;
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
	const size_t shared[] = {
		P * sizeof(float4),               // rawColor
		P * sizeof(float4),               // history[0]
		P * sizeof(float4),               // history[1]
		P * sizeof(float4),               // color[0]
		P * sizeof(float4),               // color[1]
		4 * sizeof(unsigned long long),   // rayTotals
		P * sizeof(float2),               // velocity ring
		P * sizeof(float2),
		P * sizeof(float2),
	};
	size_t total = per_frame_bytes(P, L);
	for (size_t x : shared) total += align256(x);
	char* base = nullptr;
	cudaError_t e = cudaMalloc(&base, total);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(frame buffers)");
	FrameBuffers& fb = r->fb;
	char* p = carve_per_frame(base, P, L, fb);
	auto take = [&](size_t i) { char* q = p; p += align256(shared[i]); return q; };
	fb.rawColor = (float4*)take(0);
	fb.history[0] = (float4*)take(1);
	fb.history[1] = (float4*)take(2);
	fb.color[0] = (float4*)take(3);
	fb.color[1] = (float4*)take(4);
	fb.rayTotals = (unsigned long long*)take(5);
	for (int i = 0; i < 3; i++) r->vel[i] = (float2*)take(6 + i);
	fb.sortWindow = r->sortWindow;
	fb.capacityLP = (uint32_t)(P * L);
	fb.refill = r->refill;
	r->capacityP = P;
	r->capacityL = L;
	r->allocation = base;
	r->resX = resX;
	r->resY = resY;
	r->numLights = numLights;
	if (phe_status st = clear_new(base, total)) return st;
	r->parity = 0;
	if (r->inFlight == 2 || r->frameParts >= 2) {
		phe_status st = allocate_slot1(r);
		if (!st && r->frameParts > 2) st = allocate_parts(r);
		return st;
	}
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
	make_fb1(r);
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
	if (schedule == PHE_SHADOWS_BESIDE_BOUNCE && !r->streams.side) {
		PHE_CUDA_TRY(cudaStreamCreateWithFlags(&r->streams.side, cudaStreamNonBlocking), "create renderer stream");
		PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->streams.fork, cudaEventDisableTiming), "create renderer event");
		PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->streams.join, cudaEventDisableTiming), "create renderer event");
	}
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
	if (e == cudaSuccess) e = cudaMalloc(&r->dParams1, sizeof(FrameParamsDev));
	if (e == cudaSuccess) e = cudaMallocHost(&r->hParams, sizeof(FrameParamsDev) * kParamSlots);
	for (uint32_t i = 0; i < kParamSlots && e == cudaSuccess; i++)
		e = cudaEventCreateWithFlags(&r->paramEvents[i], cudaEventDisableTiming);
	if (e != cudaSuccess) {
		if (r->dParams) cudaFree(r->dParams);
		if (r->dParams1) cudaFree(r->dParams1);
		if (r->hParams) cudaFreeHost(r->hParams);
		delete r;
		return cuda_fail(e, "allocate frame parameters");
	}
	std::memset(r->hParams, 0, sizeof(FrameParamsDev) * kParamSlots);
	// No stream of its own yet: CUDA maps streams onto a few hardware queues in creation order, so
	// streams that sit unused (the side stream of a schedule not chosen) would make the streams of
	// concurrent renderers share queues and wait on each other. The side stream comes with the
	// BESIDE_BOUNCE schedule, the frame streams with two frames in flight, the copy stream with the
	// first asynchronous read.
	*out = r;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_destroy(phe_renderer* r)
{
	if (!r) return PHE_OK;
	cudaDeviceSynchronize();
	free_buffers(r);   // first: it waits on the read-back events destroyed below
	for (int j = 0; j < 2; j++) {
		if (r->travStream[j]) cudaStreamDestroy(r->travStream[j]);
		if (r->travDone[j]) cudaEventDestroy(r->travDone[j]);
		if (r->resolveDone[j]) cudaEventDestroy(r->resolveDone[j]);
	}
	if (r->resolveStream) cudaStreamDestroy(r->resolveStream);
	if (r->callEvent) cudaEventDestroy(r->callEvent);
	for (int j = 0; j < kMaxFrameParts; j++) {
		if (r->partStream[j]) cudaStreamDestroy(r->partStream[j]);
		if (r->partJoin[j]) cudaEventDestroy(r->partJoin[j]);
		if (r->partParams[j]) cudaFree(r->partParams[j]);
	}
	if (r->partFork) cudaEventDestroy(r->partFork);
	for (cudaEvent_t e : r->latencyPool) cudaEventDestroy(e);
	for (auto& pr : r->latencyPending) {
		cudaEventDestroy(pr.first);
		cudaEventDestroy(pr.second);
	}
	for (int i = 0; i < 3; i++)
		if (r->velDone[i]) cudaEventDestroy(r->velDone[i]);
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
	cudaFree(r->dParams1);
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

// The same for entry i of the velocity ring.
static phe_status guard_velocity(phe_renderer* r, uint32_t i, cudaStream_t s)
{
	if (!r->velGuard[i]) return PHE_OK;
	PHE_CUDA_TRY(cudaStreamWaitEvent(s, r->velDone[i], 0), "wait for read-back of a velocity buffer");
	r->velGuard[i] = false;
	return PHE_OK;
}

// Orders `s` after the last frame in flight (no-op in sequential mode, where frames run on `s`).
static phe_status join_frames(const phe_renderer* r, cudaStream_t s)
{
	if (!r->framePending) return PHE_OK;
	PHE_CUDA_TRY(cudaStreamWaitEvent(s, r->resolveDone[r->lastSlot], 0), "wait for the last frame");
	return PHE_OK;
}

// Buffers of the last rendered frame's slot (slot 0 in sequential mode).
static const FrameBuffers& last_fb(const phe_renderer* r) { return r->lastSlot ? r->fb1 : r->fb; }

extern "C" phe_status phe_renderer_join(phe_renderer* r, void* stream)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_join: null renderer");
	return join_frames(r, (cudaStream_t)stream);
}

extern "C" phe_status phe_renderer_set_frames_in_flight(phe_renderer* r, int frames)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_frames_in_flight: null renderer");
	if (frames != 1 && frames != 2) return fail(PHE_ERR_INVALID_ARGUMENT, "frames in flight must be 1 or 2");
	if (frames == 2 && r->frameParts >= 2)
		return fail(PHE_ERR_INVALID_ARGUMENT, "two frames in flight and split frames cannot be combined");
	drain_streams(r);   // the slots and streams change hands only when no frame is in flight
	r->slotUsed[0] = r->slotUsed[1] = false;
	r->framePending = false;
	r->nextSlot = r->lastSlot = 0;
	if (frames == 2) {
		phe_status st = prepare_flight(r);
		if (st) return st;   // frames stay one at a time
	}
	r->inFlight = frames;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_set_frame_parts(phe_renderer* r, int parts)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_frame_parts: null renderer");
	if (parts < 1 || parts > kMaxFrameParts) return fail(PHE_ERR_INVALID_ARGUMENT, "frame parts must be 1..%d", kMaxFrameParts);
	if (parts >= 2 && r->inFlight == 2)
		return fail(PHE_ERR_INVALID_ARGUMENT, "two frames in flight and split frames cannot be combined");
	if (parts == r->frameParts) return PHE_OK;
	cudaDeviceSynchronize();   // part 1's buffers change role
	if (r->graphExec) {
		cudaGraphExecDestroy(r->graphExec);
		r->graphExec = nullptr;
	}
	const int prev = r->frameParts;
	r->frameParts = parts;
	phe_status st = parts >= 2 ? prepare_parts(r, parts) : PHE_OK;
	if (st) r->frameParts = prev;   // a failed change keeps the previous split, whose parts are all made
	make_fb1(r);
	return st;
}

extern "C" phe_status phe_renderer_set_latency_recording(phe_renderer* r, int enable)
{
	if (!r) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_set_latency_recording: null renderer");
	r->recordLatency = enable != 0;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_frame_latencies(phe_renderer* r, float* ms, uint32_t capacity, uint32_t* count)
{
	if (!r || !count || (capacity && !ms)) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_frame_latencies: null argument");
	if (capacity == 0) {   // how many are recorded
		*count = (uint32_t)r->latencyPending.size();
		return PHE_OK;
	}
	const uint32_t n = (uint32_t)std::min<size_t>(capacity, r->latencyPending.size());
	for (uint32_t i = 0; i < n; i++) {
		const auto& pr = r->latencyPending[i];
		PHE_CUDA_TRY(cudaEventSynchronize(pr.second), "wait for a recorded frame");
		PHE_CUDA_TRY(cudaEventElapsedTime(&ms[i], pr.first, pr.second), "frame latency");
		r->latencyPool.push_back(pr.first);
		r->latencyPool.push_back(pr.second);
	}
	r->latencyPending.erase(r->latencyPending.begin(), r->latencyPending.begin() + n);
	*count = n;
	return PHE_OK;
}

static phe_status take_timing_event(phe_renderer* r, cudaEvent_t* e)
{
	if (!r->latencyPool.empty()) {
		*e = r->latencyPool.back();
		r->latencyPool.pop_back();
		return PHE_OK;
	}
	PHE_CUDA_TRY(cudaEventCreate(e), "create latency event");
	return PHE_OK;
}

extern "C" phe_status phe_renderer_reset_taa(phe_renderer* r, void* stream)
{
	if (!r || !r->allocation) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_reset_taa: no frame buffers");
	size_t P = (size_t)r->resX * r->resY;
	phe_status st = join_frames(r, (cudaStream_t)stream);   // the resolve of a frame in flight uses the history
	if (st) return st;
	for (uint32_t side = 0; side < 2; side++) {
		st = guard_side(r, side, (cudaStream_t)stream);
		if (st) return st;
	}
	PHE_CUDA_TRY(cudaMemsetAsync(r->fb.history[0], 0, P * sizeof(float4), (cudaStream_t)stream), "reset TAA");
	PHE_CUDA_TRY(cudaMemsetAsync(r->fb.history[1], 0, P * sizeof(float4), (cudaStream_t)stream), "reset TAA");
	r->hasPrevCam = false;
	r->velZero[0] = r->velZero[1] = r->velZero[2] = true;
	return PHE_OK;
}

extern "C" phe_status phe_renderer_reset_ray_totals(phe_renderer* r, void* stream)
{
	if (!r || !r->allocation) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_reset_ray_totals: no frame buffers");
	phe_status st = join_frames(r, (cudaStream_t)stream);
	if (st) return st;
	PHE_CUDA_TRY(cudaMemsetAsync(r->fb.rayTotals, 0, 4 * sizeof(unsigned long long), (cudaStream_t)stream),
	             "reset ray totals");
	return PHE_OK;
}

extern "C" phe_status phe_renderer_ray_totals_async(const phe_renderer* r, uint64_t* hostTotals4, void* stream)
{
	if (!r || !r->allocation || !hostTotals4) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_ray_totals_async: no frame");
	phe_status st = join_frames(r, (cudaStream_t)stream);
	if (st) return st;
	PHE_CUDA_TRY(cudaMemcpyAsync(hostTotals4, r->fb.rayTotals, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost,
	                             (cudaStream_t)stream), "read ray totals");
	return PHE_OK;
}

// One frame on `s`: whole, or split into `parts` parts, parts 1.. on their part streams between a fork
// and joins on `s` (the same calls capture a split frame into a graph).
static phe_status launch_whole_or_split(phe_renderer* r, cudaStream_t s, uint32_t parts, const uint32_t* n)
{
	if (parts == 1)
		return launch_frame(r->scene, r->dParams, r->fb, r->resX, r->resY, s, nullptr, r->fused, r->shadowSchedule,
		                    &r->streams);
	PHE_CUDA_TRY(cudaEventRecord(r->partFork, s), "fork frame parts");
	for (uint32_t j = 1; j < parts; j++)
		PHE_CUDA_TRY(cudaStreamWaitEvent(r->partStream[j], r->partFork, 0), "fork frame parts");
	for (uint32_t j = 0; j < parts; j++) {
		cudaStream_t ps = j ? r->partStream[j] : s;
		phe_status st = launch_frame(r->scene, part_params(r, j), part_fb(r, j), r->resX, r->resY, ps, nullptr, r->fused,
		                             r->shadowSchedule, nullptr, kFrameAll, n[j]);
		if (st) return st;
		if (j) PHE_CUDA_TRY(cudaEventRecord(r->partJoin[j], ps), "join frame parts");
	}
	for (uint32_t j = 1; j < parts; j++)
		PHE_CUDA_TRY(cudaStreamWaitEvent(s, r->partJoin[j], 0), "join frame parts");
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
		drain_streams(r);
		cudaStreamSynchronize(s);
		phe_status st = allocate(r, r->resX, r->resY, L);
		if (st) return st;
	}
	// Two frames in flight, unless per-kernel timing wants the frame in order on one stream.
	const bool pipelined = r->inFlight == 2 && !r->timing;
	const uint32_t j = pipelined ? r->nextSlot : 0;
	const FrameBuffers& fb = j ? r->fb1 : r->fb;
	FrameParamsDev* dParams = j ? r->dParams1 : r->dParams;
	cudaStream_t X = pipelined ? r->travStream[j] : s;   // traversal kernels
	cudaStream_t R = pipelined ? r->resolveStream : s;   // resolve + TAA
	// A split frame: part j takes the tile rows r with r % parts == j, part 0 on `s`, the others on their
	// part streams (fused pipeline only, at most one part per tile row; frames timed per kernel stay whole).
	const uint32_t tileRows = r->resY / 8u;
	const uint32_t parts = (!pipelined && r->frameParts >= 2 && r->fused && !r->timing)
	                           ? std::min<uint32_t>((uint32_t)r->frameParts, tileRows) : 1u;
	uint32_t n[kMaxFrameParts] = {};
	for (uint32_t k = 0; k < parts; k++) n[k] = (tileRows - k + parts - 1) / parts * 8u * r->resX;
	{   // everything this frame's shape uses (only checks, unless an earlier call failed part way)
		phe_status st = pipelined ? prepare_flight(r) : parts >= 2 ? prepare_parts(r, (int)parts) : PHE_OK;
		if (st) return st;
	}
	if (pipelined) {
		// after the caller's work so far, and after the resolve that last read this slot's buffers
		PHE_CUDA_TRY(cudaEventRecord(r->callEvent, s), "record caller work");
		PHE_CUDA_TRY(cudaStreamWaitEvent(X, r->callEvent, 0), "order frame after caller work");
		if (r->slotUsed[j]) PHE_CUDA_TRY(cudaStreamWaitEvent(X, r->resolveDone[j], 0), "wait for the slot");
	} else {
		phe_status st = join_frames(r, s);   // frames still in flight from before per-kernel timing
		if (st) return st;
		r->framePending = false;
	}
	// Pinned staging ring: a slot is rewritten only after its previous copy has been consumed.
	uint32_t slot = r->paramSlot;
	r->paramSlot = (slot + 1) % kParamSlots;
	PHE_CUDA_TRY(cudaEventSynchronize(r->paramEvents[slot]), "wait for a free parameter slot");
	FrameParamsDev& fp = r->hParams[slot];
	// Camera motion: this frame writes the next entry of the velocity ring and reads the previous
	// frame's; a camera equal to the previous one has velocity 0 (nothing written or read).
	const uint32_t outSide = r->parity ^ 1u;
	const uint32_t vOut = r->velNext, vIn = r->velLast;
	const bool moving = r->hasPrevCam && std::memcmp(&r->prevCam, &r->cam, sizeof(phe_camera_def)) != 0;
	fp.prevCam = r->hasPrevCam ? r->prevCam : r->cam;
	fp.velocity = moving ? r->vel[vOut] : nullptr;
	fp.prevVelocity = r->velZero[vIn] ? nullptr : r->vel[vIn];
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
	fp.part = 0;
	fp.parts = parts;
	fp.partPixels = n[0];
	fp.pad = 0;
	std::memset(fp.lights, 0, sizeof(fp.lights));
	if (numLights) std::memcpy(fp.lights, lights, sizeof(phe_sphere_light) * numLights);
	phe_status gst = guard_velocity(r, vOut, X);   // the traversal rewrites this velocity buffer
	if (!gst) gst = guard_side(r, outSide, R);     // the resolve rewrites this colour / history side
	if (gst) return gst;
	PHE_CUDA_TRY(cudaMemcpyAsync(dParams, &fp, sizeof(FrameParamsDev), cudaMemcpyHostToDevice, X),
	             "upload frame parameters");
	PHE_CUDA_TRY(cudaEventRecord(r->paramEvents[slot], X), "record parameter slot");
	for (uint32_t k = 1; k < parts; k++) {   // the other parts' parameters: the same but for part and pixels
		const uint32_t slotK = r->paramSlot;
		r->paramSlot = (slotK + 1) % kParamSlots;
		PHE_CUDA_TRY(cudaEventSynchronize(r->paramEvents[slotK]), "wait for a free parameter slot");
		FrameParamsDev& fpk = r->hParams[slotK];
		fpk = fp;
		fpk.part = k;
		fpk.partPixels = n[k];
		PHE_CUDA_TRY(cudaMemcpyAsync(part_params(r, k), &fpk, sizeof(FrameParamsDev), cudaMemcpyHostToDevice, s),
		             "upload frame parameters");
		PHE_CUDA_TRY(cudaEventRecord(r->paramEvents[slotK], s), "record parameter slot");
	}
	if (pipelined) {
		cudaEvent_t t0 = nullptr, t1 = nullptr;
		if (r->recordLatency) {
			phe_status st = take_timing_event(r, &t0);
			if (!st) st = take_timing_event(r, &t1);
			if (st) return st;
			PHE_CUDA_TRY(cudaEventRecord(t0, X), "record frame start");
		}
		phe_status st = launch_frame(r->scene, dParams, fb, r->resX, r->resY, X, nullptr, r->fused, r->shadowSchedule,
		                             nullptr, kFrameTraversal);
		if (st) return st;
		PHE_CUDA_TRY(cudaEventRecord(r->travDone[j], X), "record frame traversal");
		PHE_CUDA_TRY(cudaStreamWaitEvent(R, r->travDone[j], 0), "order resolve after traversal");
		st = launch_frame(r->scene, dParams, fb, r->resX, r->resY, R, nullptr, r->fused, r->shadowSchedule, nullptr,
		                  kFrameResolve);
		if (st) return st;
		PHE_CUDA_TRY(cudaEventRecord(r->resolveDone[j], R), "record frame end");
		if (r->recordLatency) {
			PHE_CUDA_TRY(cudaEventRecord(t1, R), "record frame end");
			r->latencyPending.emplace_back(t0, t1);
		}
		r->slotUsed[j] = true;
		r->lastSlot = j;
		r->nextSlot = j ^ 1u;
		r->framePending = true;
	} else if (r->useGraph) {
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
				st = launch_whole_or_split(r, cap, parts, n);
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
		r->lastSlot = 0;
	} else {
		phe_status st;
		if (r->timing) {
			if ((st = collect_times(r))) return st;
			r->timedKernels = frame_kernels(r->fused, r->shadowSchedule, r->sortWindow);
			st = launch_frame(r->scene, r->dParams, r->fb, r->resX, r->resY, s, r->events, r->fused, r->shadowSchedule,
			                  nullptr);
			r->pendingTimes = true;
		} else {
			st = launch_whole_or_split(r, s, parts, n);
		}
		if (st) return st;
		r->lastSlot = 0;
	}
	r->lastParts = parts;
	r->velZero[vOut] = !moving;
	r->velLast = vOut;
	r->velNext = (vOut + 1) % 3;
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
	out->roughness = last_fb(r).roughness;
	out->velocity = r->velZero[r->velLast] ? nullptr : (const float*)r->vel[r->velLast];
	return PHE_OK;
}

extern "C" phe_status phe_renderer_ray_counts(const phe_renderer* r, uint64_t counts[4], void* stream)
{
	if (!r || !counts || !r->fb.counters) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_renderer_ray_counts: no frame");
	phe_status st = join_frames(r, (cudaStream_t)stream);
	if (st) return st;
	uint32_t c[kNumCounters];
	uint32_t cp[kMaxFrameParts][kNumCounters] = {};
	PHE_CUDA_TRY(cudaMemcpyAsync(c, last_fb(r).counters, sizeof(c), cudaMemcpyDeviceToHost, (cudaStream_t)stream),
	             "read counters");
	for (uint32_t j = 1; j < r->lastParts; j++)   // the other parts' queues
		PHE_CUDA_TRY(cudaMemcpyAsync(cp[j], part_fb(r, j).counters, sizeof(cp[j]), cudaMemcpyDeviceToHost,
		                             (cudaStream_t)stream), "read counters");
	PHE_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream), "read counters");
	counts[0] = (uint64_t)r->resX * r->resY;
	counts[1] = c[kCtrShadow0];
	counts[2] = c[kCtrBounce];
	counts[3] = c[kCtrShadow1];
	for (uint32_t j = 1; j < r->lastParts; j++) {
		counts[1] += cp[j][kCtrShadow0];
		counts[2] += cp[j][kCtrBounce];
		counts[3] += cp[j][kCtrShadow1];
	}
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
	case 3: *src = last_fb(r).roughness; *bytes = P * sizeof(float); break;
	case 4: *src = r->velZero[r->velLast] ? nullptr : r->vel[r->velLast]; *bytes = P * sizeof(float2); break;
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
	if ((st = join_frames(r, (cudaStream_t)stream))) return st;
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
		for (int i = 0; i < 3; i++)
			PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->velDone[i], cudaEventDisableTiming), "create read event");
		PHE_CUDA_TRY(cudaEventCreateWithFlags(&r->readyEvent, cudaEventDisableTiming), "create read event");
	}
	// TAA colour and history live on the side the last frame wrote, a stored velocity in the last entry
	// of the ring; the next frame only reads them, so the copy reads them in place and the frame that
	// rewrites them waits for the copy. The copy waits for the last frame itself: with frames in flight
	// the caller's stream is not ordered after them, and ordering it would hold back the next frame.
	if (src && (which == 0 || which == 1 || which == 4)) {
		if (r->framePending) {
			PHE_CUDA_TRY(cudaStreamWaitEvent(r->copyStream, r->resolveDone[r->lastSlot], 0), "order read-back");
		} else {
			PHE_CUDA_TRY(cudaEventRecord(r->readyEvent, s), "record frame end");
			PHE_CUDA_TRY(cudaStreamWaitEvent(r->copyStream, r->readyEvent, 0), "order read-back");
		}
		PHE_CUDA_TRY(cudaMemcpyAsync(hostDst, src, bytes, cudaMemcpyDeviceToHost, r->copyStream), "read result");
		if (which == 4) {
			PHE_CUDA_TRY(cudaEventRecord(r->velDone[r->velLast], r->copyStream), "record read-back");
			r->velGuard[r->velLast] = true;
		} else {
			PHE_CUDA_TRY(cudaEventRecord(r->sideDone[r->parity], r->copyStream), "record read-back");
			r->sideGuard[r->parity] = true;
		}
		return PHE_OK;
	}
	// Raw colour and roughness are rewritten by the next frame: a snapshot on the caller's stream, which
	// is first ordered after the last frame (with frames in flight this also orders the next frame after it).
	if ((st = join_frames(r, s))) return st;
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
	for (int i = 0; i < 3; i++)
		if (r->velDone[i]) PHE_CUDA_TRY(cudaEventSynchronize(r->velDone[i]), "wait for read-back");
	return PHE_OK;
}

extern "C" uint32_t phe_renderer_frame_param_bytes(void) { return (uint32_t)sizeof(FrameParamsDev); }
