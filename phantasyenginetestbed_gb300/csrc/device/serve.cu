// Serving loop: continuous batching of ray-query and render requests against device-resident
// scenes (no reference counterpart; the reference renders one frame at a time from its game loop).
//
// A scheduler thread owns the GPU work:
//   * admission — a request is admitted when it fits the device-memory budget (resident scenes
//     count against it), the in-flight limit, and, for renders, a free render slot (queries behind a
//     render that waits for a slot are admitted past it; a render on a scene a slot is rendering may
//     go before a bounded number of earlier renders). Its device state (rays and results; a render
//     slot's frame buffers) stays on the GPU until it completes.
//   * ray queries — every admitted query whose rays are on the device joins the next WAVE: one
//     batched persistent launch over all of them (any scenes, closest and any hit mixed). Requests that
//     arrive while a wave runs are admitted and go into the following wave (up to two waves queued).
//   * renders — each runs its spp frames (wavefront frame + TAA, Halton jitter) on its slot's own
//     stream, so renders overlap each other and the query waves on the device.
//   * completion — an event per request; results are copied to the caller's host buffer before the
//     event, and the request's budget is returned.
// A serial mode (one request at a time, plain per-request launches, synchronised) is the baseline.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.cuh"
#include "runtime.cuh"
#include "wavefront.cuh"

using namespace phe_gb300;

namespace {

constexpr uint32_t kWaveRing = 2;          // waves in flight at once
constexpr uint32_t kMaxWaveItems = 1024;   // queries per wave
constexpr size_t kAffinityLookAhead = 16;  // pending entries searched for a render on a scene in use
constexpr uint32_t kMaxPassed = 8;         // a render is passed over at most this many times

double now_ms(std::chrono::steady_clock::time_point t0)
{
	return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

enum ReqState { kPending, kAdmitted, kIssued, kDone };

struct Request {
	uint64_t id = 0;
	phe_request desc{};
	std::vector<phe_sphere_light> lights;
	ReqState state = kPending;
	phe_status status = PHE_OK;
	double tSubmit = 0, tAdmit = 0, tDone = 0;
	uint64_t bytes = 0;
	void* dMem = nullptr;           // query: rays then results
	cudaEvent_t done = nullptr;
	int slot = -1;                  // render slot
	uint32_t passed = 0;            // times a later render on a busier scene was admitted before it
	uint64_t rays = 0;
	std::string error;              // message of a failed request (set on the scheduler thread)
};

struct RenderSlot {
	phe_renderer* renderer = nullptr;
	cudaStream_t stream = nullptr;
	Request* busy = nullptr;
	uint64_t* totals = nullptr;     // pinned [4]
};

struct Wave {
	BatchItemDev* hostItems = nullptr;   // pinned [kMaxWaveItems]
	BatchItemDev* devItems = nullptr;    // [kMaxWaveItems]
	uint32_t* counter = nullptr;         // work counter of the wave
	cudaEvent_t done = nullptr;
	bool busy = false;
};

// Device bytes a render slot holds for a frame of P pixels and L lights (the renderer's buffers):
// per light and pixel, two contributions, visibilities, shadow rays and slots; per pixel, the bounce
// ray, pixel, throughput and permutation, roughness, raw colour, two histories, two TAA colours, two
// hit records and three velocities. With two frames in flight the per-frame part (everything but the
// colours, histories and velocities) is held twice.
uint64_t render_bytes(uint64_t P, uint64_t L, bool twoInFlight)
{
	const uint64_t perFrame = 2 * L * P * (16 + 1 + 32 + 4) + P * (32 + 4 + 16 + 4 + 4 + 16 * 2) + 256;
	const uint64_t shared = P * (16 + 16 * 2 + 16 * 2 + 8 * 3) + 4096;
	return perFrame * (twoInFlight ? 2 : 1) + shared;
}

uint64_t query_bytes(const phe_request& r)
{
	return align256((uint64_t)r.numRays * sizeof(phe_ray_in)) +
	       align256((uint64_t)r.numRays * (r.kind == PHE_REQ_ANY ? 1 : sizeof(phe_ray_hit)));
}

} // namespace

struct phe_server {
	phe_server_config cfg{};
	std::vector<const phe_scene*> scenes;
	DeviceScene* dScenes = nullptr;
	uint64_t sceneBytes = 0;
	int device = 0;
	std::chrono::steady_clock::time_point t0;

	std::mutex m;
	std::condition_variable cvWork, cvDone;
	std::deque<Request*> pending;
	std::vector<Request*> admitted;   // queries waiting for a wave
	std::vector<Request*> inflight;   // issued, not complete
	std::unordered_map<uint64_t, Request*> all;
	uint64_t nextId = 1;
	uint64_t bytesInUse = 0;
	bool stop = false;
	bool sceneTableDirty = true;
	bool wideScenes = false;               // some resident scene has its 4-wide layout selected

	cudaStream_t waveStream = nullptr;
	Wave waves[kWaveRing];
	std::vector<RenderSlot> slots;
	std::vector<cudaEvent_t> eventPool;
	std::thread worker;

	// statistics
	uint64_t wavesLaunched = 0, raysCompleted = 0;
};

namespace {

cudaEvent_t take_event(phe_server* s)
{
	if (!s->eventPool.empty()) {
		cudaEvent_t e = s->eventPool.back();
		s->eventPool.pop_back();
		return e;
	}
	cudaEvent_t e = nullptr;
	cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
	return e;
}

void finish(phe_server* s, Request* r, phe_status st)
{
	r->status = st;
	if (st != PHE_OK) r->error = phe_last_error();
	r->tDone = now_ms(s->t0);
	r->state = kDone;
	s->bytesInUse -= r->bytes;
	s->raysCompleted += r->rays;
	if (r->dMem) {   // a query that failed before its wave freed it
		cudaFreeAsync(r->dMem, s->waveStream);
		r->dMem = nullptr;
	}
	if (r->done) {
		s->eventPool.push_back(r->done);
		r->done = nullptr;
	}
}

// Issues a query's upload (admission) on the wave stream.
phe_status admit_query(phe_server* s, Request* r)
{
	const phe_request& d = r->desc;
	size_t raysBytes = align256((size_t)d.numRays * sizeof(phe_ray_in));
	size_t outBytes = align256((size_t)d.numRays * (d.kind == PHE_REQ_ANY ? 1 : sizeof(phe_ray_hit)));
	cudaError_t e = cudaMallocAsync(&r->dMem, raysBytes + outBytes, s->waveStream);
	if (e != cudaSuccess) {
		r->dMem = nullptr;
		return cuda_fail(e, "cudaMallocAsync(request)");
	}
	e = cudaMemcpyAsync(r->dMem, d.rays, (size_t)d.numRays * sizeof(phe_ray_in), cudaMemcpyHostToDevice, s->waveStream);
	if (e != cudaSuccess) return cuda_fail(e, "upload request rays");
	return PHE_OK;
}

// Host callback queued after a wave's or a render's completion event: wakes the scheduler so that it
// retires the requests at once instead of at its next timed poll. It only notifies (no CUDA call, no
// lock); phe_server_destroy synchronises the device before the server is freed.
void CUDART_CB wake_scheduler(void* server) { static_cast<phe_server*>(server)->cvWork.notify_all(); }

// Launches one wave over every admitted query (called with the lock held).
phe_status launch_wave(phe_server* s, Wave& w)
{
	NvtxRange range("phe_server wave");
	uint32_t n = (uint32_t)std::min<size_t>(s->admitted.size(), kMaxWaveItems);
	uint32_t base = 0;
	for (uint32_t i = 0; i < n; i++) {
		Request* r = s->admitted[i];
		const phe_request& d = r->desc;
		BatchItemDev& it = w.hostItems[i];
		it.scene = d.scene;
		it.kind = d.kind == PHE_REQ_ANY ? 1u : 0u;
		it.count = d.numRays;
		it.base = base;
		it.rays = (const phe_ray_in*)r->dMem;
		it.out = (char*)r->dMem + align256((size_t)d.numRays * sizeof(phe_ray_in));
		base += (d.numRays + 31u) / 32u * 32u;
	}
	cudaStream_t st = s->waveStream;
	PHE_CUDA_TRY(cudaMemcpyAsync(w.devItems, w.hostItems, n * sizeof(BatchItemDev), cudaMemcpyHostToDevice, st),
	             "upload wave table");
	PHE_CUDA_TRY(cudaMemsetAsync(w.counter, 0, 2 * sizeof(uint32_t), st), "clear wave counter");
	phe_status ps = launch_batch_table(w.devItems, n, base, s->dScenes, w.counter, 128, 0, st,
	                                   s->wideScenes);
	if (ps) return ps;
	for (uint32_t i = 0; i < n; i++) {
		Request* r = s->admitted[i];
		const phe_request& d = r->desc;
		size_t outBytes = (size_t)d.numRays * (d.kind == PHE_REQ_ANY ? 1 : sizeof(phe_ray_hit));
		PHE_CUDA_TRY(cudaMemcpyAsync(d.out, w.hostItems[i].out, outBytes, cudaMemcpyDeviceToHost, st), "download results");
		PHE_CUDA_TRY(cudaFreeAsync(r->dMem, st), "cudaFreeAsync(request)");
		r->dMem = nullptr;
		r->done = take_event(s);
		PHE_CUDA_TRY(cudaEventRecord(r->done, st), "record request event");
		r->rays = d.numRays;
		r->state = kIssued;
		s->inflight.push_back(r);
	}
	PHE_CUDA_TRY(cudaEventRecord(w.done, st), "record wave event");
	PHE_CUDA_TRY(cudaLaunchHostFunc(st, wake_scheduler, s), "queue wave completion callback");
	w.busy = true;
	s->admitted.erase(s->admitted.begin(), s->admitted.begin() + n);
	s->wavesLaunched++;
	return PHE_OK;
}

// Issues every frame of a render request on its slot's stream.
phe_status issue_render(phe_server* s, Request* r, RenderSlot& slot)
{
	const phe_request& d = r->desc;
	phe_renderer* R = slot.renderer;
	cudaStream_t st = slot.stream;
	phe_status ps;
	if ((ps = phe_renderer_set_static_scene(R, s->scenes[d.scene]))) return ps;
	if ((ps = phe_renderer_set_target_resolution(R, d.resX, d.resY))) return ps;
	if ((ps = phe_renderer_set_seed(R, d.seed, 0))) return ps;
	if ((ps = phe_renderer_reset_taa(R, st))) return ps;
	if ((ps = phe_renderer_reset_ray_totals(R, st))) return ps;
	for (uint32_t f = 0; f < d.spp; f++) {
		float j[2];
		phe_halton_jitter(f, j);
		if ((ps = phe_renderer_set_camera_def(R, &d.cam, d.camPos, j[0], j[1]))) return ps;
		if ((ps = phe_renderer_render(R, r->lights.data(), (uint32_t)r->lights.size(), st))) return ps;
	}
	phe_render_result res;
	if ((ps = phe_renderer_result(R, &res))) return ps;
	if ((ps = phe_renderer_join(R, st))) return ps;   // the frames run on the renderer's own streams
	PHE_CUDA_TRY(cudaMemcpyAsync(d.out, res.color, (size_t)d.resX * d.resY * 16, cudaMemcpyDeviceToHost, st),
	             "download render");
	if ((ps = phe_renderer_ray_totals_async(R, slot.totals, st))) return ps;
	r->done = take_event(s);
	PHE_CUDA_TRY(cudaEventRecord(r->done, st), "record request event");
	if (!s->cfg.serial) PHE_CUDA_TRY(cudaLaunchHostFunc(st, wake_scheduler, s), "queue render completion callback");
	r->slot = (int)(&slot - s->slots.data());
	slot.busy = r;
	r->state = kIssued;
	s->inflight.push_back(r);
	return PHE_OK;
}

// Scene affinity of render admission: the render at pending[pi] is next in order and a slot is free.
// If no slot is rendering its scene, a later render (within kAffinityLookAhead entries) on a scene that
// a slot is rendering goes first instead, its tree being warm in L2; every render passed over counts
// it, and one passed kMaxPassed times is taken in order. Returns the index of the render to admit.
size_t pick_render(phe_server* s, size_t pi)
{
	auto inUse = [&](uint32_t scene) {
		for (const RenderSlot& sl : s->slots)
			if (sl.busy && sl.busy->desc.scene == scene) return true;
		return false;
	};
	const Request* r = s->pending[pi];
	if (r->passed >= kMaxPassed || inUse(r->desc.scene)) return pi;
	const size_t end = std::min(s->pending.size(), pi + 1 + kAffinityLookAhead);
	for (size_t j = pi + 1; j < end; j++) {
		const Request* q = s->pending[j];
		if (q->desc.kind == PHE_REQ_RENDER && inUse(q->desc.scene) &&
		    s->sceneBytes + s->bytesInUse + q->bytes <= s->cfg.memoryBudget) {
			for (size_t k = pi; k < j; k++)
				if (s->pending[k]->desc.kind == PHE_REQ_RENDER) s->pending[k]->passed++;
			return j;
		}
	}
	return pi;
}

void upload_scene_table(phe_server* s)
{
	std::vector<DeviceScene> t;
	s->wideScenes = false;
	for (const phe_scene* sc : s->scenes) {
		t.push_back(sc->dev);
		s->wideScenes = s->wideScenes || sc->dev.nodes4 || sc->dev.nodes8;
	}
	// On the wave stream: after the waves still reading the table, before the next wave (the pageable
	// source is staged before the call returns).
	if (!t.empty())
		cudaMemcpyAsync(s->dScenes, t.data(), t.size() * sizeof(DeviceScene), cudaMemcpyHostToDevice, s->waveStream);
	s->sceneTableDirty = false;
}

// Serial baseline: one request at a time with plain launches, waiting for each. Called with the lock
// held; it is released only while waiting for the GPU, with the request in `inflight`, so that
// drain() and the stop condition still see it and every change of shared state happens under the lock.
void serve_serial(phe_server* s, Request* r, std::unique_lock<std::mutex>& lock)
{
	const phe_request& d = r->desc;
	r->tAdmit = now_ms(s->t0);
	phe_status ps = PHE_OK;
	cudaStream_t wait = nullptr;
	RenderSlot* slot = nullptr;
	if (d.kind == PHE_REQ_RENDER) {
		slot = &s->slots[0];
		ps = issue_render(s, r, *slot);   // on success the request is in inflight
		if (!ps) wait = slot->stream;
	} else {
		ps = admit_query(s, r);
		if (!ps) {
			phe_scene* sc = const_cast<phe_scene*>(s->scenes[d.scene]);
			void* out = (char*)r->dMem + align256((size_t)d.numRays * sizeof(phe_ray_in));
			ps = d.kind == PHE_REQ_ANY
			         ? phe_cast_any(sc, (const phe_ray_in*)r->dMem, (uint8_t*)out, d.numRays, nullptr, s->waveStream)
			         : phe_cast_closest(sc, (const phe_ray_in*)r->dMem, (phe_ray_hit*)out, d.numRays, s->waveStream);
			size_t outBytes = (size_t)d.numRays * (d.kind == PHE_REQ_ANY ? 1 : sizeof(phe_ray_hit));
			if (!ps) cudaMemcpyAsync(d.out, out, outBytes, cudaMemcpyDeviceToHost, s->waveStream);
			cudaFreeAsync(r->dMem, s->waveStream);
			r->dMem = nullptr;
			r->rays = d.numRays;
			r->state = kIssued;
			s->inflight.push_back(r);
			wait = s->waveStream;
		}
	}
	if (wait) {
		lock.unlock();
		cudaError_t e = cudaStreamSynchronize(wait);
		lock.lock();
		s->inflight.erase(std::find(s->inflight.begin(), s->inflight.end(), r));
		if (slot) {
			r->rays = slot->totals[0] + slot->totals[1] + slot->totals[2] + slot->totals[3];
			slot->busy = nullptr;
		}
		if (e != cudaSuccess && !ps) ps = cuda_fail(e, "request");
	}
	finish(s, r, ps);
}

void worker_loop(phe_server* s)
{
	cudaSetDevice(s->device);
	std::unique_lock<std::mutex> lock(s->m);
	while (true) {
		if (s->stop && s->pending.empty() && s->admitted.empty() && s->inflight.empty()) break;
		if (s->sceneTableDirty) upload_scene_table(s);
		bool progress = false;

		if (s->cfg.serial) {
			if (!s->pending.empty()) {
				Request* r = s->pending.front();
				s->pending.pop_front();
				s->bytesInUse += r->bytes;
				serve_serial(s, r, lock);
				s->cvDone.notify_all();
				continue;
			}
		} else {
			// 1. completions
			for (size_t i = 0; i < s->inflight.size();) {
				Request* r = s->inflight[i];
				cudaError_t q = cudaEventQuery(r->done);
				if (q == cudaErrorNotReady) { i++; continue; }
				if (r->slot >= 0) {
					RenderSlot& slot = s->slots[r->slot];
					r->rays = slot.totals[0] + slot.totals[1] + slot.totals[2] + slot.totals[3];
					slot.busy = nullptr;
				}
				finish(s, r, q == cudaSuccess ? PHE_OK : cuda_fail(q, "request"));
				s->inflight[i] = s->inflight.back();
				s->inflight.pop_back();
				progress = true;
			}
			for (Wave& w : s->waves)
				if (w.busy && cudaEventQuery(w.done) != cudaErrorNotReady) w.busy = false;
			if (progress) s->cvDone.notify_all();

			// 2. admission, in arrival order. A render waiting for a free slot does not hold back the
			//    queries behind it; renders are taken in order except for the bounded scene affinity of
			//    pick_render; a request that does not fit the memory budget or the in-flight limit stops
			//    admission.
			bool renderWaits = false;
			for (size_t pi = 0; pi < s->pending.size();) {
				Request* r = s->pending[pi];
				if (s->inflight.size() + s->admitted.size() >= s->cfg.maxInFlight) break;
				if (s->sceneBytes + s->bytesInUse + r->bytes > s->cfg.memoryBudget) break;
				RenderSlot* freeSlot = nullptr;
				size_t take = pi;
				if (r->desc.kind == PHE_REQ_RENDER) {
					if (!renderWaits)
						for (RenderSlot& sl : s->slots)
							if (!sl.busy) { freeSlot = &sl; break; }
					if (!freeSlot) {
						renderWaits = true;
						pi++;
						continue;
					}
					take = pick_render(s, pi);
					r = s->pending[take];
				}
				s->pending.erase(s->pending.begin() + take);
				s->bytesInUse += r->bytes;
				r->tAdmit = now_ms(s->t0);
				r->state = kAdmitted;
				phe_status ps = r->desc.kind == PHE_REQ_RENDER ? issue_render(s, r, *freeSlot) : admit_query(s, r);
				if (ps) {
					if (freeSlot) freeSlot->busy = nullptr;
					finish(s, r, ps);
					s->cvDone.notify_all();
					continue;
				}
				if (r->desc.kind != PHE_REQ_RENDER) s->admitted.push_back(r);
				progress = true;
			}

			// 3. a wave over the admitted queries when a wave slot is free and the batching window of
			//    the oldest admitted query has passed (or the wave is full, or nothing else is coming)
			bool waveReady = !s->admitted.empty();
			if (waveReady && s->cfg.batchWindowUs > 0 && s->admitted.size() < kMaxWaveItems) {
				double waited = now_ms(s->t0) - s->admitted.front()->tAdmit;
				waveReady = waited * 1000.0 >= (double)s->cfg.batchWindowUs;
			}
			if (waveReady)
				for (Wave& w : s->waves)
					if (!w.busy) {
						phe_status ps = launch_wave(s, w);
						if (ps) {
							// queries the wave issued before the failure complete through their events
							for (Request* r : s->admitted)
								if (r->state != kIssued) finish(s, r, ps);
							s->admitted.clear();
							s->cvDone.notify_all();
						}
						progress = true;
						break;
					}
		}
		if (!progress) {
			if (s->inflight.empty() && s->pending.empty() && s->admitted.empty())
				s->cvWork.wait(lock, [&] { return s->stop || !s->pending.empty(); });
			else
				s->cvWork.wait_for(lock, std::chrono::microseconds(20));
		}
	}
}

} // namespace

extern "C" void phe_server_default_config(phe_server_config* c)
{
	if (!c) return;
	std::memset(c, 0, sizeof(*c));
	c->memoryBudget = 120ull << 30;
	c->maxInFlight = 256;
	c->renderSlots = 4;
	c->maxRenderPixels = 1920 * 1080;
	c->maxLights = 4;
	c->serial = 0;
	c->batchWindowUs = 0;
}

extern "C" phe_status phe_server_create(const phe_server_config* cfg, phe_server** out)
{
	if (!out) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_create: out is null");
	*out = nullptr;
	phe_server_config c;
	phe_server_default_config(&c);
	if (cfg) c = *cfg;
	if (c.renderSlots == 0 || c.maxInFlight == 0) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_create: zero slots");
	DeviceInfo* d = nullptr;
	phe_status ps = device_info(&d);
	if (ps) return ps;
	phe_server* s = new phe_server();
	s->cfg = c;
	s->device = d->device;
	s->t0 = std::chrono::steady_clock::now();
	cudaError_t e = cudaStreamCreateWithFlags(&s->waveStream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaMalloc(&s->dScenes, 256 * sizeof(DeviceScene));
	for (Wave& w : s->waves) {
		if (e == cudaSuccess) e = cudaMallocHost(&w.hostItems, kMaxWaveItems * sizeof(BatchItemDev));
		if (e == cudaSuccess) e = cudaMalloc(&w.devItems, kMaxWaveItems * sizeof(BatchItemDev) + 256);
		if (e == cudaSuccess) w.counter = (uint32_t*)((char*)w.devItems + kMaxWaveItems * sizeof(BatchItemDev));
		if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming);
	}
	s->slots.resize(c.renderSlots);
	for (RenderSlot& sl : s->slots) {
		if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
		if (e == cudaSuccess) e = cudaMallocHost(&sl.totals, 4 * sizeof(uint64_t));
		if (e != cudaSuccess) break;
		if ((ps = phe_renderer_create(&sl.renderer))) break;
		// Size the slot's buffers once for the largest frame it will serve.
		if ((ps = renderer_reserve(sl.renderer, c.maxRenderPixels, std::max<uint32_t>(1, c.maxLights)))) break;
		// Continuous mode: a render's spp frames overlap two at a time (the same bytes; 2% more served
		// rays/s at 8,000 req/s). The serial baseline renders one frame at a time.
		if (!c.serial && (ps = phe_renderer_set_frames_in_flight(sl.renderer, 2))) break;
	}
	if (e == cudaSuccess && !ps) {
		// Keep freed request memory in the stream-ordered pool instead of returning it to the CUDA driver.
		cudaMemPool_t pool;
		if (cudaDeviceGetDefaultMemPool(&pool, s->device) == cudaSuccess) {
			uint64_t keep = UINT64_MAX;
			cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
		}
	}
	if (e != cudaSuccess || ps) {
		phe_status fs = ps ? ps : cuda_fail(e, "phe_server_create");
		phe_server_destroy(s);   // releases what was made (no worker thread yet)
		return fs;
	}
	s->worker = std::thread(worker_loop, s);
	*out = s;
	return PHE_OK;
}

extern "C" phe_status phe_server_add_scene(phe_server* s, const phe_scene* scene, uint32_t* id)
{
	if (!s || !scene || !id) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_add_scene: null argument");
	std::lock_guard<std::mutex> lock(s->m);
	if (s->scenes.size() >= 256) return fail(PHE_ERR_TOO_LARGE, "phe_server_add_scene: at most 256 scenes");
	if (s->sceneBytes + scene->bytes > s->cfg.memoryBudget)
		return fail(PHE_ERR_BUDGET, "phe_server_add_scene: scenes exceed the memory budget");
	*id = (uint32_t)s->scenes.size();
	s->scenes.push_back(scene);
	s->sceneBytes += scene->bytes;
	s->sceneTableDirty = true;
	return PHE_OK;
}

extern "C" phe_status phe_server_submit(phe_server* s, const phe_request* req, uint64_t* id)
{
	if (!s || !req || !id) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_submit: null argument");
	std::lock_guard<std::mutex> lock(s->m);
	if (req->scene >= s->scenes.size()) return fail(PHE_ERR_NOT_FOUND, "phe_server_submit: unknown scene %u", req->scene);
	if (!req->out) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_submit: out is null");
	Request* r = new Request();
	r->desc = *req;
	if (req->kind == PHE_REQ_RENDER) {
		if (req->resX == 0 || req->resY == 0 || req->resX % 8 || req->resY % 8 || req->spp == 0) {
			delete r;
			return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_submit: render needs a resolution multiple of 8 and spp >= 1");
		}
		if ((uint64_t)req->resX * req->resY > s->cfg.maxRenderPixels || req->resX > 1920) {
			delete r;
			return fail(PHE_ERR_TOO_LARGE, "phe_server_submit: render larger than a render slot (%u pixels)",
			            s->cfg.maxRenderPixels);
		}
		if (req->numLights > s->cfg.maxLights || (req->numLights && !req->lights)) {
			delete r;
			return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_submit: bad light list");
		}
		if (!s->scenes[req->scene]->dev.datas || !s->scenes[req->scene]->dev.materials) {
			delete r;
			return fail(PHE_ERR_INVALID_SCENE, "phe_server_submit: render needs a scene with triangle data and materials");
		}
		r->lights.assign(req->lights, req->lights + req->numLights);
		r->desc.lights = nullptr;
		r->bytes = render_bytes((uint64_t)req->resX * req->resY, std::max<uint32_t>(1, req->numLights), !s->cfg.serial);
	} else if (req->kind == PHE_REQ_CLOSEST || req->kind == PHE_REQ_ANY) {
		if (!req->rays || req->numRays == 0) {
			delete r;
			return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_submit: a query needs rays");
		}
		r->bytes = query_bytes(*req);
	} else {
		delete r;
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_submit: unknown request kind %u", req->kind);
	}
	if (s->sceneBytes + r->bytes > s->cfg.memoryBudget) {
		delete r;
		return fail(PHE_ERR_BUDGET, "phe_server_submit: request needs more than the memory budget");
	}
	r->id = s->nextId++;
	r->tSubmit = now_ms(s->t0);
	s->all[r->id] = r;
	s->pending.push_back(r);
	*id = r->id;
	s->cvWork.notify_one();
	return PHE_OK;
}

static void fill_stats(const Request* r, phe_request_stats* out)
{
	if (!out) return;
	out->submitMs = r->tSubmit;
	out->admitMs = r->tAdmit;
	out->doneMs = r->tDone;
	out->rays = r->rays;
	out->status = r->status;
}

extern "C" phe_status phe_server_poll(phe_server* s, uint64_t id, phe_request_stats* out)
{
	if (!s) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_poll: null server");
	std::lock_guard<std::mutex> lock(s->m);
	auto it = s->all.find(id);
	if (it == s->all.end()) return fail(PHE_ERR_NOT_FOUND, "phe_server_poll: unknown request %llu", (unsigned long long)id);
	if (it->second->state != kDone) return PHE_ERR_NOT_READY;
	fill_stats(it->second, out);
	return PHE_OK;
}

extern "C" phe_status phe_server_wait(phe_server* s, uint64_t id, phe_request_stats* out)
{
	if (!s) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_wait: null server");
	std::unique_lock<std::mutex> lock(s->m);
	auto it = s->all.find(id);
	if (it == s->all.end()) return fail(PHE_ERR_NOT_FOUND, "phe_server_wait: unknown request %llu", (unsigned long long)id);
	Request* r = it->second;
	s->cvDone.wait(lock, [&] { return r->state == kDone; });
	fill_stats(r, out);
	if (r->status != PHE_OK) return fail(r->status, "request %llu failed: %s", (unsigned long long)id, r->error.c_str());
	return PHE_OK;
}

extern "C" phe_status phe_server_drain(phe_server* s)
{
	if (!s) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_drain: null server");
	std::unique_lock<std::mutex> lock(s->m);
	s->cvDone.wait(lock, [&] { return s->pending.empty() && s->admitted.empty() && s->inflight.empty(); });
	return PHE_OK;
}

extern "C" phe_status phe_server_release(phe_server* s, uint64_t id)
{
	if (!s) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_release: null server");
	std::lock_guard<std::mutex> lock(s->m);
	auto it = s->all.find(id);
	if (it == s->all.end()) return fail(PHE_ERR_NOT_FOUND, "phe_server_release: unknown request");
	if (it->second->state != kDone) return fail(PHE_ERR_NOT_READY, "phe_server_release: request still running");
	delete it->second;
	s->all.erase(it);
	return PHE_OK;
}

extern "C" phe_status phe_server_cancel(phe_server* s, uint64_t id)
{
	if (!s) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_cancel: null server");
	std::lock_guard<std::mutex> lock(s->m);
	auto it = s->all.find(id);
	if (it == s->all.end()) return fail(PHE_ERR_NOT_FOUND, "phe_server_cancel: unknown request");
	Request* r = it->second;
	if (r->state == kDone) return r->status == PHE_ERR_CANCELLED ? PHE_OK : fail(PHE_ERR_NOT_READY, "phe_server_cancel: request already completed");
	auto p = std::find(s->pending.begin(), s->pending.end(), r);
	if (r->state != kPending || p == s->pending.end())
		return fail(PHE_ERR_NOT_READY, "phe_server_cancel: request already admitted");
	s->pending.erase(p);
	r->status = PHE_ERR_CANCELLED;
	r->error = "cancelled before admission";
	r->tDone = now_ms(s->t0);
	r->state = kDone;
	s->cvDone.notify_all();
	s->cvWork.notify_one();
	return PHE_OK;
}

extern "C" phe_status phe_server_get_stats(phe_server* s, phe_server_stats* out)
{
	if (!s || !out) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_server_get_stats: null argument");
	std::lock_guard<std::mutex> lock(s->m);
	out->waves = s->wavesLaunched;
	out->raysCompleted = s->raysCompleted;
	out->bytesInUse = s->bytesInUse + s->sceneBytes;
	out->pending = (uint32_t)s->pending.size();
	out->inFlight = (uint32_t)(s->inflight.size() + s->admitted.size());
	return PHE_OK;
}

extern "C" phe_status phe_server_destroy(phe_server* s)
{
	if (!s) return PHE_OK;
	{
		std::lock_guard<std::mutex> lock(s->m);
		s->stop = true;
		s->cvWork.notify_all();
	}
	if (s->worker.joinable()) s->worker.join();
	cudaDeviceSynchronize();
	for (auto& kv : s->all) delete kv.second;
	for (RenderSlot& sl : s->slots) {
		if (sl.renderer) phe_renderer_destroy(sl.renderer);
		if (sl.stream) cudaStreamDestroy(sl.stream);
		if (sl.totals) cudaFreeHost(sl.totals);
	}
	for (Wave& w : s->waves) {
		if (w.hostItems) cudaFreeHost(w.hostItems);
		if (w.devItems) cudaFree(w.devItems);
		if (w.done) cudaEventDestroy(w.done);
	}
	for (cudaEvent_t e : s->eventPool) cudaEventDestroy(e);
	if (s->dScenes) cudaFree(s->dScenes);
	if (s->waveStream) cudaStreamDestroy(s->waveStream);
	delete s;
	return PHE_OK;
}
