// Batched multi-scene ray casting: many ray batches of uneven sizes over several resident scenes,
// closest-hit and any-hit mixed, in ONE persistent launch (replayed from a CUDA graph). The
// reference has no counterpart: it launches one kernel per batch and synchronises the device after
// each (RayCastKernel.cu:806-886).
//
// Work layout: batch i owns the global ray indices [base_i, base_i + count_i) with every base a
// multiple of 32, so a warp's 32-ray fetch never straddles two batches: scene, query kind and
// buffers are warp-uniform. Warps take 32-ray chunks from one atomic counter; the batch of a chunk
// is found by binary search over the bases.
//
// Launch parameters (block size, resident blocks per SM, batch order) come from phe_batch_params,
// which the autotuner (phe_batch_autotune) picks by timing candidates on the actual batch mix.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "batch.cuh"
#include "octant_sort.cuh"
#include "runtime.cuh"
#include "traverse.cuh"

namespace phe_gb300 {

struct BatchTableDev {
	const BatchItemDev* items;
	const DeviceScene* scenes;
	uint32_t numItems;
	uint32_t totalPadded;
	const uint32_t* perm;   // ray-sort permutation: global index -> item-local ray index (null: identity)
};

// Shared-memory depth of the traversal stack the autotuner may pick besides 0.
constexpr int kBatchStackShared = 16;

__device__ __forceinline__ uint32_t find_item(const BatchItemDev* __restrict__ items, uint32_t n, uint32_t g)
{
	uint32_t lo = 0, hi = n;  // largest i with base_i <= g
	while (hi - lo > 1) {
		uint32_t mid = (lo + hi) >> 1;
		if (__ldg(&items[mid].base) <= g) lo = mid;
		else hi = mid;
	}
	return lo;
}

// Compiled for 1,280 resident threads per SM (48 registers), like the frame's bounce kernel: on the
// uneven-batch mix over 10K..2M-triangle scenes 2.553 ms vs 2.617 ms with the compiler's own budget
// (48-56 registers), and 2.932 ms at 40 registers (spills); the autotuner then picks the resident
// blocks below that limit.
// Traversal errors (stack overflow; an index outside its array in the checked build) are ORed into the
// status word of the item's scene, which phe_scene_status reads.
constexpr int kBatchThreadsPerSM = 1280;
template <int BLOCK, bool WIDE, int SN>
__global__ void __launch_bounds__(BLOCK, kBatchThreadsPerSM / BLOCK) batch_kernel(BatchTableDev t, uint32_t* __restrict__ counter)
{
	const uint32_t lane = threadIdx.x & 31u;
	for (;;) {
		uint32_t g = 0;
		if (lane == 0) g = atomicAdd(counter, 32u);
		g = __shfl_sync(0xFFFFFFFFu, g, 0);
		if (g >= t.totalPadded) break;
		uint32_t it = find_item(t.items, t.numItems, g);
		const BatchItemDev item = t.items[it];
		uint32_t i = g - item.base + lane;
		if (i < item.count) {
			if (t.perm) i = __ldg(t.perm + g + lane);   // the ray traced at this slot after sorting
			const DeviceScene s = t.scenes[item.scene];
			RayState r = load_ray(item.rays, i);
			HitRecord h = empty_hit(r);
			uint32_t err;
			if (item.kind == 0) {
				err = trace<false, WIDE, SN>(s, r, h);
				store_hit((phe_ray_hit*)item.out, i, r, h);
			} else {
				err = trace<true, WIDE, SN>(s, r, h);
				((uint8_t*)item.out)[i] = h.slot == ~0u ? 1 : 0;
			}
			if (err) atomicOr(s.status, err);
		}
		__syncwarp();
	}
}

// `wide` selects the instantiation with the 4-wide traversal (for scene tables holding 4-wide scenes),
// `stackShared` (0 or kBatchStackShared) the one keeping that many stack entries in shared memory.
template <int BLOCK>
static phe_status launch_batch_kernel(const BatchTableDev& t, bool wide, int stackShared, int blocksPerSM, int numSMs,
                                      uint32_t* counter, cudaStream_t stream, int* occupancyOut)
{
	const bool sh = stackShared > 0;
	auto kernel = wide ? (sh ? batch_kernel<BLOCK, true, kBatchStackShared> : batch_kernel<BLOCK, true, 0>)
	                   : (sh ? batch_kernel<BLOCK, false, kBatchStackShared> : batch_kernel<BLOCK, false, 0>);
	const size_t smem = stack_smem_bytes(BLOCK, sh ? kBatchStackShared : 0);
	int maxB = 0;
	PHE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxB, kernel, BLOCK, smem), "occupancy");
	if (occupancyOut) {
		*occupancyOut = maxB;
		return PHE_OK;
	}
	int b = blocksPerSM > 0 ? std::min(blocksPerSM, maxB) : maxB;
	if (b < 1) b = 1;
	uint32_t grid = (uint32_t)(b * numSMs);
	uint32_t need = (t.totalPadded + BLOCK - 1) / BLOCK;
	if (grid > need) grid = need > 0 ? need : 1;
	kernel<<<grid, BLOCK, smem, stream>>>(t, counter);
	PHE_CUDA_TRY(cudaGetLastError(), "batch_kernel launch");
	return PHE_OK;
}

// Ray-sort granularity: one block per window of W consecutive rays of one item (the item of window w
// is the last one whose first window is <= w) sorts the window by direction octant (stable) and writes
// perm[item.base + w0 + position] = item-local index of the ray traced there.
__global__ void __launch_bounds__(kOctantBlock) batch_sort_kernel(BatchTableDev t, const uint32_t* __restrict__ windowStart,
                                                                 uint32_t numWindows, int W, uint32_t* __restrict__ perm)
{
	__shared__ uint32_t cnt[8][kOctantBlock];
	__shared__ uint32_t bucketBase[8];
	const int per = W / kOctantBlock;
	const int tid = threadIdx.x;
	for (uint32_t w = blockIdx.x; w < numWindows; w += gridDim.x) {
		uint32_t lo = 0, hi = t.numItems;
		while (hi - lo > 1) {
			uint32_t mid = (lo + hi) >> 1;
			if (__ldg(windowStart + mid) <= w) lo = mid;
			else hi = mid;
		}
		const BatchItemDev item = t.items[lo];
		const uint32_t w0 = (w - __ldg(windowStart + lo)) * (uint32_t)W;
		const uint32_t n = min((uint32_t)W, item.count - w0);
		uint8_t keys[kMaxOctantWindow / kOctantBlock];
		for (int k = 0; k < per; k++) {
			uint32_t j = (uint32_t)(tid * per + k);
			keys[k] = j < n ? octant_key(__ldg(reinterpret_cast<const float4*>(item.rays + w0 + j) + 1)) : (uint8_t)0xFF;
		}
		uint32_t rank[8];
		octant_ranks(keys, per, cnt, bucketBase, rank);
		for (int k = 0; k < per; k++)
			if (keys[k] != 0xFF) perm[item.base + w0 + rank[keys[k]]++] = w0 + (uint32_t)(tid * per + k);
	}
}

phe_status launch_batch_table(const BatchItemDev* items, uint32_t numItems, uint32_t totalPadded,
                              const DeviceScene* scenes, uint32_t* counter, int blockSize, int blocksPerSM,
                              cudaStream_t stream, bool wide)
{
	DeviceInfo* d = nullptr;
	phe_status st = device_info(&d);
	if (st) return st;
	if (totalPadded == 0) return PHE_OK;
	BatchTableDev t{items, scenes, numItems, totalPadded, nullptr};
	switch (blockSize) {
	case 64: return launch_batch_kernel<64>(t, wide, 0, blocksPerSM, d->numSMs, counter, stream, nullptr);
	case 256: return launch_batch_kernel<256>(t, wide, 0, blocksPerSM, d->numSMs, counter, stream, nullptr);
	default: return launch_batch_kernel<128>(t, wide, 0, blocksPerSM, d->numSMs, counter, stream, nullptr);
	}
}

} // namespace phe_gb300

using namespace phe_gb300;

struct phe_batch {
	std::vector<phe_batch_item> items;     // as given
	std::vector<uint32_t> order;           // launch order of the items
	std::vector<DeviceScene> scenes;
	std::vector<const phe_scene*> sceneHandles;
	phe_batch_params params{};
	void* allocation = nullptr;            // items table + scene table + counter
	BatchItemDev* dItems = nullptr;
	DeviceScene* dScenes = nullptr;
	uint32_t* dCounter = nullptr;
	uint32_t totalPadded = 0;
	uint64_t totalRays = 0;
	cudaGraphExec_t graph = nullptr;
	// The last phe_batch_launch, which may still read the tables on its stream when they are rewritten.
	cudaEvent_t launchDone = nullptr;
	bool launchPending = false;
	// Ray sorting (params.sortWindow > 0): window table of the item order and the permutation.
	uint32_t* dPerm = nullptr;             // [totalPadded]
	uint32_t* dWindowStart = nullptr;      // [items + 1]
	uint32_t numWindows = 0;
	size_t permCapacity = 0, windowCapacity = 0;
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

extern "C" void phe_batch_default_params(phe_batch_params* p)
{
	if (!p) return;
	std::memset(p, 0, sizeof(*p));
	p->blockSize = 128;
	p->blocksPerSM = 0;
	p->order = PHE_BATCH_ORDER_GIVEN;
	p->useGraph = 1;
	p->layout = PHE_LAYOUT_BINARY;
	p->stackShared = 0;
	p->sortWindow = 0;
}

static phe_status check_params(const phe_batch_params* p)
{
	if (p->blockSize != 64 && p->blockSize != 128 && p->blockSize != 256)
		return fail(PHE_ERR_INVALID_ARGUMENT, "batch block size must be 64, 128 or 256");
	if (p->stackShared != 0 && p->stackShared != kBatchStackShared)
		return fail(PHE_ERR_INVALID_ARGUMENT, "batch stackShared must be 0 or %d", kBatchStackShared);
	if (p->sortWindow != 0 && (p->sortWindow < kOctantBlock || p->sortWindow > kMaxOctantWindow ||
	                           p->sortWindow % kOctantBlock))
		return fail(PHE_ERR_INVALID_ARGUMENT, "batch sortWindow must be 0 or a multiple of %d up to %d", kOctantBlock,
		            kMaxOctantWindow);
	if (p->layout != PHE_LAYOUT_BINARY && p->layout != PHE_LAYOUT_WIDE4 && p->layout != PHE_LAYOUT_WIDE8)
		return fail(PHE_ERR_INVALID_ARGUMENT, "batch layout must be PHE_LAYOUT_BINARY, PHE_LAYOUT_WIDE4 or PHE_LAYOUT_WIDE8");
	return PHE_OK;
}

static phe_status upload_table(phe_batch* b)
{
	// The tables are rewritten in place: after the last launch that reads them, on whichever stream.
	if (b->launchPending) {
		PHE_CUDA_TRY(cudaEventSynchronize(b->launchDone), "wait for the last batch launch");
		b->launchPending = false;
	}
	// Launch order.
	const size_t n = b->items.size();
	b->order.resize(n);
	for (size_t i = 0; i < n; i++) b->order[i] = (uint32_t)i;
	if (b->params.order == PHE_BATCH_ORDER_LARGEST_FIRST) {
		// Estimated cost: rays x log2(scene size); heavy batches first so the tail is made of small ones.
		auto cost = [&](uint32_t i) {
			const phe_batch_item& it = b->items[i];
			double tri = (double)b->scenes[it.scene].numSlots;
			return (double)it.count * std::log2(tri + 2.0) * (it.kind == PHE_QUERY_ANY ? 0.6 : 1.0);
		};
		std::stable_sort(b->order.begin(), b->order.end(), [&](uint32_t a, uint32_t c) { return cost(a) > cost(c); });
	}
	std::vector<BatchItemDev> dev(n);
	uint32_t base = 0;
	uint64_t total = 0;
	for (size_t k = 0; k < n; k++) {
		const phe_batch_item& it = b->items[b->order[k]];
		dev[k].scene = it.scene;
		dev[k].kind = it.kind;
		dev[k].count = it.count;
		dev[k].base = base;
		dev[k].rays = it.rays;
		dev[k].out = it.out;
		uint64_t next = (uint64_t)base + ((uint64_t)it.count + 31u) / 32u * 32u;
		if (next > kMaxPersistentRays)
			return fail(PHE_ERR_TOO_LARGE, "batch: more than %u rays (padded) in one launch", kMaxPersistentRays);
		base = (uint32_t)next;
		total += it.count;
	}
	b->totalPadded = base;
	b->totalRays = total;
	PHE_CUDA_TRY(cudaMemcpy(b->dItems, dev.data(), n * sizeof(BatchItemDev), cudaMemcpyHostToDevice), "upload batch table");
	std::vector<DeviceScene> st(b->sceneHandles.size());
	for (size_t i = 0; i < st.size(); i++) {
		const phe_scene* sc = b->sceneHandles[i];
		st[i] = sc->dev;
		st[i].nodes4 = b->params.layout == PHE_LAYOUT_WIDE4 ? sc->nodes4 : nullptr;
		st[i].nodes8 = b->params.layout == PHE_LAYOUT_WIDE8 ? sc->nodes8 : nullptr;
		st[i].leaves8 = b->params.layout == PHE_LAYOUT_WIDE8 ? sc->leaves8 : nullptr;
	}
	if (!st.empty())
		PHE_CUDA_TRY(cudaMemcpy(b->dScenes, st.data(), st.size() * sizeof(DeviceScene), cudaMemcpyHostToDevice),
		             "upload scene table");
	b->numWindows = 0;
	if (b->params.sortWindow > 0) {
		const uint32_t W = (uint32_t)b->params.sortWindow;
		std::vector<uint32_t> ws(n + 1);
		uint32_t acc = 0;
		for (size_t k = 0; k < n; k++) {
			ws[k] = acc;
			acc += (dev[k].count + W - 1) / W;
		}
		ws[n] = acc;
		b->numWindows = acc;
		if (b->permCapacity < b->totalPadded || !b->dPerm) {
			if (b->dPerm) cudaFree(b->dPerm);
			b->dPerm = nullptr;
			b->permCapacity = 0;
			PHE_CUDA_TRY(cudaMalloc(&b->dPerm, std::max<size_t>(1, b->totalPadded) * sizeof(uint32_t)),
			             "cudaMalloc(batch ray permutation)");
			b->permCapacity = std::max<size_t>(1, b->totalPadded);
		}
		if (b->windowCapacity < n + 1 || !b->dWindowStart) {
			if (b->dWindowStart) cudaFree(b->dWindowStart);
			b->dWindowStart = nullptr;
			b->windowCapacity = 0;
			PHE_CUDA_TRY(cudaMalloc(&b->dWindowStart, (n + 1) * sizeof(uint32_t)), "cudaMalloc(batch sort windows)");
			b->windowCapacity = n + 1;
		}
		PHE_CUDA_TRY(cudaMemcpy(b->dWindowStart, ws.data(), (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice),
		             "upload batch sort windows");
	}
	if (b->graph) {
		cudaGraphExecDestroy(b->graph);
		b->graph = nullptr;
	}
	return finish_uploads("upload batch tables");
}

static phe_status check_items(const phe_batch_item* items, uint32_t numItems, uint32_t numScenes)
{
	for (uint32_t i = 0; i < numItems; i++) {
		const phe_batch_item& it = items[i];
		if (it.scene >= numScenes) return fail(PHE_ERR_NOT_FOUND, "batch item %u: scene %u out of range", i, it.scene);
		if (it.kind != PHE_QUERY_CLOSEST && it.kind != PHE_QUERY_ANY)
			return fail(PHE_ERR_INVALID_ARGUMENT, "batch item %u: kind must be closest or any", i);
		if (it.count && (!it.rays || !it.out)) return fail(PHE_ERR_INVALID_ARGUMENT, "batch item %u: null buffer", i);
		if (((uintptr_t)it.rays & 15u) || (it.kind == PHE_QUERY_CLOSEST && ((uintptr_t)it.out & 15u)))
			return fail(PHE_ERR_INVALID_ARGUMENT, "batch item %u: buffers must be 16-byte aligned", i);
	}
	return PHE_OK;
}

extern "C" phe_status phe_batch_create(const phe_scene* const* scenes, uint32_t numScenes, const phe_batch_item* items,
                                       uint32_t numItems, const phe_batch_params* params, phe_batch** out)
{
	if (!out || !scenes || numScenes == 0 || (!items && numItems))
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_create: null argument");
	*out = nullptr;
	for (uint32_t i = 0; i < numScenes; i++)
		if (!scenes[i]) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_create: scene %u is null", i);
	phe_status st = check_items(items, numItems, numScenes);
	if (st) return st;
	if (params && (st = check_params(params))) return st;
	DeviceInfo* d = nullptr;
	if ((st = device_info(&d))) return st;
	for (uint32_t i = 0; i < numScenes; i++)
		if (scenes[i]->device != d->device)
			return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_create: scene %u lives on device %d, not on the current device %d",
			            i, scenes[i]->device, d->device);
	phe_batch* b = new phe_batch();
	if (params) b->params = *params;
	else phe_batch_default_params(&b->params);
	b->items.assign(items, items + numItems);
	for (uint32_t i = 0; i < numScenes; i++) {
		b->scenes.push_back(scenes[i]->dev);
		b->sceneHandles.push_back(scenes[i]);
	}
	size_t itemBytes = align256(std::max<size_t>(1, numItems) * sizeof(BatchItemDev));
	size_t sceneBytes = align256(numScenes * sizeof(DeviceScene));
	char* base = nullptr;
	cudaError_t e = cudaMalloc(&base, itemBytes + sceneBytes + 256);
	if (e != cudaSuccess) {
		delete b;
		return cuda_fail(e, "cudaMalloc(batch)");
	}
	b->allocation = base;
	if ((e = cudaEventCreateWithFlags(&b->launchDone, cudaEventDisableTiming)) != cudaSuccess) {
		cudaFree(base);
		delete b;
		return cuda_fail(e, "create batch event");
	}
	b->dItems = (BatchItemDev*)base;
	b->dScenes = (DeviceScene*)(base + itemBytes);
	b->dCounter = (uint32_t*)(base + itemBytes + sceneBytes);
	cudaMemset(b->dCounter, 0, 256);
	e = cudaMemcpy(b->dScenes, b->scenes.data(), numScenes * sizeof(DeviceScene), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		phe_batch_destroy(b);
		return cuda_fail(e, "upload scene table");
	}
	if ((st = upload_table(b))) {
		phe_batch_destroy(b);
		return st;
	}
	*out = b;
	return PHE_OK;
}

extern "C" phe_status phe_batch_update(phe_batch* b, const phe_batch_item* items, uint32_t numItems)
{
	if (!b || (!items && numItems)) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_update: null argument");
	if (numItems != b->items.size()) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_update: item count changed");
	phe_status st = check_items(items, numItems, (uint32_t)b->scenes.size());
	if (st) return st;
	b->items.assign(items, items + numItems);
	return upload_table(b);
}

static phe_status batch_enqueue(phe_batch* b, cudaStream_t stream)
{
	DeviceInfo* d = nullptr;
	phe_status st = device_info(&d);
	if (st) return st;
	const bool sorted = b->params.sortWindow > 0 && b->numWindows > 0;
	BatchTableDev t{b->dItems, b->dScenes, (uint32_t)b->items.size(), b->totalPadded, sorted ? b->dPerm : nullptr};
	PHE_CUDA_TRY(cudaMemsetAsync(b->dCounter, 0, sizeof(uint32_t), stream), "clear batch counter");
	if (b->totalPadded == 0) return PHE_OK;
	if (sorted) {
		uint32_t grid = std::min<uint32_t>(b->numWindows, (uint32_t)d->numSMs * 8u);
		batch_sort_kernel<<<grid, kOctantBlock, 0, stream>>>(t, b->dWindowStart, b->numWindows, b->params.sortWindow,
		                                                    b->dPerm);
		PHE_CUDA_TRY(cudaGetLastError(), "batch_sort_kernel launch");
	}
	const bool wide = b->params.layout == PHE_LAYOUT_WIDE4 || b->params.layout == PHE_LAYOUT_WIDE8;
	const int sh = b->params.stackShared;
	switch (b->params.blockSize) {
	case 64: return launch_batch_kernel<64>(t, wide, sh, b->params.blocksPerSM, d->numSMs, b->dCounter, stream, nullptr);
	case 256: return launch_batch_kernel<256>(t, wide, sh, b->params.blocksPerSM, d->numSMs, b->dCounter, stream, nullptr);
	case 128: return launch_batch_kernel<128>(t, wide, sh, b->params.blocksPerSM, d->numSMs, b->dCounter, stream, nullptr);
	default: return fail(PHE_ERR_INVALID_ARGUMENT, "batch block size must be 64, 128 or 256");
	}
}

extern "C" phe_status phe_batch_launch(phe_batch* b, void* stream)
{
	if (!b) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_launch: null batch");
	NvtxRange range("phe_batch_launch");
	cudaStream_t s = (cudaStream_t)stream;
	if (!b->params.useGraph) {
		phe_status st = batch_enqueue(b, s);
		if (st) return st;
		PHE_CUDA_TRY(cudaEventRecord(b->launchDone, s), "record batch launch");
		b->launchPending = true;
		return PHE_OK;
	}
	if (!b->graph) {
		// Resolve occupancy outside capture.
		int occ = 0;
		BatchTableDev t{};
		const bool wide = b->params.layout == PHE_LAYOUT_WIDE4 || b->params.layout == PHE_LAYOUT_WIDE8;
		const int sh = b->params.stackShared;
		switch (b->params.blockSize) {
		case 64: launch_batch_kernel<64>(t, wide, sh, 0, 1, nullptr, nullptr, &occ); break;
		case 256: launch_batch_kernel<256>(t, wide, sh, 0, 1, nullptr, nullptr, &occ); break;
		default: launch_batch_kernel<128>(t, wide, sh, 0, 1, nullptr, nullptr, &occ); break;
		}
		cudaStream_t cap = nullptr;
		PHE_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "create capture stream");
		cudaGraph_t g = nullptr;
		cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
		phe_status st = PHE_OK;
		if (e == cudaSuccess) {
			st = batch_enqueue(b, cap);
			e = cudaStreamEndCapture(cap, &g);
		}
		cudaStreamDestroy(cap);
		if (st) { if (g) cudaGraphDestroy(g); return st; }
		if (e != cudaSuccess) return cuda_fail(e, "capture batch graph");
		e = cudaGraphInstantiate(&b->graph, g, 0);
		cudaGraphDestroy(g);
		if (e != cudaSuccess) return cuda_fail(e, "instantiate batch graph");
	}
	PHE_CUDA_TRY(cudaGraphLaunch(b->graph, s), "launch batch graph");
	PHE_CUDA_TRY(cudaEventRecord(b->launchDone, s), "record batch launch");
	b->launchPending = true;
	return PHE_OK;
}

extern "C" phe_status phe_batch_set_params(phe_batch* b, const phe_batch_params* params)
{
	if (!b || !params) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_set_params: null argument");
	phe_status st = check_params(params);
	if (st) return st;
	b->params = *params;
	return upload_table(b);
}

extern "C" phe_status phe_batch_info(const phe_batch* b, uint64_t* totalRays, uint32_t* paddedRays)
{
	if (!b) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_info: null batch");
	if (totalRays) *totalRays = b->totalRays;
	if (paddedRays) *paddedRays = b->totalPadded;
	return PHE_OK;
}

extern "C" phe_status phe_batch_destroy(phe_batch* b)
{
	if (!b) return PHE_OK;
	if (b->graph) cudaGraphExecDestroy(b->graph);
	if (b->dPerm) cudaFree(b->dPerm);
	if (b->dWindowStart) cudaFree(b->dWindowStart);
	cudaFree(b->allocation);
	if (b->launchDone) cudaEventDestroy(b->launchDone);
	delete b;
	return PHE_OK;
}

// ------------------------------------------------------------------------------------------------
// Autotuner: times every candidate launch configuration on the batch as given (after a warm-up
// launch each) with CUDA events on `stream`, keeps the fastest, and leaves it set on the batch.
// ------------------------------------------------------------------------------------------------

extern "C" phe_status phe_batch_autotune(phe_batch* b, int repeats, void* stream, phe_batch_params* best,
                                         float* bestMs, phe_batch_tuning_row* rows, uint32_t maxRows, uint32_t* numRows)
{
	if (!b) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_autotune: null batch");
	if (repeats < 1) repeats = 3;
	cudaStream_t s = (cudaStream_t)stream;
	DeviceInfo* d = nullptr;
	phe_status st = device_info(&d);
	if (st) return st;
	const int blocks[] = {64, 128, 256};
	const int orders[] = {PHE_BATCH_ORDER_GIVEN, PHE_BATCH_ORDER_LARGEST_FIRST};
	const int occFrac[] = {4, 3, 2};  // quarters of the occupancy limit: 4/4, 3/4, 2/4
	const int layouts[] = {PHE_LAYOUT_BINARY, PHE_LAYOUT_WIDE4, PHE_LAYOUT_WIDE8};
	const int stacks[] = {0, kBatchStackShared};
	const int sorts[] = {0, 1024, 4096};
	// Candidates are timed from a cold L2 (the condition of a batch that arrives after other work): a
	// write of twice the L2 size before each timed launch, outside the timed interval.
	int l2 = 0;
	PHE_CUDA_TRY(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, d->device), "L2 size");
	const size_t flushBytes = std::max<size_t>((size_t)l2 * 2, (size_t)64 << 20);
	void* flush = nullptr;
	PHE_CUDA_TRY(cudaMalloc(&flush, flushBytes), "cudaMalloc(autotune L2 flush)");
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
		cudaFree(flush);
		if (e0) cudaEventDestroy(e0);
		return cuda_fail(cudaGetLastError(), "cudaEventCreate");
	}
	phe_batch_params saved = b->params;
	phe_batch_params winner = saved;
	float winnerMs = 1e30f;
	uint32_t n = 0;
	for (int bs : blocks) {
		int occ = 0;
		BatchTableDev t{};
		if (bs == 64) launch_batch_kernel<64>(t, false, 0, 0, 1, nullptr, nullptr, &occ);
		else if (bs == 128) launch_batch_kernel<128>(t, false, 0, 0, 1, nullptr, nullptr, &occ);
		else launch_batch_kernel<256>(t, false, 0, 0, 1, nullptr, nullptr, &occ);
		for (int ord : orders)
			for (int q : occFrac)
				for (int lay : layouts)
				for (int sh : stacks)
				for (int sw : sorts) {
				phe_batch_params p = saved;
				p.blockSize = bs;
				p.order = ord;
				p.blocksPerSM = std::max(1, occ * q / 4);
				p.useGraph = 0;
				p.layout = lay;
				p.stackShared = sh;
				p.sortWindow = sw;
				b->params = p;
				if ((st = upload_table(b))) goto done;
				if ((st = batch_enqueue(b, s))) goto done;  // warm-up
				float ms = 0;
				for (int r = 0; r < repeats; r++) {
					cudaMemsetAsync(flush, r & 1, flushBytes, s);
					cudaEventRecord(e0, s);
					if ((st = batch_enqueue(b, s))) goto done;
					cudaEventRecord(e1, s);
					cudaError_t ce = cudaEventSynchronize(e1);
					if (ce != cudaSuccess) {
						st = cuda_fail(ce, "autotune sync");
						goto done;
					}
					float one = 0;
					cudaEventElapsedTime(&one, e0, e1);
					ms += one;
				}
				ms /= (float)repeats;
				if (rows && n < maxRows) {
					rows[n].params = p;
					rows[n].ms = ms;
				}
				n++;
				if (ms < winnerMs) {
					winnerMs = ms;
					winner = p;
				}
			}
	}
done:
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(flush);
	if (st) {
		b->params = saved;
		upload_table(b);
		return st;
	}
	winner.useGraph = saved.useGraph;
	b->params = winner;
	if ((st = upload_table(b))) return st;
	if (best) *best = winner;
	if (bestMs) *bestMs = winnerMs;
	if (numRows) *numRows = n;
	return PHE_OK;
}

// ------------------------------------------------------------------------------------------------
// phe_batch_cast_noalloc: the batched launch for callers that must not allocate device memory.
//
// Some callers own every byte of device memory through their own allocator or memory budget (a game
// engine's renderer, a plugin host) and do not let a library call cudaMalloc: it can block until the
// whole device is idle and it takes memory outside their accounting. For them this entry point keeps
// its scratch (the batch descriptor table, the scene table and the work counter) in the fixed array
// below, which lives in the library image. The caller passes the scenes, rays and output buffers as
// usual.
//
// The host builds the two tables on its stack and hands them to a one-block staging kernel as its
// by-value (__grid_constant__) parameter; the staging kernel copies them into the array and clears
// the counter, and the batch kernel then runs from the array. No host-to-device copy is queued, so
// nothing waits for pageable memory and the call returns as soon as both kernels are queued.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxItems batches and kNoAllocMaxScenes scenes per call (12,544 bytes of scratch,
//     held by every GPU that loads the library until the process exits); larger calls fail with
//     PHE_ERR_TOO_LARGE;
//   * every call uses the same array and leaves its tables there; the counter is cleared at the start
//     of each call. Two calls whose work overlaps on the GPU (for example on two streams at once) race
//     on the array: serialise them on one stream;
//   * traversal errors are ORed into each scene's own status word (phe_scene_status), not kept in the
//     array;
//   * the first call on a device looks up the array's device address for that device (the call
//     must be made with that device current); make that first call before any stream capture.
// ------------------------------------------------------------------------------------------------

namespace phe_gb300 {

constexpr uint32_t kNoAllocMaxItems = 256;
constexpr uint32_t kNoAllocMaxScenes = 32;
constexpr size_t kNoAllocItemsBytes = kNoAllocMaxItems * sizeof(BatchItemDev);          // 8192
constexpr size_t kNoAllocScenesBytes = kNoAllocMaxScenes * sizeof(DeviceScene);         // 4096
constexpr size_t kNoAllocScratchBytes = kNoAllocItemsBytes + kNoAllocScenesBytes + 256; // + counter
static_assert(sizeof(DeviceScene) % 16 == 0, "scene table entries stay 16-byte aligned");
static_assert(kNoAllocScratchBytes == 12544, "the documented scratch size");

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

// Both tables as one kernel parameter (12,288 bytes, inside the 32,764-byte limit of kernel parameters).
struct NoAllocTables {
	BatchItemDev items[kNoAllocMaxItems];
	DeviceScene scenes[kNoAllocMaxScenes];
};
static_assert(sizeof(NoAllocTables) == kNoAllocItemsBytes + kNoAllocScenesBytes, "tables fill the scratch head");
static_assert(sizeof(NoAllocTables) % 16 == 0, "tables copy as 16-byte words");

constexpr int kNoAllocStageBlock = 256;

// Copies the used part of both tables from the parameter into the scratch and clears the counter.
// `scratch` is the array's device address looked up by the host.
__global__ void __launch_bounds__(kNoAllocStageBlock) noalloc_stage_kernel(const __grid_constant__ NoAllocTables tab,
                                                                          uint32_t numItems, uint32_t numScenes,
                                                                          unsigned char* __restrict__ scratch)
{
	const uint4* src = reinterpret_cast<const uint4*>(&tab);
	uint4* dst = reinterpret_cast<uint4*>(scratch);
	const uint32_t itemWords = numItems * (uint32_t)(sizeof(BatchItemDev) / 16);
	const uint32_t sceneWords = numScenes * (uint32_t)(sizeof(DeviceScene) / 16);
	const uint32_t sceneFirst = (uint32_t)(kNoAllocItemsBytes / 16);
	for (uint32_t k = threadIdx.x; k < itemWords; k += blockDim.x) dst[k] = src[k];
	for (uint32_t k = threadIdx.x; k < sceneWords; k += blockDim.x) dst[sceneFirst + k] = src[sceneFirst + k];
	if (threadIdx.x == 0) *reinterpret_cast<uint32_t*>(scratch + kNoAllocItemsBytes + kNoAllocScenesBytes) = 0u;
}

static std::mutex g_noallocMutex;
static unsigned char* g_noallocAddr[64] = {};   // device address of g_noallocScratch, per device

// Looks up (once per device) the device address of the scratch array on the current device.
static phe_status noalloc_scratch(int dev, unsigned char** out)
{
	if (dev < 0 || dev >= 64) return fail(PHE_ERR_NO_DEVICE, "device ordinal %d out of range", dev);
	std::lock_guard<std::mutex> lock(g_noallocMutex);
	if (!g_noallocAddr[dev]) {
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
		if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
		g_noallocAddr[dev] = (unsigned char*)p;
	}
	*out = g_noallocAddr[dev];
	return PHE_OK;
}

} // namespace phe_gb300

extern "C" phe_status phe_batch_cast_noalloc(const phe_scene* const* scenes, uint32_t numScenes,
                                             const phe_batch_item* items, uint32_t numItems, void* stream)
{
	if (!scenes || numScenes == 0 || (!items && numItems))
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_cast_noalloc: null argument");
	if (numItems > kNoAllocMaxItems)
		return fail(PHE_ERR_TOO_LARGE, "phe_batch_cast_noalloc: %u batches, at most %u fit the fixed scratch", numItems,
		            kNoAllocMaxItems);
	if (numScenes > kNoAllocMaxScenes)
		return fail(PHE_ERR_TOO_LARGE, "phe_batch_cast_noalloc: %u scenes, at most %u fit the fixed scratch", numScenes,
		            kNoAllocMaxScenes);
	for (uint32_t i = 0; i < numScenes; i++)
		if (!scenes[i]) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_cast_noalloc: scene %u is null", i);
	phe_status st = check_items(items, numItems, numScenes);
	if (st) return st;
	// Padded ray total (a warp's 32-ray fetch never straddles two batches).
	uint64_t total = 0;
	for (uint32_t k = 0; k < numItems; k++) {
		total += ((uint64_t)items[k].count + 31u) / 32u * 32u;
		if (total > kMaxPersistentRays)
			return fail(PHE_ERR_TOO_LARGE, "phe_batch_cast_noalloc: more than %u rays (padded)", kMaxPersistentRays);
	}
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return fail(PHE_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
	for (uint32_t i = 0; i < numScenes; i++)
		if (scenes[i]->device != dev)
			return fail(PHE_ERR_INVALID_ARGUMENT, "phe_batch_cast_noalloc: scene %u lives on device %d, not on the current device %d",
			            i, scenes[i]->device, dev);
	unsigned char* scratch = nullptr;
	if ((st = noalloc_scratch(dev, &scratch))) return st;
	if (total == 0) return PHE_OK;

	// Both tables on the host stack, passed by value to the staging kernel (no heap, no device allocation).
	NoAllocTables tab;
	uint32_t base = 0;
	for (uint32_t k = 0; k < numItems; k++) {
		tab.items[k].scene = items[k].scene;
		tab.items[k].kind = items[k].kind;
		tab.items[k].count = items[k].count;
		tab.items[k].base = base;
		tab.items[k].rays = items[k].rays;
		tab.items[k].out = items[k].out;
		base += (items[k].count + 31u) / 32u * 32u;
	}
	bool wide = false;
	for (uint32_t i = 0; i < numScenes; i++) {
		tab.scenes[i] = scenes[i]->dev;
		wide = wide || scenes[i]->dev.nodes4 || scenes[i]->dev.nodes8;
	}
	cudaStream_t s = (cudaStream_t)stream;
	noalloc_stage_kernel<<<1, kNoAllocStageBlock, 0, s>>>(tab, numItems, numScenes, scratch);
	PHE_CUDA_TRY(cudaGetLastError(), "no-alloc staging kernel launch");

	int numSMs = 0, perSM = 0;
	PHE_CUDA_TRY(cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, dev), "SM count");
	auto kernel = wide ? batch_kernel<128, true, 0> : batch_kernel<128, false, 0>;
	PHE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, 128, 0), "occupancy");
	uint32_t grid = (uint32_t)(perSM > 0 ? perSM : 1) * (uint32_t)numSMs;
	uint32_t need = (base + 127u) / 128u;
	if (grid > need) grid = need;
	BatchTableDev t{(const BatchItemDev*)scratch, (const DeviceScene*)(scratch + kNoAllocItemsBytes), numItems, base,
	                nullptr};
	kernel<<<grid, 128, 0, s>>>(t, (uint32_t*)(scratch + kNoAllocItemsBytes + kNoAllocScenesBytes));
	PHE_CUDA_TRY(cudaGetLastError(), "batch_kernel launch (no-alloc)");
	return PHE_OK;
}
