// Wavefront frame renderer: the CUDA path of CudaTracerRenderer::render (normal path,
// cuda_ray_tracer/CudaTracerRenderer.cpp:612-728) with the raster G-buffer replaced by ray-cast
// primary hits, followed by the TAA resolve of resources/shaders/taa.frag:25-71.
//
// One frame is four kernels on one stream by default (the reference issues ~10 launches, each
// followed by cudaDeviceSynchronize):
//   1. primary_kernel     persistent: camera ray -> closest hit -> shading of every light -> append
//                         the shadow rays that matter and one bounce ray per hit to compacted queues
//                         (warp-aggregated atomics; the reference casts dummy rays instead,
//                         MaterialKernel.cu:41-47,105-109)
//   2. bounce_kernel      persistent: bounce closest hit -> shading (throughput as mask) -> append
//                         shadow rays
//   3. any_queue_kernel   persistent any hit over both shadow queues (bounce shadows first), scattered
//                         to the (light, pixel) visibility slots; the other shadow schedules run it
//                         once per queue (PHE_SHADOWS_IN_ORDER, PHE_SHADOWS_BESIDE_BOUNCE)
//   4. resolve_taa_kernel sum of lit contributions (primary lights, then bounce lights, in light
//                         order: shadowLogicKernel, MaterialKernel.cu:361-388) and the TAA blend
// Queue counts stay on the device; persistent kernels read them when they start, so a frame needs
// no host synchronisation and can be captured in a CUDA graph.

#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

#include "raygen.cuh"
#include "runtime.cuh"
#include "octant_sort.cuh"
#include "sampling.cuh"
#include "shading.cuh"
#include "traverse.cuh"
#include "wavefront.cuh"

namespace phe_gb300 {

constexpr int kWaveBlock = 128;
// Resident blocks per SM asked of the compiler for the fused traversal + shading kernels: caps them
// at 64 registers (32 warps per SM instead of 20-24). The spills this costs sit in the shading code;
// measured on GB300 at 1080p: 8 blocks 0.893 ms per frame, 9 0.926, 10 0.915, 12 0.959, uncapped
// (88-92 registers) 0.970. With the branch-free triangle test (fewer live values) the bounce kernel,
// whose incoherent rays wait longest on node fetches, gains from more resident warps while the
// primary kernel does not: bounce pass 0.369 ms at 10 blocks (48 registers) vs 0.376 at 8 and 0.377
// at 12; primary 0.242 ms at 8 vs 0.245 at 9 or 10.
constexpr int kWaveMinBlocks = 8;
constexpr int kBounceMinBlocks = 10;
const size_t kStackSmem = stack_smem_bytes(kWaveBlock);   // dynamic shared memory of the traversal kernels

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated append: every lane of `mask` calls it; lanes with pred get consecutive indices.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred, uint32_t mask)
{
	uint32_t b = __ballot_sync(mask, pred);
	if (b == 0) return 0xFFFFFFFFu;
	uint32_t leader = (uint32_t)__ffs(b) - 1u;
	uint32_t base = 0;
	if (lane_id() == leader) base = atomicAdd(counter, (uint32_t)__popc(b));
	base = __shfl_sync(mask, base, leader);
	return base + (uint32_t)__popc(b & ((1u << lane_id()) - 1u));
}

__device__ __forceinline__ void store_ray(phe_ray_in* rays, uint32_t i, f3 o, float tMin, f3 d, float tMax)
{
	float4* p = reinterpret_cast<float4*>(rays + i);
	st_stream(p, make_float4(o.x, o.y, o.z, tMin));
	st_stream(p + 1, make_float4(d.x, d.y, d.z, tMax));
}

// Shades one hit for every light and appends shadow rays. `stage` 0 = primary, 1 = bounce.
__device__ __forceinline__ void shade_all_lights(const FrameParamsDev& fp, const FrameBuffers& fb, uint32_t stage,
                                                 bool valid, const HitInfo& hi, f3 mask, f3 toCamera, DevPcg& rng,
                                                 uint32_t pid)
{
	const uint32_t P = fp.numPixels;
	const uint32_t L = fp.numLights;
	uint32_t* queueCount = fb.counters + (stage == 0 ? kCtrShadow0 : kCtrShadow1);
	phe_ray_in* qRays = fb.shadowRays + (size_t)stage * fb.capacityLP;
	uint32_t* qSlots = fb.shadowSlots + (size_t)stage * fb.capacityLP;
	for (uint32_t l = 0; l < L; l++) {
		bool cast = false;
		f3 sdir = mk3(0.0f, 0.0f, 0.0f);
		float stmax = 0.0f;
		f3 c = mk3(0.0f, 0.0f, 0.0f);
		if (valid) c = shade_light(fp.lights[l], mask, hi, toCamera, rng, cast, sdir, stmax);
		uint32_t slot = (stage * L + l) * P + pid;
		uint32_t q = warp_append(queueCount, valid && cast, 0xFFFFFFFFu);
		if (valid) {
			st_stream(fb.contrib + slot, make_float4(c.x, c.y, c.z, 0.0f));
			if (cast) {
				store_ray(qRays, q, hi.pos, 0.001f, sdir, stmax);
				st_stream(qSlots + q, slot);
			} else {
				fb.inLight[slot] = 1;   // the reference's dummy ray is never occluded
			}
		}
	}
}

// Image position (uv in [0, 1]^2, the ray-generation convention of genPrimaryRaysKernel) of the camera
// ray through `d` (a point minus the camera origin, or a direction for a point at infinity); false
// when it lies behind the camera.
__device__ __forceinline__ bool project_uv(const phe_camera_def& c, f3 d, float& u, float& v)
{
	f3 dir = mk3(c.dir[0], c.dir[1], c.dir[2]);
	f3 dX = mk3(c.dX[0], c.dX[1], c.dX[2]);
	f3 dY = mk3(c.dY[0], c.dY[1], c.dY[2]);
	float z = dot3(d, dir);
	if (!(z > 0.0f)) return false;
	float cx = __fdiv_rn(dot3(d, dX), __fmul_rn(dot3(dX, dX), z));
	float cy = __fdiv_rn(dot3(d, dY), __fmul_rn(dot3(dY, dY), z));
	u = __fmul_rn(__fadd_rn(cx, 1.0f), 0.5f);
	v = __fmul_rn(__fadd_rn(cy, 1.0f), 0.5f);
	return true;
}

// Velocity of the surface seen through a pixel (velocity_gen.frag without dynamic objects): its uv in
// this frame's camera minus its uv in the previous frame's camera, both without jitter. A point behind
// either camera gets (2, 2), which sends the TAA history lookup off screen (current colour only).
__device__ __forceinline__ float2 pixel_velocity(const FrameParamsDev& fp, bool hit, f3 pos, f3 dir)
{
	f3 o = mk3(fp.cam.origin[0], fp.cam.origin[1], fp.cam.origin[2]);
	f3 po = mk3(fp.prevCam.origin[0], fp.prevCam.origin[1], fp.prevCam.origin[2]);
	float u0, v0, u1, v1;
	if (project_uv(fp.cam, hit ? sub3(pos, o) : dir, u0, v0) &&
	    project_uv(fp.prevCam, hit ? sub3(pos, po) : dir, u1, v1))
		return make_float2(__fsub_rn(u0, u1), __fsub_rn(v0, v1));
	return make_float2(2.0f, 2.0f);
}

template <bool WIDE>
__global__ void __launch_bounds__(kWaveBlock, kWaveMinBlocks) primary_kernel(DeviceScene s, const FrameParamsDev* __restrict__ fpp,
                                                             FrameBuffers fb, uint32_t* __restrict__ status)
{
	const FrameParamsDev& fp = *fpp;
	const uint32_t P = fp.numPixels, W = fp.resX, L = fp.numLights, n = fp.partPixels;
	uint32_t* work = fb.counters + kCtrWork0;
	for (;;) {
		uint32_t base = 0;
		if (lane_id() == 0) base = atomicAdd(work, 32u);
		base = __shfl_sync(0xFFFFFFFFu, base, 0);
		if (base >= n) break;
		uint32_t i = base + lane_id();
		bool active = i < n;
		// 8x8-tile-major ray order (getRayIdx, CudaDeviceHelpers.cuh:49-62): coherent warps; this part's
		// tile rows interleave with the other parts'
		uint32_t tile = i >> 6, within = i & 63u;
		uint32_t tilesX = W >> 3;
		uint32_t x = (tile % tilesX) * 8u + (within & 7u);
		uint32_t y = ((tile / tilesX) * fp.parts + fp.part) * 8u + (within >> 3);
		uint32_t pid = y * W + x;
		RayState r;
		HitRecord h;
		h.slot = ~0u;
		if (active) {
			f3 d = primary_dir(fp.cam, x, y, W, fp.resY, fp.jitter[0], fp.jitter[1]);
			r.o = mk3(fp.cam.origin[0], fp.cam.origin[1], fp.cam.origin[2]);
			r.d = d;
			r.tMin = 0.0001f;
			r.tMax = 3.402823466e+38f;
			r.inv = mk3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
			r.safe = isfinite(r.inv.x) && isfinite(r.inv.y) && isfinite(r.inv.z) && isfinite(d.x) && isfinite(d.y) &&
			         isfinite(d.z) && isfinite(r.o.x) && isfinite(r.o.y) && isfinite(r.o.z);
			h = empty_hit(r);
			uint32_t err = trace<false, WIDE>(s, r, h);
			if (err) atomicOr(status, err);
		}
		__syncwarp();
		bool hit = active && h.slot != ~0u;
		HitInfo hi;
		DevPcg rng;
		f3 toCamera = mk3(0.0f, 0.0f, 0.0f);
		f3 camPos = mk3(fp.camPos[0], fp.camPos[1], fp.camPos[2]);
		if (hit) {
			hi = interpret_hit(s, r.o, r.d, h.slot, h.t, h.u, h.v);
			pixel_stream(rng, fp.seed, fp.frame, pid, 0);
			toCamera = normalize3(sub3(camPos, hi.pos));
		} else {
			hi.pos = hi.normal = hi.albedo = mk3(0.0f, 0.0f, 0.0f);
			hi.alpha = hi.roughness = hi.metallic = 0.0f;
		}
		if (active) fb.roughness[pid] = hit ? hi.roughness : 0.0f;
		if (active && fp.velocity) fp.velocity[pid] = pixel_velocity(fp, hit, hi.pos, r.d);
		shade_all_lights(fp, fb, 0, hit, hi, mk3(1.0f, 1.0f, 1.0f), toCamera, rng, pid);
		// Bounce ray (one per hit) into the bounce queue.
		float btMin = 0.001f;
		f3 thr = mk3(0.0f, 0.0f, 0.0f), bdir = mk3(0.0f, 0.0f, 0.0f);
		if (hit) bdir = sample_bounce(hi, camPos, rng, btMin, thr);
		uint32_t q = warp_append(fb.counters + kCtrBounce, hit, 0xFFFFFFFFu);
		if (hit) {
			store_ray(fb.bounceRays, q, hi.pos, btMin, bdir, 3.402823466e+38f);
			st_stream(fb.bouncePixel + q, pid);
			st_stream(fb.bounceThroughput + q, make_float4(thr.x, thr.y, thr.z, 0.0f));
		} else if (active) {
			// no primary hit: nothing to add for this pixel in either stage
			// Visibility 0 marks both stages' slots as adding nothing, so the resolve reads no
			// contribution for them (the sum stays +0, as with zero contributions marked visible).
			for (uint32_t l = 0; l < L; l++) {
				st_stream(fb.inLight + (size_t)l * P + pid, (uint8_t)0);
				st_stream(fb.inLight + (size_t)(L + l) * P + pid, (uint8_t)0);
			}
		}
		__syncwarp();
	}
}

// Persistent any hit over one or two compacted shadow queues (A, then B when countB is given),
// each result scattered to its (light, pixel) visibility slot.
template <bool WIDE>
__global__ void __launch_bounds__(kWaveBlock) any_queue_kernel(DeviceScene s, const phe_ray_in* __restrict__ raysA,
                                                               const uint32_t* __restrict__ slotsA,
                                                               const uint32_t* __restrict__ countA,
                                                               const phe_ray_in* __restrict__ raysB,
                                                               const uint32_t* __restrict__ slotsB,
                                                               const uint32_t* __restrict__ countB,
                                                               uint8_t* __restrict__ inLight, uint32_t* __restrict__ work,
                                                               uint32_t* __restrict__ status)
{
	const uint32_t nA = *countA, n = nA + (countB ? *countB : 0u);
	for (;;) {
		uint32_t base = 0;
		if (lane_id() == 0) base = atomicAdd(work, 32u);
		base = __shfl_sync(0xFFFFFFFFu, base, 0);
		if (base >= n) break;
		uint32_t i = base + lane_id();
		if (i < n) {
			const bool a = i < nA;
			const uint32_t k = a ? i : i - nA;
			RayState r = load_ray(a ? raysA : raysB, k);
			HitRecord h = empty_hit(r);
			uint32_t err = trace<true, WIDE>(s, r, h);
			if (err) atomicOr(status, err);
			inLight[ld_stream((a ? slotsA : slotsB) + k)] = h.slot == ~0u ? 1 : 0;
		}
		__syncwarp();
	}
}

// Bins the bounce queue by direction octant inside windows of fb.sortWindow consecutive entries (a
// stable counting sort per window, octant_sort.cuh), so warps of the bounce pass trace rays of one
// octant from one neighbourhood of the image. Writes fb.bouncePerm.
constexpr int kBinBlock = kOctantBlock;

__global__ void __launch_bounds__(kBinBlock) bin_bounce_kernel(FrameBuffers fb)
{
	const int W = fb.sortWindow;
	if (W <= 0) return;
	const uint32_t n = fb.counters[kCtrBounce];
	const int per = W / kBinBlock;   // entries per thread (W is a multiple of kBinBlock, <= kMaxOctantWindow)
	__shared__ uint32_t cnt[8][kBinBlock];
	__shared__ uint32_t bucketBase[8];
	const int t = threadIdx.x;
	for (uint32_t w0 = blockIdx.x * (uint32_t)W; w0 < n; w0 += gridDim.x * (uint32_t)W) {
		uint8_t keys[kMaxOctantWindow / kBinBlock];
		for (int k = 0; k < per; k++) {
			uint32_t i = w0 + (uint32_t)(t * per + k);
			keys[k] = i < n ? octant_key(reinterpret_cast<const float4*>(fb.bounceRays + i)[1]) : (uint8_t)0xFF;
		}
		uint32_t rank[8];
		octant_ranks(keys, per, cnt, bucketBase, rank);
		for (int k = 0; k < per; k++) {
			uint8_t key = keys[k];
			if (key != 0xFF) fb.bouncePerm[w0 + rank[key]++] = w0 + (uint32_t)(t * per + k);
		}
	}
}

template <bool WIDE>
__global__ void __launch_bounds__(kWaveBlock, kBounceMinBlocks) bounce_kernel(DeviceScene s, const FrameParamsDev* __restrict__ fpp,
                                                            FrameBuffers fb, uint32_t* __restrict__ status)
{
	const FrameParamsDev& fp = *fpp;
	const uint32_t P = fp.numPixels, L = fp.numLights;
	const uint32_t n = fb.counters[kCtrBounce];
	uint32_t* work = fb.counters + kCtrWork1;
	for (;;) {
		uint32_t base = 0;
		if (lane_id() == 0) base = atomicAdd(work, 32u);
		base = __shfl_sync(0xFFFFFFFFu, base, 0);
		if (base >= n) break;
		uint32_t i = base + lane_id();
		bool active = i < n;
		RayState r;
		HitRecord h;
		h.slot = ~0u;
		uint32_t pid = 0;
		f3 thr = mk3(0.0f, 0.0f, 0.0f);
		if (active) {
			uint32_t j = fb.sortWindow > 0 ? fb.bouncePerm[i] : i;
			r = load_ray(fb.bounceRays, j);
			pid = ld_stream(fb.bouncePixel + j);
			float4 t4 = ld_stream(fb.bounceThroughput + j);
			thr = mk3(t4.x, t4.y, t4.z);
			h = empty_hit(r);
			uint32_t err = trace<false, WIDE>(s, r, h);
			if (err) atomicOr(status, err);
		}
		__syncwarp();
		bool hit = active && h.slot != ~0u;
		HitInfo hi;
		DevPcg rng;
		f3 toCamera = mk3(0.0f, 0.0f, 0.0f);
		if (hit) {
			hi = interpret_hit(s, r.o, r.d, h.slot, h.t, h.u, h.v);
			pixel_stream(rng, fp.seed, fp.frame, pid, 1);
			toCamera = mk3(-r.d.x, -r.d.y, -r.d.z);
		} else {
			hi.pos = hi.normal = hi.albedo = mk3(0.0f, 0.0f, 0.0f);
			hi.alpha = hi.roughness = hi.metallic = 0.0f;
		}
		shade_all_lights(fp, fb, 1, hit, hi, thr, toCamera, rng, pid);
		if (active && !hit) {   // the bounce ray escaped: nothing to add (visibility 0, no contribution read)
			for (uint32_t l = 0; l < L; l++) st_stream(fb.inLight + (size_t)(L + l) * P + pid, (uint8_t)0);
		}
		__syncwarp();
	}
}

// ------------------------------------------------------------------------------------------------
// Split pipeline: traversal kernels (persistent, lane refill, no shading state in registers) and
// shading kernels (one thread per hit, full warps) communicate through 16-byte hit records.
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ void tile_pixel(uint32_t i, uint32_t W, uint32_t& x, uint32_t& y)
{
	uint32_t tile = i >> 6, within = i & 63u, tilesX = W >> 3;
	x = (tile % tilesX) * 8u + (within & 7u);
	y = (tile / tilesX) * 8u + (within >> 3);
}

struct CameraSource {
	const FrameParamsDev* fp;
	__device__ __forceinline__ RayState load(uint32_t i) const
	{
		uint32_t x, y;
		tile_pixel(i, fp->resX, x, y);
		RayState r;
		f3 d = primary_dir(fp->cam, x, y, fp->resX, fp->resY, fp->jitter[0], fp->jitter[1]);
		r.o = mk3(fp->cam.origin[0], fp->cam.origin[1], fp->cam.origin[2]);
		r.d = d;
		r.tMin = 0.0001f;
		r.tMax = 3.402823466e+38f;
		r.inv = mk3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
		r.safe = isfinite(r.inv.x) && isfinite(r.inv.y) && isfinite(r.inv.z) && isfinite(d.x) && isfinite(d.y) &&
		         isfinite(d.z) && isfinite(r.o.x) && isfinite(r.o.y) && isfinite(r.o.z);
		return r;
	}
};

struct ArraySource {
	const phe_ray_in* rays;
	const uint32_t* perm;   // optional: ray i of the pass is rays[perm[i]]
	__device__ __forceinline__ RayState load(uint32_t i) const { return load_ray(rays, perm ? __ldg(perm + i) : i); }
};

struct HitSink {
	phe_ray_hit* hits;
	__device__ __forceinline__ void store(uint32_t i, const RayState& r, const HitRecord& h) const { store_hit(hits, i, r, h); }
};

struct VisibilitySink {
	uint8_t* inLight;
	const uint32_t* slots;
	__device__ __forceinline__ void store(uint32_t i, const RayState&, const HitRecord& h) const
	{
		inLight[slots ? __ldg(slots + i) : i] = h.slot == ~0u ? 1 : 0;
	}
};

__global__ void __launch_bounds__(kWaveBlock) primary_trace_kernel(DeviceScene s, const FrameParamsDev* __restrict__ fpp,
                                                                   FrameBuffers fb, uint32_t* __restrict__ status)
{
	uint32_t err = persistent_trace<false>(s.nodes, s.tris, TraversalBounds{s.numNodes, s.numSlots}, CameraSource{fpp}, HitSink{fb.primaryHits}, fpp->numPixels,
	                                       fb.counters + kCtrWork0, fb.refill);
	if (err) atomicOr(status, err);
}

__global__ void __launch_bounds__(kWaveBlock) any_refill_kernel(DeviceScene s, const phe_ray_in* __restrict__ rays,
                                                                const uint32_t* __restrict__ slots,
                                                                const uint32_t* __restrict__ count,
                                                                uint8_t* __restrict__ inLight, uint32_t* __restrict__ work,
                                                                int refill, uint32_t* __restrict__ status)
{
	uint32_t err = persistent_trace<true>(s.nodes, s.tris, TraversalBounds{s.numNodes, s.numSlots}, ArraySource{rays, nullptr}, VisibilitySink{inLight, slots}, *count,
	                                      work, refill);
	if (err) atomicOr(status, err);
}

__global__ void __launch_bounds__(kWaveBlock) bounce_trace_kernel(DeviceScene s, FrameBuffers fb, uint32_t* __restrict__ status)
{
	uint32_t err = persistent_trace<false>(s.nodes, s.tris, TraversalBounds{s.numNodes, s.numSlots}, ArraySource{fb.bounceRays, fb.sortWindow > 0 ? fb.bouncePerm : nullptr},
	                                       HitSink{fb.bounceHits},
	                                       fb.counters[kCtrBounce], fb.counters + kCtrWork1, fb.refill);
	if (err) atomicOr(status, err);
}

__global__ void __launch_bounds__(kWaveBlock) primary_shade_kernel(DeviceScene s, const FrameParamsDev* __restrict__ fpp,
                                                                   FrameBuffers fb)
{
	const FrameParamsDev& fp = *fpp;
	const uint32_t P = fp.numPixels, W = fp.resX, L = fp.numLights;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;; i += gridDim.x * blockDim.x) {
		bool active = i < P;
		if (!__any_sync(0xFFFFFFFFu, active)) break;
		uint32_t x = 0, y = 0, pid = 0;
		float4 hv = make_float4(__uint_as_float(~0u), 0.0f, 0.0f, 0.0f);
		if (active) {
			tile_pixel(i, W, x, y);
			pid = y * W + x;
			hv = reinterpret_cast<const float4*>(fb.primaryHits)[i];
		}
		uint32_t slot = __float_as_uint(hv.x);
		bool hit = active && slot != ~0u;
		HitInfo hi;
		DevPcg rng;
		f3 toCamera = mk3(0.0f, 0.0f, 0.0f);
		f3 camPos = mk3(fp.camPos[0], fp.camPos[1], fp.camPos[2]);
		if (hit) {
			f3 o = mk3(fp.cam.origin[0], fp.cam.origin[1], fp.cam.origin[2]);
			f3 d = primary_dir(fp.cam, x, y, W, fp.resY, fp.jitter[0], fp.jitter[1]);
			hi = interpret_hit(s, o, d, slot, hv.y, hv.z, hv.w);
			pixel_stream(rng, fp.seed, fp.frame, pid, 0);
			toCamera = normalize3(sub3(camPos, hi.pos));
		} else {
			hi.pos = hi.normal = hi.albedo = mk3(0.0f, 0.0f, 0.0f);
			hi.alpha = hi.roughness = hi.metallic = 0.0f;
		}
		if (active) fb.roughness[pid] = hit ? hi.roughness : 0.0f;
		if (active && fp.velocity)
			fp.velocity[pid] = pixel_velocity(fp, hit, hi.pos,
			                                  hit ? hi.pos : primary_dir(fp.cam, x, y, W, fp.resY, fp.jitter[0], fp.jitter[1]));
		shade_all_lights(fp, fb, 0, hit, hi, mk3(1.0f, 1.0f, 1.0f), toCamera, rng, pid);
		float btMin = 0.001f;
		f3 thr = mk3(0.0f, 0.0f, 0.0f), bdir = mk3(0.0f, 0.0f, 0.0f);
		if (hit) bdir = sample_bounce(hi, camPos, rng, btMin, thr);
		uint32_t q = warp_append(fb.counters + kCtrBounce, hit, 0xFFFFFFFFu);
		if (hit) {
			store_ray(fb.bounceRays, q, hi.pos, btMin, bdir, 3.402823466e+38f);
			st_stream(fb.bouncePixel + q, pid);
			st_stream(fb.bounceThroughput + q, make_float4(thr.x, thr.y, thr.z, 0.0f));
		} else if (active) {
			// Visibility 0 marks both stages' slots as adding nothing, so the resolve reads no
			// contribution for them (the sum stays +0, as with zero contributions marked visible).
			for (uint32_t l = 0; l < L; l++) {
				st_stream(fb.inLight + (size_t)l * P + pid, (uint8_t)0);
				st_stream(fb.inLight + (size_t)(L + l) * P + pid, (uint8_t)0);
			}
		}
	}
}

__global__ void __launch_bounds__(kWaveBlock) bounce_shade_kernel(DeviceScene s, const FrameParamsDev* __restrict__ fpp,
                                                                  FrameBuffers fb)
{
	const FrameParamsDev& fp = *fpp;
	const uint32_t P = fp.numPixels, L = fp.numLights;
	const uint32_t n = fb.counters[kCtrBounce];
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;; i += gridDim.x * blockDim.x) {
		bool active = i < n;
		if (!__any_sync(0xFFFFFFFFu, active)) break;
		uint32_t pid = 0, slot = ~0u;
		f3 thr = mk3(0.0f, 0.0f, 0.0f), o = thr, d = thr;
		float4 hv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		if (active) {
			uint32_t j = fb.sortWindow > 0 ? fb.bouncePerm[i] : i;
			pid = ld_stream(fb.bouncePixel + j);
			float4 t4 = ld_stream(fb.bounceThroughput + j);
			thr = mk3(t4.x, t4.y, t4.z);
			hv = reinterpret_cast<const float4*>(fb.bounceHits)[i];
			slot = __float_as_uint(hv.x);
			const float4* rp = reinterpret_cast<const float4*>(fb.bounceRays + j);
			float4 a = rp[0], b = rp[1];
			o = mk3(a.x, a.y, a.z);
			d = mk3(b.x, b.y, b.z);
		}
		bool hit = active && slot != ~0u;
		HitInfo hi;
		DevPcg rng;
		f3 toCamera = mk3(0.0f, 0.0f, 0.0f);
		if (hit) {
			hi = interpret_hit(s, o, d, slot, hv.y, hv.z, hv.w);
			pixel_stream(rng, fp.seed, fp.frame, pid, 1);
			toCamera = mk3(-d.x, -d.y, -d.z);
		} else {
			hi.pos = hi.normal = hi.albedo = mk3(0.0f, 0.0f, 0.0f);
			hi.alpha = hi.roughness = hi.metallic = 0.0f;
		}
		shade_all_lights(fp, fb, 1, hit, hi, thr, toCamera, rng, pid);
		if (active && !hit) {   // the bounce ray escaped: nothing to add (visibility 0, no contribution read)
			for (uint32_t l = 0; l < L; l++) st_stream(fb.inLight + (size_t)(L + l) * P + pid, (uint8_t)0);
		}
	}
}

// TAA (taa.frag:25-71) with the history fetched in pixel space: (x + 0.5) - velocity * res.
// The blend of taa.frag:62-70: n' = n * trust + 1, out = mix(cur, hist, 1 - 1/n'), alpha n'.
__device__ __forceinline__ void taa_blend(float4 cur, float4 h, float trust, float4& outColor, float4& outHist)
{
	float newSamples = __fadd_rn(__fmul_rn(h.w, trust), 1.0f);
	float blend = __fsub_rn(1.0f, __fdiv_rn(1.0f, newSamples));
	outHist = make_float4(glsl_mix(cur.x, h.x, blend), glsl_mix(cur.y, h.y, blend), glsl_mix(cur.z, h.z, blend),
	                      newSamples);
	outColor = make_float4(outHist.x, outHist.y, outHist.z, 1.0f);
}

__device__ __forceinline__ void taa_pixel(uint32_t x, uint32_t y, uint32_t W, uint32_t H, float4 cur,
                                          const float4* __restrict__ hist, const float2* __restrict__ vel,
                                          const float2* __restrict__ prevVel, float roughness, float4& outColor,
                                          float4& outHist)
{
	size_t p = (size_t)y * W + x;
	float vx = vel ? vel[p].x : 0.0f, vy = vel ? vel[p].y : 0.0f;
	float hx = __fsub_rn(__fadd_rn((float)x, 0.5f), __fmul_rn(vx, (float)W));
	float hy = __fsub_rn(__fadd_rn((float)y, 0.5f), __fmul_rn(vy, (float)H));
	if (hx < 0.0f || hx > (float)W || hy < 0.0f || hy > (float)H) {
		outHist = make_float4(cur.x, cur.y, cur.z, 1.0f);
		outColor = make_float4(cur.x, cur.y, cur.z, 1.0f);
		return;
	}
	bool still = vx == 0.0f && vy == 0.0f;
	float hv[2] = {0.0f, 0.0f};
	if (prevVel) {
		if (still) { hv[0] = prevVel[p].x; hv[1] = prevVel[p].y; }
		else bilinear<2>(reinterpret_cast<const float*>(prevVel), W, H, hx, hy, hv);
	}
	float pvx = __fmul_rn((float)W, vx), pvy = __fmul_rn((float)H, vy);
	float hpx = __fmul_rn((float)W, hv[0]), hpy = __fmul_rn((float)H, hv[1]);
	float lp = __fsqrt_rn(__fadd_rn(__fmul_rn(pvx, pvx), __fmul_rn(pvy, pvy)));
	float lh = __fsqrt_rn(__fadd_rn(__fmul_rn(hpx, hpx), __fmul_rn(hpy, hpy)));
	float velocityDistrust = fminf(1.0f, __fmul_rn(1.2f, __fsqrt_rn(fabsf(__fsub_rn(lp, lh)))));
	float roughnessDistrust = glsl_mix(3.0f, 1.0f, roughness);
	float trust = clampf(__fsub_rn(1.0f, __fmul_rn(roughnessDistrust, velocityDistrust)), 0.0f, 1.0f);
	float4 h;
	if (still) {
		h = hist[p];
	} else {
		float h4[4];
		bilinear<4>(reinterpret_cast<const float*>(hist), W, H, hx, hy, h4);
		h = make_float4(h4[0], h4[1], h4[2], h4[3]);
	}
	taa_blend(cur, h, trust, outColor, outHist);
}

// Two pixels a thread, 128 apart (a block covers 256 consecutive pixels, so every load and store of a
// warp stays coalesced). The still-camera path is bound by memory latency: a pixel's contribution loads
// wait on its visibility bytes. Here the visibility loads of both pixels (kResolveChunk slots each) are
// issued together, then the contribution loads of the visible slots, so a thread keeps two independent
// chains in flight; the per-pixel sums keep the slot order.
constexpr int kResolveBlock = 128;
constexpr int kResolveMinBlocks = 10;
constexpr uint32_t kResolveChunk = 2;   // light slots whose loads are issued together
__global__ void __launch_bounds__(kResolveBlock, kResolveMinBlocks)
resolve_taa_kernel(const FrameParamsDev* __restrict__ fpp, FrameBuffers fb)
{
	const FrameParamsDev& fp = *fpp;
	const uint32_t P = fp.numPixels, L = fp.numLights, np = fp.partPixels, W = fp.resX;
	// The thread's two pixels, indices q0 and q1 into this part's pixels in row order (the part's rows
	// are its tile rows, which interleave with the other parts'; with one part, q is the pixel).
	const uint32_t q0 = blockIdx.x * (2u * kResolveBlock) + threadIdx.x, q1 = q0 + kResolveBlock;
	if (q0 >= np) return;
	auto pixel = [&](uint32_t q) {
		const uint32_t lr = q / W;
		return (((lr >> 3) * fp.parts + fp.part) * 8u + (lr & 7u)) * W + q % W;
	};
	if (q0 == 0) {
		atomicAdd(&fb.rayTotals[0], (unsigned long long)np);
		atomicAdd(&fb.rayTotals[1], (unsigned long long)fb.counters[kCtrShadow0]);
		atomicAdd(&fb.rayTotals[2], (unsigned long long)fb.counters[kCtrBounce]);
		atomicAdd(&fb.rayTotals[3], (unsigned long long)fb.counters[kCtrShadow1]);
	}
	if (fp.velocity || fp.prevVelocity) {   // camera motion: the full TAA with reprojected history
		for (uint32_t q = q0; q <= q1 && q < np; q += kResolveBlock) {
			const uint32_t pid = pixel(q);
			f3 acc = mk3(0.0f, 0.0f, 0.0f);
			for (uint32_t k = 0; k < 2 * L; k++) {
				size_t slot = (size_t)k * P + pid;
				if (fb.inLight[slot]) {
					float4 c = fb.contrib[slot];
					acc = add3(acc, mk3(c.x, c.y, c.z));
				}
			}
			float4 cur = make_float4(acc.x, acc.y, acc.z, 1.0f);
			float4 oc, oh;
			taa_pixel(pid % fp.resX, pid / fp.resX, fp.resX, fp.resY, cur, fb.history[fp.parity], fp.velocity,
			          fp.prevVelocity, fb.roughness[pid], oc, oh);
			fb.rawColor[pid] = cur;
			fb.color[fp.parity ^ 1u][pid] = oc;
			fb.history[fp.parity ^ 1u][pid] = oh;
		}
		return;
	}
	// Still camera. Every load a pixel needs is issued before the first store (the stores could alias
	// them for the compiler). With zero velocity the history texel is the pixel itself and both velocity
	// lengths are 0, so velocityDistrust = 0 and trust = clamp(1 - roughnessDistrust * 0). At the end of
	// the frame the second pixel may not exist: it then repeats the first and its stores are skipped.
	const bool two = q1 < np;
	const uint32_t p0 = pixel(q0), p1 = two ? pixel(q1) : p0;
	const float4 h0 = ld_stream(fb.history[fp.parity] + p0), h1 = ld_stream(fb.history[fp.parity] + p1);
	const float r0 = ld_stream(fb.roughness + p0), r1 = ld_stream(fb.roughness + p1);
	const uint32_t n = 2 * L;
	f3 a0 = mk3(0.0f, 0.0f, 0.0f), a1 = a0;
	for (uint32_t k0 = 0; k0 < n; k0 += kResolveChunk) {
		uint8_t v0[kResolveChunk], v1[kResolveChunk];
#pragma unroll
		for (uint32_t j = 0; j < kResolveChunk; j++) {
			const size_t base = (size_t)(k0 + j) * P;
			const bool in = k0 + j < n;
			v0[j] = in ? ld_stream(fb.inLight + base + p0) : (uint8_t)0;
			v1[j] = in ? ld_stream(fb.inLight + base + p1) : (uint8_t)0;
		}
		float4 c0[kResolveChunk], c1[kResolveChunk];
#pragma unroll
		for (uint32_t j = 0; j < kResolveChunk; j++) {
			const size_t base = (size_t)(k0 + j) * P;
			c0[j] = v0[j] ? ld_stream(fb.contrib + base + p0) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
			c1[j] = v1[j] ? ld_stream(fb.contrib + base + p1) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		}
#pragma unroll
		for (uint32_t j = 0; j < kResolveChunk; j++) {
			if (v0[j]) a0 = add3(a0, mk3(c0[j].x, c0[j].y, c0[j].z));
			if (v1[j]) a1 = add3(a1, mk3(c1[j].x, c1[j].y, c1[j].z));
		}
	}
	const float4 cur0 = make_float4(a0.x, a0.y, a0.z, 1.0f), cur1 = make_float4(a1.x, a1.y, a1.z, 1.0f);
	float4 oc0, oh0, oc1, oh1;
	taa_blend(cur0, h0, clampf(__fsub_rn(1.0f, __fmul_rn(glsl_mix(3.0f, 1.0f, r0), 0.0f)), 0.0f, 1.0f), oc0, oh0);
	taa_blend(cur1, h1, clampf(__fsub_rn(1.0f, __fmul_rn(glsl_mix(3.0f, 1.0f, r1), 0.0f)), 0.0f, 1.0f), oc1, oh1);
	float4* color = fb.color[fp.parity ^ 1u];
	float4* hist = fb.history[fp.parity ^ 1u];
	st_stream(fb.rawColor + p0, cur0);
	st_stream(color + p0, oc0);
	st_stream(hist + p0, oh0);
	if (two) {
		st_stream(fb.rawColor + p1, cur1);
		st_stream(color + p1, oc1);
		st_stream(hist + p1, oh1);
	}
}

__global__ void taa_kernel(uint32_t W, uint32_t H, const float4* __restrict__ cur, const float4* __restrict__ hist,
                           const float2* __restrict__ vel, const float2* __restrict__ prevVel,
                           const float* __restrict__ roughness, float4* __restrict__ outColor, float4* __restrict__ outHist)
{
	uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
	uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= W || y >= H) return;
	size_t p = (size_t)y * W + x;
	float4 oc, oh;
	taa_pixel(x, y, W, H, cur[p], hist, vel, prevVel, roughness ? roughness[p] : 0.0f, oc, oh);
	outColor[p] = oc;
	outHist[p] = oh;
}

// ------------------------------------------------------------------------------------------------
// Launch sequence of one frame
// ------------------------------------------------------------------------------------------------

// The last three are the 4-wide instantiations of the fused kernels.
enum { kGridPrimary = 0, kGridAnyQueue, kGridBounce, kGridPrimaryTrace, kGridAnyRefill, kGridBounceTrace,
       kGridPrimaryShade, kGridBounceShade, kGridPrimaryWide, kGridAnyQueueWide, kGridBounceWide, kGridCount };
// filled on first use (threads that race store the same value)
static std::atomic<int> g_waveBlocksPerSM[kGridCount] = {};

static const void* wave_kernel(int which)
{
	switch (which) {
	case kGridPrimary: return (const void*)primary_kernel<false>;
	case kGridAnyQueue: return (const void*)any_queue_kernel<false>;
	case kGridBounce: return (const void*)bounce_kernel<false>;
	case kGridPrimaryWide: return (const void*)primary_kernel<true>;
	case kGridAnyQueueWide: return (const void*)any_queue_kernel<true>;
	case kGridBounceWide: return (const void*)bounce_kernel<true>;
	case kGridPrimaryTrace: return (const void*)primary_trace_kernel;
	case kGridAnyRefill: return (const void*)any_refill_kernel;
	case kGridBounceTrace: return (const void*)bounce_trace_kernel;
	case kGridPrimaryShade: return (const void*)primary_shade_kernel;
	default: return (const void*)bounce_shade_kernel;
	}
}

static phe_status wave_grid(int which, int* grid)
{
	DeviceInfo* d = nullptr;
	phe_status st = device_info(&d);
	if (st) return st;
	int blocks = g_waveBlocksPerSM[which].load(std::memory_order_relaxed);
	if (blocks == 0) {
		int b = 0;
		const bool traverses = which != kGridPrimaryShade && which != kGridBounceShade;
		PHE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, wave_kernel(which), kWaveBlock,
		                                                           traverses ? kStackSmem : 0), "occupancy");
		blocks = b > 0 ? b : 1;
		g_waveBlocksPerSM[which].store(blocks, std::memory_order_relaxed);
	}
	*grid = blocks * d->numSMs;
	return PHE_OK;
}

phe_status prepare_frame()
{
	int g;
	for (int k = 0; k < kGridCount; k++) {
		phe_status st = wave_grid(k, &g);
		if (st) return st;
	}
	return PHE_OK;
}

phe_status launch_frame(const phe_scene* scene, const FrameParamsDev* dParams, const FrameBuffers& fb, uint32_t resX,
                        uint32_t resY, cudaStream_t stream, cudaEvent_t* ev, bool fused, int schedule,
                        const FrameStreams* streams, int parts, uint32_t partPixels)
{
	// Timed frames keep one stream so that the per-kernel events measure one kernel each.
	const bool beside = schedule == PHE_SHADOWS_BESIDE_BOUNCE && streams && streams->side && !ev;
	phe_status st;
	int g[kGridCount];
	for (int k = 0; k < kGridCount; k++)
		if ((st = wave_grid(k, &g[k]))) return st;
	int e = 0;
	auto mark = [&]() { if (ev) cudaEventRecord(ev[e++], stream); };
	DeviceInfo* dinfo = nullptr;
	if ((st = device_info(&dinfo))) return st;
	int binGrid = dinfo->numSMs * 4;
	if (parts & kFrameTraversal) {
		PHE_CUDA_TRY(cudaMemsetAsync(fb.counters, 0, sizeof(uint32_t) * kNumCounters, stream), "clear frame counters");
		mark();
		if (fused) {
			const bool wide = scene->dev.nodes4 || scene->dev.nodes8;
			auto primary = wide ? primary_kernel<true> : primary_kernel<false>;
			auto anyQueue = wide ? any_queue_kernel<true> : any_queue_kernel<false>;
			auto bounce = wide ? bounce_kernel<true> : bounce_kernel<false>;
			// Persistent grids, but never more blocks than the frame's rays can keep busy: a small frame (a
			// 256x256 render of the serving loop) then leaves the other SMs to concurrent requests.
			const uint64_t P = partPixels ? partPixels : (uint64_t)resX * resY;
			auto clamp = [](int grid, uint64_t rays) {
				return (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)grid, (rays + kWaveBlock - 1) / kWaveBlock));
			};
			const int gPrimary = clamp(g[wide ? kGridPrimaryWide : kGridPrimary], P);
			const int gAny = clamp(g[wide ? kGridAnyQueueWide : kGridAnyQueue], 2 * (uint64_t)fb.capacityLP);
			const int gBounce = clamp(g[wide ? kGridBounceWide : kGridBounce], P);
			const phe_ray_in* rays1 = fb.shadowRays + fb.capacityLP;
			const uint32_t* slots1 = fb.shadowSlots + fb.capacityLP;
			primary<<<gPrimary, kWaveBlock, kStackSmem, stream>>>(scene->dev, dParams, fb, scene->status);
			mark();
			if (schedule != PHE_SHADOWS_MERGED) {
				cudaStream_t shadowStream = stream;
				if (beside) {
					PHE_CUDA_TRY(cudaEventRecord(streams->fork, stream), "fork frame");
					PHE_CUDA_TRY(cudaStreamWaitEvent(streams->side, streams->fork, 0), "fork frame");
					shadowStream = streams->side;
				}
				anyQueue<<<gAny, kWaveBlock, kStackSmem, shadowStream>>>(scene->dev, fb.shadowRays, fb.shadowSlots,
				                                                 fb.counters + kCtrShadow0, nullptr, nullptr, nullptr,
				                                                 fb.inLight, fb.counters + kCtrWork2, scene->status);
				if (beside) PHE_CUDA_TRY(cudaEventRecord(streams->join, shadowStream), "join frame");
				mark();
			}
			if (fb.sortWindow > 0) {
				bin_bounce_kernel<<<binGrid, kBinBlock, 0, stream>>>(fb);
				mark();
			}
			bounce<<<gBounce, kWaveBlock, kStackSmem, stream>>>(scene->dev, dParams, fb, scene->status);
			mark();
			if (schedule == PHE_SHADOWS_MERGED) {
				// bounce shadows first: their incoherent rays start early and the primary ones fill the tail
				anyQueue<<<gAny, kWaveBlock, kStackSmem, stream>>>(scene->dev, rays1, slots1, fb.counters + kCtrShadow1,
				                                           fb.shadowRays, fb.shadowSlots, fb.counters + kCtrShadow0,
				                                           fb.inLight, fb.counters + kCtrWork3, scene->status);
			} else {
				anyQueue<<<gAny, kWaveBlock, kStackSmem, stream>>>(scene->dev, rays1, slots1, fb.counters + kCtrShadow1, nullptr,
				                                           nullptr, nullptr, fb.inLight, fb.counters + kCtrWork3,
				                                           scene->status);
			}
			mark();
			if (beside) PHE_CUDA_TRY(cudaStreamWaitEvent(stream, streams->join, 0), "join frame");
		} else {
			primary_trace_kernel<<<g[kGridPrimaryTrace], kWaveBlock, kStackSmem, stream>>>(scene->dev, dParams, fb, scene->status);
			mark();
			primary_shade_kernel<<<g[kGridPrimaryShade], kWaveBlock, 0, stream>>>(scene->dev, dParams, fb);
			mark();
			any_refill_kernel<<<g[kGridAnyRefill], kWaveBlock, kStackSmem, stream>>>(scene->dev, fb.shadowRays, fb.shadowSlots,
			                                                                 fb.counters + kCtrShadow0, fb.inLight,
			                                                                 fb.counters + kCtrWork2, fb.refill,
			                                                                 scene->status);
			mark();
			if (fb.sortWindow > 0) {
				bin_bounce_kernel<<<binGrid, kBinBlock, 0, stream>>>(fb);
				mark();
			}
			bounce_trace_kernel<<<g[kGridBounceTrace], kWaveBlock, kStackSmem, stream>>>(scene->dev, fb, scene->status);
			mark();
			bounce_shade_kernel<<<g[kGridBounceShade], kWaveBlock, 0, stream>>>(scene->dev, dParams, fb);
			mark();
			any_refill_kernel<<<g[kGridAnyRefill], kWaveBlock, kStackSmem, stream>>>(scene->dev, fb.shadowRays + fb.capacityLP,
			                                                                 fb.shadowSlots + fb.capacityLP,
			                                                                 fb.counters + kCtrShadow1, fb.inLight,
			                                                                 fb.counters + kCtrWork3, fb.refill,
			                                                                 scene->status);
			mark();
		}
	}
	if (parts & kFrameResolve) {
		const uint64_t pixels = partPixels ? partPixels : (uint64_t)resX * resY;
		const uint32_t resolveGrid = (uint32_t)((pixels + 2 * kResolveBlock - 1) / (2 * kResolveBlock));
		resolve_taa_kernel<<<resolveGrid, kResolveBlock, 0, stream>>>(dParams, fb);
		mark();
	}
	PHE_CUDA_TRY(cudaGetLastError(), "frame kernel launch");
	return PHE_OK;
}

} // namespace phe_gb300

using namespace phe_gb300;

extern "C" phe_status phe_taa_resolve(uint32_t resX, uint32_t resY, const float* cur, const float* hist,
                                      const float* velocity, const float* prevVelocity, const float* roughness,
                                      float* outColor, float* outHist, void* stream)
{
	if (!cur || !hist || !outColor || !outHist) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_taa_resolve: null buffer");
	if (resX == 0 || resY == 0) return PHE_OK;
	dim3 block(16, 8);
	dim3 grid((resX + 15) / 16, (resY + 7) / 8);
	taa_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(resX, resY, (const float4*)cur, (const float4*)hist,
	                                                     (const float2*)velocity, (const float2*)prevVelocity, roughness,
	                                                     (float4*)outColor, (float4*)outHist);
	PHE_CUDA_TRY(cudaGetLastError(), "taa_kernel launch");
	return PHE_OK;
}
