// BVH traversal for one ray per thread: the while-while loop of Aila & Laine ("Understanding the
// Efficiency of Ray Traversal on GPUs", HPG 2009) as the reference's kernels use it
// (RayCastKernel.cu:286-383): inner nodes are traversed until every active lane of the warp holds a
// postponed leaf, then leaves are intersected. Closest hit visits the nearer child first; any hit
// stops at the first accepted triangle.
//
// Child boxes are tested with the reference CPU arithmetic (Intersection.hpp:77-90,
// BVHTraversal.hpp:152-156): t = (bound - origin) * (1 / dir) per plane, the std::min/std::max
// reduction, and the visit rule hit && tOut > tMin && tIn < tCurrentMax. Box culling is therefore
// the same decision the CPU oracle makes for the same current best t. For rays whose 1/dir is finite
// no NaN can appear and fminf/fmaxf give the same values; other rays use the exact std::min/max
// selects (a NaN in the x lane culls a box on the CPU, a NaN in y or z does not).
#pragma once

#include "common.cuh"

namespace phe_gb300 {

struct RayState {
	f3 o, d, inv;
	float tMin, tMax;
	bool safe;
};

__device__ __forceinline__ RayState load_ray(const phe_ray_in* __restrict__ rays, uint32_t i)
{
	const float4* p = reinterpret_cast<const float4*>(rays + i);
	float4 a = ld_stream(p), b = ld_stream(p + 1);
	RayState r;
	r.o = mk3(a.x, a.y, a.z);
	r.tMin = a.w;
	r.d = mk3(b.x, b.y, b.z);
	r.tMax = b.w;
	r.inv = mk3(__frcp_rn(b.x), __frcp_rn(b.y), __frcp_rn(b.z));
	r.safe = isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(b.x) && isfinite(b.y) && isfinite(b.z) &&
	         isfinite(r.inv.x) && isfinite(r.inv.y) && isfinite(r.inv.z);
	return r;
}

template <bool SAFE>
__device__ __forceinline__ float mn(float a, float b) { return SAFE ? fminf(a, b) : stdmin(a, b); }
template <bool SAFE>
__device__ __forceinline__ float mx(float a, float b) { return SAFE ? fmaxf(a, b) : stdmax(a, b); }

template <bool SAFE>
__device__ __forceinline__ bool visit_box(const RayState& r, float lx, float ly, float lz, float hx, float hy, float hz,
                                          float tCur, float& tIn)
{
	float t1x = __fmul_rn(__fsub_rn(lx, r.o.x), r.inv.x);
	float t1y = __fmul_rn(__fsub_rn(ly, r.o.y), r.inv.y);
	float t1z = __fmul_rn(__fsub_rn(lz, r.o.z), r.inv.z);
	float t2x = __fmul_rn(__fsub_rn(hx, r.o.x), r.inv.x);
	float t2y = __fmul_rn(__fsub_rn(hy, r.o.y), r.inv.y);
	float t2z = __fmul_rn(__fsub_rn(hz, r.o.z), r.inv.z);
	float tmin = mx<SAFE>(mx<SAFE>(mn<SAFE>(t1x, t2x), mn<SAFE>(t1y, t2y)), mn<SAFE>(t1z, t2z));
	float tmax = mn<SAFE>(mn<SAFE>(mx<SAFE>(t1x, t2x), mx<SAFE>(t1y, t2y)), mx<SAFE>(t1z, t2z));
	tIn = tmin;
	return tmax >= tmin && tmax > r.tMin && tmin < tCur;
}

struct HitRecord {
	uint32_t slot;
	float t, u, v;
};

// Traversal stack of one thread. The first kSmemStack entries live in shared memory, one column per
// thread with a stride of the block size, so the 32 lanes of a warp always touch 32 different banks
// whatever their stack depths; deeper entries spill to a per-thread local array. Kernels that
// traverse use 1-D blocks and are launched with stack_smem_bytes(blockDim.x) of dynamic shared
// memory. kSmemStack = 0 keeps the whole stack in local memory (no shared memory).
#ifndef PHE_SMEM_STACK
#define PHE_SMEM_STACK 0
#endif
constexpr int kSmemStack = PHE_SMEM_STACK;
static_assert(kSmemStack >= 0 && kSmemStack <= kStackSize, "shared stack depth");
extern __shared__ int32_t g_stackSmem[];
inline size_t stack_smem_bytes(int block, int entries = kSmemStack)
{
	return (size_t)entries * sizeof(int32_t) * (size_t)block;
}

// SN: stack entries kept in shared memory (the batch autotuner instantiates other depths).
template <int SN>
struct TraversalStackT {
	static_assert(SN >= 0 && SN <= kStackSize, "shared stack depth");
	int32_t* col;
	uint32_t stride;
	int32_t spill[kStackSize - SN > 0 ? kStackSize - SN : 1];
	__device__ __forceinline__ TraversalStackT() : col(g_stackSmem + threadIdx.x), stride(blockDim.x) {}
	__device__ __forceinline__ void set(int i, int32_t v)
	{
		if (SN > 0 && i < SN) col[(uint32_t)i * stride] = v;
		else spill[i - SN] = v;
	}
	__device__ __forceinline__ int32_t get(int i) const
	{
		return (SN > 0 && i < SN) ? col[(uint32_t)i * stride] : spill[i - SN];
	}
};
using TraversalStack = TraversalStackT<kSmemStack>;

// Traverses the scene for one ray. ANY = true stops at the first triangle with tMin <= t < tMax.
// Returns the error bits (0, or kErrStackOverflow when the stack would overflow).
template <bool SAFE, bool ANY, int SN = kSmemStack>
__device__ __forceinline__ uint32_t traverse(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                             const TraversalBounds& bd, const RayState& r, HitRecord& hit)
{
	TraversalStackT<SN> stack;
	int sp = 0;
	stack.set(0, kSentinel);
	int32_t nodeAddr = 0;
	int32_t leafAddr = 0;
	uint32_t err = 0;

	while (nodeAddr != kSentinel) {
		while (nodeAddr >= 0 && nodeAddr != kSentinel) {
			if (kDeviceChecks && (uint32_t)nodeAddr >= bd.numNodes) {
				err |= kErrBadIndex;
				nodeAddr = kSentinel;
				leafAddr = 0;
				break;
			}
			const float4* np = nodes + 4 * (size_t)nodeAddr;
			float4 b0 = __ldg(np), b1 = __ldg(np + 1), b2 = __ldg(np + 2);
			int4 ix = __ldg(reinterpret_cast<const int4*>(np + 3));
			float tIn0, tIn1;
			bool v0 = visit_box<SAFE>(r, b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, hit.t, tIn0);
			bool v1 = visit_box<SAFE>(r, b1.z, b1.w, b2.x, b2.y, b2.z, b2.w, hit.t, tIn1);
			{
				const bool both = v0 && v1;
				const bool swp = !ANY && both && tIn1 < tIn0;
				int32_t nearC = (v0 && !swp) ? ix.x : ix.y;
				int32_t farC = swp ? ix.x : ix.y;
				if (both) {
					if (sp >= kStackSize - 1) {
						err |= kErrStackOverflow;
						nodeAddr = kSentinel;
						leafAddr = 0;
						break;
					}
					stack.set(++sp, farC);
				}
				nodeAddr = (v0 || v1) ? nearC : stack.get(sp--);
			}
			if (nodeAddr < 0 && leafAddr >= 0) {
				leafAddr = nodeAddr;
				nodeAddr = stack.get(sp--);
			}
			if (!__any_sync(__activemask(), leafAddr >= 0)) break;
		}

		while (leafAddr < 0) {
			int32_t slot = ~leafAddr;
			for (;;) {
				if (kDeviceChecks && (uint32_t)slot >= bd.numSlots) {
					err |= kErrBadIndex;
					nodeAddr = kSentinel;
					leafAddr = 0;
					break;
				}
				const float4* tp = tris + 3 * (size_t)slot;
				float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
				float t, u, v;
				if (intersect_tri(a, b, c, r.o, r.d, t, u, v) && r.tMin <= t && t < hit.t) {
					hit.slot = (uint32_t)slot;
					hit.t = t;
					hit.u = u;
					hit.v = v;
					if (ANY) {
						nodeAddr = kSentinel;
						leafAddr = 0;
						break;
					}
				}
				if (a.w < 0.0f) break;
				slot++;
			}
			if ((ANY || kDeviceChecks) && nodeAddr == kSentinel && leafAddr == 0) break;
			leafAddr = nodeAddr;
			if (nodeAddr < 0) nodeAddr = stack.get(sp--);
		}
	}
	return err;
}

// Initial record: no hit, current best = std::min(tMax, FLT_MAX) (the CPU castRay starts from
// FLT_MAX; RayCastKernel.cu:267 starts from maxDist).
__device__ __forceinline__ HitRecord empty_hit(const RayState& r)
{
	HitRecord h;
	h.slot = ~0u;
	h.t = stdmin(r.tMax, 3.402823466e+38f);
	h.u = 0.0f;
	h.v = 0.0f;
	return h;
}

// Compare-and-swap of (key, payload) pairs for the near-first order of a 4-wide node.
__device__ __forceinline__ void cswap(float& ka, int32_t& pa, float& kb, int32_t& pb)
{
	bool sw = kb < ka;
	float k = sw ? kb : ka;
	int32_t q = sw ? pb : pa;
	kb = sw ? ka : kb;
	pb = sw ? pa : pb;
	ka = k;
	pa = q;
}

// Traversal of the 4-wide layout (DeviceScene::nodes4) for rays whose 1/dir is finite. The four
// child boxes of a node are tested with the same arithmetic as the binary traversal; hit children
// are visited nearest first (closest hit) and the others pushed. A child box lies inside the binary
// box it replaces and the rounded slab test is monotone in the box bounds, so a child passes here
// only if the skipped binary test would pass too: the set of reachable leaves is the binary one.
template <bool ANY>
__device__ __forceinline__ uint32_t traverse4(const float4* __restrict__ nodes4, const float4* __restrict__ tris,
                                              const TraversalBounds& bd, const RayState& r, HitRecord& hit)
{
	int32_t stack[kStackSize4];
	int sp = 0;
	stack[0] = kSentinel;
	int32_t nodeAddr = 0;
	int32_t leafAddr = 0;
	uint32_t err = 0;
	const float INF = __int_as_float(0x7f800000);

	while (nodeAddr != kSentinel) {
		while (nodeAddr >= 0 && nodeAddr != kSentinel) {
			if (kDeviceChecks && (uint32_t)nodeAddr >= bd.numNodes) {
				err |= kErrBadIndex;
				nodeAddr = kSentinel;
				leafAddr = 0;
				break;
			}
			const float4* np = nodes4 + 8 * (size_t)nodeAddr;
			float4 lx = __ldg(np), ly = __ldg(np + 1), lz = __ldg(np + 2);
			float4 hx = __ldg(np + 3), hy = __ldg(np + 4), hz = __ldg(np + 5);
			int4 ref = __ldg(reinterpret_cast<const int4*>(np + 6));
			float t0, t1, t2, t3;
			bool v0 = visit_box<true>(r, lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, hit.t, t0) && ref.x != kEmptyChild;
			bool v1 = visit_box<true>(r, lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, hit.t, t1) && ref.y != kEmptyChild;
			bool v2 = visit_box<true>(r, lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, hit.t, t2) && ref.z != kEmptyChild;
			bool v3 = visit_box<true>(r, lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, hit.t, t3) && ref.w != kEmptyChild;
			int nhit = (int)v0 + (int)v1 + (int)v2 + (int)v3;
			if (nhit == 0) {
				nodeAddr = stack[sp--];
			} else {
				float k0 = v0 ? t0 : INF, k1 = v1 ? t1 : INF, k2 = v2 ? t2 : INF, k3 = v3 ? t3 : INF;
				int32_t c0 = ref.x, c1 = ref.y, c2 = ref.z, c3 = ref.w;
				if (ANY) {
					// no order needed: compact the hit children to the front
					if (!v0) { k0 = k1; c0 = c1; k1 = k2; c1 = c2; k2 = k3; c2 = c3; v0 = v1; v1 = v2; v2 = v3; }
					if (!v0) { k0 = k1; c0 = c1; k1 = k2; c1 = c2; v0 = v1; v1 = v2; }
					if (!v0) { c0 = c1; }
					if (nhit > 1 && !v1) { c1 = c2; c2 = c3; v1 = v2; }
					if (nhit > 1 && !v1) { c1 = c2; }
					if (nhit > 2 && !v2) { c2 = c3; }
				} else {
					cswap(k0, c0, k1, c1);
					cswap(k2, c2, k3, c3);
					cswap(k0, c0, k2, c2);
					cswap(k1, c1, k3, c3);
					cswap(k1, c1, k2, c2);
				}
				if (sp + 3 >= kStackSize4 - 1) {
					err |= kErrStackOverflow;
					nodeAddr = kSentinel;
					leafAddr = 0;
					break;
				}
				if (nhit > 3) stack[++sp] = c3;
				if (nhit > 2) stack[++sp] = c2;
				if (nhit > 1) stack[++sp] = c1;
				nodeAddr = c0;
			}
			if (nodeAddr < 0 && leafAddr >= 0) {
				leafAddr = nodeAddr;
				nodeAddr = stack[sp--];
			}
			if (!__any_sync(__activemask(), leafAddr >= 0)) break;
		}

		while (leafAddr < 0) {
			int32_t slot = ~leafAddr;
			for (;;) {
				if (kDeviceChecks && (uint32_t)slot >= bd.numSlots) {
					err |= kErrBadIndex;
					nodeAddr = kSentinel;
					leafAddr = 0;
					break;
				}
				const float4* tp = tris + 3 * (size_t)slot;
				float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
				float t, u, v;
				if (intersect_tri(a, b, c, r.o, r.d, t, u, v) && r.tMin <= t && t < hit.t) {
					hit.slot = (uint32_t)slot;
					hit.t = t;
					hit.u = u;
					hit.v = v;
					if (ANY) {
						nodeAddr = kSentinel;
						leafAddr = 0;
						break;
					}
				}
				if (a.w < 0.0f) break;
				slot++;
			}
			if ((ANY || kDeviceChecks) && nodeAddr == kSentinel && leafAddr == 0) break;
			leafAddr = nodeAddr;
			if (nodeAddr < 0) nodeAddr = stack[sp--];
		}
	}
	return err;
}

} // namespace phe_gb300

#include "traverse8.cuh"

namespace phe_gb300 {

// WIDE = false compiles the binary traversal only; kernels are instantiated for both and the host
// launches the WIDE one only for scenes whose 4-wide or 8-wide layout is selected, so binary launches
// carry neither the wide code nor its stacks. Rays with a non-finite 1/dir always take the binary
// nodes (the wide tests assume finite slab distances).
template <bool ANY, bool WIDE = false, int SN = kSmemStack>
__device__ __forceinline__ uint32_t trace(const DeviceScene& s, const RayState& r, HitRecord& hit)
{
	if (r.safe) {
		if constexpr (WIDE) {
			if (s.nodes8)
				return traverse8<ANY>(s.nodes8, s.leaves8, s.tris, Wide8Bounds{s.numNodes8, s.numLeaves8, s.numSlots}, r, hit);
			if (s.nodes4) return traverse4<ANY>(s.nodes4, s.tris, TraversalBounds{s.numNodes4, s.numSlots}, r, hit);
		}
		return traverse<true, ANY, SN>(s.nodes, s.tris, TraversalBounds{s.numNodes, s.numSlots}, r, hit);
	}
	return traverse<false, ANY, SN>(s.nodes, s.tris, TraversalBounds{s.numNodes, s.numSlots}, r, hit);
}

__device__ __forceinline__ void store_hit(phe_ray_hit* __restrict__ hits, uint32_t i, const RayState& r, const HitRecord& h)
{
	float4 o;
	if (h.slot != ~0u) o = make_float4(__uint_as_float(h.slot), h.t, h.u, h.v);
	else o = make_float4(__uint_as_float(~0u), r.tMax, 0.0f, 0.0f);
	st_stream(reinterpret_cast<float4*>(hits) + i, o);
}

} // namespace phe_gb300

namespace phe_gb300 {

// ------------------------------------------------------------------------------------------------
// Persistent traversal with lane refill (Aila & Laine 2009, "persistent while-while" with dynamic ray
// fetch; the reference does the same with a threshold of 20 lanes, RayCastKernel.cu:225-393). Every
// lane keeps its own ray state across outer iterations; when fewer than `refill` lanes of a warp are
// still traversing, the warp leaves the traversal loop, idle lanes take new rays (one atomic per warp)
// and traversal resumes. Divergent incoherent rays then keep more lanes busy than with a fixed
// 32-ray batch per warp.
//
// Source: `RayState load(uint32_t i)` for i < n. Sink: `void store(uint32_t i, const RayState&, const
// HitRecord&)`, called once per ray when its traversal ends.
// ------------------------------------------------------------------------------------------------
template <bool ANY, bool SAFE>
__device__ __forceinline__ void trace_step(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                           const TraversalBounds& bd, const RayState& r, HitRecord& hit,
                                           TraversalStack& stack, int& sp, int32_t& nodeAddr, int32_t& leafAddr,
                                           uint32_t& err)
{
	while (nodeAddr >= 0 && nodeAddr != kSentinel) {
		if (kDeviceChecks && (uint32_t)nodeAddr >= bd.numNodes) {
			err |= kErrBadIndex;
			nodeAddr = kSentinel;
			leafAddr = 0;
			return;
		}
		const float4* np = nodes + 4 * (size_t)nodeAddr;
		float4 b0 = __ldg(np), b1 = __ldg(np + 1), b2 = __ldg(np + 2);
		int4 ix = __ldg(reinterpret_cast<const int4*>(np + 3));
		float tIn0, tIn1;
		bool v0 = visit_box<SAFE>(r, b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, hit.t, tIn0);
		bool v1 = visit_box<SAFE>(r, b1.z, b1.w, b2.x, b2.y, b2.z, b2.w, hit.t, tIn1);
		if (!v0 && !v1) {
			nodeAddr = stack.get(sp--);
		} else {
			nodeAddr = v0 ? ix.x : ix.y;
			if (v0 && v1) {
				int32_t other = ix.y;
				if (!ANY && tIn1 < tIn0) {
					other = ix.x;
					nodeAddr = ix.y;
				}
				if (sp >= kStackSize - 1) {
					err |= kErrStackOverflow;
					nodeAddr = kSentinel;
					leafAddr = 0;
					return;
				}
				stack.set(++sp, other);
			}
		}
		if (nodeAddr < 0 && leafAddr >= 0) {
			leafAddr = nodeAddr;
			nodeAddr = stack.get(sp--);
		}
		if (!__any_sync(__activemask(), leafAddr >= 0)) break;
	}
	while (leafAddr < 0) {
		int32_t slot = ~leafAddr;
		for (;;) {
			if (kDeviceChecks && (uint32_t)slot >= bd.numSlots) {
				err |= kErrBadIndex;
				nodeAddr = kSentinel;
				leafAddr = 0;
				return;
			}
			const float4* tp = tris + 3 * (size_t)slot;
			float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
			float t, u, v;
			if (intersect_tri(a, b, c, r.o, r.d, t, u, v) && r.tMin <= t && t < hit.t) {
				hit.slot = (uint32_t)slot;
				hit.t = t;
				hit.u = u;
				hit.v = v;
				if (ANY) {
					nodeAddr = kSentinel;
					leafAddr = 0;
					return;
				}
			}
			if (a.w < 0.0f) break;
			slot++;
		}
		leafAddr = nodeAddr;
		if (nodeAddr < 0) nodeAddr = stack.get(sp--);
	}
}

template <bool ANY, class Source, class Sink>
__device__ __forceinline__ uint32_t persistent_trace(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                                     const TraversalBounds& bd, const Source& src, const Sink& sink,
                                                     uint32_t n,
                                                     uint32_t* __restrict__ counter, int refill)
{
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t below = (1u << lane) - 1u;
	TraversalStack stack;
	int sp = 0;
	int32_t nodeAddr = kSentinel, leafAddr = 0;
	RayState r;
	HitRecord h;
	h.slot = ~0u;
	h.t = 0.0f;
	h.u = h.v = 0.0f;
	r.safe = true;
	uint32_t rayIdx = 0, err = 0;
	bool hasRay = false, exhausted = false;
	for (;;) {
		bool need = !hasRay && !exhausted;
		uint32_t needMask = __ballot_sync(0xFFFFFFFFu, need);
		if (needMask) {
			uint32_t leader = (uint32_t)__ffs(needMask) - 1u;
			uint32_t base = 0;
			if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(needMask));
			base = __shfl_sync(0xFFFFFFFFu, base, leader);
			if (need) {
				rayIdx = base + (uint32_t)__popc(needMask & below);
				if (rayIdx < n) {
					r = src.load(rayIdx);
					h = empty_hit(r);
					sp = 0;
					stack.set(0, kSentinel);
					nodeAddr = 0;
					leafAddr = 0;
					hasRay = true;
				} else {
					exhausted = true;
				}
			}
		}
		if (!__any_sync(0xFFFFFFFFu, hasRay)) break;
		if (hasRay) {
			if (r.safe) {
				while (nodeAddr != kSentinel) {
					trace_step<ANY, true>(nodes, tris, bd, r, h, stack, sp, nodeAddr, leafAddr, err);
					if (__popc(__activemask()) < refill) break;
				}
			} else {
				while (nodeAddr != kSentinel) {
					trace_step<ANY, false>(nodes, tris, bd, r, h, stack, sp, nodeAddr, leafAddr, err);
					if (__popc(__activemask()) < refill) break;
				}
			}
			if (nodeAddr == kSentinel) {
				sink.store(rayIdx, r, h);
				hasRay = false;
			}
		}
		__syncwarp();
	}
	return err;
}

} // namespace phe_gb300
