// Device helpers shared by the kernels: explicitly rounded FP32 arithmetic in the reference's
// operation order (sfz vector math, externals/sfzCore/include/sfz/math/Vector.inl), the device-side
// scene layout, PCG32 and the sampling sine/cosine. Every float operation that decides a hit or a
// sampled direction goes through __fadd_rn/__fsub_rn/__fmul_rn/__fdiv_rn/__fsqrt_rn, which the
// compiler never fuses, so results equal the host's IEEE single-precision results bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "phe_gb300.h"

namespace phe_gb300 {

// ------------------------------------------------------------------------------------------------
// Device scene layout (built on upload from the reference arrays)
//
// nodes: 64 B per node, 4 x float4 — bytes 0..47 are the reference fData (child boxes), bytes
//        48..63 are (child0, child1, count0, count1) with inner children as node indices >= 0 and
//        leaf children as ~firstSlot (< 0); count is 0 for inner children.
// tris:  48 B per slot, 3 x float4 — (p0.xyz, endMarker), (e1 = p1 - p0, 0), (e2 = p2 - p0, 0).
//        e1 and e2 are the exact float subtractions Moller-Trumbore performs first, so storing them
//        changes no result bit. endMarker is -1 on the last slot of each leaf, else 0.
// ------------------------------------------------------------------------------------------------

// nodes4 (optional): the same tree collapsed to 4-wide nodes, 128 B each — 6 float4 of child bounds
//        in SoA order (lo.x[4], lo.y[4], lo.z[4], hi.x[4], hi.y[4], hi.z[4]), one int4 of child refs
//        (4-wide node index >= 0, leaf ~firstSlot < 0, kEmptyChild for an unused slot) and one float4
//        of padding. Every child box is a box of the binary tree (a grandchild when the binary child
//        is inner), and it is built only when each grandchild box lies inside its parent box, so the
//        4-wide test of a grandchild passes only if the skipped binary test of its parent would pass.
// nodes8 / leaves8 (optional): the 8-wide compressed layout, 80 B per node and 32 B per leaf record
//        (format in host/wide8.hpp, traversal in traverse8.cuh).
// Textures of a scene: texels of texture k start at texels + offset (rows rowBytes apart, tightly
// packed); srgb[b] = powf(b / 255, 2.2) correctly rounded.
struct DeviceTexture {
	uint64_t offset;
	int32_t width, height;
	uint32_t bytesPerPixel, rowBytes;
};
static_assert(sizeof(DeviceTexture) == 24, "DeviceTexture is 24 bytes");

struct DeviceScene {
	const float4* nodes;
	const float4* tris;
	const phe_triangle_data* datas;
	const phe_material* materials;
	uint32_t numNodes, numSlots, numMaterials, numNodes4;
	const float4* nodes4;
	uint32_t* status;   // device word: OR of the error bits any kernel raised on this scene
	const DeviceTexture* textures;
	const uint8_t* texels;
	const float* srgb;
	uint32_t numTextures, pad;
	const uint4* nodes8;    // set only while the 8-wide layout is selected (host/wide8.hpp)
	const float4* leaves8;  // its leaf records
	uint32_t numNodes8, numLeaves8, pad2[2];
};
static_assert(sizeof(DeviceScene) == 128, "DeviceScene is 128 bytes");

constexpr int32_t kEmptyChild = 0x7FFFFFFE;

// Traversal stack depth: leaves of a valid scene are at most 64 levels deep, and a node pushes at
// most one entry per inner level, plus the sentinel.
constexpr int kStackSize = 68;
// 4-wide traversal: a node pushes up to 3 entries; a binary tree of depth <= 64 collapses to <= 32 levels.
constexpr int kStackSize4 = 100;
constexpr int32_t kSentinel = 0x7FFFFFFF;

// Error bits written to the per-launch status word.
constexpr uint32_t kErrStackOverflow = 1u;
constexpr uint32_t kErrBadIndex = 2u;   // checked build: a node or slot index outside its array

// The checked build (-DPHE_DEVICE_CHECKS=1, libphe_gb300_checked.so) tests every node and slot index a
// traversal is about to read against the array sizes; an index outside sets kErrBadIndex and ends that
// ray (no trap, no out-of-bounds access). The normal build relies on the host validation of the tree
// done at upload, and these tests compile away.
#ifndef PHE_DEVICE_CHECKS
#define PHE_DEVICE_CHECKS 0
#endif
constexpr bool kDeviceChecks = PHE_DEVICE_CHECKS != 0;
struct TraversalBounds {
	uint32_t numNodes;   // nodes of the layout being traversed (binary or 4-wide)
	uint32_t numSlots;
};

// Cache hints for data that is read or written once per launch (rays in, hits out, the frame's queues
// and contributions): with kStreamHints they use the evict-first ("streaming") cache policy, so these
// streams do not push scene nodes and triangles out of L2. Plain loads through the read-only path and
// plain stores otherwise.
#ifndef PHE_STREAM_HINTS
#define PHE_STREAM_HINTS 1
#endif
constexpr bool kStreamHints = PHE_STREAM_HINTS != 0;
template <class T>
__device__ __forceinline__ T ld_stream(const T* p)
{
	if constexpr (kStreamHints) return __ldcs(p);
	else return __ldg(p);
}
template <class T>
__device__ __forceinline__ void st_stream(T* p, T v)
{
	if constexpr (kStreamHints) __stcs(p, v);
	else *p = v;
}

struct f3 { float x, y, z; };

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return mk3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ f3 mul3(f3 a, f3 b) { return mk3(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)); }
__device__ __forceinline__ f3 muls3(f3 a, float s) { return mk3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
__device__ __forceinline__ f3 divs3(f3 a, float s) { return mk3(__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)); }
__device__ __forceinline__ float dot3(f3 a, f3 b)
{
	return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ f3 cross3(f3 a, f3 b)
{
	return mk3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
	           __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float length3(f3 a) { return __fsqrt_rn(dot3(a, a)); }
__device__ __forceinline__ f3 normalize3(f3 a) { return divs3(a, length3(a)); }
// std::min / std::max semantics (b < a ? b : a / a < b ? b : a), including NaN behaviour.
__device__ __forceinline__ float stdmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float stdmax(float a, float b) { return (a < b) ? b : a; }

// ------------------------------------------------------------------------------------------------
// Moller-Trumbore with the reference's absolute determinant epsilon (Intersection.hpp:24-67,
// RayCastKernel.cu:96-131), on a slot stored as (p0, e1, e2). Returns true on a hit.
//
// Every quantity is computed with the reference's operations and rounding; only the control flow
// differs. The reference returns early after the determinant, u and v tests; here all of u, v and t
// are computed and the same three tests are combined into one predicate, so a rejected triangle gives
// the same answer. In a warp the early returns saved little (the warp runs until its last lane
// rejects), while the straight-line form has no branches and overlaps the reciprocal with the other
// products. f = rn(1 / det) is taken as the correctly rounded reciprocal, the same value as the
// correctly rounded quotient 1.0f / det.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ bool intersect_tri(float4 a, float4 b, float4 c, f3 o, f3 d, float& t, float& u, float& v)
{
	const float EPS = 0.00001f;
	f3 p0 = mk3(a.x, a.y, a.z), e1 = mk3(b.x, b.y, b.z), e2 = mk3(c.x, c.y, c.z);
	f3 q = cross3(d, e2);
	float det = dot3(e1, q);
	f3 s = sub3(o, p0);
	f3 r = cross3(s, e1);
	float f = __frcp_rn(det);
	float uu = __fmul_rn(f, dot3(s, q));
	float vv = __fmul_rn(f, dot3(d, r));
	t = __fmul_rn(f, dot3(e2, r));
	u = uu;
	v = vv;
	return !(-EPS < det && det < EPS) && !(uu < 0.0f) && !(vv < 0.0f || __fadd_rn(uu, vv) > 1.0f);
}

// ------------------------------------------------------------------------------------------------
// PCG32 (O'Neill 2014), identical to the host generator (host/pcg.hpp).
// ------------------------------------------------------------------------------------------------
struct DevPcg {
	uint64_t state, inc;
	__device__ __forceinline__ uint32_t next()
	{
		uint64_t old = state;
		state = old * 6364136223846793005ull + inc;
		uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
		uint32_t rot = (uint32_t)(old >> 59u);
		return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
	}
	__device__ __forceinline__ void seed(uint64_t initstate, uint64_t initseq)
	{
		state = 0u;
		inc = (initseq << 1u) | 1u;
		next();
		state += initstate;
		next();
	}
	__device__ __forceinline__ float uniform() { return __fmul_rn((float)(next() >> 8), 0x1.0p-24f); }
};

// Stream of pixel `pixel` for shading stage `stage` of frame `frame`.
__device__ __forceinline__ void pixel_stream(DevPcg& r, uint64_t seed, uint32_t frame, uint32_t pixel, uint32_t stage)
{
	uint64_t initstate = seed ^ ((uint64_t)frame * 0x9E3779B97F4A7C15ull);
	uint64_t initseq = ((uint64_t)pixel << 2) | (uint64_t)(stage & 3u);
	r.seed(initstate, initseq);
}

// sin(2 pi r), cos(2 pi r) for r in [0, 1): exact quadrant reduction, then Taylor polynomials of
// degree 9 (sine) and 10 (cosine) on [0, pi/4] evaluated in Horner form with single roundings.
// Truncation error below 2e-9; the host restatement performs the same operations.
__device__ __forceinline__ void sincos_2pi(float r, float& s, float& c)
{
	float q = __fmul_rn(r, 4.0f);
	int k = (int)q;
	k = k > 3 ? 3 : (k < 0 ? 0 : k);
	float f = __fsub_rn(q, (float)k);
	bool swap = f > 0.5f;
	float g = swap ? __fsub_rn(1.0f, f) : f;
	float x = __fmul_rn(g, 0x1.921fb6p+0f);
	float x2 = __fmul_rn(x, x);
	float sp = __fmul_rn(x, __fadd_rn(1.0f, __fmul_rn(x2, __fadd_rn(-0x1.555556p-3f, __fmul_rn(x2, __fadd_rn(0x1.111112p-7f,
	                         __fmul_rn(x2, __fadd_rn(-0x1.a01a02p-13f, __fmul_rn(x2, 0x1.71de3ap-19f)))))))));
	float cp = __fadd_rn(1.0f, __fmul_rn(x2, __fadd_rn(-0x1.0p-1f, __fmul_rn(x2, __fadd_rn(0x1.555556p-5f,
	                         __fmul_rn(x2, __fadd_rn(-0x1.6c16c2p-10f, __fmul_rn(x2, __fsub_rn(0x1.a01a02p-16f,
	                         __fmul_rn(x2, 0x1.27e4fcp-22f))))))))));
	float sq = swap ? cp : sp;
	float cq = swap ? sp : cp;
	switch (k) {
	case 0: s = sq; c = cq; break;
	case 1: s = cq; c = -sq; break;
	case 2: s = -sq; c = -cq; break;
	default: s = -cq; c = sq; break;
	}
}

} // namespace phe_gb300
