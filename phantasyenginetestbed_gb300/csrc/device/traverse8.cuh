// Traversal of the 8-wide compressed layout (DeviceScene::nodes8, format in host/wide8.hpp) for rays
// whose 1/dir is finite, in the manner of Ylitie, Karras and Laine (HPG 2017): one node fetch tests up
// to 8 child boxes, hit inner children are kept as one stack entry (a node group: the children's base
// index, the inner-child mask and the keys still to visit), hit leaf children are visited right after
// their node, and children are taken in the order of (slot XOR ray octant), which the builder's slot
// assignment makes close to front to back.
//
// Exactness. A quantized child box contains the exact box it stands for, and its slab distances are
// computed with directed rounding: the entry distance rounded down and the exit distance rounded up,
// from bounds decoded exactly from their grid bytes. Since (b - o) x (1/d) rounds monotonically in b,
// the quantized test passes whenever the reference's test of the exact box does (for the same current
// best t), so the traversal reaches every leaf the binary traversal reaches. Before testing a leaf's
// triangles the leaf's exact box is tested with the reference arithmetic (visit_box), and because every
// child box lies inside its parent's box (checked when the layout is built) that test passing is what
// the binary traversal requires of all the leaf's ancestors. Triangle tests and the accept rule are
// the binary traversal's, so results are the same up to equal-t ties between distinct triangles
// (the near-tie rule).
// Included by traverse.cuh after the binary traversal's definitions (RayState, visit_box, intersect_tri).
#pragma once

namespace phe_gb300 {

// A node group per traversal level; the layout's depth is at most the binary depth (64), plus margin.
constexpr int kStackSize8 = 68;

// Bit i of the result is bit (i XOR oct) of m (8-bit masks).
__device__ __forceinline__ uint32_t perm8(uint32_t m, uint32_t oct)
{
	m = (oct & 1u) ? (((m & 0x55u) << 1) | ((m >> 1) & 0x55u)) : m;
	m = (oct & 2u) ? (((m & 0x33u) << 2) | ((m >> 2) & 0x33u)) : m;
	m = (oct & 4u) ? (((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu)) : m;
	return m;
}

// Grid byte c of a child bound as the exact float 2^23 + q.
template <int C>
__device__ __forceinline__ float grid_byte(uint32_t w0, uint32_t w1)
{
	return __uint_as_float(__byte_perm(C < 4 ? w0 : w1, 0x4B000000u, 0x7540u | (uint32_t)(C & 3)));
}

struct Wide8Ray {
	float so[3];     // sigma * origin, sigma = sign of the direction component
	float a[3];      // |1 / dir|
	uint32_t oct;    // bit i set when dir component i is negative
	bool neg[3];
};

__device__ __forceinline__ Wide8Ray wide8_ray(const RayState& r)
{
	Wide8Ray w;
	const float d[3] = {r.d.x, r.d.y, r.d.z}, o[3] = {r.o.x, r.o.y, r.o.z}, inv[3] = {r.inv.x, r.inv.y, r.inv.z};
	w.oct = 0;
#pragma unroll
	for (int k = 0; k < 3; k++) {
		w.neg[k] = d[k] < 0.0f;
		w.so[k] = w.neg[k] ? -o[k] : o[k];
		w.a[k] = fabsf(inv[k]);
		w.oct |= w.neg[k] ? (1u << k) : 0u;
	}
	return w;
}

// Slab test of child C on one axis in sigma space: entry distance rounded down, exit rounded up.
template <int C>
__device__ __forceinline__ void axis_span(uint32_t n0, uint32_t n1, uint32_t f0, uint32_t f1, float ss, float sp, float so,
                                          float a, float& tn, float& tf)
{
	float bn = __fmaf_rn(grid_byte<C>(n0, n1), ss, sp);   // exact: (k + q) * 2^e, sign applied
	float bf = __fmaf_rn(grid_byte<C>(f0, f1), ss, sp);
	tn = __fmul_rd(__fsub_rd(bn, so), a);
	tf = __fmul_ru(__fsub_ru(bf, so), a);
}

// Tests the 8 child boxes of node n; returns the hit mask in slot order and the node's header words.
__device__ __forceinline__ uint32_t wide8_node(const uint4* __restrict__ nodes8, uint32_t n, const Wide8Ray& w,
                                               float tMin, float tCur, uint4& hdr1, uint32_t& imask)
{
	const uint4* np = nodes8 + 5 * (size_t)n;
	const uint4 h0 = __ldg(np);
	hdr1 = __ldg(np + 1);
	const uint4 bx = __ldg(np + 2), by = __ldg(np + 3), bz = __ldg(np + 4);
	const uint32_t meta = h0.w;
	imask = meta >> 24;
	// 2^e with the sign of the direction: (e + 127) << 23 = ((byte) - 1) << 23 for byte = e + 128
	const float ssx = __uint_as_float(((((meta >> 0) & 0xFFu) - 1u) << 23) | (w.neg[0] ? 0x80000000u : 0u));
	const float ssy = __uint_as_float(((((meta >> 8) & 0xFFu) - 1u) << 23) | (w.neg[1] ? 0x80000000u : 0u));
	const float ssz = __uint_as_float(((((meta >> 16) & 0xFFu) - 1u) << 23) | (w.neg[2] ? 0x80000000u : 0u));
	const float spx = w.neg[0] ? -__uint_as_float(h0.x) : __uint_as_float(h0.x);
	const float spy = w.neg[1] ? -__uint_as_float(h0.y) : __uint_as_float(h0.y);
	const float spz = w.neg[2] ? -__uint_as_float(h0.z) : __uint_as_float(h0.z);
	// entry planes: lo bytes for a positive direction component, hi bytes for a negative one
	const uint32_t nx0 = w.neg[0] ? bx.z : bx.x, nx1 = w.neg[0] ? bx.w : bx.y;
	const uint32_t fx0 = w.neg[0] ? bx.x : bx.z, fx1 = w.neg[0] ? bx.y : bx.w;
	const uint32_t ny0 = w.neg[1] ? by.z : by.x, ny1 = w.neg[1] ? by.w : by.y;
	const uint32_t fy0 = w.neg[1] ? by.x : by.z, fy1 = w.neg[1] ? by.y : by.w;
	const uint32_t nz0 = w.neg[2] ? bz.z : bz.x, nz1 = w.neg[2] ? bz.w : bz.y;
	const uint32_t fz0 = w.neg[2] ? bz.x : bz.z, fz1 = w.neg[2] ? bz.y : bz.w;
	uint32_t hits = 0;
#define PHE_WIDE8_CHILD(C)                                                                          \
	{                                                                                               \
		float tnx, tfx, tny, tfy, tnz, tfz;                                                         \
		axis_span<C>(nx0, nx1, fx0, fx1, ssx, spx, w.so[0], w.a[0], tnx, tfx);                       \
		axis_span<C>(ny0, ny1, fy0, fy1, ssy, spy, w.so[1], w.a[1], tny, tfy);                       \
		axis_span<C>(nz0, nz1, fz0, fz1, ssz, spz, w.so[2], w.a[2], tnz, tfz);                       \
		const float tin = fmaxf(fmaxf(tnx, tny), tnz);                                              \
		const float tout = fminf(fminf(tfx, tfy), tfz);                                             \
		hits |= (tout >= tin && tout > tMin && tin < tCur) ? (1u << C) : 0u;                        \
	}
	PHE_WIDE8_CHILD(0) PHE_WIDE8_CHILD(1) PHE_WIDE8_CHILD(2) PHE_WIDE8_CHILD(3)
	PHE_WIDE8_CHILD(4) PHE_WIDE8_CHILD(5) PHE_WIDE8_CHILD(6) PHE_WIDE8_CHILD(7)
#undef PHE_WIDE8_CHILD
	return hits & hdr1.z;   // valid slots only
}

struct Wide8Bounds {
	uint32_t numNodes8, numLeaves8, numSlots;
};

// Traverses the 8-wide layout for one ray (r.safe must hold). ANY = true stops at the first triangle
// with tMin <= t < tMax. Lanes of a warp alternate between a node phase (lanes without pending leaves
// intersect nodes until every active lane has leaves or is done) and a leaf phase. Returns error bits.
template <bool ANY>
__device__ __forceinline__ uint32_t traverse8(const uint4* __restrict__ nodes8, const float4* __restrict__ leaves8,
                                              const float4* __restrict__ tris, const Wide8Bounds& bd,
                                              const RayState& r, HitRecord& hit)
{
	const Wide8Ray w = wide8_ray(r);
	uint2 stack[kStackSize8];
	int sp = 0;
	int32_t node = 0;                 // next node to intersect, -1 when none
	uint32_t leafBase = 0, leafMask = 0, leafKeys = 0;
	bool done = false;
	uint32_t err = 0;
	for (;;) {
		// node phase
		while (__any_sync(__activemask(), !done && leafKeys == 0)) {
			if (done || leafKeys != 0) continue;
			if (node < 0) {
				if (sp == 0) {
					done = true;
					continue;
				}
				const uint2 top = stack[sp - 1];
				uint32_t keys = top.y >> 8;
				const uint32_t k = (uint32_t)__ffs(keys) - 1u;
				keys &= keys - 1u;
				const uint32_t s = k ^ w.oct;
				node = (int32_t)(top.x + (uint32_t)__popc((top.y & 0xFFu) & ((1u << s) - 1u)));
				if (keys) stack[sp - 1].y = (top.y & 0xFFu) | (keys << 8);
				else sp--;
			}
			if (kDeviceChecks && (uint32_t)node >= bd.numNodes8) {
				err |= kErrBadIndex;
				done = true;
				continue;
			}
			uint4 hdr1;
			uint32_t imask;
			const uint32_t hits = wide8_node(nodes8, (uint32_t)node, w, r.tMin, hit.t, hdr1, imask);
			node = -1;
			const uint32_t keys = perm8(hits, w.oct), ikeys = perm8(imask, w.oct);
			const uint32_t inner = keys & ikeys, leaves = keys & ~ikeys;
			if (inner) {
				if (sp >= kStackSize8) {
					err |= kErrStackOverflow;
					done = true;
					continue;
				}
				stack[sp++] = make_uint2(hdr1.x, imask | (inner << 8));
			}
			leafBase = hdr1.y;
			leafMask = hdr1.z & ~imask;
			leafKeys = leaves;
		}
		// leaf phase: the leaves of the last node intersected, nearest key first
		while (leafKeys) {
			const uint32_t k = (uint32_t)__ffs(leafKeys) - 1u;
			leafKeys &= leafKeys - 1u;
			const uint32_t li = leafBase + (uint32_t)__popc(leafMask & ((1u << (k ^ w.oct)) - 1u));
			if (kDeviceChecks && li >= bd.numLeaves8) {
				err |= kErrBadIndex;
				done = true;
				leafKeys = 0;
				break;
			}
			const float4 lo = __ldg(leaves8 + 2 * (size_t)li), hi = __ldg(leaves8 + 2 * (size_t)li + 1);
			float tIn;
			if (!visit_box<true>(r, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, hit.t, tIn)) continue;
			const uint32_t first = __float_as_uint(lo.w), count = __float_as_uint(hi.w);
			if (kDeviceChecks && (uint64_t)first + count > bd.numSlots) {
				err |= kErrBadIndex;
				done = true;
				leafKeys = 0;
				break;
			}
			for (uint32_t j = 0; j < count; j++) {
				const float4* tp = tris + 3 * (size_t)(first + j);
				const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
				float t, u, v;
				if (intersect_tri(ta, tb, tc, r.o, r.d, t, u, v) && r.tMin <= t && t < hit.t) {
					hit.slot = first + j;
					hit.t = t;
					hit.u = u;
					hit.v = v;
					if (ANY) {
						done = true;
						break;
					}
				}
			}
			if (ANY && done) leafKeys = 0;
		}
		if (!__any_sync(__activemask(), !done)) break;
	}
	return err;
}

} // namespace phe_gb300
