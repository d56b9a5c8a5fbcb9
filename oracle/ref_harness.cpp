// Test infrastructure only: a thin extern "C" harness around the reference's own CPU ray-cast
// path, compiled from the reference sources where they lie by oracle/Makefile into
// oracle/_ref/libpheref.so. Nothing in the product links this file. It exists to pin the
// oracle restatement (oracle/oracle.c) against the reference itself and to generate the
// committed golden fixtures under tests/golden/.
//
// Reference entry points wrapped here (paths relative to the reference project root):
//   buildStaticFrom + sanitizeBVH   source/phantasy_engine/ray_tracer_common/StaticBVHBuilder.cpp:213-260
//   castRay / castDebugRay          source/phantasy_engine/ray_tracer_common/BVHTraversal.hpp:37-235
//   intersects (triangle)           source/phantasy_engine/ray_tracer_common/Intersection.hpp:24-67
//   generateCameraDef               source/phantasy_engine/ray_tracer_common/GenerateRays.cpp:12-35

#include <cstdint>
#include <cstring>
#include <cstdio>
#include <thread>
#include <vector>

#include "phantasy_engine/ray_tracer_common/BVH.hpp"
#include "phantasy_engine/ray_tracer_common/BVHTraversal.hpp"
#include "phantasy_engine/ray_tracer_common/GenerateRays.hpp"
#include "phantasy_engine/ray_tracer_common/StaticBVHBuilder.hpp"

using namespace phe;

namespace {

struct RefBVH {
	DynArray<BVHNode> nodes;
	DynArray<TriangleVertices> verts;
	DynArray<TriangleData> datas;
};

} // namespace

extern "C" {

// Builds the reference SBVH (default BuildParams / Platform) over `numTris` triangles given as
// 9 floats each (v0.xyz v1.xyz v2.xyz) and sanitizes it. Each output slot's original triangle index
// is recovered by passing the index through TriangleData::materialIndex (the builder copies
// TriangleData per slot, StaticBVHBuilder.cpp:242-245). Returns an opaque handle.
void* ref_build_sbvh(const float* triVerts, const uint32_t* materialIndices, uint32_t numTris)
{
	DynArray<TriangleVertices> inTris;
	DynArray<TriangleData> inDatas;
	inTris.ensureCapacity(numTris);
	inDatas.ensureCapacity(numTris);
	for (uint32_t i = 0; i < numTris; i++) {
		const float* p = triVerts + 9 * size_t(i);
		TriangleVertices tv;
		tv.v0 = sfz::vec4(p[0], p[1], p[2], 0.0f);
		tv.v1 = sfz::vec4(p[3], p[4], p[5], 0.0f);
		tv.v2 = sfz::vec4(p[6], p[7], p[8], 0.0f);
		inTris.add(tv);
		TriangleData td;
		std::memset(&td, 0, sizeof(td));
		td.materialIndex = i;
		inDatas.add(td);
	}
	(void)materialIndices;
	BVH bvh = buildStaticFrom(inTris, inDatas);
	sanitizeBVH(bvh);
	RefBVH* out = new RefBVH();
	out->nodes = std::move(bvh.nodes);
	out->verts = std::move(bvh.triangleVerts);
	out->datas = std::move(bvh.triangleDatas);
	return out;
}

void ref_bvh_sizes(const void* h, uint32_t* numNodes, uint32_t* numSlots)
{
	const RefBVH* b = (const RefBVH*)h;
	*numNodes = b->nodes.size();
	*numSlots = b->verts.size();
}

// Copies the sanitized arrays out: nodes (64 B each), slot vertices (48 B each) and the
// slot -> original triangle map.
void ref_bvh_copy(const void* h, void* nodes, void* verts, uint32_t* slotToTri)
{
	const RefBVH* b = (const RefBVH*)h;
	std::memcpy(nodes, b->nodes.data(), sizeof(BVHNode) * b->nodes.size());
	std::memcpy(verts, b->verts.data(), sizeof(TriangleVertices) * b->verts.size());
	for (uint32_t i = 0; i < b->datas.size(); i++) slotToTri[i] = b->datas[i].materialIndex;
}

void ref_bvh_free(void* h) { delete (RefBVH*)h; }

// Closest hit through the reference castRay for `n` rays in RayIn layout
// (origin.xyz, tMin, dir.xyz, tMax). Output in RayHit layout (slot, t, u, v).
// `debug` (optional) receives nodesVisited and triangleIntersectionTests per ray from castDebugRay.
void ref_cast_rays(const void* nodes, const void* verts, const float* rays, uint32_t n,
                   uint32_t* hits, uint32_t* debug, int numThreads)
{
	const BVHNode* nd = (const BVHNode*)nodes;
	const TriangleVertices* tv = (const TriangleVertices*)verts;
	if (numThreads < 1) numThreads = 1;
	auto work = [&](uint32_t begin, uint32_t end) {
		for (uint32_t i = begin; i < end; i++) {
			const float* r = rays + 8 * size_t(i);
			Ray ray(sfz::vec3(r[0], r[1], r[2]), sfz::vec3(r[4], r[5], r[6]));
			RayCastResult res;
			if (debug) {
				DebugRayCastData dbg;
				res = castDebugRay(nd, tv, ray, &dbg, r[3], r[7]);
				debug[2 * size_t(i)] = dbg.nodesVisited;
				debug[2 * size_t(i) + 1] = dbg.triangleIntersectionTests;
			} else {
				res = castRay(nd, tv, ray, r[3], r[7]);
			}
			uint32_t* o = hits + 4 * size_t(i);
			o[0] = res.triangleIndex;
			std::memcpy(&o[1], &res.t, 4);
			std::memcpy(&o[2], &res.u, 4);
			std::memcpy(&o[3], &res.v, 4);
		}
	};
	std::vector<std::thread> threads;
	uint32_t chunk = (n + numThreads - 1) / numThreads;
	for (int t = 0; t < numThreads; t++) {
		uint32_t b = t * chunk, e = b + chunk < n ? b + chunk : n;
		if (b >= e) break;
		threads.emplace_back(work, b, e);
	}
	for (auto& th : threads) th.join();
}

// Any hit through the reference castRay, the way the reference's CPU path would answer a shadow
// query (it has no any-hit traversal): inLight[i] = 1 when castRay(ray, tMin, tMax) finds no triangle.
void ref_any_rays(const void* nodes, const void* verts, const float* rays, uint32_t n, uint8_t* inLight,
                  int numThreads)
{
	const BVHNode* nd = (const BVHNode*)nodes;
	const TriangleVertices* tv = (const TriangleVertices*)verts;
	if (numThreads < 1) numThreads = 1;
	auto work = [&](uint32_t begin, uint32_t end) {
		for (uint32_t i = begin; i < end; i++) {
			const float* r = rays + 8 * size_t(i);
			Ray ray(sfz::vec3(r[0], r[1], r[2]), sfz::vec3(r[4], r[5], r[6]));
			RayCastResult res = castRay(nd, tv, ray, r[3], r[7]);
			inLight[i] = res.triangleIndex == ~0u ? 1 : 0;
		}
	};
	std::vector<std::thread> threads;
	uint32_t chunk = (n + numThreads - 1) / numThreads;
	for (int t = 0; t < numThreads; t++) {
		uint32_t b = t * chunk, e = b + chunk < n ? b + chunk : n;
		if (b >= e) break;
		threads.emplace_back(work, b, e);
	}
	for (auto& th : threads) th.join();
}

// The reference triangle test on one triangle (TriangleVertices layout).
int ref_intersect_tri(const float* tri, const float* origin, const float* dir, float* tuv)
{
	TriangleVertices tv;
	std::memcpy(&tv, tri, sizeof(tv));
	TriangleHit h = intersects(tv, sfz::vec3(origin[0], origin[1], origin[2]),
	                           sfz::vec3(dir[0], dir[1], dir[2]));
	if (h.hit) { tuv[0] = h.t; tuv[1] = h.u; tuv[2] = h.v; }
	return h.hit ? 1 : 0;
}

// generateCameraDef: out = origin.xyz, dir.xyz, dX.xyz, dY.xyz (12 floats).
void ref_camera_def(const float* pos, const float* dir, const float* up, float vfovRad,
                    float resX, float resY, float* out)
{
	CameraDef c = generateCameraDef(sfz::vec3(pos[0], pos[1], pos[2]), sfz::vec3(dir[0], dir[1], dir[2]),
	                                sfz::vec3(up[0], up[1], up[2]), vfovRad, sfz::vec2(resX, resY));
	float tmp[12] = {c.origin.x, c.origin.y, c.origin.z, c.dir.x, c.dir.y, c.dir.z,
	                 c.dX.x, c.dX.y, c.dX.z, c.dY.x, c.dY.y, c.dY.z};
	std::memcpy(out, tmp, sizeof(tmp));
}

} // extern "C"
