// Scene upload: validates the reference-layout arrays on the host, re-lays them out into the
// traversal layout (device/common.cuh) and uploads them in one allocation. Replaces setStaticScene
// (cuda_ray_tracer/CudaTracerRenderer.cpp:251-315), which uploaded the arrays unchanged into linear
// texture objects.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../host/wide8.hpp"
#include "runtime.cuh"

namespace phe_gb300 {

static std::mutex g_devMutex;
static DeviceInfo g_devices[64];
static std::atomic<uint32_t> g_counterNext{0};

phe_status device_info(DeviceInfo** out)
{
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return fail(PHE_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
	if (dev < 0 || dev >= 64) return fail(PHE_ERR_NO_DEVICE, "device ordinal %d out of range", dev);
	std::lock_guard<std::mutex> lock(g_devMutex);
	DeviceInfo& d = g_devices[dev];
	if (d.device < 0) {
		cudaDeviceProp prop;
		PHE_CUDA_TRY(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
		uint32_t* pool = nullptr;
		PHE_CUDA_TRY(cudaMalloc(&pool, sizeof(uint32_t) * kCounterPool), "cudaMalloc(counter pool)");
		PHE_CUDA_TRY(cudaMemset(pool, 0, sizeof(uint32_t) * kCounterPool), "cudaMemset(counter pool)");
		if (phe_status up = finish_uploads("clear counter pool")) return up;
		d.numSMs = prop.multiProcessorCount;
		d.maxThreadsPerSM = prop.maxThreadsPerMultiProcessor;
		d.counterPool = pool;
		d.device = dev;
	}
	*out = &d;
	return PHE_OK;
}

phe_status acquire_counter(cudaStream_t stream, uint32_t** counter)
{
	DeviceInfo* d = nullptr;
	phe_status s = device_info(&d);
	if (s) return s;
	uint32_t slot = g_counterNext.fetch_add(1) % kCounterPool;
	uint32_t* c = d->counterPool + slot;
	PHE_CUDA_TRY(cudaMemsetAsync(c, 0, sizeof(uint32_t), stream), "cudaMemsetAsync(counter)");
	*counter = c;
	return PHE_OK;
}

} // namespace phe_gb300

using namespace phe_gb300;

static_assert(sizeof(phe_bvh_node) == 64, "BVHNode is 64 bytes");
static_assert(sizeof(phe_triangle_vertices) == 48, "TriangleVertices is 48 bytes");
static_assert(sizeof(phe_triangle_data) == 64, "TriangleData is 64 bytes");
static_assert(sizeof(phe_ray_in) == 32, "RayIn is 32 bytes");
static_assert(sizeof(phe_ray_hit) == 16, "RayHit is 16 bytes");

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

namespace {

struct ChildRef {
	float box[6];   // lo.xyz, hi.xyz
	int32_t ref;    // binary inner node index (>= 0) or ~firstSlot (< 0)
};

ChildRef binary_child(const std::vector<float4>& dn, uint32_t node, int c)
{
	const float* f = reinterpret_cast<const float*>(&dn[(size_t)node * 4]);
	const int32_t* iv = reinterpret_cast<const int32_t*>(&dn[(size_t)node * 4 + 3]);
	ChildRef r;
	for (int k = 0; k < 6; k++) r.box[k] = f[6 * c + k];
	r.ref = iv[c];
	return r;
}

// True when `inner` is a non-inverted box (lo <= hi on every axis) inside `outer`. Then, for a ray
// with finite 1/dir, the rounded slab test gives inner an entry distance >= outer's and an exit
// distance <= outer's on every axis ((b - o) rounds monotonically in b, and the sign of 1/dir picks
// the same plane for both boxes), so inner passes the visit rule only if outer passes it too. An
// inverted box (lo > hi) is tested by the reference's min/max slab code as the swapped interval,
// which need not lie inside outer.
bool contains(const float* outer, const float* inner)
{
	return inner[0] >= outer[0] && inner[1] >= outer[1] && inner[2] >= outer[2] && inner[3] <= outer[3] &&
	       inner[4] <= outer[4] && inner[5] <= outer[5] && inner[0] <= inner[3] && inner[1] <= inner[4] &&
	       inner[2] <= inner[5];
}

// Collapses the binary tree (traversal layout `dn`) into 4-wide nodes: a binary node's inner children
// are replaced by their own two children. Returns false (and builds nothing) when some grandchild box
// is not inside its parent box, where skipping the parent test could change the traversal.
bool collapse4(const std::vector<float4>& dn, std::vector<float4>& out, uint32_t& depth4)
{
	out.clear();
	depth4 = 0;
	struct Item { uint32_t binary, index4, depth; };
	std::vector<Item> work;
	out.resize(8);
	work.push_back({0, 0, 1});
	while (!work.empty()) {
		Item it = work.back();
		work.pop_back();
		depth4 = std::max(depth4, it.depth);
		ChildRef kids[4];
		int n = 0;
		for (int c = 0; c < 2; c++) {
			ChildRef ch = binary_child(dn, it.binary, c);
			if (ch.ref >= 0) {
				for (int g = 0; g < 2; g++) {
					ChildRef gc = binary_child(dn, (uint32_t)ch.ref, g);
					if (!contains(ch.box, gc.box)) return false;
					kids[n++] = gc;
				}
			} else {
				kids[n++] = ch;
			}
		}
		float lanes[6][4];
		int32_t refs[4];
		for (int k = 0; k < 4; k++) {
			if (k < n) {
				for (int j = 0; j < 6; j++) lanes[j][k] = kids[k].box[j];
				if (kids[k].ref >= 0) {
					uint32_t child4 = (uint32_t)(out.size() / 8);
					out.resize(out.size() + 8);
					work.push_back({(uint32_t)kids[k].ref, child4, it.depth + 1});
					refs[k] = (int32_t)child4;
				} else {
					refs[k] = kids[k].ref;
				}
			} else {
				for (int j = 0; j < 6; j++) lanes[j][k] = 0.0f;
				refs[k] = kEmptyChild;
			}
		}
		float4* q = &out[(size_t)it.index4 * 8];
		for (int j = 0; j < 6; j++) q[j] = make_float4(lanes[j][0], lanes[j][1], lanes[j][2], lanes[j][3]);
		int4 rv = make_int4(refs[0], refs[1], refs[2], refs[3]);
		std::memcpy(&q[6], &rv, sizeof(rv));
		q[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	}
	return true;
}

// Materials and textures (setMaterialsAndTextures, CudaTracerRenderer.cpp:192-239).
phe_status check_materials(const phe_material* mats, uint32_t numMats, const phe_texture* tex, uint32_t numTex)
{
	for (uint32_t t = 0; t < numTex; t++) {
		const phe_texture& x = tex[t];
		if (!x.data) return fail(PHE_ERR_INVALID_ARGUMENT, "texture %u: null data", t);
		if (x.width < 1 || x.height < 1 || x.width > 65536 || x.height > 65536)
			return fail(PHE_ERR_INVALID_ARGUMENT, "texture %u: size %dx%d outside 1..65536", t, x.width, x.height);
		if (x.bytesPerPixel != 1 && x.bytesPerPixel != 2 && x.bytesPerPixel != 4)
			return fail(PHE_ERR_INVALID_ARGUMENT, "texture %u: %u bytes per pixel (1, 2 or 4)", t, x.bytesPerPixel);
		if ((uint64_t)x.pitch < (uint64_t)x.width * x.bytesPerPixel)
			return fail(PHE_ERR_INVALID_ARGUMENT, "texture %u: pitch %u < width x bytes per pixel", t, x.pitch);
	}
	for (uint32_t m = 0; m < numMats; m++)
		for (int k = 0; k < 3; k++) {
			int32_t ti = mats[m].texIndex[k];
			if (ti < -1 || ti >= (int32_t)numTex)
				return fail(PHE_ERR_INVALID_SCENE, "material %u: texture index %d with %u textures", m, ti, numTex);
			if (k == 0 && ti >= 0 && tex[ti].bytesPerPixel != 4)
				return fail(PHE_ERR_INVALID_SCENE, "material %u: albedo texture %d needs 4 bytes per pixel", m, ti);
		}
	return PHE_OK;
}

// One allocation: materials | texture table | sRGB table | texels (each texture 16-byte aligned, rows
// packed). Replaces the scene's previous one once the device is idle.
phe_status upload_shading(phe_scene* sc, const phe_material* mats, uint32_t numMats, const phe_texture* tex,
                          uint32_t numTex)
{
	const size_t matBytes = align256((size_t)numMats * sizeof(phe_material));
	const size_t tableBytes = align256((size_t)numTex * sizeof(DeviceTexture));
	const size_t srgbBytes = align256(256 * sizeof(float));
	std::vector<DeviceTexture> table(numTex);
	uint64_t texelBytes = 0;
	for (uint32_t t = 0; t < numTex; t++) {
		DeviceTexture& d = table[t];
		d.width = tex[t].width;
		d.height = tex[t].height;
		d.bytesPerPixel = tex[t].bytesPerPixel;
		d.rowBytes = (uint32_t)tex[t].width * tex[t].bytesPerPixel;
		d.offset = texelBytes;
		texelBytes += ((uint64_t)d.rowBytes * (uint64_t)d.height + 15u) & ~uint64_t(15);
	}
	const size_t total = matBytes + tableBytes + srgbBytes + (size_t)texelBytes;
	std::vector<uint8_t> host;
	try {
		host.assign(total, 0);
	} catch (const std::bad_alloc&) {
		return fail(PHE_ERR_OUT_OF_MEMORY, "materials and textures: host staging allocation failed");
	}
	if (numMats) std::memcpy(host.data(), mats, (size_t)numMats * sizeof(phe_material));
	if (numTex) std::memcpy(host.data() + matBytes, table.data(), (size_t)numTex * sizeof(DeviceTexture));
	float* srgb = reinterpret_cast<float*>(host.data() + matBytes + tableBytes);
	for (int b = 0; b < 256; b++) srgb[b] = (float)std::pow((double)((float)b / 255.0f), (double)2.2f);
	uint8_t* texels = host.data() + matBytes + tableBytes + srgbBytes;
	for (uint32_t t = 0; t < numTex; t++)
		for (int32_t y = 0; y < tex[t].height; y++)
			std::memcpy(texels + table[t].offset + (uint64_t)y * table[t].rowBytes,
			            tex[t].data + (uint64_t)y * tex[t].pitch, table[t].rowBytes);
	char* base = nullptr;
	PHE_CUDA_TRY(cudaMalloc(&base, total), "cudaMalloc(materials and textures)");
	cudaError_t e = cudaMemcpy(base, host.data(), total, cudaMemcpyHostToDevice);
	phe_status up = e != cudaSuccess ? cuda_fail(e, "upload materials and textures")
	                                 : finish_uploads("upload materials and textures");
	if (up) {
		cudaFree(base);
		return up;
	}
	if (sc->shading) {
		// Frames or casts queued on any stream may still read the old arrays.
		cudaDeviceSynchronize();
		cudaFree(sc->shading);
	}
	sc->shading = base;
	sc->shadingBytes = total;
	sc->dev.materials = numMats ? reinterpret_cast<const phe_material*>(base) : nullptr;
	sc->dev.numMaterials = numMats;
	sc->dev.textures = numTex ? reinterpret_cast<const DeviceTexture*>(base + matBytes) : nullptr;
	sc->dev.srgb = reinterpret_cast<const float*>(base + matBytes + tableBytes);
	sc->dev.texels = reinterpret_cast<const uint8_t*>(base + matBytes + tableBytes + srgbBytes);
	sc->dev.numTextures = numTex;
	sc->generation++;
	return PHE_OK;
}

} // namespace

extern "C" phe_status phe_scene_create(const phe_bvh_node* nodes, uint32_t numNodes, const phe_triangle_vertices* verts,
                                       const phe_triangle_data* datas, uint32_t numSlots, const phe_material* materials,
                                       uint32_t numMaterials, int where, phe_scene** out)
{
	if (!out) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_create: out is null");
	NvtxRange range("phe_scene_create");
	*out = nullptr;
	if (!nodes || !verts || numNodes == 0 || numSlots == 0)
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_create: empty scene");
	if (where != PHE_PTR_HOST && where != PHE_PTR_DEVICE)
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_create: where must be PHE_PTR_HOST or PHE_PTR_DEVICE");
	if (numNodes >= (uint32_t)kSentinel || numSlots >= 0x7FFFFFFFu)
		return fail(PHE_ERR_TOO_LARGE, "phe_scene_create: more than 2^31-2 nodes or slots");
	DeviceInfo* dinfo = nullptr;
	phe_status s = device_info(&dinfo);
	if (s) return s;

	// Host copies of the reference arrays (device input is read back once).
	std::vector<phe_bvh_node> hn;
	std::vector<phe_triangle_vertices> hv;
	std::vector<phe_triangle_data> hd;
	std::vector<phe_material> hm;
	try {
		hn.resize(numNodes);
		hv.resize(numSlots);
		if (datas) hd.resize(numSlots);
		if (materials && numMaterials) hm.resize(numMaterials);
	} catch (const std::bad_alloc&) {
		return fail(PHE_ERR_OUT_OF_MEMORY, "phe_scene_create: host staging allocation failed");
	}
	cudaMemcpyKind kind = where == PHE_PTR_HOST ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost;
	PHE_CUDA_TRY(cudaMemcpy(hn.data(), nodes, sizeof(phe_bvh_node) * (size_t)numNodes, kind), "copy nodes");
	PHE_CUDA_TRY(cudaMemcpy(hv.data(), verts, sizeof(phe_triangle_vertices) * (size_t)numSlots, kind), "copy verts");
	if (datas) PHE_CUDA_TRY(cudaMemcpy(hd.data(), datas, sizeof(phe_triangle_data) * (size_t)numSlots, kind), "copy datas");
	if (!hm.empty()) PHE_CUDA_TRY(cudaMemcpy(hm.data(), materials, sizeof(phe_material) * (size_t)numMaterials, kind), "copy materials");

	uint32_t maxDepth = 0;
	s = phe_bvh_validate(hn.data(), numNodes, numSlots, &maxDepth);
	if (s) return s;
	int64_t maxMaterialIndex = -1;
	for (const phe_triangle_data& d : hd) maxMaterialIndex = std::max<int64_t>(maxMaterialIndex, d.materialIndex);
	if (!hm.empty() && maxMaterialIndex >= (int64_t)numMaterials)
		return fail(PHE_ERR_INVALID_SCENE, "materialIndex %lld >= %u materials", (long long)maxMaterialIndex,
		            numMaterials);
	if ((s = check_materials(hm.data(), (uint32_t)hm.size(), nullptr, 0))) return s;

	// Traversal layout: child indices normalised (leaf = ~first), leaf end markers rewritten from
	// the counts so that leaf loops always stop inside the slot array, triangles as (p0, e1, e2).
	std::vector<float4> dn((size_t)numNodes * 4);
	std::vector<float4> dt((size_t)numSlots * 3);
	std::vector<uint8_t> used(numSlots, 0);
	for (uint32_t i = 0; i < numNodes; i++) {
		const phe_bvh_node& n = hn[i];
		float4* o = &dn[(size_t)i * 4];
		o[0] = make_float4(n.fData[0], n.fData[1], n.fData[2], n.fData[3]);
		o[1] = make_float4(n.fData[4], n.fData[5], n.fData[6], n.fData[7]);
		o[2] = make_float4(n.fData[8], n.fData[9], n.fData[10], n.fData[11]);
		int32_t idx[2], cnt[2];
		for (int c = 0; c < 2; c++) {
			int32_t raw = n.iData[c];
			cnt[c] = n.iData[2 + c];
			if (cnt[c] > 0) {
				int32_t first = raw < 0 ? ~raw : raw;
				idx[c] = ~first;
			} else {
				idx[c] = raw;
				cnt[c] = 0;
			}
		}
		int4 iv = make_int4(idx[0], idx[1], cnt[0], cnt[1]);
		std::memcpy(&o[3], &iv, sizeof(iv));
	}
	for (uint32_t i = 0; i < numSlots; i++) {
		const phe_triangle_vertices& t = hv[i];
		float e1x = t.v1[0] - t.v0[0], e1y = t.v1[1] - t.v0[1], e1z = t.v1[2] - t.v0[2];
		float e2x = t.v2[0] - t.v0[0], e2y = t.v2[1] - t.v0[1], e2z = t.v2[2] - t.v0[2];
		dt[(size_t)i * 3 + 0] = make_float4(t.v0[0], t.v0[1], t.v0[2], 0.0f);
		dt[(size_t)i * 3 + 1] = make_float4(e1x, e1y, e1z, 0.0f);
		dt[(size_t)i * 3 + 2] = make_float4(e2x, e2y, e2z, 0.0f);
	}
	// End markers from the leaf ranges of the reachable tree (phe_bvh_validate checked the ranges).
	{
		std::vector<uint32_t> stack{0};
		while (!stack.empty()) {
			uint32_t ni = stack.back();
			stack.pop_back();
			const int32_t* iv = reinterpret_cast<const int32_t*>(&dn[(size_t)ni * 4 + 3]);
			for (int c = 0; c < 2; c++) {
				if (iv[2 + c] > 0) {
					uint32_t first = (uint32_t)~iv[c];
					uint32_t last = first + (uint32_t)iv[2 + c] - 1;
					for (uint32_t k = first; k <= last; k++) {
						if (used[k])
							return fail(PHE_ERR_INVALID_SCENE, "slot %u belongs to two leaves", k);
						used[k] = 1;
					}
					dt[(size_t)last * 3].w = -1.0f;
				} else {
					stack.push_back((uint32_t)iv[c]);
				}
			}
		}
	}

	std::vector<float4> dn4;
	uint32_t depth4 = 0;
	bool wide = collapse4(dn, dn4, depth4);
	if (!wide) dn4.clear();
	Wide8Tree w8;
	std::string why8;
	if (!build_wide8(hn.data(), numNodes, w8, why8)) {
		w8.nodes.clear();
		w8.leaves.clear();
	}

	size_t nodeBytes = align256(dn.size() * sizeof(float4));
	size_t node4Bytes = align256(dn4.size() * sizeof(float4));
	size_t node8Bytes = align256(w8.nodes.size() * sizeof(uint32_t));
	size_t leaf8Bytes = align256(w8.leaves.size() * sizeof(uint32_t));
	size_t triBytes = align256(dt.size() * sizeof(float4));
	size_t dataBytes = align256(hd.size() * sizeof(phe_triangle_data));
	size_t statusBytes = 256;
	size_t total = nodeBytes + node4Bytes + node8Bytes + leaf8Bytes + triBytes + dataBytes + statusBytes;
	char* base = nullptr;
	cudaError_t e = cudaMalloc(&base, total);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(scene)");
	auto cleanup = [&](phe_status st) { cudaFree(base); return st; };
	char* p = base;
	float4* dNodes = (float4*)p; p += nodeBytes;
	float4* dNodes4 = dn4.empty() ? nullptr : (float4*)p; p += node4Bytes;
	uint4* dNodes8 = w8.nodes.empty() ? nullptr : (uint4*)p; p += node8Bytes;
	float4* dLeaves8 = w8.leaves.empty() ? nullptr : (float4*)p; p += leaf8Bytes;
	float4* dTris = (float4*)p; p += triBytes;
	phe_triangle_data* dDatas = hd.empty() ? nullptr : (phe_triangle_data*)p; p += dataBytes;
	uint32_t* dStatus = (uint32_t*)p;
	if ((e = cudaMemcpy(dNodes, dn.data(), dn.size() * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess)
		return cleanup(cuda_fail(e, "upload nodes"));
	if (dNodes4 && (e = cudaMemcpy(dNodes4, dn4.data(), dn4.size() * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess)
		return cleanup(cuda_fail(e, "upload 4-wide nodes"));
	if (dNodes8 && (e = cudaMemcpy(dNodes8, w8.nodes.data(), w8.nodes.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
		return cleanup(cuda_fail(e, "upload 8-wide nodes"));
	if (dLeaves8 && (e = cudaMemcpy(dLeaves8, w8.leaves.data(), w8.leaves.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
		return cleanup(cuda_fail(e, "upload 8-wide leaf records"));
	if ((e = cudaMemcpy(dTris, dt.data(), dt.size() * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess)
		return cleanup(cuda_fail(e, "upload triangles"));
	if (dDatas && (e = cudaMemcpy(dDatas, hd.data(), hd.size() * sizeof(phe_triangle_data), cudaMemcpyHostToDevice)) != cudaSuccess)
		return cleanup(cuda_fail(e, "upload triangle data"));
	if ((e = cudaMemset(dStatus, 0, statusBytes)) != cudaSuccess) return cleanup(cuda_fail(e, "clear status"));
	if (phe_status up = finish_uploads("upload scene")) return cleanup(up);

	phe_scene* sc = new phe_scene();
	sc->dev.nodes = dNodes;
	sc->dev.tris = dTris;
	sc->dev.datas = dDatas;
	sc->dev.materials = nullptr;
	sc->dev.numNodes = numNodes;
	sc->dev.numSlots = numSlots;
	sc->dev.numMaterials = 0;
	sc->maxDepth = maxDepth;
	sc->dev.textures = nullptr;
	sc->dev.texels = nullptr;
	sc->dev.srgb = nullptr;
	sc->dev.numTextures = 0;
	sc->maxMaterialIndex = maxMaterialIndex;
	sc->dev.nodes4 = nullptr;   // binary layout unless phe_scene_set_layout selects a wide one
	sc->dev.nodes8 = nullptr;
	sc->dev.leaves8 = nullptr;
	sc->nodes4 = dNodes4;
	sc->nodes8 = dNodes8;
	sc->leaves8 = dLeaves8;
	sc->numNodes8 = (uint32_t)(w8.nodes.size() / kWide8NodeWords);
	sc->numLeaves8 = (uint32_t)(w8.leaves.size() / kWide8LeafWords);
	sc->maxDepth8 = w8.depth;
	sc->dev.numNodes8 = sc->numNodes8;
	sc->dev.numLeaves8 = sc->numLeaves8;
	sc->dev.numNodes4 = (uint32_t)(dn4.size() / 8);
	sc->maxDepth4 = depth4;
	sc->allocation = base;
	sc->bytes = total;
	sc->status = dStatus;
	sc->dev.status = dStatus;
	sc->device = dinfo->device;
	if (!hm.empty() && (s = upload_shading(sc, hm.data(), (uint32_t)hm.size(), nullptr, 0))) {
		phe_scene_destroy(sc);
		return s;
	}
	*out = sc;
	return PHE_OK;
}

extern "C" phe_status phe_scene_set_materials_and_textures(phe_scene* scene, const phe_material* materials,
                                                           uint32_t numMaterials, const phe_texture* textures,
                                                           uint32_t numTextures)
{
	if (!scene) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_set_materials_and_textures: null scene");
	if ((!materials && numMaterials) || (!textures && numTextures))
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_set_materials_and_textures: null array");
	if (scene->maxMaterialIndex >= (int64_t)numMaterials)
		return fail(PHE_ERR_INVALID_SCENE, "materialIndex %lld >= %u materials", (long long)scene->maxMaterialIndex,
		            numMaterials);
	phe_status s = check_materials(materials, numMaterials, textures, numTextures);
	if (s) return s;
	return upload_shading(scene, materials, numMaterials, textures, numTextures);
}

extern "C" phe_status phe_scene_destroy(phe_scene* scene)
{
	if (!scene) return PHE_OK;
	// Work on any stream may still read the scene: a renderer's own streams with two frames in flight
	// are not ordered after the caller's.
	cudaDeviceSynchronize();
	if (scene->shading) cudaFree(scene->shading);
	cudaError_t e = cudaFree(scene->allocation);
	delete scene;
	if (e != cudaSuccess) return cuda_fail(e, "cudaFree(scene)");
	return PHE_OK;
}

extern "C" phe_status phe_scene_device_bytes(const phe_scene* scene, uint64_t* bytes)
{
	if (!scene || !bytes) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_device_bytes: null argument");
	*bytes = scene->bytes + scene->shadingBytes;
	return PHE_OK;
}

extern "C" phe_status phe_scene_status(const phe_scene* scene, uint32_t* bits)
{
	if (!scene || !bits) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_status: null argument");
	PHE_CUDA_TRY(cudaMemcpy(bits, scene->status, sizeof(uint32_t), cudaMemcpyDeviceToHost), "read scene status");
	return PHE_OK;
}

extern "C" phe_status phe_scene_set_layout(phe_scene* scene, int layout)
{
	if (!scene) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_set_layout: null scene");
	const float4* n4 = nullptr;
	const uint4* n8 = nullptr;
	const float4* l8 = nullptr;
	if (layout == PHE_LAYOUT_WIDE4) {
		if (!scene->nodes4)
			return fail(PHE_ERR_INVALID_SCENE, "phe_scene_set_layout: this tree has child boxes outside their parent box");
		n4 = scene->nodes4;
	} else if (layout == PHE_LAYOUT_WIDE8) {
		if (!scene->nodes8)
			return fail(PHE_ERR_INVALID_SCENE, "phe_scene_set_layout: this tree allows no 8-wide layout (a child box "
			                                   "outside its parent box, inverted or not finite)");
		n8 = scene->nodes8;
		l8 = scene->leaves8;
	} else if (layout != PHE_LAYOUT_BINARY) {
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_set_layout: unknown layout %d", layout);
	}
	if (scene->dev.nodes4 != n4 || scene->dev.nodes8 != n8) scene->generation++;
	scene->dev.nodes4 = n4;
	scene->dev.nodes8 = n8;
	scene->dev.leaves8 = l8;
	return PHE_OK;
}

extern "C" phe_status phe_scene_get_layout(const phe_scene* scene, int* layout, int* wideAvailable)
{
	if (!scene) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_scene_get_layout: null scene");
	if (layout)
		*layout = scene->dev.nodes8 ? PHE_LAYOUT_WIDE8 : scene->dev.nodes4 ? PHE_LAYOUT_WIDE4 : PHE_LAYOUT_BINARY;
	if (wideAvailable) *wideAvailable = (scene->nodes4 ? 1 : 0) | (scene->nodes8 ? 2 : 0);
	return PHE_OK;
}
