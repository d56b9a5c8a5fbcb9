// Host-side tools around the reference BVH layout: validation before upload, the raw BVH cache
// file format, camera definition and the TAA jitter table.

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.hpp"

using namespace phe_gb300;

// Maximum leaf depth the device traversal's stack supports. The reference SBVH builder never
// exceeds 64 (SplitBVHBuilder.h:38, MaxDepth).
static const uint32_t kMaxTraversalDepth = 64;

extern "C" phe_status phe_bvh_validate(const phe_bvh_node* nodes, uint32_t numNodes, uint32_t numSlots,
                                       uint32_t* maxDepthOut)
{
	if (!nodes || numNodes == 0) return fail(PHE_ERR_INVALID_SCENE, "phe_bvh_validate: no nodes");
	if (numSlots == 0) return fail(PHE_ERR_INVALID_SCENE, "phe_bvh_validate: no triangles");
	std::vector<uint8_t> seen(numNodes, 0);
	struct Item { uint32_t node, depth; };
	std::vector<Item> stack;
	stack.push_back({0, 0});
	seen[0] = 1;
	uint32_t maxDepth = 0;
	while (!stack.empty()) {
		Item it = stack.back();
		stack.pop_back();
		const phe_bvh_node& n = nodes[it.node];
		for (int c = 0; c < 2; c++) {
			int32_t raw = n.iData[c];
			int32_t count = n.iData[2 + c];
			uint32_t depth = it.depth + 1;
			if (count < 0) return fail(PHE_ERR_INVALID_SCENE, "node %u child %d: negative triangle count", it.node, c);
			for (int k = 0; k < 6; k++)
				if (std::isnan(n.fData[6 * c + k]))
					return fail(PHE_ERR_INVALID_SCENE, "node %u child %d: NaN in bounds", it.node, c);
			if (count > 0) {
				uint32_t first = (uint32_t)(raw < 0 ? ~raw : raw);
				if ((uint64_t)first + (uint64_t)count > numSlots)
					return fail(PHE_ERR_INVALID_SCENE, "node %u child %d: leaf [%u, +%d) beyond %u slots", it.node, c,
					            first, count, numSlots);
				if (depth > maxDepth) maxDepth = depth;
			} else {
				if (raw < 0 || (uint32_t)raw >= numNodes)
					return fail(PHE_ERR_INVALID_SCENE, "node %u child %d: inner index %d out of range", it.node, c, raw);
				if (seen[(uint32_t)raw])
					return fail(PHE_ERR_INVALID_SCENE, "node %d reached twice (not a tree)", raw);
				if (depth >= kMaxTraversalDepth)
					return fail(PHE_ERR_INVALID_SCENE, "inner node %d at depth %u: deeper than %u", raw, depth,
					            kMaxTraversalDepth);
				seen[(uint32_t)raw] = 1;
				stack.push_back({(uint32_t)raw, depth});
			}
		}
	}
	if (maxDepthOut) *maxDepthOut = maxDepth;
	return PHE_OK;
}

// ------------------------------------------------------------------------------------------------
// BVH cache (testbed_application/Main.cpp:105-154): three raw dumps, no header, so that caches move
// between the reference and this library unchanged. Beside them this library writes
// <base>_header.bin: magic, version, record sizes, counts and a 64-bit checksum of each dump. A
// cache read verifies it when present (a reference-written cache has none and is read as is).

static std::string cachePath(const char* base, const char* suffix) { return std::string(base) + suffix; }

static phe_status writeFile(const std::string& path, const void* data, size_t bytes)
{
	FILE* f = std::fopen(path.c_str(), "wb");
	if (!f) return fail(PHE_ERR_INVALID_ARGUMENT, "cannot open %s for writing", path.c_str());
	size_t w = bytes ? std::fwrite(data, 1, bytes, f) : 0;
	int rc = std::fclose(f);
	if (w != bytes || rc != 0) return fail(PHE_ERR_INVALID_ARGUMENT, "short write to %s", path.c_str());
	return PHE_OK;
}

static phe_status fileSize(const std::string& path, uint64_t* size)
{
	FILE* f = std::fopen(path.c_str(), "rb");
	if (!f) return fail(PHE_ERR_NOT_FOUND, "cannot open %s", path.c_str());
	std::fseek(f, 0, SEEK_END);
	long s = std::ftell(f);
	std::fclose(f);
	if (s < 0) return fail(PHE_ERR_INVALID_ARGUMENT, "cannot size %s", path.c_str());
	*size = (uint64_t)s;
	return PHE_OK;
}

static phe_status readFile(const std::string& path, void* data, size_t bytes)
{
	FILE* f = std::fopen(path.c_str(), "rb");
	if (!f) return fail(PHE_ERR_NOT_FOUND, "cannot open %s", path.c_str());
	size_t r = bytes ? std::fread(data, 1, bytes, f) : 0;
	std::fclose(f);
	if (r != bytes) return fail(PHE_ERR_INVALID_ARGUMENT, "short read from %s", path.c_str());
	return PHE_OK;
}

namespace {

struct CacheHeader {
	char magic[8];          // "PHEBVHC\0"
	uint32_t version;       // 1
	uint32_t nodeBytes, vertBytes, dataBytes;   // record sizes: 64, 48, 64
	uint32_t numNodes, numSlots;
	uint64_t sumNodes, sumVerts, sumDatas;      // checksum64 of each dump
};
static_assert(sizeof(CacheHeader) == 56, "cache header is 56 bytes");
constexpr char kCacheMagic[8] = {'P', 'H', 'E', 'B', 'V', 'H', 'C', 0};

// FNV-1a over little-endian 64-bit words (then the tail bytes), the word count mixed in at the end.
uint64_t checksum64(const void* data, size_t bytes)
{
	const uint64_t prime = 0x100000001b3ull;
	uint64_t h = 0xcbf29ce484222325ull;
	const unsigned char* p = static_cast<const unsigned char*>(data);
	size_t words = bytes / 8;
	for (size_t i = 0; i < words; i++) {
		uint64_t w = 0;
		for (int k = 7; k >= 0; k--) w = (w << 8) | p[8 * i + (size_t)k];
		h = (h ^ w) * prime;
	}
	for (size_t i = words * 8; i < bytes; i++) h = (h ^ p[i]) * prime;
	return (h ^ (uint64_t)bytes) * prime;
}

} // namespace

extern "C" phe_status phe_bvh_cache_write(const char* base, const phe_bvh_node* nodes, uint32_t numNodes,
                                          const phe_triangle_vertices* verts, const phe_triangle_data* datas,
                                          uint32_t numSlots)
{
	if (!base || !nodes || !verts || !datas) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_bvh_cache_write: null argument");
	phe_status s = writeFile(cachePath(base, "_nodes.bin"), nodes, sizeof(phe_bvh_node) * (size_t)numNodes);
	if (s) return s;
	s = writeFile(cachePath(base, "_verts.bin"), verts, sizeof(phe_triangle_vertices) * (size_t)numSlots);
	if (s) return s;
	s = writeFile(cachePath(base, "_datas.bin"), datas, sizeof(phe_triangle_data) * (size_t)numSlots);
	if (s) return s;
	CacheHeader h{};
	std::memcpy(h.magic, kCacheMagic, sizeof(h.magic));
	h.version = 1;
	h.nodeBytes = sizeof(phe_bvh_node);
	h.vertBytes = sizeof(phe_triangle_vertices);
	h.dataBytes = sizeof(phe_triangle_data);
	h.numNodes = numNodes;
	h.numSlots = numSlots;
	h.sumNodes = checksum64(nodes, sizeof(phe_bvh_node) * (size_t)numNodes);
	h.sumVerts = checksum64(verts, sizeof(phe_triangle_vertices) * (size_t)numSlots);
	h.sumDatas = checksum64(datas, sizeof(phe_triangle_data) * (size_t)numSlots);
	return writeFile(cachePath(base, "_header.bin"), &h, sizeof(h));
}

extern "C" phe_status phe_bvh_cache_sizes(const char* base, uint32_t* numNodes, uint32_t* numSlots)
{
	if (!base || !numNodes || !numSlots) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_bvh_cache_sizes: null argument");
	uint64_t ns = 0, vs = 0, ds = 0;
	phe_status s;
	if ((s = fileSize(cachePath(base, "_nodes.bin"), &ns))) return s;
	if ((s = fileSize(cachePath(base, "_verts.bin"), &vs))) return s;
	if ((s = fileSize(cachePath(base, "_datas.bin"), &ds))) return s;
	if (ns % sizeof(phe_bvh_node) || vs % sizeof(phe_triangle_vertices) || ds % sizeof(phe_triangle_data))
		return fail(PHE_ERR_INVALID_SCENE, "BVH cache %s: file size not a multiple of the record size", base);
	if (vs / sizeof(phe_triangle_vertices) != ds / sizeof(phe_triangle_data))
		return fail(PHE_ERR_INVALID_SCENE, "BVH cache %s: vertex and data counts differ", base);
	*numNodes = (uint32_t)(ns / sizeof(phe_bvh_node));
	*numSlots = (uint32_t)(vs / sizeof(phe_triangle_vertices));
	return PHE_OK;
}

extern "C" phe_status phe_bvh_cache_read(const char* base, phe_bvh_node* nodes, uint32_t numNodes,
                                         phe_triangle_vertices* verts, phe_triangle_data* datas, uint32_t numSlots)
{
	uint32_t nn = 0, nsl = 0;
	phe_status s = phe_bvh_cache_sizes(base, &nn, &nsl);
	if (s) return s;
	if (nn != numNodes || nsl != numSlots)
		return fail(PHE_ERR_INVALID_ARGUMENT, "BVH cache %s holds %u nodes / %u slots, caller expects %u / %u", base,
		            nn, nsl, numNodes, numSlots);
	if ((s = readFile(cachePath(base, "_nodes.bin"), nodes, sizeof(phe_bvh_node) * (size_t)nn))) return s;
	if ((s = readFile(cachePath(base, "_verts.bin"), verts, sizeof(phe_triangle_vertices) * (size_t)nsl))) return s;
	if ((s = readFile(cachePath(base, "_datas.bin"), datas, sizeof(phe_triangle_data) * (size_t)nsl))) return s;
	uint64_t hs = 0;
	if (fileSize(cachePath(base, "_header.bin"), &hs) != PHE_OK) {
		clear_error();
		return PHE_OK;   // no header: a cache written by the reference
	}
	CacheHeader h{};
	if (hs != sizeof(h) || (s = readFile(cachePath(base, "_header.bin"), &h, sizeof(h))))
		return fail(PHE_ERR_INVALID_SCENE, "BVH cache %s: unreadable header", base);
	if (std::memcmp(h.magic, kCacheMagic, sizeof(h.magic)) != 0 || h.version != 1 ||
	    h.nodeBytes != sizeof(phe_bvh_node) || h.vertBytes != sizeof(phe_triangle_vertices) ||
	    h.dataBytes != sizeof(phe_triangle_data))
		return fail(PHE_ERR_INVALID_SCENE, "BVH cache %s: unknown header format", base);
	if (h.numNodes != nn || h.numSlots != nsl)
		return fail(PHE_ERR_INVALID_SCENE, "BVH cache %s: header counts %u / %u, files hold %u / %u", base, h.numNodes,
		            h.numSlots, nn, nsl);
	if (h.sumNodes != checksum64(nodes, sizeof(phe_bvh_node) * (size_t)nn) ||
	    h.sumVerts != checksum64(verts, sizeof(phe_triangle_vertices) * (size_t)nsl) ||
	    h.sumDatas != checksum64(datas, sizeof(phe_triangle_data) * (size_t)nsl))
		return fail(PHE_ERR_INVALID_SCENE, "BVH cache %s: checksum mismatch (a file changed after it was written)", base);
	return PHE_OK;
}

// ------------------------------------------------------------------------------------------------

extern "C" void phe_generate_camera_def(const float pos[3], const float dir[3], const float up[3], float vertFovRad,
                                        float resX, float resY, phe_camera_def* out)
{
	// GenerateRays.cpp:12-35, in sfz operation order (normalize = v / sqrt(dot(v, v))).
	auto normalize = [](const float v[3], float o[3]) {
		float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
		o[0] = v[0] / l; o[1] = v[1] / l; o[2] = v[2] / l;
	};
	float d[3], u[3], r[3], c[3];
	normalize(dir, d);
	normalize(up, u);
	c[0] = d[1] * u[2] - d[2] * u[1];
	c[1] = d[2] * u[0] - d[0] * u[2];
	c[2] = d[0] * u[1] - d[1] * u[0];
	normalize(c, r);
	float aspect = resX / resY;
	float yMax = std::tan(vertFovRad * 0.5f);
	float xMax = aspect * yMax;
	for (int k = 0; k < 3; k++) {
		out->origin[k] = pos[k];
		out->dir[k] = d[k];
		out->dX[k] = r[k] * xMax;
		out->dY[k] = u[k] * yMax;
	}
}

extern "C" void phe_halton_jitter(uint32_t index, float out[2])
{
	// Halton(2,3) points 1..16 (GameScreen.cpp:21-39 lists them), minus half a pixel.
	uint32_t k = (index % 16u) + 1u;
	double f = 1.0, r = 0.0;
	for (uint32_t n = k; n; n /= 2u) { f /= 2.0; r += f * (double)(n % 2u); }
	double f3 = 1.0, r3 = 0.0;
	for (uint32_t n = k; n; n /= 3u) { f3 /= 3.0; r3 += f3 * (double)(n % 3u); }
	out[0] = (float)r - 0.5f;
	out[1] = (float)r3 - 0.5f;
}
