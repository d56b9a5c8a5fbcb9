// Spatial-split BVH builder emitting the reference's sanitized layout.
//
// Algorithm: "Spatial Splits in Bounding Volume Hierarchies" (M. Stich, H. Friedrich,
// A. Dietrich, HPG 2009): per node, the best of a leaf, an object split (SAH over sorted
// centroids; binned above kExactSweepMax references) and a spatial split (32 chopped bins per
// axis, tried only when the object split's children overlap by more than splitAlpha times the root
// area), with reference unsplitting at the chosen plane. Costs, thresholds and depth limits are the
// reference builder's defaults (sbvh-stuff/BVH.h:68-81, sbvh-stuff/Util.h:71-109,
// SplitBVHBuilder.h:38-44): node cost 1, triangle cost 1, leaf size 1.., max depth 64, no spatial
// splits at depth >= 48. Subtrees above kParallelMin references are built on their own threads;
// the output does not depend on the thread count.
//
// Output layout (what buildStaticFrom + sanitizeBVH produce, StaticBVHBuilder.cpp:19-78,213-260):
// node 0 is the root, nodes in pre-order with the left subtree first, leaf child indices are ~slot,
// slot vertices copy the input triangle with .w = 0 except -1 on each leaf's last slot.

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

#include "common.hpp"

namespace phe_gb300 {
namespace {

constexpr int kSpatialBins = 32;
constexpr int kObjectBins = 128;
constexpr size_t kExactSweepMax = 1024;
constexpr size_t kParallelMin = 16384;
// Nodes with at least kChunkedMin references bin and partition them in contiguous chunks of at
// least kChunkMin on threads from the free pool (the top levels of the tree, where too few subtrees
// exist to keep the threads busy). Binning merges boxes by min/max and counts by addition, and
// partitions concatenate the chunks in order, so the tree is the same for any thread count.
constexpr size_t kChunkedMin = 1u << 18;
constexpr size_t kChunkMin = 1u << 16;
constexpr int kMaxChunks = 64;

struct AABB {
	float lo[3] = {INFINITY, INFINITY, INFINITY};
	float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
	void grow(const float p[3])
	{
		for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
	}
	void grow(const AABB& b)
	{
		for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
	}
	void intersect(const AABB& b)
	{
		for (int k = 0; k < 3; k++) { lo[k] = std::max(lo[k], b.lo[k]); hi[k] = std::min(hi[k], b.hi[k]); }
	}
	bool valid() const { return lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2]; }
	float area() const
	{
		if (!valid()) return 0.0f;
		float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
		return 2.0f * (dx * dy + dy * dz + dz * dx);
	}
};

struct Ref {
	uint32_t tri;
	AABB box;
	float centroid2(int axis) const { return box.lo[axis] + box.hi[axis]; }
};

struct TNode {
	AABB box;
	std::unique_ptr<TNode> child[2];
	std::vector<uint32_t> tris; // leaf only
	bool leaf() const { return !child[0]; }
};

struct Builder {
	const float* verts; // 9 floats per triangle
	phe_sbvh_params params;
	float minOverlap = 0.0f;
	std::atomic<int> freeThreads{0};

	// Splits [0, n) into contiguous chunks, one per thread taken from the free pool plus the calling
	// thread, and runs fn(chunk, begin, end) on each. Returns the number of chunks (>= 1).
	static size_t maxChunks(size_t n) { return n >= kChunkedMin ? std::min<size_t>(kMaxChunks, n / kChunkMin) : 1; }

	template <class F>
	int chunked(size_t n, F&& fn)
	{
		int want = (int)maxChunks(n);
		int extra = 0;
		while (extra + 1 < want) {
			int f = freeThreads.load();
			if (f <= 0) break;
			if (freeThreads.compare_exchange_weak(f, f - 1)) extra++;
		}
		const int chunks = extra + 1;
		auto range = [&](int c, size_t& b, size_t& e) {
			b = n * (size_t)c / (size_t)chunks;
			e = n * (size_t)(c + 1) / (size_t)chunks;
		};
		std::vector<std::thread> pool;
		pool.reserve((size_t)extra);
		for (int c = 1; c < chunks; c++)
			pool.emplace_back([&, c]() {
				size_t b, e;
				range(c, b, e);
				fn(c, b, e);
			});
		size_t b0, e0;
		range(0, b0, e0);
		fn(0, b0, e0);
		for (std::thread& t : pool) t.join();
		freeThreads.fetch_add(extra);
		return chunks;
	}

	void clipTriangle(const Ref& ref, int dim, float pos, AABB& left, AABB& right) const
	{
		left = AABB();
		right = AABB();
		const float* t = verts + 9 * (size_t)ref.tri;
		for (int i = 0; i < 3; i++) {
			const float* a = t + 3 * i;
			const float* b = t + 3 * ((i + 1) % 3);
			float ap = a[dim], bp = b[dim];
			if (ap <= pos) left.grow(a);
			if (ap >= pos) right.grow(a);
			if ((ap < pos && bp > pos) || (ap > pos && bp < pos)) {
				float s = (pos - ap) / (bp - ap);
				s = std::min(1.0f, std::max(0.0f, s));
				float p[3];
				for (int k = 0; k < 3; k++) p[k] = a[k] + (b[k] - a[k]) * s;
				p[dim] = pos;
				left.grow(p);
				right.grow(p);
			}
		}
		left.hi[dim] = pos;
		right.lo[dim] = pos;
		left.intersect(ref.box);
		right.intersect(ref.box);
	}

	struct ObjectSplit {
		float sah = INFINITY;
		int axis = -1;
		bool binned = false;
		size_t numLeft = 0;     // exact sweep
		int binSplit = 0;       // binned
		float cmin = 0, cscale = 0;
		AABB lbox, rbox;
	};

	static bool lessOn(const Ref& a, const Ref& b, int axis)
	{
		float ca = a.centroid2(axis), cb = b.centroid2(axis);
		if (ca != cb) return ca < cb;
		return a.tri < b.tri;
	}

	ObjectSplit exactObjectSplit(std::vector<Ref>& refs, float nodeSAH) const
	{
		ObjectSplit best;
		size_t n = refs.size();
		std::vector<AABB> rightBoxes(n);
		for (int axis = 0; axis < 3; axis++) {
			std::sort(refs.begin(), refs.end(), [axis](const Ref& a, const Ref& b) { return lessOn(a, b, axis); });
			AABB rb;
			for (size_t i = n - 1; i > 0; i--) { rb.grow(refs[i].box); rightBoxes[i - 1] = rb; }
			AABB lb;
			for (size_t i = 1; i < n; i++) {
				lb.grow(refs[i - 1].box);
				float sah = nodeSAH + lb.area() * (float)i + rightBoxes[i - 1].area() * (float)(n - i);
				if (sah < best.sah) {
					best.sah = sah; best.axis = axis; best.numLeft = i; best.lbox = lb; best.rbox = rightBoxes[i - 1];
				}
			}
		}
		best.binned = false;
		return best;
	}

	ObjectSplit binnedObjectSplit(const std::vector<Ref>& refs, float nodeSAH)
	{
		ObjectSplit best;
		size_t n = refs.size();
		// Centroid ranges of the three axes, then the bins of the three axes, each in one chunked pass.
		struct Range { float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}; };
		std::vector<Range> ranges(maxChunks(n));
		int chunks = chunked(n, [&](int c, size_t b, size_t e) {
			Range& rg = ranges[(size_t)c];
			for (size_t i = b; i < e; i++)
				for (int a = 0; a < 3; a++) {
					float v = refs[i].centroid2(a);
					rg.lo[a] = std::min(rg.lo[a], v);
					rg.hi[a] = std::max(rg.hi[a], v);
				}
		});
		float cmins[3], scales[3];
		bool active[3];
		for (int a = 0; a < 3; a++) {
			float lo = INFINITY, hi = -INFINITY;
			for (int c = 0; c < chunks; c++) { lo = std::min(lo, ranges[(size_t)c].lo[a]); hi = std::max(hi, ranges[(size_t)c].hi[a]); }
			active[a] = hi > lo;
			cmins[a] = lo;
			scales[a] = active[a] ? (float)kObjectBins / (hi - lo) : 0.0f;
		}
		struct Bins { AABB box[3][kObjectBins]; size_t cnt[3][kObjectBins] = {}; };
		std::vector<Bins> partial(maxChunks(n));
		chunks = chunked(n, [&](int c, size_t b, size_t e) {
			Bins& pb = partial[(size_t)c];
			for (size_t i = b; i < e; i++)
				for (int a = 0; a < 3; a++) {
					if (!active[a]) continue;
					int k = std::min(kObjectBins - 1, (int)((refs[i].centroid2(a) - cmins[a]) * scales[a]));
					pb.box[a][k].grow(refs[i].box);
					pb.cnt[a][k]++;
				}
		});
		for (int axis = 0; axis < 3; axis++) {
			if (!active[axis]) continue;
			const float cmin = cmins[axis], scale = scales[axis];
			AABB bins[kObjectBins];
			size_t cnt[kObjectBins] = {};
			for (int c = 0; c < chunks; c++)
				for (int k = 0; k < kObjectBins; k++) {
					bins[k].grow(partial[(size_t)c].box[axis][k]);
					cnt[k] += partial[(size_t)c].cnt[axis][k];
				}
			AABB rboxes[kObjectBins];
			size_t rcnt[kObjectBins];
			AABB rb;
			size_t rc = 0;
			for (int b = kObjectBins - 1; b > 0; b--) { rb.grow(bins[b]); rc += cnt[b]; rboxes[b - 1] = rb; rcnt[b - 1] = rc; }
			AABB lb;
			size_t lc = 0;
			for (int b = 1; b < kObjectBins; b++) {
				lb.grow(bins[b - 1]);
				lc += cnt[b - 1];
				if (lc == 0 || rcnt[b - 1] == 0) continue;
				float sah = nodeSAH + lb.area() * (float)lc + rboxes[b - 1].area() * (float)rcnt[b - 1];
				if (sah < best.sah) {
					best.sah = sah; best.axis = axis; best.binSplit = b; best.cmin = cmin; best.cscale = scale;
					best.numLeft = lc; best.lbox = lb; best.rbox = rboxes[b - 1];
				}
			}
		}
		best.binned = true;
		(void)n;
		return best;
	}

	// Concatenates per-chunk vectors in chunk order.
	static void concat(std::vector<std::vector<Ref>>& parts, int chunks, std::vector<Ref>& out)
	{
		if (chunks == 1) {
			out.swap(parts[0]);
			return;
		}
		size_t total = 0;
		for (int c = 0; c < chunks; c++) total += parts[(size_t)c].size();
		out.clear();
		out.reserve(total);
		for (int c = 0; c < chunks; c++) out.insert(out.end(), parts[(size_t)c].begin(), parts[(size_t)c].end());
	}

	void performObjectSplit(std::vector<Ref>& refs, const ObjectSplit& s, std::vector<Ref>& left,
	                        std::vector<Ref>& right)
	{
		left.clear();
		right.clear();
		if (!s.binned) {
			int axis = s.axis;
			std::sort(refs.begin(), refs.end(), [axis](const Ref& a, const Ref& b) { return lessOn(a, b, axis); });
			left.assign(refs.begin(), refs.begin() + (ptrdiff_t)s.numLeft);
			right.assign(refs.begin() + (ptrdiff_t)s.numLeft, refs.end());
		} else {
			const size_t mc = maxChunks(refs.size());
			std::vector<std::vector<Ref>> lp(mc), rp(mc);
			int chunks = chunked(refs.size(), [&](int c, size_t b, size_t e) {
				for (size_t i = b; i < e; i++) {
					int k = std::min(kObjectBins - 1, (int)((refs[i].centroid2(s.axis) - s.cmin) * s.cscale));
					(k < s.binSplit ? lp : rp)[(size_t)c].push_back(refs[i]);
				}
			});
			concat(lp, chunks, left);
			concat(rp, chunks, right);
		}
	}

	struct SpatialSplit { float sah = INFINITY; int dim = -1; float pos = 0.0f; };

	SpatialSplit findSpatialSplit(const std::vector<Ref>& refs, const AABB& box, float nodeSAH)
	{
		SpatialSplit best;
		float origin[3], binSize[3], inv[3];
		for (int k = 0; k < 3; k++) {
			origin[k] = box.lo[k];
			binSize[k] = (box.hi[k] - box.lo[k]) * (1.0f / (float)kSpatialBins);
			inv[k] = 1.0f / binSize[k];
		}
		struct Bin { AABB box; uint32_t enter = 0, exit = 0; };
		for (int dim = 0; dim < 3; dim++) {
			if (!(binSize[dim] > 0.0f) || !std::isfinite(inv[dim])) continue;
			std::vector<std::array<Bin, kSpatialBins>> partial(maxChunks(refs.size()));
			int chunks = chunked(refs.size(), [&](int c, size_t b, size_t e) {
				Bin* pb = partial[(size_t)c].data();
				for (size_t j = b; j < e; j++) {
					const Ref& r = refs[j];
					int first = (int)((r.box.lo[dim] - origin[dim]) * inv[dim]);
					first = std::min(kSpatialBins - 1, std::max(0, first));
					int last = (int)((r.box.hi[dim] - origin[dim]) * inv[dim]);
					last = std::min(kSpatialBins - 1, std::max(first, last));
					Ref cur = r;
					for (int i = first; i < last; i++) {
						AABB l, rr;
						clipTriangle(cur, dim, origin[dim] + binSize[dim] * (float)(i + 1), l, rr);
						pb[i].box.grow(l);
						cur.box = rr;
					}
					pb[last].box.grow(cur.box);
					pb[first].enter++;
					pb[last].exit++;
				}
			});
			Bin bins[kSpatialBins];
			for (int c = 0; c < chunks; c++)
				for (int i = 0; i < kSpatialBins; i++) {
					bins[i].box.grow(partial[(size_t)c][(size_t)i].box);
					bins[i].enter += partial[(size_t)c][(size_t)i].enter;
					bins[i].exit += partial[(size_t)c][(size_t)i].exit;
				}
			AABB rboxes[kSpatialBins];
			AABB rb;
			for (int i = kSpatialBins - 1; i > 0; i--) { rb.grow(bins[i].box); rboxes[i - 1] = rb; }
			AABB lb;
			size_t ln = 0, rn = refs.size();
			for (int i = 1; i < kSpatialBins; i++) {
				lb.grow(bins[i - 1].box);
				ln += bins[i - 1].enter;
				rn -= bins[i - 1].exit;
				float sah = nodeSAH + lb.area() * (float)ln + rboxes[i - 1].area() * (float)rn;
				if (sah < best.sah) { best.sah = sah; best.dim = dim; best.pos = origin[dim] + binSize[dim] * (float)i; }
			}
		}
		return best;
	}

	void performSpatialSplit(const std::vector<Ref>& refs, const SpatialSplit& s, std::vector<Ref>& left,
	                         std::vector<Ref>& right, AABB& lbox, AABB& rbox)
	{
		lbox = AABB();
		rbox = AABB();
		// References entirely on one side keep their order; the straddling ones are decided after, in order.
		const size_t mc = maxChunks(refs.size());
		std::vector<std::vector<Ref>> lp(mc), rp(mc), sp(mc);
		std::vector<AABB> lb(mc), rb(mc);
		int chunks = chunked(refs.size(), [&](int c, size_t b, size_t e) {
			for (size_t i = b; i < e; i++) {
				const Ref& r = refs[i];
				if (r.box.hi[s.dim] <= s.pos) { lp[(size_t)c].push_back(r); lb[(size_t)c].grow(r.box); }
				else if (r.box.lo[s.dim] >= s.pos) { rp[(size_t)c].push_back(r); rb[(size_t)c].grow(r.box); }
				else sp[(size_t)c].push_back(r);
			}
		});
		concat(lp, chunks, left);
		concat(rp, chunks, right);
		std::vector<Ref> straddleRefs;
		concat(sp, chunks, straddleRefs);
		for (int c = 0; c < chunks; c++) { lbox.grow(lb[(size_t)c]); rbox.grow(rb[(size_t)c]); }
		std::vector<const Ref*> straddle;
		straddle.reserve(straddleRefs.size());
		for (const Ref& r : straddleRefs) straddle.push_back(&r);
		// Reference unsplitting: keep a straddling reference whole on one side when that is cheaper
		// than duplicating it.
		for (const Ref* rp : straddle) {
			const Ref& r = *rp;
			AABB lc, rc;
			clipTriangle(r, s.dim, s.pos, lc, rc);
			AABB lub = lbox; lub.grow(r.box);
			AABB rub = rbox; rub.grow(r.box);
			AABB ldb = lbox; ldb.grow(lc);
			AABB rdb = rbox; rdb.grow(rc);
			float nl = (float)left.size(), nr = (float)right.size();
			float unsplitLeft = lub.area() * (nl + 1.0f) + rbox.area() * nr;
			float unsplitRight = lbox.area() * nl + rub.area() * (nr + 1.0f);
			float duplicate = ldb.area() * (nl + 1.0f) + rdb.area() * (nr + 1.0f);
			float m = std::min(std::min(unsplitLeft, unsplitRight), duplicate);
			if (m == unsplitLeft) { left.push_back(r); lbox = lub; }
			else if (m == unsplitRight) { right.push_back(r); rbox = rub; }
			else {
				Ref a = r, b = r;
				a.box = lc; b.box = rc;
				left.push_back(a); lbox = ldb;
				right.push_back(b); rbox = rdb;
			}
		}
	}

	std::unique_ptr<TNode> makeLeaf(const std::vector<Ref>& refs, const AABB& box) const
	{
		auto node = std::make_unique<TNode>();
		node->box = box;
		node->tris.reserve(refs.size());
		for (const Ref& r : refs) node->tris.push_back(r.tri);
		return node;
	}

	std::unique_ptr<TNode> build(std::vector<Ref> refs, const AABB& box, int depth)
	{
		size_t n = refs.size();
		if (n <= 1 || depth >= params.maxDepth) return makeLeaf(refs, box);
		float area = box.area();
		float leafSAH = area * (float)n;
		float nodeSAH = area * 2.0f;
		ObjectSplit obj = n <= kExactSweepMax ? exactObjectSplit(refs, nodeSAH) : binnedObjectSplit(refs, nodeSAH);
		if (obj.axis < 0 && obj.binned) obj = exactObjectSplit(refs, nodeSAH);
		SpatialSplit spatial;
		if (depth < params.maxSpatialDepth && obj.axis >= 0) {
			AABB overlap = obj.lbox;
			overlap.intersect(obj.rbox);
			if (overlap.area() >= minOverlap) spatial = findSpatialSplit(refs, box, nodeSAH);
		}
		float minSAH = std::min(std::min(leafSAH, obj.sah), spatial.sah);
		if (minSAH == leafSAH || obj.axis < 0) return makeLeaf(refs, box);

		std::vector<Ref> left, right;
		AABB lbox, rbox;
		if (minSAH == spatial.sah && spatial.dim >= 0) performSpatialSplit(refs, spatial, left, right, lbox, rbox);
		if (left.empty() || right.empty()) {
			performObjectSplit(refs, obj, left, right);
			lbox = obj.lbox;
			rbox = obj.rbox;
			if (left.empty() || right.empty()) return makeLeaf(refs, box);
		}
		std::vector<Ref>().swap(refs);

		auto node = std::make_unique<TNode>();
		node->box = box;
		bool spawn = false;
		if (right.size() >= kParallelMin && left.size() >= kParallelMin) {
			int f = freeThreads.fetch_sub(1);
			if (f > 0) spawn = true;
			else freeThreads.fetch_add(1);
		}
		if (spawn) {
			std::unique_ptr<TNode> r;
			std::thread th([&]() { r = build(std::move(right), rbox, depth + 1); });
			node->child[0] = build(std::move(left), lbox, depth + 1);
			th.join();
			freeThreads.fetch_add(1);
			node->child[1] = std::move(r);
		} else {
			node->child[0] = build(std::move(left), lbox, depth + 1);
			node->child[1] = build(std::move(right), rbox, depth + 1);
		}
		return node;
	}
};

} // namespace
} // namespace phe_gb300

struct phe_host_bvh {
	std::vector<phe_bvh_node> nodes;
	std::vector<phe_triangle_vertices> verts;
	std::vector<uint32_t> slotToTri;
	uint32_t maxDepth = 0;
};

namespace phe_gb300 {
namespace {

void setBox(phe_bvh_node& n, int c, const AABB& b)
{
	float* f = n.fData + 6 * c;
	f[0] = b.lo[0]; f[1] = b.lo[1]; f[2] = b.lo[2];
	f[3] = b.hi[0]; f[4] = b.hi[1]; f[5] = b.hi[2];
}

void emitLeaf(phe_host_bvh& out, const float* verts, const std::vector<uint32_t>& tris, int32_t& first, int32_t& count)
{
	first = (int32_t)out.verts.size();
	count = (int32_t)tris.size();
	for (size_t i = 0; i < tris.size(); i++) {
		const float* t = verts + 9 * (size_t)tris[i];
		phe_triangle_vertices tv;
		float w = (i + 1 == tris.size()) ? -1.0f : 0.0f;
		tv.v0[0] = t[0]; tv.v0[1] = t[1]; tv.v0[2] = t[2]; tv.v0[3] = w;
		tv.v1[0] = t[3]; tv.v1[1] = t[4]; tv.v1[2] = t[5]; tv.v1[3] = w;
		tv.v2[0] = t[6]; tv.v2[1] = t[7]; tv.v2[2] = t[8]; tv.v2[3] = w;
		out.verts.push_back(tv);
		out.slotToTri.push_back(tris[i]);
	}
}

uint32_t flatten(phe_host_bvh& out, const float* verts, const TNode& node, uint32_t depth)
{
	uint32_t index = (uint32_t)out.nodes.size();
	out.nodes.push_back(phe_bvh_node{});
	for (int c = 0; c < 2; c++) {
		const TNode& ch = *node.child[c];
		setBox(out.nodes[index], c, ch.box);
		if (ch.leaf()) {
			int32_t first, count;
			emitLeaf(out, verts, ch.tris, first, count);
			out.nodes[index].iData[c] = ~first;
			out.nodes[index].iData[2 + c] = count;
			out.maxDepth = std::max(out.maxDepth, depth + 1);
		} else {
			uint32_t ci = flatten(out, verts, ch, depth + 1);
			out.nodes[index].iData[c] = (int32_t)ci;
			out.nodes[index].iData[2 + c] = 0;
		}
	}
	return index;
}

} // namespace
} // namespace phe_gb300

using namespace phe_gb300;

extern "C" void phe_sbvh_default_params(phe_sbvh_params* p)
{
	if (!p) return;
	p->splitAlpha = 1.0e-5f;
	p->maxDepth = 64;
	p->maxSpatialDepth = 48;
	p->numThreads = 0;
}

extern "C" phe_status phe_sbvh_build(const float* triVerts, uint32_t numTris, const phe_sbvh_params* params,
                                     phe_host_bvh** out)
{
	if (!triVerts || !out) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_sbvh_build: null argument");
	if (numTris == 0) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_sbvh_build: no triangles");
	NvtxRange range("phe_sbvh_build");
	*out = nullptr;
	Builder b;
	b.verts = triVerts;
	phe_sbvh_default_params(&b.params);
	if (params) b.params = *params;
	if (b.params.maxDepth < 1 || b.params.maxDepth > 64)
		return fail(PHE_ERR_INVALID_ARGUMENT, "phe_sbvh_build: maxDepth must be in [1, 64]");
	int threads = b.params.numThreads > 0 ? b.params.numThreads : (int)std::thread::hardware_concurrency();
	b.freeThreads = std::max(0, threads - 1);
	try {
		std::vector<Ref> refs(numTris);
		AABB root;
		for (uint32_t i = 0; i < numTris; i++) {
			refs[i].tri = i;
			for (int v = 0; v < 3; v++) refs[i].box.grow(triVerts + 9 * (size_t)i + 3 * v);
			for (int k = 0; k < 3; k++)
				if (!std::isfinite(refs[i].box.lo[k]) || !std::isfinite(refs[i].box.hi[k]))
					return fail(PHE_ERR_INVALID_ARGUMENT, "phe_sbvh_build: triangle %u has a non-finite vertex", i);
			root.grow(refs[i].box);
		}
		b.minOverlap = root.area() * b.params.splitAlpha;
		std::unique_ptr<TNode> tree = b.build(std::move(refs), root, 0);
		if (tree->leaf()) {
			// The layout needs an inner root: give it two copies of the single leaf.
			auto r = std::make_unique<TNode>();
			r->box = tree->box;
			auto dup = std::make_unique<TNode>();
			dup->box = tree->box;
			dup->tris = tree->tris;
			r->child[0] = std::move(tree);
			r->child[1] = std::move(dup);
			tree = std::move(r);
		}
		auto* h = new phe_host_bvh();
		h->nodes.reserve((size_t)numTris);
		h->verts.reserve((size_t)numTris + numTris / 4);
		flatten(*h, triVerts, *tree, 0);
		*out = h;
	} catch (const std::bad_alloc&) {
		return fail(PHE_ERR_OUT_OF_MEMORY, "phe_sbvh_build: host allocation failed");
	}
	return PHE_OK;
}

extern "C" phe_status phe_host_bvh_info(const phe_host_bvh* b, uint32_t* numNodes, uint32_t* numSlots, uint32_t* maxDepth)
{
	if (!b) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_host_bvh_info: null bvh");
	if (numNodes) *numNodes = (uint32_t)b->nodes.size();
	if (numSlots) *numSlots = (uint32_t)b->verts.size();
	if (maxDepth) *maxDepth = b->maxDepth;
	return PHE_OK;
}

extern "C" phe_status phe_host_bvh_copy(const phe_host_bvh* b, phe_bvh_node* nodes, phe_triangle_vertices* verts,
                                        uint32_t* slotToTri)
{
	if (!b) return fail(PHE_ERR_INVALID_ARGUMENT, "phe_host_bvh_copy: null bvh");
	if (nodes) std::memcpy(nodes, b->nodes.data(), b->nodes.size() * sizeof(phe_bvh_node));
	if (verts) std::memcpy(verts, b->verts.data(), b->verts.size() * sizeof(phe_triangle_vertices));
	if (slotToTri) std::memcpy(slotToTri, b->slotToTri.data(), b->slotToTri.size() * sizeof(uint32_t));
	return PHE_OK;
}

extern "C" void phe_host_bvh_free(phe_host_bvh* b) { delete b; }
