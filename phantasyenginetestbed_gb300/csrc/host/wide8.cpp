// Builder of the 8-wide compressed node layout (format in wide8.hpp).

#include "wide8.hpp"

#include "common.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>

namespace phe_gb300 {

namespace {

// A child as stored in a binary node: its box and either an inner node index or a leaf slot range.
struct Kid {
	float lo[3], hi[3];
	int32_t node;     // inner child: binary node index (count == 0)
	uint32_t first;   // leaf child: first slot
	uint32_t count;   // leaf child: triangle count (> 0)
};

Kid kid_of(const phe_bvh_node& n, int c)
{
	Kid k;
	for (int i = 0; i < 3; i++) {
		k.lo[i] = n.fData[6 * c + i];
		k.hi[i] = n.fData[6 * c + 3 + i];
	}
	int32_t raw = n.iData[c];
	k.count = (uint32_t)std::max(n.iData[2 + c], 0);
	k.node = k.count ? -1 : raw;
	k.first = k.count ? (uint32_t)(raw < 0 ? ~raw : raw) : 0u;
	return k;
}

bool finite_ordered(const Kid& k)
{
	for (int i = 0; i < 3; i++)
		if (!std::isfinite(k.lo[i]) || !std::isfinite(k.hi[i]) || k.lo[i] > k.hi[i]) return false;
	return true;
}

bool inside(const Kid& outer, const Kid& inner)
{
	for (int i = 0; i < 3; i++)
		if (inner.lo[i] < outer.lo[i] || inner.hi[i] > outer.hi[i]) return false;
	return true;
}

float area(const Kid& k)
{
	float dx = k.hi[0] - k.lo[0], dy = k.hi[1] - k.lo[1], dz = k.hi[2] - k.lo[2];
	return dx * dy + dy * dz + dz * dx;
}

// Grid of one axis: exponent e and k = floor(mn / 2^e) such that every child bound, rounded outward to
// the grid, is k + q steps with q in [0, 255], and |k| < 2^23 (so (k + q) * 2^e and (k - 2^23) * 2^e are
// exact floats). Returns false when no exponent in range works.
bool axis_grid(double mn, double mx, int& e, int64_t& k)
{
	const int64_t kLimit = (int64_t)1 << 23;
	int e0 = kWide8MinExp;
	double extent = mx - mn;
	if (extent > 0) e0 = std::max(e0, (int)std::floor(std::log2(extent / 255.0)) - 1);
	double mag = std::max(std::fabs(mn), std::fabs(mx));
	if (mag > 0) e0 = std::max(e0, (int)std::floor(std::log2(mag)) - 23);
	for (e = e0; e <= kWide8MaxExp; e++) {
		double lo = std::floor(std::ldexp(mn, -e)), hi = std::ceil(std::ldexp(mx, -e));
		if (hi - lo <= 255.0 && std::fabs(lo) < (double)kLimit && std::fabs(hi) < (double)kLimit) {
			k = (int64_t)lo;
			return true;
		}
	}
	return false;
}

uint32_t f2u(float f)
{
	uint32_t u;
	std::memcpy(&u, &f, 4);
	return u;
}

} // namespace

bool build_wide8(const phe_bvh_node* nodes, uint32_t numNodes, Wide8Tree& out, std::string& why)
{
	out.nodes.clear();
	out.leaves.clear();
	out.depth = 0;
	// Every box finite and ordered, every child box inside its parent's box (the box the grandparent
	// stores for the parent): then a leaf's own exact box test passing implies every ancestor's test
	// passes, so re-testing the leaf's exact box reproduces the binary traversal's decision for it.
	{
		struct Item { uint32_t node; Kid box; bool root; };
		std::vector<Item> st{{0, Kid{}, true}};
		while (!st.empty()) {
			Item it = st.back();
			st.pop_back();
			if (it.node >= numNodes) {
				why = "child index out of range";
				return false;
			}
			for (int c = 0; c < 2; c++) {
				Kid k = kid_of(nodes[it.node], c);
				if (!finite_ordered(k)) {
					why = "a child box is inverted or not finite";
					return false;
				}
				if (!it.root && !inside(it.box, k)) {
					why = "a child box is not inside its parent's box";
					return false;
				}
				if (!k.count) st.push_back({(uint32_t)k.node, k, false});
			}
		}
	}
	// 1. Collapse: each wide node starts from a binary node's two children and repeatedly replaces the
	//    inner child with the largest surface area by its two children, up to 8 children.
	struct WNode { std::vector<Kid> kids; std::vector<int32_t> sub; };
	std::vector<WNode> wn(1);
	std::vector<uint32_t> src{0};   // binary node of each wide node
	for (size_t w = 0; w < wn.size(); w++) {
		Kid kids[8];
		int n = 0;
		kids[n++] = kid_of(nodes[src[w]], 0);
		kids[n++] = kid_of(nodes[src[w]], 1);
		while (n < 8) {
			int best = -1;
			float bestArea = -1.0f;
			for (int i = 0; i < n; i++)
				if (!kids[i].count && area(kids[i]) > bestArea) {
					bestArea = area(kids[i]);
					best = i;
				}
			if (best < 0) break;
			const phe_bvh_node& x = nodes[kids[best].node];
			kids[best] = kid_of(x, 0);
			kids[n++] = kid_of(x, 1);
		}
		for (int i = 0; i < n; i++) {
			wn[w].kids.push_back(kids[i]);
			int32_t sub = -1;
			if (!kids[i].count) {
				sub = (int32_t)wn.size();
				wn.emplace_back();
				src.push_back((uint32_t)kids[i].node);
			}
			wn[w].sub.push_back(sub);
		}
	}
	// 2. Emit breadth-first, so that each node's inner children are contiguous.
	struct Job { int32_t w; uint32_t index, depth; };
	std::deque<Job> jobs{{0, 0, 1}};
	out.nodes.assign(kWide8NodeWords, 0u);
	while (!jobs.empty()) {
		Job job = jobs.front();
		jobs.pop_front();
		out.depth = std::max(out.depth, job.depth);
		const WNode& W = wn[job.w];
		const int n = (int)W.kids.size();
		const Kid* kids = W.kids.data();
		// Slots: child c in slot s comes first for rays of octant s; greedy assignment by the projection
		// of the child's centre (relative to the node's) on the octant's diagonal.
		float cen[3] = {0, 0, 0};
		{
			float mn[3], mx[3];
			for (int i = 0; i < 3; i++) {
				mn[i] = kids[0].lo[i];
				mx[i] = kids[0].hi[i];
				for (int c = 1; c < n; c++) {
					mn[i] = std::min(mn[i], kids[c].lo[i]);
					mx[i] = std::max(mx[i], kids[c].hi[i]);
				}
				cen[i] = 0.5f * (mn[i] + mx[i]);
			}
		}
		int slotKid[8];
		for (int s = 0; s < 8; s++) slotKid[s] = -1;
		bool used[8] = {false, false, false, false, false, false, false, false};
		for (int round = 0; round < n; round++) {
			float bestCost = 0.0f;
			int bc = -1, bs = -1;
			for (int c = 0; c < n; c++) {
				if (used[c]) continue;
				for (int s = 0; s < 8; s++) {
					if (slotKid[s] >= 0) continue;
					float cost = 0.0f;
					for (int i = 0; i < 3; i++) {
						float d = 0.5f * (kids[c].lo[i] + kids[c].hi[i]) - cen[i];
						cost += (s >> i & 1) ? -d : d;
					}
					if (bc < 0 || cost < bestCost) {
						bestCost = cost;
						bc = c;
						bs = s;
					}
				}
			}
			used[bc] = true;
			slotKid[bs] = bc;
		}
		uint32_t* w = &out.nodes[(size_t)job.index * kWide8NodeWords];
		uint32_t imask = 0, valid = 0;
		for (int s = 0; s < 8; s++) {
			if (slotKid[s] < 0) continue;
			valid |= 1u << s;
			if (!kids[slotKid[s]].count) imask |= 1u << s;
		}
		uint32_t meta = imask << 24;
		for (int i = 0; i < 3; i++) {
			double mn = INFINITY, mx = -INFINITY;
			for (int c = 0; c < n; c++) {
				mn = std::min(mn, (double)kids[c].lo[i]);
				mx = std::max(mx, (double)kids[c].hi[i]);
			}
			int e = 0;
			int64_t k = 0;
			if (!axis_grid(mn, mx, e, k)) {
				why = "a node's extent does not fit the grid exponent range";
				return false;
			}
			meta |= (uint32_t)(e + kWide8ExpBias) << (8 * i);
			float pPrime = (float)std::ldexp((double)(k - ((int64_t)1 << 23)), e);
			w[i] = f2u(pPrime);
			uint8_t lo[8], hi[8];
			for (int s = 0; s < 8; s++) {
				if (slotKid[s] < 0) {
					lo[s] = 255;
					hi[s] = 0;
					continue;
				}
				const Kid& kd = kids[slotKid[s]];
				int64_t ql = (int64_t)std::floor(std::ldexp((double)kd.lo[i], -e)) - k;
				int64_t qh = (int64_t)std::ceil(std::ldexp((double)kd.hi[i], -e)) - k;
				if (ql < 0 || qh > 255 || ql > qh) {
					why = "grid quantization out of range";
					return false;
				}
				lo[s] = (uint8_t)ql;
				hi[s] = (uint8_t)qh;
			}
			uint32_t* b = w + 8 + 4 * i;
			std::memcpy(&b[0], lo, 4);
			std::memcpy(&b[1], lo + 4, 4);
			std::memcpy(&b[2], hi, 4);
			std::memcpy(&b[3], hi + 4, 4);
		}
		w[3] = meta;
		uint32_t childBase = (uint32_t)(out.nodes.size() / kWide8NodeWords);
		uint32_t leafBase = (uint32_t)(out.leaves.size() / kWide8LeafWords);
		w[4] = childBase;
		w[5] = leafBase;
		w[6] = valid;
		w[7] = 0;
		uint32_t nInner = (uint32_t)__builtin_popcount(imask);
		out.nodes.resize(out.nodes.size() + (size_t)nInner * kWide8NodeWords, 0u);   // w is not used past here
		uint32_t innerRank = 0;
		for (int s = 0; s < 8; s++) {
			if (slotKid[s] < 0) continue;
			const Kid& kd = kids[slotKid[s]];
			if (kd.count) {
				uint32_t rec[kWide8LeafWords] = {f2u(kd.lo[0]), f2u(kd.lo[1]), f2u(kd.lo[2]), kd.first,
				                                 f2u(kd.hi[0]), f2u(kd.hi[1]), f2u(kd.hi[2]), kd.count};
				out.leaves.insert(out.leaves.end(), rec, rec + kWide8LeafWords);
			} else {
				jobs.push_back({W.sub[slotKid[s]], childBase + innerRank++, job.depth + 1});
			}
		}
	}
	return true;
}

} // namespace phe_gb300

using namespace phe_gb300;

extern "C" phe_status phe_bvh_wide8_build(const phe_bvh_node* nodes, uint32_t numNodes, uint32_t numSlots,
                                          uint32_t* nodeWords, uint32_t maxNodes, uint32_t* leafWords,
                                          uint32_t maxLeaves, uint32_t* numNodes8, uint32_t* numLeaves8,
                                          uint32_t* depth)
{
	phe_status s = phe_bvh_validate(nodes, numNodes, numSlots, nullptr);
	if (s) return s;
	Wide8Tree t;
	std::string why;
	if (!build_wide8(nodes, numNodes, t, why)) return fail(PHE_ERR_INVALID_SCENE, "no 8-wide layout: %s", why.c_str());
	uint32_t nn = (uint32_t)(t.nodes.size() / kWide8NodeWords), nl = (uint32_t)(t.leaves.size() / kWide8LeafWords);
	if (numNodes8) *numNodes8 = nn;
	if (numLeaves8) *numLeaves8 = nl;
	if (depth) *depth = t.depth;
	if ((nodeWords && maxNodes < nn) || (leafWords && maxLeaves < nl))
		return fail(PHE_ERR_TOO_LARGE, "phe_bvh_wide8_build: output arrays too small (%u nodes, %u leaves)", nn, nl);
	if (nodeWords) std::memcpy(nodeWords, t.nodes.data(), t.nodes.size() * 4);
	if (leafWords) std::memcpy(leafWords, t.leaves.data(), t.leaves.size() * 4);
	return PHE_OK;
}
