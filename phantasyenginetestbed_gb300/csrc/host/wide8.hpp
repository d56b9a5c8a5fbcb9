// 8-wide compressed node layout (PHE_LAYOUT_WIDE8), built on upload from the reference's binary tree.
//
// The binary tree is collapsed into nodes of up to 8 children (a node's inner children with the largest
// surface area are replaced by their own two children until there are 8), in the manner of Ylitie,
// Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs" (HPG
// 2017). Child boxes are stored as 8-bit offsets on a per-node, per-axis power-of-two grid, rounded
// outward, so every stored box contains the exact binary box it stands for. Leaf children point to a
// leaf record that keeps the exact binary box of the leaf and its slot range; the traversal re-tests
// that exact box with the reference arithmetic before it tests triangles.
//
// Node: 80 bytes = 5 x 16 bytes (20 words)
//   words 0..2  p'x, p'y, p'z (float): the grid origin minus 2^23 grid steps, (k - 2^23) * 2^e
//   word  3     ex | ey << 8 | ez << 16 | imask << 24: grid exponents (e + 128) and the mask of
//               slots holding inner children
//   word  4     childBase: index of the node of the first inner child (inner children are contiguous,
//               in slot order)
//   word  5     leafBase: index of the leaf record of the first leaf child (contiguous, slot order)
//   word  6     validMask: slots holding a child
//   word  7     0
//   words 8..11   x bytes: lo[0..3], lo[4..7], hi[0..3], hi[4..7]  (one byte per slot)
//   words 12..15  y bytes, words 16..19 z bytes, same order
// A child's bound on an axis is (k + q) * 2^e for its byte q; with f = 2^23 + q (an exact float) it is
// fma(f, 2^e, p') exactly, because |k| < 2^23 and so every such value is a float. Empty slots hold
// lo = 255, hi = 0.
// Leaf record: 32 bytes = (lo.x, lo.y, lo.z, firstSlot as bits), (hi.x, hi.y, hi.z, count as bits).
//
// Slots are assigned so that the child that comes first for rays of direction-sign octant o (bit i set
// when direction component i is negative) tends to sit in slot o; traversal visits hit children in
// the order of (slot XOR ray octant).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "phe_gb300.h"

namespace phe_gb300 {

constexpr uint32_t kWide8NodeWords = 20;
constexpr uint32_t kWide8LeafWords = 8;
constexpr int kWide8ExpBias = 128;
constexpr int kWide8MinExp = -100;
constexpr int kWide8MaxExp = 100;

struct Wide8Tree {
	std::vector<uint32_t> nodes;    // kWide8NodeWords per node, node 0 = root
	std::vector<uint32_t> leaves;   // kWide8LeafWords per leaf record
	uint32_t depth = 0;             // deepest level of a wide node (root = 1)
};

// Builds the 8-wide tree of a validated reference-layout tree. Returns false (with the reason) when a
// child box does not lie inside its parent's box, is inverted or not finite, or does not fit the grid
// exponent range: the scene then offers no 8-wide layout.
bool build_wide8(const phe_bvh_node* nodes, uint32_t numNodes, Wide8Tree& out, std::string& why);

} // namespace phe_gb300
