// bvh_build.h — host-side binned-SAH BVH2 builder for the GB300 tracer.
//
// Replaces BVHNode::create (src/bvh.cpp:67-94), whose median split by box
// centre gives a tree the GPU would traverse poorly. The closest hit does not
// depend on the tree; only exact-t ties may resolve differently.
#pragma once

#include <cstdint>
#include <vector>

namespace gbrt {

struct Box {
  float lo[3], hi[3];
};

// One 64-byte node: the bounds of both children and their references, laid
// out for four 128-bit loads (child 0 x/y, child 1 x/y, both z, refs).
//   a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (ref0, ref1, 0, 0)
// ref >= 0: index of an inner node. ref < 0: a leaf; ~ref = first << 4 |
// (count - 1), first indexing the leaf-ordered primitive records. A scene
// that is a single leaf gets a root whose two children both refer to it.
struct alignas(16) Node {
  float a[4], b[4], c[4];
  int32_t d[4];
};

constexpr int kMaxLeafPrims = 16;
// The traversal stack holds one entry per level. From depth kSahDepthLimit on
// the builder uses object-median splits, which halve the primitive count per
// level, so a tree over fewer than 2^27 primitives (the record-index limit)
// stays within kSahDepthLimit + 24 <= kMaxTreeDepth levels.
constexpr int kMaxTreeDepth = 62;
constexpr int kSahDepthLimit = 36;

struct BuildOptions {
  int max_leaf = 8;        // hard cap on primitives per leaf (<= 16)
  int bins = 32;           // SAH bins per axis
  float cost_node = 1.0f;  // SAH traversal cost of a node
  float cost_prim = 1.5f;  // SAH cost of a primitive test
  int threads = 0;         // 0 = hardware concurrency
};

struct BuildResult {
  std::vector<Node> nodes;        // nodes[0] is the root
  std::vector<uint32_t> order;    // leaf order -> input primitive index
  int64_t leaves = 0;
  int max_depth = 0;
  double sah_cost = 0;            // SAH cost of the tree relative to the root box
};

// Builds over boxes (all finite). Produces no node for an empty input.
BuildResult build_bvh(const std::vector<Box>& boxes, const BuildOptions& opt);

// A 4-wide node, 128 bytes: the boxes of up to four children as six float4
// planes (lo.x of children 0..3, hi.x, lo.y, hi.y, lo.z, hi.z), then the four
// child references (same encoding as Node; kEmptyRef for an unused slot, whose
// box is inverted so it never intersects).
struct alignas(16) Node4 {
  float lox[4], hix[4], loy[4], hiy[4], loz[4], hiz[4];
  int32_t ref[4];
  int32_t pad[4];
};
constexpr int32_t kEmptyRef = 0x7fffffff;

struct Collapsed {
  std::vector<Node4> nodes;  // nodes[0] is the root
  int max_depth = 0;         // levels of 4-wide nodes
};

// Collapses a binary tree into a 4-wide one: every 4-wide node takes the two
// children of a binary node and keeps opening its largest inner child until it
// holds four. Leaves (primitive ranges) are unchanged.
Collapsed collapse_bvh4(const BuildResult& b2);

}  // namespace gbrt
