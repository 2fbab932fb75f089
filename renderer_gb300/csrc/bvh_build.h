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

// Builds over boxes (all finite). Always produces at least a root node.
BuildResult build_bvh(const std::vector<Box>& boxes, const BuildOptions& opt);

}  // namespace gbrt
