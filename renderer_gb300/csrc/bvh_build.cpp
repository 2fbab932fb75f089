// bvh_build.cpp — binned-SAH BVH2 builder (Wald 2007, "On fast Construction of
// SAH-based Bounding Volume Hierarchies"): centroid binning per axis, the
// cheapest bin boundary by surface-area cost, a leaf when splitting costs more
// or the node is small. Large subtrees are built on worker threads and spliced
// into one depth-first node array (left child stored right after its parent).
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <future>
#include <limits>
#include <thread>

namespace gbrt {
namespace {

constexpr float kInf = std::numeric_limits<float>::infinity();

struct Bounds {
  float lo[3] = {kInf, kInf, kInf};
  float hi[3] = {-kInf, -kInf, -kInf};
  void grow(const float* l, const float* h) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], l[k]);
      hi[k] = std::max(hi[k], h[k]);
    }
  }
  void grow(const Bounds& b) { grow(b.lo, b.hi); }
  void growPoint(const float* p) { grow(p, p); }
  float area() const {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (!(dx >= 0) || !(dy >= 0) || !(dz >= 0)) return 0.f;
    return 2.f * (dx * dy + dy * dz + dz * dx);
  }
};

struct Ref {
  float lo[3], hi[3], c[3];
  uint32_t idx;
};

// A subtree built on its own: nodes with local indices, leaf primitive ranges
// relative to the subtree's slice of the reference array.
struct SubTree {
  std::vector<Node> nodes;
  int64_t leaves = 0;
  int max_depth = 0;
  double sah = 0;  // sum over nodes of area * cost (unnormalised)
};

struct Builder {
  const BuildOptions& opt;
  explicit Builder(const BuildOptions& o) : opt(o) {}

  static int32_t leafRef(uint32_t first, uint32_t count) {
    return ~int32_t((first << 4) | (count - 1));
  }

  static void setChild(Node& n, int which, const Bounds& b, int32_t ref) {
    float* xy = which == 0 ? n.a : n.b;
    xy[0] = b.lo[0]; xy[1] = b.hi[0]; xy[2] = b.lo[1]; xy[3] = b.hi[1];
    n.c[which * 2 + 0] = b.lo[2];
    n.c[which * 2 + 1] = b.hi[2];
    n.d[which] = ref;
  }

  // Chooses a split of refs[begin, end). Returns the split position (begin <
  // mid < end) or -1 for "make a leaf".
  int64_t split(Ref* refs, int64_t begin, int64_t end, const Bounds& nb, int depth) {
    const int64_t n = end - begin;
    if (n <= 1) return -1;
    Bounds cb;
    for (int64_t i = begin; i < end; ++i) cb.growPoint(refs[i].c);
    if (depth >= kSahDepthLimit) {
      if (n <= opt.max_leaf) return -1;
      // Object median on the widest centroid axis: halves the count per level.
      int axis = 0;
      float best = -1.f;
      for (int k = 0; k < 3; ++k) {
        float e = cb.hi[k] - cb.lo[k];
        if (e > best) { best = e; axis = k; }
      }
      int64_t mid = begin + n / 2;
      std::nth_element(refs + begin, refs + mid, refs + end,
                       [axis](const Ref& x, const Ref& y) { return x.c[axis] < y.c[axis]; });
      return mid;
    }
    const int B = opt.bins;
    float bestCost = kInf;
    int bestAxis = -1, bestBin = -1;
    std::vector<Bounds> bb(B);
    std::vector<int64_t> cnt(B);
    std::vector<float> rightArea(B);
    std::vector<int64_t> rightCnt(B);
    for (int axis = 0; axis < 3; ++axis) {
      float ext = cb.hi[axis] - cb.lo[axis];
      if (!(ext > 0)) continue;
      float scale = B / ext;
      for (int b = 0; b < B; ++b) { bb[b] = Bounds(); cnt[b] = 0; }
      for (int64_t i = begin; i < end; ++i) {
        int b = int((refs[i].c[axis] - cb.lo[axis]) * scale);
        b = std::min(std::max(b, 0), B - 1);
        bb[b].grow(refs[i].lo, refs[i].hi);
        cnt[b]++;
      }
      Bounds acc;
      int64_t c = 0;
      for (int b = B - 1; b > 0; --b) {
        acc.grow(bb[b]);
        c += cnt[b];
        rightArea[b] = acc.area();
        rightCnt[b] = c;
      }
      acc = Bounds();
      c = 0;
      for (int b = 0; b < B - 1; ++b) {
        acc.grow(bb[b]);
        c += cnt[b];
        if (c == 0 || rightCnt[b + 1] == 0) continue;
        float cost = acc.area() * float(c) + rightArea[b + 1] * float(rightCnt[b + 1]);
        if (cost < bestCost) { bestCost = cost; bestAxis = axis; bestBin = b; }
      }
    }
    float parentArea = nb.area();
    float leafCost = opt.cost_prim * float(n);
    bool mustSplit = n > opt.max_leaf;
    if (bestAxis >= 0) {
      float splitCost = opt.cost_node + (parentArea > 0 ? opt.cost_prim * bestCost / parentArea : kInf);
      if (!mustSplit && splitCost >= leafCost) return -1;
      float ext = cb.hi[bestAxis] - cb.lo[bestAxis];
      float scale = B / ext;
      Ref* mid = std::partition(refs + begin, refs + end, [&](const Ref& r) {
        int b = int((r.c[bestAxis] - cb.lo[bestAxis]) * scale);
        b = std::min(std::max(b, 0), B - 1);
        return b <= bestBin;
      });
      int64_t m = mid - refs;
      if (m > begin && m < end) return m;
    }
    if (!mustSplit) return -1;
    // Degenerate centroids: split by index.
    return begin + n / 2;
  }

  // Builds refs[begin, end) into st. Returns the child reference of the root
  // (an inner node index local to st, or a leaf with first relative to base).
  int32_t buildRec(Ref* refs, int64_t begin, int64_t end, int64_t base, const Bounds& nb, int depth,
                   SubTree& st) {
    st.max_depth = std::max(st.max_depth, depth);
    int64_t mid = split(refs, begin, end, nb, depth);
    if (mid < 0) {
      st.leaves++;
      st.sah += double(nb.area()) * opt.cost_prim * double(end - begin);
      return leafRef(uint32_t(begin - base), uint32_t(end - begin));
    }
    int32_t me = int32_t(st.nodes.size());
    st.nodes.emplace_back();
    st.sah += double(nb.area()) * opt.cost_node;
    Bounds lb, rb;
    for (int64_t i = begin; i < mid; ++i) lb.grow(refs[i].lo, refs[i].hi);
    for (int64_t i = mid; i < end; ++i) rb.grow(refs[i].lo, refs[i].hi);
    int32_t l = buildRec(refs, begin, mid, base, lb, depth + 1, st);
    int32_t r = buildRec(refs, mid, end, base, rb, depth + 1, st);
    setChild(st.nodes[me], 0, lb, l);
    setChild(st.nodes[me], 1, rb, r);
    return me;
  }
};

// Shifts a subtree's references when splicing it at node offset noff and
// primitive offset poff.
int32_t shiftRef(int32_t ref, int32_t noff, uint32_t poff) {
  if (ref >= 0) return ref + noff;
  uint32_t v = ~uint32_t(ref);
  uint32_t first = (v >> 4) + poff;
  return ~int32_t((first << 4) | (v & 15u));
}

}  // namespace

BuildResult build_bvh(const std::vector<Box>& boxes, const BuildOptions& optIn) {
  BuildOptions opt = optIn;
  opt.max_leaf = std::min(std::max(opt.max_leaf, 1), kMaxLeafPrims);
  opt.bins = std::max(opt.bins, 4);
  BuildResult res;
  const int64_t n = int64_t(boxes.size());
  std::vector<Ref> refs(n);
  Bounds root;
  for (int64_t i = 0; i < n; ++i) {
    Ref& r = refs[i];
    for (int k = 0; k < 3; ++k) {
      r.lo[k] = boxes[i].lo[k];
      r.hi[k] = boxes[i].hi[k];
      r.c[k] = 0.5f * (r.lo[k] + r.hi[k]);
    }
    r.idx = uint32_t(i);
    root.grow(r.lo, r.hi);
  }
  Builder b(opt);
  if (n == 0) return res;  // no nodes: the caller skips traversal

  // Top levels on this thread down to a task size, then subtrees in parallel.
  unsigned hw = opt.threads > 0 ? unsigned(opt.threads) : std::max(1u, std::thread::hardware_concurrency());
  const int64_t taskSize = std::max<int64_t>(n / (int64_t(hw) * 4), 4096);

  struct Task { int64_t begin, end; Bounds nb; int depth; int32_t parent; int which; };
  std::vector<Node> top;
  std::vector<Task> tasks;
  int64_t topLeaves = 0;
  int topDepth = 0;
  double topSah = 0;
  // Iterative top-level split: node slots first, big children become tasks.
  struct Pending { int64_t begin, end; Bounds nb; int depth; int32_t parent; int which; };
  std::vector<Pending> stack;
  stack.push_back({0, n, root, 0, -1, 0});
  int32_t rootRef = 0;
  while (!stack.empty()) {
    Pending p = stack.back();
    stack.pop_back();
    int64_t cnt = p.end - p.begin;
    if (cnt <= taskSize || hw == 1) {
      tasks.push_back({p.begin, p.end, p.nb, p.depth, p.parent, p.which});
      continue;
    }
    int64_t mid = b.split(refs.data(), p.begin, p.end, p.nb, p.depth);
    topDepth = std::max(topDepth, p.depth);
    if (mid < 0) {
      tasks.push_back({p.begin, p.end, p.nb, p.depth, p.parent, p.which});
      continue;
    }
    int32_t me = int32_t(top.size());
    top.emplace_back();
    topSah += double(p.nb.area()) * opt.cost_node;
    if (p.parent >= 0) top[p.parent].d[p.which] = me;
    else rootRef = me;
    Bounds lb, rb;
    for (int64_t i = p.begin; i < mid; ++i) lb.grow(refs[i].lo, refs[i].hi);
    for (int64_t i = mid; i < p.end; ++i) rb.grow(refs[i].lo, refs[i].hi);
    Builder::setChild(top[me], 0, lb, 0);
    Builder::setChild(top[me], 1, rb, 0);
    stack.push_back({mid, p.end, rb, p.depth + 1, me, 1});
    stack.push_back({p.begin, mid, lb, p.depth + 1, me, 0});
  }

  std::vector<SubTree> subs(tasks.size());
  std::vector<int32_t> subRoot(tasks.size());
  {
    std::atomic<size_t> next{0};
    auto worker = [&]() {
      for (;;) {
        size_t t = next.fetch_add(1);
        if (t >= tasks.size()) break;
        const Task& tk = tasks[t];
        subRoot[t] = b.buildRec(refs.data(), tk.begin, tk.end, tk.begin, tk.nb, tk.depth, subs[t]);
      }
    };
    unsigned nt = std::min<unsigned>(hw, unsigned(tasks.size()));
    std::vector<std::thread> th;
    for (unsigned i = 1; i < nt; ++i) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
  }

  // Splice: top nodes first, then every subtree's nodes.
  res.nodes = top;
  bool rootIsTask = top.empty();
  for (size_t t = 0; t < tasks.size(); ++t) {
    int32_t noff = int32_t(res.nodes.size());
    uint32_t poff = uint32_t(tasks[t].begin);
    for (Node nd : subs[t].nodes) {
      nd.d[0] = shiftRef(nd.d[0], noff, poff);
      nd.d[1] = shiftRef(nd.d[1], noff, poff);
      res.nodes.push_back(nd);
    }
    int32_t ref = shiftRef(subRoot[t], noff, poff);
    if (tasks[t].parent >= 0) res.nodes[tasks[t].parent].d[tasks[t].which] = ref;
    else rootRef = ref;
    res.leaves += subs[t].leaves;
    res.max_depth = std::max(res.max_depth, subs[t].max_depth);
    topSah += subs[t].sah;
  }
  res.leaves += topLeaves;
  res.max_depth = std::max(res.max_depth, topDepth);

  if (rootIsTask && rootRef < 0) {
    // The whole scene is one leaf (and no node was made): wrap it in a root
    // whose two children both refer to that leaf. The duplicate test is
    // harmless because a later hit must be strictly closer to replace one.
    Node node;
    Builder::setChild(node, 0, root, rootRef);
    Builder::setChild(node, 1, root, rootRef);
    res.nodes.insert(res.nodes.begin(), node);
  }
  res.order.resize(n);
  for (int64_t i = 0; i < n; ++i) res.order[i] = refs[i].idx;
  float ra = root.area();
  res.sah_cost = ra > 0 ? topSah / ra : 0;
  return res;
}

namespace {

struct Child {
  float lo[3], hi[3];
  int32_t ref;
  float area() const {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return 2.f * (dx * dy + dy * dz + dz * dx);
  }
};

Child childOf(const Node& n, int which) {
  Child c;
  const float* xy = which == 0 ? n.a : n.b;
  c.lo[0] = xy[0]; c.hi[0] = xy[1]; c.lo[1] = xy[2]; c.hi[1] = xy[3];
  c.lo[2] = n.c[which * 2]; c.hi[2] = n.c[which * 2 + 1];
  c.ref = n.d[which];
  return c;
}

int32_t collapseRec(const std::vector<Node>& n2, int32_t ref2, int depth, Collapsed& out) {
  out.max_depth = std::max(out.max_depth, depth + 1);
  Child ch[4];
  int cnt = 0;
  ch[cnt++] = childOf(n2[ref2], 0);
  ch[cnt++] = childOf(n2[ref2], 1);
  if (ch[0].ref == ch[1].ref) cnt = 1;  // a single-leaf scene: both slots name the same leaf
  while (cnt < 4) {
    int best = -1;
    float bestArea = -1.f;
    for (int i = 0; i < cnt; ++i)
      if (ch[i].ref >= 0 && ch[i].area() > bestArea) { bestArea = ch[i].area(); best = i; }
    if (best < 0) break;
    const Node& nd = n2[ch[best].ref];
    ch[best] = childOf(nd, 0);
    ch[cnt++] = childOf(nd, 1);
  }
  int32_t me = int32_t(out.nodes.size());
  out.nodes.emplace_back();
  Node4 node;
  for (int i = 0; i < 4; ++i) {
    if (i < cnt) {
      node.lox[i] = ch[i].lo[0]; node.hix[i] = ch[i].hi[0];
      node.loy[i] = ch[i].lo[1]; node.hiy[i] = ch[i].hi[1];
      node.loz[i] = ch[i].lo[2]; node.hiz[i] = ch[i].hi[2];
    } else {
      node.lox[i] = node.loy[i] = node.loz[i] = INFINITY;
      node.hix[i] = node.hiy[i] = node.hiz[i] = -INFINITY;
    }
    node.ref[i] = kEmptyRef;
    node.pad[i] = 0;
  }
  for (int i = 0; i < cnt; ++i) node.ref[i] = ch[i].ref >= 0 ? collapseRec(n2, ch[i].ref, depth + 1, out) : ch[i].ref;
  out.nodes[me] = node;
  return me;
}

}  // namespace

Collapsed collapse_bvh4(const BuildResult& b2) {
  Collapsed out;
  if (b2.nodes.empty()) return out;
  out.nodes.reserve(b2.nodes.size() / 2 + 1);
  collapseRec(b2.nodes, 0, 0, out);
  return out;
}

}  // namespace gbrt
