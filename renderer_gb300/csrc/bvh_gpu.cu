// bvh_gpu.cu — GPU builder of the 4-wide BVH (GBRT_SCENE_GPU_BUILD).
//
// Replaces, like bvh_build.cpp, BVHNode::create (src/bvh.cpp:67-94), for
// scenes whose host build would dominate the time to first image. It is a
// linear BVH (Karras, "Maximizing parallelism in the construction of BVHs,
// octrees, and k-d trees", HPG 2012):
//   1. 30-bit Morton codes of the box centres inside the centres' bounds;
//   2. a stable LSD radix sort of (code, index) pairs, one bit per pass
//      (count, scan, scatter), so equal codes keep their input order;
//   3. the binary radix tree over the sorted codes, one thread per inner
//      node (range by exponential and binary search on the common-prefix
//      length, ties broken by index);
//   4. node boxes bottom-up, one thread per primitive, the second thread to
//      reach a node computing its box;
//   5. a top-down collapse into the traversal's 128-byte Node4, one level per
//      launch: every 4-wide node takes a binary node's two children and opens
//      its largest inner child until it has four; a subtree becomes one leaf
//      (its primitives are contiguous in the sorted order) when that is
//      cheaper by the surface-area heuristic (decided bottom-up in step 4,
//      at most max_leaf primitives).
// The closest hit does not depend on the tree; only exact-t ties may resolve
// differently from another build.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "bvh_gpu.h"

namespace gbrt {
namespace {

constexpr int kSortThreads = 1024, kSortPerThread = 4, kSortTile = kSortThreads * kSortPerThread;

// Order-preserving float <-> uint mapping for atomic min / max.
__device__ __forceinline__ unsigned f2o(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void k_centre_bounds(const float* __restrict__ box, int64_t n, unsigned* __restrict__ bnd) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float* b = box + 6 * i;
    for (int k = 0; k < 3; ++k) {
      float c = 0.5f * (b[k] + b[3 + k]);
      lo[k] = fminf(lo[k], c);
      hi[k] = fmaxf(hi[k], c);
    }
  }
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = fminf(lo[k], __shfl_down_sync(0xffffffffu, lo[k], o));
      hi[k] = fmaxf(hi[k], __shfl_down_sync(0xffffffffu, hi[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 3; ++k) {
      atomicMin(&bnd[k], f2o(lo[k]));
      atomicMax(&bnd[3 + k], f2o(hi[k]));
    }
  }
}

__device__ __forceinline__ unsigned spread10(unsigned v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void k_morton(const float* __restrict__ box, int64_t n, const unsigned* __restrict__ bnd,
                         unsigned* __restrict__ key, unsigned* __restrict__ val) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* b = box + 6 * i;
  unsigned q[3];
  for (int k = 0; k < 3; ++k) {
    float lo = o2f(bnd[k]), hi = o2f(bnd[3 + k]);
    float c = 0.5f * (b[k] + b[3 + k]);
    float t = hi > lo ? (c - lo) / (hi - lo) : 0.f;
    q[k] = unsigned(fminf(fmaxf(t * 1024.f, 0.f), 1023.f));
  }
  key[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  val[i] = unsigned(i);
}

// ---- stable one-bit split sort --------------------------------------------
// Zeros of bit `bit` per tile of kSortTile keys.
__global__ void __launch_bounds__(kSortThreads) k_split_count(const unsigned* __restrict__ key, int64_t n, int bit,
                                                              unsigned* __restrict__ zeros) {
  __shared__ unsigned s[32];
  const int64_t base = int64_t(blockIdx.x) * kSortTile + int64_t(threadIdx.x) * kSortPerThread;
  unsigned c = 0;
  for (int j = 0; j < kSortPerThread; ++j) {
    int64_t i = base + j;
    if (i < n) c += ((key[i] >> bit) & 1u) ^ 1u;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned v = s[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) zeros[blockIdx.x] = v;
  }
}

// Exclusive scan of the tile counts in place (one block), total in zeros[nt].
__global__ void __launch_bounds__(1024) k_split_scan(unsigned* __restrict__ zeros, int nt) {
  __shared__ unsigned s[1024];
  const int per = (nt + 1023) / 1024;
  const int b = threadIdx.x * per;
  unsigned sum = 0;
  for (int j = 0; j < per; ++j)
    if (b + j < nt) sum += zeros[b + j];
  s[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    unsigned v = threadIdx.x >= unsigned(o) ? s[threadIdx.x - o] : 0u;
    __syncthreads();
    s[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned run = s[threadIdx.x] - sum;  // exclusive
  for (int j = 0; j < per; ++j) {
    if (b + j < nt) {
      unsigned z = zeros[b + j];
      zeros[b + j] = run;
      run += z;
    }
  }
  if (threadIdx.x == 1023) zeros[nt] = s[1023];
}

// Stable scatter: zeros first, in order, then ones, in order.
__global__ void __launch_bounds__(kSortThreads) k_split_scatter(const unsigned* __restrict__ key,
                                                                const unsigned* __restrict__ val, int64_t n, int bit,
                                                                const unsigned* __restrict__ zeros, int nt,
                                                                unsigned* __restrict__ key2,
                                                                unsigned* __restrict__ val2) {
  __shared__ unsigned s[32];
  const int64_t tile0 = int64_t(blockIdx.x) * kSortTile;
  const int64_t base = tile0 + int64_t(threadIdx.x) * kSortPerThread;
  unsigned k[kSortPerThread], v[kSortPerThread];
  unsigned c = 0;
  for (int j = 0; j < kSortPerThread; ++j) {
    int64_t i = base + j;
    k[j] = i < n ? key[i] : 0xffffffffu;
    v[j] = i < n ? val[i] : 0u;
    if (i < n) c += ((k[j] >> bit) & 1u) ^ 1u;
  }
  // exclusive prefix of the zero counts over the block's threads
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned incl = c;
  for (int o = 1; o < 32; o <<= 1) {
    unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned w = s[lane];
    unsigned wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    s[lane] = wi - w;
  }
  __syncthreads();
  unsigned zbefore = zeros[blockIdx.x] + s[warp] + incl - c;  // zeros before this thread's first key
  const unsigned total_zeros = zeros[nt];
  for (int j = 0; j < kSortPerThread; ++j) {
    int64_t i = base + j;
    if (i >= n) break;
    unsigned pos;
    if (((k[j] >> bit) & 1u) == 0u) {
      pos = zbefore++;
    } else {
      unsigned obefore = unsigned(i) - zbefore;  // ones before key i
      pos = total_zeros + obefore;
    }
    key2[pos] = k[j];
    val2[pos] = v[j];
  }
}

// ---- binary radix tree ----------------------------------------------------
// Inner node i (0 = root) of n - 1; child c >= 0 an inner node, c < 0 the
// sorted primitive ~c. first / last: the sorted primitives below.
struct Inner {
  int left, right, parent, first, last;
  float lo[3], hi[3];
  float cost;    // SAH cost of the subtree (per unit of its box area)
  int leafable;  // cheaper as one leaf than split (and at most max_leaf primitives)
};

// SAH costs of the leaf decision (those of the host builder).
constexpr float kCostNode = 1.0f, kCostPrim = 1.5f;

__device__ __forceinline__ float half_area(const float* lo, const float* hi) {
  float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
  return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ int delta(const unsigned* __restrict__ k, int64_t n, int64_t i, int64_t j) {
  if (j < 0 || j >= n) return -1;
  unsigned a = k[i], b = k[j];
  if (a == b) return 32 + __clz(unsigned(i) ^ unsigned(j));
  return __clz(a ^ b);
}

__global__ void k_radix_tree(const unsigned* __restrict__ k, int64_t n, Inner* __restrict__ nodes,
                             int* __restrict__ leaf_parent) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(k, n, i, i - d);
  int64_t lmax = 2;
  while (delta(k, n, i, i + lmax * d) > dmin) lmax *= 2;
  int64_t l = 0;
  for (int64_t t = lmax / 2; t >= 1; t /= 2)
    if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
  const int64_t j = i + l * d;
  const int dnode = delta(k, n, i, j);
  int64_t s = 0;
  int64_t t = l;
  do {
    t = (t + 1) / 2;
    if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int64_t split = i + s * d + min(d, 0);
  const int64_t first = min(i, j), last = max(i, j);
  Inner& nd = nodes[i];
  nd.first = int(first);
  nd.last = int(last);
  if (first == split) {
    nd.left = ~int(split);
    leaf_parent[split] = int(i);
  } else {
    nd.left = int(split);
    nodes[split].parent = int(i);
  }
  if (last == split + 1) {
    nd.right = ~int(split + 1);
    leaf_parent[split + 1] = int(i);
  } else {
    nd.right = int(split + 1);
    nodes[split + 1].parent = int(i);
  }
  if (i == 0) nd.parent = -1;
}

__device__ __forceinline__ void child_box(const Inner* nodes, const float* sbox, int c, float* lo, float* hi) {
  if (c >= 0) {
    for (int k = 0; k < 3; ++k) { lo[k] = nodes[c].lo[k]; hi[k] = nodes[c].hi[k]; }
  } else {
    const float* b = sbox + 6 * int64_t(~c);
    for (int k = 0; k < 3; ++k) { lo[k] = b[k]; hi[k] = b[3 + k]; }
  }
}

// Boxes of the sorted primitives, and the inner boxes bottom-up.
__global__ void k_gather_boxes(const float* __restrict__ box, const unsigned* __restrict__ order, int64_t n,
                               float* __restrict__ sbox) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* b = box + 6 * int64_t(order[i]);
  for (int k = 0; k < 6; ++k) sbox[6 * i + k] = b[k];
}

// A radix tree over 30-bit codes with index tie-breaks is at most 30 + 27
// levels deep; the walk stops (and flags) after kMaxWalk.
constexpr int kMaxWalk = 128;

// Boxes bottom-up; with both children known, also the node's SAH cost,
// min(leaf, split), and whether a leaf is the cheaper choice.
__global__ void k_inner_boxes(Inner* nodes, const float* __restrict__ sbox, const int* __restrict__ leaf_parent,
                              int64_t n, int max_leaf, int* __restrict__ visits, int* __restrict__ bad) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int p = leaf_parent[i];
  for (int step = 0; p >= 0; ++step) {
    if (step >= kMaxWalk || p >= n - 1) {
      atomicExch(bad, 1);
      return;
    }
    __threadfence();
    if (atomicAdd(&visits[p], 1) == 0) return;  // the other child is not done yet
    __threadfence();
    float l0[3], h0[3], l1[3], h1[3], lo[3], hi[3];
    const int cl = nodes[p].left, cr = nodes[p].right;
    child_box(nodes, sbox, cl, l0, h0);
    child_box(nodes, sbox, cr, l1, h1);
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(l0[k], l1[k]);
      hi[k] = fmaxf(h0[k], h1[k]);
      nodes[p].lo[k] = lo[k];
      nodes[p].hi[k] = hi[k];
    }
    const float a = fmaxf(half_area(lo, hi), 1e-30f);
    const float costL = cl >= 0 ? nodes[cl].cost : kCostPrim;
    const float costR = cr >= 0 ? nodes[cr].cost : kCostPrim;
    const float split = kCostNode + (half_area(l0, h0) * costL + half_area(l1, h1) * costR) / a;
    const int count = nodes[p].last - nodes[p].first + 1;
    const float leaf = kCostPrim * float(count);
    const bool canLeaf = count <= max_leaf;
    nodes[p].leafable = canLeaf && leaf <= split;
    nodes[p].cost = (canLeaf && leaf < split) ? leaf : split;
    p = nodes[p].parent;
  }
}

// ---- collapse into Node4 --------------------------------------------------
struct Task {
  int inner;  // binary inner node
  int node4;  // its 4-wide node
};

__device__ __forceinline__ int count_of(const Inner* nodes, int c) {
  return c >= 0 ? nodes[c].last - nodes[c].first + 1 : 1;
}
// A child ends in a leaf: a single primitive, or a subtree cheaper as a leaf.
__device__ __forceinline__ bool is_leaf(const Inner* nodes, int c) { return c < 0 || nodes[c].leafable; }
__device__ __forceinline__ float area_of(const Inner* nodes, int c) {
  const Inner& q = nodes[c];
  float dx = q.hi[0] - q.lo[0], dy = q.hi[1] - q.lo[1], dz = q.hi[2] - q.lo[2];
  return dx * dy + dy * dz + dz * dx;
}

__global__ void k_collapse(const Inner* __restrict__ nodes, const float* __restrict__ sbox,
                           const Task* __restrict__ in, const int* __restrict__ n_in, Task* __restrict__ out,
                           int* __restrict__ n_out, int* __restrict__ n_nodes, int capacity, float4* __restrict__ node4,
                           int max_leaf, unsigned long long* __restrict__ leaves, int* __restrict__ overflow) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= *n_in) return;
  const Task tk = in[q];
  int ch[4];
  int cnt = 2;
  ch[0] = nodes[tk.inner].left;
  ch[1] = nodes[tk.inner].right;
  while (cnt < 4) {
    int best = -1;
    float ba = -1.f;
    for (int c = 0; c < cnt; ++c) {
      if (!is_leaf(nodes, ch[c])) {
        float a = area_of(nodes, ch[c]);
        if (a > ba) { ba = a; best = c; }
      }
    }
    if (best < 0) break;
    int open = ch[best];
    ch[best] = nodes[open].left;
    ch[cnt++] = nodes[open].right;
  }
  float lo[3][4], hi[3][4];
  int ref[4];
  for (int s = 0; s < 4; ++s) {
    if (s < cnt) {
      float l[3], h[3];
      child_box(nodes, sbox, ch[s], l, h);
      for (int k = 0; k < 3; ++k) { lo[k][s] = l[k]; hi[k][s] = h[k]; }
      const int c = ch[s];
      const int count = count_of(nodes, c);
      if (is_leaf(nodes, c)) {
        const int first = c >= 0 ? nodes[c].first : ~c;
        ref[s] = ~((first << 4) | (count - 1));
        atomicAdd(leaves, 1ull);
      } else {
        int k4 = atomicAdd(n_nodes, 1);
        if (k4 >= capacity) {
          atomicExch(overflow, 1);
          ref[s] = kEmptyRef;
        } else {
          ref[s] = k4;
          int e = atomicAdd(n_out, 1);
          out[e] = Task{c, k4};
        }
      }
    } else {
      for (int k = 0; k < 3; ++k) { lo[k][s] = INFINITY; hi[k][s] = -INFINITY; }
      ref[s] = kEmptyRef;
    }
  }
  float4* nd = node4 + 8 * int64_t(tk.node4);
  nd[0] = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
  nd[1] = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
  nd[2] = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
  nd[3] = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
  nd[4] = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
  nd[5] = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
  nd[6] = make_float4(__int_as_float(ref[0]), __int_as_float(ref[1]), __int_as_float(ref[2]), __int_as_float(ref[3]));
  nd[7] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// A scene of at most max_leaf primitives: a root with one leaf.
__global__ void k_single_leaf(const float* __restrict__ sbox, int64_t n, float4* __restrict__ node4) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(lo[k], sbox[6 * i + k]);
      hi[k] = fmaxf(hi[k], sbox[6 * i + 3 + k]);
    }
  const float I = INFINITY;
  node4[0] = make_float4(lo[0], I, I, I);
  node4[1] = make_float4(hi[0], -I, -I, -I);
  node4[2] = make_float4(lo[1], I, I, I);
  node4[3] = make_float4(hi[1], -I, -I, -I);
  node4[4] = make_float4(lo[2], I, I, I);
  node4[5] = make_float4(hi[2], -I, -I, -I);
  const int ref = ~int(n - 1);
  node4[6] = make_float4(__int_as_float(ref), __int_as_float(kEmptyRef), __int_as_float(kEmptyRef),
                         __int_as_float(kEmptyRef));
  node4[7] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void k_gather_records(const float4* __restrict__ rin, const int4* __restrict__ min_,
                                 const unsigned* __restrict__ order, int64_t n, float4* __restrict__ rout,
                                 int4* __restrict__ mout) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s = order[i];
  rout[3 * i] = rin[3 * s];
  rout[3 * i + 1] = rin[3 * s + 1];
  rout[3 * i + 2] = rin[3 * s + 2];
  mout[i] = min_[s];
}

struct DevBuf {
  std::vector<void*> p;
  ~DevBuf() {
    for (void* x : p) cudaFree(x);
  }
  template <typename T>
  cudaError_t alloc(T** out, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) p.push_back(q);
    *out = static_cast<T*>(q);
    return e;
  }
};

}  // namespace

cudaError_t gpu_build_bvh4(const std::vector<Box>& boxes, int max_leaf, cudaStream_t stream, GpuBuild* out) {
  const int64_t n = int64_t(boxes.size());
  out->nodes = nullptr;
  out->order = nullptr;
  out->n_nodes = 0;
  out->depth4 = 0;
  out->leaves = 0;
  out->too_deep = false;
  if (n == 0) return cudaSuccess;
  if (n >= (int64_t(1) << 27)) {
    out->too_deep = true;  // leaf references hold 27 bits of record index
    return cudaSuccess;
  }
  DevBuf tmp;
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  float *d_box = nullptr, *d_sbox = nullptr;
  unsigned *k0 = nullptr, *v0 = nullptr, *k1 = nullptr, *v1 = nullptr, *zeros = nullptr, *bnd = nullptr;
  Inner* inner = nullptr;
  int *leaf_parent = nullptr, *visits = nullptr, *counters = nullptr;
  Task *t0 = nullptr, *t1 = nullptr;
  unsigned long long* leaves = nullptr;
  const int nt = int((n + kSortTile - 1) / kSortTile);
  A(tmp.alloc(&d_box, 6 * n));
  A(tmp.alloc(&d_sbox, 6 * n));
  A(tmp.alloc(&k0, n)); A(tmp.alloc(&v0, n)); A(tmp.alloc(&k1, n)); A(tmp.alloc(&v1, n));
  A(tmp.alloc(&zeros, nt + 1));
  A(tmp.alloc(&bnd, 6));
  A(tmp.alloc(&inner, std::max<int64_t>(n - 1, 1)));
  A(tmp.alloc(&leaf_parent, n));
  A(tmp.alloc(&visits, std::max<int64_t>(n - 1, 1)));
  A(tmp.alloc(&counters, 8));
  A(tmp.alloc(&t0, n)); A(tmp.alloc(&t1, n));
  A(tmp.alloc(&leaves, 1));
  if (e != cudaSuccess) return e;
  const int64_t cap = n;  // 4-wide nodes: at most one per inner binary node
  float4* node4 = nullptr;
  unsigned* order = nullptr;
  A(cudaMalloc(&node4, size_t(cap) * 8 * sizeof(float4)));
  A(cudaMalloc(&order, size_t(n) * sizeof(unsigned)));
  if (e != cudaSuccess) {
    cudaFree(node4);
    cudaFree(order);
    return e;
  }
  A(cudaMemcpyAsync(d_box, boxes.data(), size_t(n) * sizeof(Box), cudaMemcpyHostToDevice, stream));
  const unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  A(cudaMemcpyAsync(bnd, init, sizeof init, cudaMemcpyHostToDevice, stream));
  const unsigned blocks = unsigned((n + 255) / 256);
  k_centre_bounds<<<std::min(blocks, 1024u), 256, 0, stream>>>(d_box, n, bnd);
  k_morton<<<blocks, 256, 0, stream>>>(d_box, n, bnd, k0, v0);
  for (int bit = 0; bit < 30; ++bit) {
    k_split_count<<<nt, kSortThreads, 0, stream>>>(k0, n, bit, zeros);
    k_split_scan<<<1, 1024, 0, stream>>>(zeros, nt);
    k_split_scatter<<<nt, kSortThreads, 0, stream>>>(k0, v0, n, bit, zeros, nt, k1, v1);
    std::swap(k0, k1);
    std::swap(v0, v1);
  }
  A(cudaMemcpyAsync(order, v0, size_t(n) * sizeof(unsigned), cudaMemcpyDeviceToDevice, stream));
  k_gather_boxes<<<blocks, 256, 0, stream>>>(d_box, v0, n, d_sbox);
  A(cudaGetLastError());
  if (n <= max_leaf) {
    k_single_leaf<<<1, 1, 0, stream>>>(d_sbox, n, node4);
    A(cudaGetLastError());
    A(cudaStreamSynchronize(stream));
    if (e != cudaSuccess) {
      cudaFree(node4);
      cudaFree(order);
      return e;
    }
    out->nodes = node4;
    out->order = order;
    out->n_nodes = 1;
    out->depth4 = 1;
    out->leaves = 1;
    return cudaSuccess;
  }
  A(cudaMemsetAsync(visits, 0, size_t(n - 1) * sizeof(int), stream));
  k_radix_tree<<<unsigned((n - 1 + 255) / 256), 256, 0, stream>>>(k0, n, inner, leaf_parent);
  // counters: [0] 4-wide nodes, [1] tasks in, [2] tasks out, [3] overflow or malformed tree
  const int hc[4] = {1, 1, 0, 0};
  A(cudaMemcpyAsync(counters, hc, sizeof hc, cudaMemcpyHostToDevice, stream));
  k_inner_boxes<<<blocks, 256, 0, stream>>>(inner, d_sbox, leaf_parent, n, max_leaf, visits, counters + 3);
  A(cudaGetLastError());
  const Task root{0, 0};
  A(cudaMemcpyAsync(t0, &root, sizeof root, cudaMemcpyHostToDevice, stream));
  A(cudaMemsetAsync(leaves, 0, sizeof(unsigned long long), stream));
  int level = 0, n_in = 1;
  while (n_in > 0 && e == cudaSuccess) {
    if (level >= kGpuBuildMaxDepth4) {
      out->too_deep = true;
      break;
    }
    A(cudaMemsetAsync(counters + 2, 0, sizeof(int), stream));
    k_collapse<<<unsigned((n_in + 255) / 256), 256, 0, stream>>>(inner, d_sbox, t0, counters + 1, t1, counters + 2,
                                                                 counters, int(cap), node4, max_leaf, leaves,
                                                                 counters + 3);
    A(cudaGetLastError());
    A(cudaMemcpyAsync(counters + 1, counters + 2, sizeof(int), cudaMemcpyDeviceToDevice, stream));
    A(cudaMemcpyAsync(&n_in, counters + 2, sizeof(int), cudaMemcpyDeviceToHost, stream));
    A(cudaStreamSynchronize(stream));
    std::swap(t0, t1);
    ++level;
  }
  int hcount[4] = {0, 0, 0, 0};
  unsigned long long hl = 0;
  A(cudaMemcpyAsync(hcount, counters, sizeof hcount, cudaMemcpyDeviceToHost, stream));
  A(cudaMemcpyAsync(&hl, leaves, sizeof hl, cudaMemcpyDeviceToHost, stream));
  A(cudaStreamSynchronize(stream));
  if (e != cudaSuccess || out->too_deep || hcount[3]) {
    cudaFree(node4);
    cudaFree(order);
    if (hcount[3]) out->too_deep = true;
    return e;
  }
  out->nodes = node4;
  out->order = order;
  out->n_nodes = hcount[0];
  out->depth4 = level;
  out->leaves = int64_t(hl);
  return cudaSuccess;
}

cudaError_t gpu_gather_records(const float4* rin, const int4* min_, const unsigned* order, int64_t n, float4* rout,
                               int4* mout, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_gather_records<<<unsigned((n + 255) / 256), 256, 0, stream>>>(rin, min_, order, n, rout, mout);
  return cudaGetLastError();
}

}  // namespace gbrt
