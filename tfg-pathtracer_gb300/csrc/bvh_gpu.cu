// GPU BVH builder: linear BVH (Morton order) collapsed into the same 4-wide
// node format the host builder writes (bvh_build.cpp), for the
// `ER_BUILDER_GPU` scene option.
//
// The reference builds its BVH on the host (BVH.hpp:187-211, 291-460); the
// closest-hit result does not depend on the tree (candidates are ranked by
// the reference distance, exact ties by the tie key), so any tree will do.
// Steps, all on the device:
//  1. per triangle: bounds, centroid, shading-offset bound (as the host
//     builder computes it, in double), 63-bit Morton code of the centroid;
//  2. sort (code, index) pairs (CUB radix sort);
//  3. binary radix tree over the sorted codes (T. Karras, "Maximizing
//     parallelism in the construction of BVHs, octrees, and k-d trees",
//     HPG 2012), duplicate codes ordered by index;
//  4. bottom-up bounds, triangle counts and shading-offset maxima, the last
//     child to finish computing its parent;
//  4b. treelet restructuring (T. Karras and T. Aila, "Fast parallel
//     construction of high-quality bounding volume hierarchies", HPG 2013):
//     bottom-up again, each node grows a treelet of up to 7 leaves (opening
//     the largest-area internal leaf) and rebuilds it with the topology of
//     least SAH cost, found by dynamic programming over the leaf subsets;
//     three passes; then the triangles are renumbered into the tree's leaf
//     order so that every subtree is again a contiguous range;
//  5. top-down collapse, one launch per level: a binary node with more than
//     max_leaf triangles becomes a 4-wide node whose children are found by
//     repeatedly opening the largest-area internal child; a subtree with at
//     most max_leaf triangles becomes a leaf reference over its contiguous
//     range of sorted triangles;
//  6. the triangle arrays are gathered into leaf (sorted) order.
// Without step 4b such trees trace ~12 % slower than the host SAH tree.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "internal.h"

namespace er {
namespace {

struct BNode {            // binary radix-tree node
  float lo[3], hi[3];
  float delta;
  int32_t left, right;    // >= 0 internal node, < 0: ~leaf index
  int32_t first, last;    // sorted triangle range
  int32_t parent;
  int32_t count;
  float cost;             // SAH cost of the subtree (step 4b)
};

__device__ __forceinline__ uint64_t spread21(uint32_t v) {
  uint64_t x = v & 0x1FFFFFull;
  x = (x | x << 32) & 0x1F00000000FFFFull;
  x = (x | x << 16) & 0x1F0000FF0000FFull;
  x = (x | x << 8) & 0x100F00F00F00F00Full;
  x = (x | x << 4) & 0x10C30C30C30C30C3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

// Tri.hpp:74-92 bound on |shading position - geometric hit|, as bvh_build.cpp
__device__ double shading_bound_d(const float* p, const float* n) {
  double m = 0;
  for (int a = 0; a < 3; a++) {
    double nx = n[3 * a], ny = n[3 * a + 1], nz = n[3 * a + 2];
    double nn = sqrt(nx * nx + ny * ny + nz * nz);
    double mx = 0;
    for (int b = 0; b < 3; b++) {
      double dd = ((double)p[3 * b] - p[3 * a]) * nx + ((double)p[3 * b + 1] - p[3 * a + 1]) * ny +
                  ((double)p[3 * b + 2] - p[3 * a + 2]) * nz;
      mx = fmax(mx, fabs(dd));
    }
    m = fmax(m, nn * mx);
  }
  return m;
}

__global__ void k_tri_prep(const float* pos, const float* nrm, int64_t n, const float* scene_lo, const float* scene_ext,
                           uint64_t* codes, int32_t* idx, float* delta) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* p = pos + 9 * i;
  float c[3];
  for (int k = 0; k < 3; k++) {
    float lo = fminf(fminf(p[k], p[3 + k]), p[6 + k]), hi = fmaxf(fmaxf(p[k], p[3 + k]), p[6 + k]);
    c[k] = 0.5f * (lo + hi);
  }
  uint64_t code = 0;
  for (int k = 0; k < 3; k++) {
    float t = scene_ext[k] > 0.f ? (c[k] - scene_lo[k]) / scene_ext[k] : 0.f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    code |= spread21((uint32_t)(t * 2097151.0f)) << (2 - k);
  }
  codes[i] = code;
  idx[i] = (int32_t)i;
  double D = nrm ? shading_bound_d(p, nrm + 9 * i) : 0.0;
  delta[i] = D > 0 ? (float)(D * (1.0 + 1e-5)) : 0.0f;  // padded as the host builder
}

__device__ __forceinline__ int delta_k(const uint64_t* codes, int32_t n, int32_t i, int32_t j) {
  if (j < 0 || j >= n) return -1;
  uint64_t a = codes[i], b = codes[j];
  if (a == b) return 64 + __clz(i ^ j);
  return __clzll(a ^ b);
}

// Karras 2012: internal node i of the radix tree over n sorted keys
__global__ void k_radix_tree(const uint64_t* codes, int32_t n, BNode* nodes, int32_t* leaf_parent) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = delta_k(codes, n, i, i + 1) - delta_k(codes, n, i, i - 1) >= 0 ? 1 : -1;
  const int dmin = delta_k(codes, n, i, i - d);
  int32_t lmax = 2;
  while (delta_k(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
  int32_t l = 0;
  for (int32_t t = lmax / 2; t >= 1; t /= 2)
    if (delta_k(codes, n, i, i + (l + t) * d) > dmin) l += t;
  const int32_t j = i + l * d;
  const int dnode = delta_k(codes, n, i, j);
  int32_t s = 0;
  for (int32_t div = 2;; div *= 2) {
    int32_t t = (l + div - 1) / div;
    if (delta_k(codes, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
  }
  const int32_t g = i + s * d + min(d, 0);
  BNode& nd = nodes[i];
  nd.first = min(i, j);
  nd.last = max(i, j);
  nd.left = nd.first == g ? ~g : g;
  nd.right = nd.last == g + 1 ? ~(g + 1) : g + 1;
  if (nd.left < 0) leaf_parent[g] = i;
  else nodes[g].parent = i;
  if (nd.right < 0) leaf_parent[g + 1] = i;
  else nodes[g + 1].parent = i;
}

// Bottom-up: the second child to arrive computes its parent.
__global__ void k_bottom_up(const float* pos, const int32_t* sorted, const float* tdelta, int32_t n, BNode* nodes,
                            const int32_t* leaf_parent, int32_t* visits) {
  int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int32_t cur = leaf_parent[k];
  while (cur >= 0) {
    __threadfence();
    if (atomicAdd(&visits[cur], 1) == 0) return;  // the sibling finishes the node
    __threadfence();
    BNode& nd = nodes[cur];
    float lo[3], hi[3], dl = 0.f;
    int32_t cnt = 0;
    for (int k3 = 0; k3 < 3; k3++) { lo[k3] = INFINITY; hi[k3] = -INFINITY; }
    const int32_t ch[2] = {nd.left, nd.right};
    for (int c = 0; c < 2; c++) {
      if (ch[c] < 0) {
        const int32_t t = sorted[~ch[c]];
        const float* p = pos + 9 * (int64_t)t;
        for (int v = 0; v < 3; v++)
          for (int k3 = 0; k3 < 3; k3++) {
            lo[k3] = fminf(lo[k3], p[3 * v + k3]);
            hi[k3] = fmaxf(hi[k3], p[3 * v + k3]);
          }
        dl = fmaxf(dl, tdelta[t]);
        cnt += 1;
      } else {
        const BNode& cn = nodes[ch[c]];
        for (int k3 = 0; k3 < 3; k3++) {
          lo[k3] = fminf(lo[k3], ((volatile const float*)cn.lo)[k3]);
          hi[k3] = fmaxf(hi[k3], ((volatile const float*)cn.hi)[k3]);
        }
        dl = fmaxf(dl, *(volatile const float*)&cn.delta);
        cnt += *(volatile const int32_t*)&cn.count;
      }
    }
    for (int k3 = 0; k3 < 3; k3++) { nd.lo[k3] = lo[k3]; nd.hi[k3] = hi[k3]; }
    nd.delta = dl;
    nd.count = cnt;
    cur = nd.parent;
  }
}

__device__ __forceinline__ float area_of(const float* lo, const float* hi) {
  float x = hi[0] - lo[0], y = hi[1] - lo[1], z = hi[2] - lo[2];
  if (!(x >= 0.f) || !(y >= 0.f) || !(z >= 0.f)) return 0.f;
  return 2.f * (x * y + x * z + y * z);
}

// ------------------------------------------------------- treelets (4b) --

constexpr float kSahNode = 1.2f, kSahTri = 1.0f;  // as the host builder's SAH
constexpr int kTreelet = 7;                         // leaves per treelet

__device__ __forceinline__ void tri_box(const float* pos, const int32_t* sorted, int32_t leaf, float* lo, float* hi) {
  const float* p = pos + 9 * (int64_t)sorted[leaf];
  for (int k = 0; k < 3; k++) {
    lo[k] = fminf(fminf(p[k], p[3 + k]), p[6 + k]);
    hi[k] = fmaxf(fmaxf(p[k], p[3 + k]), p[6 + k]);
  }
}

// Bounds, count, delta and cost of a node or leaf as other threads left
// them (read through L2).
struct Sub {
  float lo[3], hi[3], delta, cost;
  int32_t count;
};
__device__ __forceinline__ Sub sub_of(const BNode* nodes, const float* pos, const int32_t* sorted, const float* tdelta,
                                      int32_t c) {
  Sub r;
  if (c < 0) {
    tri_box(pos, sorted, ~c, r.lo, r.hi);
    r.delta = tdelta[sorted[~c]];
    r.count = 1;
    r.cost = kSahTri * area_of(r.lo, r.hi);
  } else {
    const BNode* b = nodes + c;
    for (int k = 0; k < 3; k++) {
      r.lo[k] = __ldcg(&b->lo[k]);
      r.hi[k] = __ldcg(&b->hi[k]);
    }
    r.delta = __ldcg(&b->delta);
    r.count = __ldcg(&b->count);
    r.cost = __ldcg(&b->cost);
  }
  return r;
}

// Sets node nd from its two children (bounds, count, delta, cost).
__device__ __forceinline__ void refit(BNode* nodes, const float* pos, const int32_t* sorted, const float* tdelta,
                                      int32_t nd) {
  BNode& b = nodes[nd];
  const Sub l = sub_of(nodes, pos, sorted, tdelta, __ldcg(&b.left));
  const Sub r = sub_of(nodes, pos, sorted, tdelta, __ldcg(&b.right));
  for (int k = 0; k < 3; k++) {
    b.lo[k] = fminf(l.lo[k], r.lo[k]);
    b.hi[k] = fmaxf(l.hi[k], r.hi[k]);
  }
  b.delta = fmaxf(l.delta, r.delta);
  b.count = l.count + r.count;
  b.cost = kSahNode * area_of(b.lo, b.hi) + l.cost + r.cost;
}

// Bottom-up: the second child to arrive restructures the treelet rooted at
// its parent.  Everything below the root is final by then, and no other
// thread touches it again; the root keeps its place (and parent).
__global__ void k_treelets(const float* pos, const int32_t* sorted, const float* tdelta, int32_t n, BNode* nodes,
                           int32_t* leaf_parent, int32_t* visits, int32_t* err) {
  int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int32_t cur = leaf_parent[k];
  for (int32_t steps = 0; cur >= 0; steps++) {
    if (steps >= n || cur >= n - 1) {  // a walk longer than the tree: corrupt links
      atomicOr(err, 1);
      return;
    }
    __threadfence();
    if (atomicAdd(&visits[cur], 1) == 0) return;
    __threadfence();
    BNode* R = nodes + cur;
    // grow the treelet
    int32_t T[kTreelet], I[kTreelet - 1];
    int nt = 2, ni = 1;
    T[0] = __ldcg(&R->left);
    T[1] = __ldcg(&R->right);
    I[0] = cur;
    while (nt < kTreelet) {
      int pick = -1;
      float pa = -1.f;
      for (int j = 0; j < nt; j++) {
        if (T[j] < 0) continue;
        const Sub sj = sub_of(nodes, pos, sorted, tdelta, T[j]);
        const float a = area_of(sj.lo, sj.hi);
        if (a > pa) { pa = a; pick = j; }
      }
      if (pick < 0) break;
      const int32_t t = T[pick];
      I[ni++] = t;
      T[pick] = __ldcg(&nodes[t].left);
      T[nt++] = __ldcg(&nodes[t].right);
    }
    if (nt >= 3) {
      // least-cost topology over the treelet's leaves
      float tlo[kTreelet][3], thi[kTreelet][3], tc[kTreelet];
      for (int j = 0; j < nt; j++) {
        const Sub sj = sub_of(nodes, pos, sorted, tdelta, T[j]);
        for (int a = 0; a < 3; a++) { tlo[j][a] = sj.lo[a]; thi[j][a] = sj.hi[a]; }
        tc[j] = sj.cost;
      }
      float cost[1 << kTreelet];
      uint8_t part[1 << kTreelet];
      const int full = (1 << nt) - 1;
      for (int sset = 1; sset <= full; sset++) {
        if ((sset & (sset - 1)) == 0) {
          cost[sset] = tc[__ffs(sset) - 1];
          continue;
        }
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int j = 0; j < nt; j++)
          if (sset >> j & 1)
            for (int a = 0; a < 3; a++) { lo[a] = fminf(lo[a], tlo[j][a]); hi[a] = fmaxf(hi[a], thi[j][a]); }
        const int low = sset & -sset, rest = sset ^ low;
        float best = INFINITY;
        int bp = low;
        // partitions {low | q, rest \ q}, q a proper subset of rest
        for (int q = (rest - 1) & rest;; q = (q - 1) & rest) {
          const int pp = low | q;
          const float c = cost[pp] + cost[sset ^ pp];
          if (c < best) { best = c; bp = pp; }
          if (q == 0) break;
        }
        cost[sset] = kSahNode * area_of(lo, hi) + best;
        part[sset] = (uint8_t)bp;
      }
      // current cost of the treelet
      const Sub l0 = sub_of(nodes, pos, sorted, tdelta, __ldcg(&R->left));
      const Sub r0 = sub_of(nodes, pos, sorted, tdelta, __ldcg(&R->right));
      float rlo[3], rhi[3];
      for (int a = 0; a < 3; a++) { rlo[a] = fminf(l0.lo[a], r0.lo[a]); rhi[a] = fmaxf(l0.hi[a], r0.hi[a]); }
      const float now = kSahNode * area_of(rlo, rhi) + l0.cost + r0.cost;
      if (cost[full] < now * (1.0f - 1e-6f)) {
        // rebuild with the internal nodes I (I[0] = the root), parents first
        int32_t st_s[kTreelet], st_n[kTreelet];
        int sp = 0, used = 1;
        int32_t order[kTreelet - 1];
        int no = 0;
        st_s[sp] = full;
        st_n[sp++] = cur;
        while (sp > 0) {
          const int sset = st_s[--sp];
          const int32_t nd = st_n[sp];
          order[no++] = nd;
          const int sides[2] = {part[sset], sset ^ part[sset]};
          int32_t ch[2];
          for (int c = 0; c < 2; c++) {
            if ((sides[c] & (sides[c] - 1)) == 0) {
              ch[c] = T[__ffs(sides[c]) - 1];
            } else {
              ch[c] = I[used++];
              st_s[sp] = sides[c];
              st_n[sp++] = ch[c];
            }
            if (ch[c] >= 0) nodes[ch[c]].parent = nd;
            else leaf_parent[~ch[c]] = nd;
          }
          nodes[nd].left = ch[0];
          nodes[nd].right = ch[1];
        }
        // children before parents
        for (int o = no - 1; o >= 0; o--) refit(nodes, pos, sorted, tdelta, order[o]);
      } else {
        R->cost = now;
      }
    } else {
      refit(nodes, pos, sorted, tdelta, cur);
    }
    cur = __ldcg(&R->parent);
  }
}

// Position of leaf k in the tree's left-to-right leaf order.
__global__ void k_leaf_order(const BNode* nodes, const int32_t* leaf_parent, int32_t n, int32_t* pos_of, int32_t* err) {
  int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int32_t child = ~k, nd = leaf_parent[k], p = 0;
  for (int32_t steps = 0; nd >= 0; steps++) {
    if (steps >= n || nd >= n - 1) {
      atomicOr(err, 2);
      pos_of[k] = k;
      return;
    }
    const BNode& b = nodes[nd];
    if (b.right == child) p += b.left < 0 ? 1 : nodes[b.left].count;
    child = nd;
    nd = b.parent;
  }
  pos_of[k] = p;
}

// Renumbers leaves to their positions: triangle order, leaf references,
// first / last of every internal node.
__global__ void k_renumber_leaves(const int32_t* sorted, const int32_t* pos_of, int32_t n, int32_t* sorted2) {
  int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) sorted2[pos_of[k]] = sorted[k];
}
__global__ void k_renumber_nodes(BNode* nodes, const int32_t* pos_of, int32_t n_int) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_int) return;
  BNode& b = nodes[i];
  if (b.left < 0) b.left = ~pos_of[~b.left];
  if (b.right < 0) b.right = ~pos_of[~b.right];
}
__global__ void k_node_ranges(BNode* nodes, const int32_t* pos_of, int32_t n_int, int32_t* err) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_int) return;
  // leftmost leaf (references already renumbered by the previous launch)
  int32_t c = i;
  for (int32_t steps = 0; c >= 0; steps++) {
    if (steps > n_int || c >= n_int) {
      atomicOr(err, 4);
      return;
    }
    c = nodes[c].left;
  }
  nodes[i].first = ~c;
  nodes[i].last = ~c + nodes[i].count - 1;
}

struct Item {
  int32_t bnode;   // binary node to expand into a 4-wide node
  int32_t out;     // its 4-wide node index
};


// Child c (>= 0 internal, < 0 ~leaf) bounds / count / delta / range
__device__ __forceinline__ void child_info(const BNode* nodes, const float* pos, const int32_t* sorted,
                                           const float* tdelta, int32_t c, float* lo, float* hi, float* dl,
                                           int32_t* cnt, int32_t* first) {
  if (c >= 0) {
    const BNode& b = nodes[c];
    for (int k = 0; k < 3; k++) { lo[k] = b.lo[k]; hi[k] = b.hi[k]; }
    *dl = b.delta;
    *cnt = b.count;
    *first = b.first;
  } else {
    const int32_t t = sorted[~c];
    const float* p = pos + 9 * (int64_t)t;
    for (int k = 0; k < 3; k++) {
      lo[k] = fminf(fminf(p[k], p[3 + k]), p[6 + k]);
      hi[k] = fmaxf(fmaxf(p[k], p[3 + k]), p[6 + k]);
    }
    *dl = tdelta[t];
    *cnt = 1;
    *first = ~c;
  }
}

__global__ void k_collapse(const BNode* nodes, const float* pos, const int32_t* sorted, const float* tdelta,
                           const Item* items, int32_t n_items, Item* next, int32_t* n_next, int32_t* n_out,
                           float* out_nodes, int32_t max_leaf, int32_t* leaf_count) {
  int32_t it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= n_items) return;
  const Item I = items[it];
  int32_t ch[4];
  int32_t nc = 0;
  const BNode& root = nodes[I.bnode];
  ch[nc++] = root.left;
  ch[nc++] = root.right;
  while (nc < 4) {
    int pick = -1;
    float pa = -1.f;
    for (int k = 0; k < nc; k++) {
      if (ch[k] < 0) continue;
      const BNode& b = nodes[ch[k]];
      if (b.count <= max_leaf) continue;
      float a = area_of(b.lo, b.hi);
      if (a > pa) { pa = a; pick = k; }
    }
    if (pick < 0) break;
    const BNode& b = nodes[ch[pick]];
    for (int k = nc; k > pick + 1; k--) ch[k] = ch[k - 1];
    ch[pick] = b.left;
    ch[pick + 1] = b.right;
    nc++;
  }
  float* nd = out_nodes + 32 * (int64_t)I.out;
  for (int s = 0; s < 4; s++) {
    int32_t ref = kEmpty;
    // an empty slot keeps an inverted box (lo = +inf, hi = -inf)
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}, dl = 0.f;
    if (s < nc) {
      int32_t cnt, first;
      child_info(nodes, pos, sorted, tdelta, ch[s], lo, hi, &dl, &cnt, &first);
      if (cnt <= max_leaf) {
        ref = (int32_t)(kLeafBit | ((uint32_t)(cnt - 1) << kLeafCountShift) | (uint32_t)first);
        atomicAdd(leaf_count, 1);
      } else {
        ref = atomicAdd(n_out, 1);
        next[atomicAdd(n_next, 1)] = Item{ch[s], ref};
      }
    }
    nd[0 + s] = lo[0];
    nd[4 + s] = hi[0];
    nd[8 + s] = lo[1];
    nd[12 + s] = hi[1];
    nd[16 + s] = lo[2];
    nd[20 + s] = hi[2];
    nd[24 + s] = __int_as_float(ref);
    nd[28 + s] = dl;
  }
}

// leaf-order triangle data (as scene.cpp lays it out on the host)
__global__ void k_gather(const int32_t* sorted, int64_t n, const float* pos, const float* nrm, const float* uv,
                         const float* tan, const float* tsign, const int32_t* tri_obj, const int32_t* obj_mat,
                         const uint32_t* tie, float4* tv, float4* tn, float2* tuv, float4* tt) {
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int32_t i = sorted[s];
  const int32_t obj = tri_obj ? tri_obj[i] : 0;
  const int32_t mat = obj_mat ? obj_mat[obj] : 0;
  const uint32_t key = tie ? tie[i] : (uint32_t)i;
  const float w[3] = {__int_as_float(i), __uint_as_float(key), __int_as_float(mat)};
  const float ts = tsign ? tsign[i] : 1.0f;
  for (int k = 0; k < 3; k++) {
    const float* p = pos + 9 * (int64_t)i + 3 * k;
    tv[3 * s + k] = make_float4(p[0], p[1], p[2], w[k]);
    if (nrm) {
      const float* q = nrm + 9 * (int64_t)i + 3 * k;
      tn[3 * s + k] = make_float4(q[0], q[1], q[2], k == 0 ? ts : 0.0f);
    } else {
      tn[3 * s + k] = make_float4(0.f, 0.f, 0.f, k == 0 ? ts : 0.0f);
    }
    tuv[3 * s + k] = uv ? make_float2(uv[6 * (int64_t)i + 2 * k], uv[6 * (int64_t)i + 2 * k + 1]) : make_float2(0.f, 0.f);
    if (tt) {
      const float* g = tan + 9 * (int64_t)i + 3 * k;
      tt[3 * s + k] = make_float4(g[0], g[1], g[2], 0.f);
    }
  }
}

struct Scratch {
  std::vector<void*> p;
  ~Scratch() {
    for (void* q : p) cudaFree(q);
  }
  er_status get(void** out, size_t bytes) {
    cudaError_t e = cudaMalloc(out, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ER_ERR_OOM, "GPU BVH build buffers");
    }
    p.push_back(*out);
    return ER_OK;
  }
  template <typename T>
  er_status put(const T** out, const T* host, size_t count, cudaStream_t st) {
    *out = nullptr;
    if (!host) return ER_OK;
    void* p = nullptr;
    er_status s = get(&p, count * sizeof(T));
    if (s != ER_OK) return s;
    ER_CUDA(cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, st));
    *out = (const T*)p;
    return ER_OK;
  }
};

}  // namespace

er_status build_bvh_gpu(er_scene* s, const er_scene_desc* d, int max_leaf, const float scene_lo[3],
                        const float scene_hi[3], GpuBvh* out) {
  const int64_t T = d->tri_count;
  cudaStream_t st = s->stream;
  max_leaf = std::min(std::max(max_leaf, 1), 8);
  Scratch X;
  er_status e;
  // raw triangle data on the device
  const float *pos, *nrm, *uv, *tan, *tsign;
  const int32_t *tobj, *omat;
  const uint32_t* tie;
  if ((e = X.put(&pos, d->positions, (size_t)(9 * T), st)) != ER_OK) return e;
  if ((e = X.put(&nrm, d->normals, (size_t)(9 * T), st)) != ER_OK) return e;
  if ((e = X.put(&uv, d->uvs, (size_t)(6 * T), st)) != ER_OK) return e;
  if ((e = X.put(&tan, d->tangents, (size_t)(9 * T), st)) != ER_OK) return e;
  if ((e = X.put(&tsign, d->tangent_sign, (size_t)T, st)) != ER_OK) return e;
  if ((e = X.put(&tobj, d->tri_object, (size_t)T, st)) != ER_OK) return e;
  // no objects: every triangle takes material 0, as on the host builder
  if ((e = X.put(&omat, d->object_count > 0 ? d->object_material : nullptr, (size_t)std::max(d->object_count, 0),
                 st)) != ER_OK)
    return e;
  if ((e = X.put(&tie, d->tie_key, (size_t)T, st)) != ER_OK) return e;
  float hb[6] = {scene_lo[0], scene_lo[1], scene_lo[2], scene_hi[0] - scene_lo[0], scene_hi[1] - scene_lo[1],
                 scene_hi[2] - scene_lo[2]};
  const float* d_box;
  if ((e = X.put(&d_box, hb, 6, st)) != ER_OK) return e;

  auto t0 = std::chrono::steady_clock::now();
  const unsigned tb = (unsigned)((T + 255) / 256);
  uint64_t *codes, *codes2;
  int32_t *idx, *sorted;
  float* tdelta;
  if ((e = X.get((void**)&codes, (size_t)T * 8)) != ER_OK) return e;
  if ((e = X.get((void**)&codes2, (size_t)T * 8)) != ER_OK) return e;
  if ((e = X.get((void**)&idx, (size_t)T * 4)) != ER_OK) return e;
  if ((e = X.get((void**)&sorted, (size_t)T * 4)) != ER_OK) return e;
  if ((e = X.get((void**)&tdelta, (size_t)T * 4)) != ER_OK) return e;
  k_tri_prep<<<tb, 256, 0, st>>>(pos, nrm, T, d_box, d_box + 3, codes, idx, tdelta);
  size_t temp_bytes = 0;
  ER_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, codes, codes2, idx, sorted, (int)T, 0, 63, st));
  void* temp;
  if ((e = X.get(&temp, temp_bytes)) != ER_OK) return e;
  ER_CUDA(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, codes, codes2, idx, sorted, (int)T, 0, 63, st));

  // radix tree + bottom-up (a single triangle is a one-leaf root)
  const int32_t n = (int32_t)T;
  BNode* bn;
  int32_t *leaf_parent, *visits;
  if ((e = X.get((void**)&bn, (size_t)std::max(n - 1, 1) * sizeof(BNode))) != ER_OK) return e;
  if ((e = X.get((void**)&leaf_parent, (size_t)n * 4)) != ER_OK) return e;
  if ((e = X.get((void**)&visits, (size_t)std::max(n - 1, 1) * 4)) != ER_OK) return e;
  ER_CUDA(cudaMemsetAsync(visits, 0, (size_t)std::max(n - 1, 1) * 4, st));
  ER_CUDA(cudaMemsetAsync(leaf_parent, 0xFF, (size_t)n * 4, st));
  if (n > 1) {
    // the root has no parent
    int32_t m1 = -1;
    ER_CUDA(cudaMemcpyAsync(&bn[0].parent, &m1, 4, cudaMemcpyHostToDevice, st));
    k_radix_tree<<<(unsigned)((n - 1 + 255) / 256), 256, 0, st>>>(codes2, n, bn, leaf_parent);
    k_bottom_up<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pos, sorted, tdelta, n, bn, leaf_parent, visits);
  }
  ER_CUDA(cudaGetLastError());
  if (n > 2) {
    // treelet restructuring, then triangles renumbered into leaf order
    int32_t *pos_of, *sorted2, *terr;
    if ((e = X.get((void**)&pos_of, (size_t)n * 4)) != ER_OK) return e;
    if ((e = X.get((void**)&sorted2, (size_t)n * 4)) != ER_OK) return e;
    if ((e = X.get((void**)&terr, 4)) != ER_OK) return e;
    ER_CUDA(cudaMemsetAsync(terr, 0, 4, st));
    for (int pass = 0; pass < 3; pass++) {
      ER_CUDA(cudaMemsetAsync(visits, 0, (size_t)(n - 1) * 4, st));
      k_treelets<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(pos, sorted, tdelta, n, bn, leaf_parent, visits, terr);
    }
    const unsigned gb = (unsigned)((n + 255) / 256);
    k_leaf_order<<<gb, 256, 0, st>>>(bn, leaf_parent, n, pos_of, terr);
    k_renumber_leaves<<<gb, 256, 0, st>>>(sorted, pos_of, n, sorted2);
    k_renumber_nodes<<<gb, 256, 0, st>>>(bn, pos_of, n - 1);
    k_node_ranges<<<gb, 256, 0, st>>>(bn, pos_of, n - 1, terr);
    ER_CUDA(cudaGetLastError());
    int32_t herr = 0;
    ER_CUDA(cudaMemcpyAsync(&herr, terr, 4, cudaMemcpyDeviceToHost, st));
    ER_CUDA(cudaStreamSynchronize(st));
    if (herr) return fail(ER_ERR_DEVICE_CHECK, "GPU BVH treelet pass: corrupt tree links (" + std::to_string(herr) + ")");
    sorted = sorted2;
  }

  // top-down collapse into 4-wide nodes, one launch per level
  float* nodes4;
  Item *qa, *qb;
  int32_t* counters;  // [0] next items [1] nodes [2] leaves
  const size_t max_nodes = (size_t)std::max<int64_t>(T, 1);
  if ((e = X.get((void**)&nodes4, max_nodes * 128)) != ER_OK) return e;
  if ((e = X.get((void**)&qa, max_nodes * sizeof(Item))) != ER_OK) return e;
  if ((e = X.get((void**)&qb, max_nodes * sizeof(Item))) != ER_OK) return e;
  if ((e = X.get((void**)&counters, 16)) != ER_OK) return e;
  int32_t node_count = 1, leaves = 0, depth = 1;
  if (n <= max_leaf) {
    // a root with a single leaf child (or, with no triangles, no child)
    std::vector<float> root(32, 0.0f);
    int32_t ref = n > 0 ? (int32_t)(kLeafBit | ((uint32_t)(n - 1) << kLeafCountShift)) : kEmpty;
    float lo[3] = {scene_lo[0], scene_lo[1], scene_lo[2]}, hi[3] = {scene_hi[0], scene_hi[1], scene_hi[2]};
    for (int sl = 0; sl < 4; sl++) {
      int32_t r = sl == 0 ? ref : kEmpty;
      std::memcpy(&root[24 + sl], &r, 4);
      if (r == kEmpty)
        for (int k = 0; k < 3; k++) {
          root[4 * 2 * k + sl] = INFINITY;         // inverted box of an empty slot
          root[4 * (2 * k + 1) + sl] = -INFINITY;
        }
    }
    if (n > 0) {
      for (int k = 0; k < 3; k++) { root[4 * 2 * k] = lo[k]; root[4 * (2 * k + 1)] = hi[k]; }
      std::vector<float> td((size_t)n);
      ER_CUDA(cudaMemcpyAsync(td.data(), tdelta, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
      ER_CUDA(cudaStreamSynchronize(st));
      float m = 0;
      for (float v : td) m = std::max(m, v);
      root[28] = m;
      leaves = 1;
    }
    ER_CUDA(cudaMemcpyAsync(nodes4, root.data(), 128, cudaMemcpyHostToDevice, st));
  } else {
    Item first{0, 0};
    ER_CUDA(cudaMemcpyAsync(qa, &first, sizeof first, cudaMemcpyHostToDevice, st));
    int32_t init[3] = {0, 1, 0};
    ER_CUDA(cudaMemcpyAsync(counters, init, 12, cudaMemcpyHostToDevice, st));
    int32_t n_items = 1;
    depth = 0;
    while (n_items > 0) {
      depth++;
      ER_CUDA(cudaMemsetAsync(counters, 0, 4, st));
      k_collapse<<<(unsigned)((n_items + 127) / 128), 128, 0, st>>>(bn, pos, sorted, tdelta, qa, n_items, qb, counters,
                                                                      counters + 1, nodes4, max_leaf, counters + 2);
      ER_CUDA(cudaGetLastError());
      int32_t c[3];
      ER_CUDA(cudaMemcpyAsync(c, counters, 12, cudaMemcpyDeviceToHost, st));
      ER_CUDA(cudaStreamSynchronize(st));
      n_items = c[0];
      node_count = c[1];
      leaves = c[2];
      std::swap(qa, qb);
    }
  }
  // outputs owned by the scene
  void *p_nodes, *p_tv, *p_tn, *p_tuv, *p_tt = nullptr;
  const size_t slots = (size_t)std::max<int64_t>(T, 1);
  if ((e = dev_alloc(s, &p_nodes, (size_t)node_count * 128)) != ER_OK) return e;
  ER_CUDA(cudaMemcpyAsync(p_nodes, nodes4, (size_t)node_count * 128, cudaMemcpyDeviceToDevice, st));
  if ((e = dev_alloc(s, &p_tv, slots * 48)) != ER_OK) return e;
  if ((e = dev_alloc(s, &p_tn, slots * 48)) != ER_OK) return e;
  if ((e = dev_alloc(s, &p_tuv, slots * 24)) != ER_OK) return e;
  if (d->tangents && (e = dev_alloc(s, &p_tt, slots * 48)) != ER_OK) return e;
  if (T > 0)
    k_gather<<<tb, 256, 0, st>>>(sorted, T, pos, nrm, uv, tan, tsign, tobj, omat, tie, (float4*)p_tv, (float4*)p_tn,
                                 (float2*)p_tuv, (float4*)p_tt);
  ER_CUDA(cudaGetLastError());
  ER_CUDA(cudaStreamSynchronize(st));
  auto t1 = std::chrono::steady_clock::now();
  float maxd = 0;
  if (T > 0) {
    std::vector<float> td((size_t)T);
    ER_CUDA(cudaMemcpy(td.data(), tdelta, (size_t)T * 4, cudaMemcpyDeviceToHost));
    for (float v : td) maxd = std::max(maxd, v);
  }
  out->nodes = (const float4*)p_nodes;
  out->tri_v = (const float4*)p_tv;
  out->tri_n = (const float4*)p_tn;
  out->tri_uv = (const float2*)p_tuv;
  out->tri_t = (const float4*)p_tt;
  out->node_count = node_count;
  out->leaf_count = leaves;
  out->depth = depth;
  out->max_delta = maxd;
  out->build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  return ER_OK;
}

}  // namespace er
