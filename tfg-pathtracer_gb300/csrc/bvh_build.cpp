// Host SAH BVH builder: binned-SAH binary tree collapsed into a 4-wide tree
// with 128-byte FP32 nodes (each node's children picked by an SAH-optimal
// dynamic programme over the binary tree), plus the 8-bit quantised form of
// the same topology.
//
// The reference builds a fixed-depth (18) binary tree with 14 SAH bins and
// no leaf cost (BVH.hpp:291-460); closest-hit results do not depend on the
// tree (all candidate triangles are ranked by the reference distance, and
// exact ties by the tie key), so this builder is free to pick a shape that
// traverses well on the GPU.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>

#include "internal.h"

namespace er {
namespace {

struct Box {
  float lo[3], hi[3];
  void reset() {
    for (int k = 0; k < 3; k++) { lo[k] = INFINITY; hi[k] = -INFINITY; }
  }
  void grow(const Box& b) {
    for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
  }
  void grow_pt(const float* p) {
    for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
  }
  double area() const {
    double x = (double)hi[0] - lo[0], y = (double)hi[1] - lo[1], z = (double)hi[2] - lo[2];
    if (!(x >= 0) || !(y >= 0) || !(z >= 0)) return 0;
    return 2.0 * (x * y + x * z + y * z);
  }
};

struct Node2 {
  Box box;
  int32_t left = -1, right = -1;
  int32_t first = 0, count = 0;  // leaf range in the order array
  float delta = 0;
};

constexpr int kBins = 32;
// Binary depth from which nodes are halved at the median instead of by SAH
// (the 1080p 1.18M-triangle scene's SAH tree is 25 deep).
constexpr int32_t kMedianDepth = 48;

// Cost of a triangle test against a 4-wide node visit in the collapse's SAH.
// Measured on the 1.18M-triangle 1080p scene (traversal ms per sample):
// 0.15 -> 6.75, 0.2 -> 6.59, 0.3 -> 6.42, 0.5 -> 6.285, 1.0 -> 6.285;
// the greedy collapse (open the largest child) 6.38.  Below 0.5 the
// programme merges small subtrees into larger leaves, and the extra
// triangle tests cost more than the node visits they save.
constexpr double kTriCost = 1.0;

struct Builder {
  const er_scene_desc* d;
  int max_leaf;
  std::vector<Box> tbox;
  std::vector<float> cent;  // 3 per triangle
  std::vector<float> tdelta;
  std::vector<int32_t> idx;
  std::vector<Node2> nodes;
  int32_t max_depth = 0;

  int32_t build() {
    struct Task { int32_t node, b, e, depth; };
    std::vector<Task> stack;
    nodes.reserve((size_t)(2 * idx.size() / std::max(1, max_leaf) + 16));
    nodes.push_back(Node2());
    stack.push_back({0, 0, (int32_t)idx.size(), 0});
    while (!stack.empty()) {
      Task t = stack.back();
      stack.pop_back();
      max_depth = std::max(max_depth, t.depth);
      Box nb, cb;
      nb.reset();
      cb.reset();
      float dl = 0;
      for (int32_t i = t.b; i < t.e; i++) {
        nb.grow(tbox[idx[i]]);
        cb.grow_pt(&cent[3 * (size_t)idx[i]]);
        dl = std::max(dl, tdelta[idx[i]]);
      }
      int32_t n = t.e - t.b;
      nodes[t.node].box = nb;
      nodes[t.node].delta = dl;
      int32_t mid = -1;
      if (n > max_leaf && t.depth >= kMedianDepth) {
        mid = median_split(t.b, t.e, cb);
      } else if (n > max_leaf) {
        mid = split(t.b, t.e, nb, cb, n <= kMaxLeafTris);
      }
      if (mid < 0) {
        nodes[t.node].first = t.b;
        nodes[t.node].count = n;
        continue;
      }
      int32_t l = (int32_t)nodes.size();
      nodes.push_back(Node2());
      nodes.push_back(Node2());
      nodes[t.node].left = l;
      nodes[t.node].right = l + 1;
      stack.push_back({l + 1, mid, t.e, t.depth + 1});
      stack.push_back({l, t.b, mid, t.depth + 1});
    }
    return 0;
  }

  // Halves [b, e) at the centroid median of its widest axis.  Used below
  // depth kMedianDepth, which bounds the tree's depth (and the recursion of
  // the collapse) by kMedianDepth + log2(triangles) for any input.
  int32_t median_split(int32_t b, int32_t e, const Box& cb) {
    int a = 0;
    for (int k = 1; k < 3; k++)
      if (cb.hi[k] - cb.lo[k] > cb.hi[a] - cb.lo[a]) a = k;
    const int32_t mid = b + (e - b) / 2;
    std::nth_element(idx.begin() + b, idx.begin() + mid, idx.begin() + e,
                     [&](int32_t x, int32_t y) { return cent[3 * (size_t)x + a] < cent[3 * (size_t)y + a]; });
    return mid;
  }

  // Binned SAH; returns the partition point or -1 for "make a leaf".
  int32_t split(int32_t b, int32_t e, const Box& nb, const Box& cb, bool may_leaf) {
    int32_t n = e - b;
    double best = INFINITY;
    int best_axis = -1, best_bin = -1;
    for (int a = 0; a < 3; a++) {
      float ext = cb.hi[a] - cb.lo[a];
      if (!(ext > 0)) continue;
      Box bb[kBins];
      int cnt[kBins] = {0};
      for (int k = 0; k < kBins; k++) bb[k].reset();
      float sc = (float)kBins / ext;
      for (int32_t i = b; i < e; i++) {
        int32_t t = idx[i];
        int k = (int)((cent[3 * (size_t)t + a] - cb.lo[a]) * sc);
        k = std::min(std::max(k, 0), kBins - 1);
        cnt[k]++;
        bb[k].grow(tbox[t]);
      }
      double ra[kBins];
      int rc[kBins];
      Box acc;
      acc.reset();
      int c = 0;
      for (int k = kBins - 1; k > 0; k--) {
        acc.grow(bb[k]);
        c += cnt[k];
        ra[k] = acc.area();
        rc[k] = c;
      }
      acc.reset();
      c = 0;
      for (int k = 0; k < kBins - 1; k++) {
        acc.grow(bb[k]);
        c += cnt[k];
        if (c == 0 || rc[k + 1] == 0) continue;
        double cost = acc.area() * c + ra[k + 1] * rc[k + 1];
        if (cost < best) { best = cost; best_axis = a; best_bin = k; }
      }
    }
    double leaf_cost = nb.area() * n;
    const double trav = 1.2;  // node traversal vs triangle test cost ratio
    if (best_axis >= 0 && may_leaf && trav * nb.area() + best >= leaf_cost) return -1;
    if (best_axis < 0) {
      if (may_leaf) return -1;
      return b + n / 2;  // all centroids coincide: split by count
    }
    float ext = cb.hi[best_axis] - cb.lo[best_axis];
    float sc = (float)kBins / ext;
    auto it = std::partition(idx.begin() + b, idx.begin() + e, [&](int32_t t) {
      int k = (int)((cent[3 * (size_t)t + best_axis] - cb.lo[best_axis]) * sc);
      k = std::min(std::max(k, 0), kBins - 1);
      return k <= best_bin;
    });
    int32_t mid = (int32_t)(it - idx.begin());
    if (mid == b || mid == e) return b + n / 2;
    return mid;
  }
};

void put_child(float* nd, int slot, const Box& bx, int32_t child, float delta) {
  nd[0 + slot] = bx.lo[0];
  nd[4 + slot] = bx.hi[0];
  nd[8 + slot] = bx.lo[1];
  nd[12 + slot] = bx.hi[1];
  nd[16 + slot] = bx.lo[2];
  nd[20 + slot] = bx.hi[2];
  std::memcpy(&nd[24 + slot], &child, 4);
  nd[28 + slot] = delta;
}

}  // namespace

double shading_offset_bound(const er_scene_desc* d, int64_t i) {
  if (!d->normals) return 0.0;
  const float* p = d->positions + 9 * i;
  const float* n = d->normals + 9 * i;
  double m = 0;
  for (int a = 0; a < 3; a++) {
    double nn = std::sqrt((double)n[3 * a] * n[3 * a] + (double)n[3 * a + 1] * n[3 * a + 1] +
                          (double)n[3 * a + 2] * n[3 * a + 2]);
    double mx = 0;
    for (int b = 0; b < 3; b++) {
      double dd = 0;
      for (int k = 0; k < 3; k++) dd += ((double)p[3 * b + k] - p[3 * a + k]) * n[3 * a + k];
      mx = std::max(mx, std::fabs(dd));
    }
    m = std::max(m, nn * mx);
  }
  return m;
}

er_status build_bvh4(const er_scene_desc* d, int max_leaf, BuildResult* out) {
  Builder B;
  B.d = d;
  B.max_leaf = std::min(std::max(max_leaf, 1), 8);
  int64_t T = d->tri_count;
  B.tbox.resize((size_t)T);
  B.cent.resize((size_t)(3 * T));
  B.tdelta.resize((size_t)T);
  B.idx.resize((size_t)T);
  for (int64_t i = 0; i < T; i++) {
    Box bx;
    bx.reset();
    for (int v = 0; v < 3; v++) bx.grow_pt(d->positions + 9 * i + 3 * v);
    B.tbox[i] = bx;
    for (int k = 0; k < 3; k++) B.cent[3 * i + k] = 0.5f * (bx.lo[k] + bx.hi[k]);
    double D = shading_offset_bound(d, i);
    // Rounded up and padded: the kernel compares against float distances.
    B.tdelta[i] = D > 0 ? (float)(D * (1.0 + 1e-5)) : 0.0f;
    B.idx[i] = (int32_t)i;
  }
  if (T == 0) {
    out->nodes.assign(32, 0.0f);
    Box z;
    z.reset();  // inverted: lo = +inf, hi = -inf
    for (int s = 0; s < 4; s++) put_child(out->nodes.data(), s, z, kEmpty, 0.0f);
    out->node_count = 1;
    out->leaf_count = 0;
    out->depth = 1;
    return ER_OK;
  }
  B.build();

  // Collapse to 4-wide.
  std::vector<float>& N4 = out->nodes;
  N4.clear();
  int64_t leaves = 0;
  int32_t depth4 = 0;
  float maxd = 0;
  // SAH-optimal collapse (the dynamic programme of Ylitie, Karras and Laine,
  // HPG 2017, for 4 slots).  F[n][j]: least SAH cost of covering binary
  // subtree n with at most j child slots of one 4-wide node; a slot holds a
  // leaf (the subtree's contiguous leaf range, at most kMaxLeafTris
  // triangles) or a 4-wide node of its own, which costs one node visit times
  // its area plus its slots.  Children are created after their parent, so a
  // reverse sweep sees them first.
  const size_t nb = B.nodes.size();
  const double c_node = 1.0, c_tri = kTriCost;
  std::vector<int32_t> cnt(nb), first(nb);
  std::vector<double> area(nb), tc(nb);
  std::vector<std::array<double, 5>> F(nb);
  std::vector<std::array<int8_t, 5>> Fk(nb);  // slots given to the left child, 0 = n itself
  std::vector<int8_t> as_leaf(nb), k4(nb);
  for (size_t i = nb; i-- > 0;) {
    const Node2& x = B.nodes[i];
    area[i] = x.box.area();
    if (x.left < 0) {
      cnt[i] = x.count;
      first[i] = x.first;
    } else {
      cnt[i] = cnt[x.left] + cnt[x.right];
      first[i] = first[x.left];
    }
    const double leafc = cnt[i] <= kMaxLeafTris ? area[i] * cnt[i] * c_tri : INFINITY;
    double intc = INFINITY;
    int kb = 0;
    if (x.left >= 0) {
      for (int k = 1; k <= 3; k++) {
        double c = F[x.left][k] + F[x.right][4 - k];
        if (c < intc) { intc = c; kb = k; }
      }
      intc += area[i] * c_node;
    }
    as_leaf[i] = leafc <= intc;
    k4[i] = (int8_t)kb;
    tc[i] = std::min(leafc, intc);
    for (int j = 1; j <= 4; j++) {
      F[i][j] = tc[i];
      Fk[i][j] = 0;
      if (x.left < 0) continue;
      for (int k = 1; k < j; k++) {
        double c = F[x.left][k] + F[x.right][j - k];
        if (c < F[i][j]) { F[i][j] = c; Fk[i][j] = (int8_t)k; }
      }
    }
  }
  std::function<void(int32_t, int, std::vector<int32_t>&)> cut = [&](int32_t n, int j, std::vector<int32_t>& o) {
    const int k = Fk[n][j];
    if (k == 0) {
      o.push_back(n);
      return;
    }
    cut(B.nodes[n].left, k, o);
    cut(B.nodes[n].right, j - k, o);
  };
  std::function<int32_t(int32_t, int32_t)> emit = [&](int32_t n2, int32_t dep) -> int32_t {
    depth4 = std::max(depth4, dep);
    std::vector<int32_t> ch;
    if (as_leaf[n2] || B.nodes[n2].left < 0) {
      ch.push_back(n2);  // the root as one leaf child
    } else {
      cut(B.nodes[n2].left, k4[n2], ch);
      cut(B.nodes[n2].right, 4 - k4[n2], ch);
    }
    int32_t me = (int32_t)(N4.size() / 32);
    N4.resize(N4.size() + 32, 0.0f);
    int32_t refs[4];
    for (size_t k = 0; k < ch.size(); k++) {
      const int32_t c = ch[k];
      if (as_leaf[c] || B.nodes[c].left < 0 || (k == 0 && ch.size() == 1)) {
        refs[k] = make_leaf((uint32_t)first[c], (uint32_t)cnt[c]);
        leaves++;
      } else {
        refs[k] = emit(c, dep + 1);
      }
    }
    float* nd = &N4[(size_t)me * 32];
    for (int s = 0; s < 4; s++) {
      if (s < (int)ch.size()) {
        const Node2& c = B.nodes[ch[s]];
        put_child(nd, s, c.box, refs[s], c.delta);
        maxd = std::max(maxd, c.delta);
      } else {
        Box z;
        z.reset();  // inverted: lo = +inf, hi = -inf
        put_child(nd, s, z, kEmpty, 0.0f);
      }
    }
    return me;
  };
  emit(0, 1);
  out->order = B.idx;
  out->node_count = (int64_t)(N4.size() / 32);
  out->leaf_count = leaves;
  out->depth = depth4;
  out->max_delta = maxd;
  return ER_OK;
}

// Quantise every FP32 node's child boxes to 8 bits relative to the node's
// own bounds, rounding outward so the decoded box (evaluated with the same
// float operations as the kernel: origin + q * 2^e) always contains the
// FP32 box.  The topology, leaves and child order are unchanged, so the hit
// set of a closest-hit query is unchanged.
void quantize_bvh4(BuildResult* r) {
  r->qnodes.assign((size_t)r->node_count, QNode());
  for (int64_t i = 0; i < r->node_count; i++) {
    const float* nd = &r->nodes[(size_t)i * 32];
    QNode& q = r->qnodes[(size_t)i];
    std::memset(&q, 0, sizeof q);
    float org[3], top[3];
    for (int a = 0; a < 3; a++) { org[a] = INFINITY; top[a] = -INFINITY; }
    int32_t child[4];
    float dmax = 0;
    for (int s = 0; s < 4; s++) {
      std::memcpy(&child[s], &nd[24 + s], 4);
      if (child[s] == kEmpty) continue;
      for (int a = 0; a < 3; a++) {
        org[a] = std::min(org[a], nd[8 * a + s]);
        top[a] = std::max(top[a], nd[8 * a + 4 + s]);
      }
      dmax = std::max(dmax, nd[28 + s]);
    }
    int ex[3];
    for (int a = 0; a < 3; a++) {
      if (!(org[a] <= top[a])) { org[a] = 0; top[a] = 0; }
      org[a] = std::nextafter(org[a], -INFINITY);
      double ext = (double)top[a] - (double)org[a];
      int e = -126;
      while (e < 127 && std::ldexp(255.0, e) < ext * (1.0 + 1e-6)) e++;
      // the decoded top must reach `top` after float rounding
      while (e < 127 && !(org[a] + 255.0f * std::ldexp(1.0f, e) >= top[a])) e++;
      ex[a] = e;
    }
    q.ox = org[0];
    q.oy = org[1];
    q.oz = org[2];
    q.ex = (uint32_t)(uint8_t)(ex[0] + 127) | ((uint32_t)(uint8_t)(ex[1] + 127) << 8) |
           ((uint32_t)(uint8_t)(ex[2] + 127) << 16);
    uint8_t* lo[3] = {q.qlx, q.qly, q.qlz};
    uint8_t* hi[3] = {q.qhx, q.qhy, q.qhz};
    for (int s = 0; s < 4; s++) {
      for (int a = 0; a < 3; a++) {
        float sc = std::ldexp(1.0f, ex[a]);
        if (child[s] == kEmpty) { lo[a][s] = 255; hi[a][s] = 0; continue; }
        float l = nd[8 * a + s], h = nd[8 * a + 4 + s];
        int ql = (int)std::floor(((double)l - org[a]) / sc);
        int qh = (int)std::ceil(((double)h - org[a]) / sc);
        ql = std::min(std::max(ql, 0), 255);
        qh = std::min(std::max(qh, 0), 255);
        while (ql > 0 && !(org[a] + (float)ql * sc <= l)) ql--;
        while (qh < 255 && !(org[a] + (float)qh * sc >= h)) qh++;
        lo[a][s] = (uint8_t)ql;
        hi[a][s] = (uint8_t)qh;
      }
    }
    q.child01[0] = child[0];
    q.child01[1] = child[1];
    q.child23[0] = child[2];
    q.child23[1] = child[3];
    q.delta = dmax;
  }
}

}  // namespace er
