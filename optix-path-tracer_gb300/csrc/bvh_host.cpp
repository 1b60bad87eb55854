/*
 * bvh_host.cpp - host BVH8 builder: binned-SAH binary BVH, collapsed to
 * 8-wide nodes with 8-bit quantised child boxes (the node format of
 * pt_types.h).  Replaces the OptiX "Trbvh" acceleration the reference
 * requests for every group (e.g. host_includes/scenes.hpp:32,
 * host_includes/transforms.hpp:59).  The GPU builder (bvh_gpu.cu) produces
 * the same node format; this one serves small scenes and cross-checks.
 */
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>
#include "bvh_build.h"

namespace pt {

namespace {

struct BNode {
  Box box;
  int left = -1, right = -1;  // internal children
  int first = 0, count = 0;   // leaf range in `order`
  int nprims = 0;             // primitives in the subtree
};

inline Box merge(const Box& a, const Box& b) {
  Box r;
  for (int k = 0; k < 3; k++) {
    r.lo[k] = std::min(a.lo[k], b.lo[k]);
    r.hi[k] = std::max(a.hi[k], b.hi[k]);
  }
  return r;
}
inline float half_area(const Box& a) {
  float ex = a.hi[0] - a.lo[0], ey = a.hi[1] - a.lo[1], ez = a.hi[2] - a.lo[2];
  if (ex < 0) return 0.f;
  return ex * ey + ey * ez + ez * ex;
}
inline Box empty_box() {
  Box b;
  for (int k = 0; k < 3; k++) {
    b.lo[k] = FLT_MAX;
    b.hi[k] = -FLT_MAX;
  }
  return b;
}

struct Bvh2 {
  const std::vector<Box>& boxes;
  std::vector<float> cx, cy, cz;
  std::vector<uint32_t>& order;
  std::vector<BNode> nodes;
  Bvh2(const std::vector<Box>& b, std::vector<uint32_t>& o) : boxes(b), order(o) {
    size_t n = b.size();
    cx.resize(n);
    cy.resize(n);
    cz.resize(n);
    for (size_t i = 0; i < n; i++) {
      cx[i] = 0.5f * (b[i].lo[0] + b[i].hi[0]);
      cy[i] = 0.5f * (b[i].lo[1] + b[i].hi[1]);
      cz[i] = 0.5f * (b[i].lo[2] + b[i].hi[2]);
    }
  }
  float cen(uint32_t p, int ax) const { return ax == 0 ? cx[p] : (ax == 1 ? cy[p] : cz[p]); }

  int build(int begin, int end) {
    int ni = (int)nodes.size();
    nodes.emplace_back();
    Box bb = empty_box(), cb = empty_box();
    for (int k = begin; k < end; k++) {
      uint32_t p = order[k];
      bb = merge(bb, boxes[p]);
      for (int a = 0; a < 3; a++) {
        cb.lo[a] = std::min(cb.lo[a], cen(p, a));
        cb.hi[a] = std::max(cb.hi[a], cen(p, a));
      }
    }
    int n = end - begin;
    nodes[ni].box = bb;
    nodes[ni].nprims = n;
    if (n <= 3) {
      nodes[ni].first = begin;
      nodes[ni].count = n;
      return ni;
    }
    const int NB = 32;
    float best = FLT_MAX;
    int best_ax = -1, best_bin = -1;
    for (int ax = 0; ax < 3; ax++) {
      float lo = cb.lo[ax], hi = cb.hi[ax];
      if (!(hi - lo > 0.f)) continue;
      Box bins[NB];
      int cnt[NB] = {0};
      for (int k = 0; k < NB; k++) bins[k] = empty_box();
      float scale = NB / (hi - lo);
      for (int k = begin; k < end; k++) {
        uint32_t p = order[k];
        int b = std::min(NB - 1, std::max(0, (int)((cen(p, ax) - lo) * scale)));
        cnt[b]++;
        bins[b] = merge(bins[b], boxes[p]);
      }
      float la[NB];
      int lc[NB];
      Box acc = empty_box();
      int c = 0;
      for (int k = 0; k < NB; k++) {
        acc = merge(acc, bins[k]);
        c += cnt[k];
        la[k] = half_area(acc);
        lc[k] = c;
      }
      acc = empty_box();
      c = 0;
      for (int k = NB - 1; k > 0; k--) {
        acc = merge(acc, bins[k]);
        c += cnt[k];
        if (lc[k - 1] == 0 || c == 0) continue;
        float cost = la[k - 1] * lc[k - 1] + half_area(acc) * c;
        if (cost < best) {
          best = cost;
          best_ax = ax;
          best_bin = k - 1;
        }
      }
    }
    int mid = begin + n / 2;
    if (best_ax >= 0) {
      float lo = cb.lo[best_ax], hi = cb.hi[best_ax];
      float scale = NB / (hi - lo);
      auto it = std::partition(order.begin() + begin, order.begin() + end, [&](uint32_t p) {
        int b = std::min(NB - 1, std::max(0, (int)((cen(p, best_ax) - lo) * scale)));
        return b <= best_bin;
      });
      mid = (int)(it - order.begin());
      if (mid == begin || mid == end) mid = begin + n / 2;
    } else {
      // all centroids coincide: split by index
      mid = begin + n / 2;
    }
    int l = build(begin, mid);
    int r = build(mid, end);
    nodes[ni].left = l;
    nodes[ni].right = r;
    return ni;
  }
};

}  // namespace

// The quantisation grid of encode_node extends the parent box upward by up
// to 255 steps; the parent itself must cover the children, which the caller
// guarantees (parent = union of children).
int build_bvh8_host(const std::vector<Box>& boxes, Bvh8Out& out, int width) {
  if (width < 2 || width > 8) width = 8;
  size_t n = boxes.size();
  out.nodes.clear();
  out.leaf_order.clear();
  out.depth = 0;
  if (n == 0) return 0;
  std::vector<uint32_t> order(n);
  for (size_t i = 0; i < n; i++) order[i] = (uint32_t)i;
  Bvh2 b2(boxes, order);
  b2.nodes.reserve(2 * n);
  b2.build(0, (int)n);
  const std::vector<BNode>& B = b2.nodes;

  // breadth-first emission of wide nodes; each wide node records the binary
  // node it expands
  struct Pending {
    int bnode;
    int depth;
  };
  std::vector<Pending> queue;
  queue.push_back({0, 1});
  out.nodes.resize(20);  // root
  size_t head = 0;
  while (head < queue.size()) {
    Pending pd = queue[head];
    uint32_t self = (uint32_t)head;
    head++;
    out.depth = std::max(out.depth, pd.depth);
    // gather up to `width` children by expanding the largest internal child
    std::vector<int> kids;
    const BNode& bn = B[pd.bnode];
    if (bn.left < 0) {
      kids.push_back(pd.bnode);  // single-leaf root
    } else {
      kids.push_back(bn.left);
      kids.push_back(bn.right);
      while ((int)kids.size() < width) {
        int best = -1;
        float best_area = -1.f;
        for (size_t k = 0; k < kids.size(); k++) {
          const BNode& c = B[kids[k]];
          if (c.left < 0 || c.nprims <= 3) continue;  // leaf or small enough for one slot
          float a = half_area(c.box);
          if (a > best_area) {
            best_area = a;
            best = (int)k;
          }
        }
        if (best < 0) break;
        int bi = kids[best];
        kids[best] = B[bi].left;
        kids.push_back(B[bi].right);
      }
    }
    WideChild wc[8];
    int nch = (int)kids.size();
    uint32_t child_base = (uint32_t)queue.size();
    uint32_t prim_base = (uint32_t)out.leaf_order.size();
    uint32_t off = 0;
    Box parent = empty_box();
    for (int k = 0; k < nch; k++) {
      const BNode& c = B[kids[k]];
      wc[k].box = c.box;
      parent = merge(parent, c.box);
      if (c.nprims <= 3) {
        wc[k].internal = false;
        wc[k].count = (uint32_t)c.nprims;
        wc[k].prim_off = off;
        // collect the subtree's primitives (a leaf, or a small internal node)
        std::vector<int> st{kids[k]};
        while (!st.empty()) {
          int x = st.back();
          st.pop_back();
          if (B[x].left < 0) {
            for (int q = 0; q < B[x].count; q++) out.leaf_order.push_back(order[B[x].first + q]);
          } else {
            st.push_back(B[x].right);
            st.push_back(B[x].left);
          }
        }
        off += (uint32_t)c.nprims;
      } else {
        wc[k].internal = true;
        wc[k].count = 0;
        wc[k].prim_off = 0;
        queue.push_back({kids[k], pd.depth + 1});
      }
    }
    out.nodes.resize(queue.size() * 20);
    encode_node(parent, wc, nch, child_base, prim_base, &out.nodes[(size_t)self * 20]);
  }
  return 0;
}

// Structural check of a BVH8 before it is uploaded: every internal child
// index lies after its parent and inside the node array, internal children
// fill the low slots with dense ranks (slot == rank),
// leaf ranges lie inside the primitive array and cover each primitive once.
bool validate_bvh8(const Bvh8Out& b, size_t num_prims) {
  size_t nn = b.nodes.size() / 20;
  if (num_prims == 0) return nn == 0 && b.leaf_order.empty();
  if (nn == 0 || b.leaf_order.size() != num_prims) return false;
  std::vector<uint8_t> seen(num_prims, 0);
  auto cover = [&](uint64_t pi) {
    const uint32_t id = b.leaf_order[pi];
    return id < num_prims && seen[id]++ == 0;
  };
  for (size_t k = 0; k < nn; k++)
    if (!check_node8(&b.nodes[k * 20], k, nn, num_prims, cover)) return false;
  for (uint8_t v : seen)
    if (v != 1) return false;
  return true;
}

}  // namespace pt
