// Test driver for the BVH8 structural rules (check_node8 through the host
// validator, the rules the GPU builder's k_check_* kernels apply too): trees
// from the host builder must pass at every node width, and each planted
// defect must be refused.  Prints one "PASS name" / "FAIL name" line per
// case.  Built and run by tests/test_bvh_check.py with the host compiler.
#include <cstdint>
#include <cstdio>
#include <functional>
#include <vector>

#include "bvh_build.h"

using pt::Box;
using pt::Bvh8Out;

static uint32_t lcg(uint32_t& s) {
  s = s * 1664525u + 1013904223u;
  return s;
}

static float unit(uint32_t& s) { return (float)(lcg(s) >> 8) * (1.0f / 16777216.0f); }

static std::vector<Box> random_boxes(size_t n, uint32_t seed) {
  std::vector<Box> b(n);
  for (Box& x : b) {
    for (int a = 0; a < 3; a++) {
      const float c = 100.f * unit(seed), e = 0.01f + 2.f * unit(seed);
      x.lo[a] = c - e;
      x.hi[a] = c + e;
    }
  }
  return b;
}

static uint32_t meta(const Bvh8Out& t, size_t k, int i) {
  const uint32_t* w = &t.nodes[k * 20];
  return ((i < 4 ? w[6] : w[7]) >> (8 * (i & 3))) & 0xffu;
}

static void set_meta(Bvh8Out& t, size_t k, int i, uint32_t m) {
  uint32_t* w = &t.nodes[k * 20 + (i < 4 ? 6 : 7)];
  const int sh = 8 * (i & 3);
  *w = (*w & ~(0xffu << sh)) | ((m & 0xffu) << sh);
}

// First node (other than the root when `non_root`) with an internal / a leaf child.
static long find_node(const Bvh8Out& t, bool internal, bool non_root) {
  const size_t nn = t.nodes.size() / 20;
  for (size_t k = non_root ? 1 : 0; k < nn; k++)
    for (int i = 0; i < 8; i++) {
      const uint32_t m = meta(t, k, i);
      if (m && ((m & 0x80u) != 0) == internal) return (long)k;
    }
  return -1;
}

static int first_slot(const Bvh8Out& t, size_t k, bool internal) {
  for (int i = 0; i < 8; i++) {
    const uint32_t m = meta(t, k, i);
    if (m && ((m & 0x80u) != 0) == internal) return i;
  }
  return -1;
}

int main() {
  int bad = 0;
  auto report = [&](const char* name, bool ok) {
    printf("%s %s\n", ok ? "PASS" : "FAIL", name);
    if (!ok) bad++;
  };
  // valid trees, every width, several sizes
  for (int width = 2; width <= 8; width++)
    for (size_t n : {1u, 2u, 3u, 4u, 9u, 100u, 5000u}) {
      Bvh8Out t;
      pt::build_bvh8_host(random_boxes(n, (uint32_t)(n * 31 + width)), t, width);
      char name[64];
      snprintf(name, sizeof(name), "valid_w%d_n%zu", width, n);
      report(name, pt::validate_bvh8(t, n));
    }

  const size_t n = 5000;
  Bvh8Out base;
  pt::build_bvh8_host(random_boxes(n, 7u), base, 8);
  auto planted = [&](const char* name, const std::function<bool(Bvh8Out&)>& plant) {
    Bvh8Out t = base;
    const bool planted_ok = plant(t);
    report(name, planted_ok && !pt::validate_bvh8(t, n));
  };
  planted("child_not_after_parent", [&](Bvh8Out& t) {
    const long k = find_node(t, true, true);
    if (k < 0) return false;
    t.nodes[(size_t)k * 20 + 4] = (uint32_t)k;  // slot 0 would point at the node itself
    return true;
  });
  planted("child_past_end", [&](Bvh8Out& t) {
    const long k = find_node(t, true, false);
    if (k < 0) return false;
    t.nodes[(size_t)k * 20 + 4] = (uint32_t)(t.nodes.size() / 20);
    return true;
  });
  planted("internal_slot_not_rank", [&](Bvh8Out& t) {
    const long k = find_node(t, true, false);
    if (k < 0) return false;
    const int i = first_slot(t, (size_t)k, true);
    set_meta(t, (size_t)k, i, 0x80u | ((meta(t, (size_t)k, i) + 1u) & 7u));
    return true;
  });
  planted("internal_mask_wrong", [&](Bvh8Out& t) {
    const long k = find_node(t, true, false);
    if (k < 0) return false;
    t.nodes[(size_t)k * 20 + 3] ^= 0x80u << 24;  // flips the mask bit of slot 7
    return true;
  });
  planted("leaf_of_zero", [&](Bvh8Out& t) {
    const long k = find_node(t, false, false);
    if (k < 0) return false;
    const int i = first_slot(t, (size_t)k, false);
    set_meta(t, (size_t)k, i, meta(t, (size_t)k, i) & 31u);  // count 0, offset kept
    // a zero byte reads as an empty slot: give it offset 1 so it stays a leaf
    if ((meta(t, (size_t)k, i) & 31u) == 0) set_meta(t, (size_t)k, i, 1u);
    return true;
  });
  planted("leaf_of_four", [&](Bvh8Out& t) {
    const long k = find_node(t, false, false);
    if (k < 0) return false;
    const int i = first_slot(t, (size_t)k, false);
    set_meta(t, (size_t)k, i, (4u << 5) | (meta(t, (size_t)k, i) & 31u));
    return true;
  });
  planted("leaf_past_end", [&](Bvh8Out& t) {
    const long k = find_node(t, false, false);
    if (k < 0) return false;
    t.nodes[(size_t)k * 20 + 5] = (uint32_t)n;
    return true;
  });
  planted("position_covered_twice", [&](Bvh8Out& t) {
    const long k = find_node(t, false, false);
    if (k < 0) return false;
    t.nodes[(size_t)k * 20 + 5] += 1;  // shifts this node's leaves onto a neighbour's
    return true;
  });
  planted("leaf_order_not_permutation", [&](Bvh8Out& t) {
    t.leaf_order[1] = t.leaf_order[0];
    return true;
  });
  planted("leaf_order_out_of_range", [&](Bvh8Out& t) {
    t.leaf_order[n / 2] = (uint32_t)n;
    return true;
  });
  printf("%s\n", bad ? "SOME CASES FAILED" : "ALL PASS");
  return bad ? 1 : 0;
}
