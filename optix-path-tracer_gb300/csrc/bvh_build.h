/*
 * bvh_build.h - BVH8 builders (host: bvh_host.cpp, GPU: bvh_gpu.cu).  Both
 * emit the 80-byte compressed node format documented in pt_types.h.
 */
#ifndef PT_BVH_BUILD_H
#define PT_BVH_BUILD_H

#include <math.h>
#include <stdint.h>
#include <string.h>
#include <vector>

#if defined(__CUDACC__)
#define PT_BVH_HD __host__ __device__
#else
#define PT_BVH_HD
#endif

namespace pt {

struct Box {
  float lo[3], hi[3];
};

struct WideChild {
  Box box;
  bool internal;
  uint32_t count;     /* leaf: primitives (1..3) */
  uint32_t prim_off;  /* leaf: offset from the node's prim_base */
};

/* Device scratch of the GPU builder, kept by its owner across builds (grown
 * on demand, freed with cudaFree by the owner). */
struct BuildArena {
  void* p = nullptr;
  size_t bytes = 0;
};

struct Bvh8Out {
  std::vector<uint32_t> nodes;       /* 20 words per node */
  std::vector<uint32_t> leaf_order;  /* primitive index at each leaf position */
  int depth = 0;                     /* levels of wide nodes */
};

// Quantises the child boxes of one wide node into the 80-byte record: per
// axis the smallest power-of-two step s with 255 s >= the parent's extent;
// child bounds rounded outward to the step grid plus one step of slack for
// the float decode in traversal.  Float-only, so host and device agree.
PT_BVH_HD inline void encode_node_dev(const Box& parent, const WideChild* ch, int nch,
                                      uint32_t child_base, uint32_t prim_base, uint32_t out[20]) {
  for (int w = 0; w < 20; w++) out[w] = 0;
  uint32_t e[3];
  float p[3], step[3];
  for (int a = 0; a < 3; a++) {
    p[a] = parent.lo[a];
    float ext = parent.hi[a] - parent.lo[a];
    int ex = -126;
    if (ext > 0.f) {
      int k;
      frexpf(ext / 255.0f, &k);
      ex = k;
      while (ex > -126 && ldexpf(255.0f, ex - 1) >= ext) ex--;
      while (ldexpf(255.0f, ex) < ext) ex++;
      if (ex < -126) ex = -126;
    }
    e[a] = (uint32_t)(ex + 127);
    step[a] = ldexpf(1.0f, ex);
  }
  memcpy(&out[0], &p[0], 4);
  memcpy(&out[1], &p[1], 4);
  memcpy(&out[2], &p[2], 4);
  uint32_t imask = 0, rank = 0;
  // empty slots keep an inverted box (lo 255, hi 0): no ray passes its slab test
  uint32_t meta[2] = {0, 0}, qhi[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  uint32_t qlo[3][2] = {{0xffffffffu, 0xffffffffu}, {0xffffffffu, 0xffffffffu},
                        {0xffffffffu, 0xffffffffu}};
  // internal children take the low slots in their given order (slot ==
  // rank, the offset of the child node from child_base), leaves follow
  int ord[8], no = 0;
  for (int i = 0; i < nch; i++)
    if (ch[i].internal) ord[no++] = i;
  for (int i = 0; i < nch; i++)
    if (!ch[i].internal) ord[no++] = i;
  for (int i = 0; i < nch; i++) {
    const WideChild& c = ch[ord[i]];
    uint32_t m;
    if (c.internal) {
      m = 0x80u | rank;
      imask |= 1u << i;
      rank++;
    } else {
      m = (c.count << 5) | c.prim_off;
    }
    meta[i >> 2] |= m << (8 * (i & 3));
    for (int a = 0; a < 3; a++) {
      float lo = floorf((c.box.lo[a] - p[a]) / step[a]) - 1.0f;
      float hi = ceilf((c.box.hi[a] - p[a]) / step[a]) + 1.0f;
      lo = fminf(fmaxf(lo, 0.0f), 255.0f);
      hi = fminf(fmaxf(hi, 0.0f), 255.0f);
      qlo[a][i >> 2] = (qlo[a][i >> 2] & ~(0xffu << (8 * (i & 3)))) | ((uint32_t)lo << (8 * (i & 3)));
      qhi[a][i >> 2] |= (uint32_t)hi << (8 * (i & 3));
    }
  }
  out[3] = e[0] | (e[1] << 8) | (e[2] << 16) | (imask << 24);
  out[4] = child_base;
  out[5] = prim_base;
  out[6] = meta[0];
  out[7] = meta[1];
  out[8] = qlo[0][0];
  out[9] = qlo[0][1];
  out[10] = qlo[1][0];
  out[11] = qlo[1][1];
  out[12] = qlo[2][0];
  out[13] = qlo[2][1];
  out[14] = qhi[0][0];
  out[15] = qhi[0][1];
  out[16] = qhi[1][0];
  out[17] = qhi[1][1];
  out[18] = qhi[2][0];
  out[19] = qhi[2][1];
}

// World box of a moving sphere (f = centre at time0 (3), radius, time0,
// time1, centre at time1 (3)) over every time a ray can carry: ray times lie
// in [cam_t0, cam_t0 + (cam_t1 - cam_t0)] (or the reverse), the centre
// c0 + ((t - time0) / (time1 - time0)) * (c1 - c0) is monotonic in t in
// floating point too, so the boxes at the two end times hold it.
PT_BVH_HD inline void moving_sphere_box(const float* f, float cam_t0, float cam_t1, float lo[3],
                                        float hi[3]) {
  const float te = cam_t0 + (cam_t1 - cam_t0);
  const float ta = fminf(fminf(f[4], cam_t0), te), tb = fmaxf(fmaxf(f[5], cam_t0), te);
  for (int a = 0; a < 3; a++) {
    const float d = f[6 + a] - f[a];
    const float ca = f[a] + ((ta - f[4]) / (f[5] - f[4])) * d;
    const float cb = f[a] + ((tb - f[4]) / (f[5] - f[4])) * d;
    lo[a] = fminf(ca, cb) - f[3];
    hi[a] = fmaxf(ca, cb) + f[3];
  }
}

// Structural rules of node k of an nn-node BVH8 over n primitives: internal
// children fill slots 0..r-1 with child index base + slot, each above k and
// below nn, the internal-slot mask (bits 24-31 of word 3) is (1 << r) - 1,
// and every leaf slot holds 1..3 primitive positions below n, each passed to
// on_prim (which counts how often a position is covered).  Returns false on
// the first broken rule.  The host validator and the GPU builder's check
// both apply it.
template <typename F>
PT_BVH_HD inline bool check_node8(const uint32_t* w, uint64_t k, uint64_t nn, uint64_t n,
                                  F&& on_prim) {
  uint32_t rank = 0;
  for (int i = 0; i < 8; i++) {
    const uint32_t meta = ((i < 4 ? w[6] : w[7]) >> (8 * (i & 3))) & 0xffu;
    if (!meta) continue;
    if (meta & 0x80u) {
      const uint64_t c = (uint64_t)w[4] + (meta & 7u);
      if ((meta & 7u) != rank || (uint32_t)i != rank || c <= k || c >= nn) return false;
      rank++;
    } else {
      const uint32_t cnt = meta >> 5, off = meta & 31u;
      if (cnt < 1 || cnt > 3) return false;
      for (uint32_t q = 0; q < cnt; q++) {
        const uint64_t pi = (uint64_t)w[5] + off + q;
        if (pi >= n || !on_prim(pi)) return false;
      }
    }
  }
  return (w[3] >> 24) == (1u << rank) - 1u;
}

inline void encode_node(const Box& parent, const WideChild* ch, int nch, uint32_t child_base,
                        uint32_t prim_base, uint32_t out[20]) {
  encode_node_dev(parent, ch, nch, child_base, prim_base, out);
}
/* width: most children per node, 2..8 (the node format holds 8) */
int build_bvh8_host(const std::vector<Box>& boxes, Bvh8Out& out, int width = 8);
bool validate_bvh8(const Bvh8Out& b, size_t num_prims);

}  // namespace pt

#endif
