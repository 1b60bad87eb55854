/*
 * bvh_build.h - BVH8 builders (host: bvh_host.cpp, GPU: bvh_gpu.cu).  Both
 * emit the 80-byte compressed node format documented in pt_types.h.
 */
#ifndef PT_BVH_BUILD_H
#define PT_BVH_BUILD_H

#include <stdint.h>
#include <vector>

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

struct Bvh8Out {
  std::vector<uint32_t> nodes;       /* 20 words per node */
  std::vector<uint32_t> leaf_order;  /* primitive index at each leaf position */
  int depth = 0;                     /* levels of wide nodes */
};

void encode_node(const Box& parent, const WideChild* ch, int nch, uint32_t child_base,
                 uint32_t prim_base, uint32_t out[20]);
int build_bvh8_host(const std::vector<Box>& boxes, Bvh8Out& out);
bool validate_bvh8(const Bvh8Out& b, size_t num_prims);

}  // namespace pt

#endif
