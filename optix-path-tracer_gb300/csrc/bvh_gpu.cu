/*
 * bvh_gpu.cu - BVH8 builder on the GPU (replaces the OptiX "Trbvh" build the
 * reference requests for every group, e.g. host_includes/scenes.hpp:32).
 *
 *  1. k_bounds      padded world AABB and centroid of every primitive record
 *  2. k_morton      30-bit Morton code of the centroid (10 bits per axis, one
 *                   scale for all axes: the centroid box's longest side)
 *  3. radix sort    CUB DeviceRadixSort over (code, primitive) pairs
 *  4. k_karras      binary radix tree, Karras, "Maximizing Parallelism in the
 *                   Construction of BVHs, Octrees, and k-d Trees", HPG 2012
 *  5. k_bottom_up   bounds and SAH cost bottom-up (atomic arrival counters);
 *                   at every node with >= 7 primitives below it the treelet of
 *                   up to 7 leaves is rebuilt optimally for SAH by dynamic
 *                   programming over leaf subsets (Karras & Aila, "Fast
 *                   Parallel Construction of High-Quality BVHs", HPG 2013),
 *                   one warp per treelet; a first pass without restructuring,
 *                   then one per treelet round
 *  6. k_collapse    one launch per level: each binary node becomes a wide
 *                   node by expanding its largest child until 8 children
 *                   (or the requested width);
 *                   subtrees of <= 3 primitives become leaf slots; child
 *                   boxes are quantised to 8 bits (node format: pt_types.h)
 *  7. k_check_*     structural check of the finished tree before any
 *                   traversal runs on it (check_node8 on every node, every
 *                   leaf position covered once, leaf_of_id a permutation)
 * The result is order independent for rendering (closest hit is the minimum
 * of (t, primitive id)), so the atomics that place nodes do not change images.
 */
#include <cuda_runtime.h>
#include <cub/device/device_radix_sort.cuh>
#include <stdint.h>
#include <vector>

#include "bvh_build.h"
#include "pt_device.cuh"
#include "pt_internal.h"

namespace {

constexpr uint32_t LEAF_BIT = 0x80000000u;
constexpr float C_INNER = 1.2f, C_TRI = 1.0f;

struct GBox {
  float lo[3], hi[3];
};

__device__ __forceinline__ GBox box_union(const GBox& a, const GBox& b) {
  GBox r;
  for (int k = 0; k < 3; k++) {
    r.lo[k] = fminf(a.lo[k], b.lo[k]);
    r.hi[k] = fmaxf(a.hi[k], b.hi[k]);
  }
  return r;
}
__device__ __forceinline__ float box_area(const GBox& b) {
  float x = b.hi[0] - b.lo[0], y = b.hi[1] - b.lo[1], z = b.hi[2] - b.lo[2];
  return x * y + y * z + z * x;
}
__device__ __forceinline__ void box_store(float4* lo, float4* hi, uint32_t i, const GBox& b,
                                          float w0, float w1) {
  lo[i] = make_float4(b.lo[0], b.lo[1], b.lo[2], w0);
  hi[i] = make_float4(b.hi[0], b.hi[1], b.hi[2], w1);
}
__device__ __forceinline__ GBox box_load(const float4* lo, const float4* hi, uint32_t i) {
  float4 a = lo[i], b = hi[i];
  GBox r;
  r.lo[0] = a.x; r.lo[1] = a.y; r.lo[2] = a.z;
  r.hi[0] = b.x; r.hi[1] = b.y; r.hi[2] = b.z;
  return r;
}
// Loads of tree data that other threads write during the same kernel
// (k_bottom_up): L2 only (ld.global.cg), so no stale L1 line is read.
__device__ __forceinline__ GBox box_load_cg(const float4* lo, const float4* hi, uint32_t i) {
  float4 a = __ldcg(lo + i), b = __ldcg(hi + i);
  GBox r;
  r.lo[0] = a.x; r.lo[1] = a.y; r.lo[2] = a.z;
  r.hi[0] = b.x; r.hi[1] = b.y; r.hi[2] = b.z;
  return r;
}

// Padded world AABB of one primitive record (the host builder's padding).
__global__ void k_bounds(const float4* __restrict__ rec, const float4* __restrict__ xforms,
                         uint32_t n, float cam_t0, float cam_t1, float4* lo, float4* hi,
                         unsigned int* cbox) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  GBox c;
  for (int k = 0; k < 3; k++) {
    c.lo[k] = 3.0e38f;
    c.hi[k] = -3.0e38f;
  }
  if (i < n) {
    float4 r0 = rec[3 * i], r1 = rec[3 * i + 1], r2 = rec[3 * i + 2];
    uint32_t tag = __float_as_uint(r0.w);
    int type = tag & 3, axis = (tag >> 2) & 3, xf = (int)(tag >> 8) - 1;
    float f[9] = {r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r2.x, r2.y, r2.z};
    GBox b;
    if (type == PT_PRIM_TRIANGLE) {
      for (int a = 0; a < 3; a++) {
        b.lo[a] = fminf(fminf(f[a], f[3 + a]), f[6 + a]);
        b.hi[a] = fmaxf(fmaxf(f[a], f[3 + a]), f[6 + a]);
      }
    } else if (type == PT_PRIM_SPHERE && (tag & PT_PRIM_MOVING)) {
      pt::moving_sphere_box(f, cam_t0, cam_t1, b.lo, b.hi);
    } else if (type == PT_PRIM_SPHERE) {
      for (int a = 0; a < 3; a++) {
        b.lo[a] = f[a] - f[3];
        b.hi[a] = f[a] + f[3];
      }
    } else if (type == PT_PRIM_RECT) {
      int ia = axis == 0 ? 1 : 0, ib = axis == 2 ? 1 : 2;
      b.lo[axis] = b.hi[axis] = f[4];
      b.lo[ia] = f[0];
      b.hi[ia] = f[1];
      b.lo[ib] = f[2];
      b.hi[ib] = f[3];
    } else {
      for (int a = 0; a < 3; a++) {
        b.lo[a] = f[a];
        b.hi[a] = f[3 + a];
      }
    }
    if (xf >= 0) {
      const float4* M = xforms + 6 * xf;
      GBox w;
      for (int k = 0; k < 3; k++) {
        w.lo[k] = 3.0e38f;
        w.hi[k] = -3.0e38f;
      }
      for (int cc = 0; cc < 8; cc++) {
        ptd::V3 q = ptd::v3((cc & 1) ? b.hi[0] : b.lo[0], (cc & 2) ? b.hi[1] : b.lo[1],
                            (cc & 4) ? b.hi[2] : b.lo[2]);
        ptd::V3 p = ptd::xpoint(M, q);
        float pw[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; k++) {
          w.lo[k] = fminf(w.lo[k], pw[k]);
          w.hi[k] = fmaxf(w.hi[k], pw[k]);
        }
      }
      b = w;
    }
    for (int a = 0; a < 3; a++) {
      float mag = fmaxf(1.0f, fmaxf(fabsf(b.lo[a]), fabsf(b.hi[a])));
      float pad = mag * 9.5367431640625e-07f * (xf >= 0 ? 16.f : 1.f);
      b.lo[a] -= pad;
      b.hi[a] += pad;
    }
    lo[i] = make_float4(b.lo[0], b.lo[1], b.lo[2], 0.f);
    hi[i] = make_float4(b.hi[0], b.hi[1], b.hi[2], 0.f);
    for (int a = 0; a < 3; a++) c.lo[a] = c.hi[a] = 0.5f * (b.lo[a] + b.hi[a]);
  }
  // centroid bounds: block reduction, then ordered-int atomics
  for (int a = 0; a < 3; a++) {
    for (int o = 16; o > 0; o >>= 1) {
      c.lo[a] = fminf(c.lo[a], __shfl_xor_sync(0xffffffffu, c.lo[a], o));
      c.hi[a] = fmaxf(c.hi[a], __shfl_xor_sync(0xffffffffu, c.hi[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int a = 0; a < 3; a++) {
      // monotone float -> uint mapping
      uint32_t u = __float_as_uint(c.lo[a]);
      u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
      atomicMin(&cbox[a], u);
      uint32_t v = __float_as_uint(c.hi[a]);
      v = (v & 0x80000000u) ? ~v : (v | 0x80000000u);
      atomicMax(&cbox[3 + a], v);
    }
  }
}

__device__ __forceinline__ float unmap(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                         const unsigned int* cbox, uint32_t* keys, uint32_t* vals) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 a = lo[i], b = hi[i];
  float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
  // one scale for all axes (the centroid box's longest side): a flat scene
  // (a heightfield) is not split along its thin axis as often as along the
  // wide ones, which would give siblings that overlap over their whole area
  float e = 0.f;
  for (int k = 0; k < 3; k++) e = fmaxf(e, unmap(cbox[3 + k]) - unmap(cbox[k]));
  uint32_t code = 0;
  for (int k = 0; k < 3; k++) {
    float l = unmap(cbox[k]);
    float t = e > 0.f ? (c[k] - l) / e : 0.5f;
    uint32_t q = (uint32_t)fminf(fmaxf(t * 1024.f, 0.f), 1023.f);
    code |= spread10(q) << (2 - k);
  }
  keys[i] = code;
  vals[i] = i;
}

__device__ __forceinline__ int delta(const uint32_t* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint32_t a = keys[i], b = keys[j];
  if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
  return __clz(a ^ b);
}

// internal node i of the radix tree over sorted keys (Karras 2012, fig. 4)
__global__ void k_karras(const uint32_t* __restrict__ keys, int n, uint32_t* left, uint32_t* right,
                         uint32_t* parent_int, uint32_t* parent_leaf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = delta(keys, n, i, j);
  int s = 0;
  for (int div = 2;; div *= 2) {
    int t = (l + div - 1) / div;
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  int gamma = i + s * d + min(d, 0);
  int lo = min(i, j), hi = max(i, j);
  uint32_t lc = (lo == gamma) ? ((uint32_t)gamma | LEAF_BIT) : (uint32_t)gamma;
  uint32_t rc = (hi == gamma + 1) ? ((uint32_t)(gamma + 1) | LEAF_BIT) : (uint32_t)(gamma + 1);
  left[i] = lc;
  right[i] = rc;
  if (lc & LEAF_BIT) parent_leaf[lc & ~LEAF_BIT] = (uint32_t)i;
  else parent_int[lc] = (uint32_t)i;
  if (rc & LEAF_BIT) parent_leaf[rc & ~LEAF_BIT] = (uint32_t)i;
  else parent_int[rc] = (uint32_t)i;
  if (i == 0) parent_int[0] = 0xffffffffu;
}

struct Tree {
  uint32_t *left, *right, *parent_int, *parent_leaf;
  float4 *ilo, *ihi;        // internal bounds; ilo.w = SAH cost, ihi.w = primitive count
  const float4 *llo, *lhi;  // leaf bounds (sorted order)
  uint32_t* flags;
};

// Internal-node data (boxes, costs, counts, links) is written by other
// threads of k_bottom_up while it runs, so it is read through L2 only; leaf
// boxes come from an earlier kernel.
__device__ __forceinline__ GBox ref_box(const Tree& T, uint32_t r) {
  return (r & LEAF_BIT) ? box_load(T.llo, T.lhi, r & ~LEAF_BIT) : box_load_cg(T.ilo, T.ihi, r);
}
__device__ __forceinline__ float ref_cost(const Tree& T, uint32_t r) {
  return (r & LEAF_BIT) ? C_TRI * box_area(box_load(T.llo, T.lhi, r & ~LEAF_BIT))
                        : __ldcg(&T.ilo[r].w);
}
__device__ __forceinline__ float ref_count(const Tree& T, uint32_t r) {
  return (r & LEAF_BIT) ? 1.f : __ldcg(&T.ihi[r].w);
}
__device__ __forceinline__ uint32_t left_of(const Tree& T, uint32_t x) { return __ldcg(T.left + x); }
__device__ __forceinline__ uint32_t right_of(const Tree& T, uint32_t x) { return __ldcg(T.right + x); }
__device__ __forceinline__ void set_parent(const Tree& T, uint32_t r, uint32_t p) {
  if (r & LEAF_BIT) T.parent_leaf[r & ~LEAF_BIT] = p;
  else T.parent_int[r] = p;
}

// Dynamic-programming state of one treelet, one per warp in shared memory.
struct TreeletDP {
  float cost[128];    // SAH cost of the best subtree over each leaf subset
  float box[6][128];  // bounds of each leaf subset (lo xyz, hi xyz)
  uint8_t split[128]; // the subset's best first part
};

// Rebuilds the treelet rooted at internal node `root` (up to 7 leaves) with
// the SAH-optimal topology; the treelet's internal nodes are reused.  Called
// by all 32 lanes of a warp together: every lane forms the same treelet (the
// same loads), the lanes share the subsets of each size of the dynamic
// program, and lane 0 writes the new topology.
__device__ void optimize_treelet(const Tree& T, uint32_t root, TreeletDP& dp, int lane) {
  uint32_t leaves[7], inner[6];
  int nl = 2, ni = 1;
  leaves[0] = left_of(T, root);
  leaves[1] = right_of(T, root);
  inner[0] = root;
  while (nl < 7) {
    int best = -1;
    float ba = -1.f;
    for (int k = 0; k < nl; k++) {
      if (leaves[k] & LEAF_BIT) continue;
      float a = box_area(box_load_cg(T.ilo, T.ihi, leaves[k]));
      if (a > ba) {
        ba = a;
        best = k;
      }
    }
    if (best < 0) break;
    uint32_t x = leaves[best];
    inner[ni++] = x;
    leaves[best] = left_of(T, x);
    leaves[nl++] = right_of(T, x);
  }
  if (nl < 3) return;  // the same for every lane
  const int full = (1 << nl) - 1;
  if (lane < nl) {
    GBox b = ref_box(T, leaves[lane]);
    const int S = 1 << lane;
    for (int a = 0; a < 3; a++) {
      dp.box[a][S] = b.lo[a];
      dp.box[3 + a][S] = b.hi[a];
    }
    dp.cost[S] = ref_cost(T, leaves[lane]);
  }
  __syncwarp();
  // subsets by size: every proper subset of S is complete before S
  for (int size = 2; size <= nl; size++) {
    for (int S = lane + 1; S <= full; S += 32) {
      if (__popc(S) != size) continue;
      const int low = S & -S;
      GBox b;
      for (int a = 0; a < 3; a++) {
        b.lo[a] = fminf(dp.box[a][S ^ low], dp.box[a][low]);
        b.hi[a] = fmaxf(dp.box[3 + a][S ^ low], dp.box[3 + a][low]);
        dp.box[a][S] = b.lo[a];
        dp.box[3 + a][S] = b.hi[a];
      }
      // subsets P of S containing the lowest bit, P != S
      float best = 3.0e38f;
      int bp = low;
      const int rest = S ^ low;
      for (int Q = (rest - 1) & rest;; Q = (Q - 1) & rest) {
        const int P = Q | low;  // P ranges over low + proper subsets of rest
        float c = dp.cost[P] + dp.cost[S ^ P];
        if (c < best) {
          best = c;
          bp = P;
        }
        if (Q == 0) break;
      }
      dp.cost[S] = C_INNER * box_area(b) + best;
      dp.split[S] = (uint8_t)bp;
    }
    __syncwarp();
  }
  if (lane == 0) {
    // rewrite: assign internal node indices top-down (root keeps its index)
    struct Item {
      int S;
      uint32_t node;
    };
    Item stk[8];
    int sp = 0, next_inner = 1;
    stk[sp++] = {full, root};
    while (sp) {
      Item it = stk[--sp];
      int P = dp.split[it.S], R = it.S ^ P;
      uint32_t ch[2];
      int sets[2] = {P, R};
      for (int c = 0; c < 2; c++) {
        int X = sets[c];
        if ((X & (X - 1)) == 0) {
          int k = __ffs(X) - 1;
          ch[c] = leaves[k];
        } else {
          ch[c] = inner[next_inner++];
          stk[sp++] = {X, ch[c]};
        }
        set_parent(T, ch[c], it.node);
      }
      T.left[it.node] = ch[0];
      T.right[it.node] = ch[1];
      float cnt = 0.f;
      // count = sum of leaf counts in S
      for (int k = 0; k < nl; k++)
        if (it.S & (1 << k)) cnt += ref_count(T, leaves[k]);
      GBox b;
      for (int a = 0; a < 3; a++) {
        b.lo[a] = dp.box[a][it.S];
        b.hi[a] = dp.box[3 + a][it.S];
      }
      box_store(T.ilo, T.ihi, it.node, b, dp.cost[it.S], cnt);
    }
    __threadfence();  // before any lane of this warp reports the root upward
  }
  __syncwarp();
}

// Bounds, costs and counts bottom-up (the second thread to arrive at a node
// processes it); optionally treelet restructuring, done by the whole warp
// for each of its lanes' nodes in turn.  Launched with 256 threads.
__global__ void __launch_bounds__(256) k_bottom_up(Tree T, int n, int optimize) {
  __shared__ TreeletDP dps[8];
  const int lane = threadIdx.x & 31;
  TreeletDP& dp = dps[threadIdx.x >> 5];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool alive = i < n;
  uint32_t node = alive ? T.parent_leaf[i] : 0xffffffffu;
  while (__any_sync(0xffffffffu, alive)) {
    bool need = false;
    if (alive) {
      if (node == 0xffffffffu) {
        alive = false;
      } else {
        __threadfence();
        if (atomicAdd(&T.flags[node], 1u) == 0) {
          alive = false;  // the sibling subtree is not done: its thread continues
        } else {
          __threadfence();
          uint32_t l = left_of(T, node), r = right_of(T, node);
          GBox b = box_union(ref_box(T, l), ref_box(T, r));
          float cnt = ref_count(T, l) + ref_count(T, r);
          float cost = C_INNER * box_area(b) + ref_cost(T, l) + ref_cost(T, r);
          box_store(T.ilo, T.ihi, node, b, cost, cnt);
          need = optimize && cnt >= 7.f;
        }
      }
    }
    uint32_t m = __ballot_sync(0xffffffffu, need);
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      optimize_treelet(T, __shfl_sync(0xffffffffu, node, src), dp, lane);
    }
    if (alive) {
      __threadfence();
      node = __ldcg(T.parent_int + node);
    }
  }
}

struct CollapseOut {
  uint4* nodes;           // 5 per node
  float4* rec_out;        // leaf-ordered primitive records
  uint32_t* leaf_of_id;
  uint32_t* counters;     // [0] nodes, [1] primitives, [2] next-level queue length, [3] error
  uint32_t n;             // primitives = capacity of nodes, records and queues
};

// gathers the primitives of a subtree with <= 3 of them
__device__ __forceinline__ int gather_small(const Tree& T, const uint32_t* sorted_prim, uint32_t r,
                                            uint32_t* out) {
  int cnt = 0;
  uint32_t stk[4];
  int sp = 0;
  stk[sp++] = r;
  while (sp) {
    uint32_t x = stk[--sp];
    if (x & LEAF_BIT) {
      if (cnt < 3) out[cnt] = sorted_prim[x & ~LEAF_BIT];
      cnt++;
    } else if (sp < 3) {
      stk[sp++] = T.right[x];
      stk[sp++] = T.left[x];
    }
  }
  return cnt;
}

__global__ void k_collapse(Tree T, const uint32_t* __restrict__ sorted_prim,
                           const float4* __restrict__ rec_in, const uint2* __restrict__ qin,
                           uint32_t nq, uint2* qout, CollapseOut out, int width) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq) return;
  uint2 it = qin[t];
  uint32_t kids[8];
  int nk = 0;
  if (it.x & LEAF_BIT) {  // a single-primitive scene
    kids[nk++] = it.x;
  } else {
    kids[nk++] = T.left[it.x];
    kids[nk++] = T.right[it.x];
    // at most 6 expansions (2 -> 8 children); a fixed trip count keeps the
    // per-thread arrays in registers
#pragma unroll
    for (int ex = 0; ex < 6; ex++) {
      if (nk >= width) break;
      int best = -1;
      float ba = -1.f;
      for (int k = 0; k < nk; k++) {
        if ((kids[k] & LEAF_BIT) || ref_count(T, kids[k]) <= 3.f) continue;
        float a = box_area(box_load(T.ilo, T.ihi, kids[k]));
        if (a > ba) {
          ba = a;
          best = k;
        }
      }
      if (best < 0) break;
      uint32_t x = kids[best];
      kids[best] = T.left[x];
      kids[nk++] = T.right[x];
    }
  }
  // classify and allocate
  int n_int = 0;
  uint32_t nprim = 0;
  uint32_t cnts[8];
  for (int k = 0; k < nk; k++) {
    float c = ref_count(T, kids[k]);
    if (!(kids[k] & LEAF_BIT) && c > 3.f) {
      n_int++;
      cnts[k] = 0;
    } else if (c >= 1.f && c <= 3.f) {
      cnts[k] = (uint32_t)c;
      nprim += cnts[k];
    } else {  // a count a valid tree cannot have: flag it, write nothing
      atomicOr(&out.counters[3], 1u);
      return;
    }
  }
  uint32_t child_base = n_int ? atomicAdd(&out.counters[0], (uint32_t)n_int) : 0;
  uint32_t prim_base = nprim ? atomicAdd(&out.counters[1], nprim) : 0;
  uint32_t qbase = n_int ? atomicAdd(&out.counters[2], (uint32_t)n_int) : 0;
  if (it.y >= out.n || child_base + (uint32_t)n_int > out.n || prim_base + nprim > out.n ||
      qbase + (uint32_t)n_int > out.n) {
    atomicOr(&out.counters[3], 2u);  // would overrun the buffers: the host rejects the tree
    return;
  }
  pt::WideChild wc[8];
  GBox parent;
  for (int a = 0; a < 3; a++) {
    parent.lo[a] = 3.0e38f;
    parent.hi[a] = -3.0e38f;
  }
  uint32_t off = 0, rank = 0;
  for (int k = 0; k < nk; k++) {
    GBox b = ref_box(T, kids[k]);
    parent = box_union(parent, b);
    for (int a = 0; a < 3; a++) {
      wc[k].box.lo[a] = b.lo[a];
      wc[k].box.hi[a] = b.hi[a];
    }
    if (cnts[k] == 0) {
      wc[k].internal = true;
      wc[k].count = 0;
      wc[k].prim_off = 0;
      qout[qbase + rank] = make_uint2(kids[k], child_base + rank);
      rank++;
    } else {
      wc[k].internal = false;
      wc[k].count = cnts[k];
      wc[k].prim_off = off;
      uint32_t pr[3];
      if (gather_small(T, sorted_prim, kids[k], pr) != (int)cnts[k]) {
        atomicOr(&out.counters[3], 4u);
        return;
      }
      for (uint32_t q = 0; q < cnts[k]; q++) {
        uint32_t dst = prim_base + off + q;
        out.rec_out[3 * dst] = rec_in[3 * pr[q]];
        out.rec_out[3 * dst + 1] = rec_in[3 * pr[q] + 1];
        out.rec_out[3 * dst + 2] = rec_in[3 * pr[q] + 2];
        out.leaf_of_id[pr[q]] = dst;
      }
      off += cnts[k];
    }
  }
  pt::Box pb;
  for (int a = 0; a < 3; a++) {
    pb.lo[a] = parent.lo[a];
    pb.hi[a] = parent.hi[a];
  }
  uint32_t words[20];
  pt::encode_node_dev(pb, wc, nk, child_base, prim_base, words);
  uint4* dst = out.nodes + 5 * (size_t)it.y;
  for (int w = 0; w < 5; w++)
    dst[w] = make_uint4(words[4 * w], words[4 * w + 1], words[4 * w + 2], words[4 * w + 3]);
}

// leaf boxes in sorted (Morton) order
__global__ void k_gather_boxes(const float4* lo, const float4* hi, const uint32_t* order, uint32_t n,
                               float4* slo, float4* shi) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t p = order[i];
  slo[i] = lo[p];
  shi[i] = hi[p];
}

// Carves the builder's scratch arrays out of one device arena that persists
// across builds (grown only when a scene needs more), so a commit makes no
// allocation once the arena fits.
struct Carve {
  unsigned char* base;
  size_t off;
  template <typename T>
  void take(T** p, size_t n) {
    off = (off + 255) & ~(size_t)255;
    *p = base ? (T*)(base + off) : nullptr;
    off += (n ? n : 1) * sizeof(T);
  }
};

// Structural check, per node: the rules of check_node8, counting in cover
// how often each leaf position is referenced.
__global__ void __launch_bounds__(256) k_check_nodes(const uint4* __restrict__ nodes,
                                                     uint32_t nn, uint32_t n,
                                                     uint32_t* __restrict__ cover,
                                                     uint32_t* err) {
  const uint32_t k = blockIdx.x * 256u + threadIdx.x;
  if (k >= nn) return;
  const uint4 a = nodes[5 * (size_t)k], b = nodes[5 * (size_t)k + 1];
  const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};  // words 3..7 are read
  const bool ok = pt::check_node8(w, k, nn, n, [cover](uint64_t pi) {
    atomicAdd(&cover[pi], 1u);
    return true;
  });
  if (!ok) atomicOr(err, 8u);
}

// Counts in ids how often each leaf position is some primitive's position.
__global__ void __launch_bounds__(256) k_check_ids(const uint32_t* __restrict__ leaf_of_id,
                                                   uint32_t n, uint32_t* __restrict__ ids,
                                                   uint32_t* err) {
  const uint32_t i = blockIdx.x * 256u + threadIdx.x;
  if (i >= n) return;
  const uint32_t p = leaf_of_id[i];
  if (p >= n)
    atomicOr(err, 8u);
  else
    atomicAdd(&ids[p], 1u);
}

// Every leaf position must be covered by exactly one leaf slot and be the
// position of exactly one primitive.
__global__ void __launch_bounds__(256) k_check_cover(const uint32_t* __restrict__ cover,
                                                     const uint32_t* __restrict__ ids, uint32_t n,
                                                     uint32_t* err) {
  const uint32_t i = blockIdx.x * 256u + threadIdx.x;
  if (i < n && (cover[i] != 1u || ids[i] != 1u)) atomicOr(err, 8u);
}

}  // namespace

namespace pt {

// Builds the BVH8 of n primitive records (call order, on the device) into
// d_nodes / d_rec_out / d_leaf_of_id (allocated by the caller: n nodes,
// n records, n ids).  Returns the number of nodes and the depth (depth < 0:
// the collapse met an inconsistent tree and stopped before overrunning a
// buffer; -depth: 1 bad count, 2 capacity, 4 leaf gather mismatch; 8: the
// finished tree broke a structural rule).
cudaError_t build_bvh8_gpu(const float4* d_rec, const float4* d_xforms, uint32_t n,
                           uint4* d_nodes, float4* d_rec_out, uint32_t* d_leaf_of_id,
                           uint32_t* out_nodes, int* out_depth, int treelet_rounds, int width,
                           float cam_t0, float cam_t1, BuildArena* arena, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (width < 2 || width > 8) width = 8;
  float4 *lo = nullptr, *hi = nullptr, *ilo = nullptr, *ihi = nullptr, *slo = nullptr,
         *shi = nullptr;
  uint32_t *keys = nullptr, *vals = nullptr, *keys2 = nullptr, *vals2 = nullptr, *left = nullptr,
           *right = nullptr, *pint = nullptr, *pleaf = nullptr, *flags = nullptr, *counters = nullptr;
  unsigned int* cbox = nullptr;
  uint2 *qa = nullptr, *qb = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  uint32_t ni = n > 1 ? n - 1 : 1;
  int depth = 0;
  uint32_t h_cnt[4] = {1, 0, 0, 0};
  unsigned int h_cbox[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
#define BV(x)                         \
  do {                                \
    e = (x);                          \
    if (e != cudaSuccess) goto done;  \
  } while (0)
  // the radix sort's temporary size (a query: no sorting, no allocation)
  BV(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, vals, vals2, (int)n, 0, 30,
                                     st));
  {
    Carve cv{nullptr, 0};
    for (int pass = 0; pass < 2; pass++) {
      cv.off = 0;
      cv.take(&lo, n);
      cv.take(&hi, n);
      cv.take(&slo, n);
      cv.take(&shi, n);
      cv.take(&ilo, ni);
      cv.take(&ihi, ni);
      cv.take(&keys, n);
      cv.take(&vals, n);
      cv.take(&keys2, n);
      cv.take(&vals2, n);
      cv.take(&left, ni);
      cv.take(&right, ni);
      cv.take(&pint, ni);
      cv.take(&pleaf, n);
      cv.take(&flags, ni);
      cv.take(&counters, 4);
      cv.take(&cbox, 6);
      cv.take(&qa, n);
      cv.take(&qb, n);
      unsigned char* t8 = nullptr;
      cv.take(&t8, tmp_bytes);
      tmp = t8;
      if (pass == 0 && cv.off > arena->bytes) {  // grow the arena
        if (arena->p) cudaFree(arena->p);
        arena->p = nullptr;
        arena->bytes = 0;
        BV(cudaMalloc(&arena->p, cv.off));
        arena->bytes = cv.off;
      }
      cv.base = (unsigned char*)arena->p;
    }
  }
  BV(cudaMemcpyAsync(cbox, h_cbox, sizeof(h_cbox), cudaMemcpyHostToDevice, st));
  {
    uint32_t g = (n + 255) / 256;
    k_bounds<<<g, 256, 0, st>>>(d_rec, d_xforms, n, cam_t0, cam_t1, lo, hi, cbox);
    k_morton<<<g, 256, 0, st>>>(lo, hi, n, cbox, keys, vals);
    BV(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, vals, vals2, (int)n, 0, 30, st));
    // leaf bounds in sorted order
    BV(cudaMemsetAsync(pint, 0xff, ni * 4, st));
    BV(cudaMemsetAsync(pleaf, 0xff, (size_t)n * 4, st));
    Tree T;
    T.left = left;
    T.right = right;
    T.parent_int = pint;
    T.parent_leaf = pleaf;
    T.ilo = ilo;
    T.ihi = ihi;
    T.llo = slo;
    T.lhi = shi;
    T.flags = flags;
    k_gather_boxes<<<g, 256, 0, st>>>(lo, hi, vals2, n, slo, shi);
    if (n > 1) {
      k_karras<<<(ni + 255) / 256, 256, 0, st>>>(keys2, (int)n, left, right, pint, pleaf);
      for (int round = 0; round <= treelet_rounds; round++) {
        BV(cudaMemsetAsync(flags, 0, ni * 4, st));
        k_bottom_up<<<g, 256, 0, st>>>(T, (int)n, round > 0 ? 1 : 0);
      }
    }
    // collapse, level by level
    BV(cudaMemcpyAsync(counters, h_cnt, sizeof(h_cnt), cudaMemcpyHostToDevice, st));
    uint2 root = make_uint2(n > 1 ? 0u : (0u | LEAF_BIT), 0u);
    BV(cudaMemcpyAsync(qa, &root, sizeof(root), cudaMemcpyHostToDevice, st));
    uint32_t nq = 1;
    CollapseOut co{d_nodes, d_rec_out, d_leaf_of_id, counters, n};
    while (nq) {
      depth++;
      BV(cudaMemsetAsync(counters + 2, 0, 4, st));
      k_collapse<<<(nq + 127) / 128, 128, 0, st>>>(T, vals2, d_rec, qa, nq, qb, co, width);
      BV(cudaMemcpyAsync(h_cnt, counters, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
      BV(cudaStreamSynchronize(st));
      nq = h_cnt[3] ? 0u : h_cnt[2];
      uint2* tq = qa;
      qa = qb;
      qb = tq;
    }
    // structural check of the result (keys and vals are free by now)
    if (!h_cnt[3] && n > 0) {
      const uint32_t nn = h_cnt[0];
      if (nn == 0 || nn > n) {
        h_cnt[3] = 8;
      } else {
        BV(cudaMemsetAsync(keys, 0, (size_t)n * 4, st));
        BV(cudaMemsetAsync(vals, 0, (size_t)n * 4, st));
        k_check_nodes<<<(nn + 255) / 256, 256, 0, st>>>(d_nodes, nn, n, keys, counters + 3);
        k_check_ids<<<g, 256, 0, st>>>(d_leaf_of_id, n, vals, counters + 3);
        k_check_cover<<<g, 256, 0, st>>>(keys, vals, n, counters + 3);
        BV(cudaMemcpyAsync(&h_cnt[3], counters + 3, 4, cudaMemcpyDeviceToHost, st));
        BV(cudaStreamSynchronize(st));
      }
    }
    BV(cudaGetLastError());
    *out_nodes = h_cnt[3] ? 0u : h_cnt[0];
    *out_depth = h_cnt[3] ? -(int)h_cnt[3] : depth;  // < 0: the collapse found an inconsistent tree
  }
done:
#undef BV
  return e;
}

}  // namespace pt
