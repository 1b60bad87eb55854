/*
 * pt_trace.cu - BVH8 traversal kernels for sm_103a: the closest hit of
 * extension rays (replaces rtTrace into the scene's top object), the shadow
 * ray of Direct_Light (programs/hit.cu:16-24 under the closest-hit rule), the
 * occlusion rays of the consistent mode and first-hit queries.
 *
 * The BVH8 (csrc/bvh_gpu.cu, csrc/bvh_host.cpp) stores 80-byte nodes with
 * 8-bit quantised child boxes and 48-byte primitive records; rays come from
 * the wavefront's path and shadow arrays (pt_kernels.cu), results go back to
 * them.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include "pt_device.cuh"
#include "pt_internal.h"
#include "pt_wave.cuh"

using namespace ptd;

// ------------------------------------------------------------ BVH8 trace --
// Closest hit through the BVH8 with warp-collective leaf tests.
//
// Each lane traverses its own ray node by node: into the nearest hit
// internal child, with one stack entry per level for the group of the
// node's other hit internal children (the second nearest taken first, the
// rest in slot order: a node step hits at most two internal children in
// nearly every case, so two running minima replace a full sort).  Primitive
// tests are not run by the lane that reaches a leaf: after every node step
// the warp gathers all (ray, primitive) pairs its lanes produced into shared
// memory and the 32 lanes test them together, merging the results per ray
// with a 64-bit atomicMin on (t, primitive id) - the order-independent
// closest-hit rule of the oracle.  Per-lane leaf loops of 1..24 triangles
// would otherwise serialise the warp.  Lanes whose rays are done wait until
// enough of the warp is idle, then write their results and take new rays
// together (persistent threads), and a stack group whose nearest child lies
// beyond the closest hit is dropped without visiting it.
//
// One node step yields at most PT_MAX_PAIRS pairs per warp (the builders
// bound the primitives under one node's leaf children by 24); they are
// tested in rounds of PT_PAIR_CAP, so the pair buffer stays small and more
// blocks fit on an SM.
#define PT_MAX_PAIRS (32 * 24)
#ifndef PT_PAIR_CAP
#define PT_PAIR_CAP (32 * 8)
#endif

struct WarpShared {
  float4 ro[32];                  // origin, tmin
  float4 rd[32];                  // direction, tmax
  float4 wt[32];                  // watertight-test constants Sx, Sy, Sz, axes
  unsigned long long best[32];    // (t bits << 32) | primitive id
  float tm[32];                   // the ray's path time (scenes with moving spheres)
  uint32_t pair_prim[PT_PAIR_CAP];
  uint8_t pair_owner[PT_PAIR_CAP];
};

__device__ __forceinline__ uint32_t byte_of(uint32_t w, int i) { return (w >> (8 * i)) & 0xffu; }

// Three-input max / min (one instruction each on sm_100+) and the paired
// FP32 fused multiply-add: a node step evaluates 8 children x 3 axes of
// (near, far) slab distances, so pairs share one instruction.
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
// (a.x * s + t, a.y * s + t), each rounded once.
__device__ __forceinline__ float2 fma2s(float ax, float ay, float s, float t) {
  unsigned long long a, b, c, d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(a) : "f"(ax), "f"(ay));
  asm("mov.b64 %0, {%1, %1};" : "=l"(b) : "f"(s));
  asm("mov.b64 %0, {%1, %1};" : "=l"(c) : "f"(t));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(d));
  return r;
}

__device__ __forceinline__ WtRay wt_unpack(float4 w) {
  WtRay r;
  uint32_t k = __float_as_uint(w.w);
  r.kx = (int)(k & 3u);
  r.ky = (int)((k >> 2) & 3u);
  r.kz = (int)((k >> 4) & 3u);
  r.Sx = w.x;
  r.Sy = w.y;
  r.Sz = w.z;
  return r;
}

// Candidate of one primitive for a world-space ray (object space inside);
// MOTION: spheres may move (at the ray's `time`), else every sphere is static.
template <bool MOTION>
__device__ __forceinline__ bool prim_test(const DevScene& S, const PrimRec& p, V3 o, V3 d,
                                          const WtRay& wt, float tmin, float tmax, float& t,
                                          float& bu, float& bv, float time) {
  bu = bv = 0.f;
  if (S.tri_only) return tri_candidate(p, o, wt, tmin, tmax, t, bu, bv);
  int type = prim_type(p);
  if (type == PT_PRIM_TRIANGLE) return tri_candidate(p, o, wt, tmin, tmax, t, bu, bv);
  V3 oo = o, dd = d;
  int xf = prim_xform(p);
  if (xf >= 0) {
    const float4* I = S.xforms + 6 * xf + 3;
    oo = xpoint(I, o);
    dd = xvector(I, d);
  }
  if (type == PT_PRIM_SPHERE)
    return sphere_candidate_at(p, MOTION ? sphere_center(p, time) : v3(p.r0.x, p.r0.y, p.r0.z), oo,
                               dd, tmin, tmax, t);
  if (type == PT_PRIM_RECT) return rect_candidate(p, oo, dd, tmin, tmax, t);
  return box_candidate(p, oo, dd, tmin, tmax, t);
}

struct FirstHitOut {
  uint32_t* prim;
  uint32_t* mat;
  float* t;
  int width, height, frame;
  uint32_t* err;
};

#ifndef PT_ANYHIT_NEAREST
#define PT_ANYHIT_NEAREST 1  // occlusion rays enter the nearest child first
#endif

// BATCH: rays of several scenes; each starts at its scene's root node (the
// scene index is in the path state word st.z).  MOTION: the scene has moving
// spheres, so each ray carries its path's time (other scenes do without).
template <int MODE, bool COUNT, bool BATCH, bool MOTION>
__global__ void __maxnreg__(PT_TRACE_MAXREG)
    k_trace_t(DevScene S, WaveState W, const WaveCtl* __restrict__ ctlp, int max_stack,
              FirstHitOut fo, BatchRefs br, int refetch) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  WarpShared& ws = ((WarpShared*)smem)[threadIdx.x >> 5];
  unsigned char* stk_base = smem + (blockDim.x >> 5) * sizeof(WarpShared);
  uint2* stk = (uint2*)stk_base + threadIdx.x;
  float* stkt = (float*)((uint2*)stk_base + (size_t)max_stack * blockDim.x) + threadIdx.x;
  const int bd = blockDim.x;

  uint32_t n;
  WaveCounters c;
  constexpr bool consistent = MODE == TRACE_OCCLUDED;
  constexpr bool SHADOWRAY = MODE == TRACE_SHADOW || MODE == TRACE_OCCLUDED;
  if (MODE == TRACE_EXT) {
    c = *W.ctr;
    n = c.n_cur + gen_count(c, *ctlp, (uint32_t)W.slots);
  } else if (SHADOWRAY) {
    n = W.ctr->n_shadow;
  } else {
    n = (uint32_t)fo.width * (uint32_t)fo.height;
  }
  // rays are handed out to warps in arrival order from a per-launch counter
  // (first-hit queries: a fixed grid-stride assignment)
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t* take = MODE == TRACE_EXT ? &W.ctr->ray_next[0] : (SHADOWRAY ? &W.ctr->ray_next[1] : nullptr);
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool started = false;
  uint32_t nn = 0, np = 0;

  // per-lane ray state (the direction and tmax of a lane's ray live in the
  // warp's shared copy, ws.rd[lane]: the node tests need only o, tmin and
  // the reciprocal direction)
  const uint32_t parity = MODE == TRACE_EXT ? c.parity : 0u;
  V3 o = v3(0.f);
  float tmin = 0.f, ix = 0.f, iy = 0.f, iz = 0.f, tbest = 0.f;
  bool negx = false, negy = false, negz = false;
  uint32_t cur = 0, best_id = PT_NO_HIT;
  int sp = 0;
  bool active = false;

  // loads ray i into o, d, tmin, tmax
  auto load_ray = [&](V3& d, float& tmax) {
    if (MODE == TRACE_EXT) {
      float4 ro = W.path[parity].ray_o[i], rdv = W.path[parity].ray_d[i];
      o = f4xyz(ro);
      d = f4xyz(rdv);
      tmin = ro.w;
      tmax = rdv.w;
    } else if (SHADOWRAY) {
      o = f4xyz(W.sh.P[i]);
      d = f4xyz(W.sh.Wi[i]);
      tmin = 1e-3f;
      tmax = consistent ? W.sh.C[i].w : PT_RAY_TMAX;
    } else {
      uint32_t x = i % (uint32_t)fo.width, y = i / (uint32_t)fo.width;
      uint32_t seed = tea64((uint32_t)fo.width * y + x, (uint32_t)fo.frame);
      Ray3 r = camera_ray(S.cam, x, y, fo.width, fo.height, seed);
      o = v3(r.o.x, r.o.y, r.o.z);
      d = v3(r.d.x, r.d.y, r.d.z);
      tmin = 1e-6f;
      tmax = PT_RAY_TMAX;
      if (MOTION)  // color()'s prd.time, programs/raygen.cu:69
        ws.tm[lane] = S.cam.time0 + rnd(seed) * (S.cam.time1 - S.cam.time0);
    }
  };

  auto finish = [&](V3 d, float tmax) {
    if (MODE == TRACE_EXT) {
      float4 h = make_float4(tmax, 0.f, 0.f, __uint_as_float(PT_NO_HIT));
      if (best_id != PT_NO_HIT) {
        uint32_t leaf = __ldg(S.leaf_of_id + best_id);
        PrimRec p = load_prim(S.prims, leaf);
        float t = tbest, bu = 0.f, bv = 0.f;
        if (prim_type(p) == PT_PRIM_TRIANGLE) tri_candidate(p, o, wt_setup(d), tmin, tmax, t, bu, bv);
        h = make_float4(tbest, bu, bv, __uint_as_float(leaf));
      }
      W.hit[i] = h;
    } else if (SHADOWRAY) {
      bool occluded = true;
      if (consistent) {
        occluded = best_id != PT_NO_HIT;  // anything before the light
      } else if (best_id != PT_NO_HIT) {
        PrimRec p = load_prim(S.prims, __ldg(S.leaf_of_id + best_id));
        bool is_light = S.mats[prim_material(p)].type == PT_MAT_DIFFUSE_LIGHT;
        occluded = !(is_light && dot(f4xyz(W.sh.N[i]), d) > 0.f);
      }
      W.sh.Wi[i].w = occluded ? 1.f : 0.f;
    } else {
      if (best_id == PT_NO_HIT) {
        fo.prim[i] = PT_NO_HIT;
        fo.mat[i] = PT_NO_HIT;
        fo.t[i] = 0.f;
      } else {
        PrimRec p = load_prim(S.prims, __ldg(S.leaf_of_id + best_id));
        fo.prim[i] = best_id;
        fo.mat[i] = prim_material(p);
        fo.t[i] = tbest;
      }
    }
  };

  auto finish_traced = [&]() {
    float4 rdv = ws.rd[lane];
    finish(f4xyz(rdv), rdv.w);
  };

  bool idle = true;   // wants a ray (finished one, or none taken yet)
  bool done = false;  // traced a ray whose result is not written yet
  // a traversal ends: the result is written with the warp's next batch of
  // fetches, when most lanes do the same work together
  auto end_ray = [&]() {
    active = false;
    idle = true;
    done = true;
  };
  // loads ray i (< n) and sets up its traversal
  auto fetch = [&]() {
    // a ray with a NaN in its origin or direction hits nothing (every
    // primitive test fails or yields a NaN distance, which never wins the
    // closest-hit minimum), and neither does any ray of an empty scene: both
    // end here, without a traversal (a NaN ray would pass every box test)
    V3 d;
    float tmax;
    load_ray(d, tmax);
    bool nan = !(o.x == o.x && o.y == o.y && o.z == o.z && d.x == d.x && d.y == d.y &&
                 d.z == d.z);
    if (nan || S.num_prims == 0) {
      best_id = PT_NO_HIT;
      tbest = tmax;
      finish(d, tmax);
      active = false;
      idle = true;
      return;
    }
    active = true;
    const float eps = 1e-18f;
    float dx = fabsf(d.x) < eps ? copysignf(eps, d.x) : d.x;
    float dy = fabsf(d.y) < eps ? copysignf(eps, d.y) : d.y;
    float dz = fabsf(d.z) < eps ? copysignf(eps, d.z) : d.z;
    ix = 1.0f / dx;
    iy = 1.0f / dy;
    iz = 1.0f / dz;
    negx = ix < 0.f;
    negy = iy < 0.f;
    negz = iz < 0.f;
    WtRay w = wt_setup(d);
    ws.ro[lane] = make_float4(o.x, o.y, o.z, tmin);
    ws.rd[lane] = make_float4(d.x, d.y, d.z, tmax);
    ws.wt[lane] = make_float4(w.Sx, w.Sy, w.Sz,
                              __uint_as_float((uint32_t)w.kx | ((uint32_t)w.ky << 2) |
                                              ((uint32_t)w.kz << 4)));
    tbest = tmax;
    best_id = PT_NO_HIT;
    ws.best[lane] = ((unsigned long long)__float_as_uint(tmax) << 32) | 0xffffffffull;
    if (MOTION && MODE != TRACE_FIRST)  // the path's time rides in throughput.w
      ws.tm[lane] = MODE == TRACE_EXT ? W.path[parity].thr[i].w : W.sh.thr[i].w;
    cur = S.root;
    if (BATCH) {
      uint32_t z = MODE == TRACE_EXT ? W.path[parity].st[i].z : W.sh.st[i].z;
      cur = __ldg(br.roots + (z >> PT_ST_SCENE_SHIFT));
    }
    sp = 0;
  };

  while (true) {
    // idle lanes take and load their next rays together once `refetch`
    // lanes wait (or nothing else runs), so the warp pays one load latency
    // per batch; a lane whose index is past the end has no more work (the
    // counter only grows)
    uint32_t busy = __ballot_sync(0xffffffffu, active);
    uint32_t waiting = __ballot_sync(0xffffffffu, idle);
    if (waiting && (__popc(waiting) >= refetch || busy == 0)) {
      if (done) {
        finish_traced();
        done = false;
      }
      if (MODE == TRACE_FIRST) {
        if (idle) {
          if (started) i += stride;
          started = true;
        }
      } else {
        const int leader = __ffs(waiting) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(take, (uint32_t)__popc(waiting));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (idle) i = base + (uint32_t)__popc(waiting & ((1u << lane) - 1u));
      }
      if (idle) {
        idle = false;
        if (i < n) fetch();
      }
      busy = __ballot_sync(0xffffffffu, active);
      if (!busy) {
        if (__ballot_sync(0xffffffffu, idle)) continue;  // only rays that ended at load
        break;
      }
    }
    if (!busy) break;
    // ---- node step: the eight child boxes of each active lane's node.
    // Internal children fill the low slots, slot == offset of the child node
    // from child_base; leaf children follow.
    uint32_t ihit = 0, leafmask = 0, pbase = 0, mlo = 0, mhi = 0, child_base = 0;
    // the two nearest hit internal children: entry distance (tn >= 0, so its
    // bits order like the value) with the slot in the low 3 bits
    uint32_t k1 = 0xffffffffu, k2 = 0xffffffffu;
    if (active) {
      const uint4* nptr = S.nodes + 5 * (size_t)cur;
      uint4 n0 = __ldg(nptr), n1 = __ldg(nptr + 1), n2 = __ldg(nptr + 2), n3 = __ldg(nptr + 3),
            n4 = __ldg(nptr + 4);
      if (COUNT) nn++;
      child_base = n1.x;
      pbase = n1.y;
      mlo = n1.z;
      mhi = n1.w;
      const uint32_t im = n0.w >> 24;
      // child bound q (8 bits) is read as the float f = 1 + q * 2^-15 built by
      // one byte permute; t = q*a + b = f*A + B with A = 2^15 a, B = b - A
      float sx = __uint_as_float((n0.w & 0xffu) << 23);
      float sy = __uint_as_float(((n0.w >> 8) & 0xffu) << 23);
      float sz = __uint_as_float(((n0.w >> 16) & 0xffu) << 23);
      float Ax = 32768.0f * (sx * ix), Ay = 32768.0f * (sy * iy), Az = 32768.0f * (sz * iz);
      float Bx = (__uint_as_float(n0.x) - o.x) * ix - Ax;
      float By = (__uint_as_float(n0.y) - o.y) * iy - Ay;
      float Bz = (__uint_as_float(n0.z) - o.z) * iz - Az;
      uint32_t nx0 = negx ? n3.z : n2.x, nx1 = negx ? n3.w : n2.y;
      uint32_t fx0 = negx ? n2.x : n3.z, fx1 = negx ? n2.y : n3.w;
      uint32_t ny0 = negy ? n4.x : n2.z, ny1 = negy ? n4.y : n2.w;
      uint32_t fy0 = negy ? n2.z : n4.x, fy1 = negy ? n2.w : n4.y;
      uint32_t nz0 = negz ? n4.z : n3.x, nz1 = negz ? n4.w : n3.y;
      uint32_t fz0 = negz ? n3.x : n4.z, fz1 = negz ? n3.y : n4.w;
      float tlim = tbest * 1.0000005f;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const uint32_t sel = 0x7604u | ((uint32_t)(k & 3) << 4);
        float2 tx = fma2s(__uint_as_float(__byte_perm(k < 4 ? nx0 : nx1, 0x3F800000u, sel)),
                          __uint_as_float(__byte_perm(k < 4 ? fx0 : fx1, 0x3F800000u, sel)), Ax, Bx);
        float2 ty = fma2s(__uint_as_float(__byte_perm(k < 4 ? ny0 : ny1, 0x3F800000u, sel)),
                          __uint_as_float(__byte_perm(k < 4 ? fy0 : fy1, 0x3F800000u, sel)), Ay, By);
        float2 tz = fma2s(__uint_as_float(__byte_perm(k < 4 ? nz0 : nz1, 0x3F800000u, sel)),
                          __uint_as_float(__byte_perm(k < 4 ? fz0 : fz1, 0x3F800000u, sel)), Az, Bz);
        float tn = max3f(tx.x, ty.x, fmaxf(tz.x, tmin));
        float tf = min3f(tx.y, ty.y, fminf(tz.y, tlim));
        // an empty slot (meta 0) has an inverted box and fails here; were it
        // to pass (infinite slab distances), it is a leaf of no primitives.
        if (tn <= tf) {
          if ((im >> k) & 1u) {
            const uint32_t key = (__float_as_uint(tn) & 0xfffffff8u) | (uint32_t)k;
            k2 = min(k2, max(k1, key));
            k1 = min(k1, key);
            ihit |= 1u << k;
          } else {
            leafmask |= 1u << k;
          }
        }
      }
    }
    // ---- next node, chosen before the primitive tests: the nearest hit
    // internal child, the others pushed as one group (closest hit: in
    // near-to-far order with the distance of the nearest; occlusion: as a
    // mask).  With no internal child hit, a closest-hit ray pops after the
    // tests, which may shorten it and so drop groups beyond the new hit.
    const int nint = __popc(ihit);
    bool pop = false;
    float tnext = 0.f;
    if (active) {
      if (consistent) {
        if (ihit) {
          uint32_t b = (uint32_t)(__ffs(ihit) - 1);
          if (PT_ANYHIT_NEAREST) b = k1 & 7u;
          cur = child_base + b;
          const uint32_t rest = ihit & ~(1u << b);
          if (rest) {
            if (sp >= max_stack) {
              atomicOr(&W.ctr->error, 1u);
              sp = 0;  // abandon this ray (the host reports the error)
              end_ray();
            } else {
              stk[sp * bd] = make_uint2(child_base, rest);
              sp++;
            }
          }
        } else if (sp > 0) {
          uint2 e = stk[(sp - 1) * bd];
          cur = e.x + (uint32_t)(__ffs(e.y) - 1);
          e.y &= e.y - 1;
          if (e.y == 0) sp--;
          else stk[(sp - 1) * bd].y = e.y;
        } else {
          end_ray();
        }
      } else if (nint >= 1) {
        cur = child_base + (k1 & 7u);
        tnext = __uint_as_float(k1 & 0xfffffff8u);
        if (nint > 1) {
          // pending group: the other hit children as a slot mask, the second
          // nearest marked to be taken first (the rest in slot order), and
          // the entry distance of the second nearest, below every one of them
          if (sp >= max_stack) {
            atomicOr(MODE == TRACE_FIRST ? fo.err : &W.ctr->error, 1u);
            sp = 0;  // abandon this ray (the host reports the error)
            end_ray();
          } else {
            stk[sp * bd] = make_uint2(child_base, (ihit & ~(1u << (k1 & 7u))) | ((k2 & 7u) << 8) | 0x800u);
            stkt[sp * bd] = __uint_as_float(k2 & 0xfffffff8u);
            sp++;
          }
        }
      } else {
        pop = true;
      }
    }
    // ---- warp-collective primitive tests of the hit leaves (also of a lane
    // whose ray ended above: its leaves of this node still count).  pm: the
    // lane's primitives as bits over the node's range, bit j = record
    // pbase + j (a node's leaves hold at most 24 primitives).
    uint32_t pm = 0;
    {
      uint32_t m = leafmask;
      while (m) {
        const int k = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t meta = (k < 4 ? mlo : mhi) >> (8 * (k & 3));
        pm |= ((1u << ((meta >> 5) & 7u)) - 1u) << (meta & 31u);
      }
    }
    if (__any_sync(0xffffffffu, pm != 0)) {
      const uint32_t cnt = __popc(pm);
      const uint32_t total = __reduce_add_sync(0xffffffffu, cnt);
      const uint32_t mx = __reduce_max_sync(0xffffffffu, cnt);
      if (mx * 32u <= 2u * total) {
        // balanced: each lane tests its own primitives (at least half the
        // lane-slots do work)
        if (pm) {
          WtRay wt = wt_unpack(ws.wt[lane]);
          unsigned long long bk = ws.best[lane];
          const float4 rdv = ws.rd[lane];
          uint32_t m = pm;
          while (m) {
            const int j = __ffs(m) - 1;
            m &= m - 1;
            PrimRec p = load_prim(S.prims, pbase + (uint32_t)j);
            if (COUNT) np++;
            float t, bu, bv;
            if (prim_test<MOTION>(S, p, o, f4xyz(rdv), wt, tmin, rdv.w, t, bu, bv,
                                  MOTION ? ws.tm[lane] : 0.f)) {
              unsigned long long key = ((unsigned long long)__float_as_uint(t) << 32) | prim_id(p);
              bk = min(bk, key);
            }
          }
          ws.best[lane] = bk;
          tbest = __uint_as_float((uint32_t)(bk >> 32));
          best_id = (uint32_t)bk;
        }
      } else {
        // unbalanced: spread the (ray, primitive) pairs over the warp
        uint32_t incl = cnt;
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
          uint32_t t = __shfl_up_sync(0xffffffffu, incl, dd);
          if (lane >= dd) incl += t;
        }
        const uint32_t off0 = incl - cnt;
        for (uint32_t r0 = 0; r0 < total; r0 += PT_PAIR_CAP) {
          // this round's pairs: [r0, r0 + PT_PAIR_CAP) of the warp's list
          if (pm && off0 < r0 + PT_PAIR_CAP && off0 + cnt > r0) {
            uint32_t off = off0 - r0;  // wraps below the round: skipped
            uint32_t m = pm;
            while (m) {
              const int j = __ffs(m) - 1;
              m &= m - 1;
              if (off < PT_PAIR_CAP) {
                ws.pair_prim[off] = pbase + (uint32_t)j;
                ws.pair_owner[off] = (uint8_t)lane;
              }
              off++;
            }
          }
          __syncwarp();
          const uint32_t nr = min(total - r0, (uint32_t)PT_PAIR_CAP);
          for (uint32_t j = lane; j < nr; j += 32) {
            uint32_t pi = ws.pair_prim[j];
            uint32_t ow = ws.pair_owner[j];
            PrimRec p = load_prim(S.prims, pi);
            if (COUNT) np++;
            float4 ro = ws.ro[ow], rdv = ws.rd[ow];
            float t, bu, bv;
            if (prim_test<MOTION>(S, p, f4xyz(ro), f4xyz(rdv), wt_unpack(ws.wt[ow]), ro.w, rdv.w, t,
                                  bu, bv, MOTION ? ws.tm[ow] : 0.f)) {
              unsigned long long key = ((unsigned long long)__float_as_uint(t) << 32) | prim_id(p);
              atomicMin(&ws.best[ow], key);
            }
          }
          __syncwarp();
        }
        if (pm) {
          unsigned long long k = ws.best[lane];
          tbest = __uint_as_float((uint32_t)(k >> 32));
          best_id = (uint32_t)k;
        }
      }
    }
    // ---- occlusion rays end at the first confirmed hit before tmax
    if (consistent && active && best_id != PT_NO_HIT) end_ray();
    // ---- closest hit: a chosen child that now lies beyond the hit is
    // dropped; then the deepest pending group not beyond the hit
    if (!consistent && active) {
      const float tlim = tbest * 1.0000005f;
      if (!pop && tnext > tlim) pop = true;
      if (pop) {
        bool found = false;
        while (sp > 0) {
          uint2 e = stk[(sp - 1) * bd];
          if (stkt[(sp - 1) * bd] > tlim) {  // every child of the group starts beyond the hit
            sp--;
            continue;
          }
          uint32_t m = e.y & 0xffu;
          const uint32_t slot = (e.y & 0x800u) ? (e.y >> 8) & 7u : (uint32_t)(__ffs(m) - 1);
          m &= ~(1u << slot);
          cur = e.x + slot;
          if (m == 0) sp--;
          else stk[(sp - 1) * bd].y = m;
          found = true;
          break;
        }
        if (!found) end_ray();
      }
    }
  }
  if (COUNT) {
    atomicAdd(&W.ctr->node_fetches, (unsigned long long)nn);
    atomicAdd(&W.ctr->prim_tests, (unsigned long long)np);
  }
}


// ------------------------------------------------------- host launchers ---
namespace pt {

size_t trace_smem(int max_stack, int block) {
  return (size_t)(block / 32) * sizeof(WarpShared) +
         (size_t)block * max_stack * (sizeof(uint2) + sizeof(float));
}

int trace_blocks_per_sm(int block, size_t smem) {
  int blocks = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &blocks, k_trace_t<TRACE_EXT, false, false, false>, block, smem);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return blocks;
}

// Dynamic shared memory limit of kernel k: the per-block opt-in maximum
// minus its static shared memory.
template <typename K>
static cudaError_t smem_attr(K k, int optin) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, k);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - (int)fa.sharedSizeBytes);
}

template <int MODE, bool MOTION>
static cudaError_t smem_attr_mode(int optin) {
  cudaError_t e;
  if ((e = smem_attr(k_trace_t<MODE, false, false, MOTION>, optin)) != cudaSuccess) return e;
  if ((e = smem_attr(k_trace_t<MODE, true, false, MOTION>, optin)) != cudaSuccess) return e;
  if ((e = smem_attr(k_trace_t<MODE, false, true, MOTION>, optin)) != cudaSuccess) return e;
  return smem_attr(k_trace_t<MODE, true, true, MOTION>, optin);
}

static const int kMaxDev = 64;
static bool g_smem_set[kMaxDev];

cudaError_t set_trace_smem() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kMaxDev && g_smem_set[dev]) return cudaSuccess;
  int optin = 0;
  if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) !=
      cudaSuccess)
    return e;
  if ((e = smem_attr_mode<TRACE_EXT, false>(optin)) != cudaSuccess) return e;
  if ((e = smem_attr_mode<TRACE_SHADOW, false>(optin)) != cudaSuccess) return e;
  if ((e = smem_attr_mode<TRACE_OCCLUDED, false>(optin)) != cudaSuccess) return e;
  if ((e = smem_attr_mode<TRACE_EXT, true>(optin)) != cudaSuccess) return e;
  if ((e = smem_attr_mode<TRACE_SHADOW, true>(optin)) != cudaSuccess) return e;
  if ((e = smem_attr_mode<TRACE_OCCLUDED, true>(optin)) != cudaSuccess) return e;
  if ((e = smem_attr(k_trace_t<TRACE_FIRST, false, false, false>, optin)) != cudaSuccess) return e;
  if ((e = smem_attr(k_trace_t<TRACE_FIRST, false, false, true>, optin)) != cudaSuccess) return e;
  if (dev >= 0 && dev < kMaxDev) g_smem_set[dev] = true;
  return cudaSuccess;
}

template <int MODE, bool BATCH, bool MOTION>
static void launch_mode(bool counters, const DevScene& S, const WaveState& W, const WaveCtl* ctl,
                        int max_stack, const BatchRefs& br, const LaunchCfg& lc, size_t smem,
                        cudaStream_t st) {
  FirstHitOut none{};
  if (counters)
    k_trace_t<MODE, true, BATCH, MOTION><<<lc.trace_grid, lc.trace_block, smem, st>>>(
        S, W, ctl, max_stack, none, br, lc.refetch);
  else
    k_trace_t<MODE, false, BATCH, MOTION><<<lc.trace_grid, lc.trace_block, smem, st>>>(
        S, W, ctl, max_stack, none, br, lc.refetch);
}

template <bool BATCH, bool MOTION>
static void launch_kind(int mode, bool counters, const DevScene& S, const WaveState& W,
                        const WaveCtl* ctl, int max_stack, const BatchRefs& br,
                        const LaunchCfg& lc, size_t smem, cudaStream_t st) {
  if (mode == TRACE_EXT)
    launch_mode<TRACE_EXT, BATCH, MOTION>(counters, S, W, ctl, max_stack, br, lc, smem, st);
  else if (mode == TRACE_SHADOW)
    launch_mode<TRACE_SHADOW, BATCH, MOTION>(counters, S, W, ctl, max_stack, br, lc, smem, st);
  else
    launch_mode<TRACE_OCCLUDED, BATCH, MOTION>(counters, S, W, ctl, max_stack, br, lc, smem, st);
}

void launch_trace(int mode, bool counters, const DevScene& S, const WaveState& W,
                  const WaveCtl* ctl, int max_stack, const BatchRefs* br, const LaunchCfg& lc,
                  cudaStream_t st) {
  const size_t smem = trace_smem(max_stack, lc.trace_block);
  if (br && lc.motion)
    launch_kind<true, true>(mode, counters, S, W, ctl, max_stack, *br, lc, smem, st);
  else if (br)
    launch_kind<true, false>(mode, counters, S, W, ctl, max_stack, *br, lc, smem, st);
  else if (lc.motion)
    launch_kind<false, true>(mode, counters, S, W, ctl, max_stack, BatchRefs{}, lc, smem, st);
  else
    launch_kind<false, false>(mode, counters, S, W, ctl, max_stack, BatchRefs{}, lc, smem, st);
}

void launch_first_hits(const DevScene& S, int w, int h, int frame, uint32_t* prim, uint32_t* mat,
                       float* t, int max_stack, uint32_t* err, int grid, cudaStream_t st) {
  FirstHitOut fo{prim, mat, t, w, h, frame, err};
  WaveState none{};
  if (S.has_motion)
    k_trace_t<TRACE_FIRST, false, false, true>
        <<<grid, PT_TRACE_BLOCK, trace_smem(max_stack, PT_TRACE_BLOCK), st>>>(
            S, none, nullptr, max_stack, fo, BatchRefs{}, 32);
  else
    k_trace_t<TRACE_FIRST, false, false, false>
        <<<grid, PT_TRACE_BLOCK, trace_smem(max_stack, PT_TRACE_BLOCK), st>>>(
            S, none, nullptr, max_stack, fo, BatchRefs{}, 32);
}

}  // namespace pt
