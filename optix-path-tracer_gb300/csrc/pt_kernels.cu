/*
 * pt_kernels.cu - wavefront path tracing kernels for sm_103a.
 *
 * One path = one (pixel, frame) sample of programs/raygen.cu:148-167.  The
 * reference runs each path in one OptiX megakernel thread; here the live
 * paths stream through stage kernels, and new paths top the buffer up to its
 * capacity every iteration (regeneration), so the GPU stays full:
 *
 *   k_generate      renderPixel up to color()'s loop: TEA seed, jitter,
 *                   thin-lens camera ray, time draw (raygen.cu:148-162,50-69)
 *   k_trace_t<EXT>  closest hit through the BVH8 (replaces rtTrace)
 *   k_shade         miss programs, Get_HitRecord, closest-hit programs; the
 *                   NEE of Direct_Light stops at the shadow ray
 *   k_trace_t<SHADOW> shadow rays (programs/hit.cu:16-24, closest-hit rule)
 *   k_finish        rest of Direct_Light (MIS), BSDF continuation
 *   k_advance       counter bookkeeping (one thread)
 * The consistent mode (NEE over lights and the environment with MIS) uses
 * k_shade_c, k_trace_t<OCCLUDED> (any hit before the light ends the ray) and
 * k_finish_c in the same places.  Trace warps take rays from a per-launch
 * counter (ray_next), so no warp sits idle while others still have rays.
 * Path state is kept in queue order: paths that continue are appended,
 * compacted with warp-aggregated atomics (ballot + popc prefix), to the other
 * buffer of a ping-pong pair, so every kernel streams its arrays
 * contiguously.  Ended paths write their colour to a per-path result slot,
 * and k_accumulate adds results to the accumulator in frame order, so the
 * image does not depend on scheduling.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include "pt_device.cuh"
#include "pt_guide.cuh"
#include "pt_internal.h"
#include "pt_wave.cuh"

using namespace ptd;

// -------------------------------------------------- warp-aggregated push --
__device__ __forceinline__ uint32_t warp_push(uint32_t* counter, bool active) {
  uint32_t mask = __ballot_sync(0xffffffffu, active);
  if (!active) return 0;
  int lane = threadIdx.x & 31;
  int leader = __ffs(mask) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

// ---------------------------------------------------------- path state ----
// st.x = seed, st.y = path id in the chunk, st.z = depth | prevSpecular<<16 |
// scene<<17 (batch), st.w = pdf of the last BSDF sample (consistent mode)

// Depth limit and Russian roulette of a path (per render, or per scene of a
// batch).
struct PathCtl {
  int max_depth, rr_enable, rr_depth;
};
__device__ __forceinline__ void finalize_path(const WaveState& W, uint32_t pid, V3 col) {
  // de_nan, programs/raygen.cu:126-134
  if (!(col.x == col.x)) col.x = 0.f;
  if (!(col.y == col.y)) col.y = 0.f;
  if (!(col.z == col.z)) col.z = 0.f;
  __stcs(&W.results[pid], make_float4(col.x, col.y, col.z, 1.f));
}

// raygen.cu:81-122 after the closest-hit program: event dispatch, next
// ray, Russian roulette, depth limit.
struct Tail {
  int event;  // 0 bounced, 1 cancelled, 2 hit light
  bool isSpecular;
  V3 origin, direction;
};

// Ends the path or appends it, compacted, to the next path buffer.  All
// lanes of the warp call it (the append is a warp-aggregated atomic).  tm:
// the path's time (color()'s prd.time), carried in the throughput's w.
__device__ __forceinline__ void path_tail(const WaveState& W, const WaveCounters& c,
                                          const PathCtl& ctl, uint4 st, V3 thr, V3 rad,
                                          const Tail& tl, bool active, float tm) {
  bool cont = false;
  if (active) {
    uint32_t depth = st.z & PT_ST_DEPTH_MASK;
    bool prevSpec = (st.z >> PT_ST_SPEC_BIT) & 1u;
    bool done = false;
    V3 col = v3(0.f);
    if (tl.event == 2) {
      if (depth == 0 || prevSpec) rad += thr;
      col = rad;
      done = true;
    } else if (tl.event == 1) {
      col = rad;
      done = true;
    } else {
      prevSpec = tl.isSpecular;
      if (ctl.rr_enable) {
        float prob = max_component(thr);
        if ((int)depth > ctl.rr_depth) {
          if (rnd(st.x) >= prob) {
            col = rad + thr;
            done = true;
          } else {
            thr *= 1.f / prob;
          }
        }
      }
      if (!done) {
        depth++;
        if ((int)depth >= ctl.max_depth) {
          col = v3(0.f);
          done = true;
        } else {
          cont = true;
          st.z = (st.z & PT_ST_KEEP_MASK) | depth | ((uint32_t)prevSpec << PT_ST_SPEC_BIT);
        }
      }
    }
    if (done) finalize_path(W, st.y, col);
  }
  uint32_t pos = warp_push(&W.ctr->n_next, cont);
  if (cont) {
    const PathBuf& nb = W.path[c.parity ^ 1u];
    nb.ray_o[pos] = make_float4(tl.origin.x, tl.origin.y, tl.origin.z, 1e-3f);
    nb.ray_d[pos] = make_float4(tl.direction.x, tl.direction.y, tl.direction.z, PT_RAY_TMAX);
    nb.thr[pos] = make_float4(thr.x, thr.y, thr.z, tm);
    nb.rad[pos] = make_float4(rad.x, rad.y, rad.z, 0.f);
    nb.st[pos] = st;
  }
}

// ------------------------------------------------------------- kernels ----
// Segment of a batch chunk that holds path `pid` (binary search over the
// segments' first paths).
__device__ __forceinline__ uint32_t find_seg(const BatchSeg* __restrict__ segs, uint32_t lo,
                                             uint32_t hi, uint32_t pid, bool by_pixel) {
  // invariant: segs[lo].off <= pid, answer in [lo, hi)
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    uint32_t off = by_pixel ? segs[mid].pix_off : segs[mid].path_off;
    if (off <= pid) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <bool BATCH>
__global__ void k_generate(DevScene S0, WaveState W, const WaveCtl* __restrict__ ctlp,
                           BatchRefs br) {
  WaveCounters c = *W.ctr;
  WaveCtl ctl = *ctlp;
  uint32_t n = gen_count(c, ctl, (uint32_t)W.slots);
  const PathBuf& pb = W.path[c.parity];
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    uint32_t pos = c.n_cur + j;
    uint32_t pid = (uint32_t)(c.next_path + j);
    uint32_t width = (uint32_t)ctl.width, height = (uint32_t)ctl.height;
    uint32_t wh_m = ctl.wh_m, wh_l = ctl.wh_l, w_m = ctl.w_m, w_l = ctl.w_l;
    uint32_t frame0 = (uint32_t)ctl.frame0, local = pid, scene = 0;
    const DevScene* Sp = &S0;
    if (BATCH) {
      const BatchSeg& sg = br.segs[find_seg(br.segs, ctl.seg_begin, ctl.seg_end, pid, false)];
      scene = sg.scene;
      const BatchScene& B = br.scenes[scene];
      Sp = &B.S;
      width = (uint32_t)B.width;
      height = (uint32_t)B.height;
      wh_m = B.wh_m;
      wh_l = B.wh_l;
      w_m = B.w_m;
      w_l = B.w_l;
      frame0 = sg.frame0;
      local = pid - sg.path_off;
    }
    const DevScene& S = *Sp;
    uint32_t WH = width * height;
    uint32_t fr = fastdiv(local, wh_m, wh_l);
    uint32_t frame = frame0 + fr;
    uint32_t pix = local - fr * WH;
    uint32_t y = fastdiv(pix, w_m, w_l);
    uint32_t x = pix - y * width;
    uint32_t seed = tea64(width * y + x, frame);
    Ray3 r = camera_ray(S.cam, x, y, width, height, seed);
    // color(): prd.time draw, programs/raygen.cu:69
    float tm = S.cam.time0 + rnd(seed) * (S.cam.time1 - S.cam.time0);
    pb.ray_o[pos] = make_float4(r.o.x, r.o.y, r.o.z, 1e-6f);
    pb.ray_d[pos] = make_float4(r.d.x, r.d.y, r.d.z, PT_RAY_TMAX);
    pb.thr[pos] = make_float4(1.f, 1.f, 1.f, tm);
    pb.rad[pos] = make_float4(0.f, 0.f, 0.f, 0.f);
    pb.st[pos] = make_uint4(seed, pid, scene << PT_ST_SCENE_SHIFT, 0u);
  }
}

// Scene and path controls of a path: the render's, or its batch scene's.
template <bool BATCH>
__device__ __forceinline__ const DevScene& path_scene(const DevScene& S0, const BatchRefs& br,
                                                      uint32_t stz) {
  return BATCH ? br.scenes[stz >> PT_ST_SCENE_SHIFT].S : S0;
}
template <bool BATCH>
__device__ __forceinline__ PathCtl path_ctl(const WaveCtl& ctl, const BatchRefs& br,
                                            uint32_t stz) {
  PathCtl pc;
  if (BATCH) {
    const BatchScene& B = br.scenes[stz >> PT_ST_SCENE_SHIFT];
    pc.max_depth = B.max_depth;
    pc.rr_enable = B.rr_enable;
    pc.rr_depth = B.rr_depth;
  } else {
    pc.max_depth = ctl.max_depth;
    pc.rr_enable = ctl.rr_enable;
    pc.rr_depth = ctl.rr_depth;
  }
  return pc;
}

// Direct_Light (programs/materials/light_sample.cuh:36-73) up to the shadow
// ray.  Returns 0: no contribution, stop here; 1: shadow ray queued.
__device__ __forceinline__ int nee_begin(const DevScene& S, uint32_t& seed, V3 P, V3 N,
                                         bool isLight, V3& Wi, float& lightPDF, int& index) {
  int numLights = S.num_lights;
  if (numLights == 0) return 0;
  index = ((int)(rnd(seed) * numLights)) % numLights;
  if (isLight && numLights == 1) return 0;
  GpuLight L = S.lights[index];
  Wi = light_sample(L, P, seed);
  lightPDF = light_pdf(L, P, Wi);
  if (dot(Wi, N) < 0.f) return 0;
  return 1;
}

// programs/materials/light_sample.cuh:76-103: MIS after the shadow test.
__device__ __forceinline__ V3 nee_end(const DevScene& S, const GpuMaterial& m, uint32_t& seed,
                                      V3 P, V3 Wo, V3 N, V3 Wi, float lightPDF, int index,
                                      bool occluded) {
  V3 directLight = v3(0.f);
  if (occluded) return v3(0.f);
  GpuLight L = S.lights[index];
  V3 emission = v3(L.ex, L.ey, L.ez);
  if (lightPDF != 0.f && !isNull(emission)) {
    float matPDF = 0.f;
    V3 matValue = brdf_eval(m, Wo, Wi, N, matPDF);
    if (matPDF != 0.f && !isNull(matValue)) {
      float f = 1u * lightPDF, g = 1u * matPDF;
      float weight = (f * f) / (f * f + g * g);
      directLight += matValue * emission * weight / lightPDF;
    }
  }
  Wi = brdf_sample(m, Wo, N, seed);
  float matPDF = 0.f;
  V3 matValue = brdf_eval(m, Wo, Wi, N, matPDF);
  if (matPDF != 0.f && !isNull(matValue)) {
    lightPDF = light_pdf(L, P, Wi);
    if (!lightPDF || isNull(emission)) return directLight;
    float f = 1u * matPDF, g = 1u * lightPDF;
    float weight = (f * f) / (f * f + g * g);
    directLight += matValue * emission * weight / matPDF;
  }
  return directLight;
}

// Closest-hit continuation after Direct_Light for the NEE materials
// (lambertian.cu:55-72, oren_nayar.cu:56-69, diffuse_light.cu:40-47).
__device__ __forceinline__ void after_nee(const GpuMaterial& m, uint32_t& seed, V3 P, V3 Wo, V3 N,
                                          V3 direct, V3& thr, V3& rad, Tail& tl) {
  rad += thr * direct;
  if (m.type == PT_MAT_DIFFUSE_LIGHT) {
    if (dot(N, Wo) < 0.f) thr *= v3(m.c0x, m.c0y, m.c0z);
    tl.event = 2;
    return;
  }
  V3 Wi = brdf_sample(m, Wo, N, seed);
  float pdf = 0.f;
  V3 attenuation = brdf_eval(m, Wo, Wi, N, pdf);
  tl.event = 0;
  tl.origin = P;
  tl.direction = Wi;
  thr *= clamp3(attenuation / pdf, 0.f, 1.f);
  tl.isSpecular = false;
}

__device__ __forceinline__ V3 env_lookup(const GpuMiss& ms, float u, float v) {
  if (!(u == u) || !(v == v) || fabsf(u) > 1e6f || fabsf(v) > 1e6f) return v3(0.f);
  float x = u * (float)ms.w - 0.5f, y = v * (float)ms.h - 0.5f;
  float fx = floorf(x), fy = floorf(y);
  float ax = x - fx, ay = y - fy;
  int ix0 = (int)fx % ms.w; if (ix0 < 0) ix0 += ms.w;
  int iy0 = (int)fy % ms.h; if (iy0 < 0) iy0 += ms.h;
  int ix1 = ix0 + 1 == ms.w ? 0 : ix0 + 1;
  int iy1 = iy0 + 1 == ms.h ? 0 : iy0 + 1;
  float4 e00 = __ldg(ms.env + iy0 * ms.w + ix0), e10 = __ldg(ms.env + iy0 * ms.w + ix1);
  float4 e01 = __ldg(ms.env + iy1 * ms.w + ix0), e11 = __ldg(ms.env + iy1 * ms.w + ix1);
  V3 c00 = f4xyz(e00), c10 = f4xyz(e10), c01 = f4xyz(e01), c11 = f4xyz(e11);
  return (c00 * (1.f - ax) + c10 * ax) * (1.f - ay) + (c01 * (1.f - ax) + c11 * ax) * ay;
}

// The colours of a textured material at a hit (Get_Parameters of the
// closest-hit programs).  Compiled only into the shading kernels of scenes
// with textures (the TEX variants): untextured shading never computes the
// texture coordinates.
__device__ __forceinline__ void apply_textures(const DevScene& S, GpuMaterial& m, const PrimRec& p,
                                               V3 ro, V3 rd, float t, float bu, float bv,
                                               float tm) {
  HitRecord rec = hit_record(S, p, ro, rd, t, bu, bv, true, tm);
  resolve_textures(S, m, rec.u, rec.v, rec.P, rec.tindex);
}

// programs/miss.cu:30-95; returns the multiplier applied to throughput.
__device__ __forceinline__ V3 miss_color(const GpuMiss& ms, V3 d) {
  if (ms.type == 0) {
    V3 unit_direction = normalize(d);
    float t = 0.5f * (unit_direction.y + 1.f);
    V3 c = (1.f - t) * v3(ms.c1x, ms.c1y, ms.c1z);
    c += t * v3(ms.c2x, ms.c2y, ms.c2z);
    return c;
  }
  if (ms.type == 1) return v3(ms.c1x, ms.c1y, ms.c1z);
  if (ms.type == 3) {
    float theta = pt_atan2f(d.x, d.z);
    float phi = PTM_PI * 0.5f - pt_acosf(d.y);
    float u = (theta + PTM_PI) * (0.5f * (1.0f / PTM_PI));
    float v = 0.5f * (1.f + pt_sinf(phi));
    return env_lookup(ms, u, v);
  }
  float u, v;
  if (ms.spherical) {
    float r = length(d);
    float lon = pt_atan2f(d.z, d.x);
    float lat = pt_acosf(d.y / r);
    u = lon * (1.f / (PI_F * 2.f));
    v = lat * (1.f / PI_F);
  } else {
    float theta = pt_atan2f(d.x, d.z);
    theta = theta < 0.f ? theta + (2.f * PI_F) : theta;
    float phi = pt_acosf(d.y);
    u = 1.f - (theta / (2.f * PI_F));
    v = phi / PI_F;
  }
  return 2.f * env_lookup(ms, u, v);
}

// ------------------------------------------------ material-sorted tiles --
// The shade kernels take the live paths in tiles of blockDim x
// PT_SORT_ITEMS consecutive positions and shade each tile in the order of
// its material key (0 miss, 1 + material type, PT_SORT_KEYS - 1 past the
// end): a counting sort in shared memory (shared atomics give the ranks, one
// thread the key offsets).  Warps then run one material's code instead of a
// mix, which is what bounds these kernels (SIMT efficiency and instruction
// fetch).  The order does not change any path's result.
#ifndef PT_SORT_ITEMS
#define PT_SORT_ITEMS 4
#endif
#ifndef PT_SHADE_TILE_GRID
#define PT_SHADE_TILE_GRID 1
#endif
#define PT_SORT_KEYS (PT_NUM_MAT_TYPES + 2)

struct SortTile {
  uint16_t perm[PT_SHADE_BLOCK * PT_SORT_ITEMS];  // tile position in sorted order
  uint32_t cnt[PT_SORT_KEYS];
  uint32_t start[PT_SORT_KEYS];
};

__device__ __forceinline__ uint32_t shade_key(const DevScene& S0, const float4* __restrict__ hit,
                                              uint32_t i, uint32_t n) {
  if (i >= n) return PT_SORT_KEYS - 1;
  uint32_t leaf = __float_as_uint(hit[i].w);
  if (leaf == PT_NO_HIT) return 0;
  uint32_t mid = __float_as_uint(__ldg(&S0.prims[3 * (size_t)leaf + 2].w));
  return 1u + (uint32_t)__ldg(&S0.mats[mid].type);
}

__device__ __forceinline__ void sort_tile(SortTile& t, const DevScene& S0,
                                          const float4* __restrict__ hit, uint32_t base,
                                          uint32_t n) {
  const uint32_t bd = blockDim.x;
  if (threadIdx.x < PT_SORT_KEYS) t.cnt[threadIdx.x] = 0;
  __syncthreads();
  uint32_t key[PT_SORT_ITEMS], rank[PT_SORT_ITEMS];
#pragma unroll
  for (int it = 0; it < PT_SORT_ITEMS; it++) {
    key[it] = shade_key(S0, hit, base + it * bd + threadIdx.x, n);
    rank[it] = atomicAdd(&t.cnt[key[it]], 1u);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t sum = 0;
    for (int k = 0; k < PT_SORT_KEYS; k++) {
      t.start[k] = sum;
      sum += t.cnt[k];
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < PT_SORT_ITEMS; it++)
    t.perm[t.start[key[it]] + rank[it]] = (uint16_t)(it * bd + threadIdx.x);
  __syncthreads();
}

// Loop of a shade kernel over its paths: material-sorted tiles (SORT) or a
// plain grid-stride loop.  Every lane of a warp runs every step (the queue
// appends inside are warp-aggregated).
#define SHADE_LOOP(CALL)                                                           \
  if (SORT) {                                                                      \
    const uint32_t tile_n = blockDim.x * PT_SORT_ITEMS;                            \
    for (uint32_t base = blockIdx.x * tile_n; base < n; base += gridDim.x * tile_n) { \
      sort_tile(tile, S0, W.hit, base, n);                                         \
      for (int it = 0; it < PT_SORT_ITEMS; it++) {                                 \
        uint32_t i = base + tile.perm[it * blockDim.x + threadIdx.x];              \
        CALL;                                                                      \
      }                                                                            \
      __syncthreads();                                                             \
    }                                                                              \
  } else {                                                                         \
    uint32_t stride = gridDim.x * blockDim.x;                                      \
    uint32_t iters = (n + stride - 1) / stride;                                    \
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;                            \
    for (uint32_t it = 0; it < iters; it++, i += stride) {                         \
      CALL;                                                                        \
    }                                                                              \
  }

// One path of k_shade (position i of the current buffer; all lanes of the
// warp call it together: the queue appends are warp-aggregated).
template <bool BATCH, bool TEX>
__device__ __forceinline__ void shade_path(const DevScene& S0, const WaveState& W,
                                         const WaveCounters& c, const WaveCtl& ctl,
                                         const BatchRefs& br, uint32_t i, bool active) {
  const PathBuf& pb = W.path[c.parity];
  uint4 st = make_uint4(0, 0, 0, 0);
  V3 thr = v3(0.f), rad = v3(0.f);
  float tm = 0.f;
  Tail tl;
  tl.event = 1;
  tl.isSpecular = false;
  bool tail = false, shadow = false, missed = false;
  V3 col = v3(0.f);
  V3 P, N, Wo, Wi;
  float lightPDF = 0.f;
  int lindex = 0;
  uint32_t mid = 0;
  bool textured = false;  // the material's colours come from textures
  V3 tcol = v3(0.f);      // its colour at this hit (k_finish needs it for Direct_Light)
  if (active) st = pb.st[i];
  const DevScene& S = path_scene<BATCH>(S0, br, st.z);
  if (active) {
    float4 t4 = pb.thr[i], r4 = pb.rad[i];
    thr = f4xyz(t4);
    tm = t4.w;
    rad = f4xyz(r4);
    float4 hit = W.hit[i];
    float4 ro = pb.ray_o[i], rdv = pb.ray_d[i];
    uint32_t leaf = __float_as_uint(hit.w);
    if (leaf == PT_NO_HIT) {
      thr *= miss_color(S.miss, f4xyz(rdv));
      col = rad + clamp3(thr, 0.f, 1.f);  // raygen.cu:81-82
      missed = true;
    } else {
      PrimRec p = load_prim(S.prims, leaf);
      HitRecord rec = hit_record(S, p, f4xyz(ro), f4xyz(rdv), hit.x, hit.y, hit.z, false, tm);
      mid = rec.index;
      GpuMaterial m = S.mats[mid];
      textured = TEX && (m.tex0 >= 0 || m.tex1 >= 0);
      if (textured) {
        apply_textures(S, m, p, f4xyz(ro), f4xyz(rdv), hit.x, hit.y, hit.z, tm);
        tcol = v3(m.c0x, m.c0y, m.c0z);
      }
      P = rec.P;
      Wo = rec.Wo;
      N = rec.shading_normal;
      switch (m.type) {
        case PT_MAT_LAMBERTIAN:
        case PT_MAT_OREN_NAYAR:
        case PT_MAT_DIFFUSE_LIGHT: {
          bool isLight = m.type == PT_MAT_DIFFUSE_LIGHT;
          if (nee_begin(S, st.x, P, N, isLight, Wi, lightPDF, lindex)) {
            shadow = true;
          } else {
            after_nee(m, st.x, P, Wo, N, v3(0.f), thr, rad, tl);
            tail = true;
          }
          break;
        }
        case PT_MAT_METAL: {  // programs/materials/metal.cu:38-56
          V3 reflected = reflect(-Wo, N);
          tl.direction = reflected + m.p0 * random_in_unit_sphere(st.x);
          tl.event = 0;
          tl.origin = P;
          thr *= v3(m.c0x, m.c0y, m.c0z);
          tl.isSpecular = true;
          tail = true;
          break;
        }
        case PT_MAT_DIELECTRIC: {  // programs/materials/dielectric.cu:46-96
          float ref_idx = m.p0;
          V3 Wd = -rec.Wo;
          V3 Nd = N;
          V3 absorption = v3(1.f);
          float ni_over_nt;
          float cosine = dot(Wd, Nd);
          if (cosine > 0.f) {
            Nd = -Nd;
            ni_over_nt = ref_idx;
            cosine = ref_idx * cosine / length(Wd);
          } else {
            ni_over_nt = 1.f / ref_idx;
            cosine = -cosine / length(Wd);
          }
          V3 refracted = v3(0.f);
          float reflect_prob;
          if (Refract(Wd, Nd, ni_over_nt, refracted))
            reflect_prob = schlick(cosine, ref_idx);
          else
            reflect_prob = 1.f;
          if (rnd(st.x) < reflect_prob)
            tl.direction = reflect(Wd, Nd);
          else
            tl.direction = normalize(refracted);
          tl.event = 0;
          tl.origin = P;
          thr *= (v3(m.c0x, m.c0y, m.c0z) * absorption);
          tl.isSpecular = true;
          tail = true;
          break;
        }
        case PT_MAT_TORRANCE_SPARROW:
        case PT_MAT_ASHIKHMIN_SHIRLEY: {
          V3 Wn = brdf_sample(m, Wo, N, st.x);
          float pdf = 0.f;
          V3 attenuation = brdf_eval(m, Wo, Wn, N, pdf);
          tl.event = 0;
          tl.origin = P;
          tl.direction = Wn;
          if (m.type == PT_MAT_TORRANCE_SPARROW)
            thr *= clamp3(attenuation / pdf, 0.f, 1.f);
          else
            thr *= clamp3(attenuation, 0.f, 1.f);
          tl.isSpecular = true;
          tail = true;
          break;
        }
        default:
          tl.event = 1;
          tail = true;
      }
    }
  }
  // shadow rays: park the Direct_Light context and the path state
  uint32_t spos = warp_push(&W.ctr->n_shadow, shadow);
  if (shadow) {
    W.sh.P[spos] = make_float4(P.x, P.y, P.z, lightPDF);
    W.sh.N[spos] = make_float4(N.x, N.y, N.z, __int_as_float(lindex));
    W.sh.Wo[spos] = make_float4(Wo.x, Wo.y, Wo.z, __uint_as_float(mid));
    W.sh.Wi[spos] = make_float4(Wi.x, Wi.y, Wi.z, 0.f);
    if (textured) W.sh.C[spos] = make_float4(tcol.x, tcol.y, tcol.z, 0.f);
    W.sh.st[spos] = st;
    W.sh.thr[spos] = make_float4(thr.x, thr.y, thr.z, tm);
    W.sh.rad[spos] = make_float4(rad.x, rad.y, rad.z, 0.f);
  }
  if (missed) finalize_path(W, st.y, col);  // misses end here
  path_tail(W, c, path_ctl<BATCH>(ctl, br, st.z), st, thr, rad, tl, tail, tm);
}

// TEX: the scene has textured materials (their colours are evaluated at
// the hit); the other variant carries no texture code at all.
template <bool BATCH, bool SORT, bool TEX>
__global__ void __launch_bounds__(PT_SHADE_BLOCK, PT_SHADE_MINBLOCKS) k_shade(DevScene S0, WaveState W,
                                                          const WaveCtl* __restrict__ ctlp,
                                                          BatchRefs br) {
  __shared__ SortTile tile;
  WaveCounters c = *W.ctr;
  WaveCtl ctl = *ctlp;
  uint32_t n = c.n_cur + gen_count(c, ctl, (uint32_t)W.slots);
  SHADE_LOOP((shade_path<BATCH, TEX>(S0, W, c, ctl, br, i, i < n)))
}

template <bool BATCH>
__global__ void __launch_bounds__(PT_SHADE_BLOCK) k_finish(DevScene S0, WaveState W,
                                                           const WaveCtl* __restrict__ ctlp,
                                                           BatchRefs br) {
  WaveCounters c = *W.ctr;
  WaveCtl ctl = *ctlp;
  uint32_t n = c.n_shadow;
  uint32_t stride = gridDim.x * blockDim.x;
  uint32_t iters = (n + stride - 1) / stride;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t it = 0; it < iters; it++, i += stride) {
    bool active = i < n;
    uint4 st = make_uint4(0, 0, 0, 0);
    V3 thr = v3(0.f), rad = v3(0.f);
    float tm = 0.f;
    Tail tl;
    tl.event = 1;
    tl.isSpecular = false;
    if (active) st = W.sh.st[i];
    const DevScene& S = path_scene<BATCH>(S0, br, st.z);
    if (active) {
      const float4 t4 = W.sh.thr[i];
      thr = f4xyz(t4);
      tm = t4.w;
      rad = f4xyz(W.sh.rad[i]);
      float4 P4 = W.sh.P[i], N4 = W.sh.N[i], Wo4 = W.sh.Wo[i], Wi4 = W.sh.Wi[i];
      GpuMaterial m = S.mats[__float_as_uint(Wo4.w)];
      if (m.tex0 >= 0) {  // the colour its texture gave at the hit (k_shade): NEE materials
        float4 c4 = W.sh.C[i];  // (Lambertian, Oren-Nayar, diffuse light) read only c0
        m.c0x = c4.x;
        m.c0y = c4.y;
        m.c0z = c4.z;
      }
      V3 P = f4xyz(P4), N = f4xyz(N4), Wo = f4xyz(Wo4);
      V3 direct = nee_end(S, m, st.x, P, Wo, N, f4xyz(Wi4), P4.w, __float_as_int(N4.w),
                          Wi4.w != 0.f);
      after_nee(m, st.x, P, Wo, N, direct, thr, rad, tl);
    }
    path_tail(W, c, path_ctl<BATCH>(ctl, br, st.z), st, thr, rad, tl, active, tm);
  }
}

// ------------------------------------------------- consistent-mode stages --
// Sum over the lights of their sampling pdf for direction d from P (per
// light selection), the MIS partner of BSDF sampling at emitter hits.
__device__ __forceinline__ float lights_pdf_c(const DevScene& S, V3 P, V3 d, int n_sel) {
  float acc = 0.f;
  for (int k = 0; k < S.num_lights; k++) acc += light_pdf(S.lights[k], P, d);
  return acc / (float)n_sel;
}

// Appends a continuing path (consistent mode) to the next buffer; tm is the
// path's time (in the throughput's w), rad_w the guide-record word carried
// in the radiance's w (0 without the guide).
__device__ __forceinline__ void path_push(const WaveState& W, const WaveCounters& c, uint4 st,
                                          V3 thr, V3 rad, V3 o, V3 d, bool cont, float tm,
                                          float rad_w = 0.f) {
  uint32_t pos = warp_push(&W.ctr->n_next, cont);
  if (cont) {
    const PathBuf& nb = W.path[c.parity ^ 1u];
    nb.ray_o[pos] = make_float4(o.x, o.y, o.z, 1e-3f);
    nb.ray_d[pos] = make_float4(d.x, d.y, d.z, PT_RAY_TMAX);
    nb.thr[pos] = make_float4(thr.x, thr.y, thr.z, tm);
    nb.rad[pos] = make_float4(rad.x, rad.y, rad.z, rad_w);
    nb.st[pos] = st;
  }
}

// ---------------------------------------------------- guide training data --
// A path whose id is a multiple of W.grec_stride records its first two
// guided vertices (shading point, sampled direction, BSDF pdf) in
// W.grec[2 * (id / stride) + v], with the throughput arriving at the vertex
// (luminance, kept in .weight) and the radiance collected so far (pad[0]).
// The record word in the path's radiance w is 2 * records + (1 if the
// current vertex recorded), so the NEE term of that vertex, known after its
// shadow ray, joins the mark.  At the end of the path each record's weight
// becomes (radiance after the vertex) / (throughput at it) = F / q of its
// direction, the training signal.
__device__ __forceinline__ float lum3(V3 c) {
  return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
}

__device__ __forceinline__ void guide_end(const WaveState& W, uint32_t pid, float code,
                                          V3 rad_end) {
  int count = (int)code >> 1;
  if (count <= 0) return;
  uint32_t base = 2u * (pid / W.grec_stride);
  float le = lum3(rad_end);
  for (int v = 0; v < count; v++) {
    GuideSample& r = W.grec[base + v];
    float T = r.weight, w = (le - r.pad[0]) / T;
    r.weight = (T > 0.f && w > 0.f && w < 1e30f) ? fminf(w, 1e6f) : 0.f;
    r.pad[1] = 2.f;  // complete
  }
}

// One bounce of the consistent integrator (the oracle's color_c): emission
// with MIS at hits and misses, NEE over lights + environment, BSDF
// continuation, Russian roulette.  The NEE term waits for its shadow ray in
// the shadow buffer together with the already-sampled continuation.  With
// GUIDE the continuation is drawn from alpha * guide + (1 - alpha) * BSDF
// (the guide of this position from k_guide_infer) and that mixture density is
// the MIS partner of NEE and of emitter hits at the next vertex.  One path of
// k_shade_c (see shade_path).
template <bool BATCH, bool GUIDE, bool TEX>
__device__ __forceinline__ void shade_c_path(const DevScene& S0, const WaveState& W,
                                           const WaveCounters& c, const WaveCtl& ctl,
                                           const BatchRefs& br, uint32_t i, bool active) {
  const PathBuf& pb = W.path[c.parity];
  uint4 st = make_uint4(0, 0, 0, 0);
  V3 thr = v3(0.f), rad = v3(0.f), P = v3(0.f), Wi = v3(0.f), dcont = v3(0.f), C = v3(0.f);
  float tmax = 0.f, code = 0.f, tm = 0.f;
  bool ended = false, shadow = false;
  if (active) st = pb.st[i];
  const DevScene& S = path_scene<BATCH>(S0, br, st.z);
  const int n_sel = S.num_lights + (S.env_valid ? 1 : 0);
  if (active) {
    const PathCtl pc = path_ctl<BATCH>(ctl, br, st.z);
    const float4 t4 = pb.thr[i];
    thr = f4xyz(t4);
    tm = t4.w;
    float4 r4 = pb.rad[i];
    rad = f4xyz(r4);
    code = GUIDE ? r4.w : 0.f;
    float4 hit = W.hit[i];
    float4 ro = pb.ray_o[i], rdv = pb.ray_d[i];
    V3 d = f4xyz(rdv);
    uint32_t depth = st.z & PT_ST_DEPTH_MASK;
    // a camera ray counts as a specular bounce: emission it sees is not MIS-weighted
    bool prev_spec = ((st.z >> PT_ST_SPEC_BIT) & 1u) || depth == 0;
    float pdf_prev = __uint_as_float(st.w);
    uint32_t leaf = __float_as_uint(hit.w);
    if (leaf == PT_NO_HIT) {
      V3 Le = miss_color(S.miss, d);
      float w = 1.f;
      if (!prev_spec && S.env_valid) w = power_mis(pdf_prev, env_pdf_dir(S, d) / (float)n_sel);
      rad += thr * Le * w;
      ended = true;
    } else {
      PrimRec p = load_prim(S.prims, leaf);
      HitRecord rec = hit_record(S, p, f4xyz(ro), d, hit.x, hit.y, hit.z, false, tm);
      GpuMaterial m = S.mats[rec.index];
      if (TEX && (m.tex0 >= 0 || m.tex1 >= 0))
        apply_textures(S, m, p, f4xyz(ro), d, hit.x, hit.y, hit.z, tm);
      P = rec.P;
      V3 Wo = rec.Wo, N = rec.shading_normal;
      if (m.type == PT_MAT_DIFFUSE_LIGHT) {
        float w = 1.f;
        if (!prev_spec && n_sel > 0) w = power_mis(pdf_prev, lights_pdf_c(S, f4xyz(ro), d, n_sel));
        rad += thr * v3(m.c0x, m.c0y, m.c0z) * w;
        ended = true;
      } else if (m.type == PT_MAT_METAL) {  // programs/materials/metal.cu:38-56
        V3 reflected = reflect(-Wo, N);
        dcont = reflected + m.p0 * random_in_unit_sphere(st.x);
        thr *= v3(m.c0x, m.c0y, m.c0z);
        prev_spec = true;
      } else if (m.type == PT_MAT_DIELECTRIC) {  // programs/materials/dielectric.cu:46-96
        float ref_idx = m.p0;
        V3 Wd = -rec.Wo, Nd = N;
        float ni_over_nt;
        float cosine = dot(Wd, Nd);
        if (cosine > 0.f) {
          Nd = -Nd;
          ni_over_nt = ref_idx;
          cosine = ref_idx * cosine / length(Wd);
        } else {
          ni_over_nt = 1.f / ref_idx;
          cosine = -cosine / length(Wd);
        }
        V3 refracted = v3(0.f);
        float reflect_prob;
        if (Refract(Wd, Nd, ni_over_nt, refracted)) reflect_prob = schlick(cosine, ref_idx);
        else reflect_prob = 1.f;
        if (rnd(st.x) < reflect_prob) dcont = reflect(Wd, Nd);
        else dcont = normalize(refracted);
        thr *= (v3(m.c0x, m.c0y, m.c0z) * v3(1.f));
        prev_spec = true;
      } else {
        Frame fr(N);
        V3 wo_l = fr.to_local(Wo);
        // bounces past the guided depth use the BSDF alone (alpha = 0)
        const bool guided = GUIDE && depth < ctl.guide_depth;
        const GuidePacked* G = GUIDE ? W.guide + i : nullptr;
        const float G_alpha = guided ? __ldg(&G->alpha) : 0.f;
        if (n_sel > 0) {
          int k = (int)(rnd(st.x) * (float)n_sel);
          if (k > n_sel - 1) k = n_sel - 1;
          float pl = 0.f;
          V3 Le;
          tmax = PT_RAY_TMAX;
          if (k < S.num_lights) {
            GpuLight L = S.lights[k];
            if (L.type == PT_LIGHT_RECT) {
              Wi = light_sample(L, P, st.x);
              tmax = 1.f - 1e-4f;
            } else {
              Wi = sphere_light_sample_c(L, P, st.x);
              V3 lc = v3(L.cx, L.cy, L.cz);
              float a = dot(Wi, Wi), b = dot(P - lc, Wi);
              float cc = dot(P - lc, P - lc) - L.r * L.r;
              float disc = b * b - a * cc;
              float tn = disc >= 0.f ? (-b - ptm_sqrt(disc)) / a : 0.f;
              tmax = tn * (1.f - 1e-4f);
            }
            pl = light_pdf(L, P, Wi);
            Le = v3(L.ex, L.ey, L.ez);
          } else {
            float u1 = rnd(st.x);
            float u2 = rnd(st.x);
            Wi = env_sample_dir(S, u1, u2);
            pl = env_pdf_dir(S, Wi);
            Le = miss_color(S.miss, Wi);
          }
          V3 wi_n = normalize(Wi);
          float cs = dot(wi_n, N);
          float pls = pl / (float)n_sel;
          if (cs > 0.f && pls > 0.f && tmax > 1e-3f) {
            V3 wi_l = fr.to_local(wi_n);
            V3 f = bsdf_f_c(m, wo_l, wi_l);
            float pbs = bsdf_pdf_c(m, wo_l, wi_l);
            if (guided)
              pbs = G_alpha * guide_pdf_packed(G, wi_n.x, wi_n.y, wi_n.z) + (1.f - G_alpha) * pbs;
            V3 cv = f * Le * (cs * power_mis(pls, pbs) / pls);
            if (!isNull(cv)) {
              shadow = true;
              C = thr * cv;
            }
          }
        }
        V3 wi_l, wdir;
        if (guided && rnd(st.x) < G_alpha) {
          float u0 = rnd(st.x);
          float u1 = rnd(st.x);
          float u2 = rnd(st.x);
          guide_sample_packed(G, u0, u1, u2, wdir.x, wdir.y, wdir.z);
          wi_l = fr.to_local(wdir);
        } else {
          wi_l = bsdf_sample_c(m, wo_l, st.x);
          wdir = fr.to_world(wi_l);
        }
        float pbs = bsdf_pdf_c(m, wo_l, wi_l);
        float q = pbs;
        if (guided) q = G_alpha * guide_pdf_packed(G, wdir.x, wdir.y, wdir.z) + (1.f - G_alpha) * pbs;
        V3 f = bsdf_f_c(m, wo_l, wi_l);
        if (!(q > 0.f) || isNull(f) || !(wi_l.y > 0.f)) {
          ended = true;
        } else {
          if (guided) {
            int count = (int)code >> 1;
            code = (float)(2 * count);
            if (count < 2 && st.y % W.grec_stride == 0) {
              uint32_t slot = 2u * (st.y / W.grec_stride) + (uint32_t)count;
              if (slot < W.grec_n) {
                GuideSample r;
                r.P[0] = P.x; r.P[1] = P.y; r.P[2] = P.z;
                r.N[0] = N.x; r.N[1] = N.y; r.N[2] = N.z;
                r.Wo[0] = Wo.x; r.Wo[1] = Wo.y; r.Wo[2] = Wo.z;
                r.wi[0] = wdir.x; r.wi[1] = wdir.y; r.wi[2] = wdir.z;
                r.p_bsdf = pbs;
                r.weight = lum3(thr);
                r.pad[0] = lum3(rad);
                r.pad[1] = 1.f;
                W.grec[slot] = r;
                code = (float)(2 * (count + 1) + 1);
              }
            }
          }
          thr *= f * (wi_l.y / q);
          prev_spec = false;
          pdf_prev = q;
          dcont = wdir;
        }
      }
      if (!ended) {
        if (pc.rr_enable && (int)depth > pc.rr_depth) {
          float q = fminf(1.f, max_component(thr));
          if (rnd(st.x) >= q) ended = true;
          else thr *= 1.f / q;
        }
        if (!ended) {
          depth++;
          if ((int)depth >= pc.max_depth) ended = true;
        }
      }
      st.z = (st.z & PT_ST_KEEP_MASK) | depth | ((uint32_t)prev_spec << PT_ST_SPEC_BIT);
      st.w = __float_as_uint(pdf_prev);
    }
  }
  uint32_t spos = warp_push(&W.ctr->n_shadow, shadow);
  if (shadow) {
    W.sh.P[spos] = make_float4(P.x, P.y, P.z, 0.f);
    W.sh.Wi[spos] = make_float4(Wi.x, Wi.y, Wi.z, 0.f);
    W.sh.C[spos] = make_float4(C.x, C.y, C.z, tmax);
    W.sh.Wo[spos] = make_float4(dcont.x, dcont.y, dcont.z, ended ? 1.f : 0.f);
    W.sh.thr[spos] = make_float4(thr.x, thr.y, thr.z, tm);
    W.sh.rad[spos] = make_float4(rad.x, rad.y, rad.z, code);
    W.sh.st[spos] = st;
  }
  if (active && !shadow && ended) {
    finalize_path(W, st.y, rad);
    if (GUIDE) guide_end(W, st.y, code, rad);
  }
  // the next vertex starts without a pending record of its own
  float cw = GUIDE ? (float)(((int)code >> 1) * 2) : 0.f;
  path_push(W, c, st, thr, rad, P, dcont, active && !shadow && !ended, tm, cw);
}

template <bool BATCH, bool SORT, bool GUIDE, bool TEX>
__global__ void __launch_bounds__(PT_SHADE_BLOCK, GUIDE ? PT_SHADE_G_MINBLOCKS : PT_SHADE_C_MINBLOCKS) k_shade_c(DevScene S0, WaveState W,
                                                            const WaveCtl* __restrict__ ctlp,
                                                            BatchRefs br) {
  __shared__ SortTile tile;
  WaveCounters c = *W.ctr;
  WaveCtl ctl = *ctlp;
  uint32_t n = c.n_cur + gen_count(c, ctl, (uint32_t)W.slots);
  SHADE_LOOP((shade_c_path<BATCH, GUIDE, TEX>(S0, W, c, ctl, br, i, i < n)))
}

__global__ void __launch_bounds__(PT_SHADE_BLOCK) k_finish_c(DevScene S, WaveState W,
                                                             const WaveCtl* __restrict__ ctlp) {
  (void)S;
  (void)ctlp;
  WaveCounters c = *W.ctr;
  uint32_t n = c.n_shadow;
  uint32_t stride = gridDim.x * blockDim.x;
  uint32_t iters = (n + stride - 1) / stride;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t it = 0; it < iters; it++, i += stride) {
    bool active = i < n;
    uint4 st = make_uint4(0, 0, 0, 0);
    V3 thr = v3(0.f), rad = v3(0.f), P = v3(0.f), dcont = v3(0.f);
    bool ended = false;
    float code = 0.f, tm = 0.f;
    if (active) {
      st = W.sh.st[i];
      const float4 t4 = W.sh.thr[i];
      thr = f4xyz(t4);
      tm = t4.w;
      float4 r4 = W.sh.rad[i];
      rad = f4xyz(r4);
      code = r4.w;
      float4 Wi4 = W.sh.Wi[i], C4 = W.sh.C[i], Wo4 = W.sh.Wo[i];
      P = f4xyz(W.sh.P[i]);
      if (Wi4.w == 0.f) {  // unoccluded
        rad += f4xyz(C4);
        // the vertex that just recorded a guide sample: its NEE light did
        // not come along the recorded direction
        int ci = (int)code;
        if (ci & 1) W.grec[2u * (st.y / W.grec_stride) + (uint32_t)(ci >> 1) - 1u].pad[0] +=
            lum3(f4xyz(C4));
      }
      dcont = f4xyz(Wo4);
      ended = Wo4.w != 0.f;
      if (ended) {
        finalize_path(W, st.y, rad);
        if (code != 0.f) guide_end(W, st.y, code, rad);
      }
    }
    path_push(W, c, st, thr, rad, P, dcont, active && !ended, tm, (float)(((int)code >> 1) * 2));
  }
}

// Queue bookkeeping after an iteration.  With use_cond (the iteration loop
// is a graph conditional node) it also decides whether the loop goes on:
// not once the chunk has drained, an error was flagged, or the chunk's
// iteration bound is reached (then error bit 1 is set, so the loop always
// ends).
__global__ void k_advance(WaveState W, const WaveCtl* __restrict__ ctlp, int use_cond,
                          cudaGraphConditionalHandle cond) {
  WaveCounters& c = *W.ctr;
  const WaveCtl& ctl = *ctlp;
  uint32_t n_gen = gen_count(c, ctl, (uint32_t)W.slots);
  c.ext_rays += c.n_cur + n_gen;
  c.shadow_rays += c.n_shadow;
  c.next_path += n_gen;
  c.n_cur = c.n_next;
  c.n_next = 0;
  c.n_shadow = 0;
  c.ray_next[0] = 0;
  c.ray_next[1] = 0;
  c.guide_rows = 0;
  c.parity ^= 1u;
  c.iter++;
  c.iters_total++;
  if (use_cond) {
    bool more = c.n_cur != 0 || c.next_path < ctl.chunk_paths;
    if (more && (unsigned long long)c.iter >= ctl.max_iter) c.error |= 2u;
    if (c.error) more = false;
    cudaGraphSetConditional(cond, more ? 1u : 0u);
  }
}

// ------------------------------------------------------ batch chunk steps --
__global__ void k_batch_begin(WaveState W, WaveCtl* ctl, const BatchChunk* __restrict__ chunks,
                              int use_cond, cudaGraphConditionalHandle inner) {
  WaveCounters& c = *W.ctr;
  BatchChunk ch{};
  if (c.chunk < c.n_chunks) ch = chunks[c.chunk];
  else c.error |= 2u;  // no chunk left: run nothing
  ctl->chunk_paths = ch.paths;
  ctl->max_iter = ch.max_iter;
  ctl->seg_begin = ch.seg_begin;
  ctl->seg_end = ch.seg_end;
  ctl->pixels = ch.pixels;
  c.n_cur = 0;
  c.n_next = 0;
  c.n_shadow = 0;
  c.parity = 0;
  c.iter = 0;
  c.next_path = 0;
  if (use_cond) cudaGraphSetConditional(inner, c.error ? 0u : 1u);
}

// acc[x, H-1-y] += (col, 1) in frame order for every pixel of every segment
// of the chunk (the batch form of k_accumulate).
__global__ void k_accumulate_batch(const float4* __restrict__ results, const WaveCtl* __restrict__ ctlp,
                                   BatchRefs br) {
  const WaveCtl ctl = *ctlp;
  if (ctl.seg_end <= ctl.seg_begin) return;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < ctl.pixels;
       g += gridDim.x * blockDim.x) {
    const BatchSeg& sg = br.segs[find_seg(br.segs, ctl.seg_begin, ctl.seg_end, g, true)];
    const BatchScene& B = br.scenes[sg.scene];
    uint32_t w = (uint32_t)B.width, h = (uint32_t)B.height, WH = w * h;
    uint32_t p = g - sg.pix_off;
    uint32_t y = fastdiv(p, B.w_m, B.w_l), x = p - y * w;
    size_t o = (size_t)(h - 1 - y) * w + x;
    float4 a = sg.acc[o];
    for (uint32_t f = 0; f < sg.frames; f++) {
      float4 r = results[(size_t)sg.path_off + (size_t)f * WH + p];
      a.x += r.x;
      a.y += r.y;
      a.z += r.z;
      a.w += 1.f;
    }
    sg.acc[o] = a;
  }
}

__global__ void k_batch_end(WaveState W, int use_cond, cudaGraphConditionalHandle outer) {
  WaveCounters& c = *W.ctr;
  c.chunk++;
  if (use_cond) cudaGraphSetConditional(outer, (c.chunk < c.n_chunks && !c.error) ? 1u : 0u);
}

// ------------------------------------------------ batch scene relocation --
__global__ void k_relocate_nodes(uint4* nodes, size_t n, uint32_t node_off, uint32_t prim_off) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    uint4 w = nodes[5 * i + 1];
    w.x += node_off;
    w.y += prim_off;
    nodes[5 * i + 1] = w;
  }
}

__global__ void k_relocate_prims(float4* prims, size_t n, uint32_t xform_off, uint32_t id_off,
                                 uint32_t mat_off) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    float4 r0 = prims[3 * i], r1 = prims[3 * i + 1], r2 = prims[3 * i + 2];
    uint32_t tag = __float_as_uint(r0.w);
    if (tag >> 8) tag += xform_off << 8;  // transform index + 1 (0: world space)
    r0.w = __uint_as_float(tag);
    r1.w = __uint_as_float(__float_as_uint(r1.w) + id_off);
    r2.w = __uint_as_float(__float_as_uint(r2.w) + mat_off);
    prims[3 * i] = r0;
    prims[3 * i + 1] = r1;
    prims[3 * i + 2] = r2;
  }
}

__global__ void k_relocate_ids(uint32_t* leaf_of_id, uint4* tri_attr, size_t n, uint32_t prim_off,
                               uint32_t attr_off) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    leaf_of_id[i] += prim_off;
    uint4 a = tri_attr[i];
    a.x += attr_off;
    a.y += attr_off;
    a.z += attr_off;
    tri_attr[i] = a;
  }
}

// acc[x, H-1-y] += (col, 1) in frame order (programs/raygen.cu:153-166)
__global__ void k_accumulate(const float4* __restrict__ results, float4* acc, int width,
                             int height, int frames) {
  uint32_t WH = (uint32_t)width * (uint32_t)height;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < WH; p += gridDim.x * blockDim.x) {
    uint32_t x = p % (uint32_t)width, y = p / (uint32_t)width;
    size_t o = (size_t)(height - 1 - y) * width + x;
    float4 a = acc[o];
    for (int f = 0; f < frames; f++) {
      float4 r = results[(size_t)f * WH + p];
      a.x += r.x;
      a.y += r.y;
      a.z += r.z;
      a.w += 1.f;
    }
    acc[o] = a;
  }
}

// The same accumulation into double sums (acc holds 4 doubles per pixel):
// for renders beyond a few thousand frames, where float sums of per-frame
// values lose the low bits of each new frame.
__global__ void k_accumulate64(const float4* __restrict__ results, double2* acc, int width,
                               int height, int frames) {
  uint32_t WH = (uint32_t)width * (uint32_t)height;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < WH; p += gridDim.x * blockDim.x) {
    uint32_t x = p % (uint32_t)width, y = p / (uint32_t)width;
    size_t o = (size_t)(height - 1 - y) * width + x;
    double2 a0 = acc[2 * o], a1 = acc[2 * o + 1];
    for (int f = 0; f < frames; f++) {
      float4 r = results[(size_t)f * WH + p];
      a0.x += (double)r.x;
      a0.y += (double)r.y;
      a1.x += (double)r.z;
      a1.y += 1.0;
    }
    acc[2 * o] = a0;
    acc[2 * o + 1] = a1;
  }
}

__global__ void k_paths_out(const float4* __restrict__ results, float* out, uint32_t n) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    float4 r = results[p];
    out[3 * p] = r.x;
    out[3 * p + 1] = r.y;
    out[3 * p + 2] = r.z;
  }
}

// programs/raygen.cu:136-146
__global__ void k_resolve(const float4* __restrict__ acc, uchar4* out, int n, int frame) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    float4 a = acc[p];
    float d = (float)(frame + 1);
    float r = fmaxf(0.f, fminf(ptm_sqrt(a.x / d), 1.f));
    float g = fmaxf(0.f, fminf(ptm_sqrt(a.y / d), 1.f));
    float b = fmaxf(0.f, fminf(ptm_sqrt(a.z / d), 1.f));
    out[p] = make_uchar4((unsigned char)(int)(255.99 * r), (unsigned char)(int)(255.99 * g),
                         (unsigned char)(int)(255.99 * b), (unsigned char)(int)(255.99 * 1.f));
  }
}

// ------------------------------------------- environment sampling tables --
// Weight of texel (r, c) = luminance x sin(theta_r).  Each row's prefix is
// summed in double, sequentially, in the oracle's order, so the float CDFs
// come out identical on both sides.  FP64 arithmetic is scarce on this GPU,
// so the per-texel work (weights, then the normalising divisions) runs on
// every SM, and only the dependent additions of a row stay in one thread:
//   k_env_weights  pre[r][c] = weight (all texels)
//   k_env_prefix   pre[r][c] = running sum of row r, rows[r] = its total
//   k_env_cond     conditional CDFs (all entries)
__global__ void k_env_weights(const float4* __restrict__ env, int w, int h, double* pre) {
  const size_t n = (size_t)w * h;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / (size_t)w);
    float theta = PI_F * (((float)r + 0.5f) / (float)h);
    double sn = (double)pt_sinf(theta);
    float4 t = env[i];
    double lum = 0.2126 * (double)t.x + 0.7152 * (double)t.y + 0.0722 * (double)t.z;
    if (!(lum > 0.0)) lum = 0.0;
    pre[i] = lum * sn;
  }
}

__global__ void k_env_prefix(double* pre, int w, int h, double* rows) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= h) return;
  double* p = pre + (size_t)r * w;
  double acc = 0.0;
  for (int c = 0; c < w; c++) {
    acc = acc + p[c];
    p[c] = acc;
  }
  rows[r] = acc;
}

__global__ void k_env_cond(const double* __restrict__ pre, const double* __restrict__ rows, int w,
                           int h, float* cond) {
  const size_t n = (size_t)(w + 1) * h;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / (size_t)(w + 1));
    const int k = (int)(i - (size_t)r * (w + 1));
    const double a = rows[r];
    float v;
    if (k == 0) v = 0.f;
    else if (k == w) v = 1.f;
    else v = a > 0.0 ? (float)(pre[(size_t)r * w + k - 1] / a) : (float)((double)k / (double)w);
    cond[i] = v;
  }
}

// Marginal CDF over the row totals: the sums by one thread in the oracle's
// order (rows[] becomes the running sums), the divisions by the block.
__global__ void k_env_marg(double* rows, int h, float* marg, int* valid) {
  __shared__ double tot_s;
  if (blockIdx.x != 0) return;
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int r = 0; r < h; r++) tot = tot + rows[r];
    double mp = 0.0;
    for (int r = 0; r < h; r++) {
      mp = mp + rows[r];
      rows[r] = mp;
    }
    tot_s = tot;
    *valid = tot > 0.0 ? 1 : 0;
  }
  __syncthreads();
  const double tot = tot_s;
  if (!(tot > 0.0)) return;
  for (int r = threadIdx.x; r < h; r += blockDim.x) marg[r + 1] = (float)(rows[r] / tot);
  if (threadIdx.x == 0) marg[0] = 0.f;
  __syncthreads();
  if (threadIdx.x == 0) marg[h] = 1.f;
}

// ------------------------------------------------------- host launchers ---
namespace pt {

static int g_num_sms = 0;

static int num_sms() {
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

int wave_grid(int kind, int max_stack, int block) {
  int blocks = 0;
  cudaError_t e = cudaSuccess;
  if (kind == 0)
    blocks = trace_blocks_per_sm(block, trace_smem(max_stack, block));
  else
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_shade<false, true, false>, block, 0);
  if (e != cudaSuccess || blocks < 1) {
    cudaGetLastError();
    blocks = 1;
  }
  return blocks * num_sms();
}

LaunchCfg default_launch(int max_stack) {
  LaunchCfg lc;
  lc.trace_block = PT_TRACE_BLOCK;
  lc.shade_block = PT_SHADE_BLOCK;
  lc.sort = 1;
  lc.refetch = 32;
  lc.tex = 0;
  lc.motion = 0;
  lc.trace_grid = wave_grid(0, max_stack, lc.trace_block);
  lc.shade_grid = wave_grid(1, max_stack, lc.shade_block);
  return lc;
}

// The shading kernel of the integrator mode, guide, tile order and texture
// variant.
template <bool BATCH, bool TEX>
static void launch_shade(const DevScene& S, const WaveState& W, const WaveCtl* ctl, BatchRefs br,
                         int mode, bool guide, int sort, int tgs, int sg, int sb, cudaStream_t st) {
  if (mode == 1 && guide) {
    if (sort) k_shade_c<BATCH, true, true, TEX><<<tgs, sb, 0, st>>>(S, W, ctl, br);
    else k_shade_c<BATCH, false, true, TEX><<<sg, sb, 0, st>>>(S, W, ctl, br);
  } else if (mode == 1) {
    if (sort) k_shade_c<BATCH, true, false, TEX><<<tgs, sb, 0, st>>>(S, W, ctl, br);
    else k_shade_c<BATCH, false, false, TEX><<<sg, sb, 0, st>>>(S, W, ctl, br);
  } else {
    if (sort) k_shade<BATCH, true, TEX><<<tgs, sb, 0, st>>>(S, W, ctl, br);
    else k_shade<BATCH, false, TEX><<<sg, sb, 0, st>>>(S, W, ctl, br);
  }
}

template <bool BATCH>
static void launch_iteration_t(const DevScene& S, const WaveState& W, const WaveCtl* ctl,
                               int max_stack, bool counters, const LaunchCfg& lc, cudaStream_t st,
                               cudaEvent_t* ev, int mode, const BatchRefs& br, bool use_cond,
                               unsigned long long cond, const GuideInferArgs* gi) {
  const int sb = lc.shade_block, sg = lc.shade_grid;
  const BatchRefs* brp = BATCH ? &br : nullptr;
  // sorted shading: one block per tile of the buffer (blocks past the live
  // paths return at once), so the block scheduler balances uneven tiles
  const int tile = sb * PT_SORT_ITEMS;
#if PT_SHADE_TILE_GRID
  const int tgs = W.slots > 0 ? (W.slots + tile - 1) / tile : 1;
#else
  const int tgs = sg;
#endif
  if (ev) cudaEventRecordWithFlags(ev[0], st, cudaEventRecordExternal);
  k_generate<BATCH><<<sg, sb, 0, st>>>(S, W, ctl, br);
  if (ev) cudaEventRecordWithFlags(ev[1], st, cudaEventRecordExternal);
  launch_trace(TRACE_EXT, counters, S, W, ctl, max_stack, brp, lc, st);
  if (ev) cudaEventRecordWithFlags(ev[2], st, cudaEventRecordExternal);
  if (mode == 1 && gi) launch_guide_infer(S, W, ctl, *gi, 2 * num_sms(), st);
  if (lc.tex)
    launch_shade<BATCH, true>(S, W, ctl, br, mode, gi != nullptr, lc.sort, tgs, sg, sb, st);
  else
    launch_shade<BATCH, false>(S, W, ctl, br, mode, gi != nullptr, lc.sort, tgs, sg, sb, st);
  if (ev) cudaEventRecordWithFlags(ev[3], st, cudaEventRecordExternal);
  launch_trace(mode == 1 ? TRACE_OCCLUDED : TRACE_SHADOW, counters, S, W, ctl, max_stack, brp, lc,
               st);
  if (ev) cudaEventRecordWithFlags(ev[4], st, cudaEventRecordExternal);
  if (mode == 1)
    k_finish_c<<<sg, sb, 0, st>>>(S, W, ctl);
  else
    k_finish<BATCH><<<sg, sb, 0, st>>>(S, W, ctl, br);
  k_advance<<<1, 1, 0, st>>>(W, ctl, use_cond ? 1 : 0, (cudaGraphConditionalHandle)cond);
  if (ev) cudaEventRecordWithFlags(ev[5], st, cudaEventRecordExternal);
}

// One wavefront iteration (7 launches).
void launch_iteration(const DevScene& S, const WaveState& W, const WaveCtl* ctl, int max_stack,
                      bool counters, const LaunchCfg& lc, cudaStream_t st, cudaEvent_t* ev,
                      int mode, const BatchRefs* br, bool use_cond, unsigned long long cond,
                      const GuideInferArgs* gi) {
  if (br)
    launch_iteration_t<true>(S, W, ctl, max_stack, counters, lc, st, ev, mode, *br, use_cond, cond,
                             nullptr);
  else
    launch_iteration_t<false>(S, W, ctl, max_stack, counters, lc, st, ev, mode, BatchRefs{},
                              use_cond, cond, gi);
}

void launch_batch_begin(const WaveState& W, WaveCtl* ctl, const BatchChunk* chunks,
                        bool use_cond, unsigned long long inner, cudaStream_t st) {
  k_batch_begin<<<1, 1, 0, st>>>(W, ctl, chunks, use_cond ? 1 : 0,
                                 (cudaGraphConditionalHandle)inner);
}

void launch_batch_end(const WaveState& W, const WaveCtl* ctl, const BatchRefs& br,
                      bool use_cond, unsigned long long outer, cudaStream_t st) {
  k_accumulate_batch<<<num_sms() * 8, 256, 0, st>>>(W.results, ctl, br);
  k_batch_end<<<1, 1, 0, st>>>(W, use_cond ? 1 : 0, (cudaGraphConditionalHandle)outer);
}

void launch_relocate(uint4* nodes, size_t n_nodes, uint32_t node_off, uint32_t prim_off,
                     float4* prims, size_t n_prims, uint32_t xform_off, uint32_t id_off,
                     uint32_t mat_off, uint32_t* leaf_of_id, uint4* tri_attr, uint32_t attr_off,
                     cudaStream_t st) {
  int g = num_sms() * 4;
  if (n_nodes) k_relocate_nodes<<<g, 256, 0, st>>>(nodes, n_nodes, node_off, prim_off);
  if (n_prims) {
    k_relocate_prims<<<g, 256, 0, st>>>(prims, n_prims, xform_off, id_off, mat_off);
    k_relocate_ids<<<g, 256, 0, st>>>(leaf_of_id, tri_attr, n_prims, prim_off, attr_off);
  }
}

void launch_accumulate(const float4* results, float4* acc, int w, int h, int frames,
                       cudaStream_t st) {
  k_accumulate<<<num_sms() * 8, 256, 0, st>>>(results, acc, w, h, frames);
}

void launch_accumulate64(const float4* results, double* acc, int w, int h, int frames,
                         cudaStream_t st) {
  k_accumulate64<<<num_sms() * 8, 256, 0, st>>>(results, (double2*)acc, w, h, frames);
}

void launch_paths_out(const float4* results, float* out, uint32_t n, cudaStream_t st) {
  k_paths_out<<<num_sms() * 8, 256, 0, st>>>(results, out, n);
}

void launch_env_cdf(const float4* env, int w, int h, float* marg, float* cond, double* rows,
                    double* pre, int* valid, cudaStream_t st) {
  const int g = num_sms() * 8;
  k_env_weights<<<g, 256, 0, st>>>(env, w, h, pre);
  k_env_prefix<<<(h + 31) / 32, 32, 0, st>>>(pre, w, h, rows);
  k_env_cond<<<g, 256, 0, st>>>(pre, rows, w, h, cond);
  k_env_marg<<<1, 256, 0, st>>>(rows, h, marg, valid);
}

void launch_resolve(const float4* acc, uchar4* out, int n, int frame, cudaStream_t st) {
  k_resolve<<<num_sms() * 8, 256, 0, st>>>(acc, out, n, frame);
}

}  // namespace pt
