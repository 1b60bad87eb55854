/*
 * pt_internal.h - library-internal structures shared by the host API
 * (pt_api.cu, bvh_build.cu) and the wavefront kernels (pt_kernels.cu).
 */
#ifndef PT_INTERNAL_H
#define PT_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>
#include "pt_types.h"

#ifndef PT_TRACE_BLOCK
#define PT_TRACE_BLOCK 128       /* default threads per trace block */
#endif
#ifndef PT_TRACE_MAXREG
#define PT_TRACE_MAXREG 72       /* registers per trace thread: 7 blocks of 128 per SM */
#endif
#define PT_SHADE_BLOCK 256       /* default and largest shade block */
#ifndef PT_SHADE_MINBLOCKS
#define PT_SHADE_MINBLOCKS 4     /* of 256 threads: <= 64 registers, 1024 resident threads per SM */
#endif
/* consistent-mode shading: more resident blocks of fewer registers (the
 * spills go to L1) hide more of its dependent loads: 7 blocks of 256 (<= 36
 * registers) gave 1150 -> 1210 M paths/s on the 2.1 M-triangle heightfield
 * (5: 1167, 6: 1182, 8: 1210); reference-mode shading (k_shade) is faster
 * at 4 (5 blocks: 10 % slower on random spheres), and so is guided shading
 * (7 blocks: 256 guided frames of the lit box 3 % slower) */
#ifndef PT_SHADE_C_MINBLOCKS
#define PT_SHADE_C_MINBLOCKS 7
#endif
#ifndef PT_SHADE_G_MINBLOCKS
#define PT_SHADE_G_MINBLOCKS PT_SHADE_MINBLOCKS
#endif

/* Path state word st.z: depth (bits 0-15), previous bounce specular (bit 16),
 * scene of a batch (bits 17-31). */
#define PT_ST_DEPTH_MASK 0xffffu
#define PT_ST_SPEC_BIT 16
#define PT_ST_SCENE_SHIFT 17
#define PT_ST_KEEP_MASK 0xfffe0000u
#define PT_MAX_BATCH_SCENES 32767

/* Launch shape of the stage kernels. */
struct LaunchCfg {
  int trace_block, trace_grid;
  int shade_block, shade_grid;
  int sort;            /* shade in material-sorted tiles */
  int refetch;         /* idle lanes of a trace warp that take new rays together (1..32) */
  int tex;             /* some material takes a texture: the texture variants of shading */
  int motion;          /* some sphere moves: the trace variants that carry ray times */
};

struct Ray3 {
  float3 o, d;
};

/* Counters of the streaming wavefront, in device memory. */
struct WaveCounters {
  uint32_t n_cur;        /* live paths at the start of the current buffer (before generation) */
  uint32_t n_next;       /* paths written to the next buffer */
  uint32_t n_shadow;     /* paths parked at a shadow ray this iteration */
  uint32_t parity;       /* which path buffer is current */
  uint32_t error;        /* bit 0: traversal stack overflow, bit 1: iteration bound reached */
  uint32_t iter;         /* iterations of the current chunk */
  unsigned long long next_path;   /* next path id of the chunk to generate */
  unsigned long long ext_rays, shadow_rays;
  unsigned long long node_fetches, prim_tests;
  unsigned long long iters_total; /* iterations over all chunks (batch) */
  uint32_t chunk;        /* current chunk of a batch */
  uint32_t n_chunks;     /* chunks of the batch (set by the host) */
  uint32_t ray_next[2];  /* rays taken by trace warps this iteration (extension, shadow) */
  uint32_t guide_rows;   /* positions listed for guide inference this iteration */
};

/* Per-chunk render controls, in device memory (kernels read them, so one
 * captured CUDA graph serves every chunk). */
struct WaveCtl {
  int width, height;
  int frame0;                     /* frame of path id 0 of this chunk */
  int max_depth, rr_enable, rr_depth, mode, guide;
  unsigned long long chunk_paths; /* paths in this chunk */
  uint32_t wh_m, wh_l, w_m, w_l;  /* invariant-divisor constants for W*H and W */
  /* batch: segments [seg_begin, seg_end) make up this chunk, `pixels` pixels */
  uint32_t seg_begin, seg_end, pixels;
  uint32_t guide_depth;           /* guided bounces: depth < guide_depth */
  unsigned long long max_iter;    /* device-side iteration bound of this chunk */
};

/* ---- batched multi-scene rendering ---------------------------------------
 * Every scene of a batch is copied into one set of geometry arrays (nodes,
 * records, transforms, materials, attributes) with its indices shifted, so
 * traversal needs only a per-ray root node.  Camera, miss program, lights
 * and environment tables stay per scene. */
struct BatchScene {
  DevScene S;          /* geometry pointers: the batch arrays; the rest: this scene's */
  int width, height, max_depth, rr_enable, rr_depth, pad;
  uint32_t wh_m, wh_l, w_m, w_l;
};

/* Consecutive frames of one scene inside a chunk. */
struct BatchSeg {
  uint32_t path_off;   /* first path of the segment, chunk-relative */
  uint32_t pix_off;    /* first pixel of the segment among the chunk's pixels */
  uint32_t scene;      /* index into the BatchScene table */
  uint32_t frame0, frames, pad;
  float4* acc;         /* device accumulator of the scene */
};

struct BatchChunk {
  unsigned long long paths, max_iter;
  uint32_t seg_begin, seg_end, pixels, pad;
};

/* Kernel-parameter view of a batch (null pointers for a single scene). */
struct BatchRefs {
  const BatchScene* scenes;
  const BatchSeg* segs;
  const uint32_t* roots;     /* root node per scene */
};

/* Unsigned division by an invariant 32-bit divisor d >= 1 (Granlund &
 * Montgomery 1994, "Division by invariant integers using multiplication",
 * fig. 4.1): l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, then
 * n / d = (t + ((n - t) >> min(l,1))) >> max(l-1,0) with t = mulhi(m, n). */
static inline void fastdiv_magic(uint32_t d, uint32_t* m, uint32_t* l) {
  uint32_t ll = 0;
  while (ll < 32 && (1ull << ll) < d) ll++;
  *l = ll;
  *m = (uint32_t)((((1ull << 32) * ((1ull << ll) - d)) / d) + 1);
}
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t fastdiv(uint32_t n, uint32_t m, uint32_t l) {
  uint32_t t = __umulhi(m, n);
  return (t + ((n - t) >> (l > 0 ? 1u : 0u))) >> (l > 0 ? l - 1 : 0u);
}
#endif

/* Path state, structure of arrays, stored in queue order: entry i of the
 * current buffer is the i-th live path of this iteration.  Paths that
 * continue are written compacted into the other buffer of the pair, so
 * every kernel reads and writes its arrays contiguously. */
struct PathBuf {
  float4 *ray_o, *ray_d;      /* origin+tmin, direction+tmax */
  float4 *thr, *rad;          /* throughput, radiance */
  uint4* st;                  /* seed, path id, depth|prevSpecular<<16 */
};

/* Paths parked at a shadow ray (Direct_Light context), in shadow-queue
 * order. */
struct ShadowBuf {
  float4 *P, *N, *Wo, *Wi;    /* P+light pdf, N+light index, Wo+material, Wi+occluded */
  float4* C;                  /* consistent mode: NEE term + shadow tmax */
  float4 *thr, *rad;
  uint4* st;
};

struct GuidePacked;
struct GuideSample;
struct GuideInferArgs;

struct WaveState {
  PathBuf path[2];            /* ping-pong: path[parity] is current */
  float4* hit;                /* t, u, v, leaf index: by position in the current buffer */
  ShadowBuf sh;
  WaveCounters* ctr;
  float4* results;            /* per path of the chunk: colour */
  int slots;                  /* capacity of each buffer */
  /* learned guide (consistent mode, guide = 1): decoded guide by position;
   * training records, 2 per recording path (path id % grec_stride == 0) */
  GuidePacked* guide;
  GuideSample* grec;
  uint32_t grec_stride, grec_n;
};

/* float4 arrays per slot: 2 x 4 (path buffers) + 1 (hit) + 7 (shadow), and
 * 3 uint4 state arrays. */
#define PT_SLOT_F4 16
#define PT_SLOT_U4 3

/* Ray kinds of the trace kernels: closest hit of extension rays; closest
 * hit of a shadow ray (reference mode: the light must be the first thing
 * hit); first-hit queries; any hit before tmax (consistent-mode occlusion). */
enum { TRACE_EXT = 0, TRACE_SHADOW = 1, TRACE_FIRST = 2, TRACE_OCCLUDED = 3 };

namespace pt {
/* Dynamic shared memory of a trace block (pt_trace.cu). */
size_t trace_smem(int max_stack, int block);
/* Resident trace blocks per SM (0 if the shape does not fit). */
int trace_blocks_per_sm(int block, size_t smem);
/* One trace launch of `mode` (TRACE_EXT, TRACE_SHADOW or TRACE_OCCLUDED)
 * over the wavefront's rays, with the launch shape of lc. */
void launch_trace(int mode, bool counters, const DevScene& S, const WaveState& W,
                  const WaveCtl* ctl, int max_stack, const BatchRefs* br, const LaunchCfg& lc,
                  cudaStream_t st);
/* Resident blocks per SM x SMs for a trace (kind 0) or shade (kind 1)
 * kernel of `block` threads. */
int wave_grid(int kind, int max_stack, int block);
/* Raises the dynamic shared memory limit of the trace kernels to the
 * device maximum (once per device). */
cudaError_t set_trace_smem();
/* Default launch shape for a BVH of the given stack depth. */
LaunchCfg default_launch(int max_stack);
/* One wavefront iteration (7 kernels).  ev, if not null, holds 6 events
 * recorded between the stages.  br: batch tables, or null for one scene.
 * use_cond: the queue-advance kernel sets graph conditional `cond` to
 * whether the chunk has work left (device-side iteration loop).  gi: the
 * learned guide (consistent mode only): its inference kernel runs between
 * trace and shade (counted in the shade stage) and shading samples from it. */
void launch_iteration(const DevScene& S, const WaveState& W, const WaveCtl* ctl, int max_stack,
                      bool counters, const LaunchCfg& lc, cudaStream_t st, cudaEvent_t* ev,
                      int mode, const BatchRefs* br, bool use_cond,
                      unsigned long long cond, const GuideInferArgs* gi = nullptr);
/* Batch chunk boundaries: begin loads chunk c.chunk into *ctl and resets the
 * queues (and sets conditional `inner` to 1); end accumulates the chunk's
 * results into the scenes' accumulators, moves to the next chunk and sets
 * conditional `outer` to whether one is left. */
void launch_batch_begin(const WaveState& W, WaveCtl* ctl, const BatchChunk* chunks,
                        bool use_cond, unsigned long long inner, cudaStream_t st);
void launch_batch_end(const WaveState& W, const WaveCtl* ctl, const BatchRefs& br,
                      bool use_cond, unsigned long long outer, cudaStream_t st);
/* Adds offsets to the indices of one scene copied into the batch arrays. */
void launch_relocate(uint4* nodes, size_t n_nodes, uint32_t node_off, uint32_t prim_off,
                     float4* prims, size_t n_prims, uint32_t xform_off, uint32_t id_off,
                     uint32_t mat_off, uint32_t* leaf_of_id, uint4* tri_attr, uint32_t attr_off,
                     cudaStream_t st);
void launch_env_cdf(const float4* env, int w, int h, float* marg, float* cond, double* rows,
                    double* pre, int* valid, cudaStream_t st);
void launch_accumulate(const float4* results, float4* acc, int w, int h, int frames,
                       cudaStream_t st);
/* acc: 4 doubles per pixel (16-byte aligned) */
void launch_accumulate64(const float4* results, double* acc, int w, int h, int frames,
                         cudaStream_t st);
void launch_paths_out(const float4* results, float* out, uint32_t n, cudaStream_t st);
/* First hits of the camera rays of one frame (grid: blocks of PT_TRACE_BLOCK). */
void launch_first_hits(const DevScene& S, int w, int h, int frame, uint32_t* prim, uint32_t* mat,
                       float* t, int max_stack, uint32_t* err, int grid, cudaStream_t st);
void launch_resolve(const float4* acc, uchar4* out, int n, int frame, cudaStream_t st);
}  // namespace pt

#endif
