/*
 * pt_internal.h - library-internal structures shared by the host API
 * (pt_api.cu, bvh_build.cu) and the wavefront kernels (pt_kernels.cu).
 */
#ifndef PT_INTERNAL_H
#define PT_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>
#include "pt_types.h"

#define PT_TRACE_BLOCK 128
#ifndef PT_TRACE_MINBLOCKS
#define PT_TRACE_MINBLOCKS 6  /* <= 80 registers per thread, no spills */
#endif
#define PT_SHADE_BLOCK 256

struct Ray3 {
  float3 o, d;
};

/* Counters of the streaming wavefront, in device memory. */
struct WaveCounters {
  uint32_t n_cur;        /* live paths at the start of the current buffer (before generation) */
  uint32_t n_next;       /* paths written to the next buffer */
  uint32_t n_shadow;     /* paths parked at a shadow ray this iteration */
  uint32_t parity;       /* which path buffer is current */
  uint32_t error;        /* bit 0: traversal stack overflow */
  uint32_t iter;
  unsigned long long next_path;   /* next path id of the chunk to generate */
  unsigned long long ext_rays, shadow_rays;
  unsigned long long node_fetches, prim_tests;
};

/* Per-chunk render controls, in device memory (kernels read them, so one
 * captured CUDA graph serves every chunk). */
struct WaveCtl {
  int width, height;
  int frame0;                     /* frame of path id 0 of this chunk */
  int max_depth, rr_enable, rr_depth, mode, guide;
  unsigned long long chunk_paths; /* paths in this chunk */
  uint32_t wh_m, wh_l, w_m, w_l;  /* invariant-divisor constants for W*H and W */
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

struct WaveState {
  PathBuf path[2];            /* ping-pong: path[parity] is current */
  float4* hit;                /* t, u, v, leaf index: by position in the current buffer */
  ShadowBuf sh;
  WaveCounters* ctr;
  float4* results;            /* per path of the chunk: colour */
  int slots;                  /* capacity of each buffer */
};

/* float4 arrays per slot: 2 x 4 (path buffers) + 1 (hit) + 7 (shadow), and
 * 3 uint4 state arrays. */
#define PT_SLOT_F4 16
#define PT_SLOT_U4 3

namespace pt {
size_t trace_smem(int max_stack);
int wave_grid(int kind, int max_stack);
cudaError_t set_trace_smem(int max_stack);
/* One wavefront iteration (7 kernels).  ev, if not null, holds 6 events
 * recorded between the stages. */
void launch_iteration(const DevScene& S, const WaveState& W, const WaveCtl* ctl, int max_stack,
                      bool counters, int trace_grid, int shade_grid, cudaStream_t st,
                      cudaEvent_t* ev, int mode);
void launch_env_cdf(const float4* env, int w, int h, float* marg, float* cond, double* rows,
                    int* valid, cudaStream_t st);
void launch_accumulate(const float4* results, float4* acc, int w, int h, int frames,
                       cudaStream_t st);
void launch_paths_out(const float4* results, float* out, uint32_t n, cudaStream_t st);
void launch_first_hits(const DevScene& S, int w, int h, int frame, uint32_t* prim, uint32_t* mat,
                       float* t, int max_stack, uint32_t* err, cudaStream_t st);
void launch_resolve(const float4* acc, uchar4* out, int n, int frame, cudaStream_t st);
}  // namespace pt

#endif
