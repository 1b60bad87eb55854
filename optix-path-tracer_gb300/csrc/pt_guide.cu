/*
 * pt_guide.cu - tensor-core kernels of the learned sampling guide
 * (pt_guide.cuh describes the network).  sm_103a tcgen05: operands in
 * shared memory as 8x8 core-matrix tiles without swizzle, read through
 * matrix descriptors; the FP32 accumulators live in tensor memory; one thread
 * issues the MMAs and a bounded mbarrier wait hands the result to the CTA.
 *
 *   k_guide_infer  per wavefront iteration: hit record -> 76 features ->
 *                  5 layers (BF16 x BF16 -> FP32) -> decoded guide per path
 *   k_guide_grad   training: forward, loss gradient, backward over tiles of
 *                  128 samples; each persistent CTA keeps the five weight
 *                  gradients in tensor memory across its tiles (bias
 *                  gradients come out of the ones column) and writes one
 *                  partial gradient
 *   k_guide_adam   deterministic sum of the partials, Adam on the FP32
 *                  masters, BF16 copies for the next MMAs
 *
 * Layout rules (measured on GB300 by a layout probe): K-major operand, core
 * matrices 8 rows x 16 B; descriptor LBO = byte stride between cores along K,
 * SBO = along M/N.  MN-major operand (the transpose bit set): cores are 8
 * K-rows x 8 contiguous M/N elements; LBO again along K, SBO along M/N.  So
 * one activation tile serves as the K-major A of the forward MMA and as the
 * MN-major operand of the weight-gradient MMA.
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "pt_device.cuh"
#include "pt_guide.cuh"
#include "pt_internal.h"

using namespace ptd;

namespace {

// ------------------------------------------------------------ tcgen05 ------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor, no swizzle (descriptor version 1).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: BF16 A and B, FP32 D, M = 128.
__device__ __forceinline__ uint32_t idesc(int n, int ta, int tb) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)ta << 15) | ((uint32_t)tb << 16) |
         ((uint32_t)(n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

// Bounded wait for an mbarrier phase: at most `limit` try_waits; false when
// the limit ran out.  The kernels' waits take the limit from their arguments
// (pt_guide_set_wait_limit: 2^24 by default, 0 runs out at once); after a
// wait ran out, the wait for the MMAs still in flight always uses
// kDrainLimit, so no kernel reads or frees TMEM under a running MMA.
constexpr uint32_t kDrainLimit = 1u << 24;

__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < limit && !done; it++) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
  }
  return done != 0;
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

// Byte offset of element (r, c) in a tile of C columns stored as 8x8 core
// matrices: cores ordered row-group major, 128 B each, 16 B per core row.
__device__ __forceinline__ uint32_t core_off(int r, int c, int C) {
  return (uint32_t)(((r >> 3) * (C >> 3) + (c >> 3)) * 128 + (r & 7) * 16 + (c & 7) * 2);
}


__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *(uint32_t*)&h;
}
// 8 consecutive columns (c0 % 8 == 0) of row r of a C-column tile, one
// 16-byte access.
__device__ __forceinline__ void st_row8c(unsigned char* tile, int r, int c0, int C, const float* v) {
  uint4 q = make_uint4(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]), pack_bf16x2(v[4], v[5]),
                       pack_bf16x2(v[6], v[7]));
  *(uint4*)(tile + core_off(r, c0, C)) = q;
}
__device__ __forceinline__ void ld_row8c(const unsigned char* tile, int r, int c0, int C, float* v) {
  uint4 q = *(const uint4*)(tile + core_off(r, c0, C));
  uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    float2 f = __bfloat1622float2(*(__nv_bfloat162*)&w[k]);
    v[2 * k] = f.x;
    v[2 * k + 1] = f.y;
  }
}

__device__ __forceinline__ void st_row8(unsigned char* tile, int r, int c0, const float* v) {
  st_row8c(tile, r, c0, PTG_K, v);
}

// The feature row of guide_features, written 8 columns at a time (the same
// arithmetic, so inference and training see identical features), then the
// ones column and padding.
__device__ void write_features_vec(unsigned char* T, int row, const float* P, const float* N,
                                   const float* Wo, const float* bmin, const float* binv,
                                   bool valid) {
  float v[8];
  if (!valid) {
    for (int q = 0; q < 8; q++) v[q] = 0.f;
    for (int c0 = 0; c0 < 72; c0 += 8) st_row8(T, row, c0, v);
  } else {
    for (int a = 0; a < 3; a++) {
      float x = (P[a] - bmin[a]) * binv[a];
      x = fminf(fmaxf(x, 0.f), 1.f);
      float s, c;
      sincospif(x, &s, &c);
      for (int k = 0; k < PTG_FREQ; k++) {
        v[(2 * k) & 7] = s;
        v[(2 * k + 1) & 7] = c;
        if (((2 * k + 2) & 7) == 0) st_row8(T, row, a * 2 * PTG_FREQ + 2 * k - 6, v);
        float s2 = 2.f * s * c, c2 = 1.f - 2.f * s * s;
        s = s2;
        c = c2;
      }
    }
  }
  // 72..75 directions, 76 one, 77..79 zero
  for (int q = 0; q < 8; q++) v[q] = 0.f;
  if (valid) {
    const float* dirs[2] = {N, Wo};
    for (int q = 0; q < 2; q++) {
      const float* d = dirs[q];
      float y = fminf(fmaxf(d[1], -1.f), 1.f);
      v[2 * q] = acosf(y) * 0.31830988618379067f;
      v[2 * q + 1] = atan2f(d[2], d[0]) * 0.15915494309189535f + 0.5f;
    }
  }
  v[4] = 1.f;
  st_row8(T, row, 72, v);
}

// Tile sizes (bytes).
constexpr int kTileT = 128 * PTG_K * 2;   // activation tile, 128 x 80
constexpr int kTileW = PTG_H * PTG_K * 2; // W1..W4, 64 x 80
constexpr int kTileW5 = PTG_NOUT * PTG_K * 2;
constexpr int kWeights = 4 * kTileW + kTileW5;
constexpr int kTileG = 128 * PTG_H * 2;   // gradient tile, 128 x 64
constexpr int kGuard = 2048;              // the weight-gradient MMA reads M = 128 rows of
                                          // a 48/64-row operand: the extra rows land here
// TMEM columns of the training kernel: [0,64) layer accumulator, then the
// five weight gradients, 80 columns each.
constexpr int kTmemAcc = 0;
constexpr int kTmemDW = 64;

__device__ __forceinline__ int layer_rows(int l) { return l == 4 ? PTG_NOUT : PTG_H; }

// Weights (BF16, row-major [rows][80]) into K-major core tiles, 16 bytes
// (one core-matrix row: 8 consecutive columns) per copy.
__device__ void load_weights(unsigned char* W, const __nv_bfloat16* __restrict__ wg) {
  constexpr int kChunks = PTG_K / 8;  // 16-byte chunks per row
  for (int l = 0; l < 5; l++) {
    unsigned char* t = W + l * kTileW;
    const uint4* src = (const uint4*)(wg + PTG_LAYER_OFF(l));
    int n = layer_rows(l) * kChunks;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      int r = e / kChunks, c = (e % kChunks) * 8;
      *(uint4*)(t + core_off(r, c, PTG_K)) = __ldg(src + e);
    }
  }
}

// Forward MMAs of layer l: acc[N] = T (128 x 80, K-major) * W_l^T.
__device__ __forceinline__ void issue_forward(uint32_t tmem, const unsigned char* T,
                                              const unsigned char* W, int l) {
  const int n = layer_rows(l);
  const uint32_t id = idesc(n, 0, 0);
  const uint32_t ta = smem_u32(T), tw = smem_u32(W + l * kTileW);
#pragma unroll
  for (int ks = 0; ks < PTG_K / 16; ks++)
    mma(tmem + kTmemAcc, sdesc(ta + ks * 256, 128, (PTG_K / 8) * 128),
        sdesc(tw + ks * 256, 128, (PTG_K / 8) * 128), id, ks > 0 ? 1u : 0u);
}



struct TmemGuard {
  uint64_t mbar;
  uint32_t base;
};

// Runs the 5-layer forward on T[0] (features), leaving the 48 outputs of
// this thread's row in out[]: with nT == 5 layer l reads T[l] and writes
// T[l+1] (training keeps every activation), with nT == 2 it ping-pongs.
// Returns false, in every thread alike, when a wait ran out.
__device__ bool forward_tile(uint32_t tmem, TmemGuard& g, uint32_t& phase, unsigned char* W,
                             unsigned char* const* T, int nT, float* out, uint32_t limit) {
  const int row = threadIdx.x;
  const uint32_t lane_base = (uint32_t)((threadIdx.x >> 5) * 32) << 16;
  for (int l = 0; l < 5; l++) {
    const unsigned char* in = T[nT == 5 ? l : (l & 1)];
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    if (threadIdx.x == 0) {
      issue_forward(tmem, in, W, l);
      mma_commit(&g.mbar);
    }
    bool ok = mbar_wait(&g.mbar, phase, limit);
    phase ^= 1u;
    fence_after();
    if (!__syncthreads_and(ok)) return false;
    if (l < 4) {
      unsigned char* dst = T[nT == 5 ? l + 1 : ((l + 1) & 1)];
      float h[16];
      for (int c0 = 0; c0 < PTG_H; c0 += 16) {
        tmem_ld16(tmem + lane_base + kTmemAcc + c0, h);
        for (int q = 0; q < 16; q++) h[q] = fmaxf(h[q], 0.f);
        st_row8c(dst, row, c0, PTG_K, h);
        st_row8c(dst, row, c0 + 8, PTG_K, h + 8);
      }
      for (int q = 0; q < 16; q++) h[q] = 0.f;
      h[0] = 1.f;
      st_row8c(dst, row, PTG_H, PTG_K, h);
      h[0] = 0.f;
      st_row8c(dst, row, PTG_H + 8, PTG_K, h);
    } else {
      for (int c0 = 0; c0 < PTG_NOUT; c0 += 16) tmem_ld16(tmem + lane_base + kTmemAcc + c0, out + c0);
    }
  }
  return true;
}

// d(-wn log q)/d(outputs) of one sample; returns the loss term.
__device__ float loss_grad(const float* o, float wx, float wy, float wz, float p_bsdf, float wn,
                           float* d) {
  for (int k = 0; k < PTG_NOUT; k++) d[k] = 0.f;
  if (!(wn > 0.f)) return 0.f;
  GuideParams g;
  guide_decode(o, g);
  float v[PTG_LOBES], pi[PTG_LOBES], cj[PTG_LOBES];
  float pg = 0.f, prev = 0.f;
  for (int j = 0; j < PTG_LOBES; j++) {
    pi[j] = g.cdf[j] - prev;
    prev = g.cdf[j];
    cj[j] = g.lobe[j].x * wx + g.lobe[j].y * wy + g.lobe[j].z * wz;
    v[j] = vmf_pdf(g.lobe[j].x, g.lobe[j].y, g.lobe[j].z, g.lobe[j].w, wx, wy, wz);
    pg += pi[j] * v[j];
  }
  float a = g.alpha;
  float q = a * pg + (1.f - a) * p_bsdf;
  if (!(q > 1e-30f)) return 0.f;
  float dq = -wn / q;  // dL/dq
  float sig = (a - PTG_ALPHA_MIN) / PTG_ALPHA_SPAN;
  d[40] = dq * (pg - p_bsdf) * PTG_ALPHA_SPAN * sig * (1.f - sig);
  for (int j = 0; j < PTG_LOBES; j++) {
    float k = g.lobe[j].w;
    float common = dq * a * pi[j] * v[j];
    // mixture logit
    d[5 * j + 4] = dq * a * pi[j] * (v[j] - pg);
    // log concentration (zero where clamped or in the uniform branch)
    float lk = o[5 * j + 3];
    if (lk > PTG_LOGK_MIN && lk < PTG_LOGK_MAX && k >= 1e-4f)
      d[5 * j + 3] = common * (1.f + k * (cj[j] - 1.f) - 2.f * k / expm1f(2.f * k));
    // mean direction through the normalisation
    float mx = o[5 * j], my = o[5 * j + 1], mz = o[5 * j + 2];
    float n = sqrtf(mx * mx + my * my + mz * mz);
    if (n > 1e-12f && k >= 1e-4f) {
      float s = common * k / n;
      d[5 * j] = s * (wx - cj[j] * g.lobe[j].x);
      d[5 * j + 1] = s * (wy - cj[j] * g.lobe[j].y);
      d[5 * j + 2] = s * (wz - cj[j] * g.lobe[j].z);
    }
  }
  return -wn * logf(q);
}

}  // namespace

// ------------------------------------------------------------ kernels ------
__global__ void __launch_bounds__(128, 1) k_guide_grad(GuideTrainArgs A) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ TmemGuard g;
  bool failed = false;  // uniform across the CTA (decided by __syncthreads_and)
  unsigned char* W = sm;
  unsigned char* T[5];
  for (int l = 0; l < 5; l++) T[l] = sm + kWeights + l * kTileT;
  unsigned char* Gt = sm + kWeights + 5 * kTileT;             // dO (128 x 48) or dH (128 x 64)
  unsigned char* Gn = Gt + kTileG + kGuard;                   // the other dH
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&g.mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&g.base)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  load_weights(W, A.w);
  // the guard areas must hold finite numbers (their products land in
  // ignored rows, but NaN/Inf patterns are avoided all the same)
  for (int e = tid; e < kGuard / 4; e++) {
    ((uint32_t*)(Gt + kTileG))[e] = 0u;
    ((uint32_t*)(Gn + kTileG))[e] = 0u;
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = g.base;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  uint32_t phase = 0;
  uint32_t n = *A.count;
  if (A.max_count && n > A.max_count) n = A.max_count;
  const float wsum = *A.wsum;
  const uint32_t ntiles = (n + 127) / 128;
  bool first = true;
  float loss_acc = 0.f;
  for (uint32_t tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
    const uint32_t s = tile * 128 + tid;
    const bool valid = s < n;
    GuideSample smp = {};
    if (valid) smp = A.samples[s];
    write_features_vec(T[0], tid, smp.P, smp.N, smp.Wo, A.bmin, A.binv, valid);
    float o[PTG_NOUT];
    if (!forward_tile(tmem, g, phase, W, T, 5, o, A.wait_limit)) {
      failed = true;
      break;
    }
    if (A.out && valid)
      for (int k = 0; k < PTG_NOUT; k++) A.out[(size_t)s * PTG_NOUT + k] = o[k];
    if (!A.train) continue;
    // ---- loss gradient of this row -> dO tile (128 x 48, K-major)
    float d[PTG_NOUT];
    float wn = valid && wsum > 0.f ? smp.weight / wsum : 0.f;
    loss_acc += valid ? loss_grad(o, smp.wi[0], smp.wi[1], smp.wi[2], smp.p_bsdf, wn, d)
                      : loss_grad(o, 0.f, 1.f, 0.f, 0.f, 0.f, d);
    for (int k = 0; k < PTG_NOUT; k += 8) st_row8c(Gt, tid, k, PTG_NOUT, d + k);
    // ---- backward, layer 4 .. 0
    unsigned char* G = Gt;
    unsigned char* Gnext = Gn;
    for (int l = 4; l >= 0; l--) {
      const int rows = layer_rows(l);        // width of G (layer outputs)
      fence_async_smem();
      fence_before();
      __syncthreads();
      fence_after();
      if (tid == 0) {
        // dW_l += G^T T_l : A = G MN-major (M = rows, padded to 128), K = samples;
        //                   B = T_l MN-major (N = 80), K = samples
        const uint32_t ga = smem_u32(G), tb = smem_u32(T[l]);
        const uint32_t gk = (rows / 8) * 128;  // G: bytes per core row (8 samples)
        const uint32_t idw = idesc(PTG_K, 1, 1);
        for (int ks = 0; ks < 8; ks++)
          mma(tmem + kTmemDW + l * PTG_K, sdesc(ga + ks * 2 * gk, gk, 128),
              sdesc(tb + ks * 2 * (PTG_K / 8) * 128, (PTG_K / 8) * 128, 128), idw,
              (first && ks == 0) ? 0u : 1u);
        if (l > 0) {
          // dT_l = G * W_l[:, 0:64] : A = G K-major (K = rows); B = W_l MN-major (N = 64)
          const uint32_t wa = smem_u32(W + l * kTileW);
          const uint32_t idx = idesc(PTG_H, 0, 1);
          for (int ks = 0; ks < rows / 16; ks++)
            mma(tmem + kTmemAcc, sdesc(ga + ks * 256, 128, gk),
                sdesc(wa + ks * 2 * (PTG_K / 8) * 128, (PTG_K / 8) * 128, 128), idx,
                ks > 0 ? 1u : 0u);
        }
        mma_commit(&g.mbar);
      }
      bool ok = mbar_wait(&g.mbar, phase, A.wait_limit);
      phase ^= 1u;
      fence_after();
      if (!__syncthreads_and(ok)) {
        failed = true;
        break;
      }
      if (l > 0) {
        // G_{l-1} = dT_l * (T_l > 0), into the other gradient tile
        float h[16], t[8];
        for (int c0 = 0; c0 < PTG_H; c0 += 16) {
          tmem_ld16(tmem + lane_base + kTmemAcc + c0, h);
          for (int half = 0; half < 2; half++) {
            ld_row8c(T[l], tid, c0 + 8 * half, PTG_K, t);
            for (int q = 0; q < 8; q++) h[8 * half + q] = t[q] > 0.f ? h[8 * half + q] : 0.f;
            st_row8c(Gnext, tid, c0 + 8 * half, PTG_H, h + 8 * half);
          }
        }
        unsigned char* tmp = G;
        G = Gnext;
        Gnext = tmp;
      }
    }
    if (failed) break;
    first = false;
  }
  // after a wait that ran out, the MMAs in flight (phase was flipped past
  // it) finish before TMEM is read or freed; this wait is bounded too
  if (failed) mbar_wait(&g.mbar, phase ^ 1u, kDrainLimit);
  // ---- per-CTA partial gradients (rows of dW live in lanes 0..rows-1)
  fence_before();
  __syncthreads();
  fence_after();
  if (A.train && A.partial) {
    float* P = A.partial + (size_t)blockIdx.x * PTG_PARAMS;
    for (int l = 0; l < 5; l++) {
      const int rows = layer_rows(l);
      if (warp * 32 >= rows) continue;
      int row = tid;
      float vals[PTG_K];
      for (int c0 = 0; c0 < PTG_K; c0 += 16)
        tmem_ld16(tmem + lane_base + kTmemDW + l * PTG_K + c0, vals + c0);
      if (row < rows)
        for (int c = 0; c < PTG_K; c++)
          P[PTG_LAYER_OFF(l) + row * PTG_K + c] = (first || failed) ? 0.f : vals[c];
    }
  }
  if (loss_acc != 0.f && A.loss) atomicAdd(A.loss, loss_acc);
  if (failed && tid == 0) atomicOr(A.fail, 1u);
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// Sum of the per-CTA partials (fixed order) and Adam on the FP32 masters;
// padding entries (rows 41..47 of W5, columns past the bias column) stay 0.
__global__ void k_guide_adam(GuideAdamArgs A) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= PTG_PARAMS) return;
  int l = p / PTG_W_LAYER;
  int e = p - l * PTG_W_LAYER;
  int r = e / PTG_K, c = e % PTG_K;
  bool used = r < (l == 4 ? PTG_OUT : PTG_H) && c <= PTG_BIAS_COL(l);
  float gsum = 0.f;
  for (int k = 0; k < A.nparts; k++) gsum += A.partial[(size_t)k * PTG_PARAMS + p];
  if (!used) gsum = 0.f;
  if (A.grad_out) A.grad_out[p] = gsum;
  if (!A.update || !used) return;
  float m = A.b1 * A.m[p] + (1.f - A.b1) * gsum;
  float v = A.b2 * A.v[p] + (1.f - A.b2) * gsum * gsum;
  A.m[p] = m;
  A.v[p] = v;
  float w = A.w32[p] - A.lr * (m / A.bc1) / (sqrtf(v / A.bc2) + A.eps);
  A.w32[p] = w;
  A.wbf[p] = __float2bfloat16_rn(w);
}

// ------------------------------------------------------ inference --------
__device__ __forceinline__ void bar_group(int id) {
  asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory");
}
// AND of v over the 128 threads of named barrier id.
__device__ __forceinline__ bool group_and(bool v, int id) {
  uint32_t r;
  asm volatile(
      "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred p, %2, 128, q;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id)
      : "memory");
  return r != 0;
}


// Lists the positions of the current buffer whose path needs a guide at
// this bounce (depth below the guided-bounce limit, a hit on a non-delta
// material), so that inference runs the network on those rows only, and
// writes each listed row's hit record (point, shading normal, Wo): the chain
// of dependent loads behind it (hit, primitive record, material, ray) runs
// here, at full occupancy, instead of in front of the inference MMAs.  The
// list order does not matter (rows are independent).
__global__ void __launch_bounds__(256) k_guide_select(DevScene S, WaveState W,
                                                      const WaveCtl* __restrict__ ctlp,
                                                      uint32_t* rows, float4* feat) {
  const WaveCounters c = *W.ctr;
  const WaveCtl ctl = *ctlp;
  unsigned long long left = ctl.chunk_paths - c.next_path;
  const uint32_t n =
      c.n_cur + (uint32_t)min((unsigned long long)((uint32_t)W.slots - c.n_cur), left);
  const PathBuf& pb = W.path[c.parity];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t iters = (n + stride - 1) / stride;
  const int lane = threadIdx.x & 31;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  for (uint32_t it = 0; it < iters; it++, i += stride) {
    bool take = false;
    HitRecord rec;
    if (i < n && (pb.st[i].z & PT_ST_DEPTH_MASK) < ctl.guide_depth) {
      const float4 hit = W.hit[i];
      const uint32_t leaf = __float_as_uint(hit.w);
      if (leaf != PT_NO_HIT) {
        const PrimRec p = load_prim(S.prims, leaf);
        const int type = __ldg(&S.mats[prim_material(p)].type);
        take = type == PT_MAT_LAMBERTIAN || type == PT_MAT_OREN_NAYAR ||
               type == PT_MAT_TORRANCE_SPARROW || type == PT_MAT_ASHIKHMIN_SHIRLEY;
        if (take) {
          const float4 ro = pb.ray_o[i], rd = pb.ray_d[i];
          rec = hit_record(S, p, f4xyz(ro), f4xyz(rd), hit.x, hit.y, hit.z, false, pb.thr[i].w);
        }
      }
    }
    uint32_t mask = __ballot_sync(0xffffffffu, take);
    if (!mask) continue;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&W.ctr->guide_rows, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) {
      const uint32_t li = base + __popc(mask & ((1u << lane) - 1u));
      rows[li] = i;
      feat[3 * (size_t)li] = make_float4(rec.P.x, rec.P.y, rec.P.z, 0.f);
      feat[3 * (size_t)li + 1] =
          make_float4(rec.shading_normal.x, rec.shading_normal.y, rec.shading_normal.z, 0.f);
      feat[3 * (size_t)li + 2] = make_float4(rec.Wo.x, rec.Wo.y, rec.Wo.z, 0.f);
    }
  }
}

// Inference inside the wavefront, one row per position listed by
// k_guide_select; each row's packed guide goes to A.out at the path's
// position.  Each CTA runs two independent
// 128-row pipelines (warps 0-3 and 4-7) that share the weights: each has
// its own activation tile (updated in place: the epilogue writes a layer's
// output over its input once the MMA has read it), mbarrier, 64 TMEM columns
// and named barrier, so one pipeline's epilogue overlaps the other's MMAs.
__global__ void __launch_bounds__(256) k_guide_infer(DevScene S, WaveState W,
                                                     const WaveCtl* __restrict__ ctlp,
                                                     GuideInferArgs A) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tbase;
  unsigned char* Wt = sm;
  const int grp = threadIdx.x >> 7, row = threadIdx.x & 127, warp = threadIdx.x >> 5;
  const int bar_id = 1 + grp;
  unsigned char* T = sm + kWeights + grp * kTileT;
  const WaveCounters c = *W.ctr;
  const uint32_t nl = min(c.guide_rows, (uint32_t)W.slots);  // listed by k_guide_select
  const uint32_t ntiles = (nl + 127) / 128;
  if (blockIdx.x * 2 >= ntiles) return;  // no tile for this CTA: skip the setup
  if (threadIdx.x == 0) {
    for (int g = 0; g < 2; g++)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar[g])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tbase)),
                 "r"(128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  load_weights(Wt, A.w);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tbase + (uint32_t)(grp * 64);
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  uint32_t phase = 0;
  bool failed = false;
  for (uint32_t tile = blockIdx.x * 2 + grp; tile < ntiles; tile += gridDim.x * 2) {
    const uint32_t li = tile * 128 + row;
    const bool valid = li < nl;  // every listed row needs a guide
    const uint32_t i = valid ? A.rows[li] : 0xffffffffu;
    float P[3], N[3], Wo[3];
    if (valid) {
      const float4 a = A.feat[3 * (size_t)li], b = A.feat[3 * (size_t)li + 1],
                   e = A.feat[3 * (size_t)li + 2];
      P[0] = a.x; P[1] = a.y; P[2] = a.z;
      N[0] = b.x; N[1] = b.y; N[2] = b.z;
      Wo[0] = e.x; Wo[1] = e.y; Wo[2] = e.z;
    }
    // a pipeline whose 128 rows all need no guide skips the network
    if (group_and(!valid, bar_id)) continue;
    write_features_vec(T, row, P, N, Wo, A.bmin, A.binv, valid);
    float o[PTG_NOUT];
    for (int l = 0; l < 5 && !failed; l++) {
      fence_async_smem();
      fence_before();
      bar_group(bar_id);
      fence_after();
      if (row == 0) {
        issue_forward(tmem, T, Wt, l);
        mma_commit(&mbar[grp]);
      }
      bool ok = mbar_wait(&mbar[grp], phase, A.wait_limit);
      phase ^= 1u;
      fence_after();
      if (!group_and(ok, bar_id)) {
        failed = true;
        break;
      }
      if (l < 4) {
        // ReLU, BF16, in place; then the ones column and padding
        float h[16];
        for (int c0 = 0; c0 < PTG_H; c0 += 16) {
          tmem_ld16(tmem + lane_base + kTmemAcc + c0, h);
          for (int q = 0; q < 16; q++) h[q] = fmaxf(h[q], 0.f);
          st_row8(T, row, c0, h);
          st_row8(T, row, c0 + 8, h + 8);
        }
        for (int q = 0; q < 16; q++) h[q] = 0.f;
        h[0] = 1.f;
        st_row8(T, row, PTG_H, h);
        h[0] = 0.f;
        st_row8(T, row, PTG_H + 8, h);
      } else {
        for (int c0 = 0; c0 < PTG_NOUT; c0 += 16) tmem_ld16(tmem + lane_base + kTmemAcc + c0, o + c0);
      }
    }
    if (failed) break;
    if (valid) {
      GuideParams gp;
      guide_decode(o, gp);
      A.out[i] = guide_pack(gp);
    }
  }
  if (failed) {
    if (row == 0) atomicOr(A.fail, 1u);
    mbar_wait(&mbar[grp], phase ^ 1u, kDrainLimit);  // the MMAs in flight finish first
  }
  fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(128));
}

// Completed training records with a positive weight, copied to the
// training array in record order (the first `cap` of them), with the sum of
// their weights: a stable compaction over blocks of 1024 records, so the
// training array, and with it the whole training, is the same on every run.
//   k_guide_collect_count   takers per block
//   k_guide_collect_scan    block offsets (one thread, in block order), count
//   k_guide_collect_write   the copies; per-block weight sums (fixed order)
//   k_guide_collect_sum     the weight sum (one thread, in block order)
constexpr uint32_t kCollectPer = 1024;  // records per block: 4 chunks of 256

__device__ __forceinline__ bool collect_take(const GuideSample& r) {
  return r.pad[1] == 2.f && r.weight > 0.f;
}

__global__ void __launch_bounds__(256) k_guide_collect_count(const GuideSample* __restrict__ rec,
                                                             uint32_t n, uint32_t* block_cnt) {
  __shared__ uint32_t wc[8];
  uint32_t c = 0;
  for (int k = 0; k < 4; k++) {
    const uint32_t i = blockIdx.x * kCollectPer + k * 256 + threadIdx.x;
    if (i < n && collect_take(rec[i])) c++;
  }
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) wc[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; w++) t += wc[w];
    block_cnt[blockIdx.x] = t;
  }
}

__global__ void k_guide_collect_scan(const uint32_t* __restrict__ block_cnt, uint32_t nb,
                                     uint32_t* offsets, uint32_t* count, uint32_t cap) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  uint32_t t = 0;
  for (uint32_t b = 0; b < nb; b++) {
    offsets[b] = t;
    t += block_cnt[b];
  }
  *count = t < cap ? t : cap;
}

__global__ void __launch_bounds__(256) k_guide_collect_write(const GuideSample* __restrict__ rec,
                                                             uint32_t n,
                                                             const uint32_t* __restrict__ offsets,
                                                             GuideSample* out, float* block_w,
                                                             uint32_t cap, float exponent) {
  __shared__ uint32_t wtot[8];
  __shared__ float ws[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t run = offsets[blockIdx.x];
  float wacc = 0.f;
  for (int k = 0; k < 4; k++) {
    const uint32_t i = blockIdx.x * kCollectPer + k * 256 + threadIdx.x;
    GuideSample r;
    bool take = false;
    if (i < n) {
      r = rec[i];
      take = collect_take(r);
      if (take && exponent != 1.f) r.weight = powf(r.weight, exponent);
    }
    const uint32_t m = __ballot_sync(0xffffffffu, take);
    if (lane == 0) wtot[warp] = (uint32_t)__popc(m);
    __syncthreads();
    uint32_t before = 0, chunk = 0;
    for (int w = 0; w < 8; w++) {
      if (w < warp) before += wtot[w];
      chunk += wtot[w];
    }
    if (take) {
      const uint32_t dst = run + before + (uint32_t)__popc(m & ((1u << lane) - 1u));
      if (dst < cap) {
        out[dst] = r;
        wacc += r.weight;
      }
    }
    run += chunk;
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) wacc += __shfl_down_sync(0xffffffffu, wacc, o);
  if (lane == 0) ws[warp] = wacc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < 8; w++) t += ws[w];
    block_w[blockIdx.x] = t;
  }
}

__global__ void k_guide_collect_sum(const float* __restrict__ block_w, uint32_t nb, float* wsum) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  float t = 0.f;
  for (uint32_t b = 0; b < nb; b++) t += block_w[b];
  *wsum = t;
}

// ------------------------------------------------------------ launchers ----
namespace pt {

uint32_t guide_collect_blocks(uint32_t n) { return (n + kCollectPer - 1) / kCollectPer; }

void launch_guide_collect(const GuideSample* rec, uint32_t n, GuideSample* out, uint32_t* count,
                          float* wsum, uint32_t cap, float exponent, uint32_t* scratch_u,
                          float* scratch_f, cudaStream_t st) {
  const uint32_t nb = guide_collect_blocks(n);
  if (nb == 0) return;  // the caller zeroed count and wsum
  uint32_t* block_cnt = scratch_u;
  uint32_t* offsets = scratch_u + nb;
  k_guide_collect_count<<<nb, 256, 0, st>>>(rec, n, block_cnt);
  k_guide_collect_scan<<<1, 32, 0, st>>>(block_cnt, nb, offsets, count, cap);
  k_guide_collect_write<<<nb, 256, 0, st>>>(rec, n, offsets, out, scratch_f, cap, exponent);
  k_guide_collect_sum<<<1, 32, 0, st>>>(scratch_f, nb, wsum);
}

size_t guide_train_smem() { return (size_t)kWeights + 5 * kTileT + 2 * (kTileG + kGuard); }
size_t guide_infer_smem() { return (size_t)kWeights + 2 * kTileT; }  // 2 pipelines

cudaError_t guide_set_smem() {
  cudaError_t e = cudaFuncSetAttribute(k_guide_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)guide_train_smem());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)guide_infer_smem());
}

void launch_guide_grad(const GuideTrainArgs& a, int grid, cudaStream_t st) {
  k_guide_grad<<<grid, 128, guide_train_smem(), st>>>(a);
}

void launch_guide_adam(const GuideAdamArgs& a, cudaStream_t st) {
  k_guide_adam<<<(PTG_PARAMS + 255) / 256, 256, 0, st>>>(a);
}

void launch_guide_infer(const DevScene& S, const WaveState& W, const WaveCtl* ctl,
                        const GuideInferArgs& a, int grid, cudaStream_t st) {
  k_guide_select<<<grid * 4, 256, 0, st>>>(S, W, ctl, a.rows, a.feat);
  k_guide_infer<<<grid, 256, guide_infer_smem(), st>>>(S, W, ctl, a);
}

}  // namespace pt
