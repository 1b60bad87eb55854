/*
 * pt_guide.cuh - the learned sampling guide: a small MLP mapping the encoded
 * shading point (position, normal, outgoing direction) to a mixture of 8 von
 * Mises-Fisher lobes plus the probability of sampling that mixture instead of
 * the BSDF.  Shared by the guide kernels (pt_guide.cu) and consistent-mode
 * shading (pt_kernels.cu).  No counterpart in the reference.
 *
 * Network (every layer takes an 80-wide row: 64 activations or 76 features,
 * a constant 1 that carries the bias, zero padding):
 *   features (76) -> 64 -> 64 -> 64 -> 64 -> 41 (48 computed), ReLU between
 *   W1 [64 x 80] (bias in column 76), W2..W4 [64 x 80], W5 [48 x 80] (bias in
 *   column 64); rows 41..47 of W5 and the padding columns stay zero.
 * Outputs per lobe j (0..7): o[5j..5j+2] mean direction (normalised),
 *   o[5j+3] log concentration, o[5j+4] mixture logit (softmax over j);
 *   o[40] selection logit: alpha = 0.05 + 0.9 sigmoid(o[40]).
 * Sampling density of the guided bounce (one-sample MIS with the BSDF):
 *   q(w) = alpha p_guide(w) + (1 - alpha) p_bsdf(w),
 *   vMF(w; mu, k) = k / (2 pi (1 - e^{-2k})) exp(k (mu.w - 1)).
 */
#ifndef PT_GUIDE_CUH
#define PT_GUIDE_CUH

#include <stdint.h>

#define PTG_FEAT 76
#define PTG_K 80
#define PTG_H 64
#define PTG_OUT 41
#define PTG_NOUT 48
#define PTG_LOBES 8
#define PTG_FREQ 12
#define PTG_W_LAYER (64 * 80)              /* floats of W1..W4 */
#define PTG_W5 (48 * 80)
#define PTG_PARAMS (4 * PTG_W_LAYER + PTG_W5)  /* flat parameter vector (with padding) */
#define PTG_ALPHA_MIN 0.05f
#ifndef PTG_ALPHA_SPAN
#define PTG_ALPHA_SPAN 0.9f
#endif
#define PTG_LOGK_MIN -6.0f
#define PTG_LOGK_MAX 9.0f

/* Offset of layer l (0..4) in the flat parameter vector; rows of 80. */
#define PTG_LAYER_OFF(l) ((l) * PTG_W_LAYER)
#define PTG_LAYER_ROWS(l) ((l) == 4 ? PTG_NOUT : PTG_H)
#define PTG_BIAS_COL(l) ((l) == 0 ? PTG_FEAT : PTG_H)

/* Decoded guide of one shading point (the inference output). */
struct GuideParams {
  float4 lobe[PTG_LOBES];  /* mean direction xyz, concentration */
  float cdf[PTG_LOBES];    /* cumulative mixture weights (cdf[7] = 1) */
  float alpha;             /* probability of sampling the guide */
  float pad[3];
};

/* The guide as stored per path between inference and shading (96 B): eight
 * lobes as half (mean x, y, z, concentration), the cumulative mixture
 * weights as half (the last forced to 1) and alpha.  Sampling and density
 * both read these same values (means renormalised), so they stay
 * consistent. */
struct GuidePacked {
  uint2 lobe[PTG_LOBES];   /* half2 (mx, my), half2 (mz, kappa) */
  uint4 cdf;               /* 8 x half */
  float alpha;
  uint32_t pad[3];
};

/* A training sample: the shading point, the sampled direction, the BSDF pdf
 * of that direction and the sample's weight F/q (radiance carried back along
 * it times the BSDF and cosine, over the density it was sampled with). */
struct GuideSample {
  float P[3], N[3], Wo[3], wi[3];
  float p_bsdf, weight, pad[2];
};

#ifdef __CUDACC__
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

/* Kernel arguments (pt_guide.cu). */
struct GuideInferArgs {
  const __nv_bfloat16* w;   // BF16 weights, row-major, PTG_PARAMS
  GuidePacked* out;         // per buffer position
  uint32_t* rows;           // positions that need a guide this iteration (k_guide_select)
  float4* feat;             // per listed row: hit point, shading normal, Wo (3 float4)
  float bmin[3], binv[3];   // scene box for the position encoding
  uint32_t* fail;
  uint32_t wait_limit;      // try_waits per tensor-core completion wait
};

// Training / evaluation on explicit samples.
struct GuideTrainArgs {
  const __nv_bfloat16* w;
  const GuideSample* samples;
  const uint32_t* count;    // samples to use (device)
  const float* wsum;        // sum of their weights (device): loss = sum(-w log q) / wsum
  float* partial;           // per CTA: PTG_PARAMS gradient floats
  float* loss;              // accumulated loss (atomic)
  float* out;               // evaluation: 48 outputs per sample, or null
  float bmin[3], binv[3];
  int train;                // 1: backward + partial gradients
  uint32_t max_count;       // use at most this many samples (0: all)
  uint32_t* fail;
  uint32_t wait_limit;      // try_waits per tensor-core completion wait
};

struct GuideAdamArgs {
  const float* partial;
  int nparts;
  float* w32;
  __nv_bfloat16* wbf;
  float* m;
  float* v;
  float* grad_out;  // optional copy of the summed gradient
  float lr, b1, b2, eps, bc1, bc2;  // bc = 1 - beta^t
  int update;
};


struct DevScene;
struct WaveState;
struct WaveCtl;
namespace pt {
size_t guide_train_smem();
size_t guide_infer_smem();
cudaError_t guide_set_smem();
/* grid: persistent CTAs (one per SM); each writes PTG_PARAMS partial floats */
void launch_guide_grad(const GuideTrainArgs& a, int grid, cudaStream_t st);
void launch_guide_adam(const GuideAdamArgs& a, cudaStream_t st);
void launch_guide_infer(const DevScene& S, const WaveState& W, const WaveCtl* ctl,
                        const GuideInferArgs& a, int grid, cudaStream_t st);
/* Appends the completed records with a positive weight to out (at most cap;
 * count and wsum accumulate on the device). */
// scratch: 2 x guide_collect_blocks(n) uint32 and guide_collect_blocks(n) floats
uint32_t guide_collect_blocks(uint32_t n);
void launch_guide_collect(const GuideSample* rec, uint32_t n, GuideSample* out, uint32_t* count,
                          float* wsum, uint32_t cap, float exponent, uint32_t* scratch_u,
                          float* scratch_f, cudaStream_t st);
}  // namespace pt
#endif

#ifdef __CUDACC__
#define PTG_FN __host__ __device__ __forceinline__
#else
#define PTG_FN inline
#endif

/* Feature row of a shading point: position normalised by the scene box to
 * [0,1]^3, encoded as sin/cos(2^k pi x) for k = 0..11 (the doubling
 * recurrence from k = 0), then normal and outgoing direction as (theta/pi,
 * phi/2pi + 1/2).  Writes PTG_FEAT floats. */
PTG_FN void guide_features(const float P[3], const float N[3], const float Wo[3],
                           const float bmin[3], const float binv[3], float* f) {
  for (int a = 0; a < 3; a++) {
    float x = (P[a] - bmin[a]) * binv[a];
    x = fminf(fmaxf(x, 0.f), 1.f);
    float s, c;
#ifdef __CUDA_ARCH__
    sincospif(x, &s, &c);
#else
    s = (float)sin(3.14159265358979323846 * (double)x);
    c = (float)cos(3.14159265358979323846 * (double)x);
#endif
    for (int k = 0; k < PTG_FREQ; k++) {
      f[a * 2 * PTG_FREQ + 2 * k] = s;
      f[a * 2 * PTG_FREQ + 2 * k + 1] = c;
      float s2 = 2.f * s * c, c2 = 1.f - 2.f * s * s;
      s = s2;
      c = c2;
    }
  }
  const float* dirs[2] = {N, Wo};
  for (int q = 0; q < 2; q++) {
    const float* d = dirs[q];
    float y = fminf(fmaxf(d[1], -1.f), 1.f);
    f[72 + 2 * q] = acosf(y) * 0.31830988618379067f;
    f[73 + 2 * q] = atan2f(d[2], d[0]) * 0.15915494309189535f + 0.5f;
  }
}

/* Decodes the 41 outputs; lobe means fall back to +y for a zero vector. */
PTG_FN void guide_decode(const float* o, GuideParams& g) {
  float mx = -3.0e38f;
  for (int j = 0; j < PTG_LOBES; j++) mx = fmaxf(mx, o[5 * j + 4]);
  float e[PTG_LOBES], sum = 0.f;
  for (int j = 0; j < PTG_LOBES; j++) {
    e[j] = expf(o[5 * j + 4] - mx);
    sum += e[j];
  }
  float acc = 0.f;
  for (int j = 0; j < PTG_LOBES; j++) {
    float x = o[5 * j], y = o[5 * j + 1], z = o[5 * j + 2];
    float n = sqrtf(x * x + y * y + z * z);
    if (n > 1e-12f) {
      x /= n;
      y /= n;
      z /= n;
    } else {
      x = 0.f;
      y = 1.f;
      z = 0.f;
    }
    float lk = fminf(fmaxf(o[5 * j + 3], PTG_LOGK_MIN), PTG_LOGK_MAX);
    g.lobe[j] = make_float4(x, y, z, expf(lk));
    acc += e[j] / sum;
    g.cdf[j] = acc;
  }
  g.cdf[PTG_LOBES - 1] = 1.f;
  g.alpha = PTG_ALPHA_MIN + PTG_ALPHA_SPAN / (1.f + expf(-o[40]));
}

/* vMF density of unit direction w around unit mean mu, concentration k. */
PTG_FN float vmf_pdf(float mx, float my, float mz, float k, float wx, float wy, float wz) {
  float c = mx * wx + my * wy + mz * wz;
  if (k < 1e-4f) return 0.07957747154594767f;  /* 1/(4 pi) */
  return k / (6.283185307179586f * -expm1f(-2.f * k)) * expf(k * (c - 1.f));
}

PTG_FN float guide_pdf(const GuideParams& g, float wx, float wy, float wz) {
  float p = 0.f, prev = 0.f;
  for (int j = 0; j < PTG_LOBES; j++) {
    float wj = g.cdf[j] - prev;
    prev = g.cdf[j];
    p += wj * vmf_pdf(g.lobe[j].x, g.lobe[j].y, g.lobe[j].z, g.lobe[j].w, wx, wy, wz);
  }
  return p;
}

/* Samples a direction from the mixture with uniforms u0 (lobe), u1, u2
 * (Jakob 2012, "Numerically stable sampling of the von Mises Fisher
 * distribution on S^2"). */
PTG_FN void guide_sample(const GuideParams& g, float u0, float u1, float u2, float& wx, float& wy,
                         float& wz) {
  int j = 0;
  while (j < PTG_LOBES - 1 && u0 >= g.cdf[j]) j++;
  float mx = g.lobe[j].x, my = g.lobe[j].y, mz = g.lobe[j].z, k = g.lobe[j].w;
  float w;
  if (k < 1e-4f) w = 1.f - 2.f * u1;
  else w = 1.f + logf(u1 + (1.f - u1) * expf(-2.f * k)) / k;
  w = fminf(fmaxf(w, -1.f), 1.f);
  float r = sqrtf(fmaxf(0.f, 1.f - w * w));
  float s, c;
#ifdef __CUDA_ARCH__
  sincospif(2.f * u2, &s, &c);
#else
  s = (float)sin(6.283185307179586 * (double)u2);
  c = (float)cos(6.283185307179586 * (double)u2);
#endif
  // orthonormal basis around the mean (Duff et al. 2017)
  float sign = mz >= 0.f ? 1.f : -1.f;
  float a = -1.f / (sign + mz), b = mx * my * a;
  float tx = 1.f + sign * mx * mx * a, ty = sign * b, tz = -sign * mx;
  float bx = b, by = sign + my * my * a, bz = -my;
  wx = r * c * tx + r * s * bx + w * mx;
  wy = r * c * ty + r * s * by + w * my;
  wz = r * c * tz + r * s * bz + w * mz;
}

#ifdef __CUDACC__
/* ---- packed guide (device) ---------------------------------------------- */
__device__ __forceinline__ GuidePacked guide_pack(const GuideParams& g) {
  GuidePacked p;
  for (int j = 0; j < PTG_LOBES; j++) {
    __half2 a = __floats2half2_rn(g.lobe[j].x, g.lobe[j].y);
    __half2 b = __floats2half2_rn(g.lobe[j].z, g.lobe[j].w);
    p.lobe[j] = make_uint2(*(uint32_t*)&a, *(uint32_t*)&b);
  }
  __half2 c0 = __floats2half2_rn(g.cdf[0], g.cdf[1]), c1 = __floats2half2_rn(g.cdf[2], g.cdf[3]);
  __half2 c2 = __floats2half2_rn(g.cdf[4], g.cdf[5]), c3 = __floats2half2_rn(g.cdf[6], 1.f);
  p.cdf = make_uint4(*(uint32_t*)&c0, *(uint32_t*)&c1, *(uint32_t*)&c2, *(uint32_t*)&c3);
  p.alpha = g.alpha;
  p.pad[0] = p.pad[1] = p.pad[2] = 0u;
  return p;
}

/* Shading reads the packed guide with fast intrinsics (rsqrt, exp, divide):
 * the guide has no bit-exact contract, only that its sampler and its density
 * agree, which they do to float rounding (both use these same functions). */
/* Lobe j of a packed guide in global memory: unit mean and concentration. */
__device__ __forceinline__ void guide_lobe(const GuidePacked* __restrict__ g, int j, float& mx,
                                           float& my, float& mz, float& k) {
  uint2 v = __ldg(&g->lobe[j]);
  float2 a = __half22float2(*(__half2*)&v.x), b = __half22float2(*(__half2*)&v.y);
  float n2 = a.x * a.x + a.y * a.y + b.x * b.x;
  if (n2 > 1e-20f) {
    float inv = rsqrtf(n2);
    mx = a.x * inv;
    my = a.y * inv;
    mz = b.x * inv;
  } else {
    mx = 0.f;
    my = 1.f;
    mz = 0.f;
  }
  k = b.y;
}

__device__ __forceinline__ void guide_cdf(const GuidePacked* __restrict__ g, float* cdf) {
  uint4 v = __ldg(&g->cdf);
  uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    float2 f = __half22float2(*(__half2*)&w[q]);
    cdf[2 * q] = f.x;
    cdf[2 * q + 1] = f.y;
  }
  cdf[PTG_LOBES - 1] = 1.f;
}

// vMF density with intrinsics; a series near k = 0 keeps the normaliser
// k / (1 - e^{-2k}) accurate where the exponential cancels.
__device__ __forceinline__ float vmf_pdf_fast(float mx, float my, float mz, float k, float wx,
                                              float wy, float wz) {
  float c = mx * wx + my * wy + mz * wz;
  float norm;
  if (k < 1e-3f) norm = 0.5f + 0.5f * k;  // k / (1 - e^{-2k}) = 1/2 + k/2 + O(k^2)
  else norm = __fdividef(k, 1.f - __expf(-2.f * k));
  return norm * 0.15915494309189535f * __expf(k * (c - 1.f));
}

__device__ __forceinline__ float guide_pdf_packed(const GuidePacked* __restrict__ g, float wx,
                                                  float wy, float wz) {
  float cdf[PTG_LOBES];
  guide_cdf(g, cdf);
  float p = 0.f, prev = 0.f;
#pragma unroll
  for (int j = 0; j < PTG_LOBES; j++) {
    float mx, my, mz, k;
    guide_lobe(g, j, mx, my, mz, k);
    p += (cdf[j] - prev) * vmf_pdf_fast(mx, my, mz, k, wx, wy, wz);
    prev = cdf[j];
  }
  return p;
}

/* Samples lobe j with probability cdf[j] - cdf[j-1], then the lobe's vMF
 * (Jakob 2012); the same lobe values as guide_pdf_packed. */
__device__ __forceinline__ void guide_sample_packed(const GuidePacked* __restrict__ g, float u0,
                                                    float u1, float u2, float& wx, float& wy,
                                                    float& wz) {
  float cdf[PTG_LOBES];
  guide_cdf(g, cdf);
  int j = 0;
#pragma unroll
  for (int q = 0; q < PTG_LOBES - 1; q++) j += u0 >= cdf[q] ? 1 : 0;
  float mx, my, mz, k;
  guide_lobe(g, j, mx, my, mz, k);
  float w;
  if (k < 1e-3f) {
    // series of log(u + (1-u) e^{-2k}) / k for small k: -2(1-u) + ...; the
    // uniform limit at k -> 0
    w = 1.f - 2.f * (1.f - u1) * (1.f - k * u1);
  } else {
    w = 1.f + __logf(u1 + (1.f - u1) * __expf(-2.f * k)) / k;
  }
  w = fminf(fmaxf(w, -1.f), 1.f);
  float r = sqrtf(fmaxf(0.f, 1.f - w * w));
  float s, c;
  __sincosf(6.283185307179586f * u2, &s, &c);
  float sign = mz >= 0.f ? 1.f : -1.f;
  float a = -1.f / (sign + mz), b = mx * my * a;
  float tx = 1.f + sign * mx * mx * a, ty = sign * b, tz = -sign * mx;
  float bx = b, by = sign + my * my * a, bz = -my;
  wx = r * c * tx + r * s * bx + w * mx;
  wy = r * c * ty + r * s * by + w * my;
  wz = r * c * tz + r * s * bz + w * mz;
}
#endif

#endif
