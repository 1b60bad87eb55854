/*
 * pt_guide_host.cu - host side of the learned sampling guide (pt_guide_* in
 * include/pt.h): weight initialisation, Adam state, the scene box of the
 * position encoding, and the evaluation / gradient / training entry points
 * used by the renderer's online training and by the tests.
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pt.h"
#include "pt_context.h"
#include "pt_guide.cuh"
#include "pt_internal.h"

using namespace pth;

static int gfail(pt_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

#define GK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return gfail(ctx, e_ == cudaErrorMemoryAllocation ? PT_ENOMEM : PT_ECUDA,   \
                   std::string(#call) + ": " + cudaGetErrorString(e_));           \
  } while (0)

namespace {

// splitmix64 (Steele, Lea & Flood 2014) for the weight initialisation.
struct Mix64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  float uniform() { return (float)((next() >> 40) * (1.0 / 16777216.0)); }
};

bool param_used(int p) {
  int l = p / PTG_W_LAYER, e = p - l * PTG_W_LAYER;
  int r = e / PTG_K, c = e % PTG_K;
  return r < (l == 4 ? PTG_OUT : PTG_H) && c <= PTG_BIAS_COL(l);
}

}  // namespace

// Allocates the guide buffers (once) and computes the scene box of the
// position encoding (padded by 1e-3 of its extent).
int pth::guide_prepare(pt_context* ctx) {
  GuideState& G = ctx->guide;
  if (!G.w32.p) {
    GK(G.w32.ensure(PTG_PARAMS));
    GK(G.m.ensure(PTG_PARAMS));
    GK(G.v.ensure(PTG_PARAMS));
    GK(G.wbf.ensure(PTG_PARAMS));
    GK(G.grad.ensure(PTG_PARAMS));
    GK(G.scalars.ensure(2));
    GK(G.counters.ensure(4));
    GK(cudaMemset(G.counters.p, 0, 16));
    int dev = 0, sms = 0;
    GK(cudaGetDevice(&dev));
    GK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    G.grid = std::max(1, sms);
    GK(G.partial.ensure((size_t)G.grid * PTG_PARAMS));
    GK(pt::guide_set_smem());
  }
  if (!G.bounds) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (const HostPrim& p : ctx->prims) {
      pt::Box b = prim_bounds(ctx, p);
      for (int a = 0; a < 3; a++) {
        lo[a] = std::min(lo[a], b.lo[a]);
        hi[a] = std::max(hi[a], b.hi[a]);
      }
    }
    for (int a = 0; a < 3; a++) {
      if (!(lo[a] <= hi[a])) {
        lo[a] = -1.f;
        hi[a] = 1.f;
      }
      float ext = std::max(hi[a] - lo[a], 1e-6f);
      G.bmin[a] = lo[a] - 1e-3f * ext;
      G.binv[a] = 1.f / (ext * 1.002f);
    }
    G.bounds = true;
  }
  return PT_OK;
}

GuideInferArgs pth::guide_infer_args(pt_context* ctx) {
  GuideState& G = ctx->guide;
  GuideInferArgs a;
  memset(&a, 0, sizeof(a));
  a.w = (const __nv_bfloat16*)G.wbf.p;
  a.out = G.out.p;
  a.rows = G.rows.p;
  a.feat = G.feat.p;
  memcpy(a.bmin, G.bmin, sizeof(a.bmin));
  memcpy(a.binv, G.binv, sizeof(a.binv));
  a.fail = G.counters.p + 2;  // read back at the end of a guided render
  a.wait_limit = G.wait_limit;
  return a;
}

int pth::guide_frame_begin(pt_context* ctx, int w, int h) {
  GuideState& G = ctx->guide;
  const size_t target = (size_t)1 << 18;  // recording paths per frame (2 records each)
  size_t wh = (size_t)w * h;
  G.rec_stride = (uint32_t)std::max<size_t>(1, (wh + target - 1) / target);
  G.rec_n = (uint32_t)(2 * ((wh + G.rec_stride - 1) / G.rec_stride));
  GK(G.rec.ensure(G.rec_n));
  GK(G.coll_u.ensure(2 * (size_t)pt::guide_collect_blocks(G.rec_n) + 1));
  GK(G.coll_f.ensure((size_t)pt::guide_collect_blocks(G.rec_n) + 1));
  GK(G.samples.ensure((size_t)1 << 19));
  GK(cudaMemsetAsync(G.rec.p, 0, (size_t)G.rec_n * sizeof(GuideSample), ctx->stream));
  return PT_OK;
}

int pth::guide_frame_train(pt_context* ctx) {
  GuideState& G = ctx->guide;
  cudaStream_t st = ctx->stream;
  const uint32_t cap = 1u << 19;
  GK(cudaMemsetAsync(G.counters.p, 0, 4, st));  // the failure flags stay
  GK(cudaMemsetAsync(G.scalars.p, 0, 8, st));
  pt::launch_guide_collect(G.rec.p, G.rec_n, G.samples.p, G.counters.p, G.scalars.p + 1, cap,
                           G.exponent, G.coll_u.p, G.coll_f.p, st);
  GuideTrainArgs a;
  memset(&a, 0, sizeof(a));
  a.w = (const __nv_bfloat16*)G.wbf.p;
  a.samples = G.samples.p;
  a.count = G.counters.p;
  a.wsum = G.scalars.p + 1;
  a.partial = G.partial.p;
  a.loss = G.scalars.p;
  memcpy(a.bmin, G.bmin, sizeof(a.bmin));
  memcpy(a.binv, G.binv, sizeof(a.binv));
  a.train = 1;
  a.max_count = cap;
  a.fail = G.counters.p + 1;
  a.wait_limit = G.wait_limit;
  for (int k = 0; k < G.steps; k++) {
    pt::launch_guide_grad(a, G.grid, st);
    GuideAdamArgs d;
    memset(&d, 0, sizeof(d));
    d.partial = G.partial.p;
    d.nparts = G.grid;
    d.w32 = G.w32.p;
    d.wbf = (__nv_bfloat16*)G.wbf.p;
    d.m = G.m.p;
    d.v = G.v.p;
    d.update = 1;
    G.step++;
    d.lr = G.lr;
    d.b1 = 0.9f;
    d.b2 = 0.99f;
    d.eps = 1e-8f;
    d.bc1 = 1.f - powf(d.b1, (float)G.step);
    d.bc2 = 1.f - powf(d.b2, (float)G.step);
    pt::launch_guide_adam(d, st);
  }
  GK(cudaGetLastError());
  return PT_OK;
}

static int upload_params(pt_context* ctx, const std::vector<float>& w) {
  GuideState& G = ctx->guide;
  std::vector<uint16_t> bf(PTG_PARAMS);
  for (int p = 0; p < PTG_PARAMS; p++) {
    __nv_bfloat16 h = __float2bfloat16_rn(w[p]);
    memcpy(&bf[p], &h, 2);
  }
  GK(cudaMemcpyAsync(G.w32.p, w.data(), PTG_PARAMS * 4, cudaMemcpyHostToDevice, ctx->stream));
  GK(cudaMemcpyAsync(G.wbf.p, bf.data(), PTG_PARAMS * 2, cudaMemcpyHostToDevice, ctx->stream));
  GK(cudaMemsetAsync(G.m.p, 0, PTG_PARAMS * 4, ctx->stream));
  GK(cudaMemsetAsync(G.v.p, 0, PTG_PARAMS * 4, ctx->stream));
  GK(cudaStreamSynchronize(ctx->stream));
  G.step = 0;
  G.ready = true;
  return PT_OK;
}

// Runs the gradient kernel on `n` device samples (G.samples) and sums the
// partials; update: one Adam step with learning rate lr.
static int guide_step(pt_context* ctx, int n, bool update, float lr, float* loss_out,
                      float* grad_host) {
  GuideState& G = ctx->guide;
  cudaStream_t st = ctx->stream;
  uint32_t cnt[2] = {(uint32_t)n, 0u};
  GK(cudaMemcpyAsync(G.counters.p, cnt, sizeof(cnt), cudaMemcpyHostToDevice, st));
  GuideTrainArgs a;
  memset(&a, 0, sizeof(a));
  a.w = (const __nv_bfloat16*)G.wbf.p;
  a.samples = G.samples.p;
  a.count = G.counters.p;
  a.wsum = G.scalars.p + 1;
  a.partial = G.partial.p;
  a.loss = G.scalars.p;
  a.out = nullptr;
  memcpy(a.bmin, G.bmin, sizeof(a.bmin));
  memcpy(a.binv, G.binv, sizeof(a.binv));
  a.train = 1;
  a.fail = G.counters.p + 1;
  a.wait_limit = G.wait_limit;
  GK(cudaMemsetAsync(G.scalars.p, 0, 4, st));
  pt::launch_guide_grad(a, G.grid, st);
  GK(cudaGetLastError());
  GuideAdamArgs d;
  memset(&d, 0, sizeof(d));
  d.partial = G.partial.p;
  d.nparts = G.grid;
  d.w32 = G.w32.p;
  d.wbf = (__nv_bfloat16*)G.wbf.p;
  d.m = G.m.p;
  d.v = G.v.p;
  d.grad_out = G.grad.p;
  d.update = update ? 1 : 0;
  if (update) G.step++;
  d.lr = lr;
  d.b1 = 0.9f;
  d.b2 = 0.99f;
  d.eps = 1e-8f;
  d.bc1 = 1.f - powf(d.b1, (float)std::max(1, G.step));
  d.bc2 = 1.f - powf(d.b2, (float)std::max(1, G.step));
  pt::launch_guide_adam(d, st);
  GK(cudaGetLastError());
  float loss = 0.f;
  uint32_t h_cnt[2];
  GK(cudaMemcpyAsync(&loss, G.scalars.p, 4, cudaMemcpyDeviceToHost, st));
  GK(cudaMemcpyAsync(h_cnt, G.counters.p, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
  if (grad_host) GK(cudaMemcpyAsync(grad_host, G.grad.p, PTG_PARAMS * 4, cudaMemcpyDeviceToHost, st));
  GK(cudaStreamSynchronize(st));
  if (h_cnt[1]) return gfail(ctx, PT_ETIMEOUT, "guide kernel: tensor-core wait ran out");
  if (loss_out) *loss_out = loss;
  return PT_OK;
}

static int upload_samples(pt_context* ctx, const float* samples, int n) {
  GuideState& G = ctx->guide;
  GK(G.samples.ensure((size_t)std::max(n, 1)));
  const GuideSample* s = (const GuideSample*)samples;
  double wsum = 0.0;
  for (int i = 0; i < n; i++) wsum += s[i].weight;
  float ws = (float)wsum;
  GK(cudaMemcpyAsync(G.samples.p, samples, (size_t)n * sizeof(GuideSample), cudaMemcpyHostToDevice,
                     ctx->stream));
  GK(cudaMemcpyAsync(G.scalars.p + 1, &ws, 4, cudaMemcpyHostToDevice, ctx->stream));
  GK(cudaStreamSynchronize(ctx->stream));
  return PT_OK;
}

extern "C" {

PT_API int pt_guide_init(pt_context* ctx, uint64_t seed) {
  if (!ctx) return PT_EINVAL;
  GK(cudaSetDevice(ctx->device));
  int rc = guide_prepare(ctx);
  if (rc) return rc;
  // He-uniform hidden layers; a small last layer so the first mixture is
  // broad (concentration ~1, equal weights, alpha = 0.5); biases zero.  The
  // training options keep their values.
  Mix64 r{seed ^ 0x6A09E667F3BCC909ull};
  std::vector<float> w(PTG_PARAMS, 0.f);
  for (int l = 0; l < 5; l++) {
    int rows = l == 4 ? PTG_OUT : PTG_H;
    int fan_in = l == 0 ? PTG_FEAT : PTG_H;
    float lim = std::sqrt(6.f / (float)fan_in) * (l == 4 ? 0.1f : 1.f);
    for (int i = 0; i < rows; i++)
      for (int c = 0; c < fan_in; c++)
        w[PTG_LAYER_OFF(l) + i * PTG_K + c] = (2.f * r.uniform() - 1.f) * lim;
  }
  return upload_params(ctx, w);
}

PT_API int pt_guide_set_wait_limit(pt_context* ctx, uint32_t try_waits) {
  if (!ctx) return PT_EINVAL;
  ctx->guide.wait_limit = try_waits;
  return PT_OK;
}

PT_API int pt_guide_set_training(pt_context* ctx, float lr, int steps_per_frame, float exponent,
                                 int max_bounces) {
  if (!ctx) return PT_EINVAL;
  if (!(lr > 0.f) || lr > 1.f || steps_per_frame < 1 || steps_per_frame > 64 ||
      !(exponent > 0.f) || exponent > 1.f || max_bounces < 0)
    return gfail(ctx, PT_EINVAL,
                 "guide training: lr in (0,1], 1..64 steps, exponent in (0,1], bounces >= 0");
  ctx->guide.lr = lr;
  ctx->guide.steps = steps_per_frame;
  ctx->guide.exponent = exponent;
  ctx->guide.max_bounces = max_bounces;
  return PT_OK;
}

PT_API int pt_guide_get_params(pt_context* ctx, float* params) {
  if (!ctx || !params) return PT_EINVAL;
  if (!ctx->guide.ready) return gfail(ctx, PT_ESTATE, "guide not initialised (pt_guide_init)");
  GK(cudaSetDevice(ctx->device));
  GK(cudaMemcpy(params, ctx->guide.w32.p, PTG_PARAMS * 4, cudaMemcpyDeviceToHost));
  return PT_OK;
}

PT_API int pt_guide_set_params(pt_context* ctx, const float* params) {
  if (!ctx || !params) return PT_EINVAL;
  GK(cudaSetDevice(ctx->device));
  int rc = guide_prepare(ctx);
  if (rc) return rc;
  std::vector<float> w(params, params + PTG_PARAMS);
  for (int p = 0; p < PTG_PARAMS; p++) {
    if (!param_used(p)) w[p] = 0.f;
    if (!std::isfinite(w[p])) return gfail(ctx, PT_EINVAL, "guide parameters must be finite");
  }
  return upload_params(ctx, w);
}

PT_API int pt_guide_get_state(pt_context* ctx, float* state, int64_t* step) {
  if (!ctx || !state || !step) return PT_EINVAL;
  if (!ctx->guide.ready) return gfail(ctx, PT_ESTATE, "guide not initialised (pt_guide_init)");
  GK(cudaSetDevice(ctx->device));
  GuideState& G = ctx->guide;
  GK(cudaStreamSynchronize(ctx->stream));
  GK(cudaMemcpy(state, G.w32.p, PTG_PARAMS * 4, cudaMemcpyDeviceToHost));
  GK(cudaMemcpy(state + PTG_PARAMS, G.m.p, PTG_PARAMS * 4, cudaMemcpyDeviceToHost));
  GK(cudaMemcpy(state + 2 * PTG_PARAMS, G.v.p, PTG_PARAMS * 4, cudaMemcpyDeviceToHost));
  *step = G.step;
  return PT_OK;
}

PT_API int pt_guide_set_state(pt_context* ctx, const float* state, int64_t step) {
  if (!ctx || !state || step < 0 || step > 0x7fffffff) return PT_EINVAL;
  GK(cudaSetDevice(ctx->device));
  int rc = guide_prepare(ctx);
  if (rc) return rc;
  for (int p = 0; p < 3 * PTG_PARAMS; p++)
    if (!std::isfinite(state[p]) || (p >= 2 * PTG_PARAMS && state[p] < 0.f))
      return gfail(ctx, PT_EINVAL, "guide state: finite values, second moments >= 0");
  std::vector<float> w(state, state + PTG_PARAMS);
  for (int p = 0; p < PTG_PARAMS; p++)
    if (!param_used(p)) w[p] = 0.f;
  rc = upload_params(ctx, w);  // weights and their BF16 copy; moments zeroed
  if (rc) return rc;
  GuideState& G = ctx->guide;
  GK(cudaMemcpyAsync(G.m.p, state + PTG_PARAMS, PTG_PARAMS * 4, cudaMemcpyHostToDevice,
                     ctx->stream));
  GK(cudaMemcpyAsync(G.v.p, state + 2 * PTG_PARAMS, PTG_PARAMS * 4, cudaMemcpyHostToDevice,
                     ctx->stream));
  GK(cudaStreamSynchronize(ctx->stream));
  G.step = (int)step;
  return PT_OK;
}

PT_API int pt_guide_bounds(pt_context* ctx, float bmin[3], float binv[3]) {
  if (!ctx || !bmin || !binv) return PT_EINVAL;
  GK(cudaSetDevice(ctx->device));
  int rc = guide_prepare(ctx);
  if (rc) return rc;
  memcpy(bmin, ctx->guide.bmin, 12);
  memcpy(binv, ctx->guide.binv, 12);
  return PT_OK;
}

PT_API int pt_guide_eval(pt_context* ctx, const float* samples, int n, float* outputs) {
  if (!ctx || !samples || !outputs || n <= 0) return PT_EINVAL;
  if (!ctx->guide.ready) return gfail(ctx, PT_ESTATE, "guide not initialised (pt_guide_init)");
  GK(cudaSetDevice(ctx->device));
  GuideState& G = ctx->guide;
  int rc = upload_samples(ctx, samples, n);
  if (rc) return rc;
  GK(G.eval_out.ensure((size_t)n * PTG_NOUT));
  uint32_t cnt[2] = {(uint32_t)n, 0u};
  GK(cudaMemcpyAsync(G.counters.p, cnt, sizeof(cnt), cudaMemcpyHostToDevice, ctx->stream));
  GuideTrainArgs a;
  memset(&a, 0, sizeof(a));
  a.w = (const __nv_bfloat16*)G.wbf.p;
  a.samples = G.samples.p;
  a.count = G.counters.p;
  a.wsum = G.scalars.p + 1;
  a.out = G.eval_out.p;
  memcpy(a.bmin, G.bmin, sizeof(a.bmin));
  memcpy(a.binv, G.binv, sizeof(a.binv));
  a.train = 0;
  a.fail = G.counters.p + 1;
  a.wait_limit = G.wait_limit;
  pt::launch_guide_grad(a, G.grid, ctx->stream);
  GK(cudaGetLastError());
  uint32_t h_cnt[2];
  GK(cudaMemcpyAsync(outputs, G.eval_out.p, (size_t)n * PTG_NOUT * 4, cudaMemcpyDeviceToHost,
                     ctx->stream));
  GK(cudaMemcpyAsync(h_cnt, G.counters.p, sizeof(h_cnt), cudaMemcpyDeviceToHost, ctx->stream));
  GK(cudaStreamSynchronize(ctx->stream));
  if (h_cnt[1]) return gfail(ctx, PT_ETIMEOUT, "guide kernel: tensor-core wait ran out");
  return PT_OK;
}

PT_API int pt_guide_gradient(pt_context* ctx, const float* samples, int n, float* grad,
                             float* loss) {
  if (!ctx || !samples || n <= 0) return PT_EINVAL;
  if (!ctx->guide.ready) return gfail(ctx, PT_ESTATE, "guide not initialised (pt_guide_init)");
  GK(cudaSetDevice(ctx->device));
  int rc = upload_samples(ctx, samples, n);
  if (rc) return rc;
  return guide_step(ctx, n, false, 0.f, loss, grad);
}

PT_API int pt_guide_train(pt_context* ctx, const float* samples, int n, float lr, float* loss) {
  if (!ctx || !samples || n <= 0 || !(lr > 0.f)) return PT_EINVAL;
  if (!ctx->guide.ready) return gfail(ctx, PT_ESTATE, "guide not initialised (pt_guide_init)");
  GK(cudaSetDevice(ctx->device));
  int rc = upload_samples(ctx, samples, n);
  if (rc) return rc;
  return guide_step(ctx, n, true, lr, loss, nullptr);
}

}  // extern "C"
