/*
 * pt_batch.cu - batched multi-scene rendering (pt_batch_* in include/pt.h).
 *
 * Many committed scenes render in one wavefront.  The batch copies every
 * scene's geometry into one set of arrays, shifting node, record, primitive,
 * transform, material and attribute indices (k_relocate_*), so a traced ray
 * needs only its scene's root node.  Camera, miss program, lights,
 * environment tables and path controls of each item sit in a scene table
 * indexed by the scene bits of the path state.
 *
 * The work is cut into chunks: runs of whole frames of consecutive items with
 * at most 2 GiB of per-path results.  The whole batch is ONE graph launch:
 *
 *   while (a chunk is left)             conditional node, set on the device
 *     k_batch_begin                     load the chunk, reset the queues
 *     while (the chunk has paths left)  conditional node, set on the device
 *       generate, trace, shade, shadow trace, finish, advance
 *     k_accumulate_batch, k_batch_end
 *
 * Both loops are bounded on the device (by the chunk count, and per chunk by
 * (ceil(paths / slots) + 2) * (max depth + 1) + 16 iterations: every path
 * ends within max depth iterations of its generation, and generation keeps
 * the slots full while paths remain) and end on any error flag.  With
 * per-stage timing, or where the runtime refuses conditional nodes, the same
 * kernels run under a host loop.
 *
 * Frames are accumulated per pixel in frame order exactly as pt_render does,
 * so every item's accumulator is bit-identical to its own pt_render.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/pt.h"
#include "pt_context.h"
#include "pt_internal.h"

using namespace pth;

namespace {

// Everything a captured graph bakes in; a change means re-capture.
struct GraphSig {
  DevScene merged;
  WaveState W;
  BatchRefs br;
  const void* chunks;
  const void* ctl;
  LaunchCfg lc;
  int max_stack, mode, counters, timing, device_loop;
};

struct ScenePart {  // one distinct context inside the batch arrays
  pt_context* ctx;
  uint64_t gen;
  uint32_t root;
};

}  // namespace

struct pt_batch {
  int device = 0;
  std::string err;
  pt_options opt{};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  pt_tune tune{};
  // ---- batch geometry (copies of the scenes)
  std::vector<ScenePart> parts;
  int parts_width = 0;
  DevBuf<uint4> nodes, tri_attr;
  DevBuf<float4> prims, xforms;
  DevBuf<GpuMaterial> mats;
  DevBuf<float> normals, uvs;
  DevBuf<uint32_t> leaf_of_id;
  int max_stack = 1;
  size_t total_nodes = 0;
  DevScene merged{};
  // ---- tables
  DevBuf<BatchScene> d_scenes;
  DevBuf<BatchSeg> d_segs;
  DevBuf<BatchChunk> d_chunks;
  DevBuf<uint32_t> d_roots;
  DevBuf<float4> d_stage;  // device copies of host accumulators
  DevBuf<float4> d_tune_acc;
  // ---- wavefront
  int slots = 0;
  WaveState W{};
  DevBuf<float4> slot_f4;
  DevBuf<uint4> slot_u4;
  DevBuf<WaveCounters> d_ctr;
  DevBuf<WaveCtl> d_ctl;
  DevBuf<float4> d_results;
  WaveCounters* h_ctr = nullptr;
  LaunchCfg lc{};
  // ---- graphs
  cudaGraphExec_t exec = nullptr;  // device loop, or 8 iterations (host loop)
  GraphSig sig{};
  bool cond_ok = true;             // conditional nodes usable
  std::vector<cudaEvent_t> tev;
  pt_stats stats{};
};

static int bfail(pt_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

static int bcuda(pt_batch* b, cudaError_t e, const char* where) {
  return bfail(b, e == cudaErrorMemoryAllocation ? PT_ENOMEM : PT_ECUDA,
               std::string(where) + ": " + cudaGetErrorString(e));
}

#define BK(call)                                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return bcuda(b, e_, #call);  \
  } while (0)

static const int kItersPerGraph = 8;
static const size_t kResultsCap = (size_t)1 << 27;  // paths per chunk: 2 GiB of results

static bool tune_valid(const pt_tune& t) {
  return t.path_slots >= 1024 && t.path_slots <= (1 << 24) &&
         (t.trace_block == 64 || t.trace_block == 128 || t.trace_block == 256) &&
         t.shade_block >= 64 && t.shade_block <= PT_SHADE_BLOCK && t.shade_block % 32 == 0 &&
         t.bvh_width >= 2 && t.bvh_width <= 8 && t.chunk_paths >= 0 &&
         t.shade_order >= 0 && t.shade_order <= 2 && t.refetch_lanes >= 0 && t.refetch_lanes <= 32;
}

static void drop_graph(pt_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
}

// ------------------------------------------------------- batch geometry ----
// Copies the distinct scenes of the items into the batch arrays (building
// each scene's BVH again when its node width differs from the batch's).
static int ensure_geometry(pt_batch* b, const pt_batch_item* items, int n) {
  cudaStream_t st = b->stream;
  const int width = b->tune.bvh_width;
  std::vector<pt_context*> ctxs;
  std::unordered_map<pt_context*, int> index;
  for (int i = 0; i < n; i++)
    if (index.emplace(items[i].scene, (int)ctxs.size()).second) ctxs.push_back(items[i].scene);
  bool same = b->parts_width == width && b->parts.size() == ctxs.size();
  for (size_t k = 0; same && k < ctxs.size(); k++)
    same = b->parts[k].ctx == ctxs[k] && b->parts[k].gen == ctxs[k]->commit_gen;
  if (same) return PT_OK;
  drop_graph(b);
  b->parts.clear();
  b->parts_width = 0;
  // BVHs at the batch width: the context's own, or rebuilt into scratch
  struct Src {
    const uint4* nodes;
    const float4* prims;
    const uint32_t* loid;
    size_t nn;
    int depth;
  };
  std::vector<Src> src(ctxs.size());
  std::vector<DevBuf<uint4>> tn(ctxs.size());
  std::vector<DevBuf<float4>> tp(ctxs.size());
  std::vector<DevBuf<uint32_t>> tl(ctxs.size());
  auto release_scratch = [&]() {
    for (size_t k = 0; k < ctxs.size(); k++) {
      tn[k].release();
      tp[k].release();
      tl[k].release();
    }
  };
  for (size_t k = 0; k < ctxs.size(); k++) {
    pt_context* c = ctxs[k];
    if (c->bvh_width == width || c->prims.empty()) {
      src[k] = {c->d_nodes.p, c->d_prims.p, c->d_leaf_of_id.p, c->bvh_nodes, c->bvh_depth};
      continue;
    }
    size_t nn = 0;
    int depth = 0;
    int rc = build_bvh(c, width, tn[k], tp[k], tl[k], &nn, &depth);
    if (rc) {
      release_scratch();
      return bfail(b, rc, std::string("batch BVH build: ") + c->err);
    }
    src[k] = {tn[k].p, tp[k].p, tl[k].p, nn, depth};
  }
  size_t N = 0, P = 0, X = 0, M = 0, A = 0;
  int max_depth = 1;
  for (size_t k = 0; k < ctxs.size(); k++) {
    pt_context* c = ctxs[k];
    N += c->prims.empty() ? 0 : src[k].nn;
    P += c->prims.size();
    X += c->xforms.size() / 24;
    M += c->mats.size();
    A += c->normals.size() / 3;
    max_depth = std::max(max_depth, src[k].depth);
  }
  if (N + 1 >= 0xffffffffull || P >= 0x7fffffffull || A >= 0xffffffffull)
    return bfail(b, PT_EINVAL, "batch geometry exceeds 32-bit indices");
  BK(b->nodes.ensure(5 * (N + 1)));
  BK(b->prims.ensure(3 * std::max<size_t>(P, 1)));
  BK(b->leaf_of_id.ensure(std::max<size_t>(P, 1)));
  BK(b->tri_attr.ensure(std::max<size_t>(P, 1)));
  BK(b->xforms.ensure(6 * X + 1));
  BK(b->mats.ensure(std::max<size_t>(M, 1)));
  BK(b->normals.ensure(3 * A + 3));
  BK(b->uvs.ensure(2 * A + 2));
  // the trailing empty node: root of scenes without primitives
  BK(cudaMemsetAsync(b->nodes.p + 5 * N, 0, 5 * sizeof(uint4), st));
  size_t no = 0, po = 0, xo = 0, mo = 0, ao = 0;
  for (size_t k = 0; k < ctxs.size(); k++) {
    pt_context* c = ctxs[k];
    size_t np = c->prims.size(), nx = c->xforms.size() / 24, nm = c->mats.size(),
           na = c->normals.size() / 3;
    size_t nn = np ? src[k].nn : 0;
    ScenePart part{c, c->commit_gen, np ? (uint32_t)no : (uint32_t)N};
    if (nn) BK(cudaMemcpyAsync(b->nodes.p + 5 * no, src[k].nodes, nn * 80, cudaMemcpyDeviceToDevice, st));
    if (np) {
      BK(cudaMemcpyAsync(b->prims.p + 3 * po, src[k].prims, np * 48, cudaMemcpyDeviceToDevice, st));
      BK(cudaMemcpyAsync(b->leaf_of_id.p + po, src[k].loid, np * 4, cudaMemcpyDeviceToDevice, st));
      BK(cudaMemcpyAsync(b->tri_attr.p + po, c->d_tri_attr.p, np * 16, cudaMemcpyDeviceToDevice, st));
    }
    if (nx) BK(cudaMemcpyAsync(b->xforms.p + 6 * xo, c->d_xforms.p, nx * 96, cudaMemcpyDeviceToDevice, st));
    if (nm) BK(cudaMemcpyAsync(b->mats.p + mo, c->d_mats.p, nm * sizeof(GpuMaterial), cudaMemcpyDeviceToDevice, st));
    if (na) {
      BK(cudaMemcpyAsync(b->normals.p + 3 * ao, c->d_normals.p, na * 12, cudaMemcpyDeviceToDevice, st));
      BK(cudaMemcpyAsync(b->uvs.p + 2 * ao, c->d_uvs.p, na * 8, cudaMemcpyDeviceToDevice, st));
    }
    pt::launch_relocate(b->nodes.p + 5 * no, nn, (uint32_t)no, (uint32_t)po, b->prims.p + 3 * po, np,
                        (uint32_t)xo, (uint32_t)po, (uint32_t)mo, b->leaf_of_id.p + po,
                        b->tri_attr.p + po, (uint32_t)ao, st);
    BK(cudaGetLastError());
    b->parts.push_back(part);
    no += nn;
    po += np;
    xo += nx;
    mo += nm;
    ao += na;
  }
  BK(cudaStreamSynchronize(st));
  release_scratch();
  DevScene& S = b->merged;
  memset(&S, 0, sizeof(S));
  S.nodes = b->nodes.p;
  S.prims = b->prims.p;
  S.xforms = b->xforms.p;
  S.mats = b->mats.p;
  S.tri_attr = b->tri_attr.p;
  S.normals = b->normals.p;
  S.uvs = b->uvs.p;
  S.leaf_of_id = b->leaf_of_id.p;
  S.num_prims = (int)P;
  S.root = 0;
  S.tri_only = 1;
  S.has_motion = 0;
  for (const pt_context* c : ctxs) {
    if (!pth::all_triangles(c)) S.tri_only = 0;
    if (pth::has_motion(c)) S.has_motion = 1;
  }
  b->max_stack = max_depth + 1;
  b->total_nodes = N;
  b->parts_width = width;
  return PT_OK;
}

static int ensure_wave(pt_batch* b, size_t results) {
  if (b->slots != b->tune.path_slots || !b->slot_f4.p) {
    drop_graph(b);
    size_t s = (size_t)b->tune.path_slots;
    b->slot_f4.release();
    b->slot_u4.release();
    BK(b->slot_f4.ensure(s * PT_SLOT_F4));
    BK(b->slot_u4.ensure(s * PT_SLOT_U4));
    BK(b->d_ctr.ensure(1));
    BK(b->d_ctl.ensure(1));
    carve_wave(b->W, b->slot_f4.p, b->slot_u4.p, s);
    b->W.ctr = b->d_ctr.p;
    b->slots = (int)s;
  }
  if (b->d_results.n < results || !b->d_results.p) {
    drop_graph(b);
    BK(b->d_results.ensure(results));
  }
  b->W.results = b->d_results.p;
  return PT_OK;
}

// Grows a table buffer; a new address invalidates the captured graph.
template <typename T>
static cudaError_t table_upload(pt_batch* b, DevBuf<T>& buf, const std::vector<T>& v) {
  if (buf.n < v.size() || !buf.p) drop_graph(b);
  return buf.upload(v.data(), v.size(), b->stream);
}

// ------------------------------------------------------------- graphs ------
// The device-loop graph: outer while over chunks, inner while over
// iterations (see the file comment).
static cudaError_t capture_loop_graph(pt_batch* b, const BatchRefs& br, bool counters, int mode,
                                      cudaGraphExec_t* out) {
  cudaStream_t st = b->stream;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  bool capturing = false;
  auto body = [&]() -> cudaError_t {
    cudaError_t r;
    cudaGraphConditionalHandle h_out = 0, h_in = 0;
    if ((r = cudaGraphConditionalHandleCreate(&h_out, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess)
      return r;
    if ((r = cudaGraphConditionalHandleCreate(&h_in, g, 0, 0)) != cudaSuccess) return r;
    cudaGraphNodeParams po = {};
    po.type = cudaGraphNodeTypeConditional;
    po.conditional.handle = h_out;
    po.conditional.type = cudaGraphCondTypeWhile;
    po.conditional.size = 1;
    cudaGraphNode_t n_out;
    if ((r = cudaGraphAddNode(&n_out, g, nullptr, nullptr, 0, &po)) != cudaSuccess) return r;
    cudaGraph_t body_out = po.conditional.phGraph_out[0];
    if ((r = cudaStreamBeginCaptureToGraph(st, body_out, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
      return r;
    capturing = true;
    pt::launch_batch_begin(b->W, b->d_ctl.p, b->d_chunks.p, true, h_in, st);
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaGraph_t cg = nullptr;
    if ((r = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, nullptr, &nd)) != cudaSuccess)
      return r;
    cudaGraphNodeParams pi = {};
    pi.type = cudaGraphNodeTypeConditional;
    pi.conditional.handle = h_in;
    pi.conditional.type = cudaGraphCondTypeWhile;
    pi.conditional.size = 1;
    cudaGraphNode_t n_in;
    if ((r = cudaGraphAddNode(&n_in, cg, deps, nullptr, nd, &pi)) != cudaSuccess) return r;
    cudaGraph_t body_in = pi.conditional.phGraph_out[0];
    if ((r = cudaStreamUpdateCaptureDependencies(st, &n_in, nullptr, 1,
                                                 cudaStreamSetCaptureDependencies)) != cudaSuccess)
      return r;
    pt::launch_batch_end(b->W, b->d_ctl.p, br, true, h_out, st);
    capturing = false;
    if ((r = cudaStreamEndCapture(st, &body_out)) != cudaSuccess) return r;
    if ((r = cudaStreamBeginCaptureToGraph(st, body_in, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
      return r;
    capturing = true;
    pt::launch_iteration(b->merged, b->W, b->d_ctl.p, b->max_stack, counters, b->lc, st, nullptr,
                         mode, &br, true, h_in);
    capturing = false;
    if ((r = cudaStreamEndCapture(st, &body_in)) != cudaSuccess) return r;
    if ((r = cudaGetLastError()) != cudaSuccess) return r;
    return cudaGraphInstantiate(out, g, 0);
  };
  e = body();
  if (capturing) {
    cudaGraph_t junk = nullptr;
    cudaStreamEndCapture(st, &junk);
  }
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
  }
  return e;
}

// The host-loop graph: kItersPerGraph iterations, events between stages
// when timing.
static cudaError_t capture_iter_graph(pt_batch* b, const BatchRefs& br, bool counters, bool timing,
                                      int mode, cudaGraphExec_t* out) {
  cudaStream_t st = b->stream;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  for (int i = 0; i < kItersPerGraph; i++)
    pt::launch_iteration(b->merged, b->W, b->d_ctl.p, b->max_stack, counters, b->lc, st,
                         timing ? &b->tev[6 * i] : nullptr, mode, &br, false, 0);
  e = cudaStreamEndCapture(st, &g);
  if (e != cudaSuccess) return e;
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  return e;
}

// ------------------------------------------------------------- render ------
static int check_items(pt_batch* b, const pt_batch_item* items, int n) {
  if (!items || n <= 0) return bfail(b, PT_EINVAL, "no batch items");
  if (n > PT_MAX_BATCH_SCENES) return bfail(b, PT_EINVAL, "more than 32767 batch items");
  for (int i = 0; i < n; i++) {
    const pt_batch_item& it = items[i];
    std::string at = "batch item " + std::to_string(i) + ": ";
    if (!it.scene) return bfail(b, PT_EINVAL, at + "null scene");
    if (it.scene->device != b->device) return bfail(b, PT_EINVAL, at + "scene on another device");
    int rc = check_params(it.scene, &it.params);
    if (rc) return bfail(b, rc, at + it.scene->err);
    if (!it.accum_rgba) return bfail(b, PT_EINVAL, at + "null accumulator");
    if (it.params.mode != items[0].params.mode)
      return bfail(b, PT_EINVAL, at + "all items of a batch use one integrator mode");
    if (it.params.guide) return bfail(b, PT_EINVAL, at + "batches render without the guide");
  }
  return PT_OK;
}

static int batch_render(pt_batch* b, const pt_batch_item* items, int n, float4* const* acc_override) {
  cudaStream_t st = b->stream;
  int rc = ensure_geometry(b, items, n);
  if (rc) return rc;
  // launch shape for this tune and BVH depth
  if (pt::trace_smem(b->max_stack, b->tune.trace_block) > 200 * 1024)
    return bfail(b, PT_EINVAL, "BVH too deep for the traversal stack at this trace block size");
  BK(pt::set_trace_smem());
  LaunchCfg lc;
  lc.trace_block = b->tune.trace_block;
  lc.shade_block = b->tune.shade_block;
  lc.trace_grid = pt::wave_grid(0, b->max_stack, lc.trace_block);
  lc.shade_grid = pt::wave_grid(1, b->max_stack, lc.shade_block);
  lc.sort = b->tune.shade_order == 1;
  if (b->tune.shade_order == 0)
    for (const ScenePart& p : b->parts) lc.sort = lc.sort || sort_pays(p.ctx);
  lc.tex = 0;
  lc.motion = 0;
  for (const ScenePart& p : b->parts) {
    lc.tex = lc.tex || uses_textures(p.ctx);
    lc.motion = lc.motion || has_motion(p.ctx);
  }
  lc.refetch = b->tune.refetch_lanes;
  if (lc.refetch == 0) {  // automatic: by the largest scene of the batch
    size_t most = 0;
    for (const ScenePart& p : b->parts) most = std::max(most, p.ctx->prims.size());
    lc.refetch = auto_refetch(most);
  }
  b->lc = lc;
  // accumulators: the items' device buffers, or device copies of host ones
  std::vector<float4*> acc(n);
  std::vector<size_t> stage_off(n, (size_t)-1);
  size_t stage = 0, max_wh = 1;
  for (int i = 0; i < n; i++) {
    size_t wh = (size_t)items[i].params.width * items[i].params.height;
    max_wh = std::max(max_wh, wh);
    if (acc_override) {
      acc[i] = acc_override[i];
    } else if (int kind = device_ptr_kind(items[i].accum_rgba, b->device)) {
      if (kind < 0)
        return bfail(b, PT_EINVAL, "batch item " + std::to_string(i) +
                                       ": accumulator is device memory of another GPU");
      acc[i] = (float4*)items[i].accum_rgba;
    } else {
      stage_off[i] = stage;
      stage += wh;
    }
  }
  if (stage) {
    BK(b->d_stage.ensure(stage));
    for (int i = 0; i < n; i++)
      if (stage_off[i] != (size_t)-1) acc[i] = b->d_stage.p + stage_off[i];
  }
  // scene table
  std::vector<BatchScene> scenes(n);
  std::vector<uint32_t> roots(n);
  std::unordered_map<pt_context*, uint32_t> root_of;
  for (const ScenePart& p : b->parts) root_of[p.ctx] = p.root;
  for (int i = 0; i < n; i++) {
    const pt_render_params& p = items[i].params;
    BatchScene& B = scenes[i];
    memset(&B, 0, sizeof(B));
    B.S = items[i].scene->scene;  // camera, miss, lights, environment
    B.S.nodes = b->merged.nodes;
    B.S.prims = b->merged.prims;
    B.S.xforms = b->merged.xforms;
    B.S.mats = b->merged.mats;
    B.S.tri_attr = b->merged.tri_attr;
    B.S.normals = b->merged.normals;
    B.S.uvs = b->merged.uvs;
    B.S.leaf_of_id = b->merged.leaf_of_id;
    B.S.root = root_of[items[i].scene];
    B.width = p.width;
    B.height = p.height;
    B.max_depth = p.max_depth;
    B.rr_enable = p.rr_enable;
    B.rr_depth = p.rr_depth;
    fastdiv_magic((uint32_t)(p.width * p.height), &B.wh_m, &B.wh_l);
    fastdiv_magic((uint32_t)p.width, &B.w_m, &B.w_l);
    roots[i] = B.S.root;
  }
  // chunks of whole frames, in item order
  const size_t cap =
      std::max(b->tune.chunk_paths > 0 ? (size_t)b->tune.chunk_paths : kResultsCap, max_wh);
  const size_t slots = (size_t)b->tune.path_slots;
  std::vector<BatchSeg> segs;
  std::vector<BatchChunk> chunks;
  size_t max_chunk = 0;
  BatchChunk cur{};
  int cur_depth = 1;
  auto close = [&]() {
    if (!cur.paths) return;
    cur.seg_end = (uint32_t)segs.size();
    cur.max_iter = ((cur.paths + slots - 1) / slots + 2) * (unsigned long long)(cur_depth + 1) + 16;
    max_chunk = std::max<size_t>(max_chunk, cur.paths);
    chunks.push_back(cur);
    cur = BatchChunk{};
    cur.seg_begin = (uint32_t)segs.size();
    cur_depth = 1;
  };
  unsigned long long total_paths = 0;
  for (int i = 0; i < n; i++) {
    const pt_render_params& p = items[i].params;
    size_t wh = (size_t)p.width * p.height;
    int f = 0;
    while (f < p.spp) {
      size_t room = (cap - cur.paths) / wh;
      if (room == 0) {
        close();
        continue;
      }
      int take = (int)std::min<size_t>((size_t)(p.spp - f), room);
      BatchSeg sg;
      memset(&sg, 0, sizeof(sg));
      sg.path_off = (uint32_t)cur.paths;
      sg.pix_off = cur.pixels;
      sg.scene = (uint32_t)i;
      sg.frame0 = (uint32_t)(p.frame0 + f);
      sg.frames = (uint32_t)take;
      sg.acc = acc[i];
      segs.push_back(sg);
      cur.paths += (unsigned long long)take * wh;
      cur.pixels += (uint32_t)wh;
      cur_depth = std::max(cur_depth, p.max_depth);
      f += take;
    }
    total_paths += (unsigned long long)p.spp * wh;
  }
  close();
  rc = ensure_wave(b, max_chunk);
  if (rc) return rc;
  BK(table_upload(b, b->d_scenes, scenes));
  BK(table_upload(b, b->d_roots, roots));
  BK(table_upload(b, b->d_segs, segs));
  BK(table_upload(b, b->d_chunks, chunks));
  // accumulators start at zero (frame0 == 0) or from the caller's values
  for (int i = 0; i < n; i++) {
    size_t bytes = (size_t)items[i].params.width * items[i].params.height * sizeof(float4);
    if (items[i].params.frame0 == 0 || acc_override)
      BK(cudaMemsetAsync(acc[i], 0, bytes, st));
    else if (stage_off[i] != (size_t)-1)
      BK(cudaMemcpyAsync(acc[i], items[i].accum_rgba, bytes, cudaMemcpyHostToDevice, st));
  }
  const bool counters = b->opt.enable_counters != 0;
  const bool timing = b->opt.enable_timing != 0;
  const int mode = items[0].params.mode;
  WaveCounters& c = *b->h_ctr;
  memset(&c, 0, sizeof(c));
  c.n_chunks = (uint32_t)chunks.size();
  BK(cudaMemcpyAsync(b->d_ctr.p, &c, sizeof(c), cudaMemcpyHostToDevice, st));
  // batch-wide controls; k_batch_begin fills in the chunk fields
  WaveCtl hc;
  memset(&hc, 0, sizeof(hc));
  hc.mode = mode;
  BK(cudaMemcpyAsync(b->d_ctl.p, &hc, sizeof(hc), cudaMemcpyHostToDevice, st));
  BatchRefs br{b->d_scenes.p, b->d_segs.p, b->d_roots.p};
  if (timing && b->tev.empty()) {
    b->tev.resize(6 * kItersPerGraph);
    for (auto& e : b->tev) BK(cudaEventCreate(&e));
  }
  GraphSig sig;
  memset(&sig, 0, sizeof(sig));
  sig.merged = b->merged;
  sig.W = b->W;
  sig.br = br;
  sig.chunks = b->d_chunks.p;
  sig.ctl = b->d_ctl.p;
  sig.lc = b->lc;
  sig.max_stack = b->max_stack;
  sig.mode = mode;
  sig.counters = counters;
  sig.timing = timing;
  sig.device_loop = (!timing && b->cond_ok) ? 1 : 0;
  if (b->exec && memcmp(&sig, &b->sig, sizeof(sig)) != 0) drop_graph(b);
  if (!b->exec && sig.device_loop) {
    if (capture_loop_graph(b, br, counters, mode, &b->exec) != cudaSuccess) {
      b->cond_ok = false;  // the host loop below does the same work
      sig.device_loop = 0;
    }
  }
  if (!b->exec && !sig.device_loop) BK(capture_iter_graph(b, br, counters, timing, mode, &b->exec));
  b->sig = sig;
  pt_stats& s = b->stats;
  s.paths = s.ext_rays = s.shadow_rays = s.node_fetches = s.prim_tests = 0;
  s.iterations = s.kernel_launches = s.graph_launches = 0;
  for (double& x : s.stage_ms) x = 0.0;
  BK(cudaEventRecord(b->ev0, st));
  if (sig.device_loop) {
    BK(cudaGraphLaunch(b->exec, st));
    s.graph_launches = 1;
  } else {
    for (size_t k = 0; k < chunks.size(); k++) {
      pt::launch_batch_begin(b->W, b->d_ctl.p, b->d_chunks.p, false, 0, st);
      s.kernel_launches += 1;
      unsigned long long bound = chunks[k].max_iter + kItersPerGraph, iters = 0;
      while (true) {
        BK(cudaGraphLaunch(b->exec, st));
        s.graph_launches++;
        iters += kItersPerGraph;
        BK(cudaMemcpyAsync(b->h_ctr, b->d_ctr.p, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st));
        BK(cudaStreamSynchronize(st));
        if (timing) {
          for (int i = 0; i < kItersPerGraph; i++)
            for (int q = 0; q < 5; q++) {
              float ms = 0.f;
              if (cudaEventElapsedTime(&ms, b->tev[6 * i + q], b->tev[6 * i + q + 1]) == cudaSuccess)
                s.stage_ms[q] += ms;
              else
                cudaGetLastError();
            }
        }
        if (c.error) break;
        if (c.next_path >= chunks[k].paths && c.n_cur == 0) break;
        if (iters > bound) return bfail(b, PT_ETIMEOUT, "batch wavefront did not drain");
      }
      if (c.error) break;
      pt::launch_batch_end(b->W, b->d_ctl.p, br, false, 0, st);
      s.kernel_launches += 2;
    }
  }
  BK(cudaGetLastError());
  BK(cudaEventRecord(b->ev1, st));
  BK(cudaMemcpyAsync(b->h_ctr, b->d_ctr.p, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st));
  if (!acc_override)
    for (int i = 0; i < n; i++)
      if (stage_off[i] != (size_t)-1)
        BK(cudaMemcpyAsync(items[i].accum_rgba, acc[i],
                           (size_t)items[i].params.width * items[i].params.height * sizeof(float4),
                           cudaMemcpyDeviceToHost, st));
  BK(cudaStreamSynchronize(st));
  if (c.error & 1u) return bfail(b, PT_EQUEUE, "traversal stack overflow");
  if (c.error & 2u) return bfail(b, PT_ETIMEOUT, "batch wavefront did not drain within its bound");
  if (c.chunk != c.n_chunks) return bfail(b, PT_ETIMEOUT, "batch ended before its last chunk");
  float ms = 0.f;
  BK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  s.render_ms = ms;
  s.paths = total_paths;
  s.ext_rays = c.ext_rays;
  s.shadow_rays = c.shadow_rays;
  s.node_fetches = c.node_fetches;
  s.prim_tests = c.prim_tests;
  s.iterations = c.iters_total;
  if (sig.device_loop) s.kernel_launches = 7 * c.iters_total + 3 * chunks.size();
  else s.kernel_launches += 7 * c.iters_total;
  s.bvh_nodes = b->total_nodes;
  s.bvh_bytes = b->total_nodes * 80 + (size_t)b->merged.num_prims * 48;
  s.bvh_depth = b->max_stack - 1;
  return PT_OK;
}

// ============================================================== ABI ========
extern "C" {

PT_API int pt_batch_create(const pt_options* opt, pt_batch** out) {
  if (!out) return PT_EINVAL;
  *out = nullptr;
  pt_batch* b = new (std::nothrow) pt_batch();
  if (!b) return PT_ENOMEM;
  if (opt) b->opt = *opt;
  b->device = opt ? opt->device : 0;
  b->tune.path_slots = (opt && opt->path_slots > 0) ? opt->path_slots : (1 << 21);
  b->tune.trace_block = PT_TRACE_BLOCK;
  b->tune.shade_block = PT_SHADE_BLOCK;
  b->tune.bvh_width = (opt && opt->bvh_width) ? opt->bvh_width : 8;
  b->tune.shade_order = opt ? opt->shade_order : 0;
  b->tune.refetch_lanes = opt ? opt->refetch_lanes : 0;
  if (!tune_valid(b->tune)) {
    delete b;
    return PT_EINVAL;
  }
  cudaError_t e = cudaSetDevice(b->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_ctr, sizeof(WaveCounters));
  if (e != cudaSuccess) {
    int rc = (e == cudaErrorMemoryAllocation) ? PT_ENOMEM : PT_ECUDA;
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return rc;
  }
  *out = b;
  return PT_OK;
}

PT_API int pt_batch_destroy(pt_batch* b) {
  if (!b) return PT_EINVAL;
  cudaSetDevice(b->device);
  drop_graph(b);
  for (cudaEvent_t e : b->tev) cudaEventDestroy(e);
  b->nodes.release();
  b->tri_attr.release();
  b->prims.release();
  b->xforms.release();
  b->mats.release();
  b->normals.release();
  b->uvs.release();
  b->leaf_of_id.release();
  b->d_scenes.release();
  b->d_segs.release();
  b->d_chunks.release();
  b->d_roots.release();
  b->d_stage.release();
  b->d_tune_acc.release();
  b->slot_f4.release();
  b->slot_u4.release();
  b->d_ctr.release();
  b->d_ctl.release();
  b->d_results.release();
  if (b->h_ctr) cudaFreeHost(b->h_ctr);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return PT_OK;
}

PT_API const char* pt_batch_last_error(pt_batch* b) { return b ? b->err.c_str() : "null batch"; }

PT_API int pt_batch_render(pt_batch* b, const pt_batch_item* items, int n, void* stream) {
  if (!b) return PT_EINVAL;
  int rc = check_items(b, items, n);
  if (rc) return rc;
  BK(cudaSetDevice(b->device));
  BK(cudaEventRecord(b->ev0, (cudaStream_t)stream));
  BK(cudaStreamWaitEvent(b->stream, b->ev0, 0));
  rc = batch_render(b, items, n, nullptr);
  if (rc == PT_OK) {
    BK(cudaEventRecord(b->ev1, b->stream));
    BK(cudaStreamWaitEvent((cudaStream_t)stream, b->ev1, 0));
  }
  return rc;
}

PT_API int pt_batch_set_tune(pt_batch* b, const pt_tune* t) {
  if (!b || !t) return PT_EINVAL;
  if (!tune_valid(*t)) return bfail(b, PT_EINVAL, "invalid tune");
  b->tune = *t;
  return PT_OK;
}

PT_API int pt_batch_get_tune(pt_batch* b, pt_tune* t) {
  if (!b || !t) return PT_EINVAL;
  *t = b->tune;
  return PT_OK;
}

PT_API int pt_batch_get_stats(pt_batch* b, pt_stats* out) {
  if (!b || !out) return PT_EINVAL;
  *out = b->stats;
  return PT_OK;
}

PT_API int pt_batch_autotune(pt_batch* b, const pt_batch_item* items, int n, pt_tune* best_out) {
  if (!b) return PT_EINVAL;
  int rc = check_items(b, items, n);
  if (rc) return rc;
  BK(cudaSetDevice(b->device));
  // the sample: every item at low spp (about 2^25 paths in all), into
  // scratch accumulators
  size_t per_frame = 0;
  for (int i = 0; i < n; i++) per_frame += (size_t)items[i].params.width * items[i].params.height;
  int s = (int)std::max<size_t>(1, ((size_t)1 << 25) / std::max<size_t>(per_frame, 1));
  std::vector<pt_batch_item> sample(items, items + n);
  std::vector<float4*> acc(n);
  BK(b->d_tune_acc.ensure(per_frame));
  size_t off = 0;
  for (int i = 0; i < n; i++) {
    sample[i].params.spp = std::min(items[i].params.spp, s);
    sample[i].params.frame0 = 0;
    acc[i] = b->d_tune_acc.p + off;
    off += (size_t)items[i].params.width * items[i].params.height;
  }
  auto measure = [&](const pt_tune& t, double* pps) -> int {
    b->tune = t;
    double best_ms = 1e300;
    for (int rep = 0; rep < 3; rep++) {  // the first run captures the graph
      int r = batch_render(b, sample.data(), n, acc.data());
      if (r) return r;
      if (rep > 0) best_ms = std::min(best_ms, b->stats.render_ms);
    }
    *pps = (double)b->stats.paths / (best_ms * 1e-3);
    return PT_OK;
  };
  pt_tune best = b->tune;
  double best_pps = 0.0;
  rc = measure(best, &best_pps);
  if (rc) return rc;
  auto consider = [&](pt_tune t) -> int {
    if (!tune_valid(t) || memcmp(&t, &best, sizeof(t)) == 0) return PT_OK;
    double pps = 0.0;
    int r = measure(t, &pps);
    if (r == PT_EINVAL) return PT_OK;  // e.g. stack too deep for this block size
    if (r) return r;
    if (pps > best_pps * 1.02) {
      best = t;
      best_pps = pps;
    }
    return PT_OK;
  };
  const int slot_opts[] = {1 << 19, 1 << 20, 1 << 21, 1 << 22, 1 << 23};
  const int tb_opts[] = {64, 128, 256};
  const int sb_opts[] = {128, 256};
  const int w_opts[] = {8, 4};
  const int order_opts[] = {1, 2};
  const int refetch_opts[] = {24, 32};
  for (int v : slot_opts) {
    pt_tune t = best;
    t.path_slots = v;
    if ((rc = consider(t))) return rc;
  }
  for (int v : tb_opts) {
    pt_tune t = best;
    t.trace_block = v;
    if ((rc = consider(t))) return rc;
  }
  for (int v : sb_opts) {
    pt_tune t = best;
    t.shade_block = v;
    if ((rc = consider(t))) return rc;
  }
  for (int v : w_opts) {
    pt_tune t = best;
    t.bvh_width = v;
    if ((rc = consider(t))) return rc;
  }
  for (int v : order_opts) {
    pt_tune t = best;
    t.shade_order = v;
    if ((rc = consider(t))) return rc;
  }
  for (int v : refetch_opts) {
    pt_tune t = best;
    t.refetch_lanes = v;
    if ((rc = consider(t))) return rc;
  }
  best.sample_paths_per_s = best_pps;
  b->tune = best;
  if (best_out) *best_out = best;
  return PT_OK;
}

}  // extern "C"
