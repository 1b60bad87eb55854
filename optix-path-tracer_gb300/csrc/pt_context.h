/*
 * pt_context.h - host-side state of a scene context, shared by the single
 * scene API (pt_api.cu) and batched rendering (pt_batch.cu).
 */
#ifndef PT_CONTEXT_H
#define PT_CONTEXT_H

#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "../../include/pt.h"
#include "bvh_build.h"
#include "pt_guide.cuh"
#include "pt_internal.h"

namespace pth {

struct HostPrim {
  int type, axis, flip, xform;
  uint32_t material;
  float f[9];
  int moving;  // a moving sphere (type sphere, f as in pt_types.h)
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc((void**)&p, (count ? count : 1) * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  cudaError_t upload(const T* h, size_t count, cudaStream_t st) {
    cudaError_t e = ensure(count);
    if (e != cudaSuccess || count == 0) return e;
    return cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, st);
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// Page-locked host memory that grows on demand (staging of large uploads and
// read-backs at commit, which then run at full copy-engine speed).
template <typename T>
struct PinnedBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMallocHost((void**)&p, (count ? count : 1) * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace pth

using pth::DevBuf;
using pth::PinnedBuf;
using pth::HostPrim;

/* State of the learned sampling guide of a context. */
struct GuideState {
  bool ready = false;        // weights initialised
  bool bounds = false;       // scene box known
  DevBuf<float> w32, m, v;   // FP32 master weights, Adam moments (PTG_PARAMS each)
  DevBuf<uint16_t> wbf;      // BF16 copy read by the MMAs
  DevBuf<float> partial;     // per-CTA gradients
  DevBuf<float> grad;        // summed gradient (tests)
  DevBuf<float> scalars;     // [0] loss, [1] sum of sample weights
  DevBuf<uint32_t> counters; // [0] samples in the training array, [1] failure flag
  DevBuf<GuideSample> samples;
  DevBuf<float> eval_out;
  DevBuf<GuidePacked> out;   // per path slot: decoded guide
  DevBuf<uint32_t> rows;     // per path slot: positions selected for inference
  DevBuf<float4> feat;       // per path slot: their hit records (3 float4)
  DevBuf<GuideSample> rec;   // training records of the current frame
  DevBuf<uint32_t> coll_u;   // record collection scratch: per-block counts and offsets
  DevBuf<float> coll_f;      //   and per-block weight sums
  uint32_t rec_stride = 1, rec_n = 0;
  float lr = 1e-2f;          // Adam learning rate of the online training
  int steps = 12;            // Adam steps per frame on the frame's samples
  float exponent = 1.f;      // training weight = (F/q)^exponent (1: the KL target)
  int max_bounces = 4;       // guided bounces per path (0: all)
  uint32_t wait_limit = 1u << 24;  // try_waits per tensor-core completion wait
  float bmin[3] = {0, 0, 0}, binv[3] = {1, 1, 1};
  int step = 0;
  int grid = 0;
};

struct pt_context {
  int device = 0;
  std::string err;
  pt_options opt{};
  cudaStream_t stream = nullptr;
  cudaStream_t aux_stream = nullptr;  // scene table uploads during the BVH build
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // ---- host scene
  std::vector<GpuMaterial> mats;
  std::vector<HostPrim> prims;
  size_t num_non_triangles = 0;  // primitives that are not triangles
  size_t num_moving = 0;         // moving spheres
  std::vector<float> xforms;  // 24 floats each: m rows, inv rows (float4-padded 3x4)
  std::vector<uint4> tri_attr;
  std::vector<float> normals, uvs;
  std::vector<GpuLight> lights;
  std::vector<GpuTexture> textures;
  std::vector<float4> tex_data;   // image texels and noise tables
  std::vector<int> tex_list;      // vector-texture entries
  GpuMiss miss{};
  std::vector<float4> env;
  GpuCamera cam{};
  bool committed = false;
  // ---- device scene
  DevBuf<uint4> d_nodes;
  DevBuf<float4> d_prims, d_xforms, d_env;
  DevBuf<GpuMaterial> d_mats;
  DevBuf<GpuLight> d_lights;
  DevBuf<GpuTexture> d_textures;
  DevBuf<float4> d_tex_data;
  DevBuf<int> d_tex_list;
  DevBuf<uint4> d_tri_attr;
  DevBuf<float> d_normals, d_uvs;
  DevBuf<uint32_t> d_leaf_of_id;
  DevBuf<float4> d_rec_in;  // primitive records in call order (GPU builder input)
  PinnedBuf<float4> h_rec;  // their host staging
  pt::BuildArena build_arena;  // GPU builder scratch, reused by every commit
  DevBuf<float> d_env_marg, d_env_cond;  // environment sampling CDFs
  DevBuf<double> d_env_rows;
  DevBuf<double> d_env_pre;   // per texel: weights, then row prefix sums
  DevBuf<int> d_env_valid;
  int env_valid = 0;
  DevScene scene{};
  int bvh_depth = 0;
  size_t bvh_nodes = 0;
  int bvh_width = 8;          // node width the committed BVH was built with
  uint64_t commit_gen = 0;    // increases with every pt_commit
  // ---- wavefront state
  int slots = 0;
  WaveState W{};
  DevBuf<float4> d_slot_f4;   // PT_SLOT_F4 float4 arrays of `slots` entries
  DevBuf<uint4> d_slot_u4;    // PT_SLOT_U4 uint4 arrays
  DevBuf<WaveCounters> d_ctr;
  DevBuf<WaveCtl> d_ctl;
  DevBuf<float4> d_results;
  DevBuf<float4> d_acc;
  DevBuf<double> d_acc64;     // staging for host double accumulators
  DevBuf<float> d_tmp;
  DevBuf<uint32_t> d_tmpu;
  WaveCounters* h_ctr = nullptr;  // pinned, 2 (the counters after each of two graph launches)
  WaveCtl* h_ctl = nullptr;       // pinned
  cudaGraphExec_t graph = nullptr;
  cudaGraphExec_t graph2 = nullptr;  // a second instance on its own timing events (timing)
  cudaEvent_t evc[2] = {nullptr, nullptr};  // the counters of a graph launch have arrived
  bool graph_counters = false;
  bool graph_timing = false;
  int graph_mode = 0;
  WaveState graph_W{};       // the buffers the captured graph refers to
  bool graph_guide = false;
  std::vector<cudaEvent_t> tev;  // 6 per iteration of the graph (timing)
  int max_stack = 0;
  LaunchCfg lc{};
  GuideState guide;
  pt_stats stats{};
};


namespace pth {
/* Builds the scene's BVH (at most `width` children per node) into the given
 * buffers; returns a PT_ status.  *uploaded (if given) receives the bytes
 * copied host to device. */
int build_bvh(pt_context* ctx, int width, DevBuf<uint4>& d_nodes, DevBuf<float4>& d_prims,
              DevBuf<uint32_t>& d_leaf_of_id, size_t* out_nodes, int* out_depth,
              size_t* uploaded = nullptr);
/* Carves the wavefront arrays of `slots` paths out of one float4 block
 * (PT_SLOT_F4 per slot) and one uint4 block (PT_SLOT_U4 per slot). */
void carve_wave(WaveState& W, float4* f, uint4* u, size_t slots);
/* 1: device memory of `device` (or managed memory), usable by its kernels;
 * 0: host memory (pageable or pinned); -1: device memory of another GPU. */
int device_ptr_kind(const void* p, int device);
/* Whether some material of the scene takes a texture. */
bool uses_textures(const pt_context* ctx);
/* Whether every primitive of the scene is a triangle. */
bool all_triangles(const pt_context* ctx);
/* Whether some sphere of the scene moves. */
bool has_motion(const pt_context* ctx);
/* Whether shading in material-sorted tiles pays for this scene: it does when
 * one of the costly BRDFs (Oren-Nayar, Torrance-Sparrow, Ashikhmin-Shirley)
 * is present, whose code paths diverge most in a mixed warp. */
bool sort_pays(const pt_context* ctx);
int auto_refetch(size_t num_prims);
/* Padded world box of one primitive (the BVH builders' leaf box). */
pt::Box prim_bounds(const pt_context* ctx, const HostPrim& p);
/* Allocates the guide's buffers and finds the scene box of its position
 * encoding; returns a PT_ status. */
int guide_prepare(pt_context* ctx);
/* Online training around a guided frame (enqueued on the context's stream):
 * clear the record buffer for a frame of w x h paths (and size it), then
 * collect the frame's records and take one Adam step. */
int guide_frame_begin(pt_context* ctx, int w, int h);
int guide_frame_train(pt_context* ctx);
/* Inference arguments for the current buffers. */
GuideInferArgs guide_infer_args(pt_context* ctx);
/* Render parameters valid for the context (sets ctx->err otherwise). */
int check_params(pt_context* ctx, const pt_render_params* p);
}  // namespace pth

#endif
