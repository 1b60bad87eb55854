/*
 * pt_api.cu - implementation of the C ABI declared in include/pt.h.
 *
 * Host side of the drop-in boundary: it takes over what the reference's
 * host_includes/ hand to OptiX (materials.hpp, hitables.hpp, mesh.hpp,
 * pdfs.hpp, programs.hpp, camera.hpp, transforms.hpp), keeps a flat scene,
 * builds the BVH8 at pt_commit and drives the wavefront kernels in
 * pt_render (the per-sample Context::launch of main.cpp:26-39,264).
 */
#include <atomic>
#include <random>
#include <cuda_runtime.h>
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pt.h"
#include "bvh_build.h"
#include "pt_context.h"
#include "pt_internal.h"
#include "ptmath.h"

namespace pt {
cudaError_t build_bvh8_gpu(const float4* d_rec, const float4* d_xforms, uint32_t n,
                           uint4* d_nodes, float4* d_rec_out, uint32_t* d_leaf_of_id,
                           uint32_t* out_nodes, int* out_depth, int treelet_rounds, int width,
                           float cam_t0, float cam_t1, BuildArena* arena, cudaStream_t st);
}

namespace {
const float PI_F = 3.141592654f;
}  // namespace

#ifndef PT_TREELET_ROUNDS
#define PT_TREELET_ROUNDS 2  /* SAH treelet restructuring passes of the GPU builder */
#endif

using namespace pth;

static int fail(pt_context* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

static const char* const kOtherDevice =
    "buffer is device memory of another GPU than the context's (pt_options.device)";

static int cuda_fail(pt_context* ctx, cudaError_t e, const char* where) {
  return fail(ctx, PT_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                          \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

// ----------------------------------------------------------------- helpers --
static void affine_inverse(const float* m, float* out) {
  // same expression as the oracle: adjugate in double, rounded once
  double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9],
         i = m[10];
  double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  double det = a * A + b * B + c * C;
  double inv_det = 1.0 / det;
  double r[9] = {A * inv_det, -(b * i - c * h) * inv_det, (b * f - c * e) * inv_det,
                 B * inv_det, (a * i - c * g) * inv_det, -(a * f - c * d) * inv_det,
                 C * inv_det, -(a * h - b * g) * inv_det, (a * e - b * d) * inv_det};
  double tx = m[3], ty = m[7], tz = m[11];
  for (int row = 0; row < 3; row++) {
    out[row * 4 + 0] = (float)r[row * 3 + 0];
    out[row * 4 + 1] = (float)r[row * 3 + 1];
    out[row * 4 + 2] = (float)r[row * 3 + 2];
    out[row * 4 + 3] = (float)(-(r[row * 3 + 0] * tx + r[row * 3 + 1] * ty + r[row * 3 + 2] * tz));
  }
}

static bool affine_ok(const float* m) {
  double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9],
         i = m[10];
  double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
  for (int k = 0; k < 12; k++)
    if (!std::isfinite(m[k])) return false;
  return std::isfinite(det) && std::fabs(det) > 1e-30;
}

static int add_xform(pt_context* ctx, const float* x) {
  if (!x) return -1;
  float inv[12];
  affine_inverse(x, inv);
  for (int k = 0; k < 12; k++) ctx->xforms.push_back(x[k]);
  for (int k = 0; k < 12; k++) ctx->xforms.push_back(inv[k]);
  return (int)(ctx->xforms.size() / 24) - 1;
}

static inline void xpoint_h(const float* m, const float* p, float* o) {
  o[0] = m[0] * p[0] + m[1] * p[1] + m[2] * p[2] + m[3];
  o[1] = m[4] * p[0] + m[5] * p[1] + m[6] * p[2] + m[7];
  o[2] = m[8] * p[0] + m[9] * p[1] + m[10] * p[2] + m[11];
}

static bool finite3(const float* v) {
  return v && std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

bool pth::uses_textures(const pt_context* ctx) {
  for (const GpuMaterial& m : ctx->mats)
    if (m.tex0 >= 0 || m.tex1 >= 0) return true;
  return false;
}

int pth::device_ptr_kind(const void* p, int device) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (a.type == cudaMemoryTypeManaged) return 1;
  if (a.type == cudaMemoryTypeDevice) return a.device == device ? 1 : -1;
  return 0;
}

// Forgets the captured wavefront graphs (a new scene, buffers or options).
static void drop_graphs(pt_context* ctx) {
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  if (ctx->graph2) cudaGraphExecDestroy(ctx->graph2);
  ctx->graph = ctx->graph2 = nullptr;
}

// Uploads a host table, or `zeros` zeroed elements when it is empty (the
// scene's device pointers are never null).
// Adds the bytes copied to *bytes.
template <typename T>
static cudaError_t upload_or_zero(DevBuf<T>& d, const std::vector<T>& v, size_t zeros,
                                  cudaStream_t st, size_t* bytes) {
  *bytes += (v.empty() ? zeros : v.size()) * sizeof(T);
  if (!v.empty()) return d.upload(v.data(), v.size(), st);
  const std::vector<T> z(zeros);
  cudaError_t e = d.upload(z.data(), z.size(), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // z is a local
  return e;
}

// World-space AABB of a primitive, padded so that rounding in the primitive
// tests can never place a reported hit outside its box.
static pt::Box prim_box(const pt_context* ctx, const HostPrim& p) {
  float lo[3], hi[3];
  const float* f = p.f;
  if (p.type == PT_PRIM_TRIANGLE) {
    for (int a = 0; a < 3; a++) {
      lo[a] = fminf(fminf(f[a], f[3 + a]), f[6 + a]);
      hi[a] = fmaxf(fmaxf(f[a], f[3 + a]), f[6 + a]);
    }
  } else if (p.type == PT_PRIM_SPHERE && p.moving) {
    pt::moving_sphere_box(f, ctx->cam.time0, ctx->cam.time1, lo, hi);
  } else if (p.type == PT_PRIM_SPHERE) {
    for (int a = 0; a < 3; a++) {
      lo[a] = f[a] - f[3];
      hi[a] = f[a] + f[3];
    }
  } else if (p.type == PT_PRIM_RECT) {
    int ka = p.axis, ia = (p.axis == 0) ? 1 : 0, ib = (p.axis == 2) ? 1 : 2;
    lo[ka] = hi[ka] = f[4];
    lo[ia] = f[0];
    hi[ia] = f[1];
    lo[ib] = f[2];
    hi[ib] = f[3];
  } else {
    for (int a = 0; a < 3; a++) {
      lo[a] = f[a];
      hi[a] = f[3 + a];
    }
  }
  if (p.xform >= 0) {
    const float* M = &ctx->xforms[(size_t)p.xform * 24];
    float nlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, nhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int c = 0; c < 8; c++) {
      float q[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]};
      float w[3];
      xpoint_h(M, q, w);
      for (int a = 0; a < 3; a++) {
        nlo[a] = fminf(nlo[a], w[a]);
        nhi[a] = fmaxf(nhi[a], w[a]);
      }
    }
    for (int a = 0; a < 3; a++) {
      lo[a] = nlo[a];
      hi[a] = nhi[a];
    }
  }
  pt::Box b;
  for (int a = 0; a < 3; a++) {
    float mag = fmaxf(1.0f, fmaxf(fabsf(lo[a]), fabsf(hi[a])));
    float pad = mag * 9.5367431640625e-07f;  // 2^-20 relative
    if (p.xform >= 0) pad *= 16.f;
    b.lo[a] = lo[a] - pad;
    b.hi[a] = hi[a] + pad;
  }
  return b;
}

pt::Box pth::prim_bounds(const pt_context* ctx, const HostPrim& p) { return prim_box(ctx, p); }

// ====================================================================== ABI ==
extern "C" {

PT_API const char* pt_version(void) { return "gb300-pathtracer 0.1 (sm_103a)"; }

PT_API const char* pt_last_error(pt_context* ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

PT_API int pt_context_create(const pt_options* opt, pt_context** out) {
  if (!out) return PT_EINVAL;
  *out = nullptr;
  if (opt && ((opt->bvh_width != 0 && (opt->bvh_width < 2 || opt->bvh_width > 8)) ||
              opt->shade_order < 0 || opt->shade_order > 2 || opt->refetch_lanes < 0 ||
              opt->refetch_lanes > 32))
    return PT_EINVAL;
  pt_context* ctx = new (std::nothrow) pt_context();
  if (!ctx) return PT_ENOMEM;
  if (opt) ctx->opt = *opt;
  ctx->device = opt ? opt->device : 0;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&ctx->h_ctr, 2 * sizeof(WaveCounters));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->evc[0], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->evc[1], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&ctx->h_ctl, sizeof(WaveCtl));
  if (e != cudaSuccess) {
    int rc = (e == cudaErrorMemoryAllocation) ? PT_ENOMEM : PT_ECUDA;
    delete ctx;
    return rc;
  }
  ctx->miss.type = PT_MISS_CONSTANT;
  *out = ctx;
  return PT_OK;
}

PT_API int pt_context_destroy(pt_context* ctx) {
  if (!ctx) return PT_EINVAL;
  cudaSetDevice(ctx->device);
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  if (ctx->graph2) cudaGraphExecDestroy(ctx->graph2);
  for (cudaEvent_t e : ctx->evc)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->tev) cudaEventDestroy(e);
  ctx->d_nodes.release();
  ctx->d_prims.release();
  ctx->d_xforms.release();
  ctx->d_env.release();
  ctx->d_mats.release();
  ctx->d_lights.release();
  ctx->d_tri_attr.release();
  ctx->d_normals.release();
  ctx->d_uvs.release();
  ctx->d_leaf_of_id.release();
  ctx->d_rec_in.release();
  ctx->h_rec.release();
  if (ctx->build_arena.p) cudaFree(ctx->build_arena.p);
  ctx->build_arena = pt::BuildArena{};
  ctx->d_env_marg.release();
  ctx->d_env_cond.release();
  ctx->d_env_rows.release();
  ctx->d_env_pre.release();
  ctx->d_env_valid.release();
  ctx->d_slot_f4.release();
  ctx->d_slot_u4.release();
  ctx->d_ctr.release();
  ctx->d_ctl.release();
  ctx->d_results.release();
  ctx->d_acc.release();
  ctx->d_acc64.release();
  {
    GuideState& G = ctx->guide;
    G.w32.release();
    G.m.release();
    G.v.release();
    G.wbf.release();
    G.partial.release();
    G.grad.release();
    G.scalars.release();
    G.counters.release();
    G.samples.release();
    G.eval_out.release();
    G.out.release();
    G.rows.release();
    G.feat.release();
    G.rec.release();
    G.coll_u.release();
    G.coll_f.release();
  }
  ctx->d_tmp.release();
  ctx->d_tmpu.release();
  if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
  if (ctx->h_ctl) cudaFreeHost(ctx->h_ctl);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
  delete ctx;
  return PT_OK;
}

// ---------------------------------------------------------------- materials
static int add_material(pt_context* ctx, int type, const float* c0, const float* c1, float p0,
                        float p1, uint32_t* id) {
  if (!ctx || !id) return fail(ctx, PT_EINVAL, "null argument");
  if (!finite3(c0) || (c1 && !finite3(c1)) || !std::isfinite(p0) || !std::isfinite(p1))
    return fail(ctx, PT_EINVAL, "material parameters must be finite");
  GpuMaterial m;
  memset(&m, 0, sizeof(m));
  m.type = type;
  m.c0x = c0[0];
  m.c0y = c0[1];
  m.c0z = c0[2];
  if (c1) {
    m.c1x = c1[0];
    m.c1y = c1[1];
    m.c1z = c1[2];
  }
  m.p0 = p0;
  m.p1 = p1;
  m.tex0 = m.tex1 = -1;
  ctx->mats.push_back(m);
  ctx->committed = false;
  *id = (uint32_t)ctx->mats.size() - 1;
  return PT_OK;
}

// ----------------------------------------------------------------- textures
// host_includes/textures.hpp: texture callables as records; a material slot
// names a texture in place of its constant colour (pt_material_set_texture).
static int add_texture(pt_context* ctx, GpuTexture t, uint32_t* id) {
  if (!id) return fail(ctx, PT_EINVAL, "null argument");
  ctx->textures.push_back(t);
  ctx->committed = false;
  *id = (uint32_t)ctx->textures.size() - 1;
  return PT_OK;
}

static GpuTexture blank_texture(int kind) {
  GpuTexture t;
  memset(&t, 0, sizeof(t));
  t.kind = kind;
  return t;
}

PT_API int pt_texture_constant(pt_context* ctx, const float rgb[3], uint32_t* id) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(rgb)) return fail(ctx, PT_EINVAL, "texture colour must be finite");
  GpuTexture t = blank_texture(PT_TEX_CONSTANT);
  for (int k = 0; k < 3; k++) t.c[k] = rgb[k];
  return add_texture(ctx, t, id);
}

PT_API int pt_texture_checker(pt_context* ctx, uint32_t odd, uint32_t even, uint32_t* id) {
  if (!ctx) return PT_EINVAL;
  if (odd >= ctx->textures.size() || even >= ctx->textures.size())
    return fail(ctx, PT_EINVAL, "checker: unknown texture id");
  GpuTexture t = blank_texture(PT_TEX_CHECKER);
  t.a = (int)odd;
  t.b = (int)even;
  return add_texture(ctx, t, id);
}

// Perlin tables as Noise_Texture::assignTo makes them (textures.hpp:63-106):
// 256 unit vectors of (-1 + 2 rnd()) components, then perm_x, perm_y,
// perm_z, each a Fisher-Yates shuffle of 0..255 from the top; rnd() is the
// host's std::mt19937 seeded 0 with a uniform float distribution
// (host_common.hpp:59-63), drawn left to right.
static void noise_tables(float* ranvec, int32_t* perm) {
  std::mt19937 gen(0);
  std::uniform_real_distribution<float> dis(0.f, 1.f);
  for (int i = 0; i < 256; i++) {
    float x = -1 + 2 * dis(gen);
    float y = -1 + 2 * dis(gen);
    float z = -1 + 2 * dis(gen);
    float l = std::sqrt(x * x + y * y + z * z);
    ranvec[3 * i] = x / l;
    ranvec[3 * i + 1] = y / l;
    ranvec[3 * i + 2] = z / l;
  }
  for (int a = 0; a < 3; a++) {
    int32_t* p = perm + 256 * a;
    for (int i = 0; i < 256; i++) p[i] = i;
    for (int i = 256 - 1; i > 0; i--) {
      int target = int(dis(gen) * (i + 1));
      int tmp = p[i];
      p[i] = p[target];
      p[target] = tmp;
    }
  }
}

PT_API int pt_noise_tables(float* ranvec, int32_t* perm) {
  if (!ranvec || !perm) return PT_EINVAL;
  noise_tables(ranvec, perm);
  return PT_OK;
}

PT_API int pt_texture_noise(pt_context* ctx, float scale, int axis, const float* ranvec,
                            const int32_t* perm, uint32_t* id) {
  if (!ctx) return PT_EINVAL;
  if (!std::isfinite(scale)) return fail(ctx, PT_EINVAL, "noise scale must be finite");
  if (axis < 0 || axis > 2) return fail(ctx, PT_EINVAL, "invalid axis");
  float rv[768];
  int32_t pm[768];
  if (!ranvec || !perm) noise_tables(rv, pm);
  if (ranvec) memcpy(rv, ranvec, sizeof(rv));
  if (perm) memcpy(pm, perm, sizeof(pm));
  for (int k = 0; k < 768; k++) {
    if (!std::isfinite(rv[k])) return fail(ctx, PT_EINVAL, "noise vectors must be finite");
    if (pm[k] < 0 || pm[k] > 255) return fail(ctx, PT_EINVAL, "noise permutations: 0..255");
  }
  GpuTexture t = blank_texture(PT_TEX_NOISE);
  t.a = axis;
  t.c[0] = scale;
  t.data = (int)ctx->tex_data.size();
  for (int i = 0; i < 256; i++)
    ctx->tex_data.push_back(make_float4(rv[3 * i], rv[3 * i + 1], rv[3 * i + 2], 0.f));
  for (int i = 0; i < 768; i += 4) {
    float4 q;
    memcpy(&q, pm + i, sizeof(q));
    ctx->tex_data.push_back(q);
  }
  return add_texture(ctx, t, id);
}

PT_API int pt_texture_image(pt_context* ctx, const float* rgba, int w, int h, uint32_t* id) {
  if (!ctx) return PT_EINVAL;
  if (!rgba || w <= 0 || h <= 0 || (size_t)w * h > ((size_t)1 << 28))
    return fail(ctx, PT_EINVAL, "image texture: texels and a size of 1 .. 2^28 texels");
  GpuTexture t = blank_texture(PT_TEX_IMAGE);
  t.a = w;
  t.b = h;
  t.data = (int)ctx->tex_data.size();
  size_t n = (size_t)w * h;
  for (size_t k = 0; k < 4 * n; k++)
    if (!std::isfinite(rgba[k])) return fail(ctx, PT_EINVAL, "image texels must be finite");
  size_t base = ctx->tex_data.size();
  ctx->tex_data.resize(base + n);
  memcpy(ctx->tex_data.data() + base, rgba, n * sizeof(float4));
  return add_texture(ctx, t, id);
}

PT_API int pt_texture_gradient(pt_context* ctx, const float a[3], const float b[3],
                               const float c[3], uint32_t* id) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(a) || !finite3(b) || !finite3(c))
    return fail(ctx, PT_EINVAL, "gradient colours must be finite");
  GpuTexture t = blank_texture(PT_TEX_GRADIENT);
  for (int k = 0; k < 3; k++) {
    t.c[k] = a[k];
    t.c[3 + k] = b[k];
    t.c[6 + k] = c[k];
  }
  return add_texture(ctx, t, id);
}

PT_API int pt_texture_vector(pt_context* ctx, const uint32_t* ids, int n, uint32_t* id) {
  if (!ctx) return PT_EINVAL;
  if (n < 0 || (n > 0 && !ids)) return fail(ctx, PT_EINVAL, "vector texture: n >= 0 ids");
  for (int k = 0; k < n; k++)
    if (ids[k] >= ctx->textures.size()) return fail(ctx, PT_EINVAL, "vector: unknown texture id");
  GpuTexture t = blank_texture(PT_TEX_VECTOR);
  t.a = (int)ctx->tex_list.size();
  t.b = n;
  for (int k = 0; k < n; k++) ctx->tex_list.push_back((int)ids[k]);
  return add_texture(ctx, t, id);
}

PT_API int pt_material_set_texture(pt_context* ctx, uint32_t material, int slot,
                                   uint32_t texture) {
  if (!ctx) return PT_EINVAL;
  if (material >= ctx->mats.size()) return fail(ctx, PT_EINVAL, "unknown material id");
  if (slot < 0 || slot > 1) return fail(ctx, PT_EINVAL, "texture slot is 0 or 1");
  if (texture >= ctx->textures.size() && texture != PT_NO_TEXTURE)
    return fail(ctx, PT_EINVAL, "unknown texture id");
  int t = texture == PT_NO_TEXTURE ? -1 : (int)texture;
  (slot == 0 ? ctx->mats[material].tex0 : ctx->mats[material].tex1) = t;
  ctx->committed = false;
  return PT_OK;
}

PT_API int pt_mesh_set_texture_index(pt_context* ctx, uint32_t first_prim, size_t n,
                                     const uint32_t* index) {
  if (!ctx) return PT_EINVAL;
  if (!index || (size_t)first_prim + n > ctx->prims.size())
    return fail(ctx, PT_EINVAL, "texture index: primitive range out of bounds");
  for (size_t k = 0; k < n; k++) {
    if (ctx->prims[first_prim + k].type != PT_PRIM_TRIANGLE)
      return fail(ctx, PT_EINVAL, "texture index: only triangles carry one");
    if (index[k] >= (1u << 30)) return fail(ctx, PT_EINVAL, "texture index must be < 2^30");
  }
  for (size_t k = 0; k < n; k++) {
    uint4& a = ctx->tri_attr[first_prim + k];
    a.w = (a.w & 3u) | (index[k] << 2);
  }
  ctx->committed = false;
  return PT_OK;
}

PT_API int pt_material_lambertian(pt_context* ctx, const float albedo[3], uint32_t* id) {
  return add_material(ctx, PT_MAT_LAMBERTIAN, albedo, nullptr, 0.f, 0.f, id);
}
PT_API int pt_material_metal(pt_context* ctx, const float albedo[3], float fuzz, uint32_t* id) {
  return add_material(ctx, PT_MAT_METAL, albedo, nullptr, fuzz, 0.f, id);
}
PT_API int pt_material_dielectric(pt_context* ctx, const float base[3], const float extinction[3],
                                  float ref_idx, float density, uint32_t* id) {
  if (ctx && !(ref_idx > 0.f)) return fail(ctx, PT_EINVAL, "ref_idx must be > 0");
  return add_material(ctx, PT_MAT_DIELECTRIC, base, extinction, ref_idx, density, id);
}
PT_API int pt_material_diffuse_light(pt_context* ctx, const float emission[3], uint32_t* id) {
  return add_material(ctx, PT_MAT_DIFFUSE_LIGHT, emission, nullptr, 0.f, 0.f, id);
}
PT_API int pt_material_oren_nayar(pt_context* ctx, const float albedo[3], float roughness,
                                  uint32_t* id) {
  // host_includes/materials.hpp:192-198
  float R = roughness;
  float sigma = (0.f > (1.f < R ? 1.f : R)) ? 0.f : (1.f < R ? 1.f : R);  // saturate
  float div = 1.f / (PI_F + ((3.f * PI_F - 4.f) / 6.f) * sigma);
  return add_material(ctx, PT_MAT_OREN_NAYAR, albedo, nullptr, 1.0f * div, sigma * div, id);
}
PT_API int pt_material_torrance_sparrow(pt_context* ctx, const float color[3], float nu, float nv,
                                        uint32_t* id) {
  // host_includes/materials.hpp:235-238
  float R0 = fmaxf(nu, 1e-3f), R1 = fmaxf(nv, 1e-3f);
  return add_material(ctx, PT_MAT_TORRANCE_SPARROW, color, nullptr, R0 * R0, R1 * R1, id);
}
PT_API int pt_material_ashikhmin_shirley(pt_context* ctx, const float diffuse[3],
                                         const float specular[3], float nu, float nv,
                                         uint32_t* id) {
  if (ctx && !specular) return fail(ctx, PT_EINVAL, "specular colour required");
  // host_includes/materials.hpp:173-174
  return add_material(ctx, PT_MAT_ASHIKHMIN_SHIRLEY, diffuse, specular, fmaxf(1.f, nu),
                      fmaxf(1.f, nv), id);
}

// ----------------------------------------------------------------- geometry
static int push_prim(pt_context* ctx, HostPrim& p, const float* xform, uint32_t* prim_id) {
  if (p.material >= ctx->mats.size()) return fail(ctx, PT_EINVAL, "unknown material id");
  if (xform && !affine_ok(xform)) return fail(ctx, PT_EINVAL, "transform is singular or not finite");
  p.xform = add_xform(ctx, xform);
  ctx->prims.push_back(p);
  ctx->tri_attr.push_back(make_uint4(0, 0, 0, 0));
  if (p.type != PT_PRIM_TRIANGLE) ctx->num_non_triangles++;
  if (p.moving) ctx->num_moving++;
  ctx->committed = false;
  if (prim_id) *prim_id = (uint32_t)ctx->prims.size() - 1;
  return PT_OK;
}

PT_API int pt_add_sphere(pt_context* ctx, const float center[3], float radius, uint32_t material,
                         const float xform[12], uint32_t* prim_id) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(center) || !std::isfinite(radius) || !(radius > 0.f))
    return fail(ctx, PT_EINVAL, "sphere needs a finite centre and radius > 0");
  HostPrim p;
  memset(&p, 0, sizeof(p));
  p.type = PT_PRIM_SPHERE;
  p.material = material;
  p.f[0] = center[0];
  p.f[1] = center[1];
  p.f[2] = center[2];
  p.f[3] = radius;
  return push_prim(ctx, p, xform, prim_id);
}

PT_API int pt_add_moving_sphere(pt_context* ctx, const float center0[3], const float center1[3],
                                float radius, float time0, float time1, uint32_t material,
                                const float xform[12], uint32_t* prim_id) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(center0) || !finite3(center1) || !std::isfinite(radius) || !(radius > 0.f))
    return fail(ctx, PT_EINVAL, "moving sphere needs finite centres and radius > 0");
  if (!std::isfinite(time0) || !std::isfinite(time1) || !(time1 > time0))
    return fail(ctx, PT_EINVAL, "moving sphere needs finite times with time1 > time0");
  HostPrim p;
  memset(&p, 0, sizeof(p));
  p.type = PT_PRIM_SPHERE;
  p.moving = 1;
  p.material = material;
  for (int a = 0; a < 3; a++) {
    p.f[a] = center0[a];
    p.f[6 + a] = center1[a];
  }
  p.f[3] = radius;
  p.f[4] = time0;
  p.f[5] = time1;
  return push_prim(ctx, p, xform, prim_id);
}

PT_API int pt_add_rect(pt_context* ctx, float a0, float a1, float b0, float b1, float k, int flip,
                       int axis, uint32_t material, const float xform[12], uint32_t* prim_id) {
  if (!ctx) return PT_EINVAL;
  if (axis < 0 || axis > 2) return fail(ctx, PT_EINVAL, "invalid axis");
  float v[5] = {a0, a1, b0, b1, k};
  for (float x : v)
    if (!std::isfinite(x)) return fail(ctx, PT_EINVAL, "rect bounds must be finite");
  if (!(a1 >= a0) || !(b1 >= b0)) return fail(ctx, PT_EINVAL, "rect needs a0 <= a1, b0 <= b1");
  HostPrim p;
  memset(&p, 0, sizeof(p));
  p.type = PT_PRIM_RECT;
  p.axis = axis;
  p.flip = flip ? 1 : 0;
  p.material = material;
  for (int i = 0; i < 5; i++) p.f[i] = v[i];
  return push_prim(ctx, p, xform, prim_id);
}

PT_API int pt_add_box(pt_context* ctx, const float p0[3], const float p1[3], uint32_t material,
                      const float xform[12], uint32_t* prim_id) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(p0) || !finite3(p1)) return fail(ctx, PT_EINVAL, "box corners must be finite");
  HostPrim p;
  memset(&p, 0, sizeof(p));
  p.type = PT_PRIM_BOX;
  p.material = material;
  for (int i = 0; i < 3; i++) {
    p.f[i] = p0[i];
    p.f[3 + i] = p1[i];
  }
  return push_prim(ctx, p, xform, prim_id);
}

PT_API int pt_add_mesh(pt_context* ctx, const float* verts, size_t nv, const uint32_t* idx,
                       size_t nt, const uint32_t* mat_per_tri, uint32_t material,
                       const float* normals, const float* uvs, const float xform[12],
                       uint32_t* first_prim_id) {
  if (!ctx) return PT_EINVAL;
  if (!verts || !idx || nv == 0 || nt == 0) return fail(ctx, PT_EINVAL, "empty mesh");
  if (xform && !affine_ok(xform)) return fail(ctx, PT_EINVAL, "transform is singular or not finite");
  if (!mat_per_tri && material >= ctx->mats.size())
    return fail(ctx, PT_EINVAL, "unknown material id");
  for (size_t t = 0; t < nt; t++) {
    for (int k = 0; k < 3; k++)
      if (idx[3 * t + k] >= nv) return fail(ctx, PT_EINVAL, "mesh index out of range");
    if (mat_per_tri && mat_per_tri[t] >= ctx->mats.size())
      return fail(ctx, PT_EINVAL, "unknown per-triangle material id");
  }
  for (size_t i = 0; i < 3 * nv; i++)
    if (!std::isfinite(verts[i])) return fail(ctx, PT_EINVAL, "mesh vertices must be finite");
  // flatten into world space (the oracle flattens the same way)
  std::vector<float> wv(3 * nv);
  float inv[12];
  if (xform) affine_inverse(xform, inv);
  for (size_t i = 0; i < nv; i++) {
    if (xform) xpoint_h(xform, verts + 3 * i, &wv[3 * i]);
    else memcpy(&wv[3 * i], verts + 3 * i, 12);
  }
  // attribute vertices: normals and uvs share one index space (the two
  // arrays always hold the same number of vertices)
  size_t nattr = ctx->normals.size() / 3;
  uint32_t abase = (uint32_t)nattr;
  uint32_t flags = (normals ? 1u : 0u) | (uvs ? 2u : 0u);
  if (normals || uvs) {
    ctx->normals.resize(3 * (nattr + nv), 0.f);
    ctx->uvs.resize(2 * (nattr + nv), 0.f);
    for (size_t i = 0; i < nv; i++) {
      if (normals) {
        const float* n = normals + 3 * i;
        float* o = &ctx->normals[3 * (nattr + i)];
        if (xform) {  // transpose of the inverse (the oracle's xnormal)
          o[0] = inv[0] * n[0] + inv[4] * n[1] + inv[8] * n[2];
          o[1] = inv[1] * n[0] + inv[5] * n[1] + inv[9] * n[2];
          o[2] = inv[2] * n[0] + inv[6] * n[1] + inv[10] * n[2];
        } else {
          o[0] = n[0];
          o[1] = n[1];
          o[2] = n[2];
        }
      }
      if (uvs) {
        ctx->uvs[2 * (nattr + i)] = uvs[2 * i];
        ctx->uvs[2 * (nattr + i) + 1] = uvs[2 * i + 1];
      }
    }
  }
  uint32_t first = (uint32_t)ctx->prims.size();
  ctx->prims.reserve(ctx->prims.size() + nt);
  ctx->tri_attr.reserve(ctx->tri_attr.size() + nt);
  for (size_t t = 0; t < nt; t++) {
    HostPrim p;
    memset(&p, 0, sizeof(p));
    p.type = PT_PRIM_TRIANGLE;
    p.xform = -1;
    p.material = mat_per_tri ? mat_per_tri[t] : material;
    for (int k = 0; k < 3; k++) memcpy(&p.f[3 * k], &wv[3 * idx[3 * t + k]], 12);
    ctx->prims.push_back(p);
    ctx->tri_attr.push_back(make_uint4(abase + idx[3 * t], abase + idx[3 * t + 1],
                                       abase + idx[3 * t + 2], flags));
  }
  ctx->committed = false;
  if (first_prim_id) *first_prim_id = first;
  return PT_OK;
}

// ------------------------------------------------------------------- lights
PT_API int pt_add_light_rect(pt_context* ctx, float a0, float a1, float b0, float b1, float k,
                             int axis, const float emission[3]) {
  if (!ctx) return PT_EINVAL;
  if (axis < 0 || axis > 2 || !finite3(emission)) return fail(ctx, PT_EINVAL, "invalid light");
  GpuLight L;
  memset(&L, 0, sizeof(L));
  L.type = PT_LIGHT_RECT;
  L.axis = axis;
  L.a0 = a0;
  L.a1 = a1;
  L.b0 = b0;
  L.b1 = b1;
  L.k = k;
  L.ex = emission[0];
  L.ey = emission[1];
  L.ez = emission[2];
  ctx->lights.push_back(L);
  ctx->committed = false;
  return PT_OK;
}

PT_API int pt_add_light_sphere(pt_context* ctx, const float center[3], float radius,
                               const float emission[3]) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(center) || !(radius > 0.f) || !finite3(emission))
    return fail(ctx, PT_EINVAL, "invalid light");
  GpuLight L;
  memset(&L, 0, sizeof(L));
  L.type = PT_LIGHT_SPHERE;
  L.cx = center[0];
  L.cy = center[1];
  L.cz = center[2];
  L.r = radius;
  L.ex = emission[0];
  L.ey = emission[1];
  L.ez = emission[2];
  ctx->lights.push_back(L);
  ctx->committed = false;
  return PT_OK;
}

// ------------------------------------------------------------------- miss
PT_API int pt_set_env_gradient(pt_context* ctx, const float c1[3], const float c2[3]) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(c1) || !finite3(c2)) return fail(ctx, PT_EINVAL, "invalid colours");
  ctx->miss.type = PT_MISS_GRADIENT;
  ctx->miss.c1x = c1[0]; ctx->miss.c1y = c1[1]; ctx->miss.c1z = c1[2];
  ctx->miss.c2x = c2[0]; ctx->miss.c2y = c2[1]; ctx->miss.c2z = c2[2];
  ctx->committed = false;
  return PT_OK;
}

PT_API int pt_set_env_constant(pt_context* ctx, const float c[3]) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(c)) return fail(ctx, PT_EINVAL, "invalid colour");
  ctx->miss.type = PT_MISS_CONSTANT;
  ctx->miss.c1x = c[0]; ctx->miss.c1y = c[1]; ctx->miss.c1z = c[2];
  ctx->committed = false;
  return PT_OK;
}

PT_API int pt_set_env_map(pt_context* ctx, int kind, const float* rgba, int w, int h,
                          int spherical) {
  if (!ctx) return PT_EINVAL;
  if ((kind != PT_MISS_HDR && kind != PT_MISS_IMG) || !rgba || w <= 0 || h <= 0)
    return fail(ctx, PT_EINVAL, "invalid environment map");
  ctx->miss.type = kind;
  ctx->miss.w = w;
  ctx->miss.h = h;
  ctx->miss.spherical = spherical ? 1 : 0;
  ctx->env.resize((size_t)w * h);
  memcpy(ctx->env.data(), rgba, (size_t)w * h * 16);
  ctx->committed = false;
  return PT_OK;
}

// ------------------------------------------------------------------ camera
PT_API int pt_set_camera(pt_context* ctx, const float lookfrom[3], const float lookat[3],
                         const float vup[3], float vfov, float aspect, float aperture,
                         float focus_dist, float t0, float t1) {
  if (!ctx) return PT_EINVAL;
  if (!finite3(lookfrom) || !finite3(lookat) || !finite3(vup))
    return fail(ctx, PT_EINVAL, "camera vectors must be finite");
  // host_includes/camera.hpp:13-38, with the oracle's elementary functions
  GpuCamera& c = ctx->cam;
  c.lens_radius = aperture / 2.f;
  c.time0 = t0;
  c.time1 = t1;
  float theta = vfov * PI_F / 180.f;
  float half_height = pt_tanf(theta / 2.f);
  float half_width = aspect * half_height;
  float o[3] = {lookfrom[0], lookfrom[1], lookfrom[2]};
  float w[3] = {lookfrom[0] - lookat[0], lookfrom[1] - lookat[1], lookfrom[2] - lookat[2]};
  auto len = [](const float* v) { return ptm_sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
  float lw = len(w);
  w[0] = w[0] / lw; w[1] = w[1] / lw; w[2] = w[2] / lw;
  float u[3] = {vup[1] * w[2] - vup[2] * w[1], vup[2] * w[0] - vup[0] * w[2],
                vup[0] * w[1] - vup[1] * w[0]};
  float lu = len(u);
  u[0] = u[0] / lu; u[1] = u[1] / lu; u[2] = u[2] / lu;
  float v[3] = {w[1] * u[2] - w[2] * u[1], w[2] * u[0] - w[0] * u[2], w[0] * u[1] - w[1] * u[0]};
  float hf = half_width * focus_dist, vf = half_height * focus_dist;
  float llc[3], hor[3], ver[3];
  for (int k = 0; k < 3; k++) {
    llc[k] = o[k] - hf * u[k] - vf * v[k] - focus_dist * w[k];
    hor[k] = 2.f * half_width * focus_dist * u[k];
    ver[k] = 2.f * half_height * focus_dist * v[k];
  }
  c.ox = o[0]; c.oy = o[1]; c.oz = o[2];
  c.lx = llc[0]; c.ly = llc[1]; c.lz = llc[2];
  c.hx = hor[0]; c.hy = hor[1]; c.hz = hor[2];
  c.vx = ver[0]; c.vy = ver[1]; c.vz = ver[2];
  c.ux = u[0]; c.uy = u[1]; c.uz = u[2];
  c.wx = v[0]; c.wy = v[1]; c.wz = v[2];
  ctx->committed = false;
  return PT_OK;
}

// ------------------------------------------------------------------- commit
static void prim_record(const HostPrim& p, uint32_t id, float4* out) {
  uint32_t tag = (uint32_t)p.type | ((uint32_t)p.axis << 2) | ((uint32_t)p.flip << 4) |
                 (p.moving ? PT_PRIM_MOVING : 0u) | ((uint32_t)(p.xform + 1) << 8);
  float tagf, idf, matf;
  memcpy(&tagf, &tag, 4);
  memcpy(&idf, &id, 4);
  memcpy(&matf, &p.material, 4);
  out[0] = make_float4(p.f[0], p.f[1], p.f[2], tagf);
  out[1] = make_float4(p.f[3], p.f[4], p.f[5], idf);
  out[2] = make_float4(p.f[6], p.f[7], p.f[8], matf);
}

}  // extern "C"

// Builds the BVH8 of the scene's primitives (transforms already on the
// device) into nodes / leaf-ordered records / leaf_of_id, with at most
// `width` children per node, and checks its structure on the host.
int pth::build_bvh(pt_context* ctx, int width, DevBuf<uint4>& d_nodes, DevBuf<float4>& d_prims,
                   DevBuf<uint32_t>& d_leaf_of_id, size_t* out_nodes, int* out_depth,
                   size_t* uploaded) {
  size_t up = 0;
  cudaStream_t st = ctx->stream;
  size_t n = ctx->prims.size();
  int builder = ctx->opt.bvh_builder;
  if (builder == 0) builder = n >= 4096 ? 2 : 1;
  pt::Bvh8Out bvh;
  size_t nn = 0;
  if (builder == 2 && n > 0) {
    // records in call order (filled by several host threads for large
    // scenes, into page-locked staging), built into leaf order on the device
    CK(ctx->h_rec.ensure(3 * n));
    {
      const HostPrim* src = ctx->prims.data();
      float4* dst = ctx->h_rec.p;
      auto fill = [src, dst](size_t a, size_t b) {
        for (size_t i = a; i < b; i++) prim_record(src[i], (uint32_t)i, dst + 3 * i);
      };
      const size_t parts = n >= ((size_t)1 << 16) ? 8 : 1;
      std::vector<std::thread> pool;
      for (size_t k = 1; k < parts; k++) pool.emplace_back(fill, n * k / parts, n * (k + 1) / parts);
      fill(0, n / parts);
      for (std::thread& th : pool) th.join();
    }
    CK(ctx->d_rec_in.upload(ctx->h_rec.p, 3 * n, st));
    up += 3 * n * sizeof(float4);
    CK(d_nodes.ensure(5 * std::max<size_t>(1, n)));
    CK(d_prims.ensure(3 * n));
    CK(d_leaf_of_id.ensure(n));
    uint32_t nodes = 0;
    int depth = 0;
    CK(pt::build_bvh8_gpu(ctx->d_rec_in.p, ctx->d_xforms.p, (uint32_t)n, d_nodes.p,
                          d_prims.p, d_leaf_of_id.p, &nodes, &depth, PT_TREELET_ROUNDS, width,
                          ctx->cam.time0, ctx->cam.time1, &ctx->build_arena, st));
    if (depth < 0)
      return fail(ctx, PT_EINVAL,
                  "GPU BVH8 failed validation (check " + std::to_string(-depth) + ")");
    nn = nodes;
    bvh.depth = depth;  // the builder checked the tree's structure on the device
  } else {
    std::vector<pt::Box> boxes(n);
    for (size_t i = 0; i < n; i++) boxes[i] = prim_box(ctx, ctx->prims[i]);
    if (n) pt::build_bvh8_host(boxes, bvh, width);
    if (!pt::validate_bvh8(bvh, n)) return fail(ctx, PT_EINVAL, "BVH8 failed validation");
    // primitive records in leaf order
    std::vector<float4> rec(3 * (n ? n : 1));
    for (size_t k = 0; k < bvh.leaf_order.size(); k++)
      prim_record(ctx->prims[bvh.leaf_order[k]], bvh.leaf_order[k], &rec[3 * k]);
    nn = bvh.nodes.size() / 20;
    std::vector<uint4> nodes(nn ? nn * 5 : 5);
    if (nn) memcpy(nodes.data(), bvh.nodes.data(), bvh.nodes.size() * 4);
    CK(d_nodes.upload(nodes.data(), nodes.size(), st));
    CK(d_prims.upload(rec.data(), rec.size(), st));
    std::vector<uint32_t> leaf_of_id(n ? n : 1, 0);
    for (size_t k = 0; k < bvh.leaf_order.size(); k++) leaf_of_id[bvh.leaf_order[k]] = (uint32_t)k;
    CK(d_leaf_of_id.upload(leaf_of_id.data(), leaf_of_id.size(), st));
    up += nodes.size() * sizeof(uint4) + rec.size() * sizeof(float4) + leaf_of_id.size() * 4;
  }
  CK(cudaStreamSynchronize(st));
  if (uploaded) *uploaded = up;
  *out_nodes = nn;
  *out_depth = bvh.depth;
  return PT_OK;
}

extern "C" {

// Uploads the scene's tables (materials, lights, textures, triangle
// attributes, the environment) on the context's second stream and builds the
// importance-sampling tables of a spherical HDR environment; returns when
// they are on the device (*bytes: the bytes copied host to device).  Runs on
// its own host thread during the BVH build.
static cudaError_t upload_tables(pt_context* ctx, size_t* bytes) {
  cudaStream_t st = ctx->aux_stream;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_mats, ctx->mats, 1, st, bytes);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_lights, ctx->lights, 1, st, bytes);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_textures, ctx->textures, 1, st, bytes);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_tex_data, ctx->tex_data, 1, st, bytes);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_tex_list, ctx->tex_list, 1, st, bytes);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_tri_attr, ctx->tri_attr, 1, st, bytes);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_normals, ctx->normals, 3, st, bytes);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_uvs, ctx->uvs, 2, st, bytes);
  if (e == cudaSuccess) e = upload_or_zero(ctx->d_env, ctx->env, 1, st, bytes);
  ctx->env_valid = 0;
  if (e == cudaSuccess && ctx->miss.type == PT_MISS_HDR && ctx->miss.spherical &&
      !ctx->env.empty()) {
    const int w = ctx->miss.w, h = ctx->miss.h;
    e = ctx->d_env_marg.ensure((size_t)h + 1);
    if (e == cudaSuccess) e = ctx->d_env_cond.ensure((size_t)h * (w + 1));
    if (e == cudaSuccess) e = ctx->d_env_rows.ensure((size_t)h);
    if (e == cudaSuccess) e = ctx->d_env_pre.ensure((size_t)w * h);
    if (e == cudaSuccess) e = ctx->d_env_valid.ensure(1);
    if (e == cudaSuccess) {
      pt::launch_env_cdf(ctx->d_env.p, w, h, ctx->d_env_marg.p, ctx->d_env_cond.p,
                         ctx->d_env_rows.p, ctx->d_env_pre.p, ctx->d_env_valid.p, st);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&ctx->env_valid, ctx->d_env_valid.p, sizeof(int),
                          cudaMemcpyDeviceToHost, st);
  }
  cudaError_t s = cudaStreamSynchronize(st);
  return e != cudaSuccess ? e : s;
}

PT_API int pt_commit(pt_context* ctx) {
  if (!ctx) return PT_EINVAL;
  CK(cudaSetDevice(ctx->device));
  auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = ctx->stream;
  drop_graphs(ctx);
  size_t n = ctx->prims.size();
  std::vector<float4> xf(ctx->xforms.size() / 4 + 1);
  if (!ctx->xforms.empty()) memcpy(xf.data(), ctx->xforms.data(), ctx->xforms.size() * 4);
  CK(ctx->d_xforms.upload(xf.data(), xf.size(), st));
  size_t nn = 0;
  int depth = 0;
  int width = ctx->opt.bvh_width ? ctx->opt.bvh_width : 8;
  // the scene's tables go up from a helper thread on the second stream while
  // this thread builds the BVH
  cudaError_t te = cudaSuccess;
  size_t table_up = 0;
  std::thread tables;
  try {
    tables = std::thread([ctx, &te, &table_up] { te = upload_tables(ctx, &table_up); });
  } catch (...) {
    te = upload_tables(ctx, &table_up);
  }
  size_t bvh_up = 0;
  int rc = build_bvh(ctx, width, ctx->d_nodes, ctx->d_prims, ctx->d_leaf_of_id, &nn, &depth,
                     &bvh_up);
  if (tables.joinable()) tables.join();
  if (rc) return rc;
  if (te != cudaSuccess) return cuda_fail(ctx, te, "scene table upload");
  CK(cudaStreamSynchronize(st));
  DevScene& S = ctx->scene;
  memset(&S, 0, sizeof(S));
  S.nodes = ctx->d_nodes.p;
  S.prims = ctx->d_prims.p;
  S.xforms = ctx->d_xforms.p;
  S.mats = ctx->d_mats.p;
  S.lights = ctx->d_lights.p;
  S.tri_attr = ctx->d_tri_attr.p;
  S.normals = ctx->d_normals.p;
  S.uvs = ctx->d_uvs.p;
  S.leaf_of_id = ctx->d_leaf_of_id.p;
  S.textures = ctx->d_textures.p;
  S.tex_data = ctx->d_tex_data.p;
  S.tex_list = ctx->d_tex_list.p;
  S.num_lights = (int)ctx->lights.size();
  S.num_prims = (int)n;
  S.tri_only = pth::all_triangles(ctx) ? 1 : 0;
  S.has_motion = pth::has_motion(ctx) ? 1 : 0;
  S.miss = ctx->miss;
  S.miss.env = ctx->d_env.p;
  S.cam = ctx->cam;
  S.env_marg = ctx->d_env_marg.p;
  S.env_cond = ctx->d_env_cond.p;
  S.env_valid = ctx->env_valid;
  ctx->bvh_depth = depth;
  ctx->bvh_nodes = nn;
  ctx->bvh_width = width;
  ctx->max_stack = std::max(1, depth + 1);
  if (pt::trace_smem(ctx->max_stack, PT_TRACE_BLOCK) > 200 * 1024)
    return fail(ctx, PT_EINVAL, "BVH too deep for the traversal stack");
  CK(pt::set_trace_smem());
  ctx->lc = pt::default_launch(ctx->max_stack);
  ctx->lc.sort = ctx->opt.shade_order == 1 || (ctx->opt.shade_order == 0 && pth::sort_pays(ctx));
  ctx->lc.refetch = ctx->opt.refetch_lanes ? ctx->opt.refetch_lanes : pth::auto_refetch(n);
  ctx->lc.tex = pth::uses_textures(ctx) ? 1 : 0;
  ctx->lc.motion = pth::has_motion(ctx) ? 1 : 0;
  auto t1 = std::chrono::steady_clock::now();
  ctx->stats.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  ctx->stats.bvh_nodes = nn;
  ctx->stats.bvh_bytes = nn * 80 + n * 48;
  ctx->stats.bvh_depth = depth;
  ctx->stats.upload_bytes = xf.size() * sizeof(float4) + bvh_up + table_up;
  ctx->commit_gen++;
  ctx->committed = true;
  return PT_OK;
}

}  // extern "C"

// ------------------------------------------------------------------- render
// Carves the wavefront arrays out of one float4 block and one uint4 block.
void pth::carve_wave(WaveState& W, float4* f, uint4* u, size_t s) {
  for (int k = 0; k < 2; k++) {
    PathBuf& b = W.path[k];
    b.ray_o = f + (4 * k + 0) * s;
    b.ray_d = f + (4 * k + 1) * s;
    b.thr = f + (4 * k + 2) * s;
    b.rad = f + (4 * k + 3) * s;
    b.st = u + k * s;
  }
  W.hit = f + 8 * s;
  W.sh.P = f + 9 * s;
  W.sh.N = f + 10 * s;
  W.sh.Wo = f + 11 * s;
  W.sh.Wi = f + 12 * s;
  W.sh.thr = f + 13 * s;
  W.sh.rad = f + 14 * s;
  W.sh.C = f + 15 * s;
  W.sh.st = u + 2 * s;
  W.slots = (int)s;
}

extern "C" {

// Automatic wavefront size: the paths of a chunk rounded up to 64 Ki slots, at
// most 8 Mi slots (2.4 GiB of path state), never shrinking.  A larger
// wavefront needs fewer iterations for the same paths, and every iteration
// has a fixed cost (launches, the drain of each kernel): on the
// 2.1 M-triangle heightfield at 1920x1080 paths/s rose 7.9 % from 2 Mi to
// 4 Mi slots and 11.3 % to 8 Mi.  Results do not depend on the slot count.
static int auto_slots(const pt_context* ctx, size_t paths) {
  const size_t q = (size_t)1 << 16, cap = (size_t)1 << 23;
  const size_t want = std::min(cap, std::max(q, (paths + q - 1) / q * q));
  return (int)std::max<size_t>(want, (size_t)ctx->slots);
}

static int ensure_wave(pt_context* ctx, size_t results_needed) {
  int slots = ctx->opt.path_slots > 0 ? ctx->opt.path_slots : auto_slots(ctx, results_needed);
  if (ctx->slots != slots || !ctx->d_slot_f4.p) {
    drop_graphs(ctx);
    CK(ctx->d_slot_f4.ensure((size_t)slots * PT_SLOT_F4));
    CK(ctx->d_slot_u4.ensure((size_t)slots * PT_SLOT_U4));
    CK(ctx->d_ctr.ensure(1));
    CK(ctx->d_ctl.ensure(1));
    ctx->slots = slots;
    carve_wave(ctx->W, ctx->d_slot_f4.p, ctx->d_slot_u4.p, (size_t)slots);
    ctx->W.ctr = ctx->d_ctr.p;
  }
  if (ctx->d_results.n < results_needed || !ctx->d_results.p) {
    drop_graphs(ctx);
    CK(ctx->d_results.ensure(results_needed));
  }
  ctx->W.results = ctx->d_results.p;
  return PT_OK;
}

static const int kItersPerGraph = 8;

static int run_chunk(pt_context* ctx, const pt_render_params* p, int frame0, int frames) {
  cudaStream_t st = ctx->stream;
  WaveCtl& ctl = *ctx->h_ctl;
  ctl.width = p->width;
  ctl.height = p->height;
  ctl.frame0 = frame0;
  ctl.max_depth = p->max_depth;
  ctl.rr_enable = p->rr_enable;
  ctl.rr_depth = p->rr_depth;
  ctl.mode = p->mode;
  ctl.guide = p->guide;
  ctl.guide_depth = ctx->guide.max_bounces > 0 ? (uint32_t)ctx->guide.max_bounces : 0xffffffffu;
  ctl.chunk_paths = (unsigned long long)p->width * p->height * frames;
  fastdiv_magic((uint32_t)(p->width * p->height), &ctl.wh_m, &ctl.wh_l);
  fastdiv_magic((uint32_t)p->width, &ctl.w_m, &ctl.w_l);
  CK(cudaMemcpyAsync(ctx->d_ctl.p, &ctl, sizeof(WaveCtl), cudaMemcpyHostToDevice, st));
  WaveCounters& c = *ctx->h_ctr;
  memset(&c, 0, sizeof(c));
  CK(cudaMemcpyAsync(ctx->d_ctr.p, &c, sizeof(WaveCounters), cudaMemcpyHostToDevice, st));
  bool counters = ctx->opt.enable_counters != 0;
  bool timing = ctx->opt.enable_timing != 0;
  if (timing && ctx->tev.empty()) {
    ctx->tev.resize(2 * 6 * kItersPerGraph);  // a set for each graph instance
    for (auto& e : ctx->tev) CK(cudaEventCreate(&e));
  }
  const bool guide = p->guide != 0;
  GuideInferArgs gi;
  if (guide) gi = guide_infer_args(ctx);
  if (!ctx->graph || ctx->graph_counters != counters || ctx->graph_timing != timing ||
      ctx->graph_mode != p->mode || ctx->graph_guide != guide ||
      memcmp(&ctx->graph_W, &ctx->W, sizeof(WaveState)) != 0) {
    drop_graphs(ctx);
    // with timing, a second instance records on its own events, so one
    // launch can run while the host reads the other's times
    for (int inst = 0; inst < (timing ? 2 : 1); inst++) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      for (int i = 0; i < kItersPerGraph; i++)
        pt::launch_iteration(ctx->scene, ctx->W, ctx->d_ctl.p, ctx->max_stack, counters, ctx->lc,
                             st, timing ? &ctx->tev[6 * (kItersPerGraph * inst + i)] : nullptr,
                             p->mode, nullptr, false, 0, guide ? &gi : nullptr);
      cudaError_t ce = cudaStreamEndCapture(st, &g);
      if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
      cudaError_t e = cudaGraphInstantiate(inst ? &ctx->graph2 : &ctx->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
    }
    ctx->graph_counters = counters;
    ctx->graph_timing = timing;
    ctx->graph_mode = p->mode;
    ctx->graph_guide = guide;
    ctx->graph_W = ctx->W;
  }
  // bounded host loop: a path needs at most max_depth iterations after its
  // generation, and every iteration generates at least one path while any
  // remain, so this many iterations always suffice.  The loop keeps one graph
  // launch queued ahead of the one whose counters it reads (slot 0 / 1:
  // counters, completion event and, with timing, graph instance and events),
  // so the GPU does not wait for the host between launches; the launch queued
  // after the chunk drained runs empty iterations.
  unsigned long long max_iters = ctl.chunk_paths + (unsigned long long)p->max_depth + 16;
  unsigned long long iters = 0;
  auto launch = [&](int slot) -> cudaError_t {
    cudaError_t e = cudaGraphLaunch(timing && slot ? ctx->graph2 : ctx->graph, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&ctx->h_ctr[slot], ctx->d_ctr.p, sizeof(WaveCounters),
                          cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->evc[slot], st);
    ctx->stats.graph_launches++;
    iters += kItersPerGraph;
    return e;
  };
  auto harvest = [&](int slot) -> cudaError_t {
    cudaError_t e = cudaEventSynchronize(ctx->evc[slot]);
    ctx->stats.iterations += kItersPerGraph;
    ctx->stats.kernel_launches += 7 * kItersPerGraph;
    if (timing && e == cudaSuccess) {
      const cudaEvent_t* ev = &ctx->tev[6 * kItersPerGraph * slot];
      for (int i = 0; i < kItersPerGraph; i++)
        for (int k = 0; k < 5; k++) {
          float ms = 0.f;
          if (cudaEventElapsedTime(&ms, ev[6 * i + k], ev[6 * i + k + 1]) == cudaSuccess)
            ctx->stats.stage_ms[k] += ms;
          else
            cudaGetLastError();  // a missing sample is not an error of the render
        }
    }
    return e;
  };
  CK(launch(0));
  int cur = 0;  // the oldest launch in flight
  while (true) {
    CK(launch(cur ^ 1));
    CK(harvest(cur));
    const WaveCounters& cc = ctx->h_ctr[cur];
    if (cc.error) {
      CK(cudaStreamSynchronize(st));
      return fail(ctx, PT_EQUEUE, "traversal stack overflow");
    }
    if (cc.next_path >= ctl.chunk_paths && cc.n_cur == 0) {
      CK(harvest(cur ^ 1));
      c = ctx->h_ctr[cur ^ 1];
      break;
    }
    if (iters > max_iters) {
      CK(cudaStreamSynchronize(st));
      return fail(ctx, PT_ETIMEOUT, "wavefront did not drain");
    }
    cur ^= 1;
  }
  ctx->stats.paths += ctl.chunk_paths;
  ctx->stats.ext_rays += c.ext_rays;
  ctx->stats.shadow_rays += c.shadow_rays;
  ctx->stats.node_fetches += c.node_fetches;
  ctx->stats.prim_tests += c.prim_tests;
  return PT_OK;
}

static void reset_render_stats(pt_context* ctx) {
  pt_stats& s = ctx->stats;
  s.paths = s.ext_rays = s.shadow_rays = s.node_fetches = s.prim_tests = 0;
  s.iterations = s.kernel_launches = s.graph_launches = s.guide_samples = 0;
  for (double& x : s.stage_ms) x = 0.0;
  s.render_ms = 0.0;
}

}  // extern "C"

// Rays through a large scene take many more steps, with a wider spread, so
// lanes refill earlier (a quarter of the warp idle) rather than waiting for
// the whole warp; rays through a small scene are short and alike.  (GB300,
// 1080p: 2.1M-triangle heightfield 24 lanes +6% over 32; 488 spheres 32
// lanes +1% over 24.)
bool pth::has_motion(const pt_context* ctx) { return ctx->num_moving > 0; }

bool pth::all_triangles(const pt_context* ctx) { return ctx->num_non_triangles == 0; }

int pth::auto_refetch(size_t num_prims) { return num_prims > ((size_t)1 << 16) ? 24 : 32; }

bool pth::sort_pays(const pt_context* ctx) {
  for (const GpuMaterial& m : ctx->mats)
    if (m.type == PT_MAT_OREN_NAYAR || m.type == PT_MAT_TORRANCE_SPARROW ||
        m.type == PT_MAT_ASHIKHMIN_SHIRLEY)
      return true;
  return false;
}

int pth::check_params(pt_context* ctx, const pt_render_params* p) {
  if (!p) return fail(ctx, PT_EINVAL, "null params");
  if (p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->frame0 < 0 || p->max_depth <= 0 ||
      p->max_depth > 65535)
    return fail(ctx, PT_EINVAL, "invalid render parameters");
  if ((unsigned long long)p->width * p->height > (1ull << 30))
    return fail(ctx, PT_EINVAL, "image too large");
  if (p->mode != PT_MODE_REF && p->mode != PT_MODE_CONSISTENT)
    return fail(ctx, PT_EINVAL, "unknown integrator mode");
  if (p->guide != 0 && p->guide != 1) return fail(ctx, PT_EINVAL, "guide must be 0 or 1");
  if (p->guide && p->mode != PT_MODE_CONSISTENT)
    return fail(ctx, PT_EINVAL, "the learned guide needs the consistent integrator mode");
  if (!ctx->committed) return fail(ctx, PT_ESTATE, "scene not committed (call pt_commit)");
  return PT_OK;
}

extern "C" {

// Render into a device accumulator: float4 per pixel, or 4 doubles per
// pixel when acc64.
static int render_device(pt_context* ctx, const pt_render_params* p, void* d_acc,
                         bool acc64 = false) {
  cudaStream_t st = ctx->stream;
  size_t WH = (size_t)p->width * p->height;
  const size_t results_cap = (size_t)1 << 27;  // 128 M paths = 2 GiB of results
  int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)p->spp, results_cap / WH));
  if (p->guide) chunk = 1;  // the guide trains between frames
  int rc = ensure_wave(ctx, (size_t)chunk * WH);
  if (rc) return rc;
  if (p->guide) {
    rc = guide_prepare(ctx);
    if (rc) return rc;
    if (!ctx->guide.ready && (rc = pt_guide_init(ctx, 0)) != PT_OK) return rc;
    CK(ctx->guide.out.ensure((size_t)ctx->slots));
    CK(ctx->guide.rows.ensure((size_t)ctx->slots));
    CK(ctx->guide.feat.ensure(3 * (size_t)ctx->slots));
    ctx->W.guide = ctx->guide.out.p;
  }
  if (p->frame0 == 0) CK(cudaMemsetAsync(d_acc, 0, WH * (acc64 ? 32 : 16), st));
  for (int f = 0; f < p->spp; f += chunk) {
    int frames = std::min(chunk, p->spp - f);
    if (p->guide) {
      rc = guide_frame_begin(ctx, p->width, p->height);
      if (rc) return rc;
      ctx->W.grec = ctx->guide.rec.p;
      ctx->W.grec_stride = ctx->guide.rec_stride;
      ctx->W.grec_n = ctx->guide.rec_n;
    }
    rc = run_chunk(ctx, p, p->frame0 + f, frames);
    if (rc) return rc;
    if (p->guide) {
      rc = guide_frame_train(ctx);
      if (rc) return rc;
    }
    if (acc64)
      pt::launch_accumulate64(ctx->d_results.p, (double*)d_acc, p->width, p->height, frames, st);
    else
      pt::launch_accumulate(ctx->d_results.p, (float4*)d_acc, p->width, p->height, frames, st);
    ctx->stats.kernel_launches += 1;
  }
  if (p->guide) {
    uint32_t fl[4];
    CK(cudaMemcpyAsync(fl, ctx->guide.counters.p, 16, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (fl[1] || fl[2]) return fail(ctx, PT_ETIMEOUT, "guide kernel: tensor-core wait ran out");
    ctx->stats.guide_samples = std::min<uint64_t>(fl[0], (uint64_t)1 << 19);
  }
  return PT_OK;
}

PT_API int pt_render(pt_context* ctx, const pt_render_params* params, float* accum_rgba,
                     void* stream) {
  if (!ctx) return PT_EINVAL;
  int rc = check_params(ctx, params);
  if (rc) return rc;
  if (!accum_rgba) return fail(ctx, PT_EINVAL, "null accumulator");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t user = (cudaStream_t)stream;
  cudaStream_t st = ctx->stream;
  // order after the caller's stream
  CK(cudaEventRecord(ctx->ev0, user));
  CK(cudaStreamWaitEvent(st, ctx->ev0, 0));
  reset_render_stats(ctx);
  size_t WH = (size_t)params->width * params->height;
  int kind = device_ptr_kind(accum_rgba, ctx->device);
  if (kind < 0) return fail(ctx, PT_EINVAL, kOtherDevice);
  bool dev = kind > 0;
  float4* d_acc = (float4*)accum_rgba;
  if (!dev) {
    CK(ctx->d_acc.ensure(WH));
    d_acc = ctx->d_acc.p;
    if (params->frame0 != 0)
      CK(cudaMemcpyAsync(d_acc, accum_rgba, WH * sizeof(float4), cudaMemcpyHostToDevice, st));
  }
  CK(cudaEventRecord(ctx->ev0, st));
  rc = render_device(ctx, params, d_acc);
  if (rc) return rc;
  CK(cudaEventRecord(ctx->ev1, st));
  if (!dev) CK(cudaMemcpyAsync(accum_rgba, d_acc, WH * sizeof(float4), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.render_ms = ms;
  return PT_OK;
}

PT_API int pt_render_accum64(pt_context* ctx, const pt_render_params* params,
                             double* accum_rgba, void* stream) {
  if (!ctx) return PT_EINVAL;
  int rc = check_params(ctx, params);
  if (rc) return rc;
  if (!accum_rgba) return fail(ctx, PT_EINVAL, "null accumulator");
  if (((uintptr_t)accum_rgba & 15u) != 0)
    return fail(ctx, PT_EINVAL, "the double accumulator must be 16-byte aligned");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  CK(cudaEventRecord(ctx->ev0, (cudaStream_t)stream));
  CK(cudaStreamWaitEvent(st, ctx->ev0, 0));
  reset_render_stats(ctx);
  size_t WH = (size_t)params->width * params->height;
  int kind = device_ptr_kind(accum_rgba, ctx->device);
  if (kind < 0) return fail(ctx, PT_EINVAL, kOtherDevice);
  bool dev = kind > 0;
  double* d_acc = accum_rgba;
  if (!dev) {
    CK(ctx->d_acc64.ensure(4 * WH));
    d_acc = ctx->d_acc64.p;
    if (params->frame0 != 0)
      CK(cudaMemcpyAsync(d_acc, accum_rgba, WH * 32, cudaMemcpyHostToDevice, st));
  }
  CK(cudaEventRecord(ctx->ev0, st));
  rc = render_device(ctx, params, d_acc, true);
  if (rc) return rc;
  CK(cudaEventRecord(ctx->ev1, st));
  if (!dev) CK(cudaMemcpyAsync(accum_rgba, d_acc, WH * 32, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.render_ms = ms;
  return PT_OK;
}

PT_API int pt_render_paths(pt_context* ctx, const pt_render_params* params, float* out_rgb,
                           void* stream) {
  if (!ctx) return PT_EINVAL;
  int rc = check_params(ctx, params);
  if (rc) return rc;
  if (!out_rgb) return fail(ctx, PT_EINVAL, "null output");
  if (params->guide) return fail(ctx, PT_EINVAL, "pt_render_paths renders without the guide");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  CK(cudaEventRecord(ctx->ev0, (cudaStream_t)stream));
  CK(cudaStreamWaitEvent(st, ctx->ev0, 0));
  pt_render_params p = *params;
  p.spp = 1;
  size_t WH = (size_t)p.width * p.height;
  CK(ctx->d_acc.ensure(WH));
  reset_render_stats(ctx);
  p.frame0 = 0;  // acc scratch zeroed; the frame index goes into the chunk
  rc = ensure_wave(ctx, WH);
  if (rc) return rc;
  p.frame0 = params->frame0;
  rc = run_chunk(ctx, &p, p.frame0, 1);
  if (rc) return rc;
  int kind = device_ptr_kind(out_rgb, ctx->device);
  if (kind < 0) return fail(ctx, PT_EINVAL, kOtherDevice);
  bool dev = kind > 0;
  float* d_out = out_rgb;
  if (!dev) {
    CK(ctx->d_tmp.ensure(3 * WH));
    d_out = ctx->d_tmp.p;
  }
  pt::launch_paths_out(ctx->d_results.p, d_out, (uint32_t)WH, st);
  if (!dev) CK(cudaMemcpyAsync(out_rgb, d_out, 3 * WH * sizeof(float), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return PT_OK;
}

PT_API int pt_trace_first_hits(pt_context* ctx, int width, int height, int frame, uint32_t* prim,
                               uint32_t* mat, float* t, void* stream) {
  if (!ctx) return PT_EINVAL;
  if (width <= 0 || height <= 0 || frame < 0 || !prim || !mat || !t)
    return fail(ctx, PT_EINVAL, "invalid arguments");
  if (!ctx->committed) return fail(ctx, PT_ESTATE, "scene not committed (call pt_commit)");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  CK(cudaEventRecord(ctx->ev0, (cudaStream_t)stream));
  CK(cudaStreamWaitEvent(st, ctx->ev0, 0));
  size_t WH = (size_t)width * height;
  CK(ctx->d_tmpu.ensure(2 * WH + 1));
  CK(ctx->d_tmp.ensure(WH));
  uint32_t* d_err = ctx->d_tmpu.p + 2 * WH;
  CK(cudaMemsetAsync(d_err, 0, 4, st));
  pt::launch_first_hits(ctx->scene, width, height, frame, ctx->d_tmpu.p, ctx->d_tmpu.p + WH,
                        ctx->d_tmp.p, ctx->max_stack, d_err, ctx->lc.trace_grid, st);
  CK(cudaGetLastError());
  uint32_t herr = 0;
  CK(cudaMemcpyAsync(prim, ctx->d_tmpu.p, WH * 4, cudaMemcpyDefault, st));
  CK(cudaMemcpyAsync(mat, ctx->d_tmpu.p + WH, WH * 4, cudaMemcpyDefault, st));
  CK(cudaMemcpyAsync(t, ctx->d_tmp.p, WH * 4, cudaMemcpyDefault, st));
  CK(cudaMemcpyAsync(&herr, d_err, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (herr) return fail(ctx, PT_EQUEUE, "traversal stack overflow");
  return PT_OK;
}

PT_API int pt_resolve_display(pt_context* ctx, const float* accum_rgba, int width, int height,
                              int frame, uint8_t* rgba8, void* stream) {
  if (!ctx) return PT_EINVAL;
  if (!accum_rgba || !rgba8 || width <= 0 || height <= 0 || frame < 0)
    return fail(ctx, PT_EINVAL, "invalid arguments");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  CK(cudaEventRecord(ctx->ev0, (cudaStream_t)stream));
  CK(cudaStreamWaitEvent(st, ctx->ev0, 0));
  size_t WH = (size_t)width * height;
  const float4* d_acc = (const float4*)accum_rgba;
  int kind = device_ptr_kind(accum_rgba, ctx->device);
  if (kind < 0) return fail(ctx, PT_EINVAL, kOtherDevice);
  if (kind == 0) {
    CK(ctx->d_acc.ensure(WH));
    CK(cudaMemcpyAsync(ctx->d_acc.p, accum_rgba, WH * 16, cudaMemcpyHostToDevice, st));
    d_acc = ctx->d_acc.p;
  }
  CK(ctx->d_tmpu.ensure(WH));
  pt::launch_resolve(d_acc, (uchar4*)ctx->d_tmpu.p, (int)WH, frame, st);
  CK(cudaMemcpyAsync(rgba8, ctx->d_tmpu.p, WH * 4, cudaMemcpyDefault, st));
  CK(cudaStreamSynchronize(st));
  return PT_OK;
}

PT_API int pt_get_stats(pt_context* ctx, pt_stats* out) {
  if (!ctx || !out) return PT_EINVAL;
  *out = ctx->stats;
  return PT_OK;
}

}  // extern "C"

// ============================================================================
// pt_render_noalloc: rendering for callers that cannot allocate device memory
// at call time (for example code running under a memory pool that forbids
// cudaMalloc, or an application that allocates everything at start-up and
// then only launches).  It performs no cudaMalloc, cudaFree or other
// allocating call: the wavefront scratch (path-state slots, queues, counters
// and per-path results) lives in the fixed file-scope device array below,
// which every GPU that loads this library holds until the process exits.
//
// Limits: images of at most PT_NOALLOC_MAX_PIXELS pixels (the per-path
// result area holds one frame of that size); PT_NOALLOC_SLOTS paths in
// flight, so it is slower than pt_render on large images.  All calls share
// the array and it keeps the last call's contents: each call resets the
// counters it needs; the path arrays are written before they are read.  Calls whose GPU work
// overlaps (several host threads, streams or contexts on one device) race
// on the array and must be serialised by the caller.
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress; make that first call before any stream capture.
// ============================================================================
namespace {

constexpr size_t kNoAllocSlots = 16384;
constexpr size_t kNoAllocMaxPixels = 262144;  // e.g. 512 x 512
constexpr size_t kNoAllocBytes =
    kNoAllocSlots * (PT_SLOT_F4 * sizeof(float4) + PT_SLOT_U4 * sizeof(uint4)) +
    256 /* WaveCounters */ + 256 /* WaveCtl */ + kNoAllocMaxPixels * sizeof(float4);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
// device address of the array, per device; atomic because two host threads
// may make their first call on one device at the same time (both resolve
// the same address)
static std::atomic<void*> g_noalloc_ptr[kMaxDevices];

// Once per device, with that device current: the host-side name of the
// array is a stand-in, not a device address, so kernels get this pointer.
static int noalloc_setup(pt_context* ctx, unsigned char** out) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices) return fail(ctx, PT_EINVAL, "device ordinal");
  void* p = g_noalloc_ptr[ctx->device].load(std::memory_order_acquire);
  if (!p) {
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(ctx, e, "cudaGetSymbolAddress(noalloc scratch)");
    g_noalloc_ptr[ctx->device].store(p, std::memory_order_release);
  }
  *out = (unsigned char*)p;
  return PT_OK;
}

static WaveState noalloc_wave(unsigned char* base, WaveCtl** ctl) {
  WaveState W;
  memset(&W, 0, sizeof(W));
  size_t s = kNoAllocSlots;
  float4* f = (float4*)base;
  uint4* u = (uint4*)(f + PT_SLOT_F4 * s);
  carve_wave(W, f, u, s);
  unsigned char* tail = (unsigned char*)(u + PT_SLOT_U4 * s);
  W.ctr = (WaveCounters*)tail;
  *ctl = (WaveCtl*)(tail + 256);
  W.results = (float4*)(tail + 512);
  return W;
}

}  // namespace

extern "C" PT_API int pt_render_noalloc(pt_context* ctx, const pt_render_params* p,
                                        float* accum_rgba, void* stream) {
  static_assert(sizeof(WaveCounters) <= 256 && sizeof(WaveCtl) <= 256, "scratch layout");
  if (!ctx) return PT_EINVAL;
  int rc = check_params(ctx, p);
  if (rc) return rc;
  if (p->guide) return fail(ctx, PT_EINVAL, "pt_render_noalloc renders without the guide");
  size_t WH = (size_t)p->width * p->height;
  if (WH > kNoAllocMaxPixels)
    return fail(ctx, PT_EINVAL,
                "pt_render_noalloc: image has " + std::to_string(WH) + " pixels, its static "
                "scratch holds at most " + std::to_string(kNoAllocMaxPixels) + "; use pt_render");
  if (!accum_rgba || device_ptr_kind(accum_rgba, ctx->device) <= 0)
    return fail(ctx, PT_EINVAL, "pt_render_noalloc needs a device accumulator on the "
                                "context's GPU");
  CK(cudaSetDevice(ctx->device));
  unsigned char* base = nullptr;
  rc = noalloc_setup(ctx, &base);
  if (rc) return rc;
  WaveCtl* d_ctl = nullptr;
  WaveState W = noalloc_wave(base, &d_ctl);
  cudaStream_t st = ctx->stream;
  CK(cudaEventRecord(ctx->ev0, (cudaStream_t)stream));
  CK(cudaStreamWaitEvent(st, ctx->ev0, 0));
  CK(cudaEventRecord(ctx->ev0, st));  // start of the device time (render_ms)
  reset_render_stats(ctx);
  float4* acc = (float4*)accum_rgba;
  if (p->frame0 == 0) CK(cudaMemsetAsync(acc, 0, WH * sizeof(float4), st));
  int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)p->spp, kNoAllocMaxPixels / WH));
  WaveCounters& c = *ctx->h_ctr;
  WaveCtl& ctl = *ctx->h_ctl;
  for (int f = 0; f < p->spp; f += chunk) {
    int frames = std::min(chunk, p->spp - f);
    ctl.width = p->width;
    ctl.height = p->height;
    ctl.frame0 = p->frame0 + f;
    ctl.max_depth = p->max_depth;
    ctl.rr_enable = p->rr_enable;
    ctl.rr_depth = p->rr_depth;
    ctl.mode = p->mode;
    ctl.guide = p->guide;
    ctl.chunk_paths = (unsigned long long)WH * frames;
    fastdiv_magic((uint32_t)WH, &ctl.wh_m, &ctl.wh_l);
    fastdiv_magic((uint32_t)p->width, &ctl.w_m, &ctl.w_l);
    CK(cudaMemcpyAsync(d_ctl, &ctl, sizeof(WaveCtl), cudaMemcpyHostToDevice, st));
    memset(&c, 0, sizeof(c));  // no live path; the counters start at zero
    CK(cudaMemcpyAsync(W.ctr, &c, sizeof(WaveCounters), cudaMemcpyHostToDevice, st));
    unsigned long long max_iters = ctl.chunk_paths + (unsigned long long)p->max_depth + 16;
    unsigned long long iters = 0;
    while (true) {
      for (int i = 0; i < kItersPerGraph; i++)
        pt::launch_iteration(ctx->scene, W, d_ctl, ctx->max_stack, false, ctx->lc, st, nullptr,
                             p->mode, nullptr, false, 0);
      CK(cudaGetLastError());
      iters += kItersPerGraph;
      ctx->stats.iterations += kItersPerGraph;
      ctx->stats.kernel_launches += 7 * kItersPerGraph;
      CK(cudaMemcpyAsync(ctx->h_ctr, W.ctr, sizeof(WaveCounters), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (c.error) return fail(ctx, PT_EQUEUE, "traversal stack overflow");
      if (c.next_path >= ctl.chunk_paths && c.n_cur == 0) break;
      if (iters > max_iters) return fail(ctx, PT_ETIMEOUT, "wavefront did not drain");
    }
    ctx->stats.paths += ctl.chunk_paths;
    ctx->stats.ext_rays += c.ext_rays;
    ctx->stats.shadow_rays += c.shadow_rays;
    pt::launch_accumulate(W.results, acc, p->width, p->height, frames, st);
    ctx->stats.kernel_launches += 1;
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->ev1, st));
  CK(cudaStreamWaitEvent((cudaStream_t)stream, ctx->ev1, 0));
  CK(cudaStreamSynchronize(st));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.render_ms = ms;
  return PT_OK;
}

