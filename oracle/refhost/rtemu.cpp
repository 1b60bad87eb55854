/*
 * rtemu.cpp - a small emulation of the OptiX 6 runtime that runs the
 * reference's device programs (compiled unmodified by the ref_*.cpp
 * wrappers) on the CPU, and the C API of oracle/_ref/libref.so.
 *
 * TEST INFRASTRUCTURE ONLY: it exists to check the oracle (oracle.cpp)
 * against the reference's own code.  Single-threaded: the programs keep
 * their variables in file-scope statics, as OptiX programs do per launch.
 *
 * What the runtime does, where OptiX would:
 *   - rtTrace: every primitive in id order runs its intersection program on
 *     the ray in its object space (inverse instance transform; direction not
 *     renormalised, so t is shared); rtPotentialIntersection accepts t in
 *     (tmin, closest so far), rtReportIntersection makes it the closest, so
 *     among equal t the lower primitive id wins.  Triangles take the RTX
 *     path of host_includes/mesh.hpp:176-188: a watertight hardware-style
 *     test (Woop, Benthin & Wald 2013, standing in for the RT cores), then
 *     the Attributes program.  A radiance ray then runs the closest-hit
 *     program of the primitive's material, or the miss program; a shadow
 *     ray runs the any-hit program of programs/hit.cu on the closest
 *     intersection (one valid OptiX traversal order), or counts as occluded
 *     when it hits nothing.  Closest-hit and any-hit programs see the ray in
 *     the object space of the primitive that was hit, and rtTransformPoint /
 *     rtTransformNormal map with that primitive's transform (normals by the
 *     transpose of the world->object matrix).
 *   - Meshes are flattened to world space when added, like the oracle's.
 *   - Callable programs (textures, the lights' sample/pdf, the HitRecord
 *     function) are bound to the scene's objects; buffers view its arrays.
 *   - The host-side set-up that OptiX's C++ API did is restated from the
 *     reference: the camera (host_includes/camera.hpp:13-38) and the
 *     material parameter conversions (ref_convert_params, ref_units.cpp).
 */
#include <memory>

#include "rtemu.h"

extern "C" void ref_convert_params(int type, float p0, float p1, float* q);

namespace {

enum { MAT_LAMBERTIAN = 0, MAT_METAL, MAT_DIELECTRIC, MAT_DIFFUSE_LIGHT, MAT_OREN_NAYAR,
       MAT_TORRANCE_SPARROW, MAT_ASHIKHMIN_SHIRLEY };
enum { PRIM_TRIANGLE = 0, PRIM_SPHERE, PRIM_RECT, PRIM_BOX };
enum { TEX_CONSTANT = 0, TEX_IMAGE };
enum { LIGHT_RECT = 0, LIGHT_SPHERE };
enum { MISS_GRADIENT = 0, MISS_CONSTANT, MISS_HDR, MISS_IMAGE };

// Textures the runtime makes for the materials' constant colours and the
// miss programs (ids -1, -2, ... in the programs' callables), and the
// scene's own textures (ids 0, 1, ... as the oracle and the library number
// them).
struct Texture {
  int kind;
  float c[3];
  int image;  // index into Scene::images
};
struct UserTexture {
  int kind;   // the oracle's TEX_*
  int a, b;   // checker: odd, even; vector: -, size; image: w, h; noise: axis
  float c[9];
  std::vector<float> texels;  // image rgba
  std::vector<float3> ranvec; // noise
  std::vector<int> perm;      // noise: perm_x, perm_y, perm_z
  std::vector<int> ids;       // vector entries
};
struct Material {
  int type;
  int tex[2];
  float p[2];
};
struct Xform {
  float m[12], inv[12];
};
struct Prim {
  int type, axis, flip, material, xform, mesh, local;
  float f[6];
};
struct Mesh {
  std::vector<float3> v, n;
  std::vector<float2> uv;
  std::vector<int3> idx;
  std::vector<int> texidx;
};
struct Light {
  int type, axis;
  float f[5];
  float3 emission;
};
struct Image {
  std::vector<float> texels;
  int w, h;
};
struct Scene {
  std::vector<Texture> tex;
  std::vector<UserTexture> utex;
  std::vector<Material> mats;
  std::vector<Xform> xforms;
  std::vector<Prim> prims;
  std::vector<Mesh> meshes;
  std::vector<Light> lights;
  std::vector<Image> images;
  int miss_kind = MISS_GRADIENT;
  int miss_tex[2] = {0, 0};
  int spherical = 1;
  float cam[21] = {0};
  uint64_t ext = 0, shadow = 0;
};

Scene* g = nullptr;
int g_generation = 0;

void use(Scene* s) {
  if (g != s) {
    g = s;
    g_generation++;
  }
}

// State of one rtTrace (nested traces stack).
struct TraceState {
  float tmin, tmax, t_candidate;
  bool reported;
  unsigned int prim_index;
  float2 bary;
};
TraceState* ts = nullptr;
int cur_prim = -1;   // primitive whose programs run (intersection, closest/any hit)
int bound_mesh = -1;

// first-hit recording (rh_first_hits) and single-ray probes (rh_probe)
bool rec_first = false, rec_done = false, probe = false;
int rec_prim = -1;
float rec_t = 0.f;
float2 rec_bc;
EmuRec probe_rec;

inline float3 xpoint(const float* m, const float3& p) {
  return make_float3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
                     m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
                     m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
inline float3 xvector(const float* m, const float3& p) {
  return make_float3(m[0] * p.x + m[1] * p.y + m[2] * p.z, m[4] * p.x + m[5] * p.y + m[6] * p.z,
                     m[8] * p.x + m[9] * p.y + m[10] * p.z);
}
inline float3 xnormal(const float* inv, const float3& n) {
  return make_float3(inv[0] * n.x + inv[4] * n.y + inv[8] * n.z,
                     inv[1] * n.x + inv[5] * n.y + inv[9] * n.z,
                     inv[2] * n.x + inv[6] * n.y + inv[10] * n.z);
}

// Inverse of an affine 3x4 matrix in double (adjugate), rounded once to float:
// the runtime's instance-transform inverse.
void affine_inverse(const float* m, float* out) {
  double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g_ = m[8], h = m[9],
         i = m[10];
  double A = e * i - f * h, B = -(d * i - f * g_), C = d * h - e * g_;
  double det = a * A + b * B + c * C;
  double inv_det = 1.0 / det;
  double r[9] = {A * inv_det, -(b * i - c * h) * inv_det, (b * f - c * e) * inv_det,
                 B * inv_det, (a * i - c * g_) * inv_det, -(a * f - c * d) * inv_det,
                 C * inv_det, -(a * h - b * g_) * inv_det, (a * e - b * d) * inv_det};
  double tx = m[3], ty = m[7], tz = m[11];
  for (int row = 0; row < 3; row++) {
    out[row * 4 + 0] = (float)r[row * 3 + 0];
    out[row * 4 + 1] = (float)r[row * 3 + 1];
    out[row * 4 + 2] = (float)r[row * 3 + 2];
    out[row * 4 + 3] =
        (float)(-(r[row * 3 + 0] * tx + r[row * 3 + 1] * ty + r[row * 3 + 2] * tz));
  }
}

inline float comp(const float3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// Watertight ray/triangle test (Woop, Benthin & Wald, JCGT 2(1) 2013): the
// stand-in for the RT-core triangle test.  Barycentrics of v1 (u) and v2 (v).
bool watertight(const float3& v0, const float3& v1, const float3& v2, const float3& o,
                const float3& d, float& t, float& bu, float& bv) {
  float adx = fabsf(d.x), ady = fabsf(d.y), adz = fabsf(d.z);
  int kz = (adx > ady) ? ((adx > adz) ? 0 : 2) : ((ady > adz) ? 1 : 2);
  int kx = kz + 1;
  if (kx == 3) kx = 0;
  int ky = kx + 1;
  if (ky == 3) ky = 0;
  if (comp(d, kz) < 0.0f) {
    int tmp = kx;
    kx = ky;
    ky = tmp;
  }
  float Sz = 1.0f / comp(d, kz);
  float Sx = comp(d, kx) * Sz;
  float Sy = comp(d, ky) * Sz;
  float3 A = v0 - o, B = v1 - o, C = v2 - o;
  float Ax = comp(A, kx) - Sx * comp(A, kz), Ay = comp(A, ky) - Sy * comp(A, kz);
  float Bx = comp(B, kx) - Sx * comp(B, kz), By = comp(B, ky) - Sy * comp(B, kz);
  float Cx = comp(C, kx) - Sx * comp(C, kz), Cy = comp(C, ky) - Sy * comp(C, kz);
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  float det = U + V + W;
  if (det == 0.0f) return false;
  float Az = Sz * comp(A, kz), Bz = Sz * comp(B, kz), Cz = Sz * comp(C, kz);
  float T = U * Az + V * Bz + W * Cz;
  float rcp = 1.0f / det;
  t = T * rcp;
  bu = V * rcp;
  bv = W * rcp;
  return true;
}

void bind_mesh(int m) {
  if (m < 0 || m == bound_mesh) return;
  Mesh& M = g->meshes[m];
  ref_triangle_bind(M.v.data(), M.v.size(), M.n.data(), M.n.size(), M.uv.data(), M.uv.size(),
                    M.idx.data(), M.idx.size(), M.texidx.data());
  bound_mesh = m;
}

Ray object_ray(const Prim& p, const Ray& r) {
  if (p.xform < 0) return r;
  Ray o = r;
  const float* inv = g->xforms[p.xform].inv;
  o.origin = xpoint(inv, r.origin);
  o.direction = xvector(inv, r.direction);
  return o;
}

void call_closest_hit(const Material& m, void* prd, const Ray& r, float t, int gi, float2 b) {
  switch (m.type) {
    case MAT_LAMBERTIAN: ref_lambertian_hit(prd, &r, t, gi, b, m.tex, m.p); break;
    case MAT_METAL: ref_metal_hit(prd, &r, t, gi, b, m.tex, m.p); break;
    case MAT_DIELECTRIC: ref_dielectric_hit(prd, &r, t, gi, b, m.tex, m.p); break;
    case MAT_DIFFUSE_LIGHT: ref_diffuse_light_hit(prd, &r, t, gi, b, m.tex, m.p); break;
    case MAT_OREN_NAYAR: ref_oren_nayar_hit(prd, &r, t, gi, b, m.tex, m.p); break;
    case MAT_TORRANCE_SPARROW: ref_torrance_sparrow_hit(prd, &r, t, gi, b, m.tex, m.p); break;
    default: ref_ashikhmin_shirley_hit(prd, &r, t, gi, b, m.tex, m.p); break;
  }
}

}  // namespace

// ---------------------------------------------------------- runtime calls --
bool rtemu_potential_intersection(float t) {
  ts->t_candidate = t;
  return t > ts->tmin && t < ts->tmax;
}

bool rtemu_report_intersection(unsigned int) {
  ts->tmax = ts->t_candidate;
  ts->reported = true;
  return true;
}

void rtemu_terminate_ray() {}

float3 rtemu_transform_point(int kind, const float3& p) {
  if (cur_prim < 0) return p;  // a program called on its own: object = world
  const Prim& pr = g->prims[cur_prim];
  if (pr.xform < 0) return p;
  const Xform& x = g->xforms[pr.xform];
  return xpoint(kind == RT_OBJECT_TO_WORLD ? x.m : x.inv, p);
}

float3 rtemu_transform_normal(int kind, const float3& n) {
  if (cur_prim < 0) return n;
  const Prim& pr = g->prims[cur_prim];
  if (pr.xform < 0) return n;
  const Xform& x = g->xforms[pr.xform];
  return xnormal(kind == RT_OBJECT_TO_WORLD ? x.inv : x.m, n);
}

unsigned int rtemu_primitive_index() { return ts->prim_index; }
float2 rtemu_triangle_barycentrics() { return ts->bary; }

float4 rtemu_tex2d(const float* e, int w, int h, float u, float v) {
  if (!(u == u) || !(v == v) || fabsf(u) > 1e6f || fabsf(v) > 1e6f) return make_float4(0.f);
  float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
  float fx = ptm_floor(x), fy = ptm_floor(y);
  float ax = x - fx, ay = y - fy;
  int ix0 = (int)fx % w;
  if (ix0 < 0) ix0 += w;
  int iy0 = (int)fy % h;
  if (iy0 < 0) iy0 += h;
  int ix1 = ix0 + 1 == w ? 0 : ix0 + 1;
  int iy1 = iy0 + 1 == h ? 0 : iy0 + 1;
  auto tx = [&](int ix, int iy) {
    const float* p = e + ((size_t)iy * w + ix) * 4;
    return make_float3(p[0], p[1], p[2]);
  };
  float3 c = (tx(ix0, iy0) * (1.f - ax) + tx(ix1, iy0) * ax) * (1.f - ay) +
             (tx(ix0, iy1) * (1.f - ax) + tx(ix1, iy1) * ax) * ay;
  return make_float4(c.x, c.y, c.z, 0.f);
}

void rtemu_trace(const Ray& ray, void* payload) {
  TraceState st;
  st.tmin = ray.tmin;
  st.tmax = ray.tmax;
  st.t_candidate = 0.f;
  st.reported = false;
  st.prim_index = 0;
  st.bary = make_float2(0.f);
  TraceState* saved_ts = ts;
  int saved_prim = cur_prim, saved_mesh = bound_mesh;
  ts = &st;
  int best = -1, best_gi = 0;
  float2 best_bc = make_float2(0.f);
  Ray best_ray = ray;
  for (size_t i = 0; i < g->prims.size(); i++) {
    const Prim& p = g->prims[i];
    cur_prim = (int)i;
    Ray o = object_ray(p, ray);
    st.reported = false;
    int gi = 0;
    float2 b = make_float2(0.f);
    switch (p.type) {
      case PRIM_SPHERE: ref_sphere_intersect(p.f, &o, &gi, &b); break;
      case PRIM_RECT: ref_aarect_intersect(p.f, p.axis, p.flip, &o, &gi, &b); break;
      case PRIM_BOX: ref_box_intersect(p.f, &o, &gi, &b); break;
      default: {
        const Mesh& M = g->meshes[p.mesh];
        const int3 vi = M.idx[p.local];
        float t, bu, bv;
        if (watertight(M.v[vi.x], M.v[vi.y], M.v[vi.z], o.origin, o.direction, t, bu, bv) &&
            rtPotentialIntersection(t)) {
          st.prim_index = (unsigned int)p.local;
          st.bary = make_float2(bu, bv);
          bind_mesh(p.mesh);
          ref_triangle_attributes(&gi, &b);
          rtReportIntersection(0);
        }
      }
    }
    if (st.reported) {
      best = (int)i;
      best_gi = gi;
      best_bc = b;
      best_ray = o;
    }
  }
  float t_best = st.tmax;
  if (ray.ray_type == 0) {
    g->ext++;
    if (rec_first && !rec_done) {
      rec_done = true;
      rec_prim = best;
      rec_t = best >= 0 ? t_best : 0.f;
      rec_bc = best_bc;
    }
    if (probe) {
      if (best >= 0) {
        cur_prim = best;
        bind_mesh(g->prims[best].mesh);
        rtemu_hitrecord(best_gi, best_ray, t_best, best_bc, &probe_rec);
      }
    } else if (best < 0) {
      ref_miss(g->miss_kind, g->miss_tex, g->spherical, &ray, payload);
    } else {
      const Prim& p = g->prims[best];
      cur_prim = best;
      bind_mesh(p.mesh);
      call_closest_hit(g->mats[p.material], payload, best_ray, t_best, best_gi, best_bc);
    }
  } else {
    g->shadow++;
    if (best < 0) {
      ref_shadow_miss(payload);
    } else {
      const Prim& p = g->prims[best];
      cur_prim = best;
      ref_any_hit(g->mats[p.material].type == MAT_DIFFUSE_LIGHT, &best_ray, payload);
    }
  }
  ts = saved_ts;
  cur_prim = saved_prim;
  if (saved_mesh >= 0) bind_mesh(saved_mesh);
}

// ------------------------------------------------- callables of the scene --
float3 rtemu_texture(int tex, float u, float v, const float3& p, int i) {
  if (tex < 0) {
    const Texture& t = g->tex[-1 - tex];
    if (t.kind == TEX_CONSTANT) return ref_constant_texture(t.c, u, v, &p, i);
    const Image& im = g->images[t.image];
    return ref_image_texture(im.texels.data(), im.w, im.h, u, v, &p, i);
  }
  const UserTexture& t = g->utex[tex];
  switch (t.kind) {
    case 0: return ref_constant_texture(t.c, u, v, &p, i);
    case 1: return ref_checker_texture(t.a, t.b, u, v, &p, i);
    case 2: return ref_noise_texture(t.c[0], t.a, t.ranvec.data(), t.perm.data(), u, v, &p, i);
    case 3: return ref_image_texture(t.texels.data(), t.a, t.b, u, v, &p, i);
    case 4: return ref_gradient_texture(t.c, u, v, &p, i);
    default: return ref_vector_texture(tex, t.ids.data(), (int)t.ids.size(), u, v, &p, i);
  }
}

void rtemu_hitrecord(int index, const Ray& ray, float t, float2 b, EmuRec* out) {
  const Prim& p = g->prims[cur_prim];
  switch (p.type) {
    case PRIM_SPHERE: ref_sphere_hitrecord(p.f, index, &ray, t, b, out); break;
    case PRIM_RECT: ref_aarect_hitrecord(p.f, p.axis, p.flip, index, &ray, t, b, out); break;
    case PRIM_BOX: ref_box_hitrecord(p.f, index, &ray, t, b, out); break;
    default:
      bind_mesh(p.mesh);
      ref_triangle_hitrecord(index, &ray, t, b, out);
  }
}

int rtemu_num_lights() { return (int)g->lights.size(); }
float3 rtemu_light_emission(int k) { return g->lights[k].emission; }
int rtemu_scene_generation() { return g_generation; }

float3 rtemu_light_sample(int k, const float3& P, const float3& Wo, const float3& N,
                          unsigned int& seed) {
  const Light& L = g->lights[k];
  if (L.type == LIGHT_RECT) return ref_rect_light_sample(L.f, L.axis, &P, &Wo, &N, &seed);
  return ref_sphere_light_sample(L.f, &P, &Wo, &N, &seed);
}

float rtemu_light_pdf(int k, const float3& P, const float3& Wo, const float3& Wi,
                      const float3& N) {
  const Light& L = g->lights[k];
  if (L.type == LIGHT_RECT) return ref_rect_light_pdf(L.f, L.axis, &P, &Wo, &Wi, &N);
  return ref_sphere_light_pdf(L.f, &P, &Wo, &Wi, &N);
}

// ==================================================================== C API ==
namespace {
int add_texture(Scene& s, const float* c) {
  Texture t;
  t.kind = TEX_CONSTANT;
  t.c[0] = c ? c[0] : 0.f;
  t.c[1] = c ? c[1] : 0.f;
  t.c[2] = c ? c[2] : 0.f;
  t.image = -1;
  s.tex.push_back(t);
  return -(int)s.tex.size();
}
int add_xform(Scene& s, const float* x) {
  if (!x) return -1;
  Xform xf;
  memcpy(xf.m, x, sizeof(xf.m));
  affine_inverse(xf.m, xf.inv);
  s.xforms.push_back(xf);
  return (int)s.xforms.size() - 1;
}
float3 unit_vec(const float3& v) { return v / length(v); }  // programs/vec.hpp:40-42
const float kPiF = 3.141592654f;                             // PI_F, programs/common.hpp:17
}  // namespace

extern "C" {

void* rh_create(void) { return new Scene(); }
void rh_destroy(void* s) {
  if (g == (Scene*)s) g = nullptr;
  delete (Scene*)s;
}

// type as the oracle's MAT_*; c0/c1 colours; p0/p1 as the host classes take them.
int rh_add_material(void* sp, int type, const float* c0, const float* c1, float p0, float p1) {
  Scene& s = *(Scene*)sp;
  Material m;
  m.type = type;
  m.tex[0] = add_texture(s, c0);
  m.tex[1] = add_texture(s, c1);
  float q[2];
  ref_convert_params(type, p0, p1, q);
  m.p[0] = q[0];
  m.p[1] = q[1];
  s.mats.push_back(m);
  return (int)s.mats.size() - 1;
}

int rh_add_prim(void* sp, int type, const float* f, int axis, int flip, int material,
                const float* xform) {
  Scene& s = *(Scene*)sp;
  Prim p;
  memset(&p, 0, sizeof(p));
  p.type = type;
  p.axis = axis;
  p.flip = flip;
  p.material = material;
  p.mesh = -1;
  memcpy(p.f, f, sizeof(float) * (type == PRIM_SPHERE ? 4 : (type == PRIM_RECT ? 5 : 6)));
  p.xform = add_xform(s, xform);
  s.prims.push_back(p);
  return (int)s.prims.size() - 1;
}

int rh_add_mesh(void* sp, const float* verts, int nv, const uint32_t* idx, int nt,
                const int32_t* mat_per_tri, int material, const float* normals,
                const float* uvs, const float* xform) {
  Scene& s = *(Scene*)sp;
  Mesh mesh;
  float inv[12];
  if (xform) affine_inverse(xform, inv);
  mesh.v.resize(nv);
  for (int i = 0; i < nv; i++) {
    float3 v = make_float3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
    mesh.v[i] = xform ? xpoint(xform, v) : v;
  }
  if (normals) {
    mesh.n.resize(nv);
    for (int i = 0; i < nv; i++) {
      float3 n = make_float3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
      mesh.n[i] = xform ? xnormal(inv, n) : n;
    }
  }
  if (uvs) {
    mesh.uv.resize(nv);
    for (int i = 0; i < nv; i++) mesh.uv[i] = make_float2(uvs[2 * i], uvs[2 * i + 1]);
  }
  mesh.idx.resize(nt);
  mesh.texidx.assign(nt, 0);  // the faces' texture indices (rh_mesh_set_texture_index)
  for (int t = 0; t < nt; t++)
    mesh.idx[t] = make_int3((int)idx[3 * t], (int)idx[3 * t + 1], (int)idx[3 * t + 2]);
  s.meshes.push_back(std::move(mesh));
  int mid = (int)s.meshes.size() - 1;
  int first = (int)s.prims.size();
  for (int t = 0; t < nt; t++) {
    Prim p;
    memset(&p, 0, sizeof(p));
    p.type = PRIM_TRIANGLE;
    p.material = mat_per_tri ? mat_per_tri[t] : material;
    p.xform = -1;
    p.mesh = mid;
    p.local = t;
    s.prims.push_back(p);
  }
  return first;
}

// The scene's textures, as or_add_texture takes them (kind: 0 constant,
// 1 checker, 2 noise, 3 image, 4 gradient, 5 vector).
int rh_add_texture(void* sp, int kind, int a, int b, const float* c, const float* data,
                   const int32_t* perm, const uint32_t* ids) {
  Scene& s = *(Scene*)sp;
  UserTexture t;
  t.kind = kind;
  t.a = a;
  t.b = b;
  for (int k = 0; k < 9; k++) t.c[k] = c ? c[k] : 0.f;
  if (kind == 3) t.texels.assign(data, data + (size_t)a * b * 4);
  if (kind == 2) {
    t.ranvec.resize(256);
    for (int k = 0; k < 256; k++)
      t.ranvec[k] = make_float3(data[3 * k], data[3 * k + 1], data[3 * k + 2]);
    t.perm.assign(perm, perm + 768);
  }
  if (kind == 5)
    for (int k = 0; k < b; k++) t.ids.push_back((int)ids[k]);
  s.utex.push_back(std::move(t));
  return (int)s.utex.size() - 1;
}

void rh_material_set_texture(void* sp, int material, int slot, int texture) {
  ((Scene*)sp)->mats[material].tex[slot] = texture;
}

void rh_mesh_set_texture_index(void* sp, int first_prim, int n, const uint32_t* index) {
  Scene& s = *(Scene*)sp;
  for (int k = 0; k < n; k++) {
    const Prim& p = s.prims[first_prim + k];
    s.meshes[p.mesh].texidx[p.local] = (int)index[k];
  }
}

// type 0 rect: f = a0,a1,b0,b1,k (axis); 1 sphere: cx,cy,cz,r.
int rh_add_light(void* sp, int type, const float* f, int axis, const float* emission) {
  Scene& s = *(Scene*)sp;
  Light L;
  memset(&L, 0, sizeof(L));
  L.type = type;
  L.axis = axis;
  memcpy(L.f, f, sizeof(float) * (type == LIGHT_RECT ? 5 : 4));
  L.emission = make_float3(emission[0], emission[1], emission[2]);
  s.lights.push_back(L);
  return (int)s.lights.size() - 1;
}

void rh_set_miss(void* sp, int type, const float* c1, const float* c2, const float* env, int w,
                 int h, int spherical) {
  Scene& s = *(Scene*)sp;
  s.miss_kind = type;
  s.spherical = spherical;
  if (type == MISS_GRADIENT) {
    s.miss_tex[0] = add_texture(s, c1);
    s.miss_tex[1] = add_texture(s, c2);
  } else if (type == MISS_CONSTANT) {
    s.miss_tex[0] = add_texture(s, c1);
  } else {
    Image im;
    im.texels.assign(env, env + (size_t)w * h * 4);
    im.w = w;
    im.h = h;
    s.images.push_back(std::move(im));
    Texture t;
    t.kind = TEX_IMAGE;
    t.image = (int)s.images.size() - 1;
    s.tex.push_back(t);
    s.miss_tex[0] = -(int)s.tex.size();
  }
}

// host_includes/camera.hpp:13-38 (the host Camera class), then the context
// variables its set() writes (camera.hpp:40-51).
void rh_set_camera(void* sp, const float* from, const float* at, const float* up, float vfov,
                   float aspect, float aperture, float focus_dist, float t0, float t1) {
  Scene& s = *(Scene*)sp;
  float3 lookfrom = make_float3(from[0], from[1], from[2]);
  float3 lookat = make_float3(at[0], at[1], at[2]);
  float3 vup = make_float3(up[0], up[1], up[2]);
  float lens_radius = aperture / 2.f;
  float theta = vfov * kPiF / 180.f;
  float half_height = pt_tanf(theta / 2.f);
  float half_width = aspect * half_height;
  float3 origin = lookfrom;
  float3 w = unit_vec(lookfrom - lookat);
  float3 u = unit_vec(cross(vup, w));
  float3 v = cross(w, u);
  float3 llc = origin - half_width * focus_dist * u - half_height * focus_dist * v -
               focus_dist * w;
  float3 horizontal = 2.f * half_width * focus_dist * u;
  float3 vertical = 2.f * half_height * focus_dist * v;
  float3 vs[6] = {llc, horizontal, vertical, origin, u, v};
  for (int k = 0; k < 6; k++) {
    s.cam[3 * k] = vs[k].x;
    s.cam[3 * k + 1] = vs[k].y;
    s.cam[3 * k + 2] = vs[k].z;
  }
  s.cam[18] = lens_radius;
  s.cam[19] = t0;
  s.cam[20] = t1;
}

int rh_commit(void* sp) {
  g = nullptr;
  use((Scene*)sp);
  return (int)((Scene*)sp)->prims.size();
}

// params: width, height, spp, frame0, max_depth, rr_enable, rr_depth, mode,
// guide (the oracle's layout).  The reference's raygen starts Russian
// roulette after depth 10 and has no consistent mode: other values -> -1.
int rh_render_paths(void* sp, const int* params, int frame, const uint32_t* pix, int n,
                    float* out_rgb) {
  use((Scene*)sp);
  int W = params[0], H = params[1];
  if (params[6] != 10 || params[7] != 0) return -1;
  std::vector<float4> acc((size_t)W * H, make_float4(0.f));
  std::vector<uchar4> disp((size_t)W * H);
  bound_mesh = -1;
  for (int i = 0; i < n; i++) {
    uint32_t x = pix[i] % W, y = pix[i] / W;
    size_t o = (size_t)(H - 1 - y) * W + x;
    acc[o] = make_float4(0.f);
    ref_render_pixel(x, y, W, H, frame, params[5], params[4], g->cam, acc.data(), disp.data());
    out_rgb[3 * i] = acc[o].x;
    out_rgb[3 * i + 1] = acc[o].y;
    out_rgb[3 * i + 2] = acc[o].z;
  }
  return 0;
}

// First hit of every pixel's camera ray of `frame` (renderPixel's own seed,
// jitter and Camera::generateRay): primitive id (-1 on miss), its material
// (-1), t.
void rh_first_hits(void* sp, int W, int H, int frame, int32_t* prim, int32_t* mat, float* tout) {
  use((Scene*)sp);
  std::vector<float4> acc((size_t)W * H, make_float4(0.f));
  std::vector<uchar4> disp((size_t)W * H);
  bound_mesh = -1;
  for (int p = 0; p < W * H; p++) {
    rec_first = true;
    rec_done = false;
    ref_render_pixel(p % W, p / W, W, H, frame, 1, 1, g->cam, acc.data(), disp.data());
    rec_first = false;
    prim[p] = rec_prim;
    mat[p] = rec_prim >= 0 ? g->prims[rec_prim].material : -1;
    tout[p] = rec_t;
  }
}

// One ray: closest primitive (-1 if none) with t, and its HitRecord as
// P, shading normal, u, v, geometric normal, Wo, index (17 floats).
int rh_probe(void* sp, const float* o, const float* d, float tmin, float* t, float* rec) {
  use((Scene*)sp);
  bound_mesh = -1;
  Ray r = make_Ray(make_float3(o[0], o[1], o[2]), make_float3(d[0], d[1], d[2]), 0, tmin,
                   RT_DEFAULT_MAX);
  probe = true;
  rec_first = true;
  rec_done = false;
  cur_prim = -1;
  rtemu_trace(r, nullptr);
  probe = false;
  rec_first = false;
  *t = rec_t;
  if (rec_prim >= 0 && rec) {
    const EmuRec& e = probe_rec;
    float v[17] = {e.P.x, e.P.y, e.P.z, e.shading_normal.x, e.shading_normal.y,
                   e.shading_normal.z, e.u, e.v, e.geometric_normal.x, e.geometric_normal.y,
                   e.geometric_normal.z, e.Wo.x, e.Wo.y, e.Wo.z, (float)e.index, 0.f, 0.f};
    memcpy(rec, v, sizeof(v));
  }
  return rec_prim;
}

// Bounds program of primitive `prim` (box6 = min xyz, max xyz, object space).
void rh_bounds(void* sp, int prim, float* box6) {
  use((Scene*)sp);
  const Prim& p = g->prims[prim];
  switch (p.type) {
    case PRIM_SPHERE: ref_sphere_bounds(p.f, box6); break;
    case PRIM_RECT: ref_aarect_bounds(p.f, p.axis, box6); break;
    case PRIM_BOX: ref_box_bounds(p.f, box6); break;
    default:
      bound_mesh = -1;
      bind_mesh(p.mesh);
      ref_triangle_bounds(p.local, box6);
  }
}

// The non-RTX software triangle program (programs/hitables/triangle.cu:26-58)
// on one ray against triangle `prim`: 1 and t, barycentrics if it reports.
int rh_triangle_sw(void* sp, int prim, const float* o, const float* d, float tmin, float* out) {
  use((Scene*)sp);
  const Prim& p = g->prims[prim];
  if (p.type != PRIM_TRIANGLE) return -1;
  bound_mesh = -1;
  bind_mesh(p.mesh);
  Ray r = make_Ray(make_float3(o[0], o[1], o[2]), make_float3(d[0], d[1], d[2]), 0, tmin,
                   RT_DEFAULT_MAX);
  TraceState st;
  memset(&st, 0, sizeof(st));
  st.tmin = tmin;
  st.tmax = RT_DEFAULT_MAX;
  TraceState* saved = ts;
  ts = &st;
  int gi = 0;
  float2 b = make_float2(0.f);
  ref_triangle_intersect(p.local, &r, &gi, &b);
  ts = saved;
  if (!st.reported) return 0;
  out[0] = st.tmax;
  out[1] = b.x;
  out[2] = b.y;
  return 1;
}

// Light k: n samples from (P, seed) through its Sample callable and the pdf
// of each sampled direction through its PDF callable (N and Wo unused by
// both programs, passed as zero).
void rh_light(void* sp, int k, int n, const float* P, uint32_t* seeds, float* Wi, float* pdf) {
  use((Scene*)sp);
  float3 zero = make_float3(0.f);
  for (int i = 0; i < n; i++) {
    float3 p = make_float3(P[3 * i], P[3 * i + 1], P[3 * i + 2]);
    unsigned int s = seeds[i];
    float3 w = rtemu_light_sample(k, p, zero, zero, s);
    seeds[i] = s;
    Wi[3 * i] = w.x;
    Wi[3 * i + 1] = w.y;
    Wi[3 * i + 2] = w.z;
    pdf[i] = rtemu_light_pdf(k, p, zero, w, zero);
  }
}

void rh_stats(void* sp, uint64_t* out) {
  Scene& s = *(Scene*)sp;
  out[0] = s.ext;
  out[1] = s.shadow;
}

}  // extern "C"

// The moving sphere of programs/hitables/moving_sphere.cu (f = centre at
// time0 (3), radius, time0, time1, centre at time1 (3)) against one ray at
// `time`: 1 and out = t, P (3), shading normal (3), u, v, Wo (3) if it
// reports a hit; box6 = its get_bounds box.
extern "C" int rh_msphere(const float* f, const float* o, const float* d, float tmin, float tmax,
                          float time, float* out, float* box6) {
  ref_msphere_bounds(f, box6);
  Ray r = make_Ray(make_float3(o[0], o[1], o[2]), make_float3(d[0], d[1], d[2]), 0, tmin, tmax);
  TraceState st;
  memset(&st, 0, sizeof(st));
  st.tmin = tmin;
  st.tmax = tmax;
  TraceState* saved = ts;
  int saved_prim = cur_prim;
  ts = &st;
  cur_prim = -1;
  float rec[11];
  ref_msphere_intersect(f, &r, time, rec);
  ts = saved;
  cur_prim = saved_prim;
  if (!st.reported) return 0;
  out[0] = st.tmax;
  for (int k = 0; k < 11; k++) out[1 + k] = rec[k];
  return 1;
}
