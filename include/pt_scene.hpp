/*
 * pt_scene.hpp - the reference's host scene-construction API, re-created over
 * the C ABI of pt.h (header only, C++14).
 *
 * Class and function names follow joaovbs96/OptiX-Path-Tracer's
 * host_includes/ so that scene code written against them (scenes.hpp) ports
 * by changing includes: Constant_Texture, Checker_Texture, Noise_Texture,
 * Image_Texture / HDR_Texture, Gradient_Texture, Vector_Texture (textures.hpp),
 * Lambertian, Metal, Dielectric, Diffuse_Light, Oren_Nayar, Torrance_Sparrow,
 * Ashikhmin_Shirley (materials.hpp), Sphere, Moving_Sphere, AARect, Box, Mesh, Hitable_List
 * (hitables.hpp, mesh.hpp), Camera (camera.hpp), Rectangle_PDF, Sphere_PDF,
 * Light_Sampler (pdfs.hpp, host_common.hpp), setRayGenerationProgram,
 * setMissProgram, setExceptionProgram (programs.hpp).  The OptiX objects
 * (Context, Group, Program) become a thin Context over pt_context; errors are
 * thrown as pt::Error (the reference throws strings, host_common.hpp:53).
 * File loading (stb_image, tinyobjloader, HDRloader) is not part of this
 * library: meshes and environment maps are passed as arrays.
 */
#ifndef PT_SCENE_HPP
#define PT_SCENE_HPP

#include <algorithm>
#include <cmath>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "pt.h"

namespace pt {

struct float3v {
  float x, y, z;
};
inline float3v make_float3(float x, float y, float z) { return float3v{x, y, z}; }
inline float3v make_float3(float s) { return float3v{s, s, s}; }

typedef enum { X_AXIS = PT_X_AXIS, Y_AXIS = PT_Y_AXIS, Z_AXIS = PT_Z_AXIS } AXIS;
typedef enum { GRADIENT = 0, CONSTANT = 1, IMG = 3, HDR = 2 } Miss_Programs;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ------------------------------------------------------------------ Context
class ContextObj {
 public:
  explicit ContextObj(int device = 0, int path_slots = 0) {
    pt_options o{};
    o.device = device;
    o.path_slots = path_slots;
    check(pt_context_create(&o, &ctx_), "pt_context_create");
  }
  ~ContextObj() {
    if (ctx_) pt_context_destroy(ctx_);
  }
  ContextObj(const ContextObj&) = delete;
  ContextObj& operator=(const ContextObj&) = delete;
  pt_context* get() const { return ctx_; }
  void check(int rc, const char* what) const {
    if (rc != PT_OK)
      throw Error(rc, std::string(what) + ": " + (ctx_ ? pt_last_error(ctx_) : "no context"));
  }
  // context variables of main.cpp:61-63
  int samples = 500, russian = 1, maxDepth = 50, russianDepth = 10;
  bool dirty = true;
  void commit() {
    if (dirty) check(pt_commit(ctx_), "pt_commit");
    dirty = false;
  }

 private:
  pt_context* ctx_ = nullptr;
};

// optix::Context is a reference-counted handle; so is this.
class Context {
 public:
  Context() = default;
  static Context create(int device = 0, int path_slots = 0) {
    Context c;
    c.p_ = std::make_shared<ContextObj>(device, path_slots);
    return c;
  }
  ContextObj* operator->() const { return p_.get(); }
  pt_context* get() const { return p_->get(); }
  explicit operator bool() const { return (bool)p_; }

 private:
  std::shared_ptr<ContextObj> p_;
};

struct Group {};  // the top-level OptiX Group; here all primitives share one BVH8

// ----------------------------------------------------------------- textures
// host_includes/host_common.hpp:59-63: the host's random numbers (scene
// generators and the Perlin tables draw from this one stream).
inline float rnd() {
  static std::mt19937 gen(0);
  static std::uniform_real_distribution<float> dis(0.f, 1.f);
  return dis(gen);
}

// host_includes/textures.hpp: a texture registers itself in a context once
// (assignTo returns its texture id there, as the reference's returns its
// callable program).
struct Texture {
  virtual ~Texture() = default;
  uint32_t assignTo(Context& ctx) const {
    if (ctx_ != ctx.get()) {
      id_ = create(ctx);
      ctx_ = ctx.get();
      ctx->dirty = true;
    }
    return id_;
  }
  // the colour of a constant texture (a material then needs no texture)
  virtual bool constant(float3v* c) const {
    (void)c;
    return false;
  }

 protected:
  virtual uint32_t create(Context& ctx) const = 0;
  static const float* f3(const float3v& v) { return &v.x; }
  mutable pt_context* ctx_ = nullptr;
  mutable uint32_t id_ = 0;
};

struct Constant_Texture : public Texture {  // textures.hpp:19-37
  explicit Constant_Texture(const float3v& c) : c_(c) {}
  explicit Constant_Texture(float rgb) : c_(make_float3(rgb)) {}
  Constant_Texture(float r, float g, float b) : c_(make_float3(r, g, b)) {}
  bool constant(float3v* c) const override {
    *c = c_;
    return true;
  }
  float3v c_;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_texture_constant(c.get(), f3(c_), &id), "Constant_Texture");
    return id;
  }
};

struct Checker_Texture : public Texture {  // textures.hpp:39-54
  Checker_Texture(const Texture* o, const Texture* e) : odd(o), even(e) {}
  const Texture *odd, *even;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t o = odd->assignTo(c), e = even->assignTo(c), id;
    c->check(pt_texture_checker(c.get(), o, e, &id), "Checker_Texture");
    return id;
  }
};

struct Noise_Texture : public Texture {  // textures.hpp:56-112
  Noise_Texture(float s, AXIS ax = X_AXIS) : scale(s), ax(ax) {}
  const float scale;
  const AXIS ax;

 protected:
  static float3v unit_float3(float x, float y, float z) {
    float l = std::sqrt(x * x + y * y + z * z);
    return make_float3(x / l, y / l, z / l);
  }
  static void permute(int32_t* p) {
    for (int i = 256 - 1; i > 0; i--) {
      int target = int(rnd() * (i + 1));
      int32_t tmp = p[i];
      p[i] = p[target];
      p[target] = tmp;
    }
  }
  // the tables as the host class makes them, from the shared rnd() stream
  uint32_t create(Context& c) const override {
    std::vector<float> ranvec(768);
    std::vector<int32_t> perm(768);
    for (int i = 0; i < 256; ++i) {
      float3v v = unit_float3(-1 + 2 * rnd(), -1 + 2 * rnd(), -1 + 2 * rnd());
      ranvec[3 * i] = v.x;
      ranvec[3 * i + 1] = v.y;
      ranvec[3 * i + 2] = v.z;
    }
    for (int a = 0; a < 3; a++) {
      for (int i = 0; i < 256; i++) perm[256 * a + i] = i;
      permute(perm.data() + 256 * a);
    }
    uint32_t id;
    c->check(pt_texture_noise(c.get(), scale, (int)ax, ranvec.data(), perm.data(), &id),
             "Noise_Texture");
    return id;
  }
};

// Image_Texture / HDR_Texture after loading: RGBA float texels, row 0 at
// v = 0 (textures.hpp:114-230; the loaders flip the file's rows and
// normalise 8-bit texels to [0, 1]).  HDR_Texture also serves as the
// environment map of setMissProgram.
struct HDR_Texture : public Texture {
  HDR_Texture(const float* rgba, int w, int h) : rgba(rgba, rgba + (size_t)w * h * 4), w(w), h(h) {}
  std::vector<float> rgba;
  int w, h;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_texture_image(c.get(), rgba.data(), w, h, &id), "Image_Texture");
    return id;
  }
};
typedef HDR_Texture Image_Texture;

struct Gradient_Texture : public Texture {  // textures.hpp:233-251
  Gradient_Texture(const float3v& a, const float3v& b, const float3v& cc)
      : colorA(a), colorB(b), colorC(cc) {}
  const float3v colorA, colorB, colorC;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_texture_gradient(c.get(), f3(colorA), f3(colorB), f3(colorC), &id),
             "Gradient_Texture");
    return id;
  }
};

struct Vector_Texture : public Texture {  // textures.hpp:253-271
  explicit Vector_Texture(const std::vector<Texture*>& tv) : texture_vector(tv) {}
  const std::vector<Texture*> texture_vector;

 protected:
  uint32_t create(Context& c) const override {
    std::vector<uint32_t> ids;
    for (const Texture* t : texture_vector) ids.push_back(t->assignTo(c));
    uint32_t id;
    c->check(pt_texture_vector(c.get(), ids.data(), (int)ids.size(), &id), "Vector_Texture");
    return id;
  }
};

// ---------------------------------------------------------------- materials
struct BRDF {
  virtual ~BRDF() = default;
  // Registers the material once per context and returns its id.
  uint32_t assignTo(Context& ctx) const {
    if (ctx_ != ctx.get()) {
      id_ = create(ctx);
      ctx_ = ctx.get();
      ctx->dirty = true;
    }
    return id_;
  }

 protected:
  virtual uint32_t create(Context& ctx) const = 0;
  static const float* f3(const float3v& v) { return &v.x; }
  // a texture's constant colour, or black where the material takes the
  // texture itself (bind() then names it)
  static float3v colour(const Texture* t) {
    float3v c = make_float3(0.f);
    t->constant(&c);
    return c;
  }
  static void bind(Context& c, uint32_t id, int slot, const Texture* t) {
    float3v unused;
    if (!t->constant(&unused))
      c->check(pt_material_set_texture(c.get(), id, slot, t->assignTo(c)), "texture");
  }
  mutable pt_context* ctx_ = nullptr;
  mutable uint32_t id_ = 0;
};

struct Lambertian : public BRDF {
  explicit Lambertian(const Texture* t) : texture(t) {}
  const Texture* texture;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_material_lambertian(c.get(), f3(colour(texture)), &id), "Lambertian");
    bind(c, id, 0, texture);
    return id;
  }
};

struct Metal : public BRDF {
  Metal(const Texture* t, float fuzz) : texture(t), fuzz(fuzz) {}
  const Texture* texture;
  const float fuzz;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_material_metal(c.get(), f3(colour(texture)), fuzz, &id), "Metal");
    bind(c, id, 0, texture);
    return id;
  }
};

struct Dielectric : public BRDF {
  Dielectric(const Texture* base, const Texture* ext, float ref_idx, float density = 0.f)
      : baseTex(base), extTex(ext), ref_idx(ref_idx), density(density) {}
  const Texture *baseTex, *extTex;
  const float ref_idx, density;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_material_dielectric(c.get(), f3(colour(baseTex)), f3(colour(extTex)), ref_idx,
                                    density, &id),
             "Dielectric");
    bind(c, id, 0, baseTex);
    bind(c, id, 1, extTex);
    return id;
  }
};

struct Diffuse_Light : public BRDF {
  explicit Diffuse_Light(const Texture* t) : texture(t) {}
  const Texture* texture;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_material_diffuse_light(c.get(), f3(colour(texture)), &id), "Diffuse_Light");
    bind(c, id, 0, texture);
    return id;
  }
};

struct Oren_Nayar : public BRDF {
  Oren_Nayar(const Texture* t, float R) : texture(t), R(R) {}
  const Texture* texture;
  const float R;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_material_oren_nayar(c.get(), f3(colour(texture)), R, &id), "Oren_Nayar");
    bind(c, id, 0, texture);
    return id;
  }
};

struct Torrance_Sparrow : public BRDF {
  Torrance_Sparrow(const Texture* t, float nu, float nv) : texture(t), nu(nu), nv(nv) {}
  const Texture* texture;
  const float nu, nv;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_material_torrance_sparrow(c.get(), f3(colour(texture)), nu, nv, &id),
             "Torrance_Sparrow");
    bind(c, id, 0, texture);
    return id;
  }
};

struct Ashikhmin_Shirley : public BRDF {
  Ashikhmin_Shirley(const Texture* d, const Texture* s, float nu, float nv)
      : diffuse_tex(d), specular_tex(s), nu(nu), nv(nv) {}
  const Texture *diffuse_tex, *specular_tex;
  const float nu, nv;

 protected:
  uint32_t create(Context& c) const override {
    uint32_t id;
    c->check(pt_material_ashikhmin_shirley(c.get(), f3(colour(diffuse_tex)),
                                           f3(colour(specular_tex)), nu, nv, &id),
             "Ashikhmin_Shirley");
    bind(c, id, 0, diffuse_tex);
    bind(c, id, 1, specular_tex);
    return id;
  }
};

// --------------------------------------------------------------- transforms
typedef enum { Rotate_Transform, Translate_Transform, Scale_Transform } Transform_Type;

struct TransformParameter {  // host_includes/transforms.hpp:36-44
  TransformParameter(Transform_Type t, float a, AXIS ax, float3v s, float3v p)
      : type(t), angle(a), axis(ax), scale(s), pos(p) {}
  Transform_Type type;
  float angle;
  AXIS axis;
  float3v scale, pos;
};

// 4x4 (row major, double) of one transform step: right-handed rotation of
// `angle` degrees about an axis, translation, axis-aligned scale.
inline void transform_matrix(const TransformParameter& t, double m[16]) {
  for (int i = 0; i < 16; i++) m[i] = (i % 5 == 0) ? 1.0 : 0.0;
  if (t.type == Translate_Transform) {
    m[3] = t.pos.x;
    m[7] = t.pos.y;
    m[11] = t.pos.z;
  } else if (t.type == Scale_Transform) {
    m[0] = t.scale.x;
    m[5] = t.scale.y;
    m[10] = t.scale.z;
  } else {
    double a = t.angle * 3.14159265358979323846 / 180.0, c = std::cos(a), s = std::sin(a);
    int i = (t.axis == X_AXIS) ? 1 : (t.axis == Y_AXIS ? 2 : 0);
    int j = (t.axis == X_AXIS) ? 2 : (t.axis == Y_AXIS ? 0 : 1);
    m[i * 4 + i] = c;
    m[i * 4 + j] = -s;
    m[j * 4 + i] = s;
    m[j * 4 + j] = c;
  }
}

// World matrix of a transform list applied outermost-first (the list's first
// entry is the outermost transform): returns false for an empty list.
inline bool compose(const std::vector<TransformParameter>& ts, float out[12]) {
  if (ts.empty()) return false;
  double m[16];
  for (int i = 0; i < 16; i++) m[i] = (i % 5 == 0) ? 1.0 : 0.0;
  for (const auto& t : ts) {
    double s[16], r[16];
    transform_matrix(t, s);
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) {
        double acc = 0;
        for (int k = 0; k < 4; k++) acc += m[i * 4 + k] * s[k * 4 + j];
        r[i * 4 + j] = acc;
      }
    std::copy(r, r + 16, m);
  }
  for (int i = 0; i < 12; i++) out[i] = (float)m[i];
  return true;
}

// ---------------------------------------------------------------- hitables
class Hitable {
 public:
  explicit Hitable(BRDF* material) : material(material) {}
  virtual ~Hitable() = default;
  std::vector<TransformParameter> transforms;
  virtual void rotate(float angle, AXIS axis) {
    transforms.emplace_back(Rotate_Transform, angle, axis, make_float3(0.f), make_float3(0.f));
  }
  virtual void scale(float3v s) {
    transforms.emplace_back(Scale_Transform, 0.f, X_AXIS, s, make_float3(0.f));
  }
  virtual void translate(float3v p) {
    transforms.emplace_back(Translate_Transform, 0.f, X_AXIS, make_float3(0.f), p);
  }
  // Hitable::addTo reverses the list: the first call is innermost
  // (host_includes/hitables.hpp:61-70).
  virtual void addTo(Group&, Context& ctx) {
    std::vector<TransformParameter> r(transforms.rbegin(), transforms.rend());
    add(ctx, r);
  }
  // Adds the primitive with `ts` applied outermost-first.
  virtual void add(Context& ctx, const std::vector<TransformParameter>& ts) = 0;

 protected:
  BRDF* material;
};

class Sphere : public Hitable {
 public:
  Sphere(const float3v& c, float r, BRDF* m) : Hitable(m), center(c), radius(r) {}
  void add(Context& ctx, const std::vector<TransformParameter>& ts) override {
    float x[12];
    bool has = compose(ts, x);
    uint32_t mid = material->assignTo(ctx);
    ctx->check(pt_add_sphere(ctx.get(), &center.x, radius, mid, has ? x : nullptr, nullptr),
               "Sphere");
    ctx->dirty = true;
  }
  const float3v center;
  const float radius;
};

// Moving_Sphere(center0, center1, radius, time0, time1, material): the
// sphere's centre moves linearly from center0 at time0 to center1 at time1
// over each path's time (the Camera's time0..time1).
class Moving_Sphere : public Hitable {
 public:
  Moving_Sphere(const float3v& c0, const float3v& c1, float r, float t0, float t1, BRDF* m)
      : Hitable(m), center0(c0), center1(c1), radius(r), time0(t0), time1(t1) {}
  void add(Context& ctx, const std::vector<TransformParameter>& ts) override {
    float x[12];
    bool has = compose(ts, x);
    uint32_t mid = material->assignTo(ctx);
    ctx->check(pt_add_moving_sphere(ctx.get(), &center0.x, &center1.x, radius, time0, time1, mid,
                                    has ? x : nullptr, nullptr),
               "Moving_Sphere");
    ctx->dirty = true;
  }
  const float3v center0, center1;
  const float radius, time0, time1;
};

class AARect : public Hitable {
 public:
  AARect(float a0, float a1, float b0, float b1, float k, bool flip, AXIS ax, BRDF* m)
      : Hitable(m), a0(a0), a1(a1), b0(b0), b1(b1), k(k), axis(ax), flip(flip) {}
  void add(Context& ctx, const std::vector<TransformParameter>& ts) override {
    float x[12];
    bool has = compose(ts, x);
    uint32_t mid = material->assignTo(ctx);
    ctx->check(pt_add_rect(ctx.get(), a0, a1, b0, b1, k, flip ? 1 : 0, (int)axis, mid,
                           has ? x : nullptr, nullptr),
               "AARect");
    ctx->dirty = true;
  }
  const float a0, a1, b0, b1, k;
  const AXIS axis;
  const bool flip;
};

class Box : public Hitable {
 public:
  Box(const float3v& p0, const float3v& p1, BRDF* m) : Hitable(m), p0(p0), p1(p1) {}
  void add(Context& ctx, const std::vector<TransformParameter>& ts) override {
    float x[12];
    bool has = compose(ts, x);
    uint32_t mid = material->assignTo(ctx);
    ctx->check(pt_add_box(ctx.get(), &p0.x, &p1.x, mid, has ? x : nullptr, nullptr), "Box");
    ctx->dirty = true;
  }
  const float3v p0, p1;
};

// Mesh(file, folder, BRDF*) after loading: indexed triangles, optional
// per-vertex normals/uvs, optional per-triangle materials (mesh.hpp:49-204).
class Mesh : public Hitable {
 public:
  Mesh(std::vector<float> verts, std::vector<uint32_t> idx, BRDF* m,
       std::vector<float> normals = {}, std::vector<float> uvs = {},
       std::vector<BRDF*> tri_materials = {})
      : Hitable(m), verts(std::move(verts)), idx(std::move(idx)), normals(std::move(normals)),
        uvs(std::move(uvs)), tri_materials(std::move(tri_materials)) {}
  // Mesh(fileName[, assetsFolder][, givenMaterial], RTX) (mesh.hpp:22-45): an
  // OBJ file read by pt_obj_load; without a material, one Lambertian per MTL
  // material (its ambient colour).  The RTX flag has no meaning here.
  Mesh(std::string fileName, bool /*RTX*/ = false) : Hitable(nullptr), file(std::move(fileName)) {}
  Mesh(std::string fileName, std::string assetsFolder, bool /*RTX*/ = false)
      : Hitable(nullptr), file(std::move(fileName)), folder(std::move(assetsFolder)) {}
  Mesh(std::string fileName, BRDF* givenMaterial, bool /*RTX*/ = false)
      : Hitable(givenMaterial), file(std::move(fileName)) {}
  Mesh(std::string fileName, std::string assetsFolder, BRDF* givenMaterial, bool /*RTX*/ = false)
      : Hitable(givenMaterial), file(std::move(fileName)), folder(std::move(assetsFolder)) {}
  void add(Context& ctx, const std::vector<TransformParameter>& ts) override {
    float x[12];
    bool has = compose(ts, x);
    if (!file.empty()) {
      pt_obj* obj = nullptr;
      if (pt_obj_load((folder + file).c_str(), &obj) != PT_OK)
        throw Error(PT_EINVAL, std::string("Mesh: ") + pt_io_last_error());
      uint32_t mid = material ? material->assignTo(ctx) : PT_OBJ_MTL;
      int rc = pt_add_obj(ctx.get(), obj, mid, has ? x : nullptr, nullptr);
      pt_obj_free(obj);
      ctx->check(rc, "Mesh");
      ctx->dirty = true;
      return;
    }
    std::vector<uint32_t> mpt;
    for (BRDF* b : tri_materials) mpt.push_back(b->assignTo(ctx));
    uint32_t mid = material ? material->assignTo(ctx) : 0;
    ctx->check(pt_add_mesh(ctx.get(), verts.data(), verts.size() / 3, idx.data(), idx.size() / 3,
                           mpt.empty() ? nullptr : mpt.data(), mid,
                           normals.empty() ? nullptr : normals.data(),
                           uvs.empty() ? nullptr : uvs.data(), has ? x : nullptr, nullptr),
               "Mesh");
    ctx->dirty = true;
  }
  std::vector<float> verts;
  std::vector<uint32_t> idx;
  std::vector<float> normals, uvs;
  std::vector<BRDF*> tri_materials;
  std::string file, folder;
};

class Hitable_List {  // host_includes/hitables.hpp:455-528
 public:
  int push(Hitable* h) {
    list.push_back(h);
    return (int)list.size() - 1;
  }
  void rotate(float angle, AXIS axis) {
    transforms.emplace_back(Rotate_Transform, angle, axis, make_float3(0.f), make_float3(0.f));
  }
  void scale(float3v s) { transforms.emplace_back(Scale_Transform, 0.f, X_AXIS, s, make_float3(0.f)); }
  void translate(float3v p) {
    transforms.emplace_back(Translate_Transform, 0.f, X_AXIS, make_float3(0.f), p);
  }
  // each element with its own transforms; the last call is innermost
  void addElementsTo(Group&, Context& ctx) {
    for (Hitable* h : list) h->add(ctx, h->transforms);
  }
  // the whole list as one group under the list's transforms (last call
  // innermost); like getGroup (hitables.hpp:497-505) it ignores the
  // elements' own transforms
  void addListTo(Group&, Context& ctx) {
    for (Hitable* h : list) h->add(ctx, transforms);
  }
  std::vector<Hitable*> list;
  std::vector<TransformParameter> transforms;
};

// ------------------------------------------------------------------- camera
class Camera {  // host_includes/camera.hpp:9-61
 public:
  Camera(const float3v& lookfrom, const float3v& lookat, const float3v& vup, float vfov,
         float aspect, float aperture, float focus_dist, float t0, float t1)
      : from(lookfrom), at(lookat), up(vup), vfov(vfov), aspect(aspect), aperture(aperture),
        focus(focus_dist), t0(t0), t1(t1) {}
  void set(Context& ctx) {
    ctx->check(pt_set_camera(ctx.get(), &from.x, &at.x, &up.x, vfov, aspect, aperture, focus, t0,
                             t1),
               "Camera::set");
    ctx->dirty = true;
  }
  float3v from, at, up;
  float vfov, aspect, aperture, focus, t0, t1;
};

// ------------------------------------------------------------------- lights
struct LightShape {
  int type;  // 0 rect, 1 sphere
  float a0, a1, b0, b1, k;
  AXIS axis;
  float3v c;
  float r;
};

struct PDF {
  virtual ~PDF() = default;
  virtual LightShape createSample(Context&) const = 0;
  virtual LightShape createPDF(Context&) const = 0;
};

struct Rectangle_PDF : public PDF {  // host_includes/pdfs.hpp:17-80
  Rectangle_PDF(float a0, float a1, float b0, float b1, float k, AXIS ax)
      : a0(a0), a1(a1), b0(b0), b1(b1), k(k), ax(ax) {}
  LightShape createSample(Context&) const override { return shape(); }
  LightShape createPDF(Context&) const override { return shape(); }
  LightShape shape() const { return LightShape{0, a0, a1, b0, b1, k, ax, make_float3(0.f), 0.f}; }
  float a0, a1, b0, b1, k;
  AXIS ax;
};

struct Sphere_PDF : public PDF {  // host_includes/pdfs.hpp:82-109
  Sphere_PDF(const float3v& c, float r) : center(c), radius(r) {}
  LightShape createSample(Context&) const override { return shape(); }
  LightShape createPDF(Context&) const override { return shape(); }
  LightShape shape() const { return LightShape{1, 0, 0, 0, 0, 0, X_AXIS, center, radius}; }
  float3v center;
  float radius;
};

struct Light_Sampler {  // host_includes/host_common.hpp:65-68
  std::vector<LightShape> sample, pdf;
  std::vector<float3v> emissions;
};

// programs.hpp:17-30: the light buffers; numLights = emissions.size()
inline void setRayGenerationProgram(Context& ctx, Light_Sampler& lights) {
  for (size_t i = 0; i < lights.emissions.size(); i++) {
    const LightShape& s = lights.sample[i];
    const float3v& e = lights.emissions[i];
    if (s.type == 0)
      ctx->check(pt_add_light_rect(ctx.get(), s.a0, s.a1, s.b0, s.b1, s.k, (int)s.axis, &e.x),
                 "light");
    else
      ctx->check(pt_add_light_sphere(ctx.get(), &s.c.x, s.r, &e.x), "light");
  }
  ctx->dirty = true;
}

// programs.hpp:207-235
inline void setMissProgram(Context& ctx, Miss_Programs id, float3v c1 = make_float3(0.f),
                           float3v c2 = make_float3(0.f)) {
  if (id == GRADIENT)
    ctx->check(pt_set_env_gradient(ctx.get(), &c1.x, &c2.x), "setMissProgram");
  else if (id == CONSTANT)
    ctx->check(pt_set_env_constant(ctx.get(), &c1.x), "setMissProgram");
  else
    throw Error(PT_EINVAL, "Parameters invalid, miss program unknown or not yet implemented");
  ctx->dirty = true;
}

// programs.hpp:177-205, with the image already loaded
inline void setMissProgram(Context& ctx, Miss_Programs id, const HDR_Texture& img,
                           bool isSpherical = true) {
  if (id != HDR && id != IMG) throw Error(PT_EINVAL, "miss program needs HDR or IMG");
  ctx->check(pt_set_env_map(ctx.get(), (int)id, img.rgba.data(), img.w, img.h, isSpherical ? 1 : 0),
             "setMissProgram");
  ctx->dirty = true;
}

inline void setExceptionProgram(Context&) {}  // device errors are status codes here

// main.cpp:26-39 renderFrame + the per-sample loop main.cpp:264: renders
// frames [frame, frame + spp) into acc (W*H float4, host or device).
inline void renderFrame(Context& ctx, int W, int H, int frame, int spp, float* acc) {
  ctx->commit();
  pt_render_params p{};
  p.width = W;
  p.height = H;
  p.spp = spp;
  p.frame0 = frame;
  p.max_depth = ctx->maxDepth;
  p.rr_enable = ctx->russian;
  p.rr_depth = ctx->russianDepth;
  p.mode = PT_MODE_REF;
  ctx->check(pt_render(ctx.get(), &p, acc, nullptr), "renderFrame");
}

// programs/raygen.cu:136-146 display conversion (RGBA8)
inline std::vector<uint8_t> resolveDisplay(Context& ctx, const float* acc, int W, int H,
                                           int frame) {
  std::vector<uint8_t> out((size_t)W * H * 4);
  ctx->check(pt_resolve_display(ctx.get(), acc, W, H, frame, out.data(), nullptr),
             "resolveDisplay");
  return out;
}

// Save_PNG / Save_HDR (image_save.hpp:7-73) of an accumulation buffer of
// w*h RGBA float sums over spp frames; ".png" / ".hdr" is appended to the
// name as the reference does.
inline void Save_PNG(const std::string& fileName, int w, int h, const std::vector<float>& acc,
                     int spp) {
  if (acc.size() < (size_t)w * h * 4) throw Error(PT_EINVAL, "Save_PNG: buffer too small");
  if (pt_png_save((fileName + ".png").c_str(), w, h, acc.data(), spp) != PT_OK)
    throw Error(PT_EINVAL, std::string("Save_PNG: ") + pt_io_last_error());
}
inline void Save_HDR(const std::string& fileName, int w, int h, const std::vector<float>& acc,
                     int spp) {
  if (acc.size() < (size_t)w * h * 4) throw Error(PT_EINVAL, "Save_HDR: buffer too small");
  if (pt_hdr_save((fileName + ".hdr").c_str(), w, h, acc.data(), spp) != PT_OK)
    throw Error(PT_EINVAL, std::string("Save_HDR: ") + pt_io_last_error());
}

}  // namespace pt

#endif  // PT_SCENE_HPP
