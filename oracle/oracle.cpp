/*
 * oracle.cpp - CPU restatement of the reference path tracer's device programs.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * path tracer in optix-path-tracer_gb300/: tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg are the only code that may load it.  The
 * product never links or calls it.
 *
 * It transcribes, statement by statement and in the reference's evaluation
 * order, the OptiX programs of joaovbs96/OptiX-Path-Tracer:
 *   programs/random.cuh:33-65       tea<N>, lcg, rnd
 *   programs/sampling.cuh:22-59     random_in_unit_disk/_sphere, on_unit_sphere
 *   programs/raygen.cu:50-167       Camera::generateRay, color(), de_nan,
 *                                   renderPixel
 *   programs/miss.cu:30-95          gradient / constant / image / env miss
 *   programs/hit.cu:16-24           shadow any-hit (closest-hit occlusion here)
 *   programs/hitables/sphere.cu     hit_sphere, Get_HitRecord, get_bounds
 *   programs/hitables/aarect.cu     Hit_X/Y/Z, Hit_Rect, Get_HitRecord
 *   programs/hitables/box.cu        Intersect, boxnormal, Get_HitRecord
 *   programs/hitables/triangle.cu   Get_HitRecord (intersection: watertight,
 *                                   the RTX-mode hardware test of mesh.hpp:176)
 *   programs/materials/{lambertian,...}.cu[h] the BRDFs and Direct_Light
 *   programs/pdfs/{rect,sphere}_pdf.cu    rect / sphere light sample + pdf
 *   host_includes/camera.hpp:13-38, materials.hpp:173-174,194-197,235-238
 * OptiX SDK 6.0.0 helpers that the reference uses but does not vendor are
 * replaced by published methods, identically on CPU and GPU:
 *   Onb                      -> Duff et al. 2017, "Building an Orthonormal
 *                               Basis, Revisited"
 *   cosine_sample_hemisphere -> Malley's method over the Shirley-Chiu (1997)
 *                               concentric square-to-disk map
 *   normalize/length/reflect/clamp/cross/dot -> their textbook definitions
 *   Trbvh + rtTrace          -> binned-SAH BVH2 + closest-hit traversal
 * Conventions fixed here and mirrored by the GPU kernels:
 *   - several rnd() arguments in one call are drawn left to right;
 *   - closest hit is the lexicographic minimum of (t, primitive id);
 *   - each primitive proposes one candidate t independent of the current
 *     closest t (sphere: near root if > tmin else far root; box: entry if >
 *     tmin else exit), so the result does not depend on traversal order;
 *   - shadow rays report the closest hit in (1e-3, tmax); the point is
 *     unoccluded iff that hit is a diffuse light and dot(N, Wi) > 0;
 *   - a HitRecord is computed from the object-space ray and mapped to world
 *     space once, as the reference's HitRecord programs do with the ray
 *     OptiX gives them; Wo is taken from the world-space ray (the
 *     reference's comes from the object-space one);
 *   - a pdf the reference leaves uninitialised starts at 0.
 * Arithmetic: compiled with -ffp-contract=off, elementary functions from
 * ptmath.h, so every float operation rounds exactly as on the GPU.
 *
 * Pinned: oracle/refhost compiles the reference's programs/ unmodified over
 * an OptiX stand-in (oracle/_ref/libref.so), and tests/test_ref_pin.py finds
 * this restatement bit-identical to them, function by function and path by
 * path.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include <vector>
#include <algorithm>
#include <atomic>
#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../optix-path-tracer_gb300/csrc/ptmath.h"

namespace {

// ---------------------------------------------------------------- vectors --
struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 v3(float s) { return V3{s, s, s}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
inline V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
inline V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
inline V3& operator*=(V3& a, V3 b) { a = a * b; return a; }
inline V3& operator*=(V3& a, float s) { a = a * s; return a; }
inline V3& operator/=(V3& a, float s) { a = a / s; return a; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(V3 a) { return ptm_sqrt(dot(a, a)); }
inline V3 normalize(V3 a) {
  float inv = 1.0f / ptm_sqrt(dot(a, a));
  return a * inv;
}
inline float clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
inline V3 clamp3(V3 v, float a, float b) {
  return v3(clampf(v.x, a, b), clampf(v.y, a, b), clampf(v.z, a, b));
}
inline V3 reflect(V3 i, V3 n) { return i - (2.0f * n) * dot(n, i); }
// programs/vec.hpp:21-84
inline float squared_length(V3 a) { return length(a) * length(a); }
inline bool isNull(V3 a) { return (a.x == 0.f) && (a.y == 0.f) && (a.z == 0.f); }
inline V3 unit_vector(V3 v) { return v / length(v); }
inline float ffmin(float a, float b) { return a < b ? a : b; }
inline float ffmax(float a, float b) { return a > b ? a : b; }
inline V3 min_vec(V3 a, V3 b) { return v3(ffmin(a.x, b.x), ffmin(a.y, b.y), ffmin(a.z, b.z)); }
inline V3 max_vec(V3 a, V3 b) { return v3(ffmax(a.x, b.x), ffmax(a.y, b.y), ffmax(a.z, b.z)); }
inline float max_component(V3 a) { return ffmax(ffmax(a.x, a.y), a.z); }
inline float min_component(V3 a) { return ffmin(ffmin(a.x, a.y), a.z); }
inline float get(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

const float PI_F = 3.141592654f;  // programs/common.hpp:19
const float RAY_TMAX = 1e27f;

// -------------------------------------------------------------------- RNG --
// programs/random.cuh:33-65
inline uint32_t tea64(uint32_t val0, uint32_t val1) {
  uint32_t v0 = val0, v1 = val1, s0 = 0;
  for (int n = 0; n < 64; n++) {
    s0 += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  return v0;
}
inline uint32_t lcg(uint32_t& prev) {
  prev = 1664525u * prev + 1013904223u;
  return prev & 0x00FFFFFFu;
}
inline float rnd(uint32_t& prev) { return (float)lcg(prev) / (float)0x01000000; }

// ------------------------------------------------------- sampling helpers --
// programs/sampling.cuh:22-29
inline V3 random_in_unit_disk(uint32_t& seed) {
  float a = rnd(seed) * 2.f * PI_F;
  V3 xy = v3(pt_sinf(a), pt_cosf(a), 0.f);
  xy *= ptm_sqrt(rnd(seed));
  return xy;
}
// programs/sampling.cuh:31-44
inline V3 random_in_unit_sphere(uint32_t& seed) {
  float z = rnd(seed) * 2.f - 1.f;
  float t = rnd(seed) * 2.f * PI_F;
  float r = ptm_sqrt((0.f > (1.f - z * z) ? 0.f : (1.f - z * z)));
  float x = r * pt_cosf(t);
  float y = r * pt_sinf(t);
  V3 res = v3(x, y, z);
  res *= pt_powf(rnd(seed), 1.f / 3.f);
  return res;
}
// programs/sampling.cuh:46-59
inline V3 random_on_unit_sphere(uint32_t& seed) {
  return unit_vector(random_in_unit_sphere(seed));
}

// Orthonormal basis, Duff et al. 2017 (replaces OptiX's Onb).
struct Onb {
  V3 t, b, n;
  explicit Onb(V3 nn) {
    n = nn;
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float bb = n.x * n.y * a;
    t = v3(1.0f + sign * n.x * n.x * a, sign * bb, -sign * n.x);
    b = v3(bb, sign + n.y * n.y * a, -n.y);
  }
  void inverse_transform(V3& p) const { p = p.x * t + p.y * b + p.z * n; }
};

// Malley's method on the Shirley-Chiu concentric map (replaces OptiX's
// cosine_sample_hemisphere).
inline void cosine_sample_hemisphere(float u1, float u2, V3& p) {
  float ox = 2.0f * u1 - 1.0f, oy = 2.0f * u2 - 1.0f;
  float r, theta;
  if (ox == 0.0f && oy == 0.0f) {
    r = 0.0f;
    theta = 0.0f;
  } else if (fabsf(ox) > fabsf(oy)) {
    r = ox;
    theta = PTM_PI_4 * (oy / ox);
  } else {
    r = oy;
    theta = PTM_PI_2 - PTM_PI_4 * (ox / oy);
  }
  float s, c;
  pt_sincosf(theta, &s, &c);
  p.x = r * c;
  p.y = r * s;
  p.z = ptm_sqrt(fmaxf(0.0f, 1.0f - p.x * p.x - p.y * p.y));
}

// programs/math/trigonometric.cuh:5-62
inline float CosTheta(V3 w) { return w.y; }
inline float Cos2Theta(V3 w) { return w.y * w.y; }
inline float AbsCosTheta(V3 w) { return fabsf(w.y); }
inline float Sin2Theta(V3 w) { return fmaxf(0.f, 1.f - Cos2Theta(w)); }
inline float SinTheta(V3 w) { return ptm_sqrt(Sin2Theta(w)); }
inline float TanTheta(V3 w) { return SinTheta(w) / CosTheta(w); }
inline float Tan2Theta(V3 w) { return Sin2Theta(w) / Cos2Theta(w); }
inline float CosPhi(V3 w) {
  float sinTheta = SinTheta(w);
  return (sinTheta == 0) ? 1.f : clampf(w.x / sinTheta, -1.f, 1.f);
}
inline float SinPhi(V3 w) {
  float sinTheta = SinTheta(w);
  return (sinTheta == 0) ? 0.f : clampf(w.z / sinTheta, -1.f, 1.f);
}
inline float Cos2Phi(V3 w) { float c = CosPhi(w); return c * c; }
inline float Sin2Phi(V3 w) { float s = SinPhi(w); return s * s; }
inline V3 Spherical_Vector(float sintheta, float costheta, float phi) {
  return v3(sintheta * pt_cosf(phi), costheta, sintheta * pt_sinf(phi));
}

// ------------------------------------------------------------------ scene --
enum { MAT_LAMBERTIAN = 0, MAT_METAL, MAT_DIELECTRIC, MAT_DIFFUSE_LIGHT,
       MAT_OREN_NAYAR, MAT_TORRANCE_SPARROW, MAT_ASHIKHMIN_SHIRLEY };
// PRIM_MSPHERE: the moving sphere of programs/hitables/moving_sphere.cu,
// f = center0 (3), radius, time0, time1, center1 (3)
enum { PRIM_TRIANGLE = 0, PRIM_SPHERE = 1, PRIM_RECT = 2, PRIM_BOX = 3, PRIM_MSPHERE = 4 };
enum { LIGHT_RECT = 0, LIGHT_SPHERE = 1 };
enum { MISS_GRADIENT = 0, MISS_CONSTANT = 1, MISS_ENV = 2, MISS_IMAGE = 3 };

struct Material {
  int type;
  V3 c0, c1;    // colour (diffuse), second colour (specular / extinction)
  float p0, p1; // fuzz | ref_idx,density | rA,rB | nu,nv
  int tex0 = -1, tex1 = -1;  // textures of c0 / c1 (-1: the constant colour)
};

// Texture callables of programs/textures/*.cu (host_includes/textures.hpp).
enum { TEX_CONSTANT = 0, TEX_CHECKER, TEX_NOISE, TEX_IMAGE, TEX_GRADIENT, TEX_VECTOR };
struct Texture {
  int kind;
  int a = 0, b = 0;          // checker: odd, even; vector: first entry, size; image: w, h;
                             // noise: axis
  float c[9] = {0};          // constant colour; gradient A, B, C; noise scale
  std::vector<float> data;   // image: rgba texels; noise: ranvec (256 x 3)
  std::vector<int> perm;     // noise: perm_x, perm_y, perm_z (3 x 256)
};

struct Xform {
  float m[12];    // object -> world, row major 3x4
  float inv[12];  // world -> object
};

struct Prim {
  int type, material, xform;  // xform -1 = identity
  int axis, flip;
  float f[9];
  // triangles: vertex indices into the mesh-wide attribute arrays
  int32_t vi[3];
  int mesh;
  int tindex;  // texture index: 0, or the face's (mesh.hpp material_buffer)
};

struct Mesh {
  std::vector<V3> normals;
  std::vector<float> uvs;  // 2 per vertex
};

struct Light {
  int type, axis;
  float a0, a1, b0, b1, k;  // rect
  V3 c;
  float r;                  // sphere
  V3 emission;
};

struct Miss {
  int type = MISS_CONSTANT;
  V3 c1 = v3(0.f), c2 = v3(0.f);
  std::vector<float> env;  // rgba, w*h
  int w = 0, h = 0, spherical = 1;
};

struct Cam {
  V3 origin, llc, horizontal, vertical, u, v, w;
  float lens_radius, time0, time1;
};

struct AABB {
  V3 lo, hi;
};

struct BNode {
  AABB box;
  int left;   // internal: left child index; leaf: first prim index
  int count;  // 0 = internal (right = left + 1 not assumed: stored below)
  int right;
};

// Piecewise-constant importance sampling of the spherical environment map:
// weight of texel (r, c) = luminance x sin(theta_r), row (conditional) and
// row-sum (marginal) prefix sums accumulated sequentially in double, then
// normalised to float.  The GPU builds it with the same sequential sums.
struct EnvCdf {
  std::vector<float> marg;  // h+1
  std::vector<float> cond;  // h rows of w+1
  int w = 0, h = 0;
  bool valid = false;
};

struct Scene {
  EnvCdf env_cdf;
  std::vector<Material> mats;
  std::vector<Texture> textures;
  std::vector<int> tex_list;  // vector-texture entries
  std::vector<Prim> prims;
  std::vector<Xform> xforms;
  std::vector<Mesh> meshes;
  std::vector<Light> lights;
  Miss miss;
  Cam cam;
  std::vector<BNode> nodes;
  std::vector<int> order;  // leaf prim order
  bool committed = false;
};

// ---------------------------------------------------------------- xforms --
inline V3 xpoint(const float* m, V3 p) {
  return v3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
            m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
inline V3 xvector(const float* m, V3 p) {
  return v3(m[0] * p.x + m[1] * p.y + m[2] * p.z,
            m[4] * p.x + m[5] * p.y + m[6] * p.z,
            m[8] * p.x + m[9] * p.y + m[10] * p.z);
}
// normal: multiply by the transpose of the world->object matrix
inline V3 xnormal(const float* inv, V3 n) {
  return v3(inv[0] * n.x + inv[4] * n.y + inv[8] * n.z,
            inv[1] * n.x + inv[5] * n.y + inv[9] * n.z,
            inv[2] * n.x + inv[6] * n.y + inv[10] * n.z);
}

// Inverse of an affine 3x4 matrix, in double through the adjugate, rounded
// once to float.  The library's pt_api.cpp evaluates the same expression.
void affine_inverse(const float* m, float* out) {
  double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8],
         h = m[9], i = m[10];
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

// ------------------------------------------------------------- primitives --
struct Ray {
  V3 o, d;
  float tmin, tmax;
  float time = 0.f;  // the path's time (color(): prd.time, programs/raygen.cu:69)
};

struct HitRecord {
  int index;
  int tindex;  // texture index
  V3 P;
  float u, v;
  V3 geometric_normal, shading_normal, Wo;
};

// Centre of a moving sphere at `time`: programs/hitables/moving_sphere.cu:47-49
// (linear in time, also outside [time0, time1]).
inline V3 msphere_center(const Prim& p, float time) {
  V3 c0 = v3(p.f[0], p.f[1], p.f[2]), c1 = v3(p.f[6], p.f[7], p.f[8]);
  return c0 + ((time - p.f[4]) / (p.f[5] - p.f[4])) * (c1 - c0);
}

// Candidate t of one primitive for an (object-space) ray; false if none.
// programs/hitables/sphere.cu:32-62 (a moving sphere: moving_sphere.cu:57-118
// at its centre for the ray's time, the same two roots)
bool sphere_candidate(V3 center, float radius, V3 o, V3 d, float tmin, float tmax, float& t) {
  V3 oc = o - center;
  float a = dot(d, d);
  float b = dot(oc, d);
  float c = dot(oc, oc) - radius * radius;
  float discriminant = b * b - a * c;
  if (discriminant < 0.f) return false;
  float t0 = (-b - ptm_sqrt(discriminant)) / a;
  if (t0 > tmin && t0 < tmax) { t = t0; return true; }
  float t1 = (-b + ptm_sqrt(discriminant)) / a;
  if (t1 > tmin && t1 < tmax) { t = t1; return true; }
  return false;
}

// programs/hitables/aarect.cu:20-69
bool rect_candidate(const Prim& p, V3 o, V3 d, float tmin, float tmax, float& t) {
  float a0 = p.f[0], a1 = p.f[1], b0 = p.f[2], b1 = p.f[3], k = p.f[4];
  float a, b;
  if (p.axis == 0) {
    t = (k - o.x) / d.x;
    a = o.y + t * d.y;
    b = o.z + t * d.z;
  } else if (p.axis == 1) {
    t = (k - o.y) / d.y;
    a = o.x + t * d.x;
    b = o.z + t * d.z;
  } else {
    t = (k - o.z) / d.z;
    a = o.x + t * d.x;
    b = o.y + t * d.y;
  }
  if (a < a0 || a > a1 || b < b0 || b > b1) return false;
  return t > tmin && t < tmax;
}

// programs/hitables/box.cu:36-53
bool box_candidate(const Prim& p, V3 o, V3 d, float tmin, float tmax, float& t) {
  V3 boxmin = v3(p.f[0], p.f[1], p.f[2]), boxmax = v3(p.f[3], p.f[4], p.f[5]);
  V3 t0 = (boxmin - o) / d;
  V3 t1 = (boxmax - o) / d;
  float tn = max_component(min_vec(t0, t1));
  float tf = min_component(max_vec(t0, t1));
  if (tn <= tf) {
    if (tn > tmin && tn < tmax) { t = tn; return true; }
    if (tf > tmin && tf < tmax) { t = tf; return true; }
  }
  return false;
}

// Watertight ray/triangle test, Woop, Benthin & Wald, JCGT 2(1) 2013.  Same
// statement order as the GPU kernel.  Returns barycentrics of v1 (u), v2 (v).
bool tri_candidate(const Prim& p, V3 o, V3 d, float tmin, float tmax, float& t,
                   float& bu, float& bv) {
  float adx = fabsf(d.x), ady = fabsf(d.y), adz = fabsf(d.z);
  int kz = (adx > ady) ? ((adx > adz) ? 0 : 2) : ((ady > adz) ? 1 : 2);
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  if (get(d, kz) < 0.0f) { int tmp = kx; kx = ky; ky = tmp; }
  float Sz = 1.0f / get(d, kz);
  float Sx = get(d, kx) * Sz;
  float Sy = get(d, ky) * Sz;
  V3 A = v3(p.f[0], p.f[1], p.f[2]) - o;
  V3 B = v3(p.f[3], p.f[4], p.f[5]) - o;
  V3 C = v3(p.f[6], p.f[7], p.f[8]) - o;
  float Ax = get(A, kx) - Sx * get(A, kz), Ay = get(A, ky) - Sy * get(A, kz);
  float Bx = get(B, kx) - Sx * get(B, kz), By = get(B, ky) - Sy * get(B, kz);
  float Cx = get(C, kx) - Sx * get(C, kz), Cy = get(C, ky) - Sy * get(C, kz);
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
  float Az = Sz * get(A, kz), Bz = Sz * get(B, kz), Cz = Sz * get(C, kz);
  float T = U * Az + V * Bz + W * Cz;
  float rcp = 1.0f / det;
  float tt = T * rcp;
  if (!(tt > tmin && tt < tmax)) return false;
  t = tt;
  bu = V * rcp;
  bv = W * rcp;
  return true;
}

// Object-space ray of a primitive.
inline void object_ray(const Scene& s, const Prim& p, const Ray& r, V3& o, V3& d) {
  if (p.xform < 0) { o = r.o; d = r.d; return; }
  const float* inv = s.xforms[p.xform].inv;
  o = xpoint(inv, r.o);
  d = xvector(inv, r.d);
}

bool prim_candidate(const Scene& s, const Prim& p, const Ray& r, float& t, float& bu,
                    float& bv) {
  V3 o, d;
  object_ray(s, p, r, o, d);
  bu = bv = 0.0f;
  switch (p.type) {
    case PRIM_SPHERE: return sphere_candidate(v3(p.f[0], p.f[1], p.f[2]), p.f[3], o, d, r.tmin, r.tmax, t);
    case PRIM_MSPHERE: return sphere_candidate(msphere_center(p, r.time), p.f[3], o, d, r.tmin, r.tmax, t);
    case PRIM_RECT: return rect_candidate(p, o, d, r.tmin, r.tmax, t);
    case PRIM_BOX: return box_candidate(p, o, d, r.tmin, r.tmax, t);
    default: return tri_candidate(p, o, d, r.tmin, r.tmax, t, bu, bv);
  }
}

// Get_HitRecord of each primitive type.
HitRecord hit_record(const Scene& s, const Prim& p, const Ray& r, float t_hit, float bu,
                     float bv) {
  HitRecord rec;
  rec.Wo = normalize(-r.d);
  V3 o, d;
  object_ray(s, p, r, o, d);
  const float* M = p.xform >= 0 ? s.xforms[p.xform].m : nullptr;
  const float* I = p.xform >= 0 ? s.xforms[p.xform].inv : nullptr;
  rec.index = p.material;
  rec.tindex = p.type == PRIM_TRIANGLE ? p.tindex : 0;
  if (p.type == PRIM_SPHERE || p.type == PRIM_MSPHERE) {
    // programs/hitables/sphere.cu:65-93; the moving sphere's record
    // (moving_sphere.cu:80-96) is the same at its centre for the ray's time
    V3 center = p.type == PRIM_SPHERE ? v3(p.f[0], p.f[1], p.f[2]) : msphere_center(p, r.time);
    float radius = p.f[3];
    V3 hit_point = o + t_hit * d;
    rec.P = M ? xpoint(M, hit_point) : hit_point;
    V3 T = (rec.P - center) / radius;
    V3 normal = normalize(I ? xnormal(I, T) : T);
    rec.shading_normal = rec.geometric_normal = normal;
    float phi = pt_atan2f(T.z, T.x);
    float theta = pt_asinf(T.y);
    rec.u = 1.f - (phi + PI_F) / (2.f * PI_F);
    rec.v = (theta + PI_F / 2.f) / PI_F;
  } else if (p.type == PRIM_RECT) {  // programs/hitables/aarect.cu:71-115
    float a0 = p.f[0], a1 = p.f[1], b0 = p.f[2], b1 = p.f[3];
    V3 hit_point = o + t_hit * d;
    rec.P = M ? xpoint(M, hit_point) : hit_point;
    V3 normal;
    if (p.axis == 0) {
      normal = v3(1.f, 0.f, 0.f);
      rec.u = (hit_point.y - a0) / (a1 - a0);
      rec.v = (hit_point.z - b0) / (b1 - b0);
    } else if (p.axis == 1) {
      normal = v3(0.f, 1.f, 0.f);
      rec.u = (hit_point.x - a0) / (a1 - a0);
      rec.v = (hit_point.z - b0) / (b1 - b0);
    } else {
      normal = v3(0.f, 0.f, 1.f);
      rec.u = (hit_point.x - a0) / (a1 - a0);
      rec.v = (hit_point.y - b0) / (b1 - b0);
    }
    normal = p.flip ? -normal : normal;
    normal = normalize(I ? xnormal(I, normal) : normal);
    rec.shading_normal = rec.geometric_normal = normal;
  } else if (p.type == PRIM_BOX) {  // programs/hitables/box.cu:24-81
    V3 boxmin = v3(p.f[0], p.f[1], p.f[2]), boxmax = v3(p.f[3], p.f[4], p.f[5]);
    V3 hit_point = o + t_hit * d;
    rec.P = M ? xpoint(M, hit_point) : hit_point;
    V3 t0 = (boxmin - o) / d;
    V3 t1 = (boxmax - o) / d;
    V3 neg = v3(t_hit == t0.x ? 1.f : 0.f, t_hit == t0.y ? 1.f : 0.f, t_hit == t0.z ? 1.f : 0.f);
    V3 pos = v3(t_hit == t1.x ? 1.f : 0.f, t_hit == t1.y ? 1.f : 0.f, t_hit == t1.z ? 1.f : 0.f);
    V3 normal = pos - neg;
    normal = normalize(I ? xnormal(I, normal) : normal);
    rec.shading_normal = rec.geometric_normal = normal;
    rec.u = rec.v = 0.f;
  } else {  // programs/hitables/triangle.cu:85-149 (mesh already in world space)
    V3 a = v3(p.f[0], p.f[1], p.f[2]), b = v3(p.f[3], p.f[4], p.f[5]),
       c = v3(p.f[6], p.f[7], p.f[8]);
    V3 e1 = b - a, e2 = c - a;
    float b0 = 1.f - bu - bv, b1 = bu, b2 = bv;
    rec.P = a * b0 + b * b1 + c * b2;
    V3 Ng = cross(e1, e2);
    float area = length(Ng) / 2.f;
    Ng /= 2.f * area;
    Ng = normalize(normalize(Ng));
    rec.geometric_normal = Ng;
    const Mesh& mesh = s.meshes[p.mesh];
    if (mesh.normals.empty()) {
      rec.shading_normal = Ng;
    } else {
      V3 Ns = mesh.normals[p.vi[0]] * b0 + mesh.normals[p.vi[1]] * b1 +
              mesh.normals[p.vi[2]] * b2;
      rec.shading_normal = normalize(Ns);
    }
    if (mesh.uvs.empty()) {
      rec.u = rec.v = 0.f;
    } else {
      const float* uv = mesh.uvs.data();
      rec.u = uv[2 * p.vi[0]] * b0 + uv[2 * p.vi[1]] * b1 + uv[2 * p.vi[2]] * b2;
      rec.v = uv[2 * p.vi[0] + 1] * b0 + uv[2 * p.vi[1] + 1] * b1 + uv[2 * p.vi[2] + 1] * b2;
    }
  }
  return rec;
}

// -------------------------------------------------------------- textures --
// programs/textures/noise_texture.cu:12-59 (ranvec: 256 x 3, perm: 3 x 256)
float perlin_noise(const Texture& t, V3 p) {
  float u = p.x - floorf(p.x);
  float v = p.y - floorf(p.y);
  float w = p.z - floorf(p.z);
  int i = (int)floorf(p.x);
  int j = (int)floorf(p.y);
  int k = (int)floorf(p.z);
  float uu = u * u * (3 - 2 * u);
  float vv = v * v * (3 - 2 * v);
  float ww = w * w * (3 - 2 * w);
  float accum = 0;
  for (int di = 0; di < 2; di++)
    for (int dj = 0; dj < 2; dj++)
      for (int dk = 0; dk < 2; dk++) {
        int r = t.perm[(i + di) & 255] ^ t.perm[256 + ((j + dj) & 255)] ^
                t.perm[512 + ((k + dk) & 255)];
        V3 c = v3(t.data[3 * r], t.data[3 * r + 1], t.data[3 * r + 2]);
        V3 weight_v = v3(u - di, v - dj, w - dk);
        accum += (di * uu + (1 - di) * (1 - uu)) * (dj * vv + (1 - dj) * (1 - vv)) *
                 (dk * ww + (1 - dk) * (1 - ww)) * dot(c, weight_v);
      }
  return accum;
}

// noise_texture.cu:61-76
float perlin_turb(const Texture& t, V3 p) {
  float accum = 0;
  V3 temp_p = p;
  float weight = 1.0f;
  for (int i = 0; i < 7; i++) {
    accum += weight * perlin_noise(t, temp_p);
    weight *= 0.5f;
    temp_p *= 2.f;
  }
  return fabsf(accum);
}

// sample_texture(u, v, p, i) of the texture callables.
V3 texture_color(const Scene& s, int id, float u, float v, V3 p, int i) {
  for (int hop = 0; hop < 64; hop++) {
    const Texture& t = s.textures[id];
    switch (t.kind) {
      case TEX_CONSTANT:  // constant_texture.cu:5-7
        return v3(t.c[0], t.c[1], t.c[2]);
      case TEX_CHECKER: {  // checkered_texture.cu:8-15
        float sines = pt_sinf(10 * p.x) * pt_sinf(10 * p.y) * pt_sinf(10 * p.z);
        id = sines < 0 ? t.a : t.b;
        i = 0;
        break;
      }
      case TEX_VECTOR:  // vector.cu:7-12
        if (i >= t.b || i < 0) return v3(0.f);
        id = s.tex_list[t.a + i];
        i = 0;
        break;
      case TEX_NOISE: {  // noise_texture.cu:61-76: every axis falls through to Z
        float scale = t.c[0];
        float sinValue = pt_sinf(scale * p.z + 5 * perlin_turb(t, scale * p));
        return v3(1.f) * 0.5f * (1 + sinValue);
      }
      case TEX_IMAGE: {  // image_texture.cu:3-7: bilinear, repeat wrap
        int W = t.a, H = t.b;
        if (!(u == u) || !(v == v) || fabsf(u) > 1e6f || fabsf(v) > 1e6f) return v3(0.f);
        float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
        float fx = ptm_floor(x), fy = ptm_floor(y);
        float ax = x - fx, ay = y - fy;
        int ix0 = (int)fx % W; if (ix0 < 0) ix0 += W;
        int iy0 = (int)fy % H; if (iy0 < 0) iy0 += H;
        int ix1 = ix0 + 1 == W ? 0 : ix0 + 1;
        int iy1 = iy0 + 1 == H ? 0 : iy0 + 1;
        auto tx = [&](int ix, int iy) {
          const float* e = t.data.data() + ((size_t)iy * W + ix) * 4;
          return v3(e[0], e[1], e[2]);
        };
        return (tx(ix0, iy0) * (1.f - ax) + tx(ix1, iy0) * ax) * (1.f - ay) +
               (tx(ix0, iy1) * (1.f - ax) + tx(ix1, iy1) * ax) * ay;
      }
      default: {  // gradient_texture.cu:7-14
        V3 unit_direction = normalize(p);
        float x = fabsf(unit_direction.x), y = fabsf(unit_direction.y),
              z = fabsf(unit_direction.z);
        return x * v3(t.c[0], t.c[1], t.c[2]) + y * v3(t.c[3], t.c[4], t.c[5]) +
               z * v3(t.c[6], t.c[7], t.c[8]);
      }
    }
  }
  return v3(0.f);
}

// Get_Parameters of the closest-hit programs: colours from the textures.
inline void resolve_textures(const Scene& s, Material& m, const HitRecord& rec) {
  if (m.tex0 >= 0) m.c0 = texture_color(s, m.tex0, rec.u, rec.v, rec.P, rec.tindex);
  if (m.tex1 >= 0) m.c1 = texture_color(s, m.tex1, rec.u, rec.v, rec.P, rec.tindex);
}

// ------------------------------------------------------------------- BVH ---
AABB prim_bounds(const Scene& s, const Prim& p) {
  AABB b;
  V3 lo, hi;
  if (p.type == PRIM_TRIANGLE) {
    V3 a = v3(p.f[0], p.f[1], p.f[2]), bb = v3(p.f[3], p.f[4], p.f[5]),
       c = v3(p.f[6], p.f[7], p.f[8]);
    lo = v3(fminf(fminf(a.x, bb.x), c.x), fminf(fminf(a.y, bb.y), c.y), fminf(fminf(a.z, bb.z), c.z));
    hi = v3(fmaxf(fmaxf(a.x, bb.x), c.x), fmaxf(fmaxf(a.y, bb.y), c.y), fmaxf(fmaxf(a.z, bb.z), c.z));
  } else if (p.type == PRIM_SPHERE) {
    lo = v3(p.f[0] - p.f[3], p.f[1] - p.f[3], p.f[2] - p.f[3]);
    hi = v3(p.f[0] + p.f[3], p.f[1] + p.f[3], p.f[2] + p.f[3]);
  } else if (p.type == PRIM_MSPHERE) {
    // every centre a ray can meet: the ray times lie between cam.time0 and
    // cam.time0 + (cam.time1 - cam.time0), and the centre is monotonic in
    // time (moving_sphere.cu:136-147 bounds [time0, time1] only)
    float te = s.cam.time0 + (s.cam.time1 - s.cam.time0);
    float ta = fminf(fminf(p.f[4], s.cam.time0), te), tb = fmaxf(fmaxf(p.f[5], s.cam.time0), te);
    V3 ca = msphere_center(p, ta), cb = msphere_center(p, tb);
    lo = v3(fminf(ca.x, cb.x) - p.f[3], fminf(ca.y, cb.y) - p.f[3], fminf(ca.z, cb.z) - p.f[3]);
    hi = v3(fmaxf(ca.x, cb.x) + p.f[3], fmaxf(ca.y, cb.y) + p.f[3], fmaxf(ca.z, cb.z) + p.f[3]);
  } else if (p.type == PRIM_RECT) {
    float a0 = p.f[0], a1 = p.f[1], b0 = p.f[2], b1 = p.f[3], k = p.f[4];
    if (p.axis == 0) { lo = v3(k, a0, b0); hi = v3(k, a1, b1); }
    else if (p.axis == 1) { lo = v3(a0, k, b0); hi = v3(a1, k, b1); }
    else { lo = v3(a0, b0, k); hi = v3(a1, b1, k); }
  } else {
    lo = v3(p.f[0], p.f[1], p.f[2]);
    hi = v3(p.f[3], p.f[4], p.f[5]);
  }
  if (p.xform >= 0) {
    const float* M = s.xforms[p.xform].m;
    V3 nlo = v3(FLT_MAX), nhi = v3(-FLT_MAX);
    for (int c = 0; c < 8; c++) {
      V3 q = v3((c & 1) ? hi.x : lo.x, (c & 2) ? hi.y : lo.y, (c & 4) ? hi.z : lo.z);
      V3 w = xpoint(M, q);
      nlo = v3(fminf(nlo.x, w.x), fminf(nlo.y, w.y), fminf(nlo.z, w.z));
      nhi = v3(fmaxf(nhi.x, w.x), fmaxf(nhi.y, w.y), fmaxf(nhi.z, w.z));
    }
    lo = nlo;
    hi = nhi;
  }
  // conservative padding: relative to magnitude plus a small absolute term
  for (int i = 0; i < 3; i++) {
    float* l = i == 0 ? &lo.x : (i == 1 ? &lo.y : &lo.z);
    float* h = i == 0 ? &hi.x : (i == 1 ? &hi.y : &hi.z);
    float pad = 1e-4f * fmaxf(1.0f, fmaxf(fabsf(*l), fabsf(*h)));
    *l -= pad;
    *h += pad;
  }
  b.lo = lo;
  b.hi = hi;
  return b;
}

inline AABB merge(const AABB& a, const AABB& b) {
  return AABB{v3(fminf(a.lo.x, b.lo.x), fminf(a.lo.y, b.lo.y), fminf(a.lo.z, b.lo.z)),
              v3(fmaxf(a.hi.x, b.hi.x), fmaxf(a.hi.y, b.hi.y), fmaxf(a.hi.z, b.hi.z))};
}
inline float area(const AABB& a) {
  V3 e = a.hi - a.lo;
  if (e.x < 0) return 0.f;
  return 2.f * (e.x * e.y + e.y * e.z + e.z * e.x);
}

struct Builder {
  const std::vector<AABB>& boxes;
  std::vector<V3> cent;
  std::vector<int>& idx;
  std::vector<BNode>& nodes;
  Builder(const std::vector<AABB>& b, std::vector<int>& i, std::vector<BNode>& n)
      : boxes(b), idx(i), nodes(n) {
    cent.resize(b.size());
    for (size_t k = 0; k < b.size(); k++) cent[k] = (b[k].lo + b[k].hi) * 0.5f;
  }
  int build(int begin, int end) {
    int ni = (int)nodes.size();
    nodes.push_back(BNode());
    AABB bb = boxes[idx[begin]], cb{cent[idx[begin]], cent[idx[begin]]};
    for (int k = begin + 1; k < end; k++) {
      bb = merge(bb, boxes[idx[k]]);
      cb = merge(cb, AABB{cent[idx[k]], cent[idx[k]]});
    }
    nodes[ni].box = bb;
    int n = end - begin;
    if (n <= 4) {
      nodes[ni].left = begin;
      nodes[ni].count = n;
      return ni;
    }
    // binned SAH, 16 bins per axis
    const int NB = 16;
    float best = FLT_MAX;
    int best_axis = -1, best_bin = -1;
    for (int ax = 0; ax < 3; ax++) {
      float lo = get(cb.lo, ax), hi = get(cb.hi, ax);
      if (hi - lo <= 0.f) continue;
      AABB bins[NB];
      int cnt[NB] = {0};
      for (int k = 0; k < NB; k++) bins[k] = AABB{v3(FLT_MAX), v3(-FLT_MAX)};
      float scale = NB / (hi - lo);
      for (int k = begin; k < end; k++) {
        int b = (int)((get(cent[idx[k]], ax) - lo) * scale);
        if (b >= NB) b = NB - 1;
        if (b < 0) b = 0;
        cnt[b]++;
        bins[b] = merge(bins[b], boxes[idx[k]]);
      }
      float la[NB], ra[NB];
      int lc[NB], rc[NB];
      AABB acc{v3(FLT_MAX), v3(-FLT_MAX)};
      int c = 0;
      for (int k = 0; k < NB; k++) {
        acc = merge(acc, bins[k]);
        c += cnt[k];
        la[k] = area(acc);
        lc[k] = c;
      }
      acc = AABB{v3(FLT_MAX), v3(-FLT_MAX)};
      c = 0;
      for (int k = NB - 1; k >= 0; k--) {
        acc = merge(acc, bins[k]);
        c += cnt[k];
        ra[k] = area(acc);
        rc[k] = c;
      }
      for (int k = 0; k < NB - 1; k++) {
        if (lc[k] == 0 || rc[k + 1] == 0) continue;
        float cost = la[k] * lc[k] + ra[k + 1] * rc[k + 1];
        if (cost < best) { best = cost; best_axis = ax; best_bin = k; }
      }
    }
    int mid;
    if (best_axis < 0) {
      mid = begin + n / 2;
    } else {
      float lo = get(cb.lo, best_axis), hi = get(cb.hi, best_axis);
      float scale = NB / (hi - lo);
      auto it = std::partition(idx.begin() + begin, idx.begin() + end, [&](int k) {
        int b = (int)((get(cent[k], best_axis) - lo) * scale);
        if (b >= NB) b = NB - 1;
        if (b < 0) b = 0;
        return b <= best_bin;
      });
      mid = (int)(it - idx.begin());
      if (mid == begin || mid == end) mid = begin + n / 2;
    }
    int l = build(begin, mid);
    int r = build(mid, end);
    nodes[ni].left = l;
    nodes[ni].right = r;
    nodes[ni].count = 0;
    return ni;
  }
};

inline bool slab(const AABB& b, V3 o, V3 inv, float tmin, float tmax, float& tn) {
  float tx0 = (b.lo.x - o.x) * inv.x, tx1 = (b.hi.x - o.x) * inv.x;
  float ty0 = (b.lo.y - o.y) * inv.y, ty1 = (b.hi.y - o.y) * inv.y;
  float tz0 = (b.lo.z - o.z) * inv.z, tz1 = (b.hi.z - o.z) * inv.z;
  float t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
  float t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
  t1 *= 1.00000024f;  // robust: 2 ulp slack
  tn = t0;
  return t0 <= t1;
}

struct Hit {
  int prim = -1;
  float t = 0.f, u = 0.f, v = 0.f;
};

struct Counters {
  uint64_t nodes = 0, prims = 0;
};

// Closest hit: lexicographic minimum of (t, prim id) over all candidates.
Hit trace(const Scene& s, const Ray& r, Counters* cnt) {
  Hit best;
  float tbest = r.tmax;
  if (s.nodes.empty()) return best;
  V3 inv = v3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const BNode& n = s.nodes[stack[--sp]];
    float tn;
    if (cnt) cnt->nodes++;
    if (!slab(n.box, r.o, inv, r.tmin, tbest, tn)) continue;
    if (n.count) {
      for (int k = n.left; k < n.left + n.count; k++) {
        int pid = s.order[k];
        float t, bu, bv;
        if (cnt) cnt->prims++;
        if (!prim_candidate(s, s.prims[pid], r, t, bu, bv)) continue;
        if (t < tbest || (t == tbest && pid < best.prim)) {
          tbest = t;
          best.prim = pid;
          best.t = t;
          best.u = bu;
          best.v = bv;
        }
      }
    } else {
      float tl, tr;
      bool hl = slab(s.nodes[n.left].box, r.o, inv, r.tmin, tbest, tl);
      bool hr = slab(s.nodes[n.right].box, r.o, inv, r.tmin, tbest, tr);
      if (hl && hr) {
        if (tl <= tr) { stack[sp++] = n.right; stack[sp++] = n.left; }
        else { stack[sp++] = n.left; stack[sp++] = n.right; }
      } else if (hl) {
        stack[sp++] = n.left;
      } else if (hr) {
        stack[sp++] = n.right;
      }
    }
  }
  return best;
}

// ------------------------------------------------------------ lights -------
// programs/pdfs/rect_pdf.cu:11-145, programs/pdfs/sphere_pdf.cu:8-73
bool rect_light_intersect(const Light& L, V3 P, V3 Wi, float tmin, float tmax, V3& N, float& t) {
  float a, b;
  if (L.axis == 0) {
    t = (L.k - P.x) / Wi.x;
    a = P.y + t * Wi.y;
    b = P.z + t * Wi.z;
  } else if (L.axis == 1) {
    t = (L.k - P.y) / Wi.y;
    a = P.x + t * Wi.x;
    b = P.z + t * Wi.z;
  } else {
    t = (L.k - P.z) / Wi.z;
    a = P.x + t * Wi.x;
    b = P.y + t * Wi.y;
  }
  if (a < L.a0 || a > L.a1 || b < L.b0 || b > L.b1) return false;
  if (t < tmax && t > tmin) {
    N = L.axis == 0 ? v3(1.f, 0.f, 0.f) : (L.axis == 1 ? v3(0.f, 1.f, 0.f) : v3(0.f, 0.f, 1.f));
    return true;
  }
  return false;
}

float light_pdf(const Light& L, V3 P, V3 Wi) {
  if (L.type == LIGHT_RECT) {
    float t;
    V3 rectNormal;
    if (rect_light_intersect(L, P, Wi, 0.001f, FLT_MAX, rectNormal, t)) {
      float distance_squared = t * t * squared_length(Wi);
      float cosine = fabsf(dot(Wi, rectNormal) / length(Wi));
      float area = (L.a1 - L.a0) * (L.b1 - L.b0);
      return distance_squared / (cosine * area);
    }
    return 0.f;
  }
  // sphere
  V3 oc = P - L.c;
  float a = dot(Wi, Wi);
  float b = dot(oc, Wi);
  float c = dot(oc, oc) - L.r * L.r;
  float discriminant = b * b - a * c;
  bool hit = false;
  if (discriminant >= 0.f) {
    float temp = (-b - ptm_sqrt(discriminant)) / a;
    if (temp < FLT_MAX && temp > 0.001f) hit = true;
    if (!hit) {
      temp = (-b + ptm_sqrt(discriminant)) / a;
      if (temp < FLT_MAX && temp > 0.001f) hit = true;
    }
  }
  if (!hit) return 0.f;
  float distance_squared = squared_length(L.c - P);
  float cos_theta_max = ptm_sqrt(1.f - L.r * L.r / distance_squared);
  float solid_angle = 2.f * PI_F * (1.f - cos_theta_max);
  return 1.f / solid_angle;
}

V3 light_sample(const Light& L, V3 P, uint32_t& seed) {
  if (L.type == LIGHT_RECT) {
    float r0 = rnd(seed);
    float r1 = rnd(seed);
    V3 q;
    if (L.axis == 0) q = v3(L.k, L.a0 + r0 * (L.a1 - L.a0), L.b0 + r1 * (L.b1 - L.b0));
    else if (L.axis == 1) q = v3(L.a0 + r0 * (L.a1 - L.a0), L.k, L.b0 + r1 * (L.b1 - L.b0));
    else q = v3(L.a0 + r0 * (L.a1 - L.a0), L.b0 + r1 * (L.b1 - L.b0), L.k);
    return q - P;
  }
  float r1 = rnd(seed);
  float r2 = rnd(seed);
  float distance_squared = squared_length(L.c - P);
  float z = 1.f + r2 * (ptm_sqrt(1.f - L.r * L.r / distance_squared) - 1.f);
  float phi = 2.f * PI_F * r1;
  float x = pt_cosf(phi) * ptm_sqrt(1.f - z * z);
  float y = pt_sinf(phi) * ptm_sqrt(1.f - z * z);
  V3 Wi = v3(x, y, z);
  Onb uvw(normalize(Wi));
  uvw.inverse_transform(Wi);
  return Wi;
}

// -------------------------------------------------------------- materials --
// programs/materials/material.cuh:30-63
inline float schlick(float cosine, float ref_idx) {
  float r0 = (1.f - ref_idx) / (1.f + ref_idx);
  r0 = r0 * r0;
  return r0 + (1.f - r0) * pt_powf((1.f - cosine), 5.f);
}
inline V3 schlick3(V3 r0, float cosine) {
  float exponential = pt_powf(1.f - cosine, 5.f);
  return r0 + (v3(1.f) - r0) * exponential;
}
inline bool Refract(V3 v, V3 n, float ni_over_nt, V3& refracted) {
  V3 uv = normalize(v);
  float dt = dot(uv, n);
  float discriminant = 1.f - ni_over_nt * ni_over_nt * (1.f - dt * dt);
  if (discriminant > 0.f) {
    refracted = ni_over_nt * (uv - n * dt) - n * ptm_sqrt(discriminant);
    return true;
  }
  return false;
}

// programs/materials/microfacets.cuh:11-20
inline void Sample_Quadrant(float nu, float nv, float randX, float randY, float& phi,
                            float& theta) {
  phi = pt_atanf(ptm_sqrt((nu + 1.f) / (nv + 1.f)) * pt_tanf(2.f * PI_F * randX));
  float cos_phi = pt_cosf(phi);
  float sin_phi = pt_sinf(phi);
  theta = pt_powf(randY, 1.f / (nu * cos_phi * cos_phi + nv * sin_phi * sin_phi + 1.f));
}
// programs/materials/microfacets.cuh:85-201
inline float GGX_D(V3 H, float nu, float nv) {
  const float CosTheta2 = Cos2Theta(H);
  if (CosTheta2 <= 0.0f) return 0.f;
  if (nu == nv) {
    float beta = CosTheta2 * ((nu * nu) - 1) + 1;
    return (nu * nu) / (PI_F * beta * beta);
  }
  const float Sin2PhiNV = Sin2Phi(H) / (nv * nv);
  const float Cos2PhiNU = (1.f - Sin2Phi(H)) / (nu * nu);
  float beta = (CosTheta2 + (1.f - CosTheta2) * (Cos2PhiNU + Sin2PhiNV));
  return 1.f / (PI_F * nu * nv * beta * beta);
}
inline V3 GGX_Sample(V3 origin, float rx, float ry, float nu, float nv) {
  bool flip = origin.y < 0;
  V3 stretchedOrigin = v3(origin.x * nu, origin.y, origin.z * nv);
  stretchedOrigin = normalize(stretchedOrigin);
  float slopeX, slopeY;
  float cosTheta = CosTheta(stretchedOrigin);
  if (cosTheta > 0.9999f) {
    float r = ptm_sqrt(rx / (1 - rx));
    float phi = (float)(6.28318530718 * (double)ry);
    slopeX = r * pt_cosf(phi);
    slopeY = r * pt_sinf(phi);
  } else {
    float sinTheta = ptm_sqrt(fmaxf(0.f, 1.f - cosTheta * cosTheta));
    float tanTheta = sinTheta / cosTheta;
    float a = 1.f / tanTheta;
    float G1 = 2.f / (1.f + ptm_sqrt(1.f + 1.f / (a * a)));
    float A = 2.f * rx / G1 - 1.f;
    float tmp = 1.f / (A * A - 1.f);
    if (tmp > 1e10f) tmp = 1e10f;
    float B = tanTheta;
    float D = ptm_sqrt(fmaxf(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.f));
    float slopeX1 = B * tmp - D;
    float slopeX2 = B * tmp + D;
    slopeX = (A < 0 || slopeX2 > 1.f / tanTheta) ? slopeX1 : slopeX2;
    float S;
    if (ry > 0.5f) {
      S = 1.f;
      ry = 2.f * (ry - .5f);
    } else {
      S = -1.f;
      ry = 2.f * (.5f - ry);
    }
    float z = (ry * (ry * (ry * 0.27385f - 0.73369f) + 0.46341f)) /
              (ry * (ry * (ry * 0.093073f + 0.309420f) - 1.f) + 0.597999f);
    slopeY = S * z * ptm_sqrt(1.f + slopeX * slopeX);
  }
  float t = CosPhi(stretchedOrigin) * slopeX - SinPhi(stretchedOrigin) * slopeY;
  slopeY = SinPhi(stretchedOrigin) * slopeX + CosPhi(stretchedOrigin) * slopeY;
  slopeX = t;
  slopeX = nu * slopeX;
  slopeY = nv * slopeY;
  V3 H = normalize(v3(-slopeX, 1.f, -slopeY));
  if (flip) H *= -1.f;
  return H;
}
inline float GGX_Lambda(V3 V, float nu, float nv) {
  float absTanTheta = fabsf(TanTheta(V));
  if (isinf(absTanTheta)) return 0.f;
  float alpha = ptm_sqrt(Cos2Phi(V) * nu * nu + Sin2Phi(V) * nv * nv);
  float alpha2Tan2Theta = (alpha * absTanTheta) * (alpha * absTanTheta);
  return (-1.f + ptm_sqrt(1.f + alpha2Tan2Theta)) / 2.f;
}
inline float GGX_G(V3 Wo, V3 Wi, float nu, float nv) {
  return 1.f / (1.f + GGX_Lambda(Wo, nu, nv) + GGX_Lambda(Wi, nu, nv));
}
inline float GGX_PDF(V3 H, float nu, float nv) { return GGX_D(H, nu, nv) * AbsCosTheta(H); }

// BRDF sample (draws random numbers) and evaluate (sets pdf).
V3 brdf_sample(const Material& m, V3 Wo, V3 N, uint32_t& seed) {
  switch (m.type) {
    case MAT_LAMBERTIAN:    // programs/materials/lambertian.cuh:7-19
    case MAT_OREN_NAYAR: {  // programs/materials/oren_nayar.cuh:8-20
      V3 Wi;
      float r0 = rnd(seed);
      float r1 = rnd(seed);
      cosine_sample_hemisphere(r0, r1, Wi);
      Onb uvw(N);
      uvw.inverse_transform(Wi);
      return Wi;
    }
    case MAT_DIFFUSE_LIGHT:  // programs/materials/diffuse_light.cuh:7-13
      return random_on_unit_sphere(seed);
    case MAT_TORRANCE_SPARROW: {  // programs/materials/torrance_sparrow.cuh:10-35
      float nu = m.p0, nv = m.p1;
      V3 Nn = normalize(N);
      V3 T = normalize(cross(Nn, v3(0.f, 1.f, 0.f)));
      V3 B = cross(T, Nn);
      float rx = rnd(seed);
      float ry = rnd(seed);
      V3 H = normalize(GGX_Sample(Wo, rx, ry, nu, nv));
      H = H.x * B + H.y * Nn + H.z * T;
      float HdotI = dot(H, Wo);
      if (HdotI < 0.f) H = -H;
      return normalize(-Wo + 2.f * dot(Wo, H) * H);
    }
    case MAT_ASHIKHMIN_SHIRLEY: {  // programs/materials/ashikhmin_shirley.cuh:11-82
      float nu = m.p0, nv = m.p1;
      V3 Wi;
      V3 Nn = normalize(N);
      V3 T = normalize(cross(Nn, v3(0.f, 1.f, 0.f)));
      V3 B = cross(T, Nn);
      float rx = rnd(seed);
      float ry = rnd(seed);
      if (rx < 0.5) {
        rx = fminf(2 * rx, 1.f - 1e-6f);
        cosine_sample_hemisphere(rx, ry, Wi);
        Onb uvw(Nn);
        uvw.inverse_transform(Wi);
      } else {
        rx = fminf(2 * (rx - 0.5f), 1.f - 1e-6f);
        float phi, cos_theta;
        if (nu == nv) {
          phi = 2.f * PI_F * rx;
          cos_theta = pt_powf(ry, 1.f / (nu + 1.f));
        } else {
          if (rx < 0.25f) {
            float remappedRX = 4.f * rx;
            Sample_Quadrant(nu, nv, remappedRX, ry, phi, cos_theta);
          } else if (rx < 0.5f) {
            float remappedRX = 4.f * (0.5f - rx);
            Sample_Quadrant(nu, nv, remappedRX, ry, phi, cos_theta);
            phi = PI_F - phi;
          } else if (rx < 0.75f) {
            float remappedRX = 4.f * (rx - 0.5f);
            Sample_Quadrant(nu, nv, remappedRX, ry, phi, cos_theta);
            phi = PI_F + phi;
          } else {
            float remappedRX = 4.f * (1.f - rx);
            Sample_Quadrant(nu, nv, remappedRX, ry, phi, cos_theta);
            phi = 2.f * PI_F - phi;
          }
        }
        float sin_theta = ptm_sqrt(fmaxf(0.f, 1.f - cos_theta * cos_theta));
        V3 H = normalize(Spherical_Vector(sin_theta, cos_theta, phi));
        H = H.x * B + H.y * Nn + H.z * T;
        float HdotI = dot(H, Wo);
        if (HdotI < 0.f) H = -H;
        Wi = normalize(-Wo + 2.f * dot(Wo, H) * H);
      }
      return Wi;
    }
  }
  return v3(0.f);
}

V3 brdf_eval(const Material& m, V3 Wo, V3 Wi, V3 N, float& pdf) {
  switch (m.type) {
    case MAT_LAMBERTIAN: {  // programs/materials/lambertian.cuh:22-43
      float cosine = dot(normalize(Wi), normalize(N));
      if (cosine < 0.f) return v3(0.f);
      pdf = dot(normalize(Wi), normalize(N)) / PI_F;
      return (cosine * m.c0) / PI_F;
    }
    case MAT_DIFFUSE_LIGHT:  // programs/materials/diffuse_light.cuh:15-23
      pdf = 1.f;
      return m.c0;
    case MAT_OREN_NAYAR: {  // programs/materials/oren_nayar.cuh:22-66
      V3 WiN = normalize(Wi);
      float sinThetaI = SinTheta(WiN);
      float sinThetaO = SinTheta(Wo);
      float maxCos = 0;
      if (sinThetaI > 1e-4 && sinThetaO > 1e-4) {
        float sinPhiI = SinPhi(WiN), cosPhiI = CosPhi(WiN);
        float sinPhiO = SinPhi(Wo), cosPhiO = CosPhi(Wo);
        float dCos = cosPhiI * cosPhiO + sinPhiI * sinPhiO;
        maxCos = fmaxf(0.f, dCos);
      }
      float sinAlpha, tanBeta;
      if (AbsCosTheta(WiN) > AbsCosTheta(Wo)) {
        sinAlpha = sinThetaO;
        tanBeta = sinThetaI / AbsCosTheta(WiN);
      } else {
        sinAlpha = sinThetaI;
        tanBeta = sinThetaO / AbsCosTheta(Wo);
      }
      pdf = dot(normalize(Wi), normalize(N)) / PI_F;
      return m.c0 * (1.f / PI_F) * (m.p0 + m.p1 * maxCos * sinAlpha * tanBeta);
    }
    case MAT_TORRANCE_SPARROW: {  // programs/materials/torrance_sparrow.cuh:37-65
      V3 Rs = m.c0;
      float nu = m.p0, nv = m.p1;
      V3 Up = v3(0.f, 1.f, 0.f);
      float NdotI = fmaxf(dot(Up, Wi), 1e-6f), NdotO = fmaxf(dot(Up, Wo), 1e-6f);
      V3 H = Wo + Wi;
      if (isNull(H)) return v3(0.f);
      H = normalize(H);
      float HdotI = fabsf(dot(H, Wi));
      V3 F = schlick3(Rs, HdotI);
      float G = GGX_G(Wo, Wi, nu, nv);
      float D = GGX_D(H, nu, nv);
      pdf = GGX_PDF(H, nu, nv) / (4.f * dot(Wo, H));
      return Rs * D * G * F / (4.f * NdotI * NdotO);
    }
    case MAT_ASHIKHMIN_SHIRLEY: {  // programs/materials/ashikhmin_shirley.cuh:84-152
      V3 Rd = m.c0, Rs = m.c1;
      float nu = m.p0, nv = m.p1;
      V3 Up = v3(0.f, 1.f, 0.f);
      V3 Nn = normalize(N);
      V3 T = normalize(cross(Nn, Up));
      V3 B = cross(T, Nn);
      float NdotI = fabsf(dot(Up, Wi)), NdotO = fabsf(dot(Up, Wo));
      V3 diffuse_component = Rd * (28.f / (23.f * PI_F));
      diffuse_component *= (v3(1.f) - Rs);
      diffuse_component *= (1.f - pt_powf(1.f - NdotI * 0.5f, 5.f));
      diffuse_component *= (1.f - pt_powf(1.f - NdotO * 0.5f, 5.f));
      float diffuse_PDF = dot(Wi, Nn) / PI_F;
      if (diffuse_PDF < 0.f) return v3(0.f);
      V3 H = Wo + Wi;
      if (isNull(H)) return v3(0.f);
      H = normalize(H);
      float HdotI = fabsf(dot(H, Wi));
      float HdotN = fabsf(dot(H, Nn)), HdotT = fabsf(dot(H, T)), HdotB = fabsf(dot(H, B));
      float norm, lobe;
      if (nu == nv) {
        norm = (nu + 1.f) / (8.f * PI_F);
        lobe = pt_powf(HdotN, nu);
      } else {
        norm = ptm_sqrt((nu + 1.f) * (nv + 1.f)) / (8.f * PI_F);
        if (HdotN < 1.f)
          lobe = pt_powf(HdotN, (nu * HdotT * HdotT + nv * HdotB * HdotB) / (1.f - HdotN * HdotN));
        else
          lobe = 1.f;
      }
      V3 specular_component = schlick3(Rs, HdotI);
      specular_component *= norm;
      specular_component *= lobe / (HdotI * fmaxf(NdotI, NdotO));
      float specular_PDF = HdotI / (norm * lobe);
      pdf = (diffuse_PDF + specular_PDF) / 2.f;
      return (diffuse_component / diffuse_PDF) + (specular_component / specular_PDF);
    }
  }
  pdf = 0.f;
  return v3(0.f);
}

// ------------------------------------------------------------- integrator --

// ========================================================= consistent mode ==
// Unbiased variant: BRDFs evaluated in the local frame of the shading normal
// (y up, the reference's trig conventions applied to local vectors), pdfs
// that match the samplers, no throughput clamps, next-event estimation with
// MIS (power heuristic) against BSDF sampling for area lights and the
// importance-sampled environment.  Lights are two-sided emitters.

void build_env_cdf(Scene& s) {
  EnvCdf& E = s.env_cdf;
  E = EnvCdf();
  const Miss& m = s.miss;
  if (m.type != MISS_ENV || !m.spherical || m.w <= 0 || m.h <= 0) return;
  int W = m.w, H = m.h;
  E.w = W;
  E.h = H;
  E.cond.assign((size_t)H * (W + 1), 0.f);
  E.marg.assign(H + 1, 0.f);
  std::vector<double> rows(H);
  std::vector<double> pre(W + 1);
  for (int r = 0; r < H; r++) {
    float theta = PI_F * (((float)r + 0.5f) / (float)H);
    double sn = (double)pt_sinf(theta);
    double acc = 0.0;
    pre[0] = 0.0;
    for (int c = 0; c < W; c++) {
      const float* t = &m.env[((size_t)r * W + c) * 4];
      double lum = 0.2126 * (double)t[0] + 0.7152 * (double)t[1] + 0.0722 * (double)t[2];
      if (!(lum > 0.0)) lum = 0.0;
      acc = acc + lum * sn;
      pre[c + 1] = acc;
    }
    rows[r] = acc;
    float* cr = &E.cond[(size_t)r * (W + 1)];
    for (int c = 0; c <= W; c++)
      cr[c] = acc > 0.0 ? (float)(pre[c] / acc) : (float)((double)c / (double)W);
    cr[W] = 1.f;
  }
  double tot = 0.0;
  std::vector<double> mp(H + 1);
  mp[0] = 0.0;
  for (int r = 0; r < H; r++) {
    tot = tot + rows[r];
    mp[r + 1] = tot;
  }
  if (!(tot > 0.0)) return;
  for (int r = 0; r <= H; r++) E.marg[r] = (float)(mp[r] / tot);
  E.marg[H] = 1.f;
  E.valid = true;
}

// largest i in [0, n) with cdf[i] <= u (cdf[0] = 0 <= u < cdf[n] = 1)
inline int cdf_find(const float* cdf, int n, float u) {
  int lo = 0, hi = n;  // invariant: cdf[lo] <= u < cdf[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (cdf[mid] <= u) lo = mid;
    else hi = mid;
  }
  return lo;
}

// direction -> (u, v) of the spherical mapping (programs/miss.cu:66-77)
inline void env_uv(V3 d, float& u, float& v) {
  float r = length(d);
  float lon = pt_atan2f(d.z, d.x);
  float lat = pt_acosf(d.y / r);
  u = lon * (1.f / (PI_F * 2.f));
  v = lat * (1.f / PI_F);
}

float env_pdf_dir(const EnvCdf& E, V3 d) {
  if (!E.valid) return 0.f;
  float u, v;
  env_uv(d, u, v);
  if (!(u == u) || !(v == v)) return 0.f;
  if (u < 0.f) u += 1.f;
  int r = (int)(v * (float)E.h);
  if (r < 0) r = 0;
  if (r >= E.h) r = E.h - 1;
  int c = (int)(u * (float)E.w);
  if (c < 0) c = 0;
  if (c >= E.w) c = E.w - 1;
  const float* cr = &E.cond[(size_t)r * (E.w + 1)];
  float pm = E.marg[r + 1] - E.marg[r];
  float pc = cr[c + 1] - cr[c];
  float theta = PI_F * (((float)r + 0.5f) / (float)E.h);
  float st = pt_sinf(theta);
  if (!(st > 0.f)) return 0.f;
  return pm * pc * (float)E.w * (float)E.h / (2.f * PI_F * PI_F * st);
}

V3 env_sample_dir(const EnvCdf& E, float u1, float u2) {
  int r = cdf_find(E.marg.data(), E.h, u1);
  float dv = (u1 - E.marg[r]) / (E.marg[r + 1] - E.marg[r]);
  const float* cr = &E.cond[(size_t)r * (E.w + 1)];
  int c = cdf_find(cr, E.w, u2);
  float du = (u2 - cr[c]) / (cr[c + 1] - cr[c]);
  float v = ((float)r + dv) / (float)E.h;
  float u = ((float)c + du) / (float)E.w;
  float st, ct, sp, cp;
  pt_sincosf(PI_F * v, &st, &ct);
  pt_sincosf(2.f * PI_F * u, &sp, &cp);
  return v3(st * cp, ct, st * sp);
}

struct Frame {
  V3 t, n, b;
  explicit Frame(V3 N) {
    Onb o(N);
    t = o.t;
    n = o.n;
    b = o.b;
  }
  V3 to_local(V3 w) const { return v3(dot(w, t), dot(w, n), dot(w, b)); }
  V3 to_world(V3 l) const { return l.x * t + l.y * n + l.z * b; }
};

inline float GGX_G1c(V3 V, float nu, float nv) { return 1.f / (1.f + GGX_Lambda(V, nu, nv)); }

// BSDF value f (no cosine) for local y-up directions.
V3 bsdf_f_c(const Material& m, V3 wo, V3 wi) {
  if (!(wo.y > 0.f) || !(wi.y > 0.f)) return v3(0.f);
  switch (m.type) {
    case MAT_LAMBERTIAN:
      return m.c0 * (1.f / PI_F);
    case MAT_OREN_NAYAR: {
      float sinThetaI = SinTheta(wi), sinThetaO = SinTheta(wo);
      float maxCos = 0;
      if (sinThetaI > 1e-4 && sinThetaO > 1e-4) {
        float dCos = CosPhi(wi) * CosPhi(wo) + SinPhi(wi) * SinPhi(wo);
        maxCos = fmaxf(0.f, dCos);
      }
      float sinAlpha, tanBeta;
      if (AbsCosTheta(wi) > AbsCosTheta(wo)) {
        sinAlpha = sinThetaO;
        tanBeta = sinThetaI / AbsCosTheta(wi);
      } else {
        sinAlpha = sinThetaI;
        tanBeta = sinThetaO / AbsCosTheta(wo);
      }
      return m.c0 * (1.f / PI_F) * (m.p0 + m.p1 * maxCos * sinAlpha * tanBeta);
    }
    case MAT_TORRANCE_SPARROW: {
      V3 H = normalize(wo + wi);
      float D = GGX_D(H, m.p0, m.p1);
      float G = GGX_G(wo, wi, m.p0, m.p1);
      V3 F = schlick3(m.c0, fabsf(dot(H, wi)));
      return m.c0 * D * G * F / (4.f * wi.y * wo.y);
    }
    case MAT_ASHIKHMIN_SHIRLEY: {
      V3 Rd = m.c0, Rs = m.c1;
      float nu = m.p0, nv = m.p1;
      V3 diffuse = Rd * (28.f / (23.f * PI_F));
      diffuse *= (v3(1.f) - Rs);
      diffuse *= (1.f - pt_powf(1.f - wi.y * 0.5f, 5.f));
      diffuse *= (1.f - pt_powf(1.f - wo.y * 0.5f, 5.f));
      V3 H = normalize(wo + wi);
      float HdotI = fabsf(dot(H, wi));
      float HdotN = H.y;
      float norm = ptm_sqrt((nu + 1.f) * (nv + 1.f)) / (8.f * PI_F);
      float lobe = HdotN < 1.f
                       ? pt_powf(HdotN, (nu * H.x * H.x + nv * H.z * H.z) / (1.f - HdotN * HdotN))
                       : 1.f;
      V3 spec = schlick3(Rs, HdotI);
      spec *= norm;
      spec *= lobe / (HdotI * fmaxf(wi.y, wo.y));
      return diffuse + spec;
    }
  }
  return v3(0.f);
}

float bsdf_pdf_c(const Material& m, V3 wo, V3 wi) {
  if (!(wo.y > 0.f) || !(wi.y > 0.f)) return 0.f;
  switch (m.type) {
    case MAT_LAMBERTIAN:
    case MAT_OREN_NAYAR:
      return wi.y * (1.f / PI_F);
    case MAT_TORRANCE_SPARROW: {
      V3 H = normalize(wo + wi);
      float woh = dot(wo, H);
      if (!(woh > 0.f)) return 0.f;
      return GGX_G1c(wo, m.p0, m.p1) * GGX_D(H, m.p0, m.p1) / (4.f * wo.y);
    }
    case MAT_ASHIKHMIN_SHIRLEY: {
      float nu = m.p0, nv = m.p1;
      V3 H = normalize(wo + wi);
      float woh = dot(wo, H);
      float HdotN = H.y;
      float ph = 0.f;
      if (woh > 0.f && HdotN > 0.f) {
        float e = HdotN < 1.f ? (nu * H.x * H.x + nv * H.z * H.z) / (1.f - HdotN * HdotN) : 0.f;
        ph = ptm_sqrt((nu + 1.f) * (nv + 1.f)) / (2.f * PI_F) * pt_powf(HdotN, e);
        ph = ph / (4.f * woh);
      }
      return 0.5f * (wi.y * (1.f / PI_F)) + 0.5f * ph;
    }
  }
  return 0.f;
}

// local y-up direction sampled from the BSDF (draws two numbers)
V3 bsdf_sample_c(const Material& m, V3 wo, uint32_t& seed) {
  float rx = rnd(seed);
  float ry = rnd(seed);
  V3 p;
  switch (m.type) {
    case MAT_LAMBERTIAN:
    case MAT_OREN_NAYAR:
      cosine_sample_hemisphere(rx, ry, p);
      return v3(p.x, p.z, p.y);
    case MAT_TORRANCE_SPARROW: {
      V3 H = normalize(GGX_Sample(wo, rx, ry, m.p0, m.p1));
      if (dot(H, wo) < 0.f) H = -H;
      return -wo + 2.f * dot(wo, H) * H;
    }
    case MAT_ASHIKHMIN_SHIRLEY: {
      float nu = m.p0, nv = m.p1;
      if (rx < 0.5f) {
        rx = fminf(2.f * rx, 1.f - 1e-6f);
        cosine_sample_hemisphere(rx, ry, p);
        return v3(p.x, p.z, p.y);
      }
      rx = fminf(2.f * (rx - 0.5f), 1.f - 1e-6f);
      float phi, cos_theta;
      if (nu == nv) {
        phi = 2.f * PI_F * rx;
        cos_theta = pt_powf(ry, 1.f / (nu + 1.f));
      } else if (rx < 0.25f) {
        Sample_Quadrant(nu, nv, 4.f * rx, ry, phi, cos_theta);
      } else if (rx < 0.5f) {
        Sample_Quadrant(nu, nv, 4.f * (0.5f - rx), ry, phi, cos_theta);
        phi = PI_F - phi;
      } else if (rx < 0.75f) {
        Sample_Quadrant(nu, nv, 4.f * (rx - 0.5f), ry, phi, cos_theta);
        phi = PI_F + phi;
      } else {
        Sample_Quadrant(nu, nv, 4.f * (1.f - rx), ry, phi, cos_theta);
        phi = 2.f * PI_F - phi;
      }
      float sin_theta = ptm_sqrt(fmaxf(0.f, 1.f - cos_theta * cos_theta));
      V3 H = Spherical_Vector(sin_theta, cos_theta, phi);
      if (dot(H, wo) < 0.f) H = -H;
      return -wo + 2.f * dot(wo, H) * H;
    }
  }
  return v3(0.f, 1.f, 0.f);
}

// cone sampling toward a sphere light (consistent mode): direction to the
// sampled point on the cone (unnormalised) and the distance limit
inline V3 sphere_light_sample_c(const Light& L, V3 P, uint32_t& seed) {
  float r1 = rnd(seed);
  float r2 = rnd(seed);
  V3 dc = L.c - P;
  float dist2 = dot(dc, dc);
  float z = 1.f + r2 * (ptm_sqrt(fmaxf(0.f, 1.f - L.r * L.r / dist2)) - 1.f);
  float phi = 2.f * PI_F * r1;
  float sp, cp;
  pt_sincosf(phi, &sp, &cp);
  float sz = ptm_sqrt(fmaxf(0.f, 1.f - z * z));
  V3 w = v3(cp * sz, sp * sz, z);
  Onb uvw(normalize(dc));
  uvw.inverse_transform(w);
  return w;
}

inline float power_mis(float a, float b) { return (a * a) / (a * a + b * b); }

struct Params {
  int width, height, spp, frame0, max_depth, rr_enable, rr_depth, mode, guide;
};

enum { EV_BOUNCED = 0, EV_CANCELLED, EV_HIT_LIGHT, EV_MISSED };

struct PRD {
  uint32_t seed;
  float time;
  V3 throughput, radiance;
  int scatterEvent;
  bool isSpecular;
  V3 origin, direction;
};

struct Tracer {
  const Scene& s;
  Counters* cnt;
  uint64_t ext = 0, shadow = 0;
  float tm = 0.f;  // the current path's time: every ray of the path carries it

  // Shadow test: true if occluded.  programs/hit.cu:16-24 under closest-hit.
  bool occluded(V3 P, V3 Wi, V3 N) {
    Ray r{P, Wi, 1e-3f, RAY_TMAX, tm};
    shadow++;
    Hit h = trace(s, r, cnt);
    if (h.prim < 0) return true;
    const Prim& p = s.prims[h.prim];
    bool is_light = s.mats[p.material].type == MAT_DIFFUSE_LIGHT;
    return !(is_light && dot(N, Wi) > 0.f);
  }

  // programs/materials/light_sample.cuh:27-103
  V3 direct_light(const Material& m, V3 P, V3 Wo, V3 N, bool isLight, uint32_t& seed) {
    V3 directLight = v3(0.f);
    int numLights = (int)s.lights.size();
    if (numLights == 0) return v3(0.f);
    int index = ((int)(rnd(seed) * numLights)) % numLights;
    if (isLight && numLights == 1) return v3(0.f);
    const Light& L = s.lights[index];
    V3 emission = L.emission;
    V3 Wi = light_sample(L, P, seed);
    float lightPDF = light_pdf(L, P, Wi);
    if (dot(Wi, N) < 0.f) return v3(0.f);
    if (occluded(P, Wi, N)) return v3(0.f);
    if (lightPDF != 0.f && !isNull(emission)) {
      float matPDF = 0.f;
      V3 matValue = brdf_eval(m, Wo, Wi, N, matPDF);
      if (matPDF != 0.f && !isNull(matValue)) {
        float f = 1u * lightPDF, g = 1u * matPDF;
        float weight = (f * f) / (f * f + g * g);
        directLight += matValue * emission * weight / lightPDF;
      }
    }
    Wi = brdf_sample(m, Wo, N, seed);
    float matPDF = 0.f;
    V3 matValue = brdf_eval(m, Wo, Wi, N, matPDF);
    if (matPDF != 0.f && !isNull(matValue)) {
      lightPDF = light_pdf(L, P, Wi);
      if (!lightPDF || isNull(emission)) return directLight;
      float f = 1u * matPDF, g = 1u * lightPDF;
      float weight = (f * f) / (f * f + g * g);
      directLight += matValue * emission * weight / matPDF;
    }
    return directLight;
  }

  V3 env_lookup(float u, float v) {
    const Miss& ms = s.miss;
    if (!(u == u) || !(v == v) || fabsf(u) > 1e6f || fabsf(v) > 1e6f) return v3(0.f);
    float x = u * (float)ms.w - 0.5f, y = v * (float)ms.h - 0.5f;
    float fx = ptm_floor(x), fy = ptm_floor(y);
    float ax = x - fx, ay = y - fy;
    int ix0 = (int)fx % ms.w; if (ix0 < 0) ix0 += ms.w;
    int iy0 = (int)fy % ms.h; if (iy0 < 0) iy0 += ms.h;
    int ix1 = ix0 + 1 == ms.w ? 0 : ix0 + 1;
    int iy1 = iy0 + 1 == ms.h ? 0 : iy0 + 1;
    const float* e = ms.env.data();
    V3 c00 = v3(e[(iy0 * ms.w + ix0) * 4], e[(iy0 * ms.w + ix0) * 4 + 1], e[(iy0 * ms.w + ix0) * 4 + 2]);
    V3 c10 = v3(e[(iy0 * ms.w + ix1) * 4], e[(iy0 * ms.w + ix1) * 4 + 1], e[(iy0 * ms.w + ix1) * 4 + 2]);
    V3 c01 = v3(e[(iy1 * ms.w + ix0) * 4], e[(iy1 * ms.w + ix0) * 4 + 1], e[(iy1 * ms.w + ix0) * 4 + 2]);
    V3 c11 = v3(e[(iy1 * ms.w + ix1) * 4], e[(iy1 * ms.w + ix1) * 4 + 1], e[(iy1 * ms.w + ix1) * 4 + 2]);
    return (c00 * (1.f - ax) + c10 * ax) * (1.f - ay) + (c01 * (1.f - ax) + c11 * ax) * ay;
  }

  // programs/miss.cu:30-95
  void miss(PRD& prd, const Ray& ray) {
    const Miss& ms = s.miss;
    if (ms.type == MISS_GRADIENT) {
      V3 unit_direction = normalize(ray.d);
      float t = 0.5f * (unit_direction.y + 1.f);
      V3 c = (1.f - t) * ms.c1;
      c += t * ms.c2;
      prd.throughput *= c;
    } else if (ms.type == MISS_CONSTANT) {
      prd.throughput *= ms.c1;
    } else if (ms.type == MISS_IMAGE) {
      float theta = pt_atan2f(ray.d.x, ray.d.z);
      float phi = PTM_PI * 0.5f - pt_acosf(ray.d.y);
      float u = (theta + PTM_PI) * (0.5f * (1.0f / PTM_PI));
      float v = 0.5f * (1.f + pt_sinf(phi));
      prd.throughput *= env_lookup(u, v);
    } else {
      float u, v;
      if (ms.spherical) {
        float r = length(ray.d);
        float lon = pt_atan2f(ray.d.z, ray.d.x);
        float lat = pt_acosf(ray.d.y / r);
        u = lon * (1.f / (PI_F * 2.f));
        v = lat * (1.f / PI_F);
      } else {
        float theta = pt_atan2f(ray.d.x, ray.d.z);
        theta = theta < 0.f ? theta + (2.f * PI_F) : theta;
        float phi = pt_acosf(ray.d.y);
        u = 1.f - (theta / (2.f * PI_F));
        v = phi / PI_F;
      }
      prd.throughput *= 2.f * env_lookup(u, v);
    }
    prd.scatterEvent = EV_MISSED;
  }

  // closest-hit programs of programs/materials/*.cu
  void closest_hit(PRD& prd, const Ray& ray, const Hit& h) {
    const Prim& p = s.prims[h.prim];
    HitRecord rec = hit_record(s, p, ray, h.t, h.u, h.v);
    Material m = s.mats[rec.index];
    resolve_textures(s, m, rec);
    V3 P = rec.P, Wo = rec.Wo, N = rec.shading_normal;
    switch (m.type) {
      case MAT_LAMBERTIAN:     // programs/materials/lambertian.cu:49-73
      case MAT_OREN_NAYAR: {   // programs/materials/oren_nayar.cu:46-70
        V3 direct = direct_light(m, P, Wo, N, false, prd.seed);
        prd.radiance += prd.throughput * direct;
        V3 Wi = brdf_sample(m, Wo, N, prd.seed);
        float pdf = 0.f;
        V3 attenuation = brdf_eval(m, Wo, Wi, N, pdf);
        prd.scatterEvent = EV_BOUNCED;
        prd.origin = P;
        prd.direction = Wi;
        prd.throughput *= clamp3(attenuation / pdf, 0.f, 1.f);
        prd.isSpecular = false;
        break;
      }
      case MAT_METAL: {  // programs/materials/metal.cu:38-56
        V3 reflected = reflect(-Wo, N);
        prd.direction = reflected + m.p0 * random_in_unit_sphere(prd.seed);
        prd.scatterEvent = EV_BOUNCED;
        prd.origin = P;
        prd.throughput *= m.c0;
        prd.isSpecular = true;
        break;
      }
      case MAT_DIELECTRIC: {  // programs/materials/dielectric.cu:46-96
        float ref_idx = m.p0;
        V3 Wd = -rec.Wo;
        V3 Nd = N;
        V3 absorption = v3(1.f);
        float ni_over_nt;
        float cosine = dot(Wd, Nd);
        if (cosine > 0.f) {
          Nd = -Nd;
          ni_over_nt = ref_idx;
          cosine = ref_idx * cosine / length(Wd);
        } else {
          ni_over_nt = 1.f / ref_idx;
          cosine = -cosine / length(Wd);
        }
        V3 refracted = v3(0.f);
        float reflect_prob;
        if (Refract(Wd, Nd, ni_over_nt, refracted))
          reflect_prob = schlick(cosine, ref_idx);
        else
          reflect_prob = 1.f;
        if (rnd(prd.seed) < reflect_prob)
          prd.direction = reflect(Wd, Nd);
        else
          prd.direction = normalize(refracted);
        prd.scatterEvent = EV_BOUNCED;
        prd.origin = P;
        prd.throughput *= (m.c0 * absorption);
        prd.isSpecular = true;
        break;
      }
      case MAT_DIFFUSE_LIGHT: {  // programs/materials/diffuse_light.cu:30-48
        V3 direct = direct_light(m, P, Wo, N, true, prd.seed);
        prd.radiance += prd.throughput * direct;
        if (dot(N, Wo) < 0.f) prd.throughput *= m.c0;
        prd.scatterEvent = EV_HIT_LIGHT;
        break;
      }
      case MAT_TORRANCE_SPARROW: {  // programs/materials/torrance_sparrow.cu:39-59
        V3 Wi = brdf_sample(m, Wo, N, prd.seed);
        float pdf = 0.f;
        V3 attenuation = brdf_eval(m, Wo, Wi, N, pdf);
        prd.scatterEvent = EV_BOUNCED;
        prd.origin = P;
        prd.direction = Wi;
        prd.throughput *= clamp3(attenuation / pdf, 0.f, 1.f);
        prd.isSpecular = true;
        break;
      }
      case MAT_ASHIKHMIN_SHIRLEY: {  // programs/materials/ashikhmin_shirley.cu:48-68
        V3 Wi = brdf_sample(m, Wo, N, prd.seed);
        float pdf = 0.f;
        V3 attenuation = brdf_eval(m, Wo, Wi, N, pdf);
        prd.scatterEvent = EV_BOUNCED;
        prd.origin = P;
        prd.direction = Wi;
        prd.throughput *= clamp3(attenuation, 0.f, 1.f);
        prd.isSpecular = true;
        break;
      }
      default:
        prd.scatterEvent = EV_CANCELLED;
    }
  }

  // programs/raygen.cu:66-123
  V3 color(Ray ray, uint32_t seed, const Params& pr) {
    PRD prd;
    prd.seed = seed;
    prd.time = s.cam.time0 + rnd(prd.seed) * (s.cam.time1 - s.cam.time0);
    tm = prd.time;
    ray.time = tm;
    prd.throughput = v3(1.f);
    prd.radiance = v3(0.f);
    prd.isSpecular = false;
    bool previousHitSpecular = false;
    for (int depth = 0; depth < pr.max_depth; depth++) {
      ext++;
      Hit h = trace(s, ray, cnt);
      if (h.prim < 0) miss(prd, ray);
      else closest_hit(prd, ray, h);
      if (prd.scatterEvent == EV_MISSED)
        return prd.radiance + clamp3(prd.throughput, 0.f, 1.f);
      else if (prd.scatterEvent == EV_HIT_LIGHT) {
        if (depth == 0 || previousHitSpecular) prd.radiance += prd.throughput;
        return prd.radiance;
      } else if (prd.scatterEvent == EV_CANCELLED) {
        return prd.radiance;
      } else {
        ray = Ray{prd.origin, prd.direction, 1e-3f, RAY_TMAX, tm};
        previousHitSpecular = prd.isSpecular;
      }
      if (pr.rr_enable) {
        float prob = max_component(prd.throughput);
        if (depth > pr.rr_depth) {
          if (rnd(prd.seed) >= prob)
            return prd.radiance + prd.throughput;
          else
            prd.throughput *= 1.f / prob;
        }
      }
    }
    return v3(0.f);
  }


  // sum over lights of the light-sampling pdf of direction d from P (per
  // selection), for MIS at emitter hits and misses
  float lights_pdf_c(V3 P, V3 d, int n_sel) {
    float acc = 0.f;
    for (size_t k = 0; k < s.lights.size(); k++) acc += light_pdf(s.lights[k], P, d);
    return acc / (float)n_sel;
  }

  V3 color_c(Ray ray, uint32_t seed, const Params& pr) {
    tm = s.cam.time0 + rnd(seed) * (s.cam.time1 - s.cam.time0);
    ray.time = tm;
    V3 thr = v3(1.f), rad = v3(0.f);
    bool prev_spec = true;
    float pdf_prev = 0.f;
    const bool env_is = s.env_cdf.valid;
    const int n_lights = (int)s.lights.size();
    const int n_sel = n_lights + (env_is ? 1 : 0);
    for (int depth = 0; depth < pr.max_depth; depth++) {
      ext++;
      Hit h = trace(s, ray, cnt);
      if (h.prim < 0) {
        PRD prd;
        prd.throughput = v3(1.f);
        miss(prd, ray);  // radiance multiplier of the miss programs
        float w = 1.f;
        if (!prev_spec && env_is) w = power_mis(pdf_prev, env_pdf_dir(s.env_cdf, ray.d) / (float)n_sel);
        rad += thr * prd.throughput * w;
        break;
      }
      const Prim& p = s.prims[h.prim];
      HitRecord rec = hit_record(s, p, ray, h.t, h.u, h.v);
      Material m = s.mats[rec.index];
      resolve_textures(s, m, rec);
      V3 P = rec.P, Wo = rec.Wo, N = rec.shading_normal;
      if (m.type == MAT_DIFFUSE_LIGHT) {
        float w = 1.f;
        if (!prev_spec && n_sel > 0) w = power_mis(pdf_prev, lights_pdf_c(ray.o, ray.d, n_sel));
        rad += thr * m.c0 * w;
        break;
      }
      if (m.type == MAT_METAL || m.type == MAT_DIELECTRIC) {
        PRD prd;
        prd.seed = seed;
        prd.throughput = thr;
        prd.radiance = rad;
        closest_hit(prd, ray, h);
        seed = prd.seed;
        thr = prd.throughput;
        ray = Ray{prd.origin, prd.direction, 1e-3f, RAY_TMAX, tm};
        prev_spec = true;
      } else {
        Frame fr(N);
        V3 wo_l = fr.to_local(Wo);
        // next-event estimation
        if (n_sel > 0) {
          int k = (int)(rnd(seed) * (float)n_sel);
          if (k > n_sel - 1) k = n_sel - 1;
          V3 Wi;
          float pl = 0.f, tmax = RAY_TMAX;
          V3 Le;
          if (k < n_lights) {
            const Light& L = s.lights[k];
            if (L.type == LIGHT_RECT) {
              Wi = light_sample(L, P, seed);
              tmax = 1.f - 1e-4f;
            } else {
              Wi = sphere_light_sample_c(L, P, seed);
              float a = dot(Wi, Wi), b = dot(P - L.c, Wi);
              float c = dot(P - L.c, P - L.c) - L.r * L.r;
              float disc = b * b - a * c;
              float tn = disc >= 0.f ? (-b - ptm_sqrt(disc)) / a : 0.f;
              tmax = tn * (1.f - 1e-4f);
            }
            pl = light_pdf(L, P, Wi);
            Le = L.emission;
          } else {
            float u1 = rnd(seed);
            float u2 = rnd(seed);
            Wi = env_sample_dir(s.env_cdf, u1, u2);
            pl = env_pdf_dir(s.env_cdf, Wi);
            PRD q;
            q.throughput = v3(1.f);
            miss(q, Ray{P, Wi, 1e-3f, RAY_TMAX});
            Le = q.throughput;
          }
          V3 wi_n = normalize(Wi);
          float cs = dot(wi_n, N);
          float pls = pl / (float)n_sel;
          if (cs > 0.f && pls > 0.f && tmax > 1e-3f) {
            V3 wi_l = fr.to_local(wi_n);
            V3 f = bsdf_f_c(m, wo_l, wi_l);
            float pb = bsdf_pdf_c(m, wo_l, wi_l);
            V3 c = f * Le * (cs * power_mis(pls, pb) / pls);
            if (!isNull(c)) {
              shadow++;
              Ray sr{P, Wi, 1e-3f, tmax, tm};
              Hit sh = trace(s, sr, cnt);
              if (sh.prim < 0) rad += thr * c;
            }
          }
        }
        // BSDF continuation
        V3 wi_l = bsdf_sample_c(m, wo_l, seed);
        float pb = bsdf_pdf_c(m, wo_l, wi_l);
        V3 f = bsdf_f_c(m, wo_l, wi_l);
        if (!(pb > 0.f) || isNull(f) || !(wi_l.y > 0.f)) break;
        thr *= f * (wi_l.y / pb);
        prev_spec = false;
        pdf_prev = pb;
        ray = Ray{P, fr.to_world(wi_l), 1e-3f, RAY_TMAX, tm};
      }
      if (pr.rr_enable && depth > pr.rr_depth) {
        float q = fminf(1.f, max_component(thr));
        if (rnd(seed) >= q) break;
        thr *= 1.f / q;
      }
    }
    return rad;
  }

  // programs/raygen.cu:50-64 + 148-165; returns the path's colour
  Ray camera_ray(uint32_t x, uint32_t y, uint32_t W, uint32_t H, uint32_t& seed) {
    float u = float((float)x + rnd(seed)) / (float)W;
    float v = float((float)y + rnd(seed)) / (float)H;
    const Cam& c = s.cam;
    V3 rd = c.lens_radius * random_in_unit_disk(seed);
    V3 lens_offset = c.u * rd.x + c.v * rd.y;
    V3 origin = c.origin + lens_offset;
    V3 direction = c.llc + u * c.horizontal + v * c.vertical - origin;
    return Ray{origin, direction, 1e-6f, RAY_TMAX};
  }

  V3 render_path(uint32_t x, uint32_t y, const Params& pr, int frame) {
    uint32_t W = pr.width, H = pr.height;
    uint32_t seed = tea64(W * y + x, (uint32_t)frame);
    Ray ray = camera_ray(x, y, W, H, seed);
    V3 col = pr.mode == 1 ? color_c(ray, seed, pr) : color(ray, seed, pr);
    if (!(col.x == col.x)) col.x = 0.f;  // de_nan, programs/raygen.cu:126-134
    if (!(col.y == col.y)) col.y = 0.f;
    if (!(col.z == col.z)) col.z = 0.f;
    return col;
  }
};

}  // namespace

// ================================================================== C API ==
extern "C" {

void* or_create(void) { return new Scene(); }
void or_destroy(void* s) { delete (Scene*)s; }

// type: MAT_*; c0/c1: colours; p0/p1 as the host classes take them
// (materials.hpp:173-174,194-197,235-238 conversions applied here).
int or_add_material(void* sp, int type, const float* c0, const float* c1, float p0, float p1) {
  Scene& s = *(Scene*)sp;
  Material m;
  m.type = type;
  m.c0 = c0 ? v3(c0[0], c0[1], c0[2]) : v3(0.f);
  m.c1 = c1 ? v3(c1[0], c1[1], c1[2]) : v3(0.f);
  m.p0 = p0;
  m.p1 = p1;
  if (type == MAT_OREN_NAYAR) {
    float sigma = ffmax(0.f, ffmin(1.f, p0));
    float div = 1.f / (PI_F + ((3.f * PI_F - 4.f) / 6.f) * sigma);
    m.p0 = 1.0f * div;
    m.p1 = sigma * div;
  } else if (type == MAT_TORRANCE_SPARROW) {
    float R0 = fmaxf(p0, 1e-3f), R1 = fmaxf(p1, 1e-3f);
    m.p0 = R0 * R0;
    m.p1 = R1 * R1;
  } else if (type == MAT_ASHIKHMIN_SHIRLEY) {
    m.p0 = fmaxf(1.f, p0);
    m.p1 = fmaxf(1.f, p1);
  }
  s.mats.push_back(m);
  return (int)s.mats.size() - 1;
}

static int add_xform(Scene& s, const float* x) {
  if (!x) return -1;
  Xform xf;
  memcpy(xf.m, x, sizeof(xf.m));
  affine_inverse(xf.m, xf.inv);
  s.xforms.push_back(xf);
  return (int)s.xforms.size() - 1;
}

// type PRIM_SPHERE: f = cx,cy,cz,r; PRIM_RECT: a0,a1,b0,b1,k (axis, flip);
// PRIM_BOX: x0,y0,z0,x1,y1,z1; PRIM_MSPHERE: c0 (3), r, t0, t1, c1 (3).
// Returns the primitive id.
int or_add_prim(void* sp, int type, const float* f, int axis, int flip, int material,
                const float* xform) {
  Scene& s = *(Scene*)sp;
  Prim p;
  memset(&p, 0, sizeof(p));
  p.type = type;
  p.axis = axis;
  p.flip = flip;
  p.material = material;
  p.mesh = -1;
  memcpy(p.f, f, sizeof(float) * (type == PRIM_SPHERE ? 4 : (type == PRIM_RECT ? 5 : (type == PRIM_MSPHERE ? 9 : 6))));
  p.xform = add_xform(s, xform);
  s.prims.push_back(p);
  return (int)s.prims.size() - 1;
}

int or_add_mesh(void* sp, const float* verts, int nv, const uint32_t* idx, int nt,
                const int32_t* mat_per_tri, int material, const float* normals,
                const float* uvs, const float* xform) {
  Scene& s = *(Scene*)sp;
  Mesh mesh;
  std::vector<V3> wv(nv);
  float inv[12];
  if (xform) affine_inverse(xform, inv);
  for (int i = 0; i < nv; i++) {
    V3 v = v3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
    wv[i] = xform ? xpoint(xform, v) : v;
  }
  if (normals) {
    mesh.normals.resize(nv);
    for (int i = 0; i < nv; i++) {
      V3 n = v3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
      mesh.normals[i] = xform ? xnormal(inv, n) : n;
    }
  }
  if (uvs) mesh.uvs.assign(uvs, uvs + 2 * nv);
  s.meshes.push_back(mesh);
  int mid = (int)s.meshes.size() - 1;
  int first = (int)s.prims.size();
  for (int t = 0; t < nt; t++) {
    Prim p;
    memset(&p, 0, sizeof(p));
    p.type = PRIM_TRIANGLE;
    p.material = mat_per_tri ? mat_per_tri[t] : material;
    p.xform = -1;
    p.mesh = mid;
    for (int k = 0; k < 3; k++) {
      uint32_t vi = idx[3 * t + k];
      p.vi[k] = (int32_t)vi;
      p.f[3 * k] = wv[vi].x;
      p.f[3 * k + 1] = wv[vi].y;
      p.f[3 * k + 2] = wv[vi].z;
    }
    s.prims.push_back(p);
  }
  return first;
}

// A texture (kind TEX_*): ints a, b as the kind uses them (checker: odd,
// even; vector: -, size with `ids` its entries; image: w, h; noise: axis),
// c[9] its colours / scale, data: image rgba (w*h*4) or noise ranvec
// (768 floats), perm: noise permutations (768 ints).  Returns the id.
int or_add_texture(void* sp, int kind, int a, int b, const float* c, const float* data,
                   const int32_t* perm, const uint32_t* ids) {
  Scene& s = *(Scene*)sp;
  Texture t;
  t.kind = kind;
  t.a = a;
  t.b = b;
  if (c) memcpy(t.c, c, sizeof(t.c));
  if (kind == TEX_IMAGE) t.data.assign(data, data + (size_t)a * b * 4);
  if (kind == TEX_NOISE) {
    t.data.assign(data, data + 768);
    t.perm.assign(perm, perm + 768);
  }
  if (kind == TEX_VECTOR) {
    t.a = (int)s.tex_list.size();
    for (int k = 0; k < b; k++) s.tex_list.push_back((int)ids[k]);
  }
  s.textures.push_back(t);
  return (int)s.textures.size() - 1;
}

void or_material_set_texture(void* sp, int material, int slot, int texture) {
  Scene& s = *(Scene*)sp;
  (slot == 0 ? s.mats[material].tex0 : s.mats[material].tex1) = texture;
}

void or_mesh_set_texture_index(void* sp, int first_prim, int n, const uint32_t* index) {
  Scene& s = *(Scene*)sp;
  for (int k = 0; k < n; k++) s.prims[first_prim + k].tindex = (int)index[k];
}

// type LIGHT_RECT: f = a0,a1,b0,b1,k (axis); LIGHT_SPHERE: cx,cy,cz,r.
int or_add_light(void* sp, int type, const float* f, int axis, const float* emission) {
  Scene& s = *(Scene*)sp;
  Light L;
  memset(&L, 0, sizeof(L));
  L.type = type;
  L.axis = axis;
  if (type == LIGHT_RECT) {
    L.a0 = f[0]; L.a1 = f[1]; L.b0 = f[2]; L.b1 = f[3]; L.k = f[4];
  } else {
    L.c = v3(f[0], f[1], f[2]);
    L.r = f[3];
  }
  L.emission = v3(emission[0], emission[1], emission[2]);
  s.lights.push_back(L);
  return (int)s.lights.size() - 1;
}

void or_set_miss(void* sp, int type, const float* c1, const float* c2, const float* env,
                 int w, int h, int spherical) {
  Scene& s = *(Scene*)sp;
  s.miss.type = type;
  if (c1) s.miss.c1 = v3(c1[0], c1[1], c1[2]);
  if (c2) s.miss.c2 = v3(c2[0], c2[1], c2[2]);
  if (env) {
    s.miss.env.assign(env, env + (size_t)w * h * 4);
    s.miss.w = w;
    s.miss.h = h;
  }
  s.miss.spherical = spherical;
}

// host_includes/camera.hpp:13-38
void or_set_camera(void* sp, const float* from, const float* at, const float* up, float vfov,
                   float aspect, float aperture, float focus_dist, float t0, float t1) {
  Scene& s = *(Scene*)sp;
  Cam& c = s.cam;
  V3 lookfrom = v3(from[0], from[1], from[2]), lookat = v3(at[0], at[1], at[2]),
     vup = v3(up[0], up[1], up[2]);
  c.lens_radius = aperture / 2.f;
  c.time0 = t0;
  c.time1 = t1;
  float theta = vfov * PI_F / 180.f;
  float half_height = pt_tanf(theta / 2.f);
  float half_width = aspect * half_height;
  c.origin = lookfrom;
  c.w = unit_vector(lookfrom - lookat);
  c.u = unit_vector(cross(vup, c.w));
  c.v = cross(c.w, c.u);
  c.llc = c.origin - half_width * focus_dist * c.u - half_height * focus_dist * c.v -
          focus_dist * c.w;
  c.horizontal = 2.f * half_width * focus_dist * c.u;
  c.vertical = 2.f * half_height * focus_dist * c.v;
}

int or_commit(void* sp) {
  Scene& s = *(Scene*)sp;
  build_env_cdf(s);
  s.nodes.clear();
  s.order.resize(s.prims.size());
  for (size_t i = 0; i < s.prims.size(); i++) s.order[i] = (int)i;
  if (s.prims.empty()) { s.committed = true; return 0; }
  std::vector<AABB> boxes(s.prims.size());
  for (size_t i = 0; i < s.prims.size(); i++) boxes[i] = prim_bounds(s, s.prims[i]);
  s.nodes.reserve(2 * s.prims.size());
  Builder b(boxes, s.order, s.nodes);
  b.build(0, (int)s.prims.size());
  s.committed = true;
  return (int)s.nodes.size();
}

// First hit of frame `frame` for every pixel (camera ray with the jitter of
// that frame): primitive id (-1 on miss), material id (-1), t.
void or_first_hits(void* sp, int W, int H, int frame, int32_t* prim, int32_t* mat, float* tout,
                   int threads) {
  Scene& s = *(Scene*)sp;
  Tracer base{s, nullptr};
  (void)base;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
  for (int p = 0; p < W * H; p++) {
    Tracer tr{s, nullptr};
    uint32_t x = p % W, y = p / W;
    uint32_t seed = tea64((uint32_t)W * y + x, (uint32_t)frame);
    Ray ray = tr.camera_ray(x, y, W, H, seed);
    ray.time = s.cam.time0 + rnd(seed) * (s.cam.time1 - s.cam.time0);  // color()'s prd.time
    Hit h = trace(s, ray, nullptr);
    prim[p] = h.prim;
    mat[p] = h.prim >= 0 ? s.prims[h.prim].material : -1;
    tout[p] = h.prim >= 0 ? h.t : 0.f;
  }
}

// Per-path radiance of frame `frame` for the listed pixels (index y*W+x).
void or_render_paths(void* sp, const int* params, int frame, const uint32_t* pix, int n,
                     float* out_rgb, int threads) {
  Scene& s = *(Scene*)sp;
  Params pr;
  memcpy(&pr, params, sizeof(pr));
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
  for (int i = 0; i < n; i++) {
    Tracer tr{s, nullptr};
    uint32_t x = pix[i] % pr.width, y = pix[i] / pr.width;
    V3 c = tr.render_path(x, y, pr, frame);
    out_rgb[3 * i] = c.x;
    out_rgb[3 * i + 1] = c.y;
    out_rgb[3 * i + 2] = c.z;
  }
}

// Progressive render of frames frame0 .. frame0+spp-1 into acc (W*H float4,
// y-flipped like programs/raygen.cu:153).  Only pixels with index
// p % pixel_stride == pixel_offset are rendered (bounded CPU samples).
// stats[0] = extension rays, stats[1] = shadow rays, stats[2] = paths.
double or_render(void* sp, const int* params, float* acc, int pixel_stride, int pixel_offset,
                 int threads, uint64_t* stats) {
  Scene& s = *(Scene*)sp;
  Params pr;
  memcpy(&pr, params, sizeof(pr));
  int W = pr.width, H = pr.height;
  if (pixel_stride < 1) pixel_stride = 1;
  std::atomic<uint64_t> ext{0}, sh{0}, paths{0};
  auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel num_threads(threads)
  {
    Tracer tr{s, nullptr};
    uint64_t np = 0;
#pragma omp for schedule(dynamic, 16)
    for (int p = pixel_offset; p < W * H; p += pixel_stride) {
      uint32_t x = p % W, y = p / W;
      size_t o = ((size_t)(H - 1 - y) * W + x) * 4;
      if (pr.frame0 == 0) acc[o] = acc[o + 1] = acc[o + 2] = acc[o + 3] = 0.f;
      for (int f = pr.frame0; f < pr.frame0 + pr.spp; f++) {
        V3 c = tr.render_path(x, y, pr, f);
        acc[o] += c.x;
        acc[o + 1] += c.y;
        acc[o + 2] += c.z;
        acc[o + 3] += 1.f;
        np++;
      }
    }
    ext += tr.ext;
    sh += tr.shadow;
    paths += np;
  }
  auto t1 = std::chrono::steady_clock::now();
  if (stats) {
    stats[0] = ext;
    stats[1] = sh;
    stats[2] = paths;
  }
  return std::chrono::duration<double>(t1 - t0).count();
}

// Exposes the integer/elementary kernels for known-answer tests.
uint32_t or_tea64(uint32_t a, uint32_t b) { return tea64(a, b); }
void or_rnd_stream(uint32_t seed, int n, float* out) {
  for (int i = 0; i < n; i++) out[i] = rnd(seed);
}
void or_math(int fn, const float* x, const float* y, float* out, int n) {
  for (int i = 0; i < n; i++) {
    switch (fn) {
      case 0: out[i] = pt_sinf(x[i]); break;
      case 1: out[i] = pt_cosf(x[i]); break;
      case 2: out[i] = pt_tanf(x[i]); break;
      case 3: out[i] = pt_atanf(x[i]); break;
      case 4: out[i] = pt_atan2f(y[i], x[i]); break;
      case 5: out[i] = pt_asinf(x[i]); break;
      case 6: out[i] = pt_acosf(x[i]); break;
      case 7: out[i] = pt_powf(x[i], y[i]); break;
      case 8: out[i] = pt_exp2f(x[i]); break;
      case 9: out[i] = pt_log2f(x[i]); break;
    }
  }
}
// Single-ray closest hit for analytic known-answer tests.
int or_trace_ray(void* sp, const float* o, const float* d, float tmin, float* t, float* uv) {
  Scene& s = *(Scene*)sp;
  Ray r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2]), tmin, RAY_TMAX};
  Hit h = trace(s, r, nullptr);
  if (t) *t = h.t;
  if (uv) { uv[0] = h.u; uv[1] = h.v; }
  return h.prim;
}
// Shading frame of a hit for known-answer tests: P, shading normal, u, v.
int or_hit_record(void* sp, const float* o, const float* d, float* out) {
  Scene& s = *(Scene*)sp;
  Ray r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2]), 1e-6f, RAY_TMAX};
  Hit h = trace(s, r, nullptr);
  if (h.prim < 0) return -1;
  HitRecord rec = hit_record(s, s.prims[h.prim], r, h.t, h.u, h.v);
  out[0] = rec.P.x; out[1] = rec.P.y; out[2] = rec.P.z;
  out[3] = rec.shading_normal.x; out[4] = rec.shading_normal.y; out[5] = rec.shading_normal.z;
  out[6] = rec.u; out[7] = rec.v;
  return h.prim;
}

}  // extern "C"

// Consistent-mode BSDF of one material (user parameters, converted as the
// material constructors do) for local y-up directions: f (rgb) and pdf.
extern "C" void or_bsdf_c(int type, const float* c0, const float* c1, float p0, float p1,
                          const float* wo, const float* wi, float* f, float* pdf) {
  Scene tmp;
  int id = or_add_material(&tmp, type, c0, c1, p0, p1);
  const Material& m = tmp.mats[id];
  V3 a = v3(wo[0], wo[1], wo[2]), b = v3(wi[0], wi[1], wi[2]);
  V3 r = bsdf_f_c(m, a, b);
  f[0] = r.x;
  f[1] = r.y;
  f[2] = r.z;
  *pdf = bsdf_pdf_c(m, a, b);
}

// n samples of the consistent-mode BSDF sampler from one seed stream.
extern "C" void or_bsdf_sample_c(int type, const float* c0, const float* c1, float p0, float p1,
                                 const float* wo, uint32_t seed, int n, float* wi) {
  Scene tmp;
  int id = or_add_material(&tmp, type, c0, c1, p0, p1);
  const Material& m = tmp.mats[id];
  V3 a = v3(wo[0], wo[1], wo[2]);
  for (int k = 0; k < n; k++) {
    V3 r = bsdf_sample_c(m, a, seed);
    wi[3 * k] = r.x;
    wi[3 * k + 1] = r.y;
    wi[3 * k + 2] = r.z;
  }
}

// Environment sampling of a committed scene: n directions from n uniform
// pairs, and the pdf of each returned direction.
extern "C" int or_env_sample(void* sp, const float* u, int n, float* dirs, float* pdf) {
  Scene& s = *(Scene*)sp;
  if (!s.env_cdf.valid) return 0;
  for (int k = 0; k < n; k++) {
    V3 d = env_sample_dir(s.env_cdf, u[2 * k], u[2 * k + 1]);
    dirs[3 * k] = d.x;
    dirs[3 * k + 1] = d.y;
    dirs[3 * k + 2] = d.z;
    pdf[k] = env_pdf_dir(s.env_cdf, d);
  }
  return 1;
}

// Batched form of or_bsdf_c for quadrature checks.
extern "C" void or_bsdf_c_batch(int type, const float* c0, const float* c1, float p0, float p1,
                                const float* wo, int n, const float* wi, float* f, float* pdf) {
  Scene tmp;
  int id = or_add_material(&tmp, type, c0, c1, p0, p1);
  const Material& m = tmp.mats[id];
  V3 a = v3(wo[0], wo[1], wo[2]);
  for (int k = 0; k < n; k++) {
    V3 b = v3(wi[3 * k], wi[3 * k + 1], wi[3 * k + 2]);
    V3 r = bsdf_f_c(m, a, b);
    f[3 * k] = r.x;
    f[3 * k + 1] = r.y;
    f[3 * k + 2] = r.z;
    pdf[k] = bsdf_pdf_c(m, a, b);
  }
}

// ---------------------------------------------------------------------------
// Function-level entry points for the pins against the reference's own
// programs (oracle/refhost, tests/test_ref_pin.py).  Reference mode.
extern "C" void or_lcg_stream(uint32_t seed, int n, uint32_t* out) {
  for (int i = 0; i < n; i++) out[i] = lcg(seed);
}

// kind 0 random_in_unit_disk, 1 random_in_unit_sphere, 2 random_on_unit_sphere
extern "C" void or_sampling(int kind, uint32_t seed, int n, float* out) {
  for (int i = 0; i < n; i++) {
    V3 v = kind == 0 ? random_in_unit_disk(seed)
                     : (kind == 1 ? random_in_unit_sphere(seed) : random_on_unit_sphere(seed));
    out[3 * i] = v.x;
    out[3 * i + 1] = v.y;
    out[3 * i + 2] = v.z;
  }
}

extern "C" void or_brdf_sample(int type, const float* c0, const float* c1, float p0, float p1,
                               int n, const float* Wo, const float* N, uint32_t* seeds,
                               float* Wi) {
  Scene tmp;
  const Material m = tmp.mats[or_add_material(&tmp, type, c0, c1, p0, p1)];
  for (int i = 0; i < n; i++) {
    V3 w = brdf_sample(m, v3(Wo[3 * i], Wo[3 * i + 1], Wo[3 * i + 2]),
                       v3(N[3 * i], N[3 * i + 1], N[3 * i + 2]), seeds[i]);
    Wi[3 * i] = w.x;
    Wi[3 * i + 1] = w.y;
    Wi[3 * i + 2] = w.z;
  }
}

extern "C" void or_brdf_eval(int type, const float* c0, const float* c1, float p0, float p1,
                             int n, const float* Wo, const float* Wi, const float* N, float* f,
                             float* pdf) {
  Scene tmp;
  const Material m = tmp.mats[or_add_material(&tmp, type, c0, c1, p0, p1)];
  for (int i = 0; i < n; i++) {
    float pd = 0.f;
    V3 v = brdf_eval(m, v3(Wo[3 * i], Wo[3 * i + 1], Wo[3 * i + 2]),
                     v3(Wi[3 * i], Wi[3 * i + 1], Wi[3 * i + 2]),
                     v3(N[3 * i], N[3 * i + 1], N[3 * i + 2]), pd);
    f[3 * i] = v.x;
    f[3 * i + 1] = v.y;
    f[3 * i + 2] = v.z;
    pdf[i] = pd;
  }
}

// The same helper cases as the reference harness's ref_helper: inputs of 8
// floats, outputs of 4, per case.
extern "C" void or_helper(int fn, int n, const float* in, float* out) {
  for (int i = 0; i < n; i++) {
    const float* a = in + 8 * i;
    float* o = out + 4 * i;
    V3 A = v3(a[0], a[1], a[2]), B = v3(a[3], a[4], a[5]);
    switch (fn) {
      case 0: o[0] = schlick(a[0], a[1]); break;
      case 1: {
        V3 r = v3(0.f);
        bool ok = Refract(A, B, a[6], r);
        o[0] = r.x; o[1] = r.y; o[2] = r.z;
        o[3] = ok ? 1.f : 0.f;
        break;
      }
      case 2: {
        V3 h = GGX_Sample(A, a[3], a[4], a[5], a[6]);
        o[0] = h.x; o[1] = h.y; o[2] = h.z;
        break;
      }
      case 3:
        o[0] = GGX_D(A, a[6], a[7]);
        o[1] = GGX_G(A, B, a[6], a[7]);
        o[2] = GGX_PDF(A, a[6], a[7]);
        break;
      case 4: {
        float phi, theta;
        Sample_Quadrant(a[0], a[1], a[2], a[3], phi, theta);
        o[0] = phi;
        o[1] = theta;
        break;
      }
      case 5:
        o[0] = AbsCosTheta(A);
        o[1] = SinTheta(A);
        o[2] = CosPhi(A);
        o[3] = SinPhi(A);
        break;
    }
  }
}

// Light k of a committed scene: n samples from (P, N, seed) and the pdf of
// each sampled direction.
extern "C" void or_light(void* sp, int k, int n, const float* P, uint32_t* seeds, float* Wi,
                         float* pdf) {
  Scene& s = *(Scene*)sp;
  const Light& L = s.lights[k];
  for (int i = 0; i < n; i++) {
    V3 p = v3(P[3 * i], P[3 * i + 1], P[3 * i + 2]);
    V3 w = light_sample(L, p, seeds[i]);
    Wi[3 * i] = w.x;
    Wi[3 * i + 1] = w.y;
    Wi[3 * i + 2] = w.z;
    pdf[i] = light_pdf(L, p, w);
  }
}

// One ray: closest primitive (-1 if none), t and its HitRecord as P, shading
// normal, u, v, geometric normal, Wo, material (17 floats).
extern "C" int or_probe(void* sp, const float* o, const float* d, float tmin, float* t,
                        float* rec) {
  Scene& s = *(Scene*)sp;
  Ray r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2]), tmin, RAY_TMAX};
  Hit h = trace(s, r, nullptr);
  *t = h.prim >= 0 ? h.t : 0.f;
  if (h.prim < 0 || !rec) return h.prim;
  HitRecord e = hit_record(s, s.prims[h.prim], r, h.t, h.u, h.v);
  float v[17] = {e.P.x, e.P.y, e.P.z, e.shading_normal.x, e.shading_normal.y,
                 e.shading_normal.z, e.u, e.v, e.geometric_normal.x, e.geometric_normal.y,
                 e.geometric_normal.z, e.Wo.x, e.Wo.y, e.Wo.z, (float)e.index, 0.f, 0.f};
  memcpy(rec, v, sizeof(v));
  return h.prim;
}

// ===================================================== FP64 hit distances ==
// A double-precision ray-primitive oracle against which the FP32 hit
// distances (oracle and kernels alike) are stated.  The primitives are the
// same float data (an instance transform is the float matrix, inverted here
// in double without rounding); the tests run in double: sphere roots by the
// cancellation-free quadratic, rect planes, box slabs, triangles by the
// Moller-Trumbore test (exact enough in double).  Traversal reuses the float
// BVH, whose boxes are padded conservatively, with the slab test in double.
namespace {

struct D3 {
  double x, y, z;
};
inline D3 dd(V3 v) { return D3{v.x, v.y, v.z}; }
inline D3 dsub(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 dcross(D3 a, D3 b) {
  return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dget(D3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

void inverse64(const float* m, double* out) {
  double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9],
         i = m[10];
  double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  double inv_det = 1.0 / (a * A + b * B + c * C);
  double r[9] = {A * inv_det, -(b * i - c * h) * inv_det, (b * f - c * e) * inv_det,
                 B * inv_det, (a * i - c * g) * inv_det, -(a * f - c * d) * inv_det,
                 C * inv_det, -(a * h - b * g) * inv_det, (a * e - b * d) * inv_det};
  for (int row = 0; row < 3; row++) {
    out[row * 4 + 0] = r[row * 3 + 0];
    out[row * 4 + 1] = r[row * 3 + 1];
    out[row * 4 + 2] = r[row * 3 + 2];
    out[row * 4 + 3] = -(r[row * 3 + 0] * m[3] + r[row * 3 + 1] * m[7] + r[row * 3 + 2] * m[11]);
  }
}

// Candidate of one primitive for a world ray (o, d) in double.  Returns true
// on a hit with t > tmin; t is then the hit distance, else the distance to
// the primitive's surface where the ray passes nearest (plane t for
// triangles and rects, the closest approach for spheres, the slab entry for
// boxes).  The FP32 error statement uses three more numbers:
//   margin  how far inside the primitive's outline the ray passes, relative
//           to its size (triangles: the smallest barycentric; rects: the
//           nearest edge distance / extent; spheres: (r - h) / r with h the
//           ray's distance to the centre; boxes: slab overlap / box size);
//           negative on a miss;
//   mslack  the size of the rounding error of an FP32 evaluation of margin,
//           in units of epsilon (position magnitude / primitive size; for
//           spheres (|o - c|^2 + r^2) / r^2, from c = |o - c|^2 - r^2);
//   tslack  the size of the rounding error of an FP32 t, as a distance in
//           units of epsilon: |o| + t|d| (for spheres plus
//           (|o - c|^2 + r^2) / L, L the half chord: the discriminant's
//           cancellation).
struct Cand64 {
  double t, margin, mslack, tslack;
};

bool cand64(const Scene& s, const Prim& p, D3 o, D3 d, double tmin, Cand64& c64) {
  D3 wo = o, wd = d;
  if (p.xform >= 0) {
    double inv[12];
    inverse64(s.xforms[p.xform].m, inv);
    D3 oo{inv[0] * o.x + inv[1] * o.y + inv[2] * o.z + inv[3],
          inv[4] * o.x + inv[5] * o.y + inv[6] * o.z + inv[7],
          inv[8] * o.x + inv[9] * o.y + inv[10] * o.z + inv[11]};
    D3 od{inv[0] * d.x + inv[1] * d.y + inv[2] * d.z, inv[4] * d.x + inv[5] * d.y + inv[6] * d.z,
          inv[8] * d.x + inv[9] * d.y + inv[10] * d.z};
    o = oo;
    d = od;
  }
  const float* f = p.f;
  const double on = sqrt(ddot(wo, wo)), dn = sqrt(ddot(wd, wd));
  double& t = c64.t;
  c64.margin = -1.0;
  c64.mslack = 1.0;
  bool hit = false;
  if (p.type == PRIM_MSPHERE) return false;  // (the statement covers static primitives)
  if (p.type == PRIM_SPHERE) {
    double r = f[3];
    D3 oc = dsub(o, D3{f[0], f[1], f[2]});
    double a = ddot(d, d), b = ddot(oc, d), occ = ddot(oc, oc), c = occ - r * r;
    double disc = b * b - a * c;
    double h2 = std::max(0.0, occ - b * b / a);
    c64.margin = (r - sqrt(h2)) / r;
    c64.mslack = (occ + r * r) / (r * r);
    double L = disc > 0.0 ? sqrt(disc / a) : 0.0;
    if (disc < 0.0) {
      t = -b / a;
    } else {
      double sq = sqrt(disc);
      double q = b > 0.0 ? -(b + sq) : -(b - sq);
      double t0 = q / a, t1 = c / q;
      if (t0 > t1) std::swap(t0, t1);
      if (t0 > tmin) { t = t0; hit = true; }
      else if (t1 > tmin) { t = t1; hit = true; }
      else { t = t1; c64.margin = -1.0; }
    }
    c64.tslack = on + fabs(t) * dn + (occ + r * r) / std::max(L, 1e-300);
    return hit;
  }
  if (p.type == PRIM_RECT) {
    int ax = p.axis, ia = ax == 0 ? 1 : 0, ib = ax == 2 ? 1 : 2;
    t = ((double)f[4] - dget(o, ax)) / dget(d, ax);
    double a = dget(o, ia) + t * dget(d, ia), b = dget(o, ib) + t * dget(d, ib);
    double ea = (double)f[1] - f[0], eb = (double)f[3] - f[2];
    double ext = std::max(std::min(ea, eb), 1e-30);
    c64.margin = std::min(std::min(a - f[0], f[1] - a), std::min(b - f[2], f[3] - b)) / ext;
    c64.tslack = on + fabs(t) * dn;
    c64.mslack = c64.tslack / ext + 1.0;
    return c64.margin >= 0.0 && t > tmin;
  }
  if (p.type == PRIM_BOX) {
    double tn = -INFINITY, tf = INFINITY, size = INFINITY;
    for (int k = 0; k < 3; k++) {
      double t0 = ((double)f[k] - dget(o, k)) / dget(d, k);
      double t1 = ((double)f[3 + k] - dget(o, k)) / dget(d, k);
      tn = std::max(tn, std::min(t0, t1));
      tf = std::min(tf, std::max(t0, t1));
      size = std::min(size, (double)f[3 + k] - f[k]);
    }
    size = std::max(size, 1e-30);
    c64.margin = (tf - tn) * sqrt(ddot(d, d)) / size;
    if (tn <= tf) {
      if (tn > tmin) { t = tn; hit = true; }
      else if (tf > tmin) { t = tf; hit = true; }
      else t = tf;
    } else {
      t = tn;
    }
    c64.tslack = on + fabs(t) * dn;
    c64.mslack = c64.tslack / size + 1.0;
    return hit;
  }
  D3 v0{f[0], f[1], f[2]}, v1{f[3], f[4], f[5]}, v2{f[6], f[7], f[8]};
  D3 e1 = dsub(v1, v0), e2 = dsub(v2, v0);
  D3 P = dcross(d, e2);
  double det = ddot(P, e1);
  D3 R = dsub(o, v0);
  D3 Q = dcross(R, e1);
  if (det == 0.0) {
    t = INFINITY;
    c64.tslack = INFINITY;
    return false;
  }
  double u = ddot(P, R) / det, v = ddot(Q, d) / det;
  t = ddot(Q, e2) / det;
  c64.margin = std::min(std::min(u, v), 1.0 - u - v);
  D3 e3 = dsub(v2, v1);
  double area2 = sqrt(ddot(dcross(e1, e2), dcross(e1, e2)));
  double maxe = sqrt(std::max(std::max(ddot(e1, e1), ddot(e2, e2)), ddot(e3, e3)));
  double alt = std::max(area2 / maxe, 1e-30);
  c64.tslack = on + fabs(t) * dn;
  c64.mslack = c64.tslack / alt + 1.0;
  return c64.margin >= 0.0 && t > tmin;
}

struct Hit64 {
  int prim = -1;
  double t = INFINITY;
  Cand64 c{};
};

Hit64 trace64(const Scene& s, D3 o, D3 d, double tmin) {
  Hit64 best;
  if (s.nodes.empty()) return best;
  D3 inv{1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
  auto slab = [&](const AABB& b, double& tn) {
    double lo = tmin, hi = best.t;
    for (int k = 0; k < 3; k++) {
      double t0 = (dget(dd(b.lo), k) - dget(o, k)) * dget(inv, k);
      double t1 = (dget(dd(b.hi), k) - dget(o, k)) * dget(inv, k);
      if (t0 > t1) std::swap(t0, t1);
      if (t0 == t0) lo = std::max(lo, t0);  // a NaN bound (0 * inf) constrains nothing
      if (t1 == t1) hi = std::min(hi, t1);
    }
    tn = lo;
    return lo <= hi;
  };
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const BNode& n = s.nodes[stack[--sp]];
    double tn;
    if (!slab(n.box, tn)) continue;
    if (n.count) {
      for (int k = n.left; k < n.left + n.count; k++) {
        int pid = s.order[k];
        Cand64 c;
        if (!cand64(s, s.prims[pid], o, d, tmin, c)) continue;
        if (c.t < best.t || (c.t == best.t && pid < best.prim)) {
          best.prim = pid;
          best.t = c.t;
          best.c = c;
        }
      }
    } else {
      stack[sp++] = n.right;
      stack[sp++] = n.left;
    }
  }
  return best;
}

}  // namespace

// Camera rays of frame `frame` (float, as the float path generates them):
// origins and directions, 3 floats each per pixel.
extern "C" void or_camera_rays(void* sp, int W, int H, int frame, float* o, float* d) {
  Scene& s = *(Scene*)sp;
  Tracer tr{s, nullptr};
  for (int p = 0; p < W * H; p++) {
    uint32_t x = p % W, y = p / W;
    uint32_t seed = tea64((uint32_t)W * y + x, (uint32_t)frame);
    Ray r = tr.camera_ray(x, y, W, H, seed);
    o[3 * p] = r.o.x; o[3 * p + 1] = r.o.y; o[3 * p + 2] = r.o.z;
    d[3 * p] = r.d.x; d[3 * p + 1] = r.d.y; d[3 * p + 2] = r.d.z;
  }
}

// Closest hit in double of n rays (float origins and directions, tmin as
// the float path's): primitive (-1), and per ray 4 doubles: t, margin,
// mslack, tslack (see Cand64).
extern "C" void or_trace64(void* sp, int n, const float* o, const float* d, float tmin,
                           int32_t* prim, double* out, int threads) {
  Scene& s = *(Scene*)sp;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
  for (int i = 0; i < n; i++) {
    Hit64 h = trace64(s, D3{o[3 * i], o[3 * i + 1], o[3 * i + 2]},
                      D3{d[3 * i], d[3 * i + 1], d[3 * i + 2]}, (double)tmin);
    prim[i] = h.prim;
    double* q = out + 4 * i;
    q[0] = h.prim >= 0 ? h.c.t : 0.0;
    q[1] = h.c.margin;
    q[2] = h.c.mslack;
    q[3] = h.c.tslack;
  }
}

// One primitive in double for one ray: 1 on a hit; out = t, margin, mslack,
// tslack.
extern "C" int or_prim64(void* sp, int prim, const float* o, const float* d, float tmin,
                         double* out) {
  Scene& s = *(Scene*)sp;
  Cand64 c;
  bool hit = cand64(s, s.prims[prim], D3{o[0], o[1], o[2]}, D3{d[0], d[1], d[2]}, (double)tmin, c);
  out[0] = c.t;
  out[1] = c.margin;
  out[2] = c.mslack;
  out[3] = c.tslack;
  return hit ? 1 : 0;
}

// A moving sphere (f = centre at time0 (3), radius, time0, time1, centre at
// time1 (3)) against one ray at `time`: 1 on a hit, out = t, P (3), shading
// normal (3), u, v, Wo (3); and its box for camera times cam_t0, cam_t1
// (box6 = lo, hi).  Test infrastructure: pins the oracle's moving sphere to
// programs/hitables/moving_sphere.cu.
extern "C" int or_msphere(const float* f, const float* o, const float* d, float tmin, float tmax,
                          float time, float* out, float cam_t0, float cam_t1, float* box6) {
  Scene s;
  s.cam.time0 = cam_t0;
  s.cam.time1 = cam_t1;
  Prim p;
  memset(&p, 0, sizeof(p));
  p.type = PRIM_MSPHERE;
  p.xform = -1;
  p.mesh = -1;
  memcpy(p.f, f, 9 * sizeof(float));
  AABB b = prim_bounds(s, p);
  box6[0] = b.lo.x; box6[1] = b.lo.y; box6[2] = b.lo.z;
  box6[3] = b.hi.x; box6[4] = b.hi.y; box6[5] = b.hi.z;
  Ray r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2]), tmin, tmax, time};
  float t = 0.f, bu = 0.f, bv = 0.f;
  if (!prim_candidate(s, p, r, t, bu, bv)) return 0;
  HitRecord rec = hit_record(s, p, r, t, bu, bv);
  float v[13] = {t, rec.P.x, rec.P.y, rec.P.z, rec.shading_normal.x, rec.shading_normal.y,
                 rec.shading_normal.z, rec.u, rec.v, rec.Wo.x, rec.Wo.y, rec.Wo.z, 0.f};
  memcpy(out, v, 12 * sizeof(float));
  return 1;
}
