/*
 * pt_device.cuh - device restatement of the reference's OptiX programs for
 * the wavefront kernels: RNG, sampling, primitive tests and hit records,
 * light sample/pdf callables, the seven BRDFs.  Every expression keeps the
 * reference's evaluation order; with -fmad=false and the shared ptmath.h
 * functions the results are bit-identical to the CPU oracle.
 * Reference: programs/{random,sampling}.cuh, programs/hitables/*.cu,
 * programs/pdfs/*.cu, programs/materials/*.cu[h], programs/math/*.cuh.
 */
#ifndef PT_DEVICE_CUH
#define PT_DEVICE_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include "ptmath.h"
#include "pt_types.h"

#define PTD __device__ __forceinline__

namespace ptd {

struct V3 {
  float x, y, z;
};
PTD V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
PTD V3 v3(float s) { return v3(s, s, s); }
PTD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
PTD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
PTD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
PTD V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
PTD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
PTD V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
PTD V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
PTD V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
PTD V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
PTD V3& operator*=(V3& a, V3 b) { a = a * b; return a; }
PTD V3& operator*=(V3& a, float s) { a = a * s; return a; }
PTD V3& operator/=(V3& a, float s) { a = a / s; return a; }
PTD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PTD V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
PTD float length(V3 a) { return ptm_sqrt(dot(a, a)); }
PTD V3 normalize(V3 a) {
  float inv = 1.0f / ptm_sqrt(dot(a, a));
  return a * inv;
}
PTD float clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
PTD V3 clamp3(V3 v, float a, float b) {
  return v3(clampf(v.x, a, b), clampf(v.y, a, b), clampf(v.z, a, b));
}
PTD V3 reflect(V3 i, V3 n) { return i - (2.0f * n) * dot(n, i); }
PTD float squared_length(V3 a) { return length(a) * length(a); }
PTD bool isNull(V3 a) { return (a.x == 0.f) && (a.y == 0.f) && (a.z == 0.f); }
PTD V3 unit_vector(V3 v) { return v / length(v); }
PTD float ffmin(float a, float b) { return a < b ? a : b; }
PTD float ffmax(float a, float b) { return a > b ? a : b; }
PTD V3 min_vec(V3 a, V3 b) { return v3(ffmin(a.x, b.x), ffmin(a.y, b.y), ffmin(a.z, b.z)); }
PTD V3 max_vec(V3 a, V3 b) { return v3(ffmax(a.x, b.x), ffmax(a.y, b.y), ffmax(a.z, b.z)); }
PTD float max_component(V3 a) { return ffmax(ffmax(a.x, a.y), a.z); }
PTD float min_component(V3 a) { return ffmin(ffmin(a.x, a.y), a.z); }
PTD float get(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
PTD V3 f4xyz(float4 f) { return v3(f.x, f.y, f.z); }

#define PI_F 3.141592654f

// ------------------------------------------------------------------- RNG --
// programs/random.cuh:33-65
PTD uint32_t tea64(uint32_t val0, uint32_t val1) {
  uint32_t v0 = val0, v1 = val1, s0 = 0;
#pragma unroll 16
  for (int n = 0; n < 64; n++) {
    s0 += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  return v0;
}
PTD uint32_t lcg(uint32_t& prev) {
  prev = 1664525u * prev + 1013904223u;
  return prev & 0x00FFFFFFu;
}
PTD float rnd(uint32_t& prev) { return (float)lcg(prev) / (float)0x01000000; }

// ------------------------------------------------------------- sampling ---
// programs/sampling.cuh:22-59
PTD V3 random_in_unit_disk(uint32_t& seed) {
  float a = rnd(seed) * 2.f * PI_F;
  V3 xy = v3(pt_sinf(a), pt_cosf(a), 0.f);
  xy *= ptm_sqrt(rnd(seed));
  return xy;
}
PTD V3 random_in_unit_sphere(uint32_t& seed) {
  float z = rnd(seed) * 2.f - 1.f;
  float t = rnd(seed) * 2.f * PI_F;
  float r = ptm_sqrt((0.f > (1.f - z * z) ? 0.f : (1.f - z * z)));
  float x = r * pt_cosf(t);
  float y = r * pt_sinf(t);
  V3 res = v3(x, y, z);
  res *= pt_powf(rnd(seed), 1.f / 3.f);
  return res;
}
PTD V3 random_on_unit_sphere(uint32_t& seed) { return unit_vector(random_in_unit_sphere(seed)); }

// Orthonormal basis after Duff et al. 2017 (the reference uses OptiX's Onb).
struct Onb {
  V3 t, b, n;
  PTD explicit Onb(V3 nn) {
    n = nn;
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float bb = n.x * n.y * a;
    t = v3(1.0f + sign * n.x * n.x * a, sign * bb, -sign * n.x);
    b = v3(bb, sign + n.y * n.y * a, -n.y);
  }
  PTD void inverse_transform(V3& p) const { p = p.x * t + p.y * b + p.z * n; }
};

// Malley's method over the Shirley-Chiu concentric map.
PTD void cosine_sample_hemisphere(float u1, float u2, V3& p) {
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

// programs/math/trigonometric.cuh:5-62 (world "y-up" conventions)
PTD float CosTheta(V3 w) { return w.y; }
PTD float Cos2Theta(V3 w) { return w.y * w.y; }
PTD float AbsCosTheta(V3 w) { return fabsf(w.y); }
PTD float Sin2Theta(V3 w) { return fmaxf(0.f, 1.f - Cos2Theta(w)); }
PTD float SinTheta(V3 w) { return ptm_sqrt(Sin2Theta(w)); }
PTD float TanTheta(V3 w) { return SinTheta(w) / CosTheta(w); }
PTD float CosPhi(V3 w) {
  float sinTheta = SinTheta(w);
  return (sinTheta == 0) ? 1.f : clampf(w.x / sinTheta, -1.f, 1.f);
}
PTD float SinPhi(V3 w) {
  float sinTheta = SinTheta(w);
  return (sinTheta == 0) ? 0.f : clampf(w.z / sinTheta, -1.f, 1.f);
}
PTD float Cos2Phi(V3 w) { float c = CosPhi(w); return c * c; }
PTD float Sin2Phi(V3 w) { float s = SinPhi(w); return s * s; }
PTD V3 Spherical_Vector(float sintheta, float costheta, float phi) {
  return v3(sintheta * pt_cosf(phi), costheta, sintheta * pt_sinf(phi));
}

// ------------------------------------------------------------- xforms -----
PTD V3 xpoint(const float4* m, V3 p) {
  float4 r0 = m[0], r1 = m[1], r2 = m[2];
  return v3(r0.x * p.x + r0.y * p.y + r0.z * p.z + r0.w,
            r1.x * p.x + r1.y * p.y + r1.z * p.z + r1.w,
            r2.x * p.x + r2.y * p.y + r2.z * p.z + r2.w);
}
PTD V3 xvector(const float4* m, V3 p) {
  float4 r0 = m[0], r1 = m[1], r2 = m[2];
  return v3(r0.x * p.x + r0.y * p.y + r0.z * p.z,
            r1.x * p.x + r1.y * p.y + r1.z * p.z,
            r2.x * p.x + r2.y * p.y + r2.z * p.z);
}
// transpose of world->object rows applied to a normal
PTD V3 xnormal(const float4* inv, V3 n) {
  float4 r0 = inv[0], r1 = inv[1], r2 = inv[2];
  return v3(r0.x * n.x + r1.x * n.y + r2.x * n.z,
            r0.y * n.x + r1.y * n.y + r2.y * n.z,
            r0.z * n.x + r1.z * n.y + r2.z * n.z);
}

// --------------------------------------------------------- primitives -----
struct PrimRec {
  float4 r0, r1, r2;
};
PTD int prim_type(const PrimRec& p) { return (int)(__float_as_uint(p.r0.w) & 3u); }
PTD int prim_axis(const PrimRec& p) { return (int)((__float_as_uint(p.r0.w) >> 2) & 3u); }
PTD int prim_flip(const PrimRec& p) { return (int)((__float_as_uint(p.r0.w) >> 4) & 1u); }
PTD int prim_xform(const PrimRec& p) { return (int)(__float_as_uint(p.r0.w) >> 8) - 1; }
PTD bool prim_moving(const PrimRec& p) { return (__float_as_uint(p.r0.w) & PT_PRIM_MOVING) != 0u; }
PTD uint32_t prim_id(const PrimRec& p) { return __float_as_uint(p.r1.w); }
PTD uint32_t prim_material(const PrimRec& p) { return __float_as_uint(p.r2.w); }

PTD PrimRec load_prim(const float4* prims, uint32_t i) {
  PrimRec p;
  p.r0 = __ldg(prims + 3 * i);
  p.r1 = __ldg(prims + 3 * i + 1);
  p.r2 = __ldg(prims + 3 * i + 2);
  return p;
}

// Centre of a sphere at `time`: the record's centre, or for a moving sphere
// programs/hitables/moving_sphere.cu:47-49 (linear in time, also outside
// [time0, time1]).
PTD V3 sphere_center(const PrimRec& p, float time) {
  V3 c0 = v3(p.r0.x, p.r0.y, p.r0.z);
  if (!prim_moving(p)) return c0;
  V3 c1 = v3(p.r2.x, p.r2.y, p.r2.z);
  return c0 + ((time - p.r1.y) / (p.r1.z - p.r1.y)) * (c1 - c0);
}

// programs/hitables/sphere.cu:32-62 - near root if in range, else far root
// (a moving sphere, moving_sphere.cu:57-118: the same roots at its centre
// for the ray's time: sphere_candidate_at(p, sphere_center(p, time), ...))
PTD bool sphere_candidate_at(const PrimRec& p, V3 center, V3 o, V3 d, float tmin, float tmax,
                             float& t) {
  float radius = p.r1.x;
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

PTD bool sphere_candidate(const PrimRec& p, V3 o, V3 d, float tmin, float tmax, float& t,
                          float time = 0.f) {
  return sphere_candidate_at(p, sphere_center(p, time), o, d, tmin, tmax, t);
}

// programs/hitables/aarect.cu:20-69
PTD bool rect_candidate(const PrimRec& p, V3 o, V3 d, float tmin, float tmax, float& t) {
  float a0 = p.r0.x, a1 = p.r0.y, b0 = p.r0.z, b1 = p.r1.x, k = p.r1.y;
  int axis = prim_axis(p);
  float a, b;
  if (axis == 0) {
    t = (k - o.x) / d.x;
    a = o.y + t * d.y;
    b = o.z + t * d.z;
  } else if (axis == 1) {
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

// programs/hitables/box.cu:36-53 - entry if in range, else exit
PTD bool box_candidate(const PrimRec& p, V3 o, V3 d, float tmin, float tmax, float& t) {
  V3 boxmin = v3(p.r0.x, p.r0.y, p.r0.z), boxmax = v3(p.r1.x, p.r1.y, p.r1.z);
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

// Per-ray constants of the watertight triangle test.
struct WtRay {
  int kx, ky, kz;
  float Sx, Sy, Sz;
};
PTD WtRay wt_setup(V3 d) {
  WtRay w;
  float adx = fabsf(d.x), ady = fabsf(d.y), adz = fabsf(d.z);
  w.kz = (adx > ady) ? ((adx > adz) ? 0 : 2) : ((ady > adz) ? 1 : 2);
  w.kx = w.kz + 1; if (w.kx == 3) w.kx = 0;
  w.ky = w.kx + 1; if (w.ky == 3) w.ky = 0;
  if (get(d, w.kz) < 0.0f) { int tmp = w.kx; w.kx = w.ky; w.ky = tmp; }
  w.Sz = 1.0f / get(d, w.kz);
  w.Sx = get(d, w.kx) * w.Sz;
  w.Sy = get(d, w.ky) * w.Sz;
  return w;
}

// Watertight ray/triangle intersection, Woop, Benthin & Wald, JCGT 2013.
PTD bool tri_candidate(const PrimRec& p, V3 o, const WtRay& w, float tmin, float tmax,
                       float& t, float& bu, float& bv) {
  V3 A = v3(p.r0.x, p.r0.y, p.r0.z) - o;
  V3 B = v3(p.r1.x, p.r1.y, p.r1.z) - o;
  V3 C = v3(p.r2.x, p.r2.y, p.r2.z) - o;
  float Akz = get(A, w.kz), Bkz = get(B, w.kz), Ckz = get(C, w.kz);
  float Ax = get(A, w.kx) - w.Sx * Akz, Ay = get(A, w.ky) - w.Sy * Akz;
  float Bx = get(B, w.kx) - w.Sx * Bkz, By = get(B, w.ky) - w.Sy * Bkz;
  float Cx = get(C, w.kx) - w.Sx * Ckz, Cy = get(C, w.ky) - w.Sy * Ckz;
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
  float Az = w.Sz * Akz, Bz = w.Sz * Bkz, Cz = w.Sz * Ckz;
  float T = U * Az + V * Bz + W * Cz;
  float rcp = 1.0f / det;
  float tt = T * rcp;
  if (!(tt > tmin && tt < tmax)) return false;
  t = tt;
  bu = V * rcp;
  bv = W * rcp;
  return true;
}

// ------------------------------------------------------------ hit record --
struct HitRecord {
  uint32_t index;  // material id
  int tindex;      // texture index: the face's (mesh.hpp material_buffer), 0 for analytic shapes
  V3 P;
  float u, v;
  V3 geometric_normal, shading_normal, Wo;
};

// Get_HitRecord of each primitive: programs/hitables/{sphere,aarect,box,
// triangle}.cu, from the object-space ray, mapped to world space once.
// need_uv: texture coordinates are computed only when a texture reads them
// (the shading kernels pass false and compute them out of line, in
// textured_colours, for textured materials only; u, v feed nothing else).
PTD HitRecord hit_record(const DevScene& S, const PrimRec& p, V3 ro, V3 rd, float t_hit,
                         float bu, float bv, bool need_uv = true, float time = 0.f) {
  HitRecord rec;
  rec.Wo = normalize(-rd);
  int xf = prim_xform(p);
  const float4* M = xf >= 0 ? S.xforms + 6 * xf : nullptr;
  const float4* I = xf >= 0 ? S.xforms + 6 * xf + 3 : nullptr;
  V3 o = ro, d = rd;
  if (I) {
    o = xpoint(I, ro);
    d = xvector(I, rd);
  }
  rec.index = prim_material(p);
  rec.tindex = 0;
  int type = prim_type(p);
  if (type == PT_PRIM_SPHERE) {
    // a moving sphere's record (moving_sphere.cu:80-96) is the sphere's at
    // its centre for the ray's time
    V3 center = sphere_center(p, time);
    float radius = p.r1.x;
    V3 hit_point = o + t_hit * d;
    rec.P = M ? xpoint(M, hit_point) : hit_point;
    V3 T = (rec.P - center) / radius;
    V3 normal = normalize(I ? xnormal(I, T) : T);
    rec.shading_normal = rec.geometric_normal = normal;
    rec.u = rec.v = 0.f;
    if (need_uv) {
      float phi = pt_atan2f(T.z, T.x);
      float theta = pt_asinf(T.y);
      rec.u = 1.f - (phi + PI_F) / (2.f * PI_F);
      rec.v = (theta + PI_F / 2.f) / PI_F;
    }
  } else if (type == PT_PRIM_RECT) {
    float a0 = p.r0.x, a1 = p.r0.y, b0 = p.r0.z, b1 = p.r1.x;
    int axis = prim_axis(p);
    V3 hit_point = o + t_hit * d;
    rec.P = M ? xpoint(M, hit_point) : hit_point;
    V3 normal;
    if (axis == 0) {
      normal = v3(1.f, 0.f, 0.f);
      rec.u = (hit_point.y - a0) / (a1 - a0);
      rec.v = (hit_point.z - b0) / (b1 - b0);
    } else if (axis == 1) {
      normal = v3(0.f, 1.f, 0.f);
      rec.u = (hit_point.x - a0) / (a1 - a0);
      rec.v = (hit_point.z - b0) / (b1 - b0);
    } else {
      normal = v3(0.f, 0.f, 1.f);
      rec.u = (hit_point.x - a0) / (a1 - a0);
      rec.v = (hit_point.y - b0) / (b1 - b0);
    }
    normal = prim_flip(p) ? -normal : normal;
    normal = normalize(I ? xnormal(I, normal) : normal);
    rec.shading_normal = rec.geometric_normal = normal;
  } else if (type == PT_PRIM_BOX) {
    V3 boxmin = v3(p.r0.x, p.r0.y, p.r0.z), boxmax = v3(p.r1.x, p.r1.y, p.r1.z);
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
  } else {
    V3 a = v3(p.r0.x, p.r0.y, p.r0.z), b = v3(p.r1.x, p.r1.y, p.r1.z),
       c = v3(p.r2.x, p.r2.y, p.r2.z);
    V3 e1 = b - a, e2 = c - a;
    float b0 = 1.f - bu - bv, b1 = bu, b2 = bv;
    rec.P = a * b0 + b * b1 + c * b2;
    V3 Ng = cross(e1, e2);
    float area = length(Ng) / 2.f;
    Ng /= 2.f * area;
    Ng = normalize(normalize(Ng));
    rec.geometric_normal = Ng;
    uint4 at = __ldg(S.tri_attr + prim_id(p));
    rec.tindex = (int)(at.w >> 2);
    if (!(at.w & 1u)) {
      rec.shading_normal = Ng;
    } else {
      const float* N = S.normals;
      V3 na = v3(N[3 * at.x], N[3 * at.x + 1], N[3 * at.x + 2]);
      V3 nb = v3(N[3 * at.y], N[3 * at.y + 1], N[3 * at.y + 2]);
      V3 nc = v3(N[3 * at.z], N[3 * at.z + 1], N[3 * at.z + 2]);
      V3 Ns = na * b0 + nb * b1 + nc * b2;
      rec.shading_normal = normalize(Ns);
    }
    if (!(at.w & 2u) || !need_uv) {
      rec.u = rec.v = 0.f;
    } else {
      const float* uv = S.uvs;
      rec.u = uv[2 * at.x] * b0 + uv[2 * at.y] * b1 + uv[2 * at.z] * b2;
      rec.v = uv[2 * at.x + 1] * b0 + uv[2 * at.y + 1] * b1 + uv[2 * at.z + 1] * b2;
    }
  }
  return rec;
}

// ---------------------------------------------------------------- lights --
// programs/pdfs/rect_pdf.cu:11-113 and programs/pdfs/sphere_pdf.cu:8-50
PTD float light_pdf(const GpuLight& L, V3 P, V3 Wi) {
  if (L.type == PT_LIGHT_RECT) {
    float t, a, b;
    V3 N;
    if (L.axis == 0) {
      t = (L.k - P.x) / Wi.x;
      a = P.y + t * Wi.y;
      b = P.z + t * Wi.z;
      N = v3(1.f, 0.f, 0.f);
    } else if (L.axis == 1) {
      t = (L.k - P.y) / Wi.y;
      a = P.x + t * Wi.x;
      b = P.z + t * Wi.z;
      N = v3(0.f, 1.f, 0.f);
    } else {
      t = (L.k - P.z) / Wi.z;
      a = P.x + t * Wi.x;
      b = P.y + t * Wi.y;
      N = v3(0.f, 0.f, 1.f);
    }
    if (a < L.a0 || a > L.a1 || b < L.b0 || b > L.b1) return 0.f;
    if (!(t < 3.40282347e+38f && t > 0.001f)) return 0.f;
    float distance_squared = t * t * squared_length(Wi);
    float cosine = fabsf(dot(Wi, N) / length(Wi));
    float area = (L.a1 - L.a0) * (L.b1 - L.b0);
    return distance_squared / (cosine * area);
  }
  V3 c = v3(L.cx, L.cy, L.cz);
  V3 oc = P - c;
  float a = dot(Wi, Wi);
  float b = dot(oc, Wi);
  float cc = dot(oc, oc) - L.r * L.r;
  float discriminant = b * b - a * cc;
  bool hit = false;
  if (discriminant >= 0.f) {
    float temp = (-b - ptm_sqrt(discriminant)) / a;
    if (temp < 3.40282347e+38f && temp > 0.001f) hit = true;
    if (!hit) {
      temp = (-b + ptm_sqrt(discriminant)) / a;
      if (temp < 3.40282347e+38f && temp > 0.001f) hit = true;
    }
  }
  if (!hit) return 0.f;
  float distance_squared = squared_length(c - P);
  float cos_theta_max = ptm_sqrt(1.f - L.r * L.r / distance_squared);
  float solid_angle = 2.f * PI_F * (1.f - cos_theta_max);
  return 1.f / solid_angle;
}

// programs/pdfs/rect_pdf.cu:116-145 and programs/pdfs/sphere_pdf.cu:53-73
PTD V3 light_sample(const GpuLight& L, V3 P, uint32_t& seed) {
  if (L.type == PT_LIGHT_RECT) {
    float r0 = rnd(seed);
    float r1 = rnd(seed);
    V3 q;
    if (L.axis == 0) q = v3(L.k, L.a0 + r0 * (L.a1 - L.a0), L.b0 + r1 * (L.b1 - L.b0));
    else if (L.axis == 1) q = v3(L.a0 + r0 * (L.a1 - L.a0), L.k, L.b0 + r1 * (L.b1 - L.b0));
    else q = v3(L.a0 + r0 * (L.a1 - L.a0), L.b0 + r1 * (L.b1 - L.b0), L.k);
    return q - P;
  }
  V3 c = v3(L.cx, L.cy, L.cz);
  float r1 = rnd(seed);
  float r2 = rnd(seed);
  float distance_squared = squared_length(c - P);
  float z = 1.f + r2 * (ptm_sqrt(1.f - L.r * L.r / distance_squared) - 1.f);
  float phi = 2.f * PI_F * r1;
  float x = pt_cosf(phi) * ptm_sqrt(1.f - z * z);
  float y = pt_sinf(phi) * ptm_sqrt(1.f - z * z);
  V3 Wi = v3(x, y, z);
  Onb uvw(normalize(Wi));
  uvw.inverse_transform(Wi);
  return Wi;
}

// ------------------------------------------------------------- materials --
PTD float schlick(float cosine, float ref_idx) {
  float r0 = (1.f - ref_idx) / (1.f + ref_idx);
  r0 = r0 * r0;
  return r0 + (1.f - r0) * pt_powf((1.f - cosine), 5.f);
}
PTD V3 schlick3(V3 r0, float cosine) {
  float exponential = pt_powf(1.f - cosine, 5.f);
  return r0 + (v3(1.f) - r0) * exponential;
}
PTD bool Refract(V3 v, V3 n, float ni_over_nt, V3& refracted) {
  V3 uv = normalize(v);
  float dt = dot(uv, n);
  float discriminant = 1.f - ni_over_nt * ni_over_nt * (1.f - dt * dt);
  if (discriminant > 0.f) {
    refracted = ni_over_nt * (uv - n * dt) - n * ptm_sqrt(discriminant);
    return true;
  }
  return false;
}
PTD void Sample_Quadrant(float nu, float nv, float randX, float randY, float& phi, float& theta) {
  phi = pt_atanf(ptm_sqrt((nu + 1.f) / (nv + 1.f)) * pt_tanf(2.f * PI_F * randX));
  float cos_phi = pt_cosf(phi);
  float sin_phi = pt_sinf(phi);
  theta = pt_powf(randY, 1.f / (nu * cos_phi * cos_phi + nv * sin_phi * sin_phi + 1.f));
}
PTD float GGX_D(V3 H, float nu, float nv) {
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
PTD V3 GGX_Sample(V3 origin, float rx, float ry, float nu, float nv) {
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
PTD float GGX_Lambda(V3 V, float nu, float nv) {
  float absTanTheta = fabsf(TanTheta(V));
  if (isinf(absTanTheta)) return 0.f;
  float alpha = ptm_sqrt(Cos2Phi(V) * nu * nu + Sin2Phi(V) * nv * nv);
  float alpha2Tan2Theta = (alpha * absTanTheta) * (alpha * absTanTheta);
  return (-1.f + ptm_sqrt(1.f + alpha2Tan2Theta)) / 2.f;
}
PTD float GGX_G(V3 Wo, V3 Wi, float nu, float nv) {
  return 1.f / (1.f + GGX_Lambda(Wo, nu, nv) + GGX_Lambda(Wi, nu, nv));
}
PTD float GGX_PDF(V3 H, float nu, float nv) { return GGX_D(H, nu, nv) * AbsCosTheta(H); }

// Sample callables of programs/materials/{lambertian,oren_nayar,
// diffuse_light,torrance_sparrow,ashikhmin_shirley}.cuh
PTD V3 brdf_sample(const GpuMaterial& m, V3 Wo, V3 N, uint32_t& seed) {
  switch (m.type) {
    case PT_MAT_LAMBERTIAN:
    case PT_MAT_OREN_NAYAR: {
      V3 Wi;
      float r0 = rnd(seed);
      float r1 = rnd(seed);
      cosine_sample_hemisphere(r0, r1, Wi);
      Onb uvw(N);
      uvw.inverse_transform(Wi);
      return Wi;
    }
    case PT_MAT_DIFFUSE_LIGHT:
      return random_on_unit_sphere(seed);
    case PT_MAT_TORRANCE_SPARROW: {
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
    case PT_MAT_ASHIKHMIN_SHIRLEY: {
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

// Evaluate callables (set pdf; a pdf the reference leaves unset stays as the
// caller initialised it, 0).
PTD V3 brdf_eval(const GpuMaterial& m, V3 Wo, V3 Wi, V3 N, float& pdf) {
  switch (m.type) {
    case PT_MAT_LAMBERTIAN: {
      float cosine = dot(normalize(Wi), normalize(N));
      if (cosine < 0.f) return v3(0.f);
      pdf = dot(normalize(Wi), normalize(N)) / PI_F;
      return (cosine * v3(m.c0x, m.c0y, m.c0z)) / PI_F;
    }
    case PT_MAT_DIFFUSE_LIGHT:
      pdf = 1.f;
      return v3(m.c0x, m.c0y, m.c0z);
    case PT_MAT_OREN_NAYAR: {
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
      return v3(m.c0x, m.c0y, m.c0z) * (1.f / PI_F) * (m.p0 + m.p1 * maxCos * sinAlpha * tanBeta);
    }
    case PT_MAT_TORRANCE_SPARROW: {
      V3 Rs = v3(m.c0x, m.c0y, m.c0z);
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
    case PT_MAT_ASHIKHMIN_SHIRLEY: {
      V3 Rd = v3(m.c0x, m.c0y, m.c0z), Rs = v3(m.c1x, m.c1y, m.c1z);
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
  return v3(0.f);
}

// ========================================================= consistent mode ==
// Device statement of the oracle's consistent mode: BRDFs in the local frame
// of the shading normal (y up), pdfs matching the samplers, importance
// sampling of the environment through a piecewise-constant 2D CDF.
PTD void env_uv(V3 d, float& u, float& v) {
  float r = length(d);
  float lon = pt_atan2f(d.z, d.x);
  float lat = pt_acosf(d.y / r);
  u = lon * (1.f / (PI_F * 2.f));
  v = lat * (1.f / PI_F);
}

PTD int cdf_find(const float* cdf, int n, float u) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(cdf + mid) <= u) lo = mid;
    else hi = mid;
  }
  return lo;
}

PTD float env_pdf_dir(const DevScene& S, V3 d) {
  if (!S.env_valid) return 0.f;
  int W = S.miss.w, H = S.miss.h;
  float u, v;
  env_uv(d, u, v);
  if (!(u == u) || !(v == v)) return 0.f;
  if (u < 0.f) u += 1.f;
  int r = (int)(v * (float)H);
  if (r < 0) r = 0;
  if (r >= H) r = H - 1;
  int c = (int)(u * (float)W);
  if (c < 0) c = 0;
  if (c >= W) c = W - 1;
  const float* cr = S.env_cond + (size_t)r * (W + 1);
  float pm = __ldg(S.env_marg + r + 1) - __ldg(S.env_marg + r);
  float pc = __ldg(cr + c + 1) - __ldg(cr + c);
  float theta = PI_F * (((float)r + 0.5f) / (float)H);
  float st = pt_sinf(theta);
  if (!(st > 0.f)) return 0.f;
  return pm * pc * (float)W * (float)H / (2.f * PI_F * PI_F * st);
}

PTD V3 env_sample_dir(const DevScene& S, float u1, float u2) {
  int W = S.miss.w, H = S.miss.h;
  int r = cdf_find(S.env_marg, H, u1);
  float m0 = __ldg(S.env_marg + r), m1 = __ldg(S.env_marg + r + 1);
  float dv = (u1 - m0) / (m1 - m0);
  const float* cr = S.env_cond + (size_t)r * (W + 1);
  int c = cdf_find(cr, W, u2);
  float c0 = __ldg(cr + c), c1 = __ldg(cr + c + 1);
  float du = (u2 - c0) / (c1 - c0);
  float v = ((float)r + dv) / (float)H;
  float u = ((float)c + du) / (float)W;
  float st, ct, sp, cp;
  pt_sincosf(PI_F * v, &st, &ct);
  pt_sincosf(2.f * PI_F * u, &sp, &cp);
  return v3(st * cp, ct, st * sp);
}

struct Frame {
  V3 t, n, b;
  PTD explicit Frame(V3 N) {
    Onb o(N);
    t = o.t;
    n = o.n;
    b = o.b;
  }
  PTD V3 to_local(V3 w) const { return v3(dot(w, t), dot(w, n), dot(w, b)); }
  PTD V3 to_world(V3 l) const { return l.x * t + l.y * n + l.z * b; }
};

PTD float GGX_G1c(V3 V, float nu, float nv) { return 1.f / (1.f + GGX_Lambda(V, nu, nv)); }

PTD V3 bsdf_f_c(const GpuMaterial& m, V3 wo, V3 wi) {
  if (!(wo.y > 0.f) || !(wi.y > 0.f)) return v3(0.f);
  V3 c0 = v3(m.c0x, m.c0y, m.c0z);
  switch (m.type) {
    case PT_MAT_LAMBERTIAN:
      return c0 * (1.f / PI_F);
    case PT_MAT_OREN_NAYAR: {
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
      return c0 * (1.f / PI_F) * (m.p0 + m.p1 * maxCos * sinAlpha * tanBeta);
    }
    case PT_MAT_TORRANCE_SPARROW: {
      V3 H = normalize(wo + wi);
      float D = GGX_D(H, m.p0, m.p1);
      float G = GGX_G(wo, wi, m.p0, m.p1);
      V3 F = schlick3(c0, fabsf(dot(H, wi)));
      return c0 * D * G * F / (4.f * wi.y * wo.y);
    }
    case PT_MAT_ASHIKHMIN_SHIRLEY: {
      V3 Rd = c0, Rs = v3(m.c1x, m.c1y, m.c1z);
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

PTD float bsdf_pdf_c(const GpuMaterial& m, V3 wo, V3 wi) {
  if (!(wo.y > 0.f) || !(wi.y > 0.f)) return 0.f;
  switch (m.type) {
    case PT_MAT_LAMBERTIAN:
    case PT_MAT_OREN_NAYAR:
      return wi.y * (1.f / PI_F);
    case PT_MAT_TORRANCE_SPARROW: {
      V3 H = normalize(wo + wi);
      float woh = dot(wo, H);
      if (!(woh > 0.f)) return 0.f;
      return GGX_G1c(wo, m.p0, m.p1) * GGX_D(H, m.p0, m.p1) / (4.f * wo.y);
    }
    case PT_MAT_ASHIKHMIN_SHIRLEY: {
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

PTD V3 bsdf_sample_c(const GpuMaterial& m, V3 wo, uint32_t& seed) {
  float rx = rnd(seed);
  float ry = rnd(seed);
  V3 p;
  switch (m.type) {
    case PT_MAT_LAMBERTIAN:
    case PT_MAT_OREN_NAYAR:
      cosine_sample_hemisphere(rx, ry, p);
      return v3(p.x, p.z, p.y);
    case PT_MAT_TORRANCE_SPARROW: {
      V3 H = normalize(GGX_Sample(wo, rx, ry, m.p0, m.p1));
      if (dot(H, wo) < 0.f) H = -H;
      return -wo + 2.f * dot(wo, H) * H;
    }
    case PT_MAT_ASHIKHMIN_SHIRLEY: {
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

PTD V3 sphere_light_sample_c(const GpuLight& L, V3 P, uint32_t& seed) {
  float r1 = rnd(seed);
  float r2 = rnd(seed);
  V3 c = v3(L.cx, L.cy, L.cz);
  V3 dc = c - P;
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

PTD float power_mis(float a, float b) { return (a * a) / (a * a + b * b); }


// ------------------------------------------------------------ textures ----
// Bilinear lookup with repeat wrap of float4 texels (row 0 at v = 0): the
// software stand-in for OptiX's hardware texture filtering (environment and
// image textures alike).
PTD V3 bilinear_rgb(const float4* texels, int w, int h, float u, float v) {
  if (!(u == u) || !(v == v) || fabsf(u) > 1e6f || fabsf(v) > 1e6f) return v3(0.f);
  float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
  float fx = ptm_floor(x), fy = ptm_floor(y);
  float ax = x - fx, ay = y - fy;
  int ix0 = (int)fx % w; if (ix0 < 0) ix0 += w;
  int iy0 = (int)fy % h; if (iy0 < 0) iy0 += h;
  int ix1 = ix0 + 1 == w ? 0 : ix0 + 1;
  int iy1 = iy0 + 1 == h ? 0 : iy0 + 1;
  V3 c00 = f4xyz(texels[iy0 * w + ix0]), c10 = f4xyz(texels[iy0 * w + ix1]);
  V3 c01 = f4xyz(texels[iy1 * w + ix0]), c11 = f4xyz(texels[iy1 * w + ix1]);
  return (c00 * (1.f - ax) + c10 * ax) * (1.f - ay) + (c01 * (1.f - ax) + c11 * ax) * ay;
}

// programs/textures/noise_texture.cu:12-59: Perlin noise over the texture's
// tables (ranvec: 256 vectors, then perm_x, perm_y, perm_z: 256 ints each).
PTD float perlin_noise(const float4* D, V3 p) {
  const int* perm = (const int*)(D + 256);
  float u = p.x - ptm_floor(p.x);
  float v = p.y - ptm_floor(p.y);
  float w = p.z - ptm_floor(p.z);
  int i = (int)ptm_floor(p.x);
  int j = (int)ptm_floor(p.y);
  int k = (int)ptm_floor(p.z);
  float uu = u * u * (3 - 2 * u);
  float vv = v * v * (3 - 2 * v);
  float ww = w * w * (3 - 2 * w);
  float accum = 0;
  for (int di = 0; di < 2; di++)
    for (int dj = 0; dj < 2; dj++)
      for (int dk = 0; dk < 2; dk++) {
        int r = perm[(i + di) & 255] ^ perm[256 + ((j + dj) & 255)] ^ perm[512 + ((k + dk) & 255)];
        V3 c = f4xyz(D[r]);
        V3 weight_v = v3(u - di, v - dj, w - dk);
        accum += (di * uu + (1 - di) * (1 - uu)) * (dj * vv + (1 - dj) * (1 - vv)) *
                 (dk * ww + (1 - dk) * (1 - ww)) * dot(c, weight_v);
      }
  return accum;
}

// noise_texture.cu:61-76: seven octaves of turbulence.
PTD float perlin_turb(const float4* D, V3 p) {
  float accum = 0;
  V3 temp_p = p;
  float weight = 1.0f;
  for (int i = 0; i < 7; i++) {
    accum += weight * perlin_noise(D, temp_p);
    weight *= 0.5f;
    temp_p *= 2.f;
  }
  return fabsf(accum);
}

// A texture's colour at (u, v, P) with texture index i (the callable
// sample_texture(u, v, p, i) of programs/textures/*.cu).  Checker and vector
// textures hand over to another texture (with index 0, as
// checkered_texture.cu:11-14 and vector.cu:7-12 call it); the chain is
// bounded (ids only decrease along it).
PTD V3 texture_color(const DevScene& S, int id, float u, float v, V3 p, int i) {
  for (int hop = 0; hop < 64; hop++) {
    const GpuTexture& t = S.textures[id];
    switch (t.kind) {
      case PT_TEX_CONSTANT:  // constant_texture.cu:5-7
        return v3(t.c[0], t.c[1], t.c[2]);
      case PT_TEX_CHECKER: {  // checkered_texture.cu:8-15
        float sines = pt_sinf(10 * p.x) * pt_sinf(10 * p.y) * pt_sinf(10 * p.z);
        id = sines < 0 ? t.a : t.b;
        i = 0;
        break;
      }
      case PT_TEX_VECTOR:  // vector.cu:7-12
        if (i >= t.b || i < 0) return v3(0.f);
        id = S.tex_list[t.a + i];
        i = 0;
        break;
      case PT_TEX_NOISE: {  // noise_texture.cu:61-76: the switch has no breaks, so
                            // every axis ends in the Z case
        float scale = t.c[0];
        float sinValue = pt_sinf(scale * p.z + 5 * perlin_turb(S.tex_data + t.data, scale * p));
        return v3(1.f) * 0.5f * (1 + sinValue);
      }
      case PT_TEX_IMAGE:  // image_texture.cu:3-7 (texels normalised to [0, 1])
        return bilinear_rgb(S.tex_data + t.data, t.a, t.b, u, v);
      default: {  // PT_TEX_GRADIENT, gradient_texture.cu:7-14
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

// The material's colours at a hit: Get_Parameters of the closest-hit
// programs (e.g. lambertian.cu:29-38) with textures in place of constants.
PTD void resolve_textures(const DevScene& S, GpuMaterial& m, float u, float v, V3 p, int i) {
  if (m.tex0 >= 0) {
    V3 c = texture_color(S, m.tex0, u, v, p, i);
    m.c0x = c.x; m.c0y = c.y; m.c0z = c.z;
  }
  if (m.tex1 >= 0) {
    V3 c = texture_color(S, m.tex1, u, v, p, i);
    m.c1x = c.x; m.c1y = c.y; m.c1z = c.z;
  }
}

}  // namespace ptd

#endif
