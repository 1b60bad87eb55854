/*
 * rtshim.h - a host-side stand-in for the parts of the OptiX 6.0 SDK that the
 * reference's device programs (programs/ of joaovbs96/OptiX-Path-Tracer) use,
 * so that those programs compile UNMODIFIED with g++ and run on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  Together with rtemu.cpp and the ref_*.cpp
 * program wrappers this builds oracle/_ref/libref.so, which the CPU tests use
 * to pin the oracle (oracle/oracle.cpp) to the reference's own code.  Nothing
 * here is part of the product.
 *
 * What OptiX supplies and the reference does not vendor is supplied here with
 * the conventions that the oracle and the CUDA kernels state for themselves:
 *   - CUDA vector types (float2/3/4, int2/3, uint2, uchar4), their make_*
 *     functions and the optixu operators and helpers (dot, cross, length,
 *     normalize = v * (1/sqrt(dot(v,v))), clamp = fmaxf(a, fminf(f, b)),
 *     saturate, reflect = i - 2 n dot(n, i));
 *   - Onb: Duff et al. 2017, "Building an Orthonormal Basis, Revisited";
 *   - cosine_sample_hemisphere: Malley's method over the Shirley-Chiu
 *     concentric map;
 *   - elementary functions (sin, cos, tan, atan, atan2, asin, acos, pow, exp,
 *     log in their float forms) routed to ptmath.h, the functions the oracle
 *     and the kernels share, in place of the GPU's fast-math intrinsics;
 *   - Ray, make_Ray, RT_DEFAULT_MAX (1e27), Aabb, rtObject, rtBuffer,
 *     rtCallableProgramId/X, rtTextureSampler + tex2D (software bilinear,
 *     repeat wrap), and the runtime calls rtTrace, rtPotentialIntersection,
 *     rtReportIntersection, rtTerminateRay, rtTransformPoint/Normal,
 *     rtGetPrimitiveIndex, rtGetTriangleBarycentrics, implemented by the
 *     emulator in rtemu.cpp;
 *   - rtDeclareVariable(T, name, semantic, annotation) declares a file-scope
 *     variable of the program's translation unit; each ref_*.cpp wrapper sets
 *     its program's variables before it calls the program, as the OptiX
 *     runtime does.
 */
#pragma once

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/types.h>

#include <cmath>
#include <cstdlib>
#include <functional>
#include <vector>

#include "../../optix-path-tracer_gb300/csrc/ptmath.h"

using std::abs;  // abs(float) must be the float overload (trigonometric.cuh:9)

// ------------------------------------------------- CUDA / OptiX qualifiers --
#define __device__
#define __host__
#define __forceinline__ inline
#define __inline__ inline
#define RT_PROGRAM static
#define RT_CALLABLE_PROGRAM static
#define RT_DEFAULT_MAX 1.e27f
#define M_PIf 3.14159265358979323846f
#define M_1_PIf 0.318309886183790671538f
#define rtDeclareVariable(type, name, semantic, annotation) static type name

namespace optix {}

// ------------------------------------------------------------ vector types --
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct int3 { int x, y, z; };
struct uint2 { unsigned int x, y; };
struct uchar4 { unsigned char x, y, z, w; };

inline float2 make_float2(float x, float y) { return float2{x, y}; }
inline float2 make_float2(float s) { return float2{s, s}; }
inline float3 make_float3(float x, float y, float z) { return float3{x, y, z}; }
inline float3 make_float3(float s) { return float3{s, s, s}; }
inline float3 make_float3(const float4& v) { return float3{v.x, v.y, v.z}; }
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
inline float4 make_float4(float s) { return float4{s, s, s, s}; }
inline int2 make_int2(int x, int y) { return int2{x, y}; }
inline int3 make_int3(int x, int y, int z) { return int3{x, y, z}; }
inline uint2 make_uint2(unsigned int x, unsigned int y) { return uint2{x, y}; }
inline uchar4 make_uchar4(unsigned char x, unsigned char y, unsigned char z, unsigned char w) {
  return uchar4{x, y, z, w};
}

inline float3 operator+(const float3& a, const float3& b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(const float3& a, const float3& b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(const float3& a, const float3& b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(const float3& a, const float3& b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator+(const float3& a, float s) { return make_float3(a.x + s, a.y + s, a.z + s); }
inline float3 operator-(const float3& a, float s) { return make_float3(a.x - s, a.y - s, a.z - s); }
inline float3 operator*(const float3& a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator/(const float3& a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
inline float3 operator+(float s, const float3& a) { return make_float3(s + a.x, s + a.y, s + a.z); }
inline float3 operator-(float s, const float3& a) { return make_float3(s - a.x, s - a.y, s - a.z); }
inline float3 operator*(float s, const float3& a) { return make_float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator-(const float3& a) { return make_float3(-a.x, -a.y, -a.z); }
inline float3& operator+=(float3& a, const float3& b) { a = a + b; return a; }
inline float3& operator-=(float3& a, const float3& b) { a = a - b; return a; }
inline float3& operator*=(float3& a, const float3& b) { a = a * b; return a; }
inline float3& operator/=(float3& a, const float3& b) { a = a / b; return a; }
inline float3& operator*=(float3& a, float s) { a = a * s; return a; }
inline float3& operator/=(float3& a, float s) { a = a / s; return a; }
inline float4 operator+(const float4& a, const float4& b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
inline float4& operator+=(float4& a, const float4& b) { a = a + b; return a; }

inline float dot(const float3& a, const float3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(const float3& a, const float3& b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const float3& a) { return ptm_sqrt(dot(a, a)); }
inline float3 normalize(const float3& a) {
  float inv = 1.0f / ptm_sqrt(dot(a, a));
  return a * inv;
}
inline float clamp(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
inline float3 clamp(const float3& v, float a, float b) {
  return make_float3(clamp(v.x, a, b), clamp(v.y, a, b), clamp(v.z, a, b));
}
inline float saturate(float f) { return clamp(f, 0.0f, 1.0f); }
inline float3 reflect(const float3& i, const float3& n) { return i - 2.0f * n * dot(n, i); }

// Orthonormal basis around a normal, Duff et al. 2017.
struct Onb {
  float3 m_tangent, m_binormal, m_normal;
  explicit Onb(const float3& n) {
    m_normal = n;
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    m_tangent = make_float3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    m_binormal = make_float3(b, sign + n.y * n.y * a, -n.y);
  }
  void inverse_transform(float3& p) const {
    p = p.x * m_tangent + p.y * m_binormal + p.z * m_normal;
  }
};

// Cosine-weighted hemisphere sample (+z up): Malley's method over the
// Shirley-Chiu concentric square-to-disk map.
inline void cosine_sample_hemisphere(float u1, float u2, float3& p) {
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

// ---------------------------------------------------------- OptiX objects --
struct Ray {
  float3 origin;
  unsigned int ray_type;
  float3 direction;
  float tmin, tmax;
};
inline Ray make_Ray(float3 origin, float3 direction, unsigned int ray_type, float tmin,
                    float tmax) {
  Ray r;
  r.origin = origin;
  r.ray_type = ray_type;
  r.direction = direction;
  r.tmin = tmin;
  r.tmax = tmax;
  return r;
}

struct Aabb {
  float3 m_min, m_max;
  // optix::Aabb::include: grows the box to hold b (component min / max)
  void include(const Aabb& b) {
    m_min = make_float3(std::fmin(m_min.x, b.m_min.x), std::fmin(m_min.y, b.m_min.y),
                        std::fmin(m_min.z, b.m_min.z));
    m_max = make_float3(std::fmax(m_max.x, b.m_max.x), std::fmax(m_max.y, b.m_max.y),
                        std::fmax(m_max.z, b.m_max.z));
  }
};
struct rtObject {};

// The scene-graph root `world`.  light_sample.cuh:69 names it inside the
// template Direct_Light before the including program declares it (nvcc
// resolves the name late, g++ at the template's definition), so `world`
// names a static function declared here; a program's
// rtDeclareVariable(rtObject, world, , ) then only redeclares it.
static inline rtObject rtemu_world_object() { return rtObject(); }
#define world rtemu_world_object()

template <class Sig> struct rtCallableProgramId;
template <class R, class... A> struct rtCallableProgramId<R(A...)> {
  std::function<R(A...)> fn;
  R operator()(A... a) const { return fn(a...); }
};
template <class Sig> using rtCallableProgramX = rtCallableProgramId<Sig>;

// Buffers view memory owned by the emulator (bound by the wrappers).  Like
// rtDeclareVariable, a buffer declaration is local to its program's
// translation unit (OptiX compiles each program to its own module).
template <class T, int Dim = 1> struct rtBufferT {
  T* data = nullptr;
  size_t n = 0;
  size_t size() const { return n; }
  T& operator[](unsigned int i) const { return data[i]; }
};
template <class T> struct rtBufferT<T, 2> {
  T* data = nullptr;
  unsigned int w = 0, h = 0;
  T& operator[](uint2 i) const { return data[(size_t)i.y * w + i.x]; }
};
#define rtBuffer static rtBufferT

// A 2D float4 texture: texels row by row, v = 0 at row 0.
template <class T, int Dim> struct rtTextureSamplerT {
  const float* texels = nullptr;
  int w = 0, h = 0;
};
#define rtTextureSampler static rtTextureSamplerT

// ----------------------------------------------------- emulated runtime ---
enum RTtransformkind { RT_OBJECT_TO_WORLD = 0xf00, RT_WORLD_TO_OBJECT = 0xf01 };

bool rtemu_potential_intersection(float t);
bool rtemu_report_intersection(unsigned int material);
void rtemu_terminate_ray();
float3 rtemu_transform_point(int kind, const float3& p);
float3 rtemu_transform_normal(int kind, const float3& n);
unsigned int rtemu_primitive_index();
float2 rtemu_triangle_barycentrics();
void rtemu_trace(const Ray& ray, void* payload);
float4 rtemu_tex2d(const float* texels, int w, int h, float u, float v);

inline bool rtPotentialIntersection(float t) { return rtemu_potential_intersection(t); }
inline bool rtReportIntersection(unsigned int material) {
  return rtemu_report_intersection(material);
}
inline void rtTerminateRay() { rtemu_terminate_ray(); }
inline float3 rtTransformPoint(RTtransformkind kind, const float3& p) {
  return rtemu_transform_point(kind, p);
}
inline float3 rtTransformNormal(RTtransformkind kind, const float3& n) {
  return rtemu_transform_normal(kind, n);
}
inline unsigned int rtGetPrimitiveIndex() { return rtemu_primitive_index(); }
inline float2 rtGetTriangleBarycentrics() { return rtemu_triangle_barycentrics(); }
template <class Payload> inline void rtTrace(const rtObject&, const Ray& ray, Payload& prd) {
  rtemu_trace(ray, &prd);
}
template <class T, int Dim>
inline float4 tex2D(const rtTextureSamplerT<T, Dim>& s, float u, float v) {
  return rtemu_tex2d(s.texels, s.w, s.h, u, v);
}

// ---------------------------------------------- argument evaluation order --
// Some programs draw several random numbers in one argument list
// (lambertian.cuh:13, oren_nayar.cuh:14, torrance_sparrow.cuh:25,
// ashikhmin_shirley.cuh:28, rect_pdf.cu:116-145), whose evaluation order C++
// leaves unspecified.  The oracle and the kernels draw them left to right;
// so that the host compiler does too, these three calls take their
// arguments through a braced list, which is evaluated in order.
struct Float2Args {
  float2 v;
  template <class A, class B> Float2Args(A a, B b) : v{(float)a, (float)b} {}
  template <class A> Float2Args(A s) : v{(float)s, (float)s} {}
};
struct Float3Args {
  float3 v;
  template <class A, class B, class C> Float3Args(A a, B b, C c) : v{(float)a, (float)b, (float)c} {}
  template <class A> Float3Args(A s) : v{(float)s, (float)s, (float)s} {}
  Float3Args(const float4& q) : v{q.x, q.y, q.z} {}
};
struct CosineSampleArgs {
  float u1, u2;
  float3* p;
  template <class A, class B> CosineSampleArgs(A a, B b, float3& out) : u1(a), u2(b), p(&out) {}
};
inline void cosine_sample_hemisphere_in_order(const CosineSampleArgs& a) {
  cosine_sample_hemisphere(a.u1, a.u2, *a.p);
}
#define make_float2(...) (Float2Args{__VA_ARGS__}.v)
#define make_float3(...) (Float3Args{__VA_ARGS__}.v)
#define cosine_sample_hemisphere(...) cosine_sample_hemisphere_in_order(CosineSampleArgs{__VA_ARGS__})

// ------------------------------------------------- elementary functions ---
// The float forms used by programs/ (sin, cos, tan, atan, atan2, asin, acos,
// pow, exp, log) go to ptmath.h.  sqrt, fabs, floor and fmod are exact in
// IEEE arithmetic and stay with the C library.  Every system header is
// included above this point.
#define sin(x) pt_sinf(x)
#define sinf(x) pt_sinf(x)
#define cos(x) pt_cosf(x)
#define cosf(x) pt_cosf(x)
#define tanf(x) pt_tanf(x)
#define atanf(x) pt_atanf(x)
#define atan2(y, x) pt_atan2f(y, x)
#define atan2f(y, x) pt_atan2f(y, x)
#define asin(x) pt_asinf(x)
#define acos(x) pt_acosf(x)
#define acosf(x) pt_acosf(x)
#define powf(x, y) pt_powf(x, y)
#define expf(x) pt_expf(x)
#define logf(x) pt_logf(x)
