/*
 * ref_common.h - helpers shared by the program wrappers (ref_*.cpp).  Each
 * wrapper includes one of the reference's programs first, then this file, so
 * the reference's own types (HitRecord, PerRayData, the callable typedefs)
 * are in scope.  TEST INFRASTRUCTURE ONLY (see rtshim.h).
 */
#pragma once
#include <type_traits>

#include "rtemu.h"

inline EmuRec to_emu(const HitRecord& r) {
  EmuRec e;
  e.index = r.index;
  e.P = r.P;
  e.u = r.u;
  e.v = r.v;
  e.geometric_normal = r.geometric_normal;
  e.shading_normal = r.shading_normal;
  e.Wo = r.Wo;
  return e;
}

inline HitRecord from_emu(const EmuRec& e) {
  HitRecord r;
  memset(&r, 0, sizeof(r));
  r.index = e.index;
  r.P = e.P;
  r.u = e.u;
  r.v = e.v;
  r.geometric_normal = e.geometric_normal;
  r.shading_normal = e.shading_normal;
  r.Wo = e.Wo;
  return r;
}

// Binds a HitRecord_Function variable to the primitive the runtime reports.
template <class F> inline void bind_hitrecord(F& f) {
  f.fn = [](int index, Ray r, float t, float2 b) {
    EmuRec e;
    rtemu_hitrecord(index, r, t, b, &e);
    return from_emu(e);
  };
}

// Binds a Texture_Function variable to texture `tex` of the scene.
template <class F> inline void bind_texture(F& f, int tex) {
  f.fn = [tex](float u, float v, float3 p, int i) { return rtemu_texture(tex, u, v, p, i); };
}

// The light buffers of programs/materials/light_sample.cuh:13-25, bound to the
// scene's lights once per scene (rtemu_scene_generation changes on commit).
int rtemu_scene_generation();

#define REF_BIND_LIGHTS()                                                                    \
  static void bind_lights() {                                                                \
    static int gen = -1;                                                                     \
    if (gen == rtemu_scene_generation()) return;                                             \
    gen = rtemu_scene_generation();                                                          \
    using SampleFn = std::remove_reference<decltype(Light_Sample[0])>::type;                 \
    using PdfFn = std::remove_reference<decltype(Light_PDF[0])>::type;                       \
    static std::vector<float3> ev;                                                           \
    static std::vector<SampleFn> sv;                                                         \
    static std::vector<PdfFn> pv;                                                            \
    int n = rtemu_num_lights();                                                              \
    ev.assign(n, make_float3(0.f));                                                          \
    sv.assign(n, SampleFn());                                                                \
    pv.assign(n, PdfFn());                                                                   \
    for (int k = 0; k < n; k++) {                                                            \
      ev[k] = rtemu_light_emission(k);                                                       \
      sv[k].fn = [k](const float3& P, const float3& Wo, const float3& N, uint& s) {          \
        return rtemu_light_sample(k, P, Wo, N, s);                                           \
      };                                                                                     \
      pv[k].fn = [k](const float3& P, const float3& Wo, const float3& Wi, const float3& N) { \
        return rtemu_light_pdf(k, P, Wo, Wi, N);                                             \
      };                                                                                     \
    }                                                                                        \
    numLights = n;                                                                           \
    Light_Emissions.data = ev.data();                                                        \
    Light_Emissions.n = (size_t)n;                                                           \
    Light_Sample.data = sv.data();                                                           \
    Light_Sample.n = (size_t)n;                                                              \
    Light_PDF.data = pv.data();                                                              \
    Light_PDF.n = (size_t)n;                                                                 \
  }

// Sets the closest-hit program's semantic variables and payload, runs it and
// copies the payload back (OptiX passes the payload by reference).
#define REF_RUN_CLOSEST_HIT(prd_ptr, ray_ptr, t, gi, b) \
  do {                                                  \
    ray = *(ray_ptr);                                   \
    t_hit = (t);                                        \
    geo_index = (gi);                                   \
    bc = (b);                                           \
    prd = *(PerRayData*)(prd_ptr);                      \
    closest_hit();                                      \
    *(PerRayData*)(prd_ptr) = prd;                      \
  } while (0)
