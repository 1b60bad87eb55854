// Wrapper of programs/hitables/sphere.cu (test infrastructure, see rtshim.h).
#include "rtemu.h"
#include "hitables/sphere.cu"
#include "ref_common.h"

static void set_sphere(const float* f) {
  center = make_float3(f[0], f[1], f[2]);
  radius = f[3];
}

extern "C" void ref_sphere_intersect(const float* f, const Ray* r, int* gi, float2* b) {
  set_sphere(f);
  ray = *r;
  hit_sphere(0);
  *gi = geo_index;
  *b = bc;
}

extern "C" void ref_sphere_hitrecord(const float* f, int index, const Ray* r, float t,
                                     float2 b, EmuRec* out) {
  set_sphere(f);
  *out = to_emu(Get_HitRecord(index, *r, t, b));
}

extern "C" void ref_sphere_bounds(const float* f, float* box6) {
  set_sphere(f);
  get_bounds(0, box6);
}
