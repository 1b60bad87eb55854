// Wrapper of programs/hitables/box.cu (test infrastructure, see rtshim.h).
#include "rtemu.h"
#include "hitables/box.cu"
#include "ref_common.h"

static void set_box(const float* f) {
  boxmin = make_float3(f[0], f[1], f[2]);
  boxmax = make_float3(f[3], f[4], f[5]);
}

extern "C" void ref_box_intersect(const float* f, const Ray* r, int* gi, float2* b) {
  set_box(f);
  ray = *r;
  Intersect(0);
  *gi = geo_index;
  *b = bc;
}

extern "C" void ref_box_hitrecord(const float* f, int index, const Ray* r, float t, float2 b,
                                  EmuRec* out) {
  set_box(f);
  *out = to_emu(Get_HitRecord(index, *r, t, b));
}

extern "C" void ref_box_bounds(const float* f, float* box6) {
  set_box(f);
  Get_Bounds(0, box6);
}
