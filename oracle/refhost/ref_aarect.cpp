// Wrapper of programs/hitables/aarect.cu (test infrastructure, see rtshim.h).
#include "rtemu.h"
#include "hitables/aarect.cu"
#include "ref_common.h"

static void set_rect(const float* f, int ax, int fl) {
  a0 = f[0];
  a1 = f[1];
  b0 = f[2];
  b1 = f[3];
  k = f[4];
  axis = ax;
  flip = fl;
}

extern "C" void ref_aarect_intersect(const float* f, int ax, int fl, const Ray* r, int* gi,
                                     float2* b) {
  set_rect(f, ax, fl);
  ray = *r;
  Hit_Rect(0);
  *gi = geo_index;
  *b = bc;
}

extern "C" void ref_aarect_hitrecord(const float* f, int ax, int fl, int index, const Ray* r,
                                     float t, float2 b, EmuRec* out) {
  set_rect(f, ax, fl);
  *out = to_emu(Get_HitRecord(index, *r, t, b));
}

extern "C" void ref_aarect_bounds(const float* f, int ax, float* box6) {
  set_rect(f, ax, 0);
  Get_Bounds(0, box6);
}
