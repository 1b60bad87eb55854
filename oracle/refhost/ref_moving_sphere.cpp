// Wrapper of programs/hitables/moving_sphere.cu (test infrastructure, see
// rtshim.h).  The program writes its hit record as the `hit_rec` attribute
// and reads the ray's time from the radiance payload (prd.time); the wrapper
// sets both and returns the attribute.
#include "rtemu.h"
// the program's `index` variable would clash with the C library's index()
#define index ms_index
#include "hitables/moving_sphere.cu"

static void set_msphere(const float* f) {
  center0 = make_float3(f[0], f[1], f[2]);
  radius = f[3];
  time0 = f[4];
  time1 = f[5];
  center1 = make_float3(f[6], f[7], f[8]);
  ms_index = 0;
}

// out = P (3), shading normal (3), u, v, Wo (3) of the reported hit.
extern "C" void ref_msphere_intersect(const float* f, const Ray* r, float time, float* out) {
  set_msphere(f);
  ray = *r;
  prd.time = time;
  hit_sphere(0);
  const float v[11] = {hit_rec.P.x, hit_rec.P.y, hit_rec.P.z, hit_rec.shading_normal.x,
                       hit_rec.shading_normal.y, hit_rec.shading_normal.z, hit_rec.u, hit_rec.v,
                       hit_rec.Wo.x, hit_rec.Wo.y, hit_rec.Wo.z};
  for (int k = 0; k < 11; k++) out[k] = v[k];
}

extern "C" void ref_msphere_bounds(const float* f, float* box6) {
  set_msphere(f);
  get_bounds(0, box6);
}
