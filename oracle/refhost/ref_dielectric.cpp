// Wrapper of programs/materials/dielectric.cu (test infrastructure, see
// rtshim.h).
#include "rtemu.h"
#include "materials/dielectric.cu"
#include "ref_common.h"

extern "C" void ref_dielectric_hit(void* p_prd, const Ray* r, float t, int gi, float2 b,
                                   const int* tex, const float* p) {
  bind_hitrecord(Get_HitRecord);
  bind_texture(base_texture, tex[0]);
  bind_texture(extinction_texture, tex[1]);
  ref_idx = p[0];
  density = p[1];
  REF_RUN_CLOSEST_HIT(p_prd, r, t, gi, b);
}
