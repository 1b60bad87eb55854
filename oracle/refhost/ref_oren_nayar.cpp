// Wrapper of programs/materials/oren_nayar.cu (test infrastructure, see rtshim.h).
#include "rtemu.h"
#include "materials/oren_nayar.cu"
#include "ref_common.h"

REF_BIND_LIGHTS()

extern "C" void ref_oren_nayar_hit(void* p_prd, const Ray* r, float t, int gi, float2 b,
                             const int* tex, const float* p) {
  (void)p;
  bind_hitrecord(Get_HitRecord);
  bind_texture(sample_texture, tex[0]);
  bind_lights();
  rA = p[0];
  rB = p[1];
  REF_RUN_CLOSEST_HIT(p_prd, r, t, gi, b);
}
