// Wrapper of programs/materials/metal.cu (test infrastructure, see rtshim.h).
#include "rtemu.h"
#include "materials/metal.cu"
#include "ref_common.h"

extern "C" void ref_metal_hit(void* p_prd, const Ray* r, float t, int gi, float2 b,
                              const int* tex, const float* p) {
  bind_hitrecord(Get_HitRecord);
  bind_texture(sample_texture, tex[0]);
  fuzz = p[0];
  REF_RUN_CLOSEST_HIT(p_prd, r, t, gi, b);
}
