// Wrapper of programs/materials/ashikhmin_shirley.cu (test infrastructure,
// see rtshim.h).
#include "rtemu.h"
#include "materials/ashikhmin_shirley.cu"
#include "ref_common.h"

REF_BIND_LIGHTS()

extern "C" void ref_ashikhmin_shirley_hit(void* p_prd, const Ray* r, float t, int gi, float2 b,
                                          const int* tex, const float* p) {
  bind_hitrecord(Get_HitRecord);
  bind_texture(diffuse_color, tex[0]);
  bind_texture(specular_color, tex[1]);
  bind_lights();
  nu = p[0];
  nv = p[1];
  REF_RUN_CLOSEST_HIT(p_prd, r, t, gi, b);
}
