// Wrapper of programs/textures/constant_texture.cu (test infrastructure, see
// rtshim.h).
#include "rtemu.h"
#include "textures/constant_texture.cu"

extern "C" float3 ref_constant_texture(const float* c, float u, float v, const float3* p, int i) {
  color = make_float3(c[0], c[1], c[2]);
  return sample_texture(u, v, *p, i);
}
