// Wrapper of programs/textures/gradient_texture.cu (test infrastructure, see
// rtshim.h).  c: colorA, colorB, colorC.
#include "rtemu.h"
#include "textures/gradient_texture.cu"

extern "C" float3 ref_gradient_texture(const float* c, float u, float v, const float3* p, int i) {
  colorA = make_float3(c[0], c[1], c[2]);
  colorB = make_float3(c[3], c[4], c[5]);
  colorC = make_float3(c[6], c[7], c[8]);
  return sample_texture(u, v, *p, i);
}
