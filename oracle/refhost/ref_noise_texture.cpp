// Wrapper of programs/textures/noise_texture.cu (test infrastructure, see
// rtshim.h).  ranvec: 256 float3, perm: perm_x, perm_y, perm_z (3 x 256).
#include "rtemu.h"
#include "textures/noise_texture.cu"

extern "C" float3 ref_noise_texture(float s, int axis, const float3* rv, const int* perm, float u,
                                    float v, const float3* p, int i) {
  scale = s;
  ax = axis;
  ranvec.data = const_cast<float3*>(rv);
  ranvec.n = 256;
  perm_x.data = const_cast<int*>(perm);
  perm_x.n = 256;
  perm_y.data = const_cast<int*>(perm + 256);
  perm_y.n = 256;
  perm_z.data = const_cast<int*>(perm + 512);
  perm_z.n = 256;
  return sample_texture(u, v, *p, i);
}
