// Wrapper of programs/textures/image_texture.cu (test infrastructure, see
// rtshim.h).  The sampler reads float RGBA texels with the stand-in tex2D.
#include "rtemu.h"
#include "textures/image_texture.cu"

extern "C" float3 ref_image_texture(const float* texels, int w, int h, float u, float v,
                                    const float3* p, int i) {
  data.texels = texels;
  data.w = w;
  data.h = h;
  return sample_texture(u, v, *p, i);
}
