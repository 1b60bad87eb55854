// Wrapper of programs/textures/checkered_texture.cu (test infrastructure, see
// rtshim.h).  odd / even are texture ids of the scene.
#include "rtemu.h"
#include "textures/checkered_texture.cu"
#include "ref_common_tex.h"

extern "C" float3 ref_checker_texture(int odd_id, int even_id, float u, float v, const float3* p,
                                      int i) {
  bind_texture_fn(odd, odd_id);
  bind_texture_fn(even, even_id);
  return sample_texture(u, v, *p, i);
}
