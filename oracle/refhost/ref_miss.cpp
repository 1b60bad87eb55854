// Wrapper of programs/miss.cu (test infrastructure, see rtshim.h).
#include "rtemu.h"
#include "miss.cu"
#include "ref_common.h"

extern "C" void ref_miss(int kind, const int* tex, int spherical, const Ray* r, void* p) {
  ray = *r;
  prd = *(PerRayData*)p;
  switch (kind) {
    case 0:
      bind_texture(sample_color1, tex[0]);
      bind_texture(sample_color2, tex[1]);
      gradient_color();
      break;
    case 1:
      bind_texture(sample_texture, tex[0]);
      constant_color();
      break;
    case 2:
      bind_texture(sample_texture, tex[0]);
      isSpherical = spherical;
      environmental_mapping();
      break;
    default:
      bind_texture(sample_texture, tex[0]);
      image_background();
      break;
  }
  *(PerRayData*)p = prd;
}
