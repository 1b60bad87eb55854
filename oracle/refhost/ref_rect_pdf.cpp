// Wrapper of programs/pdfs/rect_pdf.cu, the rectangle light callables (test
// infrastructure, see rtshim.h).
#include "rtemu.h"
#include "pdfs/rect_pdf.cu"

static void set_rect(const float* f) {
  a0 = f[0];
  a1 = f[1];
  b0 = f[2];
  b1 = f[3];
  k = f[4];
}

extern "C" float3 ref_rect_light_sample(const float* f, int axis, const float3* P,
                                        const float3* Wo, const float3* N, unsigned int* seed) {
  set_rect(f);
  uint s = *seed;
  float3 r = axis == 0 ? Sample_X(*P, *Wo, *N, s)
                       : (axis == 1 ? Sample_Y(*P, *Wo, *N, s) : Sample_Z(*P, *Wo, *N, s));
  *seed = s;
  return r;
}

extern "C" float ref_rect_light_pdf(const float* f, int axis, const float3* P, const float3* Wo,
                                    const float3* Wi, const float3* N) {
  set_rect(f);
  return axis == 0 ? PDF_X(*P, *Wo, *Wi, *N)
                   : (axis == 1 ? PDF_Y(*P, *Wo, *Wi, *N) : PDF_Z(*P, *Wo, *Wi, *N));
}
