// Wrapper of programs/pdfs/sphere_pdf.cu, the sphere light callables (test
// infrastructure, see rtshim.h).
#include "rtemu.h"
#include "pdfs/sphere_pdf.cu"

extern "C" float3 ref_sphere_light_sample(const float* f, const float3* P, const float3* Wo,
                                          const float3* N, unsigned int* seed) {
  center = make_float3(f[0], f[1], f[2]);
  radius = f[3];
  uint s = *seed;
  float3 r = Sample(*P, *Wo, *N, s);
  *seed = s;
  return r;
}

extern "C" float ref_sphere_light_pdf(const float* f, const float3* P, const float3* Wo,
                                      const float3* Wi, const float3* N) {
  center = make_float3(f[0], f[1], f[2]);
  radius = f[3];
  return PDF(*P, *Wo, *Wi, *N);
}
