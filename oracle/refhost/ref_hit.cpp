// Wrapper of programs/hit.cu, the shadow-ray any-hit program (test
// infrastructure, see rtshim.h).
#include "rtemu.h"
#include "hit.cu"

extern "C" void ref_any_hit(int light, const Ray* r, void* p) {
  is_light = light;
  ray = *r;
  prd_shadow = *(PerRayData_Shadow*)p;
  any_hit();
  *(PerRayData_Shadow*)p = prd_shadow;
}

// A shadow ray that hits nothing: the reference has no miss program for ray
// type 1 and leaves inShadow as Direct_Light declared it (uninitialised,
// light_sample.cuh:63).  Here, as in the oracle and the kernels, a miss
// counts as occluded.
extern "C" void ref_shadow_miss(void* p) { ((PerRayData_Shadow*)p)->inShadow = true; }
