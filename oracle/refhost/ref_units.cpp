// Function-level entry points into the reference's device headers (test
// infrastructure, see rtshim.h): programs/random.cuh, sampling.cuh,
// materials/{material,microfacets,lambertian,oren_nayar,torrance_sparrow,
// ashikhmin_shirley,diffuse_light}.cuh and math/trigonometric.cuh, compiled
// unmodified.  Plain pointers and sizes, for ctypes.
#include "rtemu.h"
#include "materials/light_sample.cuh"

enum { LAMBERTIAN = 0, METAL, DIELECTRIC, DIFFUSE_LIGHT, OREN_NAYAR, TORRANCE_SPARROW,
       ASHIKHMIN_SHIRLEY };

static float3 f3(const float* p) { return make_float3(p[0], p[1], p[2]); }
static void put3(float* o, const float3& v) {
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
}

// The host material classes' parameter conversions: Oren_Nayar
// (host_includes/materials.hpp:192-198), Torrance_Sparrow roughnessToAlpha
// (:227-238), Ashikhmin_Shirley (:173-174).
extern "C" void ref_convert_params(int type, float p0, float p1, float* q) {
  q[0] = p0;
  q[1] = p1;
  if (type == OREN_NAYAR) {
    float sigma = saturate(p0);
    float div = 1.f / (PI_F + ((3.f * PI_F - 4.f) / 6.f) * sigma);
    q[0] = 1.0f * div;
    q[1] = sigma * div;
  } else if (type == TORRANCE_SPARROW) {
    float R0 = fmaxf(p0, 1e-3f), R1 = fmaxf(p1, 1e-3f);
    q[0] = R0 * R0;
    q[1] = R1 * R1;
  } else if (type == ASHIKHMIN_SHIRLEY) {
    q[0] = fmaxf(1.f, p0);
    q[1] = fmaxf(1.f, p1);
  }
}

extern "C" uint32_t ref_tea64(uint32_t a, uint32_t b) { return tea<64>(a, b); }

extern "C" void ref_lcg_stream(uint32_t seed, int n, uint32_t* out) {
  unsigned int s = seed;
  for (int i = 0; i < n; i++) out[i] = lcg(s);
}

extern "C" void ref_rnd_stream(uint32_t seed, int n, float* out) {
  unsigned int s = seed;
  for (int i = 0; i < n; i++) out[i] = rnd(s);
}

// kind 0 random_in_unit_disk, 1 random_in_unit_sphere, 2 random_on_unit_sphere
// (sampling.cuh:22-59): n draws of 3 floats from one seed stream.
extern "C" void ref_sampling(int kind, uint32_t seed, int n, float* out) {
  uint s = seed;
  for (int i = 0; i < n; i++) {
    float3 v = kind == 0 ? random_in_unit_disk(s)
                         : (kind == 1 ? random_in_unit_sphere(s) : random_on_unit_sphere(s));
    put3(out + 3 * i, v);
  }
}

template <class F> static void with_surface(int type, const float* c0, const float* c1, float p0,
                                            float p1, F&& f) {
  float q[2];
  ref_convert_params(type, p0, p1, q);
  switch (type) {
    case LAMBERTIAN: {
      Lambertian_Parameters s;
      s.color = f3(c0);
      f(s);
      break;
    }
    case DIFFUSE_LIGHT: {
      Diffuse_Light_Parameters s;
      s.color = f3(c0);
      f(s);
      break;
    }
    case OREN_NAYAR: {
      Oren_Nayar_Parameters s;
      s.color = f3(c0);
      s.rA = q[0];
      s.rB = q[1];
      f(s);
      break;
    }
    case TORRANCE_SPARROW: {
      Torrance_Sparrow_Parameters s;
      s.color = f3(c0);
      s.nu = q[0];
      s.nv = q[1];
      f(s);
      break;
    }
    case ASHIKHMIN_SHIRLEY: {
      Ashikhmin_Shirley_Parameters s;
      s.diffuse_color = f3(c0);
      s.specular_color = f3(c1);
      s.nu = q[0];
      s.nv = q[1];
      f(s);
      break;
    }
    default:
      break;
  }
}

// Sample(surface, P, Wo, N, seed) of one material for n (Wo, N, seed)
// triples; seeds are advanced in place.  P is not used by any Sample.
extern "C" void ref_brdf_sample(int type, const float* c0, const float* c1, float p0, float p1,
                                int n, const float* Wo, const float* N, uint32_t* seeds,
                                float* Wi) {
  with_surface(type, c0, c1, p0, p1, [&](const auto& s) {
    for (int i = 0; i < n; i++) {
      uint seed = seeds[i];
      float3 w = Sample(s, make_float3(0.f), f3(Wo + 3 * i), f3(N + 3 * i), seed);
      seeds[i] = seed;
      put3(Wi + 3 * i, w);
    }
  });
}

// Evaluate(surface, P, Wo, Wi, N, pdf) for n (Wo, Wi, N) triples.  A pdf
// that Evaluate does not set stays 0.
extern "C" void ref_brdf_eval(int type, const float* c0, const float* c1, float p0, float p1,
                              int n, const float* Wo, const float* Wi, const float* N, float* f,
                              float* pdf) {
  with_surface(type, c0, c1, p0, p1, [&](const auto& s) {
    for (int i = 0; i < n; i++) {
      float pd = 0.f;
      float3 v = Evaluate(s, make_float3(0.f), f3(Wo + 3 * i), f3(Wi + 3 * i), f3(N + 3 * i), pd);
      put3(f + 3 * i, v);
      pdf[i] = pd;
    }
  });
}

// Helpers of material.cuh, microfacets.cuh and trigonometric.cuh over n
// inputs of `stride` floats each (see the cases).
extern "C" void ref_helper(int fn, int n, const float* in, float* out) {
  for (int i = 0; i < n; i++) {
    const float* a = in + 8 * i;
    float* o = out + 4 * i;
    switch (fn) {
      case 0:  // schlick(cosine, ref_idx)
        o[0] = schlick(a[0], a[1]);
        break;
      case 1: {  // Refract(v, n, ni_over_nt, refracted) -> (refracted, ok)
        float3 r = make_float3(0.f);
        bool ok = Refract(f3(a), f3(a + 3), a[6], r);
        put3(o, r);
        o[3] = ok ? 1.f : 0.f;
        break;
      }
      case 2: {  // GGX_Sample(origin, (rx, ry), nu, nv)
        float3 h = GGX_Sample(f3(a), make_float2(a[3], a[4]), a[5], a[6]);
        put3(o, h);
        break;
      }
      case 3: {  // GGX_D(H, nu, nv), GGX_G(Wo=H, Wi, nu, nv) with Wi = a[3..5]
        o[0] = GGX_D(f3(a), a[6], a[7]);
        o[1] = GGX_G(f3(a), f3(a + 3), a[6], a[7]);
        o[2] = GGX_PDF(f3(a), f3(a + 3), a[6], a[7]);
        break;
      }
      case 4: {  // Sample_Quadrant(nu, nv, rx, ry) -> (phi, theta)
        float phi, theta;
        Sample_Quadrant(a[0], a[1], a[2], a[3], phi, theta);
        o[0] = phi;
        o[1] = theta;
        break;
      }
      case 5: {  // trigonometric.cuh on w: AbsCosTheta, SinTheta, CosPhi, SinPhi
        float3 w = f3(a);
        o[0] = AbsCosTheta(w);
        o[1] = SinTheta(w);
        o[2] = CosPhi(w);
        o[3] = SinPhi(w);
        break;
      }
    }
  }
}
