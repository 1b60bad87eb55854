/*
 * rtemu.h - interface between the emulated OptiX runtime (rtemu.cpp) and the
 * wrappers (ref_*.cpp) that each compile one of the reference's device
 * programs unmodified.  TEST INFRASTRUCTURE ONLY (see rtshim.h).
 *
 * A wrapper owns one program's translation unit: its rtDeclareVariable
 * variables and rtBuffers are file-scope statics there, so only the wrapper
 * can set them.  The runtime calls the wrappers' extern "C" entry points
 * declared below; the wrappers call back into the runtime for what OptiX
 * would provide across programs (texture and light callables, the HitRecord
 * callable of the primitive that was hit, nested rtTrace).
 */
#pragma once
#include "rtshim.h"

// The reference's HitRecord (programs/prd.cuh:32-42) as plain fields, so that
// translation units without prd.cuh can pass it along.
struct EmuRec {
  int index;
  float3 P;
  float u, v;
  float3 geometric_normal, shading_normal, Wo;
};

// Callables the runtime binds into programs (rtCallableProgramId targets).
float3 rtemu_texture(int texture, float u, float v, const float3& p, int i);
void rtemu_hitrecord(int index, const Ray& ray, float t_hit, float2 bc, EmuRec* out);
int rtemu_num_lights();
float3 rtemu_light_emission(int light);
float3 rtemu_light_sample(int light, const float3& P, const float3& Wo, const float3& N,
                          unsigned int& seed);
float rtemu_light_pdf(int light, const float3& P, const float3& Wo, const float3& Wi,
                      const float3& N);

extern "C" {
// programs/hitables/{sphere,aarect,box,triangle}.cu.  Intersection entry
// points run the program's intersection routine on `ray` (object space) and
// return the attributes it wrote (valid when it reported an intersection).
void ref_sphere_intersect(const float* f, const Ray* ray, int* geo_index, float2* bc);
void ref_sphere_hitrecord(const float* f, int index, const Ray* ray, float t, float2 bc,
                          EmuRec* out);
void ref_sphere_bounds(const float* f, float* box6);
void ref_aarect_intersect(const float* f, int axis, int flip, const Ray* ray, int* geo_index,
                          float2* bc);
void ref_aarect_hitrecord(const float* f, int axis, int flip, int index, const Ray* ray,
                          float t, float2 bc, EmuRec* out);
void ref_aarect_bounds(const float* f, int axis, float* box6);
void ref_box_intersect(const float* f, const Ray* ray, int* geo_index, float2* bc);
void ref_box_hitrecord(const float* f, int index, const Ray* ray, float t, float2 bc,
                       EmuRec* out);
void ref_box_bounds(const float* f, float* box6);
// programs/hitables/moving_sphere.cu (its record is the hit_rec attribute;
// out = P, shading normal, u, v, Wo of the reported hit)
void ref_msphere_intersect(const float* f, const Ray* ray, float time, float* out);
void ref_msphere_bounds(const float* f, float* box6);
void ref_triangle_bind(const float3* verts, size_t nv, const float3* normals, size_t nn,
                       const float2* uvs, size_t nuv, const int3* idx, size_t nt,
                       const int* mats);
void ref_triangle_attributes(int* geo_index, float2* bc);
void ref_triangle_intersect(int pid, const Ray* ray, int* geo_index, float2* bc);
void ref_triangle_hitrecord(int index, const Ray* ray, float t, float2 bc, EmuRec* out);
void ref_triangle_bounds(int pid, float* box6);

// programs/materials/*.cu closest-hit programs.  prd points at the
// reference's PerRayData; tex lists the material's texture callables;
// p its float variables (fuzz; ref_idx, density; rA, rB; nu, nv).
void ref_lambertian_hit(void* prd, const Ray* ray, float t, int geo_index, float2 bc,
                        const int* tex, const float* p);
void ref_metal_hit(void* prd, const Ray* ray, float t, int geo_index, float2 bc,
                   const int* tex, const float* p);
void ref_dielectric_hit(void* prd, const Ray* ray, float t, int geo_index, float2 bc,
                        const int* tex, const float* p);
void ref_diffuse_light_hit(void* prd, const Ray* ray, float t, int geo_index, float2 bc,
                           const int* tex, const float* p);
void ref_oren_nayar_hit(void* prd, const Ray* ray, float t, int geo_index, float2 bc,
                        const int* tex, const float* p);
void ref_torrance_sparrow_hit(void* prd, const Ray* ray, float t, int geo_index, float2 bc,
                              const int* tex, const float* p);
void ref_ashikhmin_shirley_hit(void* prd, const Ray* ray, float t, int geo_index, float2 bc,
                               const int* tex, const float* p);

// programs/hit.cu any-hit program (shadow rays) and the shadow-ray miss.
void ref_any_hit(int is_light, const Ray* ray, void* prd_shadow);
void ref_shadow_miss(void* prd_shadow);

// programs/miss.cu: kind 0 gradient, 1 constant, 2 HDR environment, 3 image.
void ref_miss(int kind, const int* tex, int is_spherical, const Ray* ray, void* prd);

// programs/pdfs/{rect,sphere}_pdf.cu light callables.
float3 ref_rect_light_sample(const float* f, int axis, const float3* P, const float3* Wo,
                             const float3* N, unsigned int* seed);
float ref_rect_light_pdf(const float* f, int axis, const float3* P, const float3* Wo,
                         const float3* Wi, const float3* N);
float3 ref_sphere_light_sample(const float* f, const float3* P, const float3* Wo,
                               const float3* N, unsigned int* seed);
float ref_sphere_light_pdf(const float* f, const float3* P, const float3* Wo, const float3* Wi,
                           const float3* N);

// programs/textures/*.cu texture callables
float3 ref_constant_texture(const float* color, float u, float v, const float3* p, int i);
float3 ref_image_texture(const float* texels, int w, int h, float u, float v, const float3* p,
                         int i);
float3 ref_checker_texture(int odd_id, int even_id, float u, float v, const float3* p, int i);
float3 ref_noise_texture(float scale, int axis, const float3* ranvec, const int* perm, float u,
                         float v, const float3* p, int i);
float3 ref_gradient_texture(const float* c, float u, float v, const float3* p, int i);
float3 ref_vector_texture(int self, const int* ids, int n, float u, float v, const float3* p,
                          int i);

// programs/raygen.cu renderPixel: one launch index of one frame; acc and
// display are W x H buffers (row y holds launch row H-1-y).
void ref_render_pixel(unsigned int x, unsigned int y, unsigned int W, unsigned int H, int frame,
                      int russian, int max_depth, const float* camera, float4* acc,
                      uchar4* display);
}
