/*
 * pt_types.h - data layout in device memory, shared by host and device code.
 *
 * Primitive record (48 B, 3 x float4, stored in BVH leaf order):
 *   r0 = (f0, f1, f2, tag)     tag bits 0-1 type, 2-3 axis, 4 flip, 5 moving
 *                              sphere, 8-31 transform index + 1 (0 = world space)
 *   r1 = (f3, f4, f5, prim id) prim id = call-order id (tie-break, output)
 *   r2 = (f6, f7, f8, material id)
 *   triangle: f0..2 = v0, f3..5 = v1, f6..8 = v2 (world space)
 *   sphere:   f0..2 = centre, f3 = radius
 *   moving sphere (type sphere, tag bit 5): f0..2 = centre at time0,
 *             f3 = radius, f4 = time0, f5 = time1, f6..8 = centre at time1
 *   rect:     f0..4 = a0, a1, b0, b1, k
 *   box:      f0..2 = min, f3..5 = max
 * BVH8 node (80 B, 5 x uint4), compressed child boxes after Ylitie, Karras &
 * Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
 * BVHs", HPG 2017:
 *   n0 = (p.x, p.y, p.z as float bits, ex | ey<<8 | ez<<16 | imask<<24)
 *   n1 = (child_base, prim_base, meta[0..3], meta[4..7])
 *   n2 = (qlo.x[0..3], qlo.x[4..7], qlo.y[0..3], qlo.y[4..7])
 *   n3 = (qlo.z[0..3], qlo.z[4..7], qhi.x[0..3], qhi.x[4..7])
 *   n4 = (qhi.y[0..3], qhi.y[4..7], qhi.z[0..3], qhi.z[4..7])
 *   child box = p + q * 2^(e-127) per axis (q: 8-bit, rounded outward)
 *   meta[i] = 0: empty slot (its box inverted: qlo 255, qhi 0);
 *             0x80 | r: internal child, node child_base + r; internal
 *             children fill slots 0..7 first, so r == i and imask is
 *             (1 << internal children) - 1;
 *             (count << 5) | off (count 1..3): leaf, prims prim_base + off ..
 */
#ifndef PT_TYPES_H
#define PT_TYPES_H

#include <stdint.h>

#define PT_PRIM_TRIANGLE 0
#define PT_PRIM_SPHERE 1
#define PT_PRIM_RECT 2
#define PT_PRIM_BOX 3
#define PT_PRIM_MOVING 0x20u  /* tag bit of a moving sphere */

#define PT_MAT_LAMBERTIAN 0
#define PT_MAT_METAL 1
#define PT_MAT_DIELECTRIC 2
#define PT_MAT_DIFFUSE_LIGHT 3
#define PT_MAT_OREN_NAYAR 4
#define PT_MAT_TORRANCE_SPARROW 5
#define PT_MAT_ASHIKHMIN_SHIRLEY 6
#define PT_NUM_MAT_TYPES 7

#define PT_LIGHT_RECT 0
#define PT_LIGHT_SPHERE 1

#define PT_RAY_TMAX 1e27f
#define PT_NO_HIT 0xffffffffu

struct GpuMaterial {
  int type;
  float c0x, c0y, c0z;  /* colour / albedo / diffuse / base */
  float c1x, c1y, c1z;  /* specular / extinction */
  float p0, p1;         /* fuzz | ref_idx,density | rA,rB | nu,nv */
  int tex0, tex1;       /* texture ids of c0 / c1, or -1 for the constant colour */
  int pad;
};

/* Texture callables (programs/textures/, host_includes/textures.hpp): a
 * texture maps (u, v, P, index) to a colour.  Checker and vector textures
 * name other textures (ids below their own: the graph has no cycles). */
#define PT_TEX_CONSTANT 0
#define PT_TEX_CHECKER 1
#define PT_TEX_NOISE 2
#define PT_TEX_IMAGE 3
#define PT_TEX_GRADIENT 4
#define PT_TEX_VECTOR 5

struct GpuTexture {
  int kind;
  int a, b;     /* checker: odd, even ids; vector: first list entry, size; image: w, h;
                   noise: axis */
  int data;     /* image: first texel in tex_data; noise: ranvec (256 float4) then
                   perm_x, perm_y, perm_z (64 float4 each, 4 ints per float4) */
  float c[9];   /* constant: c[0..2]; gradient: colorA, colorB, colorC; noise: scale */
  int pad[3];
};

struct GpuLight {
  int type, axis;
  float a0, a1, b0, b1, k;  /* rect */
  float cx, cy, cz, r;      /* sphere */
  float ex, ey, ez;         /* emission */
  int pad[2];
};

struct GpuCamera {
  float ox, oy, oz;     /* origin */
  float lx, ly, lz;     /* lower_left_corner */
  float hx, hy, hz;     /* horizontal */
  float vx, vy, vz;     /* vertical */
  float ux, uy, uz;     /* u */
  float wx, wy, wz;     /* v (camera up) */
  float lens_radius, time0, time1;
};

struct GpuMiss {
  int type;             /* pt_miss_kind */
  float c1x, c1y, c1z, c2x, c2y, c2z;
  int w, h, spherical;
  const float4* env;    /* rgba texels, row 0 at v = 0 */
};

struct DevScene {
  const uint4* nodes;       /* BVH8 nodes */
  const float4* prims;      /* 3 float4 per primitive, leaf order */
  const float4* xforms;     /* 6 float4 per transform: object->world rows, world->object rows */
  const GpuMaterial* mats;
  const GpuLight* lights;
  const uint4* tri_attr;    /* per prim id: absolute attribute-vertex indices (x,y,z),
                               .w bit0 = has normals, bit1 = has uvs, bits 2-31 the
                               face's texture index (mesh.hpp material_buffer) */
  const float* normals;     /* 3 floats per attribute vertex */
  const float* uvs;         /* 2 floats per attribute vertex */
  const uint32_t* leaf_of_id; /* primitive id -> position in the leaf-ordered records */
  const float* env_marg;    /* environment sampling: marginal CDF over rows (h+1) */
  const float* env_cond;    /* conditional CDFs, h rows of w+1 */
  int env_valid;            /* 1 if the environment can be importance sampled */
  int num_lights;
  int num_prims;
  uint32_t root;            /* BVH8 node where traversal starts (0 for one scene) */
  int tri_only;             /* every primitive is a triangle (no type dispatch in traversal) */
  int has_motion;           /* some sphere moves: rays carry their path's time */
  int pad;
  const GpuTexture* textures;
  const float4* tex_data;   /* image texels (rgba, row 0 at v = 0) and noise tables */
  const int* tex_list;      /* entries of vector textures */
  GpuMiss miss;
  GpuCamera cam;
};

#endif
