/*
 * pt.h - C ABI of the GB300 path tracer (libpt.so).
 *
 * This is the drop-in boundary for the hot path of joaovbs96/OptiX-Path-Tracer:
 * everything the reference's host code hands to OptiX (context variables,
 * geometry instances, materials, light callables, miss programs, the launch)
 * crosses this interface instead.  The C++ classes of host_includes/ are
 * re-created on top of it in pt_scene.hpp.
 *
 * Conventions
 *  - Every function returns PT_OK (0) or a negative PT_E* status; no C++
 *    exception crosses the ABI.  pt_last_error() describes the last failure.
 *  - The library copies every scene input at the call; the caller keeps
 *    ownership of its arrays and of output buffers.
 *  - One context per host thread; calls on a context are serialised by the
 *    caller.  GPU work is issued on the stream passed to pt_render (a
 *    cudaStream_t given as void*, NULL = the legacy default stream).
 *  - Output pointers may be host or device memory (detected per call).
 *  - Transforms are affine 3x4 object-to-world matrices, row major
 *    (m[0..3] is the first row); NULL means identity.
 */
#ifndef PT_H
#define PT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define PT_API __declspec(dllexport)
#else
#define PT_API __attribute__((visibility("default")))
#endif

enum pt_status {
  PT_OK = 0,
  PT_EINVAL = -1,   /* invalid argument or scene state */
  PT_ENOMEM = -2,   /* host or device allocation failed */
  PT_ECUDA = -3,    /* CUDA runtime error */
  PT_ETIMEOUT = -4, /* a bounded device wait ran out */
  PT_EQUEUE = -5,   /* a work queue overflowed */
  PT_ESTATE = -6    /* call not valid in the current state (e.g. not committed) */
};

enum pt_axis { PT_X_AXIS = 0, PT_Y_AXIS = 1, PT_Z_AXIS = 2 }; /* programs/common.hpp:28 */

enum pt_miss_kind { /* host_includes/programs.hpp:32 Miss_Programs */
  PT_MISS_GRADIENT = 0,
  PT_MISS_CONSTANT = 1,
  PT_MISS_HDR = 2,  /* environmental_mapping, programs/miss.cu:64-95 */
  PT_MISS_IMG = 3   /* image_background, programs/miss.cu:51-59 */
};

enum pt_mode {
  PT_MODE_REF = 0,        /* statement-for-statement semantics of programs/ */
  PT_MODE_CONSISTENT = 1  /* local shading frames, matching pdfs, env NEE */
};

typedef struct pt_context pt_context;

typedef struct pt_options {
  int device;          /* CUDA device ordinal */
  int path_slots;      /* wavefront path-state slots; 0 = automatic (a render's
                          paths per chunk rounded up to 64 Ki, at most 8 Mi) */
  int enable_counters; /* count BVH node fetches and primitive tests */
  int enable_timing;   /* per-stage device times (CUDA events in the graph) */
  int bvh_builder;     /* 0 automatic, 1 host (binned SAH), 2 GPU (LBVH + treelets) */
  int bvh_width;       /* most children per BVH node, 2..8; 0 = 8 */
  int shade_order;     /* 0 automatic (material-sorted tiles when the scene uses
                          Oren-Nayar, Torrance-Sparrow or Ashikhmin-Shirley), 1 sorted,
                          2 path order */
  int refetch_lanes;   /* idle lanes of a trace warp that take new rays together, 1..32;
                          0 automatic (24 for scenes of more than 2^16 primitives, else 32) */
} pt_options;

typedef struct pt_render_params {
  int width, height;   /* launch size (programs/raygen.cu:22-23) */
  int spp;             /* frames to accumulate in this call */
  int frame0;          /* first frame index ("frame", main.cpp:264) */
  int max_depth;       /* "maxDepth", main.cpp:63 (default 50) */
  int rr_enable;       /* "russian", main.cpp:62 */
  int rr_depth;        /* RR starts when depth > rr_depth (raygen.cu:112: 10) */
  int mode;            /* pt_mode */
  int guide;           /* learned sampling guide: 0 = off */
} pt_render_params;

typedef struct pt_stats {
  uint64_t paths;          /* paths completed by the last pt_render */
  uint64_t ext_rays;       /* extension rays traced */
  uint64_t shadow_rays;    /* shadow rays traced */
  uint64_t node_fetches;   /* BVH8 nodes fetched (counters enabled only) */
  uint64_t prim_tests;     /* primitive tests (counters enabled only) */
  uint64_t bvh_nodes;      /* BVH8 node count of the committed scene */
  uint64_t bvh_bytes;      /* bytes of nodes + primitive records */
  int bvh_depth;           /* depth of the BVH8 */
  double build_ms;         /* last pt_commit, host wall time */
  double render_ms;        /* last pt_render, device time */
  uint64_t iterations;     /* wavefront iterations of the last render */
  uint64_t kernel_launches;/* kernels launched by the last render */
  /* device time per stage (enable_timing): generate, trace, shade,
     shadow trace, finish + queue advance */
  double stage_ms[5];
  uint64_t graph_launches; /* CUDA-graph launches of the last render */
  uint64_t guide_samples;  /* training samples of each Adam step after the last guided
                              frame (0 without the guide) */
  uint64_t upload_bytes;   /* bytes copied host to device by the last pt_commit */
} pt_stats;

/* ---- context (replaces optix::Context, host_includes/host_common.hpp:21-45) */
PT_API int pt_context_create(const pt_options* opt, pt_context** out);
PT_API int pt_context_destroy(pt_context* ctx);
PT_API const char* pt_last_error(pt_context* ctx);
PT_API const char* pt_version(void);

/* ---- materials (host_includes/materials.hpp) ----------------------------
 * Colours are the constant textures the reference passes
 * (Constant_Texture, host_includes/textures.hpp:20-37).  Each returns the
 * material id in *id. */
/* Lambertian(Texture*)                         materials.hpp:43-58 */
PT_API int pt_material_lambertian(pt_context* ctx, const float albedo[3], uint32_t* id);
/* Metal(Texture*, fuzz)                        materials.hpp:61-78 */
PT_API int pt_material_metal(pt_context* ctx, const float albedo[3], float fuzz, uint32_t* id);
/* Dielectric(base, extinction, ref_idx, density) materials.hpp:81-103 */
PT_API int pt_material_dielectric(pt_context* ctx, const float base[3], const float extinction[3],
                                  float ref_idx, float density, uint32_t* id);
/* Diffuse_Light(Texture*)                      materials.hpp:106-122 */
PT_API int pt_material_diffuse_light(pt_context* ctx, const float emission[3], uint32_t* id);
/* Oren_Nayar(Texture*, R) with the sigma->A,B mapping of materials.hpp:191-198 */
PT_API int pt_material_oren_nayar(pt_context* ctx, const float albedo[3], float roughness,
                                  uint32_t* id);
/* Torrance_Sparrow(Texture*, nu, nv), alpha = max(r,1e-3)^2, materials.hpp:218-238 */
PT_API int pt_material_torrance_sparrow(pt_context* ctx, const float color[3], float nu, float nv,
                                        uint32_t* id);
/* Ashikhmin_Shirley(diffuse, specular, nu, nv), nu,nv >= 1, materials.hpp:162-179 */
PT_API int pt_material_ashikhmin_shirley(pt_context* ctx, const float diffuse[3],
                                         const float specular[3], float nu, float nv,
                                         uint32_t* id);

/* ---- textures (host_includes/textures.hpp, the programs of programs/textures/)
 * A texture maps a hit's (u, v, P, texture index) to a colour; a material
 * slot that names one uses it in place of its constant colour.  Each call
 * returns the texture id in *id; checker and vector textures name textures
 * made before them.  Texture coordinates are the primitives' (sphere.cu:84-87,
 * aarect.cu:71-115, triangle uvs); the texture index is 0 on analytic shapes
 * and the face's index on meshes (pt_mesh_set_texture_index, the
 * material_buffer of mesh.hpp:140-150). */
#define PT_NO_TEXTURE 0xffffffffu
/* Constant_Texture(float3)                     textures.hpp:19-37 */
PT_API int pt_texture_constant(pt_context* ctx, const float rgb[3], uint32_t* id);
/* Checker_Texture(odd, even): odd where sin(10x) sin(10y) sin(10z) < 0,
 * checkered_texture.cu:8-15, textures.hpp:39-54 */
PT_API int pt_texture_checker(pt_context* ctx, uint32_t odd, uint32_t even, uint32_t* id);
/* Noise_Texture(scale, axis): Perlin turbulence, noise_texture.cu:12-76,
 * textures.hpp:56-112.  ranvec: 256 x 3 floats, perm: perm_x, perm_y, perm_z
 * (3 x 256 ints, values 0..255); null tables are made as the host class makes
 * them (std::mt19937 seeded 0, uniform floats).  As in noise_texture.cu:66-73,
 * whose switch has no breaks, every axis evaluates the Z-axis formula. */
PT_API int pt_texture_noise(pt_context* ctx, float scale, int axis, const float* ranvec,
                            const int32_t* perm, uint32_t* id);
/* The default tables of pt_texture_noise (host only, no device work). */
PT_API int pt_noise_tables(float* ranvec, int32_t* perm);
/* Image_Texture / HDR_Texture: w x h RGBA float texels, row 0 at v = 0
 * (the loaders flip the file's rows, textures.hpp:140-151), bilinear with
 * repeat wrap; image_texture.cu:3-7, textures.hpp:114-230 */
PT_API int pt_texture_image(pt_context* ctx, const float* rgba, int w, int h, uint32_t* id);
/* Gradient_Texture(A, B, C): |n.x| A + |n.y| B + |n.z| C with n = P / |P|,
 * gradient_texture.cu:7-14, textures.hpp:233-251 */
PT_API int pt_texture_gradient(pt_context* ctx, const float a[3], const float b[3],
                               const float c[3], uint32_t* id);
/* Vector_Texture(textures): entry `texture index` (black outside 0..n-1),
 * vector.cu:7-12, textures.hpp:253-271 */
PT_API int pt_texture_vector(pt_context* ctx, const uint32_t* textures, int n, uint32_t* id);
/* Material colour from a texture: slot 0 is the colour / albedo / diffuse /
 * base / emission, slot 1 the Ashikhmin-Shirley specular or the dielectric
 * extinction; PT_NO_TEXTURE restores the constant colour. */
PT_API int pt_material_set_texture(pt_context* ctx, uint32_t material, int slot,
                                   uint32_t texture);
/* Texture index of n consecutive triangles from first_prim (their faces'
 * entries of a vector texture; 0 by default), mesh.hpp:140-150 */
PT_API int pt_mesh_set_texture_index(pt_context* ctx, uint32_t first_prim, size_t n,
                                     const uint32_t* index);

/* ---- geometry (host_includes/hitables.hpp, mesh.hpp) ---------------------
 * Primitive ids are assigned in call order (a mesh takes nt consecutive ids);
 * equal hit distances resolve to the lower id. */
/* Sphere(center, radius, BRDF*)                hitables.hpp:89-128 */
PT_API int pt_add_sphere(pt_context* ctx, const float center[3], float radius, uint32_t material,
                         const float xform[12], uint32_t* prim_id);
/* Moving_Sphere(c0, c1, r, t0, t1, BRDF*)     hitables.hpp:130-181: centre c0
 * at time t0, c1 at t1 (t1 > t0), linear in each path's time (the camera's
 * time0 + rnd * (time1 - time0), programs/raygen.cu:69), extrapolated outside
 * [t0, t1]; intersection and record of moving_sphere.cu:57-118.  Its bounds
 * cover every time the camera can give: a camera change needs pt_commit. */
PT_API int pt_add_moving_sphere(pt_context* ctx, const float center0[3], const float center1[3],
                                float radius, float time0, float time1, uint32_t material,
                                const float xform[12], uint32_t* prim_id);
/* AARect(a0,a1,b0,b1,k,flip,axis,BRDF*)        hitables.hpp:210-270 */
PT_API int pt_add_rect(pt_context* ctx, float a0, float a1, float b0, float b1, float k, int flip,
                       int axis, uint32_t material, const float xform[12], uint32_t* prim_id);
/* Box(p0, p1, BRDF*)                           hitables.hpp:273-316 */
PT_API int pt_add_box(pt_context* ctx, const float p0[3], const float p1[3], uint32_t material,
                      const float xform[12], uint32_t* prim_id);
/* Mesh(file, folder, BRDF*) after loading: indexed triangles with optional
 * per-vertex normals and uvs and a per-triangle material (mesh.hpp:49-204).
 * mat_per_tri may be NULL (then every triangle uses `material`). */
PT_API int pt_add_mesh(pt_context* ctx, const float* verts, size_t nv, const uint32_t* idx,
                       size_t nt, const uint32_t* mat_per_tri, uint32_t material,
                       const float* normals, const float* uvs, const float xform[12],
                       uint32_t* first_prim_id);

/* ---- file formats (host side, no device work) ----------------------------
 * Wavefront OBJ/MTL, as the reference's Mesh(file, folder[, BRDF*]) reads it
 * through tinyobjloader (mesh.hpp:49-204, lib/tiny_obj_loader.h): v / vt /
 * vn / f (any of v, v/vt, v//vn, v/vt/vn; negative indices count back),
 * polygons ear-clipped as that loader does, usemtl / mtllib (newmtl, Ka,
 * Kd, map_Kd).  Triangles are de-indexed: three corners each, in file order
 * (mesh.hpp:123-138).  Normals / uvs are kept when every corner has one. */
typedef struct pt_obj pt_obj;
#define PT_OBJ_NO_MATERIAL 0xffffffffu /* mat_per_tri of a face without usemtl */
#define PT_OBJ_MTL 0xfffffffeu         /* pt_add_obj: materials from the MTL file */
PT_API int pt_obj_load(const char* path, pt_obj** out);
PT_API int pt_obj_free(pt_obj* mesh);
PT_API int pt_obj_info(const pt_obj* mesh, size_t* n_tris, size_t* n_materials,
                       int* has_normals, int* has_uvs);
/* verts 9 floats per triangle, normals 9, uvs 6, mat_per_tri 1 (any may be NULL) */
PT_API int pt_obj_get(const pt_obj* mesh, float* verts, float* normals, float* uvs,
                      uint32_t* mat_per_tri);
PT_API int pt_obj_material(const pt_obj* mesh, size_t k, char* name, size_t name_cap,
                           float ka[3], float kd[3], char* map_kd, size_t map_cap);
/* Mesh::getGeometryInstance (mesh.hpp:49-204): the mesh into the scene with
 * `material` on every face, or, with PT_OBJ_MTL, as the reference builds it
 * without a given material (mesh.hpp:78-98): one Lambertian whose colour is
 * a Vector_Texture of the MTL materials (an image texture of map_Kd, read
 * with pt_image_load relative to the OBJ file's folder, rows flipped as
 * Image_Texture does; else a constant texture of Ka), each face indexing
 * its material (faces without usemtl: the first). */
PT_API int pt_add_obj(pt_context* ctx, const pt_obj* mesh, uint32_t material,
                      const float xform[12], uint32_t* first_prim_id);
/* Radiance HDR in (lib/HDRloader.cpp): rgba NULL returns the size only;
 * else w*h*4 floats, first scanline first, (r,g,b)/256 * 2^(e-128), a = 1.
 * Only the "-Y h +X w" orientation, as the reference reads. */
PT_API int pt_hdr_load(const char* path, int* w, int* h, float* rgba);
/* Save_HDR (image_save.hpp:40-73): sum/spp, Reinhard c/(1+c), RGBE. */
PT_API int pt_hdr_save(const char* path, int w, int h, const float* accum_rgba, int spp);
/* Save_PNG (image_save.hpp:7-37): sqrt(sum/spp) clamped, x255.99, 8-bit RGB. */
PT_API int pt_png_save(const char* path, int w, int h, const float* accum_rgba, int spp);
/* message of the last failed file-format call of this thread */
PT_API const char* pt_io_last_error(void);
/* Image_Texture's file reading (textures.hpp:117-155, through stb_image):
 * PNG (8/16-bit grey, grey+alpha, RGB, RGBA, 8-bit palette; not interlaced),
 * PPM (P6, P3) and Radiance HDR; rgba NULL returns the size only, else
 * w*h*4 floats, first file row first, 8-bit samples / 255 (16-bit / 65535),
 * alpha 1 where the file has none.  JPEG is not decoded. */
PT_API int pt_image_load(const char* path, int* w, int* h, float* rgba);
PT_API const char* pt_image_last_error(void);

/* ---- lights (host_includes/pdfs.hpp + Light_Sampler, host_common.hpp:65-68) */
/* Rectangle_PDF(a0,a1,b0,b1,k,axis) + emission  pdfs.hpp:17-80 */
PT_API int pt_add_light_rect(pt_context* ctx, float a0, float a1, float b0, float b1, float k,
                             int axis, const float emission[3]);
/* Sphere_PDF(center, radius) + emission         pdfs.hpp:82-109 */
PT_API int pt_add_light_sphere(pt_context* ctx, const float center[3], float radius,
                               const float emission[3]);

/* ---- miss programs (setMissProgram, host_includes/programs.hpp:32-92) -- */
PT_API int pt_set_env_gradient(pt_context* ctx, const float c1[3], const float c2[3]);
PT_API int pt_set_env_constant(pt_context* ctx, const float c[3]);
/* HDR_Texture(file) / Image_Texture(file) after loading: RGBA float w*h,
 * row 0 at v = 0, bilinear with repeat wrap.  kind = PT_MISS_HDR or PT_MISS_IMG. */
PT_API int pt_set_env_map(pt_context* ctx, int kind, const float* rgba, int w, int h,
                          int spherical);

/* ---- camera (Camera(...).set(Context&), host_includes/camera.hpp:13-51) */
PT_API int pt_set_camera(pt_context* ctx, const float lookfrom[3], const float lookat[3],
                         const float vup[3], float vfov_deg, float aspect, float aperture,
                         float focus_dist, float t0, float t1);

/* ---- build: BVH8 over all primitives (replaces Trbvh) --------------------
 * Automatic builder choice: the GPU builder (Morton codes, radix sort,
 * Karras radix tree, SAH treelet restructuring, 8-wide collapse) from 4096
 * primitives up, the host binned-SAH builder below. */
PT_API int pt_commit(pt_context* ctx);

/* ---- render (renderFrame / Context::launch, main.cpp:26-39,264) ----------
 * Accumulates frames frame0 .. frame0+spp-1 into accum_rgba (W*H float4,
 * y-flipped as programs/raygen.cu:153; zeroed first when frame0 == 0). */
PT_API int pt_render(pt_context* ctx, const pt_render_params* params, float* accum_rgba,
                     void* stream);

/* pt_render with per-pixel sums in double precision: accum_rgba holds 4
 * doubles per pixel (W*H*4, host or device memory, 16-byte aligned), the same
 * layout and frame order as pt_render's float4 accumulator; each path's
 * float colour is widened and added in frame order.  For long progressive
 * renders (beyond about 4096 frames float sums drop the low bits of each new
 * frame).  No counterpart in the reference (its acc_buffer is float4,
 * host_includes/buffers.hpp:13-18). */
PT_API int pt_render_accum64(pt_context* ctx, const pt_render_params* params,
                             double* accum_rgba, void* stream);

/* Per-path colour of one frame (W*H*3 floats, row y*W+x, not flipped): the
 * value renderPixel adds to the accumulator, for parity checks. */
PT_API int pt_render_paths(pt_context* ctx, const pt_render_params* params, float* out_rgb,
                           void* stream);

/* First hit of the camera rays of frame `frame`: primitive id (UINT32_MAX on
 * a miss), material id and t, each W*H, row y*W+x. */
PT_API int pt_trace_first_hits(pt_context* ctx, int width, int height, int frame, uint32_t* prim,
                               uint32_t* mat, float* t, void* stream);

/* Display conversion of programs/raygen.cu:136-146: sqrt(acc/(frame+1)),
 * clamp, x255.99 -> RGBA8 (W*H*4 bytes). */
PT_API int pt_resolve_display(pt_context* ctx, const float* accum_rgba, int width, int height,
                              int frame, uint8_t* rgba8, void* stream);

PT_API int pt_get_stats(pt_context* ctx, pt_stats* out);

/* pt_render for callers that cannot allocate device memory while rendering
 * (a strict memory pool, or an application that allocates only at start-up).
 * No counterpart in the reference.  It calls no cudaMalloc/cudaFree: its
 * wavefront scratch is a fixed 8.75 MiB device array inside libpt.so that
 * every GPU loading the library holds until exit.  Same results as
 * pt_render.  accum_rgba must be device memory; images of at most 262144
 * pixels (PT_EINVAL beyond); fewer paths in flight, so slower.  All calls
 * share the array: calls whose GPU work overlaps race and must be
 * serialised.  The first call on a device resolves the array's address
 * (cudaGetSymbolAddress); make it before any stream capture. */
PT_API int pt_render_noalloc(pt_context* ctx, const pt_render_params* params, float* accum_rgba,
                             void* stream);

/* ---- learned sampling guide ----------------------------------------------
 * No counterpart in the reference.  A small MLP (BF16 tensor-core kernels,
 * FP32 accumulation) maps the encoded shading point (position in the scene
 * box, normal, outgoing direction: 76 features) through 4 hidden layers of 64
 * to a mixture of 8 von Mises-Fisher lobes and the probability of sampling it
 * instead of the BSDF; consistent-mode renders with params.guide = 1 sample
 * their bounces from alpha * guide + (1 - alpha) * BSDF (one-sample MIS, so
 * the estimate stays unbiased) and train the network online on the radiance
 * they carry back.  Parameters: PT_GUIDE_PARAMS floats, five row-major
 * [rows x 80] matrices (W1..W4: 64 rows, W5: 48 rows) whose column 76 (W1)
 * or 64 (W2..W5) is the bias; padding entries are kept 0.
 * Samples: PT_GUIDE_SAMPLE_FLOATS floats each: position, normal, outgoing
 * direction, sampled direction (3 each), BSDF pdf of that direction, weight
 * (F / q: the integrand over the density it was drawn from), 2 unused. */
#define PT_GUIDE_PARAMS 24320
#define PT_GUIDE_OUTPUTS 48
#define PT_GUIDE_SAMPLE_FLOATS 16
/* Seeded He-uniform initialisation; resets the Adam state. */
PT_API int pt_guide_init(pt_context* ctx, uint64_t seed);
/* Online training during guided renders: Adam learning rate, Adam steps
 * per frame on that frame's samples, the exponent applied to the sample
 * weights F/q (1 = the KL target; below 1 tempers the heavy tail of bright,
 * rare paths), and how many bounces of a path are guided (0 = all; deeper
 * bounces sample the BSDF alone).  Defaults: 1e-2, 12 steps, exponent 1,
 * 4 bounces. */
PT_API int pt_guide_set_training(pt_context* ctx, float lr, int steps_per_frame, float exponent,
                                 int max_bounces);
/* Bound on each wait of the guide kernels for their tensor-core results, in
 * mbarrier try_wait attempts (default PT_GUIDE_WAIT_DEFAULT = 2^24).  A wait
 * that runs out makes the kernel stop, let its MMAs in flight finish, free
 * its tensor memory and report PT_ETIMEOUT; the context stays usable.  0
 * makes every wait run out at once: it exists to exercise that path (a
 * working kernel never needs a small bound). */
#define PT_GUIDE_WAIT_DEFAULT (1u << 24)
PT_API int pt_guide_set_wait_limit(pt_context* ctx, uint32_t try_waits);
PT_API int pt_guide_get_params(pt_context* ctx, float* params);
PT_API int pt_guide_set_params(pt_context* ctx, const float* params);
/* Checkpoint of the online training: FP32 weights, Adam first and second
 * moments (PT_GUIDE_STATE_FLOATS floats) and the Adam step count.  Training
 * is deterministic, so a guided render resumed from a checkpoint continues
 * bit for bit as the uninterrupted one (with the same pt_guide_set_training
 * options).  The reference keeps only its in-memory accumulation
 * (raygen.cu:153-154). */
#define PT_GUIDE_STATE_FLOATS (3 * PT_GUIDE_PARAMS)
PT_API int pt_guide_get_state(pt_context* ctx, float* state, int64_t* step);
PT_API int pt_guide_set_state(pt_context* ctx, const float* state, int64_t step);
/* Scene box of the position encoding: x01 = (p - bmin) * binv. */
PT_API int pt_guide_bounds(pt_context* ctx, float bmin[3], float binv[3]);
/* Raw network outputs (PT_GUIDE_OUTPUTS per sample) of n samples. */
PT_API int pt_guide_eval(pt_context* ctx, const float* samples, int n, float* outputs);
/* Loss sum(-w log q(wi)) / sum(w) of n samples and its gradient
 * (PT_GUIDE_PARAMS floats); no update. */
PT_API int pt_guide_gradient(pt_context* ctx, const float* samples, int n, float* grad,
                             float* loss);
/* One Adam step (beta 0.9/0.99) with learning rate lr on n samples. */
PT_API int pt_guide_train(pt_context* ctx, const float* samples, int n, float lr, float* loss);

/* ---- batched multi-scene rendering ---------------------------------------
 * No counterpart in the reference (its main.cpp renders one scene per
 * process).  Renders many committed scenes in one wavefront: the paths of
 * all scenes share the path-state buffers, so small scenes and the drained
 * tail of each render do not leave the GPU idle.  The whole batch is one
 * CUDA-graph launch whose chunk and iteration loops are device-side
 * conditional (while) nodes, each bounded on the device.  Each item's
 * accumulator receives exactly what pt_render gives for the same scene and
 * parameters.  The batch keeps its own copy of the scenes' geometry
 * (rebuilt when a scene is re-committed or the node width changes). */
typedef struct pt_batch pt_batch;

typedef struct pt_batch_item {
  pt_context* scene;        /* committed context on the batch's device */
  pt_render_params params;  /* per item; `mode` must be equal for all items, guide 0 */
  float* accum_rgba;        /* W*H float4, host or device memory (as pt_render) */
} pt_batch_item;

/* Launch configuration of a batch, chosen by pt_batch_autotune. */
typedef struct pt_tune {
  int path_slots;           /* paths in flight */
  int trace_block;          /* threads per trace block: 64, 128 or 256 */
  int shade_block;          /* threads per shade block: 64..256, multiple of 32 */
  int bvh_width;            /* most children per BVH node, 2..8 */
  int chunk_paths;          /* paths per chunk (per-path result area), 0 = 2^27 */
  int shade_order;          /* as pt_options.shade_order */
  int refetch_lanes;        /* as pt_options.refetch_lanes */
  double sample_paths_per_s;/* autotune: throughput of this configuration on its sample */
} pt_tune;

/* opt: device and builder as for a context (path_slots and bvh_width give
 * the initial tune). */
PT_API int pt_batch_create(const pt_options* opt, pt_batch** out);
PT_API int pt_batch_destroy(pt_batch* b);
PT_API const char* pt_batch_last_error(pt_batch* b);
/* Renders n items (1..32767).  Stats (pt_batch_get_stats) sum all items. */
PT_API int pt_batch_render(pt_batch* b, const pt_batch_item* items, int n, void* stream);
/* Times short renders of a sample of the items (every item at low spp, into
 * scratch accumulators; the items' accumulators are not touched) over path
 * slots, trace and shade block sizes, BVH node width and shade order (material-
 * sorted tiles or path order), keeps the fastest
 * configuration for later pt_batch_render calls and returns it in *best. */
PT_API int pt_batch_autotune(pt_batch* b, const pt_batch_item* items, int n, pt_tune* best);
PT_API int pt_batch_set_tune(pt_batch* b, const pt_tune* t);
PT_API int pt_batch_get_tune(pt_batch* b, pt_tune* t);
PT_API int pt_batch_get_stats(pt_batch* b, pt_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* PT_H */
