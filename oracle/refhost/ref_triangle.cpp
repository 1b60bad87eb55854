// Wrapper of programs/hitables/triangle.cu (test infrastructure, see rtshim.h).
// The mesh buffers view the runtime's arrays.  Intersection in the
// reference's default RTX mode is the hardware triangle test followed by the
// Attributes program (host_includes/mesh.hpp:176-188); the runtime supplies
// the test and this wrapper runs Attributes.  ref_triangle_intersect runs
// the software Intersect program of the non-RTX mode.
#include "rtemu.h"
#include "hitables/triangle.cu"
#include "ref_common.h"

extern "C" void ref_triangle_bind(const float3* verts, size_t nv, const float3* normals,
                                  size_t nn, const float2* uvs, size_t nuv, const int3* idx,
                                  size_t nt, const int* mats) {
  vertex_buffer.data = const_cast<float3*>(verts);
  vertex_buffer.n = nv;
  normal_buffer.data = const_cast<float3*>(normals);
  normal_buffer.n = nn;
  texcoord_buffer.data = const_cast<float2*>(uvs);
  texcoord_buffer.n = nuv;
  index_buffer.data = const_cast<int3*>(idx);
  index_buffer.n = nt;
  material_buffer.data = const_cast<int*>(mats);
  material_buffer.n = nt;
}

extern "C" void ref_triangle_attributes(int* gi, float2* b) {
  Attributes();
  *gi = geo_index;
  *b = bc;
}

extern "C" void ref_triangle_intersect(int pid, const Ray* r, int* gi, float2* b) {
  ray = *r;
  Intersect(pid);
  *gi = geo_index;
  *b = bc;
}

extern "C" void ref_triangle_hitrecord(int index, const Ray* r, float t, float2 b,
                                       EmuRec* out) {
  *out = to_emu(Get_HitRecord(index, *r, t, b));
}

extern "C" void ref_triangle_bounds(int pid, float* box6) { Get_Bounds(pid, box6); }
