/*
 * pt_wave.cuh - device helpers shared by the wavefront stage kernels
 * (pt_kernels.cu) and the trace kernels (pt_trace.cu).
 */
#pragma once
#include "pt_device.cuh"
#include "pt_internal.h"

namespace ptd {
// Paths generated this iteration: the free slots of the buffer, at most the
// chunk's paths not yet generated.
__device__ __forceinline__ uint32_t gen_count(const WaveCounters& c, const WaveCtl& ctl,
                                              uint32_t slots) {
  unsigned long long left = ctl.chunk_paths - c.next_path;
  return (uint32_t)min((unsigned long long)(slots - c.n_cur), left);
}

__device__ __forceinline__ Ray3 camera_ray(const GpuCamera& cam, uint32_t x, uint32_t y,
                                           uint32_t Wd, uint32_t Hd, uint32_t& seed) {
  float u = float((float)x + rnd(seed)) / (float)Wd;
  float v = float((float)y + rnd(seed)) / (float)Hd;
  V3 rd = cam.lens_radius * random_in_unit_disk(seed);
  V3 lens_offset = v3(cam.ux, cam.uy, cam.uz) * rd.x + v3(cam.wx, cam.wy, cam.wz) * rd.y;
  V3 origin = v3(cam.ox, cam.oy, cam.oz) + lens_offset;
  V3 direction = v3(cam.lx, cam.ly, cam.lz) + u * v3(cam.hx, cam.hy, cam.hz) +
                 v * v3(cam.vx, cam.vy, cam.vz) - origin;
  Ray3 r;
  r.o = make_float3(origin.x, origin.y, origin.z);
  r.d = make_float3(direction.x, direction.y, direction.z);
  return r;
}
}  // namespace ptd
