// Wrapper of programs/raygen.cu, the ray-generation program renderPixel (test
// infrastructure, see rtshim.h).  camera: lower-left corner, horizontal,
// vertical, origin, u, v (3 floats each), lens radius, time0, time1.
#include "rtemu.h"
#include "raygen.cu"

extern "C" void ref_render_pixel(unsigned int x, unsigned int y, unsigned int W, unsigned int H,
                                 int frame_index, int rr, int max_depth, const float* cam,
                                 float4* acc, uchar4* display) {
  pixelID = make_uint2(x, y);
  launchDim = make_uint2(W, H);
  frame = frame_index;
  russian = rr;
  maxDepth = max_depth;
  samples = 1;
  camera_lower_left_corner = make_float3(cam[0], cam[1], cam[2]);
  camera_horizontal = make_float3(cam[3], cam[4], cam[5]);
  camera_vertical = make_float3(cam[6], cam[7], cam[8]);
  camera_origin = make_float3(cam[9], cam[10], cam[11]);
  camera_u = make_float3(cam[12], cam[13], cam[14]);
  camera_v = make_float3(cam[15], cam[16], cam[17]);
  camera_lens_radius = cam[18];
  time0 = cam[19];
  time1 = cam[20];
  acc_buffer.data = acc;
  acc_buffer.w = W;
  acc_buffer.h = H;
  display_buffer.data = display;
  display_buffer.w = W;
  display_buffer.h = H;
  renderPixel();
}
