/*
 * ref_common_tex.h - binding of texture callables for the texture wrappers
 * (whose translation units have no HitRecord).  TEST INFRASTRUCTURE ONLY
 * (see rtshim.h).
 */
#pragma once
#include "rtemu.h"

int rtemu_scene_generation();

template <class F> inline void bind_texture_fn(F& f, int tex) {
  f.fn = [tex](float u, float v, float3 p, int i) { return rtemu_texture(tex, u, v, p, i); };
}
