// Wrapper of programs/textures/vector.cu (test infrastructure, see rtshim.h).
// The entries' callables are kept per vector texture (a nested vector
// texture rebinds the buffer, never destroys a callable that is running).
#include <map>

#include "rtemu.h"
#include "textures/vector.cu"
#include "ref_common_tex.h"

using EntryFn = std::remove_reference<decltype(texture_vector[0])>::type;

extern "C" float3 ref_vector_texture(int self, const int* ids, int n, float u, float v,
                                     const float3* p, int i) {
  static int gen = -1;
  static std::map<int, std::vector<EntryFn>> entries;
  if (gen != rtemu_scene_generation()) {
    gen = rtemu_scene_generation();
    entries.clear();
  }
  auto it = entries.find(self);
  if (it == entries.end()) {
    std::vector<EntryFn> e((size_t)n);
    for (int k = 0; k < n; k++) bind_texture_fn(e[k], ids[k]);
    it = entries.emplace(self, std::move(e)).first;
  }
  size = n;
  texture_vector.data = it->second.data();
  texture_vector.n = (size_t)n;
  return sample_texture(u, v, *p, i);
}
