// Malformed-file driver for the host file readers (pt_image_load: PNG, PPM,
// Radiance HDR; pt_hdr_load; pt_obj_load and its MTL): every seed file is
// mutated many times (bytes flipped, cut short, spans duplicated or
// dropped) and read back; a reader must return an error or a consistent
// image / mesh.  Built by tests/test_io_fuzz.py with the address and
// undefined-behaviour sanitizers, so an out-of-bounds access or an uncaught
// exception fails the run.
//
//   io_fuzz_driver <work dir> <mutations per seed> <seed file>...
#include <cstdint>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pt.h"

// The mesh reader's neighbours in the library (pt_add_obj builds a scene
// with them); the readers exercised here never call them.
extern "C" {
int pt_add_mesh(pt_context*, const float*, size_t, const uint32_t*, size_t, const uint32_t*,
                uint32_t, const float*, const float*, const float*, uint32_t*) {
  return PT_EINVAL;
}
int pt_material_lambertian(pt_context*, const float*, uint32_t*) { return PT_EINVAL; }
int pt_texture_constant(pt_context*, const float*, uint32_t*) { return PT_EINVAL; }
int pt_texture_image(pt_context*, const float*, int, int, uint32_t*) { return PT_EINVAL; }
int pt_texture_vector(pt_context*, const uint32_t*, int, uint32_t*) { return PT_EINVAL; }
int pt_material_set_texture(pt_context*, uint32_t, int, uint32_t) { return PT_EINVAL; }
int pt_mesh_set_texture_index(pt_context*, uint32_t, size_t, const uint32_t*) {
  return PT_EINVAL;
}
}

static uint32_t g_state = 12345u;
static uint32_t rnd32() {
  g_state = g_state * 1664525u + 1013904223u;
  return g_state ^ (g_state >> 16);
}

static bool read_file(const std::string& p, std::vector<uint8_t>& out) {
  FILE* f = fopen(p.c_str(), "rb");
  if (!f) return false;
  uint8_t buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
  fclose(f);
  return true;
}

static void write_file(const std::string& p, const std::vector<uint8_t>& d) {
  FILE* f = fopen(p.c_str(), "wb");
  if (!f) return;
  if (!d.empty()) fwrite(d.data(), 1, d.size(), f);
  fclose(f);
}

static std::vector<uint8_t> mutate(const std::vector<uint8_t>& src) {
  std::vector<uint8_t> d = src;
  const int kind = (int)(rnd32() % 6);
  if (d.empty()) return d;
  if (kind == 0) {  // a few bytes flipped
    for (int k = 0, m = 1 + (int)(rnd32() % 8); k < m; k++) d[rnd32() % d.size()] ^= (uint8_t)(1u << (rnd32() % 8));
  } else if (kind == 1) {  // bytes replaced by random values
    for (int k = 0, m = 1 + (int)(rnd32() % 16); k < m; k++) d[rnd32() % d.size()] = (uint8_t)rnd32();
  } else if (kind == 2) {  // cut short
    d.resize(rnd32() % d.size());
  } else if (kind == 3) {  // a span duplicated
    const size_t a = rnd32() % d.size(), n = 1 + rnd32() % 64;
    std::vector<uint8_t> span(d.begin() + a, d.begin() + std::min(d.size(), a + n));
    d.insert(d.begin() + rnd32() % d.size(), span.begin(), span.end());
  } else if (kind == 4) {  // a span dropped
    const size_t a = rnd32() % d.size(), n = 1 + rnd32() % 64;
    d.erase(d.begin() + a, d.begin() + std::min(d.size(), a + n));
  } else {  // a 32-bit field (sizes, lengths, counts) overwritten
    if (d.size() >= 4) {
      const size_t a = rnd32() % (d.size() - 3);
      const uint32_t v = (rnd32() % 2) ? rnd32() : (rnd32() % 70000);
      d[a] = (uint8_t)(v >> 24);
      d[a + 1] = (uint8_t)(v >> 16);
      d[a + 2] = (uint8_t)(v >> 8);
      d[a + 3] = (uint8_t)v;
    }
  }
  return d;
}

static int check_image(const std::string& path, bool hdr_only) {
  int w = 0, h = 0;
  const int rc = hdr_only ? pt_hdr_load(path.c_str(), &w, &h, nullptr)
                          : pt_image_load(path.c_str(), &w, &h, nullptr);
  if (rc != PT_OK) return 0;
  if (w <= 0 || h <= 0) {
    printf("BAD size %d x %d accepted: %s\n", w, h, path.c_str());
    return 1;
  }
  if ((uint64_t)w * (uint64_t)h > ((uint64_t)1 << 24)) return 0;  // a valid but large header
  std::vector<float> px((size_t)w * h * 4 + 4, -7.f);
  int w2 = 0, h2 = 0;
  const int rc2 = hdr_only ? pt_hdr_load(path.c_str(), &w2, &h2, px.data())
                           : pt_image_load(path.c_str(), &w2, &h2, px.data());
  if (rc2 == PT_OK && (w2 != w || h2 != h)) {
    printf("BAD size changed between calls: %s\n", path.c_str());
    return 1;
  }
  for (int k = 0; k < 4; k++)
    if (px[(size_t)w * h * 4 + k] != -7.f) {
      printf("BAD write past w*h*4 floats: %s\n", path.c_str());
      return 1;
    }
  return 0;
}

static int check_obj(const std::string& path) {
  pt_obj* m = nullptr;
  if (pt_obj_load(path.c_str(), &m) != PT_OK) return 0;
  size_t nt = 0, nm = 0;
  int hn = 0, hu = 0;
  int bad = 0;
  if (pt_obj_info(m, &nt, &nm, &hn, &hu) == PT_OK && nt < ((size_t)1 << 22)) {
    std::vector<float> v(9 * nt + 1), n(9 * nt + 1), uv(6 * nt + 1);
    std::vector<uint32_t> mat(nt + 1);
    pt_obj_get(m, v.data(), hn ? n.data() : nullptr, hu ? uv.data() : nullptr, mat.data());
    for (size_t t = 0; t < nt; t++)
      if (mat[t] != PT_OBJ_NO_MATERIAL && mat[t] >= nm) {
        printf("BAD material index %u of %zu: %s\n", mat[t], nm, path.c_str());
        bad = 1;
        break;
      }
    for (size_t k = 0; k < nm; k++) {
      char name[64], tex[256];
      float ka[3], kd[3];
      pt_obj_material(m, k, name, sizeof(name), ka, kd, tex, sizeof(tex));
    }
  }
  pt_obj_free(m);
  return bad;
}

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s <work dir> <mutations per seed> <seed file>...\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  const int muts = atoi(argv[2]);
  int bad = 0, files = 0;
  for (int a = 3; a < argc; a++) {
    const std::string seed = argv[a];
    std::vector<uint8_t> src;
    if (!read_file(seed, src)) {
      printf("BAD cannot read seed %s\n", seed.c_str());
      return 2;
    }
    const bool obj = seed.size() > 4 && seed.compare(seed.size() - 4, 4, ".obj") == 0;
    // a material library is mutated in place as <work dir>/fz.mtl and read
    // through <work dir>/mtlref.obj, which names it
    const bool mtl = seed.size() > 4 && seed.compare(seed.size() - 4, 4, ".mtl") == 0;
    const bool hdr = seed.size() > 4 && seed.compare(seed.size() - 4, 4, ".hdr") == 0;
    const std::string ext = seed.substr(seed.rfind('.'));
    for (int k = 0; k < muts; k++) {
      const std::string path =
          mtl ? dir + "/fz.mtl" : dir + "/m" + std::to_string(a) + "_" + std::to_string(k % 4) + ext;
      write_file(path, k == 0 ? src : mutate(src));
      if (mtl)
        bad += check_obj(dir + "/mtlref.obj");
      else
        bad += obj ? check_obj(path) : check_image(path, false);
      if (hdr) bad += check_image(path, true);
      files++;
    }
  }
  printf("%s %d files\n", bad ? "FAILURES" : "ALL PASS", files);
  return bad ? 1 : 0;
}
