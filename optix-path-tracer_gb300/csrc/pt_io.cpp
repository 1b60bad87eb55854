/*
 * pt_io.cpp - host-side file formats on either side of the path: Wavefront
 * OBJ/MTL meshes in (the reference's Mesh class over tinyobjloader,
 * host_includes/mesh.hpp:49-204), Radiance HDR images in (lib/HDRloader.cpp)
 * and out, and PNG out (host_includes/image_save.hpp:7-73).  No third-party
 * code: the parsers and writers below follow the published formats (Ward's
 * RGBE encoding, the PNG specification with stored deflate blocks).
 */
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/pt.h"

namespace {

thread_local std::string g_io_err;

int io_fail(int code, const std::string& msg) {
  g_io_err = msg;
  return code;
}

bool read_file(const char* path, std::string& out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  std::string s;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
  bool ok = !ferror(f);
  fclose(f);
  out.swap(s);
  return ok;
}

std::vector<std::string> split_ws(const std::string& line) {
  std::vector<std::string> t;
  size_t i = 0, n = line.size();
  while (i < n) {
    while (i < n && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r')) i++;
    size_t j = i;
    while (j < n && line[j] != ' ' && line[j] != '\t' && line[j] != '\r') j++;
    if (j > i) t.push_back(line.substr(i, j - i));
    i = j;
  }
  return t;
}

// Locale-independent decimal parse (the host program's locale may use a
// decimal comma): read as double, rounded once to float.
bool to_float(const std::string& s, float& v) {
  const char* b = s.c_str();
  const char* e = b + s.size();
  if (b != e && *b == '+') b++;
  double d = 0.0;
  auto r = std::from_chars(b, e, d);
  if (r.ec != std::errc() || r.ptr == b) return false;
  v = (float)d;
  return true;
}

std::string dir_of(const std::string& path) {
  size_t k = path.find_last_of("/\\");
  return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

// ------------------------------------------------------------- OBJ ----------
struct Corner {
  long v, vt, vn;  // 0-based, -1 = absent
};

// One face index triple "v", "v/vt", "v//vn" or "v/vt/vn"; negative indices
// count back from the current end of the list.
bool parse_corner(const std::string& tok, size_t nv, size_t nvt, size_t nvn, Corner& c) {
  long idx[3] = {0, 0, 0};
  bool has[3] = {false, false, false};
  size_t part = 0, i = 0;
  while (i <= tok.size() && part < 3) {
    size_t j = tok.find('/', i);
    if (j == std::string::npos) j = tok.size();
    if (j > i) {
      char* end = nullptr;
      long x = strtol(tok.c_str() + i, &end, 10);
      if (end != tok.c_str() + j || x == 0) return false;
      idx[part] = x;
      has[part] = true;
    }
    part++;
    i = j + 1;
  }
  if (!has[0]) return false;
  const size_t counts[3] = {nv, nvt, nvn};
  long out[3] = {-1, -1, -1};
  for (int k = 0; k < 3; k++) {
    if (!has[k]) continue;
    long x = idx[k] > 0 ? idx[k] - 1 : (long)counts[k] + idx[k];
    if (x < 0 || x >= (long)counts[k]) return false;
    out[k] = x;
  }
  c.v = out[0];
  c.vt = out[1];
  c.vn = out[2];
  return true;
}

// Point in triangle by the crossing-number rule (W. R. Franklin's pnpoly).
bool inside3(const float* vx, const float* vy, float tx, float ty) {
  bool c = false;
  for (int i = 0, j = 2; i < 3; j = i++) {
    if (((vy[i] > ty) != (vy[j] > ty)) &&
        (tx < (vx[j] - vx[i]) * (ty - vy[i]) / (vy[j] - vy[i]) + vx[i]))
      c = !c;
  }
  return c;
}

// Triangulates one polygon the way the reference's loader does (ear
// clipping in the plane of the two axes that the first non-degenerate
// corner's normal does not dominate; a triangle is an ear when its corner
// turns with the polygon's orientation and no other vertex lies inside it;
// the ear's middle vertex is removed).  Appends corner triples to `out`.
// The steps are those of tinyobjloader (Syoyo Fujita, MIT licence), the OBJ
// reader the reference vendors (lib/tiny_obj_loader.h), kept so that a file
// gives the same triangles and primitive ids.
void triangulate(const std::vector<Corner>& face, const std::vector<float>& pos,
                 std::vector<Corner>& out) {
  const size_t n0 = face.size();
  if (n0 < 3) return;
  auto P = [&](const Corner& c, int a) { return pos[3 * (size_t)c.v + a]; };
  int axes[2] = {1, 2};
  for (size_t k = 0; k < n0; k++) {
    const Corner &a = face[k], &b = face[(k + 1) % n0], &c = face[(k + 2) % n0];
    float e0x = P(b, 0) - P(a, 0), e0y = P(b, 1) - P(a, 1), e0z = P(b, 2) - P(a, 2);
    float e1x = P(c, 0) - P(b, 0), e1y = P(c, 1) - P(b, 1), e1z = P(c, 2) - P(b, 2);
    float cx = std::fabs(e0y * e1z - e0z * e1y);
    float cy = std::fabs(e0z * e1x - e0x * e1z);
    float cz = std::fabs(e0x * e1y - e0y * e1x);
    const float eps = std::numeric_limits<float>::epsilon();
    if (cx > eps || cy > eps || cz > eps) {
      if (!(cx > cy && cx > cz)) {
        axes[0] = 0;
        if (cz > cx && cz > cy) axes[1] = 1;
      }
      break;
    }
  }
  float area = 0.f;
  for (size_t k = 0; k < n0; k++) {
    const Corner &a = face[k], &b = face[(k + 1) % n0];
    area += (P(a, axes[0]) * P(b, axes[1]) - P(a, axes[1]) * P(b, axes[0])) * 0.5f;
  }
  std::vector<Corner> rem = face;
  size_t guess = 0, tries = rem.size(), prev = rem.size();
  while (rem.size() > 3 && tries > 0) {
    const size_t n = rem.size();
    if (guess >= n) guess -= n;
    if (prev != n) {
      prev = n;
      tries = n;
    } else {
      tries--;
    }
    Corner ind[3];
    float vx[3], vy[3];
    for (int k = 0; k < 3; k++) {
      ind[k] = rem[(guess + k) % n];
      vx[k] = P(ind[k], axes[0]);
      vy[k] = P(ind[k], axes[1]);
    }
    float cross = (vx[1] - vx[0]) * (vy[2] - vy[1]) - (vy[1] - vy[0]) * (vx[2] - vx[1]);
    if (cross * area < 0.f) {
      guess++;
      continue;
    }
    bool overlap = false;
    for (size_t o = 3; o < n && !overlap; o++) {
      const Corner& q = rem[(guess + o) % n];
      overlap = inside3(vx, vy, P(q, axes[0]), P(q, axes[1]));
    }
    if (overlap) {
      guess++;
      continue;
    }
    out.push_back(ind[0]);
    out.push_back(ind[1]);
    out.push_back(ind[2]);
    rem.erase(rem.begin() + (long)((guess + 1) % n));
  }
  if (rem.size() == 3) {
    out.push_back(rem[0]);
    out.push_back(rem[1]);
    out.push_back(rem[2]);
  }
}

struct Mtl {
  std::string name, map_kd;
  float ka[3] = {0, 0, 0}, kd[3] = {0, 0, 0};
};

bool load_mtl(const std::string& path, std::vector<Mtl>& mats, std::map<std::string, int>& index) {
  std::string text;
  if (!read_file(path.c_str(), text)) return false;
  size_t pos = 0;
  int cur = -1;  // index of the material being read
  while (pos < text.size()) {
    size_t e = text.find('\n', pos);
    if (e == std::string::npos) e = text.size();
    std::string line = text.substr(pos, e - pos);
    pos = e + 1;
    size_t h = line.find('#');
    if (h != std::string::npos) line.resize(h);
    std::vector<std::string> t = split_ws(line);
    if (t.empty()) continue;
    if (t[0] == "newmtl" && t.size() >= 2) {
      auto it = index.find(t[1]);
      if (it == index.end()) {
        cur = (int)mats.size();
        index[t[1]] = cur;
        mats.push_back(Mtl());
        mats.back().name = t[1];
      } else {
        cur = it->second;
      }
    } else if (cur >= 0 && (t[0] == "Ka" || t[0] == "Kd") && t.size() >= 4) {
      float* d = t[0] == "Ka" ? mats[cur].ka : mats[cur].kd;
      for (int a = 0; a < 3; a++)
        if (!to_float(t[1 + a], d[a])) d[a] = 0.f;
    } else if (cur >= 0 && t[0] == "map_Kd" && t.size() >= 2) {
      mats[cur].map_kd = t.back();
    }
  }
  return true;
}

}  // namespace

struct pt_obj {
  std::vector<float> pos, nrm, uv;  // three corners per triangle
  std::vector<uint32_t> mat;        // per triangle: MTL material, or PT_OBJ_NO_MATERIAL
  bool has_nrm = false, has_uv = false;
  std::vector<Mtl> mats;
  std::string dir;                  // the OBJ file's folder (map_Kd paths are relative to it)
};

extern "C" {

PT_API const char* pt_io_last_error(void) { return g_io_err.c_str(); }

static int obj_load_body(const char* path, pt_obj** out) {
  if (!path || !out) return io_fail(PT_EINVAL, "null argument");
  *out = nullptr;
  std::string text;
  if (!read_file(path, text)) return io_fail(PT_EINVAL, std::string("cannot read ") + path);
  std::vector<float> v, vt, vn;
  std::vector<Mtl> mats;
  std::map<std::string, int> mat_index;
  int cur_mat = -1;
  std::vector<Corner> tris;
  std::vector<int> tri_mat;
  size_t pos = 0, line_no = 0;
  while (pos < text.size()) {
    size_t e = text.find('\n', pos);
    if (e == std::string::npos) e = text.size();
    std::string line = text.substr(pos, e - pos);
    pos = e + 1;
    line_no++;
    size_t h = line.find('#');
    if (h != std::string::npos) line.resize(h);
    std::vector<std::string> t = split_ws(line);
    if (t.empty()) continue;
    const std::string& k = t[0];
    if (k == "v" || k == "vn") {
      float x[3];
      if (t.size() < 4 || !to_float(t[1], x[0]) || !to_float(t[2], x[1]) || !to_float(t[3], x[2]))
        return io_fail(PT_EINVAL, "bad " + k + " at line " + std::to_string(line_no));
      std::vector<float>& dst = k == "v" ? v : vn;
      dst.insert(dst.end(), x, x + 3);
    } else if (k == "vt") {
      float x[2] = {0.f, 0.f};
      if (t.size() < 2 || !to_float(t[1], x[0]) || (t.size() >= 3 && !to_float(t[2], x[1])))
        return io_fail(PT_EINVAL, "bad vt at line " + std::to_string(line_no));
      vt.insert(vt.end(), x, x + 2);
    } else if (k == "f") {
      std::vector<Corner> face;
      for (size_t i = 1; i < t.size(); i++) {
        Corner c;
        if (!parse_corner(t[i], v.size() / 3, vt.size() / 2, vn.size() / 3, c))
          return io_fail(PT_EINVAL, "bad face index at line " + std::to_string(line_no));
        face.push_back(c);
      }
      size_t before = tris.size();
      triangulate(face, v, tris);
      for (size_t i = before; i < tris.size(); i += 3) tri_mat.push_back(cur_mat);
    } else if (k == "usemtl" && t.size() >= 2) {
      auto it = mat_index.find(t[1]);
      cur_mat = it == mat_index.end() ? -1 : it->second;
    } else if (k == "mtllib" && t.size() >= 2) {
      for (size_t i = 1; i < t.size(); i++)
        if (!load_mtl(dir_of(path) + t[i], mats, mat_index))
          return io_fail(PT_EINVAL, "cannot read material library " + t[i]);
    }
  }
  std::unique_ptr<pt_obj> m(new (std::nothrow) pt_obj());
  if (!m) return io_fail(PT_ENOMEM, "out of host memory");
  const size_t nc = tris.size();
  bool all_n = nc > 0, all_t = nc > 0;
  for (const Corner& c : tris) {
    all_n = all_n && c.vn >= 0;
    all_t = all_t && c.vt >= 0;
  }
  m->has_nrm = all_n;
  m->has_uv = all_t;
  m->pos.resize(3 * nc);
  if (all_n) m->nrm.resize(3 * nc);
  if (all_t) m->uv.resize(2 * nc);
  for (size_t i = 0; i < nc; i++) {
    const Corner& c = tris[i];
    for (int a = 0; a < 3; a++) m->pos[3 * i + a] = v[3 * (size_t)c.v + a];
    if (all_n)
      for (int a = 0; a < 3; a++) m->nrm[3 * i + a] = vn[3 * (size_t)c.vn + a];
    if (all_t)
      for (int a = 0; a < 2; a++) m->uv[2 * i + a] = vt[2 * (size_t)c.vt + a];
  }
  m->mat.resize(tri_mat.size());
  for (size_t i = 0; i < tri_mat.size(); i++)
    m->mat[i] = tri_mat[i] < 0 ? PT_OBJ_NO_MATERIAL : (uint32_t)tri_mat[i];
  m->mats = std::move(mats);
  m->dir = dir_of(path);
  *out = m.release();
  return PT_OK;
}

// Host memory running out while reading an untrusted file (a header can
// claim sizes its data cannot hold) is an error of the call, not an abort.
PT_API int pt_obj_load(const char* path, pt_obj** out) {
  try {
    return obj_load_body(path, out);
  } catch (const std::bad_alloc&) {
    return io_fail(PT_ENOMEM, "out of host memory reading the OBJ file");
  }
}

PT_API int pt_obj_free(pt_obj* m) {
  delete m;
  return PT_OK;
}

PT_API int pt_obj_info(const pt_obj* m, size_t* n_tris, size_t* n_materials, int* has_normals,
                       int* has_uvs) {
  if (!m) return io_fail(PT_EINVAL, "null mesh");
  if (n_tris) *n_tris = m->mat.size();
  if (n_materials) *n_materials = m->mats.size();
  if (has_normals) *has_normals = m->has_nrm ? 1 : 0;
  if (has_uvs) *has_uvs = m->has_uv ? 1 : 0;
  return PT_OK;
}

PT_API int pt_obj_get(const pt_obj* m, float* verts, float* normals, float* uvs,
                      uint32_t* mat_per_tri) {
  if (!m) return io_fail(PT_EINVAL, "null mesh");
  // (a mesh without faces has empty arrays: nothing is copied)
  if (verts && !m->pos.empty()) memcpy(verts, m->pos.data(), m->pos.size() * sizeof(float));
  if (normals) {
    if (!m->has_nrm) return io_fail(PT_EINVAL, "the mesh has no normals on every corner");
    if (!m->nrm.empty()) memcpy(normals, m->nrm.data(), m->nrm.size() * sizeof(float));
  }
  if (uvs) {
    if (!m->has_uv) return io_fail(PT_EINVAL, "the mesh has no texture coordinates on every corner");
    if (!m->uv.empty()) memcpy(uvs, m->uv.data(), m->uv.size() * sizeof(float));
  }
  if (mat_per_tri && !m->mat.empty())
    memcpy(mat_per_tri, m->mat.data(), m->mat.size() * sizeof(uint32_t));
  return PT_OK;
}

PT_API int pt_obj_material(const pt_obj* m, size_t k, char* name, size_t name_cap, float ka[3],
                           float kd[3], char* map_kd, size_t map_cap) {
  if (!m || k >= m->mats.size()) return io_fail(PT_EINVAL, "no such material");
  const Mtl& t = m->mats[k];
  if (name && name_cap) snprintf(name, name_cap, "%s", t.name.c_str());
  if (map_kd && map_cap) snprintf(map_kd, map_cap, "%s", t.map_kd.c_str());
  if (ka) memcpy(ka, t.ka, sizeof(t.ka));
  if (kd) memcpy(kd, t.kd, sizeof(t.kd));
  return PT_OK;
}

PT_API int pt_add_obj(pt_context* ctx, const pt_obj* m, uint32_t material, const float xform[12],
                      uint32_t* first_prim_id) {
  if (!ctx || !m) return PT_EINVAL;
  const size_t nt = m->mat.size();
  std::vector<uint32_t> idx(3 * nt);
  for (size_t i = 0; i < idx.size(); i++) idx[i] = (uint32_t)i;
  uint32_t mat_id = material;
  std::vector<uint32_t> tex_index;
  if (material == PT_OBJ_MTL) {
    // as the reference's Mesh without a given material (mesh.hpp:78-98):
    // Lambertian(Vector_Texture(per MTL material: Image_Texture(map_Kd) or
    // Constant_Texture(Ka))), each face indexing its material; without an
    // MTL file, a grey Lambertian
    if (m->mats.empty()) {
      const float grey[3] = {0.5f, 0.5f, 0.5f};
      int rc = pt_material_lambertian(ctx, grey, &mat_id);
      if (rc) return rc;
    } else {
      std::vector<uint32_t> texs(m->mats.size());
      for (size_t k = 0; k < m->mats.size(); k++) {
        const Mtl& t = m->mats[k];
        int rc;
        if (!t.map_kd.empty()) {
          std::string file = m->dir + t.map_kd;
          int w = 0, h = 0;
          if (pt_image_load(file.c_str(), &w, &h, nullptr))
            return io_fail(PT_EINVAL, std::string("map_Kd: ") + pt_image_last_error());
          std::vector<float> px((size_t)w * h * 4), flip((size_t)w * h * 4);
          if (pt_image_load(file.c_str(), &w, &h, px.data()))
            return io_fail(PT_EINVAL, std::string("map_Kd: ") + pt_image_last_error());
          // Image_Texture stores the file's last row first (textures.hpp:140-151)
          for (int y = 0; y < h; y++)
            memcpy(&flip[(size_t)y * w * 4], &px[(size_t)(h - 1 - y) * w * 4], (size_t)w * 16);
          rc = pt_texture_image(ctx, flip.data(), w, h, &texs[k]);
        } else {
          rc = pt_texture_constant(ctx, t.ka, &texs[k]);
        }
        if (rc) return rc;
      }
      uint32_t vec;
      const float black[3] = {0.f, 0.f, 0.f};
      int rc = pt_texture_vector(ctx, texs.data(), (int)texs.size(), &vec);
      if (!rc) rc = pt_material_lambertian(ctx, black, &mat_id);
      if (!rc) rc = pt_material_set_texture(ctx, mat_id, 0, vec);
      if (rc) return rc;
      tex_index.resize(nt);
      for (size_t i = 0; i < nt; i++) tex_index[i] = m->mat[i] == PT_OBJ_NO_MATERIAL ? 0u : m->mat[i];
    }
  }
  if (nt == 0) return PT_OK;
  uint32_t first = 0;
  int rc = pt_add_mesh(ctx, m->pos.data(), 3 * nt, idx.data(), nt, nullptr, mat_id,
                       m->has_nrm ? m->nrm.data() : nullptr, m->has_uv ? m->uv.data() : nullptr,
                       xform, &first);
  if (!rc && !tex_index.empty()) rc = pt_mesh_set_texture_index(ctx, first, nt, tex_index.data());
  if (!rc && first_prim_id) *first_prim_id = first;
  return rc;
}

// ------------------------------------------------------------- HDR ----------
// Radiance RGBE: text header ("#?RADIANCE" or "#?RGBE", lines, blank line),
// the resolution line "-Y h +X w", then h scanlines of w pixels, flat or run
// length encoded (the 2 2 hi lo scanline form, and the older repeat-pixel
// form).  A pixel (r, g, b, e) is (r, g, b) / 256 * 2^(e - 128), first
// scanline first, as the reference's loader stores it.
static int hdr_load_body(const char* path, int* w, int* h, float* rgba) {
  if (!path || !w || !h) return io_fail(PT_EINVAL, "null argument");
  std::string s;
  if (!read_file(path, s)) return io_fail(PT_EINVAL, std::string("cannot read ") + path);
  if (s.compare(0, 10, "#?RADIANCE") != 0 && s.compare(0, 6, "#?RGBE") != 0)
    return io_fail(PT_EINVAL, "not a Radiance HDR file");
  size_t p = s.find("\n\n");
  if (p == std::string::npos) return io_fail(PT_EINVAL, "no end of header");
  p += 2;
  size_t e = s.find('\n', p);
  if (e == std::string::npos) return io_fail(PT_EINVAL, "no resolution line");
  long H = 0, W = 0;
  if (sscanf(s.substr(p, e - p).c_str(), "-Y %ld +X %ld", &H, &W) != 2 || H <= 0 || W <= 0 ||
      H > 65536 || W > 65536)
    return io_fail(PT_EINVAL, "unsupported resolution line (expected -Y h +X w)");
  // at most 2^28 pixels (4 GiB of float texels), and at least one 4-byte
  // pixel of data per scanline, before the size is reported
  if ((uint64_t)W * (uint64_t)H > ((uint64_t)1 << 28)) return io_fail(PT_EINVAL, "HDR image too large");
  if ((size_t)H * 4 > s.size() - (e + 1)) return io_fail(PT_EINVAL, "truncated HDR data");
  *w = (int)W;
  *h = (int)H;
  if (!rgba) return PT_OK;
  p = e + 1;
  const unsigned char* d = (const unsigned char*)s.data();
  const size_t n = s.size();
  std::vector<unsigned char> line((size_t)W * 4);
  for (long y = 0; y < H; y++) {
    unsigned char* L = line.data();
    bool rle = W >= 8 && W <= 0x7fff && p + 4 <= n && d[p] == 2 && d[p + 1] == 2 &&
               !(d[p + 2] & 0x80) && (((long)d[p + 2] << 8) | d[p + 3]) == W;
    if (rle) {
      p += 4;
      for (int c = 0; c < 4; c++) {
        long x = 0;
        while (x < W) {
          if (p >= n) return io_fail(PT_EINVAL, "truncated scanline");
          unsigned code = d[p++];
          if (code > 128) {
            code &= 127;
            if (p >= n || x + (long)code > W) return io_fail(PT_EINVAL, "bad run");
            unsigned char val = d[p++];
            for (unsigned r = 0; r < code; r++) L[4 * (x++) + c] = val;
          } else {
            if (code == 0 || p + code > n || x + (long)code > W)
              return io_fail(PT_EINVAL, "bad literal run");
            for (unsigned r = 0; r < code; r++) L[4 * (x++) + c] = d[p++];
          }
        }
      }
    } else {
      // flat pixels; (1, 1, 1, k) repeats the previous pixel k << shift times
      long x = 0;
      int shift = 0;
      while (x < W) {
        if (p + 4 > n) return io_fail(PT_EINVAL, "truncated scanline");
        const unsigned char* q = d + p;
        p += 4;
        if (q[0] == 1 && q[1] == 1 && q[2] == 1) {
          if (x == 0) return io_fail(PT_EINVAL, "repeat before the first pixel");
          long cnt = (long)q[3] << shift;
          if (x + cnt > W) return io_fail(PT_EINVAL, "bad repeat");
          for (long r = 0; r < cnt; r++, x++) memcpy(L + 4 * x, L + 4 * (x - 1), 4);
          shift += 8;
        } else {
          memcpy(L + 4 * x, q, 4);
          x++;
          shift = 0;
        }
      }
    }
    float* out = rgba + (size_t)y * W * 4;
    for (long x = 0; x < W; x++) {
      const unsigned char* q = L + 4 * x;
      const int ex = (int)q[3] - 128;
      for (int c = 0; c < 3; c++) out[4 * x + c] = ldexpf((float)q[c] / 256.0f, ex);
      out[4 * x + 3] = 1.f;
    }
  }
  return PT_OK;
}

// Host memory running out while reading an untrusted file (a header can
// claim sizes its data cannot hold) is an error of the call, not an abort.
PT_API int pt_hdr_load(const char* path, int* w, int* h, float* rgba) {
  try {
    return hdr_load_body(path, w, h, rgba);
  } catch (const std::bad_alloc&) {
    return io_fail(PT_ENOMEM, "out of host memory reading the HDR file");
  }
}

// Save_HDR (image_save.hpp:40-73): the average over spp, Reinhard's c/(1+c)
// per channel, written as flat RGBE scanlines in buffer row order.  The
// reference's row loop runs over the width (image_save.hpp:46); every row of
// the image is written here.
PT_API int pt_hdr_save(const char* path, int w, int h, const float* accum_rgba, int spp) {
  if (!path || !accum_rgba || w <= 0 || h <= 0 || spp <= 0) return io_fail(PT_EINVAL, "bad argument");
  FILE* f = fopen(path, "wb");
  if (!f) return io_fail(PT_EINVAL, std::string("cannot write ") + path);
  fprintf(f, "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n", h, w);
  std::vector<unsigned char> row((size_t)w * 4);
  for (int y = 0; y < h; y++) {
    for (int x = 0; x < w; x++) {
      const float* a = accum_rgba + 4 * ((size_t)y * w + x);
      float c[3];
      for (int k = 0; k < 3; k++) {
        float v = a[k] / (float)spp;
        c[k] = v / (1.f + v);
      }
      // Ward's RGBE: the largest component's mantissa in [0.5, 1) x 256
      float m = std::max(c[0], std::max(c[1], c[2]));
      unsigned char* q = row.data() + 4 * x;
      if (!(m > 1e-32f)) {
        q[0] = q[1] = q[2] = q[3] = 0;
      } else {
        int ex = 0;
        float scale = frexpf(m, &ex) * 256.0f / m;
        for (int k = 0; k < 3; k++) q[k] = (unsigned char)std::min(255.f, std::max(0.f, c[k] * scale));
        q[3] = (unsigned char)(ex + 128);
      }
    }
    fwrite(row.data(), 1, row.size(), f);
  }
  bool ok = !ferror(f);
  ok = (fclose(f) == 0) && ok;
  return ok ? PT_OK : io_fail(PT_EINVAL, std::string("write failed: ") + path);
}

// ------------------------------------------------------------- PNG ----------
namespace {

struct CrcTable {
  uint32_t t[256];
  CrcTable() {
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t c = i;
      for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[i] = c;
    }
  }
};

uint32_t crc32_update(uint32_t crc, const unsigned char* p, size_t n) {
  static const CrcTable table;  // built once, safely under concurrent first calls
  for (size_t i = 0; i < n; i++) crc = table.t[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
  return crc;
}

void put32(std::vector<unsigned char>& v, uint32_t x) {
  v.push_back((unsigned char)(x >> 24));
  v.push_back((unsigned char)(x >> 16));
  v.push_back((unsigned char)(x >> 8));
  v.push_back((unsigned char)x);
}

void chunk(std::vector<unsigned char>& out, const char* type, const std::vector<unsigned char>& data) {
  put32(out, (uint32_t)data.size());
  size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  uint32_t crc = crc32_update(0xffffffffu, out.data() + start, out.size() - start) ^ 0xffffffffu;
  put32(out, crc);
}

}  // namespace

// Save_PNG (image_save.hpp:7-37): per channel sqrt(sum / spp), clamped to
// [0, 1], times 255.99, truncated; 8-bit RGB rows in buffer row order.  The
// zlib stream uses stored (uncompressed) deflate blocks.
PT_API int pt_png_save(const char* path, int w, int h, const float* accum_rgba, int spp) {
  if (!path || !accum_rgba || w <= 0 || h <= 0 || spp <= 0) return io_fail(PT_EINVAL, "bad argument");
  std::vector<unsigned char> raw;
  raw.reserve((size_t)h * (1 + 3 * (size_t)w));
  for (int y = 0; y < h; y++) {
    raw.push_back(0);  // filter: none
    for (int x = 0; x < w; x++) {
      const float* a = accum_rgba + 4 * ((size_t)y * w + x);
      for (int k = 0; k < 3; k++) {
        float v = sqrtf(a[k] / (float)spp);
        v = 255.99f * std::min(1.f, std::max(0.f, v));
        raw.push_back((unsigned char)(int)v);
      }
    }
  }
  std::vector<unsigned char> z;
  z.push_back(0x78);
  z.push_back(0x01);
  size_t off = 0;
  do {
    size_t len = std::min<size_t>(65535, raw.size() - off);
    bool last = off + len == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((unsigned char)(len & 0xff));
    z.push_back((unsigned char)(len >> 8));
    z.push_back((unsigned char)(~len & 0xff));
    z.push_back((unsigned char)((~len >> 8) & 0xff));
    z.insert(z.end(), raw.begin() + (long)off, raw.begin() + (long)(off + len));
    off += len;
  } while (off < raw.size());
  uint32_t s1 = 1, s2 = 0;  // Adler-32
  for (unsigned char c : raw) {
    s1 = (s1 + c) % 65521u;
    s2 = (s2 + s1) % 65521u;
  }
  put32(z, (s2 << 16) | s1);
  std::vector<unsigned char> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  std::vector<unsigned char> ihdr;
  put32(ihdr, (uint32_t)w);
  put32(ihdr, (uint32_t)h);
  ihdr.push_back(8);  // bit depth
  ihdr.push_back(2);  // colour type: RGB
  ihdr.push_back(0);
  ihdr.push_back(0);
  ihdr.push_back(0);
  chunk(out, "IHDR", ihdr);
  chunk(out, "IDAT", z);
  chunk(out, "IEND", {});
  FILE* f = fopen(path, "wb");
  if (!f) return io_fail(PT_EINVAL, std::string("cannot write ") + path);
  bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
  ok = (fclose(f) == 0) && ok;
  return ok ? PT_OK : io_fail(PT_EINVAL, std::string("write failed: ") + path);
}

}  // extern "C"
