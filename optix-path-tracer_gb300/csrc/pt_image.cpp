/*
 * pt_image.cpp - image files for image textures (host side, no device
 * work): PNG (RFC 2083; inflate per RFC 1951 / 1950 written here), binary
 * and ASCII PPM, and Radiance HDR (through pt_hdr_load).
 *
 * The reference reads texture images with stb_image (lib/stb_image.h, a
 * vendored third-party decoder; host_includes/textures.hpp:114-175) and
 * reads the texels as normalised floats; pt_image_load returns the same
 * values, 8-bit samples / 255 (16-bit / 65535), RGBA, first file row first.
 * JPEG and the other formats stb_image also reads are not decoded here.
 */
#include <ctype.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <new>
#include <string>
#include <vector>

#include "../../include/pt.h"

namespace {

thread_local std::string g_img_err;

int img_fail(int code, const std::string& msg) {
  g_img_err = msg;
  return code;
}

bool read_all(const char* path, std::vector<uint8_t>& out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  uint8_t buf[65536];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
  fclose(f);
  return true;
}

// ------------------------------------------------------------- inflate ----
// DEFLATE (RFC 1951): stored, fixed-Huffman and dynamic-Huffman blocks.
// Canonical Huffman codes are decoded one bit at a time against the count
// of codes of each length.
class Inflater {
 public:
  Inflater(const uint8_t* in, size_t n, std::vector<uint8_t>& out) : in_(in), n_(n), out_(out) {}

  bool run() {
    int last;
    do {
      last = bits(1);
      int type = bits(2);
      if (err_) return false;
      bool ok = type == 0 ? stored() : type == 1 ? fixed() : type == 2 ? dynamic() : false;
      if (!ok || err_) return false;
    } while (!last);
    return true;
  }
  size_t consumed() const { return pos_; }

 private:
  struct Huff {
    uint16_t count[16];
    uint16_t symbol[320];
  };

  uint32_t bits(int need) {
    uint32_t v = bitbuf_;
    while (bitcnt_ < need) {
      if (pos_ >= n_) {
        err_ = true;
        return 0;
      }
      v |= (uint32_t)in_[pos_++] << bitcnt_;
      bitcnt_ += 8;
    }
    bitbuf_ = need < 32 ? v >> need : 0;
    bitcnt_ -= need;
    return need < 32 ? v & ((1u << need) - 1u) : v;
  }

  // Builds the decoding table of n code lengths; false if over-subscribed.
  static bool build(Huff& h, const uint8_t* len, int n) {
    memset(h.count, 0, sizeof(h.count));
    for (int s = 0; s < n; s++) h.count[len[s]]++;
    if (h.count[0] == n) return true;  // no codes: the block uses none
    int left = 1;
    for (int l = 1; l < 16; l++) {
      left <<= 1;
      left -= h.count[l];
      if (left < 0) return false;
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; l++) offs[l + 1] = offs[l] + h.count[l];
    for (int s = 0; s < n; s++)
      if (len[s]) h.symbol[offs[len[s]]++] = (uint16_t)s;
    return true;
  }

  int decode(const Huff& h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; l++) {
      code |= (int)bits(1);
      int count = h.count[l];
      if (code - count < first) return h.symbol[index + (code - first)];
      index += count;
      first += count;
      first <<= 1;
      code <<= 1;
    }
    err_ = true;
    return -1;
  }

  bool stored() {
    bitbuf_ = 0;
    bitcnt_ = 0;
    if (pos_ + 4 > n_) return false;
    unsigned len = in_[pos_] | (in_[pos_ + 1] << 8);
    unsigned nlen = in_[pos_ + 2] | (in_[pos_ + 3] << 8);
    pos_ += 4;
    if (len != (~nlen & 0xffffu) || pos_ + len > n_) return false;
    out_.insert(out_.end(), in_ + pos_, in_ + pos_ + len);
    pos_ += len;
    return true;
  }

  bool codes(const Huff& lit, const Huff& dist) {
    static const uint16_t lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                       31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                     2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,
                                       33,  49,  65,  97,  129, 193,  257,  385,  513,  769,
                                       1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                     6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    for (;;) {
      int sym = decode(lit);
      if (err_ || sym < 0) return false;
      if (sym < 256) {
        out_.push_back((uint8_t)sym);
      } else if (sym == 256) {
        return true;
      } else {
        sym -= 257;
        if (sym >= 29) return false;
        size_t len = lbase[sym] + bits(lext[sym]);
        int ds = decode(dist);
        if (err_ || ds < 0 || ds >= 30) return false;
        size_t d = dbase[ds] + bits(dext[ds]);
        if (err_ || d > out_.size()) return false;
        size_t from = out_.size() - d;
        for (size_t k = 0; k < len; k++) out_.push_back(out_[from + k]);
      }
    }
  }

  bool fixed() {
    uint8_t len[320];
    for (int s = 0; s < 144; s++) len[s] = 8;
    for (int s = 144; s < 256; s++) len[s] = 9;
    for (int s = 256; s < 280; s++) len[s] = 7;
    for (int s = 280; s < 288; s++) len[s] = 8;
    Huff lit, dist;
    build(lit, len, 288);
    for (int s = 0; s < 30; s++) len[s] = 5;
    build(dist, len, 30);
    return codes(lit, dist);
  }

  bool dynamic() {
    static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    int nlen = (int)bits(5) + 257, ndist = (int)bits(5) + 1, ncode = (int)bits(4) + 4;
    if (err_ || nlen > 286 || ndist > 30) return false;
    uint8_t len[320];
    memset(len, 0, sizeof(len));
    for (int k = 0; k < ncode; k++) len[order[k]] = (uint8_t)bits(3);
    Huff lencode;
    if (!build(lencode, len, 19)) return false;
    int k = 0;
    while (k < nlen + ndist) {
      int sym = decode(lencode);
      if (err_ || sym < 0) return false;
      if (sym < 16) {
        len[k++] = (uint8_t)sym;
      } else {
        uint8_t v = 0;
        int rep;
        if (sym == 16) {
          if (k == 0) return false;
          v = len[k - 1];
          rep = 3 + (int)bits(2);
        } else if (sym == 17) {
          rep = 3 + (int)bits(3);
        } else {
          rep = 11 + (int)bits(7);
        }
        if (k + rep > nlen + ndist) return false;
        while (rep--) len[k++] = v;
      }
    }
    if (len[256] == 0) return false;  // the block needs its end code
    Huff lit, dist;
    if (!build(lit, len, nlen) || !build(dist, len + nlen, ndist)) return false;
    return codes(lit, dist);
  }

  const uint8_t* in_;
  size_t n_, pos_ = 0;
  uint32_t bitbuf_ = 0;
  int bitcnt_ = 0;
  bool err_ = false;
  std::vector<uint8_t>& out_;
};

uint32_t be32(const uint8_t* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

// --------------------------------------------------------------- PNG ------
int load_png(const std::vector<uint8_t>& f, int* W, int* H, std::vector<float>* rgba) {
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
  if (f.size() < 8 || memcmp(f.data(), sig, 8) != 0) return img_fail(PT_EINVAL, "not a PNG file");
  uint32_t w = 0, h = 0;
  int depth = 0, ctype = -1;
  std::vector<uint8_t> idat, plte, trns;
  size_t p = 8;
  bool end = false;
  while (!end && p + 8 <= f.size()) {
    uint32_t len = be32(&f[p]);
    if (p + 12 + (size_t)len > f.size()) return img_fail(PT_EINVAL, "truncated PNG chunk");
    const uint8_t* type = &f[p + 4];
    const uint8_t* d = &f[p + 8];
    if (!memcmp(type, "IHDR", 4)) {
      if (len < 13) return img_fail(PT_EINVAL, "bad PNG header");
      w = be32(d);
      h = be32(d + 4);
      depth = d[8];
      ctype = d[9];
      if (d[10] != 0 || d[11] != 0) return img_fail(PT_EINVAL, "unknown PNG compression/filter");
      if (d[12] != 0) return img_fail(PT_EINVAL, "interlaced PNG is not supported");
    } else if (!memcmp(type, "PLTE", 4)) {
      plte.assign(d, d + len);
    } else if (!memcmp(type, "tRNS", 4)) {
      trns.assign(d, d + len);
    } else if (!memcmp(type, "IDAT", 4)) {
      idat.insert(idat.end(), d, d + len);
    } else if (!memcmp(type, "IEND", 4)) {
      end = true;
    }
    p += 12 + (size_t)len;
  }
  if (w == 0 || h == 0 || w > 32768 || h > 32768) return img_fail(PT_EINVAL, "PNG size");
  int chans;
  switch (ctype) {
    case 0: chans = 1; break;
    case 2: chans = 3; break;
    case 3: chans = 1; break;
    case 4: chans = 2; break;
    case 6: chans = 4; break;
    default: return img_fail(PT_EINVAL, "unknown PNG colour type");
  }
  if (!(depth == 8 || (depth == 16 && ctype != 3)))
    return img_fail(PT_EINVAL, "PNG bit depth " + std::to_string(depth) + " is not supported");
  if (ctype == 3 && plte.size() < 3) return img_fail(PT_EINVAL, "PNG palette missing");
  const size_t bpp = (size_t)chans * (depth / 8), row = (size_t)w * bpp;
  // deflate expands its input at most 1032-fold: a header whose image cannot
  // come out of the data it carries is refused before anything is sized by it
  if ((row + 1) * h > idat.size() * 1032 + 1024)
    return img_fail(PT_EINVAL, "PNG data too short for its size");
  *W = (int)w;
  *H = (int)h;
  if (!rgba) return PT_OK;
  // zlib stream (RFC 1950): CMF, FLG, deflate data, Adler-32
  if (idat.size() < 6 || (idat[0] & 15) != 8 || ((idat[0] << 8) | idat[1]) % 31 != 0 ||
      (idat[1] & 0x20))
    return img_fail(PT_EINVAL, "bad zlib stream in PNG");
  std::vector<uint8_t> raw;
  raw.reserve((row + 1) * h);
  Inflater inf(idat.data() + 2, idat.size() - 2, raw);
  if (!inf.run() || raw.size() < (row + 1) * h) return img_fail(PT_EINVAL, "corrupt PNG data");
  // undo the scanline filters (none, sub, up, average, Paeth)
  std::vector<uint8_t> px(row * h);
  for (uint32_t y = 0; y < h; y++) {
    const uint8_t* src = &raw[y * (row + 1)];
    uint8_t ft = src[0];
    uint8_t* cur = &px[y * row];
    const uint8_t* prev = y ? &px[(y - 1) * row] : nullptr;
    for (size_t i = 0; i < row; i++) {
      int a = i >= bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0,
          c = (prev && i >= bpp) ? prev[i - bpp] : 0;
      int x = src[1 + i], v;
      switch (ft) {
        case 0: v = x; break;
        case 1: v = x + a; break;
        case 2: v = x + b; break;
        case 3: v = x + ((a + b) >> 1); break;
        case 4: {
          int pp = a + b - c, pa = pp > a ? pp - a : a - pp, pb = pp > b ? pp - b : b - pp,
              pc = pp > c ? pp - c : c - pp;
          v = x + ((pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c));
          break;
        }
        default: return img_fail(PT_EINVAL, "bad PNG filter type");
      }
      cur[i] = (uint8_t)v;
    }
  }
  rgba->assign((size_t)w * h * 4, 0.f);
  const float s = depth == 8 ? 255.f : 65535.f;  // texel = sample / maximum
  for (size_t i = 0; i < (size_t)w * h; i++) {
    const uint8_t* q = &px[i * bpp];
    auto sample = [&](int k) {
      return depth == 8 ? (float)q[k] : (float)((q[2 * k] << 8) | q[2 * k + 1]);
    };
    float* o = &(*rgba)[4 * i];
    if (ctype == 3) {
      size_t e = q[0];
      if (3 * e + 2 >= plte.size()) return img_fail(PT_EINVAL, "PNG palette index out of range");
      o[0] = plte[3 * e] / s;
      o[1] = plte[3 * e + 1] / s;
      o[2] = plte[3 * e + 2] / s;
      o[3] = e < trns.size() ? trns[e] / s : 1.f;
    } else if (chans <= 2) {
      o[0] = o[1] = o[2] = sample(0) / s;
      o[3] = chans == 2 ? sample(1) / s : 1.f;
    } else {
      o[0] = sample(0) / s;
      o[1] = sample(1) / s;
      o[2] = sample(2) / s;
      o[3] = chans == 4 ? sample(3) / s : 1.f;
    }
  }
  return PT_OK;
}

// --------------------------------------------------------------- PPM ------
int load_ppm(const std::vector<uint8_t>& f, int* W, int* H, std::vector<float>* rgba) {
  size_t p = 2;
  auto token = [&](long& v) {
    for (;;) {
      while (p < f.size() && isspace(f[p])) p++;
      if (p < f.size() && f[p] == '#') {
        while (p < f.size() && f[p] != '\n') p++;
        continue;
      }
      break;
    }
    if (p >= f.size() || !isdigit(f[p])) return false;
    v = 0;
    while (p < f.size() && isdigit(f[p])) {
      if (v > 100000000) return false;  // larger than any valid size or sample
      v = v * 10 + (f[p++] - '0');
    }
    return true;
  };
  long w, h, mx;
  if (!token(w) || !token(h) || !token(mx) || w <= 0 || h <= 0 || w > 32768 || h > 32768 ||
      mx <= 0 || mx > 65535)
    return img_fail(PT_EINVAL, "bad PPM header");
  const bool binary = f[1] == '6';
  const size_t n = (size_t)w * h;
  const size_t bs = mx > 255 ? 2 : 1;
  // the samples must fit in the file (binary ones exactly, text ones one
  // digit and one separator each at the least) before the size is reported
  if (binary ? p + 1 + n * 3 * bs > f.size() : 2 * 3 * n > f.size() - p + 1)
    return img_fail(PT_EINVAL, "truncated PPM data");
  *W = (int)w;
  *H = (int)h;
  if (!rgba) return PT_OK;
  rgba->assign(n * 4, 1.f);
  if (binary) {
    p++;  // the single whitespace after maxval
    for (size_t i = 0; i < 3 * n; i++) {
      long v = bs == 2 ? ((f[p + 2 * i] << 8) | f[p + 2 * i + 1]) : f[p + i];
      (*rgba)[4 * (i / 3) + i % 3] = (float)v / (float)mx;
    }
  } else {
    for (size_t i = 0; i < 3 * n; i++) {
      long v;
      if (!token(v)) return img_fail(PT_EINVAL, "truncated PPM data");
      (*rgba)[4 * (i / 3) + i % 3] = (float)v / (float)mx;
    }
  }
  return PT_OK;
}

}  // namespace

extern "C" {

// Any supported image: w x h, RGBA floats, first file row first.  rgba NULL
// returns the size only.
static int image_load_body(const char* path, int* w, int* h, float* rgba) {
  if (!path || !w || !h) return img_fail(PT_EINVAL, "null argument");
  std::vector<uint8_t> f;
  if (!read_all(path, f)) return img_fail(PT_EINVAL, std::string("cannot read ") + path);
  if (f.size() >= 2 && f[0] == 'P' && (f[1] == '6' || f[1] == '3')) {
    std::vector<float> px;
    int rc = load_ppm(f, w, h, rgba ? &px : nullptr);
    if (rc == PT_OK && rgba) memcpy(rgba, px.data(), px.size() * sizeof(float));
    return rc;
  }
  if (f.size() >= 8 && f[0] == 0x89 && f[1] == 'P') {
    std::vector<float> px;
    int rc = load_png(f, w, h, rgba ? &px : nullptr);
    if (rc == PT_OK && rgba) memcpy(rgba, px.data(), px.size() * sizeof(float));
    return rc;
  }
  if (f.size() >= 2 && f[0] == '#' && f[1] == '?') {
    int rc = pt_hdr_load(path, w, h, rgba);
    if (rc) g_img_err = pt_io_last_error();
    return rc;
  }
  if (f.size() >= 2 && f[0] == 0xff && f[1] == 0xd8)
    return img_fail(PT_EINVAL, std::string(path) + ": JPEG images are not decoded (PNG, PPM, "
                                                  "Radiance HDR are)");
  return img_fail(PT_EINVAL, std::string(path) + ": unknown image format");
}

// Host memory running out while reading an untrusted file (a header can
// claim sizes its data cannot hold) is an error of the call, not an abort.
PT_API int pt_image_load(const char* path, int* w, int* h, float* rgba) {
  try {
    return image_load_body(path, w, h, rgba);
  } catch (const std::bad_alloc&) {
    return img_fail(PT_ENOMEM, "out of host memory reading the image");
  }
}

PT_API const char* pt_image_last_error(void) { return g_img_err.c_str(); }

}  // extern "C"
