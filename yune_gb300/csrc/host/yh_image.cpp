// yh_image.cpp -- headless image output: RendererCore::saveImage (src/RendererCore.cpp:608-646)
// without the GL read-back, from the float RGBA frames yc_tonemap / yc_read_accum return.
//
// Like the reference (stbi_flip_vertically_on_write over glReadPixels, whose row 0 is
// the bottom of the frame), the file's first row is the frame's last row (y = H - 1).
//   PNG  8-bit RGB, each channel converted as GL converts a float to an 8-bit normalized
//        value for glReadPixels(GL_UNSIGNED_BYTE): round(clamp(c, 0, 1) * 255), NaN -> 0.
//        Written with filter type 0 and stored (uncompressed) deflate blocks, so the file
//        needs no compression library; CRC-32 (PNG chunks) and Adler-32 (zlib stream)
//        computed here from their definitions.
//   HDR  Radiance RGBE, flat scanlines: per pixel the largest channel m = f * 2^e with
//        f in [0.5, 1) gives the shared exponent byte e + 128 and the mantissa bytes
//        floor(c * 256 / 2^e); pixels whose largest channel is below 1e-32 (or not
//        positive) are written as zero.
// JPEG output (lossy) is not provided.
#include "yune_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
  for (uint32_t n = 0; n < 256; ++n) {
    uint32_t c = n;
    for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    crc_table[n] = c;
  }
  crc_ready = true;
}

uint32_t crc32_of(const unsigned char* p, size_t n, uint32_t c = 0xFFFFFFFFu) {
  if (!crc_ready) crc_init();
  for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
  return c;
}

void be32(std::vector<unsigned char>& o, uint32_t v) {
  o.push_back((unsigned char)(v >> 24));
  o.push_back((unsigned char)(v >> 16));
  o.push_back((unsigned char)(v >> 8));
  o.push_back((unsigned char)v);
}

void chunk(std::vector<unsigned char>& out, const char* type, const std::vector<unsigned char>& data) {
  be32(out, (uint32_t)data.size());
  const size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  be32(out, crc32_of(out.data() + start, out.size() - start) ^ 0xFFFFFFFFu);
}

unsigned char unorm8(float c) {
  if (!(c > 0.0f)) return 0;   // negative, zero or NaN
  if (c >= 1.0f) return 255;
  return (unsigned char)std::lround(c * 255.0f);
}

bool write_file(const char* path, const std::vector<unsigned char>& bytes) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return false;
  const bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
  return std::fclose(f) == 0 && ok;
}

}  // namespace

extern "C" int yh_write_png(const char* path, int width, int height, const float* rgba) {
  if (!path || !rgba || width <= 0 || height <= 0) return YH_E_INVALID;
  try {
    // raw scanlines: filter byte 0, then RGB
    const size_t row = (size_t)width * 3 + 1;
    std::vector<unsigned char> raw(row * height);
    for (int r = 0; r < height; ++r) {
      const float* src = rgba + (size_t)(height - 1 - r) * width * 4;
      unsigned char* dst = raw.data() + (size_t)r * row;
      dst[0] = 0;
      for (int x = 0; x < width; ++x)
        for (int c = 0; c < 3; ++c) dst[1 + 3 * x + c] = unorm8(src[4 * x + c]);
    }
    // zlib stream of stored deflate blocks (at most 65535 bytes each)
    std::vector<unsigned char> z = {0x78, 0x01};
    size_t pos = 0;
    do {
      const size_t n = std::min<size_t>(65535, raw.size() - pos);
      const bool last = pos + n == raw.size();
      z.push_back(last ? 1 : 0);
      z.push_back((unsigned char)(n & 0xFF));
      z.push_back((unsigned char)(n >> 8));
      z.push_back((unsigned char)(~n & 0xFF));
      z.push_back((unsigned char)((~n >> 8) & 0xFF));
      z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
      pos += n;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;   // Adler-32 of the raw scanlines
    for (unsigned char v : raw) {
      a = (a + v) % 65521u;
      b = (b + a) % 65521u;
    }
    be32(z, (b << 16) | a);
    std::vector<unsigned char> out = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    std::vector<unsigned char> ihdr;
    be32(ihdr, (uint32_t)width);
    be32(ihdr, (uint32_t)height);
    const unsigned char rest[5] = {8, 2, 0, 0, 0};   // 8-bit, truecolour, deflate, filter 0, no interlace
    ihdr.insert(ihdr.end(), rest, rest + 5);
    chunk(out, "IHDR", ihdr);
    chunk(out, "IDAT", z);
    chunk(out, "IEND", {});
    return write_file(path, out) ? YH_OK : YH_E_INVALID;
  } catch (const std::bad_alloc&) {
    return YH_E_NOMEM;
  }
}

extern "C" int yh_write_hdr(const char* path, int width, int height, const float* rgba) {
  if (!path || !rgba || width <= 0 || height <= 0) return YH_E_INVALID;
  try {
    std::vector<unsigned char> out;
    char head[96];
    const int n = std::snprintf(head, sizeof(head), "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n", height,
                                width);
    out.insert(out.end(), head, head + n);
    out.reserve(out.size() + (size_t)width * height * 4);
    for (int r = 0; r < height; ++r) {
      const float* src = rgba + (size_t)(height - 1 - r) * width * 4;
      for (int x = 0; x < width; ++x) {
        const float c[3] = {src[4 * x], src[4 * x + 1], src[4 * x + 2]};
        float m = c[0] > c[1] ? c[0] : c[1];
        m = m > c[2] ? m : c[2];
        unsigned char e4[4] = {0, 0, 0, 0};
        if (m > 1e-32f && std::isfinite(m)) {
          int e = 0;
          std::frexp(m, &e);   // m = f * 2^e, f in [0.5, 1)
          const float scale = std::ldexp(256.0f, -e);
          for (int k = 0; k < 3; ++k) e4[k] = c[k] > 0.0f ? (unsigned char)(c[k] * scale) : 0;
          e4[3] = (unsigned char)(e + 128);
        }
        out.insert(out.end(), e4, e4 + 4);
      }
    }
    return write_file(path, out) ? YH_OK : YH_E_INVALID;
  } catch (const std::bad_alloc&) {
    return YH_E_NOMEM;
  }
}
