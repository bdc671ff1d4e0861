// PNG writer for the exported image (the reference writes its render target
// with stbi_write_png, TextureUtility.cpp:52-65).  RGBA8, no interlacing,
// filter type 0 on every row, the zlib stream in stored (uncompressed)
// deflate blocks: a valid PNG whose decoded pixels are the bytes given.
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../include/friendsrender.h"

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
  for (uint32_t n = 0; n < 256; ++n) {
    uint32_t c = n;
    for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;  // reflected CRC-32 (ISO 3309)
    crc_table[n] = c;
  }
  crc_ready = true;
}

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xFFFFFFFFu) {
  for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
  return c;
}

void put32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& out, const char type[4], const std::vector<uint8_t>& data) {
  put32(out, (uint32_t)data.size());
  const size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  put32(out, crc32(out.data() + start, out.size() - start) ^ 0xFFFFFFFFu);
}

}  // namespace

extern "C" int fr_write_png(const char* path, int32_t width, int32_t height, const uint8_t* rgba) {
  if (!path || !rgba || width <= 0 || height <= 0 || (int64_t)width * 4 + 1 > 0x7FFFFFFF) return FR_ERR_INVALID;
  if (!crc_ready) crc_init();
  // Raw scanlines: a filter byte (0) and width * 4 bytes each.
  const size_t row = (size_t)width * 4 + 1;
  std::vector<uint8_t> raw(row * (size_t)height);
  for (int32_t y = 0; y < height; ++y) {
    raw[row * y] = 0;
    for (size_t k = 0; k < (size_t)width * 4; ++k) raw[row * y + 1 + k] = rgba[(size_t)y * width * 4 + k];
  }
  // zlib stream: header 0x78 0x01, stored blocks of at most 65535 bytes, Adler-32.
  std::vector<uint8_t> z = {0x78, 0x01};
  uint32_t a = 1, b = 0;
  for (size_t i = 0; i < raw.size(); ++i) {
    a = (a + raw[i]) % 65521u;
    b = (b + a) % 65521u;
  }
  for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
    const size_t len = raw.size() - off < 65535 ? raw.size() - off : 65535;
    const bool last = off + len >= raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)len);
    z.push_back((uint8_t)(len >> 8));
    z.push_back((uint8_t)~len);
    z.push_back((uint8_t)(~len >> 8));
    z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
    if (last) break;
  }
  put32(z, (b << 16) | a);
  std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  std::vector<uint8_t> ihdr;
  put32(ihdr, (uint32_t)width);
  put32(ihdr, (uint32_t)height);
  ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, filter 0, no interlace
  chunk(png, "IHDR", ihdr);
  chunk(png, "IDAT", z);
  chunk(png, "IEND", {});
  FILE* f = std::fopen(path, "wb");
  if (!f) return FR_ERR_INVALID;
  const bool ok = std::fwrite(png.data(), 1, png.size(), f) == png.size();
  return (std::fclose(f) == 0 && ok) ? FR_OK : FR_ERR_INVALID;
}
