// Image decoding for scene ingest: PNG (ISO/IEC 15948) over a zlib / deflate
// decoder (RFC 1950, RFC 1951), written from those specifications.
//
// The result is what the reference's texture loader holds after
// stbi_load(file, &X, &Y, &C, 0) and the channel copy of
// TextureUtility::LoadTextureFromFile (TextureUtility.cpp:12-35), with stb_image
// 2.12's choices where the PNG specification leaves room:
//  * the decoded buffer holds grey 1, grey+alpha 2, RGB 3, RGBA 4 or palette 3
//    channels per pixel; a tRNS chunk adds an alpha channel (palette: 4);
//  * the channel count C stbi_load reports is the file's (grey 1, grey+alpha
//    2, RGB 3, RGBA 4), or for a palette image the expanded one (3, or 4 with
//    tRNS), so for a grey or RGB image with tRNS it is one less than the
//    buffer holds;
//  * 16-bit samples keep their high byte; grey below 8 bits is scaled to
//    0..255 (x255, x85, x17 for 1, 2, 4 bits); palette indices are not scaled;
//  * tRNS on grey/RGB makes a pixel transparent when every sample equals the
//    key: at 16 bits on the 16-bit samples, otherwise on the 8-bit (scaled)
//    samples against the key's low byte times the grey scale, kept to 8 bits;
//  * chunk CRCs and the zlib Adler-32 are not checked; an unknown chunk whose
//    name starts with an upper-case letter (critical) is an error.
// LoadTextureFromFile then fills pixel i's colour (0, 0, 0, 1) from bytes
// i*C .. i*C + C-1 of the buffer, which is what the RGBA8 rows here hold (for
// grey or RGB with tRNS that reads the buffer with a stride one short of its
// own, as the reference does).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/friendsrender.h"
#include "fr_ingest.h"

namespace fr {
namespace {

// ------------------------------------------------------------------ inflate

struct BitReader {
  const uint8_t* p;
  size_t n;
  size_t pos = 0;
  uint64_t buf = 0;
  int cnt = 0;

  void refill() {
    while (cnt <= 56 && pos < n) {
      buf |= (uint64_t)p[pos++] << cnt;
      cnt += 8;
    }
  }
  // Takes `bits` (<= 32) bits, least significant first; false past the end.
  bool take(int bits, uint32_t* v) {
    if (cnt < bits) refill();
    if (cnt < bits) return false;
    *v = (uint32_t)(buf & ((1ull << bits) - 1));
    buf >>= bits;
    cnt -= bits;
    return true;
  }
  void align_to_byte() {
    const int drop = cnt & 7;
    buf >>= drop;
    cnt -= drop;
  }
};

constexpr int kFastBits = 9;

// Canonical Huffman code (RFC 1951 3.2.2): codes of each length are
// consecutive integers, assigned to the symbols in increasing order.
struct Huffman {
  uint16_t count[16];
  uint16_t symbol[320];
  uint16_t fast[1 << kFastBits];  // (length << 9) | symbol for codes <= 9 bits, 0 otherwise
};

uint32_t reverse_bits(uint32_t v, int bits) {
  uint32_t r = 0;
  for (int i = 0; i < bits; ++i) r = (r << 1) | ((v >> i) & 1u);
  return r;
}

// False for an over-subscribed set of lengths; an incomplete set is accepted
// (a code that is not assigned then fails to decode).
bool build_huffman(Huffman* h, const uint8_t* lengths, int n) {
  std::memset(h->count, 0, sizeof(h->count));
  std::memset(h->fast, 0, sizeof(h->fast));
  for (int i = 0; i < n; ++i) h->count[lengths[i]]++;
  h->count[0] = 0;
  int left = 1;
  for (int len = 1; len < 16; ++len) {
    left = (left << 1) - h->count[len];
    if (left < 0) return false;
  }
  uint16_t offset[16];
  offset[1] = 0;
  for (int len = 1; len < 15; ++len) offset[len + 1] = (uint16_t)(offset[len] + h->count[len]);
  for (int i = 0; i < n; ++i)
    if (lengths[i]) h->symbol[offset[lengths[i]]++] = (uint16_t)i;
  uint32_t code = 0;
  int k = 0;
  for (int len = 1; len <= kFastBits; ++len) {
    for (int j = 0; j < h->count[len]; ++j, ++code, ++k) {
      const uint32_t r = reverse_bits(code, len);
      for (uint32_t idx = r; idx < (1u << kFastBits); idx += 1u << len)
        h->fast[idx] = (uint16_t)((len << 9) | h->symbol[k]);
    }
    code <<= 1;
  }
  return true;
}

bool decode_symbol(BitReader& br, const Huffman& h, int* sym) {
  if (br.cnt < 15) br.refill();
  const uint16_t e = h.fast[br.buf & ((1u << kFastBits) - 1)];
  if (e) {
    const int len = e >> 9;
    if (len > br.cnt) return false;
    br.buf >>= len;
    br.cnt -= len;
    *sym = e & 511;
    return true;
  }
  // Longer codes: walk the lengths one bit at a time.
  int code = 0, first = 0, index = 0;
  for (int len = 1; len < 16; ++len) {
    if (len > br.cnt) return false;
    code |= (int)((br.buf >> (len - 1)) & 1u);
    const int count = h.count[len];
    if (code - first < count) {
      br.buf >>= len;
      br.cnt -= len;
      *sym = h.symbol[index + code - first];
      return true;
    }
    index += count;
    first = (first + count) << 1;
    code <<= 1;
  }
  return false;
}

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

// Decodes a zlib stream into at most `limit` bytes.
std::string inflate_zlib(const uint8_t* data, size_t n, size_t limit, std::vector<uint8_t>* out) {
  if (n < 2) return "zlib stream too short";
  const uint32_t cmf = data[0], flg = data[1];
  if ((cmf * 256 + flg) % 31 != 0) return "bad zlib header check";
  if ((cmf & 15) != 8 || (cmf >> 4) > 7) return "zlib stream is not deflate";
  if (flg & 32) return "zlib preset dictionary";
  BitReader br{data + 2, n - 2};
  out->clear();
  out->reserve(limit);
  // The fixed codes of RFC 1951 3.2.6 (built once, thread-safe static init).
  struct FixedCodes {
    Huffman lit, dist;
    FixedCodes() {
      uint8_t l[288];
      for (int i = 0; i < 288; ++i) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
      build_huffman(&lit, l, 288);
      uint8_t d[30];
      for (int i = 0; i < 30; ++i) d[i] = 5;
      build_huffman(&dist, d, 30);
    }
  };
  static const FixedCodes fixed;
  Huffman dyn_lit, dyn_dist;
  for (;;) {
    uint32_t final_block, type;
    if (!br.take(1, &final_block) || !br.take(2, &type)) return "truncated deflate block header";
    if (type == 0) {  // stored
      br.align_to_byte();
      uint32_t len, nlen;
      if (!br.take(16, &len) || !br.take(16, &nlen)) return "truncated stored block";
      if ((len ^ 0xFFFFu) != nlen) return "stored block length check";
      if (out->size() + len > limit) return "more image data than the image holds";
      while (len > 0 && br.cnt >= 8) {
        uint32_t b;
        br.take(8, &b);
        out->push_back((uint8_t)b);
        --len;
      }
      if (br.pos + len > br.n) return "truncated stored block";
      out->insert(out->end(), br.p + br.pos, br.p + br.pos + len);
      br.pos += len;
    } else if (type == 1 || type == 2) {
      const Huffman* lit = &fixed.lit;
      const Huffman* dist = &fixed.dist;
      if (type == 2) {
        uint32_t hlit, hdist, hclen;
        if (!br.take(5, &hlit) || !br.take(5, &hdist) || !br.take(4, &hclen)) return "truncated dynamic header";
        hlit += 257;
        hdist += 1;
        hclen += 4;
        if (hlit > 286 || hdist > 30) return "bad dynamic block code counts";
        static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
        uint8_t cl[19] = {0};
        for (uint32_t i = 0; i < hclen; ++i) {
          uint32_t v;
          if (!br.take(3, &v)) return "truncated code length codes";
          cl[order[i]] = (uint8_t)v;
        }
        Huffman clh;
        if (!build_huffman(&clh, cl, 19)) return "bad code length code";
        uint8_t lens[286 + 30];
        uint32_t k = 0;
        while (k < hlit + hdist) {
          int sym;
          if (!decode_symbol(br, clh, &sym)) return "bad code length symbol";
          if (sym < 16) {
            lens[k++] = (uint8_t)sym;
            continue;
          }
          uint32_t rep, v;
          uint8_t value = 0;
          if (sym == 16) {
            if (k == 0) return "length repeat with no previous length";
            value = lens[k - 1];
            if (!br.take(2, &v)) return "truncated repeat";
            rep = 3 + v;
          } else if (sym == 17) {
            if (!br.take(3, &v)) return "truncated repeat";
            rep = 3 + v;
          } else {
            if (!br.take(7, &v)) return "truncated repeat";
            rep = 11 + v;
          }
          if (k + rep > hlit + hdist) return "code lengths overrun";
          while (rep--) lens[k++] = value;
        }
        if (lens[256] == 0) return "no end-of-block code";
        if (!build_huffman(&dyn_lit, lens, (int)hlit) || !build_huffman(&dyn_dist, lens + hlit, (int)hdist))
          return "bad literal or distance code";
        lit = &dyn_lit;
        dist = &dyn_dist;
      }
      for (;;) {
        int sym;
        if (!decode_symbol(br, *lit, &sym)) return "bad literal/length code";
        if (sym < 256) {
          if (out->size() >= limit) return "more image data than the image holds";
          out->push_back((uint8_t)sym);
          continue;
        }
        if (sym == 256) break;
        sym -= 257;
        if (sym >= 29) return "bad length symbol";
        uint32_t extra = 0;
        if (kLenExtra[sym] && !br.take(kLenExtra[sym], &extra)) return "truncated length";
        const size_t len = kLenBase[sym] + extra;
        int dsym;
        if (!decode_symbol(br, *dist, &dsym) || dsym >= 30) return "bad distance code";
        uint32_t dextra = 0;
        if (kDistExtra[dsym] && !br.take(kDistExtra[dsym], &dextra)) return "truncated distance";
        const size_t d = kDistBase[dsym] + dextra;
        if (d > out->size()) return "distance before the start of the data";
        if (out->size() + len > limit) return "more image data than the image holds";
        const size_t from = out->size() - d;
        for (size_t i = 0; i < len; ++i) out->push_back((*out)[from + i]);
      }
    } else {
      return "bad deflate block type";
    }
    if (final_block) break;
  }
  return "";
}

// ---------------------------------------------------------------------- PNG

uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

struct PngInfo {
  uint32_t width, height;
  int depth, color, interlace;
  int samples;   // samples per pixel in the file
  int out_n;     // channels out (stb's img_out_n)
  bool has_trns = false;
  uint16_t key[3] = {0, 0, 0};  // tRNS key of a grey / RGB image
  std::vector<uint8_t> palette;  // RGBA per entry
};

// Unfilters the rows of one pass (`num_rows` rows of `row_bytes`, each after
// its filter byte) into `rows`; false on a bad filter type.
bool unfilter(const uint8_t* raw, uint32_t num_rows, size_t row_bytes, int bpp, std::vector<uint8_t>* rows) {
  rows->assign((size_t)num_rows * row_bytes, 0);
  for (uint32_t y = 0; y < num_rows; ++y) {
    const uint8_t* src = raw + (size_t)y * (row_bytes + 1);
    const int filter = src[0];
    ++src;
    uint8_t* cur = rows->data() + (size_t)y * row_bytes;
    const uint8_t* prev = y ? cur - row_bytes : nullptr;
    for (size_t i = 0; i < row_bytes; ++i) {
      const int a = i >= (size_t)bpp ? cur[i - bpp] : 0;
      const int b = prev ? prev[i] : 0;
      const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
      int v = src[i];
      switch (filter) {
        case 0: break;
        case 1: v += a; break;
        case 2: v += b; break;
        case 3: v += (a + b) >> 1; break;
        case 4: v += paeth(a, b, c); break;
        default: return false;
      }
      cur[i] = (uint8_t)v;
    }
  }
  return true;
}

// Converts unfiltered rows of a pass (pw x ph pixels) to out_n 8-bit
// channels and scatters them into the image at (x0 + i*dx, y0 + j*dy).
std::string convert_pass(const PngInfo& info, const std::vector<uint8_t>& rows, size_t row_bytes, uint32_t pw,
                         uint32_t ph, uint32_t x0, uint32_t y0, uint32_t dx, uint32_t dy, std::vector<uint8_t>* img) {
  static const int grey_scale[9] = {0, 0xff, 0x55, 0, 0x11, 0, 0, 0, 0x01};
  const int depth = info.depth, spp = info.samples, out_n = info.out_n;
  for (uint32_t j = 0; j < ph; ++j) {
    const uint8_t* row = rows.data() + (size_t)j * row_bytes;
    for (uint32_t i = 0; i < pw; ++i) {
      uint8_t* px = img->data() + (((size_t)(y0 + j * dy)) * info.width + (x0 + i * dx)) * out_n;
      uint32_t s16[4] = {0, 0, 0, 0};  // the pixel's samples at file depth
      for (int k = 0; k < spp; ++k) {
        const size_t bit = ((size_t)i * spp + k) * depth;
        if (depth == 16) {
          s16[k] = ((uint32_t)row[bit / 8] << 8) | row[bit / 8 + 1];
        } else if (depth == 8) {
          s16[k] = row[bit / 8];
        } else {
          const int shift = 8 - depth - (int)(bit & 7);
          s16[k] = (row[bit / 8] >> shift) & ((1u << depth) - 1);
        }
      }
      if (info.color == 3) {
        if (s16[0] * 4 >= info.palette.size()) return "palette index out of range";
        for (int c = 0; c < out_n; ++c) px[c] = info.palette[s16[0] * 4 + c];
        continue;
      }
      uint8_t s8[4];
      for (int k = 0; k < spp; ++k)
        s8[k] = depth == 16 ? (uint8_t)(s16[k] >> 8) : (uint8_t)(s16[k] * (depth < 8 && info.color == 0 ? grey_scale[depth] : 1));
      for (int k = 0; k < spp; ++k) px[k] = s8[k];
      if (info.has_trns) {
        bool match = true;
        for (int k = 0; k < spp; ++k) {
          if (depth == 16) {
            match = match && s16[k] == info.key[k];
          } else {
            const uint8_t key8 = (uint8_t)((info.key[k] & 255) * grey_scale[depth]);
            match = match && s8[k] == key8;
          }
        }
        px[spp] = match ? 0 : 255;
      }
    }
  }
  return "";
}

std::string decode_png(const std::vector<uint8_t>& file, DecodedImage* out) {
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  if (file.size() < 8 || std::memcmp(file.data(), sig, 8) != 0) return "not a PNG file (only PNG images are decoded)";
  PngInfo info{};
  std::vector<uint8_t> idat;
  bool have_header = false, have_plte = false, done = false;
  size_t pos = 8;
  while (!done) {
    if (pos + 8 > file.size()) return "truncated PNG chunk";
    const uint32_t len = be32(&file[pos]);
    const uint8_t* type = &file[pos + 4];
    if (len > 0x7FFFFFFFu || pos + 12 + (size_t)len > file.size()) return "truncated PNG chunk";
    const uint8_t* d = &file[pos + 8];
    const bool is_ihdr = std::memcmp(type, "IHDR", 4) == 0;
    if (!have_header && !is_ihdr) return "first PNG chunk is not IHDR";
    if (is_ihdr) {
      if (have_header || len != 13) return "bad IHDR";
      info.width = be32(d);
      info.height = be32(d + 4);
      info.depth = d[8];
      info.color = d[9];
      if (d[10] != 0 || d[11] != 0) return "unknown PNG compression or filter method";
      info.interlace = d[12];
      if (info.interlace > 1) return "bad interlace method";
      if (info.width == 0 || info.height == 0 || info.width > (1u << 24) || info.height > (1u << 24))
        return "bad image size";
      if ((uint64_t)info.width * info.height > (1ull << 30)) return "image too large";
      const int dp = info.depth, ct = info.color;
      if (dp != 1 && dp != 2 && dp != 4 && dp != 8 && dp != 16) return "bad bit depth";
      if (ct == 0) info.samples = 1;
      else if (ct == 2) info.samples = 3;
      else if (ct == 3) info.samples = 1;
      else if (ct == 4) info.samples = 2;
      else if (ct == 6) info.samples = 4;
      else return "bad colour type";
      if (ct == 3 && dp == 16) return "bad colour type";
      if ((ct == 2 || ct == 4 || ct == 6) && dp < 8) return "bad bit depth for the colour type";
      have_header = true;
    } else if (std::memcmp(type, "PLTE", 4) == 0) {
      if (len > 768 || len % 3 != 0) return "bad PLTE";
      info.palette.assign((size_t)(len / 3) * 4, 255);
      for (uint32_t i = 0; i < len / 3; ++i)
        for (int c = 0; c < 3; ++c) info.palette[i * 4 + c] = d[i * 3 + c];
      have_plte = true;
    } else if (std::memcmp(type, "tRNS", 4) == 0) {
      if (!idat.empty()) return "tRNS after IDAT";
      if (info.color == 3) {
        if (!have_plte) return "tRNS before PLTE";
        if (len > info.palette.size() / 4) return "bad tRNS length";
        for (uint32_t i = 0; i < len; ++i) info.palette[i * 4 + 3] = d[i];
      } else {
        if (info.color == 4 || info.color == 6) return "tRNS with alpha";
        if (len != (uint32_t)info.samples * 2) return "bad tRNS length";
        for (int k = 0; k < info.samples; ++k) info.key[k] = (uint16_t)((d[2 * k] << 8) | d[2 * k + 1]);
      }
      info.has_trns = true;
    } else if (std::memcmp(type, "IDAT", 4) == 0) {
      if (info.color == 3 && !have_plte) return "no PLTE";
      idat.insert(idat.end(), d, d + len);
    } else if (std::memcmp(type, "IEND", 4) == 0) {
      done = true;
    } else if (!(type[0] & 0x20)) {
      return std::string("unknown critical PNG chunk ") + std::string((const char*)type, 4);
    }
    pos += 12 + (size_t)len;
  }
  if (idat.empty()) return "no image data";
  info.out_n = info.color == 3 ? (info.has_trns ? 4 : 3) : info.samples + (info.has_trns ? 1 : 0);

  // The passes: one for a plain image, Adam7's seven otherwise.
  static const uint32_t ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
  static const uint32_t adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
  const int npass = info.interlace ? 7 : 1;
  struct Pass { uint32_t w, h, x0, y0, dx, dy; size_t row_bytes; };
  std::vector<Pass> passes;
  size_t expected = 0;
  for (int p = 0; p < npass; ++p) {
    Pass ps{};
    if (info.interlace) {
      ps.x0 = ax0[p]; ps.y0 = ay0[p]; ps.dx = adx[p]; ps.dy = ady[p];
      ps.w = info.width > ps.x0 ? (info.width - ps.x0 + ps.dx - 1) / ps.dx : 0;
      ps.h = info.height > ps.y0 ? (info.height - ps.y0 + ps.dy - 1) / ps.dy : 0;
    } else {
      ps = Pass{info.width, info.height, 0, 0, 1, 1, 0};
    }
    ps.row_bytes = ((size_t)ps.w * info.samples * info.depth + 7) / 8;
    if (ps.w && ps.h) expected += (ps.row_bytes + 1) * ps.h;
    passes.push_back(ps);
  }
  std::vector<uint8_t> raw;
  const std::string zerr = inflate_zlib(idat.data(), idat.size(), expected, &raw);
  if (!zerr.empty()) return zerr;
  if (raw.size() != expected) return "not enough image data";
  const int bpp = (info.samples * info.depth + 7) / 8;
  std::vector<uint8_t> img((size_t)info.width * info.height * info.out_n, 0);
  std::vector<uint8_t> rows;
  size_t off = 0;
  for (const Pass& ps : passes) {
    if (!ps.w || !ps.h) continue;
    if (!unfilter(raw.data() + off, ps.h, ps.row_bytes, bpp, &rows)) return "bad PNG filter type";
    const std::string cerr = convert_pass(info, rows, ps.row_bytes, ps.w, ps.h, ps.x0, ps.y0, ps.dx, ps.dy, &img);
    if (!cerr.empty()) return cerr;
    off += (ps.row_bytes + 1) * ps.h;
  }
  const int reported = info.color == 3 ? info.out_n : info.samples;
  out->width = (int32_t)info.width;
  out->height = (int32_t)info.height;
  out->channels = reported;
  out->rgba.assign((size_t)info.width * info.height * 4, 0);
  for (size_t i = 0; i < (size_t)info.width * info.height; ++i) {
    out->rgba[i * 4 + 3] = 255;
    for (int c = 0; c < reported; ++c) out->rgba[i * 4 + c] = img[i * reported + c];
  }
  return "";
}

}  // namespace

std::string decode_image_file(const std::string& path, DecodedImage* out) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return "cannot open " + path;
  std::vector<uint8_t> file;
  uint8_t chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) file.insert(file.end(), chunk, chunk + got);
  std::fclose(f);
  const std::string err = decode_png(file, out);
  return err.empty() ? err : path + ": " + err;
}

}  // namespace fr

extern "C" int fr_texture_load(const char* file, int32_t* width, int32_t* height, int32_t* channels, uint8_t* rgba) {
  if (!file) return fr::set_last_error(FR_ERR_INVALID, "fr_texture_load: file is NULL");
  fr::DecodedImage img;
  const std::string err = fr::decode_image_file(file, &img);
  if (!err.empty()) return fr::set_last_error(FR_ERR_IO, err);
  if (width) *width = img.width;
  if (height) *height = img.height;
  if (channels) *channels = img.channels;
  if (rgba) std::memcpy(rgba, img.rgba.data(), img.rgba.size());
  return FR_OK;
}
