// Image decoding for textures, as core/ResourceManager.cpp:288-315 loads them: stbi_load with
// four requested channels, i.e. 8-bit RGBA whatever the file holds. stb_image is not available
// here, so the formats it would read for an environment map are decoded by this file:
//
//  * PNG (ISO/IEC 15948): zlib/deflate streams (RFC 1950/1951: stored, fixed and dynamic
//    Huffman blocks), the five scan-line filters, Adam7 interlacing, every colour type and bit
//    depth. Grey expands to RGB, a missing alpha is 255, sub-byte grey is scaled to 0..255 (1 bit
//    x255, 2 bits x85, 4 bits x17), palettes expand through PLTE/tRNS, a tRNS colour key makes the
//    matching pixels transparent, and 16-bit samples keep their high byte (stb's 16 -> 8 rule).
//  * Binary PNM (P5 grey, P6 RGB): samples as stored (no rescaling by maxval; 16-bit samples
//    keep their high byte).
//
// JPEG and Radiance HDR are not decoded (NE_ERR_UNSUPPORTED).
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "image_load.h"

namespace neimg {
namespace {

// ---------------------------------------------------------------- inflate (RFC 1951)
struct BitReader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t buf = 0;
  int cnt = 0;
  bool over = false;
  int bit() {
    if (cnt == 0) {
      if (pos >= n) {
        over = true;
        return 0;
      }
      buf = p[pos++];
      cnt = 8;
    }
    int b = buf & 1;
    buf >>= 1;
    cnt--;
    return b;
  }
  uint32_t bits(int k) {  // k <= 16, least significant bit first
    uint32_t v = 0;
    for (int i = 0; i < k; i++) v |= (uint32_t)bit() << i;
    return v;
  }
  void alignByte() {
    buf = 0;
    cnt = 0;
  }
};

// Canonical Huffman code: count[len] codes of each length, symbols in code order.
struct Huffman {
  uint16_t count[16];
  std::vector<uint16_t> symbol;
  bool build(const uint8_t* lengths, int n) {
    memset(count, 0, sizeof(count));
    for (int i = 0; i < n; i++) count[lengths[i]]++;
    count[0] = 0;
    int left = 1;
    for (int len = 1; len < 16; len++) {
      left <<= 1;
      left -= count[len];
      if (left < 0) return false;  // over-subscribed
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int len = 1; len < 15; len++) offs[len + 1] = offs[len] + count[len];
    symbol.assign(n, 0);
    for (int i = 0; i < n; i++)
      if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
    return true;
  }
  // Reads one symbol: codes are read most significant bit first.
  int decode(BitReader& br) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; len++) {
      code |= br.bit();
      int c = count[len];
      if (code - first < c) return symbol[index + code - first];
      index += c;
      first += c;
      first <<= 1;
      code <<= 1;
      if (br.over) return -1;
    }
    return -1;
  }
};

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflateCodes(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out) {
  for (;;) {
    int sym = lit.decode(br);
    if (sym < 0) return false;
    if (sym < 256) {
      out.push_back((uint8_t)sym);
    } else if (sym == 256) {
      return true;
    } else {
      sym -= 257;
      if (sym >= 29) return false;
      size_t len = kLenBase[sym] + br.bits(kLenExtra[sym]);
      int ds = dist.decode(br);
      if (ds < 0 || ds >= 30) return false;
      size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
      if (d > out.size() || br.over) return false;
      size_t from = out.size() - d;
      for (size_t i = 0; i < len; i++) out.push_back(out[from + i]);
    }
  }
}

// The fixed literal/length and distance codes of block type 1 (RFC 1951 3.2.6).
struct FixedCodes {
  Huffman lit, dist;
};
FixedCodes makeFixedCodes() {
  FixedCodes f;
  uint8_t l[288];
  for (int i = 0; i < 144; i++) l[i] = 8;
  for (int i = 144; i < 256; i++) l[i] = 9;
  for (int i = 256; i < 280; i++) l[i] = 7;
  for (int i = 280; i < 288; i++) l[i] = 8;
  f.lit.build(l, 288);
  uint8_t d[30];
  for (int i = 0; i < 30; i++) d[i] = 5;
  f.dist.build(d, 30);
  return f;
}

bool inflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, std::string& err) {
  BitReader br{p, n};
  int last;
  do {
    last = br.bit();
    int type = (int)br.bits(2);
    if (br.over) break;
    if (type == 0) {
      br.alignByte();
      if (br.pos + 4 > n) {
        br.over = true;
        break;
      }
      uint32_t len = p[br.pos] | (p[br.pos + 1] << 8), nlen = p[br.pos + 2] | (p[br.pos + 3] << 8);
      br.pos += 4;
      if ((len ^ 0xFFFFu) != nlen || br.pos + len > n) {
        err = "corrupt stored deflate block";
        return false;
      }
      out.insert(out.end(), p + br.pos, p + br.pos + len);
      br.pos += len;
    } else if (type == 1) {
      static const FixedCodes fixed = makeFixedCodes();  // initialised once, thread-safe
      if (!inflateCodes(br, fixed.lit, fixed.dist, out)) {
        err = "corrupt fixed-Huffman deflate block";
        return false;
      }
    } else if (type == 2) {
      int nlen = (int)br.bits(5) + 257, ndist = (int)br.bits(5) + 1, ncode = (int)br.bits(4) + 4;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < ncode; i++) cl[order[i]] = (uint8_t)br.bits(3);
      Huffman clh;
      if (nlen > 286 || ndist > 30 || !clh.build(cl, 19)) {
        err = "corrupt dynamic deflate header";
        return false;
      }
      uint8_t lengths[320] = {0};
      int i = 0;
      while (i < nlen + ndist) {
        int sym = clh.decode(br);
        if (sym < 0) {
          err = "corrupt code lengths";
          return false;
        }
        if (sym < 16) {
          lengths[i++] = (uint8_t)sym;
        } else {
          int rep;
          uint8_t val = 0;
          if (sym == 16) {
            if (i == 0) {
              err = "corrupt code lengths";
              return false;
            }
            val = lengths[i - 1];
            rep = 3 + (int)br.bits(2);
          } else if (sym == 17) {
            rep = 3 + (int)br.bits(3);
          } else {
            rep = 11 + (int)br.bits(7);
          }
          if (i + rep > nlen + ndist) {
            err = "corrupt code lengths";
            return false;
          }
          while (rep--) lengths[i++] = val;
        }
      }
      Huffman lit, dist;
      if (!lit.build(lengths, nlen) || !dist.build(lengths + nlen, ndist) || !inflateCodes(br, lit, dist, out)) {
        err = "corrupt dynamic-Huffman deflate block";
        return false;
      }
    } else {
      err = "invalid deflate block type";
      return false;
    }
  } while (!last);
  if (br.over) {
    err = "truncated deflate stream";
    return false;
  }
  return true;
}

uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c) {
  int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

// Undoes the scan-line filters of one (sub-)image in place; `raw` holds h lines of 1 + stride bytes.
bool unfilter(uint8_t* raw, uint32_t h, size_t stride, int bpp, std::vector<uint8_t>& img) {
  img.assign((size_t)h * stride, 0);
  for (uint32_t y = 0; y < h; y++) {
    int f = raw[y * (stride + 1)];
    const uint8_t* src = raw + y * (stride + 1) + 1;
    uint8_t* cur = img.data() + (size_t)y * stride;
    const uint8_t* prev = y ? cur - stride : nullptr;
    for (size_t i = 0; i < stride; i++) {
      int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0, c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
      int v = src[i];
      switch (f) {
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

struct PngInfo {
  uint32_t w, h;
  int depth, ctype, interlace;
  int channels;
  std::vector<uint8_t> plte, trns;
};

// Sample k (0-based) of a line of `depth`-bit samples.
uint32_t sampleAt(const uint8_t* line, size_t k, int depth) {
  if (depth == 8) return line[k];
  if (depth == 16) return ((uint32_t)line[2 * k] << 8) | line[2 * k + 1];
  size_t bit = k * depth;
  return (line[bit >> 3] >> (8 - depth - (bit & 7))) & ((1u << depth) - 1);
}

// Writes the pixels of a decoded (sub-)image line to RGBA8 at the given pixel positions.
void emitLine(const PngInfo& P, const uint8_t* line, uint32_t n, uint8_t* out, const uint32_t* xs, size_t rowOff) {
  const int d = P.depth;
  for (uint32_t i = 0; i < n; i++) {
    uint8_t* o = out + (rowOff + xs[i]) * 4;
    uint32_t s[4] = {0, 0, 0, 0};
    for (int c = 0; c < P.channels; c++) s[c] = sampleAt(line, (size_t)i * P.channels + c, d);
    auto to8 = [&](uint32_t v) -> uint8_t {
      if (d == 16) return (uint8_t)(v >> 8);
      if (d == 8) return (uint8_t)v;
      return (uint8_t)(v * (255u / ((1u << d) - 1)));  // 1 bit x255, 2 bits x85, 4 bits x17
    };
    switch (P.ctype) {
      case 0: {
        uint8_t g = to8(s[0]);
        o[0] = o[1] = o[2] = g;
        o[3] = 255;
        if (P.trns.size() >= 2 && s[0] == (((uint32_t)P.trns[0] << 8) | P.trns[1])) o[3] = 0;
        break;
      }
      case 2:
        o[0] = to8(s[0]); o[1] = to8(s[1]); o[2] = to8(s[2]); o[3] = 255;
        if (P.trns.size() >= 6 && s[0] == (((uint32_t)P.trns[0] << 8) | P.trns[1]) &&
            s[1] == (((uint32_t)P.trns[2] << 8) | P.trns[3]) && s[2] == (((uint32_t)P.trns[4] << 8) | P.trns[5]))
          o[3] = 0;
        break;
      case 3: {
        uint32_t k = s[0];
        if (3 * k + 2 < P.plte.size()) {
          o[0] = P.plte[3 * k]; o[1] = P.plte[3 * k + 1]; o[2] = P.plte[3 * k + 2];
        } else {
          o[0] = o[1] = o[2] = 0;
        }
        o[3] = k < P.trns.size() ? P.trns[k] : 255;
        break;
      }
      case 4: {
        uint8_t g = to8(s[0]);
        o[0] = o[1] = o[2] = g;
        o[3] = to8(s[1]);
        break;
      }
      default:
        o[0] = to8(s[0]); o[1] = to8(s[1]); o[2] = to8(s[2]); o[3] = to8(s[3]);
        break;
    }
  }
}

bool decodePng(const std::vector<uint8_t>& f, Image& img, std::string& err) {
  PngInfo P{};
  std::vector<uint8_t> idat;
  size_t pos = 8;
  bool haveHdr = false;
  while (pos + 8 <= f.size()) {
    uint32_t len = be32(&f[pos]);
    if (pos + 12 + (size_t)len > f.size()) {
      err = "truncated PNG chunk";
      return false;
    }
    const uint8_t* d = &f[pos + 8];
    std::string type((const char*)&f[pos + 4], 4);
    if (type == "IHDR" && len >= 13) {
      P.w = be32(d);
      P.h = be32(d + 4);
      P.depth = d[8];
      P.ctype = d[9];
      P.interlace = d[12];
      haveHdr = true;
    } else if (type == "PLTE") {
      P.plte.assign(d, d + len);
    } else if (type == "tRNS") {
      P.trns.assign(d, d + len);
    } else if (type == "IDAT") {
      idat.insert(idat.end(), d, d + len);
    } else if (type == "IEND") {
      break;
    }
    pos += 12 + len;
  }
  if (!haveHdr || P.w == 0 || P.h == 0 || P.w > (1u << 16) || P.h > (1u << 16)) {
    err = "bad PNG header";
    return false;
  }
  switch (P.ctype) {
    case 0: P.channels = 1; break;
    case 2: P.channels = 3; break;
    case 3: P.channels = 1; break;
    case 4: P.channels = 2; break;
    case 6: P.channels = 4; break;
    default: err = "bad PNG colour type"; return false;
  }
  const int d = P.depth;
  bool depthOk = (d == 8 || d == 16) ? P.ctype != 3 || d == 8
                                     : ((d == 1 || d == 2 || d == 4) && (P.ctype == 0 || P.ctype == 3));
  if (!depthOk || P.interlace > 1 || (P.ctype == 3 && P.plte.empty())) {
    err = "unsupported PNG bit depth, palette or interlace method";
    return false;
  }
  if (idat.size() < 2 || (idat[0] & 0x0F) != 8 || ((idat[0] << 8) | idat[1]) % 31 != 0 || (idat[1] & 0x20)) {
    err = "bad zlib header";
    return false;
  }
  std::vector<uint8_t> raw;
  if (!inflate(idat.data() + 2, idat.size() - 2, raw, err)) return false;
  const int bitsPerPixel = d * P.channels;
  const int bpp = (bitsPerPixel + 7) / 8;
  img.width = (int)P.w;
  img.height = (int)P.h;
  img.rgba.assign((size_t)P.w * P.h * 4, 0);
  // passes: (x0, y0, dx, dy); a non-interlaced image is one pass over every pixel
  const int adam[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4}, {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
  const int npass = P.interlace ? 7 : 1;
  size_t off = 0;
  std::vector<uint8_t> pix;
  std::vector<uint32_t> xs;
  for (int ps = 0; ps < npass; ps++) {
    int x0 = P.interlace ? adam[ps][0] : 0, y0 = P.interlace ? adam[ps][1] : 0;
    int dx = P.interlace ? adam[ps][2] : 1, dy = P.interlace ? adam[ps][3] : 1;
    uint32_t pw = P.w > (uint32_t)x0 ? (P.w - x0 + dx - 1) / dx : 0;
    uint32_t ph = P.h > (uint32_t)y0 ? (P.h - y0 + dy - 1) / dy : 0;
    if (pw == 0 || ph == 0) continue;
    size_t stride = ((size_t)pw * bitsPerPixel + 7) / 8;
    if (off + ph * (stride + 1) > raw.size()) {
      err = "PNG image data too short";
      return false;
    }
    if (!unfilter(raw.data() + off, ph, stride, bpp, pix)) {
      err = "bad PNG filter type";
      return false;
    }
    off += ph * (stride + 1);
    xs.resize(pw);
    for (uint32_t i = 0; i < pw; i++) xs[i] = x0 + i * dx;
    for (uint32_t y = 0; y < ph; y++)
      emitLine(P, pix.data() + y * stride, pw, img.rgba.data(), xs.data(), (size_t)(y0 + y * dy) * P.w);
  }
  return true;
}

// Binary PNM: "P5"/"P6", whitespace, width, height, maxval (comments start with '#'), one
// whitespace byte, then the samples.
bool decodePnm(const std::vector<uint8_t>& f, Image& img, std::string& err) {
  size_t pos = 2;
  auto number = [&](uint32_t& v) -> bool {
    for (;;) {
      while (pos < f.size() && (f[pos] == ' ' || f[pos] == '\t' || f[pos] == '\n' || f[pos] == '\r')) pos++;
      if (pos < f.size() && f[pos] == '#') {
        while (pos < f.size() && f[pos] != '\n') pos++;
        continue;
      }
      break;
    }
    if (pos >= f.size() || f[pos] < '0' || f[pos] > '9') return false;
    uint64_t x = 0;
    while (pos < f.size() && f[pos] >= '0' && f[pos] <= '9') {
      x = x * 10 + (f[pos++] - '0');
      if (x > 0xFFFFFFFFull) return false;
    }
    v = (uint32_t)x;
    return true;
  };
  uint32_t w, h, maxval;
  if (!number(w) || !number(h) || !number(maxval) || w == 0 || h == 0 || w > (1u << 16) || h > (1u << 16) ||
      maxval == 0 || maxval > 65535) {
    err = "bad PNM header";
    return false;
  }
  pos++;  // the single whitespace byte after maxval
  const int ch = f[1] == '6' ? 3 : 1;
  const int bytes = maxval > 255 ? 2 : 1;
  size_t need = (size_t)w * h * ch * bytes;
  if (pos + need > f.size()) {
    err = "PNM data too short";
    return false;
  }
  img.width = (int)w;
  img.height = (int)h;
  img.rgba.assign((size_t)w * h * 4, 255);
  const uint8_t* s = &f[pos];
  for (size_t i = 0; i < (size_t)w * h; i++)
    for (int c = 0; c < 3; c++) img.rgba[4 * i + c] = s[(i * ch + (ch == 3 ? c : 0)) * bytes];  // high byte first
  return true;
}

}  // namespace

bool zlibInflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, std::string& err) {
  // RFC 1950: CMF (deflate, window <= 32 KiB), FLG (check bits, no preset dictionary), the
  // deflate stream, then the Adler-32 of the data, big-endian
  if (n < 6 || (p[0] & 0x0F) != 8 || (p[0] >> 4) > 7 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20)) {
    err = "bad zlib header";
    return false;
  }
  const size_t start = out.size();
  if (!inflate(p + 2, n - 2, out, err)) return false;
  uint32_t a = 1, b = 0;
  for (size_t i = start; i < out.size(); i++) {
    a = (a + out[i]) % 65521u;
    b = (b + a) % 65521u;
  }
  const uint8_t* t = p + n - 4;
  const uint32_t want = ((uint32_t)t[0] << 24) | ((uint32_t)t[1] << 16) | ((uint32_t)t[2] << 8) | t[3];
  if (((b << 16) | a) != want) {
    err = "zlib checksum mismatch";
    return false;
  }
  return true;
}

ne_status loadRGBA8(const std::string& path, Image& img, std::string& err) {
  FILE* fp = fopen(path.c_str(), "rb");
  if (!fp) {
    err = "cannot open " + path;
    return NE_ERR_MISSING_ASSET;
  }
  std::vector<uint8_t> f;
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), fp)) > 0) f.insert(f.end(), buf, buf + n);
  fclose(fp);
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  bool ok;
  if (f.size() >= 8 && memcmp(f.data(), sig, 8) == 0) {
    ok = decodePng(f, img, err);
  } else if (f.size() >= 3 && f[0] == 'P' && (f[1] == '5' || f[1] == '6')) {
    ok = decodePnm(f, img, err);
  } else {
    err = path + ": only PNG and binary PNM (P5/P6) images are decoded";
    return NE_ERR_UNSUPPORTED;
  }
  if (!ok) {
    err = path + ": " + err;
    return NE_ERR_PARSE;
  }
  return NE_OK;
}

}  // namespace neimg

extern "C" ne_status ne_image_load_rgba8(const char* path, int32_t* width, int32_t* height, uint8_t* out,
                                         size_t cap) {
  if (!path || !width || !height) return NE_ERR_INVALID_ARG;
  neimg::Image img;
  std::string err;
  ne_status st = neimg::loadRGBA8(path, img, err);
  if (st != NE_OK) return st;
  *width = img.width;
  *height = img.height;
  if (!out) return NE_OK;
  if (cap < img.rgba.size()) return NE_ERR_INVALID_ARG;
  memcpy(out, img.rgba.data(), img.rgba.size());
  return NE_OK;
}
