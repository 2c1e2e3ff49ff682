// Image output of the render: materials/Texture.h:44-75 saveImage.
//
//  * PNG: RGB, each channel clamped to [0, 1] and converted as (uint8_t)(v * 255) like the
//    reference, 8 bits per channel. The reference writes through stb_image_write; here the
//    zlib stream uses stored (uncompressed) deflate blocks, so the file is larger but decodes
//    to the same pixels.
//  * EXR: RGB FP32 scanline image, as tinyexr's SaveEXR with FP32 output. Channels are stored
//    in the EXR's required alphabetical order (B, G, R), one scan line per block, without
//    compression.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "narval_gb300.h"

namespace {

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0) {
  c = ~c;
  for (size_t i = 0; i < n; i++) {
    c ^= p[i];
    for (int k = 0; k < 8; k++) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
  }
  return ~c;
}

void put32be(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  put32be(out, (uint32_t)data.size());
  size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  put32be(out, crc32(out.data() + start, out.size() - start));
}

template <class T>
void putLE(std::vector<uint8_t>& v, T x) {
  uint8_t b[sizeof(T)];
  memcpy(b, &x, sizeof(T));
  v.insert(v.end(), b, b + sizeof(T));  // the image formats are little endian, as every supported host
}

void attr(std::vector<uint8_t>& h, const char* name, const char* type, const std::vector<uint8_t>& value) {
  h.insert(h.end(), name, name + strlen(name) + 1);
  h.insert(h.end(), type, type + strlen(type) + 1);
  putLE<int32_t>(h, (int32_t)value.size());
  h.insert(h.end(), value.begin(), value.end());
}

bool writeFile(const char* path, const std::vector<uint8_t>& bytes) {
  FILE* f = fopen(path, "wb");
  if (!f) return false;
  bool ok = fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
  return fclose(f) == 0 && ok;
}

}  // namespace

extern "C" ne_status ne_save_png(const char* path, const float* rgb, int width, int height) {
  if (!path || !rgb || width <= 0 || height <= 0) return NE_ERR_INVALID_ARG;
  // raw scan lines: filter byte 0, then RGB bytes
  std::vector<uint8_t> raw;
  raw.reserve((size_t)height * (1 + 3 * (size_t)width));
  for (int y = 0; y < height; y++) {
    raw.push_back(0);
    for (int x = 0; x < 3 * width; x++) {
      float v = rgb[(size_t)y * 3 * width + x];
      // glm::clamp(v, 0, 1); a NaN (whose conversion is undefined in the reference) becomes 0
      v = !(v >= 0.0f) ? 0.0f : (v > 1.0f ? 1.0f : v);
      raw.push_back((uint8_t)(v * 255));
    }
  }
  // zlib stream with stored deflate blocks
  std::vector<uint8_t> z = {0x78, 0x01};
  size_t pos = 0;
  do {
    size_t n = raw.size() - pos < 65535 ? raw.size() - pos : 65535;
    z.push_back(pos + n == raw.size() ? 1 : 0);
    z.push_back((uint8_t)n);
    z.push_back((uint8_t)(n >> 8));
    z.push_back((uint8_t)~n);
    z.push_back((uint8_t)(~n >> 8));
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
    pos += n;
  } while (pos < raw.size());
  uint32_t a = 1, b = 0;
  for (uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  put32be(z, (b << 16) | a);
  std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  std::vector<uint8_t> ihdr;
  put32be(ihdr, (uint32_t)width);
  put32be(ihdr, (uint32_t)height);
  ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit, truecolour, deflate, adaptive filters, no interlace
  chunk(out, "IHDR", ihdr);
  chunk(out, "IDAT", z);
  chunk(out, "IEND", {});
  return writeFile(path, out) ? NE_OK : NE_ERR_INVALID_ARG;
}

extern "C" ne_status ne_save_exr(const char* path, const float* rgb, int width, int height) {
  if (!path || !rgb || width <= 0 || height <= 0) return NE_ERR_INVALID_ARG;
  std::vector<uint8_t> out;
  putLE<uint32_t>(out, 20000630u);  // magic
  putLE<uint32_t>(out, 2u);         // version 2, single-part scan lines
  std::vector<uint8_t> v;
  for (const char* ch : {"B", "G", "R"}) {
    v.insert(v.end(), ch, ch + 2);
    putLE<int32_t>(v, 2);  // FLOAT
    v.insert(v.end(), {0, 0, 0, 0});  // pLinear, reserved
    putLE<int32_t>(v, 1);
    putLE<int32_t>(v, 1);
  }
  v.push_back(0);
  attr(out, "channels", "chlist", v);
  attr(out, "compression", "compression", {0});
  v.clear();
  for (int32_t x : {0, 0, width - 1, height - 1}) putLE<int32_t>(v, x);
  attr(out, "dataWindow", "box2i", v);
  attr(out, "displayWindow", "box2i", v);
  attr(out, "lineOrder", "lineOrder", {0});
  v.clear();
  putLE<float>(v, 1.0f);
  attr(out, "pixelAspectRatio", "float", v);
  v.clear();
  putLE<float>(v, 0.0f);
  putLE<float>(v, 0.0f);
  attr(out, "screenWindowCenter", "v2f", v);
  v.clear();
  putLE<float>(v, 1.0f);
  attr(out, "screenWindowWidth", "float", v);
  out.push_back(0);  // end of header
  const uint64_t lineBytes = 4 + 4 + 3 * 4 * (uint64_t)width;
  uint64_t offset = out.size() + 8 * (uint64_t)height;
  for (int y = 0; y < height; y++) putLE<uint64_t>(out, offset + lineBytes * (uint64_t)y);
  for (int y = 0; y < height; y++) {
    putLE<int32_t>(out, y);
    putLE<int32_t>(out, 3 * 4 * width);
    for (int c : {2, 1, 0})
      for (int x = 0; x < width; x++) putLE<float>(out, rgb[((size_t)y * width + x) * 3 + c]);
  }
  return writeFile(path, out) ? NE_OK : NE_ERR_INVALID_ARG;
}
