// Texture image decoding (image_load.cpp): 8-bit RGBA as the reference's stbi_load(..., 4).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "narval_gb300.h"

namespace neimg {

struct Image {
  int width = 0, height = 0;
  std::vector<uint8_t> rgba;  // width * height * 4, row-major from the top row
};

// NE_ERR_MISSING_ASSET if the file cannot be read, NE_ERR_UNSUPPORTED for formats other
// than PNG and binary PNM, NE_ERR_PARSE for a corrupt file; `err` says which.
ne_status loadRGBA8(const std::string& path, Image& img, std::string& err);

// Appends the data of a zlib stream (RFC 1950: header, deflate blocks, Adler-32) to `out`;
// false with `err` set if the stream is corrupt or its checksum does not match.
bool zlibInflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, std::string& err);

}  // namespace neimg
