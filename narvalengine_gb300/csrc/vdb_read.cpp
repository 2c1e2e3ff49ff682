// OpenVDB files for grid media (vdb_read.h). The layout is that of OpenVDB 6.2 (file formats
// 222-224), the library the reference links (core/ResourceManager.cpp:165-218):
//
//  * header (io/Archive.cc readHeader): int64 magic 0x56444220, uint32 format, uint32 library
//    major and minor, a byte "has grid offsets", the UUID as 36 characters, the file's metadata;
//    int32 grid count, then per grid a descriptor (io/GridDescriptor.cc read): unique name
//    (name, optionally "\x1e" and an index), type (suffix "_HalfFloat" when values are stored as
//    half floats), instance parent, int64 grid / block / end positions;
//  * a grid (io/Archive.cc readGrid): uint32 compression flags (zip 1, active mask 2, Blosc 4),
//    metadata, the transform (math/Transform.cc, math/Maps.h: a map type name and its doubles),
//    the tree's topology, then its buffers;
//  * metadata (MetaMap.cc readMeta): uint32 count, per entry name, type name, uint32 size, bytes;
//    strings are a uint32 length and the characters;
//  * topology (tree/Tree.h, RootNode.h, InternalNode.h, LeafNode.h readTopology): int32 buffer
//    count, the root's background (float), uint32 tile and child counts, tiles (int32 x3 origin,
//    float value, byte active), children (origin, then the 32^3 node); a 32^3 or 16^3 internal
//    node: child mask, value mask (bit i of 64-bit word i / 64), its values (below), its children
//    in index order; a leaf (8^3): its value mask;
//  * buffers (readBuffers): for every leaf, depth first with the root's children in coordinate
//    order: the value mask again (the topology's copy is the one used), then its 512 values;
//  * values (io/Compression.h readCompressedValues): a metadata byte m; inactive value 0 is the
//    background for m = 0, else minus the background, inactive value 1 the background; m = 2, 4
//    or 5 store inactive value 0 (float), m = 5 also inactive value 1; m = 3, 4 or 5 store a
//    selection mask; with active-mask compression and m != 6 only the active values are stored
//    and each inactive one is restored as inactive value 1 where the selection mask is on, else
//    inactive value 0; values are floats, or half floats in a "_HalfFloat" grid;
//  * data (io/Compression.cc): with zip an int64 n, then n bytes of a zlib stream (n <= 0: -n raw
//    bytes); with Blosc the same with a Blosc frame (LZ4 streams, byte shuffle); else raw bytes.
//
// The files are read as little-endian, as every machine this library builds for is.
#include "vdb_read.h"

#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <map>
#include <vector>

#include "image_load.h"

namespace nevdb {
namespace {

constexpr int64_t kMagic = 0x56444220;
constexpr uint32_t kZip = 0x1, kActiveMask = 0x2, kBlosc = 0x4;

struct Fail {
  ne_status st;
  std::string msg;
};
[[noreturn]] void corrupt(const std::string& why) { throw Fail{NE_ERR_PARSE, why}; }

struct In {
  const uint8_t* p;
  size_t n, pos;
  void need(size_t k) const {
    if (k > n - pos) corrupt("truncated file");
  }
  template <class T>
  T get() {
    need(sizeof(T));
    T v;
    memcpy(&v, p + pos, sizeof(T));
    pos += sizeof(T);
    return v;
  }
  const uint8_t* take(size_t k) {
    need(k);
    const uint8_t* q = p + pos;
    pos += k;
    return q;
  }
  std::string str() {
    const uint32_t k = get<uint32_t>();
    const uint8_t* q = take(k);
    return std::string(reinterpret_cast<const char*>(q), k);
  }
  void seek(int64_t at) {
    if (at < 0 || (uint64_t)at > n) corrupt("stream position outside the file");
    pos = (size_t)at;
  }
};

// A name from the file for an error message: printable ASCII, the rest as '?'.
std::string printable(const std::string& s) {
  std::string out = s.substr(0, 64);
  for (char& ch : out)
    if ((unsigned char)ch < 0x20 || (unsigned char)ch > 0x7E) ch = '?';
  return out;
}

uint32_t le32(const uint8_t* q) {
  return (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24);
}

struct Mask {
  std::vector<uint64_t> w;
  void load(In& in, uint32_t bits) {
    w.resize(bits / 64);
    memcpy(w.data(), in.take(bits / 8), bits / 8);
  }
  bool on(uint32_t i) const { return !w.empty() && ((w[i >> 6] >> (i & 63u)) & 1u); }
  uint32_t count() const {
    uint32_t c = 0;
    for (uint64_t x : w) c += (uint32_t)__builtin_popcountll(x);
    return c;
  }
};

// IEEE binary16 -> binary32 (exact).
float halfToFloat(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu, bits;
  if (e == 0) {
    if (m == 0) {
      bits = sign;
    } else {  // subnormal: normalise the mantissa
      int shift = 0;
      while (!(m & 0x400u)) {
        m <<= 1;
        shift++;
      }
      bits = sign | ((uint32_t)(127 - 15 + 1 - shift) << 23) | ((m & 0x3FFu) << 13);
    }
  } else if (e == 31) {
    bits = sign | 0x7F800000u | (m << 13);
  } else {
    bits = sign | ((e - 15 + 127) << 23) | (m << 13);
  }
  float f;
  memcpy(&f, &bits, 4);
  return f;
}

// LZ4 block format: sequences of a token (literal count, match length - 4), literals, a 16-bit
// offset and the match; the last sequence has literals only. Returns the bytes written.
size_t lz4Decode(const uint8_t* src, size_t n, uint8_t* dst, size_t cap) {
  size_t ip = 0, op = 0;
  while (ip < n) {
    const uint8_t token = src[ip++];
    size_t lit = token >> 4;
    if (lit == 15) {
      uint8_t b;
      do {
        if (ip >= n) corrupt("truncated LZ4 stream");
        b = src[ip++];
        lit += b;
      } while (b == 255);
    }
    if (lit > n - ip || lit > cap - op) corrupt("corrupt LZ4 literals");
    memcpy(dst + op, src + ip, lit);
    ip += lit;
    op += lit;
    if (ip >= n) break;
    if (n - ip < 2) corrupt("truncated LZ4 offset");
    const size_t off = (size_t)src[ip] | ((size_t)src[ip + 1] << 8);
    ip += 2;
    if (off == 0 || off > op) corrupt("corrupt LZ4 offset");
    size_t len = token & 15u;
    if (len == 15) {
      uint8_t b;
      do {
        if (ip >= n) corrupt("truncated LZ4 stream");
        b = src[ip++];
        len += b;
      } while (b == 255);
    }
    len += 4;
    if (len > cap - op) corrupt("corrupt LZ4 match");
    for (size_t k = 0; k < len; k++, op++) dst[op] = dst[op - off];  // may overlap its source
  }
  return op;
}

// One Blosc (version 1) frame of `want` bytes: a 16-byte header (flags: 1 byte shuffle, 2 stored
// uncompressed, 4 bit shuffle, 16 blocks not split, codec in bits 5-7, 1 = LZ4; type size,
// uncompressed size, block size, frame size), the blocks' start offsets, then per block its
// streams (one, or one per byte of the type), each an int32 size and its bytes (stored raw when
// the size equals the stream's).
void bloscDecode(const uint8_t* b, size_t n, size_t want, uint8_t* out) {
  if (n < 16) corrupt("truncated Blosc frame");
  const uint8_t flags = b[2];
  const uint32_t typesize = b[3], nbytes = le32(b + 4), blocksize = le32(b + 8), cbytes = le32(b + 12);
  if (nbytes != want || cbytes > n) corrupt("Blosc frame of an unexpected size");
  if (flags & 0x02) {
    if (16 + (size_t)nbytes > n) corrupt("truncated Blosc frame");
    memcpy(out, b + 16, nbytes);
    return;
  }
  if ((flags >> 5) != 1) throw Fail{NE_ERR_UNSUPPORTED, "Blosc codec other than LZ4"};
  if (flags & 0x04) throw Fail{NE_ERR_UNSUPPORTED, "Blosc bit shuffle"};
  if (nbytes == 0) return;
  if (blocksize == 0 || blocksize > nbytes || typesize == 0) corrupt("corrupt Blosc header");
  const uint32_t nblocks = nbytes / blocksize + (nbytes % blocksize ? 1u : 0u);
  if (16 + (size_t)nblocks * 4 > n) corrupt("truncated Blosc frame");
  std::vector<uint8_t> tmp(blocksize);
  for (uint32_t j = 0; j < nblocks; j++) {
    const bool leftover = (j == nblocks - 1) && (nbytes % blocksize != 0);
    const uint32_t bsize = leftover ? nbytes % blocksize : blocksize;
    const uint32_t nsplit =
        (!(flags & 0x10) && typesize <= 16 && bsize / typesize >= 128 && !leftover) ? typesize : 1u;
    if (bsize % nsplit) corrupt("corrupt Blosc block");
    const uint32_t neblock = bsize / nsplit;
    size_t at = le32(b + 16 + 4 * (size_t)j);
    for (uint32_t s = 0; s < nsplit; s++) {
      if (at + 4 > n) corrupt("truncated Blosc block");
      const int32_t cs = (int32_t)le32(b + at);
      at += 4;
      if (cs < 0 || (size_t)cs > n - at) corrupt("corrupt Blosc stream size");
      if ((uint32_t)cs == neblock)
        memcpy(tmp.data() + (size_t)s * neblock, b + at, neblock);
      else if (lz4Decode(b + at, (size_t)cs, tmp.data() + (size_t)s * neblock, neblock) != neblock)
        corrupt("LZ4 stream of an unexpected size");
      at += (size_t)cs;
    }
    uint8_t* dst = out + (size_t)j * blocksize;
    if ((flags & 0x01) && typesize > 1) {  // byte j of element i was stored at j * count + i
      const uint32_t count = bsize / typesize;
      for (uint32_t i = 0; i < count; i++)
        for (uint32_t k = 0; k < typesize; k++) dst[(size_t)i * typesize + k] = tmp[(size_t)k * count + i];
      memcpy(dst + (size_t)count * typesize, tmp.data() + (size_t)count * typesize, bsize - count * typesize);
    } else {
      memcpy(dst, tmp.data(), bsize);
    }
  }
}

// `bytes` of data under the grid's compression (io::readData).
void copyBytes(uint8_t* out, const uint8_t* src, size_t bytes) {
  if (bytes) memcpy(out, src, bytes);  // an empty destination may be a null pointer
}

void readData(In& in, uint32_t comp, size_t bytes, uint8_t* out) {
  if (!(comp & (kZip | kBlosc))) {
    copyBytes(out, in.take(bytes), bytes);
    return;
  }
  const int64_t nz = in.get<int64_t>();
  if (nz <= 0) {  // stored uncompressed: -nz bytes (without negating INT64_MIN)
    if ((uint64_t)0 - (uint64_t)nz != bytes) corrupt("raw chunk of an unexpected size");
    copyBytes(out, in.take(bytes), bytes);
    return;
  }
  const uint8_t* z = in.take((size_t)nz);
  if (comp & kBlosc) {
    bloscDecode(z, (size_t)nz, bytes, out);
    return;
  }
  std::vector<uint8_t> o;
  o.reserve(bytes);
  std::string e;
  if (!neimg::zlibInflate(z, (size_t)nz, o, e)) corrupt("zip chunk: " + e);
  if (o.size() != bytes) corrupt("zip chunk of an unexpected size");
  copyBytes(out, o.data(), bytes);
}

struct Codec {
  uint32_t comp;
  bool half;
  float background;
};

// `count` values of a node (io::readCompressedValues), inactive ones restored.
void readValues(In& in, const Codec& c, float* dest, uint32_t count, const Mask& valueMask) {
  const int8_t meta = in.get<int8_t>();
  float in1 = c.background, in0 = (meta == 0) ? c.background : -c.background;
  if (meta == 2 || meta == 4 || meta == 5) {
    in0 = in.get<float>();
    if (meta == 5) in1 = in.get<float>();
  }
  Mask sel;
  if (meta == 3 || meta == 4 || meta == 5) sel.load(in, count);
  const bool maskComp = (c.comp & kActiveMask) != 0;
  const uint32_t stored = (maskComp && meta != 6) ? valueMask.count() : count;
  std::vector<float> tmp(stored);
  if (c.half) {
    if (stored > 0) {  // half floats, converted
      std::vector<uint16_t> h(stored);
      readData(in, c.comp, 2 * (size_t)stored, reinterpret_cast<uint8_t*>(h.data()));
      for (uint32_t i = 0; i < stored; i++) tmp[i] = halfToFloat(h[i]);
    }
  } else {
    readData(in, c.comp, 4 * (size_t)stored, reinterpret_cast<uint8_t*>(tmp.data()));
  }
  if (maskComp && stored != count) {
    for (uint32_t d = 0, t = 0; d < count; d++) dest[d] = valueMask.on(d) ? tmp[t++] : (sel.on(d) ? in1 : in0);
  } else {
    memcpy(dest, tmp.data(), 4 * (size_t)count);
  }
}

using Key = std::array<int32_t, 3>;  // ordered as OpenVDB's Coord: x, then y, then z

struct Leaf {
  Key o;
  Mask vm;
  float v[512];
};
// An internal node of 2^(3 log2) entries, each a child (`kid`) or a tile value.
struct Inner {
  Key o;
  Mask cm, vm;
  std::vector<float> tile;
  std::vector<int32_t> kid;
};
struct RootEntry {
  int32_t child = -1;  // index into Tree::n5
  float value = 0;
  bool active = false;
};
struct Tree {
  float background = 0;
  std::map<Key, RootEntry> root;
  std::vector<Inner> n5, n4;
  std::vector<Leaf> leaves;
};

// Offset i of a node with 2^log2 entries per axis -> its entry's origin, children of `childTotal`
// log2 voxels per axis.
Key entryOrigin(const Key& o, uint32_t i, int log2, int childTotal) {
  const uint32_t m = (1u << log2) - 1u;
  return Key{o[0] + (int32_t)((i >> (2 * log2)) << childTotal), o[1] + (int32_t)(((i >> log2) & m) << childTotal),
             o[2] + (int32_t)((i & m) << childTotal)};
}

int32_t readInner(In& in, const Codec& c, Tree& t, const Key& o, int log2) {
  const uint32_t size = 1u << (3 * log2);
  Inner nd;
  // the node's origin is its first voxel (InternalNode's constructor clears the low bits)
  const int32_t low = (1 << (log2 == 5 ? 12 : 7)) - 1;
  nd.o = Key{o[0] & ~low, o[1] & ~low, o[2] & ~low};
  nd.cm.load(in, size);
  nd.vm.load(in, size);
  nd.tile.resize(size);
  readValues(in, c, nd.tile.data(), size, nd.vm);
  nd.kid.assign(size, -1);
  std::vector<Inner>& pool = log2 == 5 ? t.n5 : t.n4;
  const int32_t idx = (int32_t)pool.size();
  pool.push_back(std::move(nd));
  for (uint32_t i = 0; i < size; i++) {
    if (!pool[idx].cm.on(i)) continue;
    int32_t k;
    if (log2 == 5) {
      k = readInner(in, c, t, entryOrigin(pool[idx].o, i, 5, 7), 4);
    } else {
      Leaf lf;
      lf.o = entryOrigin(pool[idx].o, i, 4, 3);
      lf.vm.load(in, 512);
      k = (int32_t)t.leaves.size();
      t.leaves.push_back(std::move(lf));
    }
    std::vector<Inner>& again = log2 == 5 ? t.n5 : t.n4;  // the recursion may have moved `pool`
    again[idx].kid[i] = k;
  }
  return idx;
}

void readBuffers(In& in, const Codec& c, Tree& t) {
  for (const auto& kv : t.root) {
    if (kv.second.child < 0) continue;
    const Inner& a = t.n5[kv.second.child];
    for (uint32_t i = 0; i < 32768; i++) {
      if (!a.cm.on(i)) continue;
      const Inner& b = t.n4[a.kid[i]];
      for (uint32_t j = 0; j < 4096; j++) {
        if (!b.cm.on(j)) continue;
        Leaf& lf = t.leaves[b.kid[j]];
        in.take(64);  // the value mask again
        readValues(in, c, lf.v, 512, lf.vm);
      }
    }
  }
}

void skipMeta(In& in) {
  const uint32_t count = in.get<uint32_t>();
  for (uint32_t i = 0; i < count; i++) {
    in.str();
    in.str();
    in.take(in.get<uint32_t>());
  }
}

// math/Maps.h read(): the doubles each map type stores.
void skipMap(In& in, const std::string& type, bool nested) {
  if (type == "AffineMap" || type == "UnitaryMap") {
    in.take(16 * 8);
  } else if (type == "ScaleMap" || type == "UniformScaleMap") {
    in.take(15 * 8);
  } else if (type == "TranslationMap") {
    in.take(3 * 8);
  } else if (type == "ScaleTranslateMap" || type == "UniformScaleTranslateMap") {
    in.take(18 * 8);
  } else if (type == "NonlinearFrustumMap" && !nested) {  // box, taper, depth, then an affine map
    in.take(8 * 8);
    skipMap(in, in.str(), true);
  } else {
    throw Fail{NE_ERR_UNSUPPORTED, "VDB transform " + printable(type)};
  }
}

Tree readGrid(In& in, bool half) {
  Tree t;
  const uint32_t comp = in.get<uint32_t>();
  skipMeta(in);
  skipMap(in, in.str(), false);
  in.get<int32_t>();  // buffer count (1)
  t.background = in.get<float>();
  const Codec c{comp, half, t.background};
  const uint32_t ntiles = in.get<uint32_t>(), nchildren = in.get<uint32_t>();
  for (uint32_t i = 0; i < ntiles; i++) {
    Key o{in.get<int32_t>(), in.get<int32_t>(), in.get<int32_t>()};
    RootEntry e;
    e.value = in.get<float>();
    e.active = in.get<uint8_t>() != 0;
    t.root[o] = e;
  }
  for (uint32_t i = 0; i < nchildren; i++) {
    Key o{in.get<int32_t>(), in.get<int32_t>(), in.get<int32_t>()};
    RootEntry e;
    e.child = readInner(in, c, t, o, 5);
    t.root[o] = e;
  }
  readBuffers(in, c, t);
  return t;
}

struct Box {
  bool any = false;
  int64_t lo[3], hi[3];
  void expand(const Key& p, int64_t dim) {
    for (int a = 0; a < 3; a++) {
      lo[a] = any ? std::min<int64_t>(lo[a], p[a]) : p[a];
      hi[a] = any ? std::max<int64_t>(hi[a], p[a] + dim - 1) : p[a] + dim - 1;
    }
    any = true;
  }
};

// Tree::evalActiveVoxelBoundingBox: active tiles with their whole extent, active leaf voxels.
Box activeBox(const Tree& t) {
  Box b;
  for (const auto& kv : t.root) {
    if (kv.second.child < 0) {
      if (kv.second.active) b.expand(kv.first, 4096);
      continue;
    }
    const Inner& a = t.n5[kv.second.child];
    for (uint32_t i = 0; i < 32768; i++) {
      if (!a.cm.on(i)) {
        if (a.vm.on(i)) b.expand(entryOrigin(a.o, i, 5, 7), 128);
        continue;
      }
      const Inner& c = t.n4[a.kid[i]];
      for (uint32_t j = 0; j < 4096; j++) {
        if (!c.cm.on(j)) {
          if (c.vm.on(j)) b.expand(entryOrigin(c.o, j, 4, 3), 8);
          continue;
        }
        const Leaf& lf = t.leaves[c.kid[j]];
        for (uint32_t k = 0; k < 512; k++)
          if (lf.vm.on(k)) b.expand(entryOrigin(lf.o, k, 3, 0), 1);
      }
    }
  }
  return b;
}

// The dense box [org, org + dim) filled with the tree's values (tools::copyToDense): the
// background, then each root tile, internal tile and leaf painted over its part of the box.
struct Dense {
  int64_t org[3], dim[3];
  std::vector<float> v;
  void paint(const Key& p, int64_t size, float value) {
    int64_t a[3], b[3];
    for (int k = 0; k < 3; k++) {
      a[k] = std::max<int64_t>(p[k], org[k]);
      b[k] = std::min<int64_t>(p[k] + size, org[k] + dim[k]);
      if (a[k] >= b[k]) return;
    }
    for (int64_t x = a[0]; x < b[0]; x++)
      for (int64_t y = a[1]; y < b[1]; y++) {
        float* row = v.data() + ((x - org[0]) * dim[1] + (y - org[1])) * dim[2];
        for (int64_t z = a[2]; z < b[2]; z++) row[z - org[2]] = value;
      }
  }
  // A leaf's 8^3 values (x-major, z fastest) over its part of the box.
  void copyLeaf(const Key& p, const float* vals) {
    int64_t a[3], b[3];
    for (int k = 0; k < 3; k++) {
      a[k] = std::max<int64_t>(p[k], org[k]);
      b[k] = std::min<int64_t>(p[k] + 8, org[k] + dim[k]);
      if (a[k] >= b[k]) return;
    }
    for (int64_t x = a[0]; x < b[0]; x++)
      for (int64_t y = a[1]; y < b[1]; y++) {
        float* row = v.data() + ((x - org[0]) * dim[1] + (y - org[1])) * dim[2];
        const float* src = vals + ((x - p[0]) << 6) + ((y - p[1]) << 3);
        for (int64_t z = a[2]; z < b[2]; z++) row[z - org[2]] = src[z - p[2]];
      }
  }
};

void fillDense(const Tree& t, Dense& d) {
  d.v.assign((size_t)(d.dim[0] * d.dim[1] * d.dim[2]), t.background);
  for (const auto& kv : t.root) {
    const Key& key = kv.first;
    if ((key[0] & 4095) || (key[1] & 4095) || (key[2] & 4095)) continue;  // no lookup reaches it
    if (kv.second.child < 0) {
      d.paint(key, 4096, kv.second.value);
      continue;
    }
    const Inner& a = t.n5[kv.second.child];
    for (uint32_t i = 0; i < 32768; i++) {
      const Key oi = entryOrigin(a.o, i, 5, 7);
      if (!a.cm.on(i)) {
        d.paint(oi, 128, a.tile[i]);
        continue;
      }
      const Inner& c = t.n4[a.kid[i]];
      for (uint32_t j = 0; j < 4096; j++) {
        const Key oj = entryOrigin(c.o, j, 4, 3);
        if (!c.cm.on(j)) {
          d.paint(oj, 8, c.tile[j]);
          continue;
        }
        const Leaf& lf = t.leaves[c.kid[j]];
        d.copyLeaf(lf.o, lf.v);
      }
    }
  }
}

void load(const uint8_t* data, size_t n, uint32_t res[3], std::vector<float>& grid) {
  In in{data, n, 0};
  if (in.get<int64_t>() != kMagic) corrupt("not a VDB file");
  const uint32_t version = in.get<uint32_t>();
  if (version < 222) throw Fail{NE_ERR_UNSUPPORTED, "VDB file format " + std::to_string(version) + " (before 222)"};
  in.take(8);  // library version
  const bool offsets = in.get<uint8_t>() != 0;
  in.take(36);  // UUID
  skipMeta(in);
  const int32_t count = in.get<int32_t>();
  for (int32_t g = 0; g < count; g++) {
    const std::string unique = in.str();
    std::string type = in.str();
    const std::string parent = in.str();
    const int64_t gridPos = in.get<int64_t>();
    in.get<int64_t>();  // block position
    const int64_t endPos = in.get<int64_t>();
    const std::string name = unique.substr(0, unique.find('\x1e'));
    const std::string halfSuffix = "_HalfFloat";
    bool half = false;
    if (type.size() >= halfSuffix.size() && type.compare(type.size() - halfSuffix.size(), halfSuffix.size(), halfSuffix) == 0) {
      half = true;
      type.resize(type.size() - halfSuffix.size());
    }
    const bool isFloat = type == "Tree_float_5_4_3";
    if (name != "density") {
      if (offsets) {
        in.seek(endPos);
      } else if (isFloat && parent.empty()) {
        readGrid(in, half);  // read through to the next descriptor
      } else {
        throw Fail{NE_ERR_UNSUPPORTED, "VDB stream without grid offsets holding a " + printable(type) + " grid"};
      }
      continue;
    }
    if (!isFloat) throw Fail{NE_ERR_UNSUPPORTED, "density grid of type " + printable(type) + " (not a float grid)"};
    if (!parent.empty()) throw Fail{NE_ERR_UNSUPPORTED, "density grid instanced from " + printable(parent)};
    if (offsets) in.seek(gridPos);
    const Tree t = readGrid(in, half);
    const Box b = activeBox(t);
    if (!b.any) corrupt("the density grid has no active voxels");
    // ResourceManager.cpp:186-205: |min| + |max| voxels (one more across 0) from -|min|
    Dense d;
    int64_t total = 1;
    for (int a = 0; a < 3; a++) {
      const int64_t lo = b.lo[a], hi = b.hi[a];
      d.dim[a] = (lo < 0 ? -lo : lo) + (hi < 0 ? -hi : hi) + ((lo < 0 && hi >= 0) ? 1 : 0);
      d.org[a] = -(lo < 0 ? -lo : lo);
      if (d.dim[a] <= 0) corrupt("the dense box of the density grid is empty");
      total *= d.dim[a];
      if (total * 4 > INT32_MAX) throw Fail{NE_ERR_UNSUPPORTED, "dense density grid of 2 GiB or more"};
    }
    fillDense(t, d);
    res[0] = (uint32_t)d.dim[2];
    res[1] = (uint32_t)d.dim[1];
    res[2] = (uint32_t)d.dim[0];
    grid.swap(d.v);
    return;
  }
  corrupt("no grid named density");
}

}  // namespace

ne_status loadDensity(const std::string& path, uint32_t res[3], std::vector<float>& grid, std::string& err) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) {
    err = "Couldn't read the file at " + path + ".";
    return NE_ERR_MISSING_ASSET;
  }
  std::vector<uint8_t> bytes;
  uint8_t buf[1 << 16];
  size_t k;
  while ((k = fread(buf, 1, sizeof(buf), f)) > 0) bytes.insert(bytes.end(), buf, buf + k);
  fclose(f);
  try {
    load(bytes.data(), bytes.size(), res, grid);
  } catch (const Fail& e) {
    err = "VDB " + path + ": " + e.msg;
    return e.st;
  }
  return NE_OK;
}

}  // namespace nevdb
