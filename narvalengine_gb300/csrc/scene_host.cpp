// Host side of the scene interface: the reference's JSON scene descriptor turned into
// the flat ne_scene_desc that ne_scene_upload copies to the device.
//
// Follows io/SceneReader.cpp (loadScene :10-54, processMaterial :67-222,
// processPrimitives :224-648, processCameraAndRenderer :650-675), core/Camera.cpp:7-26,
// utils/Math.h:848-859 (getTransform), core/ResourceManager.cpp:222-288 (.vol grids) and
// core/ResourceManager.cpp:165-218 (.vdb grids, read by vdb_read.cpp).
// Instead of aborting with LOG(FATAL) on a malformed scene it returns NE_ERR_PARSE or
// NE_ERR_MISSING_ASSET with a message.
//
// Extensions of the descriptor (not in the reference; every one is opt-in):
//  * material "volume": "grid": {"generator": "fbm", ...} builds the density grid from
//    seeded simplex fBm; "grid": {"path": "x.f32", "resolution": [W,H,D]} reads raw
//    little-endian float32 voxels.
//  * material "infiniteAreaLight": "radiance": [r,g,b] (instead of "path") is a constant
//    environment, i.e. the reference's InfiniteAreaLight over a 1x1 map of that value. A
//    "path" texture is decoded by image_load.cpp (PNG, binary PNM).
//  * primitive "obj": read from the OBJ file directly (positions and faces) instead of through
//    assimp, with the JSON materialName; primitives naming the same file and material share
//    one model (one BVH), each with its own transform.
//  * primitive "mesh": a triangle mesh given inline ("positions", "indices") or by the
//    "icosphere" generator, loaded as the reference loads an obj/gltf model (bounding
//    box and BVH); optional "groups" assign seeded GGX materials per triangle group.
//  * renderer "rr": {"after": n} enables Russian roulette after bounce n.
//  * renderer "bvh": "sah" builds mesh BVHs with the GPU binned-SAH builder ("reference", the
//    default: BVH::init's midpoint build).
// Elementary functions come from ne_fmath.h so that the same descriptor yields the
// same matrices on x86-64 and aarch64 hosts.

#include <ctype.h>
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>
#include <map>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "narval_gb300.h"
#include "image_load.h"
#include "ne_fmath.h"
#include "scene_gen.h"
#include "vdb_read.h"

namespace {

// ---------------------------------------------------------------- minimal JSON
struct JVal {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  bool b = false;
  double num = 0;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;
  const JVal* get(const char* k) const {
    if (kind != OBJ) return nullptr;
    for (auto& kv : obj)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
};

struct ParseError : std::runtime_error {
  int code;
  ParseError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

struct JParser {
  const char* p;
  const char* end;
  int depth = 0;  // open objects and arrays; the recursion stops at kMaxDepth
  static constexpr int kMaxDepth = 256;
  void ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
  }
  [[noreturn]] void fail(const char* what) { throw ParseError(NE_ERR_PARSE, std::string("malformed json: ") + what); }
  JVal parse() {
    ws();
    if (p >= end) fail("unexpected end");
    JVal v;
    char c = *p;
    if ((c == '{' || c == '[') && depth >= kMaxDepth) fail("nesting too deep");
    struct Level {
      int& d;
      explicit Level(int& x) : d(++x) {}
      ~Level() { d--; }
    } level(depth);
    if (c == '{') {
      v.kind = JVal::OBJ;
      p++;
      ws();
      if (p < end && *p == '}') { p++; return v; }
      for (;;) {
        ws();
        if (p >= end || *p != '"') fail("expected key");
        std::string k = str();
        ws();
        if (p >= end || *p != ':') fail("expected ':'");
        p++;
        JVal x = parse();
        v.obj.emplace_back(k, std::move(x));
        ws();
        if (p < end && *p == ',') { p++; continue; }
        if (p < end && *p == '}') { p++; break; }
        fail("expected ',' or '}'");
      }
    } else if (c == '[') {
      v.kind = JVal::ARR;
      p++;
      ws();
      if (p < end && *p == ']') { p++; return v; }
      for (;;) {
        v.arr.push_back(parse());
        ws();
        if (p < end && *p == ',') { p++; continue; }
        if (p < end && *p == ']') { p++; break; }
        fail("expected ',' or ']'");
      }
    } else if (c == '"') {
      v.kind = JVal::STR;
      v.str = str();
    } else if (c == 't' && end - p >= 4 && !strncmp(p, "true", 4)) {
      v.kind = JVal::BOOL; v.b = true; p += 4;
    } else if (c == 'f' && end - p >= 5 && !strncmp(p, "false", 5)) {
      v.kind = JVal::BOOL; v.b = false; p += 5;
    } else if (c == 'n' && end - p >= 4 && !strncmp(p, "null", 4)) {
      p += 4;
    } else {
      // a JSON number: -?(0|[1-9][0-9]*)(.[0-9]+)?([eE][+-]?[0-9]+)? (no NaN, infinity, hex or
      // leading '+', which a JSON reader rejects); an integer literal is an integer, so "-0"
      // is the integer 0, read as +0.0 (a fraction or exponent makes it a double: "-0.0")
      const char* q = p;
      bool integer = true;
      auto digit = [&](const char* r) { return r < end && *r >= '0' && *r <= '9'; };
      if (q < end && *q == '-') q++;
      if (!digit(q)) fail("bad value");
      if (*q == '0') {
        q++;
      } else {
        while (digit(q)) q++;
      }
      if (q < end && *q == '.') {
        integer = false;
        q++;
        if (!digit(q)) fail("bad number");
        while (digit(q)) q++;
      }
      if (q < end && (*q == 'e' || *q == 'E')) {
        integer = false;
        q++;
        if (q < end && (*q == '+' || *q == '-')) q++;
        if (!digit(q)) fail("bad number");
        while (digit(q)) q++;
      }
      const std::string token(p, q);
      v.num = strtod(token.c_str(), nullptr);
      if (integer && v.num == 0.0) v.num = 0.0;
      v.kind = JVal::NUM;
      p = q;
    }
    return v;
  }
  // A JSON string: the escapes \" \\ \/ \b \f \n \r \t and \uXXXX (a surrogate pair for
  // one code point above U+FFFF), stored as UTF-8; an unescaped control character or any other
  // escape is an error, as a JSON reader has it.
  uint32_t hex4() {
    if (end - p < 4) fail("bad escape");
    uint32_t u = 0;
    for (int k = 0; k < 4; k++, p++) {
      const char ch = *p;
      const int d = ch >= '0' && ch <= '9' ? ch - '0' : ch >= 'a' && ch <= 'f' ? ch - 'a' + 10
                  : ch >= 'A' && ch <= 'F' ? ch - 'A' + 10 : -1;
      if (d < 0) fail("bad escape");
      u = u * 16 + (uint32_t)d;
    }
    return u;
  }
  static void utf8(std::string& s, uint32_t u) {
    if (u < 0x80) {
      s.push_back((char)u);
    } else if (u < 0x800) {
      s.push_back((char)(0xC0 | (u >> 6)));
      s.push_back((char)(0x80 | (u & 0x3F)));
    } else if (u < 0x10000) {
      s.push_back((char)(0xE0 | (u >> 12)));
      s.push_back((char)(0x80 | ((u >> 6) & 0x3F)));
      s.push_back((char)(0x80 | (u & 0x3F)));
    } else {
      s.push_back((char)(0xF0 | (u >> 18)));
      s.push_back((char)(0x80 | ((u >> 12) & 0x3F)));
      s.push_back((char)(0x80 | ((u >> 6) & 0x3F)));
      s.push_back((char)(0x80 | (u & 0x3F)));
    }
  }
  std::string str() {
    std::string s;
    p++;
    while (p < end && *p != '"') {
      if ((unsigned char)*p < 0x20) fail("control character in a string");
      if (*p != '\\') {
        s.push_back(*p++);
        continue;
      }
      if (++p >= end) break;
      const char e = *p++;
      switch (e) {
        case '"': case '\\': case '/': s.push_back(e); break;
        case 'b': s.push_back('\b'); break;
        case 'f': s.push_back('\f'); break;
        case 'n': s.push_back('\n'); break;
        case 'r': s.push_back('\r'); break;
        case 't': s.push_back('\t'); break;
        case 'u': {
          uint32_t u = hex4();
          if (u >= 0xD800 && u < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
            const char* save = p;
            p += 2;
            const uint32_t lo = hex4();
            if (lo >= 0xDC00 && lo < 0xE000)
              u = 0x10000 + ((u - 0xD800) << 10) + (lo - 0xDC00);
            else
              p = save;  // a lone high surrogate, then another escape
          }
          utf8(s, u);
          break;
        }
        default: fail("bad escape");
      }
    }
    if (p >= end) fail("unterminated string");
    p++;
    return s;
  }
};

const JVal& need(const JVal& o, const char* k, const std::string& ctx) {
  const JVal* v = o.get(k);
  if (!v) throw ParseError(NE_ERR_PARSE, ctx + " is missing the property " + k + ".");
  return *v;
}
float num(const JVal& v, const std::string& ctx) {
  if (v.kind == JVal::NUM) return (float)v.num;
  if (v.kind == JVal::BOOL) return v.b ? 1.0f : 0.0f;
  throw ParseError(NE_ERR_PARSE, ctx + " is not a number.");
}
// A whole-number field: a number in [lo, hi], truncated toward zero as the reference's int
// conversions do; anything else (out of range, not finite) is a parse error rather than an
// undefined conversion.
int64_t wholeIn(double v, double lo, double hi, const std::string& what) {
  if (!(v >= lo && v < hi + 1.0)) throw ParseError(NE_ERR_PARSE, what + " is out of range.");
  return (int64_t)v;
}
std::string sval(const JVal& v, const std::string& ctx) {
  if (v.kind != JVal::STR) throw ParseError(NE_ERR_PARSE, ctx + " is not a string.");
  return v.str;
}
// SceneReader::getVec3 (:60-65): reads up to three components.
void vec3(const JVal& v, float* out, const std::string& ctx) {
  if (v.kind != JVal::ARR) throw ParseError(NE_ERR_PARSE, ctx + " is not an array.");
  for (size_t i = 0; i < v.arr.size() && i < 3; i++) out[i] = num(v.arr[i], ctx);
}

// ---------------------------------------------------------------- matrices (glm layout)
struct M4 {
  float m[16];  // column-major
  float& at(int r, int c) { return m[c * 4 + r]; }
  float at(int r, int c) const { return m[c * 4 + r]; }
};
M4 ident() {
  M4 r;
  memset(r.m, 0, sizeof(r.m));
  r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
  return r;
}
// glm operator* for mat4: column j of the product = (a0 b0j + a1 b1j) + a2 b2j) + a3 b3j.
M4 mul(const M4& a, const M4& b) {
  M4 r;
  for (int j = 0; j < 4; j++)
    for (int i = 0; i < 4; i++) {
      float s = a.at(i, 0) * b.at(0, j) + a.at(i, 1) * b.at(1, j);
      s = s + a.at(i, 2) * b.at(2, j);
      s = s + a.at(i, 3) * b.at(3, j);
      r.at(i, j) = s;
    }
  return r;
}
// glm::eulerAngleXYZ(t1, t2, t3) (glm's gtx/euler_angles.inl), the rotation utils/Math.h:848-850
// builds: the closed form of X(t1) Y(t2) Z(t3) over c_i = cos(-t_i), s_i = sin(-t_i), term by
// term as glm writes it.
M4 eulerXYZ(float t1, float t2, float t3) {
  float c1 = nefm::cos(-t1), c2 = nefm::cos(-t2), c3 = nefm::cos(-t3);
  float s1 = nefm::sin(-t1), s2 = nefm::sin(-t2), s3 = nefm::sin(-t3);
  M4 r = ident();
  r.at(0, 0) = c2 * c3;
  r.at(1, 0) = -c1 * s3 + s1 * s2 * c3;
  r.at(2, 0) = s1 * s3 + c1 * s2 * c3;
  r.at(0, 1) = c2 * s3;
  r.at(1, 1) = c1 * c3 + s1 * s2 * s3;
  r.at(2, 1) = -s1 * c3 + c1 * s2 * s3;
  r.at(0, 2) = -s2;
  r.at(1, 2) = s1 * c2;
  r.at(2, 2) = c1 * c2;
  return r;
}
// utils/Math.h:852-859 getTransform = translate(I, t) * rotate(r) * scale(s); degrees.
M4 getTransform(const float* t, const float* rdeg, const float* s) {
  const float toRad = 0.01745329251994329576923690768489f;  // glm::radians
  // glm::translate(I, t): column 3 = ((I0 t0 + I1 t1) + I2 t2) + I3
  M4 id = ident(), tr = ident();
  for (int k = 0; k < 4; k++)
    tr.at(k, 3) = ((id.at(k, 0) * t[0] + id.at(k, 1) * t[1]) + id.at(k, 2) * t[2]) + id.at(k, 3);
  M4 r = mul(tr, eulerXYZ(rdeg[0] * toRad, rdeg[1] * toRad, rdeg[2] * toRad));
  for (int c = 0; c < 3; c++)
    for (int k = 0; k < 4; k++) r.m[c * 4 + k] = r.m[c * 4 + k] * s[c];
  return r;
}
// glm::inverse for a 4x4 (glm's func_matrix.inl, compute_inverse), which InstancedModel's
// constructor calls (primitives/InstancedModel.cpp:11-16): 18 2x2 minors, the cofactor columns
// with alternating signs, the determinant as (d0 + d1) + (d2 + d3) of the first column times the
// first cofactor row, and every element times its reciprocal. Same operations in the same order,
// so the same bits (including the signs of zero elements).
M4 inverse(const M4& a) {
  auto m = [&](int c, int r) { return a.at(r, c); };  // glm's m[column][row]
  float c00 = m(2, 2) * m(3, 3) - m(3, 2) * m(2, 3);
  float c02 = m(1, 2) * m(3, 3) - m(3, 2) * m(1, 3);
  float c03 = m(1, 2) * m(2, 3) - m(2, 2) * m(1, 3);
  float c04 = m(2, 1) * m(3, 3) - m(3, 1) * m(2, 3);
  float c06 = m(1, 1) * m(3, 3) - m(3, 1) * m(1, 3);
  float c07 = m(1, 1) * m(2, 3) - m(2, 1) * m(1, 3);
  float c08 = m(2, 1) * m(3, 2) - m(3, 1) * m(2, 2);
  float c10 = m(1, 1) * m(3, 2) - m(3, 1) * m(1, 2);
  float c11 = m(1, 1) * m(2, 2) - m(2, 1) * m(1, 2);
  float c12 = m(2, 0) * m(3, 3) - m(3, 0) * m(2, 3);
  float c14 = m(1, 0) * m(3, 3) - m(3, 0) * m(1, 3);
  float c15 = m(1, 0) * m(2, 3) - m(2, 0) * m(1, 3);
  float c16 = m(2, 0) * m(3, 2) - m(3, 0) * m(2, 2);
  float c18 = m(1, 0) * m(3, 2) - m(3, 0) * m(1, 2);
  float c19 = m(1, 0) * m(2, 2) - m(2, 0) * m(1, 2);
  float c20 = m(2, 0) * m(3, 1) - m(3, 0) * m(2, 1);
  float c22 = m(1, 0) * m(3, 1) - m(3, 0) * m(1, 1);
  float c23 = m(1, 0) * m(2, 1) - m(2, 0) * m(1, 1);
  const float fac[6][4] = {{c00, c00, c02, c03}, {c04, c04, c06, c07}, {c08, c08, c10, c11},
                           {c12, c12, c14, c15}, {c16, c16, c18, c19}, {c20, c20, c22, c23}};
  float vec[4][4];  // vec[j] = (m[1][j], m[0][j], m[0][j], m[0][j])
  for (int j = 0; j < 4; j++) {
    vec[j][0] = m(1, j);
    vec[j][1] = vec[j][2] = vec[j][3] = m(0, j);
  }
  // Inv0 = Vec1 Fac0 - Vec2 Fac1 + Vec3 Fac2, Inv1 = Vec0 Fac0 - Vec2 Fac3 + Vec3 Fac4,
  // Inv2 = Vec0 Fac1 - Vec1 Fac3 + Vec3 Fac5, Inv3 = Vec0 Fac2 - Vec1 Fac4 + Vec2 Fac5
  const int va[4] = {1, 0, 0, 0}, fa[4] = {0, 0, 1, 2};
  const int vb[4] = {2, 2, 1, 1}, fb[4] = {1, 3, 3, 4};
  const int vc[4] = {3, 3, 3, 2}, fc[4] = {2, 4, 5, 5};
  float inv[4][4];  // [column][row]
  for (int c = 0; c < 4; c++) {
    float sign0 = (c % 2 == 0) ? 1.0f : -1.0f;  // SignA = (+,-,+,-), SignB = (-,+,-,+)
    for (int k = 0; k < 4; k++) {
      float v = (vec[va[c]][k] * fac[fa[c]][k] - vec[vb[c]][k] * fac[fb[c]][k]) + vec[vc[c]][k] * fac[fc[c]][k];
      float sign = (k % 2 == 0) ? sign0 : -sign0;
      inv[c][k] = v * sign;
    }
  }
  float d0 = m(0, 0) * inv[0][0], d1 = m(0, 1) * inv[1][0], d2 = m(0, 2) * inv[2][0], d3 = m(0, 3) * inv[3][0];
  float det = (d0 + d1) + (d2 + d3);
  float od = 1.0f / det;
  M4 r;
  for (int c = 0; c < 4; c++)
    for (int k = 0; k < 4; k++) r.at(k, c) = inv[c][k] * od;
  return r;
}

// small float3 helpers for the camera (glm order)
struct F3 {
  float x, y, z;
};
F3 f3(const float* p) { return F3{p[0], p[1], p[2]}; }
F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 operator-(F3 a) { return F3{-a.x, -a.y, -a.z}; }
F3 operator*(float s, F3 a) { return F3{s * a.x, s * a.y, s * a.z}; }
float dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
F3 normalize(F3 a) {
  float k = 1.0f / nefm::fsqrt(dot(a, a));
  return F3{a.x * k, a.y * k, a.z * k};
}
F3 cross(F3 a, F3 b) { return F3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
void put(float* o, F3 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }

// core/Camera.cpp:7-26 Camera::Camera as SceneReader.cpp:650-675 calls it: aperture 0.0001
// and up (0, 1, 0) whatever the file says.
void lookAtCamera(const float position[3], const float lookAt[3], float vfov, int W, int H, float focus,
                  ne_camera* out) {
  float aspect = float(W) / float(H);
  float aperture = 0.0001f;
  F3 upv = F3{0, 1, 0};
  ne_camera& c = *out;
  c.lens_radius = aperture / 2.0f;
  const float toRad = 0.01745329251994329576923690768489f;
  float half = (vfov * toRad) / 2.0f;
  float halfHeight = nefm::sin(half) / nefm::cos(half);
  float halfWidth = aspect * halfHeight;
  F3 pos = f3(position), la = f3(lookAt);
  F3 front = normalize(pos - la);
  F3 side = normalize(cross(upv, front));
  F3 t1 = (focus * halfWidth) * (-side);
  F3 t2 = (focus * halfHeight) * upv;
  F3 t3 = focus * (-front);
  F3 ll = ((pos - t1) - t2) - t3;
  F3 hz = ((2.0f * focus) * halfWidth) * (-side);
  F3 vt = ((2.0f * focus) * halfHeight) * upv;
  put(c.position, pos);
  put(c.lower_left, ll);
  put(c.horizontal, hz);
  put(c.vertical, vt);
  put(c.side, side);
  put(c.up, upv);
}

}  // namespace

struct ne_scene_host {
  std::vector<ne_instance> instances;       // instancedModels
  std::vector<ne_instance> light_instances; // lights
  std::vector<ne_model> models;
  std::vector<ne_primitive> prims;
  std::vector<ne_material> materials;
  std::vector<uint32_t> model_materials;
  std::vector<ne_light> lights;
  std::vector<ne_medium> media;
  std::vector<std::vector<float>> grids;
  std::vector<std::vector<uint8_t>> textures;  // RGBA8 environment maps and albedo textures (their buffers never move)
  std::vector<ne_instance> all_instances;
  ne_scene_desc desc;
  std::map<std::string, int> material_by_name;
};

namespace {

struct Reader {
  ne_scene_host& S;
  std::string res_dir;
  std::map<std::string, uint32_t> objModels;  // (path, material) -> model, shared by instances

  std::string assetPath(const std::string& rel) const {
    if (!rel.empty() && rel[0] == '/') return rel;
    if (res_dir.empty()) return rel;
    std::string d = res_dir;
    if (d.back() != '/') d.push_back('/');
    return d + rel;
  }

  int addGrid(std::vector<float>&& g) {
    S.grids.push_back(std::move(g));
    return (int)S.grids.size() - 1;
  }

  // std::stof (leading whitespace skipped, the longest number prefix read): a piece without a
  // number, or with a finite number beyond float's range, makes std::stof throw, so the file
  // is rejected.
  static float stofPiece(const std::string& piece, const std::string& what) {
    const char* s = piece.c_str();
    char* end = nullptr;
    errno = 0;
    const float v = strtof(s, &end);
    if (end == s) throw ParseError(NE_ERR_PARSE, what + ": a value is not a number.");
    if (errno == ERANGE && std::isinf(v)) throw ParseError(NE_ERR_PARSE, what + ": a value is out of float range.");
    return v;
  }

  // core/ResourceManager.cpp:222-288 loadVolasTexture: first line "X Y Z " (values
  // followed by a space), second line skipped, then space-separated floats.
  void loadVol(const std::string& path, uint32_t res[3], std::vector<float>& grid) {
    FILE* f = fopen(assetPath(path).c_str(), "rb");
    if (!f) throw ParseError(NE_ERR_MISSING_ASSET, "Couldn't read the file at " + assetPath(path) + ".");
    std::string text;
    char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
    fclose(f);
    size_t l1 = text.find('\n');
    std::string first = text.substr(0, l1 == std::string::npos ? text.size() : l1);
    float r3[3] = {0, 0, 0};
    int count = 0;
    size_t start = 0, e = first.find(' ');
    while (e != std::string::npos && count < 3) {
      r3[count++] = stofPiece(first.substr(start, e - start), "volume " + path);
      start = e + 1;
      e = first.find(' ', start);
    }
    if (count < 3) throw ParseError(NE_ERR_PARSE, "volume " + path + ": resolution line needs three values.");
    for (int a = 0; a < 3; a++) res[a] = (uint32_t)wholeIn(r3[a], 1, 65536, "volume " + path + " resolution");
    size_t total = (size_t)res[0] * res[1] * res[2];
    grid.assign(total, 0.0f);
    size_t l2 = (l1 == std::string::npos) ? std::string::npos : text.find('\n', l1 + 1);
    std::string data = (l2 == std::string::npos) ? std::string() : text.substr(l2 + 1);
    size_t k = 0;
    start = 0;
    e = data.find(' ');
    while (e != std::string::npos) {
      if (k >= total) throw ParseError(NE_ERR_PARSE, "volume " + path + ": more values than the resolution.");
      grid[k++] = stofPiece(data.substr(start, e - start), "volume " + path);
      start = e + 1;
      e = data.find(' ', start);
    }
  }

  void loadF32(const std::string& path, const uint32_t res[3], std::vector<float>& grid) {
    FILE* f = fopen(assetPath(path).c_str(), "rb");
    if (!f) throw ParseError(NE_ERR_MISSING_ASSET, "Couldn't read the file at " + assetPath(path) + ".");
    size_t total = (size_t)res[0] * res[1] * res[2];
    grid.assign(total, 0.0f);
    size_t got = fread(grid.data(), sizeof(float), total, f);
    fclose(f);
    if (got != total) throw ParseError(NE_ERR_PARSE, "grid " + path + ": file shorter than the resolution.");
  }

  // io/SceneReader.cpp:67-222 processMaterial.
  void material(const JVal& m) {
    std::string name = sval(need(m, "name", "Material"), "Material name");
    std::string type = sval(need(m, "type", "Material " + name), "Material type");
    ne_material mat;
    memset(&mat, 0, sizeof(mat));
    mat.light = -1;
    mat.medium = -1;
    std::string ctx = "Material " + name;
    if (type == "microfacet") {
      const JVal& alb = need(m, "albedo", ctx);
      float albedo[3] = {1, 0, 1};
      if (alb.kind == JVal::STR) {
        // SceneReader.cpp:80-103: the albedo texture at resources/path, decoded to RGBA8
        neimg::Image img;
        std::string err;
        ne_status st = neimg::loadRGBA8(assetPath(alb.str), img, err);
        if (st != NE_OK) throw ParseError(st, ctx + ": " + err);
        S.textures.push_back(std::move(img.rgba));
        mat.albedo_width = img.width;
        mat.albedo_height = img.height;
        mat.albedo_texels = S.textures.back().data();
      } else {
        vec3(alb, albedo, ctx + " albedo");
      }
      memcpy(mat.albedo, albedo, sizeof(albedo));
      float nm[3] = {0, 0, 1};
      bool hasNormal = m.get("normalMap") != nullptr;
      if (hasNormal) vec3(*m.get("normalMap"), nm, ctx + " normalMap");
      memcpy(mat.normal_map, nm, sizeof(nm));
      mat.roughness = num(need(m, "roughness", ctx), ctx + " roughness");
      mat.metallic = num(need(m, "metallic", ctx), ctx + " metallic");
      mat.bsdf = NE_BSDF_GLOSSY;
      // addTexture order ALBEDO, METALLIC, ROUGHNESS[, NORMAL]; textureTypes keeps the
      // last one only (materials/Material.h:38-44).
      mat.tex_present = NE_TEX_ALBEDO | NE_TEX_METALLIC | NE_TEX_ROUGHNESS | (hasNormal ? NE_TEX_NORMAL : 0);
      mat.tex_types = hasNormal ? NE_TEX_NORMAL : NE_TEX_ROUGHNESS;
    } else if (type == "emitter") {
      ne_light L;
      memset(&L, 0, sizeof(L));
      L.type = NE_LIGHT_DIFFUSE;
      L.primitive = -1;
      vec3(need(m, "albedo", ctx), L.li, ctx + " albedo");
      memcpy(mat.albedo, L.li, sizeof(L.li));
      S.lights.push_back(L);
      mat.light = (int)S.lights.size() - 1;
      mat.tex_present = NE_TEX_ALBEDO;
      mat.tex_types = NE_TEX_ALBEDO;
    } else if (type == "directionalLight") {
      ne_light L;
      memset(&L, 0, sizeof(L));
      L.type = NE_LIGHT_DIRECTIONAL;
      L.primitive = -1;
      vec3(need(m, "albedo", ctx), L.le, ctx + " albedo");
      float pos[3] = {0, 0, 0};
      vec3(need(m, "position", ctx), pos, ctx + " position");
      F3 dir = normalize(F3{0.0f - pos[0], 0.0f - pos[1], 0.0f - pos[2]});
      put(L.direction, dir);
      S.lights.push_back(L);
      mat.light = (int)S.lights.size() - 1;
    } else if (type == "infiniteAreaLight") {
      ne_light L;
      memset(&L, 0, sizeof(L));
      L.type = NE_LIGHT_INFINITE;
      L.primitive = -1;
      if (const JVal* p = m.get("path")) {
        // SceneReader.cpp:169-185: the texture at resources/path, decoded to RGBA8
        neimg::Image img;
        std::string err;
        ne_status st = neimg::loadRGBA8(assetPath(sval(*p, ctx + " path")), img, err);
        if (st != NE_OK) throw ParseError(st, ctx + ": " + err);
        if (img.height > img.width)
          throw ParseError(NE_ERR_UNSUPPORTED, ctx + ": environment maps taller than wide are not supported (the "
                                               "reference's Distribution2D reads past such an image).");
        S.textures.push_back(std::move(img.rgba));
        L.env_width = img.width;
        L.env_height = img.height;
        L.env_texels = S.textures.back().data();
      } else {
        vec3(need(m, "radiance", ctx), L.env_radiance, ctx + " radiance");
        // Distribution2D over a 1x1 map of value G (InfiniteAreaLight.h:51-65, Sampling.h:12-28):
        // the sampled pdf is func/funcInt = 1 when G > 0, else 0.
        L.env_map_pdf = (L.env_radiance[1] > 0.0f) ? 1.0f : 0.0f;
      }
      S.lights.push_back(L);
      mat.light = (int)S.lights.size() - 1;
      mat.tex_present = NE_TEX_TEX1;
      mat.tex_types = NE_TEX_TEX1;
    } else if (type == "volume") {
      ne_medium md;
      memset(&md, 0, sizeof(md));
      vec3(need(m, "scattering", ctx), md.sigma_s, ctx + " scattering");
      vec3(need(m, "absorption", ctx), md.sigma_a, ctx + " absorption");
      std::string pf = sval(need(m, "phaseFunction", ctx), ctx + " phaseFunction");
      if (pf == "isotropic") {
        mat.phase = NE_PHASE_ISOTROPIC;
      } else if (pf == "hg" || pf == "henyey-greenstein") {
        mat.phase = NE_PHASE_HG;
        mat.g = num(need(m, "g", ctx), ctx + " g");
      } else {
        throw ParseError(NE_ERR_PARSE, ctx + ": unknown phase function " + pf + ".");
      }
      md.density = num(need(m, "density", ctx), ctx + " density");
      for (int a = 0; a < 3; a++) {  // the tracking steps divide by these: they must stay finite
        const float sigmaT = (md.sigma_s[a] + md.sigma_a[a]) * md.density;
        if (!std::isfinite(sigmaT) || !std::isfinite(md.sigma_s[a]) || !std::isfinite(md.sigma_a[a]))
          throw ParseError(NE_ERR_PARSE, ctx + ": scattering, absorption and density must stay finite.");
      }
      std::vector<float> grid;
      bool isGrid = false;
      if (const JVal* p = m.get("path")) {
        std::string path = sval(*p, ctx + " path");
        if (path.find(".vdb") != std::string::npos) {
          // core/ResourceManager.cpp:165-218 loadVDBasTexture
          std::string err;
          const ne_status st = nevdb::loadDensity(assetPath(path), md.res, grid, err);
          if (st != NE_OK) throw ParseError(st, ctx + ": " + err);
        } else if (path.find(".vol") != std::string::npos) {
          loadVol(path, md.res, grid);
        } else {
          throw ParseError(NE_ERR_PARSE, ctx + ": volume path must be a .vol or .vdb file.");
        }
        isGrid = true;
      } else if (const JVal* g = m.get("grid")) {
        const JVal& r = need(*g, "resolution", ctx + " grid");
        float rf[3] = {0, 0, 0};
        vec3(r, rf, ctx + " grid resolution");
        for (int a = 0; a < 3; a++)  // whole voxels, 1 to 65536 per axis
          if (!(rf[a] >= 1.0f && rf[a] < 65537.0f))
            throw ParseError(NE_ERR_PARSE, ctx + ": grid resolution must be 1 to 65536 voxels per axis.");
        md.res[0] = (uint32_t)rf[0]; md.res[1] = (uint32_t)rf[1]; md.res[2] = (uint32_t)rf[2];
        if (const JVal* gp = g->get("path")) {
          loadF32(sval(*gp, ctx + " grid path"), md.res, grid);
        } else {
          std::string gen = sval(need(*g, "generator", ctx + " grid"), ctx + " grid generator");
          if (gen != "fbm") throw ParseError(NE_ERR_PARSE, ctx + ": unknown grid generator " + gen + ".");
          negen::FbmParams fp;
          const double oct = g->get("octaves") ? num(*g->get("octaves"), "octaves") : 5.0;
          if (!(oct >= 1.0 && oct < 33.0)) throw ParseError(NE_ERR_PARSE, ctx + ": grid octaves must be 1 to 32.");
          fp.octaves = (int)oct;
          fp.frequency = g->get("frequency") ? g->get("frequency")->num : 4.0 / md.res[0];
          fp.lacunarity = g->get("lacunarity") ? g->get("lacunarity")->num : 2.0;
          fp.gain = g->get("gain") ? g->get("gain")->num : 0.5;
          fp.falloff_radius = g->get("falloff_radius") ? g->get("falloff_radius")->num : md.res[0] * 0.5;
          const double seed = g->get("seed") ? g->get("seed")->num : (double)0x4E415256ull;
          if (!(seed >= 0.0 && seed <= 9007199254740992.0))
            throw ParseError(NE_ERR_PARSE, ctx + ": grid seed must be an integer from 0 to 2^53.");
          fp.seed = (uint64_t)seed;
          negen::fbm_grid(md.res, fp, grid);
        }
        isGrid = true;
      }
      if (isGrid) {
        md.type = NE_MEDIUM_GRID;
        int gi = addGrid(std::move(grid));
        (void)gi;
        md.grid = nullptr;  // bound after all grids are stored
        md.res[0] = md.res[0];
        grids_of_media.push_back(gi);
      } else {
        md.type = NE_MEDIUM_HOMOGENEOUS;
        grids_of_media.push_back(-1);
      }
      S.media.push_back(md);
      mat.medium = (int)S.media.size() - 1;
      mat.bsdf = NE_BSDF_VOLUME;
      mat.tex_present = NE_TEX_TEX1;
      mat.tex_types = NE_TEX_TEX1;
    } else {
      throw ParseError(NE_ERR_PARSE, "Invalid material type while reading scene from json file.");
    }
    S.materials.push_back(mat);
    S.material_by_name[name] = (int)S.materials.size() - 1;
  }
  std::vector<int> grids_of_media;

  int materialNamed(const std::string& name, const std::string& ctx) {
    auto it = S.material_by_name.find(name);
    if (it == S.material_by_name.end()) throw ParseError(NE_ERR_PARSE, ctx + ": unknown material " + name + ".");
    return it->second;
  }

  void addInstance(const M4& M, uint32_t model, bool collision, bool isLight) {
    ne_instance in;
    memset(&in, 0, sizeof(in));
    memcpy(in.to_wcs, M.m, sizeof(M.m));
    M4 inv = inverse(M);
    memcpy(in.to_ocs, inv.m, sizeof(inv.m));
    in.model = model;
    in.collision = collision ? 1 : 0;
    (isLight ? S.light_instances : S.instances).push_back(in);
  }

  // A Model holding one primitive, either in Model::lights (emissive material) or in
  // Model::primitives, with Model::materials = [material].
  uint32_t singlePrimModel(ne_primitive p, int mat, bool emissive) {
    ne_model md;
    memset(&md, 0, sizeof(md));
    p.material = mat;
    S.prims.push_back(p);
    uint32_t pi = (uint32_t)S.prims.size() - 1;
    if (emissive) {
      md.light_begin = pi; md.light_count = 1;
      md.prim_begin = pi; md.prim_count = 0;
      S.lights[S.materials[mat].light].primitive = (int)pi;  // material->light->primitive = prim
    } else {
      md.prim_begin = pi; md.prim_count = 1;
      md.light_begin = pi; md.light_count = 0;
    }
    md.mat_begin = (uint32_t)S.model_materials.size();
    md.mat_count = 1;
    S.model_materials.push_back((uint32_t)mat);
    S.models.push_back(md);
    return (uint32_t)S.models.size() - 1;
  }

  // io/SceneReader.cpp:224-648 processPrimitives.
  void primitive(const JVal& p) {
    std::string name = sval(need(p, "name", "Primitive"), "Primitive name");
    std::string ctx = "Primitive " + name;
    std::string type = sval(need(p, "type", ctx), ctx + " type");
    const JVal& tr = need(p, "transform", ctx);
    float pos[3] = {0, 0, 0}, scale[3] = {1, 1, 1}, rot[3] = {0, 0, 0};
    vec3(need(tr, "position", ctx + " transform"), pos, ctx + " position");
    bool collision = true;
    if (const JVal* c = p.get("collision")) collision = c->kind == JVal::BOOL ? c->b : num(*c, "collision") != 0;
    auto readSR = [&]() {
      vec3(need(tr, "scale", ctx + " transform"), scale, ctx + " scale");
      vec3(need(tr, "rotation", ctx + " transform"), rot, ctx + " rotation");
    };
    ne_primitive pr;
    memset(&pr, 0, sizeof(pr));
    if (type == "point") {
      readSR();
      int mat = materialNamed(sval(need(p, "materialName", ctx), ctx), ctx);
      pr.type = NE_PRIM_POINT;
      memcpy(pr.p0, pos, sizeof(pos));
      bool em = S.materials[mat].light >= 0;
      uint32_t mi = singlePrimModel(pr, mat, em);
      addInstance(getTransform(pos, rot, scale), mi, true, em);
    } else if (type == "sphere") {
      pr.type = NE_PRIM_SPHERE;
      pr.radius = num(need(p, "radius", ctx), ctx + " radius");
      int mat = materialNamed(sval(need(p, "materialName", ctx), ctx), ctx);
      bool em = S.materials[mat].light >= 0;
      uint32_t mi = singlePrimModel(pr, mat, em);
      float zero[3] = {0, 0, 0}, one[3] = {1, 1, 1};
      addInstance(getTransform(pos, zero, one), mi, collision, em);
    } else if (type == "rectangle") {
      readSR();
      int mat = materialNamed(sval(need(p, "materialName", ctx), ctx), ctx);
      pr.type = NE_PRIM_RECTANGLE;
      // OCS unit square z = 0; vertexData[0] = bottom left, vertexData[1] = vertex 2
      // (top right); normal (0,0,-1) (SceneReader.cpp:407-482).
      pr.p0[0] = -0.5f; pr.p0[1] = -0.5f; pr.p0[2] = 0.0f;
      pr.p1[0] = 0.5f; pr.p1[1] = 0.5f; pr.p1[2] = 0.0f;
      pr.p2[0] = 0.0f; pr.p2[1] = 0.0f; pr.p2[2] = -1.0f;
      bool em = S.materials[mat].light >= 0;
      uint32_t mi = singlePrimModel(pr, mat, em);
      addInstance(getTransform(pos, rot, scale), mi, true, em);
    } else if (type == "volume") {
      readSR();
      int mat = materialNamed(sval(need(p, "materialName", ctx), ctx), ctx);
      pr.type = NE_PRIM_AABB;
      for (int i = 0; i < 3; i++) { pr.p0[i] = -0.5f; pr.p1[i] = 0.5f; }
      uint32_t mi = singlePrimModel(pr, mat, false);
      addInstance(getTransform(pos, rot, scale), mi, true, false);
    } else if (type == "mesh") {
      readSR();
      mesh(p, ctx);
      addInstance(getTransform(pos, rot, scale), (uint32_t)S.models.size() - 1, collision, false);
    } else if (type == "obj") {
      // SceneReader.cpp:245-266: a model file under RESOURCES_DIR with an InstancedModel. The
      // reference loads it through assimp (ResourceManager::loadModel, Model.cpp:137-370); here
      // the OBJ text is read directly, with the JSON materialName for every triangle.
      readSR();
      std::string path = sval(need(p, "path", ctx), ctx + " path");
      if (!p.get("materialName"))
        throw ParseError(NE_ERR_UNSUPPORTED, ctx + ": obj models need a materialName (MTL materials are not read).");
      std::string matName = sval(*p.get("materialName"), ctx);
      std::string key = path + "\n" + matName;
      uint32_t mi;
      auto it = objModels.find(key);
      if (it != objModels.end()) {
        mi = it->second;  // same file and material: instances share one model and its BVH
      } else {
        std::vector<float> vpos;
        std::vector<uint32_t> vidx;
        readObj(assetPath(path), vpos, vidx, ctx);
        meshModel(vpos, vidx, p, ctx);
        mi = (uint32_t)S.models.size() - 1;
        objModels[key] = mi;
      }
      // SceneReader.cpp:262-263 does not pass "collision" on to model instances
      // (InstancedModel::isCollisionEnabled keeps its default, true)
      addInstance(getTransform(pos, rot, scale), mi, true, false);
    } else if (type == "gltf") {
      throw ParseError(NE_ERR_UNSUPPORTED, ctx + ": gltf models are not supported (obj only).");
    } else {
      throw ParseError(NE_ERR_PARSE, "Invalid primitive type while reading scene from json file.");
    }
  }

  // Extension: triangle mesh loaded like Model(aiScene) (primitives/Model.cpp:4-7, 337-370):
  // bounding box over the vertices, BVH over the triangles.
  void mesh(const JVal& p, const std::string& ctx) {
    std::vector<float> pos;
    std::vector<uint32_t> idx;
    if (const JVal* g = p.get("generator")) {
      std::string gen = sval(*g, ctx + " generator");
      if (gen != "icosphere") throw ParseError(NE_ERR_PARSE, ctx + ": unknown mesh generator " + gen + ".");
      negen::IcoParams ip;
      const double sub = p.get("subdivisions") ? num(*p.get("subdivisions"), "subdivisions") : 3.0;
      if (!(sub >= 0.0 && sub < 11.0)) throw ParseError(NE_ERR_PARSE, ctx + ": subdivisions must be 0 to 10.");
      ip.subdivisions = (int)sub;
      if (const JVal* d = p.get("displacement")) {
        ip.amplitude = d->get("amplitude") ? d->get("amplitude")->num : 0.0;
        ip.frequency = d->get("frequency") ? d->get("frequency")->num : 1.0;
        const double seed = d->get("seed") ? d->get("seed")->num : (double)0x4E415256ull;
        if (!(seed >= 0.0 && seed <= 9007199254740992.0))
          throw ParseError(NE_ERR_PARSE, ctx + ": displacement seed must be an integer from 0 to 2^53.");
        ip.seed = (uint64_t)seed;
      }
      negen::icosphere(ip, pos, idx);
    } else {
      const JVal& P = need(p, "positions", ctx);
      const JVal& I = need(p, "indices", ctx);
      for (auto& v : P.arr) pos.push_back(num(v, ctx + " positions"));
      for (auto& v : I.arr) {
        const double k = v.kind == JVal::NUM ? v.num : (double)num(v, ctx + " indices");
        if (!(k >= 0.0 && k < 4294967296.0)) throw ParseError(NE_ERR_PARSE, ctx + ": index out of range.");
        idx.push_back((uint32_t)k);
      }
      if (pos.size() % 3 || idx.size() % 3) throw ParseError(NE_ERR_PARSE, ctx + ": positions/indices not multiples of 3.");
      for (uint32_t i : idx)
        if ((size_t)i * 3 + 2 >= pos.size()) throw ParseError(NE_ERR_PARSE, ctx + ": index out of range.");
    }
    meshModel(pos, idx, p, ctx);
  }

  // Wavefront OBJ positions and faces: "v x y z", "f a b c ..." with a, a/t, a/t/n or a//n
  // (1-based, negative = relative to the end); polygons become triangle fans (v0, vi, vi+1),
  // as assimp's triangulation of convex faces. Lines split at '\n' (one trailing '\r'
  // dropped), tokens at spaces and tabs; a first token starting with '#' is a comment, other
  // keywords are ignored. A vertex needs three decimal numbers (sign, digits, point,
  // exponent; read as double, then rounded to float), extra tokens ignored; a face needs
  // three vertex indices (a signed integer before any '/').
  static bool decimalToken(const std::string& t) {
    size_t i = 0, n = t.size(), digits = 0;
    if (i < n && (t[i] == '+' || t[i] == '-')) i++;
    while (i < n && isdigit((unsigned char)t[i])) i++, digits++;
    if (i < n && t[i] == '.') {
      i++;
      while (i < n && isdigit((unsigned char)t[i])) i++, digits++;
    }
    if (!digits) return false;
    if (i < n && (t[i] == 'e' || t[i] == 'E')) {
      i++;
      if (i < n && (t[i] == '+' || t[i] == '-')) i++;
      size_t e = 0;
      while (i < n && isdigit((unsigned char)t[i])) i++, e++;
      if (!e) return false;
    }
    return i == n;
  }
  static bool integerToken(const std::string& t) {
    size_t i = (!t.empty() && (t[0] == '+' || t[0] == '-')) ? 1 : 0;
    if (i == t.size() || t.size() - i > 18) return false;
    for (; i < t.size(); i++)
      if (!isdigit((unsigned char)t[i])) return false;
    return true;
  }
  void readObj(const std::string& file, std::vector<float>& pos, std::vector<uint32_t>& idx, const std::string& ctx) {
    FILE* f = fopen(file.c_str(), "rb");
    if (!f) throw ParseError(NE_ERR_MISSING_ASSET, ctx + ": cannot open " + file);
    std::string text;
    char buf[1 << 16];
    size_t r;
    while ((r = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, r);
    fclose(f);
    size_t i = 0, line = 0;
    std::vector<std::string> tok;
    std::vector<long> face;
    while (i <= text.size()) {
      size_t e = text.find('\n', i);
      if (e == std::string::npos) e = text.size();
      std::string ln = text.substr(i, e - i);
      i = e + 1;
      line++;
      if (!ln.empty() && ln.back() == '\r') ln.pop_back();
      tok.clear();
      for (size_t a = 0; a < ln.size();) {
        while (a < ln.size() && (ln[a] == ' ' || ln[a] == '\t')) a++;
        size_t b = a;
        while (b < ln.size() && ln[b] != ' ' && ln[b] != '\t') b++;
        if (b > a) tok.push_back(ln.substr(a, b - a));
        a = b;
      }
      if (tok.empty() || tok[0][0] == '#') continue;
      const std::string where = " at line " + std::to_string(line);
      if (tok[0] == "v") {
        if (tok.size() < 4) throw ParseError(NE_ERR_PARSE, ctx + ": bad vertex" + where);
        for (int k = 1; k <= 3; k++) {
          if (!decimalToken(tok[k])) throw ParseError(NE_ERR_PARSE, ctx + ": bad vertex" + where);
          pos.push_back((float)strtod(tok[k].c_str(), nullptr));
        }
      } else if (tok[0] == "f") {
        face.clear();
        const long nv = (long)(pos.size() / 3);
        for (size_t k = 1; k < tok.size(); k++) {
          const std::string num = tok[k].substr(0, tok[k].find('/'));
          if (!integerToken(num)) throw ParseError(NE_ERR_PARSE, ctx + ": bad face" + where);
          const long v = strtol(num.c_str(), nullptr, 10);
          const long vi = v > 0 ? v - 1 : nv + v;
          if (vi < 0 || vi >= nv) throw ParseError(NE_ERR_PARSE, ctx + ": face index out of range" + where);
          face.push_back(vi);
        }
        if (face.size() < 3) throw ParseError(NE_ERR_PARSE, ctx + ": face with fewer than 3 vertices" + where);
        for (size_t t = 1; t + 1 < face.size(); t++) {
          idx.push_back((uint32_t)face[0]);
          idx.push_back((uint32_t)face[t]);
          idx.push_back((uint32_t)face[t + 1]);
        }
      }
    }
  }

  // A triangle model (primitives/Model.cpp:4-7, 337-370): bounding box over the vertices,
  // BVH over the triangles; materials from "materialName" or seeded "groups".
  void meshModel(const std::vector<float>& pos, const std::vector<uint32_t>& idx, const JVal& p,
                 const std::string& ctx) {
    uint32_t nt = (uint32_t)(idx.size() / 3);
    if (nt == 0) throw ParseError(NE_ERR_PARSE, ctx + ": mesh has no triangles.");
    // materials: one named material, or seeded groups
    std::vector<int> triMat(nt, -1);
    ne_model md;
    memset(&md, 0, sizeof(md));
    md.mat_begin = (uint32_t)S.model_materials.size();
    if (const JVal* gr = p.get("groups")) {
      const int count = gr->get("count") ? (int)wholeIn(num(*gr->get("count"), "count"), 1, 65536, ctx + " group count") : 1;
      float rr[2] = {0.05f, 0.9f}, ar[2] = {0.2f, 0.9f};
      if (const JVal* v = gr->get("roughness")) { rr[0] = num(v->arr.at(0), "roughness"); rr[1] = num(v->arr.at(1), "roughness"); }
      if (const JVal* v = gr->get("albedo")) { ar[0] = num(v->arr.at(0), "albedo"); ar[1] = num(v->arr.at(1), "albedo"); }
      const uint64_t seed =
          gr->get("seed") ? (uint64_t)wholeIn(gr->get("seed")->num, 0, 9007199254740992.0, ctx + " group seed") : 0x4E415256ull;
      int first = (int)S.materials.size();
      for (int k = 0; k < count; k++) {
        ne_material mat;
        memset(&mat, 0, sizeof(mat));
        mat.light = -1;
        mat.medium = -1;
        mat.bsdf = NE_BSDF_GLOSSY;
        double u0 = negen::hash_u01(seed, (uint64_t)k * 4 + 0);
        double u1 = negen::hash_u01(seed, (uint64_t)k * 4 + 1);
        mat.roughness = (float)(rr[0] + (rr[1] - rr[0]) * u0);
        float a = (float)(ar[0] + (ar[1] - ar[0]) * u1);
        mat.albedo[0] = mat.albedo[1] = mat.albedo[2] = a;
        mat.metallic = 0.0f;
        mat.tex_present = NE_TEX_ALBEDO | NE_TEX_METALLIC | NE_TEX_ROUGHNESS;
        mat.tex_types = NE_TEX_ROUGHNESS;
        S.materials.push_back(mat);
        S.model_materials.push_back((uint32_t)(first + k));
      }
      for (uint32_t t = 0; t < nt; t++) triMat[t] = first + (int)((uint64_t)t * (uint64_t)count / nt);
      md.mat_count = (uint32_t)count;
    } else if (const JVal* mn = p.get("materialName")) {
      int mat = materialNamed(sval(*mn, ctx), ctx);
      for (auto& m : triMat) m = mat;
      S.model_materials.push_back((uint32_t)mat);
      md.mat_count = 1;
    }
    md.prim_begin = (uint32_t)S.prims.size();
    md.prim_count = nt;
    md.light_begin = md.prim_begin + nt;
    md.light_count = 0;
    const float inf = INFINITY;
    float mn[3] = {inf, inf, inf}, mx[3] = {-inf, -inf, -inf};
    for (uint32_t t = 0; t < nt; t++) {
      ne_primitive pr;
      memset(&pr, 0, sizeof(pr));
      pr.type = NE_PRIM_TRIANGLE;
      pr.material = triMat[t];
      float* dst[3] = {pr.p0, pr.p1, pr.p2};
      for (int k = 0; k < 3; k++) {
        const float* v = &pos[(size_t)idx[3 * t + k] * 3];
        memcpy(dst[k], v, 12);
        for (int c = 0; c < 3; c++) {
          mn[c] = (v[c] < mn[c]) ? v[c] : mn[c];
          mx[c] = (mx[c] < v[c]) ? v[c] : mx[c];
        }
      }
      // Triangle::calculateArea (primitives/Triangle.cpp:149-157)
      F3 a = f3(pr.p0), b = f3(pr.p1), c = f3(pr.p2);
      F3 n = cross(b - a, c - a);
      pr.area = nefm::fsqrt(dot(n, n)) / 2.0f;
      S.prims.push_back(pr);
    }
    md.has_bbox = 1;
    memcpy(md.bbox_min, mn, 12);
    memcpy(md.bbox_max, mx, 12);
    md.use_bvh = 1;
    S.models.push_back(md);
  }

  // io/SceneReader.cpp:650-675 processCameraAndRenderer and core/Camera.cpp:7-26.
  void cameraAndRenderer(const JVal& cam, const JVal& ren) {
    float position[3], lookAt[3], up[3];
    vec3(need(cam, "position", "camera"), position, "camera position");
    vec3(need(cam, "lookAt", "camera"), lookAt, "camera lookAt");
    vec3(need(cam, "up", "camera"), up, "camera up");
    float vfov = num(need(cam, "vfov", "camera"), "camera vfov");
    const JVal& res = need(ren, "resolution", "renderer");
    if (res.kind != JVal::ARR || res.arr.size() < 2) throw ParseError(NE_ERR_PARSE, "renderer resolution needs [W, H].");
    if (!(res.arr[0].num >= 1.0 && res.arr[1].num >= 1.0))
      throw ParseError(NE_ERR_PARSE, "renderer resolution must be positive.");
    const int W = (int)wholeIn(res.arr[0].num, 1, 2147483647.0, "renderer resolution");
    const int H = (int)wholeIn(res.arr[1].num, 1, 2147483647.0, "renderer resolution");
    float focus;
    const JVal* af = cam.get("autoFocus");
    if (af && af->kind == JVal::BOOL && af->b)
      focus = 3.0f;  // (position - lookAt).length(): glm's component count
    else
      focus = num(need(cam, "focus", "camera"), "camera focus");
    (void)up;
    lookAtCamera(position, lookAt, vfov, W, H, focus, &S.desc.camera);
    ne_settings& st = S.desc.settings;
    st.width = W;
    st.height = H;
    st.spp = (int)wholeIn(num(need(ren, "spp", "renderer"), "renderer spp"), -2147483648.0, 2147483647.0, "renderer spp");
    st.bounces = (int)wholeIn(num(need(ren, "bounces", "renderer"), "renderer bounces"), -2147483648.0, 2147483647.0,
                              "renderer bounces");
    const JVal* hdr = ren.get("HDR");
    st.hdr = (hdr && hdr->kind == JVal::BOOL && hdr->b) ? 1 : 0;
    st.rr_enabled = 0;
    st.rr_after = 3;
    if (const JVal* rr = ren.get("rr")) {
      st.rr_enabled = 1;
      if (const JVal* a = rr->get("after"))
        st.rr_after = (int)wholeIn(num(*a, "rr after"), -2147483648.0, 2147483647.0, "renderer rr after");
    }
    st.bvh_build = 0;
    if (const JVal* bv = ren.get("bvh")) {
      std::string kind = sval(*bv, "renderer bvh");
      if (kind == "sah")
        st.bvh_build = 1;
      else if (kind != "reference")
        throw ParseError(NE_ERR_PARSE, "renderer bvh must be \"reference\" or \"sah\".");
    }
  }

  // io/SceneReader.cpp:10-54 loadScene.
  void load(const JVal& doc) {
    if (doc.kind != JVal::OBJ) throw ParseError(NE_ERR_PARSE, "Malformatted json file. Not a valid json object.");
    if (!doc.get("version")) throw ParseError(NE_ERR_PARSE, "Incomplete json file. Version is not present.");
    const JVal& mats = need(doc, "materials", "scene");
    for (auto& m : mats.arr) material(m);
    const JVal& prims = need(doc, "primitives", "scene");
    for (auto& p : prims.arr) primitive(p);
    cameraAndRenderer(need(doc, "camera", "scene"), need(doc, "renderer", "scene"));
  }
};

void finalize(ne_scene_host& S, const std::vector<int>& grids_of_media) {
  S.all_instances = S.instances;
  S.all_instances.insert(S.all_instances.end(), S.light_instances.begin(), S.light_instances.end());
  for (size_t i = 0; i < S.media.size(); i++) {
    int g = grids_of_media[i];
    S.media[i].grid = g >= 0 ? S.grids[g].data() : nullptr;
  }
  ne_scene_desc& d = S.desc;
  d.n_instances = (uint32_t)S.instances.size();
  d.n_light_instances = (uint32_t)S.light_instances.size();
  d.instances = S.all_instances.data();
  d.n_models = (uint32_t)S.models.size();
  d.models = S.models.data();
  d.n_prims = (uint32_t)S.prims.size();
  d.prims = S.prims.data();
  d.n_materials = (uint32_t)S.materials.size();
  d.materials = S.materials.data();
  d.n_model_materials = (uint32_t)S.model_materials.size();
  d.model_materials = S.model_materials.data();
  d.n_lights = (uint32_t)S.lights.size();
  d.lights = S.lights.data();
  d.n_media = (uint32_t)S.media.size();
  d.media = S.media.data();
}

ne_status loadFromText(const std::string& text, const char* resources_dir, ne_scene_host** out, char* err,
                       size_t err_len) {
  if (!out) return NE_ERR_INVALID_ARG;
  *out = nullptr;
  std::unique_ptr<ne_scene_host> S(new ne_scene_host());
  memset(&S->desc, 0, sizeof(S->desc));
  try {
    JParser jp{text.data(), text.data() + text.size()};
    JVal doc = jp.parse();
    jp.ws();
    if (jp.p != jp.end) jp.fail("data after the document");
    Reader r{*S, resources_dir ? resources_dir : ""};
    r.load(doc);
    finalize(*S, r.grids_of_media);
  } catch (const ParseError& e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    if (err && err_len) snprintf(err, err_len, "out of host memory while reading the scene");
    return NE_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    if (err && err_len) snprintf(err, err_len, "%s", e.what());
    return NE_ERR_PARSE;
  }
  *out = S.release();
  return NE_OK;
}

}  // namespace

extern "C" {

ne_status ne_scene_host_load_json(const char* path, const char* resources_dir, ne_scene_host** out, char* err,
                                  size_t err_len) {
  if (!path || !out) return NE_ERR_INVALID_ARG;
  FILE* f = fopen(path, "rb");
  if (!f) {
    if (err && err_len) snprintf(err, err_len, "Couldn't read %s.", path);
    return NE_ERR_MISSING_ASSET;
  }
  std::string text;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
  fclose(f);
  return loadFromText(text, resources_dir, out, err, err_len);
}

ne_status ne_scene_host_load_json_string(const char* json, const char* resources_dir, ne_scene_host** out, char* err,
                                         size_t err_len) {
  if (!json || !out) return NE_ERR_INVALID_ARG;
  return loadFromText(std::string(json), resources_dir, out, err, err_len);
}

const ne_scene_desc* ne_scene_host_desc(const ne_scene_host* s) { return s ? &s->desc : nullptr; }

void ne_scene_host_destroy(ne_scene_host* s) { delete s; }

}  // extern "C"

extern "C" ne_status ne_camera_look_at(const float position[3], const float look_at[3], float vfov_deg, int width,
                                       int height, float focus, ne_camera* out) {
  if (!position || !look_at || !out || width <= 0 || height <= 0) return NE_ERR_INVALID_ARG;
  lookAtCamera(position, look_at, vfov_deg, width, height, focus, out);
  return NE_OK;
}
