// CPU oracle of the NarvalEngine path-tracing hot path (test infrastructure; see oracle.h).
//
// Every function below restates one reference function; the citation in front of it
// gives the reference file:line (paths relative to the reference's src/). Arithmetic
// follows the reference's expression order and types: float where the reference uses
// float, double where a double literal promotes the expression (EPSILON, PI, TWO_PI),
// and glm's evaluation order for vector operations (dot = (x*x' + y*y') + z*z',
// mat4*vec4 = (c0 v0 + c1 v1) + (c2 v2 + c3 v3), min(a,b) = b<a?b:a, max(a,b) = a<b?b:a,
// mix(x,y,a) = x(1-a) + y a). Built with -ffp-contract=off so no multiply-add is fused.
//
// Deviations, each also taken by the GPU code:
//  1. random() -> nerng::u01(key, dim) (ne_rng.h), drawn in the reference's order;
//     arguments of one constructor call (glm::vec2(random(), random())) are drawn
//     left to right.
//  2. libm -> nefm:: (ne_fmath.h).
//  3. intersectTr (VolumetricPathIntegrator.cpp:10-32) never terminates in the
//     reference when a surface query returns a hit at the ray origin (the "inside"
//     rule of Model.cpp:418-424 for a sphere whose surface point rounds inside): the
//     next segment starts at the same point and repeats forever. Here the loop
//     returns "no medium reached" when the next origin equals the current one or
//     after 256 segments.
//  4. Delta and ratio tracking stop after 2^20 steps and a path ends after 2^16 medium
//     pass-throughs (the reference loops without a bound; counts that large need a
//     majorant/extinction pair or a volume arrangement no scene uses).
//  5. A scene with no lights returns zero from uniformSampleOneLight after the light
//     index draw (the reference throws std::out_of_range from vector::at).

#include "oracle.h"

#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <limits>
#include <thread>
#include <vector>

#include "ne_fmath.h"
#include "ne_rng.h"

namespace {

using std::vector;

const float kInf = std::numeric_limits<float>::infinity();
const double kPiD = 3.14159265358979323846264338327950288;     // utils/Math.h:23
const double kTwoPiD = 6.283185307179586476925286766559;       // utils/Math.h:27
const double kInvPiD = 0.31830988618379067154;                 // utils/Math.h:24
const double kInv2PiD = 0.15915494309189533577;                // utils/Math.h:25
const double kFourPiD = 12.566370614359172953850573533118;     // utils/Math.h:28
const double kEpsilonD = 0.0000000001;                         // utils/Math.h:20
const float kInv4Pi = float(0.07957747154594766788);           // utils/Math.h:26
const float kEps3F = float(0.001);                             // EPSILON3 passed as a float tMin
const float kEps12F = float(0.00000000001);                    // EPSILON12 passed as a float tMin
const int kMaxTrackSteps = 1 << 20;
const int kMaxTrSegments = 256;
const int kMaxPassThrough = 1 << 16;

// ---------------------------------------------------------------- glm-like vectors
struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
inline V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(V3 a) { return nefm::fsqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a * (1.0f / nefm::fsqrt(dot(a, a))); }
inline float gmin(float a, float b) { return (b < a) ? b : a; }
inline float gmax(float a, float b) { return (a < b) ? b : a; }
inline double gmaxd(double a, double b) { return (a < b) ? b : a; }
inline V3 vmin(V3 a, V3 b) { return v3(gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return v3(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)); }
inline V3 vabs(V3 a) { return v3(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)); }
inline float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
inline void setc(V3& a, int i, float v) { (i == 0 ? a.x : (i == 1 ? a.y : a.z)) = v; }
inline V3 ld3(const float* p) { return v3(p[0], p[1], p[2]); }
inline bool isBlack(V3 v) { return v.x == 0 && v.y == 0 && v.z == 0; }      // Math.h:641-647
inline bool areAllOne(V3 v) { return v.x == 1 && v.y == 1 && v.z == 1; }    // Math.h:649-651
inline float avg(V3 v) { return (v.x + v.y + v.z) / 3.0f; }                  // Math.h:930-932
inline float absDot(V3 a, V3 b) { return std::fabs(dot(a, b)); }              // Math.h:657-659
inline float maxc(V3 v) { return gmax(gmax(v.x, v.y), v.z); }
inline bool same_bits(V3 a, V3 b) { return memcmp(&a, &b, sizeof(V3)) == 0; }

// glm::mat4 (column-major) times vec4(p, w): (c0 x + c1 y) + (c2 z + c3 w).
inline V3 mul4(const float* m, V3 p, float w) {
  return v3((m[0] * p.x + m[4] * p.y) + (m[8] * p.z + m[12] * w),
            (m[1] * p.x + m[5] * p.y) + (m[9] * p.z + m[13] * w),
            (m[2] * p.x + m[6] * p.y) + (m[10] * p.z + m[14] * w));
}

struct Ray {
  V3 o, d;
  V3 at(float t) const { return o + t * d; }  // primitives/Ray.h:24-26
};

// RayIntersection (primitives/Ray.h:8-15); instance/primitive by index.
struct Hit {
  V3 hitPoint{0, 0, 0}, normal{0, 0, 0};
  float tNear = 0, tFar = 0;
  int inst = -1, prim = -1;
  float u = 0, v = 0;  // RayIntersection::uv
};

struct Sampler {
  nerng::PathKey key;
  uint32_t dim;
  float random() { return nerng::u01(key, dim++); }
};

// utils/Math.h:942-948 transformRay: direction not normalised.
inline Ray transformRay(const Ray& r, const float* m) { return Ray{mul4(m, r.o, 1.0f), mul4(m, r.d, 0.0f)}; }

// utils/Math.h:591-599 generateOrthonormalCS.
inline void orthonormal(V3 n, V3& v, V3& u) {
  if (std::fabs(n.x) > std::fabs(n.y))
    v = v3(-n.z, 0, n.x) / nefm::fsqrt(n.x * n.x + n.z * n.z);
  else
    v = v3(0, n.z, -n.y) / nefm::fsqrt(n.y * n.y + n.z * n.z);
  u = normalize(cross(n, v));
}
// utils/Math.h:612-617 toWorld and :629-631 toLCS.
inline V3 toWorld(V3 v, V3 ns, V3 ss, V3 ts) {
  return v3(ss.x * v.x + ts.x * v.y + ns.x * v.z, ss.y * v.x + ts.y * v.y + ns.y * v.z,
            ss.z * v.x + ts.z * v.y + ns.z * v.z);
}
inline V3 toLCS(V3 v, V3 ns, V3 ss, V3 ts) { return v3(dot(v, ss), dot(v, ts), dot(v, ns)); }
inline bool sameHemisphere(V3 a, V3 b) { return dot(a, b) > 0; }  // Math.h:670-672
inline float powerHeuristic(float p0, float p1) { return (p0 * p0) / (p0 * p0 + p1 * p1); }  // Math.h:751-753

// utils/Math.h:442-457 sampleUnitSphere(e1, e2).
inline V3 sampleUnitSphere(float e1, float e2) {
  float theta = float(kTwoPiD * e1);
  float phi = nefm::acos(1.0f - 2.0f * e2);
  return v3(nefm::sin(phi) * nefm::cos(theta), nefm::sin(phi) * nefm::sin(theta), nefm::cos(phi));
}

// glm::reflect(I, N) = I - N * dot(N, I) * 2.
inline V3 reflect(V3 i, V3 n) { return i - (n * dot(n, i)) * 2.0f; }

// utils/Math.h:1112-1126 convertAreaToSolidAngle.
inline float convertAreaToSolidAngle(float pdfArea, V3 normal, V3 p1, V3 p2) {
  V3 wi = p1 - p2;
  if (dot(wi, wi) == 0) return 0;
  wi = normalize(wi);
  V3 d = p2 - p1;
  pdfArea = pdfArea * (dot(d, d) / absDot(normal, -wi));
  if (nefm::isinf_(pdfArea)) return 0;
  return pdfArea;
}

// utils/Math.h:874-912 getScale (glm::decompose's scale part): columns of the upper
// 3x3, Gram-Schmidt orthogonalised in order.
inline V3 getScale(const float* t) {
  float w = t[15];
  V3 r0 = v3(t[0] / w, t[1] / w, t[2] / w);
  V3 r1 = v3(t[4] / w, t[5] / w, t[6] / w);
  V3 r2 = v3(t[8] / w, t[9] / w, t[10] / w);
  V3 s;
  s.x = length(r0);
  r0 = (r0 * 1.0f) / length(r0);
  float skz = dot(r0, r1);
  r1 = r1 * 1.0f + r0 * (-skz);
  s.y = length(r1);
  r1 = (r1 * 1.0f) / length(r1);
  float sky = dot(r0, r2);
  r2 = r2 * 1.0f + r0 * (-sky);
  float skx = dot(r1, r2);
  r2 = r2 * 1.0f + r1 * (-skx);
  s.z = length(r2);
  return s;
}

// utils/Math.h (convertNormalFromTextureMap, end of file).
inline V3 convertNormalFromTextureMap(V3 texNormal, V3 worldNormal) {
  V3 nts = texNormal * 2.0f - v3(1, 1, 1);
  V3 t = cross(worldNormal, v3(0, 1, 0));
  V3 b = normalize(cross(worldNormal, t));
  V3 r = (t * nts.x + b * nts.y) + worldNormal * nts.z;
  return normalize(r);
}

// ---------------------------------------------------------------- scene
struct BVHNode {
  V3 mn, mx;
  uint32_t start, count, rightOffset;
  bool isLeaf() const { return rightOffset == 0; }
};

struct OModel {
  vector<uint32_t> prims;  // Model::primitives, in BVH order after BVH::init
  vector<BVHNode> nodes;
  uint32_t nodeCount = 0;
};

// Distribution1D (utils/Sampling.h:5-69).
struct ODist1D {
  vector<float> func, cdf;
  float funcInt = 0;
  ODist1D() {}
  ODist1D(const float* f, int n) {  // Sampling.h:12-28
    func.assign(f, f + n);
    cdf.assign(n + 1, 0.0f);
    cdf[0] = 0;
    for (int i = 1; i < n + 1; i++) cdf[i] = cdf[i - 1] + func[i - 1] / n;
    funcInt = cdf[n];
    if (funcInt == 0)
      for (int i = 1; i < n + 1; i++) cdf[i] = float(i) / float(n);
    else
      for (int i = 1; i < n + 1; i++) cdf[i] /= funcInt;
  }
  int count() const { return (int)func.size(); }
  float sampleContinuous(float u, float* pdf, int* off) const {  // Sampling.h:34-51
    // binarySearch (utils/Math.h:1130-1146) over the CDF
    int size = (int)cdf.size(), first = 0, len = size;
    while (len > 0) {
      int half = len >> 1, middle = first + half;
      if (cdf[middle] <= u) {
        first = middle + 1;
        len -= half + 1;
      } else {
        len = half;
      }
    }
    int offset = std::min(std::max(first - 1, 0), size - 2);
    if (off) *off = offset;
    float du = u - cdf[offset];
    if ((cdf[offset + 1] - cdf[offset]) > 0) du /= (cdf[offset + 1] - cdf[offset]);
    if (pdf) *pdf = (funcInt > 0) ? func[offset] / funcInt : 0;
    return (offset + du) / count();
  }
};

// InfiniteAreaLight's texture (RGBA8) and Distribution2D (utils/Sampling.h:71-112).
struct OEnv {
  int W = 0, H = 0;
  vector<uint8_t> texels;
  vector<ODist1D> cond;
  ODist1D marg;
};

}  // namespace

struct orc_scene {
  ne_scene_desc d;
  vector<ne_instance> instances;
  vector<ne_model> models;
  vector<ne_primitive> prims;
  vector<ne_material> materials;
  vector<uint32_t> model_materials;
  vector<ne_light> lights;
  vector<ne_medium> media;
  vector<vector<float>> grids;
  vector<float> invMax;   // GridMedia::invMaxDensity
  vector<V3> sigmaT;      // GridMedia::extinction = absorption + scattering
  vector<float> triArea;  // Triangle::area per primitive
  vector<OModel> omodels;
  vector<OEnv> env;       // per light: InfiniteAreaLight texture and Distribution2D (empty otherwise)
  vector<vector<uint8_t>> albedoTex;  // per material: the RGBA8 albedo texture (empty: constant)
};

namespace {

struct Params {
  int bounces;
  int rr;
  int rr_after;
  nerng::PathKey base;
};

struct Ctx {
  const orc_scene& s;
  Sampler S;
  uint64_t lookups = 0;
};

inline const ne_primitive& P(const orc_scene& s, int i) { return s.prims[i]; }
inline const ne_material* matOf(const orc_scene& s, int prim) {
  if (prim < 0) return nullptr;
  int m = s.prims[prim].material;
  return m < 0 ? nullptr : &s.materials[m];
}

// Material::sampleMaterial (materials/Material.h:62-69) for constant textures.
inline V3 texValue(const ne_material& m, int bit) {
  if (!(m.tex_present & bit)) return v3(0, 0, 0);
  switch (bit) {
    case NE_TEX_ALBEDO: return ld3(m.albedo);
    case NE_TEX_ROUGHNESS: return v3(m.roughness, 0, 0);
    case NE_TEX_METALLIC: return v3(m.metallic, 0, 0);
    case NE_TEX_NORMAL: return ld3(m.normal_map);
  }
  return v3(0, 0, 0);
}

// ---------------------------------------------------------------- primitives (OCS)
// primitives/AABB.cpp:48-80 AABB::intersect.
bool aabbIntersect(V3 mn, V3 mx, const Ray& r, Hit& h) {
  V3 s = v3((r.d.x < 0.0) ? 1.0f : -1.0f, (r.d.y < 0.0) ? 1.0f : -1.0f, (r.d.z < 0.0) ? 1.0f : -1.0f);
  V3 invD = v3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
  V3 size = mx - mn;
  V3 center = mx - size / 2.0f;
  V3 half = size / 2.0f;
  V3 t1 = ((center - r.o) + s * half) * invD;
  V3 t2 = ((center - r.o) - s * half) * invD;
  V3 tmin = vmin(t1, t2);
  V3 tmax = vmax(t1, t2);
  float tNear = gmax(gmax(tmin.x, tmin.y), tmin.z);
  float tFar = gmin(gmin(tmax.x, tmax.y), tmax.z);
  auto sgn = [](float x) { return float((0.0f < x) - (x < 0.0f)); };
  auto step = [](float edge, float x) { return x < edge ? 0.0f : 1.0f; };
  V3 nsg = -v3(sgn(r.d.x), sgn(r.d.y), sgn(r.d.z));
  V3 st1 = v3(step(t1.y, t1.x), step(t1.z, t1.y), step(t1.x, t1.z));
  V3 st2 = v3(step(t1.z, t1.x), step(t1.x, t1.y), step(t1.y, t1.z));
  h.normal = (nsg * st1) * st2;
  h.tNear = tNear;
  h.tFar = tFar;
  h.hitPoint = r.at(h.tNear);
  if (tNear > tFar) {
    h.tNear = kInf;
    h.tFar = -kInf;
    return false;
  }
  return true;
}

// primitives/Sphere.cpp:21-44 Sphere::intersect (returns both roots, even behind).
bool sphereIntersect(const ne_primitive& p, const Ray& r, Hit& h) {
  V3 center = ld3(p.p0);
  V3 oc = r.o - center;
  float a = dot(r.d, r.d);
  float b = dot(oc, r.d);
  float c = dot(oc, oc) - p.radius * p.radius;
  float disc = b * b - a * c;
  if (disc >= 0) {
    float sq = nefm::fsqrt(disc);
    float t1 = (-b - sq) / a;
    float t2 = (-b + sq) / a;
    h.tNear = gmin(t1, t2);
    h.tFar = gmax(t1, t2);
    h.hitPoint = r.at(h.tNear);
    h.normal = normalize((h.hitPoint - center) / p.radius);
    return true;
  }
  return false;
}

// primitives/Rectangle.cpp:16-25 getSize.
inline V3 rectSize(V3 v0, V3 v1) {
  for (int i = 0; i < 3; i++)
    if (comp(v0, i) == comp(v1, i)) { setc(v0, i, 0); setc(v1, i, 0); }
  return vabs(v0) + vabs(v1);
}

// primitives/Rectangle.cpp:91-113 Rectangle::barycentricCoordinates: (lambda, 0) in the
// triangle (a, b, c), or (lambda, 1) in (d, b, c) when the first leaves [0, 1].
void rectBarycentric(V3 p, V3 a, V3 b, V3 c, V3 d, float lambda[3], int& second) {
  float t1[3], t2[3];
  V3 v0 = b - a, v1 = c - a, v2 = p - a;
  float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
  float denom = d00 * d11 - d01 * d01;
  t1[1] = (d11 * d20 - d01 * d21) / denom;
  t1[2] = (d00 * d21 - d01 * d20) / denom;
  t1[0] = 1.0f - t1[1] - t1[2];
  v0 = b - d, v1 = c - d, v2 = p - d;
  d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
  denom = d00 * d11 - d01 * d01;
  t2[1] = (d11 * d20 - d01 * d21) / denom;
  t2[2] = (d00 * d21 - d01 * d20) / denom;
  t2[0] = 1.0f - t2[1] - t2[2];
  second = (t1[0] < 0 || t1[1] < 0 || t1[2] < 0 || t1[0] > 1 || t1[1] > 1 || t1[2] > 1) ? 1 : 0;
  for (int k = 0; k < 3; k++) lambda[k] = second ? t2[k] : t1[k];
}
// primitives/Rectangle.cpp:115-157 Rectangle::samplePointOnTexture for the corners SceneReader
// lays out (io/SceneReader.cpp:407-463): vertex 0 = p0 with uv (0,0), 1 = (p1.x, p0.y, p0.z)
// with (1,0), 2 = p1 with (1,1), 3 = (p0.x, p1.y, p0.z) with (0,1).
void rectSamplePointOnTexture(const ne_primitive& p, V3 q, float& u, float& v) {
  V3 c0 = ld3(p.p0), c2 = ld3(p.p1);
  V3 c1 = v3(c2.x, c0.y, c0.z), c3 = v3(c0.x, c2.y, c0.z);
  const float uv[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
  float l[3];
  int second;
  rectBarycentric(q, c0, c1, c2, c3, l, second);
  const float* first = second ? uv[3] : uv[0];
  u = (l[0] * first[0] + l[1] * uv[1][0]) + l[2] * uv[2][0];
  v = (l[0] * first[1] + l[1] * uv[1][1]) + l[2] * uv[2][1];
}

// primitives/Rectangle.cpp:50-76 Rectangle::intersect and :32-48 containsPoint.
bool rectIntersect(const ne_primitive& p, const Ray& r, Hit& h) {
  V3 v0 = ld3(p.p0), v1 = ld3(p.p1), n = ld3(p.p2);
  float denom = dot(n, r.d);
  if ((double)std::fabs(denom) < kEpsilonD) return false;
  float num = dot(n, v1 - r.o);
  float t = num / denom;
  if (t < 0) return false;
  V3 q = r.at(t);
  V3 mn = vmin(v0, v1), mx = vmax(v0, v1), size = rectSize(v0, v1);
  if (size.x > 0 && (q.x < mn.x || q.x > mx.x)) return false;
  if (size.y > 0 && (q.y < mn.y || q.y > mx.y)) return false;
  if (size.z > 0 && (q.z < mn.z || q.z > mx.z)) return false;
  h.tNear = t;
  h.tFar = t;
  h.normal = n;
  h.hitPoint = q;
  rectSamplePointOnTexture(p, q, h.u, h.v);
  return true;
}

// primitives/Triangle.cpp:49-80 Triangle::intersect. denom = 1.0 / dot is a double
// division rounded to float, which equals the float division 1.0f / dot exactly.
bool triIntersect(const orc_scene& s, const ne_primitive& p, const Ray& r, Hit& h) {
  V3 a = ld3(p.p0), b = ld3(p.p1), c = ld3(p.p2);
  V3 v1v0 = b - a, v2v0 = c - a, rov0 = r.o - a;
  V3 normal = cross(v1v0, v2v0);
  V3 q = cross(rov0, r.d);
  float denom = (float)(1.0 / (double)dot(r.d, normal));
  float u = dot(-q, v2v0) * denom;
  float v = dot(q, v1v0) * denom;
  float t = dot(-normal, rov0) * denom;
  if (nefm::isnan_(t) || t < 0) return false;
  if (u < 0.0f || u > 1.0f || v < 0.0f || (u + v) > 1.0f) return false;
  h.tNear = t;
  h.tFar = t;
  h.hitPoint = r.at(h.tNear);
  const ne_material* m = p.material >= 0 ? &s.materials[p.material] : nullptr;
  if (m && (m->tex_types & NE_TEX_NORMAL))
    h.normal = convertNormalFromTextureMap(texValue(*m, NE_TEX_NORMAL), normalize(normal));
  else
    h.normal = normalize(normal);
  return true;
}

bool primIntersect(const orc_scene& s, int idx, const Ray& r, Hit& h) {
  const ne_primitive& p = s.prims[idx];
  bool hit = false;
  // uv (0, 0) unless the primitive computes it (Sphere.cpp:37, AABB.cpp:68; a triangle without
  // texture coordinates, Triangle.cpp:121-123)
  h.u = 0;
  h.v = 0;
  switch (p.type) {
    case NE_PRIM_SPHERE: hit = sphereIntersect(p, r, h); break;
    case NE_PRIM_RECTANGLE: hit = rectIntersect(p, r, h); break;
    case NE_PRIM_AABB: hit = aabbIntersect(ld3(p.p0), ld3(p.p1), r, h); h.prim = idx; return hit;
    case NE_PRIM_TRIANGLE: hit = triIntersect(s, p, r, h); break;
    default: return false;  // Point::intersect (primitives/Point.cpp:10-12)
  }
  if (hit) h.prim = idx;
  return hit;
}

inline void triBounds(const ne_primitive& p, V3& mn, V3& mx) {  // Triangle.cpp:10-13 calculateAABB
  V3 a = ld3(p.p0), b = ld3(p.p1), c = ld3(p.p2);
  mn = vmin(a, vmin(b, c));
  mx = vmax(a, vmax(b, c));
}
inline V3 boxCenter(V3 mn, V3 mx) { return mx - (mx - mn) / 2.0f; }  // AABB::getCenter

// primitives/BVH.cpp:6-106 BVH::init (midpoint split on the longest centroid axis).
void bvhInit(const orc_scene& s, OModel& om) {
  const uint32_t perLeaf = 4, notVisited = 0xffffffffu, visitedTwice = 0xfffffffdu, rootParent = 0xfffffffcu;
  struct Item { uint32_t parent, start, end; };
  om.nodes.assign(om.prims.size() * 2 + 1, BVHNode{});
  vector<Item> stack;
  om.nodeCount = 0;
  stack.push_back(Item{rootParent, 0, (uint32_t)om.prims.size()});
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    om.nodeCount++;
    BVHNode node;
    node.start = it.start;
    node.count = it.end - it.start;
    node.rightOffset = notVisited;
    V3 bbMin = v3(kInf, kInf, kInf), bbMax = v3(-kInf, -kInf, -kInf);
    V3 pmn, pmx;
    triBounds(s.prims[om.prims[node.start]], pmn, pmx);
    bbMin = vmin(bbMin, pmn);
    bbMax = vmax(bbMax, pmx);
    V3 bcMin = boxCenter(bbMin, bbMax), bcMax = bcMin;
    for (uint32_t i = it.start + 1; i < it.end; i++) {
      triBounds(s.prims[om.prims[i]], pmn, pmx);
      bbMin = vmin(bbMin, pmn);
      bbMax = vmax(bbMax, pmx);
      V3 c = boxCenter(pmn, pmx);
      bcMin = vmin(bcMin, c);
      bcMax = vmax(bcMax, c);
    }
    node.mn = bbMin;
    node.mx = bbMax;
    if (node.count <= perLeaf) node.rightOffset = 0;
    om.nodes[om.nodeCount - 1] = node;
    if (it.parent != rootParent) {
      om.nodes[it.parent].rightOffset--;
      if (om.nodes[it.parent].rightOffset == visitedTwice) om.nodes[it.parent].rightOffset = om.nodeCount - 1 - it.parent;
    }
    if (node.rightOffset == 0) continue;
    V3 ext = bcMax - bcMin;
    int dim = 0;
    if (comp(ext, 1) > comp(ext, dim)) dim = 1;
    if (comp(ext, 2) > comp(ext, dim)) dim = 2;
    float split = 0.5f * (comp(bcMin, dim) + comp(bcMax, dim));
    uint32_t mid = it.start;
    for (uint32_t i = it.start; i < it.end; i++) {
      triBounds(s.prims[om.prims[i]], pmn, pmx);
      if (comp(boxCenter(pmn, pmx), dim) < split) {
        std::swap(om.prims[i], om.prims[mid]);
        mid++;
      }
    }
    if (mid == it.start || mid == it.end) mid = it.start + (it.end - it.start) / 2;
    stack.push_back(Item{om.nodeCount - 1, mid, it.end});
    stack.push_back(Item{om.nodeCount - 1, it.start, mid});
  }
}

// primitives/BVH.cpp:108-193 BVH::intersect (near-first stack traversal).
bool bvhIntersect(const orc_scene& s, const OModel& om, const Ray& r, Hit& out) {
  struct T { uint32_t node; float tNear; };
  T todo[128];
  int sp = 0;
  todo[0] = T{0, kInf};
  Hit closest;
  closest.tNear = kInf;
  closest.tFar = -kInf;
  bool anyHit = false;
  while (sp >= 0) {
    uint32_t ni = todo[sp].node;
    float nearest = todo[sp].tNear;
    sp--;
    const BVHNode& node = om.nodes[ni];
    if (nearest > closest.tNear) continue;
    if (node.isLeaf()) {
      for (uint32_t i = 0; i < node.count; i++) {
        Hit tmp;
        bool cur = primIntersect(s, om.prims[node.start + i], r, tmp);
        anyHit = anyHit || cur;
        if (cur && tmp.tNear < closest.tNear) closest = tmp;
      }
    } else {
      Hit lh, rh;
      uint32_t c0 = ni + 1, c1 = ni + node.rightOffset;
      bool h0 = aabbIntersect(om.nodes[c0].mn, om.nodes[c0].mx, r, lh);
      bool h1 = aabbIntersect(om.nodes[c1].mn, om.nodes[c1].mx, r, rh);
      if (h0 && h1) {
        uint32_t closer = c0, other = c1;
        if (rh.tNear < lh.tNear) {
          std::swap(lh, rh);
          std::swap(closer, other);
        }
        if (sp + 2 >= 128) break;  // deeper than any tree the builders make (the device stops at 64)
        todo[++sp] = T{other, rh.tNear};
        todo[++sp] = T{closer, lh.tNear};
      } else if (h0) {
        if (sp + 1 >= 128) break;
        todo[++sp] = T{c0, lh.tNear};
      } else if (h1) {
        if (sp + 1 >= 128) break;
        todo[++sp] = T{c1, rh.tNear};
      }
    }
  }
  out = closest;
  return anyHit;
}

const ne_light& lightOfMaterial(const orc_scene& s, int mat) { return s.lights[s.materials[mat].light]; }

// Texture::sample, NE_TEX_SAMPLER_UVW_MIRROR, nearest (materials/Texture.cpp:88-129): one
// coordinate. Not-a-number or beyond the int range (undefined in the reference): texel 0.
int texCoord(float u, int n) {
  if (!(u >= -2147483520.0f && u <= 2147483520.0f)) return 0;
  u = gmin(gmax(std::fabs(u - (int)u), 0.0f), 1.0f);
  int x = (int)(u * n);
  if (x > 0 && x == n) x--;
  return x;
}
// RGBA8 texel as Texture::sampleAtIndex reads it (Texture.cpp:69-81), RGB.
V3 envTexel(const OEnv& e, float u, float v) {
  const uint8_t* p = &e.texels[4 * ((size_t)texCoord(v, e.H) * e.W + texCoord(u, e.W))];
  return v3(p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f);
}
// getSphericalPhi / getSphericalTheta (utils/Math.h:1148-1155).
float sphericalPhi(V3 v) {
  float p = nefm::atan2(v.y, v.x);
  return (p < 0) ? (float)(p + kTwoPiD) : p;
}
float sphericalTheta(V3 v) { return nefm::acos(gmin(gmax(v.z, -1.0f), 1.0f)); }
// InfiniteAreaLight::Le (lights/InfiniteAreaLight.h:46-55).
V3 envLe(const OEnv& e, const float* M, V3 d) {
  V3 w = normalize(mul4(M, d, 0.0f));
  V3 normal = v3(0, 0, 1), ss, ts;
  orthonormal(normal, ss, ts);
  V3 incoming = toLCS(w, normal, ss, ts);
  float stx = (float)(sphericalPhi(incoming) * kInv2PiD), sty = (float)(sphericalTheta(incoming) * kInvPiD);
  return envTexel(e, stx, sty);
}
const OEnv* envOf(const orc_scene& s, const ne_light& L) {
  size_t i = &L - s.lights.data();
  return (i < s.env.size() && s.env[i].W > 0) ? &s.env[i] : nullptr;
}
// Light::Le(ray, M) (lights/Light.h:20-22), DirectionalLight::Le (DirectionalLight.cpp:4-6),
// InfiniteAreaLight::Le (InfiniteAreaLight.h:46-55; a constant map without a texture).
inline V3 lightLe(const orc_scene& s, const ne_light& L, const float* M, V3 d) {
  if (L.type == NE_LIGHT_INFINITE) {
    if (const OEnv* e = envOf(s, L)) return envLe(*e, M, d);
    return ld3(L.env_radiance);
  }
  return ld3(L.le);
}
const float kIdentity16[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};  // glm::mat4(1)
// Light::Li / DirectionalLight::Li (returns le) / InfiniteAreaLight::Li.
inline V3 lightLi(const ne_light& L) {
  if (L.type == NE_LIGHT_DIRECTIONAL) return ld3(L.le);
  return ld3(L.li);
}

// primitives/Model.cpp:372-447 Model::intersect (ray in OCS, tMin/tMax by reference).
bool modelIntersect(const orc_scene& s, uint32_t mi, const Ray& ray, Hit& hit, float& tMin, float& tMax) {
  const ne_model& m = s.models[mi];
  bool did = false;
  Hit temp;
  if (m.has_bbox)
    if (!aabbIntersect(ld3(m.bbox_min), ld3(m.bbox_max), ray, temp)) return false;
  const OModel& om = s.omodels[mi];
  if (m.use_bvh && om.nodeCount > 0) {
    bool local = bvhIntersect(s, om, ray, temp);
    if (local && temp.tNear > tMin && temp.tNear < tMax) {
      tMax = temp.tNear;
      hit = temp;
      did = true;
    }
    return did;
  }
  for (uint32_t k = 0; k < om.prims.size(); k++) {
    int pi = (int)om.prims[k];
    const ne_primitive& p = s.prims[pi];
    if (p.material >= 0 && s.materials[p.material].medium >= 0 &&
        s.media[s.materials[p.material].medium].type == NE_MEDIUM_GRID) {
      primIntersect(s, pi, ray, temp);
      float rx = gmax(0.0f, temp.tNear), ry = temp.tFar;
      if (rx <= ry && !nefm::isinf_(ry) && !nefm::isinf_(rx)) {
        temp.prim = pi;
        temp.tNear = rx;
        temp.tFar = ry;
        temp.hitPoint = ray.at(rx);
        temp.normal = -ray.d;
        tMax = temp.tNear;
        hit = temp;
        did = true;
      }
      continue;
    }
    bool local = primIntersect(s, pi, ray, temp);
    if (local && temp.tNear != temp.tFar && temp.tNear < 0 && temp.tFar > 0) {
      temp.tNear = 0;
      temp.hitPoint = ray.o;
      tMax = temp.tNear;
      hit = temp;
      did = true;
    }
    if (local && temp.tNear > tMin && temp.tNear < tMax) {
      tMax = temp.tNear;
      hit = temp;
      did = true;
    }
  }
  for (uint32_t k = 0; k < m.light_count; k++) {
    int pi = (int)(m.light_begin + k);
    const ne_primitive& p = s.prims[pi];
    if (!isBlack(lightLe(s, lightOfMaterial(s, p.material), kIdentity16, ray.d))) continue;  // Model.cpp:435
    bool local = primIntersect(s, pi, ray, temp);
    if (local && temp.tNear > tMin && temp.tNear < tMax) {
      tMax = temp.tNear;
      hit = temp;
      did = true;
    }
  }
  return did;
}

// primitives/InstancedModel.cpp:24-38 InstancedModel::intersect.
bool instanceIntersect(const orc_scene& s, uint32_t ii, const Ray& ray, Hit& hit, float& tMin, float& tMax) {
  const ne_instance& in = s.instances[ii];
  if (!in.collision) return false;
  Ray r = transformRay(ray, in.to_ocs);
  bool did = modelIntersect(s, in.model, r, hit, tMin, tMax);
  if (did) {
    hit.hitPoint = mul4(in.to_wcs, hit.hitPoint, 1.0f);
    hit.normal = normalize(mul4(in.to_wcs, hit.normal, 0.0f));
    hit.inst = (int)ii;
  }
  return did;
}

// core/Scene.cpp:30-56 Scene::intersectScene.
bool intersectScene(Ctx& c, const Ray& ray, Hit& hit, float tMin, float tMax) {
  const orc_scene& s = c.s;
  bool did = false;
  hit.prim = -1;
  Hit temp;
  float curMin = tMin, curMax = tMax;
  uint32_t total = s.d.n_instances + s.d.n_light_instances;
  for (uint32_t i = 0; i < total; i++) {
    bool t = instanceIntersect(s, i, ray, temp, curMin, curMax);
    if (t) hit = temp;
    did = did || t;
  }
  return did;
}

// ---------------------------------------------------------------- materials
// core/Microfacet.cpp:5-14 GGXDistribution::D.
inline float ggxD(float alpha, V3 m) {
  float a2 = alpha * alpha;
  float NdotH = m.z;
  float NdotH2 = NdotH * NdotH;
  float denom = NdotH2 * (a2 - 1.0f) + 1.0f;
  denom = (float)gmaxd(kEpsilonD, kPiD * (double)denom * (double)denom);
  return a2 / denom;
}
// core/Microfacet.cpp:16-23 geometrySchlickGGX.
inline float schlickGGX(float alpha, float NdotV) {
  float k = alpha / 2.0f;
  float nom = NdotV;
  float denom = (float)gmaxd(kEpsilonD, (double)NdotV * (1.0 - (double)k) + (double)k);
  return nom / denom;
}
// core/Microfacet.cpp:25-35 GGXDistribution::G.
inline float ggxG(float alpha, V3 wi, V3 wo) {
  V3 n = normalize(wi + wo);
  float NoV = dot(n, wi), NoL = dot(n, wo);
  float NdotV = gmax(NoV, 0.0f), NdotL = gmax(NoL, 0.0f);
  return schlickGGX(alpha, NdotV) * schlickGGX(alpha, NdotL);
}
// core/Microfacet.cpp:37-56 sampleMicrofacet + sample.
inline V3 ggxSample(float alpha, V3 wi, Sampler& S) {
  float rx = S.random();
  float ry = S.random();
  float a2 = alpha * alpha;
  float theta = nefm::acos(gmin(1.0f, nefm::fsqrt((1.0f - rx) / gmax(float(kEpsilonD), (rx * (a2 - 1.0f) + 1.0f)))));
  float phi = (float)(kTwoPiD * (double)ry);
  V3 m = v3(nefm::sin(theta) * nefm::cos(phi), nefm::sin(theta) * nefm::sin(phi), nefm::cos(theta));
  return reflect(normalize(wi), normalize(m));
}
// core/Microfacet.cpp:58-65 GGXDistribution::pdf.
inline float ggxPdf(float alpha, V3 scattered, V3 m) {
  float NdotH = m.z;
  float VdotH = dot(scattered, m);
  float Dp = ggxD(alpha, m) * NdotH;
  return Dp / (4 * VdotH);
}
// core/BSDF.h:150-157 FresnelSchilck::eval.
inline V3 fresnel(float cosTheta) {
  V3 f0 = v3(0.04f, 0.04f, 0.04f);
  return f0 + (v3(1, 1, 1) - f0) * nefm::pow5(1.0f - cosTheta);
}
// core/GlossyBSDF.cpp:25-48 GlossyBSDF::eval (alpha = roughness^2 at every call).
V3 glossyEval(const ne_material& m, V3 wi, V3 wo, V3 albedo) {
  float rough = texValue(m, NE_TEX_ROUGHNESS).x;
  float alpha = rough * rough;
  V3 H = normalize(wi + wo);
  float HdotV = dot(wi, H);
  float NdotV = wi.z, NdotL = wo.z;
  float D = ggxD(alpha, H);
  float G = ggxG(alpha, wi, wo);
  V3 F = fresnel(HdotV);
  V3 numerator = (D * G) * F;
  float denominator = (4.0f * gmax(NdotV, 0.0f)) * gmax(NdotL, 0.0f);
  V3 specular = numerator / gmax(denominator, float(kEpsilonD));
  V3 kD = v3(1, 1, 1) - F;
  float metallic = texValue(m, NE_TEX_METALLIC).x;
  kD = kD * (float)(1.0 - (double)metallic);
  return ((albedo / float(kPiD)) * kD + specular) * NdotL;
}
inline float glossyPdf(const ne_material& m, V3 wi, V3 wo) {  // GlossyBSDF.cpp:17-23
  V3 mh = normalize(wi + wo);
  float rough = texValue(m, NE_TEX_ROUGHNESS).x;
  return ggxPdf(rough * rough, wo, mh);
}
inline V3 glossySample(const ne_material& m, V3 wi, Sampler& S) {  // GlossyBSDF.cpp:10-15
  float rough = texValue(m, NE_TEX_ROUGHNESS).x;
  return ggxSample(rough * rough, wi, S);
}

// materials/Medium.h:116-128 HG::pdf / HG::eval (identical), :56-62 isotropic.
inline float phaseEval(const ne_material& m, V3 wi, V3 wo) {
  if (m.phase == NE_PHASE_ISOTROPIC) return (float)(1.0 / kFourPiD);
  float g = m.g;
  float cosT = dot(normalize(wi), normalize(wo));
  float denom = (1.0f + g * g) - (2.0f * g) * cosT;
  return (kInv4Pi * (1.0f - g * g)) / (denom * nefm::fsqrt(denom));
}
// materials/Medium.h:96-114 HG::sample (ignores the incoming direction), :45-47 isotropic.
inline V3 phaseSample(const ne_material& m, Sampler& S) {
  if (m.phase == NE_PHASE_ISOTROPIC) {
    float e1 = S.random();
    float e2 = S.random();
    return sampleUnitSphere(e1, e2);
  }
  float g = m.g;
  float u0 = S.random();
  float u1 = S.random();
  float cosTheta;
  if (std::fabs(g) < 1e-3f)
    cosTheta = 1.0f - 2.0f * u0;
  else {
    float sqr = (1.0f - g * g) / ((1.0f + g) - (2.0f * g) * u0);
    sqr = sqr * sqr;
    cosTheta = (-1.0f / (2.0f * g)) * ((1.0f + g * g) - sqr);
  }
  float sinTheta = nefm::fsqrt(1.0f - cosTheta * cosTheta);
  float phi = (float)((2.0f * kPiD) * (double)u1);
  return v3(nefm::cos(phi) * sinTheta, nefm::sin(phi) * sinTheta, cosTheta);
}

// core/BSDF.h:100-106 BSDF::sample.
V3 bsdfSample(const ne_material& m, V3 incoming, V3 normal, Sampler& S) {
  V3 ss, ts;
  orthonormal(normal, ss, ts);
  V3 wi = toLCS(-normalize(incoming), normal, ss, ts);
  V3 sc = (m.bsdf == NE_BSDF_VOLUME) ? phaseSample(m, S) : glossySample(m, wi, S);
  return toWorld(sc, normal, ss, ts);
}
// core/BSDF.h:117-125 BSDF::pdf.
float bsdfPdf(const ne_material& m, V3 incoming, V3 scattered, V3 normal) {
  bool trans = (m.bsdf == NE_BSDF_VOLUME);
  if (!trans && (!sameHemisphere(-incoming, normal) || !sameHemisphere(scattered, normal))) return 0;
  V3 ss, ts;
  orthonormal(normal, ss, ts);
  V3 wi = toLCS(-normalize(incoming), normal, ss, ts);
  V3 wo = toLCS(scattered, normal, ss, ts);
  return trans ? phaseEval(m, wi, wo) : glossyPdf(m, wi, wo);
}
// core/BSDF.h:135-142 BSDF::eval (frame of ri.normal).
// Material::sampleMaterial(ALBEDO, ri.uv) (materials/Material.h:62-69) as GlossyBSDF::eval reads
// it (GlossyBSDF.cpp:44): the texture at the hit's uv (Texture::sample, mirror wrap and
// nearest texel), or the constant.
V3 albedoOf(const orc_scene& s, const ne_material& m, const Hit& isect) {
  size_t mi = (size_t)(&m - s.materials.data());
  if (m.albedo_width > 0 && mi < s.albedoTex.size() && !s.albedoTex[mi].empty()) {
    const uint8_t* t = &s.albedoTex[mi][4 * ((size_t)texCoord(isect.v, m.albedo_height) * m.albedo_width +
                                             texCoord(isect.u, m.albedo_width))];
    return v3(t[0] / 255.0f, t[1] / 255.0f, t[2] / 255.0f);
  }
  return texValue(m, NE_TEX_ALBEDO);
}
// core/BSDF.h:135-142 for the intersection `isect`.
V3 bsdfEval(const orc_scene& s, const ne_material& m, V3 incoming, V3 scattered, const Hit& isect) {
  const V3 normal = isect.normal;
  bool trans = (m.bsdf == NE_BSDF_VOLUME);
  if (!trans && (!sameHemisphere(-incoming, normal) || !sameHemisphere(scattered, normal))) return v3(0, 0, 0);
  V3 ss, ts;
  orthonormal(normal, ss, ts);
  V3 wi = toLCS(-normalize(incoming), normal, ss, ts);
  V3 wo = toLCS(scattered, normal, ss, ts);
  if (trans) {
    float p = phaseEval(m, wi, wo);
    return v3(p, p, p);
  }
  return glossyEval(m, wi, wo, albedoOf(s, m, isect));
}

// ---------------------------------------------------------------- media
// materials/GridMedia.cpp:15-21 density and :25-39 interpolatedDensity.
inline float gridDensity(const orc_scene& s, int med, float gx, float gy, float gz) {
  const ne_medium& M = s.media[med];
  if (gx >= (float)M.res[0] || gy >= (float)M.res[1] || gz >= (float)M.res[2]) return 0;
  uint32_t x = (uint32_t)(int)gx, y = (uint32_t)(int)gy, z = (uint32_t)(int)gz;
  return s.grids[med][M.res[1] * M.res[0] * z + M.res[0] * y + x];
}
inline float lerp(float a, float b, float t) { return a * (1.0f - t) + b * t; }
float interpolatedDensity(Ctx& c, int med, V3 g) {
  const ne_medium& M = c.s.media[med];
  c.lookups++;
  V3 res = v3((float)M.res[0], (float)M.res[1], (float)M.res[2]);
  g = vmin(vmax(v3(0, 0, 0), g), res);
  int ix = (int)nefm::ffloor(g.x), iy = (int)nefm::ffloor(g.y), iz = (int)nefm::ffloor(g.z);
  V3 d = g - v3((float)ix, (float)iy, (float)iz);
  float fx = (float)ix, fy = (float)iy, fz = (float)iz;
  const orc_scene& s = c.s;
  float d00 = lerp(gridDensity(s, med, fx, fy, fz), gridDensity(s, med, fx + 1, fy, fz), d.x);
  float d10 = lerp(gridDensity(s, med, fx, fy + 1, fz), gridDensity(s, med, fx + 1, fy + 1, fz), d.x);
  float d01 = lerp(gridDensity(s, med, fx, fy, fz + 1), gridDensity(s, med, fx + 1, fy, fz + 1), d.x);
  float d11 = lerp(gridDensity(s, med, fx, fy + 1, fz + 1), gridDensity(s, med, fx + 1, fy + 1, fz + 1), d.x);
  float d0 = lerp(d00, d10, d.y);
  float d1 = lerp(d01, d11, d.y);
  return lerp(d0, d1, d.z);
}
// materials/GridMedia.cpp:41-43 sampleAt with GridMedia.h:33-35 fromOCStoGCS.
inline float sampleAt(Ctx& c, int med, const Ray& r, float t) {
  const ne_medium& M = c.s.media[med];
  V3 p = r.at(t);
  V3 res = v3((float)M.res[0], (float)M.res[1], (float)M.res[2]);
  return interpolatedDensity(c, med, (p + v3(0.5f, 0.5f, 0.5f)) * res);
}

// materials/GridMedia.cpp:45-69 GridMedia::Tr (ratio tracking with Russian roulette).
V3 gridTr(Ctx& c, int med, Ray incoming, Hit isect) {
  const orc_scene& s = c.s;
  incoming = transformRay(incoming, s.instances[isect.inst].to_ocs);
  incoming.o = incoming.at(isect.tNear);
  isect.tFar = isect.tFar - isect.tNear;
  isect.tNear = 0;
  float invMax = s.invMax[med];
  float mu = avg(s.sigmaT[med] * s.media[med].density);
  float Tr = 1, t = isect.tNear;
  for (int step = 0; step < kMaxTrackSteps; step++) {
    t -= (nefm::log(1 - c.S.random()) * invMax) / mu;
    if (t >= isect.tFar) break;
    float density = sampleAt(c, med, incoming, t);
    Tr *= 1 - std::max(0.0f, density * invMax);
    const float rrThreshold = .1f;
    if (Tr < rrThreshold) {
      float q = std::max(0.05f, 1.0f - Tr);
      if (c.S.random() < q) return v3(0, 0, 0);
      Tr /= 1 - q;
    }
  }
  return v3(Tr, Tr, Tr);
}

// materials/GridMedia.cpp:71-99 GridMedia::sample (delta tracking).
V3 gridSample(Ctx& c, int med, Ray incoming, Ray& scattered, const Hit& isect) {
  const orc_scene& s = c.s;
  scattered.o = incoming.o;
  scattered.d = incoming.d;
  const ne_instance& in = s.instances[isect.inst];
  incoming = transformRay(incoming, in.to_ocs);
  float invMax = s.invMax[med];
  float mu = avg(s.sigmaT[med] * s.media[med].density);
  float t = isect.tNear;
  for (int step = 0; step < kMaxTrackSteps; step++) {
    float r = c.S.random();
    float sampledDist = (nefm::log(1 - r) * invMax) / mu;
    t -= sampledDist;
    if (t >= isect.tFar) {
      scattered.o = incoming.at(isect.tFar + 0.0001f);
      break;
    }
    float density = sampleAt(c, med, incoming, t);
    float ra = c.S.random();
    if (density * invMax > ra) {
      scattered.o = incoming.at(t);
      const ne_material& m = *matOf(s, isect.prim);
      scattered.d = bsdfSample(m, incoming.d, v3(0, 1, 0), c.S);
      scattered = transformRay(scattered, in.to_wcs);
      return ld3(s.media[med].sigma_s) / s.sigmaT[med];
    }
  }
  return v3(1, 1, 1);
}

// materials/HomogeneousMedia.cpp:15-51.
inline V3 homogTr(const orc_scene& s, int med, float distance) {
  V3 v = (s.sigmaT[med] * distance) * s.media[med].density;
  return v3(nefm::exp(-v.x), nefm::exp(-v.y), nefm::exp(-v.z));
}
V3 homogSample(Ctx& c, int med, Ray incoming, Ray& scattered, const Hit& isect) {
  const orc_scene& s = c.s;
  float t = (-nefm::log(1 - c.S.random())) / avg(s.sigmaT[med]);
  float dist = isect.tFar - isect.tNear;
  t = t / dist;
  bool sampled = t < dist;
  if (sampled) {
    scattered.o = incoming.at(t);
    scattered.d = bsdfSample(*matOf(s, isect.prim), incoming.d, isect.normal, c.S);
  } else {
    scattered.o = incoming.at(dist + 0.001f);
    scattered.d = incoming.d;
  }
  V3 Tr = homogTr(s, med, t);
  V3 density = sampled ? (s.sigmaT[med] * Tr) : Tr;
  float pdf = avg(density);
  if (pdf == 0) pdf = 1;
  return sampled ? ((Tr * ld3(s.media[med].sigma_s)) / pdf) : Tr / pdf;
}

V3 mediumTr(Ctx& c, int med, const Ray& r, const Hit& isect) {
  if (c.s.media[med].type == NE_MEDIUM_GRID) return gridTr(c, med, r, isect);
  return homogTr(c.s, med, isect.tFar - isect.tNear);
}
V3 mediumSample(Ctx& c, int med, const Ray& r, Ray& scattered, const Hit& isect) {
  if (c.s.media[med].type == NE_MEDIUM_GRID) return gridSample(c, med, r, scattered, isect);
  return homogSample(c, med, r, scattered, isect);
}

// ---------------------------------------------------------------- lights
// Primitive::samplePointOnSurface: Rectangle.cpp:78-88, Sphere.cpp:46-52, Triangle.cpp:114-119,
// Point.cpp:14-18, AABB.cpp:81-83.
V3 samplePointOnSurface(const orc_scene& s, int pi, const Hit& isect, const float* M, Sampler& S) {
  const ne_primitive& p = s.prims[pi];
  switch (p.type) {
    case NE_PRIM_RECTANGLE: {
      float e0 = S.random();
      float e1 = S.random();
      float e2 = S.random();
      V3 v0 = ld3(p.p0);
      V3 size = rectSize(ld3(p.p0), ld3(p.p1));
      V3 q = v3(v0.x + size.x * e0, v0.y + size.y * e1, v0.z + size.z * e2);
      return mul4(M, q, 1.0f);
    }
    case NE_PRIM_SPHERE: {
      V3 c = mul4(M, ld3(p.p0), 1.0f);
      V3 n = normalize(isect.hitPoint - c);
      return c + n * p.radius;
    }
    case NE_PRIM_TRIANGLE: {
      float ex = S.random();
      float ey = S.random();
      float sq = nefm::fsqrt(ex);
      float a = 1.0f - sq, b = ey * sq;
      return (a * ld3(p.p0) + b * ld3(p.p1)) + ((1 - a) - b) * ld3(p.p2);
    }
    case NE_PRIM_POINT: return mul4(M, ld3(p.p0), 1.0f);
    default: return v3(0, 0, 0);
  }
}
// Primitive::pdf: Rectangle.cpp:159-171, Sphere.cpp:58-68, Triangle.cpp:159-161, Point/AABB = 1.
float primPdf(const orc_scene& s, int pi, const Hit& isect, const float* M, Sampler& S) {
  const ne_primitive& p = s.prims[pi];
  switch (p.type) {
    case NE_PRIM_RECTANGLE: {
      V3 size = rectSize(ld3(p.p0), ld3(p.p1));
      V3 sizeWCS = getScale(M) * size;
      float area = 1;
      for (int i = 0; i < 3; i++)
        if (comp(sizeWCS, i) != 0) area = area * comp(sizeWCS, i);
      return convertAreaToSolidAngle(1.0f / area, isect.normal, isect.hitPoint,
                                     samplePointOnSurface(s, pi, isect, M, S));
    }
    case NE_PRIM_SPHERE: {
      float pdfArea = (float)((double)(1.0f / 4.0f) * kPiD * (double)p.radius * (double)p.radius);
      return convertAreaToSolidAngle(pdfArea, isect.normal, isect.hitPoint, samplePointOnSurface(s, pi, isect, M, S));
    }
    case NE_PRIM_TRIANGLE:
      return convertAreaToSolidAngle(1.0f / s.triArea[pi], isect.normal, isect.hitPoint,
                                     samplePointOnSurface(s, pi, isect, M, S));
    default: return 1;
  }
}

// Light::sampleLi: DiffuseLight.cpp:8-20, DirectionalLight.cpp:12-18,
// InfiniteAreaLight.h:83-113 (1x1 map: Distribution2D returns u unchanged).
V3 sampleLi(const orc_scene& s, const ne_light& L, const Hit& isect, const float* M, Ray& wo, float& pdf, Sampler& S) {
  switch (L.type) {
    case NE_LIGHT_DIFFUSE: {
      wo.o = isect.hitPoint;
      V3 q = samplePointOnSurface(s, L.primitive, isect, M, S);
      V3 d = q - wo.o;
      wo.d = normalize(d);
      pdf = primPdf(s, L.primitive, isect, M, S);
      return ld3(L.li);
    }
    case NE_LIGHT_DIRECTIONAL:
      wo.o = isect.hitPoint;
      wo.d = -ld3(L.direction);
      pdf = 1;
      return ld3(L.li);
    default: {
      float u0 = S.random();
      float u1 = S.random();
      const OEnv* e = envOf(s, L);
      float uv0 = u0, uv1 = u1, mapPdf = L.env_map_pdf;  // the 1x1 map returns u with pdf 1 (or 0)
      if (e) {  // Distribution2D::sampleContinuous (Sampling.h:98-105)
        float pdfs[2];
        int v;
        uv1 = e->marg.sampleContinuous(u1, &pdfs[1], &v);
        uv0 = e->cond[v].sampleContinuous(u0, &pdfs[0], nullptr);
        mapPdf = pdfs[0] * pdfs[1];
      }
      if (mapPdf == 0) return v3(0, 0, 0);
      float theta = (float)((double)uv1 * kPiD);
      float phi = (float)((double)(uv0 * 2) * kPiD);
      float cosTheta = nefm::cos(theta), sinTheta = nefm::sin(theta);
      float sinPhi = nefm::sin(phi), cosPhi = nefm::cos(phi);
      wo.o = isect.hitPoint;
      V3 polar = v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
      V3 ss, ts;
      orthonormal(v3(0, 1, 0), ss, ts);
      wo.d = toLCS(polar, v3(0, 1, 0), ss, ts);
      pdf = (float)((double)mapPdf / (2 * kPiD * kPiD * (double)sinTheta));
      if (sinTheta == 0) pdf = 0;
      if (e) return envTexel(*e, uv0, uv1);
      return ld3(L.env_radiance);
    }
  }
}

// ---------------------------------------------------------------- integrator
// integrators/VolumetricPathIntegrator.cpp:10-32 intersectTr (deviation 3).
bool intersectTr(Ctx& c, Ray ray, Hit& intersection, V3* Tr) {
  *Tr = v3(1, 1, 1);
  for (int seg = 0; seg < kMaxTrSegments; seg++) {
    Hit isect;
    bool hitSurface = intersectScene(c, ray, isect, kEps3F, kInf);
    intersection = isect;
    int m = -1;
    const ne_material* mat = hitSurface ? matOf(c.s, isect.prim) : nullptr;
    if (mat) m = mat->medium;
    if (m >= 0) *Tr = *Tr * mediumTr(c, m, ray, isect);
    if (!hitSurface) return false;
    if (m >= 0) return true;
    if (same_bits(isect.hitPoint, ray.o)) return false;
    ray.o = isect.hitPoint;
  }
  return false;
}

// integrators/VolumetricPathIntegrator.cpp:34-72 visibilityTr.
V3 visibilityTr(Ctx& c, V3 p, V3 lightPoint) {
  Ray ray{p, lightPoint - p};
  V3 Tr = v3(1, 1, 1);
  Hit isect;
  bool hitSurface = intersectScene(c, ray, isect, kEps3F, kInf);
  if (!hitSurface) return Tr;
  const ne_material* mat = matOf(c.s, isect.prim);
  if (!mat) return v3(0, 0, 0);
  if (mat->light >= 0) return Tr;
  if (mat->medium >= 0) Tr = Tr * mediumTr(c, mat->medium, ray, isect);
  return v3(0, 0, 0);
}

// integrators/VolumetricPathIntegrator.cpp:74-157 estimateDirect.
V3 estimateDirect(Ctx& c, const Ray& incoming, const Hit& isect, const ne_light& light, uint32_t lightInst) {
  const orc_scene& s = c.s;
  const float* M = s.instances[lightInst].to_wcs;
  V3 Ld = v3(0, 0, 0);
  Ray wo{v3(0, 0, 0), v3(0, 0, 0)};
  float lightPdf = 0, scatteringPdf = 0;
  V3 Li = sampleLi(s, light, isect, M, wo, lightPdf, c.S);
  V3 f = v3(0, 0, 0);
  const ne_material& mat = *matOf(s, isect.prim);
  bool surface = !(mat.medium >= 0);
  if (lightPdf > 0 && !isBlack(Li)) {
    if (surface) {
      f = bsdfEval(s, mat, incoming.d, wo.d, isect) * std::fabs(dot(wo.d, isect.normal));
      scatteringPdf = bsdfPdf(mat, incoming.d, wo.d, isect.normal);
    } else {
      f = bsdfEval(s, mat, incoming.d, wo.d, isect);
      scatteringPdf = f.x;
    }
    if (!isBlack(f)) {
      V3 pointOnLight = samplePointOnSurface(s, light.primitive, isect, M, c.S);
      Li = Li * visibilityTr(c, isect.hitPoint, pointOnLight);
      if (!isBlack(Li)) {
        float weight = powerHeuristic(lightPdf, scatteringPdf);
        Ld = Ld + ((f * Li) * weight) / lightPdf;
      }
    }
  }
  if (surface) {
    wo.d = bsdfSample(mat, incoming.d, isect.normal, c.S);
    f = bsdfEval(s, mat, incoming.d, wo.d, isect);
    f = f * std::fabs(dot(wo.d, isect.normal));
    scatteringPdf = bsdfPdf(mat, incoming.d, wo.d, isect.normal);
  } else {
    f = bsdfEval(s, mat, incoming.d, wo.d, isect);
    wo.d = bsdfSample(mat, incoming.d, v3(0, 1, 0), c.S);
    scatteringPdf = f.x;
  }
  if (!isBlack(f) && scatteringPdf > 0) {
    float weight = 1;
    lightPdf = primPdf(s, light.primitive, isect, M, c.S);
    if (lightPdf == 0) return Ld;
    weight = powerHeuristic(scatteringPdf, lightPdf);
    Hit lightIsect;
    Ray ray{isect.hitPoint, wo.d};
    V3 Tr = v3(1, 1, 1);
    bool found = intersectTr(c, ray, lightIsect, &Tr);
    V3 Li2 = v3(0, 0, 0);
    if (found) Li2 = lightLi(light);
    if (!isBlack(Li2)) Ld = Ld + (((f * Li2) * Tr) * weight) / scatteringPdf;
  }
  return Ld;
}

// integrators/VolumetricPathIntegrator.cpp:159-174 uniformSampleOneLight with
// primitives/Model.cpp:478-485 getRandomLightPrimitive (deviation 5).
V3 uniformSampleOneLight(Ctx& c, const Ray& incoming, const Hit& isect) {
  const orc_scene& s = c.s;
  float r = c.S.random();
  uint32_t nL = s.d.n_light_instances;
  if (nL == 0) return v3(0, 0, 0);
  int i = (int)((float)nL * r);
  float lightPdf = 1.0f / (float)nL;
  uint32_t inst = s.d.n_instances + (uint32_t)i;
  const ne_model& m = s.models[s.instances[inst].model];
  if (m.light_count == 0) return v3(0, 0, 0);
  c.S.random();  // first getRandomLightPrimitive(): only tested against null
  float r2 = c.S.random();
  int k = (int)((float)m.light_count * r2);
  const ne_primitive& lp = s.prims[m.light_begin + k];
  const ne_light& light = s.lights[s.materials[lp.material].light];
  return estimateDirect(c, incoming, isect, light, inst) / lightPdf;
}

// integrators/VolumetricPathIntegrator.cpp:176-301 Li, plus the optional Russian
// roulette of resources/shaders/MS_monteCarlo.frag:539-544.
V3 Li(Ctx& c, const Params& P, Ray incoming) {
  const orc_scene& s = c.s;
  V3 L = v3(0, 0, 0);
  V3 T = v3(1, 1, 1);
  Hit isect;
  int passes = 0;
  for (int b = 0; b < P.bounces; b++) {
    bool did = intersectScene(c, incoming, isect, kEps12F, kInf);
    if (isBlack(T)) break;
    const ne_material* mat = did ? matOf(s, isect.prim) : nullptr;
    if (did && mat && mat->bsdf == NE_BSDF_VOLUME) {
      incoming.o = incoming.at(isect.tNear);
      isect.tFar = isect.tFar - isect.tNear;
      isect.tNear = 0;
      Ray scattered{v3(0, 0, 0), v3(0, 0, 0)};
      V3 sampledT = mediumSample(c, mat->medium, incoming, scattered, isect);
      if (areAllOne(sampledT)) {
        incoming.o = incoming.at(isect.tFar + 0.01f);
        if (++passes >= kMaxPassThrough) break;
        b--;
        continue;
      }
      T = T * sampledT;
      V3 phaseFr = bsdfEval(s, *mat, incoming.d, scattered.d, isect);
      float phasePdf = bsdfPdf(*mat, incoming.d, scattered.d, isect.normal);
      if (isBlack(phaseFr) || phasePdf == 0.f) break;
      V3 lightSample = uniformSampleOneLight(c, scattered, isect);
      T = T * (phaseFr / phasePdf);
      L = L + T * lightSample;
      incoming = scattered;
    } else {
      if (b == 0) {
        if (did && mat && mat->light >= 0) {
          L = L + T * lightLi(s.lights[mat->light]);
        } else {
          for (uint32_t li = 0; li < s.d.n_light_instances; li++) {
            const ne_instance& inst = s.instances[s.d.n_instances + li];
            const ne_model& lm = s.models[inst.model];
            for (uint32_t k = 0; k < lm.mat_count; k++) {
              const ne_material& mm = s.materials[s.model_materials[lm.mat_begin + k]];
              L = L + T * lightLe(s, s.lights[mm.light], inst.to_ocs, incoming.d);
            }
          }
        }
      }
      if (!did || !mat || mat->bsdf == NE_BSDF_NONE) break;
      L = L + T * uniformSampleOneLight(c, incoming, isect);
      Ray scattered;
      scattered.o = isect.hitPoint;
      scattered.d = bsdfSample(*mat, incoming.d, isect.normal, c.S);
      float pdf = bsdfPdf(*mat, incoming.d, scattered.d, isect.normal);
      V3 fr = bsdfEval(s, *mat, incoming.d, scattered.d, isect);
      if (isBlack(fr) || pdf == 0.f) break;
      T = T * ((fr * absDot(incoming.d, isect.normal)) / pdf);
      incoming = scattered;
    }
    if (P.rr && b > P.rr_after) {
      float mx = maxc(T);
      if (mx < 0.01f) {
        float q = gmax(0.05f, 1.0f - mx);
        if (c.S.random() < q) break;
        T = T / (1.0f - q);
      }
    }
  }
  return L;
}

// core/Camera.cpp:140-144 getRayPassingThrough with utils/Math.h:502-507 randomInUnitDisk.
Ray cameraRay(const ne_camera& cam, float u, float v, Sampler& S) {
  float theta = (float)((2 * kPiD) * (double)S.random());
  float r = nefm::fsqrt(S.random());
  V3 disk = r * v3(nefm::cos(theta), nefm::sin(theta), 0);
  V3 rd = cam.lens_radius * disk;
  V3 offset = ld3(cam.side) * rd.x + ld3(cam.up) * rd.y;
  V3 pos = ld3(cam.position);
  V3 dir = ((((ld3(cam.lower_left) + u * ld3(cam.horizontal)) + v * ld3(cam.vertical)) - pos) - offset);
  return Ray{pos + offset, -normalize(dir)};
}

Params makeParams(const orc_scene& s, const ne_render_params* p) {
  Params P;
  P.bounces = (p && p->bounces >= 0) ? p->bounces : s.d.settings.bounces;
  int rr = (p && p->rr >= 0) ? p->rr : s.d.settings.rr_enabled;
  P.rr = rr;
  P.rr_after = (p && p->rr >= 0) ? p->rr_after : s.d.settings.rr_after;
  uint64_t seed = p ? p->seed : 0;
  P.base.seed_lo = (uint32_t)seed;
  P.base.seed_hi = (uint32_t)(seed >> 32);
  P.base.pixel = 0;
  P.base.sample = 0;
  P.base.stream = 0;
  return P;
}

// core/OfflineEngine.cpp:61-68: jittered pixel position, camera ray, Li; for a given
// camera and image size, on random stream `stream` (0 for the scene's own camera).
V3 cameraPathCam(Ctx& c, const Params& P, const ne_camera& cam, int W, int H, uint32_t pixel, uint32_t sample,
                 uint32_t stream) {
  uint32_t x = pixel % (uint32_t)W, y = pixel / (uint32_t)W;
  c.S.key = P.base;
  c.S.key.pixel = pixel;
  c.S.key.sample = sample;
  c.S.key.stream = stream;
  c.S.dim = 0;
  float u = (float)((float)(int)x + c.S.random()) / (float)W;
  float v = (float)((float)(int)y + c.S.random()) / (float)H;
  Ray r = cameraRay(cam, u, v, c.S);
  return Li(c, P, r);
}

V3 cameraPath(Ctx& c, const Params& P, uint32_t pixel, uint32_t sample) {
  const ne_settings& st = c.s.d.settings;
  return cameraPathCam(c, P, c.s.d.camera, st.width, st.height, pixel, sample, 0);
}

template <class F>
void parallelFor(size_t n, int nThreads, F f) {
  if (nThreads <= 1 || n < 2) {
    f(0, n);
    return;
  }
  std::atomic<size_t> next(0);
  const size_t chunk = 64;
  vector<std::thread> ts;
  for (int t = 0; t < nThreads; t++)
    ts.emplace_back([&]() {
      for (;;) {
        size_t b = next.fetch_add(chunk);
        if (b >= n) break;
        f(b, std::min(n, b + chunk));
      }
    });
  for (auto& t : ts) t.join();
}

}  // namespace

extern "C" {

orc_scene* orc_scene_create(const ne_scene_desc* d) {
  if (!d) return nullptr;
  orc_scene* s = new orc_scene();
  s->d = *d;
  uint32_t ni = d->n_instances + d->n_light_instances;
  s->instances.assign(d->instances, d->instances + ni);
  s->models.assign(d->models, d->models + d->n_models);
  s->prims.assign(d->prims, d->prims + d->n_prims);
  s->materials.assign(d->materials, d->materials + d->n_materials);
  if (d->n_model_materials) s->model_materials.assign(d->model_materials, d->model_materials + d->n_model_materials);
  if (d->n_lights) s->lights.assign(d->lights, d->lights + d->n_lights);
  if (d->n_media) s->media.assign(d->media, d->media + d->n_media);
  s->grids.resize(d->n_media);
  s->invMax.assign(d->n_media, 1.0f);
  s->sigmaT.resize(d->n_media);
  for (uint32_t i = 0; i < d->n_media; i++) {
    const ne_medium& m = s->media[i];
    // GridMedia.cpp:4-13: extinction = absorption + scattering, invMaxDensity = 1/max.
    s->sigmaT[i] = ld3(m.sigma_a) + ld3(m.sigma_s);
    if (m.type == NE_MEDIUM_GRID) {
      size_t n = (size_t)m.res[0] * m.res[1] * m.res[2];
      s->grids[i].assign(m.grid, m.grid + n);
      float mx = 0;
      for (size_t k = 0; k < n; k++) mx = gmax(mx, s->grids[i][k]);  // GridMedia.h:16-21
      s->invMax[i] = 1.0f / mx;
    }
  }
  s->albedoTex.resize(d->n_materials);
  for (uint32_t i = 0; i < d->n_materials; i++) {
    const ne_material& m = s->materials[i];
    if (m.albedo_width > 0 && m.albedo_height > 0 && m.albedo_texels)
      s->albedoTex[i].assign(m.albedo_texels, m.albedo_texels + (size_t)m.albedo_width * m.albedo_height * 4);
  }
  // InfiniteAreaLight's constructor (lights/InfiniteAreaLight.h:20-40) for textured lights
  s->env.resize(d->n_lights);
  for (uint32_t i = 0; i < d->n_lights; i++) {
    const ne_light& L = s->lights[i];
    if (L.type != NE_LIGHT_INFINITE || L.env_width <= 0 || L.env_height <= 0 || !L.env_texels ||
        L.env_height > L.env_width)
      continue;
    OEnv& e = s->env[i];
    e.W = L.env_width;
    e.H = L.env_height;
    e.texels.assign(L.env_texels, L.env_texels + (size_t)e.W * e.H * 4);
    vector<float> img((size_t)e.W * e.H);
    for (int v = 0; v < e.H; v++) {
      float vp = (float)v / (float)e.H;
      float sinTheta = std::sin(kPiD * float(v + 0.5f) / float(e.H));
      for (int u = 0; u < e.W; u++) {
        float up = (float)u / (float)e.W;
        img[u + v * e.W] = envTexel(e, up, vp).y;
        img[u + v * e.W] *= sinTheta;
      }
    }
    for (int v = 0; v < e.H; ++v) e.cond.emplace_back(&img[v * e.W], e.H);  // Sampling.h:87: length = height
    vector<float> marginalFunc;
    for (int v = 0; v < e.H; ++v) marginalFunc.push_back(e.cond[v].funcInt);
    e.marg = ODist1D(&marginalFunc[0], e.H);
  }
  s->triArea.assign(d->n_prims, 0.0f);
  for (uint32_t i = 0; i < d->n_prims; i++) {
    const ne_primitive& p = s->prims[i];
    if (p.type == NE_PRIM_TRIANGLE) {  // Triangle.cpp:149-157 calculateArea
      V3 a = ld3(p.p0), b = ld3(p.p1), c = ld3(p.p2);
      s->triArea[i] = length(cross(b - a, c - a)) / 2.0f;
    }
  }
  s->omodels.resize(d->n_models);
  for (uint32_t i = 0; i < d->n_models; i++) {
    const ne_model& m = s->models[i];
    OModel& om = s->omodels[i];
    for (uint32_t k = 0; k < m.prim_count; k++) om.prims.push_back(m.prim_begin + k);
    if (m.use_bvh && m.prim_count > 0) bvhInit(*s, om);
  }
  return s;
}

void orc_scene_destroy(orc_scene* s) { delete s; }

void orc_trace_paths(const orc_scene* s, const ne_render_params* p, const ne_path_key* keys, size_t n, float* out,
                     int n_threads) {
  Params P = makeParams(*s, p);
  uint32_t off = p ? p->sample_offset : 0;
  parallelFor(n, n_threads, [&](size_t b, size_t e) {
    Ctx c{*s, Sampler{}, 0};
    for (size_t i = b; i < e; i++) {
      V3 L = cameraPath(c, P, keys[i].pixel, keys[i].sample + off);
      out[i * 3 + 0] = L.x;
      out[i * 3 + 1] = L.y;
      out[i * 3 + 2] = L.z;
    }
  });
}

void orc_trace_view_paths(const orc_scene* s, const ne_render_params* p, const ne_camera* cam, int width, int height,
                          uint32_t stream, const ne_path_key* keys, size_t n, float* out, int n_threads) {
  Params P = makeParams(*s, p);
  uint32_t off = p ? p->sample_offset : 0;
  parallelFor(n, n_threads, [&](size_t b, size_t e) {
    Ctx c{*s, Sampler{}, 0};
    for (size_t i = b; i < e; i++) {
      V3 L = cameraPathCam(c, P, *cam, width, height, keys[i].pixel, keys[i].sample + off, stream);
      out[i * 3 + 0] = L.x;
      out[i * 3 + 1] = L.y;
      out[i * 3 + 2] = L.z;
    }
  });
}

void orc_li_batch(const orc_scene* s, const ne_render_params* p, const ne_ray* rays, const ne_path_key* keys, size_t n,
                  uint32_t first_dim, float* out, int n_threads) {
  Params P = makeParams(*s, p);
  parallelFor(n, n_threads, [&](size_t b, size_t e) {
    Ctx c{*s, Sampler{}, 0};
    for (size_t i = b; i < e; i++) {
      c.S.key = P.base;
      c.S.key.pixel = keys[i].pixel;
      c.S.key.sample = keys[i].sample;
      c.S.dim = first_dim;
      V3 L = Li(c, P, Ray{ld3(rays[i].o), ld3(rays[i].d)});
      out[i * 3 + 0] = L.x;
      out[i * 3 + 1] = L.y;
      out[i * 3 + 2] = L.z;
    }
  });
}

double orc_render_pixels(const orc_scene* s, const ne_render_params* p, uint32_t pixel_begin, uint32_t n_pixels,
                         float* out, int n_threads, uint64_t* density_lookups) {
  Params P = makeParams(*s, p);
  int spp = (p && p->spp > 0) ? p->spp : s->d.settings.spp;
  uint32_t off = p ? p->sample_offset : 0;
  std::atomic<uint64_t> lookups(0);
  auto t0 = std::chrono::steady_clock::now();
  parallelFor(n_pixels, n_threads, [&](size_t b, size_t e) {
    Ctx c{*s, Sampler{}, 0};
    for (size_t i = b; i < e; i++) {
      uint32_t pix = pixel_begin + (uint32_t)i;
      V3 color = v3(0, 0, 0);
      for (int k = 0; k < spp; k++) color = color + cameraPath(c, P, pix, off + (uint32_t)k);
      color = color / (float)spp;
      out[i * 3 + 0] = color.x;
      out[i * 3 + 1] = color.y;
      out[i * 3 + 2] = color.z;
    }
    lookups.fetch_add(c.lookups);
  });
  auto t1 = std::chrono::steady_clock::now();
  if (density_lookups) *density_lookups = lookups.load();
  return std::chrono::duration<double>(t1 - t0).count();
}

// Renders the listed pixels (all spp each), as renderTile does for the pixels of a tile
// (core/OfflineEngine.cpp:54-76); chunks of 64 pixels are taken from a shared counter, as the
// reference's threads take tiles. Returns wall seconds.
double orc_render_pixel_list(const orc_scene* s, const ne_render_params* p, const uint32_t* pixels, uint32_t n_pixels,
                             float* out, int n_threads, uint64_t* density_lookups) {
  Params P = makeParams(*s, p);
  int spp = (p && p->spp > 0) ? p->spp : s->d.settings.spp;
  uint32_t off = p ? p->sample_offset : 0;
  std::atomic<uint64_t> lookups(0);
  auto t0 = std::chrono::steady_clock::now();
  parallelFor(n_pixels, n_threads, [&](size_t b, size_t e) {
    Ctx c{*s, Sampler{}, 0};
    for (size_t i = b; i < e; i++) {
      V3 color = v3(0, 0, 0);
      for (int k = 0; k < spp; k++) color = color + cameraPath(c, P, pixels[i], off + (uint32_t)k);
      color = color / (float)spp;
      out[i * 3 + 0] = color.x;
      out[i * 3 + 1] = color.y;
      out[i * 3 + 2] = color.z;
    }
    lookups.fetch_add(c.lookups);
  });
  auto t1 = std::chrono::steady_clock::now();
  if (density_lookups) *density_lookups = lookups.load();
  return std::chrono::duration<double>(t1 - t0).count();
}

// core/OfflineEngine.cpp:54-113: tiles of (W/40) x (H/10) pixels taken from a shared
// counter by n_threads threads (the reference's busy-polled pool of 16 threads).
double orc_render(const orc_scene* s, const ne_render_params* p, float* out, int n_threads) {
  Params P = makeParams(*s, p);
  const ne_settings& st = s->d.settings;
  int W = st.width, H = st.height;
  int spp = (p && p->spp > 0) ? p->spp : st.spp;
  uint32_t off = p ? p->sample_offset : 0;
  bool refTiles = p && (p->flags & NE_RENDER_REF_TILES);
  int tw = std::max(1, W / 40), th = std::max(1, H / 10);
  int tilesX = refTiles ? 40 : (W + tw - 1) / tw;
  int tilesY = refTiles ? 10 : (H + th - 1) / th;
  for (size_t i = 0; i < (size_t)W * H * 3; i++) out[i] = 0;
  std::atomic<int> next(0);
  auto work = [&]() {
    Ctx c{*s, Sampler{}, 0};
    for (;;) {
      int t = next.fetch_add(1);
      if (t >= tilesX * tilesY) break;
      int mx = (t % tilesX) * tw, my = (t / tilesX) * th;
      for (int y = my; y < std::min(H, my + th); y++)
        for (int x = mx; x < std::min(W, mx + tw); x++) {
          V3 color = v3(0, 0, 0);
          uint32_t pix = (uint32_t)(W * y + x);
          for (int k = 0; k < spp; k++) color = color + cameraPath(c, P, pix, off + (uint32_t)k);
          color = color / (float)spp;
          out[pix * 3 + 0] = color.x;
          out[pix * 3 + 1] = color.y;
          out[pix * 3 + 2] = color.z;
        }
    }
  };
  auto t0 = std::chrono::steady_clock::now();
  if (n_threads <= 1) {
    work();
  } else {
    vector<std::thread> ts;
    for (int i = 0; i < n_threads; i++) ts.emplace_back(work);
    for (auto& t : ts) t.join();
  }
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

void orc_trace_closest(const orc_scene* s, const ne_ray* rays, size_t n, float t_min, float t_max, ne_hit* out) {
  Ctx c{*s, Sampler{}, 0};
  for (size_t i = 0; i < n; i++) {
    Hit h;
    bool did = intersectScene(c, Ray{ld3(rays[i].o), ld3(rays[i].d)}, h, t_min, t_max);
    ne_hit& o = out[i];
    memset(&o, 0, sizeof(o));
    o.hit = did ? 1 : 0;
    if (did) {
      o.t_near = h.tNear;
      o.t_far = h.tFar;
      o.point[0] = h.hitPoint.x; o.point[1] = h.hitPoint.y; o.point[2] = h.hitPoint.z;
      o.normal[0] = h.normal.x; o.normal[1] = h.normal.y; o.normal[2] = h.normal.z;
      o.instance = h.inst;
      o.primitive = h.prim;
    } else {
      o.instance = -1;
      o.primitive = -1;
    }
  }
}

// ---- unit restatements for the reference's known-answer tests
int orc_triangle_intersect(const float* a, const float* b, const float* c, const ne_ray* r, float* tn, float* tf,
                           float* point, float* normal) {
  orc_scene s;
  ne_primitive p;
  memset(&p, 0, sizeof(p));
  p.type = NE_PRIM_TRIANGLE;
  p.material = -1;
  memcpy(p.p0, a, 12); memcpy(p.p1, b, 12); memcpy(p.p2, c, 12);
  Hit h;
  bool ok = triIntersect(s, p, Ray{ld3(r->o), ld3(r->d)}, h);
  *tn = h.tNear; *tf = h.tFar;
  point[0] = h.hitPoint.x; point[1] = h.hitPoint.y; point[2] = h.hitPoint.z;
  normal[0] = h.normal.x; normal[1] = h.normal.y; normal[2] = h.normal.z;
  return ok ? 1 : 0;
}

int orc_aabb_intersect(const float* mn, const float* mx, const ne_ray* r, float* tn, float* tf, float* point,
                       float* normal) {
  Hit h;
  bool ok = aabbIntersect(ld3(mn), ld3(mx), Ray{ld3(r->o), ld3(r->d)}, h);
  *tn = h.tNear; *tf = h.tFar;
  point[0] = h.hitPoint.x; point[1] = h.hitPoint.y; point[2] = h.hitPoint.z;
  normal[0] = h.normal.x; normal[1] = h.normal.y; normal[2] = h.normal.z;
  return ok ? 1 : 0;
}

void orc_orthonormal(const float* n, float* v, float* u) {
  V3 a, b;
  orthonormal(ld3(n), a, b);
  v[0] = a.x; v[1] = a.y; v[2] = a.z;
  u[0] = b.x; u[1] = b.y; u[2] = b.z;
}
void orc_to_lcs(const float* v, const float* ns, const float* ss, const float* ts, float* out) {
  V3 r = toLCS(ld3(v), ld3(ns), ld3(ss), ld3(ts));
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void orc_to_world(const float* v, const float* ns, const float* ss, const float* ts, float* out) {
  V3 r = toWorld(ld3(v), ld3(ns), ld3(ss), ld3(ts));
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void orc_sample_unit_sphere(float e1, float e2, float* out) {
  V3 r = sampleUnitSphere(e1, e2);
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
float orc_hg_eval(float g, const float* wi, const float* wo) {
  ne_material m;
  memset(&m, 0, sizeof(m));
  m.bsdf = NE_BSDF_VOLUME;
  m.phase = NE_PHASE_HG;
  m.g = g;
  return phaseEval(m, ld3(wi), ld3(wo));
}
void orc_hg_sample(float g, float u0, float u1, float* out) {
  // HG::sample with the two draws given explicitly (seeded through a fixed key).
  float cosTheta;
  if (std::fabs(g) < 1e-3f)
    cosTheta = 1.0f - 2.0f * u0;
  else {
    float sqr = (1.0f - g * g) / ((1.0f + g) - (2.0f * g) * u0);
    sqr = sqr * sqr;
    cosTheta = (-1.0f / (2.0f * g)) * ((1.0f + g * g) - sqr);
  }
  float sinTheta = nefm::fsqrt(1.0f - cosTheta * cosTheta);
  float phi = (float)((2.0f * kPiD) * (double)u1);
  out[0] = nefm::cos(phi) * sinTheta;
  out[1] = nefm::sin(phi) * sinTheta;
  out[2] = cosTheta;
}
float orc_iso_pdf(void) { return (float)(1.0 / kFourPiD); }

// primitives/Triangle.cpp:93-108 barycentricCoordinates.
void orc_barycentric(const float* pp, const float* aa, const float* bb, const float* cc, float* out) {
  V3 p = ld3(pp), a = ld3(aa), b = ld3(bb), c = ld3(cc);
  V3 v0 = b - a, v1 = c - a, v2 = p - a;
  float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
  float denom = d00 * d11 - d01 * d01;
  float v = (d11 * d20 - d01 * d21) / denom;
  float w = (d00 * d21 - d01 * d20) / denom;
  out[1] = v;
  out[2] = w;
  out[0] = 1.0f - v - w;
}
float orc_triangle_area(const float* a, const float* b, const float* c) {
  return length(cross(ld3(b) - ld3(a), ld3(c) - ld3(a))) / 2.0f;
}
// primitives/Triangle.cpp:79-91 contains (EPSILON3 plane test + barycentric range).
int orc_triangle_contains(const float* a, const float* b, const float* c, const float* p) {
  V3 A = ld3(a), B = ld3(b), C = ld3(c), Q = ld3(p);
  V3 n = cross(B - A, C - A);
  float lenSq = length(n);
  float d = dot(n, B - Q);
  if ((double)(d * d) > 0.001 * (double)lenSq) return 0;
  float uvw[3];
  orc_barycentric(p, a, b, c, uvw);
  return (uvw[0] >= 0 && uvw[1] >= 0 && uvw[0] + uvw[1] <= 1) ? 1 : 0;
}
// utils/Math.h isSameSide / isPointInsideTriangleRange.
int orc_point_in_triangle_range(const float* p, const float* a, const float* b, const float* c) {
  auto same = [](V3 P, V3 ref, V3 A, V3 B) { return dot(cross(B - A, P - A), cross(B - A, ref - A)) >= 0; };
  V3 Pp = ld3(p), A = ld3(a), B = ld3(b), C = ld3(c);
  return (same(Pp, A, B, C) && same(Pp, B, A, C) && same(Pp, C, A, B)) ? 1 : 0;
}

int orc_triangle_model_intersect(const float* verts, uint32_t n_verts, const uint32_t* idx, uint32_t n_idx,
                                 const ne_ray* r, float t_min, float t_max, float* t_hit) {
  (void)n_verts;
  orc_scene s;
  uint32_t nt = n_idx / 3;
  for (uint32_t i = 0; i < nt; i++) {
    ne_primitive p;
    memset(&p, 0, sizeof(p));
    p.type = NE_PRIM_TRIANGLE;
    p.material = -1;
    memcpy(p.p0, verts + idx[3 * i] * 3, 12);
    memcpy(p.p1, verts + idx[3 * i + 1] * 3, 12);
    memcpy(p.p2, verts + idx[3 * i + 2] * 3, 12);
    s.prims.push_back(p);
  }
  ne_model m;
  memset(&m, 0, sizeof(m));
  m.prim_begin = 0;
  m.prim_count = nt;
  // Model(vertexData, indexData, layout) sets boundingBox from the vertices (Model.cpp:36-79).
  V3 mn = v3(kInf, kInf, kInf), mx = v3(-kInf, -kInf, -kInf);
  for (uint32_t i = 0; i < n_idx; i++) {
    V3 v = ld3(verts + idx[i] * 3);
    mn = vmin(v, mn);
    mx = vmax(v, mx);
  }
  m.has_bbox = 1;
  m.bbox_min[0] = mn.x; m.bbox_min[1] = mn.y; m.bbox_min[2] = mn.z;
  m.bbox_max[0] = mx.x; m.bbox_max[1] = mx.y; m.bbox_max[2] = mx.z;
  s.models.push_back(m);
  s.omodels.resize(1);
  for (uint32_t k = 0; k < nt; k++) s.omodels[0].prims.push_back(k);
  Hit h;
  float tmin = t_min, tmax = t_max;
  bool ok = modelIntersect(s, 0, Ray{ld3(r->o), ld3(r->d)}, h, tmin, tmax);
  *t_hit = h.tNear;
  return ok ? 1 : 0;
}

uint32_t orc_bvh_build_count(const float* verts, const uint32_t* idx, uint32_t n_tris) {
  orc_scene s;
  for (uint32_t i = 0; i < n_tris; i++) {
    ne_primitive p;
    memset(&p, 0, sizeof(p));
    p.type = NE_PRIM_TRIANGLE;
    p.material = -1;
    memcpy(p.p0, verts + idx[3 * i] * 3, 12);
    memcpy(p.p1, verts + idx[3 * i + 1] * 3, 12);
    memcpy(p.p2, verts + idx[3 * i + 2] * 3, 12);
    s.prims.push_back(p);
  }
  OModel om;
  for (uint32_t k = 0; k < n_tris; k++) om.prims.push_back(k);
  bvhInit(s, om);
  return om.nodeCount;
}

void orc_fmath(int fn, const float* x, size_t n, float* out) {
  for (size_t i = 0; i < n; i++) {
    float v = x[i];
    switch (fn) {
      case 0: out[i] = nefm::log(v); break;
      case 1: out[i] = nefm::exp(v); break;
      case 2: out[i] = nefm::sin(v); break;
      case 3: out[i] = nefm::cos(v); break;
      case 4: out[i] = nefm::acos(v); break;
      case 6: out[i] = nefm::atan2(v, (i ^ 1) < n ? x[i ^ 1] : 1.0f); break;
      case 7: out[i] = nefm::log1m_draw(v); break;
      default: out[i] = nefm::pow5(v); break;
    }
  }
}

void orc_rng(uint64_t seed, const ne_path_key* keys, const uint32_t* dims, size_t n, float* out) {
  for (size_t i = 0; i < n; i++) {
    nerng::PathKey k;
    k.seed_lo = (uint32_t)seed;
    k.seed_hi = (uint32_t)(seed >> 32);
    k.pixel = keys[i].pixel;
    k.sample = keys[i].sample;
    k.stream = 0;
    out[i] = nerng::u01(k, dims[i]);
  }
}

void orc_philox(const uint32_t* c, const uint32_t* k, uint32_t* out) {
  nerng::Block b = nerng::philox4x32_10(c[0], c[1], c[2], c[3], k[0], k[1]);
  for (int i = 0; i < 4; i++) out[i] = b.w[i];
}

// The BVH of model `m` as built by BVH::init: per node (min xyz, max xyz, start, count,
// rightOffset) as 9 words (floats then uint32 bit patterns); `order` receives the primitive
// order. Returns the node count (0 when the model has no BVH); writes at most `cap` nodes.
size_t orc_model_bvh(const orc_scene* s, uint32_t m, float* nodes, size_t cap, uint32_t* order) {
  if (!s || m >= s->omodels.size()) return 0;
  const OModel& om = s->omodels[m];
  if (om.nodeCount == 0) return 0;
  for (size_t i = 0; i < om.nodeCount && i < cap; i++) {
    const BVHNode& n = om.nodes[i];
    float* o = nodes + 9 * i;
    o[0] = n.mn.x; o[1] = n.mn.y; o[2] = n.mn.z;
    o[3] = n.mx.x; o[4] = n.mx.y; o[5] = n.mx.z;
    memcpy(o + 6, &n.start, 4);
    memcpy(o + 7, &n.count, 4);
    memcpy(o + 8, &n.rightOffset, 4);
  }
  if (order) memcpy(order, om.prims.data(), om.prims.size() * sizeof(uint32_t));
  return om.nodeCount;
}

// Replaces model m's BVH by a tree given in orc_model_bvh's format (a tree the GPU built, for
// checks of the device's traversal over it). order: the model's primitives in leaf order.
int orc_model_set_bvh(orc_scene* s, uint32_t m, const float* nodes, size_t n, const uint32_t* order, size_t n_order) {
  if (!s || m >= s->omodels.size() || !nodes || !order || n == 0) return -1;
  if (n_order != s->models[m].prim_count) return -1;
  OModel& om = s->omodels[m];
  om.nodes.assign(n, BVHNode{});
  for (size_t i = 0; i < n; i++) {
    const float* o = nodes + 9 * i;
    BVHNode& b = om.nodes[i];
    b.mn = v3(o[0], o[1], o[2]);
    b.mx = v3(o[3], o[4], o[5]);
    memcpy(&b.start, o + 6, 4);
    memcpy(&b.count, o + 7, 4);
    memcpy(&b.rightOffset, o + 8, 4);
    if (b.isLeaf() ? (size_t)b.start + b.count > n_order : i + b.rightOffset >= n) return -1;
  }
  om.nodeCount = (uint32_t)n;
  om.prims.assign(order, order + n_order);
  return 0;
}

}  // extern "C"
