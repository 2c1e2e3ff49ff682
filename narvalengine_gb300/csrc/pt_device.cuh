// Device implementation of the NarvalEngine path integrator for sm_103a.
//
// One function per reference function, named after it; each cites the reference
// file:line it implements (paths relative to the reference's src/). Arithmetic keeps
// the reference's expression order and types (float, with double where a double
// literal such as PI or EPSILON promotes the expression) and glm's evaluation order:
// dot = (x*x' + y*y') + z*z', mat4*vec4 = (c0 v0 + c1 v1) + (c2 v2 + c3 v3),
// min(a,b) = b<a?b:a, max(a,b) = a<b?b:a, mix(x,y,a) = x(1-a) + y a. The file is
// compiled with -fmad=false and IEEE division and square root, so each operation
// rounds exactly as on the host.
//
// Deliberate deviations from the reference (taken identically by the CPU oracle):
//  * random() is the counter-based generator of ne_rng.h in the reference's draw order;
//  * libm functions are those of ne_fmath.h;
//  * intersectTr stops when the next segment would start at the same point or after
//    256 segments (the reference loops forever there), tracking loops stop after 2^20
//    steps, a path ends after 2^16 medium pass-throughs (which the reference does not
//    count as bounces), and a scene without lights contributes no direct light;
//  * a BVH traversal stack deeper than 64 entries raises an error flag.
#pragma once
#include <cooperative_groups.h>
#include <stdint.h>

#include "device_scene.h"
#include "ne_fmath.h"
#include "ne_rng.h"

namespace nedev {

#define NE_D __device__ __forceinline__
#define NE_NI __device__ __forceinline__

constexpr double kPiD = 3.14159265358979323846264338327950288;
constexpr double kTwoPiD = 6.283185307179586476925286766559;
constexpr double kFourPiD = 12.566370614359172953850573533118;
constexpr double kEpsilonD = 0.0000000001;
constexpr double kInvPiD = 0.31830988618379067154;   // INVPI (utils/Math.h:24)
constexpr double kInv2PiD = 0.15915494309189533577;  // INV2PI (utils/Math.h:25)
constexpr float kInv4Pi = float(0.07957747154594766788);
constexpr float kEps3F = float(0.001);
constexpr float kEps12F = float(0.00000000001);
constexpr int kMaxTrackSteps = 1 << 20;
constexpr int kMaxTrSegments = 256;
constexpr int kMaxPassThrough = 1 << 16;
constexpr int kBvhStack = 64;

enum : uint32_t { ERR_BVH_STACK = 1u };

// Kernel specialisation: K = feature bits of the scene (which primitive, BSDF, medium and
// light kinds occur) | K_COUNT for the instrumented variant. Every type switch below tests
// the feature bit first, so a kernel compiled for a scene's features carries no code for the
// rest: the fully general kernel is large enough to stall on instruction fetch.
enum : uint32_t {
  FT_SPHERE = 1u << 0,
  FT_RECT = 1u << 1,
  FT_AABB = 1u << 2,
  FT_TRI = 1u << 3,       // triangles and their BVH
  FT_POINT = 1u << 4,
  FT_GLOSSY = 1u << 5,
  FT_VOLBSDF = 1u << 6,   // VolumeBSDF with HG or isotropic phase
  FT_GRID = 1u << 7,
  FT_HOMOG = 1u << 8,
  FT_LDIFF = 1u << 9,
  FT_LDIR = 1u << 10,
  FT_LINF = 1u << 11,
  FT_NORMALMAP = 1u << 12,
  FT_BBOX = 1u << 13,     // model bounding boxes (meshes)
  FT_ENVMAP = 1u << 14,   // InfiniteAreaLight with a texture and its Distribution2D
  FT_TEXALB = 1u << 15,   // microfacet albedo from a texture (per-hit texture coordinates)
  FT_ALL = (1u << 16) - 1,
  K_COUNT = 1u << 31,
  K_CACHE = 1u << 30,  // paths end in the learned radiance cache (see CacheIO)
  K_SPLIT = 1u << 29,  // paths are deferred at their first medium scattering (see DeferQueue)
  // feature sets with a compiled kernel (the host picks the smallest superset)
  K_VOLUME = FT_AABB | FT_POINT | FT_SPHERE | FT_VOLBSDF | FT_GRID | FT_LDIR | FT_LINF,
  K_SURFACE = FT_RECT | FT_SPHERE | FT_GLOSSY | FT_LDIFF,
  K_MESH = FT_TRI | FT_BBOX | FT_RECT | FT_SPHERE | FT_GLOSSY | FT_LDIFF,
  K_GENERAL = FT_ALL
};

// ---------------------------------------------------------------- vectors
struct V3 {
  float x, y, z;
};
NE_D V3 v3(float x, float y, float z) { return V3{x, y, z}; }
NE_D V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
NE_D V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
NE_D V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
NE_D V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
NE_D V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
NE_D V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
NE_D V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
NE_D V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
NE_D float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
NE_D V3 cross(V3 a, V3 b) { return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
NE_D float length(V3 a) { return nefm::fsqrt(dot(a, a)); }
NE_D V3 normalize(V3 a) { return a * (1.0f / nefm::fsqrt(dot(a, a))); }
NE_D float gmin(float a, float b) { return (b < a) ? b : a; }
NE_D float gmax(float a, float b) { return (a < b) ? b : a; }
NE_D double gmaxd(double a, double b) { return (a < b) ? b : a; }
NE_D V3 vmin(V3 a, V3 b) { return v3(gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)); }
NE_D V3 vmax(V3 a, V3 b) { return v3(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)); }
NE_D V3 vabs(V3 a) { return v3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
NE_D V3 ld3(const float* p) { return v3(p[0], p[1], p[2]); }
NE_D bool isBlack(V3 v) { return v.x == 0 && v.y == 0 && v.z == 0; }
NE_D bool areAllOne(V3 v) { return v.x == 1 && v.y == 1 && v.z == 1; }
NE_D float avg(V3 v) { return (v.x + v.y + v.z) / 3.0f; }
NE_D float absDot(V3 a, V3 b) { return fabsf(dot(a, b)); }
NE_D float maxc(V3 v) { return gmax(gmax(v.x, v.y), v.z); }
NE_D bool sameBits(V3 a, V3 b) {
  return __float_as_uint(a.x) == __float_as_uint(b.x) && __float_as_uint(a.y) == __float_as_uint(b.y) &&
         __float_as_uint(a.z) == __float_as_uint(b.z);
}

// glm::mat4 (affine, 12 stored floats) times vec4(p, w).
NE_D V3 mul4(const float* m, V3 p, float w) {
  return v3((m[0] * p.x + m[3] * p.y) + (m[6] * p.z + m[9] * w),
            (m[1] * p.x + m[4] * p.y) + (m[7] * p.z + m[10] * w),
            (m[2] * p.x + m[5] * p.y) + (m[8] * p.z + m[11] * w));
}

struct Ray {
  V3 o, d;
  NE_D V3 at(float t) const { return o + t * d; }
};

struct Hit {
  V3 hitPoint, normal;
  float tNear, tFar;
  int inst, prim;
};

NE_D Hit emptyHit() {
  Hit h;
  h.hitPoint = v3(0, 0, 0);
  h.normal = v3(0, 0, 0);
  h.tNear = 0;
  h.tFar = 0;
  h.inst = -1;
  h.prim = -1;
  return h;
}

// Counter RNG with the current four-word block cached in registers.
// One Philox block, compiled once and called from every draw site. A free function with
// value arguments: a member function would take the sampler's address and push the whole
// per-path context out of registers into local memory.
static __device__ __noinline__ uint4 philoxBlock(uint32_t b, uint32_t sample, uint32_t pixel, uint32_t stream,
                                                  uint32_t k0, uint32_t k1) {
  nerng::Block r = nerng::philox4x32_10(b, sample, pixel, stream, k0, k1);
  return make_uint4(r.w[0], r.w[1], r.w[2], r.w[3]);
}

struct Sampler {
  nerng::PathKey key;
  uint32_t dim;
  uint32_t blk;
  uint32_t w0, w1, w2, w3;
  NE_D void refill(uint32_t b) {
    uint4 r = philoxBlock(b, key.sample, key.pixel, key.stream, key.seed_lo, key.seed_hi);
    w0 = r.x; w1 = r.y; w2 = r.z; w3 = r.w;
    blk = b;
  }
  NE_D void reset(const nerng::PathKey& k, uint32_t d) {
    key = k;
    dim = d;
    blk = 0xffffffffu;
  }
  NE_D float random() {
    float r = peek();
    dim++;
    return r;
  }
  // random() with the block computed inline: for the tracking loops, which draw most often
  // (elsewhere the out-of-line block keeps the kernel small).
  NE_D float randomInline() {
    uint32_t b = dim >> 2;
    if (b != blk) {
      nerng::Block r = nerng::philox4x32_10_unrolled(b, key.sample, key.pixel, key.stream, key.seed_lo, key.seed_hi);
      w0 = r.w[0]; w1 = r.w[1]; w2 = r.w[2]; w3 = r.w[3];
      blk = b;
    }
    uint32_t s = dim & 3u;
    dim++;
    uint32_t w = (s == 0) ? w0 : (s == 1) ? w1 : (s == 2) ? w2 : w3;
    return nerng::word_to_u01(w);
  }
  // The next draw, without consuming it.
  NE_D float peek() {
    uint32_t b = dim >> 2;
    if (b != blk) refill(b);
    uint32_t s = dim & 3u;
    uint32_t w = (s == 0) ? w0 : (s == 1) ? w1 : (s == 2) ? w2 : w3;
    return nerng::word_to_u01(w);
  }
};

struct Counters {
  unsigned long long lookups, queries, nodes, tests;
};

template <uint32_t K>
struct Ctx {
  const DScene& s;
  Sampler S;
  Counters c;
  uint32_t* err;
  // K_CACHE only: this path's index, whether it is a training path, and the cache buffers
  uint32_t pidx;
  bool train;
  const struct CacheIO* cio;
  // K_SPLIT only: the queue deferred paths go to, the bounce at whose scattering event they
  // are deferred (-1: never), the path's radiance slot, set when the path was deferred
  const struct DeferQueue* dq;
  unsigned long long idx;
  bool deferred;
  int deferAt;
  int deferHalf;  // 1: deferral points every half bounce (after sampling, and after the bounce)
  bool deferTop = false;  // K_SPLIT first pass: defer every new path before its first intersection
  // K_SPLIT passes of surface scenes whose shadow rays are traced ahead: stop a path at its
  // light sample's visibility test (shadowSlot: its queue entry, shadowPoint: the point on the
  // light), or take the test's known result (shadowVis: 1 visible, 2 blocked, 0 unknown)
  bool deferShadow = false;
  int shadowVis = 0;
  int shadowSlot = -1;
  V3 shadowPoint = V3{0, 0, 0};
};

// Kernels whose paths can stop at a shadow ray: split kernels of surface-only feature sets (the
// visibility test there draws no random numbers and gives all or nothing).
// Slot in an append-only buffer: one atomic per group of lanes that append together.
NE_D uint32_t appendSlot(uint32_t* count) {
  namespace cg = cooperative_groups;
  cg::coalesced_group g = cg::coalesced_threads();
  uint32_t base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(count, (uint32_t)g.size());
  return g.shfl(base, 0) + g.thread_rank();
}

template <uint32_t K>
__host__ __device__ constexpr bool shadowQueue() {
  return (K & K_SPLIT) && !(K & (FT_GRID | FT_HOMOG | FT_VOLBSDF | K_CACHE | K_COUNT));
}

// Buffers of a render that ends paths in the learned radiance cache. A path that reaches
// a scattering vertex in a grid medium at or after bounce `bounce` either stops there and
// appends a query (object-space position, incoming direction, throughput, path index) for
// the network to answer, or, on a training path, runs on unchanged and appends a training
// sample: the radiance gathered after that vertex divided by the throughput at it.
struct CacheIO {
  float* q_pos;
  float* q_dir;
  float* q_thr;
  uint32_t* q_idx;
  uint32_t* q_count;
  uint32_t q_cap;
  float* t_pos;
  float* t_dir;
  float* t_val;
  uint32_t* t_count;
  uint32_t t_cap;
  uint32_t train_stride;  // a path is a training path when hash(index) % train_stride == 0
  int bounce;
  // training paths ending in the cache (train_suffix > 0): at their first scattering vertex
  // train_suffix or more bounces after the recorded one, a query whose answer times tq_thr is
  // added to the training sample tq_idx's target
  int train_suffix;
  float* tq_pos;
  float* tq_dir;
  float* tq_thr;
  uint32_t* tq_idx;
  uint32_t* tq_count;
};

NE_D Ray transformRay(const Ray& r, const float* m) { return Ray{mul4(m, r.o, 1.0f), mul4(m, r.d, 0.0f)}; }

// utils/Math.h:591-599 generateOrthonormalCS.
NE_D void orthonormal(V3 n, V3& v, V3& u) {
  if (fabsf(n.x) > fabsf(n.y))
    v = v3(-n.z, 0, n.x) / nefm::fsqrt(n.x * n.x + n.z * n.z);
  else
    v = v3(0, n.z, -n.y) / nefm::fsqrt(n.y * n.y + n.z * n.z);
  u = normalize(cross(n, v));
}
NE_D V3 toWorld(V3 v, V3 ns, V3 ss, V3 ts) {  // utils/Math.h:612-617
  return v3(ss.x * v.x + ts.x * v.y + ns.x * v.z, ss.y * v.x + ts.y * v.y + ns.y * v.z,
            ss.z * v.x + ts.z * v.y + ns.z * v.z);
}
NE_D V3 toLCS(V3 v, V3 ns, V3 ss, V3 ts) { return v3(dot(v, ss), dot(v, ts), dot(v, ns)); }  // Math.h:629-631
NE_D bool sameHemisphere(V3 a, V3 b) { return dot(a, b) > 0; }
NE_D float powerHeuristic(float p0, float p1) { return (p0 * p0) / (p0 * p0 + p1 * p1); }

// utils/Math.h:442-457 sampleUnitSphere.
NE_D V3 sampleUnitSphere(float e1, float e2) {
  float theta = __double2float_rn(kTwoPiD * (double)e1);
  float phi = nefm::acos(1.0f - 2.0f * e2);
  return v3(nefm::sin(phi) * nefm::cos(theta), nefm::sin(phi) * nefm::sin(theta), nefm::cos(phi));
}
NE_D V3 reflect(V3 i, V3 n) { return i - (n * dot(n, i)) * 2.0f; }

// utils/Math.h:1112-1126 convertAreaToSolidAngle.
NE_D float convertAreaToSolidAngle(float pdfArea, V3 normal, V3 p1, V3 p2) {
  V3 wi = p1 - p2;
  if (dot(wi, wi) == 0) return 0;
  wi = normalize(wi);
  V3 d = p2 - p1;
  pdfArea = pdfArea * (dot(d, d) / absDot(normal, -wi));
  if (nefm::isinf_(pdfArea)) return 0;
  return pdfArea;
}

NE_D V3 convertNormalFromTextureMap(V3 texNormal, V3 worldNormal) {
  V3 nts = texNormal * 2.0f - v3(1, 1, 1);
  V3 t = cross(worldNormal, v3(0, 1, 0));
  V3 b = normalize(cross(worldNormal, t));
  V3 r = (t * nts.x + b * nts.y) + worldNormal * nts.z;
  return normalize(r);
}

// ---------------------------------------------------------------- primitives (OCS)
// primitives/AABB.cpp:48-80 AABB::intersect.
NE_D bool aabbIntersect(V3 mn, V3 mx, const Ray& r, Hit& h) {
  V3 s = v3((r.d.x < 0.0f) ? 1.0f : -1.0f, (r.d.y < 0.0f) ? 1.0f : -1.0f, (r.d.z < 0.0f) ? 1.0f : -1.0f);
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
    h.tNear = __int_as_float(0x7f800000);
    h.tFar = -__int_as_float(0x7f800000);
    return false;
  }
  return true;
}

// Box test used only to steer BVH traversal: same arithmetic, no hit record.
NE_D bool aabbNear(V3 mn, V3 mx, const Ray& r, V3 invD, V3 s, float& tNearOut) {
  V3 size = mx - mn;
  V3 center = mx - size / 2.0f;
  V3 half = size / 2.0f;
  V3 t1 = ((center - r.o) + s * half) * invD;
  V3 t2 = ((center - r.o) - s * half) * invD;
  V3 tmin = vmin(t1, t2);
  V3 tmax = vmax(t1, t2);
  float tNear = gmax(gmax(tmin.x, tmin.y), tmin.z);
  float tFar = gmin(gmin(tmax.x, tmax.y), tmax.z);
  tNearOut = tNear;
  return !(tNear > tFar);
}

// primitives/Sphere.cpp:21-44.
NE_D bool sphereIntersect(const DPrim& p, const Ray& r, Hit& h) {
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
NE_D V3 rectSize(V3 v0, V3 v1) {
  if (v0.x == v1.x) { v0.x = 0; v1.x = 0; }
  if (v0.y == v1.y) { v0.y = 0; v1.y = 0; }
  if (v0.z == v1.z) { v0.z = 0; v1.z = 0; }
  return vabs(v0) + vabs(v1);
}

// primitives/Rectangle.cpp:50-76 and :32-48.
NE_D bool rectIntersect(const DPrim& p, const Ray& r, Hit& h) {
  V3 v0 = ld3(p.p0), v1 = ld3(p.p1), n = ld3(p.p2);
  float denom = dot(n, r.d);
  if ((double)fabsf(denom) < kEpsilonD) return false;
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
  return true;
}

// primitives/Triangle.cpp:49-80.
template <uint32_t K>
NE_D bool triIntersect(const DScene& s, const DPrim& p, const Ray& r, Hit& h) {
  V3 a = ld3(p.p0), b = ld3(p.p1), c = ld3(p.p2);
  V3 v1v0 = b - a, v2v0 = c - a, rov0 = r.o - a;
  V3 normal = cross(v1v0, v2v0);
  V3 q = cross(rov0, r.d);
  float denom = 1.0f / dot(r.d, normal);  // equals (float)(1.0 / (double)dot)
  float u = dot(-q, v2v0) * denom;
  float v = dot(q, v1v0) * denom;
  float t = dot(-normal, rov0) * denom;
  if (nefm::isnan_(t) || t < 0) return false;
  if (u < 0.0f || u > 1.0f || v < 0.0f || (u + v) > 1.0f) return false;
  h.tNear = t;
  h.tFar = t;
  h.hitPoint = r.at(h.tNear);
  if ((K & FT_NORMALMAP) && p.material >= 0 && (s.materials[p.material].tex_types & NE_TEX_NORMAL)) {
    const DMaterial& m = s.materials[p.material];
    V3 tn = (m.tex_present & NE_TEX_NORMAL) ? ld3(m.normal_map) : v3(0, 0, 0);
    h.normal = convertNormalFromTextureMap(tn, normalize(normal));
  } else {
    h.normal = normalize(normal);
  }
  return true;
}

template <uint32_t K>
NE_D bool primIntersect(const DScene& s, Counters& cnt, int idx, const Ray& r, Hit& h) {
  const DPrim& p = s.prims[idx];
  if ((K & K_COUNT) && p.type == NE_PRIM_TRIANGLE) cnt.tests++;
  bool hit = false;
  if ((K & FT_SPHERE) && p.type == NE_PRIM_SPHERE) {
    hit = sphereIntersect(p, r, h);
  } else if ((K & FT_RECT) && p.type == NE_PRIM_RECTANGLE) {
    hit = rectIntersect(p, r, h);
  } else if ((K & FT_AABB) && p.type == NE_PRIM_AABB) {
    hit = aabbIntersect(ld3(p.p0), ld3(p.p1), r, h);
    h.prim = idx;
    return hit;
  } else if ((K & FT_TRI) && p.type == NE_PRIM_TRIANGLE) {
    hit = triIntersect<K>(s, p, r, h);
  } else {
    return false;
  }
  if (hit) h.prim = idx;
  return hit;
}

// primitives/BVH.cpp:108-193 BVH::intersect (near-first stack traversal).
template <uint32_t K>
NE_D bool bvhIntersect(const DScene& sc, uint32_t* err, Counters& cnt, const DModel& m, const Ray& r, Hit& out) {
  const float inf = __int_as_float(0x7f800000);
  uint32_t stackNode[kBvhStack];
  float stackT[kBvhStack];
  int sp = 0;
  stackNode[0] = 0;
  stackT[0] = inf;
  Hit closest = emptyHit();
  closest.tNear = inf;
  closest.tFar = -inf;
  bool anyHit = false;
  V3 s = v3((r.d.x < 0.0f) ? 1.0f : -1.0f, (r.d.y < 0.0f) ? 1.0f : -1.0f, (r.d.z < 0.0f) ? 1.0f : -1.0f);
  V3 invD = v3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
  const DNode* nodes = sc.bvh + m.bvh_node0;
  const uint32_t* slots = sc.bvh_prims + m.bvh_slot0;
  while (sp >= 0) {
    uint32_t ni = stackNode[sp];
    float nearest = stackT[sp];
    sp--;
    if (nearest > closest.tNear) continue;
    float4 hi = __ldg(reinterpret_cast<const float4*>(&nodes[ni].hi));
    uint32_t b = __float_as_uint(hi.w);
    if (K & K_COUNT) cnt.nodes++;
    if (b & 0x80000000u) {
      float4 lo = __ldg(reinterpret_cast<const float4*>(&nodes[ni].lo));
      uint32_t start = __float_as_uint(lo.w), count = b & 0x7fffffffu;
      for (uint32_t i = 0; i < count; i++) {
        Hit tmp = emptyHit();
        bool cur = primIntersect<K>(sc, cnt, (int)slots[start + i], r, tmp);
        anyHit = anyHit || cur;
        if (cur && tmp.tNear < closest.tNear) closest = tmp;
      }
    } else {
      float4 lo = __ldg(reinterpret_cast<const float4*>(&nodes[ni].lo));
      uint32_t ro = __float_as_uint(lo.w);
      uint32_t c0 = ni + 1, c1 = ni + ro;
      float4 l0 = __ldg(reinterpret_cast<const float4*>(&nodes[c0].lo));
      float4 h0 = __ldg(reinterpret_cast<const float4*>(&nodes[c0].hi));
      float4 l1 = __ldg(reinterpret_cast<const float4*>(&nodes[c1].lo));
      float4 h1 = __ldg(reinterpret_cast<const float4*>(&nodes[c1].hi));
      float tn0, tn1;
      bool hit0 = aabbNear(v3(l0.x, l0.y, l0.z), v3(h0.x, h0.y, h0.z), r, invD, s, tn0);
      bool hit1 = aabbNear(v3(l1.x, l1.y, l1.z), v3(h1.x, h1.y, h1.z), r, invD, s, tn1);
      if (hit0 && hit1) {
        uint32_t closer = c0, other = c1;
        float tc = tn0, to = tn1;
        if (tn1 < tn0) {
          closer = c1; other = c0;
          tc = tn1; to = tn0;
        }
        if (sp + 2 >= kBvhStack) { atomicOr(err, ERR_BVH_STACK); break; }
        stackNode[++sp] = other; stackT[sp] = to;
        stackNode[++sp] = closer; stackT[sp] = tc;
      } else if (hit0) {
        if (sp + 1 >= kBvhStack) { atomicOr(err, ERR_BVH_STACK); break; }
        stackNode[++sp] = c0; stackT[sp] = tn0;
      } else if (hit1) {
        if (sp + 1 >= kBvhStack) { atomicOr(err, ERR_BVH_STACK); break; }
        stackNode[++sp] = c1; stackT[sp] = tn1;
      }
    }
  }
  out = closest;
  return anyHit;
}

// Kernels for meshes with media call the traversal from three places per bounce (bounce ray,
// shadow ray, the MIS walk); there one out-of-line copy keeps the kernel's instruction
// footprint small (64 views: 94 -> 104 Mpaths/s, both built for 8 resident blocks per SM).
// Kernels for meshes without media have two call sites and stay inlined (outlined: 443 -> 437
// at 10 blocks per SM).
#ifndef NE_OUTLINE_BVH
#define NE_OUTLINE_BVH 1
#endif
template <uint32_t K>
struct OutlineBvh {
  static constexpr bool value = NE_OUTLINE_BVH && !(K & K_COUNT) && (K & FT_TRI) && (K & (FT_GRID | FT_HOMOG));
};
template <uint32_t K>
__device__ __noinline__ bool bvhIntersectOutlined(const DScene* sc, uint32_t* err, const DModel* m, Ray r, Hit* out) {
  Counters none{0, 0, 0, 0};
  return bvhIntersect<K>(*sc, err, none, *m, r, *out);
}

// ---------------------------------------------------------------- environment maps
// One texture coordinate of Texture::sample with NE_TEX_SAMPLER_UVW_MIRROR and nearest lookup
// (materials/Texture.cpp:88-129): mirror wrap |u - (int)u| clamped to [0, 1], texel (int)(u n),
// the edge u = 1 folded onto the last texel. A coordinate that is not a number or exceeds the
// int range (a NaN direction; undefined behaviour in the reference) reads texel 0.
NE_D int texCoord(float u, int n) {
  if (!(u >= -2147483520.0f && u <= 2147483520.0f)) return 0;
  u = gmin(gmax(fabsf(u - (float)(int)u), 0.0f), 1.0f);
  int x = (int)(u * (float)n);
  if (x > 0 && x == n) x--;
  return x;
}
// RGB of an RGBA8 texel, each channel / 255 (Texture.cpp:69-81).
NE_D V3 envTexel(const DLight& L, float u, float v) {
  uchar4 t = L.env_tex[(uint32_t)texCoord(v, L.env_h) * (uint32_t)L.env_w + (uint32_t)texCoord(u, L.env_w)];
  return v3((float)t.x / 255.0f, (float)t.y / 255.0f, (float)t.z / 255.0f);
}
// InfiniteAreaLight::Le (lights/InfiniteAreaLight.h:46-55): the direction through `M` (the
// light instance's invTransformToWCS, or the identity), normalised, in the frame of (0, 0, 1);
// (getSphericalPhi / 2pi, getSphericalTheta / pi) of it (utils/Math.h:1148-1155) indexes the map.
NE_D V3 envLe(const DLight& L, const float* M, V3 d) {
  V3 w = normalize(mul4(M, d, 0.0f));
  V3 n = v3(0, 0, 1), ss, ts;
  orthonormal(n, ss, ts);
  V3 inc = toLCS(w, n, ss, ts);
  float p = nefm::atan2(inc.y, inc.x);
  float phi = (p < 0) ? __double2float_rn((double)p + kTwoPiD) : p;
  float theta = nefm::acos(gmin(gmax(inc.z, -1.0f), 1.0f));
  return envTexel(L, __double2float_rn((double)phi * kInv2PiD), __double2float_rn((double)theta * kInvPiD));
}
// Distribution1D::sampleContinuous (utils/Sampling.h:34-51) with binarySearch
// (utils/Math.h:1130-1146) over the n + 1 CDF entries.
NE_D float sample1D(const float* func, const float* cdf, int n, float funcInt, float u, float* pdf, int* off) {
  int first = 0, len = n + 1;
  while (len > 0) {
    int half = len >> 1, middle = first + half;
    if (cdf[middle] <= u) {
      first = middle + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  int o = first - 1 < 0 ? 0 : (first - 1 > n - 1 ? n - 1 : first - 1);
  float du = u - cdf[o];
  if ((cdf[o + 1] - cdf[o]) > 0) du /= (cdf[o + 1] - cdf[o]);
  *pdf = (funcInt > 0) ? func[o] / funcInt : 0;
  *off = o;
  return ((float)o + du) / (float)n;
}
// Distribution2D::sampleContinuous (utils/Sampling.h:98-105): the row from the marginal, then
// the position within it.
NE_D void envSample(const DLight& L, float u0, float u1, float& d0, float& d1, float& pdf) {
  const int H = L.env_h;
  float p0, p1;
  int v, unused;
  d1 = sample1D(L.env_marg_func, L.env_marg_cdf, H, L.env_marg_int, u1, &p1, &v);
  d0 = sample1D(L.env_cond_func + (size_t)v * H, L.env_cond_cdf + (size_t)v * (H + 1), H, L.env_cond_int[v], u0, &p0,
                &unused);
  pdf = p0 * p1;
}

// Light::Le(ray, M) (lights/Light.h:20-22), DirectionalLight::Le, InfiniteAreaLight::Le.
template <uint32_t K>
NE_D V3 lightLe(const DLight& L, const float* M, V3 d) {
  if (L.type == NE_LIGHT_INFINITE) {
    if ((K & FT_ENVMAP) && L.env_w > 0) return envLe(L, M, d);
    return ld3(L.env_radiance);
  }
  return ld3(L.le);
}
// The identity matrix Model::intersect passes to Light::Le (primitives/Model.cpp:435).
__device__ __constant__ const float kIdentity12[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
NE_D V3 lightLi(const DLight& L) {  // Light::Li, DirectionalLight::Li
  if (L.type == NE_LIGHT_DIRECTIONAL) return ld3(L.le);
  return ld3(L.li);
}

// primitives/Model.cpp:372-447 Model::intersect.
template <uint32_t K>
NE_D bool modelIntersect(Ctx<K>& c, uint32_t mi, const Ray& ray, Hit& hit, float& tMin, float& tMax) {
  const DModel& m = c.s.models[mi];
  bool did = false;
  Hit temp = emptyHit();
  if ((K & FT_BBOX) && m.has_bbox)
    if (!aabbIntersect(ld3(m.bbox_min), ld3(m.bbox_max), ray, temp)) return false;
  if ((K & FT_TRI) && m.use_bvh) {
    bool local;
    if constexpr (OutlineBvh<K>::value)
      local = bvhIntersectOutlined<K>(&c.s, c.err, &m, ray, &temp);
    else
      local = bvhIntersect<K>(c.s, c.err, c.c, m, ray, temp);
    if (local && temp.tNear > tMin && temp.tNear < tMax) {
      tMax = temp.tNear;
      hit = temp;
      did = true;
    }
    return did;
  }
  for (uint32_t k = 0; k < m.prim_count; k++) {
    int pi = (int)(m.prim_begin + k);
    const DPrim& p = c.s.prims[pi];
    if ((K & FT_GRID) && (p.flags & DPRIM_GRID_MEDIUM)) {
      primIntersect<K>(c.s, c.c, pi, ray, temp);
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
    bool local = primIntersect<K>(c.s, c.c, pi, ray, temp);
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
    const DPrim& p = c.s.prims[pi];
    const DLight& L = c.s.lights[c.s.materials[p.material].light];
    if (!isBlack(lightLe<K>(L, kIdentity12, ray.d))) continue;
    bool local = primIntersect<K>(c.s, c.c, pi, ray, temp);
    if (local && temp.tNear > tMin && temp.tNear < tMax) {
      tMax = temp.tNear;
      hit = temp;
      did = true;
    }
  }
  return did;
}

// primitives/InstancedModel.cpp:24-38.
template <uint32_t K>
NE_D bool instanceIntersect(Ctx<K>& c, uint32_t ii, const Ray& ray, Hit& hit, float& tMin, float& tMax) {
  const DInstance& in = c.s.instances[ii];
  if (!in.collision || in.never_hit) return false;
  Ray r = transformRay(ray, in.ocs);
  bool did = modelIntersect(c, in.model, r, hit, tMin, tMax);
  if (did) {
    hit.hitPoint = mul4(in.wcs, hit.hitPoint, 1.0f);
    hit.normal = normalize(mul4(in.wcs, hit.normal, 0.0f));
    hit.inst = (int)ii;
  }
  return did;
}

// core/Scene.cpp:30-56.
template <uint32_t K>
NE_NI bool intersectScene(Ctx<K>& c, const Ray& ray, Hit& hit, float tMin, float tMax) {
  bool did = false;
  hit.prim = -1;
  if (K & K_COUNT) c.c.queries++;
  Hit temp = emptyHit();
  float curMin = tMin, curMax = tMax;
  uint32_t total = c.s.n_instances + c.s.n_light_instances;
  for (uint32_t i = 0; i < total; i++) {
    bool t = instanceIntersect(c, i, ray, temp, curMin, curMax);
    if (t) hit = temp;
    did = did || t;
  }
  return did;
}

// ---------------------------------------------------------------- materials
NE_D V3 texValue(const DMaterial& m, int bit) {  // Material::sampleMaterial, constant textures
  if (!(m.tex_present & bit)) return v3(0, 0, 0);
  switch (bit) {
    case NE_TEX_ALBEDO: return ld3(m.albedo);
    case NE_TEX_ROUGHNESS: return v3(m.roughness, 0, 0);
    case NE_TEX_METALLIC: return v3(m.metallic, 0, 0);
    case NE_TEX_NORMAL: return ld3(m.normal_map);
  }
  return v3(0, 0, 0);
}
// core/Microfacet.cpp:5-14.
NE_D float ggxD(float alpha, V3 m) {
  float a2 = alpha * alpha;
  float NdotH = m.z;
  float NdotH2 = NdotH * NdotH;
  float denom = NdotH2 * (a2 - 1.0f) + 1.0f;
  denom = __double2float_rn(gmaxd(kEpsilonD, kPiD * (double)denom * (double)denom));
  return a2 / denom;
}
// core/Microfacet.cpp:16-23.
NE_D float schlickGGX(float alpha, float NdotV) {
  float k = alpha / 2.0f;
  float nom = NdotV;
  float denom = __double2float_rn(gmaxd(kEpsilonD, (double)NdotV * (1.0 - (double)k) + (double)k));
  return nom / denom;
}
// core/Microfacet.cpp:25-35.
NE_D float ggxG(float alpha, V3 wi, V3 wo) {
  V3 n = normalize(wi + wo);
  float NoV = dot(n, wi), NoL = dot(n, wo);
  float NdotV = gmax(NoV, 0.0f), NdotL = gmax(NoL, 0.0f);
  return schlickGGX(alpha, NdotV) * schlickGGX(alpha, NdotL);
}
// core/Microfacet.cpp:37-56.
NE_D V3 ggxSample(float alpha, V3 wi, Sampler& S) {
  float rx = S.random();
  float ry = S.random();
  float a2 = alpha * alpha;
  float theta = nefm::acos(gmin(1.0f, nefm::fsqrt((1.0f - rx) / gmax(float(kEpsilonD), (rx * (a2 - 1.0f) + 1.0f)))));
  float phi = __double2float_rn(kTwoPiD * (double)ry);
  V3 m = v3(nefm::sin(theta) * nefm::cos(phi), nefm::sin(theta) * nefm::sin(phi), nefm::cos(theta));
  return reflect(normalize(wi), normalize(m));
}
// core/Microfacet.cpp:58-65.
NE_D float ggxPdf(float alpha, V3 scattered, V3 m) {
  float NdotH = m.z;
  float VdotH = dot(scattered, m);
  float Dp = ggxD(alpha, m) * NdotH;
  return Dp / (4 * VdotH);
}
// core/BSDF.h:150-157.
NE_D V3 fresnel(float cosTheta) {
  V3 f0 = v3(0.04f, 0.04f, 0.04f);
  return f0 + (v3(1, 1, 1) - f0) * nefm::pow5(1.0f - cosTheta);
}
// core/GlossyBSDF.cpp:25-48.
NE_D V3 glossyEval(const DMaterial& m, V3 wi, V3 wo, V3 albedo) {
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
  kD = kD * __double2float_rn(1.0 - (double)metallic);
  return ((albedo / float(kPiD)) * kD + specular) * NdotL;
}
NE_D float glossyPdf(const DMaterial& m, V3 wi, V3 wo) {  // GlossyBSDF.cpp:17-23
  V3 mh = normalize(wi + wo);
  float rough = texValue(m, NE_TEX_ROUGHNESS).x;
  return ggxPdf(rough * rough, wo, mh);
}
NE_D V3 glossySample(const DMaterial& m, V3 wi, Sampler& S) {  // GlossyBSDF.cpp:10-15
  float rough = texValue(m, NE_TEX_ROUGHNESS).x;
  return ggxSample(rough * rough, wi, S);
}
// materials/Medium.h:116-128 HG eval/pdf, :56-62 isotropic.
template <uint32_t K>
NE_D float phaseEval(const DMaterial& m, V3 wi, V3 wo) {
  if (m.phase == NE_PHASE_ISOTROPIC) return __double2float_rn(1.0 / kFourPiD);
  float g = m.g;
  float cosT = dot(normalize(wi), normalize(wo));
  float denom = (1.0f + g * g) - (2.0f * g) * cosT;
  return (kInv4Pi * (1.0f - g * g)) / (denom * nefm::fsqrt(denom));
}
// materials/Medium.h:96-114 HG sample, :45-47 isotropic.
template <uint32_t K>
NE_D V3 phaseSample(const DMaterial& m, Sampler& S) {
  if (m.phase == NE_PHASE_ISOTROPIC) {
    float e1 = S.random();
    float e2 = S.random();
    return sampleUnitSphere(e1, e2);
  }
  float g = m.g;
  float u0 = S.random();
  float u1 = S.random();
  float cosTheta;
  if (fabsf(g) < 1e-3f)
    cosTheta = 1.0f - 2.0f * u0;
  else {
    float sqr = (1.0f - g * g) / ((1.0f + g) - (2.0f * g) * u0);
    sqr = sqr * sqr;
    cosTheta = (-1.0f / (2.0f * g)) * ((1.0f + g * g) - sqr);
  }
  float sinTheta = nefm::fsqrt(1.0f - cosTheta * cosTheta);
  float phi = __double2float_rn((2.0 * kPiD) * (double)u1);
  return v3(nefm::cos(phi) * sinTheta, nefm::sin(phi) * sinTheta, cosTheta);
}
// core/BSDF.h:100-106.
template <uint32_t K>
NE_NI V3 bsdfSample(const DMaterial& m, V3 incoming, V3 normal, Sampler& S) {
  V3 ss, ts;
  orthonormal(normal, ss, ts);
  V3 wi = toLCS(-normalize(incoming), normal, ss, ts);
  V3 sc = v3(0, 0, 0);
  if ((K & FT_VOLBSDF) && m.bsdf == NE_BSDF_VOLUME)
    sc = phaseSample<K>(m, S);
  else if (K & FT_GLOSSY)
    sc = glossySample(m, wi, S);
  return toWorld(sc, normal, ss, ts);
}
// core/BSDF.h:117-125.
template <uint32_t K>
NE_NI float bsdfPdf(const DMaterial& m, V3 incoming, V3 scattered, V3 normal) {
  bool trans = (K & FT_VOLBSDF) && (m.bsdf == NE_BSDF_VOLUME);
  if (!trans && (!sameHemisphere(-incoming, normal) || !sameHemisphere(scattered, normal))) return 0;
  V3 ss, ts;
  orthonormal(normal, ss, ts);
  V3 wi = toLCS(-normalize(incoming), normal, ss, ts);
  V3 wo = toLCS(scattered, normal, ss, ts);
  if (trans) return phaseEval<K>(m, wi, wo);
  return (K & FT_GLOSSY) ? glossyPdf(m, wi, wo) : 0.0f;
}
// Rectangle::samplePointOnTexture (primitives/Rectangle.cpp:115-157) at the object-space point
// q of a hit: barycentric coordinates (:91-113) of q in the triangle (v0, v1, v2) of the
// rectangle's corners, or in (v3, v1, v2) when those leave [0, 1], weighting the corners'
// texture coordinates (0,0), (1,0), (1,1), (0,1). The corners as SceneReader lays them out
// (io/SceneReader.cpp:407-463): v0 = p0, v2 = p1 (opposite), v1 = (p1.x, p0.y, p0.z),
// v3 = (p0.x, p1.y, p0.z).
NE_D void rectBary(V3 p, V3 a, V3 b, V3 c, float& l0, float& l1, float& l2) {
  V3 v0 = b - a, v1 = c - a, v2 = p - a;
  float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
  float d20 = dot(v2, v0), d21 = dot(v2, v1);
  float denom = d00 * d11 - d01 * d01;
  l1 = (d11 * d20 - d01 * d21) / denom;
  l2 = (d00 * d21 - d01 * d20) / denom;
  l0 = 1.0f - l1 - l2;
}
NE_D void rectUV(const DPrim& p, V3 q, float& u, float& v) {
  V3 c0 = ld3(p.p0), c2 = ld3(p.p1);
  V3 c1 = v3(c2.x, c0.y, c0.z), c3 = v3(c0.x, c2.y, c0.z);
  float a0, a1, a2;
  rectBary(q, c0, c1, c2, a0, a1, a2);
  if (a0 < 0 || a1 < 0 || a2 < 0 || a0 > 1 || a1 > 1 || a2 > 1) {
    rectBary(q, c3, c1, c2, a0, a1, a2);
    u = (a0 * 0.0f + a1 * 1.0f) + a2 * 1.0f;  // uv3 = (0, 1), uv1 = (1, 0), uv2 = (1, 1)
    v = (a0 * 1.0f + a1 * 0.0f) + a2 * 1.0f;
  } else {
    u = (a0 * 0.0f + a1 * 1.0f) + a2 * 1.0f;  // uv0 = (0, 0), uv1 = (1, 0), uv2 = (1, 1)
    v = (a0 * 0.0f + a1 * 0.0f) + a2 * 1.0f;
  }
}
// Material::sampleMaterial(ALBEDO, hit.uv) (materials/Material.h:62-69): a textured albedo is
// looked up at the hit's texture coordinates, which the rectangle computes from its
// object-space hit point (Rectangle.cpp:71) and every other primitive leaves at (0, 0)
// (Sphere.cpp:37, AABB.cpp:68; triangles read no texture coordinates here). The point is
// recomputed from the ray that produced the hit, in the same operations as the intersection.
template <uint32_t K>
NE_D V3 albedoAt(const DScene& s, const DMaterial& m, const Ray& incoming, const Hit& h) {
  if ((K & FT_TEXALB) && m.albedo_w > 0) {
    float u = 0.0f, v = 0.0f;
    const DPrim& p = s.prims[h.prim];
    if ((K & FT_RECT) && p.type == NE_PRIM_RECTANGLE) {
      Ray r = transformRay(incoming, s.instances[h.inst].ocs);
      rectUV(p, r.at(h.tNear), u, v);
    }
    uchar4 t = m.albedo_tex[(uint32_t)texCoord(v, m.albedo_h) * (uint32_t)m.albedo_w + (uint32_t)texCoord(u, m.albedo_w)];
    return v3((float)t.x / 255.0f, (float)t.y / 255.0f, (float)t.z / 255.0f);
  }
  return texValue(m, NE_TEX_ALBEDO);
}
// core/BSDF.h:135-142, for the hit `isect` of the ray `incoming`.
template <uint32_t K>
NE_NI V3 bsdfEval(const DScene& s, const DMaterial& m, const Ray& incoming, V3 scattered, const Hit& isect) {
  const V3 normal = isect.normal;
  bool trans = (K & FT_VOLBSDF) && (m.bsdf == NE_BSDF_VOLUME);
  if (!trans && (!sameHemisphere(-incoming.d, normal) || !sameHemisphere(scattered, normal))) return v3(0, 0, 0);
  V3 ss, ts;
  orthonormal(normal, ss, ts);
  V3 wi = toLCS(-normalize(incoming.d), normal, ss, ts);
  V3 wo = toLCS(scattered, normal, ss, ts);
  if (trans) {
    float p = phaseEval<K>(m, wi, wo);
    return v3(p, p, p);
  }
  return (K & FT_GLOSSY) ? glossyEval(m, wi, wo, albedoAt<K>(s, m, incoming, isect)) : v3(0, 0, 0);
}

// ---------------------------------------------------------------- media
NE_D float lerp(float a, float b, float t) { return a * (1.0f - t) + b * t; }

// materials/GridMedia.cpp:25-43 interpolatedDensity(fromOCStoGCS(p)): clamp to [0,res],
// floor, trilinear over the 8 corners with density 0 at index >= res. The 8 corners of
// cell (ix,iy,iz) are stored together (two float4, one 32-byte sector), so a lookup is
// one aligned read; the values and the interpolation order are those of the dense grid.
template <uint32_t K>
NE_D float sampleAt(Ctx<K>& c, const DMedium& M, const Ray& r, float t) {
  if (K & K_COUNT) c.c.lookups++;
  V3 p = r.at(t);
  V3 res = ld3(M.resf);
  V3 g = (p + v3(0.5f, 0.5f, 0.5f)) * res;
  g = vmin(vmax(v3(0, 0, 0), g), res);
  float fx = floorf(g.x), fy = floorf(g.y), fz = floorf(g.z);
  int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  // g is clamped to [0, res] (res <= 2^24), so each floor is an integer-valued float that
  // equals (float)(int) of itself: the fraction needs no conversion back
  V3 d = g - v3(fx, fy, fz);
  float c000, c100, c010, c110, c001, c101, c011, c111;
  if (M.cells) {
    size_t cell = ((size_t)iz * (M.res[1] + 1) + (size_t)iy) * (M.res[0] + 1) + (size_t)ix;
    float4 a = __ldg(&M.cells[2 * cell]);
    float4 b = __ldg(&M.cells[2 * cell + 1]);
    c000 = a.x; c100 = a.y; c010 = a.z; c110 = a.w;
    c001 = b.x; c101 = b.y; c011 = b.z; c111 = b.w;
  } else {
    const uint32_t W = M.res[0], H = M.res[1], D = M.res[2];
    auto den = [&](int x, int y, int z) -> float {
      if ((uint32_t)x >= W || (uint32_t)y >= H || (uint32_t)z >= D) return 0.0f;
      return __ldg(&M.grid[(size_t)H * W * (uint32_t)z + (size_t)W * (uint32_t)y + (uint32_t)x]);
    };
    c000 = den(ix, iy, iz); c100 = den(ix + 1, iy, iz);
    c010 = den(ix, iy + 1, iz); c110 = den(ix + 1, iy + 1, iz);
    c001 = den(ix, iy, iz + 1); c101 = den(ix + 1, iy, iz + 1);
    c011 = den(ix, iy + 1, iz + 1); c111 = den(ix + 1, iy + 1, iz + 1);
  }
  float d00 = lerp(c000, c100, d.x);
  float d10 = lerp(c010, c110, d.x);
  float d01 = lerp(c001, c101, d.x);
  float d11 = lerp(c011, c111, d.x);
  float d0 = lerp(d00, d10, d.y);
  float d1 = lerp(d01, d11, d.y);
  return lerp(d0, d1, d.z);
}

// materials/GridMedia.cpp:45-69 GridMedia::Tr (ratio tracking).
template <uint32_t K>
NE_NI V3 gridTr(Ctx<K>& c, const DMedium& M, Ray incoming, Hit isect) {
  incoming = transformRay(incoming, c.s.instances[isect.inst].ocs);
  incoming.o = incoming.at(isect.tNear);
  isect.tFar = isect.tFar - isect.tNear;
  isect.tNear = 0;
  float invMax = M.inv_max_density;
  float mu = M.mu;
  float Tr = 1, t = isect.tNear;
  for (int step = 0; step < kMaxTrackSteps; step++) {
    t -= (nefm::log1m_draw(c.S.randomInline()) * invMax) / mu;
    if (t >= isect.tFar) break;
    float density = sampleAt(c, M, incoming, t);
    float x = density * invMax;
    Tr *= 1 - ((0.0f < x) ? x : 0.0f);
    if (Tr < 0.1f) {
      float q = (0.05f < 1.0f - Tr) ? (1.0f - Tr) : 0.05f;
      if (c.S.random() < q) return v3(0, 0, 0);
      Tr /= 1 - q;
    }
  }
  return v3(Tr, Tr, Tr);
}

// materials/GridMedia.cpp:71-99 GridMedia::sample (delta tracking).
template <uint32_t K>
NE_D V3 gridSample(Ctx<K>& c, const DMedium& M, Ray incoming, Ray& scattered, const Hit& isect) {
  scattered.o = incoming.o;
  scattered.d = incoming.d;
  const DInstance& in = c.s.instances[isect.inst];
  incoming = transformRay(incoming, in.ocs);
  float invMax = M.inv_max_density;
  float mu = M.mu;
  float t = isect.tNear;
  for (int step = 0; step < kMaxTrackSteps; step++) {
    float r = c.S.randomInline();
    float sampledDist = (nefm::log1m_draw(r) * invMax) / mu;
    t -= sampledDist;
    if (t >= isect.tFar) {
      scattered.o = incoming.at(isect.tFar + 0.0001f);
      break;
    }
    float density = sampleAt(c, M, incoming, t);
    float ra = c.S.randomInline();
    if (density * invMax > ra) {
      scattered.o = incoming.at(t);
      const DMaterial& m = c.s.materials[c.s.prims[isect.prim].material];
      scattered.d = bsdfSample<K>(m, incoming.d, v3(0, 1, 0), c.S);
      scattered = transformRay(scattered, in.wcs);
      return ld3(M.sigma_s) / ld3(M.sigma_t);
    }
  }
  return v3(1, 1, 1);
}

// materials/HomogeneousMedia.cpp:15-51.
NE_D V3 homogTr(const DMedium& M, float distance) {
  V3 v = (ld3(M.sigma_t) * distance) * M.density;
  return v3(nefm::exp(-v.x), nefm::exp(-v.y), nefm::exp(-v.z));
}
template <uint32_t K>
NE_D V3 homogSample(Ctx<K>& c, const DMedium& M, Ray incoming, Ray& scattered, const Hit& isect) {
  float t = (-nefm::log(1 - c.S.random())) / avg(ld3(M.sigma_t));
  float dist = isect.tFar - isect.tNear;
  t = t / dist;
  bool sampled = t < dist;
  if (sampled) {
    scattered.o = incoming.at(t);
    scattered.d = bsdfSample<K>(c.s.materials[c.s.prims[isect.prim].material], incoming.d, isect.normal, c.S);
  } else {
    scattered.o = incoming.at(dist + 0.001f);
    scattered.d = incoming.d;
  }
  V3 Tr = homogTr(M, t);
  V3 density = sampled ? (ld3(M.sigma_t) * Tr) : Tr;
  float pdf = avg(density);
  if (pdf == 0) pdf = 1;
  return sampled ? ((Tr * ld3(M.sigma_s)) / pdf) : Tr / pdf;
}

template <uint32_t K>
NE_D V3 mediumTr(Ctx<K>& c, int med, const Ray& r, const Hit& isect) {
  const DMedium& M = c.s.media[med];
  if ((K & FT_GRID) && M.type == NE_MEDIUM_GRID) return gridTr(c, M, r, isect);
  if (K & FT_HOMOG) return homogTr(M, isect.tFar - isect.tNear);
  return v3(1, 1, 1);
}
template <uint32_t K>
NE_D V3 mediumSample(Ctx<K>& c, int med, const Ray& r, Ray& scattered, const Hit& isect) {
  const DMedium& M = c.s.media[med];
  if ((K & FT_GRID) && M.type == NE_MEDIUM_GRID) return gridSample(c, M, r, scattered, isect);
  if (K & FT_HOMOG) return homogSample(c, M, r, scattered, isect);
  return v3(1, 1, 1);
}

// ---------------------------------------------------------------- lights
// Primitive::samplePointOnSurface (Rectangle.cpp:78-88, Sphere.cpp:46-52,
// Triangle.cpp:114-119, Point.cpp:14-18, AABB.cpp:81-83).
template <uint32_t K>
NE_NI V3 samplePointOnSurface(const DScene& s, int pi, const Hit& isect, const float* M, Sampler& S) {
  const DPrim& p = s.prims[pi];
  switch (p.type) {
    case NE_PRIM_RECTANGLE: {
      if (!(K & FT_RECT)) break;
      float e0 = S.random();
      float e1 = S.random();
      float e2 = S.random();
      V3 v0 = ld3(p.p0);
      V3 size = rectSize(ld3(p.p0), ld3(p.p1));
      V3 q = v3(v0.x + size.x * e0, v0.y + size.y * e1, v0.z + size.z * e2);
      return mul4(M, q, 1.0f);
    }
    case NE_PRIM_SPHERE: {
      if (!(K & FT_SPHERE)) break;
      V3 cc = mul4(M, ld3(p.p0), 1.0f);
      V3 n = normalize(isect.hitPoint - cc);
      return cc + n * p.radius;
    }
    case NE_PRIM_TRIANGLE: {
      if (!(K & FT_TRI)) break;
      float ex = S.random();
      float ey = S.random();
      float sq = nefm::fsqrt(ex);
      float a = 1.0f - sq, b = ey * sq;
      return (a * ld3(p.p0) + b * ld3(p.p1)) + ((1 - a) - b) * ld3(p.p2);
    }
    case NE_PRIM_POINT:
      if (K & FT_POINT) return mul4(M, ld3(p.p0), 1.0f);
      break;
    default: break;
  }
  return v3(0, 0, 0);
}
// Primitive::pdf (Rectangle.cpp:159-171, Sphere.cpp:58-68, Triangle.cpp:159-161).
template <uint32_t K>
NE_NI float primPdf(const DScene& s, int pi, const Hit& isect, const DInstance& lin, Sampler& S) {
  const DPrim& p = s.prims[pi];
  switch (p.type) {
    case NE_PRIM_RECTANGLE: {
      if (!(K & FT_RECT)) return 1;
      V3 size = rectSize(ld3(p.p0), ld3(p.p1));
      V3 sizeWCS = ld3(lin.scale) * size;
      float area = 1;
      if (sizeWCS.x != 0) area = area * sizeWCS.x;
      if (sizeWCS.y != 0) area = area * sizeWCS.y;
      if (sizeWCS.z != 0) area = area * sizeWCS.z;
      return convertAreaToSolidAngle(1.0f / area, isect.normal, isect.hitPoint,
                                     samplePointOnSurface<K>(s, pi, isect, lin.wcs, S));
    }
    case NE_PRIM_SPHERE: {
      if (!(K & FT_SPHERE)) return 1;
      float pdfArea = __double2float_rn((double)(1.0f / 4.0f) * kPiD * (double)p.radius * (double)p.radius);
      return convertAreaToSolidAngle(pdfArea, isect.normal, isect.hitPoint, samplePointOnSurface<K>(s, pi, isect, lin.wcs, S));
    }
    case NE_PRIM_TRIANGLE:
      if (!(K & FT_TRI)) return 1;
      return convertAreaToSolidAngle(1.0f / p.area, isect.normal, isect.hitPoint,
                                     samplePointOnSurface<K>(s, pi, isect, lin.wcs, S));
    default: return 1;
  }
}

// Light::sampleLi (DiffuseLight.cpp:8-20, DirectionalLight.cpp:12-18, InfiniteAreaLight.h:83-113).
template <uint32_t K>
NE_NI V3 sampleLi(const DScene& s, const DLight& L, const Hit& isect, const DInstance& lin, Ray& wo, float& pdf,
                 Sampler& S) {
  switch (L.type) {
    case NE_LIGHT_DIFFUSE: {
      if (!(K & FT_LDIFF)) return v3(0, 0, 0);
      wo.o = isect.hitPoint;
      V3 q = samplePointOnSurface<K>(s, L.primitive, isect, lin.wcs, S);
      V3 d = q - wo.o;
      wo.d = normalize(d);
      pdf = primPdf<K>(s, L.primitive, isect, lin, S);
      return ld3(L.li);
    }
    case NE_LIGHT_DIRECTIONAL:
      if (!(K & FT_LDIR)) return v3(0, 0, 0);
      wo.o = isect.hitPoint;
      wo.d = -ld3(L.direction);
      pdf = 1;
      return ld3(L.li);
    default: {
      if (!(K & FT_LINF)) return v3(0, 0, 0);
      float u0 = S.random();
      float u1 = S.random();
      // Distribution2D::sampleContinuous; over the 1x1 map of a constant environment it returns
      // (u0, u1) itself with pdf 1 (or 0 for a black map)
      float uv0 = u0, uv1 = u1, mapPdf = L.env_map_pdf;
      if ((K & FT_ENVMAP) && L.env_w > 0) envSample(L, u0, u1, uv0, uv1, mapPdf);
      if (mapPdf == 0) return v3(0, 0, 0);
      float theta = __double2float_rn((double)uv1 * kPiD);
      float phi = __double2float_rn((double)(uv0 * 2) * kPiD);
      float cosTheta = nefm::cos(theta), sinTheta = nefm::sin(theta);
      float sinPhi = nefm::sin(phi), cosPhi = nefm::cos(phi);
      wo.o = isect.hitPoint;
      V3 polar = v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
      V3 ss, ts;
      orthonormal(v3(0, 1, 0), ss, ts);
      wo.d = toLCS(polar, v3(0, 1, 0), ss, ts);
      pdf = __double2float_rn((double)mapPdf / (2 * kPiD * kPiD * (double)sinTheta));
      if (sinTheta == 0) pdf = 0;
      if ((K & FT_ENVMAP) && L.env_w > 0) return envTexel(L, uv0, uv1);
      return ld3(L.env_radiance);
    }
  }
}

// ---------------------------------------------------------------- integrator
NE_D const DMaterial* matOf(const DScene& s, int prim) {
  if (prim < 0) return nullptr;
  int m = s.prims[prim].material;
  return m < 0 ? nullptr : &s.materials[m];
}

// integrators/VolumetricPathIntegrator.cpp:10-32 intersectTr.
template <uint32_t K>
NE_D bool intersectTr(Ctx<K>& c, Ray ray, Hit& intersection, V3* Tr) {
  const float inf = __int_as_float(0x7f800000);
  *Tr = v3(1, 1, 1);
  for (int seg = 0; seg < kMaxTrSegments; seg++) {
    Hit isect = emptyHit();
    bool hitSurface = intersectScene(c, ray, isect, kEps3F, inf);
    intersection = isect;
    int m = -1;
    const DMaterial* mat = hitSurface ? matOf(c.s, isect.prim) : nullptr;
    if (mat) m = mat->medium;
    if (m >= 0) *Tr = *Tr * mediumTr(c, m, ray, isect);
    if (!hitSurface) return false;
    if (m >= 0) return true;
    if (sameBits(isect.hitPoint, ray.o)) return false;
    ray.o = isect.hitPoint;
  }
  return false;
}

// False only when the ray's line, from its origin on, misses every medium's world-space box
// (widened at upload against rounding): intersectTr's walk along the ray can then reach no
// medium, so it returns false and draws nothing. NaN in the ray narrows nothing and answers
// true.
NE_D bool mayReachMedium(const DScene& s, const Ray& r) {
  if (s.n_medium_boxes < 0) return true;
  const float o[3] = {r.o.x, r.o.y, r.o.z}, d[3] = {r.d.x, r.d.y, r.d.z};
  for (int i = 0; i < s.n_medium_boxes; i++) {
    const float* b = s.medium_boxes + 6 * i;
    float tNear = 0.0f, tFar = __int_as_float(0x7f800000);
    bool miss = false;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const float lo = __ldg(b + a), hi = __ldg(b + 3 + a);
      if (d[a] == 0.0f) {
        if (o[a] < lo || o[a] > hi) miss = true;
      } else {
        const float t0 = (lo - o[a]) / d[a], t1 = (hi - o[a]) / d[a];
        const float tn = t0 < t1 ? t0 : t1, tf = t0 < t1 ? t1 : t0;
        if (tn > tNear) tNear = tn;
        if (tf < tFar) tFar = tf;
      }
    }
    if (!miss && !(tNear > tFar)) return true;
  }
  return false;
}

// integrators/VolumetricPathIntegrator.cpp:34-72 visibilityTr.
template <uint32_t K>
NE_D V3 visibilityTr(Ctx<K>& c, V3 p, V3 lightPoint) {
  const float inf = __int_as_float(0x7f800000);
  Ray ray{p, lightPoint - p};
  V3 Tr = v3(1, 1, 1);
  Hit isect = emptyHit();
  bool hitSurface = intersectScene(c, ray, isect, kEps3F, inf);
  if (!hitSurface) return Tr;
  const DMaterial* mat = matOf(c.s, isect.prim);
  if (!mat) return v3(0, 0, 0);
  if (mat->light >= 0) return Tr;
  if (mat->medium >= 0) Tr = Tr * mediumTr(c, mat->medium, ray, isect);
  return v3(0, 0, 0);
}

// integrators/VolumetricPathIntegrator.cpp:74-157 estimateDirect.
template <uint32_t K>
NE_NI V3 estimateDirect(Ctx<K>& c, const Ray& incoming, const Hit& isect, const DLight& light, uint32_t lightInst) {
  const DScene& s = c.s;
  const DInstance& lin = s.instances[lightInst];
  V3 Ld = v3(0, 0, 0);
  Ray wo{v3(0, 0, 0), v3(0, 0, 0)};
  float lightPdf = 0, scatteringPdf = 0;
  V3 Li = sampleLi<K>(s, light, isect, lin, wo, lightPdf, c.S);
  V3 f = v3(0, 0, 0);
  const DMaterial& mat = *matOf(s, isect.prim);
  bool surface = !(mat.medium >= 0);
  bool mediumF = false;  // f holds the phase value for (incoming.d, wo.d)
  if (lightPdf > 0 && !isBlack(Li)) {
    if (surface) {
      f = bsdfEval<K>(s, mat, incoming, wo.d, isect) * fabsf(dot(wo.d, isect.normal));
      scatteringPdf = bsdfPdf<K>(mat, incoming.d, wo.d, isect.normal);
    } else {
      f = bsdfEval<K>(s, mat, incoming, wo.d, isect);
      scatteringPdf = f.x;
      mediumF = true;
    }
    if (!isBlack(f)) {
      V3 pointOnLight = samplePointOnSurface<K>(s, light.primitive, isect, lin.wcs, c.S);
      V3 vis;
      if (shadowQueue<K>() && c.shadowVis) {
        // traced ahead by k_trace (the same visibilityTr on the same segment)
        vis = c.shadowVis == 1 ? v3(1, 1, 1) : v3(0, 0, 0);
        c.shadowVis = 0;
      } else {
        if (shadowQueue<K>() && c.deferShadow) {
          const uint32_t slot = appendSlot(c.dq->count);
          if (slot < c.dq->cap) {  // stop here: the caller queues the path with this segment
            c.shadowSlot = (int)slot;
            c.shadowPoint = pointOnLight;
            return Ld;
          }
        }
        vis = visibilityTr(c, isect.hitPoint, pointOnLight);
      }
      Li = Li * vis;
      if (!isBlack(Li)) {
        float weight = powerHeuristic(lightPdf, scatteringPdf);
        Ld = Ld + ((f * Li) * weight) / lightPdf;
      }
    }
  }
  if (surface) {
    wo.d = bsdfSample<K>(mat, incoming.d, isect.normal, c.S);
    f = bsdfEval<K>(s, mat, incoming, wo.d, isect);
    f = f * fabsf(dot(wo.d, isect.normal));
    scatteringPdf = bsdfPdf<K>(mat, incoming.d, wo.d, isect.normal);
  } else {
    // the reference evaluates the phase function at the light sample's direction again here
    // (VolumetricPathIntegrator.cpp:121-125); the value computed above is the same
    if (!mediumF) f = bsdfEval<K>(s, mat, incoming, wo.d, isect);
    wo.d = bsdfSample<K>(mat, incoming.d, v3(0, 1, 0), c.S);
    scatteringPdf = f.x;
  }
  if (!isBlack(f) && scatteringPdf > 0) {
    float weight = 1;
    lightPdf = primPdf<K>(s, light.primitive, isect, lin, c.S);
    if (lightPdf == 0) return Ld;
    weight = powerHeuristic(scatteringPdf, lightPdf);
    Hit lightIsect = emptyHit();
    Ray ray{isect.hitPoint, wo.d};
    V3 Tr = v3(1, 1, 1);
    // intersectTr reports a hit only where its ray reaches a medium: in a scene without media,
    // or (kernels for meshes with media) for a ray that misses every medium's box, it draws no
    // random number and returns false, so its walk through every surface on the ray cannot
    // change the result and is skipped
    bool found = false;
    if ((K & (FT_GRID | FT_HOMOG)) && s.n_media > 0 && (!(K & FT_TRI) || mayReachMedium(s, ray)))
      found = intersectTr(c, ray, lightIsect, &Tr);
    V3 Li2 = v3(0, 0, 0);
    if (found) Li2 = lightLi(light);
    if (!isBlack(Li2)) Ld = Ld + (((f * Li2) * Tr) * weight) / scatteringPdf;
  }
  return Ld;
}

// integrators/VolumetricPathIntegrator.cpp:159-174 and primitives/Model.cpp:478-485.
template <uint32_t K>
NE_D V3 uniformSampleOneLight(Ctx<K>& c, const Ray& incoming, const Hit& isect) {
  const DScene& s = c.s;
  float r = c.S.random();
  uint32_t nL = s.n_light_instances;
  if (nL == 0) return v3(0, 0, 0);
  int i = (int)((float)nL * r);
  float lightPdf = 1.0f / (float)nL;
  uint32_t inst = s.n_instances + (uint32_t)i;
  const DModel& m = s.models[s.instances[inst].model];
  if (m.light_count == 0) return v3(0, 0, 0);
  c.S.random();
  float r2 = c.S.random();
  int k = (int)((float)m.light_count * r2);
  const DPrim& lp = s.prims[m.light_begin + k];
  const DLight& light = s.lights[s.materials[lp.material].light];
  return estimateDirect(c, incoming, isect, light, inst) / lightPdf;
}


struct PathParams {
  int bounces;
  int rr;
  int rr_after;
};

// Everything Li keeps across its bounce loop.
struct LiVars {
  V3 L, T;
  Ray incoming, scattered;
  Hit isect;
  int b, passes;
};

// A path deferred at a scattering event in a grid medium, right after the throughput took
// the medium's sampled albedo: the loop state, the sampler position and the index of the
// path's radiance slot. It moves to and from the queues as ten 16-byte words.
struct alignas(16) PathState {
  LiVars v;
  nerng::PathKey key;
  uint32_t dim;
  // 0: resume inside a medium bounce after sampling; 1: at the top of bounce v.b; 3 / 4: at the
  // top of bounce v.b with v.isect already the closest hit of v.incoming (3) or no hit (4)
  uint32_t mode;
  unsigned long long idx;
};
static_assert(sizeof(PathState) == 160, "PathState is ten 16-byte words");
// The words k_trace reads (the ray and the mode) and writes (the hit and the mode).
static_assert(offsetof(PathState, v) == 0 && offsetof(LiVars, incoming) == 24 && offsetof(LiVars, isect) == 72 &&
                  sizeof(Hit) == 40 && offsetof(PathState, mode) == 144,
              "PathState word layout");
constexpr uint32_t kModeTop = 1, kModeHit = 3, kModeMiss = 4;
// 5: at the top of bounce v.b, v.isect its hit, stopped at the light sample's visibility test
// from v.isect.hitPoint to v.scattered.o; 6 / 7: the same with the test's result (visible /
// blocked) known
constexpr uint32_t kModeShadow = 5, kModeVisible = 6, kModeBlocked = 7;


// Deferred paths of one pass. With count_hi set, paths deferred right after a free-flight
// sample are binned by the light their next draw will pick (uniformSampleOneLight's first draw,
// peeked, not consumed): class 0 in entries [0, cap), class 1 in [cap, cap + cap_hi), so that
// the warps of the next pass mostly run one light's sampling code. Every other deferral is
// class 0. Without count_hi: one class. Storage is structure-of-arrays: word k (of ten 16-byte
// words) of entry i at items[k * (cap + cap_hi) + i], so that a warp's lanes, which take
// consecutive entries, move each word as one contiguous 512-byte access.
struct DeferQueue {
  PathState* items;              // (cap + cap_hi) x 160 bytes
  uint32_t* count;
  uint32_t cap;                  // class 0 entries
  uint32_t* count_hi = nullptr;  // class 1 count (null: one class)
  uint32_t cap_hi = 0;           // class 1 entries
};
NE_D void storeState(const DeferQueue& q, size_t i, const PathState& src) {
  const uint4* s = reinterpret_cast<const uint4*>(&src);
  uint4* d = reinterpret_cast<uint4*>(q.items) + i;
  const size_t plane = (size_t)q.cap + q.cap_hi;
#pragma unroll
  for (int k = 0; k < 10; k++) d[k * plane] = s[k];
}
NE_D PathState loadState(const DeferQueue& q, size_t i) {
  PathState r;
  const uint4* s = reinterpret_cast<const uint4*>(q.items) + i;
  uint4* d = reinterpret_cast<uint4*>(&r);
  const size_t plane = (size_t)q.cap + q.cap_hi;
#pragma unroll
  for (int k = 0; k < 10; k++) d[k] = s[k * plane];
  return r;
}

// integrators/VolumetricPathIntegrator.cpp:176-301 Li, plus the optional Russian
// roulette of resources/shaders/MS_monteCarlo.frag:539-544, written as a loop over `v` that
// can start at the scattering point where a K_SPLIT path was deferred (`resume`) and can
// stop at the first deferral point at or after c.deferAt to be deferred again. Deferral
// points: the scattering event of bounce b (position b, or 2b with half-bounce deferral) and
// the end of bounce b (surfaces at position b; every bounce at 2b + 1 with half-bounce
// deferral). Every operation and every random draw happens in the same order either way.
template <uint32_t K>
NE_D V3 liLoop(Ctx<K>& c, const PathParams& P, LiVars& v, bool resume, int pretraced = 0) {
  const DScene& s = c.s;
  const float inf = __int_as_float(0x7f800000);
  // K_CACHE training paths: the vertex the sample is recorded at
  bool recorded = false;
  int recordB = 0;
  V3 vPos = v3(0, 0, 0), vDir = v3(0, 0, 0), vL = v3(0, 0, 0), vT = v3(0, 0, 0);
  for (; v.b < P.bounces; v.b++) {
    const int b = v.b;
    // the bounce's starting radiance and sampler position, for a stop at its shadow ray
    const V3 L0 = v.L;
    const uint32_t dim0 = c.S.dim;
    bool did = true;
    const DMaterial* mat;
    bool medium;
    if ((K & K_SPLIT) && resume) {
      resume = false;
      mat = matOf(s, v.isect.prim);
      medium = true;
    } else {
      // pretraced: k_trace already intersected this bounce's ray (1: hit, 2: no hit)
      if (pretraced) {
        did = pretraced == 1;
        pretraced = 0;
      } else {
        did = intersectScene(c, v.incoming, v.isect, kEps12F, inf);
      }
      if (isBlack(v.T)) break;
      mat = did ? matOf(s, v.isect.prim) : nullptr;
      medium = (K & FT_VOLBSDF) && did && mat && mat->bsdf == NE_BSDF_VOLUME;
      if (medium) {
        v.incoming.o = v.incoming.at(v.isect.tNear);
        v.isect.tFar = v.isect.tFar - v.isect.tNear;
        v.isect.tNear = 0;
        v.scattered = Ray{v3(0, 0, 0), v3(0, 0, 0)};
        V3 sampledT = mediumSample(c, mat->medium, v.incoming, v.scattered, v.isect);
        if (areAllOne(sampledT)) {
          v.incoming.o = v.incoming.at(v.isect.tFar + 0.01f);
          if (++v.passes >= kMaxPassThrough) break;
          v.b--;
          continue;
        }
        v.T = v.T * sampledT;
        if ((K & K_SPLIT) && c.deferAt >= 0 && (b << c.deferHalf) >= c.deferAt && !recorded) {
          const DeferQueue& q = *c.dq;
          uint32_t cls = 0;
          if (q.count_hi && s.n_light_instances > 1)
            cls = (uint32_t)(int)((float)s.n_light_instances * c.S.peek()) & 1u;
          uint32_t slot = cls ? appendSlot(q.count_hi) : appendSlot(q.count);
          if (slot < (cls ? q.cap_hi : q.cap)) {
            PathState ps;
            ps.v = v;
            ps.key = c.S.key;
            ps.dim = c.S.dim;
            ps.mode = 0;
            ps.idx = c.idx;
            storeState(q, (cls ? (size_t)q.cap : 0) + slot, ps);
            c.deferred = true;
            return v.L;
          }
        }
      }
    }
    if ((K & K_CACHE) && medium && b >= c.cio->bounce && !recorded) {
      V3 xo = mul4(s.instances[v.isect.inst].ocs, v.scattered.o, 1.0f);
      if (!c.train) {
        const CacheIO& io = *c.cio;
        uint32_t q = appendSlot(io.q_count);
        if (q < io.q_cap) {
          io.q_pos[3 * q] = xo.x; io.q_pos[3 * q + 1] = xo.y; io.q_pos[3 * q + 2] = xo.z;
          io.q_dir[3 * q] = v.incoming.d.x; io.q_dir[3 * q + 1] = v.incoming.d.y;
          io.q_dir[3 * q + 2] = v.incoming.d.z;
          io.q_thr[3 * q] = v.T.x; io.q_thr[3 * q + 1] = v.T.y; io.q_thr[3 * q + 2] = v.T.z;
          io.q_idx[q] = c.pidx;
        }
        return v.L;
      }
      recorded = true;
      recordB = b;
      vPos = xo;
      vDir = v.incoming.d;
      vL = v.L;
      vT = v.T;
    } else if ((K & K_CACHE) && medium && recorded && c.cio->train_suffix > 0 && b >= recordB + c.cio->train_suffix) {
      // a training path ends in the cache as well: the image gets throughput x cache(vertex),
      // the training sample the radiance gathered so far plus (throughput ratio) x cache(vertex)
      const CacheIO& io = *c.cio;
      V3 xo = mul4(s.instances[v.isect.inst].ocs, v.scattered.o, 1.0f);
      uint32_t q = appendSlot(io.q_count);
      if (q < io.q_cap) {
        io.q_pos[3 * q] = xo.x; io.q_pos[3 * q + 1] = xo.y; io.q_pos[3 * q + 2] = xo.z;
        io.q_dir[3 * q] = v.incoming.d.x; io.q_dir[3 * q + 1] = v.incoming.d.y;
        io.q_dir[3 * q + 2] = v.incoming.d.z;
        io.q_thr[3 * q] = v.T.x; io.q_thr[3 * q + 1] = v.T.y; io.q_thr[3 * q + 2] = v.T.z;
        io.q_idx[q] = c.pidx;
      }
      uint32_t ts = appendSlot(io.t_count);
      if (ts < io.t_cap) {
        V3 d = v.L - vL;
        io.t_pos[3 * ts] = vPos.x; io.t_pos[3 * ts + 1] = vPos.y; io.t_pos[3 * ts + 2] = vPos.z;
        io.t_dir[3 * ts] = vDir.x; io.t_dir[3 * ts + 1] = vDir.y; io.t_dir[3 * ts + 2] = vDir.z;
        io.t_val[3 * ts] = vT.x > 0 ? d.x / vT.x : 0.0f;
        io.t_val[3 * ts + 1] = vT.y > 0 ? d.y / vT.y : 0.0f;
        io.t_val[3 * ts + 2] = vT.z > 0 ? d.z / vT.z : 0.0f;
        uint32_t tq = appendSlot(io.tq_count);  // at most one per training sample: tq < t_cap
        io.tq_pos[3 * tq] = xo.x; io.tq_pos[3 * tq + 1] = xo.y; io.tq_pos[3 * tq + 2] = xo.z;
        io.tq_dir[3 * tq] = v.incoming.d.x; io.tq_dir[3 * tq + 1] = v.incoming.d.y;
        io.tq_dir[3 * tq + 2] = v.incoming.d.z;
        io.tq_thr[3 * tq] = vT.x > 0 ? v.T.x / vT.x : 0.0f;
        io.tq_thr[3 * tq + 1] = vT.y > 0 ? v.T.y / vT.y : 0.0f;
        io.tq_thr[3 * tq + 2] = vT.z > 0 ? v.T.z / vT.z : 0.0f;
        io.tq_idx[tq] = ts;
      }
      return v.L;
    }
    if (medium) {
      // VolumeBSDF: eval is (p, p, p) and pdf is p for the same phase value p (BSDF.h:117-142),
      // so one evaluation gives both
      V3 phaseFr = bsdfEval<K>(s, *mat, v.incoming, v.scattered.d, v.isect);
      float phasePdf = phaseFr.x;
      if (isBlack(phaseFr) || phasePdf == 0.f) break;
      V3 lightSample = uniformSampleOneLight(c, v.scattered, v.isect);
      v.T = v.T * (phaseFr / phasePdf);
      v.L = v.L + v.T * lightSample;
      v.incoming = v.scattered;
    } else {
      if (b == 0) {
        if (did && mat && mat->light >= 0) {
          v.L = v.L + v.T * lightLi(s.lights[mat->light]);
        } else {
          for (uint32_t li = 0; li < s.n_light_instances; li++) {
            const DInstance& inst = s.instances[s.n_instances + li];
            const DModel& lm = s.models[inst.model];
            for (uint32_t k = 0; k < lm.mat_count; k++) {
              const DMaterial& mm = s.materials[s.model_materials[lm.mat_begin + k]];
              v.L = v.L + v.T * lightLe<K>(s.lights[mm.light], inst.ocs, v.incoming.d);
            }
          }
        }
      }
      if (!did || !mat || mat->bsdf == NE_BSDF_NONE) break;
      {
        const V3 lightSample = uniformSampleOneLight(c, v.incoming, v.isect);
        if (shadowQueue<K>() && c.shadowSlot >= 0) {
          // stopped at the light sample's visibility test: queue the path as it was at the top
          // of this bounce (L and the sampler before the bounce), the hit known, with the
          // segment's end on the light (in scattered.o, unused at the top of a surface bounce);
          // the next pass runs the bounce again with the test's result
          PathState ps;
          ps.v = v;
          ps.v.L = L0;
          ps.v.scattered.o = c.shadowPoint;
          ps.key = c.S.key;
          ps.dim = dim0;
          ps.mode = kModeShadow;
          ps.idx = c.idx;
          storeState(*c.dq, (size_t)c.shadowSlot, ps);
          c.shadowSlot = -1;
          c.deferred = true;
          return v.L;
        }
        v.L = v.L + v.T * lightSample;
      }
      Ray scattered;
      scattered.o = v.isect.hitPoint;
      scattered.d = bsdfSample<K>(*mat, v.incoming.d, v.isect.normal, c.S);
      float pdf = bsdfPdf<K>(*mat, v.incoming.d, scattered.d, v.isect.normal);
      V3 fr = bsdfEval<K>(s, *mat, v.incoming, scattered.d, v.isect);
      if (isBlack(fr) || pdf == 0.f) break;
      v.T = v.T * ((fr * absDot(v.incoming.d, v.isect.normal)) / pdf);
      v.incoming = scattered;
    }
    if (P.rr && b > P.rr_after) {
      float mx = maxc(v.T);
      if (mx < 0.01f) {
        float q = gmax(0.05f, 1.0f - mx);
        if (c.S.random() < q) break;
        v.T = v.T / (1.0f - q);
      }
    }
    if ((K & K_SPLIT) && c.deferAt >= 0 && (c.deferHalf || !medium) && (b << c.deferHalf) + c.deferHalf >= c.deferAt &&
        b + 1 < P.bounces && !recorded) {
      // a bounce done (a surface bounce, or any bounce with half-bounce deferral): defer the
      // path to the top of the next bounce
      const DeferQueue& q = *c.dq;
      uint32_t slot = appendSlot(q.count);
      if (slot < q.cap) {
        PathState ps;
        ps.v = v;
        ps.v.b = b + 1;
        ps.key = c.S.key;
        ps.dim = c.S.dim;
        ps.mode = 1;
        ps.idx = c.idx;
        storeState(q, slot, ps);
        c.deferred = true;
        return v.L;
      }
    }
  }
  if ((K & K_CACHE) && recorded) {
    const CacheIO& io = *c.cio;
    uint32_t q = appendSlot(io.t_count);
    if (q < io.t_cap) {
      V3 d = v.L - vL;
      io.t_pos[3 * q] = vPos.x; io.t_pos[3 * q + 1] = vPos.y; io.t_pos[3 * q + 2] = vPos.z;
      io.t_dir[3 * q] = vDir.x; io.t_dir[3 * q + 1] = vDir.y; io.t_dir[3 * q + 2] = vDir.z;
      io.t_val[3 * q] = vT.x > 0 ? d.x / vT.x : 0.0f;
      io.t_val[3 * q + 1] = vT.y > 0 ? d.y / vT.y : 0.0f;
      io.t_val[3 * q + 2] = vT.z > 0 ? d.z / vT.z : 0.0f;
    }
  }
  return v.L;
}

template <uint32_t K>
NE_D V3 Li(Ctx<K>& c, const PathParams& P, Ray incoming) {
  LiVars v;
  v.L = v3(0, 0, 0);
  v.T = v3(1, 1, 1);
  v.incoming = incoming;
  v.scattered = Ray{v3(0, 0, 0), v3(0, 0, 0)};
  v.isect = emptyHit();
  v.b = 0;
  v.passes = 0;
  if ((K & K_SPLIT) && c.deferTop) {
    // the camera ray goes to k_trace with the bounce rays: the path stops at the top of bounce 0
    const DeferQueue& q = *c.dq;
    const uint32_t slot = appendSlot(q.count);
    if (slot < q.cap) {
      PathState ps;
      ps.v = v;
      ps.key = c.S.key;
      ps.dim = c.S.dim;
      ps.mode = kModeTop;
      ps.idx = c.idx;
      storeState(q, slot, ps);
      c.deferred = true;
      return v.L;
    }
  }
  return liLoop(c, P, v, false);
}

// core/Camera.cpp:140-144 with utils/Math.h:502-507.
NE_D Ray cameraRay(const DCamera& cam, float u, float v, Sampler& S) {
  float theta = __double2float_rn((2 * kPiD) * (double)S.random());
  float r = nefm::fsqrt(S.random());
  V3 disk = r * v3(nefm::cos(theta), nefm::sin(theta), 0);
  V3 rd = cam.lens_radius * disk;
  V3 offset = ld3(cam.side) * rd.x + ld3(cam.up) * rd.y;
  V3 pos = ld3(cam.position);
  V3 dir = ((((ld3(cam.lower_left) + u * ld3(cam.horizontal)) + v * ld3(cam.vertical)) - pos) - offset);
  return Ray{pos + offset, -normalize(dir)};
}

// core/OfflineEngine.cpp:61-68 for a given camera and image size; `stream` selects an
// independent random stream (views of a batch use their own).
template <uint32_t K>
NE_D V3 cameraPathCam(Ctx<K>& c, const PathParams& P, const nerng::PathKey& base, const DCamera& cam, int W, int H,
                      uint32_t pixel, uint32_t sample, uint32_t stream) {
  uint32_t x = pixel % (uint32_t)W, y = pixel / (uint32_t)W;
  nerng::PathKey k = base;
  k.pixel = pixel;
  k.sample = sample;
  k.stream = stream;
  c.S.reset(k, 0);
  float u = (float)((float)(int)x + c.S.random()) / (float)W;
  float v = (float)((float)(int)y + c.S.random()) / (float)H;
  Ray r = cameraRay(cam, u, v, c.S);
  return Li(c, P, r);
}

template <uint32_t K>
NE_D V3 cameraPath(Ctx<K>& c, const PathParams& P, const nerng::PathKey& base, uint32_t pixel, uint32_t sample) {
  return cameraPathCam(c, P, base, c.s.camera, c.s.width, c.s.height, pixel, sample, base.stream);
}

}  // namespace nedev
