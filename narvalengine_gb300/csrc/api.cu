// C ABI of the GB300 path integrator: contexts, scene upload and the path kernels.
//
// Kernels (all sm_103a, one CUDA stream per context):
//  k_paths      persistent camera-path kernel: warps take 32 consecutive (pixel, sample)
//               work items at a time from a global counter, trace camera ray + Li
//               (core/OfflineEngine.cpp:61-68) and store each path's radiance.
//  k_reduce     per-pixel mean over its samples in sample order (OfflineEngine.cpp:63-70),
//               so the image is the same sum the reference forms.
//  k_li         Integrator::Li for caller rays (integrators/Integrator.h:13-25).
//  k_closest    Scene::intersectScene (core/Scene.cpp:30-56).
//  k_cells      builds the 8-corner cell layout of a density grid at upload.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <deque>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "narval_gb300.h"
#include "bvh_build.h"
#include "host_parallel.h"
#include "kernels.cuh"
#include "mlp.h"
#include "views.cuh"

using namespace nedev;

// Device buffers a context keeps for reuse. cudaFree synchronises the whole device and
// cudaMalloc of gigabytes costs milliseconds; a caller that uploads, renders and destroys
// scenes frame after frame (or renders into host memory) would pay both every time. Buffers
// released by a scene or a render stay here, idle, and the next request of a similar size
// (the smallest cached buffer of at least the requested size and at most twice it) takes one.
// All users enqueue on the context's one stream, so a reused buffer is never still in use by
// earlier work. At most `limit` bytes stay cached (the rest is freed, largest first): a
// quarter of the device's memory, at least 16 GiB, unless ne_context_set_cache_limit says
// otherwise. A frame with camera rays traced ahead on a 1024^2 x 32 spp image holds two 8 GB
// deferred-path buffers, so a smaller limit would free and reallocate one of them every
// frame. A failed cudaMalloc frees the cache and retries.
constexpr size_t kPoolMinLimit = size_t(16) << 30;
struct DevicePool {
  std::multimap<size_t, void*> idle;          // size -> buffer
  std::unordered_map<void*, size_t> size_of;  // every buffer handed out or idle
  size_t idle_bytes = 0;
  size_t limit = kPoolMinLimit;
  cudaError_t get(size_t bytes, void** out) {
    *out = nullptr;
    bytes = std::max<size_t>(bytes, 256);
    auto it = idle.lower_bound(bytes);
    if (it != idle.end() && it->first <= 2 * bytes) {
      *out = it->second;
      idle_bytes -= it->first;
      idle.erase(it);
      return cudaSuccess;
    }
    cudaError_t e = cudaMalloc(out, bytes);
    if (e == cudaErrorMemoryAllocation && !idle.empty()) {
      cudaGetLastError();
      trim(0);
      e = cudaMalloc(out, bytes);
    }
    if (e != cudaSuccess) {
      *out = nullptr;
      return e;
    }
    size_of[*out] = bytes;
    return cudaSuccess;
  }
  void put(void* p) {
    if (!p) return;
    auto it = size_of.find(p);
    if (it == size_of.end()) return;
    idle.emplace(it->second, p);
    idle_bytes += it->second;
    trim(limit);
  }
  // Frees idle buffers, largest first, until at most `keep` bytes stay cached.
  void trim(size_t keep) {
    while (idle_bytes > keep && !idle.empty()) {
      auto it = std::prev(idle.end());
      cudaFree(it->second);
      size_of.erase(it->second);
      idle_bytes -= it->first;
      idle.erase(it);
    }
  }
};

constexpr int kGridSlabs = 8;
struct ne_context {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t user_ev[8] = {};
  void* flush_buf = nullptr;
  size_t flush_bytes = 0;
  std::string err;
  unsigned long long* d_counter = nullptr;  // [0] work counter, [1..4] work counters
  uint32_t* d_err = nullptr;
  std::vector<ne_scene*> scenes;            // live scenes, destroyed with the context
  std::vector<ne_cache*> caches;            // live radiance caches, destroyed with the context
  DevicePool pool;                          // scene and render buffers, reused
  // grid uploads: slabs copied on copy_stream while the main stream builds the cells of the
  // slabs already there (created at the first grid upload)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t slab_ev[kGridSlabs + 1] = {};
};

struct ne_cache {
  ne_context* ctx = nullptr;
  float* P = nullptr;        // FP32 master parameters
  float* m = nullptr;        // Adam moments
  float* v = nullptr;
  uint8_t* wfwd = nullptr;   // packed BF16 tiles
  uint8_t* wbwd = nullptr;
  float* bias = nullptr;
  float* part = nullptr;     // per-block partial gradients
  int part_blocks = 0;
  float* loss_part = nullptr;
  float* d_loss = nullptr;
  float* grad = nullptr;
  uint8_t* acts = nullptr;  // training activations
  float* out = nullptr;      // training outputs
  size_t cap = 0;
  int step = 0;
  // ne_render_cached: query and training-sample buffers, counters, device copy of CacheIO
  float* q = nullptr;        // q_cap x (pos 3, dir 3, thr 3)
  uint32_t* q_idx = nullptr;
  size_t q_cap = 0;
  float* tr = nullptr;       // t_cap x (pos 3, dir 3, value 3)
  float* tq = nullptr;       // t_cap x (pos 3, dir 3, throughput ratio 3): training paths' end queries
  uint32_t* tq_idx = nullptr;
  size_t t_cap = 0;
  uint32_t* counts = nullptr;  // [0] queries, [1] training samples, [2] training end queries
  CacheIO* d_io = nullptr;
  CacheIO io;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

struct ne_scene {
  ne_context* ctx = nullptr;
  DScene d;
  ne_settings settings;
  std::vector<void*> allocs;
  float* d_paths = nullptr;  // per-path radiance scratch of ne_render
  size_t paths_cap = 0;
  int blocks_per_sm = 1;
  int variant = 0;           // path kernel: 0 straight, 1 regrouped, 2 lane refill, 3 split
  int split_passes = 16;      // kernel 3: passes (the last runs deferred paths to the end)
  int split_half = 1;         // kernel 3: deferral points every half bounce
  int queue_quarters = 3;     // kernel 3: deferred-path capacity, quarters of the render's paths
  int pretrace = 0;           // kernel 3 by bounce, surface sets: bounce rays traced by k_trace
  size_t dq_cap_uploaded = 0; // capacity the uploaded queue descriptors give
  PathState* d_defer[2] = {nullptr, nullptr};  // split renders: two queues of deferred paths
  size_t defer_cap = 0;
  // split renders: queue descriptor p (device) is what pass p appends to, over buffer p & 1;
  // d_pass holds the passes' queue counts (kMaxSplitPasses x u32) and then their work
  // counters (kMaxSplitPasses x u64), all cleared by one memset per render
  DeferQueue* d_dq = nullptr;
  unsigned char* d_pass = nullptr;
  std::vector<uint32_t> bvh_nodes_of;  // BVH node count per model (0: none), for ne_scene_bvh
  std::vector<DModel> bvh_models;      // host copy of the device models (their BVH offsets)
  bool dq_uploaded = false;
  int track_share = 16;      // k_sched tracking-phase threshold (32nds of live lanes)
  uint32_t features = 0;     // FT_* bits of the scene
  uint32_t feature_set = 0;  // compiled kernel specialisation covering them
  std::vector<ne_views*> view_batches;  // destroyed with the scene
};

struct ne_views {
  ne_scene* sc = nullptr;
  std::vector<ne_view> views;      // caller order
  std::vector<uint32_t> order;     // processing slot -> caller index
  std::vector<uint32_t> slot_of;   // caller index -> processing slot
  std::vector<DView> dv;           // processing order
  DView* d_views = nullptr;
  float* d_paths = nullptr;
  float* d_img = nullptr;
  unsigned long long* d_done = nullptr;   // n finished counts, n completion times, start time, work counter
  uint64_t total = 0;
  uint32_t total_pixels = 0;
  PathParams P;
  nerng::PathKey base;
  ne_views_tuning tune = {32, 0, 0, 1, 0, 0, 1};
  std::vector<uint64_t> group_first;  // first path of each group (processing order), then total
  int blocks = 1;
  // split batches: two queues of deferred paths, the views' path spans, completion hook
  PathState* d_defer[2] = {nullptr, nullptr};
  size_t defer_cap = 0;
  DeferQueue* d_dq = nullptr;
  uint32_t* d_dcount = nullptr;
  ViewSpan* d_spans = nullptr;
  ViewDone* d_vd = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::vector<float> latency;      // caller order, last batch
};

namespace {

ne_status fail(ne_context* c, ne_status code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}
ne_status cudaFail(ne_context* c, cudaError_t e, const char* where) {
  return fail(c, e == cudaErrorMemoryAllocation ? NE_ERR_OUT_OF_MEMORY : NE_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}
#define NE_CUDA(call, where)                          \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cudaFail(ctx, e_, where); \
  } while (0)

template <class T>
ne_status upload(ne_scene* sc, const T* host, size_t n, const T** out) {
  ne_context* ctx = sc->ctx;
  *out = nullptr;
  if (n == 0) return NE_OK;
  void* p = nullptr;
  NE_CUDA(ctx->pool.get(n * sizeof(T), &p), "cudaMalloc");
  sc->allocs.push_back(p);
  NE_CUDA(cudaMemcpyAsync(p, host, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  *out = (const T*)p;
  return NE_OK;
}

// A buffer from the context's pool for the duration of one call (given back on return).
struct PoolBuf {
  DevicePool* pool = nullptr;
  void* p = nullptr;
  ~PoolBuf() {
    if (pool) pool->put(p);
  }
  cudaError_t get(DevicePool& pl, size_t bytes) {
    pool = &pl;
    return pl.get(bytes, &p);
  }
};

// ---- InfiniteAreaLight's importance-sampling tables (built at upload, read by envSample)
// Distribution1D's constructor (utils/Sampling.h:12-28): func, CDF of func / n normalised by
// its integral (a uniform CDF if the integral is 0).
void dist1D(const float* f, int n, float* func, float* cdf, float* funcInt) {
  for (int i = 0; i < n; i++) func[i] = f[i];
  cdf[0] = 0;
  for (int i = 1; i < n + 1; i++) cdf[i] = cdf[i - 1] + func[i - 1] / (float)n;
  *funcInt = cdf[n];
  if (*funcInt == 0)
    for (int i = 1; i < n + 1; i++) cdf[i] = (float)i / (float)n;
  else
    for (int i = 1; i < n + 1; i++) cdf[i] /= *funcInt;
}
// Texture::sample's mirror-wrapped nearest texel coordinate (materials/Texture.cpp:88-129).
int hostTexCoord(float u, int n) {
  if (!(u >= -2147483520.0f && u <= 2147483520.0f)) return 0;
  float a = u - (float)(int)u;
  a = a < 0 ? -a : a;
  a = (a < 0.0f) ? 0.0f : a;
  a = (1.0f < a) ? 1.0f : a;
  int x = (int)(a * (float)n);
  if (x > 0 && x == n) x--;
  return x;
}
struct EnvTables {
  std::vector<float> condFunc, condCdf, condInt, margFunc, margCdf;
  float margInt = 0;
};
// InfiniteAreaLight's constructor (lights/InfiniteAreaLight.h:20-40): the green channel of the
// texel at (u/W, v/H) times sin(pi (v + 0.5) / H), then Distribution2D (utils/Sampling.h:82-96)
// whose conditional rows take H values from the start of each image row (Sampling.h:87).
EnvTables buildEnvTables(const ne_light& L) {
  const int W = L.env_width, H = L.env_height;
  std::vector<float> img((size_t)W * H);
  for (int v = 0; v < H; v++) {
    float vp = (float)v / (float)H;
    // glm::sin(PI * float(v + 0.5f) / float(height)): the double literal PI promotes the product
    float sinTheta = (float)std::sin(3.14159265358979323846264338327950288 * (double)((float)v + 0.5f) /
                                     (double)(float)H);
    for (int u = 0; u < W; u++) {
      float up = (float)u / (float)W;
      const uint8_t* t = L.env_texels + 4 * ((size_t)hostTexCoord(vp, H) * W + hostTexCoord(up, W));
      img[u + (size_t)v * W] = (float)t[1] / 255.0f;
      img[u + (size_t)v * W] *= sinTheta;
    }
  }
  EnvTables e;
  e.condFunc.resize((size_t)H * H);
  e.condCdf.resize((size_t)H * (H + 1));
  e.condInt.resize(H);
  for (int v = 0; v < H; v++)
    dist1D(&img[(size_t)v * W], H, &e.condFunc[(size_t)v * H], &e.condCdf[(size_t)v * (H + 1)], &e.condInt[v]);
  e.margFunc.resize(H);
  e.margCdf.resize(H + 1);
  dist1D(e.condInt.data(), H, e.margFunc.data(), e.margCdf.data(), &e.margInt);
  return e;
}

// ---- host helpers shared by the upload (same arithmetic as the integrator's host side)
struct H3 {
  float x, y, z;
};
inline H3 h3(float x, float y, float z) { return H3{x, y, z}; }
inline H3 hsub(H3 a, H3 b) { return h3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline H3 hmul(H3 a, float s) { return h3(a.x * s, a.y * s, a.z * s); }
inline H3 hdiv(H3 a, float s) { return h3(a.x / s, a.y / s, a.z / s); }
inline H3 hadd(H3 a, H3 b) { return h3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float hdot(H3 a, H3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float hlen(H3 a) { return nefm::fsqrt(hdot(a, a)); }
inline float hmin(float a, float b) { return (b < a) ? b : a; }
inline float hmax(float a, float b) { return (a < b) ? b : a; }
inline H3 hvmin(H3 a, H3 b) { return h3(hmin(a.x, b.x), hmin(a.y, b.y), hmin(a.z, b.z)); }
inline H3 hvmax(H3 a, H3 b) { return h3(hmax(a.x, b.x), hmax(a.y, b.y), hmax(a.z, b.z)); }
inline float hcomp(H3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

// utils/Math.h:874-912 getScale: scale part of glm's decomposition.
H3 getScale(const float* t) {
  float w = t[15];
  H3 r0 = h3(t[0] / w, t[1] / w, t[2] / w);
  H3 r1 = h3(t[4] / w, t[5] / w, t[6] / w);
  H3 r2 = h3(t[8] / w, t[9] / w, t[10] / w);
  H3 s;
  s.x = hlen(r0);
  r0 = hdiv(hmul(r0, 1.0f), hlen(r0));
  float skz = hdot(r0, r1);
  r1 = hadd(hmul(r1, 1.0f), hmul(r0, -skz));
  s.y = hlen(r1);
  r1 = hdiv(hmul(r1, 1.0f), hlen(r1));
  float sky = hdot(r0, r2);
  r2 = hadd(hmul(r2, 1.0f), hmul(r0, -sky));
  float skx = hdot(r1, r2);
  r2 = hadd(hmul(r2, 1.0f), hmul(r1, -skx));
  s.z = hlen(r2);
  return s;
}

struct HNode {
  H3 mn, mx;
  uint32_t start, count, rightOffset;
};

void triBounds(const ne_primitive& p, H3& mn, H3& mx) {
  H3 a = h3(p.p0[0], p.p0[1], p.p0[2]), b = h3(p.p1[0], p.p1[1], p.p1[2]), c = h3(p.p2[0], p.p2[1], p.p2[2]);
  mn = hvmin(a, hvmin(b, c));
  mx = hvmax(a, hvmax(b, c));
}
inline H3 boxCenter(H3 mn, H3 mx) { return hsub(mx, hdiv(hsub(mx, mn), 2.0f)); }

// primitives/BVH.cpp:6-106 BVH::init, one node: bounds of order[start, end), the leaf
// decision (<= 4 triangles) and, for an interior node, the midpoint split on the longest axis
// of the centroid bounds with a median fallback, partitioning `order` in place. Returns the
// node (rightOffset 0 for a leaf) and the split position in `mid`.
HNode bvhNode(const ne_primitive* prims, uint32_t* order, uint32_t start, uint32_t end, uint32_t& mid) {
  const uint32_t perLeaf = 4;
  const float inf = INFINITY;
  HNode node;
  node.start = start;
  node.count = end - start;
  node.rightOffset = 1;
  H3 bbMin = h3(inf, inf, inf), bbMax = h3(-inf, -inf, -inf), pmn, pmx;
  triBounds(prims[order[start]], pmn, pmx);
  bbMin = hvmin(bbMin, pmn);
  bbMax = hvmax(bbMax, pmx);
  H3 bcMin = boxCenter(bbMin, bbMax), bcMax = bcMin;
  for (uint32_t i = start + 1; i < end; i++) {
    triBounds(prims[order[i]], pmn, pmx);
    bbMin = hvmin(bbMin, pmn);
    bbMax = hvmax(bbMax, pmx);
    H3 c = boxCenter(pmn, pmx);
    bcMin = hvmin(bcMin, c);
    bcMax = hvmax(bcMax, c);
  }
  node.mn = bbMin;
  node.mx = bbMax;
  mid = 0;
  if (node.count <= perLeaf) {
    node.rightOffset = 0;
    return node;
  }
  H3 ext = hsub(bcMax, bcMin);
  int dim = 0;
  if (hcomp(ext, 1) > hcomp(ext, dim)) dim = 1;
  if (hcomp(ext, 2) > hcomp(ext, dim)) dim = 2;
  float split = 0.5f * (hcomp(bcMin, dim) + hcomp(bcMax, dim));
  mid = start;
  for (uint32_t i = start; i < end; i++) {
    triBounds(prims[order[i]], pmn, pmx);
    if (hcomp(boxCenter(pmn, pmx), dim) < split) {
      std::swap(order[i], order[mid]);
      mid++;
    }
  }
  if (mid == start || mid == end) mid = start + (end - start) / 2;
  return node;
}

// BVH::init of order[start, end) appended to `nodes` in depth-first order (left child = i + 1,
// right child = i + rightOffset), the reference's stack traversal.
void buildRange(const ne_primitive* prims, uint32_t* order, uint32_t start, uint32_t end, std::vector<HNode>& nodes) {
  struct Item { uint32_t parent, start, end; bool right; };
  const uint32_t rootParent = 0xffffffffu;
  const size_t base = nodes.size();
  std::vector<Item> stack;
  stack.push_back(Item{rootParent, start, end, false});
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    uint32_t mid;
    HNode node = bvhNode(prims, order, it.start, it.end, mid);
    uint32_t self = (uint32_t)(nodes.size() - base);
    nodes.push_back(node);
    if (it.right) nodes[base + it.parent].rightOffset = self - it.parent;
    if (node.rightOffset == 0) continue;
    stack.push_back(Item{self, mid, it.end, true});
    stack.push_back(Item{self, it.start, mid, false});
  }
}

// The same tree built with subtrees in parallel: nodes above depth kBvhTaskDepth are split by
// one task while another builds their left child; every node is computed exactly as in the
// sequential build (ranges of `order` are disjoint), and the subtrees are laid out in the
// same depth-first order, so the node array is identical.
struct BvhTop {
  HNode node;
  bool sub = false;
  std::vector<HNode> subtree;
  std::unique_ptr<BvhTop> l, r;
};
constexpr int kBvhTaskDepth = 6;
constexpr uint32_t kBvhTaskMin = 4096;

std::unique_ptr<BvhTop> buildTop(const ne_primitive* prims, uint32_t* order, uint32_t start, uint32_t end, int depth) {
  std::unique_ptr<BvhTop> t(new BvhTop());
  if (depth >= kBvhTaskDepth || end - start < kBvhTaskMin) {
    t->sub = true;
    t->subtree.reserve((size_t)(end - start) / 2 + 8);
    buildRange(prims, order, start, end, t->subtree);
    return t;
  }
  uint32_t mid;
  t->node = bvhNode(prims, order, start, end, mid);
  if (t->node.rightOffset == 0) return t;
  auto left = std::async(std::launch::async, buildTop, prims, order, start, mid, depth + 1);
  t->r = buildTop(prims, order, mid, end, depth + 1);
  t->l = left.get();
  return t;
}

void emitTop(BvhTop* t, std::vector<HNode>& out) {
  if (t->sub) {
    out.insert(out.end(), t->subtree.begin(), t->subtree.end());
    return;
  }
  size_t self = out.size();
  out.push_back(t->node);
  if (t->node.rightOffset == 0) return;
  emitTop(t->l.get(), out);
  out[self].rightOffset = (uint32_t)(out.size() - self);
  emitTop(t->r.get(), out);
}

void buildBvh(const ne_primitive* prims, std::vector<uint32_t>& order, std::vector<HNode>& nodes) {
  nodes.clear();
  if (order.empty()) return;
  std::unique_ptr<BvhTop> top = buildTop(prims, order.data(), 0, (uint32_t)order.size(), 0);
  nodes.reserve(order.size() / 2 + 16);
  emitTop(top.get(), nodes);
}

// ---------------------------------------------------------------- kernels
// The descriptor's primitives in the device layout: Triangle::calculateArea for triangles (the
// float arithmetic of the host helpers, in the same order), the grid-medium flag from the
// primitive's material.
__global__ void k_convert_prims(const ne_primitive* __restrict__ src, uint32_t n, const uint8_t* __restrict__ gridMat,
                                DPrim* __restrict__ dst) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const ne_primitive s = src[i];
    DPrim d;
    d.type = s.type;
    d.material = s.material;
    d.flags = (s.material >= 0 && gridMat[s.material]) ? DPRIM_GRID_MEDIUM : 0;
    d.radius = s.radius;
    for (int k = 0; k < 3; k++) {
      d.p0[k] = s.p0[k];
      d.p1[k] = s.p1[k];
      d.p2[k] = s.p2[k];
    }
    d.area = 0.0f;
    if (s.type == NE_PRIM_TRIANGLE) {
      const float e1x = s.p1[0] - s.p0[0], e1y = s.p1[1] - s.p0[1], e1z = s.p1[2] - s.p0[2];
      const float e2x = s.p2[0] - s.p0[0], e2y = s.p2[1] - s.p0[1], e2z = s.p2[2] - s.p0[2];
      const float nx = e1y * e2z - e2y * e1z, ny = e1z * e2x - e2z * e1x, nz = e1x * e2y - e2x * e1y;
      d.area = nefm::fsqrt((nx * nx + ny * ny) + nz * nz) / 2.0f;
    }
    dst[i] = d;
  }
}

// The cells of cell slabs [z0, z1): a block takes rows (y, z) of W + 1 cells, its threads
// the cells of a row.
__global__ void k_cells(const float* __restrict__ grid, uint32_t W, uint32_t H, uint32_t D, uint32_t z0, uint32_t z1,
                        float4* __restrict__ cells) {
  const uint32_t rows = (z1 - z0) * (H + 1);
  for (uint32_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const uint32_t y = r % (H + 1), z = z0 + r / (H + 1);
    const size_t row = ((size_t)z * (H + 1) + y) * (W + 1);
    auto den = [&](uint32_t a, uint32_t b, uint32_t c) -> float {
      if (a >= W || b >= H || c >= D) return 0.0f;
      return grid[(size_t)H * W * c + (size_t)W * b + a];
    };
    for (uint32_t x = threadIdx.x; x <= W; x += blockDim.x) {
      const size_t i = row + x;
      cells[2 * i] = make_float4(den(x, y, z), den(x + 1, y, z), den(x, y + 1, z), den(x + 1, y + 1, z));
      cells[2 * i + 1] =
          make_float4(den(x, y, z + 1), den(x + 1, y, z + 1), den(x, y + 1, z + 1), den(x + 1, y + 1, z + 1));
    }
  }
}

// GridMedia::calculateMaxDensity (materials/GridMedia.h:16-21): mx = 0; mx = (mx < v) ? v : mx
// over the voxels, i.e. the largest value and 0 (NaN voxels never replace it), as an
// order-preserving unsigned key combined by atomicMax (*key starts at the key of 0).
__device__ __forceinline__ uint32_t maxKey(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__global__ void k_grid_max(const float* __restrict__ grid, size_t n, uint32_t* __restrict__ key) {
  uint32_t best = maxKey(0.0f);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float v = grid[i];
    if (v == v) best = max(best, maxKey(v));
  }
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0) atomicMax(key, best);
}
// invMaxDensity = 1 / max, written into the medium's device record.
__global__ void k_grid_inv_max(const uint32_t* __restrict__ key, DMedium* __restrict__ m) {
  uint32_t k = *key;
  float mx = __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
  m->inv_max_density = 1.0f / mx;
}

// Per-pixel mean in sample order: color += Li for s = 0..spp-1, then color / spp.
__global__ void k_reduce(const float* __restrict__ paths, uint32_t n_pix, uint32_t spp, uint32_t cover_w, int W,
                         float* __restrict__ out) {
  for (uint32_t pi = blockIdx.x * blockDim.x + threadIdx.x; pi < n_pix; pi += gridDim.x * blockDim.x) {
    const float* p = paths + (size_t)pi * spp * 3;
    float r = 0, g = 0, b = 0;
    for (uint32_t k = 0; k < spp; k++) {
      r = r + p[3 * k + 0];
      g = g + p[3 * k + 1];
      b = b + p[3 * k + 2];
    }
    float fs = (float)spp;
    size_t pixel = (size_t)(pi / cover_w) * (size_t)W + (pi % cover_w);
    out[3 * pixel + 0] = r / fs;
    out[3 * pixel + 1] = g / fs;
    out[3 * pixel + 2] = b / fs;
  }
}

// FP64 accumulation of per-path radiance, samples in order. With `drop`, a path whose
// radiance has a non-finite channel is skipped and counted in *dropped.
__global__ void k_accum(const float* __restrict__ paths, uint32_t n_pix, uint32_t spp, uint32_t cover_w, int W,
                        double* __restrict__ acc, int drop, unsigned long long* dropped) {
  for (uint32_t pi = blockIdx.x * blockDim.x + threadIdx.x; pi < n_pix; pi += gridDim.x * blockDim.x) {
    const float* p = paths + (size_t)pi * spp * 3;
    size_t pixel = (size_t)(pi / cover_w) * (size_t)W + (pi % cover_w);
    double r = acc[3 * pixel + 0], g = acc[3 * pixel + 1], b = acc[3 * pixel + 2];
    unsigned long long nd = 0;
    for (uint32_t k = 0; k < spp; k++) {
      float x = p[3 * k + 0], y = p[3 * k + 1], z = p[3 * k + 2];
      if (drop && !(isfinite(x) && isfinite(y) && isfinite(z))) {
        nd++;
        continue;
      }
      r += (double)x;
      g += (double)y;
      b += (double)z;
    }
    if (nd) atomicAdd(dropped, nd);
    acc[3 * pixel + 0] = r;
    acc[3 * pixel + 1] = g;
    acc[3 * pixel + 2] = b;
  }
}

// Read-only bandwidth probe: every thread reads 16-byte words (ld.global.cg: cached in L2,
// not L1; volatile, so repeated passes are not merged) with a grid stride, four in flight,
// over the whole buffer `reps` times, and folds them into one word that is written only if it
// equals a value the data never produces (so the loads are not removed).
__device__ __forceinline__ uint4 ld_cg_v4(const uint4* p) {
  uint4 v;
  asm volatile("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
  return v;
}
__global__ void __launch_bounds__(512) k_read_bw(const uint4* __restrict__ p, size_t n, int reps, uint32_t* sink) {
  uint32_t acc = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; r++) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
      uint4 a = ld_cg_v4(p + i), b = ld_cg_v4(p + i + stride), c = ld_cg_v4(p + i + 2 * stride),
            d = ld_cg_v4(p + i + 3 * stride);
      acc = acc * 31u + ((a.x + a.y + a.z + a.w) ^ (b.x + b.y + b.z + b.w) ^ (c.x + c.y + c.z + c.w) ^
                         (d.x + d.y + d.z + d.w));
    }
    for (; i < n; i += stride) {
      uint4 a = ld_cg_v4(p + i);
      acc = acc * 31u + (a.x + a.y + a.z + a.w);
    }
  }
  if (acc == 0x9e3779b9u) sink[0] = acc;
}

// Random 32-byte reads (two 16-byte loads through the read-only path, as a density-cell
// lookup makes them) at hashed record indices: each thread issues its reads in groups of D
// independent ones, so the rate measured is the memory system's, not one thread's latency.
// Index hash: the "lowbias32" integer mix (Wellons), over a counter per read.
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
template <int D>
__global__ void __launch_bounds__(512) k_random_read(const float4* __restrict__ p, uint32_t nrec, uint32_t reads,
                                                     uint32_t seed, uint32_t* sink) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.0f;
  for (uint32_t r = 0; r < reads; r += D) {
    float4 a[D], b[D];
#pragma unroll
    for (int k = 0; k < D; k++) {
      const uint32_t h = mix32((tid * reads + r + (uint32_t)k) ^ seed);
      const size_t i = (size_t)(((uint64_t)h * nrec) >> 32);
      a[k] = __ldg(p + 2 * i);
      b[k] = __ldg(p + 2 * i + 1);
    }
#pragma unroll
    for (int k = 0; k < D; k++) acc += (a[k].x + a[k].w) * (b[k].y + b[k].z);
  }
  if (acc == 1234.5f) sink[0] = tid;
}

// Reads per second of `iters` launches of k_random_read<D> (one wave of resident blocks).
template <int D>
cudaError_t randomReadRate(ne_context* ctx, const float4* buf, uint32_t nrec, int iters, uint32_t* sink, double* rate) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_random_read<D>, 512, 0);
  if (e != cudaSuccess) return e;
  const int blocks = ctx->sm_count * std::max(1, per_sm);
  const uint32_t reads = 256;  // per thread and launch
  k_random_read<D><<<blocks, 512, 0, ctx->stream>>>(buf, nrec, reads, 0x1234567u, sink);  // warm-up
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(ctx->ev[0], ctx->stream)) != cudaSuccess) return e;
  for (int k = 0; k < iters; k++)
    k_random_read<D><<<blocks, 512, 0, ctx->stream>>>(buf, nrec, reads, 0x9e3779b9u * (uint32_t)(k + 1), sink);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(ctx->ev[1], ctx->stream)) != cudaSuccess) return e;
  if ((e = cudaEventSynchronize(ctx->ev[1])) != cudaSuccess) return e;
  float ms = 0;
  if ((e = cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1])) != cudaSuccess) return e;
  *rate = (double)blocks * 512 * reads * iters / (ms / 1e3);
  return cudaSuccess;
}

__global__ void k_fmath(int fn, const float* __restrict__ x, size_t n, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float v = x[i], r;
    switch (fn) {
      case 0: r = nefm::log(v); break;
      case 1: r = nefm::exp(v); break;
      case 2: r = nefm::sin(v); break;
      case 3: r = nefm::cos(v); break;
      case 4: r = nefm::acos(v); break;
      case 6: r = nefm::atan2(v, (i ^ 1) < n ? x[i ^ 1] : 1.0f); break;
      case 7: r = nefm::log1m_draw(v); break;
      default: r = nefm::pow5(v); break;
    }
    out[i] = r;
  }
}

__global__ void k_rng(nerng::PathKey base, const ne_path_key* __restrict__ keys, const uint32_t* __restrict__ dims,
                      size_t n, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    nerng::PathKey k = base;
    k.pixel = keys[i].pixel;
    k.sample = keys[i].sample;
    out[i] = nerng::u01(k, dims[i]);
  }
}

PathParams pathParams(const ne_scene* sc, const ne_render_params* p) {
  PathParams P;
  P.bounces = (p && p->bounces >= 0) ? p->bounces : sc->settings.bounces;
  int rr = (p && p->rr >= 0) ? p->rr : sc->settings.rr_enabled;
  P.rr = rr;
  P.rr_after = (p && p->rr >= 0) ? p->rr_after : sc->settings.rr_after;
  return P;
}
nerng::PathKey baseKey(const ne_render_params* p) {
  uint64_t seed = p ? p->seed : 0;
  nerng::PathKey k;
  k.seed_lo = (uint32_t)seed;
  k.seed_hi = (uint32_t)(seed >> 32);
  k.pixel = 0;
  k.sample = 0;
  k.stream = 0;
  return k;
}

ne_status checkErr(ne_context* ctx) {
  uint32_t e = 0;
  NE_CUDA(cudaMemcpyAsync(&e, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync(err)");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (e & ERR_BVH_STACK) return fail(ctx, NE_ERR_UNSUPPORTED, "BVH traversal stack exceeded 64 entries");
  return NE_OK;
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

int persistentBlocks(ne_scene* sc) { return sc->ctx->sm_count * sc->blocks_per_sm; }

constexpr int kMaxSplitPasses = 64;

// Path-kernel launches of one launchPaths call.
int pathLaunches(const ne_scene* sc, bool count) {
  if (sc->variant != 3 || count) return 1;
  const bool traces = sc->pretrace && !sc->split_half && (sc->feature_set == K_MESH || sc->feature_set == K_SURFACE);
  const int passes = std::min(kMaxSplitPasses, std::max(2, sc->split_passes) + (traces && sc->pretrace >= 2 ? 1 : 0));
  return passes + (traces ? passes - 1 : 0);  // k_trace before every resume pass
}

// Split render: the first pass finishes every path that ends at its first event and queues
// the others (at their first scattering in a grid medium or after their first surface
// bounce); pass p resumes the queued paths and queues them again one bounce (or half a
// bounce) later, the last pass runs them to the end. Two buffers alternate, each with room for
// three quarters of the render's paths (at most kMaxDeferEntries): half in class 0, a quarter
// in class 1 (see DeferQueue); paths beyond a class's capacity continue in the pass that had
// them. Each pass
// has its own queue count and work counter, so the passes follow one another with no
// launches in between. `launch(pass, blocks, args, counter)` launches one pass (0: first
// pass; pass 0 uses the context's counter, cleared by the caller).
// Entries of each deferred-path buffer at most (2^26 paths, 10 GiB): a render with more
// paths lets the rest continue in the pass that has them.
constexpr size_t kMaxDeferEntries = size_t(1) << 26;

// With `trace` (a launcher of k_trace over a queue) and the scene tuned to pretrace, the
// bounce rays of each queue between passes are intersected by k_trace before the next pass.
struct NoTrace {
  cudaError_t operator()(const DeferQueue*, unsigned long long*) const { return cudaSuccess; }
};
template <class F, class T = NoTrace>
ne_status launchSplit(ne_scene* sc, PathArgs b, int blocks, F launch, T trace = NoTrace(), bool canTrace = false) {
  ne_context* ctx = sc->ctx;
  // queue_quarters / 4 of the paths (default 3: class 0 half the paths, class 1 a quarter)
  const bool traces = canTrace && sc->pretrace && !sc->split_half;
  // pretrace 2: the first pass queues every path before its camera ray (class 0 holds them all);
  // 3: also the shadow rays (every pass then takes each path one traversal further)
  const bool gen = traces && sc->pretrace >= 2;
  const bool shadows = traces && sc->pretrace == 3;
  size_t cap = std::min(kMaxDeferEntries,
                        std::max<size_t>(3072, (size_t)(b.total / 4) * (size_t)sc->queue_quarters));
  if (gen) cap = std::min(kMaxDeferEntries, std::max(cap, (size_t)b.total / 2 * 3 + 3));
  if (sc->defer_cap < cap) {
    for (PathState*& q : sc->d_defer) {
      ctx->pool.put(q);
      q = nullptr;
    }
    sc->defer_cap = 0;
    sc->dq_uploaded = false;
    for (PathState*& q : sc->d_defer) {
      void* qp = nullptr;
      NE_CUDA(ctx->pool.get(cap * sizeof(PathState), &qp), "cudaMalloc(deferred paths)");
      q = (PathState*)qp;
    }
    sc->defer_cap = cap;
  }
  const size_t countBytes = 2 * kMaxSplitPasses * sizeof(uint32_t);  // both classes
  // then the passes' work counters and k_trace's
  const size_t passBytes = countBytes + 2 * kMaxSplitPasses * sizeof(unsigned long long);
  if (!sc->d_dq) {
    void* qp = nullptr;
    NE_CUDA(ctx->pool.get(kMaxSplitPasses * sizeof(DeferQueue), &qp), "cudaMalloc");
    sc->d_dq = (DeferQueue*)qp;
  }
  if (!sc->d_pass) {
    void* pp = nullptr;
    NE_CUDA(ctx->pool.get(passBytes, &pp), "cudaMalloc");
    sc->d_pass = (unsigned char*)pp;
  }
  if (!sc->dq_uploaded || sc->dq_cap_uploaded != cap) {
    // this render's capacity (the buffers may be larger, from an earlier render)
    DeferQueue dq[kMaxSplitPasses];
    for (int p = 0; p < kMaxSplitPasses; p++) {
      dq[p].items = sc->d_defer[p & 1];
      dq[p].count = reinterpret_cast<uint32_t*>(sc->d_pass) + p;
      dq[p].count_hi = reinterpret_cast<uint32_t*>(sc->d_pass) + kMaxSplitPasses + p;
      dq[p].cap = (uint32_t)(cap / 3 * 2);
      dq[p].cap_hi = (uint32_t)(cap - dq[p].cap);
    }
    // from pageable memory: the call returns once `dq` has been staged
    NE_CUDA(cudaMemcpyAsync(sc->d_dq, dq, sizeof(dq), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
    sc->dq_uploaded = true;
    sc->dq_cap_uploaded = cap;
  }
  NE_CUDA(cudaMemsetAsync(sc->d_pass, 0, passBytes, ctx->stream), "cudaMemsetAsync");
  unsigned long long* counters = reinterpret_cast<unsigned long long*>(sc->d_pass + countBytes);
  unsigned long long* traceCounters = counters + kMaxSplitPasses;
  // with `gen` a first pass that only queues the new paths precedes the split passes
  const int passes = std::min(kMaxSplitPasses, std::max(2, sc->split_passes) + (gen ? 1 : 0));
  b.defer_out = sc->d_dq;
  b.defer_at = 0;
  b.defer_half = sc->split_half;
  b.defer_top = gen ? 1 : 0;
  NE_CUDA(launch(0, blocks, b, ctx->d_counter), "path kernel launch");
  b.defer_top = 0;
  for (int pass = 1; pass < passes; pass++) {
    if (traces) NE_CUDA(trace(sc->d_dq + pass - 1, traceCounters + pass), "k_trace launch");
    b.defer_in = sc->d_dq + pass - 1;
    b.defer_out = sc->d_dq + pass;
    b.defer_at = pass == passes - 1 ? -1 : (shadows ? 0 : pass - (gen ? 1 : 0));
    b.defer_shadow = shadows && pass != passes - 1;
    NE_CUDA(launch(pass, persistentBlocks(sc), b, counters + pass), "resume kernel launch");
  }
  return NE_OK;
}

ne_status launchPaths(ne_scene* sc, const PathArgs& a, bool count) {
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaMemsetAsync(ctx->d_counter, 0, 5 * sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
  int blocks = persistentBlocks(sc);
  unsigned long long needed = (a.total + kThreads - 1) / kThreads;
  if ((unsigned long long)blocks > needed) blocks = (int)std::max<unsigned long long>(1, needed);
  PathArgs b = a;
  b.track_share = sc->track_share;
  if (sc->variant == 3 && !count) {
    return launchSplit(
        sc, b, blocks,
        [&](int pass, int nb, const PathArgs& pa, unsigned long long* ctr) {
          return ne_launch_path_split(pass, sc->feature_set, nb, ctx->stream, sc->d, pa, ctr, ctx->d_err);
        },
        [&](const DeferQueue* q, unsigned long long* ctr) {
          return sc->feature_set == K_MESH
                     ? nedev::launchTrace_mesh(ctx->sm_count, ctx->stream, sc->d, q, ctr, ctx->d_err)
                     : nedev::launchTrace_surface(ctx->sm_count, ctx->stream, sc->d, q, ctr, ctx->d_err);
        },
        sc->feature_set == K_MESH || sc->feature_set == K_SURFACE);
  }
  NE_CUDA(ne_launch_path_kernel(sc->variant, sc->feature_set, count, blocks, ctx->stream, sc->d, b, ctx->d_counter,
                                ctx->d_err),
          "path kernel launch");
  return NE_OK;
}

}  // namespace

uint32_t ne_feature_set_for(uint32_t f) {
  const uint32_t sets[3] = {K_VOLUME, K_SURFACE, K_MESH};
  for (uint32_t s : sets)
    if ((f & ~s) == 0) return s;
  return K_GENERAL;
}

template <uint32_t K>
static cudaError_t launchK(int kernel, int blocks, cudaStream_t st, const DScene& s, const PathArgs& a,
                           unsigned long long* counter, uint32_t* err) {
  // kernel 3 (split) runs through launchPaths; callers without its queue use the straight kernel
  if (kernel == 0 || kernel == 3) return launchPathKernel<0, K>(blocks, st, s, a, counter, err);
  if (kernel == 1) return launchPathKernel<1, K>(blocks, st, s, a, counter, err);
  return launchPathKernel<2, K>(blocks, st, s, a, counter, err);
}

template <uint32_t K>
static cudaError_t occupancyK(int kernel, int* bps) {
  if (kernel == 0) return pathKernelOccupancy<0, K>(bps);
  if (kernel == 1) return pathKernelOccupancy<1, K>(bps);
  if (kernel == 3) return ne_path_split_occupancy(K, bps);
  return pathKernelOccupancy<2, K>(bps);
}

cudaError_t ne_launch_path_kernel(int kernel, uint32_t set, bool count, int blocks, cudaStream_t st, const DScene& s,
                                  const PathArgs& a, unsigned long long* counter, uint32_t* err) {
  if (count) return launchK<K_GENERAL | K_COUNT>(kernel, blocks, st, s, a, counter, err);
  switch (set) {
    case K_VOLUME: return launchK<K_VOLUME>(kernel, blocks, st, s, a, counter, err);
    case K_SURFACE: return launchK<K_SURFACE>(kernel, blocks, st, s, a, counter, err);
    case K_MESH: return launchK<K_MESH>(kernel, blocks, st, s, a, counter, err);
    default: return launchK<K_GENERAL>(kernel, blocks, st, s, a, counter, err);
  }
}

namespace nedev {
#define NE_SPLIT_DECL(set)                                                                                \
  cudaError_t launchSplit_##set(int, int, cudaStream_t, const DScene&, const PathArgs&, unsigned long long*, \
                                uint32_t*);                                                             \
  cudaError_t occupancySplit_##set(int*);
NE_SPLIT_DECL(volume)
NE_SPLIT_DECL(surface)
NE_SPLIT_DECL(mesh)
NE_SPLIT_DECL(general)
#undef NE_SPLIT_DECL
}  // namespace nedev

cudaError_t ne_launch_path_split(int pass, uint32_t set, int blocks, cudaStream_t st, const DScene& s,
                                 const PathArgs& a, unsigned long long* counter, uint32_t* err) {
  switch (set) {
    case K_VOLUME: return launchSplit_volume(pass, blocks, st, s, a, counter, err);
    case K_SURFACE: return launchSplit_surface(pass, blocks, st, s, a, counter, err);
    case K_MESH: return launchSplit_mesh(pass, blocks, st, s, a, counter, err);
    default: return launchSplit_general(pass, blocks, st, s, a, counter, err);
  }
}

cudaError_t ne_path_split_occupancy(uint32_t set, int* bps) {
  switch (set) {
    case K_VOLUME: return occupancySplit_volume(bps);
    case K_SURFACE: return occupancySplit_surface(bps);
    case K_MESH: return occupancySplit_mesh(bps);
    default: return occupancySplit_general(bps);
  }
}

cudaError_t ne_path_kernel_occupancy(int kernel, uint32_t set, int* bps) {
  switch (set) {
    case K_VOLUME: return occupancyK<K_VOLUME>(kernel, bps);
    case K_SURFACE: return occupancyK<K_SURFACE>(kernel, bps);
    case K_MESH: return occupancyK<K_MESH>(kernel, bps);
    default: return occupancyK<K_GENERAL>(kernel, bps);
  }
}

// ---------------------------------------------------------------------------------------
// Allocation-free render. Some callers cannot call cudaMalloc at render time: a host
// application that reserves the device's memory up front for its own pool (cudaMalloc then
// fails), and frame loops that must not stall, since cudaFree synchronises the whole device.
// ne_render allocates its per-path radiance buffer lazily and, for a host image, a device
// image; ne_render_noalloc renders into a caller-owned device image and takes its scratch
// (per-path radiance, work counters, error flag) from the fixed array below.
//
// The array is file-scope device memory: every GPU that loads this library holds its
// kNoAllocScratchBytes until the process exits. All calls on a device share it and it keeps
// the last call's contents; the counters and error flag are cleared at the start of each
// call (per-path radiance is written in full before it is read). Calls whose work overlaps
// on the GPU (two contexts on one device, or streams not ordered with one another) race on
// the array and must be serialised by the caller.
// ---------------------------------------------------------------------------------------
namespace {

constexpr uint64_t kNoAllocMaxPaths = NE_NOALLOC_MAX_PATHS;  // e.g. 256 x 256 pixels x 16 samples
constexpr size_t kNoAllocHeaderBytes = 256;        // work counters [0..7], error flag
constexpr size_t kNoAllocScratchBytes = kNoAllocHeaderBytes + kNoAllocMaxPaths * 3 * sizeof(float);
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the array on the current device, looked up once per device by the first
// call after a context is created on that device (ne_context_create forgets the address, so
// a device reset between contexts, which reloads the module, is followed by a fresh lookup).
// In host code g_noalloc_scratch names a host-side stand-in, so the address must come from
// the runtime.
void noallocForget(int device) {
  if (device < 0 || device >= kNoAllocMaxDevices) return;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  g_noalloc_ptr[device] = nullptr;
}

ne_status noallocScratch(ne_context* ctx, unsigned char** out) {
  if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
    return fail(ctx, NE_ERR_UNSUPPORTED, "ne_render_noalloc supports device ordinals below 64");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[ctx->device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(ctx, NE_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_noalloc_ptr[ctx->device] = (unsigned char*)p;
  }
  *out = g_noalloc_ptr[ctx->device];
  return NE_OK;
}

}  // namespace

// ---------------------------------------------------------------- radiance cache
namespace {

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// He-uniform initial weights (bound sqrt(6 / fan_in)), zero biases; the unused output rows
// 3..15 and input columns 88..95 stay zero.
void cacheInitParams(uint64_t seed, std::vector<float>& P) {
  static const int in[5] = {96, 64, 64, 64, 64}, out[5] = {64, 64, 64, 64, 16};
  P.assign(kNeMlpParams, 0.0f);
  uint64_t s = seed;
  size_t off = 0;
  for (int l = 0; l < 5; l++) {
    float bound = (float)sqrt(6.0 / in[l]);
    for (int o = 0; o < out[l]; o++)
      for (int k = 0; k < in[l]; k++) {
        float u = (float)((splitmix64(s) >> 40) * (1.0 / 16777216.0));
        bool used = !(l == 4 && o >= 3) && !(l == 0 && k >= 88);
        P[off + (size_t)o * in[l] + k] = used ? (2.0f * u - 1.0f) * bound : 0.0f;
      }
    off += (size_t)in[l] * out[l] + out[l];
  }
}

ne_status cacheUpload(ne_cache* c, const float* host) {
  ne_context* ctx = c->ctx;
  NE_CUDA(cudaMemcpyAsync(c->P, host, kNeMlpParams * 4, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemsetAsync(c->m, 0, kNeMlpParams * 4, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(cudaMemsetAsync(c->v, 0, kNeMlpParams * 4, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(cudaMemsetAsync(c->wfwd, 0, kNeMlpFwdBytes, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(cudaMemsetAsync(c->wbwd, 0, kNeMlpBwdBytes, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(ne_mlp_pack(ctx->stream, c->P, c->wfwd, c->wbwd, c->bias), "k_mlp_pack launch");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  c->step = 0;
  return NE_OK;
}

// Device view of a caller array: the pointer itself with NE_CACHE_DEVICE_PTRS, else a copy.
template <class T>
ne_status stageIn(ne_context* ctx, const T* src, size_t n, bool dev, DevBuf<T>& tmp, const T** out) {
  *out = nullptr;
  if (!src) return NE_OK;
  if (dev) {
    *out = src;
    return NE_OK;
  }
  NE_CUDA(cudaMalloc(&tmp.p, n * sizeof(T)), "cudaMalloc");
  NE_CUDA(cudaMemcpyAsync(tmp.p, src, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  *out = tmp.p;
  return NE_OK;
}

ne_status cacheErr(ne_context* ctx) {
  uint32_t e = 0;
  NE_CUDA(cudaMemcpyAsync(&e, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync(err)");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (e & 6u) return fail(ctx, NE_ERR_TIMEOUT, "radiance cache: a tensor-core product did not complete");
  return NE_OK;
}

}  // namespace

// ---------------------------------------------------------------- view batches
namespace {

// Lays the views out in the tuning's order and uploads the table.
ne_status viewsLayout(ne_views* vw) {
  ne_context* ctx = vw->sc->ctx;
  const uint32_t n = (uint32_t)vw->views.size();
  vw->order.resize(n);
  for (uint32_t i = 0; i < n; i++) vw->order[i] = i;
  auto paths = [&](uint32_t i) { return (uint64_t)vw->views[i].width * vw->views[i].height * vw->views[i].spp; };
  if (vw->tune.order == 1)
    std::stable_sort(vw->order.begin(), vw->order.end(), [&](uint32_t x, uint32_t y) { return paths(x) > paths(y); });
  else if (vw->tune.order == 2)
    std::stable_sort(vw->order.begin(), vw->order.end(), [&](uint32_t x, uint32_t y) { return paths(x) < paths(y); });
  vw->slot_of.assign(n, 0);
  vw->dv.resize(n);
  uint64_t pb = 0;
  uint32_t pix = 0;
  for (uint32_t s = 0; s < n; s++) {
    const ne_view& v = vw->views[vw->order[s]];
    vw->slot_of[vw->order[s]] = s;
    DView& d = vw->dv[s];
    memcpy(&d.cam, &v.camera, sizeof(DCamera));
    d.width = v.width;
    d.height = v.height;
    d.spp = (uint32_t)v.spp;
    d.pix_begin = pix;
    d.stream = vw->order[s] + 1;
    d.pad = 0;
    d.path_begin = pb;
    d.paths = (uint64_t)v.width * v.height * v.spp;
    pb += d.paths;
    pix += (uint32_t)(v.width * v.height);
  }
  // groups: cut the processing order where the running path count passes g / groups of the
  // total, never inside a view
  const int groups = std::max(1, std::min<int>(vw->tune.groups, (int)n));
  vw->group_first.assign(1, 0);
  for (uint32_t s = 0; s + 1 < n && (int)vw->group_first.size() < groups; s++) {
    uint64_t end = vw->dv[s].path_begin + vw->dv[s].paths;
    if (end * (uint64_t)groups >= pb * (uint64_t)vw->group_first.size()) vw->group_first.push_back(end);
  }
  vw->group_first.push_back(pb);
  NE_CUDA(cudaMemcpyAsync(vw->d_views, vw->dv.data(), n * sizeof(DView), cudaMemcpyHostToDevice, ctx->stream),
          "cudaMemcpyAsync");
  std::vector<ViewSpan> spans(n);
  for (uint32_t s = 0; s < n; s++) spans[s] = ViewSpan{vw->dv[s].path_begin, vw->dv[s].paths};
  NE_CUDA(cudaMemcpyAsync(vw->d_spans, spans.data(), n * sizeof(ViewSpan), cudaMemcpyHostToDevice, ctx->stream),
          "cudaMemcpyAsync");
  ViewDone vd = {vw->d_spans, n, vw->d_done, vw->d_done + n};
  NE_CUDA(cudaMemcpyAsync(vw->d_vd, &vd, sizeof(ViewDone), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  return NE_OK;
}

int viewsPasses(const ne_views* vw) { return vw->tune.split_passes == 0 ? 6 : vw->tune.split_passes; }

ne_status viewsEnqueue(ne_views* vw) {
  ne_context* ctx = vw->sc->ctx;
  const uint32_t n = (uint32_t)vw->views.size();
  unsigned long long* done = vw->d_done;
  unsigned long long* tdone = done + n;
  unsigned long long* tstart = done + 2 * n;
  unsigned long long* counter = done + 2 * n + 1;
  NE_CUDA(cudaMemsetAsync(done, 0, 2 * n * sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
  NE_CUDA(cudaMemsetAsync(tstart, 0xFF, sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  const bool split = viewsPasses(vw) > 1;
  // pretrace 2: a first pass that only queues the paths precedes the split passes
  const bool gen = split && vw->tune.pretrace == 2;
  const int passes = viewsPasses(vw) + (gen ? 1 : 0);
  for (size_t g = 0; g + 1 < vw->group_first.size(); g++) {
  NE_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
  ViewArgs a;
  a.P = vw->P;
  a.base = vw->base;
  a.views = vw->d_views;
  a.n_views = n;
  a.first = vw->group_first[g];
  a.total = vw->group_first[g + 1];
  a.fetch = vw->tune.fetch;
  a.out = vw->d_paths;
  a.done = done;
  a.t_done = tdone;
  a.t_start = tstart;
  a.defer_out = split ? vw->d_dq : nullptr;
  a.defer_half = vw->tune.split_half;
  a.defer_top = gen ? 1 : 0;
  if (split) NE_CUDA(cudaMemsetAsync(vw->d_dcount, 0, sizeof(uint32_t), ctx->stream), "cudaMemsetAsync");
  NE_CUDA(ne_launch_views(split, vw->blocks, ctx->stream, vw->sc->d, a, counter, ctx->d_err), "k_views launch");
  for (int pass = 1; pass < passes; pass++) {
    const int in = (pass - 1) & 1, out = pass & 1;
    PathArgs pa;
    pa.P = vw->P;
    pa.base = vw->base;
    pa.total = 0;
    pa.spp = 1;
    pa.sample_offset = 0;
    pa.cover_w = 1;
    pa.keys = nullptr;
    pa.out = vw->d_paths;
    pa.track_share = 16;
    pa.defer_in = vw->d_dq + in;
    pa.defer_out = vw->d_dq + out;
    pa.defer_at = pass == passes - 1 ? -1 : pass - (gen ? 1 : 0);
    pa.defer_half = vw->tune.split_half;
    pa.views = vw->d_vd;
    if (vw->tune.pretrace) {
      // the queued paths' bounce rays, intersected ahead of the pass (k_trace)
      NE_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
      NE_CUDA(nedev::launchTrace_general(ctx->sm_count, ctx->stream, vw->sc->d, vw->d_dq + in, counter, ctx->d_err),
              "k_trace launch");
    }
    NE_CUDA(cudaMemsetAsync(vw->d_dcount + out, 0, sizeof(uint32_t), ctx->stream), "cudaMemsetAsync");
    NE_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
    NE_CUDA(ne_launch_path_split(pass, K_GENERAL, vw->blocks, ctx->stream, vw->sc->d, pa, counter, ctx->d_err),
            "resume kernel launch");
  }
  }
  int rblocks = (int)std::min<uint64_t>((vw->total_pixels + 255) / 256, (uint64_t)ctx->sm_count * 16);
  NE_CUDA(ne_launch_reduce_views(std::max(1, rblocks), ctx->stream, vw->d_paths, vw->d_views, n, vw->total_pixels,
                                 vw->d_img),
          "k_reduce_views launch");
  return NE_OK;
}

// (Re)builds the launch configuration and, with tune.graph, the captured graph.
ne_status viewsPrepare(ne_views* vw) {
  ne_context* ctx = vw->sc->ctx;
  if (vw->exec) {
    cudaGraphExecDestroy(vw->exec);
    vw->exec = nullptr;
  }
  int fit = 1;
  NE_CUDA(ne_views_occupancy(&fit), "occupancy query");
  fit = std::max(1, fit);
  int bps = vw->tune.blocks_per_sm > 0 ? std::min(vw->tune.blocks_per_sm, fit) : fit;
  vw->blocks = ctx->sm_count * bps;
  ne_status st = viewsLayout(vw);
  if (st) return st;
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (vw->tune.pretrace == 2) {
    // the first pass queues every path of a group: the queues grow to the largest group
    size_t need = 1024;
    for (size_t g = 0; g + 1 < vw->group_first.size(); g++)
      need = std::max<size_t>(need, (size_t)(vw->group_first[g + 1] - vw->group_first[g]) + 1024);
    if (need > vw->defer_cap) {
      if (need > 0xFFFFFFFFull) return fail(ctx, NE_ERR_INVALID_ARG, "views: a group above 2^32 paths");
      for (PathState*& q : vw->d_defer) {
        if (q) cudaFree(q);
        q = nullptr;
      }
      vw->defer_cap = need;
      for (PathState*& q : vw->d_defer) NE_CUDA(cudaMalloc(&q, need * sizeof(PathState)), "cudaMalloc(view queues)");
      DeferQueue dq[2];
      for (int i = 0; i < 2; i++) dq[i] = DeferQueue{vw->d_defer[i], vw->d_dcount + i, (uint32_t)need};
      NE_CUDA(cudaMemcpy(vw->d_dq, dq, sizeof(dq), cudaMemcpyHostToDevice), "cudaMemcpy");
    }
  }
  if (vw->tune.graph) {
    cudaGraph_t g = nullptr;
    NE_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    st = viewsEnqueue(vw);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (st) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return cudaFail(ctx, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&vw->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cudaFail(ctx, e, "cudaGraphInstantiate");
  }
  return NE_OK;
}

}  // namespace

extern "C" {

ne_status ne_context_create(int device, ne_context** out) {
  if (!out) return NE_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return NE_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return NE_ERR_INVALID_ARG;
  ne_context* ctx = new ne_context();
  ctx->device = device;
  noallocForget(device);
  auto bad = [&](cudaError_t e, const char* w) {
    ne_status st = cudaFail(ctx, e, w);
    ne_context_destroy(ctx);
    return st;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return bad(e, "cudaSetDevice");
  e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return bad(e, "cudaDeviceGetAttribute");
  e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bad(e, "cudaStreamCreate");
  for (int i = 0; i < 4; i++) {
    e = cudaEventCreate(&ctx->ev[i]);
    if (e != cudaSuccess) return bad(e, "cudaEventCreate");
  }
  e = cudaMalloc(&ctx->d_counter, 8 * sizeof(unsigned long long));
  if (e != cudaSuccess) return bad(e, "cudaMalloc");
  e = cudaMalloc(&ctx->d_err, sizeof(uint32_t));
  if (e != cudaSuccess) return bad(e, "cudaMalloc");
  e = cudaMemset(ctx->d_err, 0, sizeof(uint32_t));
  if (e != cudaSuccess) return bad(e, "cudaMemset");
  size_t freeMem = 0, totalMem = 0;
  e = cudaMemGetInfo(&freeMem, &totalMem);
  if (e != cudaSuccess) return bad(e, "cudaMemGetInfo");
  ctx->pool.limit = std::max(kPoolMinLimit, totalMem / 4);
  *out = ctx;
  return NE_OK;
}

ne_status ne_context_set_cache_limit(ne_context* ctx, size_t bytes) {
  if (!ctx) return NE_ERR_INVALID_ARG;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  ctx->pool.limit = bytes;
  ctx->pool.trim(bytes);
  return NE_OK;
}

void ne_context_destroy(ne_context* ctx) {
  if (!ctx) return;
  while (!ctx->scenes.empty()) ne_scene_destroy(ctx->scenes.back());
  while (!ctx->caches.empty()) ne_cache_destroy(ctx->caches.back());
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (int i = 0; i < 4; i++)
    if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
  for (int i = 0; i < 8; i++)
    if (ctx->user_ev[i]) cudaEventDestroy(ctx->user_ev[i]);
  for (cudaEvent_t e : ctx->slab_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->flush_buf) cudaFree(ctx->flush_buf);
  if (ctx->d_counter) cudaFree(ctx->d_counter);
  if (ctx->d_err) cudaFree(ctx->d_err);
  ctx->pool.trim(0);
  for (auto& kv : ctx->pool.size_of) cudaFree(kv.first);  // buffers never given back
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* ne_last_error(const ne_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

// World-space bounds of the primitives whose material has a medium: a walk of intersectTr
// whose ray misses all of them can reach no medium. Each primitive's OCS bounds (box corners,
// sphere centre +- radius, rectangle corners, triangle vertices) go through the instance's
// transform in double precision and are widened by 1e-3 of their extent and position, far
// beyond the rounding of the float transforms and of the walk's successive origins.
// Returns the number of boxes (6 floats each: min xyz, max xyz), or -1 when they are not
// known (a non-finite bound, a rectangle whose hits its corners do not bound, or more than 64
// boxes): every ray may then reach a medium.
static int32_t mediumBoxesOf(const ne_scene_desc& D, std::vector<float>& boxes) {
  boxes.clear();
  int32_t nMediumBoxes = 0;
  const uint32_t ninst = D.n_instances + D.n_light_instances;
  for (uint32_t i = 0; i < ninst && nMediumBoxes >= 0; i++) {
    const ne_model& m = D.models[D.instances[i].model];
    const float* W = D.instances[i].to_wcs;
    auto addPrim = [&](const ne_primitive& p) {
      if (p.material < 0 || D.materials[p.material].medium < 0) return;
      double lo[3], hi[3];
      for (int a = 0; a < 3; a++) {
        if (p.type == NE_PRIM_SPHERE) {
          lo[a] = (double)p.p0[a] - fabs((double)p.radius);
          hi[a] = (double)p.p0[a] + fabs((double)p.radius);
        } else {
          lo[a] = std::min((double)p.p0[a], (double)p.p1[a]);
          hi[a] = std::max((double)p.p0[a], (double)p.p1[a]);
          if (p.type == NE_PRIM_TRIANGLE) {
            lo[a] = std::min(lo[a], (double)p.p2[a]);
            hi[a] = std::max(hi[a], (double)p.p2[a]);
          }
        }
      }
      double wlo[3] = {INFINITY, INFINITY, INFINITY}, whi[3] = {-INFINITY, -INFINITY, -INFINITY};
      for (int corner = 0; corner < 8; corner++) {
        double q[3] = {(corner & 1) ? hi[0] : lo[0], (corner & 2) ? hi[1] : lo[1], (corner & 4) ? hi[2] : lo[2]};
        for (int r = 0; r < 3; r++) {
          double w = (double)W[12 + r];
          for (int c = 0; c < 3; c++) w += (double)W[c * 4 + r] * q[c];
          wlo[r] = std::min(wlo[r], w);
          whi[r] = std::max(whi[r], w);
        }
      }
      bool finite = true;
      for (int a = 0; a < 3; a++) finite = finite && std::isfinite(wlo[a]) && std::isfinite(whi[a]);
      if (p.type == NE_PRIM_RECTANGLE) {
        // Rectangle::intersect checks containment only on the axes where the corners differ;
        // its hits stay inside the corners' box only if the corners agree on exactly one axis
        // and the plane normal lies along it
        int same = 0;
        for (int a = 0; a < 3; a++) {
          if (p.p0[a] == p.p1[a]) same++;
          else if (p.p2[a] != 0.0f) finite = false;
        }
        if (same != 1) finite = false;
      }
      if (!finite || p.type == NE_PRIM_POINT) {
        if (!finite) nMediumBoxes = -1;  // unbounded, or not known to be bounded
        return;
      }
      for (int a = 0; a < 3; a++) {
        double margin = 1e-3 * ((whi[a] - wlo[a]) + std::max(fabs(wlo[a]), fabs(whi[a]))) + 1e-6;
        boxes.push_back((float)(wlo[a] - margin));
      }
      for (int a = 0; a < 3; a++) {
        double margin = 1e-3 * ((whi[a] - wlo[a]) + std::max(fabs(wlo[a]), fabs(whi[a]))) + 1e-6;
        boxes.push_back((float)(whi[a] + margin));
      }
      if (nMediumBoxes >= 0) nMediumBoxes++;
    };
    for (uint32_t k = 0; k < m.prim_count && nMediumBoxes >= 0; k++) addPrim(D.prims[m.prim_begin + k]);
    for (uint32_t k = 0; k < m.light_count && nMediumBoxes >= 0; k++) addPrim(D.prims[m.light_begin + k]);
  }
  if (nMediumBoxes > 64) nMediumBoxes = -1;  // many media: the test would cost more than it saves
  if (nMediumBoxes < 0) boxes.clear();
  return nMediumBoxes;
}

ne_status ne_scene_upload(ne_context* ctx, const ne_scene_desc* desc, ne_scene** out) {
  if (!ctx || !desc || !out) return NE_ERR_INVALID_ARG;
  *out = nullptr;
  const ne_scene_desc& D = *desc;
  uint32_t ninst = D.n_instances + D.n_light_instances;
  if (D.settings.width <= 0 || D.settings.height <= 0) return fail(ctx, NE_ERR_INVALID_ARG, "scene has no resolution");
  // validate indices so that no kernel reads out of bounds
  for (uint32_t i = 0; i < ninst; i++)
    if (D.instances[i].model >= D.n_models) return fail(ctx, NE_ERR_INVALID_ARG, "instance model index out of range");
  for (uint32_t i = 0; i < D.n_models; i++) {
    const ne_model& m = D.models[i];
    if ((uint64_t)m.prim_begin + m.prim_count > D.n_prims || (uint64_t)m.light_begin + m.light_count > D.n_prims ||
        (uint64_t)m.mat_begin + m.mat_count > D.n_model_materials)
      return fail(ctx, NE_ERR_INVALID_ARG, "model ranges out of range");
    for (uint32_t k = 0; k < m.light_count; k++) {
      int mat = D.prims[m.light_begin + k].material;
      if (mat < 0 || mat >= (int)D.n_materials || D.materials[mat].light < 0)
        return fail(ctx, NE_ERR_INVALID_ARG, "emissive primitive without a light material");
    }
    if (m.use_bvh) {
      std::atomic<bool> other{false};
      nehost::parallelFor(m.prim_count, 1u << 16, [&](size_t b, size_t e) {
        for (size_t k = b; k < e; k++)
          if (D.prims[m.prim_begin + k].type != NE_PRIM_TRIANGLE) other = true;
      });
      if (other) return fail(ctx, NE_ERR_INVALID_ARG, "BVH models hold triangles only");
    }
  }
  for (uint32_t i = 0; i < D.n_light_instances; i++) {
    const ne_model& m = D.models[D.instances[D.n_instances + i].model];
    for (uint32_t k = 0; k < m.mat_count; k++) {
      uint32_t mm = D.model_materials[m.mat_begin + k];
      if (mm >= D.n_materials || D.materials[mm].light < 0)
        return fail(ctx, NE_ERR_INVALID_ARG, "light instance material without a light");
    }
  }
  {
    std::atomic<size_t> firstBad{SIZE_MAX};  // the first bad primitive in index order
    nehost::parallelFor(D.n_prims, 1u << 16, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; i++) {
        const int mat = D.prims[i].material, type = D.prims[i].type;
        const int why = mat >= (int)D.n_materials ? 1 : ((type < 0 || type > NE_PRIM_POINT) ? 2 : 0);
        if (!why) continue;
        size_t cur = firstBad.load();
        while (i < cur && !firstBad.compare_exchange_weak(cur, i)) {
        }
        break;
      }
    });
    if (firstBad.load() != SIZE_MAX) {
      const size_t i = firstBad.load();
      if (D.prims[i].material >= (int)D.n_materials)
        return fail(ctx, NE_ERR_INVALID_ARG, "primitive material out of range");
      return fail(ctx, NE_ERR_INVALID_ARG, "bad primitive type");
    }
  }
  for (uint32_t i = 0; i < D.n_materials; i++) {
    const ne_material& m = D.materials[i];
    if (m.light >= (int)D.n_lights || m.medium >= (int)D.n_media) return fail(ctx, NE_ERR_INVALID_ARG, "material index out of range");
    if (m.bsdf == NE_BSDF_VOLUME && m.medium < 0) return fail(ctx, NE_ERR_INVALID_ARG, "volume material without a medium");
  }
  for (uint32_t i = 0; i < D.n_lights; i++) {
    const ne_light& L = D.lights[i];
    if (L.primitive >= (int)D.n_prims) return fail(ctx, NE_ERR_INVALID_ARG, "light primitive out of range");
    if (L.type == NE_LIGHT_INFINITE && L.env_width != 0 &&
        (L.env_width < 0 || L.env_height <= 0 || !L.env_texels || L.env_width > (1 << 16)))
      return fail(ctx, NE_ERR_INVALID_ARG, "environment map without texels");
    if (L.type == NE_LIGHT_INFINITE && L.env_width > 0 && L.env_height > L.env_width)
      return fail(ctx, NE_ERR_UNSUPPORTED,
                  "environment maps taller than wide are not supported (the reference's Distribution2D reads past "
                  "such an image)");
  }
  // every light reachable from a light instance is sampled through Light::primitive
  for (uint32_t i = 0; i < D.n_light_instances; i++) {
    const ne_model& m = D.models[D.instances[D.n_instances + i].model];
    for (uint32_t k = 0; k < m.light_count; k++) {
      const ne_light& L = D.lights[D.materials[D.prims[m.light_begin + k].material].light];
      if (L.primitive < 0) return fail(ctx, NE_ERR_INVALID_ARG, "light without a primitive");
    }
  }

  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  ne_scene* sc = new ne_scene();
  sc->ctx = ctx;
  ctx->scenes.push_back(sc);
  sc->settings = D.settings;
  memset(&sc->d, 0, sizeof(sc->d));
  auto cleanup = [&](ne_status st) {
    ne_scene_destroy(sc);
    return st;
  };
  // a failed CUDA call from here on also releases the half-built scene
#define NE_CUDA_SC(call, where)                                           \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) return cleanup(cudaFail(ctx, e_, where));      \
  } while (0)

  // instances
  std::vector<DInstance> inst(ninst);
  for (uint32_t i = 0; i < ninst; i++) {
    const ne_instance& s = D.instances[i];
    DInstance& d = inst[i];
    memset(&d, 0, sizeof(d));
    for (int c = 0; c < 4; c++)
      for (int r = 0; r < 3; r++) {
        d.wcs[c * 3 + r] = s.to_wcs[c * 4 + r];
        d.ocs[c * 3 + r] = s.to_ocs[c * 4 + r];
      }
    H3 sc3 = getScale(s.to_wcs);
    d.scale[0] = sc3.x; d.scale[1] = sc3.y; d.scale[2] = sc3.z;
    d.model = s.model;
    d.collision = s.collision;
    // InstancedModel::intersect can only return false for a model whose primitives are points
    // (Point::intersect) and whose light primitives are points or carry a light whose Le is a
    // non-black constant (every light but a textured environment: Model.cpp:432-434 skips
    // them); the queries then skip the instance's ray transform too
    const ne_model& m = D.models[s.model];
    bool never = true;
    for (uint32_t k = 0; k < m.prim_count && never; k++) never = D.prims[m.prim_begin + k].type == NE_PRIM_POINT;
    for (uint32_t k = 0; k < m.light_count && never; k++) {
      const ne_primitive& lp = D.prims[m.light_begin + k];
      if (lp.type == NE_PRIM_POINT) continue;
      const ne_light& L = D.lights[D.materials[lp.material].light];
      const float* le = L.type == NE_LIGHT_INFINITE ? L.env_radiance : L.le;
      bool constant = !(L.type == NE_LIGHT_INFINITE && L.env_width > 0);
      never = constant && (le[0] != 0.0f || le[1] != 0.0f || le[2] != 0.0f);
    }
    d.never_hit = never ? 1 : 0;
  }
  std::vector<float> mediumBoxes;
  const int32_t nMediumBoxes = mediumBoxesOf(D, mediumBoxes);
  // primitives
  // per material: does its medium make the primitive a grid-medium boundary (DPrim::flags)
  std::vector<uint8_t> gridMat(std::max<uint32_t>(1, D.n_materials), 0);
  for (uint32_t i = 0; i < D.n_materials; i++) {
    const ne_material& m = D.materials[i];
    gridMat[i] = (m.medium >= 0 && D.media[m.medium].type == NE_MEDIUM_GRID) ? 1 : 0;
  }
  // models + BVHs
  std::vector<DModel> models(D.n_models);
  std::vector<DNode> nodes;
  std::vector<uint32_t> slots;
  for (uint32_t i = 0; i < D.n_models; i++) {
    const ne_model& s = D.models[i];
    DModel& d = models[i];
    memset(&d, 0, sizeof(d));
    d.prim_begin = s.prim_begin; d.prim_count = s.prim_count;
    d.light_begin = s.light_begin; d.light_count = s.light_count;
    d.mat_begin = s.mat_begin; d.mat_count = s.mat_count;
    d.has_bbox = s.has_bbox;
    memcpy(d.bbox_min, s.bbox_min, 12);
    memcpy(d.bbox_max, s.bbox_max, 12);
    if (s.use_bvh && s.prim_count > 0 && D.settings.bvh_build == 1) {
      d.use_bvh = 1;  // built on the GPU once the primitives are there (below)
    } else if (s.use_bvh && s.prim_count > 0) {
      std::vector<uint32_t> order(s.prim_count);
      for (uint32_t k = 0; k < s.prim_count; k++) order[k] = s.prim_begin + k;
      std::vector<HNode> hn;
      buildBvh(D.prims, order, hn);
      d.use_bvh = 1;
      d.bvh_node0 = (uint32_t)nodes.size();
      d.bvh_slot0 = (uint32_t)slots.size();
      for (const HNode& h : hn) {
        DNode n;
        n.lo[0] = h.mn.x; n.lo[1] = h.mn.y; n.lo[2] = h.mn.z;
        n.hi[0] = h.mx.x; n.hi[1] = h.mx.y; n.hi[2] = h.mx.z;
        uint32_t a, b;
        if (h.rightOffset == 0) { a = h.start; b = h.count | 0x80000000u; }
        else { a = h.rightOffset; b = 0; }
        memcpy(&n.lo[3], &a, 4);
        memcpy(&n.hi[3], &b, 4);
        nodes.push_back(n);
      }
      slots.insert(slots.end(), order.begin(), order.end());
    }
  }
  // materials, lights
  std::vector<DMaterial> mats(D.n_materials);
  for (uint32_t i = 0; i < D.n_materials; i++) {
    const ne_material& s = D.materials[i];
    DMaterial& d = mats[i];
    memset(&d, 0, sizeof(d));
    d.bsdf = s.bsdf; d.light = s.light; d.medium = s.medium; d.phase = s.phase; d.g = s.g;
    memcpy(d.albedo, s.albedo, 12);
    d.roughness = s.roughness; d.metallic = s.metallic;
    memcpy(d.normal_map, s.normal_map, 12);
    d.tex_present = s.tex_present; d.tex_types = s.tex_types;
    if (s.bsdf == NE_BSDF_GLOSSY && s.albedo_width > 0) {
      if (!s.albedo_texels || s.albedo_height <= 0)
        return cleanup(fail(ctx, NE_ERR_INVALID_ARG, "albedo texture without texels"));
      const uint8_t* tex = nullptr;
      ne_status st = upload(sc, s.albedo_texels, (size_t)s.albedo_width * s.albedo_height * 4, &tex);
      if (st) return cleanup(st);
      d.albedo_w = s.albedo_width;
      d.albedo_h = s.albedo_height;
      d.albedo_tex = (const uchar4*)tex;
    }
  }
  std::vector<DLight> lights(D.n_lights);
  std::deque<EnvTables> envTables;  // host sources of the table copies, alive until the upload syncs
  for (uint32_t i = 0; i < D.n_lights; i++) {
    const ne_light& s = D.lights[i];
    DLight& d = lights[i];
    memset(&d, 0, sizeof(d));
    d.type = s.type; d.primitive = s.primitive;
    memcpy(d.li, s.li, 12); memcpy(d.le, s.le, 12);
    memcpy(d.direction, s.direction, 12); memcpy(d.env_radiance, s.env_radiance, 12);
    d.env_map_pdf = s.env_map_pdf;
    if (s.type == NE_LIGHT_INFINITE && s.env_width > 0) {
      envTables.push_back(buildEnvTables(s));
      const EnvTables& e = envTables.back();
      d.env_w = s.env_width;
      d.env_h = s.env_height;
      d.env_marg_int = e.margInt;
      const uint8_t* tex = nullptr;
      ne_status st = NE_OK;
      if ((st = upload(sc, s.env_texels, (size_t)s.env_width * s.env_height * 4, &tex)) ||
          (st = upload(sc, e.condFunc.data(), e.condFunc.size(), &d.env_cond_func)) ||
          (st = upload(sc, e.condCdf.data(), e.condCdf.size(), &d.env_cond_cdf)) ||
          (st = upload(sc, e.condInt.data(), e.condInt.size(), &d.env_cond_int)) ||
          (st = upload(sc, e.margFunc.data(), e.margFunc.size(), &d.env_marg_func)) ||
          (st = upload(sc, e.margCdf.data(), e.margCdf.size(), &d.env_marg_cdf)))
        return cleanup(st);
      d.env_tex = (const uchar4*)tex;
    }
  }
  // media: dense grid + 8-corner cells
  std::vector<DMedium> media(D.n_media);
  std::vector<uint32_t> gridMedia;
  for (uint32_t i = 0; i < D.n_media; i++) {
    const ne_medium& s = D.media[i];
    DMedium& d = media[i];
    memset(&d, 0, sizeof(d));
    d.type = s.type;
    memcpy(d.sigma_s, s.sigma_s, 12);
    for (int k = 0; k < 3; k++) d.sigma_t[k] = s.sigma_a[k] + s.sigma_s[k];
    d.density = s.density;
    // avg(extinction * densityMultiplier) (materials/GridMedia.cpp:56,82)
    float e0 = d.sigma_t[0] * s.density, e1 = d.sigma_t[1] * s.density, e2 = d.sigma_t[2] * s.density;
    d.mu = (e0 + e1 + e2) / 3.0f;
    d.inv_max_density = 1.0f;
    if (s.type == NE_MEDIUM_GRID) {
      if (!s.grid || !s.res[0] || !s.res[1] || !s.res[2]) return cleanup(fail(ctx, NE_ERR_INVALID_ARG, "grid medium without voxels"));
      if (s.res[0] > (1u << 24) || s.res[1] > (1u << 24) || s.res[2] > (1u << 24))
        return cleanup(fail(ctx, NE_ERR_INVALID_ARG, "grid resolution above 2^24 voxels per axis"));
      size_t n = (size_t)s.res[0] * s.res[1] * s.res[2];
      gridMedia.push_back(i);  // invMaxDensity from the device copy of the grid, below
      memcpy(d.res, s.res, 12);
      d.resf[0] = (float)s.res[0]; d.resf[1] = (float)s.res[1]; d.resf[2] = (float)s.res[2];
      void* gp = nullptr;
      cudaError_t e = ctx->pool.get(n * sizeof(float), &gp);
      if (e != cudaSuccess) return cleanup(cudaFail(ctx, e, "cudaMalloc(grid)"));
      sc->allocs.push_back(gp);
      const float* dg = (const float*)gp;
      d.grid = dg;
      size_t ncell = (size_t)(s.res[0] + 1) * (s.res[1] + 1) * (s.res[2] + 1);
      void* cp = nullptr;
      e = ctx->pool.get(ncell * 2 * sizeof(float4), &cp);
      if (e != cudaSuccess) return cleanup(cudaFail(ctx, e, "cudaMalloc(cells)"));
      sc->allocs.push_back(cp);
      // the grid in slabs of z slices on the copy stream; the cells of each slab (which read
      // its slices and the next one) built on the main stream once they are there
      if (!ctx->copy_stream) {
        NE_CUDA_SC(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        for (cudaEvent_t& ev : ctx->slab_ev)
          NE_CUDA_SC(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
      }
      const uint32_t W = s.res[0], H = s.res[1], Dz = s.res[2];
      const size_t slice = (size_t)W * H;
      const int slabs = (int)std::min<uint32_t>(kGridSlabs, Dz);
      // the buffers may have been in use on the main stream until now
      NE_CUDA_SC(cudaEventRecord(ctx->slab_ev[kGridSlabs], ctx->stream), "cudaEventRecord");
      NE_CUDA_SC(cudaStreamWaitEvent(ctx->copy_stream, ctx->slab_ev[kGridSlabs], 0), "cudaStreamWaitEvent");
      uint32_t cellsDone = 0;
      for (int k = 0; k < slabs; k++) {
        const uint32_t z0 = (uint32_t)((uint64_t)Dz * k / slabs), z1 = (uint32_t)((uint64_t)Dz * (k + 1) / slabs);
        NE_CUDA_SC(cudaMemcpyAsync((float*)gp + z0 * slice, s.grid + z0 * slice, (size_t)(z1 - z0) * slice * sizeof(float),
                                cudaMemcpyHostToDevice, ctx->copy_stream),
                "cudaMemcpyAsync(grid)");
        NE_CUDA_SC(cudaEventRecord(ctx->slab_ev[k], ctx->copy_stream), "cudaEventRecord");
        NE_CUDA_SC(cudaStreamWaitEvent(ctx->stream, ctx->slab_ev[k], 0), "cudaStreamWaitEvent");
        // cell slab z reads grid slices z and z + 1: with slices [0, z1) there, cells [.., z1 - 1)
        const uint32_t cellsTo = k == slabs - 1 ? Dz + 1 : z1 - 1;
        if (cellsTo > cellsDone) {
          const uint32_t rows = (cellsTo - cellsDone) * (H + 1);
          const int blocks = (int)std::min<uint32_t>(rows, (uint32_t)ctx->sm_count * 16);
          k_cells<<<blocks, 256, 0, ctx->stream>>>(dg, W, H, Dz, cellsDone, cellsTo, (float4*)cp);
          e = cudaGetLastError();
          if (e != cudaSuccess) return cleanup(cudaFail(ctx, e, "k_cells launch"));
          cellsDone = cellsTo;
        }
      }
      d.cells = (const float4*)cp;
    }
  }
  ne_status st = NE_OK;
  if (D.n_prims) {
    // the descriptor's primitives converted on the device (k_convert_prims)
    void* raw = nullptr;
    void* dp = nullptr;
    const uint8_t* dGrid = nullptr;
    NE_CUDA_SC(ctx->pool.get((size_t)D.n_prims * sizeof(ne_primitive), &raw), "cudaMalloc(primitives)");
    cudaError_t ce = cudaMemcpyAsync(raw, D.prims, (size_t)D.n_prims * sizeof(ne_primitive), cudaMemcpyHostToDevice,
                                     ctx->stream);
    if (ce != cudaSuccess) {
      ctx->pool.put(raw);
      return cleanup(cudaFail(ctx, ce, "cudaMemcpyAsync(primitives)"));
    }
    if ((st = upload(sc, gridMat.data(), gridMat.size(), &dGrid))) {
      ctx->pool.put(raw);
      return cleanup(st);
    }
    cudaError_t e = ctx->pool.get((size_t)D.n_prims * sizeof(DPrim), &dp);
    if (e != cudaSuccess) {
      ctx->pool.put(raw);
      return cleanup(cudaFail(ctx, e, "cudaMalloc(primitives)"));
    }
    sc->allocs.push_back(dp);
    const int blocks = (int)std::min<size_t>(((size_t)D.n_prims + 255) / 256, (size_t)ctx->sm_count * 8);
    k_convert_prims<<<blocks, 256, 0, ctx->stream>>>((const ne_primitive*)raw, D.n_prims, dGrid, (DPrim*)dp);
    e = cudaGetLastError();
    ctx->pool.put(raw);  // stream order: its next user runs after the conversion
    if (e != cudaSuccess) return cleanup(cudaFail(ctx, e, "k_convert_prims launch"));
    sc->d.prims = (const DPrim*)dp;
  }
  if (D.settings.bvh_build == 1) {
    // binned-SAH trees built on the GPU from the uploaded primitives
    for (uint32_t i = 0; i < D.n_models; i++) {
      const ne_model& s = D.models[i];
      if (!s.use_bvh || s.prim_count == 0) continue;
      std::vector<DNode> bn;
      std::vector<uint32_t> bs;
      std::string err;
      cudaError_t e = buildSahBvh(ctx->stream, sc->d.prims, s.prim_begin, s.prim_count, bn, bs, err);
      if (e != cudaSuccess) {
        if (!err.empty()) return cleanup(fail(ctx, NE_ERR_CUDA, err.c_str()));
        return cleanup(cudaFail(ctx, e, "GPU BVH build"));
      }
      models[i].bvh_node0 = (uint32_t)nodes.size();
      models[i].bvh_slot0 = (uint32_t)slots.size();
      nodes.insert(nodes.end(), bn.begin(), bn.end());
      slots.insert(slots.end(), bs.begin(), bs.end());
    }
  }
  sc->bvh_nodes_of.assign(D.n_models, 0);
  for (uint32_t i = 0; i < D.n_models; i++) {
    if (!models[i].use_bvh) continue;
    uint32_t end = (uint32_t)nodes.size();
    for (uint32_t j = 0; j < D.n_models; j++)
      if (models[j].use_bvh && models[j].bvh_node0 > models[i].bvh_node0) end = std::min(end, models[j].bvh_node0);
    sc->bvh_nodes_of[i] = end - models[i].bvh_node0;
  }
  sc->bvh_models.assign(models.begin(), models.end());
  if ((st = upload(sc, inst.data(), inst.size(), &sc->d.instances))) return cleanup(st);
  if ((st = upload(sc, models.data(), models.size(), &sc->d.models))) return cleanup(st);
  if ((st = upload(sc, mats.data(), mats.size(), &sc->d.materials))) return cleanup(st);
  if ((st = upload(sc, D.model_materials, D.n_model_materials, &sc->d.model_materials))) return cleanup(st);
  if ((st = upload(sc, lights.data(), lights.size(), &sc->d.lights))) return cleanup(st);
  if ((st = upload(sc, media.data(), media.size(), &sc->d.media))) return cleanup(st);
  if (nMediumBoxes > 0 && (st = upload(sc, mediumBoxes.data(), mediumBoxes.size(), &sc->d.medium_boxes)))
    return cleanup(st);
  sc->d.n_medium_boxes = nMediumBoxes;
  if (!gridMedia.empty()) {
    std::vector<uint32_t> keys(gridMedia.size(), 0x80000000u);  // the key of 0
    const uint32_t* dkeys = nullptr;
    if ((st = upload(sc, keys.data(), keys.size(), &dkeys))) return cleanup(st);
    for (size_t k = 0; k < gridMedia.size(); k++) {
      const uint32_t i = gridMedia[k];
      const size_t n = (size_t)media[i].res[0] * media[i].res[1] * media[i].res[2];
      uint32_t* key = const_cast<uint32_t*>(dkeys) + k;
      int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx->sm_count * 8);
      k_grid_max<<<std::max(1, blocks), 256, 0, ctx->stream>>>(media[i].grid, n, key);
      k_grid_inv_max<<<1, 1, 0, ctx->stream>>>(key, const_cast<DMedium*>(sc->d.media) + i);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return cleanup(cudaFail(ctx, e, "k_grid_max launch"));
    }
  }
  if ((st = upload(sc, nodes.data(), nodes.size(), &sc->d.bvh))) return cleanup(st);
  if ((st = upload(sc, slots.data(), slots.size(), &sc->d.bvh_prims))) return cleanup(st);
  sc->d.n_instances = D.n_instances;
  sc->d.n_light_instances = D.n_light_instances;
  sc->d.n_prims = D.n_prims;
  sc->d.n_media = D.n_media;
  const ne_camera& cm = D.camera;
  memcpy(sc->d.camera.position, cm.position, 12);
  memcpy(sc->d.camera.lower_left, cm.lower_left, 12);
  memcpy(sc->d.camera.horizontal, cm.horizontal, 12);
  memcpy(sc->d.camera.vertical, cm.vertical, 12);
  memcpy(sc->d.camera.side, cm.side, 12);
  memcpy(sc->d.camera.up, cm.up, 12);
  sc->d.camera.lens_radius = cm.lens_radius;
  sc->d.width = D.settings.width;
  sc->d.height = D.settings.height;
  // feature bits: which primitive, BSDF, medium and light kinds the kernels must handle
  std::atomic<uint32_t> primBits{0};
  nehost::parallelFor(D.n_prims, 1u << 16, [&](size_t i0, size_t i1) {
    uint32_t f = 0;
    for (size_t i = i0; i < i1; i++) {
      switch (D.prims[i].type) {
        case NE_PRIM_SPHERE: f |= FT_SPHERE; break;
        case NE_PRIM_RECTANGLE: f |= FT_RECT; break;
        case NE_PRIM_AABB: f |= FT_AABB; break;
        case NE_PRIM_TRIANGLE: f |= FT_TRI; break;
        default: f |= FT_POINT; break;
      }
    }
    primBits.fetch_or(f);
  });
  uint32_t F = primBits.load();
  for (uint32_t i = 0; i < D.n_models; i++) {
    if (D.models[i].has_bbox) F |= FT_BBOX;
    if (D.models[i].use_bvh) F |= FT_TRI;
  }
  for (uint32_t i = 0; i < D.n_materials; i++) {
    const ne_material& m = D.materials[i];
    if (m.bsdf == NE_BSDF_GLOSSY) F |= FT_GLOSSY;
    if (m.bsdf == NE_BSDF_VOLUME) F |= FT_VOLBSDF;
    if (m.tex_types & NE_TEX_NORMAL) F |= FT_NORMALMAP;
    if (m.bsdf == NE_BSDF_GLOSSY && m.albedo_width > 0) F |= FT_TEXALB;
  }
  for (uint32_t i = 0; i < D.n_media; i++) F |= D.media[i].type == NE_MEDIUM_GRID ? FT_GRID : FT_HOMOG;
  for (uint32_t i = 0; i < D.n_lights; i++) {
    F |= D.lights[i].type == NE_LIGHT_DIFFUSE ? FT_LDIFF : (D.lights[i].type == NE_LIGHT_DIRECTIONAL ? FT_LDIR : FT_LINF);
    if (D.lights[i].type == NE_LIGHT_INFINITE && D.lights[i].env_width > 0) F |= FT_ENVMAP;
  }
  sc->features = F;
  sc->feature_set = ne_feature_set_for(F);
  ne_tuning tn;
  // the split kernel is the fastest measured on every scene (Mpaths/s, one pass -> split by
  // bounce, 8 passes -> split by half bounce, 16 passes: medium 386 -> 1366 -> 1510, Cornell
  // 209 -> 592 -> 574, mesh 127 -> 171 -> 171, dense cloud 115 -> 239 -> 268)
  tn.kernel = 3;
  tn.track_share = sc->track_share;
  tn.blocks_per_sm = 0;
  tn.split_passes = 0;
  tn.split_half = 1;
  tn.queue_quarters = 3;
  tn.pretrace = 0;
  if (ne_scene_set_tuning(sc, &tn) != NE_OK) return cleanup(NE_ERR_INVALID_ARG);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cleanup(cudaFail(ctx, e, "scene upload"));
  *out = sc;
  return NE_OK;
}

#undef NE_CUDA_SC

ne_status ne_scene_set_tuning(ne_scene* sc, const ne_tuning* t) {
  if (!sc || !t || t->kernel < 0 || t->kernel > 3 || t->track_share < 1 || t->track_share > 32 ||
      t->blocks_per_sm < 0 || t->blocks_per_sm > 64 || t->split_passes < 0 || t->split_passes == 1 ||
      t->split_passes > 64 || t->split_half < 0 || t->split_half > 1 || t->queue_quarters < 0 ||
      t->queue_quarters > 8 || t->pretrace < 0 || t->pretrace > 3)
    return NE_ERR_INVALID_ARG;
  ne_context* ctx = sc->ctx;
  int fit = 1;
  cudaError_t e = ne_path_kernel_occupancy(t->kernel, sc->feature_set, &fit);
  if (e != cudaSuccess) return cudaFail(ctx, e, "occupancy query");
  if (fit < 1) fit = 1;
  sc->variant = t->kernel;
  sc->split_passes = t->split_passes ? t->split_passes : (t->split_half ? 16 : 8);
  sc->split_half = t->split_half;
  sc->track_share = t->track_share;
  sc->blocks_per_sm = t->blocks_per_sm > 0 ? std::min(t->blocks_per_sm, fit) : fit;
  sc->queue_quarters = t->queue_quarters ? t->queue_quarters : 3;
  sc->pretrace = t->pretrace;
  return NE_OK;
}

ne_status ne_scene_get_tuning(const ne_scene* sc, ne_tuning* t) {
  if (!sc || !t) return NE_ERR_INVALID_ARG;
  t->kernel = sc->variant;
  t->track_share = sc->track_share;
  t->blocks_per_sm = sc->blocks_per_sm;
  t->split_passes = sc->split_passes;
  t->split_half = sc->split_half;
  t->queue_quarters = sc->queue_quarters;
  t->pretrace = sc->pretrace;
  return NE_OK;
}

void ne_scene_destroy(ne_scene* sc) {
  if (!sc) return;
  while (!sc->view_batches.empty()) ne_views_destroy(sc->view_batches.back());
  auto& v = sc->ctx->scenes;
  v.erase(std::remove(v.begin(), v.end(), sc), v.end());
  cudaSetDevice(sc->ctx->device);
  cudaStreamSynchronize(sc->ctx->stream);
  DevicePool& pool = sc->ctx->pool;
  for (void* p : sc->allocs) pool.put(p);
  pool.put(sc->d_paths);
  for (PathState* q : sc->d_defer) pool.put(q);
  pool.put(sc->d_dq);
  pool.put(sc->d_pass);
  delete sc;
}

ne_status ne_render(ne_scene* sc, const ne_render_params* p, float* out_rgb, ne_render_stats* stats) {
  if (!sc || !out_rgb) return NE_ERR_INVALID_ARG;
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const int W = sc->settings.width, H = sc->settings.height;
  int spp = (p && p->spp > 0) ? p->spp : sc->settings.spp;
  if (spp <= 0) return fail(ctx, NE_ERR_INVALID_ARG, "spp must be positive");
  uint32_t flags = p ? p->flags : 0;
  uint32_t cw = (uint32_t)W, ch = (uint32_t)H;
  if (flags & NE_RENDER_REF_TILES) {  // OfflineEngine.cpp:18-21: 40 x 10 tiles of (W/40, H/10)
    cw = 40u * (uint32_t)(W / 40);
    ch = 10u * (uint32_t)(H / 10);
  }
  uint64_t npix = (uint64_t)cw * ch;
  uint64_t total = npix * (uint64_t)spp;
  if (sc->paths_cap < total) {
    ctx->pool.put(sc->d_paths);
    sc->d_paths = nullptr;
    sc->paths_cap = 0;
    void* pp = nullptr;
    NE_CUDA(ctx->pool.get(total * 3 * sizeof(float), &pp), "cudaMalloc(paths)");
    sc->d_paths = (float*)pp;
    sc->paths_cap = total;
  }
  bool devOut = flags & NE_RENDER_OUT_DEVICE;
  float* d_img = nullptr;
  PoolBuf tmpImg;  // given back after the copy to the host, which this call waits for
  size_t imgBytes = (size_t)W * H * 3 * sizeof(float);
  if (devOut) {
    d_img = out_rgb;
  } else {
    NE_CUDA(tmpImg.get(ctx->pool, imgBytes), "cudaMalloc(image)");
    d_img = (float*)tmpImg.p;
  }
  bool timed = !(flags & NE_RENDER_NO_SYNC);
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  if (timed) NE_CUDA(cudaEventRecord(ctx->ev[0], ctx->stream), "cudaEventRecord");
  if (cw != (uint32_t)W || ch != (uint32_t)H) NE_CUDA(cudaMemsetAsync(d_img, 0, imgBytes, ctx->stream), "cudaMemsetAsync");
  PathArgs a;
  a.P = pathParams(sc, p);
  a.base = baseKey(p);
  a.total = total;
  a.spp = (uint32_t)spp;
  a.sample_offset = p ? p->sample_offset : 0;
  a.cover_w = cw;
  a.keys = nullptr;
  a.out = sc->d_paths;
  a.track_share = 16;
  if (timed) NE_CUDA(cudaEventRecord(ctx->ev[1], ctx->stream), "cudaEventRecord");
  ne_status st = launchPaths(sc, a, (flags & NE_RENDER_COUNT_WORK) != 0);
  if (st) return st;
  if (timed) NE_CUDA(cudaEventRecord(ctx->ev[2], ctx->stream), "cudaEventRecord");
  int rblocks = (int)std::min<uint64_t>((npix + 255) / 256, (uint64_t)ctx->sm_count * 16);
  k_reduce<<<std::max(1, rblocks), 256, 0, ctx->stream>>>(sc->d_paths, (uint32_t)npix, (uint32_t)spp, cw, W, d_img);
  NE_CUDA(cudaGetLastError(), "k_reduce launch");
  if (!devOut) NE_CUDA(cudaMemcpyAsync(out_rgb, d_img, imgBytes, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync(image)");
  if (timed) NE_CUDA(cudaEventRecord(ctx->ev[3], ctx->stream), "cudaEventRecord");
  if (!timed) {
    if (stats) {
      memset(stats, 0, sizeof(*stats));
      stats->paths = total;
      stats->kernel_launches = (uint32_t)pathLaunches(sc, (flags & NE_RENDER_COUNT_WORK) != 0) + 1;
    }
    return NE_OK;
  }
  unsigned long long cnt[5] = {0, 0, 0, 0, 0};
  NE_CUDA(cudaMemcpyAsync(cnt, ctx->d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  st = checkErr(ctx);
  if (st) return st;
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    float kms = 0, tms = 0;
    cudaEventElapsedTime(&kms, ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&tms, ctx->ev[0], ctx->ev[3]);
    stats->kernel_ms = kms;
    stats->total_ms = tms;
    stats->paths = total;
    stats->density_lookups = cnt[1];
    stats->scene_queries = cnt[2];
    stats->bvh_nodes = cnt[3];
    stats->prim_tests = cnt[4];
    stats->kernel_launches = (uint32_t)pathLaunches(sc, (flags & NE_RENDER_COUNT_WORK) != 0) + 1;
  }
  return NE_OK;
}

ne_status ne_render_accumulate(ne_scene* sc, const ne_render_params* p, double* accum, ne_render_stats* stats) {
  if (!sc || !accum) return NE_ERR_INVALID_ARG;
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const int W = sc->settings.width, H = sc->settings.height;
  int spp = (p && p->spp > 0) ? p->spp : sc->settings.spp;
  if (spp <= 0) return fail(ctx, NE_ERR_INVALID_ARG, "spp must be positive");
  uint32_t flags = p ? p->flags : 0;
  uint32_t cw = (uint32_t)W, ch = (uint32_t)H;
  if (flags & NE_RENDER_REF_TILES) {
    cw = 40u * (uint32_t)(W / 40);
    ch = 10u * (uint32_t)(H / 10);
  }
  uint64_t npix = (uint64_t)cw * ch, total = npix * (uint64_t)spp;
  if (sc->paths_cap < total) {
    ctx->pool.put(sc->d_paths);
    sc->d_paths = nullptr;
    sc->paths_cap = 0;
    void* pp = nullptr;
    NE_CUDA(ctx->pool.get(total * 3 * sizeof(float), &pp), "cudaMalloc(paths)");
    sc->d_paths = (float*)pp;
    sc->paths_cap = total;
  }
  bool devAcc = flags & NE_RENDER_OUT_DEVICE;
  size_t accBytes = (size_t)W * H * 3 * sizeof(double);
  DevBuf<double> tmp;
  double* d_acc = accum;
  if (!devAcc) {
    NE_CUDA(cudaMalloc(&tmp.p, accBytes), "cudaMalloc(accum)");
    d_acc = tmp.p;
    NE_CUDA(cudaMemcpyAsync(d_acc, accum, accBytes, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  }
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(cudaEventRecord(ctx->ev[1], ctx->stream), "cudaEventRecord");
  PathArgs a;
  a.P = pathParams(sc, p);
  a.base = baseKey(p);
  a.total = total;
  a.spp = (uint32_t)spp;
  a.sample_offset = p ? p->sample_offset : 0;
  a.cover_w = cw;
  a.keys = nullptr;
  a.out = sc->d_paths;
  a.track_share = sc->track_share;
  ne_status st = launchPaths(sc, a, (flags & NE_RENDER_COUNT_WORK) != 0);
  if (st) return st;
  NE_CUDA(cudaEventRecord(ctx->ev[2], ctx->stream), "cudaEventRecord");
  int rblocks = (int)std::min<uint64_t>((npix + 255) / 256, (uint64_t)ctx->sm_count * 16);
  NE_CUDA(cudaMemsetAsync(ctx->d_counter + 5, 0, sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
  k_accum<<<std::max(1, rblocks), 256, 0, ctx->stream>>>(sc->d_paths, (uint32_t)npix, (uint32_t)spp, cw, W, d_acc,
                                                         (flags & NE_RENDER_DROP_NONFINITE) ? 1 : 0,
                                                         ctx->d_counter + 5);
  NE_CUDA(cudaGetLastError(), "k_accum launch");
  if (!devAcc) NE_CUDA(cudaMemcpyAsync(accum, d_acc, accBytes, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  unsigned long long cnt[6] = {0, 0, 0, 0, 0, 0};
  NE_CUDA(cudaMemcpyAsync(cnt, ctx->d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  st = checkErr(ctx);
  if (st) return st;
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    float kms = 0;
    cudaEventElapsedTime(&kms, ctx->ev[1], ctx->ev[2]);
    stats->kernel_ms = kms;
    stats->paths = total;
    stats->density_lookups = cnt[1];
    stats->scene_queries = cnt[2];
    stats->bvh_nodes = cnt[3];
    stats->prim_tests = cnt[4];
    stats->kernel_launches = (uint32_t)pathLaunches(sc, (flags & NE_RENDER_COUNT_WORK) != 0) + 1;
    stats->dropped_paths = (uint32_t)std::min<unsigned long long>(cnt[5], 0xFFFFFFFFull);
  }
  return NE_OK;
}

ne_status ne_trace_paths(ne_scene* sc, const ne_render_params* p, const ne_path_key* keys, size_t n, float* out_L) {
  if (!sc || (!keys && n) || (!out_L && n)) return NE_ERR_INVALID_ARG;
  if (n == 0) return NE_OK;
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  uint32_t npix = (uint32_t)sc->settings.width * (uint32_t)sc->settings.height;
  for (size_t i = 0; i < n; i++)
    if (keys[i].pixel >= npix) return fail(ctx, NE_ERR_INVALID_ARG, "path key pixel out of range");
  DevBuf<ne_path_key> dk;
  DevBuf<float> dout;
  NE_CUDA(cudaMalloc(&dk.p, n * sizeof(ne_path_key)), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dout.p, n * 3 * sizeof(float)), "cudaMalloc");
  NE_CUDA(cudaMemcpyAsync(dk.p, keys, n * sizeof(ne_path_key), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  PathArgs a;
  a.P = pathParams(sc, p);
  a.base = baseKey(p);
  a.total = n;
  a.spp = 1;
  a.sample_offset = p ? p->sample_offset : 0;
  a.cover_w = (uint32_t)sc->settings.width;
  a.keys = dk.p;
  a.out = dout.p;
  a.track_share = 16;
  ne_status st = launchPaths(sc, a, false);
  if (st) return st;
  NE_CUDA(cudaMemcpyAsync(out_L, dout.p, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  return checkErr(ctx);
}

ne_status ne_li_batch(ne_scene* sc, const ne_render_params* p, const ne_ray* rays, const ne_path_key* keys, size_t n,
                      uint32_t first_dim, float* out_L) {
  if (!sc || (n && (!rays || !keys || !out_L))) return NE_ERR_INVALID_ARG;
  if (n == 0) return NE_OK;
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  DevBuf<ne_ray> dr;
  DevBuf<ne_path_key> dk;
  DevBuf<float> dout;
  NE_CUDA(cudaMalloc(&dr.p, n * sizeof(ne_ray)), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dk.p, n * sizeof(ne_path_key)), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dout.p, n * 3 * sizeof(float)), "cudaMalloc");
  NE_CUDA(cudaMemcpyAsync(dr.p, rays, n * sizeof(ne_ray), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemcpyAsync(dk.p, keys, n * sizeof(ne_path_key), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  int blocks = (int)std::min<size_t>((n + kThreads - 1) / kThreads, (size_t)ctx->sm_count * 8);
  NE_CUDA(ne_launch_li(std::max(1, blocks), ctx->stream, sc->d, pathParams(sc, p), baseKey(p), dr.p, dk.p, n, first_dim,
                       dout.p, ctx->d_err),
          "k_li launch");
  NE_CUDA(cudaMemcpyAsync(out_L, dout.p, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  return checkErr(ctx);
}

ne_status ne_trace_closest(ne_scene* sc, const ne_ray* rays, size_t n, float t_min, float t_max, ne_hit* out) {
  if (!sc || (n && (!rays || !out))) return NE_ERR_INVALID_ARG;
  if (n == 0) return NE_OK;
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  DevBuf<ne_ray> dr;
  DevBuf<ne_hit> dh;
  NE_CUDA(cudaMalloc(&dr.p, n * sizeof(ne_ray)), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dh.p, n * sizeof(ne_hit)), "cudaMalloc");
  NE_CUDA(cudaMemcpyAsync(dr.p, rays, n * sizeof(ne_ray), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  int blocks = (int)std::min<size_t>((n + kThreads - 1) / kThreads, (size_t)ctx->sm_count * 8);
  NE_CUDA(ne_launch_closest(std::max(1, blocks), ctx->stream, sc->d, dr.p, n, t_min, t_max, dh.p, ctx->d_err),
          "k_closest launch");
  NE_CUDA(cudaMemcpyAsync(out, dh.p, n * sizeof(ne_hit), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  return checkErr(ctx);
}

ne_status ne_context_event_record(ne_context* ctx, int slot) {
  if (!ctx || slot < 0 || slot >= 8) return NE_ERR_INVALID_ARG;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (!ctx->user_ev[slot]) NE_CUDA(cudaEventCreate(&ctx->user_ev[slot]), "cudaEventCreate");
  NE_CUDA(cudaEventRecord(ctx->user_ev[slot], ctx->stream), "cudaEventRecord");
  return NE_OK;
}

ne_status ne_context_event_elapsed(ne_context* ctx, int a, int b, float* ms) {
  if (!ctx || !ms || a < 0 || a >= 8 || b < 0 || b >= 8 || !ctx->user_ev[a] || !ctx->user_ev[b]) return NE_ERR_INVALID_ARG;
  NE_CUDA(cudaEventSynchronize(ctx->user_ev[b]), "cudaEventSynchronize");
  NE_CUDA(cudaEventElapsedTime(ms, ctx->user_ev[a], ctx->user_ev[b]), "cudaEventElapsedTime");
  return NE_OK;
}

ne_status ne_context_synchronize(ne_context* ctx) {
  if (!ctx) return NE_ERR_INVALID_ARG;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  return NE_OK;
}

ne_status ne_context_flush_l2(ne_context* ctx, size_t bytes) {
  if (!ctx || bytes == 0) return NE_ERR_INVALID_ARG;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (ctx->flush_bytes < bytes) {
    if (ctx->flush_buf) cudaFree(ctx->flush_buf);
    ctx->flush_buf = nullptr;
    ctx->flush_bytes = 0;
    NE_CUDA(cudaMalloc(&ctx->flush_buf, bytes), "cudaMalloc(flush)");
    ctx->flush_bytes = bytes;
  }
  NE_CUDA(cudaMemsetAsync(ctx->flush_buf, (int)(bytes & 0xff), bytes, ctx->stream), "cudaMemsetAsync(flush)");
  return NE_OK;
}

ne_status ne_measure_read_bandwidth(ne_context* ctx, size_t bytes, int iters, double* gbs) {
  if (!ctx || !gbs || bytes < 16 || iters <= 0) return NE_ERR_INVALID_ARG;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  size_t n = bytes / 16;
  DevBuf<uint4> buf;
  DevBuf<uint32_t> sink;
  NE_CUDA(cudaMalloc(&buf.p, n * 16), "cudaMalloc(read probe)");
  NE_CUDA(cudaMalloc(&sink.p, 4), "cudaMalloc(read probe)");
  NE_CUDA(cudaMemsetAsync(buf.p, 0x5a, n * 16, ctx->stream), "cudaMemsetAsync(read probe)");
  int per_sm = 0;
  NE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_read_bw, 512, 0), "occupancy");
  int blocks = ctx->sm_count * std::max(1, per_sm);
  // passes per launch: at least 1 GiB read per launch, so launch gaps do not count
  int reps = (int)std::max<size_t>(1, std::min<size_t>(1024, ((size_t)1 << 30) / (n * 16)));
  k_read_bw<<<blocks, 512, 0, ctx->stream>>>(buf.p, n, 1, sink.p);  // warm-up: brings the buffer into L2
  NE_CUDA(cudaGetLastError(), "k_read_bw launch");
  NE_CUDA(cudaEventRecord(ctx->ev[0], ctx->stream), "cudaEventRecord");
  for (int k = 0; k < iters; k++) k_read_bw<<<blocks, 512, 0, ctx->stream>>>(buf.p, n, reps, sink.p);
  NE_CUDA(cudaGetLastError(), "k_read_bw launch");
  NE_CUDA(cudaEventRecord(ctx->ev[1], ctx->stream), "cudaEventRecord");
  NE_CUDA(cudaEventSynchronize(ctx->ev[1]), "cudaEventSynchronize");
  float ms = 0;
  NE_CUDA(cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]), "cudaEventElapsedTime");
  *gbs = (double)n * 16 * reps * iters / (ms / 1e3) / 1e9;
  return NE_OK;
}

ne_status ne_measure_random_read(ne_context* ctx, size_t bytes, int iters, double* reads_per_s) {
  if (!ctx || !reads_per_s || bytes < 32 || bytes / 32 > 0xffffffffull || iters <= 0) return NE_ERR_INVALID_ARG;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const uint32_t nrec = (uint32_t)(bytes / 32);
  DevBuf<float4> buf;
  DevBuf<uint32_t> sink;
  NE_CUDA(cudaMalloc(&buf.p, (size_t)nrec * 32), "cudaMalloc(read probe)");
  NE_CUDA(cudaMalloc(&sink.p, 4), "cudaMalloc(read probe)");
  NE_CUDA(cudaMemsetAsync(buf.p, 0, (size_t)nrec * 32, ctx->stream), "cudaMemsetAsync(read probe)");
  // the best of 2, 4, 8 and 16 independent reads in flight per thread
  double r[4] = {0, 0, 0, 0};
  NE_CUDA(randomReadRate<2>(ctx, buf.p, nrec, iters, sink.p, &r[0]), "k_random_read");
  NE_CUDA(randomReadRate<4>(ctx, buf.p, nrec, iters, sink.p, &r[1]), "k_random_read");
  NE_CUDA(randomReadRate<8>(ctx, buf.p, nrec, iters, sink.p, &r[2]), "k_random_read");
  NE_CUDA(randomReadRate<16>(ctx, buf.p, nrec, iters, sink.p, &r[3]), "k_random_read");
  *reads_per_s = std::max(std::max(r[0], r[1]), std::max(r[2], r[3]));
  return NE_OK;
}

ne_status ne_debug_fmath(ne_context* ctx, int fn, const float* x, size_t n, float* out) {
  if (!ctx || (n && (!x || !out))) return NE_ERR_INVALID_ARG;
  if (n == 0) return NE_OK;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  DevBuf<float> dx, dy;
  NE_CUDA(cudaMalloc(&dx.p, n * 4), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dy.p, n * 4), "cudaMalloc");
  NE_CUDA(cudaMemcpyAsync(dx.p, x, n * 4, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx->sm_count * 8);
  k_fmath<<<std::max(1, blocks), 256, 0, ctx->stream>>>(fn, dx.p, n, dy.p);
  NE_CUDA(cudaGetLastError(), "k_fmath launch");
  NE_CUDA(cudaMemcpyAsync(out, dy.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  return NE_OK;
}

ne_status ne_debug_rng(ne_context* ctx, uint64_t seed, const ne_path_key* keys, const uint32_t* dims, size_t n,
                       float* out) {
  if (!ctx || (n && (!keys || !dims || !out))) return NE_ERR_INVALID_ARG;
  if (n == 0) return NE_OK;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  DevBuf<ne_path_key> dk;
  DevBuf<uint32_t> dd;
  DevBuf<float> dy;
  NE_CUDA(cudaMalloc(&dk.p, n * sizeof(ne_path_key)), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dd.p, n * 4), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dy.p, n * 4), "cudaMalloc");
  NE_CUDA(cudaMemcpyAsync(dk.p, keys, n * sizeof(ne_path_key), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemcpyAsync(dd.p, dims, n * 4, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  ne_render_params p;
  memset(&p, 0, sizeof(p));
  p.seed = seed;
  int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx->sm_count * 8);
  k_rng<<<std::max(1, blocks), 256, 0, ctx->stream>>>(baseKey(&p), dk.p, dd.p, n, dy.p);
  NE_CUDA(cudaGetLastError(), "k_rng launch");
  NE_CUDA(cudaMemcpyAsync(out, dy.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  return NE_OK;
}

ne_status ne_render_noalloc(ne_scene* sc, const ne_render_params* p, float* out_rgb_device, ne_render_stats* stats) {
  if (!sc || !out_rgb_device) return NE_ERR_INVALID_ARG;
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const int W = sc->settings.width, H = sc->settings.height;
  int spp = (p && p->spp > 0) ? p->spp : sc->settings.spp;
  if (spp <= 0) return fail(ctx, NE_ERR_INVALID_ARG, "spp must be positive");
  uint32_t flags = p ? p->flags : 0;
  uint32_t cw = (uint32_t)W, ch = (uint32_t)H;
  if (flags & NE_RENDER_REF_TILES) {
    cw = 40u * (uint32_t)(W / 40);
    ch = 10u * (uint32_t)(H / 10);
  }
  uint64_t npix = (uint64_t)cw * ch;
  uint64_t total = npix * (uint64_t)spp;
  if (total > kNoAllocMaxPaths)
    return fail(ctx, NE_ERR_INVALID_ARG,
                "ne_render_noalloc: " + std::to_string(total) + " paths (pixels x spp) exceed its scratch of " +
                    std::to_string(kNoAllocMaxPaths) + " paths; render fewer samples per call");
  unsigned char* scratch = nullptr;
  ne_status st = noallocScratch(ctx, &scratch);
  if (st) return st;
  unsigned long long* d_counter = (unsigned long long*)scratch;
  uint32_t* d_err = (uint32_t*)(scratch + 8 * sizeof(unsigned long long));
  float* d_paths = (float*)(scratch + kNoAllocHeaderBytes);
  NE_CUDA(cudaMemsetAsync(scratch, 0, kNoAllocHeaderBytes, ctx->stream), "cudaMemsetAsync");
  size_t imgBytes = (size_t)W * H * 3 * sizeof(float);
  NE_CUDA(cudaEventRecord(ctx->ev[0], ctx->stream), "cudaEventRecord");
  if (cw != (uint32_t)W || ch != (uint32_t)H)
    NE_CUDA(cudaMemsetAsync(out_rgb_device, 0, imgBytes, ctx->stream), "cudaMemsetAsync");
  PathArgs a;
  a.P = pathParams(sc, p);
  a.base = baseKey(p);
  a.total = total;
  a.spp = (uint32_t)spp;
  a.sample_offset = p ? p->sample_offset : 0;
  a.cover_w = cw;
  a.keys = nullptr;
  a.out = d_paths;
  a.track_share = sc->track_share;
  // The split kernel (tuning kernel 3) needs deferred-path queues sized to the render, which
  // the fixed array does not hold: a scene tuned to it renders with the one-pass kernel
  // (kernel 0), at that kernel's own occupancy. Kernels 0-2 run as tuned.
  const bool count = (flags & NE_RENDER_COUNT_WORK) != 0;
  const int kernel = sc->variant == 3 ? 0 : sc->variant;
  int blocks = persistentBlocks(sc);
  if (sc->variant == 3 && !count) {
    int fit = 0;
    NE_CUDA(ne_path_kernel_occupancy(0, sc->feature_set, &fit), "occupancy query");
    blocks = ctx->sm_count * std::max(1, fit);
  }
  unsigned long long needed = (total + kThreads - 1) / kThreads;
  if ((unsigned long long)blocks > needed) blocks = (int)std::max<unsigned long long>(1, needed);
  NE_CUDA(cudaEventRecord(ctx->ev[1], ctx->stream), "cudaEventRecord");
  NE_CUDA(ne_launch_path_kernel(kernel, sc->feature_set, count, blocks, ctx->stream, sc->d, a, d_counter, d_err),
          "path kernel launch");
  NE_CUDA(cudaEventRecord(ctx->ev[2], ctx->stream), "cudaEventRecord");
  int rblocks = (int)std::min<uint64_t>((npix + 255) / 256, (uint64_t)ctx->sm_count * 16);
  k_reduce<<<std::max(1, rblocks), 256, 0, ctx->stream>>>(d_paths, (uint32_t)npix, (uint32_t)spp, cw, W,
                                                          out_rgb_device);
  NE_CUDA(cudaGetLastError(), "k_reduce launch");
  NE_CUDA(cudaEventRecord(ctx->ev[3], ctx->stream), "cudaEventRecord");
  unsigned long long cnt[5] = {0, 0, 0, 0, 0};
  uint32_t e = 0;
  NE_CUDA(cudaMemcpyAsync(cnt, d_counter, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemcpyAsync(&e, d_err, 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync(err)");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (e & ERR_BVH_STACK) return fail(ctx, NE_ERR_UNSUPPORTED, "BVH traversal stack exceeded 64 entries");
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    float kms = 0, tms = 0;
    cudaEventElapsedTime(&kms, ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&tms, ctx->ev[0], ctx->ev[3]);
    stats->kernel_ms = kms;
    stats->total_ms = tms;
    stats->paths = total;
    stats->density_lookups = cnt[1];
    stats->scene_queries = cnt[2];
    stats->bvh_nodes = cnt[3];
    stats->prim_tests = cnt[4];
    stats->kernel_launches = 2;
  }
  return NE_OK;
}

ne_status ne_debug_mma(ne_context* ctx, const uint16_t* a, const uint16_t* b, int n, int k, float* d) {
  if (!ctx || !a || !b || !d) return NE_ERR_INVALID_ARG;
  if (n < 16 || n > 256 || n % 16 || k < 16 || k > 128 || k % 16)
    return fail(ctx, NE_ERR_INVALID_ARG, "ne_debug_mma: n must be 16..256 and k 16..128, multiples of 16");
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  DevBuf<uint16_t> da, db;
  DevBuf<float> dd;
  NE_CUDA(cudaMalloc(&da.p, (size_t)128 * k * 2), "cudaMalloc");
  NE_CUDA(cudaMalloc(&db.p, (size_t)n * k * 2), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dd.p, (size_t)128 * n * 4), "cudaMalloc");
  NE_CUDA(cudaMemcpyAsync(da.p, a, (size_t)128 * k * 2, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemcpyAsync(db.p, b, (size_t)n * k * 2, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(ne_launch_debug_mma(ctx->stream, da.p, db.p, n, k, dd.p, ctx->d_err), "k_debug_mma launch");
  NE_CUDA(cudaMemcpyAsync(d, dd.p, (size_t)128 * n * 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  uint32_t e = 0;
  NE_CUDA(cudaMemcpyAsync(&e, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (e) return fail(ctx, NE_ERR_TIMEOUT, "tensor-core product did not complete");
  return NE_OK;
}

ne_status ne_debug_mma_layout(ne_context* ctx, const uint16_t* a, const uint16_t* b, int n, int k, uint32_t layout,
                              float* d) {
  if (!ctx || !a || !b || !d) return NE_ERR_INVALID_ARG;
  if (n < 16 || n > 64 || n % 16 || k < 16 || k > 64 || k % 16 || layout > 3)
    return fail(ctx, NE_ERR_INVALID_ARG, "ne_debug_mma_layout: n and k must be 16..64, multiples of 16");
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  DevBuf<uint16_t> da, db;
  DevBuf<float> dd;
  NE_CUDA(cudaMalloc(&da.p, (size_t)128 * k * 2), "cudaMalloc");
  NE_CUDA(cudaMalloc(&db.p, (size_t)n * k * 2), "cudaMalloc");
  NE_CUDA(cudaMalloc(&dd.p, (size_t)128 * n * 4), "cudaMalloc");
  NE_CUDA(cudaMemcpyAsync(da.p, a, (size_t)128 * k * 2, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemcpyAsync(db.p, b, (size_t)n * k * 2, cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(ne_launch_debug_mma_mn(ctx->stream, da.p, db.p, n, k, layout, dd.p, ctx->d_err), "k_debug_mma_mn launch");
  NE_CUDA(cudaMemcpyAsync(d, dd.p, (size_t)128 * n * 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  uint32_t e = 0;
  NE_CUDA(cudaMemcpyAsync(&e, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (e) return fail(ctx, NE_ERR_TIMEOUT, "tensor-core product did not complete");
  return NE_OK;
}

ne_status ne_debug_wait_timeout(ne_context* ctx, uint32_t max_polls) {
  if (!ctx || max_polls == 0 || max_polls > (1u << 20)) return NE_ERR_INVALID_ARG;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(ne_launch_debug_wait(ctx->stream, max_polls, ctx->d_err), "k_debug_wait launch");
  uint32_t e = 0;
  NE_CUDA(cudaMemcpyAsync(&e, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  if (e) return fail(ctx, NE_ERR_TIMEOUT, "tensor-core wait gave up after " + std::to_string(max_polls) + " polls");
  return NE_OK;
}

ne_status ne_cache_create(ne_context* ctx, uint64_t seed, ne_cache** out) {
  if (!ctx || !out) return NE_ERR_INVALID_ARG;
  *out = nullptr;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  ne_cache* c = new ne_cache();
  c->ctx = ctx;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&c->P, kNeMlpParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->m, kNeMlpParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->v, kNeMlpParams * 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->wfwd, kNeMlpFwdBytes);
  if (e == cudaSuccess) e = cudaMalloc(&c->wbwd, kNeMlpBwdBytes);
  if (e == cudaSuccess) e = cudaMalloc(&c->bias, kNeMlpBiasFloats * 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_loss, 4);
  if (e == cudaSuccess) e = cudaMalloc(&c->grad, kNeMlpParams * 4);
  ctx->caches.push_back(c);
  if (e != cudaSuccess) {
    ne_cache_destroy(c);
    return fail(ctx, NE_ERR_OUT_OF_MEMORY, std::string("radiance cache: ") + cudaGetErrorString(e));
  }
  std::vector<float> P;
  cacheInitParams(seed, P);
  ne_status st = cacheUpload(c, P.data());
  if (st) {
    ne_cache_destroy(c);
    return st;
  }
  *out = c;
  return NE_OK;
}

void ne_cache_destroy(ne_cache* c) {
  if (!c) return;
  auto& v = c->ctx->caches;
  v.erase(std::remove(v.begin(), v.end(), c), v.end());
  cudaSetDevice(c->ctx->device);
  cudaStreamSynchronize(c->ctx->stream);
  void* bufs[] = {c->P, c->m, c->v, c->wfwd, c->wbwd, c->bias, c->part, c->loss_part, c->d_loss, c->grad, c->acts,
                  c->out, c->q, c->q_idx, c->tr, c->tq, c->tq_idx, c->counts, c->d_io};
  for (void* p : bufs)
    if (p) cudaFree(p);
  for (cudaEvent_t e : c->ev)
    if (e) cudaEventDestroy(e);
  delete c;
}

ne_status ne_cache_set_params(ne_cache* c, const float* params) {
  if (!c || !params) return NE_ERR_INVALID_ARG;
  ne_context* ctx = c->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  return cacheUpload(c, params);
}

ne_status ne_cache_get_params(ne_cache* c, float* params) {
  if (!c || !params) return NE_ERR_INVALID_ARG;
  ne_context* ctx = c->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  NE_CUDA(cudaMemcpyAsync(params, c->P, kNeMlpParams * 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  return NE_OK;
}

ne_status ne_cache_encode(ne_cache* c, const float* pos, const float* dirs, size_t n, float* feats) {
  if (!c || (n && (!pos || !dirs || !feats))) return NE_ERR_INVALID_ARG;
  if (n == 0) return NE_OK;
  ne_context* ctx = c->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  DevBuf<float> tp, td, tf;
  const float *dp, *dd;
  ne_status st = stageIn(ctx, pos, n * 3, false, tp, &dp);
  if (!st) st = stageIn(ctx, dirs, n * 3, false, td, &dd);
  if (st) return st;
  NE_CUDA(cudaMalloc(&tf.p, n * 96 * 4), "cudaMalloc");
  NE_CUDA(ne_mlp_encode(ctx->stream, dp, dd, (uint32_t)n, tf.p), "k_mlp_encode launch");
  NE_CUDA(cudaMemcpyAsync(feats, tf.p, n * 96 * 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  return NE_OK;
}

ne_status ne_cache_infer(ne_cache* c, const float* pos, const float* dirs, const float* feats, size_t n, float* rgb,
                         uint32_t flags) {
  if (!c || !rgb || (n && !feats && (!pos || !dirs))) return NE_ERR_INVALID_ARG;
  if (n == 0) return NE_OK;
  if (n > 0xFFFFFF80u) return fail(c->ctx, NE_ERR_INVALID_ARG, "radiance cache: too many queries");
  ne_context* ctx = c->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  bool dev = flags & NE_CACHE_DEVICE_PTRS;
  DevBuf<float> tp, td, tf, to;
  const float *dp = nullptr, *dd = nullptr, *df = nullptr;
  ne_status st = NE_OK;
  if (feats) st = stageIn(ctx, feats, n * 96, dev, tf, &df);
  else {
    st = stageIn(ctx, pos, n * 3, dev, tp, &dp);
    if (!st) st = stageIn(ctx, dirs, n * 3, dev, td, &dd);
  }
  if (st) return st;
  float* dout = rgb;
  if (!dev) {
    NE_CUDA(cudaMalloc(&to.p, n * 3 * 4), "cudaMalloc");
    dout = to.p;
  }
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  NeMlpForward f = {dp, dd, df, (uint32_t)n, nullptr, c->wfwd, c->bias, dout, nullptr, nullptr, nullptr, nullptr};
  NE_CUDA(ne_mlp_forward(ctx->stream, f, ctx->d_err), "k_mlp_forward launch");
  if (!dev) NE_CUDA(cudaMemcpyAsync(rgb, dout, n * 3 * 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  return cacheErr(ctx);
}

// One optimiser step on device arrays (pos/dir or features, targets).
static ne_status cacheTrainDevice(ne_cache* c, const float* dp, const float* dd, const float* df, const float* dt,
                                  size_t n, int apply, bool wantGrads) {
  ne_context* ctx = c->ctx;
  if (c->cap < n) {
    if (c->acts) cudaFree(c->acts);
    if (c->out) cudaFree(c->out);
    c->acts = nullptr;
    c->out = nullptr;
    c->cap = 0;
    NE_CUDA(cudaMalloc(&c->acts, (n + 127) / 128 * (size_t)kNeMlpActTileBytes), "cudaMalloc(activations)");
    NE_CUDA(cudaMalloc(&c->out, n * 3 * 4), "cudaMalloc(outputs)");
    c->cap = n;
  }
  int blocks = ne_mlp_backward_blocks((uint32_t)n);
  if (c->part_blocks < blocks) {
    if (c->part) cudaFree(c->part);
    if (c->loss_part) cudaFree(c->loss_part);
    c->part = nullptr;
    c->loss_part = nullptr;
    c->part_blocks = 0;
    NE_CUDA(cudaMalloc(&c->part, (size_t)blocks * kNeMlpParams * 4), "cudaMalloc(partial gradients)");
    NE_CUDA(cudaMalloc(&c->loss_part, (size_t)blocks * 4), "cudaMalloc");
    c->part_blocks = blocks;
  }
  NeMlpForward f = {dp, dd, df, (uint32_t)n, nullptr, c->wfwd, c->bias, c->out, c->acts, nullptr, nullptr, nullptr};
  NE_CUDA(ne_mlp_forward(ctx->stream, f, ctx->d_err), "k_mlp_forward launch");
  NeMlpBackward b = {c->acts, c->out, dt, (uint32_t)n, c->wbwd, c->part, c->loss_part};
  NE_CUDA(ne_mlp_backward(ctx->stream, b, ctx->d_err), "k_mlp_backward launch");
  if (apply) c->step++;
  NE_CUDA(ne_mlp_adam(ctx->stream, c->P, c->m, c->v, c->part, blocks, c->loss_part, wantGrads ? c->grad : nullptr,
                      c->d_loss, 1e-2f, apply ? c->step : 1, apply, apply ? c->wfwd : nullptr, c->wbwd, c->bias),
          "k_mlp_adam launch");
  return NE_OK;
}

ne_status ne_cache_train(ne_cache* c, const float* pos, const float* dirs, const float* feats, const float* targets,
                         size_t n, int apply, float* loss, float* grads, uint32_t flags) {
  if (!c || !targets || n == 0 || (!feats && (!pos || !dirs))) return NE_ERR_INVALID_ARG;
  if (n > (1u << 24)) return fail(c->ctx, NE_ERR_INVALID_ARG, "radiance cache: at most 2^24 samples per step");
  ne_context* ctx = c->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  bool dev = flags & NE_CACHE_DEVICE_PTRS;
  DevBuf<float> tp, td, tf, tt;
  const float *dp = nullptr, *dd = nullptr, *df = nullptr, *dt = nullptr;
  ne_status st = NE_OK;
  if (feats) st = stageIn(ctx, feats, n * 96, dev, tf, &df);
  else {
    st = stageIn(ctx, pos, n * 3, dev, tp, &dp);
    if (!st) st = stageIn(ctx, dirs, n * 3, dev, td, &dd);
  }
  if (!st) st = stageIn(ctx, targets, n * 3, dev, tt, &dt);
  if (st) return st;
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  st = cacheTrainDevice(c, dp, dd, df, dt, n, apply, grads != nullptr);
  if (st) return st;
  float lsum = 0;
  NE_CUDA(cudaMemcpyAsync(&lsum, c->d_loss, 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  if (grads)
    NE_CUDA(cudaMemcpyAsync(grads, c->grad, kNeMlpParams * 4, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            ctx->stream),
            "cudaMemcpyAsync");
  st = cacheErr(ctx);
  if (st) return st;
  if (loss) *loss = lsum / (3.0f * (float)n);
  return NE_OK;
}

ne_status ne_render_cached(ne_scene* sc, ne_cache* c, const ne_render_params* p, const ne_cache_render_params* cp,
                           float* out_rgb, ne_render_stats* stats, ne_cache_render_stats* cstats) {
  if (!sc || !c || !cp || !out_rgb || c->ctx != sc->ctx) return NE_ERR_INVALID_ARG;
  ne_context* ctx = sc->ctx;
  if (sc->feature_set != K_VOLUME || !(sc->features & FT_GRID))
    return fail(ctx, NE_ERR_UNSUPPORTED, "ne_render_cached: the scene's media must be grid media");
  if (cp->bounce < 0 || cp->train_steps < 0 || cp->train_suffix < 0)
    return fail(ctx, NE_ERR_INVALID_ARG, "ne_render_cached: bad parameters");
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const int W = sc->settings.width, H = sc->settings.height;
  int spp = (p && p->spp > 0) ? p->spp : sc->settings.spp;
  if (spp <= 0) return fail(ctx, NE_ERR_INVALID_ARG, "spp must be positive");
  uint32_t flags = p ? p->flags : 0;
  uint32_t cw = (uint32_t)W, ch = (uint32_t)H;
  if (flags & NE_RENDER_REF_TILES) {
    cw = 40u * (uint32_t)(W / 40);
    ch = 10u * (uint32_t)(H / 10);
  }
  uint64_t npix = (uint64_t)cw * ch, total = npix * (uint64_t)spp;
  if (total > 0xFFFFFFFFull) return fail(ctx, NE_ERR_INVALID_ARG, "ne_render_cached: at most 2^32 paths per call");
  if (sc->paths_cap < total) {
    ctx->pool.put(sc->d_paths);
    sc->d_paths = nullptr;
    sc->paths_cap = 0;
    void* pp = nullptr;
    NE_CUDA(ctx->pool.get(total * 3 * sizeof(float), &pp), "cudaMalloc(paths)");
    sc->d_paths = (float*)pp;
    sc->paths_cap = total;
  }
  size_t tcap = cp->train_stride ? (size_t)std::min<uint64_t>(total, total / cp->train_stride * 2 + 4096) : 1;
  if (c->q_cap < total) {
    if (c->q) cudaFree(c->q);
    if (c->q_idx) cudaFree(c->q_idx);
    c->q = nullptr;
    c->q_idx = nullptr;
    c->q_cap = 0;
    NE_CUDA(cudaMalloc(&c->q, total * 9 * sizeof(float)), "cudaMalloc(cache queries)");
    NE_CUDA(cudaMalloc(&c->q_idx, total * sizeof(uint32_t)), "cudaMalloc(cache queries)");
    c->q_cap = total;
  }
  if (c->t_cap < tcap) {
    void* bufs[] = {c->tr, c->tq, c->tq_idx};
    for (void* b : bufs)
      if (b) cudaFree(b);
    c->tr = c->tq = nullptr;
    c->tq_idx = nullptr;
    c->t_cap = 0;
    NE_CUDA(cudaMalloc(&c->tr, tcap * 9 * sizeof(float)), "cudaMalloc(training samples)");
    NE_CUDA(cudaMalloc(&c->tq, tcap * 9 * sizeof(float)), "cudaMalloc(training end queries)");
    NE_CUDA(cudaMalloc(&c->tq_idx, tcap * sizeof(uint32_t)), "cudaMalloc(training end queries)");
    c->t_cap = tcap;
  }
  if (!c->counts) NE_CUDA(cudaMalloc(&c->counts, 3 * sizeof(uint32_t)), "cudaMalloc");
  if (!c->d_io) NE_CUDA(cudaMalloc(&c->d_io, sizeof(CacheIO)), "cudaMalloc");
  for (cudaEvent_t& e : c->ev)
    if (!e) NE_CUDA(cudaEventCreate(&e), "cudaEventCreate");
  CacheIO& io = c->io;
  io.q_pos = c->q;
  io.q_dir = c->q + 3 * c->q_cap;
  io.q_thr = c->q + 6 * c->q_cap;
  io.q_idx = c->q_idx;
  io.q_count = c->counts;
  io.q_cap = (uint32_t)c->q_cap;
  io.t_pos = c->tr;
  io.t_dir = c->tr + 3 * c->t_cap;
  io.t_val = c->tr + 6 * c->t_cap;
  io.t_count = c->counts + 1;
  io.t_cap = (uint32_t)c->t_cap;
  io.train_stride = cp->train_stride;
  io.bounce = cp->bounce;
  io.train_suffix = cp->train_suffix;
  io.tq_pos = c->tq;
  io.tq_dir = c->tq + 3 * c->t_cap;
  io.tq_thr = c->tq + 6 * c->t_cap;
  io.tq_idx = c->tq_idx;
  io.tq_count = c->counts + 2;
  NE_CUDA(cudaMemcpyAsync(c->d_io, &io, sizeof(CacheIO), cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaMemsetAsync(c->counts, 0, 3 * sizeof(uint32_t), ctx->stream), "cudaMemsetAsync");
  NE_CUDA(cudaMemsetAsync(ctx->d_err, 0, 4, ctx->stream), "cudaMemsetAsync");
  NE_CUDA(cudaMemsetAsync(ctx->d_counter, 0, 5 * sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
  bool devOut = flags & NE_RENDER_OUT_DEVICE;
  size_t imgBytes = (size_t)W * H * 3 * sizeof(float);
  PoolBuf tmpImg;
  float* d_img = out_rgb;
  if (!devOut) {
    NE_CUDA(tmpImg.get(ctx->pool, imgBytes), "cudaMalloc(image)");
    d_img = (float*)tmpImg.p;
  }
  NE_CUDA(cudaEventRecord(c->ev[0], ctx->stream), "cudaEventRecord");
  if (cw != (uint32_t)W || ch != (uint32_t)H) NE_CUDA(cudaMemsetAsync(d_img, 0, imgBytes, ctx->stream), "cudaMemsetAsync");
  PathArgs a;
  a.P = pathParams(sc, p);
  a.base = baseKey(p);
  a.total = total;
  a.spp = (uint32_t)spp;
  a.sample_offset = p ? p->sample_offset : 0;
  a.cover_w = cw;
  a.keys = nullptr;
  a.out = sc->d_paths;
  a.track_share = sc->track_share;
  a.cache = c->d_io;
  int fit = 1;
  NE_CUDA(ne_path_cache_occupancy(&fit), "occupancy query");
  int blocks = ctx->sm_count * std::max(1, fit);
  unsigned long long needed = (total + kThreads - 1) / kThreads;
  if ((unsigned long long)blocks > needed) blocks = (int)std::max<unsigned long long>(1, needed);
  {
    ne_status sst = launchSplit(sc, a, blocks, [&](int pass, int nb, const PathArgs& pa, unsigned long long* ctr) {
      return ne_launch_path_kernel_cache(pass, pass ? ctx->sm_count * std::max(1, fit) : nb, ctx->stream, sc->d, pa,
                                         ctr, ctx->d_err);
    });
    if (sst) return sst;
  }
  NE_CUDA(cudaEventRecord(c->ev[1], ctx->stream), "cudaEventRecord");
  // the network answers however many queries the path kernel appended (count read on the device)
  NeMlpForward f = {io.q_pos, io.q_dir, nullptr, io.q_cap, c->counts, c->wfwd, c->bias, nullptr, nullptr, io.q_thr,
                    io.q_idx, sc->d_paths};
  NE_CUDA(ne_mlp_forward(ctx->stream, f, ctx->d_err), "k_mlp_forward launch");
  if (cp->train_suffix > 0 && cp->train_stride) {
    // the training paths' end vertices: their answers complete the training targets
    NeMlpForward ft = {io.tq_pos, io.tq_dir, nullptr, io.t_cap, c->counts + 2, c->wfwd, c->bias, nullptr, nullptr,
                       io.tq_thr, io.tq_idx, io.t_val};
    NE_CUDA(ne_mlp_forward(ctx->stream, ft, ctx->d_err), "k_mlp_forward launch");
  }
  int rblocks = (int)std::min<uint64_t>((npix + 255) / 256, (uint64_t)ctx->sm_count * 16);
  k_reduce<<<std::max(1, rblocks), 256, 0, ctx->stream>>>(sc->d_paths, (uint32_t)npix, (uint32_t)spp, cw, W, d_img);
  NE_CUDA(cudaGetLastError(), "k_reduce launch");
  if (!devOut) NE_CUDA(cudaMemcpyAsync(out_rgb, d_img, imgBytes, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaEventRecord(c->ev[2], ctx->stream), "cudaEventRecord");
  uint32_t counts[2] = {0, 0};
  NE_CUDA(cudaMemcpyAsync(counts, c->counts, sizeof(counts), cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  uint32_t nq = std::min<uint32_t>(counts[0], io.q_cap), nt = std::min<uint32_t>(counts[1], io.t_cap);
  float loss = 0;
  int launches = 3;
  if (cp->train_steps > 0 && nt > 0) {
    uint32_t batch = cp->train_batch ? std::min<uint32_t>(cp->train_batch, nt) : nt;
    uint32_t off = 0;
    for (int s = 0; s < cp->train_steps; s++) {
      if (off + batch > nt) off = 0;
      ne_status st = cacheTrainDevice(c, io.t_pos + 3 * (size_t)off, io.t_dir + 3 * (size_t)off, nullptr,
                                      io.t_val + 3 * (size_t)off, batch, 1, false);
      if (st) return st;
      off += batch;
      launches += 4;
    }
    float lsum = 0;
    NE_CUDA(cudaMemcpyAsync(&lsum, c->d_loss, 4, cudaMemcpyDeviceToHost, ctx->stream), "cudaMemcpyAsync");
    NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    loss = lsum / (3.0f * (float)batch);
  }
  NE_CUDA(cudaEventRecord(c->ev[3], ctx->stream), "cudaEventRecord");
  ne_status st = checkErr(ctx);
  if (st) return st;
  st = cacheErr(ctx);
  if (st) return st;
  float pms = 0, ims = 0, tms = 0;
  cudaEventElapsedTime(&pms, c->ev[0], c->ev[1]);
  cudaEventElapsedTime(&ims, c->ev[1], c->ev[2]);
  cudaEventElapsedTime(&tms, c->ev[2], c->ev[3]);
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->kernel_ms = pms;
    stats->total_ms = pms + ims + tms;
    stats->paths = total;
    stats->kernel_launches = (uint32_t)launches;
  }
  if (cstats) {
    cstats->queries = nq;
    cstats->train_samples = nt;
    cstats->loss = loss;
    cstats->path_ms = pms;
    cstats->infer_ms = ims;
    cstats->train_ms = tms;
  }
  return NE_OK;
}

ne_status ne_views_create(ne_scene* sc, const ne_view* views, uint32_t n, const ne_render_params* p, ne_views** out) {
  if (!sc || !views || !out || n == 0) return NE_ERR_INVALID_ARG;
  *out = nullptr;
  ne_context* ctx = sc->ctx;
  uint64_t total = 0, pixels = 0;
  for (uint32_t i = 0; i < n; i++) {
    if (views[i].width <= 0 || views[i].height <= 0 || views[i].spp <= 0)
      return fail(ctx, NE_ERR_INVALID_ARG, "ne_views_create: every view needs a positive size and spp");
    total += (uint64_t)views[i].width * views[i].height * views[i].spp;
    pixels += (uint64_t)views[i].width * views[i].height;
  }
  if (pixels > 0xFFFFFFFFull) return fail(ctx, NE_ERR_INVALID_ARG, "ne_views_create: too many pixels");
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  ne_views* vw = new ne_views();
  vw->sc = sc;
  vw->views.assign(views, views + n);
  vw->total = total;
  vw->total_pixels = (uint32_t)pixels;
  vw->P = pathParams(sc, p);
  vw->base = baseKey(p);
  vw->latency.assign(n, 0.0f);
  sc->view_batches.push_back(vw);
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&vw->d_views, n * sizeof(DView));
  if (e == cudaSuccess) e = cudaMalloc(&vw->d_paths, total * 3 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&vw->d_img, pixels * 3 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&vw->d_done, (2 * (size_t)n + 2) * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaEventCreate(&vw->ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&vw->ev[1]);
  vw->defer_cap = std::max<size_t>(1024, (size_t)(total / 2));
  for (PathState*& q : vw->d_defer)
    if (e == cudaSuccess) e = cudaMalloc(&q, vw->defer_cap * sizeof(PathState));
  if (e == cudaSuccess) e = cudaMalloc(&vw->d_dq, 2 * sizeof(DeferQueue));
  if (e == cudaSuccess) e = cudaMalloc(&vw->d_dcount, 2 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&vw->d_spans, n * sizeof(ViewSpan));
  if (e == cudaSuccess) e = cudaMalloc(&vw->d_vd, sizeof(ViewDone));
  if (e == cudaSuccess) {
    DeferQueue dq[2];
    for (int i = 0; i < 2; i++) dq[i] = DeferQueue{vw->d_defer[i], vw->d_dcount + i,
                                                   (uint32_t)std::min<size_t>(vw->defer_cap, 0xFFFFFFFFu)};
    e = cudaMemcpy(vw->d_dq, dq, sizeof(dq), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    ne_views_destroy(vw);
    return fail(ctx, NE_ERR_OUT_OF_MEMORY, std::string("ne_views_create: ") + cudaGetErrorString(e));
  }
  ne_status st = viewsPrepare(vw);
  if (st) {
    ne_views_destroy(vw);
    return st;
  }
  *out = vw;
  return NE_OK;
}

void ne_views_destroy(ne_views* vw) {
  if (!vw) return;
  auto& v = vw->sc->view_batches;
  v.erase(std::remove(v.begin(), v.end(), vw), v.end());
  cudaSetDevice(vw->sc->ctx->device);
  cudaStreamSynchronize(vw->sc->ctx->stream);
  if (vw->exec) cudaGraphExecDestroy(vw->exec);
  void* bufs[] = {vw->d_views, vw->d_paths, vw->d_img, vw->d_done, vw->d_defer[0], vw->d_defer[1], vw->d_dq,
                  vw->d_dcount, vw->d_spans, vw->d_vd};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (cudaEvent_t e : vw->ev)
    if (e) cudaEventDestroy(e);
  delete vw;
}

ne_status ne_views_set_tuning(ne_views* vw, const ne_views_tuning* t) {
  if (!vw || !t || t->fetch < 32 || t->fetch > 4096 || t->fetch % 32 || t->blocks_per_sm < 0 ||
      t->blocks_per_sm > 64 || t->order < 0 || t->order > 2 || t->graph < 0 || t->graph > 1 || t->split_passes < 0 ||
      t->split_passes > 64 || t->split_half < 0 || t->split_half > 1 || t->groups < 0 || t->groups > 16 ||
      t->pretrace < 0 || t->pretrace > 2)
    return NE_ERR_INVALID_ARG;
  ne_context* ctx = vw->sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  vw->tune = *t;
  if (vw->tune.groups == 0) vw->tune.groups = 1;
  return viewsPrepare(vw);
}

ne_status ne_views_get_tuning(const ne_views* vw, ne_views_tuning* t) {
  if (!vw || !t) return NE_ERR_INVALID_ARG;
  *t = vw->tune;
  return NE_OK;
}

ne_status ne_views_render(ne_views* vw, ne_views_stats* stats) {
  if (!vw) return NE_ERR_INVALID_ARG;
  ne_context* ctx = vw->sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const uint32_t n = (uint32_t)vw->views.size();
  NE_CUDA(cudaEventRecord(vw->ev[0], ctx->stream), "cudaEventRecord");
  if (vw->exec) {
    NE_CUDA(cudaGraphLaunch(vw->exec, ctx->stream), "cudaGraphLaunch");
  } else {
    ne_status st = viewsEnqueue(vw);
    if (st) return st;
  }
  NE_CUDA(cudaEventRecord(vw->ev[1], ctx->stream), "cudaEventRecord");
  std::vector<unsigned long long> t(n + 1);
  NE_CUDA(cudaMemcpyAsync(t.data(), vw->d_done + n, (n + 1) * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                          ctx->stream),
          "cudaMemcpyAsync");
  ne_status st = checkErr(ctx);
  if (st) return st;
  std::vector<float> lat(n);
  for (uint32_t s = 0; s < n; s++) {
    float ms = t[s] >= t[n] ? (float)((double)(t[s] - t[n]) * 1e-6) : 0.0f;
    vw->latency[vw->order[s]] = ms;
    lat[s] = ms;
  }
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    float ems = 0;
    cudaEventElapsedTime(&ems, vw->ev[0], vw->ev[1]);
    stats->ms = ems;
    stats->paths = vw->total;
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) { return lat[std::min<size_t>(n - 1, (size_t)(q * (n - 1) + 0.5))]; };
    stats->latency_p50_ms = pct(0.5);
    stats->latency_p99_ms = pct(0.99);
    stats->latency_max_ms = lat[n - 1];
    const int passes = viewsPasses(vw) + (vw->tune.pretrace == 2 && viewsPasses(vw) > 1 ? 1 : 0);
    stats->kernel_launches =
        (uint32_t)((vw->group_first.size() - 1) * (passes + (vw->tune.pretrace && passes > 1 ? passes - 1 : 0)) + 1);
  }
  return NE_OK;
}

ne_status ne_views_autotune(ne_views* vw, int repeats, ne_views_tuning* best, double* best_ms) {
  if (!vw || repeats < 1) return NE_ERR_INVALID_ARG;
  ne_context* ctx = vw->sc->ctx;
  int fit = 1;
  NE_CUDA(ne_views_occupancy(&fit), "occupancy query");
  fit = std::max(1, fit);
  const uint32_t fetches[2] = {32, 128};
  // (order, groups): largest first in one group, or smallest first in 1, 2 or 4 groups
  const int ogs[4][2] = {{1, 1}, {2, 1}, {2, 2}, {2, 4}};
  // (passes, by half bounce): by bounce, by half bounce
  const int passess[3][2] = {{8, 0}, {12, 1}, {16, 1}};
  struct Trial {
    ne_views_tuning t;
    double ms;
    float p50;
  };
  std::vector<Trial> trials;
  for (uint32_t f : fetches)
    for (const auto& og : ogs)
      for (const auto& sp : passess) {
        ne_views_tuning t = {f, fit, og[0], 1, sp[0], sp[1], og[1], 0};
        ne_status st = ne_views_set_tuning(vw, &t);
        if (st) return st;
        ne_views_stats s;
        st = ne_views_render(vw, &s);
        if (st) return st;
        Trial tr = {t, 1e30, 0.0f};
        for (int r = 0; r < repeats; r++) {
          st = ne_views_render(vw, &s);
          if (st) return st;
          if (s.ms < tr.ms) {
            tr.ms = s.ms;
            tr.p50 = s.latency_p50_ms;
          }
        }
        trials.push_back(tr);
      }
  // throughput first: among the configurations within 3% of the fastest, the lowest median
  // view latency
  double fastest = 1e30;
  for (const Trial& tr : trials) fastest = std::min(fastest, tr.ms);
  const Trial* pick = nullptr;
  for (const Trial& tr : trials)
    if (tr.ms <= fastest * 1.03 && (!pick || tr.p50 < pick->p50)) pick = &tr;
  // then the pick with the bounce rays (1) and the camera rays too (2) traced ahead of each pass
  Trial chosen = *pick;
  const ne_views_tuning picked = pick->t;
  for (int pre = 1; pre <= 2 && picked.split_passes != 1; pre++) {
    ne_views_tuning t = picked;
    t.pretrace = pre;
    ne_status st = ne_views_set_tuning(vw, &t);
    if (st) return st;
    ne_views_stats s;
    st = ne_views_render(vw, &s);
    if (st) return st;
    Trial tr = {t, 1e30, 0.0f};
    for (int r = 0; r < repeats; r++) {
      st = ne_views_render(vw, &s);
      if (st) return st;
      if (s.ms < tr.ms) {
        tr.ms = s.ms;
        tr.p50 = s.latency_p50_ms;
      }
    }
    if (tr.ms < chosen.ms) chosen = tr;
  }
  ne_status st = ne_views_set_tuning(vw, &chosen.t);
  if (st) return st;
  if (best) *best = chosen.t;
  if (best_ms) *best_ms = chosen.ms;
  return NE_OK;
}

ne_status ne_views_latency(const ne_views* vw, float* ms) {
  if (!vw || !ms) return NE_ERR_INVALID_ARG;
  memcpy(ms, vw->latency.data(), vw->latency.size() * sizeof(float));
  return NE_OK;
}

ne_status ne_views_image(const ne_views* vw, uint32_t v, float* out) {
  if (!vw || !out || v >= vw->views.size()) return NE_ERR_INVALID_ARG;
  ne_context* ctx = vw->sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const DView& d = vw->dv[vw->slot_of[v]];
  size_t bytes = (size_t)d.width * d.height * 3 * sizeof(float);
  NE_CUDA(cudaMemcpyAsync(out, vw->d_img + 3 * (size_t)d.pix_begin, bytes, cudaMemcpyDeviceToHost, ctx->stream),
          "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  return NE_OK;
}

ne_status ne_scene_autotune(ne_scene* sc, const ne_render_params* p, int repeats, ne_tuning* best, double* best_ms) {
  if (!sc || repeats < 1) return NE_ERR_INVALID_ARG;
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const int W = sc->settings.width, H = sc->settings.height;
  DevBuf<float> img;
  NE_CUDA(cudaMalloc(&img.p, (size_t)W * H * 3 * sizeof(float)), "cudaMalloc(image)");
  ne_render_params rp = p ? *p : ne_render_params{0, 0, -1, -1, 3, 0, 0};
  rp.flags = (rp.flags | NE_RENDER_OUT_DEVICE) & ~(NE_RENDER_COUNT_WORK | NE_RENDER_NO_SYNC);
  ne_tuning keep;
  ne_scene_get_tuning(sc, &keep);
  std::vector<ne_tuning> cands;
  for (int k : {0, 2}) cands.push_back(ne_tuning{k, 16, 0, 0, 0, 3});
  // the regrouped kernel at three regrouping thresholds (32nds of a warp's live lanes in one
  // kind of event)
  for (int share : {8, 16, 24}) cands.push_back(ne_tuning{1, share, 0, 0, 0, 3});
  for (int passes : {3, 4, 6, 8, 12, 16, 24}) cands.push_back(ne_tuning{3, 16, 0, passes, 0, 3});
  for (int passes : {12, 16, 20, 24, 32}) cands.push_back(ne_tuning{3, 16, 0, passes, 1, 3});
  ne_tuning bt = keep;
  double bms = 1e30;
  auto tryTuning = [&](const ne_tuning& t) -> ne_status {
    ne_status st = ne_scene_set_tuning(sc, &t);
    if (st) return st;
    ne_render_stats s;
    st = ne_render(sc, &rp, img.p, &s);  // warm-up
    if (st) return st;
    double m = 1e30;
    for (int r = 0; r < repeats; r++) {
      st = ne_render(sc, &rp, img.p, &s);
      if (st) return st;
      m = std::min(m, s.kernel_ms);
    }
    if (m < bms) {
      bms = m;
      bt = t;
    }
    return NE_OK;
  };
  for (const ne_tuning& t : cands) {
    ne_status st = tryTuning(t);
    if (st) return st;
  }
  // then the best split configuration's deferred-path capacity: 2 or 4 quarters of the paths
  if (bt.kernel == 3) {
    ne_tuning base = bt;
    for (int q : {2, 4}) {
      ne_tuning t = base;
      t.queue_quarters = q;
      ne_status st = tryTuning(t);
      if (st) return st;
    }
  }
  // and, for surface scenes split by bounce, the bounce rays traced ahead of each pass
  if (bt.kernel == 3 && !bt.split_half && (sc->feature_set == K_MESH || sc->feature_set == K_SURFACE)) {
    const ne_tuning base = bt;
    for (int pre : {1, 2}) {  // the bounce rays; the camera rays too
      ne_tuning t = base;
      t.pretrace = pre;
      ne_status st = tryTuning(t);
      if (st) return st;
    }
    // the shadow rays too: every pass takes each path one traversal further, so more passes
    for (int passes : {6, 8, 12, 16, 24}) {
      ne_tuning t = base;
      t.pretrace = 3;
      t.split_passes = passes;
      ne_status st = tryTuning(t);
      if (st) return st;
    }
  }
  ne_status st = ne_scene_set_tuning(sc, &bt);
  if (st) return st;
  if (best) ne_scene_get_tuning(sc, best);
  if (best_ms) *best_ms = bms;
  return NE_OK;
}

ne_status ne_scene_bvh(const ne_scene* sc, uint32_t model, float* nodes, size_t cap, uint32_t* order,
                       size_t* n_nodes) {
  if (!sc || !n_nodes || model >= sc->bvh_nodes_of.size()) return NE_ERR_INVALID_ARG;
  const uint32_t nn = sc->bvh_nodes_of[model];
  *n_nodes = nn;
  if (!nodes) return NE_OK;
  if (nn == 0) return NE_OK;
  if (cap < nn || !order) return NE_ERR_INVALID_ARG;
  ne_context* ctx = sc->ctx;
  NE_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
  const DModel& m = sc->bvh_models[model];
  std::vector<DNode> dn(nn);
  NE_CUDA(cudaMemcpyAsync(dn.data(), sc->d.bvh + m.bvh_node0, nn * sizeof(DNode), cudaMemcpyDeviceToHost, ctx->stream),
          "cudaMemcpyAsync");
  NE_CUDA(cudaMemcpyAsync(order, sc->d.bvh_prims + m.bvh_slot0, m.prim_count * sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, ctx->stream),
          "cudaMemcpyAsync");
  NE_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
  for (uint32_t i = 0; i < nn; i++) {
    float* o = nodes + 9 * (size_t)i;
    memcpy(o, dn[i].lo, 12);
    memcpy(o + 3, dn[i].hi, 12);
    uint32_t a, b, zero = 0;
    memcpy(&a, &dn[i].lo[3], 4);
    memcpy(&b, &dn[i].hi[3], 4);
    if (b & 0x80000000u) {  // leaf: start, count, rightOffset 0
      uint32_t cnt = b & 0x7fffffffu;
      memcpy(o + 6, &a, 4);
      memcpy(o + 7, &cnt, 4);
      memcpy(o + 8, &zero, 4);
    } else {  // interior: rightOffset
      memcpy(o + 6, &zero, 4);
      memcpy(o + 7, &zero, 4);
      memcpy(o + 8, &a, 4);
    }
  }
  return NE_OK;
}

ne_status ne_debug_medium_boxes(const ne_scene_desc* desc, float* boxes, size_t cap, int32_t* n_boxes) {
  if (!desc || !n_boxes) return NE_ERR_INVALID_ARG;
  const ne_scene_desc& D = *desc;
  for (uint32_t i = 0; i < D.n_instances + D.n_light_instances; i++) {
    if (D.instances[i].model >= D.n_models) return NE_ERR_INVALID_ARG;
    const ne_model& m = D.models[D.instances[i].model];
    if ((uint64_t)m.prim_begin + m.prim_count > D.n_prims || (uint64_t)m.light_begin + m.light_count > D.n_prims)
      return NE_ERR_INVALID_ARG;
  }
  for (uint32_t i = 0; i < D.n_prims; i++)
    if (D.prims[i].material >= (int)D.n_materials) return NE_ERR_INVALID_ARG;
  std::vector<float> b;
  *n_boxes = mediumBoxesOf(*desc, b);
  if (*n_boxes <= 0) return NE_OK;
  if (!boxes || cap < (size_t)*n_boxes) return NE_ERR_INVALID_ARG;
  memcpy(boxes, b.data(), b.size() * sizeof(float));
  return NE_OK;
}

ne_status ne_debug_bvh(const ne_primitive* prims, uint32_t first, uint32_t count, float* nodes, size_t cap,
                       uint32_t* order, size_t* n_nodes) {
  if (!prims || !nodes || !order || !n_nodes || count == 0) return NE_ERR_INVALID_ARG;
  std::vector<uint32_t> ord(count);
  for (uint32_t k = 0; k < count; k++) ord[k] = first + k;
  std::vector<HNode> hn;
  buildBvh(prims, ord, hn);
  *n_nodes = hn.size();
  if (hn.size() > cap) return NE_ERR_INVALID_ARG;
  for (size_t i = 0; i < hn.size(); i++) {
    float* o = nodes + 9 * i;
    o[0] = hn[i].mn.x; o[1] = hn[i].mn.y; o[2] = hn[i].mn.z;
    o[3] = hn[i].mx.x; o[4] = hn[i].mx.y; o[5] = hn[i].mx.z;
    memcpy(o + 6, &hn[i].start, 4);
    memcpy(o + 7, &hn[i].count, 4);
    memcpy(o + 8, &hn[i].rightOffset, 4);
  }
  memcpy(order, ord.data(), count * sizeof(uint32_t));
  return NE_OK;
}

}  // extern "C"
