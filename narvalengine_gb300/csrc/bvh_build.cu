// GPU binned-SAH BVH build for triangle meshes.
//
// The reference builds its BVH on the CPU by midpoint splits (primitives/BVH.cpp:6-106); a scene
// may instead ask for this builder ("bvh": "sah" in its renderer block). The tree has the
// reference's node layout and leaf size, so the same traversal (BVH.cpp:108-193) runs over it:
// depth-first node order (left child = i + 1, right child = i + rightOffset), at most four
// triangles per leaf. Closest hits equal those over the reference's tree except where two
// triangles are hit at exactly the same distance (the traversal order decides those).
//
// The build runs level by level. Each level's tasks (contiguous ranges of the primitive order)
// of up to 65536 triangles get one CTA each in two kernels:
//  * k_sah_bin: node bounds and centroid bounds (block reduction), then 32 bins per axis over the
//    centroid bounds (shared-memory atomics on order-preserving float keys), then the split of
//    least surface-area cost A_L N_L + A_R N_R; a range of at most four triangles becomes a
//    leaf; no split with both sides non-empty, or depth 36 and beyond, gives the median split.
//  * k_sah_partition: stable partition of the range by the chosen split (block scans of the
//    side flags), through a scratch array.
// Levels whose ranges all hold at most 2048 triangles use a warp per range instead (k_sah_*_warp).
// Larger ranges (the first levels) are cut into segments of 16384 triangles, one CTA each, that
// combine their bounds and bins through global atomics (k_wide_*); one thread per range then
// picks the split, and the segments partition at offsets from a per-range prefix of their left
// counts. The host reads each level's results back, numbers the nodes and issues the next level; at
// the end it lays the nodes out depth first. Every step is deterministic (integer counts,
// min/max, stable partitions), so a scene always gets the same tree.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include "bvh_build.h"
#include "host_parallel.h"

namespace nedev {
namespace {

constexpr int kBins = 32;
constexpr uint32_t kLeafPrims = 4;      // BVH::init's primitives per leaf (BVH.cpp)
constexpr uint32_t kMedianDepth = 36;   // from this depth on every split is the median
constexpr int kMaxLevels = 64;
constexpr int kThreads = 1024;  // most threads a task's CTA has (levels with few, large tasks)

struct Task {
  uint32_t begin, end, depth;
  uint32_t wide;  // 1: binned and partitioned by several CTAs (the k_wide_* kernels)
};
// One CTA's share of a wide task: [begin, end) of the primitive order.
struct Segment {
  uint32_t task, wide, begin, end;
};
constexpr uint32_t kWideMin = 65536;   // tasks of more triangles use several CTAs
constexpr uint32_t kSegment = 16384;   // triangles per CTA of a wide task
struct TaskResult {
  float mn[3], mx[3];
  int32_t axis;      // -1: median split
  uint32_t split;    // bins [0, split) go left
  uint32_t nLeft;
  int32_t leaf;
  float cmin, scale; // bin of centroid c: (int)((c - cmin) * scale), clamped to [0, kBins)
  float cb[2][6];    // binned split: the children's bounds (min xyz, max xyz), left then right
};

// Order-preserving map of floats to unsigned keys (for atomicMin/atomicMax).
__device__ __forceinline__ uint32_t fkey(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float funkey(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
__device__ __forceinline__ int binOf(float c, float cmin, float scale) {
  int b = (int)((c - cmin) * scale);
  return b < 0 ? 0 : (b >= kBins ? kBins - 1 : b);
}
__device__ __forceinline__ float area(const float* mn, const float* mx) {
  float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
  return 2.0f * (dx * dy + dy * dz + dz * dx);
}

__global__ void k_prim_bounds(const DPrim* __restrict__ prims, uint32_t first, uint32_t n, float4* __restrict__ lo,
                              float4* __restrict__ hi, float4* __restrict__ cen, uint32_t* __restrict__ order) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const DPrim& p = prims[first + i];
    float mn[3], mx[3];
    for (int k = 0; k < 3; k++) {
      mn[k] = fminf(fminf(p.p0[k], p.p1[k]), p.p2[k]);
      mx[k] = fmaxf(fmaxf(p.p0[k], p.p1[k]), p.p2[k]);
    }
    lo[i] = make_float4(mn[0], mn[1], mn[2], 0.0f);
    hi[i] = make_float4(mx[0], mx[1], mx[2], 0.0f);
    cen[i] = make_float4(0.5f * (mn[0] + mx[0]), 0.5f * (mn[1] + mx[1]), 0.5f * (mn[2] + mx[2]), 0.0f);
    order[i] = i;
  }
}

// Block-wide min (op 0) or max (op 1) of one value per thread; every thread gets the result.
__device__ float blockReduce(float v, int op, float* scratch) {
  for (int o = 16; o > 0; o >>= 1) {
    float w = __shfl_xor_sync(0xffffffffu, v, o);
    v = op ? fmaxf(v, w) : fminf(v, w);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  float r = scratch[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); w++) r = op ? fmaxf(r, scratch[w]) : fminf(r, scratch[w]);
  return r;
}

// The least-cost binned split (A_L N_L + A_R N_R over the 31 split planes of each axis with a
// non-zero centroid extent) from bins laid out [axis][bin][xyz] (min/max keys) and [axis][bin]
// (counts); fills axis, split, nLeft, cmin, scale and the children's bounds of `r`, or leaves
// r.axis = -1 when no split has both sides non-empty.
__device__ void evalSah(const uint32_t* bminp, const uint32_t* bmaxp, const uint32_t* bcntp, const float* cmn,
                        const float* scale, TaskResult& r) {
  const float inf = __int_as_float(0x7f800000);
  auto bmin = [&](int a, int b, int k) { return funkey(bminp[(a * kBins + b) * 3 + k]); };
  auto bmax = [&](int a, int b, int k) { return funkey(bmaxp[(a * kBins + b) * 3 + k]); };
  auto bcnt = [&](int a, int b) { return bcntp[a * kBins + b]; };
  float best = inf;
  for (int a = 0; a < 3; a++) {
    if (scale[a] == 0.0f) continue;
    // right-hand sweep: bounds and counts of bins [s, kBins)
    float rArea[kBins];
    uint32_t rCnt[kBins];
    float rmn[3] = {inf, inf, inf}, rmx[3] = {-inf, -inf, -inf};
    uint32_t rc = 0;
    for (int b = kBins - 1; b >= 0; b--) {
      if (bcnt(a, b)) {
        for (int k = 0; k < 3; k++) {
          rmn[k] = fminf(rmn[k], bmin(a, b, k));
          rmx[k] = fmaxf(rmx[k], bmax(a, b, k));
        }
        rc += bcnt(a, b);
      }
      rArea[b] = rc ? area(rmn, rmx) : 0.0f;
      rCnt[b] = rc;
    }
    float lmn[3] = {inf, inf, inf}, lmx[3] = {-inf, -inf, -inf};
    uint32_t lc = 0;
    for (int sp = 1; sp < kBins; sp++) {
      int b = sp - 1;
      if (bcnt(a, b)) {
        for (int k = 0; k < 3; k++) {
          lmn[k] = fminf(lmn[k], bmin(a, b, k));
          lmx[k] = fmaxf(lmx[k], bmax(a, b, k));
        }
        lc += bcnt(a, b);
      }
      if (lc == 0 || rCnt[sp] == 0) continue;
      float cost = area(lmn, lmx) * (float)lc + rArea[sp] * (float)rCnt[sp];
      if (cost < best) {
        best = cost;
        r.axis = a;
        r.split = (uint32_t)sp;
        r.nLeft = lc;
        r.cmin = cmn[a];
        r.scale = scale[a];
        for (int k = 0; k < 3; k++) { r.cb[0][k] = lmn[k]; r.cb[0][3 + k] = lmx[k]; }
      }
    }
  }
  if (r.axis >= 0) {  // the right child's bounds: bins [split, kBins) of the chosen axis
    float rmn[3] = {inf, inf, inf}, rmx[3] = {-inf, -inf, -inf};
    for (int b = (int)r.split; b < kBins; b++)
      if (bcnt(r.axis, b))
        for (int k = 0; k < 3; k++) {
          rmn[k] = fminf(rmn[k], bmin(r.axis, b, k));
          rmx[k] = fmaxf(rmx[k], bmax(r.axis, b, k));
        }
    for (int k = 0; k < 3; k++) { r.cb[1][k] = rmn[k]; r.cb[1][3 + k] = rmx[k]; }
  }
}

__global__ void __launch_bounds__(kThreads) k_sah_bin(const Task* __restrict__ tasks, const float4* __restrict__ lo,
                                                     const float4* __restrict__ hi, const float4* __restrict__ cen,
                                                     const uint32_t* __restrict__ order, TaskResult* __restrict__ res) {
  __shared__ float scratch[kThreads / 32];
  __shared__ uint32_t bmin[3][kBins][3], bmax[3][kBins][3], bcnt[3][kBins];
  const Task t = tasks[blockIdx.x];
  if (t.wide) return;  // k_wide_* handle it
  const uint32_t count = t.end - t.begin;
  const float inf = __int_as_float(0x7f800000);
  float mn[3] = {inf, inf, inf}, mx[3] = {-inf, -inf, -inf}, cmn[3] = {inf, inf, inf}, cmx[3] = {-inf, -inf, -inf};
  for (uint32_t i = t.begin + threadIdx.x; i < t.end; i += blockDim.x) {
    uint32_t p = order[i];
    float4 a = lo[p], b = hi[p], c = cen[p];
    mn[0] = fminf(mn[0], a.x); mn[1] = fminf(mn[1], a.y); mn[2] = fminf(mn[2], a.z);
    mx[0] = fmaxf(mx[0], b.x); mx[1] = fmaxf(mx[1], b.y); mx[2] = fmaxf(mx[2], b.z);
    cmn[0] = fminf(cmn[0], c.x); cmn[1] = fminf(cmn[1], c.y); cmn[2] = fminf(cmn[2], c.z);
    cmx[0] = fmaxf(cmx[0], c.x); cmx[1] = fmaxf(cmx[1], c.y); cmx[2] = fmaxf(cmx[2], c.z);
  }
  for (int k = 0; k < 3; k++) {
    mn[k] = blockReduce(mn[k], 0, scratch);
    mx[k] = blockReduce(mx[k], 1, scratch);
    cmn[k] = blockReduce(cmn[k], 0, scratch);
    cmx[k] = blockReduce(cmx[k], 1, scratch);
  }
  TaskResult r;
  for (int k = 0; k < 3; k++) { r.mn[k] = mn[k]; r.mx[k] = mx[k]; }
  r.axis = -1;
  r.split = 0;
  r.nLeft = count / 2;
  r.leaf = count <= kLeafPrims;
  r.cmin = 0.0f;
  r.scale = 0.0f;
  if (r.leaf || t.depth >= kMedianDepth) {
    if (threadIdx.x == 0) res[blockIdx.x] = r;
    return;
  }
  float scale[3];
  for (int a = 0; a < 3; a++) {
    float ext = cmx[a] - cmn[a];
    scale[a] = ext > 0.0f ? (float)kBins / ext : 0.0f;
  }
  for (int j = threadIdx.x; j < 3 * kBins; j += blockDim.x) {
    int a = j / kBins, b = j % kBins;
    for (int k = 0; k < 3; k++) { bmin[a][b][k] = 0xffffffffu; bmax[a][b][k] = 0u; }
    bcnt[a][b] = 0;
  }
  __syncthreads();
  for (uint32_t i = t.begin + threadIdx.x; i < t.end; i += blockDim.x) {
    uint32_t p = order[i];
    float4 a4 = lo[p], b4 = hi[p], c4 = cen[p];
    const float pl[3] = {a4.x, a4.y, a4.z}, ph[3] = {b4.x, b4.y, b4.z}, pc[3] = {c4.x, c4.y, c4.z};
    for (int a = 0; a < 3; a++) {
      if (scale[a] == 0.0f) continue;
      int b = binOf(pc[a], cmn[a], scale[a]);
      for (int k = 0; k < 3; k++) {
        atomicMin(&bmin[a][b][k], fkey(pl[k]));
        atomicMax(&bmax[a][b][k], fkey(ph[k]));
      }
      atomicAdd(&bcnt[a][b], 1u);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    evalSah(&bmin[0][0][0], &bmax[0][0][0], &bcnt[0][0], cmn, scale, r);
    res[blockIdx.x] = r;
  }
}

// A range whose left count differs from the binning's (which would mean the two kernels binned
// differently) writes nothing out of its range and raises *bad; the host then fails the build.
__global__ void __launch_bounds__(kThreads) k_sah_partition(const Task* __restrict__ tasks,
                                                           const TaskResult* __restrict__ res,
                                                           const float4* __restrict__ cen, uint32_t* __restrict__ order,
                                                           uint32_t* __restrict__ tmp, uint32_t* __restrict__ bad) {
  __shared__ uint32_t warpLeft[kThreads / 32];
  __shared__ uint32_t run[2];
  const Task t = tasks[blockIdx.x];
  if (t.wide) return;  // k_wide_* handle it
  const TaskResult r = res[blockIdx.x];
  if (r.leaf) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) { run[0] = 0; run[1] = 0; }
  __syncthreads();
  for (uint32_t base = t.begin; base < t.end; base += blockDim.x) {
    uint32_t i = base + threadIdx.x;
    bool valid = i < t.end;
    uint32_t p = valid ? order[i] : 0;
    bool left = false;
    if (valid) {
      if (r.axis < 0) {
        left = (i - t.begin) < r.nLeft;
      } else {
        float4 c = cen[p];
        float v = r.axis == 0 ? c.x : (r.axis == 1 ? c.y : c.z);
        left = binOf(v, r.cmin, r.scale) < (int)r.split;
      }
    }
    uint32_t ball = __ballot_sync(0xffffffffu, left);
    uint32_t rank = __popc(ball & ((1u << lane) - 1u));
    if (lane == 0) warpLeft[warp] = __popc(ball);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < nwarps; w++) {
      if (w < warp) before += warpLeft[w];
      total += warpLeft[w];
    }
    if (valid) {
      uint32_t leftBefore = before + rank;
      uint32_t rightBefore = threadIdx.x - leftBefore;
      uint32_t dest = left ? t.begin + run[0] + leftBefore : t.begin + r.nLeft + run[1] + rightBefore;
      if (left ? (run[0] + leftBefore < r.nLeft) : (dest < t.end)) tmp[dest] = p;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t chunk = min((uint32_t)blockDim.x, t.end - base);
      run[0] += total;
      run[1] += chunk - total;
    }
    __syncthreads();
  }
  if (run[0] != r.nLeft) {  // every thread reads the same value: leave the range as it is
    if (threadIdx.x == 0) atomicOr(bad, 1u);
    return;
  }
  for (uint32_t i = t.begin + threadIdx.x; i < t.end; i += blockDim.x) order[i] = tmp[i];
}

// ---- small tasks: one warp per task (the last levels, with many ranges of a few triangles)
constexpr int kWarpTasks = 8;          // warps (tasks) per CTA
constexpr uint32_t kSmallMax = 2048;   // levels whose ranges are all this small use these kernels

__device__ __forceinline__ float warpMin(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warpMax(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void __launch_bounds__(32 * kWarpTasks) k_sah_bin_warp(const Task* __restrict__ tasks, uint32_t nt,
                                                                 const float4* __restrict__ lo,
                                                                 const float4* __restrict__ hi,
                                                                 const float4* __restrict__ cen,
                                                                 const uint32_t* __restrict__ order,
                                                                 TaskResult* __restrict__ res) {
  __shared__ uint32_t binsAll[kWarpTasks][3 * kBins * 3 * 2 + 3 * kBins];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t ti = blockIdx.x * kWarpTasks + warp;
  if (ti >= nt) return;  // the whole warp: no block-wide barrier follows
  const Task t = tasks[ti];
  const uint32_t count = t.end - t.begin;
  const float inf = __int_as_float(0x7f800000);
  float mn[3] = {inf, inf, inf}, mx[3] = {-inf, -inf, -inf}, cmn[3] = {inf, inf, inf}, cmx[3] = {-inf, -inf, -inf};
  for (uint32_t i = t.begin + lane; i < t.end; i += 32) {
    uint32_t p = order[i];
    float4 a = lo[p], b = hi[p], c = cen[p];
    mn[0] = fminf(mn[0], a.x); mn[1] = fminf(mn[1], a.y); mn[2] = fminf(mn[2], a.z);
    mx[0] = fmaxf(mx[0], b.x); mx[1] = fmaxf(mx[1], b.y); mx[2] = fmaxf(mx[2], b.z);
    cmn[0] = fminf(cmn[0], c.x); cmn[1] = fminf(cmn[1], c.y); cmn[2] = fminf(cmn[2], c.z);
    cmx[0] = fmaxf(cmx[0], c.x); cmx[1] = fmaxf(cmx[1], c.y); cmx[2] = fmaxf(cmx[2], c.z);
  }
  for (int k = 0; k < 3; k++) {
    mn[k] = warpMin(mn[k]);
    mx[k] = warpMax(mx[k]);
    cmn[k] = warpMin(cmn[k]);
    cmx[k] = warpMax(cmx[k]);
  }
  TaskResult r;
  for (int k = 0; k < 3; k++) { r.mn[k] = mn[k]; r.mx[k] = mx[k]; }
  r.axis = -1;
  r.split = 0;
  r.nLeft = count / 2;
  r.leaf = count <= kLeafPrims;
  r.cmin = 0.0f;
  r.scale = 0.0f;
  if (r.leaf || t.depth >= kMedianDepth) {
    if (lane == 0) res[ti] = r;
    return;
  }
  float scale[3];
  for (int a = 0; a < 3; a++) {
    float ext = cmx[a] - cmn[a];
    scale[a] = ext > 0.0f ? (float)kBins / ext : 0.0f;
  }
  uint32_t* bins = binsAll[warp];
  uint32_t* bmin = bins;
  uint32_t* bmax = bins + 3 * kBins * 3;
  uint32_t* bcnt = bins + 2 * 3 * kBins * 3;
  for (int j = lane; j < 3 * kBins * 3 * 2 + 3 * kBins; j += 32) bins[j] = j < 3 * kBins * 3 ? 0xffffffffu : 0u;
  __syncwarp();
  for (uint32_t i = t.begin + lane; i < t.end; i += 32) {
    uint32_t p = order[i];
    float4 a4 = lo[p], b4 = hi[p], c4 = cen[p];
    const float pl[3] = {a4.x, a4.y, a4.z}, ph[3] = {b4.x, b4.y, b4.z}, pc[3] = {c4.x, c4.y, c4.z};
    for (int a = 0; a < 3; a++) {
      if (scale[a] == 0.0f) continue;
      int b = binOf(pc[a], cmn[a], scale[a]);
      for (int k = 0; k < 3; k++) {
        atomicMin(&bmin[(a * kBins + b) * 3 + k], fkey(pl[k]));
        atomicMax(&bmax[(a * kBins + b) * 3 + k], fkey(ph[k]));
      }
      atomicAdd(&bcnt[a * kBins + b], 1u);
    }
  }
  __syncwarp();
  if (lane == 0) {
    evalSah(bmin, bmax, bcnt, cmn, scale, r);
    res[ti] = r;
  }
}

__global__ void __launch_bounds__(32 * kWarpTasks) k_sah_partition_warp(const Task* __restrict__ tasks, uint32_t nt,
                                                                       const TaskResult* __restrict__ res,
                                                                       const float4* __restrict__ cen,
                                                                       uint32_t* __restrict__ order,
                                                                       uint32_t* __restrict__ tmp,
                                                                       uint32_t* __restrict__ bad) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t ti = blockIdx.x * kWarpTasks + warp;
  if (ti >= nt) return;
  const Task t = tasks[ti];
  const TaskResult r = res[ti];
  if (r.leaf) return;
  uint32_t leftRun = 0, rightRun = 0;
  for (uint32_t base = t.begin; base < t.end; base += 32) {
    uint32_t i = base + lane;
    bool valid = i < t.end;
    uint32_t p = valid ? order[i] : 0;
    bool left = false;
    if (valid) {
      if (r.axis < 0) {
        left = (i - t.begin) < r.nLeft;
      } else {
        float4 c = cen[p];
        float v = r.axis == 0 ? c.x : (r.axis == 1 ? c.y : c.z);
        left = binOf(v, r.cmin, r.scale) < (int)r.split;
      }
    }
    uint32_t ball = __ballot_sync(0xffffffffu, left);
    uint32_t rank = __popc(ball & ((1u << lane) - 1u));
    if (valid) {
      uint32_t dest = left ? t.begin + leftRun + rank : t.begin + r.nLeft + rightRun + ((uint32_t)lane - rank);
      if (left ? (leftRun + rank < r.nLeft) : (dest < t.end)) tmp[dest] = p;
    }
    uint32_t total = __popc(ball);
    leftRun += total;
    rightRun += min(32u, t.end - base) - total;
  }
  __syncwarp();
  if (leftRun != r.nLeft) {
    if (lane == 0) atomicOr(bad, 1u);
    return;
  }
  for (uint32_t i = t.begin + lane; i < t.end; i += 32) order[i] = tmp[i];
}

// ---- wide tasks: several CTAs per task (the first levels, with few large ranges)
// Per wide task w: acc[w] = 12 keys (node min xyz, node max xyz, centroid min xyz, centroid
// max xyz) and bins gb[w] = min keys [3][kBins][3], max keys [3][kBins][3], counts [3][kBins].
constexpr int kBinWords = 3 * kBins * 3 * 2 + 3 * kBins;

__global__ void k_wide_init(uint32_t nwide, uint32_t* __restrict__ acc, uint32_t* __restrict__ gb) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nwide * 12; i += gridDim.x * blockDim.x)
    acc[i] = ((i % 12) < 3 || ((i % 12) >= 6 && (i % 12) < 9)) ? 0xffffffffu : 0u;  // min keys start high
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nwide * kBinWords; i += gridDim.x * blockDim.x)
    gb[i] = (i % kBinWords) < 3 * kBins * 3 ? 0xffffffffu : 0u;
}

__global__ void __launch_bounds__(kThreads) k_wide_bounds(const Segment* __restrict__ segs,
                                                         const float4* __restrict__ lo, const float4* __restrict__ hi,
                                                         const float4* __restrict__ cen,
                                                         const uint32_t* __restrict__ order, uint32_t* __restrict__ acc) {
  __shared__ float scratch[kThreads / 32];
  const Segment g = segs[blockIdx.x];
  const float inf = __int_as_float(0x7f800000);
  float v[12] = {inf, inf, inf, -inf, -inf, -inf, inf, inf, inf, -inf, -inf, -inf};
  for (uint32_t i = g.begin + threadIdx.x; i < g.end; i += blockDim.x) {
    uint32_t p = order[i];
    float4 a = lo[p], b = hi[p], c = cen[p];
    v[0] = fminf(v[0], a.x); v[1] = fminf(v[1], a.y); v[2] = fminf(v[2], a.z);
    v[3] = fmaxf(v[3], b.x); v[4] = fmaxf(v[4], b.y); v[5] = fmaxf(v[5], b.z);
    v[6] = fminf(v[6], c.x); v[7] = fminf(v[7], c.y); v[8] = fminf(v[8], c.z);
    v[9] = fmaxf(v[9], c.x); v[10] = fmaxf(v[10], c.y); v[11] = fmaxf(v[11], c.z);
  }
  for (int k = 0; k < 12; k++) {
    bool isMax = (k >= 3 && k < 6) || k >= 9;
    float r = blockReduce(v[k], isMax ? 1 : 0, scratch);
    if (threadIdx.x == 0) {
      if (isMax) atomicMax(&acc[g.wide * 12 + k], fkey(r));
      else atomicMin(&acc[g.wide * 12 + k], fkey(r));
    }
  }
}

__device__ void wideScale(const uint32_t* acc, float* cmn, float* scale) {
  for (int a = 0; a < 3; a++) {
    cmn[a] = funkey(acc[6 + a]);
    float ext = funkey(acc[9 + a]) - cmn[a];
    scale[a] = ext > 0.0f ? (float)kBins / ext : 0.0f;
  }
}

__global__ void __launch_bounds__(kThreads) k_wide_bin(const Segment* __restrict__ segs, const float4* __restrict__ lo,
                                                      const float4* __restrict__ hi, const float4* __restrict__ cen,
                                                      const uint32_t* __restrict__ order,
                                                      const uint32_t* __restrict__ acc, uint32_t* __restrict__ gb) {
  __shared__ uint32_t bins[kBinWords];
  const Segment g = segs[blockIdx.x];
  float cmn[3], scale[3];
  wideScale(acc + g.wide * 12, cmn, scale);
  for (int j = threadIdx.x; j < kBinWords; j += blockDim.x) bins[j] = j < 3 * kBins * 3 ? 0xffffffffu : 0u;
  __syncthreads();
  uint32_t* bmin = bins;
  uint32_t* bmax = bins + 3 * kBins * 3;
  uint32_t* bcnt = bins + 2 * 3 * kBins * 3;
  for (uint32_t i = g.begin + threadIdx.x; i < g.end; i += blockDim.x) {
    uint32_t p = order[i];
    float4 a4 = lo[p], b4 = hi[p], c4 = cen[p];
    const float pl[3] = {a4.x, a4.y, a4.z}, ph[3] = {b4.x, b4.y, b4.z}, pc[3] = {c4.x, c4.y, c4.z};
    for (int a = 0; a < 3; a++) {
      if (scale[a] == 0.0f) continue;
      int b = binOf(pc[a], cmn[a], scale[a]);
      for (int k = 0; k < 3; k++) {
        atomicMin(&bmin[(a * kBins + b) * 3 + k], fkey(pl[k]));
        atomicMax(&bmax[(a * kBins + b) * 3 + k], fkey(ph[k]));
      }
      atomicAdd(&bcnt[a * kBins + b], 1u);
    }
  }
  __syncthreads();
  uint32_t* out = gb + (size_t)g.wide * kBinWords;
  for (int j = threadIdx.x; j < 3 * kBins; j += blockDim.x) {
    if (!bcnt[j]) continue;
    for (int k = 0; k < 3; k++) {
      atomicMin(&out[j * 3 + k], bmin[j * 3 + k]);
      atomicMax(&out[3 * kBins * 3 + j * 3 + k], bmax[j * 3 + k]);
    }
    atomicAdd(&out[2 * 3 * kBins * 3 + j], bcnt[j]);
  }
}

// One thread per wide task: its node bounds and split, written where k_sah_bin would.
__global__ void k_wide_sah(uint32_t nwide, const uint32_t* __restrict__ taskOf, const Task* __restrict__ tasks,
                           const uint32_t* __restrict__ acc, const uint32_t* __restrict__ gb,
                           TaskResult* __restrict__ res) {
  uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nwide) return;
  const uint32_t ti = taskOf[w];
  const Task t = tasks[ti];
  const uint32_t* a = acc + w * 12;
  TaskResult r;
  for (int k = 0; k < 3; k++) { r.mn[k] = funkey(a[k]); r.mx[k] = funkey(a[3 + k]); }
  r.axis = -1;
  r.split = 0;
  r.nLeft = (t.end - t.begin) / 2;
  r.leaf = 0;
  r.cmin = 0.0f;
  r.scale = 0.0f;
  float cmn[3], scale[3];
  wideScale(a, cmn, scale);
  const uint32_t* b = gb + (size_t)w * kBinWords;
  evalSah(b, b + 3 * kBins * 3, b + 2 * 3 * kBins * 3, cmn, scale, r);
  res[ti] = r;
}

// Left count of each segment under its task's split.
__global__ void __launch_bounds__(kThreads) k_wide_count(const Segment* __restrict__ segs, const Task* __restrict__ tasks,
                                                        const TaskResult* __restrict__ res,
                                                        const float4* __restrict__ cen,
                                                        const uint32_t* __restrict__ order, uint32_t* __restrict__ segLeft) {
  __shared__ uint32_t total;
  const Segment g = segs[blockIdx.x];
  const TaskResult r = res[g.task];
  const uint32_t tBegin = tasks[g.task].begin;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  uint32_t mine = 0;
  for (uint32_t i = g.begin + threadIdx.x; i < g.end; i += blockDim.x) {
    bool left;
    if (r.axis < 0) {
      left = (i - tBegin) < r.nLeft;
    } else {
      float4 c = cen[order[i]];
      float v = r.axis == 0 ? c.x : (r.axis == 1 ? c.y : c.z);
      left = binOf(v, r.cmin, r.scale) < (int)r.split;
    }
    mine += left;
  }
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(&total, mine);
  __syncthreads();
  if (threadIdx.x == 0) segLeft[blockIdx.x] = total;
}

// Per wide task (one thread each): exclusive prefix of its segments' left counts; a total that
// differs from the split's raises *bad.
__global__ void k_wide_offsets(uint32_t nwide, const uint32_t* __restrict__ segFirst, const uint32_t* __restrict__ taskOf,
                               const TaskResult* __restrict__ res, const uint32_t* __restrict__ segLeft,
                               uint32_t* __restrict__ segOff, uint32_t* __restrict__ bad) {
  uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nwide) return;
  uint32_t run = 0;
  for (uint32_t s = segFirst[w]; s < segFirst[w + 1]; s++) {
    segOff[s] = run;
    run += segLeft[s];
  }
  if (run != res[taskOf[w]].nLeft) atomicOr(bad, 1u);
}

// Stable partition of one segment into tmp at its offsets within the task, then nothing else:
// k_wide_copy moves the task's range back once every segment has been written.
__global__ void __launch_bounds__(kThreads) k_wide_scatter(const Segment* __restrict__ segs, const Task* __restrict__ tasks,
                                                          const TaskResult* __restrict__ res,
                                                          const float4* __restrict__ cen,
                                                          const uint32_t* __restrict__ order,
                                                          const uint32_t* __restrict__ segOff, uint32_t* __restrict__ tmp) {
  __shared__ uint32_t warpLeft[kThreads / 32];
  __shared__ uint32_t run[2];
  const Segment g = segs[blockIdx.x];
  const Task t = tasks[g.task];
  const TaskResult r = res[g.task];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) {
    run[0] = segOff[blockIdx.x];                       // lefts of the task before this segment
    run[1] = (g.begin - t.begin) - segOff[blockIdx.x]; // rights before it
  }
  __syncthreads();
  for (uint32_t base = g.begin; base < g.end; base += blockDim.x) {
    uint32_t i = base + threadIdx.x;
    bool valid = i < g.end;
    uint32_t p = valid ? order[i] : 0;
    bool left = false;
    if (valid) {
      if (r.axis < 0) {
        left = (i - t.begin) < r.nLeft;
      } else {
        float4 c = cen[p];
        float v = r.axis == 0 ? c.x : (r.axis == 1 ? c.y : c.z);
        left = binOf(v, r.cmin, r.scale) < (int)r.split;
      }
    }
    uint32_t ball = __ballot_sync(0xffffffffu, left);
    uint32_t rank = __popc(ball & ((1u << lane) - 1u));
    if (lane == 0) warpLeft[warp] = __popc(ball);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < nwarps; w++) {
      if (w < warp) before += warpLeft[w];
      total += warpLeft[w];
    }
    if (valid) {
      uint32_t leftBefore = before + rank;
      uint32_t rightBefore = threadIdx.x - leftBefore;
      uint32_t dest = left ? t.begin + run[0] + leftBefore : t.begin + r.nLeft + run[1] + rightBefore;
      if (left ? (run[0] + leftBefore < r.nLeft) : (dest < t.end)) tmp[dest] = p;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t chunk = min((uint32_t)blockDim.x, g.end - base);
      run[0] += total;
      run[1] += chunk - total;
    }
    __syncthreads();
  }
}

__global__ void k_wide_copy(const Segment* __restrict__ segs, const uint32_t* __restrict__ tmp,
                            uint32_t* __restrict__ order, const uint32_t* __restrict__ bad) {
  if (*bad) return;  // leave the order as it was: the build fails
  const Segment g = segs[blockIdx.x];
  for (uint32_t i = g.begin + threadIdx.x; i < g.end; i += blockDim.x) order[i] = tmp[i];
}

template <class T>
struct DeviceArray {
  T* p = nullptr;
  ~DeviceArray() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, (n ? n : 1) * sizeof(T)); }
};

struct BNode {
  float mn[3], mx[3];
  uint32_t begin, count;
  int32_t left, right;
};

}  // namespace

cudaError_t buildSahBvh(cudaStream_t st, const DPrim* prims, uint32_t first, uint32_t n, std::vector<DNode>& nodesOut,
                        std::vector<uint32_t>& slotsOut, std::string& err) {
  nodesOut.clear();
  slotsOut.clear();
  if (n == 0) return cudaSuccess;
  DeviceArray<float4> lo, hi, cen;
  DeviceArray<uint32_t> order, tmp;
  DeviceArray<Task> dTasks;
  DeviceArray<TaskResult> dRes;
  DeviceArray<uint32_t> dBad;
  // wide tasks: at most n / kWideMin per level, with at most n / kSegment + that many segments
  const size_t maxWide = n / kWideMin + 2, maxSegs = n / kSegment + maxWide;
  DeviceArray<Segment> dSegs;
  DeviceArray<uint32_t> dTaskOf, dSegFirst, dSegLeft, dSegOff, dAcc, dGb;
  cudaError_t e;
  if ((e = lo.alloc(n)) || (e = hi.alloc(n)) || (e = cen.alloc(n)) || (e = order.alloc(n)) || (e = tmp.alloc(n)) ||
      (e = dTasks.alloc(n)) || (e = dRes.alloc(n)) || (e = dBad.alloc(1)) || (e = dSegs.alloc(maxSegs)) ||
      (e = dTaskOf.alloc(maxWide)) || (e = dSegFirst.alloc(maxWide + 1)) || (e = dSegLeft.alloc(maxSegs)) ||
      (e = dSegOff.alloc(maxSegs)) || (e = dAcc.alloc(maxWide * 12)) || (e = dGb.alloc(maxWide * kBinWords)))
    return e;
  if ((e = cudaMemsetAsync(dBad.p, 0, sizeof(uint32_t), st))) return e;
  int blocks = (int)std::min<uint32_t>((n + 255) / 256, 4096u);
  k_prim_bounds<<<blocks, 256, 0, st>>>(prims, first, n, lo.p, hi.p, cen.p, order.p);
  if ((e = cudaGetLastError())) return e;
  std::vector<BNode> nodes(1);
  nodes.reserve(2 * (size_t)n / kLeafPrims + 64);  // a binary tree with at least ~kLeafPrims / 2 per leaf
  std::vector<Task> tasks = {Task{0, n, 0, 0}};  // wide flags set per level
  std::vector<int32_t> ids = {0};
  std::vector<TaskResult> res;
  std::vector<Task> next;
  std::vector<int32_t> nextIds;
  // nodes are created in batches (the root, then each level's children): a node's children are
  // in the batch after its own
  std::vector<size_t> batches = {0};
  int level = 0;
  for (; level < kMaxLevels && !tasks.empty(); level++) {
    const uint32_t nt = (uint32_t)tasks.size();
    // large ranges are binned and partitioned by several CTAs (segments of kSegment triangles)
    std::vector<uint32_t> taskOf, segFirst;
    std::vector<Segment> segs;
    for (uint32_t k = 0; k < nt; k++) {
      Task& t = tasks[k];
      t.wide = (t.end - t.begin > kWideMin && t.depth < kMedianDepth) ? 1u : 0u;
      if (!t.wide) continue;
      const uint32_t w = (uint32_t)taskOf.size();
      taskOf.push_back(k);
      segFirst.push_back((uint32_t)segs.size());
      for (uint32_t b = t.begin; b < t.end; b += kSegment) segs.push_back(Segment{k, w, b, std::min(t.end, b + kSegment)});
    }
    const uint32_t nwide = (uint32_t)taskOf.size(), nseg = (uint32_t)segs.size();
    segFirst.push_back(nseg);
    if ((e = cudaMemcpyAsync(dTasks.p, tasks.data(), nt * sizeof(Task), cudaMemcpyHostToDevice, st))) return e;
    if (nwide) {
      if ((e = cudaMemcpyAsync(dSegs.p, segs.data(), nseg * sizeof(Segment), cudaMemcpyHostToDevice, st)) ||
          (e = cudaMemcpyAsync(dTaskOf.p, taskOf.data(), nwide * sizeof(uint32_t), cudaMemcpyHostToDevice, st)) ||
          (e = cudaMemcpyAsync(dSegFirst.p, segFirst.data(), (nwide + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice,
                               st)))
        return e;
      k_wide_init<<<64, 256, 0, st>>>(nwide, dAcc.p, dGb.p);
      k_wide_bounds<<<nseg, kThreads, 0, st>>>(dSegs.p, lo.p, hi.p, cen.p, order.p, dAcc.p);
      k_wide_bin<<<nseg, kThreads, 0, st>>>(dSegs.p, lo.p, hi.p, cen.p, order.p, dAcc.p, dGb.p);
      k_wide_sah<<<(nwide + 31) / 32, 32, 0, st>>>(nwide, dTaskOf.p, dTasks.p, dAcc.p, dGb.p, dRes.p);
      if ((e = cudaGetLastError())) return e;
    }
    uint32_t largest = 0;
    for (const Task& t : tasks) largest = std::max(largest, t.end - t.begin);
    if (largest <= kSmallMax) {
      // only small ranges: a warp each
      const uint32_t blocks = (nt + kWarpTasks - 1) / kWarpTasks;
      k_sah_bin_warp<<<blocks, 32 * kWarpTasks, 0, st>>>(dTasks.p, nt, lo.p, hi.p, cen.p, order.p, dRes.p);
      if ((e = cudaGetLastError())) return e;
      k_sah_partition_warp<<<blocks, 32 * kWarpTasks, 0, st>>>(dTasks.p, nt, dRes.p, cen.p, order.p, tmp.p, dBad.p);
      if ((e = cudaGetLastError())) return e;
    } else {
      // a CTA per range, sized by the level's task count: the first levels hold few tasks of
      // many triangles
      const int threads = nt <= 2048 ? 1024 : (nt <= 32768 ? 256 : 64);
      k_sah_bin<<<nt, threads, 0, st>>>(dTasks.p, lo.p, hi.p, cen.p, order.p, dRes.p);
      if ((e = cudaGetLastError())) return e;
      k_sah_partition<<<nt, threads, 0, st>>>(dTasks.p, dRes.p, cen.p, order.p, tmp.p, dBad.p);
      if ((e = cudaGetLastError())) return e;
    }
    if (nwide) {
      k_wide_count<<<nseg, kThreads, 0, st>>>(dSegs.p, dTasks.p, dRes.p, cen.p, order.p, dSegLeft.p);
      k_wide_offsets<<<(nwide + 31) / 32, 32, 0, st>>>(nwide, dSegFirst.p, dTaskOf.p, dRes.p, dSegLeft.p, dSegOff.p,
                                                      dBad.p);
      k_wide_scatter<<<nseg, kThreads, 0, st>>>(dSegs.p, dTasks.p, dRes.p, cen.p, order.p, dSegOff.p, tmp.p);
      k_wide_copy<<<nseg, kThreads, 0, st>>>(dSegs.p, tmp.p, order.p, dBad.p);
      if ((e = cudaGetLastError())) return e;
    }
    res.resize(nt);
    if ((e = cudaMemcpyAsync(res.data(), dRes.p, nt * sizeof(TaskResult), cudaMemcpyDeviceToHost, st))) return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    // the level's results in parallel: each task's node, its two children (leaves the bins
    // already bound, or next-level tasks), at offsets from prefix sums over the tasks, so the
    // node and task order is that of a sequential pass over the tasks
    std::vector<uint32_t> kidTasks(nt + 1), kidNodes(nt + 1);
    std::atomic<bool> empty{false};
    auto childIsLeaf = [&](const Task& t, const TaskResult& r, int c) {
      const uint32_t len = c == 0 ? r.nLeft : (t.end - t.begin) - r.nLeft;
      return r.axis >= 0 && len <= kLeafPrims;
    };
    nehost::parallelFor(nt, 1u << 13, [&](size_t k0, size_t k1) {
      for (size_t k = k0; k < k1; k++) {
        const Task& t = tasks[k];
        const TaskResult& r = res[k];
        uint32_t nodesK = 0, tasksK = 0;
        if (!r.leaf) {
          if (r.nLeft == 0 || r.nLeft >= t.end - t.begin) empty = true;
          nodesK = 2;
          tasksK = (childIsLeaf(t, r, 0) ? 0u : 1u) + (childIsLeaf(t, r, 1) ? 0u : 1u);
        }
        kidNodes[k] = nodesK;
        kidTasks[k] = tasksK;
      }
    });
    if (empty) {
      err = "BVH build: empty child";
      return cudaErrorUnknown;
    }
    uint32_t sumN = 0, sumT = 0;
    for (uint32_t k = 0; k <= nt; k++) {  // exclusive scans; entry nt holds the totals
      const uint32_t a0 = k < nt ? kidNodes[k] : 0u, a1 = k < nt ? kidTasks[k] : 0u;
      kidNodes[k] = sumN;
      kidTasks[k] = sumT;
      sumN += a0;
      sumT += a1;
    }
    const size_t node0 = nodes.size();
    batches.push_back(node0);
    nodes.resize(node0 + sumN);
    next.resize(sumT);
    nextIds.resize(sumT);
    nehost::parallelFor(nt, 1u << 13, [&](size_t k0, size_t k1) {
      for (size_t k = k0; k < k1; k++) {
        const Task& t = tasks[k];
        const TaskResult& r = res[k];
        BNode& b = nodes[ids[k]];
        for (int j = 0; j < 3; j++) { b.mn[j] = r.mn[j]; b.mx[j] = r.mx[j]; }
        b.begin = t.begin;
        b.count = t.end - t.begin;
        b.left = b.right = -1;
        if (r.leaf) continue;
        const int32_t l = (int32_t)(node0 + kidNodes[k]);
        b.left = l;
        b.right = l + 1;
        uint32_t q = kidTasks[k];
        const uint32_t cBegin[2] = {t.begin, t.begin + r.nLeft}, cEnd[2] = {t.begin + r.nLeft, t.end};
        for (int c = 0; c < 2; c++) {
          if (childIsLeaf(t, r, c)) {
            // a small child of a binned split is a leaf whose bounds the bins already hold
            BNode& leaf = nodes[l + c];
            for (int j = 0; j < 3; j++) { leaf.mn[j] = r.cb[c][j]; leaf.mx[j] = r.cb[c][3 + j]; }
            leaf.begin = cBegin[c];
            leaf.count = cEnd[c] - cBegin[c];
            leaf.left = leaf.right = -1;
          } else {
            next[q] = Task{cBegin[c], cEnd[c], t.depth + 1, 0};
            nextIds[q] = l + c;
            q++;
          }
        }
      }
    });
    tasks.swap(next);
    ids.swap(nextIds);
  }
  if (!tasks.empty()) {
    err = "BVH build: deeper than 64 levels";
    return cudaErrorUnknown;
  }
  std::vector<uint32_t> ord(n);
  uint32_t bad = 0;
  if ((e = cudaMemcpyAsync(ord.data(), order.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st))) return e;
  if ((e = cudaMemcpyAsync(&bad, dBad.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st))) return e;
  if ((e = cudaStreamSynchronize(st))) return e;
  if (bad) {
    err = "BVH build: partition disagrees with the binning";
    return cudaErrorUnknown;
  }
  // depth-first layout: subtree sizes bottom-up (children follow their parent in `nodes`),
  // then positions top-down
  const size_t nn = nodes.size();
  std::vector<uint32_t> size(nn, 1), pos(nn, 0);
  batches.push_back(nn);
  for (size_t k = batches.size() - 1; k-- > 0;)  // batch by batch, the last first
    nehost::parallelFor(batches[k + 1] - batches[k], 1u << 14, [&](size_t i0, size_t i1) {
      for (size_t i = batches[k] + i0; i < batches[k] + i1; i++)
        if (nodes[i].left >= 0) size[i] = 1 + size[nodes[i].left] + size[nodes[i].right];
    });
  for (size_t k = 0; k + 1 < batches.size(); k++)
    nehost::parallelFor(batches[k + 1] - batches[k], 1u << 14, [&](size_t i0, size_t i1) {
      for (size_t i = batches[k] + i0; i < batches[k] + i1; i++)
        if (nodes[i].left >= 0) {
          pos[nodes[i].left] = pos[i] + 1;
          pos[nodes[i].right] = pos[i] + 1 + size[nodes[i].left];
        }
    });
  nodesOut.resize(nn);
  nehost::parallelFor(nn, 1u << 15, [&](size_t i0, size_t i1) {
    for (size_t i = i0; i < i1; i++) {
      const BNode& b = nodes[i];
      DNode d;
      for (int j = 0; j < 3; j++) { d.lo[j] = b.mn[j]; d.hi[j] = b.mx[j]; }
      uint32_t a, c;
      if (b.left < 0) {
        a = b.begin;
        c = b.count | 0x80000000u;
      } else {
        a = pos[b.right] - pos[i];
        c = 0;
      }
      memcpy(&d.lo[3], &a, 4);
      memcpy(&d.hi[3], &c, 4);
      nodesOut[pos[i]] = d;
    }
  });
  slotsOut.resize(n);
  nehost::parallelFor(n, 1u << 16, [&](size_t i0, size_t i1) {
    for (size_t i = i0; i < i1; i++) slotsOut[i] = first + ord[i];
  });
  return cudaSuccess;
}

}  // namespace nedev
