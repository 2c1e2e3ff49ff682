// Radiance-cache network on the fifth-generation tensor cores (tcgen05, BF16 in, FP32
// accumulate in tensor memory). See tc.cuh for the operand layout.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "mlp.h"
#include "tc.cuh"

using namespace netc;

namespace {

constexpr int kMmaThreads = 128;

__device__ __forceinline__ uint32_t tmem_cols_for(uint32_t n) {
  uint32_t c = 32;
  while (c < n) c <<= 1;
  return c;
}

// One 128 x n x k product through shared memory and tensor memory (known-answer kernel for
// the descriptor and TMEM conventions the network kernels use).
__global__ void __launch_bounds__(kMmaThreads) k_debug_mma(const uint16_t* __restrict__ A,
                                                           const uint16_t* __restrict__ B, uint32_t N, uint32_t K,
                                                           float* __restrict__ D, uint32_t* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  uint8_t* sA = smem;
  uint8_t* sB = smem + 128u * K * 2u;
  const uint32_t t = threadIdx.x;
  for (uint32_t i = t; i < 128u * K; i += kMmaThreads)
    *reinterpret_cast<uint16_t*>(sA + cm_offset(i / K, i % K, K)) = A[i];
  for (uint32_t i = t; i < N * K; i += kMmaThreads)
    *reinterpret_cast<uint16_t*>(sB + cm_offset(i / K, i % K, K)) = B[i];
  fence_smem_to_async();
  const uint32_t ncols = tmem_cols_for(N);
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  if (t < 32) {
    tmem_alloc(&tbase, ncols);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tb = tbase;
  if (t == 0) {
    const uint32_t id = idesc_bf16(128, N);
    for (uint32_t k = 0; k < K / 16; k++)
      mma_bf16(tb, tile_desc(smem_u32(sA), K, k), tile_desc(smem_u32(sB), K, k), id, k > 0 ? 1u : 0u);
    mma_commit(&bar);
  }
  bool ok = mbar_wait(&bar, 0);
  ok = __syncthreads_and(ok);
  fence_after_sync();
  if (ok) {
    const uint32_t w = t / 32;
    for (uint32_t c = 0; c < N; c += 16) {
      float v[16];
      tmem_ld16(tmem_at(tb, 32 * w, c), v);
      tmem_wait_ld();
#pragma unroll
      for (int j = 0; j < 16; j++) D[(size_t)t * N + c + j] = v[j];
    }
  } else if (t == 0) {
    atomicOr(err, 1u);
  }
  fence_before_sync();
  __syncthreads();
  if (t < 32) tmem_dealloc(tb, ncols);
}

// Failure-detection check of the bounded waits: the block allocates tensor memory and
// initialises an mbarrier exactly as the product kernels do, then waits for a completion
// that nothing signals (no MMA is issued, nobody arrives). The wait gives up after
// `max_polls` polls, the block sets err bit 1, releases its tensor memory and exits.
__global__ void __launch_bounds__(kMmaThreads) k_debug_wait(uint32_t max_polls, uint32_t* err) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  const uint32_t t = threadIdx.x;
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  if (t < 32) {
    tmem_alloc(&tbase, 32);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tb = tbase;
  bool ok = mbar_wait(&bar, 0, max_polls);
  ok = __syncthreads_and(ok);
  if (!ok && t == 0) atomicOr(err, 1u);
  fence_before_sync();
  __syncthreads();
  if (t < 32) tmem_dealloc(tb, 32);
}

}  // namespace

cudaError_t ne_launch_debug_wait(cudaStream_t st, uint32_t max_polls, uint32_t* err) {
  k_debug_wait<<<1, kMmaThreads, 0, st>>>(max_polls, err);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Network definition (identical to the CPU restatement used to check it).
//   features 96 -> 64 -> 64 -> 64 -> 64 -> 16 (RGB in rows 0..2), ReLU on hidden layers.
// Master parameters: FP32, layer l weights W_l[out][in] then bias b_l[out], layers in order.
// Packed BF16 copies for the tensor core (K-major core-matrix tiles, see tc.cuh):
//   forward  tile of layer l:      B operand W_l   [out rows x in cols]
//   backward tile of layer l >= 1: B operand W_l^T [in rows x out cols] (for dX = G * W)
// ---------------------------------------------------------------------------------------
namespace {

constexpr int kLayers = 5;
__constant__ int cIn[kLayers] = {96, 64, 64, 64, 64};
__constant__ int cOut[kLayers] = {64, 64, 64, 64, 16};
__constant__ int cWOff[kLayers] = {0, 6208, 10368, 14528, 18688};
__constant__ int cBOff[kLayers] = {6144, 10304, 14464, 18624, 19712};
__constant__ int cFwdOff[kLayers] = {0, 12288, 20480, 28672, 36864};   // bytes
__constant__ int cBwdOff[kLayers] = {0, 18432, 10240, 2048, 0};        // bytes, layers 1..4
constexpr int kFwdBytes = 38912;
constexpr int kBwdBytes = 26624;
constexpr int kBiasFloats = 272;  // 4 x 64 + 16
constexpr int kTile = 128;

__device__ __forceinline__ int biasIndex(int l) { return l * 64; }

// Feature encoding of one query (96 values, 88 used): sin/cos of pi * scalar, then each
// further band by angle doubling (sin 2x = 2 sin x cos x, cos 2x = cos^2 x - sin^2 x).
__device__ void encodeQuery(float px, float py, float pz, float wx, float wy, float wz, float* f) {
  const float kPi = 3.14159265358979323846f;
  float wyc = fminf(fmaxf(wy, -1.0f), 1.0f);
  float a = acosf(wyc) / kPi;
  float b = atan2f(wz, wx) / (2.0f * kPi) + 0.5f;
  const float v[5] = {px + 0.5f, py + 0.5f, pz + 0.5f, a, b};
  int col = 0;
#pragma unroll
  for (int s = 0; s < 5; s++) {
    const int bands = s < 3 ? 12 : 4;
    float sn, cs;
    sincosf(__fmul_rn(kPi, v[s]), &sn, &cs);
#pragma unroll
    for (int k = 0; k < bands; k++) {
      f[col] = sn;
      f[col + 1] = cs;
      col += 2;
      float s2 = __fmul_rn(__fmul_rn(2.0f, sn), cs);
      float c2 = __fsub_rn(__fmul_rn(cs, cs), __fmul_rn(sn, sn));
      sn = s2;
      cs = c2;
    }
  }
#pragma unroll
  for (int c = 88; c < 96; c++) f[c] = 0.0f;
}

// Stores 8 consecutive BF16 values (columns c..c+7 of row r) into a core-matrix tile.
__device__ __forceinline__ void storeRow8(uint8_t* tile, uint32_t r, uint32_t c, uint32_t kcols, const float* v) {
  uint32_t w[4];
#pragma unroll
  for (int i = 0; i < 4; i++) w[i] = f2bf2(v[2 * i], v[2 * i + 1]);
  *reinterpret_cast<uint4*>(tile + cm_offset(r, c, kcols)) = make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void k_mlp_encode(const float* __restrict__ pos, const float* __restrict__ dir, uint32_t n,
                             float* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float f[96];
    encodeQuery(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], dir[3 * i], dir[3 * i + 1], dir[3 * i + 2], f);
    for (int c = 0; c < 96; c++) out[(size_t)i * 96 + c] = f[c];
  }
}

// FP32 master parameters -> packed BF16 tiles and the FP32 bias table.
__global__ void k_mlp_pack(const float* __restrict__ P, uint8_t* __restrict__ fwd, uint8_t* __restrict__ bwd,
                           float* __restrict__ bias) {
  for (int l = 0; l < kLayers; l++) {
    const int in = cIn[l], out = cOut[l];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < in * out; i += gridDim.x * blockDim.x) {
      int o = i / in, k = i % in;
      uint16_t h = f2bf(P[cWOff[l] + i]);
      *reinterpret_cast<uint16_t*>(fwd + cFwdOff[l] + cm_offset(o, k, in)) = h;
      if (l >= 1) *reinterpret_cast<uint16_t*>(bwd + cBwdOff[l] + cm_offset(k, o, out)) = h;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < out; i += gridDim.x * blockDim.x)
      bias[biasIndex(l) + i] = P[cBOff[l] + i];
  }
}

struct FwdArgs {
  const float* pos;      // n x 3, medium object space
  const float* dir;      // n x 3, unit
  const float* feats;    // n x 96 precomputed features, or null (encode pos/dir)
  uint32_t n;
  const uint32_t* n_dev; // optional device count: the kernel runs min(*n_dev, n) queries
  const uint8_t* wfwd;   // packed forward tiles
  const float* bias;     // 272 floats
  float* out;            // n x 3 raw RGB outputs, or null
  uint16_t* acts;        // training: n x (96 + 4 x 64) BF16 layer inputs, or null
  const float* thr;      // optional n x 3 path throughput: radiance[idx[i]] += thr * max(out, 0)
  const uint32_t* idx;
  float* radiance;
};

constexpr uint32_t kActRow = 96 + 4 * 64;  // BF16 values stored per training sample

// Persistent fused forward pass: each block runs tiles of 128 queries through all five
// layers, activations staying in shared memory and accumulators in tensor memory.
__global__ void __launch_bounds__(kTile) k_mlp_forward(const FwdArgs a, uint32_t* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  __shared__ float sBias[kBiasFloats];
  uint8_t* sW = smem;                    // kFwdBytes
  uint8_t* sX = smem + kFwdBytes;        // 128 x 96 BF16: the encoded input, then each layer's output
  uint8_t* sH = sX;                      // (a layer's product has completed before its output is stored)
  const uint32_t t = threadIdx.x, warp = t / 32;
  for (uint32_t i = t; i < kFwdBytes / 16; i += kTile)
    reinterpret_cast<uint4*>(sW)[i] = reinterpret_cast<const uint4*>(a.wfwd)[i];
  for (uint32_t i = t; i < kBiasFloats; i += kTile) sBias[i] = a.bias[i];
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&tbase, 64);
    tmem_relinquish();
  }
  fence_smem_to_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tb = tbase;
  const uint32_t tl = tmem_at(tb, 32 * warp, 0);
  uint32_t phase = 0;
  bool ok = true;
  const uint32_t n = a.n_dev ? min(*a.n_dev, a.n) : a.n;
  const uint32_t nTiles = (n + kTile - 1) / kTile;
  for (uint32_t tile = blockIdx.x; tile < nTiles && ok; tile += gridDim.x) {
    const uint32_t row = tile * kTile + t;
    const bool valid = row < n;
    {
      float f[96];
      if (!valid) {
        for (int c = 0; c < 96; c++) f[c] = 0.0f;
      } else if (a.feats) {
        for (int c = 0; c < 96; c++) f[c] = a.feats[(size_t)row * 96 + c];
      } else {
        encodeQuery(a.pos[3 * row], a.pos[3 * row + 1], a.pos[3 * row + 2], a.dir[3 * row], a.dir[3 * row + 1],
                    a.dir[3 * row + 2], f);
      }
      for (int c = 0; c < 96; c += 8) storeRow8(sX, t, c, 96, f + c);
      if (a.acts && valid) {
        uint32_t* dst = reinterpret_cast<uint32_t*>(a.acts + (size_t)row * kActRow);
        for (int c = 0; c < 96; c += 2) dst[c / 2] = f2bf2(f[c], f[c + 1]);
      }
    }
    float o16[16];
    for (int l = 0; l < kLayers; l++) {
      const int in = cIn[l], out = cOut[l];
      const uint8_t* sA = (l == 0) ? sX : sH;
      fence_smem_to_async();
      fence_before_sync();
      __syncthreads();
      if (t == 0) {
        fence_after_sync();
        const uint32_t id = idesc_bf16(128, (uint32_t)out);
        for (int k = 0; k < in / 16; k++)
          mma_bf16(tb, tile_desc(smem_u32(sA), in, k), tile_desc(smem_u32(sW + cFwdOff[l]), in, k), id,
                   k > 0 ? 1u : 0u);
        mma_commit(&bar);
      }
      bool done = mbar_wait(&bar, phase);
      phase ^= 1u;
      ok = __syncthreads_and(done);
      if (!ok) break;
      fence_after_sync();
      if (l < kLayers - 1) {
        for (int c = 0; c < 64; c += 16) {
          float v[16];
          tmem_ld16(tl + c, v);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] = fmaxf(v[j] + sBias[biasIndex(l) + c + j], 0.0f);
          storeRow8(sH, t, c, 64, v);
          storeRow8(sH, t, c + 8, 64, v + 8);
          if (a.acts && valid) {
            uint32_t* dst = reinterpret_cast<uint32_t*>(a.acts + (size_t)row * kActRow + 96 + l * 64 + c);
#pragma unroll
            for (int j = 0; j < 8; j++) dst[j] = f2bf2(v[2 * j], v[2 * j + 1]);
          }
        }
      } else {
        tmem_ld16(tl, o16);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; j++) o16[j] += sBias[biasIndex(l) + j];
      }
    }
    if (!ok) break;
    if (valid) {
      if (a.out) {
        a.out[3 * row] = o16[0];
        a.out[3 * row + 1] = o16[1];
        a.out[3 * row + 2] = o16[2];
      }
      if (a.radiance) {
        uint32_t p = a.idx[row];
        for (int c = 0; c < 3; c++) a.radiance[3 * (size_t)p + c] += a.thr[3 * row + c] * fmaxf(o16[c], 0.0f);
      }
    }
  }
  if (!ok && t == 0) atomicOr(err, 2u);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tb, 64);
}

struct BwdArgs {
  const uint16_t* acts;   // n x kActRow BF16 layer inputs from the forward pass
  const float* out;       // n x 3 raw outputs from the forward pass
  const float* target;    // n x 3
  uint32_t n;
  float inv_count;        // 1 / (3 n)
  const uint8_t* wbwd;    // packed backward tiles
  float* part;            // gridDim.x x kParams partial gradients (master-parameter layout)
  float* loss_part;       // gridDim.x partial sums of the relative L2 terms
};

constexpr int kParams = 19728;
constexpr uint32_t kBwdCols = 512;
__constant__ int cDWCol[kLayers] = {320, 256, 192, 128, 64};  // TMEM column of each dW^T accumulator

__device__ __forceinline__ int actOffset(int l) { return l == 0 ? 0 : 96 + (l - 1) * 64; }

// Loads this sample's input of layer l into the transposed tile sXT (rows = features,
// columns = the block's 128 samples) and returns its "> 0" mask (the ReLU that made it).
__device__ __forceinline__ unsigned long long loadInputT(const BwdArgs& a, uint8_t* sXT, int l, uint32_t t,
                                                         uint32_t row, bool valid) {
  const int in = cIn[l];
  unsigned long long mask = 0;
  const uint16_t* src = a.acts + (size_t)row * kActRow + actOffset(l);
  for (int i = 0; i < in; i++) {
    uint16_t h = valid ? src[i] : (uint16_t)0;
    *reinterpret_cast<uint16_t*>(sXT + cm_offset(i, t, 128)) = h;
    if (i < 64 && bf2f(h) > 0.0f) mask |= 1ull << i;
  }
  return mask;
}

// Writes this sample's error signal g (out values) as row t of sG (K = out) and as column t
// of the transposed tile sGT (rows = outputs, columns = samples), both BF16.
__device__ __forceinline__ void storeGrad(uint8_t* sG, uint8_t* sGT, uint32_t t, int out, const float* g) {
  for (int c = 0; c < out; c += 8) storeRow8(sG, t, c, out, g + c);
  for (int o = 0; o < out; o++) *reinterpret_cast<uint16_t*>(sGT + cm_offset(o, t, 128)) = f2bf(g[o]);
}

__device__ __forceinline__ float warpSum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Persistent backward pass: per tile of 128 samples, output-layer error -> for each layer
// (last to first) weight-gradient product dW^T += X^T G^T accumulated in tensor memory
// across the block's tiles, and the error product dX = G W with the ReLU mask. The
// block's sums are written once at the end (deterministic reduction in k_mlp_adam).
__global__ void __launch_bounds__(kTile) k_mlp_backward(const BwdArgs a, uint32_t* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  __shared__ float sDb[kBiasFloats];
  __shared__ float sLoss[4];
  uint8_t* sWT = smem;                  // kBwdBytes
  uint8_t* sG = sWT + kBwdBytes;        // 128 x 64
  uint8_t* sGT = sG + kTile * 64 * 2;   // 64 x 128
  uint8_t* sXT = sGT + 64 * kTile * 2;  // 128 x 128
  const uint32_t t = threadIdx.x, warp = t / 32, lane = t % 32;
  for (uint32_t i = t; i < kBwdBytes / 16; i += kTile)
    reinterpret_cast<uint4*>(sWT)[i] = reinterpret_cast<const uint4*>(a.wbwd)[i];
  for (uint32_t i = t; i < kBiasFloats; i += kTile) sDb[i] = 0.0f;
  // rows 96..127 of the transposed input tile are never written by a layer: zero them once
  for (uint32_t i = t; i < 32 * kTile; i += kTile)
    *reinterpret_cast<uint16_t*>(sXT + cm_offset(96 + i / kTile, i % kTile, 128)) = 0;
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&tbase, kBwdCols);
    tmem_relinquish();
  }
  fence_smem_to_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tb = tbase;
  const uint32_t tl = tmem_at(tb, 32 * warp, 0);
  uint32_t phase = 0;
  bool ok = true, first = true;
  float lossAcc = 0.0f;
  const uint32_t nTiles = (a.n + kTile - 1) / kTile;
  for (uint32_t tile = blockIdx.x; tile < nTiles && ok; tile += gridDim.x) {
    const uint32_t row = tile * kTile + t;
    const bool valid = row < a.n;
    float g[64];
    for (int c = 0; c < 16; c++) g[c] = 0.0f;
    if (valid) {
      for (int c = 0; c < 3; c++) {
        float y = a.out[3 * row + c], tg = a.target[3 * row + c];
        float den = y * y + 0.01f;
        float d = y - tg;
        g[c] = 2.0f * d / den * a.inv_count;
        lossAcc += d * d / den;
      }
    }
    int l = kLayers - 1;
    storeGrad(sG, sGT, t, 16, g);
    for (int c = 0; c < 3; c++) {
      float s = warpSum(g[c]);
      if (lane == 0) atomicAdd(&sDb[biasIndex(l) + c], s);
    }
    unsigned long long mask = loadInputT(a, sXT, l, t, row, valid);
    for (; l >= 0; l--) {
      const int in = cIn[l], out = cOut[l];
      fence_smem_to_async();
      fence_before_sync();
      __syncthreads();
      if (t == 0) {
        fence_after_sync();
        if (l >= 1) {
          const uint32_t id = idesc_bf16(128, (uint32_t)in);
          for (int k = 0; k < out / 16; k++)
            mma_bf16(tb, tile_desc(smem_u32(sG), out, k), tile_desc(smem_u32(sWT + cBwdOff[l]), out, k), id,
                     k > 0 ? 1u : 0u);
        }
        const uint32_t idw = idesc_bf16(128, (uint32_t)out);
        for (int k = 0; k < kTile / 16; k++)
          mma_bf16(tb + cDWCol[l], tile_desc(smem_u32(sXT), 128, k), tile_desc(smem_u32(sGT), 128, k), idw,
                   (first && k == 0) ? 0u : 1u);
        mma_commit(&bar);
      }
      bool done = mbar_wait(&bar, phase);
      phase ^= 1u;
      ok = __syncthreads_and(done);
      if (!ok) break;
      if (l == 0) break;
      fence_after_sync();
      // error of layer l-1 = (G W_l) masked by the ReLU that produced layer l's input
      for (int c = 0; c < 64; c += 16) {
        float v[16];
        tmem_ld16(tl + c, v);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; j++) g[c + j] = ((mask >> (c + j)) & 1ull) ? v[j] : 0.0f;
      }
      for (int c = 0; c < 64; c++) {
        float s = warpSum(g[c]);
        if (lane == 0) atomicAdd(&sDb[biasIndex(l - 1) + c], s);
      }
      storeGrad(sG, sGT, t, 64, g);
      mask = loadInputT(a, sXT, l - 1, t, row, valid);
    }
    first = false;
  }
  if (!ok && t == 0) atomicOr(err, 4u);
  // block results: dW (from tensor memory, transposed back to [out][in]), db, loss
  float* part = a.part + (size_t)blockIdx.x * kParams;
  fence_after_sync();
  for (int l = 0; l < kLayers; l++) {
    const int in = cIn[l], out = cOut[l];
    for (int c = 0; c < out; c += 16) {
      float v[16];
      if (ok && !first) {
        tmem_ld16(tl + cDWCol[l] + c, v);
        tmem_wait_ld();
      } else {
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = 0.0f;
      }
      if ((int)t < in)
        for (int j = 0; j < 16; j++) part[cWOff[l] + (c + j) * in + t] = v[j];
    }
  }
  __syncthreads();
  for (int l = 0; l < kLayers; l++)
    for (int o = t; o < cOut[l]; o += kTile) part[cBOff[l] + o] = sDb[biasIndex(l) + o];
  float ls = warpSum(lossAcc);
  if (lane == 0) sLoss[warp] = ls;
  __syncthreads();
  if (t == 0) a.loss_part[blockIdx.x] = (sLoss[0] + sLoss[1]) + (sLoss[2] + sLoss[3]);
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tb, kBwdCols);
}

// Sums the blocks' partial gradients in block order and applies one Adam step to the FP32
// master parameters (lr, beta1, beta2, eps as the CPU restatement).
__global__ void k_mlp_adam(float* __restrict__ P, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ part, int nParts, const float* __restrict__ loss_part,
                           float* __restrict__ grad_out, float* __restrict__ loss_out, float lr, float c1, float c2,
                           int apply) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kParams; p += gridDim.x * blockDim.x) {
    float g = 0.0f;
    for (int c = 0; c < nParts; c++) g += part[(size_t)c * kParams + p];
    if (grad_out) grad_out[p] = g;
    if (apply) {
      float mm = 0.9f * m[p] + 0.1f * g;
      float vv = 0.99f * v[p] + 0.01f * g * g;
      m[p] = mm;
      v[p] = vv;
      P[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + 1e-8f);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && loss_out) {
    float s = 0.0f;
    for (int c = 0; c < nParts; c++) s += loss_part[c];
    *loss_out = s;
  }
}

}  // namespace


namespace {
int g_sms = 0;
int smCount() {
  if (!g_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 1;
  }
  return g_sms;
}
}  // namespace

cudaError_t ne_mlp_encode(cudaStream_t st, const float* pos, const float* dir, uint32_t n, float* feats) {
  if (!n) return cudaSuccess;
  int blocks = (int)((n + 127) / 128);
  if (blocks > smCount() * 8) blocks = smCount() * 8;
  k_mlp_encode<<<blocks, 128, 0, st>>>(pos, dir, n, feats);
  return cudaGetLastError();
}

cudaError_t ne_mlp_pack(cudaStream_t st, const float* params, uint8_t* wfwd, uint8_t* wbwd, float* bias) {
  k_mlp_pack<<<16, 256, 0, st>>>(params, wfwd, wbwd, bias);
  return cudaGetLastError();
}

cudaError_t ne_mlp_forward(cudaStream_t st, const NeMlpForward& f, uint32_t* err) {
  if (!f.n) return cudaSuccess;
  FwdArgs a;
  a.pos = f.pos;
  a.dir = f.dir;
  a.feats = f.feats;
  a.n = f.n;
  a.n_dev = f.n_dev;
  a.wfwd = f.wfwd;
  a.bias = f.bias;
  a.out = f.out;
  a.acts = f.acts;
  a.thr = f.thr;
  a.idx = f.idx;
  a.radiance = f.radiance;
  const size_t smem = kFwdBytes + (size_t)kTile * 96 * 2;
  cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  uint32_t tiles = (f.n + kTile - 1) / kTile;
  uint32_t blocks = tiles < (uint32_t)smCount() * 3 ? tiles : (uint32_t)smCount() * 3;
  k_mlp_forward<<<blocks, kTile, smem, st>>>(a, err);
  return cudaGetLastError();
}

int ne_mlp_backward_blocks(uint32_t n) {
  uint32_t tiles = (n + kTile - 1) / kTile;
  return (int)(tiles < (uint32_t)smCount() ? tiles : (uint32_t)smCount());
}

cudaError_t ne_mlp_backward(cudaStream_t st, const NeMlpBackward& b, uint32_t* err) {
  if (!b.n) return cudaSuccess;
  BwdArgs a;
  a.acts = b.acts;
  a.out = b.out;
  a.target = b.target;
  a.n = b.n;
  a.inv_count = 1.0f / (3.0f * (float)b.n);
  a.wbwd = b.wbwd;
  a.part = b.part;
  a.loss_part = b.loss_part;
  const size_t smem = kBwdBytes + (size_t)kTile * 64 * 2 + (size_t)64 * kTile * 2 + (size_t)kTile * kTile * 2;
  cudaError_t e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_mlp_backward<<<ne_mlp_backward_blocks(b.n), kTile, smem, st>>>(a, err);
  return cudaGetLastError();
}

cudaError_t ne_mlp_adam(cudaStream_t st, float* params, float* m, float* v, const float* part, int parts,
                        const float* loss_part, float* grad_out, float* loss_out, float lr, int step, int apply) {
  float c1 = (float)(1.0 - pow(0.9, (double)step));
  float c2 = (float)(1.0 - pow(0.99, (double)step));
  k_mlp_adam<<<(kParams + 255) / 256, 256, 0, st>>>(params, m, v, part, parts, loss_part, grad_out, loss_out, lr, c1,
                                                     c2, apply);
  return cudaGetLastError();
}

cudaError_t ne_launch_debug_mma(cudaStream_t st, const uint16_t* a, const uint16_t* b, int n, int k, float* d,
                                uint32_t* err) {
  size_t smem = (size_t)(128 + n) * k * 2;
  cudaError_t e = cudaFuncSetAttribute(k_debug_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_debug_mma<<<1, kMmaThreads, smem, st>>>(a, b, (uint32_t)n, (uint32_t)k, d, err);
  return cudaGetLastError();
}
