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

// The same product with either operand in the MN-major layout (layout bit 0: A, bit 1: B),
// read through mn_desc. n, k <= 64; the operand regions are 64 KB each, well beyond what the
// descriptors address.
constexpr uint32_t kMnRegion = 65536;
__global__ void __launch_bounds__(kMmaThreads) k_debug_mma_mn(const uint16_t* __restrict__ A,
                                                              const uint16_t* __restrict__ B, uint32_t N, uint32_t K,
                                                              uint32_t layout, float* __restrict__ D, uint32_t* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  uint8_t* sA = smem;
  uint8_t* sB = smem + kMnRegion;
  const uint32_t t = threadIdx.x;
  const bool aMn = layout & 1u, bMn = layout & 2u;
  for (uint32_t i = t; i < 2 * kMnRegion / 16; i += kMmaThreads) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  for (uint32_t i = t; i < 128u * K; i += kMmaThreads)
    *reinterpret_cast<uint16_t*>(sA + (aMn ? mn_offset(i / K, i % K, 128) : cm_offset(i / K, i % K, K))) = A[i];
  for (uint32_t i = t; i < N * K; i += kMmaThreads)
    *reinterpret_cast<uint16_t*>(sB + (bMn ? mn_offset(i / K, i % K, N) : cm_offset(i / K, i % K, K))) = B[i];
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
    const uint32_t id = idesc_bf16(128, N) | (aMn ? kIdescAMn : 0u) | (bMn ? kIdescBMn : 0u);
    for (uint32_t k = 0; k < K / 16; k++) {
      const uint64_t da = aMn ? mn_desc(smem_u32(sA), 128, k) : tile_desc(smem_u32(sA), K, k);
      const uint64_t db = bMn ? mn_desc(smem_u32(sB), N, k) : tile_desc(smem_u32(sB), K, k);
      mma_bf16(tb, da, db, id, k > 0 ? 1u : 0u);
    }
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
  uint8_t* acts;         // training: each tile's layer inputs (kActTileBytes per tile), or null
  const float* thr;      // optional n x 3 path throughput: radiance[idx[i]] += thr * max(out, 0)
  const uint32_t* idx;
  float* radiance;
};

// A layer's input tile, as the products read it: 128 samples x xcols(l) BF16 columns in the
// K-major core-matrix layout, the layer's `in` features, then a chunk of 8 holding 1.0 and 7
// zeros (the forward products stop at `in`; the weight-gradient product reads the 1.0 as
// the bias row). Training stores each tile's five inputs one after another, kActTileBytes per
// tile, for the backward pass to copy back whole.
__host__ __device__ constexpr int xcols(int l) { return l == 0 ? 104 : 72; }
__host__ __device__ constexpr uint32_t xTileBytes(int l) { return 128u * (uint32_t)xcols(l) * 2u; }
__host__ __device__ constexpr uint32_t actTileOff(int l) { return l == 0 ? 0u : xTileBytes(0) + (uint32_t)(l - 1) * xTileBytes(1); }
constexpr size_t kActTileBytes = xTileBytes(0) + 4 * (size_t)xTileBytes(1);
static_assert(kActTileBytes == kNeMlpActTileBytes, "activation tile size");

// Row r's ones chunk of an input tile with `cols` columns (at column cols - 8).
__device__ __forceinline__ void storeOnes(uint8_t* tile, uint32_t r, uint32_t cols) {
  *reinterpret_cast<uint4*>(tile + cm_offset(r, cols - 8, cols)) = make_uint4(0x3f80u, 0u, 0u, 0u);
}

// Persistent fused forward pass: each block runs tiles of 128 queries through all five
// layers, activations staying in shared memory and accumulators in tensor memory.
__global__ void __launch_bounds__(kTile) k_mlp_forward(const FwdArgs a, uint32_t* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tbase;
  __shared__ float sBias[kBiasFloats];
  uint8_t* sW = smem;                    // kFwdBytes
  uint8_t* sX = smem + kFwdBytes;        // the layer-0 input tile, then each layer's output
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
      for (int c = 0; c < 96; c += 8) storeRow8(sX, t, c, xcols(0), f + c);
      storeOnes(sX, t, xcols(0));
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
          mma_bf16(tb, tile_desc(smem_u32(sA), xcols(l), k), tile_desc(smem_u32(sW + cFwdOff[l]), in, k), id,
                   k > 0 ? 1u : 0u);
        mma_commit(&bar);
        // training: the input tile goes to global memory whole, while the product runs
        if (a.acts) bulk_store(a.acts + (size_t)tile * kActTileBytes + actTileOff(l), sA, xTileBytes(l));
      }
      bool done = mbar_wait(&bar, phase);
      phase ^= 1u;
      // the next layer's stores overwrite the tile: the copy must have read it
      if (t == 0 && a.acts) bulk_wait_read();
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
          storeRow8(sH, t, c, xcols(l + 1), v);
          storeRow8(sH, t, c + 8, xcols(l + 1), v + 8);
        }
        storeOnes(sH, t, xcols(l + 1));
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
  if (t == 0 && a.acts) bulk_wait();
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tb, 64);
}

struct BwdArgs {
  const uint8_t* acts;    // the forward pass's activation tiles (kActTileBytes per tile)
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
// Tiles in flight per block: each epilogue warpgroup owns one, so one group's epilogue runs
// while the tensor core works on the other's products.
constexpr int kBwdGroups = 2;
constexpr int kBwdThreads = kBwdGroups * 128 + 32;  // the groups, then the MMA-issuing warp
// Tensor memory: each group's error product dX (64 columns) at 64 g, then the weight-gradient
// accumulators dW^T of layers 4..0 (features, plus the bias row, in lanes; outputs in columns).
__constant__ int cDWCol[kLayers] = {448, 384, 320, 256, 192};
constexpr uint32_t kGBytes = 128 * 64 * 2;  // a group's error tile: 128 samples x <= 64 outputs
// A group's input-tile buffers: round k's tile is requested when round k - (kXBufs - 1)
// completes, while later rounds' products run. Each buffer has room past the largest tile for what the
// weight-gradient product's descriptor addresses beyond it (see xT_desc).
constexpr uint32_t kXBufs = 3;
constexpr uint32_t kXBuf = xTileBytes(0) + 1024;
constexpr uint32_t kGroupBytes = kGBytes + kXBufs * kXBuf;
constexpr size_t kBwdSmem = kBwdBytes + (size_t)kBwdGroups * kGroupBytes;

__device__ __forceinline__ float warpSum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Descriptor of the k-th K=16 slice of the weight-gradient product's A operand [X 1]^T
// (M = features, K = the tile's samples), read MN-major from an input tile stored K-major
// with `cols` columns: the next 8 samples are cols * 16 bytes on, the next 8 features 128
// bytes on. M is 128: rows past the tile's columns read the next samples' values (or, for the
// last 8 samples, the buffer's spare bytes) and only fill accumulator lanes nobody reads.
__device__ __forceinline__ uint64_t xT_desc(uint32_t tile_saddr, uint32_t cols, uint32_t kstep) {
  return smem_desc(tile_saddr + kstep * 2u * cols * 16u, cols * 16u, 128u);
}

// Round k of a group: its (k / 5)-th tile's layer 4 - k % 5; the input tile comes into buffer
// k % kXBufs, that buffer's (k / kXBufs)-th fill.
__device__ __forceinline__ int roundLayer(uint32_t k) { return kLayers - 1 - (int)(k % kLayers); }
__device__ __forceinline__ uint32_t fillParity(uint32_t k) { return (k / kXBufs) & 1u; }

// Persistent backward pass. kBwdGroups epilogue warpgroups each run their own tiles of 128
// samples: output-layer error, then for each layer (last to first) the weight-gradient
// product dW^T += [X 1]^T G (features and the bias row against outputs, accumulated in tensor
// memory over the block's tiles) and the error product dX = G W with the ReLU mask. A
// group's input tiles come whole from the forward pass's activations by the bulk copy engine,
// one layer ahead. The group writes its error tile (one row per sample), arrives on its
// `ready` barrier and waits on its `done` barrier; the issuing warp takes the groups in turn,
// issues their products and commits each group's to its `done`. The error tile is read both
// ways: as the K-major A of dX and the MN-major B of dW. The block's sums are written once at
// the end (deterministic reduction in k_mlp_adam).
__global__ void __launch_bounds__(kBwdThreads) k_mlp_backward(const BwdArgs a, uint32_t* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t ready[kBwdGroups], done[kBwdGroups], xfull[kBwdGroups][kXBufs], fin;
  __shared__ uint32_t tbase;
  __shared__ float sLoss[kBwdThreads / 32];
  __shared__ int sFail;
  uint8_t* sWT = smem;  // kBwdBytes
  const uint32_t t = threadIdx.x, warp = t / 32, lane = t % 32;
  for (uint32_t i = t; i < kBwdBytes / 16; i += kBwdThreads)
    reinterpret_cast<uint4*>(sWT)[i] = reinterpret_cast<const uint4*>(a.wbwd)[i];
  if (t == 0) {
    for (int g = 0; g < kBwdGroups; g++) {
      mbar_init(&ready[g], 128);
      mbar_init(&done[g], 1);
      for (uint32_t b = 0; b < kXBufs; b++) mbar_init(&xfull[g][b], 1);
    }
    mbar_init(&fin, 1);
    mbar_fence_init();
    sFail = 0;
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
  const uint32_t nTiles = (a.n + kTile - 1) / kTile;
  const uint32_t stride = gridDim.x * kBwdGroups;
  float lossAcc = 0.0f;
  bool ok = true;
  if (warp < kBwdGroups * 4) {
    // ---- epilogue group g, sample row r of its tiles
    const uint32_t g = warp / 4, r = t % 128;
    uint8_t* sG = smem + kBwdBytes + g * kGroupBytes;
    uint8_t* sXb = sG + kGBytes;  // buffer b at sXb + b * kXBuf
    const uint32_t tl = tmem_at(tb, 32 * (warp % 4), 0) + 64 * g;  // this thread's lane, the group's dX
    const uint32_t first = blockIdx.x * kBwdGroups + g;
    const uint32_t rounds = first < nTiles ? 5u * ((nTiles - first + stride - 1) / stride) : 0u;
    uint32_t rnd = 0;
    uint32_t fills = 0;  // row 0: input tiles requested so far (round k's is the k-th)
    // row 0 requests round k's input tile
    auto fill = [&](uint32_t k) {
      const uint32_t ft = first + (k / kLayers) * stride;
      const int fl = roundLayer(k);
      bulk_load(sXb + (k % kXBufs) * kXBuf, a.acts + (size_t)ft * kActTileBytes + actTileOff(fl), xTileBytes(fl),
                &xfull[g][k % kXBufs]);
      fills++;
    };
    if (r == 0)
      for (uint32_t k = 0; k < kXBufs - 1 && k < rounds; k++) fill(k);
    uint32_t tile = first;
    for (; tile < nTiles && ok; tile += stride) {
      const uint32_t row = tile * kTile + r;
      const bool valid = row < a.n;
      float gv[16];
#pragma unroll
      for (int c = 0; c < 16; c++) gv[c] = 0.0f;
      if (valid) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
          float y = a.out[3 * row + c], tg = a.target[3 * row + c];
          float den = y * y + 0.01f;
          float d = y - tg;
          gv[c] = 2.0f * d / den * a.inv_count;
          lossAcc += d * d / den;
        }
      }
      storeRow8(sG, r, 0, 16, gv);
      storeRow8(sG, r, 8, 16, gv + 8);
      for (int l = kLayers - 1; l >= 0; l--) {
        uint8_t* sX = sXb + (rnd % kXBufs) * kXBuf;
        // this layer's input tile
        bool got = mbar_wait(&xfull[g][rnd % kXBufs], fillParity(rnd));
        fence_smem_to_async();
        fence_before_sync();
        mbar_arrive(&ready[g]);
        // warp-uniform, so the aligned tensor-memory loads below run on whole warps
        got = __all_sync(0xffffffffu, got && mbar_wait(&done[g], rnd & 1u));
        if (!got) {
          rnd++;
          ok = false;
          break;
        }
        // a later round's input tile into the buffer the previous round used: its products
        // completed before this round's, and every row read its ReLU mask from it before
        // arriving for this round, which this round's completion implies
        if (r == 0 && rnd + kXBufs - 1 < rounds) fill(rnd + kXBufs - 1);
        rnd++;
        fence_after_sync();
        if (l == 0) break;
        // error of layer l-1 = (G W_l) masked by the ReLU that produced layer l's input: where
        // this row's input value is > 0 (as a BF16 bit pattern read as a signed integer: +0,
        // -0 and negatives are not), stored as the next round's error tile
        float v[64];
#pragma unroll
        for (int c = 0; c < 64; c += 16) tmem_ld16(tl + c, v + c);
        tmem_wait_ld();
#pragma unroll
        for (int c = 0; c < 64; c += 8) {
          const uint4 x = *reinterpret_cast<const uint4*>(sX + cm_offset(r, c, xcols(l)));
          const uint32_t xw[4] = {x.x, x.y, x.z, x.w};
          uint32_t o[4];
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const float lo = (int32_t)(xw[j] << 16) > 0 ? v[c + 2 * j] : 0.0f;
            const float hi = (int32_t)(xw[j] & 0xffff0000u) > 0 ? v[c + 2 * j + 1] : 0.0f;
            o[j] = f2bf2(lo, hi);
          }
          *reinterpret_cast<uint4*>(sG + cm_offset(r, c, 64)) = make_uint4(o[0], o[1], o[2], o[3]);
        }
      }
    }
    // a round that failed may leave a copy in flight: it must land before the block exits
    if (r == 0)
      for (uint32_t k = rnd; k < fills; k++)
        if (!mbar_wait(&xfull[g][k % kXBufs], fillParity(k))) ok = false;
    if (!ok) atomicOr(&sFail, 1);
  } else if (lane == 0) {
    // ---- the issuing thread: each group's rounds (5 per tile) in turn
    uint32_t total[kBwdGroups], rnd[kBwdGroups];
    for (int g = 0; g < kBwdGroups; g++) {
      const uint32_t first = blockIdx.x * kBwdGroups + g;
      total[g] = first < nTiles ? 5u * ((nTiles - first + stride - 1) / stride) : 0u;
      rnd[g] = 0;
    }
    bool initW[kLayers] = {false, false, false, false, false};
    bool more = true;
    while (more && ok) {
      more = false;
      for (int g = 0; g < kBwdGroups && ok; g++) {
        if (rnd[g] >= total[g]) continue;
        const uint32_t buf = rnd[g] % kXBufs;
        if (!mbar_wait(&ready[g], rnd[g] & 1u) || !mbar_wait(&xfull[g][buf], fillParity(rnd[g]))) {
          ok = false;
          break;
        }
        fence_after_sync();
        const int l = roundLayer(rnd[g]);
        const int in = cIn[l], out = cOut[l];
        const uint8_t* sG = smem + kBwdBytes + g * kGroupBytes;
        const uint8_t* sX = sG + kGBytes + buf * kXBuf;
        // a slice's descriptor is the first one's plus the slice's start offset / 16 (the
        // address field's unit; shared addresses stay far below its 2^18-byte range)
        if (l >= 1) {
          const uint32_t id = idesc_bf16(128, (uint32_t)in);
          const uint64_t da = tile_desc(smem_u32(sG), out, 0), db = tile_desc(smem_u32(sWT + cBwdOff[l]), out, 0);
          mma_bf16(tb + 64 * g, da, db, id, 0u);
          for (int k = 1; k < out / 16; k++) mma_bf16(tb + 64 * g, da + 16u * k, db + 16u * k, id, 1u);
        }
        const uint32_t idw = idesc_bf16(128, (uint32_t)out) | kIdescAMn | kIdescBMn;
        const uint64_t dx = xT_desc(smem_u32(sX), xcols(l), 0), dg = mn_desc(smem_u32(sG), out, 0);
        const uint64_t sx = 2u * (uint32_t)xcols(l), sg = 2u * (uint32_t)out;
        mma_bf16(tb + cDWCol[l], dx, dg, idw, initW[l] ? 1u : 0u);
#pragma unroll
        for (int k = 1; k < kTile / 16; k++) mma_bf16(tb + cDWCol[l], dx + sx * k, dg + sg * k, idw, 1u);
        initW[l] = true;
        mma_commit(&done[g]);
        rnd[g]++;
        more = true;
      }
      for (int g = 0; g < kBwdGroups; g++) more = more || rnd[g] < total[g];
    }
    // completes once every product issued above has
    mma_commit(&fin);
    if (!ok) atomicOr(&sFail, 1);
  }
  // every product must be complete before tensor memory is read or released
  if (warp == 0) {
    if (!mbar_wait(&fin, 0)) atomicOr(&sFail, 2);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const int fail = sFail;
  if (fail && t == 0) atomicOr(err, 4u);
  // block results: dW (from tensor memory, transposed back to [out][in]) and db (the bias
  // row), then the loss
  float* part = a.part + (size_t)blockIdx.x * kParams;
  const bool any = blockIdx.x * kBwdGroups < nTiles;
  if (warp < 4) {
    for (int l = 0; l < kLayers; l++) {
      const int in = cIn[l], out = cOut[l];
      for (int c = 0; c < out; c += 16) {
        float v[16];
        if (!(fail & 2) && any) {
          tmem_ld16(tmem_at(tb, 32 * warp, cDWCol[l] + c), v);
          tmem_wait_ld();
        } else {
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] = 0.0f;
        }
        if (fail) {
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] = 0.0f;
        }
        if ((int)t < in) {
          for (int j = 0; j < 16; j++) part[cWOff[l] + (c + j) * in + t] = v[j];
        } else if ((int)t == in) {
          for (int j = 0; j < 16; j++) part[cBOff[l] + c + j] = v[j];
        }
      }
    }
  }
  float ls = warpSum(lossAcc);
  if (lane == 0) sLoss[warp] = ls;
  __syncthreads();
  if (t == 0) {
    float s = 0.0f;
    for (int w = 0; w < kBwdThreads / 32; w++) s += sLoss[w];
    a.loss_part[blockIdx.x] = s;
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tb, kBwdCols);
}

// Sums the blocks' partial gradients and applies one Adam step to the FP32 master parameters
// (lr, beta1, beta2, eps as the CPU restatement). A block takes 32 parameters; its warp w sums
// parts w, w + 8, ... (coalesced over the 32 parameters), then the 8 warp sums are added in
// warp order: a fixed order, so the result does not depend on scheduling.
constexpr int kAdamWarps = 8;
// The packed copies of master parameter p (as k_mlp_pack writes them).
__device__ __forceinline__ void packParam(int p, float value, uint8_t* fwd, uint8_t* bwd, float* bias) {
#pragma unroll
  for (int l = 0; l < kLayers; l++) {
    const int in = cIn[l], out = cOut[l];
    const int i = p - cWOff[l];
    if (i >= 0 && i < in * out) {
      const int o = i / in, k = i % in;
      const uint16_t h = f2bf(value);
      *reinterpret_cast<uint16_t*>(fwd + cFwdOff[l] + cm_offset(o, k, in)) = h;
      if (l >= 1) *reinterpret_cast<uint16_t*>(bwd + cBwdOff[l] + cm_offset(k, o, out)) = h;
      return;
    }
    const int j = p - cBOff[l];
    if (j >= 0 && j < out) {
      bias[biasIndex(l) + j] = value;
      return;
    }
  }
}
__global__ void __launch_bounds__(kAdamWarps * 32) k_mlp_adam(float* __restrict__ P, float* __restrict__ m,
                                                             float* __restrict__ v, const float* __restrict__ part,
                                                             int nParts, const float* __restrict__ loss_part,
                                                             float* __restrict__ grad_out,
                                                             float* __restrict__ loss_out, float lr, float c1,
                                                             float c2, int apply, uint8_t* __restrict__ fwd,
                                                             uint8_t* __restrict__ bwd, float* __restrict__ bias) {
  __shared__ float sPart[kAdamWarps][32];
  const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
  const int p = blockIdx.x * 32 + lane;
  float acc = 0.0f;
  if (p < kParams)
    for (int c = w; c < nParts; c += kAdamWarps) acc += part[(size_t)c * kParams + p];
  sPart[w][lane] = acc;
  __syncthreads();
  if (w == 0 && p < kParams) {
    float g = 0.0f;
#pragma unroll
    for (int k = 0; k < kAdamWarps; k++) g += sPart[k][lane];
    if (grad_out) grad_out[p] = g;
    if (apply) {
      float mm = 0.9f * m[p] + 0.1f * g;
      float vv = 0.99f * v[p] + 0.01f * g * g;
      m[p] = mm;
      v[p] = vv;
      const float np = P[p] - lr * (mm / c1) / (sqrtf(vv / c2) + 1e-8f);
      P[p] = np;
      if (fwd) packParam(p, np, fwd, bwd, bias);
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
  k_mlp_pack<<<(kParams + 255) / 256, 256, 0, st>>>(params, wfwd, wbwd, bias);
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
  const size_t smem = kFwdBytes + (size_t)xTileBytes(0);
  cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  uint32_t tiles = (f.n + kTile - 1) / kTile;
  uint32_t blocks = tiles < (uint32_t)smCount() * 3 ? tiles : (uint32_t)smCount() * 3;
  k_mlp_forward<<<blocks, kTile, smem, st>>>(a, err);
  return cudaGetLastError();
}

int ne_mlp_backward_blocks(uint32_t n) {
  uint32_t tiles = (n + kTile - 1) / kTile;
  uint32_t blocks = (tiles + kBwdGroups - 1) / kBwdGroups;
  return (int)(blocks < (uint32_t)smCount() ? (blocks ? blocks : 1u) : (uint32_t)smCount());
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
  cudaError_t e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBwdSmem);
  if (e != cudaSuccess) return e;
  k_mlp_backward<<<ne_mlp_backward_blocks(b.n), kBwdThreads, kBwdSmem, st>>>(a, err);
  return cudaGetLastError();
}

cudaError_t ne_mlp_adam(cudaStream_t st, float* params, float* m, float* v, const float* part, int parts,
                        const float* loss_part, float* grad_out, float* loss_out, float lr, int step, int apply,
                        uint8_t* wfwd, uint8_t* wbwd, float* bias) {
  float c1 = (float)(1.0 - pow(0.9, (double)step));
  float c2 = (float)(1.0 - pow(0.99, (double)step));
  k_mlp_adam<<<(kParams + 31) / 32, kAdamWarps * 32, 0, st>>>(params, m, v, part, parts, loss_part, grad_out, loss_out, lr, c1,
                                                     c2, apply, wfwd, wbwd, bias);
  return cudaGetLastError();
}

cudaError_t ne_launch_debug_mma_mn(cudaStream_t st, const uint16_t* a, const uint16_t* b, int n, int k,
                                   uint32_t layout, float* d, uint32_t* err) {
  if (n < 16 || n > 64 || k < 16 || k > 64 || n % 16 || k % 16) return cudaErrorInvalidValue;
  const size_t smem = 2 * (size_t)kMnRegion;
  cudaError_t e = cudaFuncSetAttribute(k_debug_mma_mn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_debug_mma_mn<<<1, kMmaThreads, smem, st>>>(a, b, (uint32_t)n, (uint32_t)k, layout, d, err);
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
