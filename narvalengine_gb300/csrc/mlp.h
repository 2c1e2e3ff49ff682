// Radiance-cache network kernels (mlp.cu): launchers called by the C ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// D[128 x n] = A[128 x k] * B[n x k]^T, BF16 inputs (row-major bit patterns), FP32 output,
// one tcgen05 product per launch. n in 16..256 step 16, k in 16..128 step 16. err bit 1:
// a wait on the MMA's completion timed out.
cudaError_t ne_launch_debug_mma(cudaStream_t st, const uint16_t* a, const uint16_t* b, int n, int k, float* d,
                                uint32_t* err);

// The same product with operands in the MN-major layout: layout bit 0 = A, bit 1 = B.
// n, k in 16..64 step 16.
cudaError_t ne_launch_debug_mma_mn(cudaStream_t st, const uint16_t* a, const uint16_t* b, int n, int k,
                                   uint32_t layout, float* d, uint32_t* err);

// A block that allocates tensor memory and waits on an mbarrier nothing signals, bounded by
// `max_polls` polls: err bit 1 once the wait has given up (tensor memory released).
cudaError_t ne_launch_debug_wait(cudaStream_t st, uint32_t max_polls, uint32_t* err);

// Parameters: FP32, per layer W[out][in] then b[out]; layers 96->64, 64->64 (x3), 64->16.
constexpr int kNeMlpParams = 19728;
constexpr int kNeMlpFwdBytes = 38912;   // packed BF16 forward weight tiles
constexpr int kNeMlpBwdBytes = 26624;   // packed BF16 transposed weight tiles (layers 1..4)
constexpr int kNeMlpBiasFloats = 272;
// Training activations: per tile of 128 samples the five layer inputs in the tensor core's
// tile layout (features plus a ones chunk: 104 columns for layer 0, 72 for the others).
constexpr int kNeMlpActTileBytes = 128 * 2 * (104 + 4 * 72);

struct NeMlpForward {
  const float* pos;          // n x 3 query positions (medium object space)
  const float* dir;          // n x 3 unit directions
  const float* feats;        // or n x 96 precomputed features (pos/dir ignored)
  uint32_t n;
  const uint32_t* n_dev;     // optional device-side count: min(*n_dev, n) queries are run
  const uint8_t* wfwd;
  const float* bias;
  float* out;                // n x 3 raw outputs, or null
  uint8_t* acts;             // training: ceil(n / 128) x kNeMlpActTileBytes, or null
  const float* thr;          // with idx and radiance: radiance[idx[i]] += thr[i] * max(out[i], 0)
  const uint32_t* idx;
  float* radiance;
};

struct NeMlpBackward {
  const uint8_t* acts;       // the forward pass's training activations
  const float* out;
  const float* target;
  uint32_t n;
  const uint8_t* wbwd;
  float* part;               // ne_mlp_backward_blocks(n) x kNeMlpParams
  float* loss_part;          // ne_mlp_backward_blocks(n)
};

cudaError_t ne_mlp_encode(cudaStream_t st, const float* pos, const float* dir, uint32_t n, float* feats);
cudaError_t ne_mlp_pack(cudaStream_t st, const float* params, uint8_t* wfwd, uint8_t* wbwd, float* bias);
// err bit 2: a tensor-core wait of the forward pass timed out; bit 4: of the backward pass.
cudaError_t ne_mlp_forward(cudaStream_t st, const NeMlpForward& f, uint32_t* err);
int ne_mlp_backward_blocks(uint32_t n);
cudaError_t ne_mlp_backward(cudaStream_t st, const NeMlpBackward& b, uint32_t* err);
// Sums the partial gradients; when apply != 0 takes Adam step `step` (1-based) and, when
// wfwd is not null, writes the updated parameters' packed copies (as ne_mlp_pack).
cudaError_t ne_mlp_adam(cudaStream_t st, float* params, float* m, float* v, const float* part, int parts,
                        const float* loss_part, float* grad_out, float* loss_out, float lr, int step, int apply,
                        uint8_t* wfwd, uint8_t* wbwd, float* bias);
