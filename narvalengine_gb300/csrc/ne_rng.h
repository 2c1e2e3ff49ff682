// Counter-based random numbers shared by the GPU integrator and its CPU oracle.
//
// The reference draws every sample from one global std::mt19937(123) through
// `random()` (utils/Math.h:51-66), shared without synchronisation by all render
// threads, so its output depends on thread timing. Here every draw is a pure
// function of (seed, pixel, sample, dim): dim counts the draws a path has made, in
// the order the reference makes them. The same path therefore sees the same
// numbers on any device, in any thread, in any launch order.
//
// Generator: Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
// as easy as 1, 2, 3", SC 2011): ten rounds of two 32x32->64 multiplies with the
// published multipliers and Weyl key increments. One block of four 32-bit words is
// produced per counter; draw `dim` takes word (dim & 3) of the block with counter
// (dim >> 2, sample, pixel, stream), so a path that draws consecutively needs one
// block per four draws. A word becomes a float in [0, 1) as (w >> 8) * 2^-24, which
// never reaches 1 (the reference clamps values >= 1 to 0.999999, Math.h:62-63).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define NE_RNG_HD __host__ __device__ __forceinline__
#else
#define NE_RNG_HD inline
#endif

namespace nerng {

struct Block { uint32_t w[4]; };

// One widening multiply (a single 32x32->64 instruction on the device) gives both halves.
NE_RNG_HD void mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

NE_RNG_HD Block philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  // Rounds stay a loop on the device: the generator is inlined at every draw site and an
  // unrolled copy at each would dominate the path kernel's code size.
#if defined(__CUDA_ARCH__)
#pragma unroll 1
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(M0, c0, &hi0, &lo0);
    mulhilo(M1, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += W0; k1 += W1;
  }
  Block b;
  b.w[0] = c0; b.w[1] = c1; b.w[2] = c2; b.w[3] = c3;
  return b;
}

// The same generator with its ten rounds unrolled (identical words), for the few call sites
// that draw inside the tracking loops, where the loop's branch and counter per round cost
// more than the extra code.
NE_RNG_HD Block philox4x32_10_unrolled(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(M0, c0, &hi0, &lo0);
    mulhilo(M1, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += W0; k1 += W1;
  }
  Block b;
  b.w[0] = c0; b.w[1] = c1; b.w[2] = c2; b.w[3] = c3;
  return b;
}

NE_RNG_HD float word_to_u01(uint32_t w) {
  return (float)(w >> 8) * 0x1.0p-24f;
}

// Identity of one camera path: the seed of the render, the pixel (y * width + x),
// the sample index within the pixel and a stream selector (0 for camera paths).
struct PathKey {
  uint32_t seed_lo, seed_hi;
  uint32_t pixel, sample;
  uint32_t stream;
};

NE_RNG_HD float u01(const PathKey& k, uint32_t dim) {
  Block b = philox4x32_10(dim >> 2, k.sample, k.pixel, k.stream, k.seed_lo, k.seed_hi);
  return word_to_u01(b.w[dim & 3u]);
}

}  // namespace nerng
