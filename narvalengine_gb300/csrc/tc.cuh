// Fifth-generation tensor-core primitives (sm_100 family, tcgen05) in inline PTX.
//
// Operands live in shared memory in the canonical K-major layout without swizzling: a
// tile of R rows x K BF16 columns is cut into 8 x 8 "core matrices" (8 rows of 16 bytes,
// stored as 128 contiguous bytes), core matrix (row group g, column group j) at byte
// g * (K / 8) * 128 + j * 128. In the matrix descriptor the leading-dimension offset is then
// 128 B (next 8 columns) and the stride-dimension offset (K / 8) * 128 B (next 8 rows); one
// MMA of K = 16 covers two column groups, so the k-th MMA of a product starts 256 * k bytes
// into the tile. The accumulator D (M = 128 rows x N FP32 columns) lives in tensor memory,
// row m in TMEM lane m; warp w of a warpgroup reads lanes 32w..32w+31.
//
// Every wait on an mbarrier is bounded: after kTcMaxPolls polls it reports failure, the
// caller sets an error flag, and TMEM is still released before the block exits.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace netc {

constexpr uint32_t kTcMaxPolls = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of element (r, k) in a K-major core-matrix tile with `kcols` columns.
__device__ __forceinline__ uint32_t cm_offset(uint32_t r, uint32_t k, uint32_t kcols) {
  return ((r >> 3) * (kcols >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor, no swizzle (layout type 0), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Byte offset of element (r, k) in an MN-major core-matrix tile with `rows` rows (r along M
// or N, k along K): core matrices of 8 K-rows x 8 MN-elements (16 bytes per K-row, 128
// contiguous bytes), the next 8 MN-elements 128 B on, the next 8 K-rows (rows / 8) * 128 B on.
// A row-per-sample tile stored K-major (samples along M, features along K) is, read with the
// roles swapped, the MN-major tile of its transpose (features along M, samples along K).
__device__ __forceinline__ uint32_t mn_offset(uint32_t r, uint32_t k, uint32_t rows) {
  return ((k >> 3) * (rows >> 3) + (r >> 3)) * 128u + (k & 7u) * 16u + (r & 7u) * 2u;
}

// Descriptor of the k-th K=16 slice of a K-major core-matrix tile with `kcols` columns.
__device__ __forceinline__ uint64_t tile_desc(uint32_t tile_saddr, uint32_t kcols, uint32_t kstep) {
  return smem_desc(tile_saddr + kstep * 256u, 128u, (kcols >> 3) * 128u);
}

// Descriptor of the k-th K=16 slice of an MN-major tile with `rows` MN-rows (mn_offset): the
// leading-dimension offset is the step to the next 8 K-rows, (rows / 8) * 128 B, the
// stride-dimension offset the step to the next 8 MN-elements, 128 B (the instruction
// descriptor marks the operand MN-major: bit 15 for A, bit 16 for B).
__device__ __forceinline__ uint64_t mn_desc(uint32_t tile_saddr, uint32_t rows, uint32_t kstep) {
  return smem_desc(tile_saddr + kstep * 2u * rows * 16u, rows * 16u, 128u);
}
constexpr uint32_t kIdescAMn = 1u << 15;
constexpr uint32_t kIdescBMn = 1u << 16;

// Instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32 D, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// ---- tensor memory (one full warp executes these)
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- ordering
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes this thread's ordinary shared-memory stores visible to the tensor core.
__device__ __forceinline__ void fence_smem_to_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Polls the barrier's phase `parity`; false if it did not complete within `max_polls` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_polls = kTcMaxPolls) {
  uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < max_polls; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n selp.b32 %0, 1, 0, P1;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---- MMA (issued by one thread)
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// One arrival of this thread on `bar` (release at CTA scope).
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// ---- bulk copies (the asynchronous copy engine; addresses 16-byte aligned, sizes multiples of
// 16 bytes)
// Global -> shared: `bytes` from src into dst; completes as `bytes` of transaction count on
// `bar`, whose current phase this thread's arrive.expect_tx opens for them.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// Shared -> global, in this thread's bulk group.
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// This thread's bulk stores have read their shared-memory sources.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// This thread's bulk stores are complete.
__device__ __forceinline__ void bulk_wait() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Arrives on `bar` once every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ---- TMEM -> registers: 16 consecutive FP32 columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// TMEM address of (lane, column) relative to an allocation base.
__device__ __forceinline__ uint32_t tmem_at(uint32_t base, uint32_t lane, uint32_t col) {
  return base + (lane << 16) + col;
}

// FP32 -> BF16, round to nearest even (cvt.rn).
__device__ __forceinline__ uint16_t f2bf(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
// Two values packed low, high (one cvt.rn.bf16x2.f32).
__device__ __forceinline__ uint32_t f2bf2(float lo, float hi) {
  __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

}  // namespace netc
