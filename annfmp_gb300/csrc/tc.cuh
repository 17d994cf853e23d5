// tc.cuh -- fifth-generation tensor core (tcgen05) building blocks for sm_103a, in inline PTX.
//
// One CTA issues tcgen05.mma from a single thread with both operands in shared memory (K-major,
// no swizzle: 8-row x 16-byte core matrices) and the FP32 accumulator in tensor memory (TMEM);
// completion is signalled through an mbarrier (tcgen05.commit) and the epilogue reads TMEM with
// tcgen05.ld (warp w of a warpgroup sees lanes 32w..32w+31). Every wait is bounded: on time-out
// the caller records an error status, frees its TMEM and returns.
#pragma once

#include <cuda_fp16.h>

#include <stdint.h>

namespace annf {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- TMEM (one warp allocates and frees; ncols a power of two >= 32) ----
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- shared-memory matrix descriptor, K-major, no swizzle ----
// lbo: byte step between core matrices along K; sbo: byte step between 8-row groups
__device__ __forceinline__ uint64_t sdesc(const void* base, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_addr(base) & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version bits 46-48 = 0b001
  return d;                // base offset 0, relative LBO mode, no swizzle
}

// instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 accumulator, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// instruction descriptor, kind::f16: FP16 A and B (K-major), FP32 accumulator, M x N
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D (TMEM) (+)= A . B^T, single thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// D (TMEM) (+)= A . B^T, single thread, 8-bit operands (kind::f8f6f4; types from the descriptor,
// whose F32-accumulator / E4M3 x E4M3 encoding has the same bits as idesc_f16)
__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive on the mbarrier once every MMA issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
               : "memory");
}

// ---- mbarrier ----
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_addr(mbar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// bounded wait: false if the phase did not complete within max_polls polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mbar, uint32_t phase, uint32_t max_polls) {
  for (uint32_t i = 0; i < max_polls; ++i)
    if (mbar_try_wait(mbar, phase)) return true;
  return false;
}

// ---- fences ----
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- TMEM -> registers: 16 consecutive 32-bit columns of this thread's lane ----
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// 8 consecutive 32-bit columns of this thread's lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// byte offset of element (r, k) of a K-major bf16 tile (rows x K) stored as core matrices,
// 8-row groups outermost: core (r/8, k/8) at ((r/8) * (K/8) + k/8) * 128, row r%8 at 16 B steps
__host__ __device__ __forceinline__ uint32_t core_offset(int r, int k, int K) {
  return (uint32_t)(((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// eight FP16 values of eight consecutive bytes (w0 = bytes 0..3, w1 = bytes 4..7): a byte permute
// pairs each byte b with the byte 0x64, giving the half 1024 + b (bits 0x64bb, exact: 1024 + b <
// 2048), and one packed subtraction of 1024 leaves b exactly. Bytes past the patch row meet zero
// components in the B tile, so they need no masking (callers decide what the bytes meet).
__device__ __forceinline__ uint4 bytes_to_f16x8(uint32_t w0, uint32_t w1) {
  constexpr uint32_t kMagic = 0x64646464u;
  const __half2 k1024 = __halves2half2(__ushort_as_half((unsigned short)0x6400), __ushort_as_half((unsigned short)0x6400));
  const uint32_t p[4] = {__byte_perm(w0, kMagic, 0x4140), __byte_perm(w0, kMagic, 0x4342),
                         __byte_perm(w1, kMagic, 0x4140), __byte_perm(w1, kMagic, 0x4342)};
  uint32_t o[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const __half2 h = __hsub2(*reinterpret_cast<const __half2*>(&p[u]), k1024);
    o[u] = *reinterpret_cast<const uint32_t*>(&h);
  }
  return make_uint4(o[0], o[1], o[2], o[3]);
}

}  // namespace tc
}  // namespace annf
