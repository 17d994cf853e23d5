// gram_tc.cu -- the exact Gram matrix of the PCA subset on the tensor cores (sm_103a).
//
// G = X^T X over n uint8 samples of F features (blocked layout XB [ns_pad / 64][F][64]: per block
// of 64 samples, each feature's 64 bytes are contiguous; feature P is the row of ones, so G also
// holds the column sums and n). Every sample byte x is
// split into nibbles x = 16 h + l. A tile of 128 features of X (FP16, exact: 0..255) times 128
// features of H and of L (FP16, exact: 0..15) gives XH and XL; every product is at most
// 255 * 15 = 3825 and an FP32 sum of such integers is exact below 2^24, so a task sums at most
// 4352 samples (4352 * 3825 < 2^24) in TMEM and adds G = 16 XH + XL to the 64-bit Gram with
// atomics. tcgen05.mma kind::f16, M = N = 128, both accumulators FP32 in TMEM (256 columns), two
// staging buffers so that the next 64 samples are converted while the tensor cores run.
// Bit-identical to the integer dp4a Gram (pca.cu), which remains for F > 256.
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "handle.cuh"
#include "tc.cuh"

namespace annf {

int num_sms();

constexpr int kGtThreads = 128;     // thread t <-> feature row t of the tile <-> TMEM lane t
constexpr int kGtK = 64;            // samples per staged block
constexpr int kGtChunkMax = 4352;   // samples per task at most: 4352 * 255 * 15 < 2^24
constexpr int kGtTile = 128 * kGtK * 2;  // bytes of one FP16 operand tile (128 rows x 64 samples)
constexpr long long kGtWaitCycles = 2000000000LL;

__device__ __forceinline__ bool gt_wait(uint64_t* mbar, uint32_t phase) {
  const long long t0 = clock64();
  while (!tc::mbar_try_wait(mbar, phase)) {
    if (clock64() - t0 > kGtWaitCycles) return false;
  }
  return true;
}

// FP16 halves of the high and of the low nibbles of four bytes (exact: 0..15)
__device__ __forceinline__ void nibbles_f16(uint32_t w0, uint32_t w1, uint4& hi, uint4& lo) {
  hi = tc::bytes_to_f16x8((w0 >> 4) & 0x0F0F0F0Fu, (w1 >> 4) & 0x0F0F0F0Fu);
  lo = tc::bytes_to_f16x8(w0 & 0x0F0F0F0Fu, w1 & 0x0F0F0F0Fu);
}

// one task: features [128 ha, 128 ha + 128) x [128 hb, 128 hb + 128) over samples [s0, s1)
__global__ void __launch_bounds__(kGtThreads) gram_tc_kernel(const uint8_t* __restrict__ XT, int F, int ns_pad,
                                                             int chunk_len, int nchunks, int npairs,
                                                             unsigned long long* __restrict__ G, unsigned* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  unsigned char* sX[2];
  unsigned char* sH[2];
  unsigned char* sL[2];
  for (int b = 0; b < 2; ++b) {
    sX[b] = p;
    p += kGtTile;
    sH[b] = p;
    p += kGtTile;
    sL[b] = p;
    p += kGtTile;
  }
  uint64_t* mbar = reinterpret_cast<uint64_t*>(p);  // [2], one per buffer
  p += 16;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(p);
  p += 8;
  int* sflag = reinterpret_cast<int*>(p);
  p += 8;
  if (smem_overrun(smem_raw, p, status)) return;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(tslot, 256);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::mbar_fence_init();
    sflag[0] = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_f16(128, 128);
  uint32_t ph[2] = {0u, 0u};
  bool aborted = false;
  const long long ntasks = (long long)npairs * nchunks;
  for (long long task = blockIdx.x; task < ntasks && !aborted; task += gridDim.x) {
    const int pair = (int)(task / nchunks), chunk = (int)(task - (long long)pair * nchunks);
    // pair -> (ha, hb), ha <= hb: (0,0), (0,1), (1,1), ...
    int ha = 0, rem = pair, width = npairs == 1 ? 1 : 2;
    while (rem >= width - ha) {
      rem -= width - ha;
      ++ha;
    }
    const int hb = ha + rem;
    const int s0 = chunk * chunk_len, s1 = min(ns_pad, s0 + chunk_len);
    const int nblk = (s1 - s0) / kGtK;
    const int fa = ha * 128 + tid, fb = hb * 128 + tid;
    // this thread's two feature rows of a block (64 samples each); the next block's are loaded
    // while the current one is converted
    auto load_block = [&](int blk, uint4 (&xa)[4], uint4 (&xb)[4]) {
      const size_t gb = (size_t)(s0 / kGtK + blk) * F;  // this block's feature rows, 64 bytes each
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        xa[q] = fa < F ? __ldg(reinterpret_cast<const uint4*>(XT + (gb + fa) * kGtK) + q) : make_uint4(0u, 0u, 0u, 0u);
        xb[q] = ha == hb ? xa[q]
                         : (fb < F ? __ldg(reinterpret_cast<const uint4*>(XT + (gb + fb) * kGtK) + q)
                                   : make_uint4(0u, 0u, 0u, 0u));
      }
    };
    // two blocks in flight ahead of the one being converted
    uint4 na[4], nb[4], n2a[4], n2b[4];
    if (nblk > 0) load_block(0, na, nb);
    if (nblk > 1) load_block(1, n2a, n2b);
    for (int blk = 0; blk < nblk; ++blk) {
      const int buf = blk & 1;
      uint4 xa[4], xb[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        xa[q] = na[q];
        xb[q] = nb[q];
        na[q] = n2a[q];
        nb[q] = n2b[q];
      }
      if (blk + 2 < nblk) load_block(blk + 2, n2a, n2b);
      if (blk >= 2) {  // the MMAs that read this buffer (block blk - 2) are done
        if (!gt_wait(&mbar[buf], ph[buf])) sflag[0] = 1;
        ph[buf] ^= 1u;
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {  // samples 16q .. 16q + 15
        *reinterpret_cast<uint4*>(sX[buf] + tc::core_offset(tid, 16 * q, kGtK)) = tc::bytes_to_f16x8(xa[q].x, xa[q].y);
        *reinterpret_cast<uint4*>(sX[buf] + tc::core_offset(tid, 16 * q + 8, kGtK)) = tc::bytes_to_f16x8(xa[q].z, xa[q].w);
        uint4 h0, l0, h1, l1;
        nibbles_f16(xb[q].x, xb[q].y, h0, l0);
        nibbles_f16(xb[q].z, xb[q].w, h1, l1);
        *reinterpret_cast<uint4*>(sH[buf] + tc::core_offset(tid, 16 * q, kGtK)) = h0;
        *reinterpret_cast<uint4*>(sH[buf] + tc::core_offset(tid, 16 * q + 8, kGtK)) = h1;
        *reinterpret_cast<uint4*>(sL[buf] + tc::core_offset(tid, 16 * q, kGtK)) = l0;
        *reinterpret_cast<uint4*>(sL[buf] + tc::core_offset(tid, 16 * q + 8, kGtK)) = l1;
      }
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      if (sflag[0]) {
        aborted = true;
        break;
      }
      if (tid == 0) {
        tc::fence_after_sync();
#pragma unroll
        for (int kk = 0; kk < kGtK / 16; ++kk) {
          const uint64_t ad = tc::sdesc(sX[buf] + kk * 256, 128, (kGtK / 8) * 128);
          const uint32_t acc = (blk > 0 || kk > 0) ? 1u : 0u;
          tc::mma_bf16(tmem, ad, tc::sdesc(sH[buf] + kk * 256, 128, (kGtK / 8) * 128), idesc, acc);
          tc::mma_bf16(tmem + 128, ad, tc::sdesc(sL[buf] + kk * 256, 128, (kGtK / 8) * 128), idesc, acc);
        }
        tc::mma_commit(&mbar[buf]);
      }
    }
    if (aborted) break;
    // the last two blocks' commits: every MMA of the task is then done
    for (int blk = std::max(0, nblk - 2); blk < nblk; ++blk) {
      const int buf = blk & 1;
      if (!gt_wait(&mbar[buf], ph[buf])) sflag[0] = 1;
      ph[buf] ^= 1u;
    }
    __syncthreads();
    if (sflag[0]) {
      aborted = true;
      break;
    }
    tc::fence_after_sync();
    // epilogue: row fa of the tile; G = 16 XH + XL, upper triangle only
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < 128; c0 += 16) {
      uint32_t rh[16], rl[16];
      tc::tmem_ld16(trow + (uint32_t)c0, rh);
      tc::tmem_ld16(trow + 128u + (uint32_t)c0, rl);
      tc::tmem_wait_ld();
      if (nblk > 0 && fa < F) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int gj = hb * 128 + c0 + j;
          if (gj < F && (ha != hb || fa <= gj)) {
            const unsigned long long v = 16ull * __float2uint_rn(__uint_as_float(rh[j])) +
                                         (unsigned long long)__float2uint_rn(__uint_as_float(rl[j]));
            if (v) atomicAdd(&G[(size_t)fa * F + gj], v);
          }
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  if (aborted) {  // let the MMAs in flight finish (bounded) before the columns are freed
    if (tid == 0) atomicOr(status, DEV_TC_TIMEOUT);
    gt_wait(&mbar[0], ph[0]);
    gt_wait(&mbar[1], ph[1]);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

bool gram_tc_supported(int F, int ns_pad) { return F >= 1 && F <= 256 && ns_pad % kGtK == 0; }

// G [F][F] (zeroed by the caller) += the upper triangle of XT XT^T
int gram_tc(const uint8_t* XT, int F, int ns_pad, unsigned long long* G, unsigned* status, cudaStream_t st) {
  ANNF_REQUIRE(gram_tc_supported(F, ns_pad), "tensor-core Gram: unsupported shape");
  const int nh = (F + 127) / 128, npairs = nh * (nh + 1) / 2;
  // chunks (whole 64-sample blocks, at most kGtChunkMax) so that all tasks fit one wave of
  // two CTAs per SM when the samples allow
  const int slots = std::max(1, (2 * num_sms()) / npairs);
  int chunk_len = (int)std::min<long long>(kGtChunkMax, ((long long)ns_pad + slots - 1) / slots);
  chunk_len = std::max(kGtK, (chunk_len + kGtK - 1) / kGtK * kGtK);
  if (chunk_len > kGtChunkMax) chunk_len = kGtChunkMax / kGtK * kGtK;
  const int nchunks = (ns_pad + chunk_len - 1) / chunk_len;
  const size_t smem = 6 * (size_t)kGtTile + 16 + 8 + 8 + 64;
  ANNF_CUDA_TRY(cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long ntasks = (long long)npairs * nchunks;
  const int grid = (int)std::max(1LL, std::min<long long>(ntasks, 2LL * num_sms()));  // two per SM by TMEM
  gram_tc_kernel<<<grid, kGtThreads, smem, st>>>(XT, F, ns_pad, chunk_len, nchunks, npairs, G, status);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

}  // namespace annf
