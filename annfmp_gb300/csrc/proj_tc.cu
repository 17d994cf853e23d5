// proj_tc.cu -- patch extraction fused with the PCA projection on the tensor cores (sm_103a).
//
// Three kernels: the row form (project_rows_tc_kernel, images of at most 4 channels) and the tile
// form (project_tc_kernel, any channel count) of the approximate forms' FP16 projection, and the
// exact projection (project_exact_tc_kernel, the drop-in form's; its dp4a twin is in pca.cu).
//
// Tile form: every psize x psize x c patch of an image times the FP16-rounded
// components, FP32 accumulation, minus the projected mean. One tile = 128 consecutive patches of one
// row: the psize image rows they cover are staged in shared memory (aligned 32-bit loads), each thread
// pair expands one patch into the K-major FP16 A tile (core-matrix layout; K runs over the patch
// rows, each padded to a multiple of 8 bytes so that a group of 8 is 8 consecutive image bytes, and
// the components are permuted to match), and tcgen05.mma kind::f16
// (M = 128, N = components rounded up to 16) accumulates in TMEM; the epilogue reads TMEM, subtracts
// the mean term and writes FP32 reduced patches. Pixel values 0..255 are exact in FP16 and every
// product is exact in FP32, so the only rounding beyond FP32 summation is that of the components
// (FP16: 11 significant bits).
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "fixed.cuh"
#include "handle.cuh"
#include "tc.cuh"

namespace annf {

int num_sms();

constexpr int kPjThreads = 256;  // two threads per patch row of the tile
constexpr long long kPjWaitCycles = 2000000000LL;

__device__ __forceinline__ bool pj_wait(uint64_t* mbar, uint32_t phase) {
  const long long t0 = clock64();
  while (!tc::mbar_try_wait(mbar, phase)) {
    if (clock64() - t0 > kPjWaitCycles) return false;
  }
  return true;
}

// B operand [npad][kpad] FP16 row-major, K in the tile's order (patch row r occupies
// [r*rs, r*rs + psize*C) with rs = psize*C rounded up to 8; padding zero), and the FP32 mean term
// m_j = sum_k f16(c_jk) mean_k
__global__ void pj_prep_kernel(const double* __restrict__ comps, const double* __restrict__ mean, int d, int P,
                               int rowlen, int rs, int npad, int kpad, uint16_t* __restrict__ bmat,
                               float* __restrict__ mterm) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < npad * kpad; e += gridDim.x * blockDim.x) {
    const int j = e / kpad, k = e - j * kpad;
    const int r = k / rs, el = k - r * rs;
    const int src = r * rowlen + el;
    const float v = (j < d && el < rowlen && src < P) ? (float)comps[(size_t)j * P + src] : 0.f;
    bmat[e] = __half_as_ushort(__float2half_rn(v));
  }
  if (blockIdx.x == 0) {
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      double s = 0.0;
      for (int k = 0; k < P; ++k)
        s += (double)__half2float(__float2half_rn((float)comps[(size_t)j * P + k])) * mean[k];
      mterm[j] = (float)s;
    }
  }
}

// 4-byte asynchronous global -> shared copy (both addresses 4-byte aligned), and its group fences
__device__ __forceinline__ void cp_async4(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(tc::smem_addr(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// stage the psize image rows of tile t as aligned words: byte b of row r sits at
// sI[r*sw + s0(r) + b] with s0(r) = (start of row r) mod 4 (rows need not start 4-byte aligned: W * C
// may be odd). Interior words are copied asynchronously; the image's last bytes synchronously.
__device__ __forceinline__ void pj_stage(const uint8_t* __restrict__ img, long long t, int tiles_x, int ncols, int W,
                                         int C, int psize, long long nbytes, int sw, uint8_t* sI) {
  const int y = (int)(t / tiles_x), x0 = (int)(t - (long long)y * tiles_x) * 128;
  const int np = min(128, ncols - x0);
  const long long row0 = ((long long)y * W + x0) * C;
  const long long pitch = (long long)W * C;
  const int span = (np + psize - 1) * C;
  const int nw = (3 + span + 3) >> 2;  // words per staged row, enough for any shift
  for (int e = threadIdx.x; e < psize * nw; e += kPjThreads) {
    const int r = e / nw, wi = e - r * nw;
    const long long a = ((row0 + (long long)r * pitch) & ~3LL) + 4LL * wi;  // 4-byte aligned
    uint8_t* dst = sI + r * sw + 4 * wi;
    if (a + 4 <= nbytes) {
      cp_async4(dst, img + a);
    } else {
      uint32_t v = 0;
      for (int u = 0; u < 4; ++u)
        if (a + u < nbytes) v |= (uint32_t)__ldg(img + a + u) << (8 * u);
      *reinterpret_cast<uint32_t*>(dst) = v;
    }
  }
}

template <int NPAD>
__global__ void __launch_bounds__(kPjThreads) project_tc_kernel(const uint8_t* __restrict__ img, int H, int W, int C,
                                                                int psize, int d, int kpad,
                                                                const uint16_t* __restrict__ bmat,
                                                                const float* __restrict__ mterm, float* __restrict__ out,
                                                                unsigned* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int rowlen = psize * C, rs = (rowlen + 7) & ~7;
  const int ncols = W - psize + 1, nrows = H - psize + 1;
  const int tiles_x = (ncols + 127) / 128;
  const long long ntiles = (long long)tiles_x * nrows;
  const long long nbytes = (long long)H * W * C;
  const int sw = (((128 + psize - 1) * C + 3 + 16) + 15) & ~15;  // staged row pitch: span + alignment shift + slack
  unsigned char* p = smem_raw;
  unsigned char* sA = p;
  p += (size_t)128 * kpad * 2;
  unsigned char* sB = p;
  p += (size_t)NPAD * kpad * 2;
  uint8_t* sI0 = p;  // staged rows, double buffered: the next tile's rows arrive during this tile
  p += (size_t)psize * sw;
  uint8_t* sI1 = p;
  p += (size_t)psize * sw;
  p = reinterpret_cast<unsigned char*>(((uintptr_t)p + 15) & ~uintptr_t(15));
  uint64_t* mbar = reinterpret_cast<uint64_t*>(p);
  p += 8;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(p);
  p += 8;
  int* sflag = reinterpret_cast<int*>(p);
  p += 8;
  if (smem_overrun(smem_raw, p, status)) return;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(tslot, 32);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    tc::mbar_fence_init();
    sflag[0] = 0;
  }
  // components tile (core layout)
  for (int e = tid; e < NPAD * (kpad / 8); e += kPjThreads) {
    const int r = e / (kpad / 8), k8 = (e - r * (kpad / 8)) * 8;
    *reinterpret_cast<uint4*>(sB + tc::core_offset(r, k8, kpad)) =
        *reinterpret_cast<const uint4*>(bmat + (size_t)r * kpad + k8);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_f16(128, NPAD);
  const int row = tid & 127, half = tid >> 7;  // patch row of the tile; K half (expansion) / column half
  const int ngrp = kpad / 8, gpr = rs / 8;     // K groups in all / per patch row
  uint32_t phase = 0;
  if (blockIdx.x < ntiles) pj_stage(img, blockIdx.x, tiles_x, ncols, W, C, psize, nbytes, sw, sI0);
  cp_async_commit();
  int buf = 0;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, buf ^= 1) {
    const int y = (int)(t / tiles_x), x0 = (int)(t - (long long)y * tiles_x) * 128;
    const int np = min(128, ncols - x0);
    const long long row0 = ((long long)y * W + x0) * C;
    const long long pitch = (long long)W * C;
    uint8_t* sI = buf ? sI1 : sI0;
    // the next tile's rows go to the other buffer (last read by the previous tile's expansion,
    // which every thread finished before the barrier that precedes its MMA)
    if (t + gridDim.x < ntiles) pj_stage(img, t + gridDim.x, tiles_x, ncols, W, C, psize, nbytes, sw, buf ? sI0 : sI1);
    cp_async_commit();
    cp_async_wait<1>();  // this tile's copies (all but the group just committed)
    __syncthreads();
    // expand: group g of patch `row` = bytes [e0, e0 + 8) of its patch row r (zero beyond rowlen)
    const int g0 = half ? ngrp / 2 : 0, g1 = half ? ngrp : ngrp / 2;
    for (int g = g0; g < g1; ++g) {
      const int r = g / gpr, e0 = (g - r * gpr) * 8;
      uint4 w = make_uint4(0u, 0u, 0u, 0u);
      if (r < psize && row < np) {
        const int off = r * sw + (int)((row0 + (long long)r * pitch) & 3) + row * C + e0;
        const uint32_t* wp = reinterpret_cast<const uint32_t*>(sI + (off & ~3));
        const int sh = (off & 3) * 8;
        const uint32_t q0 = wp[0], q1 = wp[1], q2 = wp[2];
        w = tc::bytes_to_f16x8(__funnelshift_r(q0, q1, sh), __funnelshift_r(q1, q2, sh));
      }
      *reinterpret_cast<uint4*>(sA + tc::core_offset(row, g * 8, kpad)) = w;
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      for (int kk = 0; kk < kpad / 16; ++kk)
        tc::mma_bf16(tmem, tc::sdesc(sA + kk * 256, 128, (kpad / 8) * 128),
                     tc::sdesc(sB + kk * 256, 128, (kpad / 8) * 128), idesc, kk > 0 ? 1u : 0u);
      tc::mma_commit(mbar);
    }
    if (!pj_wait(mbar, phase)) sflag[0] = 1;
    phase ^= 1u;
    __syncthreads();
    if (sflag[0]) break;
    tc::fence_after_sync();
    // epilogue: warp w reads lanes 32 (w & 3).. and column half (w >> 2)
    {
      constexpr int HC = NPAD / 2;
      const int lane_row = (warp & 3) * 32 + (tid & 31);
      const int c0 = (warp >> 2) * HC;
      const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0;
      uint32_t r[HC];
      if constexpr (HC == 8) {
        tc::tmem_ld8(taddr, r);
      } else {
        uint32_t (&r16)[16] = *reinterpret_cast<uint32_t(*)[16]>(r);
        tc::tmem_ld16(taddr, r16);
      }
      tc::tmem_wait_ld();
      if (lane_row < np) {
        float* dst = out + ((size_t)y * ncols + x0 + lane_row) * d;
        if (d == NPAD) {  // whole 16-byte groups (rows of d floats are 16-byte aligned)
#pragma unroll
          for (int j = 0; j < HC; j += 4)
            *reinterpret_cast<float4*>(dst + c0 + j) =
                make_float4(__uint_as_float(r[j]) - mterm[c0 + j], __uint_as_float(r[j + 1]) - mterm[c0 + j + 1],
                            __uint_as_float(r[j + 2]) - mterm[c0 + j + 2], __uint_as_float(r[j + 3]) - mterm[c0 + j + 3]);
        } else {
#pragma unroll
          for (int j = 0; j < HC; ++j)
            if (c0 + j < d) dst[c0 + j] = __uint_as_float(r[j]) - mterm[c0 + j];
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  cp_async_wait<0>();  // no copy may still target this CTA's shared memory when it exits
  if (sflag[0]) {
    if (tid == 0) atomicOr(status, DEV_TC_TIMEOUT);
    pj_wait(mbar, phase ^ 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------------------------
// Row form (images of at most 4 channels): no per-patch expansion. An image row is converted once
// into FP16 with every pixel padded to 4 channels (8 bytes), so consecutive pixels are 8 bytes
// apart and every second one 16 bytes: exactly the row pitch of a K-major core matrix. With the
// A tile's rows taken as the patches x0, x0 + 2, ..., x0 + 254 and the K-adjacent core matrices
// 16 bytes apart (LBO = 16), the converted row itself is the A operand of filter row r: element
// (patch i, k) sits at byte 16 i + 2 k, i.e. channel k mod 4 of pixel 2 i + k / 4. A second copy
// shifted by one pixel gives the odd patches. Each output row is then 2 x psize x KS MMAs
// (M = 128, N = components padded to 16/32, K = 16 per MMA, KS = 4 psize / 16 rounded up) into two
// TMEM accumulators, over a ring of psize + 1 converted rows; a CTA walks a strip of 256 patches
// down kPrRows output rows, converting the next image row into the spare slot while the tensor
// cores work on the current one.
// ---------------------------------------------------------------------------------------------
constexpr int kPrThreads = 128;  // one thread per TMEM lane: the even patch 2 i and the odd one 2 i + 1
constexpr int kPrRows = 16;      // output rows per CTA

__host__ __device__ constexpr int pr_kr(int psize) { return (4 * psize + 15) / 16 * 16; }  // K per filter row
__host__ __device__ constexpr int pr_pe(int psize) { return 254 + pr_kr(psize) / 4; }      // pixels per copy

// B operand per filter row r: [psize][npad][kr] FP16 row-major, k = 4 s + ch (pixel s of the
// filter row, channel ch; zero for s >= psize or ch >= C), and the FP32 mean term as pj_prep_kernel
__global__ void pr_prep_kernel(const double* __restrict__ comps, const double* __restrict__ mean, int d, int P,
                               int psize, int C, int npad, int kr, uint16_t* __restrict__ bmat,
                               float* __restrict__ mterm) {
  const int total = psize * npad * kr;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int r = e / (npad * kr), rem = e - r * npad * kr, j = rem / kr, k = rem - j * kr;
    const int px = k >> 2, ch = k & 3;
    const float v = (j < d && px < psize && ch < C) ? (float)comps[(size_t)j * P + (r * psize + px) * C + ch] : 0.f;
    bmat[e] = __half_as_ushort(__float2half_rn(v));
  }
  if (blockIdx.x == 0) {  // a warp per component, lanes over the patch elements
    const int lane = threadIdx.x & 31;
    for (int j = threadIdx.x >> 5; j < d; j += blockDim.x >> 5) {
      double s = 0.0;
      for (int k = lane; k < P; k += 32)
        s += (double)__half2float(__float2half_rn((float)comps[(size_t)j * P + k])) * mean[k];
#pragma unroll
      for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) mterm[j] = (float)s;
    }
  }
}

// image row Y, pixels x0 .. x0 + pe (zero beyond the image) -> the even copy (pixel x0 + q at q)
// and the odd copy (pixel x0 + 1 + q at q), 4 FP16 channels per pixel
__device__ __forceinline__ void pr_convert_row(const uint8_t* __restrict__ img, int W, int C, int Y, int x0, int pe,
                                               uint2* even, uint2* odd) {
  for (int q = threadIdx.x; q <= pe; q += kPrThreads) {
    const int X = x0 + q;
    uint32_t ch[4] = {0u, 0u, 0u, 0u};
    if (X < W) {
      const uint8_t* px = img + ((size_t)Y * W + X) * C;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (u < C) ch[u] = __ldg(px + u);
    }
    // a byte b is the FP16 value b: exact, via the integer-to-half conversion
    const uint32_t lo = (uint32_t)__half_as_ushort(__uint2half_rn(ch[0])) |
                        ((uint32_t)__half_as_ushort(__uint2half_rn(ch[1])) << 16);
    const uint32_t hi = (uint32_t)__half_as_ushort(__uint2half_rn(ch[2])) |
                        ((uint32_t)__half_as_ushort(__uint2half_rn(ch[3])) << 16);
    const uint2 v = make_uint2(lo, hi);
    if (q < pe) even[q] = v;
    if (q >= 1) odd[q - 1] = v;
  }
}

template <int NPAD, int KS>
__global__ void __launch_bounds__(kPrThreads) project_rows_tc_kernel(
    const uint8_t* __restrict__ img, int H, int W, int C, int psize, int d, const uint16_t* __restrict__ bmat,
    const float* __restrict__ mterm, float* __restrict__ out, int vec_out, unsigned* status) {
  constexpr int KR = KS * 16;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int ncols = W - psize + 1, nrows = H - psize + 1;
  const int pe = 254 + KR / 4;  // pixels per copy (even: 0 .. pe - 1 relative to x0)
  const int strips = (ncols + 255) / 256;
  const int strip = blockIdx.x % strips, chunk = blockIdx.x / strips;
  const int x0 = strip * 256, yb = chunk * kPrRows, ye = min(nrows, yb + kPrRows);
  unsigned char* p = smem_raw;
  unsigned char* sB = p;  // [psize] filter rows of NPAD x KR FP16, core layout
  p += (size_t)psize * NPAD * KR * 2;
  const int nslot = psize + 1;
  unsigned char* ring = p;  // [psize + 1 slots][even, odd][pe pixels][8 bytes]
  p += (size_t)nslot * 2 * pe * 8;
  p = reinterpret_cast<unsigned char*>(((uintptr_t)p + 15) & ~uintptr_t(15));
  uint64_t* mbar = reinterpret_cast<uint64_t*>(p);  // [2]: one per accumulator
  p += 16;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(p);
  p += 8;
  int* sflag = reinterpret_cast<int*>(p);
  p += 8;
  if (smem_overrun(smem_raw, p, status)) return;
  if (yb >= nrows) return;  // uniform per block
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(tslot, 4 * NPAD);  // two accumulators x (even, odd) x NPAD columns
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    tc::mbar_init(mbar + 1, 1);
    tc::mbar_fence_init();
    sflag[0] = 0;
  }
  for (int e = tid; e < psize * NPAD * (KR / 8); e += kPrThreads) {  // components, core layout per filter row
    const int r = e / (NPAD * (KR / 8)), rem = e - r * NPAD * (KR / 8);
    const int n = rem / (KR / 8), k8 = (rem - n * (KR / 8)) * 8;
    *reinterpret_cast<uint4*>(sB + (size_t)r * NPAD * KR * 2 + tc::core_offset(n, k8, KR)) =
        *reinterpret_cast<const uint4*>(bmat + ((size_t)r * NPAD + n) * KR + k8);
  }
  auto slot_even = [&](int Y) { return reinterpret_cast<uint2*>(ring + (size_t)(2 * (Y % nslot)) * pe * 8); };
  auto slot_odd = [&](int Y) { return reinterpret_cast<uint2*>(ring + (size_t)(2 * (Y % nslot) + 1) * pe * 8); };
  for (int Y = yb; Y < yb + psize; ++Y) pr_convert_row(img, W, C, Y, x0, pe, slot_even(Y), slot_odd(Y));
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_f16(128, NPAD);
  // the MMAs of output row y (image rows y .. y + psize - 1) into accumulator buf
  auto issue = [&](int y, int buf) {
    for (int half = 0; half < 2; ++half) {
      for (int r = 0; r < psize; ++r) {
        const unsigned char* a = reinterpret_cast<const unsigned char*>(half ? slot_odd(y + r) : slot_even(y + r));
        const unsigned char* b = sB + (size_t)r * NPAD * KR * 2;
#pragma unroll
        for (int kk = 0; kk < KS; ++kk)
          tc::mma_bf16(tmem + (uint32_t)(buf * 2 * NPAD + half * NPAD), tc::sdesc(a + kk * 32, 16, 128),
                       tc::sdesc(b + kk * 256, 128, (KR / 8) * 128), idesc, (r > 0 || kk > 0) ? 1u : 0u);
      }
    }
    tc::mma_commit(mbar + buf);
  };
  uint32_t phase = 0u;    // bit b: the parity to wait for on mbar[b]
  uint32_t pending = 1u;  // bit b: a commit on mbar[b] not waited for yet
  if (tid == 0) issue(yb, 0);
  for (int y = yb; y < ye; ++y) {
    const int buf = (y - yb) & 1;
    // the image row the next output row adds goes to the slot of row y - 1, whose MMAs were waited
    // for in the previous iteration (row y's MMAs do not read it)
    if (y + 1 < ye) {
      pr_convert_row(img, W, C, y + psize, x0, pe, slot_even(y + psize), slot_odd(y + psize));
      tc::fence_async_smem();
    }
    tc::fence_before_sync();
    __syncthreads();  // the row is converted, and the epilogue of row y - 1 has left accumulator buf ^ 1
    if (sflag[0]) break;
    // the next output row's MMAs run while this row's epilogue reads accumulator buf
    if (y + 1 < ye) {
      if (tid == 0) {
        tc::fence_after_sync();
        issue(y + 1, buf ^ 1);
      }
      pending |= 2u >> buf;  // bit buf ^ 1
    }
    const bool ok = __all_sync(0xffffffffu, pj_wait(mbar + buf, (phase >> buf) & 1u));
    phase ^= 1u << buf;
    pending &= ~(1u << buf);
    if (!ok) {
      if ((tid & 31) == 0) sflag[0] = 1;
      continue;
    }
    tc::fence_after_sync();
    // epilogue: lane i holds patch x0 + 2 i (columns 0..NPAD) and x0 + 2 i + 1 (NPAD..2 NPAD)
    {
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(buf * 2 * NPAD);
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        uint32_t r[NPAD];
        if constexpr (NPAD == 16) {
          tc::tmem_ld16(taddr + (uint32_t)(half * NPAD), r);
        } else {
          uint32_t(&r0)[16] = *reinterpret_cast<uint32_t(*)[16]>(r);
          uint32_t(&r1)[16] = *reinterpret_cast<uint32_t(*)[16]>(r + 16);
          tc::tmem_ld16(taddr + (uint32_t)(half * NPAD), r0);
          tc::tmem_ld16(taddr + (uint32_t)(half * NPAD + 16), r1);
        }
        tc::tmem_wait_ld();
        const int x = x0 + 2 * tid + half;
        if (x < ncols) {
          float* dst = out + ((size_t)y * ncols + x) * d;
          if (vec_out) {  // d a multiple of 4 and out 16-byte aligned
#pragma unroll
            for (int j = 0; j < NPAD; j += 4)
              if (j < d)
                *reinterpret_cast<float4*>(dst + j) =
                    make_float4(__uint_as_float(r[j]) - mterm[j], __uint_as_float(r[j + 1]) - mterm[j + 1],
                                __uint_as_float(r[j + 2]) - mterm[j + 2], __uint_as_float(r[j + 3]) - mterm[j + 3]);
          } else {
#pragma unroll
            for (int j = 0; j < NPAD; ++j)
              if (j < d) dst[j] = __uint_as_float(r[j]) - mterm[j];
          }
        }
      }
    }
  }
  if (sflag[0] && tid == 0) atomicOr(status, DEV_TC_TIMEOUT);
  // no MMA may still write TMEM when it is freed (after a time-out the next row's may be in flight)
  for (int b = 0; b < 2; ++b)
    if ((pending >> b) & 1u) pj_wait(mbar + b, (phase >> b) & 1u);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 4 * NPAD);
}

// ---------------------------------------------------------------------------------------------
// Exact projection (annf_project) on the tensor cores. pca.cu splits every FP64 coefficient into
// 8 signed 7-bit digits (c = 2^-E sum_k s_k 2^-7k); the product of a patch with one digit slice
// is an integer of magnitude below 2^24 (at most 256 products of a pixel <= 255 and a digit
// <= 64), so FP16 operands with an FP32 accumulator give it exactly, in any summation order. The
// MMAs are the row form's (converted image rows as the A operand); the B columns of a CTA are the
// 8 slices of 8 components (column 8 c + k = slice k of component 8 g + c, g = the CTA's component
// group). The epilogue recombines a component's slices in 128-bit fixed point, subtracts the mean
// term in the same units and rounds once to FP32: the arithmetic of project_kernel (pca.cu), so
// the two give the same bits. Eight warps per CTA: warp w reads TMEM lanes 32 (w mod 4) .. + 31
// for the even patches (w < 4) or the odd ones; two TMEM accumulators, so the MMAs of the next
// output row run while this row's epilogue reads the other.
// ---------------------------------------------------------------------------------------------
constexpr int kPxThreads = 256;
constexpr int kPxCols = 64;  // B columns per CTA: 8 components x 8 digit slices

// B operand per component group g and filter row r: [groups][psize][64][kr] FP16, k = 4 s + ch as
// pr_prep_kernel; from digits_kernel's table digits[j][slice][r * rw + s * C + ch] (W4 words per
// slice); zero past the patch or past the last component
__global__ void px_prep_kernel(const int8_t* __restrict__ digits, int d, int groups, int psize, int C, int rw, int W4,
                               int kr, uint16_t* __restrict__ bmat) {
  const long long total = (long long)groups * psize * kPxCols * kr;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e % kr);
    const long long t = e / kr;
    const int n = (int)(t % kPxCols);
    const long long t2 = t / kPxCols;
    const int r = (int)(t2 % psize), g = (int)(t2 / psize);
    const int j = 8 * g + (n >> 3), sl = n & 7;
    const int px = k >> 2, ch = k & 3;
    int v = 0;
    if (j < d && px < psize && ch < C) v = digits[((size_t)j * 8 + sl) * W4 * 4 + r * rw + px * C + ch];
    bmat[e] = __half_as_ushort(__int2half_rn(v));
  }
}

// image row Y into the even / odd copies, as pr_convert_row, with kPxThreads threads
__device__ __forceinline__ void px_convert_row(const uint8_t* __restrict__ img, int W, int C, int Y, int x0, int pe,
                                               uint2* even, uint2* odd) {
  for (int q = threadIdx.x; q <= pe; q += kPxThreads) {
    const int X = x0 + q;
    uint32_t ch[4] = {0u, 0u, 0u, 0u};
    if (X < W) {
      const uint8_t* px = img + ((size_t)Y * W + X) * C;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (u < C) ch[u] = __ldg(px + u);
    }
    const uint32_t lo = (uint32_t)__half_as_ushort(__uint2half_rn(ch[0])) |
                        ((uint32_t)__half_as_ushort(__uint2half_rn(ch[1])) << 16);
    const uint32_t hi = (uint32_t)__half_as_ushort(__uint2half_rn(ch[2])) |
                        ((uint32_t)__half_as_ushort(__uint2half_rn(ch[3])) << 16);
    const uint2 v = make_uint2(lo, hi);
    if (q < pe) even[q] = v;
    if (q >= 1) odd[q - 1] = v;
  }
}

template <int KS>
__global__ void __launch_bounds__(kPxThreads) project_exact_tc_kernel(
    const uint8_t* __restrict__ img, int H, int W, int C, int psize, int d, int groups,
    const uint16_t* __restrict__ bmat, const int* __restrict__ expo, const unsigned long long* __restrict__ mfix,
    float* __restrict__ out, int vec_out, unsigned* status) {
  constexpr int KR = KS * 16;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int ncols = W - psize + 1, nrows = H - psize + 1;
  const int pe = 254 + KR / 4;
  const int strips = (ncols + 255) / 256;
  const int g = blockIdx.x % groups;  // component group: neighbouring CTAs read the same image rows
  const int rest = blockIdx.x / groups;
  const int strip = rest % strips, chunk = rest / strips;
  const int x0 = strip * 256, yb = chunk * kPrRows, ye = min(nrows, yb + kPrRows);
  unsigned char* p = smem_raw;
  unsigned char* sB = p;  // [psize] filter rows of 64 x KR FP16, core layout
  p += (size_t)psize * kPxCols * KR * 2;
  const int nslot = psize + 1;
  unsigned char* ring = p;  // [psize + 1 slots][even, odd][pe pixels][8 bytes]
  p += (size_t)nslot * 2 * pe * 8;
  p = reinterpret_cast<unsigned char*>(((uintptr_t)p + 15) & ~uintptr_t(15));
  uint64_t* mbar = reinterpret_cast<uint64_t*>(p);  // [2]: one per TMEM accumulator
  p += 16;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(p);
  p += 8;
  int* sflag = reinterpret_cast<int*>(p);
  p += 8;
  if (smem_overrun(smem_raw, p, status)) return;
  if (yb >= nrows) return;  // uniform per block
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    tc::tmem_alloc(tslot, 4 * kPxCols);  // two accumulators x (even, odd) x 64 columns
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    tc::mbar_init(mbar + 1, 1);
    tc::mbar_fence_init();
    sflag[0] = 0;
  }
  const uint16_t* bg = bmat + (size_t)g * psize * kPxCols * KR;
  for (int e = tid; e < psize * kPxCols * (KR / 8); e += kPxThreads) {
    const int r = e / (kPxCols * (KR / 8)), rem = e - r * kPxCols * (KR / 8);
    const int n = rem / (KR / 8), k8 = (rem - n * (KR / 8)) * 8;
    *reinterpret_cast<uint4*>(sB + (size_t)r * kPxCols * KR * 2 + tc::core_offset(n, k8, KR)) =
        *reinterpret_cast<const uint4*>(bg + ((size_t)r * kPxCols + n) * KR + k8);
  }
  auto slot_even = [&](int Y) { return reinterpret_cast<uint2*>(ring + (size_t)(2 * (Y % nslot)) * pe * 8); };
  auto slot_odd = [&](int Y) { return reinterpret_cast<uint2*>(ring + (size_t)(2 * (Y % nslot) + 1) * pe * 8); };
  for (int Y = yb; Y < yb + psize; ++Y) px_convert_row(img, W, C, Y, x0, pe, slot_even(Y), slot_odd(Y));
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_f16(128, kPxCols);
  // the MMAs of output row y (image rows y .. y + psize - 1) into accumulator buf
  auto issue = [&](int y, int buf) {
    for (int half = 0; half < 2; ++half) {
      for (int r = 0; r < psize; ++r) {
        const unsigned char* a = reinterpret_cast<const unsigned char*>(half ? slot_odd(y + r) : slot_even(y + r));
        const unsigned char* b = sB + (size_t)r * kPxCols * KR * 2;
#pragma unroll
        for (int kk = 0; kk < KS; ++kk)
          tc::mma_bf16(tmem + (uint32_t)(buf * 2 * kPxCols + half * kPxCols), tc::sdesc(a + kk * 32, 16, 128),
                       tc::sdesc(b + kk * 256, 128, (KR / 8) * 128), idesc, (r > 0 || kk > 0) ? 1u : 0u);
      }
    }
    tc::mma_commit(mbar + buf);
  };
  uint32_t phase = 0u;    // bit b: the parity to wait for on mbar[b]
  uint32_t pending = 1u;  // bit b: a commit on mbar[b] not waited for yet
  if (tid == 0) issue(yb, 0);
  const int quarter = warp & 3, half = warp >> 2;
  const int x = x0 + 2 * (quarter * 32 + lane) + half;
  const bool vec = vec_out && 8 * g + 8 <= d;  // vec_out: d a multiple of 4 and out 16-byte aligned
  for (int y = yb; y < ye; ++y) {
    const int buf = (y - yb) & 1;
    // the image row the next output row adds goes to the slot of row y - 1, whose MMAs were
    // waited for in the previous iteration (row y's MMAs do not read it)
    if (y + 1 < ye) {
      px_convert_row(img, W, C, y + psize, x0, pe, slot_even(y + psize), slot_odd(y + psize));
      tc::fence_async_smem();
    }
    tc::fence_before_sync();
    __syncthreads();  // the row is converted, and the epilogue of row y - 1 has left accumulator buf ^ 1
    if (sflag[0]) break;
    if (y + 1 < ye) {
      if (tid == 0) {
        tc::fence_after_sync();
        issue(y + 1, buf ^ 1);
      }
      pending |= 2u >> buf;  // bit buf ^ 1
    }
    const bool ok = __all_sync(0xffffffffu, pj_wait(mbar + buf, (phase >> buf) & 1u));
    phase ^= 1u << buf;
    pending &= ~(1u << buf);
    if (!ok) {
      if (lane == 0) sflag[0] = 1;
      continue;
    }
    tc::fence_after_sync();
    const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * 2 * kPxCols + half * kPxCols);
    float res[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {  // two components per 16 columns
      uint32_t r[16];
      tc::tmem_ld16(taddr + (uint32_t)(16 * q), r);
      tc::tmem_wait_ld();
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int j = 8 * g + 2 * q + u;
        long long hi = __float2int_rn(__uint_as_float(r[8 * u]));
        long long lo = __float2int_rn(__uint_as_float(r[8 * u + 4]));
#pragma unroll
        for (int k = 1; k < 4; ++k) {
          hi = hi * 128 + __float2int_rn(__uint_as_float(r[8 * u + k]));
          lo = lo * 128 + __float2int_rn(__uint_as_float(r[8 * u + 4 + k]));
        }
        res[2 * q + u] = 0.f;
        if (j < d) {
          const __int128 X = (__int128)hi * ((__int128)1 << 28) + lo;  // sum_k s_k 2^(7 (7 - k))
          const __int128 M =
              ((__int128)(long long)__ldg(mfix + 2 * j + 1) << 64) | (unsigned long long)__ldg(mfix + 2 * j);
          res[2 * q + u] = fixed_to_float(X - M, 49 + __ldg(expo + j));
        }
      }
    }
    if (x < ncols) {
      float* dst = out + ((size_t)y * ncols + x) * d + 8 * g;
      if (vec) {
        *reinterpret_cast<float4*>(dst) = make_float4(res[0], res[1], res[2], res[3]);
        *reinterpret_cast<float4*>(dst + 4) = make_float4(res[4], res[5], res[6], res[7]);
      } else {
#pragma unroll
        for (int c = 0; c < 8; ++c)
          if (8 * g + c < d) dst[c] = res[c];
      }
    }
  }
  if (sflag[0] && tid == 0) atomicOr(status, DEV_TC_TIMEOUT);
  // no MMA may still write TMEM when it is freed (after a time-out the next row's may be in flight)
  for (int b = 0; b < 2; ++b)
    if ((pending >> b) & 1u) pj_wait(mbar + b, (phase >> b) & 1u);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 4 * kPxCols);
}

static size_t px_smem(int psize) {
  return (size_t)psize * kPxCols * pr_kr(psize) * 2 + (size_t)(psize + 1) * 2 * pr_pe(psize) * 8 + 16 + 16 + 16 + 64;
}

bool project_rows_exact_supported(int psize, int c, int ncomp) {
  return psize >= 1 && psize <= 12 && c >= 1 && c <= 4 && ncomp >= 1 && ncomp <= 32 && px_smem(psize) <= 227 * 1024;
}

// the exact projection (annf_project) on the tensor cores: digits, expo and mfix as digits_kernel
// leaves them (8 slices, rw bytes per patch row, W4 words per slice)
int project_rows_exact(annf_handle* h, const uint8_t* img, int H, int W, int c, int psize, int ncomp,
                       const int8_t* digits, int rw, int W4, const int* expo, const unsigned long long* mfix,
                       float* out, cudaStream_t st) {
  const int kr = pr_kr(psize), ks = kr / 16;
  const int groups = (ncomp + 7) / 8;
  const size_t bbytes = (size_t)groups * psize * kPxCols * kr * 2;
  ANNF_ENSURE(h->pj_buf, bbytes + 256);
  uint16_t* bmat = h->pj_buf.as<uint16_t>();
  px_prep_kernel<<<std::max(1, std::min(ceil_div((long long)(bbytes / 2), 256), 256)), 256, 0, st>>>(
      digits, ncomp, groups, psize, c, rw, W4, kr, bmat);
  ANNF_CHECK_LAUNCH();
  // 256 TMEM columns per CTA: the shared memory request keeps at most two CTAs on an SM
  const size_t smem = std::max(px_smem(psize), (size_t)78 * 1024);
  ANNF_REQUIRE(smem <= 227 * 1024, "annf_project: tile too large for shared memory");
  const int ncols = W - psize + 1, nrows = H - psize + 1;
  const long long blocks = (long long)((ncols + 255) / 256) * ((nrows + kPrRows - 1) / kPrRows) * groups;
  ANNF_REQUIRE(blocks <= 0x7fffffffLL, "annf_project: image too large");
  const int vec = (ncomp % 4 == 0 && ((uintptr_t)out & 15) == 0) ? 1 : 0;
#define ANNF_PX(KS_)                                                                                           \
  if (ks == KS_) {                                                                                             \
    ANNF_CUDA_TRY(cudaFuncSetAttribute(project_exact_tc_kernel<KS_>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                       (int)smem));                                                            \
    project_exact_tc_kernel<KS_><<<(unsigned)blocks, kPxThreads, smem, st>>>(img, H, W, c, psize, ncomp, groups, \
                                                                           bmat, expo, mfix, out, vec,         \
                                                                           h->status.as<unsigned>());          \
  }
  ANNF_PX(1) ANNF_PX(2) ANNF_PX(3)
#undef ANNF_PX
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

bool project_rows_supported(int psize, int c, int ncomp) {
  return psize >= 1 && psize <= 12 && c >= 1 && c <= 4 && ncomp >= 1 && ncomp <= 32;
}

bool project_tc_supported(int psize, int c, int ncomp) {
  const int rs = (psize * c + 7) & ~7;
  return psize >= 1 && c >= 1 && psize * rs <= 320 && ncomp >= 1 && ncomp <= 32 && (128 + psize - 1) * c <= 4096;
}

static int project_rows_tc(annf_handle* h, const uint8_t* img, int H, int W, int c, int psize, const double* comps,
                          const double* mean, int ncomp, float* out, cudaStream_t st) {
  const int P = psize * psize * c;
  const int kr = pr_kr(psize), ks = kr / 16, pe = pr_pe(psize);
  const int npad = ncomp <= 16 ? 16 : 32;
  const size_t bbytes = (size_t)psize * npad * kr * 2;
  ANNF_ENSURE(h->pj_buf, bbytes + 64 * sizeof(float) + 256);
  uint16_t* bmat = h->pj_buf.as<uint16_t>();
  float* mterm = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(h->pj_buf.p) + ((bbytes + 255) & ~size_t(255)));
  prof_mark(h, "project:begin", st);
  pr_prep_kernel<<<std::max(1, std::min(ceil_div((int)(bbytes / 2), 256), 64)), 256, 0, st>>>(
      comps, mean, ncomp, P, psize, c, npad, kr, bmat, mterm);
  ANNF_CHECK_LAUNCH();
  // 4 npad TMEM columns per CTA (two accumulators): at most 512 / (4 npad) CTAs may share an SM's
  // columns, and the shared memory request keeps any more from being resident
  const int tmem_per_sm = 512 / (4 * npad);
  const size_t smem = std::max(bbytes + (size_t)(psize + 1) * 2 * pe * 8 + 16 + 32 + 64,
                               (size_t)233472 / (tmem_per_sm + 1) + 1024);
  ANNF_REQUIRE(smem <= 227 * 1024, "annf_project_f16: tile too large for shared memory");
  const int ncols = W - psize + 1, nrows = H - psize + 1;
  const long long blocks = (long long)((ncols + 255) / 256) * ((nrows + kPrRows - 1) / kPrRows);
  ANNF_REQUIRE(blocks <= 0x7fffffffLL, "annf_project_f16: image too large");
  const int vec = (ncomp % 4 == 0 && ((uintptr_t)out & 15) == 0) ? 1 : 0;
#define ANNF_PR(NP, KS_)                                                                                          \
  if (npad == NP && ks == KS_) {                                                                                 \
    ANNF_CUDA_TRY(cudaFuncSetAttribute(project_rows_tc_kernel<NP, KS_>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                       (int)smem));                                                              \
    project_rows_tc_kernel<NP, KS_><<<(unsigned)blocks, kPrThreads, smem, st>>>(img, H, W, c, psize, ncomp, bmat,  \
                                                                               mterm, out, vec,                  \
                                                                               h->status.as<unsigned>());        \
  }
  ANNF_PR(16, 1) ANNF_PR(16, 2) ANNF_PR(16, 3) ANNF_PR(32, 1) ANNF_PR(32, 2) ANNF_PR(32, 3)
#undef ANNF_PR
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "project", st);
  return ANNF_OK;
}

int project_tc(annf_handle* h, const uint8_t* img, int H, int W, int c, int psize, const double* comps,
               const double* mean, int ncomp, float* out, cudaStream_t st) {
  if (project_rows_supported(psize, c, ncomp)) return project_rows_tc(h, img, H, W, c, psize, comps, mean, ncomp, out, st);
  ANNF_REQUIRE(project_tc_supported(psize, c, ncomp), "annf_project_f16: patch or components too large");
  const int P = psize * psize * c;
  const int rowlen = psize * c, rs = (rowlen + 7) & ~7;
  const int kpad = (psize * rs + 15) / 16 * 16;
  const int npad = ncomp <= 16 ? 16 : 32;
  ANNF_ENSURE(h->pj_buf, (size_t)npad * kpad * 2 + 64 * sizeof(float) + 256);
  uint16_t* bmat = h->pj_buf.as<uint16_t>();
  float* mterm = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(h->pj_buf.p) + (((size_t)npad * kpad * 2 + 255) & ~size_t(255)));
  prof_mark(h, "project:begin", st);
  pj_prep_kernel<<<std::max(1, std::min(ceil_div(npad * kpad, 256), 64)), 256, 0, st>>>(comps, mean, ncomp, P, rowlen,
                                                                                         rs, npad, kpad, bmat, mterm);
  ANNF_CHECK_LAUNCH();
  const int sw = (((128 + psize - 1) * c + 3 + 16) + 15) & ~15;
  const size_t smem = (size_t)128 * kpad * 2 + (size_t)npad * kpad * 2 + 2 * (size_t)psize * sw + 16 + 24 + 64;
  ANNF_REQUIRE(smem <= 227 * 1024, "annf_project_f16: tile too large for shared memory");
  const long long ntiles = (long long)((W - psize + 1 + 127) / 128) * (H - psize + 1);
  // TMEM: 32 columns per CTA, so any residency fits; two CTAs per SM by shared memory at P = 243
  const int grid = (int)std::max(1LL, std::min<long long>(ntiles, 4LL * num_sms()));
  if (npad == 16) {
    ANNF_CUDA_TRY(cudaFuncSetAttribute(project_tc_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    project_tc_kernel<16><<<grid, kPjThreads, smem, st>>>(img, H, W, c, psize, ncomp, kpad, bmat, mterm, out,
                                                         h->status.as<unsigned>());
  } else {
    ANNF_CUDA_TRY(cudaFuncSetAttribute(project_tc_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    project_tc_kernel<32><<<grid, kPjThreads, smem, st>>>(img, H, W, c, psize, ncomp, kpad, bmat, mterm, out,
                                                         h->status.as<unsigned>());
  }
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "project", st);
  return ANNF_OK;
}

}  // namespace annf
