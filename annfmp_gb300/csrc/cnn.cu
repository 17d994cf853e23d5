// cnn.cu -- the offset-proposal network: input, 3x3 convolutions (forward, backward-data,
// backward-weights), relaxed winner-takes-all truncated L1 loss over block sub-targets, Adam,
// training targets and inference
// proposals (sm_103a).
//
// Network (an addition of this project; the reference's only propagation candidates are the row
// above, annfmp/openmp/kdtree/src/base.c:255-282): the pair at 1/4 resolution (4x4 box mean of A
// and of B, (v - 127.5) / 64, 6 channels + 2 zero) through six 3x3 convolutions (8->32, 32->32 x4,
// 32->8), zero padding, bias, ReLU after the first five. Activations are stored NHWC in BF16,
// weights are used BF16-rounded, every sum is FP32. The 8 outputs of a low-resolution pixel are 4
// hypotheses (dx, dy) in units of 16 full-resolution pixels.
//
// One generic convolution kernel serves the forward pass and the input gradient:
//   out[n][p][o] = sum_tap sum_i in[n][p + d(tap)][i] * Wg[tap][i][o]  (+ bias, ReLU)
// with Wg[tap][ci][co] = W[co][tap][ci] forward and Wg[tap][co][ci] = W[co][8 - tap][ci] for the
// input gradient (correlation with the flipped kernel). A 16x16 output tile per CTA: the 18x18 input
// halo sits channel-major in shared memory (row stride 325 floats: conflict-free), the weights as
// FP32 [9][I][O]; each of 128 threads computes two pixels x O outputs.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "handle.cuh"
#include "tc.cuh"

namespace annf {

int num_sms();

constexpr int kCT = 16;             // output tile side
constexpr int kCH = kCT + 2;        // halo tile side
constexpr int kCS = kCH * kCH + 1;  // channel stride of the halo tile in shared memory
constexpr float kOutScale = 16.0f;
constexpr float kWtaEps = 0.05f;
constexpr float kWtaTrunc = 40.0f;  // px: a hypothesis farther than this from the target gets no gradient

__device__ __forceinline__ float ld_act(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float ld_act(const float* p) { return *p; }

// ---------------------------------------------------------------------------------------------
// input: X[h4][w4][8] = ((4x4 mean of A.rgb, B.rgb) - 127.5) / 64, 0, 0
// ---------------------------------------------------------------------------------------------
__global__ void cnn_input_kernel(const uint8_t* __restrict__ A, const uint8_t* __restrict__ B, int H, int W, int h4,
                                 int w4, __nv_bfloat16* __restrict__ X) {
  const int n = h4 * w4;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int y = i / w4, x = i - y * w4;
    float v[8];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const uint8_t* img = s ? B : A;
      int acc[3] = {0, 0, 0};
      for (int u = 0; u < 4; ++u) {
        const uint8_t* row = img + ((size_t)(4 * y + u) * W + 4 * x) * 3;
#pragma unroll
        for (int t = 0; t < 12; ++t) acc[t % 3] += row[t];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) v[3 * s + c] = ((float)acc[c] * 0.0625f - 127.5f) * 0.015625f;
    }
    v[6] = v[7] = 0.f;
    __nv_bfloat16* o = X + (size_t)i * 8;
#pragma unroll
    for (int c = 0; c < 8; ++c) o[c] = __float2bfloat16_rn(v[c]);
  }
  (void)H;
}

// ---------------------------------------------------------------------------------------------
// weights: master FP32 W[co][9][ci] -> Wg forward [9][ci][co] and input-gradient [9][co][ci],
// both BF16-rounded (kept FP32)
// ---------------------------------------------------------------------------------------------
__global__ void cnn_prep_weights_kernel(const float* __restrict__ W, int co_n, int ci_n, float* __restrict__ wf,
                                        float* __restrict__ wb) {
  const int n = co_n * 9 * ci_n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int co = e / (9 * ci_n), r = e - co * 9 * ci_n, tap = r / ci_n, ci = r - tap * ci_n;
    const float w = __bfloat162float(__float2bfloat16_rn(W[e]));
    wf[((size_t)tap * ci_n + ci) * co_n + co] = w;
    if (wb) wb[((size_t)(8 - tap) * co_n + co) * ci_n + ci] = w;
  }
}

// ---------------------------------------------------------------------------------------------
// generic 3x3 convolution (see the file comment). MODE 0: bias + ReLU, BF16 out; MODE 1: bias,
// FP32 out; MODE 2: no bias, FP32 out (input gradient). MASK: input multiplied by (mask > 0).
// ---------------------------------------------------------------------------------------------
template <int CI, int CO, typename TIN, bool MASK, int MODE>
__global__ void __launch_bounds__(128) cnn_conv_kernel(const TIN* __restrict__ in, const __nv_bfloat16* __restrict__ mask,
                                                       int h, int w, const float* __restrict__ wg,
                                                       const float* __restrict__ bias, void* __restrict__ out,
                                                       unsigned* status) {
  extern __shared__ __align__(16) float csm[];
  float* xs = csm;                   // [CI][kCS]
  float* ws = csm + CI * kCS;        // [9][CI][CO]
  ws = reinterpret_cast<float*>(((uintptr_t)ws + 15) & ~uintptr_t(15));
  if (smem_overrun(csm, ws + 9 * CI * CO, status)) return;
  const int n = blockIdx.z, y0 = blockIdx.y * kCT, x0 = blockIdx.x * kCT;
  const size_t img = (size_t)n * h * w;
  for (int e = threadIdx.x; e < kCH * kCH * CI; e += blockDim.x) {
    const int q = e / CI, c = e - q * CI;
    const int qy = q / kCH, qx = q - qy * kCH;
    const int y = y0 + qy - 1, x = x0 + qx - 1;
    float v = 0.f;
    if (y >= 0 && y < h && x >= 0 && x < w) {
      const size_t off = (img + (size_t)y * w + x) * CI + c;
      v = ld_act(in + off);
      if (MASK && !(__bfloat162float(mask[off]) > 0.f)) v = 0.f;
    }
    xs[c * kCS + q] = v;
  }
  for (int e = threadIdx.x; e < 9 * CI * CO; e += blockDim.x) ws[e] = wg[e];
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // pixels (ty, tx) and (ty + 8, tx)
  float a0[CO], a1[CO];
#pragma unroll
  for (int o = 0; o < CO; ++o) {
    const float b = (MODE == 2) ? 0.f : bias[o];
    a0[o] = b;
    a1[o] = b;
  }
#pragma unroll 1
  for (int tap = 0; tap < 9; ++tap) {
    const int ky = tap / 3, kx = tap - ky * 3;
    const float* i0 = xs + (ty + ky) * kCH + tx + kx;
    const float* wt = ws + tap * CI * CO;
#pragma unroll 4
    for (int c = 0; c < CI; ++c) {
      const float x0v = i0[c * kCS], x1v = i0[c * kCS + 8 * kCH];
      const float4* w4 = reinterpret_cast<const float4*>(wt + c * CO);
#pragma unroll
      for (int o4 = 0; o4 < CO / 4; ++o4) {
        const float4 wv = w4[o4];
        a0[4 * o4 + 0] = fmaf(x0v, wv.x, a0[4 * o4 + 0]);
        a0[4 * o4 + 1] = fmaf(x0v, wv.y, a0[4 * o4 + 1]);
        a0[4 * o4 + 2] = fmaf(x0v, wv.z, a0[4 * o4 + 2]);
        a0[4 * o4 + 3] = fmaf(x0v, wv.w, a0[4 * o4 + 3]);
        a1[4 * o4 + 0] = fmaf(x1v, wv.x, a1[4 * o4 + 0]);
        a1[4 * o4 + 1] = fmaf(x1v, wv.y, a1[4 * o4 + 1]);
        a1[4 * o4 + 2] = fmaf(x1v, wv.z, a1[4 * o4 + 2]);
        a1[4 * o4 + 3] = fmaf(x1v, wv.w, a1[4 * o4 + 3]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int y = y0 + ty + 8 * r, x = x0 + tx;
    if (y >= h || x >= w) continue;
    const float* a = r ? a1 : a0;
    const size_t off = (img + (size_t)y * w + x) * CO;
    if (MODE == 0) {
      __nv_bfloat16* o = static_cast<__nv_bfloat16*>(out) + off;
#pragma unroll
      for (int c = 0; c < CO; c += 2)
        *reinterpret_cast<__nv_bfloat162*>(o + c) = __floats2bfloat162_rn(fmaxf(a[c], 0.f), fmaxf(a[c + 1], 0.f));
    } else {
      float* o = static_cast<float*>(out) + off;
#pragma unroll
      for (int c = 0; c < CO; c += 4) *reinterpret_cast<float4*>(o + c) = make_float4(a[c], a[c + 1], a[c + 2], a[c + 3]);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// weight and bias gradients: dW[co][tap][ci] += sum_p G[p][co] * X[p + d(tap)][ci],
// db[co] += sum_p G[p][co], G = upstream gradient (times (mask > 0) when MASK). One thread per
// (tap, ci) with CO accumulators; CTAs loop over 16x16 tiles and add their sums once at the end.
// ---------------------------------------------------------------------------------------------
template <int CI, int CO, bool MASK>
__global__ void __launch_bounds__(9 * CI) cnn_wgrad_kernel(const __nv_bfloat16* __restrict__ X, const float* __restrict__ G,
                                                           const __nv_bfloat16* __restrict__ mask, int nimg, int h,
                                                           int w, float* __restrict__ dW, float* __restrict__ db,
                                                           unsigned* status) {
  extern __shared__ __align__(16) float csm[];
  float* xs = csm;                                    // [CI][kCS]
  float* gs = csm + ((CI * kCS + 3) & ~3);            // [256][CO]
  if (smem_overrun(csm, gs + kCT * kCT * CO, status)) return;
  const int tid = threadIdx.x, tap = tid / CI, ci = tid - tap * CI;
  const int ky = tap / 3, kx = tap - ky * 3;
  const int tiles_x = (w + kCT - 1) / kCT, tiles_y = (h + kCT - 1) / kCT;
  const long long ntiles = (long long)tiles_x * tiles_y * nimg;
  float acc[CO], bacc[CO];
#pragma unroll
  for (int o = 0; o < CO; ++o) acc[o] = bacc[o] = 0.f;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int n = (int)(t / ((long long)tiles_x * tiles_y));
    const int r = (int)(t - (long long)n * tiles_x * tiles_y);
    const int y0 = (r / tiles_x) * kCT, x0 = (r % tiles_x) * kCT;
    const size_t img = (size_t)n * h * w;
    __syncthreads();
    for (int e = tid; e < kCH * kCH * CI; e += blockDim.x) {
      const int q = e / CI, c = e - q * CI;
      const int qy = q / kCH, qx = q - qy * kCH;
      const int y = y0 + qy - 1, x = x0 + qx - 1;
      xs[c * kCS + q] = (y >= 0 && y < h && x >= 0 && x < w) ? __bfloat162float(X[(img + (size_t)y * w + x) * CI + c]) : 0.f;
    }
    for (int e = tid; e < kCT * kCT * CO; e += blockDim.x) {
      const int q = e / CO, c = e - q * CO;
      const int y = y0 + q / kCT, x = x0 + q % kCT;
      float g = 0.f;
      if (y < h && x < w) {
        const size_t off = (img + (size_t)y * w + x) * CO + c;
        g = G[off];
        if (MASK && !(__bfloat162float(mask[off]) > 0.f)) g = 0.f;
      }
      gs[e] = g;
    }
    __syncthreads();
    const float* xb = xs + ci * kCS + ky * kCH + kx;
#pragma unroll 2
    for (int p = 0; p < kCT * kCT; ++p) {
      const float xv = xb[(p >> 4) * kCH + (p & 15)];
      const float4* g4 = reinterpret_cast<const float4*>(gs + p * CO);
#pragma unroll
      for (int o4 = 0; o4 < CO / 4; ++o4) {
        const float4 gv = g4[o4];
        acc[4 * o4 + 0] = fmaf(xv, gv.x, acc[4 * o4 + 0]);
        acc[4 * o4 + 1] = fmaf(xv, gv.y, acc[4 * o4 + 1]);
        acc[4 * o4 + 2] = fmaf(xv, gv.z, acc[4 * o4 + 2]);
        acc[4 * o4 + 3] = fmaf(xv, gv.w, acc[4 * o4 + 3]);
        if (tid == 0) {
          bacc[4 * o4 + 0] += gv.x;
          bacc[4 * o4 + 1] += gv.y;
          bacc[4 * o4 + 2] += gv.z;
          bacc[4 * o4 + 3] += gv.w;
        }
      }
    }
  }
#pragma unroll
  for (int o = 0; o < CO; ++o) atomicAdd(dW + ((size_t)o * 9 + tap) * CI + ci, acc[o]);
  if (tid == 0) {
#pragma unroll
    for (int o = 0; o < CO; ++o) atomicAdd(db + o, bacc[o]);
  }
}

// ---------------------------------------------------------------------------------------------
// relaxed winner-takes-all truncated L1 loss over each pixel's 16 sub-targets (the matches of the
// 16 A pixels of its 4x4 block): every valid sub-target pulls its nearest hypothesis (weight 1) and
// the others (weight kWtaEps); loss_sum += the batch loss
// ---------------------------------------------------------------------------------------------
__global__ void cnn_wta_kernel(const float* __restrict__ out, const float* __restrict__ tgt,
                               const uint8_t* __restrict__ valid, long long npix, float inv_nv,
                               float* __restrict__ dout, float* __restrict__ loss_sum) {
  float lsum = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npix; i += (long long)gridDim.x * blockDim.x) {
    float o[8], g[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      o[c] = kOutScale * out[i * 8 + c];
      g[c] = 0.f;
    }
    for (int s = 0; s < 16; ++s) {
      if (!valid[i * 16 + s]) continue;
      const float tx = tgt[(i * 16 + s) * 2], ty = tgt[(i * 16 + s) * 2 + 1];
      float e[4];
      int js = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        e[j] = fabsf(o[2 * j] - tx) + fabsf(o[2 * j + 1] - ty);
        if (e[j] < e[js]) js = j;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float wj = (j == js ? 1.f : kWtaEps) * inv_nv;
        const bool live = e[j] < kWtaTrunc;
        lsum += wj * (live ? e[j] : kWtaTrunc);
        const float dx = o[2 * j] - tx, dy = o[2 * j + 1] - ty;
        const float w = live ? wj * kOutScale : 0.f;
        g[2 * j] += w * (dx > 0.f ? 1.f : (dx < 0.f ? -1.f : 0.f));
        g[2 * j + 1] += w * (dy > 0.f ? 1.f : (dy < 0.f ? -1.f : 0.f));
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) dout[i * 8 + c] = g[c];
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((threadIdx.x & 31) == 0 && lsum != 0.f) atomicAdd(loss_sum, lsum);
}

// Adam (bias-corrected), in place on FP32 master parameters
__global__ void cnn_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1,
                                float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// ---------------------------------------------------------------------------------------------
// training targets from an NNF and inference proposals
// ---------------------------------------------------------------------------------------------
__global__ void cnn_targets_kernel(const int* __restrict__ nnf, int H, int W, int Wb, int psize, int h4, int w4,
                                   float* __restrict__ tgt, uint8_t* __restrict__ valid) {
  const int n_cols = W - psize + 1, n_rows = H - psize + 1, ncb = Wb - psize + 1, half = psize / 2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < h4 * w4; i += gridDim.x * blockDim.x) {
    const int yy = i / w4, xx = i - yy * w4;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int y = 4 * yy + (u >> 2) - half, x = 4 * xx + (u & 3) - half;
      const bool ok = y >= 0 && y < n_rows && x >= 0 && x < n_cols;
      float dx = 0.f, dy = 0.f;
      if (ok) {
        const int b = nnf[(size_t)y * n_cols + x];
        const int by = b / ncb, bx = b - by * ncb;
        dx = (float)(bx - x);
        dy = (float)(by - y);
      }
      valid[(size_t)i * 16 + u] = ok ? 1 : 0;
      tgt[((size_t)i * 16 + u) * 2] = dx;
      tgt[((size_t)i * 16 + u) * 2 + 1] = dy;
    }
  }
}

// per_pixel 4: every A patch takes its block's 4 hypotheses; 2: (x + y) even takes 0, 1 and odd 2, 3;
// 1: patch (y, x) takes hypothesis 2 (y mod 2) + (x mod 2), so each 2 x 2 group verifies all four
__global__ void cnn_proposals_kernel(const float* __restrict__ out, int h4, int w4, int n_rows, int n_cols, int nrb,
                                     int ncb, int psize, int per_pixel, int* __restrict__ props) {
  const long long nA = (long long)n_rows * n_cols;
  const int half = psize / 2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nA; i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / n_cols), x = (int)(i - (long long)y * n_cols);
    const int li = min((y + half) >> 2, h4 - 1), lj = min((x + half) >> 2, w4 - 1);
    const float* o = out + ((size_t)li * w4 + lj) * 8;
    const int j0 = per_pixel == 4 ? 0 : per_pixel == 2 ? 2 * ((x + y) & 1) : 2 * (y & 1) + (x & 1);
    for (int u = 0; u < per_pixel; ++u) {
      const int j = j0 + u;
      const int by = min(max(y + __float2int_rn(o[2 * j + 1] * kOutScale), 0), nrb - 1);
      const int bx = min(max(x + __float2int_rn(o[2 * j] * kOutScale), 0), ncb - 1);
      props[i * per_pixel + u] = by * ncb + bx;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// forward convolution on the tensor cores (inference and training forward): an implicit GEMM per
// tile of 128 consecutive pixels of one row, M = 128 pixels, N = Cout padded to 16/32, K = taps x
// Cin in the weights' own order (k = (ky*3 + kx)*Cin + ci). The three input rows are staged in
// shared memory. For Cin = 32 they are staged as planes of 8 channels (16 bytes per pixel), so the
// pixels of a plane are 16 bytes apart like the rows of a K-major core matrix: the staged rows are
// the A operand itself (tap (ky, kx) starts kx pixels into row ky's planes, the next 8 channels
// one plane further: LBO = the plane size), and a tile is 9 taps x 2 MMAs with no A tile built.
// For Cin = 8 all 9 taps are expanded into an A tile at once (K = 72 padded to 80). FP32 TMEM
// accumulator; epilogue adds the bias, applies the ReLU and stores BF16 (or FP32 for the last layer).
// ---------------------------------------------------------------------------------------------
constexpr long long kConvWaitCycles = 2000000000LL;

__device__ __forceinline__ bool conv_wait(uint64_t* mbar, uint32_t phase) {
  const long long t0 = clock64();
  while (!tc::mbar_try_wait(mbar, phase)) {
    if (clock64() - t0 > kConvWaitCycles) return false;
  }
  return true;
}

// W [co][9][ci] FP32 -> wt [cop][kpad] BF16 bits, zero padded
__global__ void cnn_prep_weights_tc_kernel(const float* __restrict__ W, int co_n, int ci_n, int cop, int kpad,
                                           uint16_t* __restrict__ wt) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cop * kpad; e += gridDim.x * blockDim.x) {
    const int co = e / kpad, k = e - co * kpad;
    const float v = (co < co_n && k < 9 * ci_n) ? W[(size_t)co * 9 * ci_n + k] : 0.f;
    __nv_bfloat16 b = __float2bfloat16_rn(v);
    wt[e] = *reinterpret_cast<uint16_t*>(&b);
  }
}

template <int CI, int COP, int MODE>  // MODE 0: bias + ReLU, BF16 out; MODE 1: bias, FP32 out
__global__ void __launch_bounds__(128) cnn_conv_tc_kernel(const __nv_bfloat16* __restrict__ X, int nimg, int h, int w,
                                                          const uint16_t* __restrict__ wt, const float* __restrict__ bias,
                                                          int co_n, void* __restrict__ out, unsigned* status) {
  constexpr int KPAD = CI == 32 ? 288 : 80;           // full K (B tile)
  constexpr int KR = CI == 32 ? 96 : 80;              // K of one round (A tile)
  constexpr int ROUNDS = CI == 32 ? 3 : 1;
  constexpr int SPIX = 130;                           // staged pixels per input row
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  unsigned char* sA = p;  // the expanded A tile (Cin = 8 only)
  if (CI != 32) p += 128 * KR * 2;
  unsigned char* sB = p;
  p += COP * KPAD * 2;
  __nv_bfloat16* sIn = reinterpret_cast<__nv_bfloat16*>(p);  // [3][SPIX][CI]
  p += 3 * SPIX * CI * 2;
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
  for (int e = tid; e < COP * (KPAD / 8); e += 128) {  // weights tile (core layout)
    const int r = e / (KPAD / 8), k8 = (e - r * (KPAD / 8)) * 8;
    *reinterpret_cast<uint4*>(sB + tc::core_offset(r, k8, KPAD)) =
        *reinterpret_cast<const uint4*>(wt + (size_t)r * KPAD + k8);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_bf16(128, COP);
  const int tiles_x = (w + 127) / 128;
  const long long ntiles = (long long)nimg * h * tiles_x;
  uint32_t phase = 0;
  bool aborted = false;
  for (long long t = blockIdx.x; t < ntiles && !aborted; t += gridDim.x) {
    const int n = (int)(t / ((long long)h * tiles_x));
    const int rem = (int)(t - (long long)n * h * tiles_x);
    const int y = rem / tiles_x, x0 = (rem - y * tiles_x) * 128;
    // stage input rows y-1..y+1, pixels x0-1..x0+128 (zero outside the image), 8 channels per uint4
    for (int e = tid; e < 3 * SPIX * (CI / 8); e += 128) {
      const int c8 = e % (CI / 8), q = e / (CI / 8);
      const int ry = q / SPIX, px = q - ry * SPIX;
      const int yy = y + ry - 1, xx = x0 + px - 1;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (yy >= 0 && yy < h && xx >= 0 && xx < w)
        v = *reinterpret_cast<const uint4*>(X + (((size_t)n * h + yy) * w + xx) * CI + c8 * 8);
      if (CI == 32)  // plane (row ry, channels 8 c8 .. 8 c8 + 7): SPIX pixels x 16 bytes
        *reinterpret_cast<uint4*>(sIn + ((size_t)(ry * (CI / 8) + c8) * SPIX + px) * 8) = v;
      else
        *reinterpret_cast<uint4*>(sIn + (size_t)q * CI + c8 * 8) = v;
    }
    if constexpr (CI == 32) {
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
        constexpr uint32_t kPlane = SPIX * 16;  // bytes per plane
        for (int tap = 0; tap < 9; ++tap) {
          const int ky = tap / 3, kx = tap - ky * 3;
          const unsigned char* a = reinterpret_cast<const unsigned char*>(sIn) + (size_t)ky * (CI / 8) * kPlane + kx * 16;
#pragma unroll
          for (int kk = 0; kk < CI / 16; ++kk)
            tc::mma_bf16(tmem, tc::sdesc(a + 2 * kk * kPlane, kPlane, 128),
                         tc::sdesc(sB + ((tap * CI + 16 * kk) / 8) * 128, 128, (KPAD / 8) * 128), idesc,
                         (tap > 0 || kk > 0) ? 1u : 0u);
        }
        tc::mma_commit(mbar);
      }
      if (!conv_wait(mbar, phase)) sflag[0] = 1;
      phase ^= 1u;
      __syncthreads();
      if (sflag[0]) aborted = true;
      tc::fence_after_sync();
    } else {
      __syncthreads();
    }
    for (int round = 0; round < (CI == 32 ? 0 : ROUNDS); ++round) {
      // A tile of this round: pixel tid, K = taps of kernel row `round` (CI 32) or all taps (CI 8)
      for (int g = 0; g < KR / 8; ++g) {
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        int ky, kx, c8;
        if (CI == 32) {
          ky = round;
          kx = g / 4;
          c8 = g % 4;
        } else {
          ky = g / 3;
          kx = g % 3;
          c8 = 0;
        }
        if (ky < 3) v = *reinterpret_cast<const uint4*>(sIn + ((size_t)ky * SPIX + tid + kx) * CI + c8 * 8);
        *reinterpret_cast<uint4*>(sA + tc::core_offset(tid, g * 8, KR)) = v;
      }
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
#pragma unroll
        for (int kk = 0; kk < KR / 16; ++kk)
          tc::mma_bf16(tmem, tc::sdesc(sA + kk * 256, 128, (KR / 8) * 128),
                       tc::sdesc(sB + (round * KR / 8) * 128 + kk * 256, 128, (KPAD / 8) * 128), idesc,
                       (round > 0 || kk > 0) ? 1u : 0u);
        tc::mma_commit(mbar);
      }
      if (!conv_wait(mbar, phase)) sflag[0] = 1;
      phase ^= 1u;
      __syncthreads();
      if (sflag[0]) {
        aborted = true;
        break;
      }
      tc::fence_after_sync();
    }
    if (aborted) break;
    // epilogue: thread tid = pixel x0 + tid = TMEM lane tid
    const int x = x0 + tid;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int c0 = 0; c0 < COP; c0 += 16) {
      uint32_t r[16];
      tc::tmem_ld16(trow + (uint32_t)c0, r);
      tc::tmem_wait_ld();
      if (x < w) {
        const size_t base = (((size_t)n * h + y) * w + x) * co_n;
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          const int c = c0 + j;
          if (c >= co_n) break;
          const float a0 = __uint_as_float(r[j]) + bias[c], a1 = __uint_as_float(r[j + 1]) + bias[c + 1];
          if (MODE == 0) {
            *reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(out) + base + c) =
                __floats2bfloat162_rn(fmaxf(a0, 0.f), fmaxf(a1, 0.f));
          } else {
            *reinterpret_cast<float2*>(static_cast<float*>(out) + base + c) = make_float2(a0, a1);
          }
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  if (aborted) {
    if (tid == 0) atomicOr(status, DEV_TC_TIMEOUT);
    conv_wait(mbar, phase ^ 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 32);
}

// ---------------------------------------------------------------------------------------------
// host wrappers
// ---------------------------------------------------------------------------------------------
static int grid_for(long long n, int block) { return (int)std::max(1LL, std::min<long long>((n + block - 1) / block, 16LL * num_sms())); }

int cnn_input(const uint8_t* A, const uint8_t* B, int H, int W, void* X, cudaStream_t st) {
  ANNF_REQUIRE(H >= 4 && W >= 4, "annf_cnn_input: image smaller than 4x4");
  const int h4 = H / 4, w4 = W / 4;
  cnn_input_kernel<<<grid_for((long long)h4 * w4, 256), 256, 0, st>>>(A, B, H, W, h4, w4,
                                                                       static_cast<__nv_bfloat16*>(X));
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

int cnn_prep_weights(const float* W, int co, int ci, float* wf, float* wb, cudaStream_t st) {
  cnn_prep_weights_kernel<<<grid_for((long long)co * 9 * ci, 256), 256, 0, st>>>(W, co, ci, wf, wb);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

template <int CI, int CO, typename TIN, bool MASK, int MODE>
static int launch_conv(const TIN* in, const __nv_bfloat16* mask, int nimg, int h, int w, const float* wg,
                       const float* bias, void* out, unsigned* status, cudaStream_t st) {
  const size_t smem = ((size_t)CI * kCS + 4) * sizeof(float) + (size_t)9 * CI * CO * sizeof(float);
  ANNF_CUDA_TRY(cudaFuncSetAttribute(cnn_conv_kernel<CI, CO, TIN, MASK, MODE>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((w + kCT - 1) / kCT, (h + kCT - 1) / kCT, nimg);
  cnn_conv_kernel<CI, CO, TIN, MASK, MODE><<<grid, 128, smem, st>>>(in, mask, h, w, wg, bias, out, status);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

// forward convolution: ci in {8, 32}, co in {8, 32}; relu -> BF16 out, else FP32 out
int cnn_conv_forward(const void* X, int nimg, int h, int w, int ci, int co, const float* wf, const float* bias,
                     int relu, void* Y, unsigned* status, cudaStream_t st) {
  const __nv_bfloat16* x = static_cast<const __nv_bfloat16*>(X);
  if (ci == 8 && co == 32 && relu) return launch_conv<8, 32, __nv_bfloat16, false, 0>(x, nullptr, nimg, h, w, wf, bias, Y, status, st);
  if (ci == 32 && co == 32 && relu) return launch_conv<32, 32, __nv_bfloat16, false, 0>(x, nullptr, nimg, h, w, wf, bias, Y, status, st);
  if (ci == 32 && co == 8 && !relu) return launch_conv<32, 8, __nv_bfloat16, false, 1>(x, nullptr, nimg, h, w, wf, bias, Y, status, st);
  set_error("annf_cnn_conv_forward: unsupported layer shape");
  return ANNF_ERR_UNSUPPORTED;
}

int cnn_prep_weights_tc(const float* W, int co, int ci, uint16_t* wt, cudaStream_t st) {
  ANNF_REQUIRE((ci == 8 || ci == 32) && (co == 8 || co == 32), "annf_cnn_prep_weights_tc: unsupported layer shape");
  const int cop = co <= 16 ? 16 : 32, kpad = ci == 32 ? 288 : 80;
  cnn_prep_weights_tc_kernel<<<grid_for((long long)cop * kpad, 256), 256, 0, st>>>(W, co, ci, cop, kpad, wt);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

template <int CI, int COP, int MODE>
static int launch_conv_tc(const __nv_bfloat16* x, int nimg, int h, int w, const uint16_t* wt, const float* bias,
                          int co, void* y, unsigned* status, cudaStream_t st) {
  constexpr int KPAD = CI == 32 ? 288 : 80, KR = CI == 32 ? 96 : 80;
  const size_t smem = (CI == 32 ? 0 : (size_t)128 * KR * 2) + (size_t)COP * KPAD * 2 + (size_t)3 * 130 * CI * 2 + 16 + 24 + 64;
  ANNF_CUDA_TRY(cudaFuncSetAttribute(cnn_conv_tc_kernel<CI, COP, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
  const long long tiles = (long long)nimg * h * ((w + 127) / 128);
  // two persistent CTAs per SM: in the NNF the network runs on a side stream beside the main
  // chain, and fewer long-lived CTAs leave it more of the GPU (measured faster than four)
  const int grid = (int)std::max(1LL, std::min<long long>(tiles, 2LL * num_sms()));
  cnn_conv_tc_kernel<CI, COP, MODE><<<grid, 128, smem, st>>>(x, nimg, h, w, wt, bias, co, y, status);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

// forward convolution on the tensor cores, same shapes and outputs as cnn_conv_forward
int cnn_conv_forward_tc(const void* X, int nimg, int h, int w, int ci, int co, const uint16_t* wt, const float* bias,
                        int relu, void* Y, unsigned* status, cudaStream_t st) {
  const __nv_bfloat16* x = static_cast<const __nv_bfloat16*>(X);
  if (ci == 8 && co == 32 && relu) return launch_conv_tc<8, 32, 0>(x, nimg, h, w, wt, bias, co, Y, status, st);
  if (ci == 32 && co == 32 && relu) return launch_conv_tc<32, 32, 0>(x, nimg, h, w, wt, bias, co, Y, status, st);
  if (ci == 32 && co == 8 && !relu) return launch_conv_tc<32, 16, 1>(x, nimg, h, w, wt, bias, co, Y, status, st);
  set_error("annf_cnn_conv_forward_tc: unsupported layer shape");
  return ANNF_ERR_UNSUPPORTED;
}

// input gradient: G [nimg,h,w,co] FP32 (times (mask > 0) if mask) -> dX [nimg,h,w,ci] FP32
int cnn_conv_backward_data(const float* G, const void* mask, int nimg, int h, int w, int co, int ci, const float* wb,
                           float* dX, unsigned* status, cudaStream_t st) {
  const __nv_bfloat16* m = static_cast<const __nv_bfloat16*>(mask);
  if (co == 32 && ci == 32) {
    return m ? launch_conv<32, 32, float, true, 2>(G, m, nimg, h, w, wb, nullptr, dX, status, st)
             : launch_conv<32, 32, float, false, 2>(G, m, nimg, h, w, wb, nullptr, dX, status, st);
  }
  if (co == 8 && ci == 32 && !m) return launch_conv<8, 32, float, false, 2>(G, m, nimg, h, w, wb, nullptr, dX, status, st);
  if (co == 32 && ci == 8) {
    return m ? launch_conv<32, 8, float, true, 2>(G, m, nimg, h, w, wb, nullptr, dX, status, st)
             : launch_conv<32, 8, float, false, 2>(G, m, nimg, h, w, wb, nullptr, dX, status, st);
  }
  set_error("annf_cnn_conv_backward_data: unsupported layer shape");
  return ANNF_ERR_UNSUPPORTED;
}

template <int CI, int CO, bool MASK>
static int launch_wgrad(const __nv_bfloat16* X, const float* G, const __nv_bfloat16* mask, int nimg, int h, int w,
                        float* dW, float* db, unsigned* status, cudaStream_t st) {
  const size_t smem = ((size_t)((CI * kCS + 3) & ~3) + (size_t)kCT * kCT * CO) * sizeof(float);
  ANNF_CUDA_TRY(cudaFuncSetAttribute(cnn_wgrad_kernel<CI, CO, MASK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
  const long long tiles = (long long)((w + kCT - 1) / kCT) * ((h + kCT - 1) / kCT) * nimg;
  const int grid = (int)std::max(1LL, std::min<long long>(tiles, 2LL * num_sms()));
  cnn_wgrad_kernel<CI, CO, MASK><<<grid, 9 * CI, smem, st>>>(X, G, mask, nimg, h, w, dW, db, status);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

// weight / bias gradients (accumulated into dW [co][9][ci], db [co])
int cnn_conv_backward_weights(const void* X, const float* G, const void* mask, int nimg, int h, int w, int ci, int co,
                              float* dW, float* db, unsigned* status, cudaStream_t st) {
  const __nv_bfloat16* x = static_cast<const __nv_bfloat16*>(X);
  const __nv_bfloat16* m = static_cast<const __nv_bfloat16*>(mask);
  if (ci == 8 && co == 32) {
    return m ? launch_wgrad<8, 32, true>(x, G, m, nimg, h, w, dW, db, status, st)
             : launch_wgrad<8, 32, false>(x, G, m, nimg, h, w, dW, db, status, st);
  }
  if (ci == 32 && co == 32) {
    return m ? launch_wgrad<32, 32, true>(x, G, m, nimg, h, w, dW, db, status, st)
             : launch_wgrad<32, 32, false>(x, G, m, nimg, h, w, dW, db, status, st);
  }
  if (ci == 32 && co == 8 && !m) return launch_wgrad<32, 8, false>(x, G, m, nimg, h, w, dW, db, status, st);
  set_error("annf_cnn_conv_backward_weights: unsupported layer shape");
  return ANNF_ERR_UNSUPPORTED;
}

int cnn_wta_loss(const float* out, const float* tgt, const uint8_t* valid, long long npix, float inv_nv, float* dout,
                 float* loss_sum, cudaStream_t st) {
  cnn_wta_kernel<<<grid_for(npix, 256), 256, 0, st>>>(out, tgt, valid, npix, inv_nv, dout, loss_sum);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

int cnn_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps, int step,
             cudaStream_t st) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  cnn_adam_kernel<<<grid_for(n, 256), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

int cnn_targets(const int* nnf, int H, int W, int Wb, int psize, float* tgt, uint8_t* valid, cudaStream_t st) {
  const int h4 = H / 4, w4 = W / 4;
  cnn_targets_kernel<<<grid_for((long long)h4 * w4, 128), 128, 0, st>>>(nnf, H, W, Wb, psize, h4, w4, tgt, valid);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

int cnn_proposals(const float* out, int h4, int w4, int H, int W, int Hb, int Wb, int psize, int per_pixel, int* props,
                  cudaStream_t st) {
  const int n_rows = H - psize + 1, n_cols = W - psize + 1;
  cnn_proposals_kernel<<<grid_for((long long)n_rows * n_cols, 256), 256, 0, st>>>(
      out, h4, w4, n_rows, n_cols, Hb - psize + 1, Wb - psize + 1, psize, per_pixel, props);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

}  // namespace annf
