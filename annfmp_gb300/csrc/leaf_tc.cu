// leaf_tc.cu -- natural-leaf k nearest neighbours on the fifth-generation tensor cores (sm_103a).
//
// Queries are grouped by the leaf their descent reaches (counting sort on the leaf id). For each
// leaf, the leaf's points (<= 256) and up to 128 of its queries are centred on the leaf's bounding
// box midpoint and staged in shared memory as K-major core-matrix tiles: BF16 hi/lo splits of each
// coordinate ([hi|lo|hi] against [hi|hi|lo], three MMAs per 16 dims) or one FP16 term. tcgen05.mma
// (M = 128 queries, N = leaf points) accumulates a.b in FP32 in TMEM. Each thread owns one query
// (one TMEM lane): it reads its row with tcgen05.ld and re-ranks with the exact FP32 distance
// (reference operation order) only the points whose estimate passes a proven error bound (below),
// so the k-list written equals the FP32 leaf scan's. Centring keeps the products free of the
// cancellation that |a|^2 + |b|^2 - 2 a.b suffers on uncentred reduced coordinates.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <algorithm>

#include "common.cuh"
#include "handle.cuh"
#include "tc.cuh"
#include "tree_walk.cuh"

namespace annf {

int num_sms();

constexpr int kTcThreads = 128;                    // one warpgroup: thread t <-> TMEM lane t <-> query t
constexpr int kTcQueue = 48;                       // columns a query queues for the exact re-rank
constexpr long long kTcWaitCycles = 2000000000LL;  // ~1 s at 2 GHz: bound of every mbarrier wait

// Operand precision of the leaf tiles. BF16 (PREC 0) splits every centred coordinate x into
// hi = bf16(x) and lo = bf16(x - hi) (|x - hi - lo| <= 2^-16 |x|) and accumulates
// hi.hi + hi.lo + lo.hi, so that |dot - (a-c).(b-c)| <= (3 * 2^-16 + 2^-20) |a-c| |b-c|; FP16 (PREC 1)
// uses one term, |dot - (a-c).(b-c)| <= (2^-10 + 2^-20) |a-c| |b-c|. kDot is that coefficient with a
// margin; the K extent of a tile is kSplit x the padded dimension.
template <int PREC> struct TcPrec;
template <> struct TcPrec<0> {
  static constexpr int kSplit = 3;
  static constexpr int kES = 2;  // bytes per element
  static constexpr float kDot = 5.0e-5f;  // > 3 * 2^-16 + 2^-20 = 4.67e-5
  static constexpr float kAbs = 0.f;
  __device__ static void split(float x, float& hi, float& lo) {
    hi = __bfloat162float(__float2bfloat16_rn(x));
    lo = __bfloat162float(__float2bfloat16_rn(x - hi));
  }
  __device__ static uint32_t pack(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
  }
  __host__ __device__ static constexpr uint32_t idesc(int M, int N) { return tc::idesc_bf16(M, N); }
};
template <> struct TcPrec<1> {
  static constexpr int kSplit = 1;
  static constexpr int kES = 2;
  static constexpr float kDot = 1.0e-3f;  // > 2^-10 + 2^-20 = 9.77e-4 (centred values far below 65504)
  static constexpr float kAbs = 0.f;
  __device__ static void split(float x, float& hi, float& lo) {
    hi = __half2float(__float2half_rn(x));
    lo = 0.f;
  }
  __device__ static uint32_t pack(float lo, float hi) {
    __half2 v = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
  }
  __host__ __device__ static constexpr uint32_t idesc(int M, int N) { return tc::idesc_f16(M, N); }
};

// FP8 (E4M3) hi/lo split of values scaled by a power of two into [-256, 256] (|x| < 256 once
// scaled; the largest E4M3 value is 448). Per element, hi + lo represents v within 2^-8 |v| +
// 2^-10 (lo's relative rounding 2^-4 of |v - hi| <= 2^-4 |v|, or half the subnormal step 2^-9);
// the tiles [hi|lo|hi] . [hi|hi|lo] drop lo.lo (<= 2^-8 |a||b| + small), every product is exact
// in FP32, and the FP32 accumulation is charged 1e-3 (a margin far above 64 roundings at 2^-24,
// which also covers an accumulator narrower than FP32). In the scaled units:
//   |dot - a.b| <= kDot |a||b| + kAbs sqrt(d) (|a| + |b|) + kConst d.
template <> struct TcPrec<2> {
  static constexpr int kSplit = 3;
  static constexpr int kES = 1;
  static constexpr float kDot = 1.3e-2f;   // > 2^-7 + 2^-8 + 2^-16 + 1e-3 = 1.273e-2
  static constexpr float kAbs = 1.1e-3f;   // > 2^-10 + 2^-14 + 2^-18 = 1.04e-3
  static constexpr float kConst = 2.1e-6f;  // > 2 * 2^-20 per dimension
  __device__ static uint8_t q8(float v) { return (uint8_t)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3); }
  __device__ static float f8(uint8_t b) {
    return __half2float(__half(__nv_cvt_fp8_to_halfraw((__nv_fp8_storage_t)b, __NV_E4M3)));
  }
  __host__ __device__ static constexpr uint32_t idesc(int M, int N) { return tc::idesc_f16(M, N); }
};

// power-of-two scale that maps a magnitude m > 0 into [128, 256) (1 for m == 0)
__device__ __forceinline__ float pow2_scale_256(float m) { return m > 0.f ? ldexpf(1.f, 7 - ilogbf(m)) : 1.f; }

// byte offset of element byte kb of row r in a K-major no-swizzle core-matrix tile whose rows are
// RB bytes (core matrix: 8 rows x 16 bytes; LBO 128 along K, SBO (RB / 16) * 128 along rows)
template <int RB>
__device__ __forceinline__ int core_off_b(int r, int kb) {
  return ((r >> 3) * (RB >> 4) + (kb >> 4)) * 128 + (r & 7) * 16 + (kb & 15);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// bounded wait on an mbarrier phase (clock-limited); false on time-out
__device__ __forceinline__ bool mbar_wait_clock(uint64_t* mbar, uint32_t phase) {
  const long long t0 = clock64();
  while (!tc::mbar_try_wait(mbar, phase)) {
    if (clock64() - t0 > kTcWaitCycles) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------------------------
// grouping queries by natural leaf
// ---------------------------------------------------------------------------------------------
// the top kQleafLevels levels of nodes in shared memory (one 1024-thread CTA per SM holds them)
constexpr int kQleafLevels = 14;
constexpr int kQleafThreads = 1024;
__global__ void __launch_bounds__(kQleafThreads) qleaf_kernel(TreeView<float> tv, const float* __restrict__ Q,
                                                              long long nq, int* __restrict__ qleaf,
                                                              int* __restrict__ cnt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  NodeCache<float> nc;
  nc.carve(p, tv.depth, kQleafLevels);
  if (smem_overrun(smem_raw, p, tv.status)) return;
  nc.fill(tv, kQleafLevels);
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nq; i += (long long)gridDim.x * blockDim.x) {
    const int lf = descend(tv, nc, Q + i * tv.d);
    qleaf[i] = lf;
    atomicAdd(cnt + lf, 1);
  }
}

// exclusive scans of cnt[L] into off[L+1] and cursor[L], and of the 128-query chunk counts into
// choff[L+1], in two kernels over 1024-leaf tiles: per-tile totals, then each tile's scan from the
// totals before it (coalesced loads, one block-wide scan of both counts per tile)
constexpr int kScanTile = 1024;

__device__ __forceinline__ int chunks_of(int v) { return (v + kTcThreads - 1) / kTcThreads; }

// block-wide inclusive scan of two counters (kScanTile threads); *tot_q / *tot_c get the totals
__device__ __forceinline__ void scan_tile2(int vq, int vc, int& iq, int& ic, int* tot_q, int* tot_c) {
  __shared__ int wt[2][kScanTile / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  iq = vq;
  ic = vc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int yq = __shfl_up_sync(0xffffffffu, iq, o), yc = __shfl_up_sync(0xffffffffu, ic, o);
    if (lane >= o) {
      iq += yq;
      ic += yc;
    }
  }
  if (lane == 31) {
    wt[0][w] = iq;
    wt[1][w] = ic;
  }
  __syncthreads();
  if (w == 0) {
    int tq = wt[0][lane], tc = wt[1][lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int yq = __shfl_up_sync(0xffffffffu, tq, o), yc = __shfl_up_sync(0xffffffffu, tc, o);
      if (lane >= o) {
        tq += yq;
        tc += yc;
      }
    }
    wt[0][lane] = tq;
    wt[1][lane] = tc;
  }
  __syncthreads();
  if (w) {
    iq += wt[0][w - 1];
    ic += wt[1][w - 1];
  }
  *tot_q = wt[0][kScanTile / 32 - 1];
  *tot_c = wt[1][kScanTile / 32 - 1];
}

__global__ void __launch_bounds__(kScanTile) leaf_tile_sums_kernel(const int* __restrict__ cnt, int L,
                                                                   int* __restrict__ tile_tot) {
  const int i = blockIdx.x * kScanTile + threadIdx.x;
  const int v = i < L ? __ldg(cnt + i) : 0;
  int iq, ic, tq, tc;
  scan_tile2(v, chunks_of(v), iq, ic, &tq, &tc);
  if (threadIdx.x == 0) {
    tile_tot[2 * blockIdx.x] = tq;
    tile_tot[2 * blockIdx.x + 1] = tc;
  }
}

__global__ void __launch_bounds__(kScanTile) leaf_scan_kernel(const int* __restrict__ cnt, int L,
                                                              const int* __restrict__ tile_tot, int* __restrict__ off,
                                                              int* __restrict__ cursor, int* __restrict__ choff) {
  __shared__ int base[2];
  if (threadIdx.x < 32) {  // totals of the tiles before this one
    int bq = 0, bc = 0;
    for (int t = threadIdx.x; t < (int)blockIdx.x; t += 32) {
      bq += tile_tot[2 * t];
      bc += tile_tot[2 * t + 1];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      bq += __shfl_xor_sync(0xffffffffu, bq, o);
      bc += __shfl_xor_sync(0xffffffffu, bc, o);
    }
    if (threadIdx.x == 0) {
      base[0] = bq;
      base[1] = bc;
    }
  }
  const int i = blockIdx.x * kScanTile + threadIdx.x;
  const int v = i < L ? __ldg(cnt + i) : 0, vc = chunks_of(v);
  int iq, ic, tq, tc;
  scan_tile2(v, vc, iq, ic, &tq, &tc);  // (its barriers also publish base)
  const int eq = base[0] + iq - v, ec = base[1] + ic - vc;
  if (i < L) {
    off[i] = eq;
    cursor[i] = eq;
    choff[i] = ec;
  }
  if (i == L - 1) {
    off[L] = eq + v;
    choff[L] = ec + vc;
  }
}

// work item -> leaf: leaf l owns items choff[l] .. choff[l+1]-1 (one per 128 of its queries)
__global__ void item_leaf_kernel(const int* __restrict__ choff, int L, int* __restrict__ item_leaf) {
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x)
    for (int c = choff[l]; c < choff[l + 1]; ++c) item_leaf[c] = l;
}

__global__ void qscatter_kernel(const int* __restrict__ qleaf, long long nq, int* __restrict__ cursor,
                                int* __restrict__ qorder) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nq; i += (long long)gridDim.x * blockDim.x)
    qorder[atomicAdd(cursor + qleaf[i], 1)] = (int)i;
}

// ---------------------------------------------------------------------------------------------
// the tensor-core leaf kernel
//
// Selection with a proven error bound. With centre c, est_j = |b_j - c|^2 - 2 dot_j (the norm in
// FP32 from the FP32 points, dot_j from the tile) estimates D_j^2 - |a - c|^2, D_j = |a - b_j|, to
// within delta = 2 kDot |a-c| R + FP32 slack (R bounds |b - c| over the leaf). Every point of the
// true (and of the FP32-computed) k nearest then has est_j <= est_(k) + 2 delta, est_(k) the k-th
// smallest estimate. Pass 1 finds est_(k) from the tile; pass 2 re-ranks exactly (FP32, reference
// order) every point within that band, so the k-list equals the FP32 leaf scan's. With the BF16
// split the band is ~1e-4 |a-c| R, which leaves about k points to re-rank.
// ---------------------------------------------------------------------------------------------
// branch-free insertion into an ascending list (lanes of a warp hold different queries, so a
// data-dependent branch would run the insertion for every column in which any lane inserts)
template <int KM>
__device__ __forceinline__ void sorted_insert(float (&dv)[KM], int (&iv)[KM], float v, int c) {
  // the new entry goes before the first strictly larger one (after equal ones); every entry from
  // there on shifts one place, keeping the order of equal entries
  bool shifting = false;
  float cd = 0.f;
  int ci = 0;
#pragma unroll
  for (int j = 0; j < KM; ++j) {
    const bool put = !shifting && v < dv[j];
    const float od = dv[j];
    const int oi = iv[j];
    dv[j] = put ? v : (shifting ? cd : od);
    iv[j] = put ? c : (shifting ? ci : oi);
    cd = od;
    ci = oi;
    shifting = shifting || put;
  }
}
// the KM smallest values only (min/max network)
template <int KM>
__device__ __forceinline__ void smallest_insert(float (&dv)[KM], float v) {
#pragma unroll
  for (int j = 0; j < KM; ++j) {
    const float lo = fminf(v, dv[j]);
    v = fmaxf(v, dv[j]);
    dv[j] = lo;
  }
}

struct TcLeafArgs {
  TreeView<float> tv;
  const float* Q;
  const int* qoff;    // [L+1] queries of leaf l: qorder[qoff[l] .. qoff[l+1])
  const int* qorder;  // [nq]
  const int* choff;   // [L+1] work items (128-query chunks) of leaf l: choff[l] .. choff[l+1]-1
  const int* item_leaf;  // [choff[L]] leaf of each work item
  int K;              // neighbours written per query (<= KM)
  int npad;           // point rows staged per leaf (multiple of 16, >= largest leaf, <= 256)
  int ncols;          // TMEM columns allocated (power of two >= max(32, npad))
  int* out_pos;       // [nq*K] tree positions
};

template <int KM, int KPAD, int PREC>
__global__ void __launch_bounds__(kTcThreads) leaf_tc_kernel(TcLeafArgs a) {
  using PR = TcPrec<PREC>;
  constexpr int KT = PR::kSplit * KPAD;  // K extent of the tiles (elements)
  constexpr int RB = (KT * PR::kES + 31) / 32 * 32;  // tile row bytes: whole MMA K steps (32 bytes)
  constexpr int KPS = KPAD + 4;  // FP32 point row stride: 16-byte rows that spread over the banks
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const TreeView<float>& tv = a.tv;
  const int d = tv.d, L = 1 << tv.depth, npad = a.npad, K = a.K;
  // carve: A tile, B tile (core-matrix layouts), FP32 leaf points, norms, centre, barrier, TMEM slot
  unsigned char* p = smem_raw;
  unsigned char* sA = p;
  p += kTcThreads * RB;
  unsigned char* sB = p;
  p += (size_t)npad * RB;
  float* sP = reinterpret_cast<float*>(p);  // [npad][KPS] FP32 leaf points (zero padded)
  p += (size_t)npad * KPS * 4;
  float* sN = reinterpret_cast<float*>(p);
  p += (size_t)npad * 4;
  float* sC = reinterpret_cast<float*>(p);  // [KPAD] centre, then [KPAD] = R, [KPAD+1] = FP8 point scale
  p += (KPAD + 4) * 4;
  p = reinterpret_cast<unsigned char*>(((uintptr_t)p + 15) & ~uintptr_t(15));
  uint64_t* mbar = reinterpret_cast<uint64_t*>(p);
  p += 8;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(p);
  p += 8;
  int* sflag = reinterpret_cast<int*>(p);  // [0] leaf, [1] abort
  p += 8;
  unsigned char* sQ = p;  // [kTcQueue][kTcThreads] columns each query re-ranks
  p += kTcQueue * kTcThreads;
  if (smem_overrun(smem_raw, p, tv.status)) return;

  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(tslot, (uint32_t)a.ncols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    tc::mbar_fence_init();
    sflag[1] = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = PR::idesc(128, npad);
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  bool aborted = false;
  const bool vec4 = (d & 3) == 0;

  const int total = __ldg(a.choff + L);
  int staged = -1;  // leaf whose points are in shared memory
  // work items in a fixed round robin (items are at most 128 queries of one leaf, so they cost
  // about the same); the next item's leaf is read one item ahead
  int l_next = (int)blockIdx.x < total ? __ldg(a.item_leaf + blockIdx.x) : 0;
  for (int w = blockIdx.x; w < total; w += gridDim.x) {
    __syncthreads();  // every thread has finished the previous work item
    const int l = l_next;
    if (w + (int)gridDim.x < total) l_next = __ldg(a.item_leaf + w + gridDim.x);
    const int qlb = __ldg(a.qoff + l), qle = __ldg(a.qoff + l + 1);
    const int qb = qlb + (w - __ldg(a.choff + l)) * kTcThreads, qe = min(qle, qb + kTcThreads);
    const int pb = __ldg(tv.leaf_begin + l);
    int np = __ldg(tv.leaf_begin + l + 1) - pb;
    if (np > npad) {
      if (tid == 0 && l != staged) atomicOr(tv.status, DEV_BAD_LEAF);
      np = npad;
    }
    if (l != staged) {  // uniform
    staged = l;
    // centre (box midpoint) and half-diagonal R of the leaf box
    if (tid < 32) {
      float r2 = 0.f, emax = 0.f;
      for (int j = tid; j < KPAD; j += 32) {
        float c = 0.f;
        if (j < d) {
          const float lo = __ldg(tv.leaf_box + (size_t)l * 2 * d + j), hi = __ldg(tv.leaf_box + (size_t)l * 2 * d + d + j);
          c = 0.5f * (lo + hi);
          const float e = 0.5f * (hi - lo);
          r2 = fmaf(e, e, r2);
          emax = fmaxf(emax, e);
        }
        sC[j] = c;
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        emax = fmaxf(emax, __shfl_xor_sync(0xffffffffu, emax, o));
      }
      if (tid == 0) {
        sC[KPAD] = sqrtf(r2) * 1.000001f + 1e-30f;
        // FP8: every centred coordinate is within the largest half extent (plus the centre's
        // rounding, far inside the E4M3 range above 256)
        sC[KPAD + 1] = pow2_scale_256(emax);
      }
    }
    __syncthreads();
    // the leaf's points: FP32 copy, BF16 centred tile, BF16 norms
    for (int r = tid; r < npad; r += kTcThreads) {
      float f[KPAD];
      const float* src = tv.pts + (size_t)(pb + r) * d;
      if (r < np && vec4) {
#pragma unroll
        for (int j = 0; j < KPAD; j += 4) {
          if (j < d) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(src + j));
            f[j] = v.x;
            f[j + 1] = v.y;
            f[j + 2] = v.z;
            f[j + 3] = v.w;
          } else {
            f[j] = f[j + 1] = f[j + 2] = f[j + 3] = 0.f;
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < KPAD; ++j) f[j] = (r < np && j < d) ? __ldg(src + j) : 0.f;
      }
      float nrm = 0.f;
      if constexpr (PREC != 2) {
#pragma unroll
        for (int k8 = 0; k8 < KPAD; k8 += 8) {
          float hi[8], lo[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int j = k8 + u;
            const float x = (r < np && j < d) ? f[j] - sC[j] : 0.f;
            nrm = fmaf(x, x, nrm);
            PR::split(x, hi[u], lo[u]);
          }
          uint4 wh, wl;
          wh.x = PR::pack(hi[0], hi[1]);
          wh.y = PR::pack(hi[2], hi[3]);
          wh.z = PR::pack(hi[4], hi[5]);
          wh.w = PR::pack(hi[6], hi[7]);
          wl.x = PR::pack(lo[0], lo[1]);
          wl.y = PR::pack(lo[2], lo[3]);
          wl.z = PR::pack(lo[4], lo[5]);
          wl.w = PR::pack(lo[6], lo[7]);
          // B row: [hi | hi | lo] against A row [hi | lo | hi]
          *reinterpret_cast<uint4*>(sB + tc::core_offset(r, k8, KT)) = wh;
          if constexpr (PR::kSplit == 3) {
            *reinterpret_cast<uint4*>(sB + tc::core_offset(r, KPAD + k8, KT)) = wh;
            *reinterpret_cast<uint4*>(sB + tc::core_offset(r, 2 * KPAD + k8, KT)) = wl;
          }
        }
      } else {  // FP8: [hi | hi | lo] of the scaled centred point, zero bytes up to RB
        const float sb = sC[KPAD + 1];
        uint32_t hw[KPAD / 4], lw[KPAD / 4];
#pragma unroll
        for (int j4 = 0; j4 < KPAD / 4; ++j4) {
          uint32_t h4 = 0, l4 = 0;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int j = 4 * j4 + u;
            const float x = (r < np && j < d) ? f[j] - sC[j] : 0.f;
            nrm = fmaf(x, x, nrm);
            const float v = x * sb;
            const uint8_t h = PR::q8(v), lq = PR::q8(v - PR::f8(h));
            h4 |= (uint32_t)h << (8 * u);
            l4 |= (uint32_t)lq << (8 * u);
          }
          hw[j4] = h4;
          lw[j4] = l4;
        }
#pragma unroll
        for (int c16 = 0; c16 < KPAD / 16; ++c16) {
          const uint4 H = make_uint4(hw[4 * c16], hw[4 * c16 + 1], hw[4 * c16 + 2], hw[4 * c16 + 3]);
          const uint4 Lw = make_uint4(lw[4 * c16], lw[4 * c16 + 1], lw[4 * c16 + 2], lw[4 * c16 + 3]);
          *reinterpret_cast<uint4*>(sB + core_off_b<RB>(r, 16 * c16)) = H;
          *reinterpret_cast<uint4*>(sB + core_off_b<RB>(r, KPAD + 16 * c16)) = H;
          *reinterpret_cast<uint4*>(sB + core_off_b<RB>(r, 2 * KPAD + 16 * c16)) = Lw;
        }
#pragma unroll
        for (int kb = 3 * KPAD; kb < RB; kb += 16) *reinterpret_cast<uint4*>(sB + core_off_b<RB>(r, kb)) = make_uint4(0u, 0u, 0u, 0u);
      }
#pragma unroll
      for (int j = 0; j < KPAD; j += 4)
        *reinterpret_cast<float4*>(sP + r * KPS + j) = make_float4(f[j], f[j + 1], f[j + 2], f[j + 3]);
      sN[r] = r < np ? nrm : FLT_MAX;
    }
    }  // staging
    const float R = sC[KPAD];
    {
      const int q0 = qb;
      const int qi = (q0 + tid < qe) ? __ldg(a.qorder + q0 + tid) : -1;
      float qf[KPAD];
      if (qi >= 0 && vec4) {
#pragma unroll
        for (int j = 0; j < KPAD; j += 4) {
          if (j < d) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(a.Q + (size_t)qi * d + j));
            qf[j] = v.x;
            qf[j + 1] = v.y;
            qf[j + 2] = v.z;
            qf[j + 3] = v.w;
          } else {
            qf[j] = qf[j + 1] = qf[j + 2] = qf[j + 3] = 0.f;
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < KPAD; ++j) qf[j] = (qi >= 0 && j < d) ? __ldg(a.Q + (size_t)qi * d + j) : 0.f;
      }
      float ac2 = 0.f, amax = 0.f, sa = 1.f;
      if constexpr (PREC != 2) {
#pragma unroll
        for (int k8 = 0; k8 < KPAD; k8 += 8) {
          float hi[8], lo[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const float t = (qi >= 0 && k8 + u < d) ? qf[k8 + u] - sC[k8 + u] : 0.f;
            ac2 = fmaf(t, t, ac2);
            amax = fmaxf(amax, fabsf(t));
            PR::split(t, hi[u], lo[u]);
          }
          uint4 wh, wl;
          wh.x = PR::pack(hi[0], hi[1]);
          wh.y = PR::pack(hi[2], hi[3]);
          wh.z = PR::pack(hi[4], hi[5]);
          wh.w = PR::pack(hi[6], hi[7]);
          wl.x = PR::pack(lo[0], lo[1]);
          wl.y = PR::pack(lo[2], lo[3]);
          wl.z = PR::pack(lo[4], lo[5]);
          wl.w = PR::pack(lo[6], lo[7]);
          *reinterpret_cast<uint4*>(sA + tc::core_offset(tid, k8, KT)) = wh;
          if constexpr (PR::kSplit == 3) {
            *reinterpret_cast<uint4*>(sA + tc::core_offset(tid, KPAD + k8, KT)) = wl;
            *reinterpret_cast<uint4*>(sA + tc::core_offset(tid, 2 * KPAD + k8, KT)) = wh;
          }
        }
      } else {  // FP8: [hi | lo | hi] of the scaled centred query, zero bytes up to RB
        float tq[KPAD];
#pragma unroll
        for (int u = 0; u < KPAD; ++u) {
          tq[u] = (qi >= 0 && u < d) ? qf[u] - sC[u] : 0.f;
          ac2 = fmaf(tq[u], tq[u], ac2);
          amax = fmaxf(amax, fabsf(tq[u]));
        }
        sa = pow2_scale_256(amax);
        uint32_t hw[KPAD / 4], lw[KPAD / 4];
#pragma unroll
        for (int j4 = 0; j4 < KPAD / 4; ++j4) {
          uint32_t h4 = 0, l4 = 0;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const float v = tq[4 * j4 + u] * sa;
            const uint8_t h = PR::q8(v), lq = PR::q8(v - PR::f8(h));
            h4 |= (uint32_t)h << (8 * u);
            l4 |= (uint32_t)lq << (8 * u);
          }
          hw[j4] = h4;
          lw[j4] = l4;
        }
#pragma unroll
        for (int c16 = 0; c16 < KPAD / 16; ++c16) {
          const uint4 H = make_uint4(hw[4 * c16], hw[4 * c16 + 1], hw[4 * c16 + 2], hw[4 * c16 + 3]);
          const uint4 Lw = make_uint4(lw[4 * c16], lw[4 * c16 + 1], lw[4 * c16 + 2], lw[4 * c16 + 3]);
          *reinterpret_cast<uint4*>(sA + core_off_b<RB>(tid, 16 * c16)) = H;
          *reinterpret_cast<uint4*>(sA + core_off_b<RB>(tid, KPAD + 16 * c16)) = Lw;
          *reinterpret_cast<uint4*>(sA + core_off_b<RB>(tid, 2 * KPAD + 16 * c16)) = H;
        }
#pragma unroll
        for (int kb = 3 * KPAD; kb < RB; kb += 16)
          *reinterpret_cast<uint4*>(sA + core_off_b<RB>(tid, kb)) = make_uint4(0u, 0u, 0u, 0u);
      }
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      if (tid == 0) {
        tc::fence_after_sync();
#pragma unroll
        for (int kk = 0; kk < RB / 32; ++kk) {  // one MMA per 32 bytes of K
          const uint64_t ad = tc::sdesc(sA + kk * 256, 128, (RB / 16) * 128);
          const uint64_t bd = tc::sdesc(sB + kk * 256, 128, (RB / 16) * 128);
          if constexpr (PREC == 2)
            tc::mma_f8(tmem, ad, bd, idesc, kk > 0 ? 1u : 0u);
          else
            tc::mma_bf16(tmem, ad, bd, idesc, kk > 0 ? 1u : 0u);
        }
        tc::mma_commit(mbar);
      }
      // while the MMAs run: start the next item's leaf points and queries on their way to L2
      if (w + (int)gridDim.x < total) {
        const int wn = w + (int)gridDim.x;
        const int pbn = __ldg(tv.leaf_begin + l_next), pen = __ldg(tv.leaf_begin + l_next + 1);
        const char* base = reinterpret_cast<const char*>(tv.pts + (size_t)pbn * d);
        const int bytes = (pen - pbn) * d * 4;
        for (int off = tid * 128; off < bytes; off += kTcThreads * 128)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(base + off));
        const int qbn = __ldg(a.qoff + l_next) + (wn - __ldg(a.choff + l_next)) * kTcThreads;
        if (qbn + tid < __ldg(a.qoff + l_next + 1))
          asm volatile("prefetch.global.L2 [%0];" ::"l"(a.Q + (size_t)__ldg(a.qorder + qbn + tid) * d));
      }
      if (!mbar_wait_clock(mbar, phase)) sflag[1] = 1;
      phase ^= 1u;
      __syncthreads();
      if (sflag[1]) {
        aborted = true;
        break;
      }
      tc::fence_after_sync();
      // the tile holds dot products of scaled vectors (FP8: powers of two, exact to undo)
      const float dsc = PREC == 2 ? -2.f / (sa * sC[KPAD + 1]) : -2.f;
      // pass 1: est_b, an upper bound of est_(k), the k-th smallest estimate: the k-th smallest
      // of the minima of groups of four columns (k groups' minima are k distinct estimates, so
      // their k-th smallest is at least est_(k)); padding columns carry sN = FLT_MAX
      float ev[KM];
#pragma unroll
      for (int j = 0; j < KM; ++j) ev[j] = FLT_MAX;
      for (int c0 = 0; c0 < npad; c0 += 16) {
        uint32_t r[16];
        tc::tmem_ld16(trow + (uint32_t)c0, r);
        float nv[16];
#pragma unroll
        for (int j = 0; j < 16; j += 4) {
          const float4 n4 = *reinterpret_cast<const float4*>(sN + c0 + j);
          nv[j] = n4.x;
          nv[j + 1] = n4.y;
          nv[j + 2] = n4.z;
          nv[j + 3] = n4.w;
        }
        tc::tmem_wait_ld();
#pragma unroll
        for (int g = 0; g < 16; g += 4) {
          const float e0 = fmaf(dsc, __uint_as_float(r[g]), nv[g]);
          const float e1 = fmaf(dsc, __uint_as_float(r[g + 1]), nv[g + 1]);
          const float e2 = fmaf(dsc, __uint_as_float(r[g + 2]), nv[g + 2]);
          const float e3 = fmaf(dsc, __uint_as_float(r[g + 3]), nv[g + 3]);
          smallest_insert<KM>(ev, fminf(fminf(e0, e1), fminf(e2, e3)));
        }
      }
      // band: est_j <= est_b + 2 delta, delta = 2 kDot |a-c| R + FP32 slack
      float evk = FLT_MAX;
#pragma unroll
      for (int j = 0; j < KM; ++j)
        if (j == K - 1) evk = ev[j];
      const float acn = sqrtf(ac2) * 1.000001f;
      float delta = 2.f * PR::kDot * acn * R + 4e-6f * (ac2 + R * R + fabsf(evk));
      if constexpr (PREC == 2) {  // FP8: the subnormal-step terms, back in unscaled units
        const float sb = sC[KPAD + 1];
        delta += 2.f * (PR::kAbs * sqrtf((float)d) * (acn / sb + R / sa) + PR::kConst * (float)d / (sa * sb));
      }
      // FP16 cannot hold centred values beyond its range: such queries and leaves take every point
      const bool unsafe = PREC == 1 && (amax > 60000.f || R > 60000.f);
      const float tau = (evk >= FLT_MAX || unsafe) ? FLT_MAX : evk + 2.f * delta;
      // pass 2: queue the columns whose estimate passes the bound, in column order (a query that
      // takes every point, or whose queue overflows, re-ranks the whole leaf below)
      const bool every = tau == FLT_MAX;
      int cnt = 0;
      for (int c0 = 0; c0 < npad; c0 += 16) {
        uint32_t r[16];
        tc::tmem_ld16(trow + (uint32_t)c0, r);
        float nv[16];
#pragma unroll
        for (int j = 0; j < 16; j += 4) {
          const float4 n4 = *reinterpret_cast<const float4*>(sN + c0 + j);
          nv[j] = n4.x;
          nv[j + 1] = n4.y;
          nv[j + 2] = n4.z;
          nv[j + 3] = n4.w;
        }
        tc::tmem_wait_ld();
        unsigned pass = 0;
#pragma unroll
        for (int j = 0; j < 16; ++j) pass |= fmaf(dsc, __uint_as_float(r[j]), nv[j]) <= tau ? (1u << j) : 0u;
        if (c0 + 16 > np) pass &= np > c0 ? (1u << (np - c0)) - 1u : 0u;
        if (qi < 0 || every) pass = 0u;
        while (pass) {
          if (cnt < kTcQueue) sQ[cnt * kTcThreads + tid] = (unsigned char)(c0 + __ffs(pass) - 1);
          pass &= pass - 1;
          ++cnt;
        }
      }
      // the exact FP32 distance (reference order) of every queued point; padding coordinates are
      // zero on both sides and add exact zeros
      float xv[KM];
      int xi[KM];
#pragma unroll
      for (int j = 0; j < KM; ++j) {
        xv[j] = FLT_MAX;
        xi[j] = -1;
      }
      if (qi >= 0) {
        const bool whole = every || cnt > kTcQueue;
        const int n_do = whole ? np : cnt;
        for (int t = 0; t < n_do; ++t) {
          const int col = whole ? t : (int)sQ[t * kTcThreads + tid];
          const float* pp = sP + col * KPS;
          float s = 0.f;
#pragma unroll
          for (int u = 0; u < KPAD; u += 4)
            s = dist_step4(s, *reinterpret_cast<const float4*>(pp + u), qf[u], qf[u + 1], qf[u + 2], qf[u + 3]);
          sorted_insert<KM>(xv, xi, s, col);
        }
      }
      if (qi >= 0) {
        int* out = a.out_pos + (size_t)qi * K;
        const int first = xi[0] >= 0 ? xi[0] : 0;
#pragma unroll
        for (int t = 0; t < KM; ++t)
          if (t < K) out[t] = min(max(pb + (xi[t] >= 0 ? xi[t] : first), 0), tv.n - 1);
      }
      tc::fence_before_sync();
      __syncthreads();
    }
    if (aborted) break;
  }
  if (aborted) {  // let the MMA in flight finish (bounded) before the columns are freed
    if (tid == 0) atomicOr(tv.status, DEV_TC_TIMEOUT);
    mbar_wait_clock(mbar, phase);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)a.ncols);
}

template <int KM, int KPAD, int PREC>
static int launch_leaf_tc(const TcLeafArgs& args, size_t smem, int grid, cudaStream_t st) {
  ANNF_CUDA_TRY(cudaFuncSetAttribute(leaf_tc_kernel<KM, KPAD, PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
  leaf_tc_kernel<KM, KPAD, PREC><<<grid, kTcThreads, smem, st>>>(args);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

static int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

// true when the tree's shape fits the tensor-core kernel (FP32 points, d <= 32, leaves <= 256)
bool leaf_tc_supported(const annf_handle* h, int K) {
  return h->real_type == ANNF_REAL_F32 && h->d >= 1 && h->d <= 32 && h->max_leaf >= 1 && h->max_leaf <= 256 &&
         K >= 1 && K <= 32;
}

int natural_knn_tc(annf_handle* h, const float* Q, long long nq, int K, int prec, int* out_pos, cudaStream_t st) {
  ANNF_REQUIRE(leaf_tc_supported(h, K), "tensor-core leaf kNN: unsupported tree shape");
  ANNF_REQUIRE(nq <= 0x7fffffffLL, "tensor-core leaf kNN: too many queries");
  const int L = 1 << h->depth;
  TreeView<float> tv;
  tv.n = h->n;
  tv.d = h->d;
  tv.depth = h->depth;
  tv.leaf_bits = h->leaf_bits;
  tv.pts = h->pts.as<float>();
  tv.perm = h->perm.as<int>();
  tv.node_axis = h->node_axis.as<int>();
  tv.node_split = h->node_split.as<float>();
  tv.leaf_begin = h->leaf_begin.as<int>();
  tv.point_leaf = h->point_leaf.as<int>();
  tv.status = h->status.as<unsigned>();
  tv.leaf_box = h->leaf_box.as<float>();
  // scratch: qleaf[nq], qorder[nq], cnt[L], off[L+1], cursor[L], choff[L+1], item_leaf[items]
  // (items <= L + nq / 128: each leaf's queries in chunks of 128)
  const size_t need = ((size_t)2 * nq + 4 * (size_t)L + 16 + (size_t)L + (size_t)nq / kTcThreads + 1 +
                       2 * (size_t)ceil_div(L, kScanTile) + 2) * sizeof(int);
  ANNF_ENSURE(h->tc_buf, need);
  int* qleaf = h->tc_buf.as<int>();
  int* qorder = qleaf + nq;
  int* cnt = qorder + nq;
  int* off = cnt + L;
  int* cursor = off + L + 1;
  int* choff = cursor + L;
  int* item_leaf = choff + L + 1;
  int* tile_tot = item_leaf + (size_t)L + (size_t)nq / kTcThreads + 1;  // [2 * tiles]
  ANNF_CUDA_TRY(cudaMemsetAsync(cnt, 0, (size_t)L * sizeof(int), st));
  const size_t ncs = NodeCache<float>::bytes(h->depth, kQleafLevels);
  ANNF_CUDA_TRY(cudaFuncSetAttribute(qleaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ncs));
  const int blocks = (int)std::min<long long>(ceil_div(nq, 256), 8LL * num_sms());
  const int qblocks = (int)std::min<long long>(ceil_div(nq, kQleafThreads), num_sms());
  qleaf_kernel<<<qblocks, kQleafThreads, ncs, st>>>(tv, Q, nq, qleaf, cnt);
  ANNF_CHECK_LAUNCH();
  const int tiles = ceil_div(L, kScanTile);
  leaf_tile_sums_kernel<<<tiles, kScanTile, 0, st>>>(cnt, L, tile_tot);
  ANNF_CHECK_LAUNCH();
  leaf_scan_kernel<<<tiles, kScanTile, 0, st>>>(cnt, L, tile_tot, off, cursor, choff);
  ANNF_CHECK_LAUNCH();
  qscatter_kernel<<<blocks, 256, 0, st>>>(qleaf, nq, cursor, qorder);
  ANNF_CHECK_LAUNCH();
  item_leaf_kernel<<<ceil_div(L, 256), 256, 0, st>>>(choff, L, item_leaf);
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "tc_group", st);

  TcLeafArgs args;
  args.tv = tv;
  args.Q = Q;
  args.qoff = off;
  args.qorder = qorder;
  args.choff = choff;
  args.K = K;
  args.npad = (h->max_leaf + 15) / 16 * 16;
  args.ncols = std::max(32, next_pow2(args.npad));
  args.out_pos = out_pos;
  args.item_leaf = item_leaf;
  const int kpad = h->d <= 16 ? 16 : 32;
  // tile row bytes: K extent (BF16 / FP8 hi-lo splits: 3 terms) times the element size, in whole
  // 32-byte MMA K steps (the kernel's RB)
  const int rb = ((prec == 1 ? 1 : 3) * kpad * (prec == 2 ? 1 : 2) + 31) / 32 * 32;
  const size_t carve = (size_t)kTcThreads * rb + (size_t)args.npad * rb + (size_t)args.npad * (kpad + 4) * 4 +
                       (size_t)args.npad * 4 + (kpad + 4) * 4 + 16 + 24 + (size_t)kTcQueue * kTcThreads + 64;
  // at most 512 / ncols CTAs may hold TMEM on one SM: pad the shared memory so no more fit
  const int per_sm = std::max(1, 512 / args.ncols);
  const size_t cap = 227 * 1024;
  const size_t floor_smem = (size_t)233472 / (per_sm + 1) + 1024;
  const size_t smem = std::min(cap, std::max(carve, floor_smem));
  ANNF_REQUIRE(carve <= cap, "tensor-core leaf kNN: leaf too large for shared memory");
  const int grid = std::max(1, std::min(per_sm * num_sms(), L));
  const int km = K <= 1 ? 1 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
  int rc;
#define ANNF_TC_LAUNCH(KMV)                                                                            \
  case KMV:                                                                                            \
    if (prec == 0)                                                                                     \
      rc = kpad == 16 ? launch_leaf_tc<KMV, 16, 0>(args, smem, grid, st) : launch_leaf_tc<KMV, 32, 0>(args, smem, grid, st); \
    else if (prec == 1)                                                                                \
      rc = kpad == 16 ? launch_leaf_tc<KMV, 16, 1>(args, smem, grid, st) : launch_leaf_tc<KMV, 32, 1>(args, smem, grid, st); \
    else                                                                                               \
      rc = kpad == 16 ? launch_leaf_tc<KMV, 16, 2>(args, smem, grid, st) : launch_leaf_tc<KMV, 32, 2>(args, smem, grid, st); \
    break;
  switch (km) {
    ANNF_TC_LAUNCH(1)
    ANNF_TC_LAUNCH(4)
    ANNF_TC_LAUNCH(8)
    ANNF_TC_LAUNCH(16)
    ANNF_TC_LAUNCH(32)
    default:
      rc = ANNF_ERR_UNSUPPORTED;
  }
#undef ANNF_TC_LAUNCH
  return rc;
}

// ---------------------------------------------------------------------------------------------
// single-tile check of the tcgen05 path: D[128][N] = A[128][K] . B[N][K]^T (BF16 in, FP32 out)
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTcThreads) tc_tile_kernel(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                             int N, int K, int ncols, float* __restrict__ D,
                                                             unsigned* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* sA = smem_raw;
  unsigned char* sB = sA + (size_t)128 * K * 2;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sB + (size_t)N * K * 2);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  int* sflag = reinterpret_cast<int*>(tslot + 2);
  if (smem_overrun(smem_raw, sflag + 2, status)) return;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tc::tmem_alloc(tslot, (uint32_t)ncols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(mbar, 1);
    tc::mbar_fence_init();
    sflag[0] = 0;
  }
  for (int e = tid; e < 128 * (K / 8); e += kTcThreads) {
    const int r = e / (K / 8), k8 = (e - r * (K / 8)) * 8;
    *reinterpret_cast<uint4*>(sA + tc::core_offset(r, k8, K)) = *reinterpret_cast<const uint4*>(A + (size_t)r * K + k8);
  }
  for (int e = tid; e < N * (K / 8); e += kTcThreads) {
    const int r = e / (K / 8), k8 = (e - r * (K / 8)) * 8;
    *reinterpret_cast<uint4*>(sB + tc::core_offset(r, k8, K)) = *reinterpret_cast<const uint4*>(B + (size_t)r * K + k8);
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, N);
    for (int kk = 0; kk < K / 16; ++kk)
      tc::mma_bf16(tmem, tc::sdesc(sA + kk * 256, 128, (K / 8) * 128), tc::sdesc(sB + kk * 256, 128, (K / 8) * 128),
                   idesc, kk > 0 ? 1u : 0u);
    tc::mma_commit(mbar);
  }
  if (!mbar_wait_clock(mbar, 0)) sflag[0] = 1;
  __syncthreads();
  if (sflag[0]) {
    if (tid == 0) atomicOr(status, DEV_TC_TIMEOUT);
    mbar_wait_clock(mbar, 0);
  } else {
    tc::fence_after_sync();
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t r[16];
      tc::tmem_ld16(trow + (uint32_t)c0, r);
      tc::tmem_wait_ld();
#pragma unroll
      for (int j = 0; j < 16; ++j) D[(size_t)tid * N + c0 + j] = __uint_as_float(r[j]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)ncols);
}

int tc_tile(const uint16_t* A, const uint16_t* B, int N, int K, float* D, unsigned* status, cudaStream_t st) {
  ANNF_REQUIRE(N >= 16 && N <= 256 && N % 16 == 0, "annf_tc_tile: N must be a multiple of 16 in [16, 256]");
  ANNF_REQUIRE(K >= 16 && K <= 256 && K % 16 == 0, "annf_tc_tile: K must be a multiple of 16 in [16, 256]");
  const size_t smem = (size_t)128 * K * 2 + (size_t)N * K * 2 + 64;
  ANNF_CUDA_TRY(cudaFuncSetAttribute(tc_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  tc_tile_kernel<<<1, kTcThreads, smem, st>>>(A, B, N, K, std::max(32, next_pow2(N)), D, status);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

}  // namespace annf
