// tree_build.cu -- level-synchronous k-d tree build on the GPU (sm_103a).
//
// Reproduces the reference build bit for bit (annfmp/openmp/kdtree/src/kdtree.c:76-117, 363-489,
// helper.c:63-113, util.c:146-186):
//   * node ranges are data-independent: a node over count points gives its left child the first
//     count/2 positions and its right child the rest;
//   * axis = first axis whose bounding-box width (max - min, rounded) is strictly the largest;
//   * pivot = the order statistic of rank count/2 on that axis (any exact selection agrees);
//   * element order after the split: "< pivot" elements in input order, then ">= pivot" elements
//     in reverse input order, then a forward pass that swaps the elements equal to the pivot, in
//     the order met, to the front of the ">=" block; split value = element at position count/2.
//
// Large segments (top levels) are processed by many CTAs per segment, with the points column-major
// (a level's split coordinate is one contiguous column): an 11/11/10-bit radix select of the median
// over the split column, a stable scatter of every column that finds each chunk's offset by a
// decoupled look-back and forms the children's bounding boxes (atomics on order-preserving keys),
// and a one-warp fix-up for the equal elements. When a level's segments fit in shared memory, one
// CTA per segment finishes the whole subtree in shared memory (bounding box, 8-bit-digit radix
// select and stable partition on a 16-bit index permutation) and writes the points out once, row
// by row, in leaf order.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "handle.cuh"

namespace annf {

int num_sms();

constexpr int kChunk = 2048;     // positions per CTA in the global levels
constexpr int kThreads = 256;
constexpr int kItems = kChunk / kThreads;

// [lo, hi) of node j (0-based within its level) at level t of a tree over n points
__device__ __forceinline__ void seg_range(int n, int t, int j, int& lo, int& hi) {
  int a = 0, c = n;
  for (int b = t - 1; b >= 0; --b) {
    int half = c >> 1;
    if ((j >> b) & 1) {
      a += half;
      c -= half;
    } else {
      c = half;
    }
  }
  lo = a;
  hi = a + c;
}

template <typename K> __device__ __forceinline__ K key_max();
template <> __device__ __forceinline__ uint32_t key_max<uint32_t>() { return 0xffffffffu; }
template <> __device__ __forceinline__ unsigned long long key_max<unsigned long long>() { return ~0ull; }

template <typename K>
__global__ void fill_keys_kernel(K* a, long long cnt, K v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x) a[i] = v;
}

__global__ void iota_kernel(int* a, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

// ---------------------------------------------------------------------------------------------
// global levels
// ---------------------------------------------------------------------------------------------
// Between the input and the finisher the points are column-major ([d][n]): a level reads its
// split coordinate as one contiguous column, and the scatter moves columns.
//
// row-major [n][d] -> column-major [d][n] through shared memory (tile rows of stride d | 1), and
// the bounding box of all points as order keys (level 0's box): a reading thread always reads the
// same dimension
template <typename T>
__host__ __device__ __forceinline__ int col_tile_rows(int d) {
  const int r = 16384 / ((d | 1) * (int)sizeof(T));
  return r < 32 ? 32 : (r > 256 ? 256 : r);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) to_columns_kernel(int n, int d, const T* __restrict__ in,
                                                              T* __restrict__ out, typename key_of<T>::type* gmin,
                                                              typename key_of<T>::type* gmax) {
  using K = typename key_of<T>::type;
  extern __shared__ __align__(16) unsigned char csm[];
  T* tile = reinterpret_cast<T*>(csm);
  const int rows = col_tile_rows<T>(d), ds = d | 1;
  const int per = kThreads / d, used = per * d;  // readers: thread t reads dimension t % d of rows t / d + k * per
  const int rj = (int)threadIdx.x % d, rr = (int)threadIdx.x / d;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  K kmn = key_max<K>(), kmx = 0;
  for (long long r0 = (long long)blockIdx.x * rows; r0 < n; r0 += (long long)gridDim.x * rows) {
    const int m = (int)(n - r0 < rows ? n - r0 : rows);
    if ((int)threadIdx.x < used) {
      const T* src = in + r0 * d + rj;
#pragma unroll 4
      for (int r = rr; r < m; r += per) {
        const T v = src[(long long)r * d];
        tile[r * ds + rj] = v;
        const K k = (K)ord_key(v);
        kmn = k < kmn ? k : kmn;
        kmx = k > kmx ? k : kmx;
      }
    }
    __syncthreads();
    for (int j = warp; j < d; j += kThreads / 32) {
      T* dst = out + (long long)j * n + r0;
#pragma unroll 4
      for (int r = lane; r < m; r += 32) dst[r] = tile[r * ds + j];
    }
    __syncthreads();
  }
  __shared__ K smin[kThreads], smax[kThreads];
  smin[threadIdx.x] = kmn;
  smax[threadIdx.x] = kmx;
  __syncthreads();
  if ((int)threadIdx.x < d) {
    for (int u = threadIdx.x + d; u < used; u += d) {
      kmn = smin[u] < kmn ? smin[u] : kmn;
      kmx = smax[u] > kmx ? smax[u] : kmx;
    }
    if (kmn != key_max<K>()) atomicMin(&gmin[threadIdx.x], kmn);
    if (kmx != (K)0) atomicMax(&gmax[threadIdx.x], kmx);
  }
}

// column-major [d][n] -> row-major [n][d] (the leaves when no level fits the finisher)
template <typename T>
__global__ void __launch_bounds__(kThreads) to_rows_kernel(int n, int d, const T* __restrict__ in, T* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char csm[];
  T* tile = reinterpret_cast<T*>(csm);
  const int rows = col_tile_rows<T>(d), ds = d | 1;
  const int per = kThreads / d, used = per * d;
  const int rj = (int)threadIdx.x % d, rr = (int)threadIdx.x / d;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long r0 = (long long)blockIdx.x * rows; r0 < n; r0 += (long long)gridDim.x * rows) {
    const int m = (int)(n - r0 < rows ? n - r0 : rows);
    for (int j = warp; j < d; j += kThreads / 32) {
      const T* src = in + (long long)j * n + r0;
      for (int r = lane; r < m; r += 32) tile[r * ds + j] = src[r];
    }
    __syncthreads();
    if ((int)threadIdx.x < used) {
      T* dst = out + r0 * d + rj;
      for (int r = rr; r < m; r += per) dst[(long long)r * d] = tile[r * ds + rj];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void axis_kernel(int n, int d, int t, int S, int splitting, const typename key_of<T>::type* gmin,
                            const typename key_of<T>::type* gmax, int* axis,
                            typename key_of<T>::type* prefix, int* rank, int* nlt,
                            typename key_of<T>::type* cmin, typename key_of<T>::type* cmax) {
  using K = typename key_of<T>::type;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  if (cmin != nullptr) {  // the children's boxes, filled by this level's scatter: start empty
    for (int j = 0; j < 2 * d; ++j) {
      cmin[(long long)2 * s * d + j] = key_max<K>();
      cmax[(long long)2 * s * d + j] = (K)0;
    }
  }
  int lo, hi;
  seg_range(n, t, s, lo, hi);
  T best = 0;
  int ax = 0;
  for (int j = 0; j < d; ++j) {
    T mn, mx;
    if constexpr (sizeof(T) == 4) {
      mn = key_to_float((uint32_t)gmin[(long long)s * d + j]);
      mx = key_to_float((uint32_t)gmax[(long long)s * d + j]);
    } else {
      mn = key_to_real(gmin[(long long)s * d + j]);
      mx = key_to_real(gmax[(long long)s * d + j]);
    }
    T w = real_traits<T>::sub(mx, mn);
    if (w > best) {
      best = w;
      ax = j;
    }
  }
  axis[s] = splitting == 0 ? t % d : ax;  // cyclic: node depth mod d (kdtree.c:369-371)
  prefix[s] = 0;
  rank[s] = (hi - lo) / 2;
  nlt[s] = 0;
}

// one radix-select pass: histogram of the current digit (width bits at shift, at most kSelBits)
// over the keys that match the prefix found so far. The first pass reads the split axis from the
// points and writes the keys. Lanes of a warp that hit the same bin (common: a segment's keys share
// their high digits) add once, together.
constexpr int kSelBits = 11;                 // widest digit: 32-bit keys take three passes (11, 11, 10)
constexpr int kHistChunks = 2;               // chunks per histogram CTA
constexpr int kSelBins = 1 << kSelBits;
template <typename T>
__global__ void hist_kernel(int n, int d, int t, int HB, int shift, int width, bool extract, const T* __restrict__ pts,
                            const int* __restrict__ axis, typename key_of<T>::type* __restrict__ keys,
                            const typename key_of<T>::type* __restrict__ prefix, unsigned* ghist) {
  using K = typename key_of<T>::type;
  __shared__ unsigned h[kSelBins];
  // a CTA takes kHistChunks consecutive chunks of its segment (HB CTAs per segment): one shared
  // histogram, flushed once
  const int s = blockIdx.x / HB, bb = blockIdx.x % HB;
  int lo, hi;
  seg_range(n, t, s, lo, hi);
  const int nb = 1 << width;
  for (int z = threadIdx.x; z < nb; z += blockDim.x) h[z] = 0;
  __syncthreads();
  const K pre = prefix[s];
  const K hmask = (shift + width >= (int)(8 * sizeof(K))) ? (K)0 : (~(K)0 << (shift + width));
  const int ax = axis[s];
  const int lane = threadIdx.x & 31;
  for (int cc = 0; cc < kHistChunks; ++cc) {
    const int c0 = lo + (bb * kHistChunks + cc) * kChunk, c1 = min(hi, c0 + kChunk);
    if (c0 >= c1) break;  // uniform per block
    // every load of the thread's kItems elements first (all in flight at once), then the bins
    K kv[kItems];
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
      const int i = c0 + (int)threadIdx.x + q * kThreads;
      kv[q] = 0;
      if (i < c1) kv[q] = extract ? (K)ord_key(pts[(long long)ax * n + i]) : keys[i];
    }
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
      const int i = c0 + (int)threadIdx.x + q * kThreads;
      if (c0 + q * kThreads >= c1) break;  // uniform: no element of this round in the chunk
      unsigned bin = kSelBins;
      if (i < c1) {
        const K k = kv[q];
        if (extract) keys[i] = k;
        if (((k ^ pre) & hmask) == 0) bin = (unsigned)(k >> shift) & (unsigned)(nb - 1);
      }
      const unsigned peers = __match_any_sync(0xffffffffu, bin);
      if (bin != (unsigned)kSelBins && lane == __ffs(peers) - 1) atomicAdd(&h[bin], (unsigned)__popc(peers));
    }
  }
  __syncthreads();
  for (int z = threadIdx.x; z < nb; z += blockDim.x) {
    const unsigned v = h[z];
    if (v) atomicAdd(&ghist[(long long)s * kSelBins + z], v);
  }
}

// block-wide exclusive scan of two counters (kThreads threads)
__device__ __forceinline__ void block_excl_scan2(int a, int b, int& ea, int& eb, int& ta, int& tb) {
  __shared__ int wa[kThreads / 32], wb[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) {
      ia += xa;
      ib += xb;
    }
  }
  if (lane == 31) {
    wa[w] = ia;
    wb[w] = ib;
  }
  __syncthreads();
  int pa = 0, pb = 0, sa = 0, sb = 0;
  for (int u = 0; u < kThreads / 32; ++u) {
    if (u < w) {
      pa += wa[u];
      pb += wb[u];
    }
    sa += wa[u];
    sb += wb[u];
  }
  ea = pa + ia - a;
  eb = pb + ib - b;
  ta = sa;
  tb = sb;
  __syncthreads();
}

// the bin of the digit that holds rank r (kThreads threads, kSelBins / kThreads bins each, read
// and cleared for the next pass)
template <typename K>
__global__ void pick_kernel(int shift, bool last, unsigned* ghist, K* prefix, int* rank, int* nlt,
                            int* neq) {
  constexpr int kPer = kSelBins / kThreads;
  const int s = blockIdx.x;
  unsigned* h = ghist + (long long)s * kSelBins;
  int c[kPer], sum = 0;
#pragma unroll
  for (int u = 0; u < kPer; ++u) {
    c[u] = (int)h[threadIdx.x * kPer + u];
    h[threadIdx.x * kPer + u] = 0;  // ready for the next pass
    sum += c[u];
  }
  int ex, dummy_e, tot, dummy_t;
  block_excl_scan2(sum, 0, ex, dummy_e, tot, dummy_t);
  const int r = rank[s];
  __syncthreads();
  if (ex <= r && r < ex + sum) {
    int run = ex;
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      if (run <= r && r < run + c[u]) {
        prefix[s] |= ((K)(threadIdx.x * kPer + u)) << shift;
        rank[s] = r - run;
        nlt[s] += run;
        if (last) neq[s] = c[u];
      }
      run += c[u];
    }
  }
}

// Per-chunk state of a level's scatter (decoupled look-back, zeroed before the level): a 64-bit
// word per chunk, flag in bits 62-63 (0 not ready, 1 the chunk's own counts, 2 the inclusive
// counts of the segment's chunks up to it), "<" count in bits 31-61, "==" count in bits 0-30.
constexpr long long kLookSpins = 1LL << 21;  // bound of a chunk's wait for a predecessor (~0.1 s)
__device__ __forceinline__ unsigned long long chunk_word(unsigned flag, int lt, int eq) {
  return ((unsigned long long)flag << 62) | ((unsigned long long)(unsigned)lt << 31) | (unsigned)eq;
}

// the counts of the segment's chunks before chunk bb ("<" and "==" of the pivot), by thread 0;
// publishes this chunk's own counts first and its inclusive counts last. Predecessors have lower
// block indices, so they started first; a wait that runs out sets DEV_LOOKBACK_TIMEOUT.
__device__ __forceinline__ void chunk_lookback(unsigned long long* st, int bb, int lt, int eq, int& pre_lt,
                                               int& pre_eq, unsigned* status) {
  pre_lt = 0;
  pre_eq = 0;
  if (bb == 0) {
    atomicExch(st, chunk_word(2u, lt, eq));
    return;
  }
  atomicExch(st + bb, chunk_word(1u, lt, eq));
  long long spins = 0;
  for (int u = bb - 1; u >= 0;) {
    const unsigned long long v = *reinterpret_cast<volatile unsigned long long*>(st + u);
    const unsigned flag = (unsigned)(v >> 62);
    if (flag == 0u) {
      if (++spins > kLookSpins) {
        atomicOr(status, DEV_LOOKBACK_TIMEOUT);
        break;
      }
      __nanosleep(32);
      continue;
    }
    pre_lt += (int)((v >> 31) & 0x7fffffffu);
    pre_eq += (int)(v & 0x7fffffffu);
    if (flag == 2u) break;
    --u;
  }
  atomicExch(st + bb, chunk_word(2u, pre_lt + lt, pre_eq + eq));
}

template <typename T>
__global__ void __launch_bounds__(kThreads) scatter_kernel(
    int n, int d, int t, int B, const typename key_of<T>::type* __restrict__ keys,
    const typename key_of<T>::type* __restrict__ pivot, const int* __restrict__ nlt,
    const int* __restrict__ neq, unsigned long long* __restrict__ chunk_st, unsigned* status,
    const T* __restrict__ pts_in, const int* __restrict__ perm_in, T* __restrict__ pts_out,
    int* __restrict__ perm_out, int* __restrict__ eqpos, typename key_of<T>::type* cmin,
    typename key_of<T>::type* cmax) {
  using K = typename key_of<T>::type;
  __shared__ int sdst[kChunk];
  __shared__ unsigned char sside[kChunk];  // child of each element: 0 left, 1 right
  const int s = blockIdx.x / B, bb = blockIdx.x % B;
  int lo, hi;
  seg_range(n, t, s, lo, hi);
  const int c0 = lo + bb * kChunk, c1 = min(hi, c0 + kChunk);
  const int m = c1 - c0;
  if (m <= 0) return;  // uniform per block
  const K pv = pivot[s];
  __shared__ K skeys[kChunk];
  for (int i = threadIdx.x; i < m; i += blockDim.x) skeys[i] = keys[c0 + i];  // coalesced
  __syncthreads();
  const int base = threadIdx.x * kItems;
  unsigned flt = 0, feq = 0;
  int mlt = 0, meq = 0;
#pragma unroll
  for (int q = 0; q < kItems; ++q) {
    int i = base + q;
    if (i < m) {
      K k = skeys[i];
      if (k < pv) {
        flt |= 1u << q;
        ++mlt;
      } else if (k == pv) {
        feq |= 1u << q;
        ++meq;
      }
    }
  }
  int elt, eeq, tl, te;
  block_excl_scan2(mlt, meq, elt, eeq, tl, te);
  // this chunk's offsets among its segment's chunks
  __shared__ int spre[2];
  if (threadIdx.x == 0) {
    int pl, pe;
    chunk_lookback(chunk_st + (long long)s * B, bb, tl, te, pl, pe, status);
    spre[0] = pl;
    spre[1] = pe;
  }
  __syncthreads();
  const int sum_lt = spre[0], sum_eq = spre[1];
  int lt_before = sum_lt + elt;
  int eq_before = sum_eq + eeq;
  const int seg_neq = neq[s];
  // after the fix-up the left child holds the "<" elements and the first (half - nlt) equal
  // elements of the ">=" block, i.e. the equal elements of input rank >= neq - (half - nlt)
  const int eq_left_from = seg_neq - ((hi - lo) / 2 - nlt[s]);
#pragma unroll
  for (int q = 0; q < kItems; ++q) {
    int i = base + q;
    if (i < m) {
      int r = (c0 - lo) + i;  // rank of the element in its segment (input order)
      int dst;
      unsigned char side = 1;
      if ((flt >> q) & 1u) {
        dst = lo + lt_before;
        ++lt_before;
        side = 0;
      } else {
        dst = hi - 1 - (r - lt_before);  // ">=" elements fill from the back
        if ((feq >> q) & 1u) {
          eqpos[lo + (seg_neq - 1 - eq_before)] = dst;  // ascending position order
          side = eq_before >= eq_left_from ? 0 : 1;
          ++eq_before;
        }
      }
      sdst[i] = dst;
      sside[i] = side;
    }
  }
  __syncthreads();
  // the columns move one at a time, a warp per column, lanes on consecutive positions (coalesced
  // reads; a warp's writes fall in the two runs of its children). With cmin, the children's
  // bounding boxes on the way, as order keys (the same keys as to_columns_kernel's)
  constexpr int kU = 8;  // loads in flight per lane
  const int lane = threadIdx.x & 31;
  for (int j = threadIdx.x >> 5; j < d; j += kThreads / 32) {
    const T* src = pts_in + (long long)j * n + c0;
    T* dcol = pts_out + (long long)j * n;
    K mn0 = key_max<K>(), mx0 = (K)0, mn1 = key_max<K>(), mx1 = (K)0;
    bool h0 = false, h1 = false;
    for (int r0 = lane; r0 < m; r0 += 32 * kU) {
      T v[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u)
        if (r0 + 32 * u < m) v[u] = src[r0 + 32 * u];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int r = r0 + 32 * u;
        if (r < m) {
          dcol[sdst[r]] = v[u];
          if (cmin != nullptr) {
            const K k = (K)ord_key(v[u]);
            if (sside[r]) {
              h1 = true;
              mn1 = k < mn1 ? k : mn1;
              mx1 = k > mx1 ? k : mx1;
            } else {
              h0 = true;
              mn0 = k < mn0 ? k : mn0;
              mx0 = k > mx0 ? k : mx0;
            }
          }
        }
      }
    }
    if (cmin != nullptr) {
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        K x = __shfl_xor_sync(0xffffffffu, mn0, o);
        mn0 = x < mn0 ? x : mn0;
        x = __shfl_xor_sync(0xffffffffu, mx0, o);
        mx0 = x > mx0 ? x : mx0;
        x = __shfl_xor_sync(0xffffffffu, mn1, o);
        mn1 = x < mn1 ? x : mn1;
        x = __shfl_xor_sync(0xffffffffu, mx1, o);
        mx1 = x > mx1 ? x : mx1;
      }
      h0 = __any_sync(0xffffffffu, h0);
      h1 = __any_sync(0xffffffffu, h1);
      if (lane == 0) {
        if (h0) {
          atomicMin(&cmin[(long long)(2 * s) * d + j], mn0);
          atomicMax(&cmax[(long long)(2 * s) * d + j], mx0);
        }
        if (h1) {
          atomicMin(&cmin[(long long)(2 * s + 1) * d + j], mn1);
          atomicMax(&cmax[(long long)(2 * s + 1) * d + j], mx1);
        }
      }
    }
  }
  int pv_[kItems];
#pragma unroll
  for (int q = 0; q < kItems; ++q) {
    const int i = (int)threadIdx.x + q * kThreads;
    if (i < m) pv_[q] = perm_in[c0 + i];
  }
#pragma unroll
  for (int q = 0; q < kItems; ++q) {
    const int i = (int)threadIdx.x + q * kThreads;
    if (i < m) perm_out[sdst[i]] = pv_[q];
  }
}

// one warp per segment: the reference's forward swap pass over the equal elements, then the node
template <typename T>
__global__ void fixup_kernel(int n, int d, int t, int S, const int* __restrict__ axis,
                             const int* __restrict__ nlt, const int* __restrict__ neq,
                             const int* __restrict__ eqpos, T* pts, int* perm, int* node_axis,
                             T* node_split) {
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (s >= S) return;
  int lo, hi;
  seg_range(n, t, s, lo, hi);
  const int m = neq[s], h0 = lo + nlt[s];
  for (int j = 0; j < m; ++j) {
    const int p = eqpos[lo + j], q = h0 + j;
    if (p != q) {
      for (int c = lane; c < d; c += 32) {
        T a = pts[(long long)c * n + p];
        pts[(long long)c * n + p] = pts[(long long)c * n + q];
        pts[(long long)c * n + q] = a;
      }
      if (lane == 0) {
        int a = perm[p];
        perm[p] = perm[q];
        perm[q] = a;
      }
    }
    __syncwarp();
  }
  if (lane == 0) {
    const int node = (1 << t) - 1 + s;
    const int ax = axis[s];
    node_axis[node] = ax;
    node_split[node] = pts[(long long)ax * n + lo + (hi - lo) / 2];
  }
}

// leaves produced by the global levels (depth reached without the shared-memory finisher)
__global__ void leaves_kernel(int n, int depth, int B, const int* __restrict__ perm, int* leaf_begin,
                              int* point_leaf) {
  const int s = blockIdx.x / B, bb = blockIdx.x % B;
  int lo, hi;
  seg_range(n, depth, s, lo, hi);
  const int c0 = lo + bb * kChunk, c1 = min(hi, c0 + kChunk);
  if (bb == 0 && threadIdx.x == 0) {
    leaf_begin[s] = lo;
    if (s == (1 << depth) - 1) leaf_begin[s + 1] = n;
  }
  for (int i = c0 + threadIdx.x; i < c1; i += blockDim.x) point_leaf[perm[i]] = s;
}

// per-leaf bounding box (warp per leaf): box[l][0][j] = min, box[l][1][j] = max over the leaf
template <typename T>
__global__ void leaf_box_kernel(int L, int d, const T* __restrict__ pts, const int* __restrict__ leaf_begin,
                                T* __restrict__ box) {
  const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (l >= L) return;
  const int beg = leaf_begin[l], end = leaf_begin[l + 1];
  for (int j = 0; j < d; ++j) {
    T mn = real_traits<T>::big(), mx = -real_traits<T>::big();
    for (int p = beg + lane; p < end; p += 32) {
      const T v = pts[(long long)p * d + j];
      mn = v < mn ? v : mn;
      mx = v > mx ? v : mx;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const T a = __shfl_xor_sync(0xffffffffu, mn, o), b = __shfl_xor_sync(0xffffffffu, mx, o);
      mn = a < mn ? a : mn;
      mx = b > mx ? b : mx;
    }
    if (lane == 0) {
      box[((long long)l * 2) * d + j] = mn;
      box[((long long)l * 2 + 1) * d + j] = mx;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// shared-memory subtree finisher: one CTA per segment of level t0, levels t0..depth-1
//
// Staged points use an odd row stride (d | 1), so that lanes reading one coordinate of different
// rows fall in different banks. While a level has fewer segments than warps, a segment is shared
// by G = warps / segments warps: each takes a contiguous chunk of the segment's positions; their
// bounding-box partials, histogram counts and "<" counts are combined in shared memory, so the
// result is the one a single warp walking the segment in order produces. From the level with one
// segment per warp on, each warp splits its segments alone.
// ---------------------------------------------------------------------------------------------
constexpr int kSubThreads = 512;
constexpr int kSubWarps = kSubThreads / 32;

__host__ __device__ __forceinline__ int sub_stride(int d) { return d | 1; }

// radix-select step of one warp: from the 256-bin histogram of the keys that match the prefix,
// the bin holding rank 'rank' and the number of keys in lower bins
__device__ __forceinline__ void select_bin(const unsigned* hist, int lane, int rank, int& bin, int& before) {
  int c[8], tot = 0;
#pragma unroll
  for (int z = 0; z < 8; ++z) {
    c[z] = (int)hist[8 * lane + z];  // lane owns bins [8*lane, 8*lane+8)
    tot += c[z];
  }
  int inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int x = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += x;
  }
  const int ex = inc - tot;
  const unsigned own = __ballot_sync(0xffffffffu, ex <= rank && rank < inc);
  const int src = __ffs(own) - 1;
  bin = 0;
  before = 0;
  if (lane == src) {
    int run = ex;
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      if (run <= rank && rank < run + c[z]) {
        bin = 8 * lane + z;
        before = run;
      }
      run += c[z];
    }
  }
  bin = __shfl_sync(0xffffffffu, bin, src);
  before = __shfl_sync(0xffffffffu, before, src);
}

// histogram of the keys in [ca, cb) that match prefix under hmask, by one warp (aggregated atomics)
template <typename K>
__device__ __forceinline__ void warp_hist(const K* skey, int ca, int cb, int lane, K prefix, K hmask, int shift,
                                          unsigned* hist) {
  for (int base = ca; base < cb; base += 32) {
    const int i = base + lane;
    unsigned bin = 256u;
    if (i < cb) {
      const K k = skey[i];
      if (((k ^ prefix) & hmask) == 0) bin = (unsigned)(k >> shift) & 255u;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, bin);
    if (bin != 256u && lane == __ffs(peers) - 1) atomicAdd(&hist[bin], (unsigned)__popc(peers));
  }
}

// stable partition of positions [ca, cb) by key < pivot: "<" forward from a + ltb, ">=" backward
// from b - 1 - geb (cur -> nxt)
template <typename K>
__device__ __forceinline__ void warp_partition(const K* skey, const uint16_t* cur, uint16_t* nxt, int ca, int cb,
                                               int a, int b, int lane, K pivot, int ltb, int geb) {
  for (int base = ca; base < cb; base += 32) {
    const int i = base + lane;
    const bool valid = i < cb;
    const K k = valid ? skey[i] : (K)0;
    const bool lt = valid && (k < pivot), ge = valid && !(k < pivot);
    const unsigned mlt = __ballot_sync(0xffffffffu, lt), mge = __ballot_sync(0xffffffffu, ge);
    const unsigned below = (1u << lane) - 1u;
    if (lt) nxt[a + ltb + __popc(mlt & below)] = cur[i];
    if (ge) nxt[b - 1 - (geb + __popc(mge & below))] = cur[i];
    ltb += __popc(mlt);
    geb += __popc(mge);
  }
}

// forward swap pass of the elements equal to the pivot over the ">=" block [a + nlt, b), then the
// node's axis and split value (one warp)
template <typename T, typename K>
__device__ __forceinline__ void warp_finish_split(const T* spts, int ds, uint16_t* nxt, int a, int b, int nlt,
                                                  int half, int axis, K pivot, int lane, int node,
                                                  int* __restrict__ node_axis, T* __restrict__ node_split) {
  int w = a + nlt;
  for (int base = a + nlt; base < b; base += 32) {
    const int i = base + lane;
    const bool eq = i < b && ord_key(spts[(size_t)nxt[i] * ds + axis]) == pivot;
    unsigned msk = __ballot_sync(0xffffffffu, eq);
    while (msk) {
      const int p = base + __ffs(msk) - 1;
      msk &= msk - 1;
      if (lane == 0 && p != w) {
        uint16_t tmp = nxt[p];
        nxt[p] = nxt[w];
        nxt[w] = tmp;
      }
      ++w;
      __syncwarp();
    }
  }
  if (lane == 0) {
    node_axis[node] = axis;
    node_split[node] = spts[(size_t)nxt[a + half] * ds + axis];
  }
}

// bounding box of rows [ca, cb) (through cur) over dimensions [j0, j0 + 16) by one warp, row by
// row: each lane keeps the minima and the negated maxima of its rows (32 values), then a
// recursive-halving reduction (31 shuffles) leaves slot l in lane l: slots 0..15 the minima of
// dimensions j0.., slots 16..31 the negated maxima. Start values as the per-dimension loops used
// (big, -big); only widths are taken from these boxes, so the order of the reduction is free.
template <typename T>
__device__ __forceinline__ T warp_box16(const T* spts, int ds, const uint16_t* cur, int ca, int cb, int j0, int d,
                                        int lane) {
  T v[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = real_traits<T>::big();
  const int nj = d - j0;
  for (int i = ca + lane; i < cb; i += 32) {
    const T* row = spts + (size_t)cur[i] * ds + j0;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k < nj) {
        const T x = row[k];
        v[k] = x < v[k] ? x : v[k];
        v[16 + k] = -x < v[16 + k] ? -x : v[16 + k];
      }
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < o; ++k) {
      const T send = up ? v[k] : v[k + o];
      const T keep = up ? v[k + o] : v[k];
      const T recv = __shfl_xor_sync(0xffffffffu, send, o);
      v[k] = recv < keep ? recv : keep;
    }
  }
  return v[0];
}

template <typename T>
__global__ void __launch_bounds__(kSubThreads) subtree_kernel(
    int n, int d, int depth, int t0, int smax, int splitting, const T* __restrict__ pts_in,
    const int* __restrict__ perm_in, T* __restrict__ pts_out, int* __restrict__ perm_out,
    int* __restrict__ node_axis, T* __restrict__ node_split, int* __restrict__ leaf_begin,
    int* __restrict__ point_leaf, T* __restrict__ leaf_box, unsigned* status) {
  using K = typename key_of<T>::type;
  constexpr int kBits = 8 * sizeof(K);
  const int ds = sub_stride(d);
  extern __shared__ __align__(16) unsigned char smem[];
  T* spts = reinterpret_cast<T*>(smem);                         // [smax][ds]
  T* spmn = spts + (size_t)smax * ds;                           // [warps][d] bounding-box partials
  T* spmx = spmn + (size_t)kSubWarps * d;
  K* skey = reinterpret_cast<K*>(spmx + (size_t)kSubWarps * d);  // [smax]
  K* sprefix = skey + smax;                                     // [warps] per-group select state
  int* sperm = reinterpret_cast<int*>(sprefix + kSubWarps);     // [smax]
  int* saxis = sperm + smax;
  int* srank = saxis + kSubWarps;
  int* snlt = srank + kSubWarps;
  int* scnt = snlt + kSubWarps;
  unsigned* shist = reinterpret_cast<unsigned*>(scnt + kSubWarps);  // [warps][256]
  uint16_t* sidx0 = reinterpret_cast<uint16_t*>(shist + kSubWarps * 256);
  uint16_t* sidx1 = sidx0 + smax;
  if (smem_overrun(smem, sidx1 + smax, status)) return;

  const int s = blockIdx.x;
  int lo, hi;
  seg_range(n, t0, s, lo, hi);
  const int cnt = hi - lo;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  // the segment's columns (column-major points), sixteen loads in flight per thread, into padded rows
  for (int j0 = 0; j0 < d; j0 += 16) {
    for (int r = threadIdx.x; r < cnt; r += kSubThreads) {
      T v[16];
#pragma unroll
      for (int u = 0; u < 16; ++u)
        if (j0 + u < d) v[u] = __ldg(pts_in + (long long)(j0 + u) * n + lo + r);
#pragma unroll
      for (int u = 0; u < 16; ++u)
        if (j0 + u < d) spts[(size_t)r * ds + j0 + u] = v[u];
    }
  }
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    sperm[i] = perm_in[lo + i];
    sidx0[i] = (uint16_t)i;
  }
  __syncthreads();

  uint16_t* cur = sidx0;
  uint16_t* nxt = sidx1;

  for (int l = t0; l < depth; ++l) {
    const int nsub = 1 << (l - t0);
    if (nsub >= kSubWarps) {
      // ---- one warp per segment ----
      unsigned* hist = shist + warp * 256;
      for (int u = warp; u < nsub; u += kSubWarps) {
        int a, b;
        seg_range(cnt, l - t0, u, a, b);
        const int half = (b - a) / 2;
        T best = 0;
        int axis = splitting == 0 ? l % d : 0;
        for (int j0 = 0; splitting != 0 && j0 < d; j0 += 16) {
          // widths of dimensions j0 + lane (lanes < 16), then the serial rule: the first strictly
          // widest, over the chunk's lanes in order and across chunks
          const T r = warp_box16<T>(spts, ds, cur, a, b, j0, d, lane);
          const T mx = -__shfl_sync(0xffffffffu, r, (lane & 15) + 16);
          T bw = (lane < 16 && j0 + lane < d) ? real_traits<T>::sub(mx, r) : -real_traits<T>::big();
          int bj = j0 + lane;
#pragma unroll
          for (int o = 16; o; o >>= 1) {
            const T ow = __shfl_xor_sync(0xffffffffu, bw, o);
            const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
            if (ow > bw || (ow == bw && oj < bj)) {
              bw = ow;
              bj = oj;
            }
          }
          if (bw > best) {
            best = bw;
            axis = bj;
          }
        }
        for (int i = a + lane; i < b; i += 32) skey[i] = ord_key(spts[(size_t)cur[i] * ds + axis]);
        K prefix = 0;
        int rank = half, nlt = 0;
        for (int shift = kBits - 8; shift >= 0; shift -= 8) {
          for (int z = lane; z < 256; z += 32) hist[z] = 0;
          __syncwarp();
          const K hmask = (shift + 8 >= kBits) ? (K)0 : (~(K)0 << (shift + 8));
          warp_hist<K>(skey, a, b, lane, prefix, hmask, shift, hist);
          __syncwarp();
          int bin, before;
          select_bin(hist, lane, rank, bin, before);
          prefix |= ((K)bin) << shift;
          nlt += before;
          rank -= before;
          __syncwarp();
        }
        warp_partition<K>(skey, cur, nxt, a, b, a, b, lane, prefix, 0, 0);
        __syncwarp();
        warp_finish_split<T, K>(spts, ds, nxt, a, b, nlt, half, axis, prefix, lane,
                                (1 << l) - 1 + (s << (l - t0)) + u, node_axis, node_split);
      }
    } else {
      // ---- G warps per segment, each on a contiguous chunk ----
      const int G = kSubWarps / nsub;
      const int u = warp / G, gw = warp - u * G, w0 = u * G;
      int a, b;
      seg_range(cnt, l - t0, u, a, b);
      const int half = (b - a) / 2;
      const int cs = (((b - a) + G - 1) / G + 31) & ~31;
      const int ca = min(b, a + gw * cs), cb = min(b, ca + cs);
      if (splitting != 0) {
        for (int j0 = 0; j0 < d; j0 += 16) {
          const T r = warp_box16<T>(spts, ds, cur, ca, cb, j0, d, lane);
          const int j = j0 + (lane & 15);
          if (j < d) {
            if (lane < 16) spmn[warp * d + j] = r;
            else spmx[warp * d + j] = -r;
          }
        }
      }
      // the group's two histogram buffers, used by alternate digit passes
      unsigned* ghist = shist + u * 512;
      for (int z = gw * 32 + lane; z < 512; z += G * 32) ghist[z] = 0;
      __syncthreads();
      if (gw == 0) {
        // lanes take dimensions (lane, lane + 32, ...): the widest, first on ties, as one scan
        T best = 0;
        int axis = splitting == 0 ? l % d : 0;
        if (splitting != 0) {
          for (int j0 = 0; j0 < d; j0 += 32) {
            const int j = j0 + lane;
            T wd = -real_traits<T>::big();
            if (j < d) {
              T mn = spmn[w0 * d + j], mx = spmx[w0 * d + j];
              for (int g = 1; g < G; ++g) {
                const T omn = spmn[(w0 + g) * d + j], omx = spmx[(w0 + g) * d + j];
                mn = omn < mn ? omn : mn;
                mx = omx > mx ? omx : mx;
              }
              wd = real_traits<T>::sub(mx, mn);
            }
            // the chunk's widest (lowest dimension on ties), then the serial rule across chunks
            T bw = wd;
            int bj = j;
#pragma unroll
            for (int o = 16; o; o >>= 1) {
              const T ow = __shfl_xor_sync(0xffffffffu, bw, o);
              const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
              if (ow > bw || (ow == bw && oj < bj)) {
                bw = ow;
                bj = oj;
              }
            }
            if (bw > best) {
              best = bw;
              axis = bj;
            }
          }
        }
        if (lane == 0) {
          saxis[u] = axis;
          sprefix[u] = 0;
          srank[u] = half;
          snlt[u] = 0;
        }
      }
      __syncthreads();
      const int axis = saxis[u];
      for (int i = ca + lane; i < cb; i += 32) skey[i] = ord_key(spts[(size_t)cur[i] * ds + axis]);
      int pass = 0;
      for (int shift = kBits - 8; shift >= 0; shift -= 8, ++pass) {
        unsigned* hist = ghist + (pass & 1) * 256;
        const K hmask = (shift + 8 >= kBits) ? (K)0 : (~(K)0 << (shift + 8));
        warp_hist<K>(skey, ca, cb, lane, sprefix[u], hmask, shift, hist);
        __syncthreads();
        if (gw == 0) {
          int bin, before;
          select_bin(hist, lane, srank[u], bin, before);
          __syncwarp();
          if (lane == 0) {
            sprefix[u] |= ((K)bin) << shift;
            snlt[u] += before;
            srank[u] -= before;
          }
        }
        // the other buffer was read two passes ago: clear it for the next pass
        unsigned* other = ghist + ((pass + 1) & 1) * 256;
        for (int z = gw * 32 + lane; z < 256; z += G * 32) other[z] = 0;
        __syncthreads();
      }
      const K pivot = sprefix[u];
      int clt = 0;
      for (int base = ca; base < cb; base += 32) {
        const int i = base + lane;
        clt += __popc(__ballot_sync(0xffffffffu, i < cb && skey[i] < pivot));
      }
      if (lane == 0) scnt[warp] = clt;
      __syncthreads();
      int ltb = 0, geb = 0;
      for (int g = 0; g < gw; ++g) {
        const int ga = min(b, a + g * cs), gb = min(b, ga + cs);
        ltb += scnt[w0 + g];
        geb += (gb - ga) - scnt[w0 + g];
      }
      warp_partition<K>(skey, cur, nxt, ca, cb, a, b, lane, pivot, ltb, geb);
      __syncthreads();
      if (gw == 0)
        warp_finish_split<T, K>(spts, ds, nxt, a, b, snlt[u], half, axis, pivot, lane,
                                (1 << l) - 1 + (s << (l - t0)) + u, node_axis, node_split);
    }
    __syncthreads();
    uint16_t* tmp = cur;
    cur = nxt;
    nxt = tmp;
  }
  // leaves of this subtree
  const int nleaf = 1 << (depth - t0);
  for (int u = warp; u < nleaf; u += kSubWarps) {
    int a, b;
    seg_range(cnt, depth - t0, u, a, b);
    const int leaf = (s << (depth - t0)) + u;
    if (lane == 0) {
      leaf_begin[leaf] = lo + a;
      if (leaf == (1 << depth) - 1) leaf_begin[leaf + 1] = n;
    }
    for (int i = a + lane; i < b; i += 32) point_leaf[sperm[cur[i]]] = leaf;
    // the leaf's bounding box, lanes and reduction as leaf_box_kernel (bit-identical)
    for (int j = 0; j < d; ++j) {
      T mn = real_traits<T>::big(), mx = -real_traits<T>::big();
      for (int i = a + lane; i < b; i += 32) {
        const T v = spts[(size_t)cur[i] * ds + j];
        mn = v < mn ? v : mn;
        mx = v > mx ? v : mx;
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const T oa = __shfl_xor_sync(0xffffffffu, mn, o), ob = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = oa < mn ? oa : mn;
        mx = ob > mx ? ob : mx;
      }
      if (lane == 0) {
        leaf_box[((long long)leaf * 2) * d + j] = mn;
        leaf_box[((long long)leaf * 2 + 1) * d + j] = mx;
      }
    }
  }
  if (sizeof(T) == 4 && (d & 3) == 0) {
    float4* dst = reinterpret_cast<float4*>(pts_out + (long long)lo * d);
    const int nq = cnt * d / 4, qpr = d / 4;
    for (int e = threadIdx.x; e < nq; e += kSubThreads) {
      const int r = e / qpr, c = (e - r * qpr) * 4;
      const float* sp = reinterpret_cast<const float*>(spts) + (size_t)cur[r] * ds + c;
      dst[e] = make_float4(sp[0], sp[1], sp[2], sp[3]);
    }
  } else {
    for (long long e = threadIdx.x; e < (long long)cnt * d; e += blockDim.x) {
      const int r = (int)(e / d), c = (int)(e - (long long)r * d);
      pts_out[(long long)(lo + r) * d + c] = spts[(size_t)cur[r] * ds + c];
    }
  }
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) perm_out[lo + i] = sperm[cur[i]];
}

template <typename T>
static size_t subtree_smem(int smax, int d) {
  using K = typename key_of<T>::type;
  return (size_t)smax * sub_stride(d) * sizeof(T) + 2 * (size_t)kSubWarps * d * sizeof(T) +
         (size_t)(smax + kSubWarps) * sizeof(K) + (size_t)(smax + 4 * kSubWarps) * sizeof(int) +
         kSubWarps * 256 * sizeof(unsigned) + 2 * (size_t)smax * sizeof(uint16_t);
}

template <typename T>
static int subtree_capacity(int d) {
  const size_t budget = 112 * 1024;  // two finisher CTAs per SM
  int smax = 4096;
  while (smax > 1 && subtree_smem<T>(smax, d) > budget) smax >>= 1;
  return smax;
}

template <typename T>
static int build_impl(annf_handle* h, const T* points, int n, int d, int depth, int splitting, cudaStream_t st) {
  using K = typename key_of<T>::type;
  const int L = 1 << depth;
  ANNF_ENSURE(h->pts, (size_t)n * d * sizeof(T));
  ANNF_ENSURE(h->pts_tmp, (size_t)n * d * sizeof(T));
  ANNF_ENSURE(h->perm, (size_t)n * sizeof(int));
  ANNF_ENSURE(h->perm_tmp, (size_t)n * sizeof(int));
  ANNF_ENSURE(h->node_axis, (size_t)std::max(L - 1, 1) * sizeof(int));
  ANNF_ENSURE(h->node_split, (size_t)std::max(L - 1, 1) * sizeof(T));
  ANNF_ENSURE(h->leaf_begin, (size_t)(L + 1) * sizeof(int));
  ANNF_ENSURE(h->point_leaf, (size_t)n * sizeof(int));
  ANNF_ENSURE(h->keys, (size_t)n * sizeof(K));
  ANNF_ENSURE(h->eqpos, (size_t)n * sizeof(int));

  T* cur_pts = h->pts.as<T>();
  T* alt_pts = h->pts_tmp.as<T>();
  int* cur_perm = h->perm.as<int>();
  int* alt_perm = h->perm_tmp.as<int>();
  prof_mark(h, "build:begin", st);
  iota_kernel<<<std::min(ceil_div(n, 256), 4096), 256, 0, st>>>(cur_perm, n);
  ANNF_CHECK_LAUNCH();

  const int smax = subtree_capacity<T>(d);
  const size_t sub_smem = subtree_smem<T>(smax, d);
  // global levels run while a segment exceeds the finisher's capacity; their bounding boxes live
  // in two halves of bmin / bmax (this level's, the children's)
  int tg = 0;
  while (tg < depth && ((long long)n + (1LL << tg) - 1) / (1LL << tg) > smax) ++tg;
  const long long cap = 1LL << tg;  // segments of the deepest level that needs a box
  if (tg > 0) {
    ANNF_ENSURE(h->bmin, (size_t)2 * cap * d * sizeof(K));
    ANNF_ENSURE(h->bmax, (size_t)2 * cap * d * sizeof(K));
    ANNF_ENSURE(h->hist, (size_t)(cap / 2) * kSelBins * sizeof(unsigned));
    ANNF_CUDA_TRY(cudaMemsetAsync(h->hist.p, 0, (size_t)(cap / 2) * kSelBins * sizeof(unsigned), st));  // picks re-zero it
  }
  ANNF_ENSURE(h->leaf_box, (size_t)2 * L * d * sizeof(T));
  // the points, column-major from here to the finisher (or to the leaves); level 0's box on the way
  const int crows = col_tile_rows<T>(d);
  const size_t csmem = (size_t)crows * (d | 1) * sizeof(T);
  const int cblocks = std::min(ceil_div(n, crows), 16 * num_sms());
  if (depth == 0) {
    ANNF_CUDA_TRY(cudaMemcpyAsync(cur_pts, points, (size_t)n * d * sizeof(T), cudaMemcpyDeviceToDevice, st));
  } else {
    K* gmin0 = h->bmin.as<K>();
    K* gmax0 = h->bmax.as<K>();
    if (tg == 0) {  // the finisher takes the root: no level needs a box, but the kernel wants two
      ANNF_ENSURE(h->bmin, (size_t)2 * d * sizeof(K));
      ANNF_ENSURE(h->bmax, (size_t)2 * d * sizeof(K));
      gmin0 = h->bmin.as<K>();
      gmax0 = h->bmax.as<K>();
    }
    fill_keys_kernel<K><<<1, 256, 0, st>>>(gmin0, d, ~(K)0);
    ANNF_CHECK_LAUNCH();
    fill_keys_kernel<K><<<1, 256, 0, st>>>(gmax0, d, (K)0);
    ANNF_CHECK_LAUNCH();
    to_columns_kernel<T><<<cblocks, kThreads, csmem, st>>>(n, d, points, cur_pts, gmin0, gmax0);
    ANNF_CHECK_LAUNCH();
  }
  bool finished = false;
  for (int t = 0; t < depth; ++t) {
    const int S = 1 << t;
    const int maxcnt = (int)(((long long)n + S - 1) / S);
    if (maxcnt <= smax) {
      ANNF_CUDA_TRY(cudaFuncSetAttribute(subtree_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sub_smem));
      subtree_kernel<T><<<S, kSubThreads, sub_smem, st>>>(
          n, d, depth, t, smax, splitting, cur_pts, cur_perm, alt_pts, alt_perm, h->node_axis.as<int>(),
          h->node_split.as<T>(), h->leaf_begin.as<int>(), h->point_leaf.as<int>(), h->leaf_box.as<T>(),
          h->status.as<unsigned>());
      ANNF_CHECK_LAUNCH();
      std::swap(cur_pts, alt_pts);
      std::swap(cur_perm, alt_perm);
      finished = true;
      prof_mark(h, "build_subtree", st);
      break;
    }
    const int B = ceil_div(maxcnt, kChunk);
    const long long nblk = (long long)S * B;
    const int HB = ceil_div(B, kHistChunks);  // histogram CTAs per segment
    if (nblk > 0x7fffffffLL) {
      set_error("tree too large for the level kernels");
      return ANNF_ERR_UNSUPPORTED;
    }
    ANNF_ENSURE(h->axis, (size_t)S * sizeof(int));
    ANNF_ENSURE(h->sel_prefix, (size_t)S * sizeof(K));
    ANNF_ENSURE(h->sel_rank, (size_t)S * sizeof(int));
    ANNF_ENSURE(h->sel_nlt, (size_t)S * sizeof(int));
    ANNF_ENSURE(h->sel_neq, (size_t)S * sizeof(int));
    ANNF_ENSURE(h->chunk_state, (size_t)nblk * sizeof(unsigned long long));
    K* gmin = h->bmin.as<K>() + (size_t)(t & 1) * cap * d;
    K* gmax = h->bmax.as<K>() + (size_t)(t & 1) * cap * d;
    // the children's boxes, when the next level is a global one: the scatter computes them (level
    // 0's came with the column-major copy)
    K* cmin = t + 1 < tg ? h->bmin.as<K>() + (size_t)((t + 1) & 1) * cap * d : nullptr;
    K* cmax = t + 1 < tg ? h->bmax.as<K>() + (size_t)((t + 1) & 1) * cap * d : nullptr;
    axis_kernel<T><<<ceil_div(S, 128), 128, 0, st>>>(n, d, t, S, splitting, gmin, gmax, h->axis.as<int>(),
                                                   h->sel_prefix.as<K>(), h->sel_rank.as<int>(),
                                                   h->sel_nlt.as<int>(), cmin, cmax);
    ANNF_CHECK_LAUNCH();
    constexpr int kBits = 8 * sizeof(K);
    // digits from the top: kSelBits wide, the rest of the key in the last pass
    for (int hi_bit = kBits; hi_bit > 0;) {
      const int width = hi_bit >= 2 * kSelBits ? kSelBits : (hi_bit > kSelBits ? hi_bit - hi_bit / 2 : hi_bit);
      const int shift = hi_bit - width;
      hist_kernel<T><<<(unsigned)((long long)S * HB), 256, 0, st>>>(n, d, t, HB, shift, width, hi_bit == kBits, cur_pts,
                                                     h->axis.as<int>(), h->keys.as<K>(), h->sel_prefix.as<K>(),
                                                     h->hist.as<unsigned>());
      ANNF_CHECK_LAUNCH();
      pick_kernel<K><<<S, 256, 0, st>>>(shift, shift == 0, h->hist.as<unsigned>(), h->sel_prefix.as<K>(),
                                        h->sel_rank.as<int>(), h->sel_nlt.as<int>(), h->sel_neq.as<int>());
      ANNF_CHECK_LAUNCH();
      hi_bit -= width;
    }
    ANNF_CUDA_TRY(cudaMemsetAsync(h->chunk_state.p, 0, (size_t)nblk * sizeof(unsigned long long), st));
    scatter_kernel<T><<<(unsigned)nblk, kThreads, 0, st>>>(
        n, d, t, B, h->keys.as<K>(), h->sel_prefix.as<K>(), h->sel_nlt.as<int>(), h->sel_neq.as<int>(),
        h->chunk_state.as<unsigned long long>(), h->status.as<unsigned>(), cur_pts, cur_perm, alt_pts, alt_perm,
        h->eqpos.as<int>(), cmin, cmax);
    ANNF_CHECK_LAUNCH();
    fixup_kernel<T><<<ceil_div((long long)S * 32, 256), 256, 0, st>>>(
        n, d, t, S, h->axis.as<int>(), h->sel_nlt.as<int>(), h->sel_neq.as<int>(), h->eqpos.as<int>(),
        alt_pts, alt_perm, h->node_axis.as<int>(), h->node_split.as<T>());
    ANNF_CHECK_LAUNCH();
    std::swap(cur_pts, alt_pts);
    std::swap(cur_perm, alt_perm);
    prof_mark(h, "build_level", st);
  }
  if (!finished) {
    const int S = L;
    const int maxcnt = (int)(((long long)n + S - 1) / S);
    const int B = ceil_div(maxcnt, kChunk);
    leaves_kernel<<<(unsigned)((long long)S * B), kThreads, 0, st>>>(n, depth, B, cur_perm,
                                                                    h->leaf_begin.as<int>(), h->point_leaf.as<int>());
    ANNF_CHECK_LAUNCH();
    if (depth > 0) {  // the leaves' points back to rows
      to_rows_kernel<T><<<cblocks, kThreads, csmem, st>>>(n, d, cur_pts, alt_pts);
      ANNF_CHECK_LAUNCH();
      std::swap(cur_pts, alt_pts);
    }
  }
  // the final arrays live in h->pts / h->perm
  if (cur_pts != h->pts.as<T>()) std::swap(h->pts, h->pts_tmp);
  if (cur_perm != h->perm.as<int>()) std::swap(h->perm, h->perm_tmp);
  // per-leaf bounding boxes: lower bounds for the exact search (the finisher computed them when
  // it built the leaves)
  if (!finished) {
    leaf_box_kernel<T><<<ceil_div((long long)L * 32, 256), 256, 0, st>>>(L, d, h->pts.as<T>(), h->leaf_begin.as<int>(),
                                                                       h->leaf_box.as<T>());
    ANNF_CHECK_LAUNCH();
  }
  prof_mark(h, "build_leafbox", st);
  const int maxleaf = (int)(((long long)n + L - 1) / L);
  int bits = 1;
  while ((1LL << bits) <= maxleaf) ++bits;
  h->leaf_bits = bits;
  h->max_leaf = maxleaf;
  return ANNF_OK;
}

int build_tree(annf_handle* h, const void* points, int n, int d, int real_type, int depth, int splitting,
               cudaStream_t st) {
  ANNF_REQUIRE(points != nullptr, "annf_build_tree: points is NULL");
  ANNF_REQUIRE(n >= 1 && d >= 1, "annf_build_tree: need n >= 1 and d >= 1");
  ANNF_REQUIRE(d <= 128, "annf_build_tree: d > 128 is not supported");
  ANNF_REQUIRE(depth >= 0 && depth <= 30 && (1LL << depth) <= n,
               "annf_build_tree: depth must satisfy 0 <= depth and 2^depth <= n");
  ANNF_REQUIRE(real_type == ANNF_REAL_F32 || real_type == ANNF_REAL_F64, "annf_build_tree: bad real_type");
  ANNF_REQUIRE(splitting == ANNF_SPLIT_CYCLIC || splitting == ANNF_SPLIT_LONGEST, "annf_build_tree: bad splitting_type");
  h->built = 0;
  int rc = (real_type == ANNF_REAL_F32) ? build_impl<float>(h, static_cast<const float*>(points), n, d, depth, splitting, st)
                                        : build_impl<double>(h, static_cast<const double*>(points), n, d, depth, splitting, st);
  if (rc != ANNF_OK) return rc;
  h->n = n;
  h->d = d;
  h->depth = depth;
  h->real_type = real_type;
  if (depth + h->leaf_bits > 32) {
    set_error("annf_build_tree: depth + log2(leaf size) exceeds 32 bits of tie-break");
    return ANNF_ERR_UNSUPPORTED;
  }
  h->built = 1;
  return ANNF_OK;
}

}  // namespace annf
