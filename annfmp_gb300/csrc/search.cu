// search.cu -- queries against the device k-d tree (sm_103a): exact kNN, the row-propagation
// NNF and the raw-patch re-rank.
//
// Candidate order. The reference keeps a sorted K-list and inserts candidates one by one with a
// strict '<' (annfmp/openmp/kdtree/src/kdtree.c:502-532), so the final list is the first K of the
// candidates sorted stably by distance in visiting order; a point met twice is listed twice. Here
// every candidate carries a 64-bit key (distance bits, tie) whose tie field encodes the visiting
// order, so any parallel top-K over keys returns exactly the reference list:
//   * row propagation (kdtree.c:305-352): tie = slot << leaf_bits | offset in leaf, slot 1 = the
//     natural leaf, slots 2.. = the propagated leaves in neighbour order;
//   * exact search (kdtree.c:129-268): the backtracking search visits leaves depth first, near
//     child first, and prunes only subtrees whose every point is strictly farther than the current
//     K-th distance, so its result equals the brute-force top-K with tie = dfs_rank(leaf) <<
//     leaf_bits | offset, dfs_rank being the leaf's position in that query's visiting order
//     (bit t = the leaf's branch at level t XOR the query's near side there);
//   * the K initial entries (K-th distance = max real, position 0; kdtree.c:141-144) carry tie 0.
// Distances use the reference's order of operations with explicit round-to-nearest intrinsics so
// that nothing is contracted into an FMA (helper.c:164-179).
#include <algorithm>

#include "common.cuh"
#include "handle.cuh"

namespace annf {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------------------------
// per-lane sorted list of KM (key, position) pairs and the warp-wide top-K merge
// ---------------------------------------------------------------------------------------------
template <typename T> struct KeyOps;
template <> struct KeyOps<float> {
  using K = unsigned long long;
  __device__ static K make(float d, uint32_t tie) { return ((K)__float_as_uint(d) << 32) | tie; }
  __device__ static K init() { return ((K)0x7f7fffffu << 32); }
  __device__ static K inf() { return ~0ull; }
  __device__ static float dist(K k) { return __uint_as_float((uint32_t)(k >> 32)); }
  __device__ static bool lt(K a, K b) { return a < b; }
  __device__ static bool eq(K a, K b) { return a == b; }
  __device__ static K shfl_xor(K v, int m) { return __shfl_xor_sync(kFull, v, m); }
};
template <> struct KeyOps<double> {
  using K = dkey;
  __device__ static K make(double d, uint32_t tie) { return dkey{(unsigned long long)__double_as_longlong(d), tie}; }
  __device__ static K init() { return dkey{0x7fefffffffffffffull, 0u}; }
  __device__ static K inf() { return dkey{~0ull, ~0u}; }
  __device__ static double dist(K k) { return __longlong_as_double((long long)k.d); }
  __device__ static bool lt(K a, K b) { return a.d < b.d || (a.d == b.d && a.tie < b.tie); }
  __device__ static bool eq(K a, K b) { return a.d == b.d && a.tie == b.tie; }
  __device__ static K shfl_xor(K v, int m) { return dkey{__shfl_xor_sync(kFull, v.d, m), __shfl_xor_sync(kFull, v.tie, m)}; }
};

template <typename T, int KM>
struct LaneList {
  using Ops = KeyOps<T>;
  using K = typename Ops::K;
  K key[KM];
  int pos[KM];
  __device__ void init_entries() {
#pragma unroll
    for (int j = 0; j < KM; ++j) {
      key[j] = Ops::init();
      pos[j] = 0;
    }
  }
  __device__ void init_inf() {
#pragma unroll
    for (int j = 0; j < KM; ++j) {
      key[j] = Ops::inf();
      pos[j] = 0;
    }
  }
  __device__ __forceinline__ void offer(K k, int p) {
    if (!Ops::lt(k, key[KM - 1])) return;
#pragma unroll
    for (int j = KM - 1; j >= 0; --j) {
      if (j > 0 && Ops::lt(k, key[j - 1])) {
        key[j] = key[j - 1];
        pos[j] = pos[j - 1];
      } else if (Ops::lt(k, key[j])) {
        key[j] = k;
        pos[j] = p;
      }
    }
  }
  __device__ __forceinline__ void pop() {
#pragma unroll
    for (int j = 0; j < KM - 1; ++j) {
      key[j] = key[j + 1];
      pos[j] = pos[j + 1];
    }
    key[KM - 1] = Ops::inf();
  }
};

// lanes r < K receive the r-th smallest (key, pos) over all lanes' lists
template <typename T, int KM>
__device__ __forceinline__ void warp_topk(LaneList<T, KM>& L, int K, int lane, typename KeyOps<T>::K& okey, int& opos) {
  using Ops = KeyOps<T>;
  using K_ = typename Ops::K;
  for (int r = 0; r < K; ++r) {
    K_ head = L.key[0];
    K_ m = head;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      K_ x = Ops::shfl_xor(m, o);
      m = Ops::lt(x, m) ? x : m;
    }
    const unsigned who = __ballot_sync(kFull, Ops::eq(head, m));
    const int src = __ffs(who) - 1;
    const int p = __shfl_sync(kFull, L.pos[0], src);
    if (lane == r) {
      okey = m;
      opos = p;
    }
    if (lane == src) L.pop();
  }
}

// ---------------------------------------------------------------------------------------------
// distances
// ---------------------------------------------------------------------------------------------
template <typename T, int D>
struct QReg {
  T v[D];
  __device__ __forceinline__ void load(const T* __restrict__ q, int) {
#pragma unroll
    for (int j = 0; j < D; ++j) v[j] = q[j];
  }
  __device__ __forceinline__ T dist(const T* __restrict__ p, int) const {
    using R = real_traits<T>;
    T acc = 0;
    if constexpr (sizeof(T) == 4 && D % 4 == 0) {
      const float4* p4 = reinterpret_cast<const float4*>(p);
#pragma unroll
      for (int j = 0; j < D / 4; ++j) {
        const float4 w = __ldg(p4 + j);
        float t;
        t = R::sub(w.x, v[4 * j + 0]); acc = R::add(acc, R::mul(t, t));
        t = R::sub(w.y, v[4 * j + 1]); acc = R::add(acc, R::mul(t, t));
        t = R::sub(w.z, v[4 * j + 2]); acc = R::add(acc, R::mul(t, t));
        t = R::sub(w.w, v[4 * j + 3]); acc = R::add(acc, R::mul(t, t));
      }
    } else {
#pragma unroll
      for (int j = 0; j < D; ++j) {
        T t = R::sub(__ldg(p + j), v[j]);
        acc = R::add(acc, R::mul(t, t));
      }
    }
    return acc;
  }
  __device__ __forceinline__ T coord(int j) const {  // runtime index: rarely used
    T r = v[0];
#pragma unroll
    for (int i = 1; i < D; ++i) r = (i == j) ? v[i] : r;
    return r;
  }
};

// runtime dimension: the query sits in a per-warp shared-memory slot
constexpr int kMaxDynD = 128;
template <typename T>
struct QReg<T, 0> {
  const T* v;
  int d;
  __device__ __forceinline__ void load(const T* __restrict__, int) {}
  __device__ __forceinline__ T dist(const T* __restrict__ p, int) const {
    using R = real_traits<T>;
    T acc = 0;
    for (int j = 0; j < d; ++j) {
      T t = R::sub(__ldg(p + j), v[j]);
      acc = R::add(acc, R::mul(t, t));
    }
    return acc;
  }
  __device__ __forceinline__ T coord(int j) const { return v[j]; }
};

template <typename T>
__device__ __forceinline__ int natural_leaf(const TreeView<T>& tv, const T* __restrict__ q) {
  int node = 0;
  for (int l = 0; l < tv.depth; ++l) {
    const int ax = __ldg(tv.node_axis + node);
    const T s = __ldg(tv.node_split + node);
    node = (q[ax] >= s) ? 2 * node + 2 : 2 * node + 1;  // q - split >= 0 (kdtree.c:204)
  }
  return node - ((1 << tv.depth) - 1);
}

// ---------------------------------------------------------------------------------------------
// natural leaf of every query + its top-K (slot 1)
// ---------------------------------------------------------------------------------------------
template <typename T, int D, int KM>
__global__ void __launch_bounds__(256) natural_knn_kernel(TreeView<T> tv, const T* __restrict__ Q, long long q0,
                                                          long long nq, int K, typename KeyOps<T>::K* __restrict__ out_key,
                                                          int* __restrict__ out_pos) {
  __shared__ T sq[8][D > 0 ? 1 : kMaxDynD];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const int d = tv.d;
  for (long long qi = q0 + gw; qi < q0 + nq; qi += nw) {
    const T* q = Q + qi * d;
    QReg<T, D> qr;
    if constexpr (D == 0) {
      for (int j = lane; j < d; j += 32) sq[wib][j] = q[j];
      __syncwarp();
      qr.v = sq[wib];
      qr.d = d;
    } else {
      qr.load(q, d);
    }
    const int leaf = natural_leaf(tv, D == 0 ? sq[wib] : q);
    const int beg = __ldg(tv.leaf_begin + leaf), end = __ldg(tv.leaf_begin + leaf + 1);
    LaneList<T, KM> L;
    L.init_entries();
    const uint32_t slot = 1u << tv.leaf_bits;
    for (int p = beg + lane; p < end; p += 32) {
      const T dd = qr.dist(tv.pts + (long long)p * d, d);
      L.offer(KeyOps<T>::make(dd, slot | (uint32_t)(p - beg)), p);
    }
    typename KeyOps<T>::K k;
    int pos;
    warp_topk<T, KM>(L, K, lane, k, pos);
    if (lane < K) {
      if (out_key) out_key[qi * K + lane] = k;
      out_pos[qi * K + lane] = pos;
    }
    if constexpr (D == 0) __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------------
// exact kNN by brute force in the reference's visiting order: thread per query, leaves staged in
// shared memory, leaf ranges split over blockIdx.y; partial lists merged afterwards
// ---------------------------------------------------------------------------------------------
constexpr int kExactThreads = 128;

template <typename T, int D, int KM>
__global__ void __launch_bounds__(kExactThreads) exact_part_kernel(
    TreeView<T> tv, const T* __restrict__ Q, int nq, int K, int leaves_per_split, int stage_pts,
    typename KeyOps<T>::K* __restrict__ part_key, int* __restrict__ part_pos) {
  using Ops = KeyOps<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int d = tv.d;
  const int dstride = d + 1;  // padded row for runtime-axis reads without bank conflicts
  T* sq = reinterpret_cast<T*>(smem_raw);                       // [kExactThreads][d+1]
  T* spts = sq + kExactThreads * dstride;                       // [stage_pts][d]
  spts = reinterpret_cast<T*>((reinterpret_cast<uintptr_t>(spts) + 15) & ~uintptr_t(15));
  const int qi = blockIdx.x * kExactThreads + threadIdx.x;
  const bool active = qi < nq;
  for (int j = 0; j < d; ++j) sq[threadIdx.x * dstride + j] = active ? Q[(long long)qi * d + j] : T(0);
  QReg<T, D> qr;
  if constexpr (D == 0) {
    qr.v = sq + threadIdx.x * dstride;
    qr.d = d;
  } else {
#pragma unroll
    for (int j = 0; j < D; ++j) qr.v[j] = sq[threadIdx.x * dstride + j];
  }
  LaneList<T, KM> L;
  L.init_entries();
  const int nleaves = 1 << tv.depth;
  const int l0 = blockIdx.y * leaves_per_split, l1 = min(nleaves, l0 + leaves_per_split);
  for (int lf = l0; lf < l1; ++lf) {
    const int beg = __ldg(tv.leaf_begin + lf), end = __ldg(tv.leaf_begin + lf + 1);
    const int cnt = end - beg;
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * d; e += blockDim.x) spts[e] = tv.pts[(long long)beg * d + e];
    __syncthreads();
    // dfs rank of this leaf for this query
    uint32_t rank = 0;
    for (int t = 0; t < tv.depth; ++t) {
      const int node = (1 << t) - 1 + (lf >> (tv.depth - t));
      const int dir = (lf >> (tv.depth - 1 - t)) & 1;
      const int ax = __ldg(tv.node_axis + node);
      const int side = sq[threadIdx.x * dstride + ax] >= __ldg(tv.node_split + node) ? 1 : 0;
      rank = (rank << 1) | (uint32_t)(dir ^ side);
    }
    const uint32_t hi = rank << tv.leaf_bits;
    if (active) {
      for (int p = 0; p < cnt; ++p) {
        T dd;
        if constexpr (D > 0) {
          using R = real_traits<T>;
          const T* pp = spts + p * D;
          T acc = 0;
#pragma unroll
          for (int j = 0; j < D; ++j) {
            T t = R::sub(pp[j], qr.v[j]);
            acc = R::add(acc, R::mul(t, t));
          }
          dd = acc;
        } else {
          using R = real_traits<T>;
          const T* pp = spts + p * d;
          T acc = 0;
          for (int j = 0; j < d; ++j) {
            T t = R::sub(pp[j], qr.v[j]);
            acc = R::add(acc, R::mul(t, t));
          }
          dd = acc;
        }
        L.offer(Ops::make(dd, hi | (uint32_t)p), beg + p);
      }
    }
  }
  if (active) {
    const long long base = ((long long)blockIdx.y * nq + qi) * K;
    for (int j = 0; j < K && j < KM; ++j) {
      part_key[base + j] = L.key[j];
      part_pos[base + j] = L.pos[j];
    }
  }
}

// merge the per-split lists: warp per query. mode 0: tree positions to out_pos; mode 1: square
// rooted distances + original indices (kneighbors)
template <typename T, int KM>
__global__ void exact_merge_kernel(TreeView<T> tv, int nq, int K, int nsplit,
                                   const typename KeyOps<T>::K* __restrict__ part_key,
                                   const int* __restrict__ part_pos, int mode, int* __restrict__ out_pos,
                                   T* __restrict__ out_dist, int* __restrict__ out_idx) {
  const int lane = threadIdx.x & 31;
  const long long qi = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  if (qi >= nq) return;
  LaneList<T, KM> L;
  L.init_entries();
  for (int e = lane; e < nsplit * K; e += 32) {
    const int sp = e / K, j = e - sp * K;
    const long long src = ((long long)sp * nq + qi) * K + j;
    L.offer(part_key[src], part_pos[src]);
  }
  typename KeyOps<T>::K k;
  int pos;
  warp_topk<T, KM>(L, K, lane, k, pos);
  if (lane < K) {
    if (mode == 0) {
      out_pos[qi * K + lane] = pos;
    } else {
      out_dist[qi * K + lane] = real_traits<T>::sqrt_(KeyOps<T>::dist(k));
      out_idx[qi * K + lane] = __ldg(tv.perm + pos);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// row propagation
// ---------------------------------------------------------------------------------------------
// for every tree position: the leaf span of its point's "one row below" index (base.c:260-277)
template <typename T>
__global__ void next_range_kernel(TreeView<T> tv, int n_cols, long long nA, int2* __restrict__ out,
                                  unsigned* status) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < tv.n; p += (long long)gridDim.x * blockDim.x) {
    long long b = __ldg(tv.perm + p);
    if (b + n_cols < nA) b += n_cols;
    if (b >= tv.n) {  // index outside B (A larger than B): keep the point's own row
      b = __ldg(tv.perm + p);
      atomicOr(status, DEV_BAD_INDEX);
    }
    const int lf = __ldg(tv.point_leaf + b);
    out[p] = make_int2(__ldg(tv.leaf_begin + lf), __ldg(tv.leaf_begin + lf + 1));
  }
}

// one warp per column walks the rows downwards; lane j < K carries entry j of the row above
template <typename T, int D, int KM>
__global__ void __launch_bounds__(128) chain_kernel(TreeView<T> tv, const T* __restrict__ Q, int n_rows, int n_cols,
                                                    int K, const typename KeyOps<T>::K* __restrict__ nat_key,
                                                    const int* __restrict__ nat_pos, const int2* __restrict__ next_range,
                                                    int* __restrict__ lists) {
  using Ops = KeyOps<T>;
  __shared__ T sq[4][D > 0 ? 1 : kMaxDynD];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int x = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (x >= n_cols) return;
  const int d = tv.d;
  int my_pos = lane < K ? lists[(long long)x * K + lane] : 0;
  for (int y = 1; y < n_rows; ++y) {
    const long long qi = (long long)y * n_cols + x;
    const T* q = Q + qi * d;
    QReg<T, D> qr;
    if constexpr (D == 0) {
      __syncwarp();
      for (int j = lane; j < d; j += 32) sq[wib][j] = q[j];
      __syncwarp();
      qr.v = sq[wib];
      qr.d = d;
    } else {
      qr.load(q, d);
    }
    typename Ops::K nk = Ops::inf();
    int np = 0;
    if (lane < K) {
      nk = nat_key[qi * K + lane];
      np = nat_pos[qi * K + lane];
    }
    const int2 my_rng = lane < K ? __ldg(next_range + my_pos) : make_int2(0, 0);
    LaneList<T, KM> L;
    L.init_entries();
    L.offer(nk, np);
    for (int j = 0; j < K; ++j) {
      const int beg = __shfl_sync(kFull, my_rng.x, j), end = __shfl_sync(kFull, my_rng.y, j);
      const uint32_t slot = (uint32_t)(j + 2) << tv.leaf_bits;
      for (int p = beg + lane; p < end; p += 32) {
        const T dd = qr.dist(tv.pts + (long long)p * d, d);
        L.offer(Ops::make(dd, slot | (uint32_t)(p - beg)), p);
      }
    }
    typename Ops::K k;
    int pos = 0;
    warp_topk<T, KM>(L, K, lane, k, pos);
    if (lane < K) lists[qi * K + lane] = pos;
    my_pos = pos;
  }
}

// ---------------------------------------------------------------------------------------------
// tree positions -> original indices, and the raw-patch re-rank (base.c:309-353, 362-374)
// ---------------------------------------------------------------------------------------------


template <typename T>
__device__ __forceinline__ T patch_dist(const PatchSrc& A, long long ia, const PatchSrc& B, long long ib) {
  const int rowlen = A.psize * A.c;
  const int P = rowlen * A.psize;
  if (sizeof(T) == 8 || (long long)P * 65025 < (1LL << 24)) {
    long long acc = 0;  // every partial sum is exact in the reference's accumulator
    for (int r = 0; r < A.psize; ++r) {
      const uint8_t* a = A.row(ia, r);
      const uint8_t* b = B.row(ib, r);
      int s = 0;
      for (int e = 0; e < rowlen; ++e) {
        const int t = (int)__ldg(a + e) - (int)__ldg(b + e);
        s += t * t;
      }
      acc += s;
    }
    return real_traits<T>::sqrt_((T)acc);
  } else {  // large patches: replay the reference's rounding of the running sum
    using R = real_traits<T>;
    T acc = 0;
    for (int r = 0; r < A.psize; ++r) {
      const uint8_t* a = A.row(ia, r);
      const uint8_t* b = B.row(ib, r);
      for (int e = 0; e < rowlen; ++e) {
        const T t = (T)((int)__ldg(a + e) - (int)__ldg(b + e));
        acc = R::add(acc, R::mul(t, t));
      }
    }
    return R::sqrt_(acc);
  }
}

template <typename T>
__global__ void select_kernel(TreeView<T> tv, long long nA, int K, const int* __restrict__ lists, int select_best,
                              PatchSrc A, PatchSrc B, int* __restrict__ final_idx, float* __restrict__ dist_out,
                              int* __restrict__ knn_out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nA; i += (long long)gridDim.x * blockDim.x) {
    int best = -1;
    T bestd = real_traits<T>::big();
    for (int j = 0; j < K; ++j) {
      const int o = __ldg(tv.perm + __ldg(lists + i * K + j));
      if (knn_out) knn_out[i * K + j] = o;
      if (select_best) {
        const T dd = patch_dist<T>(A, i, B, o);
        if (dd < bestd) {
          bestd = dd;
          best = o;
        }
      } else if (j == 0) {
        best = o;
      }
    }
    final_idx[i] = best;
    if (dist_out) dist_out[i] = select_best ? (float)bestd : __int_as_float(0x7fc00000);
  }
}

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
template <typename T>
static TreeView<T> view_of(const annf_handle* h) {
  TreeView<T> tv;
  tv.n = h->n;
  tv.d = h->d;
  tv.depth = h->depth;
  tv.leaf_bits = h->leaf_bits;
  tv.pts = h->pts.as<T>();
  tv.perm = h->perm.as<int>();
  tv.node_axis = h->node_axis.as<int>();
  tv.node_split = h->node_split.as<T>();
  tv.leaf_begin = h->leaf_begin.as<int>();
  tv.point_leaf = h->point_leaf.as<int>();
  return tv;
}

static int pick_km(int K) { return K <= 1 ? 1 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32; }

static int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  return sms;
}

// dispatch on (D, KM) for float and KM for double
#define ANNF_DISPATCH_KM(KMV, ...)                         \
  switch (KMV) {                                           \
    case 1: { constexpr int KM = 1; __VA_ARGS__; } break;  \
    case 4: { constexpr int KM = 4; __VA_ARGS__; } break;  \
    case 8: { constexpr int KM = 8; __VA_ARGS__; } break;  \
    case 16: { constexpr int KM = 16; __VA_ARGS__; } break; \
    default: { constexpr int KM = 32; __VA_ARGS__; } break; \
  }

template <typename T, int D, int KM>
static int exact_knn_typed(annf_handle* h, const T* Q, int nq, int K, int mode, int* out_pos, T* out_dist,
                           int* out_idx, cudaStream_t st) {
  using Kt = typename KeyOps<T>::K;
  TreeView<T> tv = view_of<T>(h);
  const int nleaves = 1 << h->depth;
  const int tiles = ceil_div(nq, kExactThreads);
  int want = std::max(1, (8 * num_sms()) / tiles);
  int lps = std::max(1, ceil_div(nleaves, want));
  int nsplit = ceil_div(nleaves, lps);
  ANNF_ENSURE(h->part_keys, (size_t)nsplit * nq * K * sizeof(Kt));
  ANNF_ENSURE(h->part_pos, (size_t)nsplit * nq * K * sizeof(int));
  const size_t smem = (size_t)kExactThreads * (h->d + 1) * sizeof(T) + 16 + (size_t)h->max_leaf * h->d * sizeof(T);
  if (smem > 200 * 1024) {
    set_error("exact search: leaf too large to stage in shared memory");
    return ANNF_ERR_UNSUPPORTED;
  }
  ANNF_CUDA_TRY(cudaFuncSetAttribute(exact_part_kernel<T, D, KM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid(tiles, nsplit);
  exact_part_kernel<T, D, KM><<<grid, kExactThreads, smem, st>>>(tv, Q, nq, K, lps, h->max_leaf,
                                                                  h->part_keys.as<Kt>(), h->part_pos.as<int>());
  ANNF_CHECK_LAUNCH();
  exact_merge_kernel<T, KM><<<ceil_div((long long)nq * 32, 256), 256, 0, st>>>(
      tv, nq, K, nsplit, h->part_keys.as<Kt>(), h->part_pos.as<int>(), mode, out_pos, out_dist, out_idx);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

template <typename T>
static int exact_knn(annf_handle* h, const T* Q, int nq, int K, int mode, int* out_pos, T* out_dist, int* out_idx,
                     cudaStream_t st) {
  const int km = pick_km(K);
  if constexpr (sizeof(T) == 4) {
    switch (h->d) {
      case 8: ANNF_DISPATCH_KM(km, return exact_knn_typed<T, 8, KM>(h, Q, nq, K, mode, out_pos, out_dist, out_idx, st));
      case 12: ANNF_DISPATCH_KM(km, return exact_knn_typed<T, 12, KM>(h, Q, nq, K, mode, out_pos, out_dist, out_idx, st));
      case 16: ANNF_DISPATCH_KM(km, return exact_knn_typed<T, 16, KM>(h, Q, nq, K, mode, out_pos, out_dist, out_idx, st));
      default: break;
    }
  }
  ANNF_DISPATCH_KM(km, return exact_knn_typed<T, 0, KM>(h, Q, nq, K, mode, out_pos, out_dist, out_idx, st));
  return ANNF_OK;
}

template <typename T, int D, int KM>
static int rows_typed(annf_handle* h, const T* ared, int n_rows, int n_cols, int K, int propagate, cudaStream_t st) {
  using Kt = typename KeyOps<T>::K;
  TreeView<T> tv = view_of<T>(h);
  const long long nA = (long long)n_rows * n_cols;
  int* lists = h->lists.as<int>();
  if (n_rows > 1) {
    const long long nq = nA - n_cols;
    const int blocks = (int)std::min<long long>(ceil_div(nq * 32, 256), 64LL * num_sms());
    if (propagate) {
      ANNF_ENSURE(h->nat_keys, (size_t)nA * K * sizeof(Kt));
      ANNF_ENSURE(h->nat_pos, (size_t)nA * K * sizeof(int));
      natural_knn_kernel<T, D, KM><<<blocks, 256, 0, st>>>(tv, ared, n_cols, nq, K, h->nat_keys.as<Kt>(), h->nat_pos.as<int>());
      ANNF_CHECK_LAUNCH();
      prof_mark(h, "natural_knn", st);
      ANNF_ENSURE(h->next_range, (size_t)h->n * sizeof(int2));
      next_range_kernel<T><<<std::min(ceil_div(h->n, 256), 16 * num_sms()), 256, 0, st>>>(
          tv, n_cols, nA, h->next_range.as<int2>(), h->status.as<unsigned>());
      ANNF_CHECK_LAUNCH();
      prof_mark(h, "next_range", st);
      chain_kernel<T, D, KM><<<ceil_div((long long)n_cols * 32, 128), 128, 0, st>>>(
          tv, ared, n_rows, n_cols, K, h->nat_keys.as<Kt>(), h->nat_pos.as<int>(), h->next_range.as<int2>(), lists);
      ANNF_CHECK_LAUNCH();
      prof_mark(h, "chain", st);
    } else {
      natural_knn_kernel<T, D, KM><<<blocks, 256, 0, st>>>(tv, ared, n_cols, nq, K, nullptr, lists);
      ANNF_CHECK_LAUNCH();
      prof_mark(h, "natural_knn", st);
    }
  }
  return ANNF_OK;
}

template <typename T>
static int rows_dispatch(annf_handle* h, const T* ared, int n_rows, int n_cols, int K, int propagate, cudaStream_t st) {
  const int km = pick_km(K);
  if constexpr (sizeof(T) == 4) {
    switch (h->d) {
      case 8: ANNF_DISPATCH_KM(km, return rows_typed<T, 8, KM>(h, ared, n_rows, n_cols, K, propagate, st));
      case 12: ANNF_DISPATCH_KM(km, return rows_typed<T, 12, KM>(h, ared, n_rows, n_cols, K, propagate, st));
      case 16: ANNF_DISPATCH_KM(km, return rows_typed<T, 16, KM>(h, ared, n_rows, n_cols, K, propagate, st));
      default: break;
    }
  }
  ANNF_DISPATCH_KM(km, return rows_typed<T, 0, KM>(h, ared, n_rows, n_cols, K, propagate, st));
  return ANNF_OK;
}

template <typename T>
static int process_rows_impl(annf_handle* h, int* final_idx, PatchSrc A, PatchSrc B, const T* ared, int n_rows,
                             int n_cols, int K, int propagate, int select_best, int* knn_out, float* dist_out,
                             cudaStream_t st) {
  const long long nA = (long long)n_rows * n_cols;
  ANNF_ENSURE(h->lists, (size_t)nA * K * sizeof(int));
  prof_mark(h, "rows:begin", st);
  int rc = exact_knn<T>(h, ared, n_cols, K, 0, h->lists.as<int>(), nullptr, nullptr, st);
  if (rc != ANNF_OK) return rc;
  prof_mark(h, "first_row", st);
  rc = rows_dispatch<T>(h, ared, n_rows, n_cols, K, propagate, st);
  if (rc != ANNF_OK) return rc;
  TreeView<T> tv = view_of<T>(h);
  select_kernel<T><<<(int)std::min<long long>(ceil_div(nA, 256), 32LL * num_sms()), 256, 0, st>>>(
      tv, nA, K, h->lists.as<int>(), select_best, A, B, final_idx, dist_out, knn_out);
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "select_best", st);
  return ANNF_OK;
}

int process_rows_generic(annf_handle* h, int* final_idx, const PatchSrc& A, const PatchSrc& B, const void* ared,
                         int n_rows, int n_cols, int K, int propagate, int select_best, int* knn_out,
                         float* dist_out, cudaStream_t st) {
  if (h->real_type == ANNF_REAL_F32)
    return process_rows_impl<float>(h, final_idx, A, B, static_cast<const float*>(ared), n_rows, n_cols, K, propagate,
                                    select_best, knn_out, dist_out, st);
  return process_rows_impl<double>(h, final_idx, A, B, static_cast<const double*>(ared), n_rows, n_cols, K, propagate,
                                   select_best, knn_out, dist_out, st);
}

int kneighbors_generic(annf_handle* h, const void* Q, int nq, int K, void* dist, int* idx, cudaStream_t st) {
  if (h->real_type == ANNF_REAL_F32)
    return exact_knn<float>(h, static_cast<const float*>(Q), nq, K, 1, nullptr, static_cast<float*>(dist), idx, st);
  return exact_knn<double>(h, static_cast<const double*>(Q), nq, K, 1, nullptr, static_cast<double*>(dist), idx, st);
}

}  // namespace annf
