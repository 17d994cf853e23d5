// search.cu -- queries against the device k-d tree (sm_103a): exact kNN, the row-propagation
// NNF and the raw-patch re-rank.
//
// Candidate order. The reference keeps a sorted K-list and inserts candidates one by one with a
// strict '<' (annfmp/openmp/kdtree/src/kdtree.c:502-532), so the final list is the first K of the
// candidates sorted stably by distance in visiting order; a point met twice is listed twice. Here
// every candidate carries a key (distance bits, tie) whose tie field encodes the visiting order, so
// a top-K over keys, computed in any order, returns exactly the reference list:
//   * row propagation (kdtree.c:305-352): tie = slot << leaf_bits | offset in leaf, slot 1 = the
//     natural leaf, slots 2.. = the propagated leaves in neighbour order;
//   * exact search (kdtree.c:129-268): tie = dfs_rank(leaf) << leaf_bits | offset, dfs_rank being
//     the leaf's position in that query's depth-first, near-child-first visiting order;
//   * the K initial entries (K-th distance = max real, position 0; kdtree.c:141-144) carry tie 0.
// Distances use the reference's order of operations with explicit round-to-nearest intrinsics so
// that nothing is contracted into an FMA (helper.c:164-179).
//
// Lists. A warp owns one query at a time and keeps its K-list distributed over lanes (lane j holds
// entry j, sorted); each batch of 32 candidates is checked against the K-th key with one ballot
// and the few that qualify are inserted with a shuffle-shift, so the pruning threshold is always
// exact. Lists longer than 32 (kneighbors takes k up to 1000, helper.c:32-35) belong to one CTA
// per query and stay sorted in shared memory (exact_dfs_big_kernel).
#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "handle.cuh"
#include "tree_walk.cuh"

namespace annf {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------------------------
// keys
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
  __device__ static K shfl(K v, int src) { return __shfl_sync(kFull, v, src); }
  __device__ static K shfl_up(K v, int d) { return __shfl_up_sync(kFull, v, d); }
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
  __device__ static K shfl(K v, int src) { return dkey{__shfl_sync(kFull, v.d, src), __shfl_sync(kFull, v.tie, src)}; }
  __device__ static K shfl_up(K v, int d) { return dkey{__shfl_up_sync(kFull, v.d, d), __shfl_up_sync(kFull, v.tie, d)}; }
  __device__ static K shfl_xor(K v, int m) { return dkey{__shfl_xor_sync(kFull, v.d, m), __shfl_xor_sync(kFull, v.tie, m)}; }
};

// K-list distributed over the warp: lane j < K holds entry j (ascending); other lanes hold +inf
template <typename T>
struct WarpList {
  using Ops = KeyOps<T>;
  using Kt = typename Ops::K;
  Kt key;
  int pos;
  Kt thr;  // entry K-1 (uniform)
  int K, lane;
  __device__ __forceinline__ void init(int K_, int lane_) {
    K = K_;
    lane = lane_;
    key = lane < K ? Ops::init() : Ops::inf();
    pos = 0;
    thr = Ops::init();
  }
  __device__ __forceinline__ void insert(Kt c, int p) {  // c < thr, warp-uniform
    const unsigned m = __ballot_sync(kFull, lane < K && Ops::lt(c, key));
    const int ins = __ffs(m) - 1;
    const Kt up = Ops::shfl_up(key, 1);
    const int pup = __shfl_up_sync(kFull, pos, 1);
    if (lane < K && lane > ins) {
      key = up;
      pos = pup;
    }
    if (lane == ins) {
      key = c;
      pos = p;
    }
    thr = Ops::shfl(key, K - 1);
  }
  // every lane offers at most one candidate; all that beat the K-th entry are inserted
  __device__ __forceinline__ void offer(bool valid, Kt c, int p) {
    unsigned m = __ballot_sync(kFull, valid && Ops::lt(c, thr));
    while (m) {
      const int src = __ffs(m) - 1;
      insert(Ops::shfl(c, src), __shfl_sync(kFull, p, src));
      m &= m - 1;
      m &= __ballot_sync(kFull, valid && Ops::lt(c, thr));
    }
  }
};

// per-lane sorted list of KM entries + warp merge (used where every lane scans many candidates)
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
      for (int j = 0; j < D / 4; ++j)
        acc = dist_step4(acc, __ldg(p4 + j), v[4 * j + 0], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    } else {
#pragma unroll
      for (int j = 0; j < D; ++j) {
        T t = R::sub(__ldg(p + j), v[j]);
        acc = R::add(acc, R::mul(t, t));
      }
    }
    return acc;
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
};

// Four distances at once. Each keeps the reference's dimension order, but the four dependent
// add chains are interleaved, so a lane has four independent instructions in flight instead of
// one (a distance is a chain of d dependent rounded adds). kSmem: points in shared memory.
template <bool kSmem, typename T, int D>
__device__ __forceinline__ void dist4(const QReg<T, D>& q, const T* p0, const T* p1, const T* p2, const T* p3, int d,
                                      T (&acc)[4]) {
  using R = real_traits<T>;
  const T* p[4] = {p0, p1, p2, p3};
#pragma unroll
  for (int u = 0; u < 4; ++u) acc[u] = T(0);
  if constexpr (D > 0 && sizeof(T) == 4 && D % 4 == 0) {
#pragma unroll
    for (int j = 0; j < D / 4; ++j) {
      float4 w[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        w[u] = kSmem ? reinterpret_cast<const float4*>(p[u])[j] : __ldg(reinterpret_cast<const float4*>(p[u]) + j);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        acc[u] = dist_step4(acc[u], w[u], q.v[4 * j + 0], q.v[4 * j + 1], q.v[4 * j + 2], q.v[4 * j + 3]);
    }
  } else {
    const int dd = D > 0 ? D : d;
#pragma unroll(D > 0 ? D : 1)
    for (int j = 0; j < dd; ++j) {
      const T qj = q.v[j];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const T t = R::sub(kSmem ? p[u][j] : __ldg(p[u] + j), qj);
        acc[u] = R::add(acc[u], R::mul(t, t));
      }
    }
  }
}

// N distances at once (N interleaved chains), points in global memory
template <int N, typename T, int D>
__device__ __forceinline__ void distN(const QReg<T, D>& q, const T* const (&p)[N], T (&acc)[N]) {
  using R = real_traits<T>;
#pragma unroll
  for (int u = 0; u < N; ++u) acc[u] = T(0);
  if constexpr (sizeof(T) == 4 && D % 4 == 0) {
#pragma unroll
    for (int j = 0; j < D / 4; ++j) {
      float4 w[N];
#pragma unroll
      for (int u = 0; u < N; ++u) w[u] = __ldg(reinterpret_cast<const float4*>(p[u]) + j);
#pragma unroll
      for (int u = 0; u < N; ++u)
        acc[u] = dist_step4(acc[u], w[u], q.v[4 * j + 0], q.v[4 * j + 1], q.v[4 * j + 2], q.v[4 * j + 3]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < D; ++j) {
#pragma unroll
      for (int u = 0; u < N; ++u) {
        const T t = R::sub(__ldg(p[u] + j), q.v[j]);
        acc[u] = R::add(acc[u], R::mul(t, t));
      }
    }
  }
}

// natural leaf span of every query (thread per query)
template <typename T>
__global__ void __launch_bounds__(256) natural_leaf_kernel(TreeView<T> tv, const T* __restrict__ Q, long long q0,
                                                           long long nq, int2* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  NodeCache<T> nc;
  nc.carve(p, tv.depth);
  if (smem_overrun(smem_raw, p, tv.status)) return;
  nc.fill(tv);
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nq; i += (long long)gridDim.x * blockDim.x) {
    const int lf = descend(tv, nc, Q + (q0 + i) * tv.d);
    out[i] = make_int2(__ldg(tv.leaf_begin + lf), __ldg(tv.leaf_begin + lf + 1));
  }
}

// natural leaf + its top-K for every query (warp per query); used when propagation is off
template <typename T, int D, int KM>
__global__ void __launch_bounds__(256) natural_knn_kernel(TreeView<T> tv, const T* __restrict__ Q, long long q0,
                                                          long long nq, int K, int* __restrict__ out_pos,
                                                          typename KeyOps<T>::K* __restrict__ out_key) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  NodeCache<T> nc;
  nc.carve(p, tv.depth);
  T* sq = reinterpret_cast<T*>(p) + (threadIdx.x >> 5) * kMaxDynD;
  if (smem_overrun(smem_raw, reinterpret_cast<T*>(p) + (blockDim.x >> 5) * kMaxDynD, tv.status)) return;
  nc.fill(tv);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const int d = tv.d;
  for (long long qi = q0 + gw; qi < q0 + nq; qi += nw) {
    const T* q = Q + qi * d;
    __syncwarp();
    for (int j = lane; j < d; j += 32) sq[j] = q[j];
    __syncwarp();
    QReg<T, D> qr;
    if constexpr (D == 0) {
      qr.v = sq;
      qr.d = d;
    } else {
      qr.load(sq, d);
    }
    const int leaf = descend(tv, nc, sq);
    const int beg = __ldg(tv.leaf_begin + leaf), end = __ldg(tv.leaf_begin + leaf + 1);
    LaneList<T, KM> L;
    L.init_entries();
    const uint32_t slot = 1u << tv.leaf_bits;
    for (int base = beg; base < end; base += 128) {  // four candidates per lane per pass
      int pp[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) pp[u] = base + lane + 32 * u;
      T dd[4];
      dist4<false>(qr, tv.pts + (long long)min(pp[0], end - 1) * d, tv.pts + (long long)min(pp[1], end - 1) * d,
                   tv.pts + (long long)min(pp[2], end - 1) * d, tv.pts + (long long)min(pp[3], end - 1) * d, d, dd);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (pp[u] < end) L.offer(KeyOps<T>::make(dd[u], slot | (uint32_t)(pp[u] - beg)), pp[u]);
    }
    typename KeyOps<T>::K k;
    int pos = 0;
    warp_topk<T, KM>(L, K, lane, k, pos);
    if (lane < K) {
      out_pos[qi * K + lane] = pos;
      if (out_key) out_key[qi * K + lane] = k;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// exact kNN with backtracking (first row, kneighbors): warp per query, DFS near child first,
// far child pruned when (q[axis]-split)^2 > K-th distance, at most max_leaves leaves scanned --
// the reference's traversal (kdtree.c:129-268), leaf scans spread over the lanes
// ---------------------------------------------------------------------------------------------
constexpr int kDfsWarps = 8;

template <typename T, int D>
__global__ void __launch_bounds__(32 * kDfsWarps) exact_dfs_kernel(TreeView<T> tv, const T* __restrict__ Q, int nq,
                                                                    int K, long long max_leaves, int mode,
                                                                    int* __restrict__ out_pos, T* __restrict__ out_dist,
                                                                    int* __restrict__ out_idx) {
  using Ops = KeyOps<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  NodeCache<T> nc;
  nc.carve(p, tv.depth);
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* sq = reinterpret_cast<T*>(p) + wib * kMaxDynD;
  p += kDfsWarps * kMaxDynD * sizeof(T);
  T* sbound = reinterpret_cast<T*>(p) + wib * 32;
  p += kDfsWarps * 32 * sizeof(T);
  int* snode = reinterpret_cast<int*>(p) + wib * 32;
  p += kDfsWarps * 32 * sizeof(int);
  uint32_t* srank = reinterpret_cast<uint32_t*>(p) + wib * 32;
  p += kDfsWarps * 32 * sizeof(uint32_t);
  if (smem_overrun(smem_raw, p, tv.status)) return;
  nc.fill(tv);
  __syncthreads();
  const int d = tv.d, depth = tv.depth;
  const int first_leaf = (1 << depth) - 1;
  for (int qi = blockIdx.x * kDfsWarps + wib; qi < nq; qi += gridDim.x * kDfsWarps) {
    __syncwarp();
    for (int j = lane; j < d; j += 32) sq[j] = Q[(long long)qi * d + j];
    __syncwarp();
    QReg<T, D> qr;
    if constexpr (D == 0) {
      qr.v = sq;
      qr.d = d;
    } else {
      qr.load(sq, d);
    }
    WarpList<T> L;
    L.init(K, lane);
    long long budget = max_leaves;
    // stack of pending far children: node, dfs-rank prefix, lower bound on their distances
    if (lane == 0) {
      snode[0] = 0;
      srank[0] = 0;
      sbound[0] = T(0);
    }
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
      --sp;
      int node = snode[sp];
      uint32_t rank = srank[sp];
      const T bound = sbound[sp];
      __syncwarp();
      if (bound > Ops::dist(L.thr)) continue;  // (q-s)^2 > d_min[K-1]: skip (kdtree.c:219, 236)
      int level = 31 - __clz(node + 1);         // depth of 'node'
      while (level < depth) {
        int ax;
        T s;
        nc.get(tv, node, ax, s);
        const T diff = real_traits<T>::sub(sq[ax], s);
        const bool right = diff >= T(0);
        if (lane == 0) {
          snode[sp] = right ? 2 * node + 1 : 2 * node + 2;
          srank[sp] = (rank << 1) | 1u;
          sbound[sp] = real_traits<T>::mul(diff, diff);
        }
        ++sp;
        node = right ? 2 * node + 2 : 2 * node + 1;
        rank <<= 1;
        ++level;
      }
      __syncwarp();
      if (budget <= 0) break;  // the reference stops at the leaf that exceeds max_leaves
      --budget;
      const int lf = node - first_leaf;
      const int beg = __ldg(tv.leaf_begin + lf), end = __ldg(tv.leaf_begin + lf + 1);
      const uint32_t hi = rank << tv.leaf_bits;
      for (int base = beg; base < end; base += 32) {
        const int pp = base + lane;
        const bool valid = pp < end;
        const T dd = valid ? qr.dist(tv.pts + (long long)pp * d, d) : T(0);
        L.offer(valid, Ops::make(dd, hi | (uint32_t)(pp - beg)), pp);
      }
    }
    if (lane < K) {
      if (mode == 0) {
        out_pos[(long long)qi * K + lane] = L.pos;
      } else {
        out_dist[(long long)qi * K + lane] = real_traits<T>::sqrt_(Ops::dist(L.key));
        out_idx[(long long)qi * K + lane] = __ldg(tv.perm + L.pos);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// the same backtracking search for K above 32 (the reference accepts K up to 1000): one CTA per
// query. The K-list lives in shared memory, sorted by key; warp 0's lane 0 runs the traversal
// (the same stack, pruning and leaf budget as exact_dfs_kernel) and hands each leaf to the CTA,
// which computes the leaf's distances kBigBatch points at a time, keeps those below the current
// K-th key, sorts them (bitonic) and merges them into the list by rank. Keys are unique (distance,
// the leaf's depth-first rank, the offset), so the merged list is the one the reference's
// one-by-one insertion builds.
// ---------------------------------------------------------------------------------------------
constexpr int kBigThreads = 256;
constexpr int kBigBatch = 256;  // candidates merged at a time (a power of two <= kBigThreads)
constexpr int kBigStack = 64;  // > the deepest tree (30 levels) + 1

template <typename T>
static size_t dfs_big_smem(int depth, int K) {
  using Kt = typename KeyOps<T>::K;
  return NodeCache<T>::bytes(depth) + 2 * (size_t)K * (sizeof(Kt) + sizeof(int)) +
         (size_t)kBigBatch * (sizeof(Kt) + sizeof(int)) + kMaxDynD * sizeof(T) +
         (size_t)kBigStack * (sizeof(T) + sizeof(int) + sizeof(uint32_t)) + 8 * sizeof(int) + 128;
}

template <typename T>
__global__ void __launch_bounds__(kBigThreads) exact_dfs_big_kernel(TreeView<T> tv, const T* __restrict__ Q, int nq,
                                                                    int K, long long max_leaves, int mode,
                                                                    int* __restrict__ out_pos,
                                                                    T* __restrict__ out_dist,
                                                                    int* __restrict__ out_idx) {
  using Ops = KeyOps<T>;
  using Kt = typename Ops::K;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  NodeCache<T> nc;
  nc.carve(p, tv.depth);
  auto align16 = [](unsigned char* q) { return reinterpret_cast<unsigned char*>(((uintptr_t)q + 15) & ~uintptr_t(15)); };
  p = align16(p);
  Kt* lk[2];
  int* lp[2];
  lk[0] = reinterpret_cast<Kt*>(p);
  lk[1] = lk[0] + K;
  p = align16(reinterpret_cast<unsigned char*>(lk[1] + K));
  Kt* ck = reinterpret_cast<Kt*>(p);  // [kBigBatch] this batch's candidates
  p = align16(reinterpret_cast<unsigned char*>(ck + kBigBatch));
  lp[0] = reinterpret_cast<int*>(p);
  lp[1] = lp[0] + K;
  int* cp = lp[1] + K;                       // [kBigBatch]
  T* sq = reinterpret_cast<T*>(align16(reinterpret_cast<unsigned char*>(cp + kBigBatch)));  // [kMaxDynD]
  T* sbound = sq + kMaxDynD;                 // [kBigStack]
  int* snode = reinterpret_cast<int*>(sbound + kBigStack);
  uint32_t* srank = reinterpret_cast<uint32_t*>(snode + kBigStack);
  int* sctl = reinterpret_cast<int*>(srank + kBigStack);  // [0] leaf, [1] rank, [2] candidates
  if (smem_overrun(smem_raw, sctl + 8, tv.status)) return;
  nc.fill(tv);
  __syncthreads();
  const int tid = threadIdx.x, d = tv.d, depth = tv.depth;
  const int first_leaf = (1 << depth) - 1;
  QReg<T, 0> qr;
  qr.v = sq;
  qr.d = d;
  for (int qi = blockIdx.x; qi < nq; qi += gridDim.x) {
    for (int j = tid; j < d; j += kBigThreads) sq[j] = Q[(long long)qi * d + j];
    for (int i = tid; i < K; i += kBigThreads) {
      lk[0][i] = Ops::init();  // (max real, position 0) fill any shortfall, as the reference
      lp[0][i] = 0;
    }
    int cur = 0;
    int sp = 1;  // traversal state: lane 0 of warp 0 only
    long long budget = max_leaves;
    if (tid == 0) {
      snode[0] = 0;
      srank[0] = 0;
      sbound[0] = T(0);
    }
    __syncthreads();
    while (true) {
      if (tid == 0) {
        int leaf = -1;
        uint32_t lrank = 0;
        const T kth = Ops::dist(lk[cur][K - 1]);
        while (sp > 0) {
          --sp;
          int node = snode[sp];
          uint32_t rank = srank[sp];
          if (sbound[sp] > kth) continue;  // (q-s)^2 > d_min[K-1]: skip (kdtree.c:219, 236)
          int level = 31 - __clz(node + 1);
          while (level < depth) {  // depth <= 30: at most depth entries pending, below kBigStack
            int ax;
            T s;
            nc.get(tv, node, ax, s);
            const T diff = real_traits<T>::sub(sq[ax], s);
            const bool right = diff >= T(0);
            snode[sp] = right ? 2 * node + 1 : 2 * node + 2;
            srank[sp] = (rank << 1) | 1u;
            sbound[sp] = real_traits<T>::mul(diff, diff);
            ++sp;
            node = right ? 2 * node + 2 : 2 * node + 1;
            rank <<= 1;
            ++level;
          }
          if (budget <= 0) {  // the reference stops at the leaf that exceeds max_leaves
            sp = 0;
            break;
          }
          --budget;
          leaf = node - first_leaf;
          lrank = rank;
          break;
        }
        sctl[0] = leaf;
        sctl[1] = (int)lrank;
      }
      __syncthreads();
      const int leaf = sctl[0];
      const uint32_t hi = (uint32_t)sctl[1] << tv.leaf_bits;
      __syncthreads();  // every thread has read the hand-off before lane 0 writes the next one
      if (leaf < 0) break;  // uniform
      const int beg = __ldg(tv.leaf_begin + leaf), end = __ldg(tv.leaf_begin + leaf + 1);
      for (int base = beg; base < end; base += kBigBatch) {
        // this batch's points whose keys beat the current K-th, compacted in point order
        const Kt thr = lk[cur][K - 1];
        const int pp = base + tid;
        Kt key = Ops::inf();
        bool take = false;
        if (tid < kBigBatch && pp < end) {
          key = Ops::make(qr.dist(tv.pts + (long long)pp * d, d), hi | (uint32_t)(pp - beg));
          take = Ops::lt(key, thr);
        }
        if (tid == 0) sctl[2] = 0;
        __syncthreads();
        const unsigned bal = __ballot_sync(0xffffffffu, take);
        int wbase = 0;
        if ((tid & 31) == 0 && bal) wbase = atomicAdd(&sctl[2], __popc(bal));
        wbase = __shfl_sync(0xffffffffu, wbase, 0);
        if (take) {
          const int at = wbase + __popc(bal & ((1u << (tid & 31)) - 1u));
          ck[at] = key;
          cp[at] = pp;
        }
        __syncthreads();
        const int m = sctl[2];
        __syncthreads();  // every thread has read the count before the next batch resets it
        if (m == 0) continue;  // uniform
        int M = 1;
        while (M < m) M <<= 1;
        for (int i = m + tid; i < M; i += kBigThreads) ck[i] = Ops::inf();
        __syncthreads();
        // bitonic sort of ck[0 .. M) (ascending), positions with their keys
        for (int k2 = 2; k2 <= M; k2 <<= 1) {
          for (int j = k2 >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < M; i += kBigThreads) {
              const int ixj = i ^ j;
              if (ixj > i) {
                const Kt a = ck[i], b = ck[ixj];
                const bool asc = (i & k2) == 0;
                if (asc ? Ops::lt(b, a) : Ops::lt(a, b)) {
                  ck[i] = b;
                  ck[ixj] = a;
                  const int t = cp[i];
                  cp[i] = cp[ixj];
                  cp[ixj] = t;
                }
              }
            }
            __syncthreads();
          }
        }
        // merge by rank into the other buffer: an entry's place is its index plus the number of
        // the other list's keys below it (no key of one list equals a key of the other)
        const int nxt = cur ^ 1;
        for (int i = tid; i < K; i += kBigThreads) {
          const Kt t = lk[cur][i];
          int lo = 0, hi2 = m;
          while (lo < hi2) {
            const int mid = (lo + hi2) >> 1;
            if (Ops::lt(ck[mid], t)) lo = mid + 1; else hi2 = mid;
          }
          const int r = i + lo;
          if (r < K) {
            lk[nxt][r] = t;
            lp[nxt][r] = lp[cur][i];
          }
        }
        for (int j = tid; j < m; j += kBigThreads) {
          const Kt c = ck[j];
          int lo = 0, hi2 = K;
          while (lo < hi2) {
            const int mid = (lo + hi2) >> 1;
            if (Ops::lt(lk[cur][mid], c)) lo = mid + 1; else hi2 = mid;
          }
          const int r = j + lo;
          if (r < K) {
            lk[nxt][r] = c;
            lp[nxt][r] = cp[j];
          }
        }
        __syncthreads();
        cur = nxt;
      }
    }
    for (int i = tid; i < K; i += kBigThreads) {
      if (mode == 0) {
        out_pos[(long long)qi * K + i] = lp[cur][i];
      } else {
        out_dist[(long long)qi * K + i] = real_traits<T>::sqrt_(Ops::dist(lk[cur][i]));
        out_idx[(long long)qi * K + i] = __ldg(tv.perm + lp[cur][i]);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// exact kNN without a leaf budget: the same result as the backtracking search (top-K by key over
// all points), computed as a tiled brute force over the leaves that cannot be skipped. A leaf is
// skipped when the distance from the query to its bounding box, evaluated with the same rounded
// operations as the point distances (so it bounds every point's distance from below), exceeds the
// query's current K-th distance; the natural leaf's K-th distance seeds that threshold. Thread
// per query (128-query tiles of adjacent pixels), leaf ranges split over blockIdx.y, partial
// lists merged by exact_merge_kernel.
// ---------------------------------------------------------------------------------------------
constexpr int kBoxThreads = 128;

template <typename T, int D, int KM>
__global__ void __launch_bounds__(kBoxThreads) exact_box_kernel(
    TreeView<T> tv, const T* __restrict__ Q, int nq, int K, const typename KeyOps<T>::K* __restrict__ seed_key,
    int leaves_per_split, typename KeyOps<T>::K* __restrict__ part_key, int* __restrict__ part_pos) {
  using Ops = KeyOps<T>;
  using R = real_traits<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int d = tv.d;
  const int dstride = d + 1;
  unsigned char* p = smem_raw;
  NodeCache<T> nc;
  nc.carve(p, tv.depth);
  T* sq = reinterpret_cast<T*>(p);                       // [kBoxThreads][d+1]
  T* sbox = sq + kBoxThreads * dstride;                  // [2][d]
  T* spts = reinterpret_cast<T*>(((uintptr_t)(sbox + 2 * d) + 15) & ~uintptr_t(15));  // [max_leaf][d]
  const int max_leaf = (int)(((long long)tv.n + (1 << tv.depth) - 1) >> tv.depth);
  if (smem_overrun(smem_raw, spts + (size_t)max_leaf * d, tv.status)) return;
  nc.fill(tv);
  const int qi = blockIdx.x * kBoxThreads + threadIdx.x;
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
  // every candidate of the global top-K is at most the seed list's K-th distance away
  const T seed = (active && seed_key) ? Ops::dist(seed_key[(long long)qi * K + K - 1]) : real_traits<T>::big();
  LaneList<T, KM> L;
  L.init_entries();
  const int nleaves = 1 << tv.depth;
  const int l0 = blockIdx.y * leaves_per_split, l1 = min(nleaves, l0 + leaves_per_split);
  __syncthreads();
  for (int lf = l0; lf < l1; ++lf) {
    for (int e = threadIdx.x; e < 2 * d; e += blockDim.x) sbox[e] = __ldg(tv.leaf_box + (long long)lf * 2 * d + e);
    __syncthreads();
    T lb = 0;
    for (int j = 0; j < (D > 0 ? D : d); ++j) {
      const T qv = sq[threadIdx.x * dstride + j];
      const T lo = sbox[j], hi = sbox[d + j];
      const T g = qv < lo ? R::sub(lo, qv) : (qv > hi ? R::sub(qv, hi) : T(0));
      lb = R::add(lb, R::mul(g, g));
    }
    const T kth = Ops::dist(L.key[KM - 1]);
    const T thr = kth < seed ? kth : seed;
    const bool need = active && !(lb > thr);
    if (__syncthreads_or(need)) {
      const int beg = __ldg(tv.leaf_begin + lf), end = __ldg(tv.leaf_begin + lf + 1);
      const int cnt = end - beg;
      for (int e = threadIdx.x; e < cnt * d; e += blockDim.x) spts[e] = tv.pts[(long long)beg * d + e];
      __syncthreads();
      if (need) {
        uint32_t rank = 0;  // this leaf's position in the query's depth-first visiting order
        for (int t = 0; t < tv.depth; ++t) {
          const int node = (1 << t) - 1 + (lf >> (tv.depth - t));
          const int dir = (lf >> (tv.depth - 1 - t)) & 1;
          int ax;
          T s;
          nc.get(tv, node, ax, s);
          const int side = sq[threadIdx.x * dstride + ax] >= s ? 1 : 0;
          rank = (rank << 1) | (uint32_t)(dir ^ side);
        }
        const uint32_t hi = rank << tv.leaf_bits;
        for (int pp = 0; pp < cnt; pp += 4) {
          const int last = cnt - 1;
          T acc[4];
          dist4<true>(qr, spts + min(pp, last) * d, spts + min(pp + 1, last) * d, spts + min(pp + 2, last) * d,
                      spts + min(pp + 3, last) * d, d, acc);
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (pp + u < cnt && !(acc[u] > seed)) L.offer(Ops::make(acc[u], hi | (uint32_t)(pp + u)), beg + pp + u);
        }
      }
    }
    __syncthreads();
  }
  if (active) {
    const long long base = ((long long)blockIdx.y * nq + qi) * K;
    for (int j = 0; j < K && j < KM; ++j) {
      part_key[base + j] = L.key[j];
      part_pos[base + j] = L.pos[j];
    }
  }
}

// Exact kNN for a moderate number of queries: warp per query; the lanes test 32 leaf boxes at a
// time and the warp scans only the leaves whose box lies within the query's current K-th distance
// (seeded by the natural leaf's K-th distance). The K-list lives distributed over the lanes, so
// the threshold is exact after every leaf.
template <typename T, int D>
__global__ void __launch_bounds__(256) exact_scan_kernel(TreeView<T> tv, const T* __restrict__ Q, int nq, int K,
                                                         const typename KeyOps<T>::K* __restrict__ seed_key, int mode,
                                                         int* __restrict__ out_pos, T* __restrict__ out_dist,
                                                         int* __restrict__ out_idx) {
  using Ops = KeyOps<T>;
  using R = real_traits<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  NodeCache<T> nc;
  nc.carve(p, tv.depth);
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* sq = reinterpret_cast<T*>(p) + wib * kMaxDynD;
  if (smem_overrun(smem_raw, reinterpret_cast<T*>(p) + (blockDim.x >> 5) * kMaxDynD, tv.status)) return;
  nc.fill(tv);
  __syncthreads();
  const int d = tv.d, depth = tv.depth;
  const int nleaves = 1 << depth;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int qi = blockIdx.x * (blockDim.x >> 5) + wib; qi < nq; qi += nw) {
    __syncwarp();
    for (int j = lane; j < d; j += 32) sq[j] = Q[(long long)qi * d + j];
    __syncwarp();
    QReg<T, D> qr;
    if constexpr (D == 0) {
      qr.v = sq;
      qr.d = d;
    } else {
      qr.load(sq, d);
    }
    const T seed = seed_key ? Ops::dist(seed_key[(long long)qi * K + K - 1]) : real_traits<T>::big();
    WarpList<T> L;
    L.init(K, lane);
    for (int base = 0; base < nleaves; base += 32) {
      const int lf = base + lane;
      T lb = real_traits<T>::big();
      if (lf < nleaves) {
        const T* box = tv.leaf_box + (long long)lf * 2 * d;
        lb = T(0);
        for (int j = 0; j < d; ++j) {
          const T qv = sq[j], lo = __ldg(box + j), hi = __ldg(box + d + j);
          const T g = qv < lo ? R::sub(lo, qv) : (qv > hi ? R::sub(qv, hi) : T(0));
          lb = R::add(lb, R::mul(g, g));
        }
      }
      T kth = Ops::dist(L.thr);
      unsigned m = __ballot_sync(kFull, lf < nleaves && !(lb > (kth < seed ? kth : seed)));
      while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        kth = Ops::dist(L.thr);
        if (__shfl_sync(kFull, lb, src) > (kth < seed ? kth : seed)) continue;  // pruned by now
        const int leaf = base + src;
        uint32_t rank = 0;  // the leaf's position in this query's depth-first visiting order
        for (int t = 0; t < depth; ++t) {
          const int node = (1 << t) - 1 + (leaf >> (depth - t));
          int ax;
          T s;
          nc.get(tv, node, ax, s);
          rank = (rank << 1) | (uint32_t)(((leaf >> (depth - 1 - t)) & 1) ^ (sq[ax] >= s ? 1 : 0));
        }
        const uint32_t hi = rank << tv.leaf_bits;
        const int beg = __ldg(tv.leaf_begin + leaf), end = __ldg(tv.leaf_begin + leaf + 1);
        for (int pb = beg; pb < end; pb += 128) {
          int pp[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) pp[u] = pb + lane + 32 * u;
          T dd[4];
          dist4<false>(qr, tv.pts + (long long)min(pp[0], end - 1) * d, tv.pts + (long long)min(pp[1], end - 1) * d,
                       tv.pts + (long long)min(pp[2], end - 1) * d, tv.pts + (long long)min(pp[3], end - 1) * d, d, dd);
#pragma unroll
          for (int u = 0; u < 4; ++u)
            L.offer(pp[u] < end && !(dd[u] > seed), Ops::make(dd[u], hi | (uint32_t)(pp[u] - beg)), pp[u]);
        }
      }
    }
    if (lane < K) {
      if (mode == 0) {
        out_pos[(long long)qi * K + lane] = L.pos;
      } else {
        out_dist[(long long)qi * K + lane] = R::sqrt_(Ops::dist(L.key));
        out_idx[(long long)qi * K + lane] = __ldg(tv.perm + L.pos);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Exact kNN by marked leaves, for a moderate number of queries (the first row of a pair: 2040
// queries over 32768 leaves at 2048x2048). A leaf can hold one of a query's exact K nearest only
// if its box lies within the query's seed distance (the K-th distance inside its natural leaf:
// the box bound never exceeds the distance of any point inside, in FP32 too, since the bound
// takes the same rounded steps on smaller differences). So:
//   1. leaf_mark_kernel: a CTA per (128-query tile, range of leaves) tests the ranges' boxes,
//      staged in shared memory and read by every thread at once, and writes one bit per
//      (query, leaf);
//   2. leaf_chunk_scan_kernel: a warp per (query, chunk of 32*CW leaves) scans the marked leaves
//      of its chunk with the reference's arithmetic and keeps the chunk's K best keys. Tasks run
//      chunk-major: warps that run together read the same leaves, which neighbouring pixels of a
//      row mostly share;
//   3. exact_merge_kernel: the K smallest keys over a query's chunks.
// Every key is unique (distance bits, the leaf's depth-first rank for that query, the offset in
// the leaf), so the K smallest over the marked leaves are the reference's K, found in any order.
// ---------------------------------------------------------------------------------------------
constexpr int kMarkThreads = 128;
constexpr int kMarkStage = 32;       // leaves whose boxes are staged at a time
constexpr int kChunkCacheLevels = 10;  // node levels the chunk scan keeps in shared memory (8 KB)

template <typename T, int D>
__global__ void __launch_bounds__(kMarkThreads) leaf_mark_kernel(TreeView<T> tv, const T* __restrict__ Q, int nq,
                                                                 int K, const typename KeyOps<T>::K* __restrict__ seed_key,
                                                                 int leaves_per_split, int nwords,
                                                                 uint32_t* __restrict__ marks) {
  using Ops = KeyOps<T>;
  using R = real_traits<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int d = D > 0 ? D : tv.d;
  T* sbox = reinterpret_cast<T*>(smem_raw);  // [kMarkStage][2][d]
  if (smem_overrun(smem_raw, sbox + kMarkStage * 2 * d, tv.status)) return;
  const int qi = blockIdx.x * kMarkThreads + threadIdx.x;
  const bool active = qi < nq;
  T q[D > 0 ? D : 1];
  const T* qg = Q + (long long)(active ? qi : 0) * d;
  if constexpr (D > 0) {
#pragma unroll
    for (int j = 0; j < D; ++j) q[j] = qg[j];
  }
  const T thr = active ? Ops::dist(seed_key[(long long)qi * K + K - 1]) : T(0);
  const int nleaves = 1 << tv.depth;
  const int l0 = blockIdx.y * leaves_per_split, l1 = min(nleaves, l0 + leaves_per_split);
  for (int s0 = l0; s0 < l1; s0 += kMarkStage) {
    const int ns = min(kMarkStage, l1 - s0);
    __syncthreads();
    for (int e = threadIdx.x; e < ns * 2 * d; e += kMarkThreads) sbox[e] = __ldg(tv.leaf_box + (long long)s0 * 2 * d + e);
    __syncthreads();
    uint32_t bits = 0;
    for (int i = 0; i < ns; ++i) {
      const T* lo = sbox + i * 2 * d;
      const T* hi = lo + d;
      T lb = 0;
      if constexpr (D > 0) {
#pragma unroll
        for (int j = 0; j < D; ++j) {
          const T g = q[j] < lo[j] ? R::sub(lo[j], q[j]) : (q[j] > hi[j] ? R::sub(q[j], hi[j]) : T(0));
          lb = R::add(lb, R::mul(g, g));
        }
      } else {
        for (int j = 0; j < d; ++j) {
          const T qv = qg[j];
          const T g = qv < lo[j] ? R::sub(lo[j], qv) : (qv > hi[j] ? R::sub(qv, hi[j]) : T(0));
          lb = R::add(lb, R::mul(g, g));
        }
      }
      bits |= (uint32_t)(!(lb > thr)) << i;
    }
    if (active) marks[(long long)qi * nwords + (s0 >> 5)] = bits;
  }
}

template <typename T, int D>
__global__ void __launch_bounds__(256, 3) leaf_chunk_scan_kernel(TreeView<T> tv, const T* __restrict__ Q, int nq, int K,
                                                              const typename KeyOps<T>::K* __restrict__ seed_key,
                                                              int nwords, int cw, const uint32_t* __restrict__ marks,
                                                              typename KeyOps<T>::K* __restrict__ part_key,
                                                              int* __restrict__ part_pos) {
  using Ops = KeyOps<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* p = smem_raw;
  NodeCache<T> nc;
  nc.carve(p, tv.depth, kChunkCacheLevels);
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* sq = reinterpret_cast<T*>(p) + wib * kMaxDynD;
  if (smem_overrun(smem_raw, reinterpret_cast<T*>(p) + (blockDim.x >> 5) * kMaxDynD, tv.status)) return;
  nc.fill(tv, kChunkCacheLevels);
  __syncthreads();
  const int d = tv.d, depth = tv.depth;
  const int nchunks = (nwords + cw - 1) / cw;
  const long long ntasks = (long long)nchunks * nq;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long task = blockIdx.x * (long long)(blockDim.x >> 5) + wib; task < ntasks; task += nw) {
    const int chunk = (int)(task / nq);
    const int qi = (int)(task - (long long)chunk * nq);
    WarpList<T> L;
    L.init(K, lane);
    const int w0 = chunk * cw, w1 = min(nwords, w0 + cw);
    // the chunk's marked words, one per lane
    const uint32_t myword = (w0 + lane < w1) ? __ldg(marks + (long long)qi * nwords + w0 + lane) : 0u;
    if (__ballot_sync(kFull, myword != 0u)) {
      __syncwarp();
      for (int j = lane; j < d; j += 32) sq[j] = Q[(long long)qi * d + j];
      __syncwarp();
      QReg<T, D> qr;
      if constexpr (D == 0) {
        qr.v = sq;
        qr.d = d;
      } else {
        qr.load(sq, d);
      }
      const T seed = Ops::dist(seed_key[(long long)qi * K + K - 1]);
      for (int wi = 0; wi < w1 - w0; ++wi) {
        const uint32_t bits = __shfl_sync(kFull, myword, wi);
        const int nset = __popc(bits);
        // lane i prepares the word's i-th marked leaf: its depth-first rank for this query (the
        // node lookups of all leaves in flight together) and its point range
        int pleaf = 0, pbeg = 0, pend = 0;
        uint32_t phi = 0;
        if (lane < nset) {
          pleaf = ((w0 + wi) << 5) + (int)__fns(bits, 0, lane + 1);
          uint32_t rank = 0;  // the leaf's position in this query's depth-first visiting order
          for (int t = 0; t < depth; ++t) {
            const int node = (1 << t) - 1 + (pleaf >> (depth - t));
            int ax;
            T s;
            nc.get(tv, node, ax, s);
            rank = (rank << 1) | (uint32_t)(((pleaf >> (depth - 1 - t)) & 1) ^ (sq[ax] >= s ? 1 : 0));
          }
          phi = rank << tv.leaf_bits;
          pbeg = __ldg(tv.leaf_begin + pleaf);
          pend = __ldg(tv.leaf_begin + pleaf + 1);
        }
        for (int li = 0; li < nset; ++li) {
          const uint32_t hi = __shfl_sync(kFull, phi, li);
          const int beg = __shfl_sync(kFull, pbeg, li), end = __shfl_sync(kFull, pend, li);
          for (int pb = beg; pb < end; pb += 128) {
            int pp[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) pp[u] = pb + lane + 32 * u;
            T dd[4];
            dist4<false>(qr, tv.pts + (long long)min(pp[0], end - 1) * d, tv.pts + (long long)min(pp[1], end - 1) * d,
                         tv.pts + (long long)min(pp[2], end - 1) * d, tv.pts + (long long)min(pp[3], end - 1) * d, d,
                         dd);
#pragma unroll
            for (int u = 0; u < 4; ++u)
              L.offer(pp[u] < end && !(dd[u] > seed), Ops::make(dd[u], hi | (uint32_t)(pp[u] - beg)), pp[u]);
          }
        }
      }
    }
    if (lane < K) {
      const long long o = ((long long)chunk * nq + qi) * K + lane;
      part_key[o] = L.key;
      part_pos[o] = L.pos;
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
  int pos = 0;
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

// L2 prefetch of the points [b, e) (contiguous in tree order), one 128-byte line per lane per pass
template <typename T>
__device__ __forceinline__ void prefetch_span_l2(const T* pts, int b, int e, int d, int lane) {
  if (e <= b) return;
  const char* base = reinterpret_cast<const char*>(pts + (long long)b * d);
  const int bytes = (e - b) * d * (int)sizeof(T);
  for (int off = lane * 128; off < bytes; off += 32 * 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(base + off));
}

// One warp per column walks the rows downwards (row y depends only on row y-1 of the same column).
// Per step: the natural leaf (span precomputed for every pixel) and the K propagated leaves; a
// leaf that several slots share is scanned once and its points are offered once per slot.
template <typename T, int D>
__global__ void __launch_bounds__(128, 1) chain_kernel(TreeView<T> tv, const T* __restrict__ Q, int n_rows, int n_cols,
                                                    int K, const int2* __restrict__ nat_range,
                                                    const int2* __restrict__ next_range, int* __restrict__ lists) {
  using Ops = KeyOps<T>;
  __shared__ T sqbuf[4][D > 0 ? 1 : kMaxDynD];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int x = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (x >= n_cols) return;
  const int d = tv.d;
  const int lb = tv.leaf_bits;
  int my_pos = lane < K ? lists[(long long)x * K + lane] : 0;
  // nat_range is indexed from row 1: entry (y-1)*n_cols + x
  int2 nat_next = __ldg(nat_range + x);
  QReg<T, D> q_next;
  if constexpr (D > 0) q_next.load(Q + ((long long)n_cols + x) * d, d);
  long long qi = (long long)n_cols + x;
  for (int y = 1; y < n_rows; ++y, qi += n_cols) {
    const int2 nat = nat_next;
    QReg<T, D> qr;
    if constexpr (D > 0) {
      qr = q_next;
      if (y + 1 < n_rows) {
        q_next.load(Q + (qi + n_cols) * d, d);
        nat_next = __ldg(nat_range + qi);  // row y+1
      }
    } else {
      __syncwarp();
      for (int j = lane; j < d; j += 32) sqbuf[wib][j] = Q[qi * d + j];
      __syncwarp();
      qr.v = sqbuf[wib];
      qr.d = d;
      if (y + 1 < n_rows) nat_next = __ldg(nat_range + qi);
    }
    const int2 rng = lane < K ? __ldg(next_range + my_pos) : make_int2(-1, -1);
    // start every propagated leaf on its way to L2 before the first distance needs it
    for (int j = 0; j < K; ++j) prefetch_span_l2(tv.pts, __shfl_sync(kFull, rng.x, j), __shfl_sync(kFull, rng.y, j), d, lane);
    // and the next row's natural leaf, which does not depend on this step
    if (y + 1 < n_rows) prefetch_span_l2(tv.pts, nat_next.x, nat_next.y, d, lane);
    WarpList<T> L;
    L.init(K, lane);
    // slots: bit 0 = natural leaf, bit j+1 = propagated neighbour j
    unsigned todo = (2u << K) - 1u;
    while (todo) {
      const int s0 = __ffs(todo) - 1;
      const int b = s0 == 0 ? nat.x : __shfl_sync(kFull, rng.x, s0 - 1);
      const int e = s0 == 0 ? nat.y : __shfl_sync(kFull, rng.y, s0 - 1);
      const unsigned same = ((nat.x == b ? 1u : 0u) | (__ballot_sync(kFull, lane < K && rng.x == b) << 1)) & todo;
      todo &= ~same;
      for (int base = b; base < e; base += 128) {  // four candidates per lane per pass
        int pp[4];
        bool valid[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          pp[u] = base + lane + 32 * u;
          valid[u] = pp[u] < e;
        }
        T dd[4];
        dist4<false>(qr, tv.pts + (long long)(valid[0] ? pp[0] : b) * d, tv.pts + (long long)(valid[1] ? pp[1] : b) * d,
                     tv.pts + (long long)(valid[2] ? pp[2] : b) * d, tv.pts + (long long)(valid[3] ? pp[3] : b) * d, d, dd);
        unsigned sl = same;
        while (sl) {
          const int s = __ffs(sl) - 1;
          sl &= sl - 1;
          const uint32_t hi = (uint32_t)(s + 1) << lb;
#pragma unroll
          for (int u = 0; u < 4; ++u) L.offer(valid[u], Ops::make(dd[u], hi | (uint32_t)(pp[u] - b)), pp[u]);
        }
      }
    }
    if (lane < K) lists[qi * K + lane] = L.pos;
    my_pos = L.pos;
  }
}

// The same step with compile-time bounds (FP32, fixed dimension, at most LM distinct leaves per
// step, at most 32*CPL points per leaf). All distinct leaves' distances are computed up front --
// their loads overlap -- and the K-list is then selected by K rounds of a warp-wide minimum over
// per-candidate keys. A candidate whose leaf serves several slots carries the mask of those slots
// and re-enters with its next slot once extracted, so points met twice are listed twice exactly
// as the reference's insertion does.
template <int D, int CPL, int LM>
__global__ void __launch_bounds__(64, 7) chain_sel_kernel(TreeView<float> tv, const float* __restrict__ Q, int n_rows,
                                                            int n_cols, int K, const int2* __restrict__ nat_range,
                                                            const int2* __restrict__ next_range, int* __restrict__ lists) {
  using Ops = KeyOps<float>;
  using Kt = Ops::K;
  const int lane = threadIdx.x & 31;
  const int x = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (x >= n_cols) return;
  const int lb = tv.leaf_bits;
  int my_pos = lane < K ? lists[(long long)x * K + lane] : 0;
  int2 nat_next = __ldg(nat_range + x);  // nat_range is indexed from row 1
  QReg<float, D> q_next;
  q_next.load(Q + ((long long)n_cols + x) * D, D);
  long long qi = (long long)n_cols + x;
  for (int y = 1; y < n_rows; ++y, qi += n_cols) {
    const int2 nat = nat_next;
    const QReg<float, D> qr = q_next;
    if (y + 1 < n_rows) {
      q_next.load(Q + (qi + n_cols) * D, D);
      nat_next = __ldg(nat_range + qi);
    }
    const int2 rng = lane < K ? __ldg(next_range + my_pos) : make_int2(-1, -1);
    if (y + 1 < n_rows) prefetch_span_l2(tv.pts, nat_next.x, nat_next.y, D, lane);
    // distinct leaves: slot bit 0 = natural leaf, bit j+1 = propagated neighbour j
    int lbeg[LM], lend[LM];
    unsigned lmask[LM];
    unsigned todo = (2u << K) - 1u;
#pragma unroll
    for (int i = 0; i < LM; ++i) {
      lbeg[i] = 0;
      lend[i] = 0;
      lmask[i] = 0;
      if (todo) {
        const int s0 = __ffs(todo) - 1;
        const int b = s0 == 0 ? nat.x : __shfl_sync(kFull, rng.x, s0 - 1);
        const int e = s0 == 0 ? nat.y : __shfl_sync(kFull, rng.y, s0 - 1);
        const unsigned same = ((nat.x == b ? 1u : 0u) | (__ballot_sync(kFull, lane < K && rng.x == b) << 1)) & todo;
        todo &= ~same;
        lbeg[i] = b;
        lend[i] = e;
        lmask[i] = same;
      }
    }
    // per-lane sorted list of its KM best (key, position, remaining slots)
    constexpr int KM = LM <= 2 ? 1 : (LM <= 5 ? 4 : 8);
    Kt lk[KM];
    int lp[KM];
    unsigned lr[KM];
#pragma unroll
    for (int j = 0; j < KM; ++j) {
      lk[j] = Ops::inf();
      lp[j] = 0;
      lr[j] = 0;
    }
    auto lane_offer = [&](Kt k, int p, unsigned r) {
      if (!(k < lk[KM - 1])) return;
#pragma unroll
      for (int j = KM - 1; j >= 0; --j) {
        if (j > 0 && k < lk[j - 1]) {
          lk[j] = lk[j - 1];
          lp[j] = lp[j - 1];
          lr[j] = lr[j - 1];
        } else if (k < lk[j]) {
          lk[j] = k;
          lp[j] = p;
          lr[j] = r;
        }
      }
    };
#pragma unroll
    for (int i = 0; i < LM; ++i) {
      if (lend[i] > lbeg[i]) {
        const float* pp[CPL];
#pragma unroll
        for (int u = 0; u < CPL; ++u) {
          const int p = lbeg[i] + lane + 32 * u;
          pp[u] = tv.pts + (long long)(p < lend[i] ? p : lbeg[i]) * D;
        }
        float dd[CPL];
        distN<CPL>(qr, pp, dd);
        const uint32_t slot = (uint32_t)__ffs(lmask[i]) << lb;
#pragma unroll
        for (int u = 0; u < CPL; ++u)
          if (lbeg[i] + lane + 32 * u < lend[i])
            lane_offer(Ops::make(dd[u], slot | (uint32_t)(lane + 32 * u)), lbeg[i] + lane + 32 * u, lmask[i]);
      }
    }
    // K rounds of warp-wide minimum over the lane heads; the initial entries (max real,
    // position 0) fill any shortfall
    const Kt low_mask = (Kt)((1u << lb) - 1u);
    int outpos = 0;
    for (int r = 0; r < K; ++r) {
      Kt wmin = lk[0];
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const Kt t = Ops::shfl_xor(wmin, o);
        wmin = t < wmin ? t : wmin;
      }
      if (!(wmin < Ops::init())) break;  // remaining entries stay (max real, position 0)
      const int winner = __ffs(__ballot_sync(kFull, lk[0] == wmin)) - 1;
      const int pos = __shfl_sync(kFull, lp[0], winner);
      if (lane == winner) {
        const unsigned nr = lr[0] & (lr[0] - 1u);  // next slot of the same point, if any
#pragma unroll
        for (int j = 0; j < KM - 1; ++j) {
          lk[j] = lk[j + 1];
          lp[j] = lp[j + 1];
          lr[j] = lr[j + 1];
        }
        lk[KM - 1] = Ops::inf();
        if (nr) lane_offer((wmin & ~(Kt)0xffffffffu) | ((Kt)((uint32_t)__ffs(nr) << lb)) | (wmin & low_mask), pos, nr);
      }
      if (lane == r) outpos = pos;
    }
    if (lane < K) lists[qi * K + lane] = outpos;
    my_pos = outpos;
  }
}

// ---------------------------------------------------------------------------------------------
// tree positions -> original indices, and the raw-patch re-rank (base.c:309-353, 362-374)
// ---------------------------------------------------------------------------------------------
// sum over a row of n bytes of (a-b)^2, exact in int (abytes / bbytes: the buffers' sizes)
__device__ __forceinline__ int row_ssd(const uint8_t* abase, long long aoff, long long abytes, const uint8_t* bbase,
                                       long long boff, long long bbytes, int n) {
  int s = 0;
  int e = 0;
  for (; e + 4 <= n; e += 4) {
    const unsigned x =
        __vabsdiffu4(load_word_bounded(abase, aoff + e, abytes), load_word_bounded(bbase, boff + e, bbytes));
    s = (int)__dp4a(x, x, (unsigned)s);
  }
  for (; e < n; ++e) {
    const int t = (int)__ldg(abase + aoff + e) - (int)__ldg(bbase + boff + e);
    s += t * t;
  }
  return s;
}

template <typename T>
__device__ __forceinline__ T patch_dist(const PatchSrc& A, long long ia, const PatchSrc& B, long long ib) {
  const int rowlen = A.psize * A.c;
  const int P = rowlen * A.psize;
  if (sizeof(T) == 8 || (long long)P * 65025 < (1LL << 24)) {
    long long acc = 0;  // every partial sum is exact in the reference's accumulator
    for (int r = 0; r < A.psize; ++r) {
      const long long ao = A.row(ia, r) - A.img, bo = B.row(ib, r) - B.img;
      acc += row_ssd(A.img, ao, A.bytes, B.img, bo, B.bytes, rowlen);
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
  tv.status = h->status.as<unsigned>();
  tv.leaf_box = h->leaf_box.as<T>();
  return tv;
}

static int pick_km(int K) { return K <= 1 ? 1 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32; }

int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  return sms;
}

#define ANNF_DISPATCH_KM(KMV, ...)                          \
  switch (KMV) {                                            \
    case 1: { constexpr int KM = 1; __VA_ARGS__; } break;   \
    case 4: { constexpr int KM = 4; __VA_ARGS__; } break;   \
    case 8: { constexpr int KM = 8; __VA_ARGS__; } break;   \
    case 16: { constexpr int KM = 16; __VA_ARGS__; } break; \
    default: { constexpr int KM = 32; __VA_ARGS__; } break; \
  }

// compile-time dimension for the common reduced sizes (FP32), runtime dimension otherwise
#define ANNF_DISPATCH_D(T, dval, ...)                                         \
  do {                                                                        \
    bool done_ = false;                                                       \
    if constexpr (sizeof(T) == 4) {                                           \
      switch (dval) {                                                         \
        case 8: { constexpr int D = 8; __VA_ARGS__; done_ = true; } break;    \
        case 12: { constexpr int D = 12; __VA_ARGS__; done_ = true; } break;  \
        case 16: { constexpr int D = 16; __VA_ARGS__; done_ = true; } break;  \
        default: break;                                                       \
      }                                                                       \
    }                                                                         \
    if (!done_) { constexpr int D = 0; __VA_ARGS__; }                         \
  } while (0)

template <typename T, int D>
static int exact_dfs_launch(annf_handle* h, const T* Q, int nq, int K, long long max_leaves, int mode, int* out_pos,
                            T* out_dist, int* out_idx, cudaStream_t st) {
  TreeView<T> tv = view_of<T>(h);
  // node cache + per warp: query copy, stack of bounds, stack of nodes, stack of rank prefixes
  const size_t smem = NodeCache<T>::bytes(h->depth) +
                      kDfsWarps * (kMaxDynD * sizeof(T) + 32 * sizeof(T) + 32 * sizeof(int) + 32 * sizeof(uint32_t)) + 64;
  ANNF_CUDA_TRY(cudaFuncSetAttribute(exact_dfs_kernel<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = std::max(1, std::min(ceil_div(nq, kDfsWarps), 32 * num_sms()));
  exact_dfs_kernel<T, D><<<blocks, 32 * kDfsWarps, smem, st>>>(tv, Q, nq, K, max_leaves, mode, out_pos, out_dist,
                                                                 out_idx);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

template <typename T, int D, int KM>
static int exact_box_launch(annf_handle* h, const T* Q, int nq, int K, int mode, int* out_pos, T* out_dist,
                            int* out_idx, cudaStream_t st) {
  using Kt = typename KeyOps<T>::K;
  TreeView<T> tv = view_of<T>(h);
  const int nleaves = 1 << h->depth;
  // seeds: each query's natural-leaf top-K
  ANNF_ENSURE(h->nat_keys, (size_t)nq * K * sizeof(Kt));
  ANNF_ENSURE(h->nat_pos, (size_t)nq * K * sizeof(int));
  const size_t nsm = NodeCache<T>::bytes(h->depth) + 8 * kMaxDynD * sizeof(T);
  ANNF_CUDA_TRY(cudaFuncSetAttribute(natural_knn_kernel<T, D, KM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nsm));
  natural_knn_kernel<T, D, KM><<<(int)std::min<long long>(ceil_div((long long)nq * 32, 256), 64LL * num_sms()), 256, nsm,
                                 st>>>(tv, Q, 0, nq, K, h->nat_pos.as<int>(), h->nat_keys.as<Kt>());
  ANNF_CHECK_LAUNCH();
  if ((long long)nq * nleaves <= (1LL << 28)) {  // few queries: marked leaves, scanned in chunks
    if (nq <= 0) return ANNF_OK;
    const int nwords = ceil_div(nleaves, 32);
    // chunk width: 2 words (64 leaves), wider when the partial lists would pass 256 MB
    int cw = 2;
    while (cw < nwords && (long long)ceil_div(nwords, cw) * nq * K * (long long)(sizeof(Kt) + sizeof(int)) > (256LL << 20))
      cw *= 2;
    const int nchunks = ceil_div(nwords, cw);
    ANNF_ENSURE(h->leaf_marks, (size_t)nq * nwords * sizeof(uint32_t));
    ANNF_ENSURE(h->part_keys, (size_t)nchunks * nq * K * sizeof(Kt));
    ANNF_ENSURE(h->part_pos, (size_t)nchunks * nq * K * sizeof(int));
    const int tiles = ceil_div(nq, kMarkThreads);
    const int want = std::max(1, (4 * num_sms()) / tiles);
    const int lps = std::max(32, ceil_div(ceil_div(nleaves, want), 32) * 32);
    const int nsplit = ceil_div(nleaves, lps);
    const size_t msm = (size_t)kMarkStage * 2 * h->d * sizeof(T) + 64;
    ANNF_CUDA_TRY(cudaFuncSetAttribute(leaf_mark_kernel<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msm));
    leaf_mark_kernel<T, D><<<dim3(tiles, nsplit), kMarkThreads, msm, st>>>(tv, Q, nq, K, h->nat_keys.as<Kt>(), lps,
                                                                          nwords, h->leaf_marks.as<uint32_t>());
    ANNF_CHECK_LAUNCH();
    const size_t ssm = NodeCache<T>::bytes(h->depth, kChunkCacheLevels) + 8 * kMaxDynD * sizeof(T) + 64;
    ANNF_CUDA_TRY(cudaFuncSetAttribute(leaf_chunk_scan_kernel<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
    const long long ntasks = (long long)nchunks * nq;
    leaf_chunk_scan_kernel<T, D><<<(int)std::max(1LL, std::min<long long>(ceil_div(ntasks, 8LL), 16LL * num_sms())), 256, ssm, st>>>(
        tv, Q, nq, K, h->nat_keys.as<Kt>(), nwords, cw, h->leaf_marks.as<uint32_t>(), h->part_keys.as<Kt>(),
        h->part_pos.as<int>());
    ANNF_CHECK_LAUNCH();
    exact_merge_kernel<T, KM><<<ceil_div((long long)nq * 32, 256), 256, 0, st>>>(
        tv, nq, K, nchunks, h->part_keys.as<Kt>(), h->part_pos.as<int>(), mode, out_pos, out_dist, out_idx);
    ANNF_CHECK_LAUNCH();
    return ANNF_OK;
  }
  const int tiles = ceil_div(nq, kBoxThreads);
  const int want = std::max(1, (4 * num_sms()) / tiles);
  const int lps = std::max(1, ceil_div(nleaves, want));
  const int nsplit = ceil_div(nleaves, lps);
  ANNF_ENSURE(h->part_keys, (size_t)nsplit * nq * K * sizeof(Kt));
  ANNF_ENSURE(h->part_pos, (size_t)nsplit * nq * K * sizeof(int));
  const size_t smem = NodeCache<T>::bytes(h->depth) + (size_t)kBoxThreads * (h->d + 1) * sizeof(T) +
                      2 * h->d * sizeof(T) + 32 + (size_t)h->max_leaf * h->d * sizeof(T) + 64;
  ANNF_CUDA_TRY(cudaFuncSetAttribute(exact_box_kernel<T, D, KM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  exact_box_kernel<T, D, KM><<<dim3(tiles, nsplit), kBoxThreads, smem, st>>>(tv, Q, nq, K, h->nat_keys.as<Kt>(), lps,
                                                                             h->part_keys.as<Kt>(), h->part_pos.as<int>());
  ANNF_CHECK_LAUNCH();
  exact_merge_kernel<T, KM><<<ceil_div((long long)nq * 32, 256), 256, 0, st>>>(
      tv, nq, K, nsplit, h->part_keys.as<Kt>(), h->part_pos.as<int>(), mode, out_pos, out_dist, out_idx);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

template <typename T>
static int exact_dfs_big_launch(annf_handle* h, const T* Q, int nq, int K, long long max_leaves, int mode,
                                int* out_pos, T* out_dist, int* out_idx, cudaStream_t st) {
  TreeView<T> tv = view_of<T>(h);
  const size_t smem = dfs_big_smem<T>(h->depth, K);
  ANNF_REQUIRE(smem <= 227 * 1024, "kneighbors: K too large for the shared-memory list");
  ANNF_CUDA_TRY(cudaFuncSetAttribute(exact_dfs_big_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = std::max(1, std::min(nq, 8 * num_sms()));
  exact_dfs_big_kernel<T><<<blocks, kBigThreads, smem, st>>>(tv, Q, nq, K, max_leaves, mode, out_pos, out_dist,
                                                              out_idx);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

template <typename T, int D>
static int exact_knn_typed(annf_handle* h, const T* Q, int nq, int K, long long max_leaves, int mode, int* out_pos,
                           T* out_dist, int* out_idx, cudaStream_t st) {
  if (K > 32)  // the warp-list kernels hold at most 32 entries
    return exact_dfs_big_launch<T>(h, Q, nq, K, max_leaves, mode, out_pos, out_dist, out_idx, st);
  const size_t box_smem = NodeCache<T>::bytes(h->depth) + (size_t)kBoxThreads * (h->d + 1) * sizeof(T) +
                          2 * h->d * sizeof(T) + 32 + (size_t)h->max_leaf * h->d * sizeof(T) + 64;
  if (max_leaves < (1LL << h->depth) || box_smem > 200 * 1024)  // budgeted search: the reference's order
    return exact_dfs_launch<T, D>(h, Q, nq, K, max_leaves, mode, out_pos, out_dist, out_idx, st);
  int rc = ANNF_OK;
  ANNF_DISPATCH_KM(pick_km(K), rc = (exact_box_launch<T, D, KM>(h, Q, nq, K, mode, out_pos, out_dist, out_idx, st)));
  return rc;
}

template <typename T>
static int exact_knn(annf_handle* h, const T* Q, int nq, int K, long long max_leaves, int mode, int* out_pos,
                     T* out_dist, int* out_idx, cudaStream_t st) {
  int rc = ANNF_OK;
  ANNF_DISPATCH_D(T, h->d, rc = (exact_knn_typed<T, D>(h, Q, nq, K, max_leaves, mode, out_pos, out_dist, out_idx, st)));
  return rc;
}

template <typename T, int D>
static int rows_typed(annf_handle* h, const T* ared, int n_rows, int n_cols, int K, int propagate, cudaStream_t st) {
  TreeView<T> tv = view_of<T>(h);
  const long long nA = (long long)n_rows * n_cols;
  int* lists = h->lists.as<int>();
  if (n_rows <= 1) return ANNF_OK;
  const long long nq = nA - n_cols;
  if (propagate) {
    ANNF_ENSURE(h->nat_pos, (size_t)nq * sizeof(int2));
    const size_t smem = NodeCache<T>::bytes(h->depth);
    natural_leaf_kernel<T><<<(int)std::min<long long>(ceil_div(nq, 256), 16LL * num_sms()), 256, smem, st>>>(
        tv, ared, n_cols, nq, h->nat_pos.as<int2>());
    ANNF_CHECK_LAUNCH();
    prof_mark(h, "natural_leaf", st);
    ANNF_ENSURE(h->next_range, (size_t)h->n * sizeof(int2));
    next_range_kernel<T><<<std::min(ceil_div(h->n, 256), 16 * num_sms()), 256, 0, st>>>(
        tv, n_cols, nA, h->next_range.as<int2>(), h->status.as<unsigned>());
    ANNF_CHECK_LAUNCH();
    prof_mark(h, "next_range", st);
    const int cblocks = ceil_div((long long)n_cols * 32, 128);
    bool launched = false;
    if constexpr (sizeof(T) == 4 && D > 0) {
      if (K <= 8 && h->max_leaf <= 128) {
        const int2* nr = h->nat_pos.as<int2>();
        const int2* xr = h->next_range.as<int2>();
        const bool small_leaf = h->max_leaf <= 64;
        // two columns per CTA at <= 128 registers: 16 warps per SM, so every column of a 2048-wide
        // image (2040 warps on 152 SMs) is resident at once -- a column left for a second wave
        // would double the chain's time
        const int sblocks = ceil_div((long long)n_cols * 32, 64);
#define ANNF_CHAIN_SEL(CPLV, LMV) \
  chain_sel_kernel<D, CPLV, LMV><<<sblocks, 64, 0, st>>>(tv, ared, n_rows, n_cols, K, nr, xr, lists)
        if (K == 1) {
          if (small_leaf) ANNF_CHAIN_SEL(2, 2); else ANNF_CHAIN_SEL(4, 2);
        } else if (K <= 4) {
          if (small_leaf) ANNF_CHAIN_SEL(2, 5); else ANNF_CHAIN_SEL(4, 5);
        } else {
          if (small_leaf) ANNF_CHAIN_SEL(2, 9); else ANNF_CHAIN_SEL(4, 9);
        }
#undef ANNF_CHAIN_SEL
        launched = true;
      }
    }
    if (!launched)
      chain_kernel<T, D><<<cblocks, 128, 0, st>>>(tv, ared, n_rows, n_cols, K, h->nat_pos.as<int2>(),
                                                  h->next_range.as<int2>(), lists);
    ANNF_CHECK_LAUNCH();
    prof_mark(h, "chain", st);
  } else {
    const size_t smem = NodeCache<T>::bytes(h->depth) + 8 * kMaxDynD * sizeof(T);
    const int blocks = (int)std::min<long long>(ceil_div(nq * 32, 256), 64LL * num_sms());
    const int km = pick_km(K);
    int rc = ANNF_OK;
    ANNF_DISPATCH_KM(km, {
      cudaError_t e = cudaFuncSetAttribute(natural_knn_kernel<T, D, KM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
      if (e != cudaSuccess) rc = ANNF_ERR_CUDA;
      natural_knn_kernel<T, D, KM><<<blocks, 256, smem, st>>>(tv, ared, n_cols, nq, K, lists, nullptr);
    });
    if (rc != ANNF_OK) {
      set_error("natural_knn_kernel: cudaFuncSetAttribute failed");
      return rc;
    }
    ANNF_CHECK_LAUNCH();
    prof_mark(h, "natural_knn", st);
  }
  return ANNF_OK;
}

template <typename T>
static int rows_dispatch(annf_handle* h, const T* ared, int n_rows, int n_cols, int K, int propagate, cudaStream_t st) {
  int rc = ANNF_OK;
  ANNF_DISPATCH_D(T, h->d, rc = (rows_typed<T, D>(h, ared, n_rows, n_cols, K, propagate, st)));
  return rc;
}

template <typename T>
static int process_rows_impl(annf_handle* h, int* final_idx, PatchSrc A, PatchSrc B, const T* ared, int n_rows,
                             int n_cols, int K, int propagate, int select_best, long long max_leaves, int* knn_out,
                             float* dist_out, cudaStream_t st) {
  const long long nA = (long long)n_rows * n_cols;
  ANNF_ENSURE(h->lists, (size_t)nA * K * sizeof(int));
  prof_mark(h, "rows:begin", st);
  int rc = exact_knn<T>(h, ared, n_cols, K, max_leaves, 0, h->lists.as<int>(), nullptr, nullptr, st);
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
                         int n_rows, int n_cols, int K, int propagate, int select_best, long long max_leaves,
                         int* knn_out, float* dist_out, cudaStream_t st) {
  if (h->real_type == ANNF_REAL_F32)
    return process_rows_impl<float>(h, final_idx, A, B, static_cast<const float*>(ared), n_rows, n_cols, K, propagate,
                                    select_best, max_leaves, knn_out, dist_out, st);
  return process_rows_impl<double>(h, final_idx, A, B, static_cast<const double*>(ared), n_rows, n_cols, K, propagate,
                                   select_best, max_leaves, knn_out, dist_out, st);
}

int kneighbors_generic(annf_handle* h, const void* Q, int nq, int K, long long max_leaves, void* dist, int* idx,
                       cudaStream_t st) {
  if (h->real_type == ANNF_REAL_F32)
    return exact_knn<float>(h, static_cast<const float*>(Q), nq, K, max_leaves, 1, nullptr, static_cast<float*>(dist),
                            idx, st);
  return exact_knn<double>(h, static_cast<const double*>(Q), nq, K, max_leaves, 1, nullptr,
                           static_cast<double*>(dist), idx, st);
}

// natural-leaf top-K (tree positions) of every query, for the parallel form
template <typename T, int D>
static int natural_all_typed(annf_handle* h, const T* Q, long long nq, int K, int* out_pos, cudaStream_t st) {
  TreeView<T> tv = view_of<T>(h);
  const size_t smem = NodeCache<T>::bytes(h->depth) + 8 * kMaxDynD * sizeof(T);
  const int blocks = (int)std::min<long long>(ceil_div(nq * 32, 256), 64LL * num_sms());
  int rc = ANNF_OK;
  ANNF_DISPATCH_KM(pick_km(K), {
    cudaError_t e = cudaFuncSetAttribute(natural_knn_kernel<T, D, KM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) rc = ANNF_ERR_CUDA;
    natural_knn_kernel<T, D, KM><<<blocks, 256, smem, st>>>(tv, Q, 0, nq, K, out_pos, nullptr);
  });
  if (rc != ANNF_OK) {
    set_error("natural_knn_kernel: cudaFuncSetAttribute failed");
    return rc;
  }
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

int natural_knn_all(annf_handle* h, const void* Q, long long nq, int K, int* out_pos, cudaStream_t st) {
  int rc = ANNF_OK;
  if (h->real_type == ANNF_REAL_F32) {
    ANNF_DISPATCH_D(float, h->d, rc = (natural_all_typed<float, D>(h, static_cast<const float*>(Q), nq, K, out_pos, st)));
  } else {
    rc = natural_all_typed<double, 0>(h, static_cast<const double*>(Q), nq, K, out_pos, st);
  }
  return rc;
}

// ---------------------------------------------------------------------------------------------
// Exact kNN that allocates nothing.
//
// Some callers cannot allocate device memory at query time: a serving process whose device
// memory was reserved up front, a host application that owns all device memory through its own
// pool, or a caller running under an allocator that forbids growth. They build the tree once
// (that call allocates), and then query with this variant, whose only scratch -- the natural-leaf
// seeds of every query -- lives in one fixed array in device memory. The array is statically
// sized for kNoAllocMaxEntries query*k entries of the widest seed (a 16-byte double key and a
// 4-byte position: 5 MiB), exists on every GPU that loads the library until the process exits,
// and is shared by all calls: two calls that overlap on the GPU (different streams, no ordering)
// race on it. Nothing in it needs clearing: every entry a call reads was written earlier in the
// same call.
// ---------------------------------------------------------------------------------------------
constexpr long long kNoAllocMaxEntries = 1LL << 18;  // queries * k per call, both real types
constexpr size_t kNoAllocKeyBytes = (size_t)kNoAllocMaxEntries * sizeof(dkey);
static_assert(sizeof(dkey) >= sizeof(cand_key<float>::type), "the key region is sized by the widest key");
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocKeyBytes + (size_t)kNoAllocMaxEntries * 4];

// device address of g_noalloc_scratch per device, looked up once (a host-side stand-in, not the
// symbol itself, must be passed to kernels). Atomic slots: two host threads making their first
// call on one device both look the address up and store the same value.
static std::atomic<unsigned char*> g_noalloc_addr[64];

static int noalloc_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= 64) {
    set_error("annf_kneighbors_noalloc: device index out of range");
    return ANNF_ERR_INVALID;
  }
  unsigned char* addr = g_noalloc_addr[device].load(std::memory_order_acquire);
  if (!addr) {  // first call on this device (the device is current)
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("annf_kneighbors_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return ANNF_ERR_CUDA;
    }
    addr = static_cast<unsigned char*>(p);
    g_noalloc_addr[device].store(addr, std::memory_order_release);
  }
  *out = addr;
  return ANNF_OK;
}

template <typename T, int D>
static int noalloc_typed(annf_handle* h, unsigned char* scratch, const T* Q, int nq, int K, long long max_leaves,
                         T* dist, int* idx, cudaStream_t st) {
  using Kt = typename KeyOps<T>::K;
  TreeView<T> tv = view_of<T>(h);
  if (max_leaves < (1LL << h->depth)) {  // budgeted search needs no scratch at all
    const size_t smem = NodeCache<T>::bytes(h->depth) +
                        kDfsWarps * (kMaxDynD * sizeof(T) + 32 * sizeof(T) + 32 * sizeof(int) + 32 * sizeof(uint32_t)) + 64;
    exact_dfs_kernel<T, D><<<std::max(1, std::min(ceil_div(nq, kDfsWarps), 32 * num_sms())), 32 * kDfsWarps, smem, st>>>(
        tv, Q, nq, K, max_leaves, 1, nullptr, dist, idx);
    ANNF_CHECK_LAUNCH();
    return ANNF_OK;
  }
  static_assert(sizeof(Kt) * kNoAllocMaxEntries <= kNoAllocKeyBytes, "seed keys overrun their region");
  Kt* seed_key = reinterpret_cast<Kt*>(scratch);
  int* seed_pos = reinterpret_cast<int*>(scratch + kNoAllocKeyBytes);
  int rc = ANNF_OK;
  const size_t nsm = NodeCache<T>::bytes(h->depth) + 8 * kMaxDynD * sizeof(T);
  ANNF_DISPATCH_KM(pick_km(K), {
    natural_knn_kernel<T, D, KM><<<(int)std::min<long long>(ceil_div((long long)nq * 32, 256), 64LL * num_sms()), 256,
                                   nsm, st>>>(tv, Q, 0, nq, K, seed_pos, seed_key);
  });
  ANNF_CHECK_LAUNCH();
  const size_t ssm = NodeCache<T>::bytes(h->depth) + 8 * kMaxDynD * sizeof(T) + 64;
  exact_scan_kernel<T, D><<<std::max(1, std::min(ceil_div(nq, 8), 32 * num_sms())), 256, ssm, st>>>(
      tv, Q, nq, K, seed_key, 1, nullptr, dist, idx);
  ANNF_CHECK_LAUNCH();
  return rc;
}

int kneighbors_noalloc(annf_handle* h, const void* Q, int nq, int K, long long max_leaves, void* dist, int* idx,
                       cudaStream_t st) {
  if ((long long)nq * K > kNoAllocMaxEntries) {
    set_error("annf_kneighbors_noalloc: n_queries * k exceeds the fixed scratch of " +
              std::to_string(kNoAllocMaxEntries) + " entries; split the queries or use annf_kneighbors");
    return ANNF_ERR_INVALID;
  }
  // every shared-memory footprint used below stays under the 48 KiB default, so no launch needs
  // an attribute change; check it rather than assume it
  const size_t sz = h->real_type == ANNF_REAL_F32 ? sizeof(float) : sizeof(double);
  const int lv = h->depth < kCacheLevels ? h->depth : kCacheLevels;
  const size_t worst = (size_t)(1 << lv) * (4 + sz) + 32 + 8 * kMaxDynD * sz +
                       kDfsWarps * (32 * sz + 32 * sizeof(int) + 32 * sizeof(uint32_t)) + 64;
  if (worst > 48 * 1024) {
    set_error("annf_kneighbors_noalloc: shared-memory footprint too large for this tree");
    return ANNF_ERR_UNSUPPORTED;
  }
  unsigned char* scratch = nullptr;
  int rc = noalloc_scratch(h->device, &scratch);
  if (rc != ANNF_OK) return rc;
  if (h->real_type == ANNF_REAL_F32) {
    ANNF_DISPATCH_D(float, h->d,
                    rc = (noalloc_typed<float, D>(h, scratch, static_cast<const float*>(Q), nq, K, max_leaves,
                                                  static_cast<float*>(dist), idx, st)));
  } else {
    rc = noalloc_typed<double, 0>(h, scratch, static_cast<const double*>(Q), nq, K, max_leaves,
                                  static_cast<double*>(dist), idx, st);
  }
  return rc;
}

}  // namespace annf
