// openclopt.cu -- the NNF algorithm of annfmp's GPU backend ("openclopt",
// annfmp/openclopt/src/futhark/{buildKDtree,kd-traverse,brute-force,driverKNN}.fut, orchestrated by
// annfmp/openclopt/src/base.c:fit_extern) as a mode of this library, for comparison with that
// backend: K fixed at 8, a tree of 2^(h+1) leaves of exactly ppl points (the input padded with
// +inf rows), splits at the mean of the two middle values of a stable sort, descent left on
// "<=", an exact first row by the backend's incremental-distance traversal, propagated leaves
// deduplicated against the natural leaf, "one row below" clamped to the last row, and select best
// by the squared raw-patch distance.
//
// Where the Futhark program leaves an order unspecified this mode fixes one: ties of the widest
// axis go to the lowest dimension; distances are sequential FP32 sums without contraction into
// FMA. The reduced patches are the caller's (the backend's own FP32 reduction has no specified
// summation order).
//
// Work: the tree level by level (one thread per node for the axis, a stable radix sort of every
// point by (node, coordinate) per level); the natural-leaf lists a warp per query; the exact first
// row a warp per query (the traversal state is uniform over the warp, the lanes share each leaf's
// distances); the rows a warp per column, rows in order (row y reads row y-1 of its column).
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>

#include "common.cuh"
#include "handle.cuh"

namespace annf {

int num_sms();

constexpr int kOclK = 8;               // the backend's fixed K (driverKNN.fut:13)
constexpr int kOclWarps = 4;           // warps per CTA in the query kernels
constexpr int kOclMaxPpl = 1024;       // points per leaf the shared distance buffers hold
constexpr unsigned kFull32 = 0xffffffffu;

// the float radix sort's order: sign flipped, negatives inverted (-0 < +0, +inf after all finite)
__device__ __forceinline__ uint32_t ocl_fkey(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ocl_funkey(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

struct OclTreeView {
  int m, d, h, q, ppl, mp;
  const float* pts;    // [mp*d] leaf order, +inf pads
  const int* indir;    // [mp]
  const int* dims;     // [q]
  const float* vals;   // [q]
  const int* clanc;    // [q]
  const int* o2l;      // [mp]
};

// sequential squared distance, no contraction (brute-force.fut:1-3)
__device__ __forceinline__ float ocl_sqdist(const float* __restrict__ x, const float* __restrict__ y, int d) {
  float r = 0.f;
  for (int j = 0; j < d; ++j) {
    const float z = __fsub_rn(x[j], y[j]);
    r = __fadd_rn(r, __fmul_rn(z, z));
  }
  return r;
}

// ---------------------------------------------------------------------------------------------
// tree (buildKDtree.fut:65-157)
// ---------------------------------------------------------------------------------------------
// global bounds over the unpadded points as ordered keys (buildKDtree.fut:74-77); +/-0 fold (only
// their spreads are used)
__global__ void ocl_bounds_kernel(const float* __restrict__ X, int m, int d, unsigned* __restrict__ kmin,
                                  unsigned* __restrict__ kmax) {
  for (int j = 0; j < d; ++j) {
    unsigned lo = 0xffffffffu, hi = 0u;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
      const unsigned k = ord_key(__ldg(X + i * d + j));
      lo = min(lo, k);
      hi = max(hi, k);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(kFull32, lo, o));
      hi = max(hi, __shfl_xor_sync(kFull32, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(kmin + j, lo);
      atomicMax(kmax + j, hi);
    }
  }
}

// axis and closest same-axis ancestor of every node of level lev (a thread per node): the box is
// the global bounds narrowed by the ancestors' split values on the way down (updateBounds,
// buildKDtree.fut:26-40), the axis its widest side (lowest dimension on ties), the ancestor by
// walking up (findClosestMed, buildKDtree.fut:42-51)
__global__ void ocl_axis_kernel(int lev, int d, const unsigned* __restrict__ kmin, const unsigned* __restrict__ kmax,
                                int* __restrict__ dims, const float* __restrict__ vals, int* __restrict__ clanc) {
  const int nodes = 1 << lev;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nodes) return;
  const int node = i + nodes - 1;
  float best_w = 0.f;
  int best = -1;
  for (int j = 0; j < d; ++j) {
    float lo = key_to_float(__ldg(kmin + j)), hi = key_to_float(__ldg(kmax + j));
    int anc = 0;
    for (int s = 0; s < lev; ++s) {
      const int k = lev - s - 1;
      const int child = (node + 1 - (1 << k)) >> k;
      if (dims[anc] == j) {
        const float v = vals[anc];
        if (!isinf(v)) {
          if ((child & 1) == 0) lo = v;  // right child: the split is its lower bound
          else hi = v;
        }
      }
      anc = child;
    }
    const float w = fabsf(__fsub_rn(hi, lo));
    if (best < 0 || w > best_w) {
      best_w = w;
      best = j;
    }
  }
  int pa = -1;
  for (int c = node; c != 0 && pa == -1;) {
    const int par = (c - 1) >> 1;
    if (dims[par] == best) pa = par;
    c = par;
  }
  dims[node] = best;
  clanc[node] = pa;
}

// sort keys of level lev: (node, coordinate on the node's axis); pads are +inf
__global__ void ocl_keys_kernel(int lev, int m, int d, int mp, const float* __restrict__ X, const int* __restrict__ indir,
                                const int* __restrict__ dims, unsigned long long* __restrict__ keys) {
  const int nodes = 1 << lev, ppn = mp >> lev;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < mp; p += (long long)gridDim.x * blockDim.x) {
    const int seg = (int)(p / ppn);
    const int ax = dims[seg + nodes - 1];
    const int o = indir[p];
    const float v = o < m ? __ldg(X + (long long)o * d + ax) : __int_as_float(0x7f800000);
    keys[p] = ((unsigned long long)seg << 32) | ocl_fkey(v);
  }
}

// split value of every node of level lev: the mean of the two middle sorted values
// (buildKDtree.fut:132-136)
__global__ void ocl_median_kernel(int lev, int mp, const unsigned long long* __restrict__ sorted, float* __restrict__ vals) {
  const int nodes = 1 << lev, ppn = mp >> lev;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nodes) return;
  const long long base = (long long)i * ppn, mi = ppn / 2;
  const float a = ocl_funkey((uint32_t)sorted[base + mi]), b = ocl_funkey((uint32_t)sorted[base + mi - 1]);
  vals[i + nodes - 1] = __fmul_rn(__fadd_rn(a, b), 0.5f);  // (a + b) / 2: halving is exact
}

__global__ void ocl_iota_kernel(int* __restrict__ a, int n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = (int)i;
}

// points in leaf order (pads +inf) and the leaf of every original index (driverKNN.fut:142-151)
__global__ void ocl_finish_kernel(int m, int d, int mp, int ppl, const float* __restrict__ X, const int* __restrict__ indir,
                                  float* __restrict__ pts, int* __restrict__ o2l) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < mp; p += (long long)gridDim.x * blockDim.x) {
    const int o = indir[p];
    for (int j = 0; j < d; ++j) pts[p * d + j] = o < m ? __ldg(X + (long long)o * d + j) : __int_as_float(0x7f800000);
    o2l[o] = (int)(p / ppl);
  }
}

// ---------------------------------------------------------------------------------------------
// queries
// ---------------------------------------------------------------------------------------------
// findLeaf (kd-traverse.fut:5-14)
__device__ __forceinline__ int ocl_find_leaf(const OclTreeView& t, const float* x) {
  int node = 0;
  while (node < t.q) node = (x[__ldg(t.dims + node)] <= __ldg(t.vals + node)) ? 2 * node + 1 : 2 * node + 2;
  return node - t.q;
}

// natural leaf and its list of every query (driverKNN.fut:153-172, bruteForce brute-force.fut:5-23):
// a warp per query. The sequential insertion keeps the 8 smallest (distance, offset) pairs of
// distance below FLT_MAX (a tie goes behind the entries it ties); the lanes keep their own
// sorted 8 and the warp merges them. Outputs tree positions (-1, FLT_MAX where none).
__global__ void __launch_bounds__(32 * kOclWarps) ocl_natural_kernel(OclTreeView t, const float* __restrict__ Q, int nq,
                                                                    int* __restrict__ ki, float* __restrict__ kd,
                                                                    int* __restrict__ nat) {
  __shared__ float sq[kOclWarps][128];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nw = gridDim.x * kOclWarps;
  for (int qi = blockIdx.x * kOclWarps + w; qi < nq; qi += nw) {
    __syncwarp();
    for (int j = lane; j < t.d; j += 32) sq[w][j] = Q[(long long)qi * t.d + j];
    __syncwarp();
    const int leaf = t.h < 0 ? 0 : ocl_find_leaf(t, sq[w]);
    unsigned long long lk[kOclK];
#pragma unroll
    for (int j = 0; j < kOclK; ++j) lk[j] = ~0ull;
    for (int i = lane; i < t.ppl; i += 32) {
      const float dist = ocl_sqdist(sq[w], t.pts + ((long long)leaf * t.ppl + i) * t.d, t.d);
      if (!(dist < FLT_MAX)) continue;
      unsigned long long key = ((unsigned long long)__float_as_uint(dist) << 32) | (unsigned)i;
#pragma unroll
      for (int j = 0; j < kOclK; ++j) {
        if (key < lk[j]) {
          const unsigned long long tk = lk[j];
          lk[j] = key;
          key = tk;
        }
      }
    }
    // warp merge: eight rounds of the warp-wide smallest head
    for (int r = 0; r < kOclK; ++r) {
      unsigned long long mn = lk[0];
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const unsigned long long x = __shfl_xor_sync(kFull32, mn, o);
        mn = x < mn ? x : mn;
      }
      const unsigned who = __ballot_sync(kFull32, lk[0] == mn && mn != ~0ull);
      if (who && lane == __ffs(who) - 1) {
#pragma unroll
        for (int j = 0; j < kOclK - 1; ++j) lk[j] = lk[j + 1];
        lk[kOclK - 1] = ~0ull;
      }
      if (lane == 0) {
        const bool ok = mn != ~0ull;
        ki[(long long)qi * kOclK + r] = ok ? leaf * t.ppl + (int)(mn & 0xffffffffu) : -1;
        kd[(long long)qi * kOclK + r] = ok ? __uint_as_float((uint32_t)(mn >> 32)) : FLT_MAX;
      }
    }
    if (lane == 0) nat[qi] = leaf;
  }
}

// bruteForcePar + sortPartSortedSeqs (brute-force.fut:25-66) by one warp: the leaf's distances in
// the warp's buffer, then up to 8 rounds of the smallest (lowest offset on ties) replacing the
// list's largest while smaller, then the merge of the two sorted runs (a tie takes the new entry
// first). The list (li, ld) is the same in every lane.
__device__ void ocl_brute_par(const OclTreeView& t, const float* x, int leaf, int* li, float* ld, float* sdist, int lane) {
  const int ppl = t.ppl;
  for (int i = lane; i < ppl; i += 32) sdist[i] = ocl_sqdist(x, t.pts + ((long long)leaf * ppl + i) * t.d, t.d);
  __syncwarp();
  for (int j = 0; j < kOclK; ++j) {
    float mv = __int_as_float(0x7f800000);
    int mi = ppl;
    for (int i = lane; i < ppl; i += 32) {
      const float v = sdist[i];
      if (v < mv || (v == mv && i < mi)) {
        mv = v;
        mi = i;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const float ov = __shfl_xor_sync(kFull32, mv, o);
      const int oi = __shfl_xor_sync(kFull32, mi, o);
      if (ov < mv || (ov == mv && oi < mi)) {
        mv = ov;
        mi = oi;
      }
    }
    if (!(mv < ld[kOclK - 1 - j])) break;  // uniform
    __syncwarp();
    if (lane == 0) sdist[mi] = FLT_MAX;
    __syncwarp();
    li[kOclK - 1 - j] = leaf * ppl + mi;
    ld[kOclK - 1 - j] = mv;
  }
  int si[kOclK];
  float sd[kOclK];
  int beg = 0, end = kOclK - 1;
#pragma unroll
  for (int i = 0; i < kOclK; ++i) {
    if (ld[beg] < ld[end]) {
      si[i] = li[beg];
      sd[i] = ld[beg];
      ++beg;
    } else {
      si[i] = li[end];
      sd[i] = ld[end];
      --end;
    }
  }
#pragma unroll
  for (int i = 0; i < kOclK; ++i) {
    li[i] = si[i];
    ld[i] = sd[i];
  }
  __syncwarp();
}

__device__ __forceinline__ int ocl_level(int node) { return 31 - __clz(node + 1); }
__device__ __forceinline__ int ocl_stk_get(int s, int i) { return (s >> i) & 1; }
__device__ __forceinline__ int ocl_stk_set(int s, int i, int v) { return (s & ~(1 << i)) | (v ? (1 << i) : 0); }

// getAncSameDimContrib (kd-traverse.fut:48-58)
__device__ float ocl_anc_contrib(const OclTreeView& t, float qm, int stack, int node) {
  int idx = node;
  for (int guard = 0; idx >= 0 && guard < 64; ++guard) {
    const int anc = __ldg(t.clanc + idx);
    if (anc == -1) return 0.f;
    if (!ocl_stk_get(stack, ocl_level(anc))) {
      idx = anc;
      continue;
    }
    return __fsub_rn(__ldg(t.vals + anc), qm);
  }
  return 0.f;
}

// traverseOnce (kd-traverse.fut:27-116): the next leaf to visit (q + 1: none)
__device__ int ocl_traverse_once(const OclTreeView& t, const float* x, float wnn, int last_leaf, int& stack, float& dist) {
  const int q = t.q;
  if (last_leaf >= q + 1) return q + 1;
  int node = last_leaf + q, count = t.h, rec = -1, stk = stack;
  float dd = dist;
  while (node != 0 && rec < 0) {
    const int parent = (node - 1) >> 1;
    const int second = ocl_stk_get(stk, count);
    const float qm = x[__ldg(t.dims + parent)];
    const float cur = __fsub_rn(__ldg(t.vals + parent), qm);
    const float cur2 = __fmul_rn(cur, cur);
    const float prv = ocl_anc_contrib(t, qm, stk, parent);
    const float prv2 = __fmul_rn(prv, prv);
    const float minu = fabsf(__fadd_rn(__fsub_rn(dd, cur2), prv2));
    const float plus = fabsf(__fadd_rn(__fsub_rn(dd, prv2), cur2));
    if (second) {
      node = parent;
      count -= 1;
      dd = minu;
    } else if (!(plus < wnn)) {
      node = parent;
      count -= 1;
    } else {
      const int snd = (node % 2 == 0) ? node - 1 : node + 1;
      stk = ocl_stk_set(stk, count, 1);
      node = parent;
      dd = plus;
      rec = snd;
    }
  }
  int leaf;
  if (node == 0 && rec == -1) {
    leaf = 2 * q + 1;
  } else {
    int nd = rec, c = count;
    while (nd < q) {
      c += 1;
      stk = ocl_stk_set(stk, c, 0);
      nd = (x[__ldg(t.dims + nd)] <= __ldg(t.vals + nd)) ? 2 * nd + 1 : 2 * nd + 2;
    }
    leaf = nd;
  }
  stack = stk;
  dist = dd;
  return leaf - q;
}

// exact lists of the first nq queries from their natural-leaf lists (driverKNN.fut:231-266),
// a warp per query
__global__ void __launch_bounds__(32 * kOclWarps) ocl_exact_kernel(OclTreeView t, const float* __restrict__ Q, int nq,
                                                                  const int* __restrict__ nat, int* __restrict__ ki,
                                                                  float* __restrict__ kd) {
  __shared__ float sq[kOclWarps][128];
  __shared__ float sdist[kOclWarps][kOclMaxPpl];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nleaves = t.q + 1;
  for (int qi = blockIdx.x * kOclWarps + w; qi < nq; qi += gridDim.x * kOclWarps) {
    __syncwarp();
    for (int j = lane; j < t.d; j += 32) sq[w][j] = Q[(long long)qi * t.d + j];
    __syncwarp();
    if (t.h < 0) continue;
    int li[kOclK];
    float ld[kOclK];
#pragma unroll
    for (int j = 0; j < kOclK; ++j) {
      li[j] = ki[(long long)qi * kOclK + j];
      ld[j] = kd[(long long)qi * kOclK + j];
    }
    int leaf = nat[qi], stack = 0;
    float dd = 0.f;
    for (int guard = 0; guard < nleaves + 1; ++guard) {  // every leaf is visited at most once
      leaf = ocl_traverse_once(t, sq[w], ld[kOclK - 1], leaf, stack, dd);
      if (leaf >= nleaves) break;
      ocl_brute_par(t, sq[w], leaf, li, ld, sdist[w], lane);
    }
    if (lane < kOclK) {
      ki[(long long)qi * kOclK + lane] = li[lane];
      kd[(long long)qi * kOclK + lane] = ld[lane];
    }
  }
}

// the leaf of the patch one row below (the last row clamped) of a tree position's original index
// (estimateIndex, driverKNN.fut:293-303); -1 beyond the tree's index range
__device__ __forceinline__ int ocl_estimate_leaf(const OclTreeView& t, int n_rows, int n_cols, int pos) {
  const int orig = __ldg(t.indir + pos);
  const int y = orig / n_cols, x = orig - y * n_cols;
  const int cy = y < n_rows - 1 ? y + 1 : n_rows - 1;
  const long long cand = (long long)cy * n_cols + x;
  if (cand < 0 || cand >= t.mp) return -1;
  return __ldg(t.o2l + cand);
}

// row propagation (driverKNN.fut:305-357): a warp per column, rows 1.. in order. Each list starts
// from the pixel's natural-leaf list and merges the distinct leaves (not the natural one) below
// the tree positions in the list of the pixel above, in list order.
__global__ void __launch_bounds__(32 * kOclWarps) ocl_rows_kernel(OclTreeView t, const float* __restrict__ Q,
                                                                 int n_rows, int n_cols, const int* __restrict__ nat,
                                                                 int* __restrict__ ki, float* __restrict__ kd,
                                                                 unsigned* status) {
  __shared__ float sq[kOclWarps][128];
  __shared__ float sdist[kOclWarps][kOclMaxPpl];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c = blockIdx.x * kOclWarps + w;
  if (c >= n_cols) return;
  for (int r = 1; r < n_rows; ++r) {
    const long long i = (long long)r * n_cols + c, up = i - n_cols;
    __syncwarp();
    for (int j = lane; j < t.d; j += 32) sq[w][j] = Q[i * t.d + j];
    __syncwarp();
    int u[kOclK], nu = 0;
    const int nl = nat[i];
#pragma unroll
    for (int j = 0; j < kOclK; ++j) {
      const int pos = ki[up * kOclK + j];
      if (pos < 0) continue;
      const int lf = ocl_estimate_leaf(t, n_rows, n_cols, pos);
      if (lf < 0) {
        if (lane == 0) atomicOr(status, DEV_BAD_INDEX);
        continue;
      }
      bool found = lf == nl;
      for (int z = 0; z < nu; ++z) found = found || u[z] == lf;
      if (!found) u[nu++] = lf;
    }
    int li[kOclK];
    float ld[kOclK];
#pragma unroll
    for (int j = 0; j < kOclK; ++j) {
      li[j] = ki[i * kOclK + j];
      ld[j] = kd[i * kOclK + j];
    }
    for (int z = 0; z < nu; ++z) ocl_brute_par(t, sq[w], u[z], li, ld, sdist[w], lane);
    if (lane < kOclK) {
      ki[i * kOclK + lane] = li[lane];
      kd[i * kOclK + lane] = ld[lane];
    }
    __syncwarp();
  }
}

// tree positions -> original indices, then select best (driverKNN.fut:90-133): the entry with the
// smallest exact squared raw-patch distance, the first on ties; a thread per pixel
__global__ void ocl_select_kernel(OclTreeView t, long long n, const int* __restrict__ ki, const uint8_t* __restrict__ A,
                                  int wa, const uint8_t* __restrict__ B, int wb, int ch, int psize, int n_cols,
                                  int n_cols_b, int* __restrict__ final_idx, int* __restrict__ knn_out,
                                  float* __restrict__ dist_out) {
  const int rowlen = psize * ch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ay = (int)(i / n_cols), ax = (int)(i - (long long)ay * n_cols);
    int best = -1;
    long long bd = -1;
    for (int j = 0; j < kOclK; ++j) {
      const int pos = ki[i * kOclK + j];
      const int o = pos < 0 ? -1 : __ldg(t.indir + pos);
      if (knn_out) knn_out[i * kOclK + j] = o;
      if (o < 0 || o >= t.m) continue;
      const int by = o / n_cols_b, bx = o - by * n_cols_b;
      long long s = 0;
      for (int rr = 0; rr < psize; ++rr) {
        const uint8_t* pa = A + ((long long)(ay + rr) * wa + ax) * ch;
        const uint8_t* pb = B + ((long long)(by + rr) * wb + bx) * ch;
        for (int e = 0; e < rowlen; ++e) {
          const int v = (int)__ldg(pb + e) - (int)__ldg(pa + e);
          s += v * v;
        }
      }
      if (bd < 0 || s < bd) {
        bd = s;
        best = o;
      }
    }
    final_idx[i] = best;
    if (dist_out) dist_out[i] = bd < 0 ? __int_as_float(0x7fc00000) : __fsqrt_rn((float)bd);
  }
}

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
static int ocl_closest_log2(int p) {
  if (p <= 1) return 0;
  int r = 0, x = p;
  while (x > 1) {
    x >>= 1;
    ++r;
  }
  return (p - (1 << r)) <= ((1 << (r + 1)) - p) ? r : r + 1;
}

static OclTreeView ocl_view(const annf_handle* h) {
  OclTreeView t;
  t.m = h->ocl_m;
  t.d = h->ocl_d;
  t.h = h->ocl_h;
  t.q = h->ocl_q;
  t.ppl = h->ocl_ppl;
  t.mp = h->ocl_mp;
  t.pts = h->ocl_pts.as<float>();
  t.indir = h->ocl_indir.as<int>();
  t.dims = h->ocl_dims.as<int>();
  t.vals = h->ocl_vals.as<float>();
  t.clanc = h->ocl_clanc.as<int>();
  t.o2l = h->ocl_o2l.as<int>();
  return t;
}

int ocl_build_tree(annf_handle* h, const float* X, int m, int d, int leaf_size, cudaStream_t st) {
  ANNF_REQUIRE(m >= 1 && d >= 1 && d <= 128 && leaf_size >= 1, "annf_ocl_build_tree: bad sizes");
  const int dnl = (int)(((long long)m + leaf_size - 1) / leaf_size);
  const int hp1 = ocl_closest_log2(dnl);
  int th, q, ppl, mp;
  if (hp1 <= 0) {
    th = -1;
    q = 0;
    ppl = m;
    mp = m;
  } else {
    ANNF_REQUIRE(hp1 <= 24, "annf_ocl_build_tree: too many leaves");
    const int nl = 1 << hp1;
    th = hp1 - 1;
    q = nl - 1;
    ppl = (int)(((long long)m + nl - 1) / nl);
    ANNF_REQUIRE((long long)nl * ppl <= 0x7fffffffLL, "annf_ocl_build_tree: too many points");
    mp = nl * ppl;
  }
  ANNF_REQUIRE(ppl <= kOclMaxPpl, "annf_ocl_build_tree: more than 1024 points per leaf");
  h->ocl_built = 0;
  ANNF_ENSURE(h->ocl_pts, (size_t)mp * d * sizeof(float));
  ANNF_ENSURE(h->ocl_indir, (size_t)mp * sizeof(int));
  ANNF_ENSURE(h->ocl_indir_tmp, (size_t)mp * sizeof(int));
  ANNF_ENSURE(h->ocl_dims, (size_t)std::max(q, 1) * sizeof(int));
  ANNF_ENSURE(h->ocl_vals, (size_t)std::max(q, 1) * sizeof(float));
  ANNF_ENSURE(h->ocl_clanc, (size_t)std::max(q, 1) * sizeof(int));
  ANNF_ENSURE(h->ocl_o2l, (size_t)mp * sizeof(int));
  ANNF_ENSURE(h->ocl_keys, (size_t)2 * mp * sizeof(unsigned long long));
  ANNF_ENSURE(h->ocl_bounds, (size_t)2 * d * sizeof(unsigned));
  int* indir = h->ocl_indir.as<int>();
  int* indir2 = h->ocl_indir_tmp.as<int>();
  unsigned long long* k0 = h->ocl_keys.as<unsigned long long>();
  unsigned long long* k1 = k0 + mp;
  const int g = std::min(ceil_div(mp, 256), 16 * num_sms());
  ocl_iota_kernel<<<g, 256, 0, st>>>(indir, mp);
  ANNF_CHECK_LAUNCH();
  if (q > 0) {
    unsigned* kmin = h->ocl_bounds.as<unsigned>();
    unsigned* kmax = kmin + d;
    ANNF_CUDA_TRY(cudaMemsetAsync(kmin, 0xff, (size_t)d * sizeof(unsigned), st));
    ANNF_CUDA_TRY(cudaMemsetAsync(kmax, 0, (size_t)d * sizeof(unsigned), st));
    ANNF_CUDA_TRY(cudaMemsetAsync(h->ocl_dims.p, 0xff, (size_t)q * sizeof(int), st));  // -1: not split yet
    ocl_bounds_kernel<<<std::min(ceil_div(m, 256), 4 * num_sms()), 256, 0, st>>>(X, m, d, kmin, kmax);
    ANNF_CHECK_LAUNCH();
    size_t tmp_bytes = 0;
    const int seg_bits = th + 1;  // node index within the level
    if (cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, k0, k1, indir, indir2, mp, 0, 32 + seg_bits, st) !=
        cudaSuccess) {
      set_error("annf_ocl_build_tree: sort workspace query failed");
      return ANNF_ERR_CUDA;
    }
    ANNF_ENSURE(h->ocl_sort_ws, tmp_bytes + 256);
    for (int lev = 0; lev <= th; ++lev) {
      const int nodes = 1 << lev;
      ocl_axis_kernel<<<ceil_div(nodes, 128), 128, 0, st>>>(lev, d, kmin, kmax, h->ocl_dims.as<int>(),
                                                           h->ocl_vals.as<float>(), h->ocl_clanc.as<int>());
      ANNF_CHECK_LAUNCH();
      ocl_keys_kernel<<<g, 256, 0, st>>>(lev, m, d, mp, X, indir, h->ocl_dims.as<int>(), k0);
      ANNF_CHECK_LAUNCH();
      size_t tb = tmp_bytes;
      ANNF_CUDA_TRY(cub::DeviceRadixSort::SortPairs(h->ocl_sort_ws.p, tb, k0, k1, indir, indir2, mp, 0, 32 + lev, st));
      count_launch();
      ocl_median_kernel<<<ceil_div(nodes, 128), 128, 0, st>>>(lev, mp, k1, h->ocl_vals.as<float>());
      ANNF_CHECK_LAUNCH();
      std::swap(indir, indir2);
    }
  }
  // the final order lives in h->ocl_indir
  if (indir != h->ocl_indir.as<int>()) std::swap(h->ocl_indir, h->ocl_indir_tmp);
  ocl_finish_kernel<<<g, 256, 0, st>>>(m, d, mp, ppl, X, h->ocl_indir.as<int>(), h->ocl_pts.as<float>(),
                                       h->ocl_o2l.as<int>());
  ANNF_CHECK_LAUNCH();
  h->ocl_m = m;
  h->ocl_d = d;
  h->ocl_h = th;
  h->ocl_q = q;
  h->ocl_ppl = ppl;
  h->ocl_mp = mp;
  h->ocl_built = 1;
  return ANNF_OK;
}

int ocl_rows(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb,
             int wb, int ch, int psize, const float* ared, int n_rows, int n_cols, int* knn_out, float* knn_sqdist_out,
             float* dist_out, cudaStream_t st) {
  ANNF_REQUIRE(h->ocl_built, "annf_ocl_rows: no tree (annf_ocl_build_tree)");
  ANNF_REQUIRE(n_rows >= 1 && n_cols >= 1, "annf_ocl_rows: empty grid");
  ANNF_REQUIRE(n_rows == ha - psize + 1 && n_cols == wa - psize + 1, "annf_ocl_rows: grid does not match image A");
  ANNF_REQUIRE((long long)(hb - psize + 1) * (wb - psize + 1) == h->ocl_m,
               "annf_ocl_rows: the tree is not over image B's patches");
  const OclTreeView t = ocl_view(h);
  const long long n = (long long)n_rows * n_cols;
  ANNF_ENSURE(h->ocl_ki, (size_t)n * kOclK * sizeof(int));
  ANNF_ENSURE(h->ocl_kd, (size_t)n * kOclK * sizeof(float));
  ANNF_ENSURE(h->ocl_nat, (size_t)n * sizeof(int));
  int* ki = h->ocl_ki.as<int>();
  float* kd = knn_sqdist_out ? knn_sqdist_out : h->ocl_kd.as<float>();
  int* nat = h->ocl_nat.as<int>();
  ocl_natural_kernel<<<(int)std::min<long long>(ceil_div(n, kOclWarps), 32LL * num_sms()), 32 * kOclWarps, 0, st>>>(
      t, ared, (int)n, ki, kd, nat);
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "ocl_natural", st);
  ocl_exact_kernel<<<std::max(1, ceil_div(n_cols, kOclWarps)), 32 * kOclWarps, 0, st>>>(t, ared, n_cols, nat, ki, kd);
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "ocl_first_row", st);
  if (n_rows > 1) {
    ocl_rows_kernel<<<ceil_div(n_cols, kOclWarps), 32 * kOclWarps, 0, st>>>(t, ared, n_rows, n_cols, nat, ki, kd,
                                                                            h->status.as<unsigned>());
    ANNF_CHECK_LAUNCH();
  }
  prof_mark(h, "ocl_rows", st);
  ocl_select_kernel<<<(int)std::min<long long>(ceil_div(n, 256), 16LL * num_sms()), 256, 0, st>>>(
      t, n, ki, img_a, wa, img_b, wb, ch, psize, n_cols, wb - psize + 1, final_idx, knn_out, dist_out);
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "ocl_select", st);
  return ANNF_OK;
}

}  // namespace annf
