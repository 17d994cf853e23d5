// fast.cu -- the parallel NNF form (no row chain) and the exact raw-patch nearest neighbour used
// to measure distance error (sm_103a).
//
// The plain form follows the reference's row-sequential propagation (each row waits for the one
// above). This form has no such dependency: every pixel gets candidates from its natural leaf
// (tensor-core leaf distances, every point within their proven error bound re-ranked exactly in
// FP32, so the FP32 scan's k-list), from offset proposals (a learned predictor, optional), and
// from a few parallel propagation / random-search passes over its neighbours' current matches. Every candidate is verified with the exact integer raw-patch SSD,
// so the answer is always a real patch distance.
#include <algorithm>

#include "common.cuh"
#include "handle.cuh"

namespace annf {

int num_sms();

// ---------------------------------------------------------------------------------------------
// exact integer SSD between two psize x psize x c patches of two images (rows padded reads)
// ---------------------------------------------------------------------------------------------
struct Img {
  const uint8_t* p;
  int h, w, c, psize, ncols;  // ncols = w - psize + 1
  long long bytes;            // h * w * c
};

__device__ __forceinline__ unsigned ldw_at(const Img& I, long long off) { return load_word_bounded(I.p, off, I.bytes); }

__device__ __forceinline__ int patch_ssd(const Img& A, int ay, int ax, const Img& B, int by, int bx) {
  const int rowlen = A.psize * A.c;
  int s = 0;
  for (int r = 0; r < A.psize; ++r) {
    const long long ao = ((long long)(ay + r) * A.w + ax) * A.c, bo = ((long long)(by + r) * B.w + bx) * B.c;
    int e = 0;
    for (; e + 4 <= rowlen; e += 4) {
      const unsigned x = __vabsdiffu4(ldw_at(A, ao + e), ldw_at(B, bo + e));
      s = (int)__dp4a(x, x, (unsigned)s);
    }
    for (; e < rowlen; ++e) {
      const int t = (int)__ldg(A.p + ao + e) - (int)__ldg(B.p + bo + e);
      s += t * t;
    }
  }
  return s;
}

// ---------------------------------------------------------------------------------------------
// exact nearest B patch of sampled A pixels (the distance-error reference): every B patch is
// compared with 32 queries held in shared memory; best (ssd, index) per query by 64-bit atomicMin
// ---------------------------------------------------------------------------------------------
constexpr int kRawQ = 32;
constexpr int kRawMaxWords = 128;  // padded patch words (psize * ceil(psize*c/4))

template <int NW>
__global__ void __launch_bounds__(256) raw_nn_kernel(Img A, Img B, const int* __restrict__ qpix, int nq, int nb_split,
                                                     unsigned long long* __restrict__ best) {
  __shared__ unsigned sq[kRawQ][kRawMaxWords + 1];
  __shared__ unsigned long long sbest[kRawQ];
  const int rowlen = A.psize * A.c, wpr = (rowlen + 3) / 4;
  const int nw = NW > 0 ? NW : A.psize * wpr;
  const int q0 = blockIdx.x * kRawQ;
  const int nqt = min(kRawQ, nq - q0);
  for (int e = threadIdx.x; e < kRawQ * nw; e += blockDim.x) {
    const int qi = e / nw, w = e - qi * nw;
    unsigned v = 0;
    if (qi < nqt) {
      const int pix = qpix[q0 + qi];
      const int y = pix / A.ncols, x = pix - y * A.ncols;
      const int r = w / wpr, wi = w - r * wpr;
      const long long off = ((long long)(y + r) * A.w + x) * A.c + wi * 4;
      const int valid = min(4, rowlen - wi * 4);
      v = ldw_at(A, off);
      if (valid < 4) v &= (1u << (8 * valid)) - 1u;
    }
    sq[qi][w] = v;
  }
  for (int i = threadIdx.x; i < kRawQ; i += blockDim.x) sbest[i] = ~0ull;
  __syncthreads();
  const long long nb = (long long)(B.h - B.psize + 1) * B.ncols;
  const long long per = (nb + gridDim.y - 1) / gridDim.y;
  const long long b0 = blockIdx.y * per, b1 = min(nb, b0 + per);
  unsigned long long mine[kRawQ];
#pragma unroll
  for (int i = 0; i < kRawQ; ++i) mine[i] = ~0ull;
  for (long long b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
    const int by = (int)(b / B.ncols), bx = (int)(b - (long long)by * B.ncols);
    unsigned bw[NW > 0 ? NW : kRawMaxWords];
#pragma unroll
    for (int w = 0; w < (NW > 0 ? NW : kRawMaxWords); ++w) {
      if (NW == 0 && w >= nw) break;
      const int r = w / wpr, wi = w - r * wpr;
      const int valid = min(4, rowlen - wi * 4);
      unsigned v = ldw_at(B, ((long long)(by + r) * B.w + bx) * B.c + wi * 4);
      if (valid < 4) v &= (1u << (8 * valid)) - 1u;
      bw[w] = v;
    }
#pragma unroll 4
    for (int qi = 0; qi < kRawQ; ++qi) {
      unsigned s = 0;
#pragma unroll
      for (int w = 0; w < (NW > 0 ? NW : kRawMaxWords); ++w) {
        if (NW == 0 && w >= nw) break;
        const unsigned x = __vabsdiffu4(sq[qi][w], bw[w]);
        s = __dp4a(x, x, s);
      }
      const unsigned long long key = ((unsigned long long)s << 32) | (unsigned long long)b;
      mine[qi] = key < mine[qi] ? key : mine[qi];
    }
  }
#pragma unroll
  for (int qi = 0; qi < kRawQ; ++qi)
    if (qi < nqt && mine[qi] != ~0ull) atomicMin(&sbest[qi], mine[qi]);
  __syncthreads();
  for (int qi = threadIdx.x; qi < nqt; qi += blockDim.x) atomicMin(&best[q0 + qi], sbest[qi]);
}

// ---------------------------------------------------------------------------------------------
// parallel NNF: initial choice among candidates, then propagation / random-search passes
// ---------------------------------------------------------------------------------------------
struct Match {
  int* idx;  // [nA] best B index
  int* ssd;  // [nA] its exact raw SSD
};

__device__ __forceinline__ uint32_t hash3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ (c + 0x165667B1u) * 0xC2B2AE3Du;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return h;
}

// candidates: k natural-leaf neighbours (tree positions -> B indices) and n_prop proposals
__global__ void fast_init_kernel(Img A, Img B, int nA, int K, const int* __restrict__ nat_pos,
                                 const int* __restrict__ perm, const int* __restrict__ prop, int n_prop,
                                 const int* __restrict__ seed, Match out) {
  const int nb_rows = B.h - B.psize + 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nA; i += gridDim.x * blockDim.x) {
    const int y = i / A.ncols, x = i - y * A.ncols;
    int best = seed ? seed[i] : -1, bs = seed ? seed[nA + i] : 0x7fffffff;
    for (int j = 0; j < K + n_prop; ++j) {
      int b = j < K ? __ldg(perm + __ldg(nat_pos + (long long)i * K + j)) : __ldg(prop + (long long)i * n_prop + (j - K));
      if (b < 0) continue;
      const int by = b / B.ncols, bx = b - by * B.ncols;
      if (by >= nb_rows) continue;
      const int s = patch_ssd(A, y, x, B, by, bx);
      if (s < bs || (s == bs && b < best)) {
        bs = s;
        best = b;
      }
    }
    out.idx[i] = best;
    out.ssd[i] = bs;
  }
}

// one pass: the four neighbours' matches at distance 'jump', shifted to this pixel, and 'nrand'
// random offsets around the current match within 'radius'
//
// chg_in (optional): per pixel, whether its match changed in the previous pass (same jump). A
// neighbour that did not change offers the candidate this pixel already tried in that pass,
// against a best no better than the current one, so it is skipped: the result is the same as
// trying it. chg_out receives this pass's flags.
__global__ void fast_prop_kernel(Img A, Img B, int nA, int jump, int radius, int nrand, uint32_t seed, Match in,
                                 Match out, const uint8_t* __restrict__ chg_in, uint8_t* __restrict__ chg_out) {
  const int nb_rows = B.h - B.psize + 1, na_rows = nA / A.ncols;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nA; i += gridDim.x * blockDim.x) {
    const int y = i / A.ncols, x = i - y * A.ncols;
    const int start = in.idx[i];
    int best = start, bs = in.ssd[i];
    const int b0y = best / B.ncols, b0x = best - b0y * B.ncols;
    auto consider = [&](int by, int bx) {
      if (by < 0 || bx < 0 || by >= nb_rows || bx >= B.ncols) return;
      const int b = by * B.ncols + bx;
      if (b == best) return;
      const int s = patch_ssd(A, y, x, B, by, bx);
      if (s < bs || (s == bs && b < best)) {
        bs = s;
        best = b;
      }
    };
    const int dy[4] = {-1, 1, 0, 0}, dx[4] = {0, 0, -1, 1};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int ny = y + dy[t] * jump, nx = x + dx[t] * jump;
      if (ny < 0 || nx < 0 || ny >= na_rows || nx >= A.ncols) continue;
      if (chg_in && !chg_in[ny * A.ncols + nx]) continue;
      const int nb = in.idx[ny * A.ncols + nx];
      if (nb < 0) continue;
      const int nby = nb / B.ncols, nbx = nb - nby * B.ncols;
      consider(nby - dy[t] * jump, nbx - dx[t] * jump);
    }
    for (int t = 0; t < nrand && radius > 0; ++t) {
      const uint32_t r = hash3(seed, (uint32_t)i, (uint32_t)t);
      const int ox = (int)(r % (2 * radius + 1)) - radius, oy = (int)((r >> 16) % (2 * radius + 1)) - radius;
      consider(b0y + oy, b0x + ox);
    }
    out.idx[i] = best;
    out.ssd[i] = bs;
    if (chg_out) chg_out[i] = best != start;
  }
}

__global__ void fast_final_kernel(int nA, Match m, int* __restrict__ final_idx, float* __restrict__ dist_out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nA; i += gridDim.x * blockDim.x) {
    final_idx[i] = m.idx[i];
    if (dist_out) dist_out[i] = __fsqrt_rn((float)m.ssd[i]);
  }
}

// ---------------------------------------------------------------------------------------------
// the same kernels for common patch shapes (rows of RL <= 33 bytes): a patch row is three aligned
// 16-byte loads shifted into word alignment; the A patch stays in registers for all candidates,
// and a candidate's sum stops once it exceeds the current best
// ---------------------------------------------------------------------------------------------
template <int RL>
__device__ __forceinline__ void row_words(const uint8_t* __restrict__ img, long long off, long long nbytes,
                                          unsigned (&w)[(RL + 3) / 4]) {
  constexpr int NW = (RL + 3) / 4;
  static_assert(RL <= 33, "row too long for three 16-byte loads");
  const long long c0 = off & ~15LL;
  const int s = (int)(off - c0);
  if (c0 + 48 <= nbytes) {
    const uint4 q0 = __ldg(reinterpret_cast<const uint4*>(img + c0));
    const uint4 q1 = __ldg(reinterpret_cast<const uint4*>(img + c0 + 16));
    // the third 16 bytes only when the row reaches past the first 32 (lanes whose row fits skip it)
    uint4 q2 = make_uint4(0u, 0u, 0u, 0u);
    if (RL > 32 || s + RL > 32) q2 = __ldg(reinterpret_cast<const uint4*>(img + c0 + 32));
    const unsigned x[13] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, 0u};
    // w[j] = bytes s + 4j .. s + 4j + 3: pick the word pair (s >> 2) + j in two branch-free steps
    // (lanes of a warp have different alignments), then shift
    const int q = s >> 2, sh = (s & 3) * 8;
    unsigned y2[NW + 2], y1[NW + 1];
#pragma unroll
    for (int k = 0; k < NW + 2; ++k) y2[k] = (q & 2) ? x[k + 2] : x[k];
#pragma unroll
    for (int k = 0; k < NW + 1; ++k) y1[k] = (q & 1) ? y2[k + 1] : y2[k];
#pragma unroll
    for (int j = 0; j < NW; ++j) w[j] = __funnelshift_r(y1[j], y1[j + 1], sh);
  } else {  // the last bytes of the image: byte loads, all in bounds
#pragma unroll
    for (int j = 0; j < NW; ++j) {
      unsigned v = 0;
#pragma unroll
      for (int b = 0; b < 4; ++b)
        if (4 * j + b < RL) v |= (unsigned)__ldg(img + off + 4 * j + b) << (8 * b);
      w[j] = v;
    }
  }
  if (RL % 4) w[NW - 1] &= (1u << (8 * (RL % 4))) - 1u;
}

// exact SSDs of G candidate B patches (top-left rows cy, columns cx; cy < 0 marks an empty slot)
// against the A patch (y, x). Row by row, the loads of every live candidate are issued together;
// a candidate stops once its partial sum exceeds limit (its value is then > limit, so it cannot
// beat a match of distance limit).
template <int PS, int RL, int G>
__device__ __forceinline__ void ssd_group(const Img& A, int y, int x, const Img& B, const int (&cy)[G],
                                          const int (&cx)[G], int limit, int (&out)[G]) {
  constexpr int NW = (RL + 3) / 4;
  unsigned s[G];
  bool live[G];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    s[g] = 0;
    live[g] = cy[g] >= 0;
  }
#pragma unroll 1
  for (int r = 0; r < PS; ++r) {
    bool any = false;
#pragma unroll
    for (int g = 0; g < G; ++g) any |= live[g];
    if (!any) break;
    unsigned aw[NW];
    row_words<RL>(A.p, ((long long)(y + r) * A.w + x) * A.c, A.bytes, aw);
    unsigned bw[G][NW];
#pragma unroll
    for (int g = 0; g < G; ++g)
      if (live[g]) row_words<RL>(B.p, ((long long)(cy[g] + r) * B.w + cx[g]) * B.c, B.bytes, bw[g]);
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (!live[g]) continue;
#pragma unroll
      for (int j = 0; j < NW; ++j) {
        const unsigned dd = __vabsdiffu4(aw[j], bw[g][j]);
        s[g] = __dp4a(dd, dd, s[g]);
      }
      if ((int)s[g] > limit) live[g] = false;
    }
  }
#pragma unroll
  for (int g = 0; g < G; ++g) out[g] = cy[g] < 0 ? 0x7fffffff : (int)s[g];
}

// the lexicographic minimum of (distance, index): the order-independent result of trying the
// candidates one by one with "s < bs || (s == bs && b < best)"
template <int G>
__device__ __forceinline__ void take_best(const int (&cy)[G], const int (&cx)[G], const int (&ssd)[G], int ncols,
                                          int& best, int& bs) {
#pragma unroll
  for (int g = 0; g < G; ++g) {
    if (cy[g] < 0) continue;
    const int b = cy[g] * ncols + cx[g];
    if (ssd[g] < bs || (ssd[g] == bs && b < best)) {
      bs = ssd[g];
      best = b;
    }
  }
}

constexpr int kGroup = 4;  // candidates evaluated together (initial choice)

// exact SSDs of G listed candidates, each against its own pixel's A patch, read from the CTA's A
// strip in shared memory: strip row r holds image row y + r from the tile's first pixel on as
// aligned words (its first byte at offset delta_r = row start & 3 of word 0), so pixel p's patch
// row starts at byte delta_r + p * c and its words are funnel shifts of neighbouring strip words.
// A candidate stops once its partial sum exceeds lim[g] (its value is then > lim[g]).
template <int PS, int RL, int G>
__device__ __forceinline__ void ssd_jobs(const unsigned* __restrict__ strip, int sw, long long row0, long long rstep,
                                         int c, const int (&pj)[G], const Img& B, const int (&cy)[G],
                                         const int (&cx)[G], const int (&lim)[G], int (&out)[G]) {
  constexpr int NW = (RL + 3) / 4;
  constexpr unsigned kLastMask = (RL % 4) ? (1u << (8 * (RL % 4))) - 1u : 0xffffffffu;
  unsigned s[G];
  bool live[G];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    s[g] = 0;
    live[g] = cy[g] >= 0;
  }
#pragma unroll 1
  for (int r = 0; r < PS; ++r) {
    bool any = false;
#pragma unroll
    for (int g = 0; g < G; ++g) any |= live[g];
    if (!any) break;
    unsigned bw[G][NW];
#pragma unroll
    for (int g = 0; g < G; ++g)
      if (live[g]) row_words<RL>(B.p, ((long long)(cy[g] + r) * B.w + cx[g]) * B.c, B.bytes, bw[g]);
    const int delta = (int)((row0 + r * rstep) & 3);
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (!live[g]) continue;
      const int o = delta + pj[g] * c;
      const unsigned* a = strip + r * sw + (o >> 2);
      const int sh = (o & 3) * 8;
      unsigned lo = a[0];
#pragma unroll
      for (int j = 0; j < NW; ++j) {
        const unsigned hi = a[j + 1];
        unsigned aw = __funnelshift_r(lo, hi, sh);
        if (j == NW - 1) aw &= kLastMask;
        lo = hi;
        const unsigned dd = __vabsdiffu4(aw, bw[g][j]);
        s[g] = __dp4a(dd, dd, s[g]);
      }
      if ((int)s[g] > lim[g]) live[g] = false;
    }
  }
#pragma unroll
  for (int g = 0; g < G; ++g) out[g] = cy[g] < 0 ? 0x7fffffff : (int)s[g];
}

constexpr int kPropThreads = 256;
constexpr int kPropGroup = 1;  // listed candidates per thread at a time (one keeps six CTAs per SM)
constexpr int kPropSlots = 6;  // candidate slots per pixel of the listing pass: 4 neighbours + up to 2 random offsets

// words per A strip row of fast_prop_t_kernel: a tile's kPropThreads patches of psize pixels of c
// bytes from an unaligned start, plus a word of slack for the funnel shifts
__host__ __device__ __forceinline__ int prop_strip_words(int psize, int c) {
  return ((kPropThreads + psize - 1) * c + 3) / 4 + 3;
}

// dynamic shared memory of fast_prop_t_kernel: best keys, the A strip, the candidate list
static size_t prop_smem(int ps, int c, int nrand) {
  return (size_t)kPropThreads * (sizeof(unsigned long long) + (size_t)(4 + nrand) * (sizeof(int) + 1)) +
         (size_t)ps * prop_strip_words(ps, c) * sizeof(unsigned);
}

// seed (optional, [2 nA]: B index, then SSD): a match to start from, e.g. the best proposal found
// earlier; the result is the lexicographic minimum over the seed and the candidates either way
template <int PS, int RL>
__global__ void __launch_bounds__(256, 3) fast_init_t_kernel(Img A, Img B, int nA, int K, const int* __restrict__ nat_pos,
                                                          const int* __restrict__ perm, const int* __restrict__ prop,
                                                          int n_prop, const int* __restrict__ seed, Match out) {
  const int nb_rows = B.h - B.psize + 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nA; i += gridDim.x * blockDim.x) {
    const int y = i / A.ncols, x = i - y * A.ncols;
    int best = seed ? seed[i] : -1, bs = seed ? seed[nA + i] : 0x7fffffff;
    for (int j0 = 0; j0 < K + n_prop; j0 += kGroup) {
      int cy[kGroup], cx[kGroup], ssd[kGroup];
#pragma unroll
      for (int g = 0; g < kGroup; ++g) {
        const int j = j0 + g;
        cy[g] = -1;
        cx[g] = 0;
        if (j >= K + n_prop) continue;
        const int b = j < K ? __ldg(perm + __ldg(nat_pos + (long long)i * K + j))
                            : __ldg(prop + (long long)i * n_prop + (j - K));
        if (b < 0) continue;
        const int by = b / B.ncols;
        if (by >= nb_rows) continue;
        cy[g] = by;
        cx[g] = b - by * B.ncols;
      }
      ssd_group<PS, RL, kGroup>(A, y, x, B, cy, cx, bs, ssd);
      take_best<kGroup>(cy, cx, ssd, B.ncols, best, bs);
    }
    out.idx[i] = best;
    out.ssd[i] = bs;
  }
}

// one pass: the four neighbours' matches at distance 'jump', shifted to this pixel, and 'nrand'
// random offsets around the pass's starting match within 'radius'. A CTA takes a tile of up to
// kPropThreads pixels of one row: it stages the tile's A strip (the psize image rows under the
// tile, aligned words) in shared memory, and each thread lists its pixel's candidates that can
// change the result (not the starting match, not a repeat of an earlier candidate of the pixel,
// with chg_in not a neighbour whose match did not change in the previous pass: fast_prop_kernel).
// The CTA then works through the listed candidates, kPropGroup per thread at a time. The list is
// slot-major (every pixel's "up" candidate, then every "down", ..., then the random offsets), so
// the 32 candidates of a warp come from neighbouring pixels and the same direction, and their B
// rows share cache lines as they would in a thread-per-pixel pass, while no lane idles on a
// candidate it does not have. Each candidate folds (SSD, index) into its pixel's 64-bit best key
// with atomicMin: the lexicographic minimum, the same result as trying the candidates one by one.
template <int PS, int RL>
__global__ void __launch_bounds__(kPropThreads, 6) fast_prop_t_kernel(Img A, Img B, int nA, int jump, int radius,
                                                                   int nrand, uint32_t seed, Match in, Match out,
                                                                   const uint8_t* __restrict__ chg_in,
                                                                   uint8_t* __restrict__ chg_out) {
  constexpr int G = kPropGroup;
  constexpr int kWarps = kPropThreads / 32;
  extern __shared__ unsigned long long sdyn[];
  const int sw = prop_strip_words(PS, A.c);
  unsigned long long* sbest = sdyn;                                        // [kPropThreads]
  int* sjob = reinterpret_cast<int*>(sbest + kPropThreads);                // [slots * kPropThreads]
  unsigned* strip = reinterpret_cast<unsigned*>(sjob + (4 + nrand) * kPropThreads);  // [PS][sw]
  unsigned char* sjp = reinterpret_cast<unsigned char*>(strip + PS * sw);  // [slots * kPropThreads]
  __shared__ int swcnt[kPropSlots][kWarps];
  const int nb_rows = B.h - B.psize + 1, na_rows = nA / A.ncols;
  const int nr = radius > 0 ? min(nrand, kPropSlots - 4) : 0;
  const int slots = 4 + nr;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int tpr = (A.ncols + kPropThreads - 1) / kPropThreads;  // tiles per row
  const long long ntiles = (long long)na_rows * tpr;
  const long long rstep = (long long)A.w * A.c;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int y = (int)(tile / tpr), x0 = (int)(tile - (long long)y * tpr) * kPropThreads;
    const int x = x0 + threadIdx.x;
    const bool have = x < A.ncols;
    const int i = y * A.ncols + x;
    const long long row0 = ((long long)y * A.w + x0) * A.c;  // strip row 0's first byte
    // the A strip: aligned words of rows y .. y + PS - 1 from the tile's first pixel on
    for (int e = threadIdx.x; e < PS * sw; e += kPropThreads) {
      const int r = e / sw, w = e - r * sw;
      const long long a = ((row0 + r * rstep) & ~3LL) + 4LL * w;
      unsigned v = 0;
      if (a + 4 <= A.bytes) {
        v = __ldg(reinterpret_cast<const unsigned*>(A.p + a));
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (a + u < A.bytes) v |= (unsigned)__ldg(A.p + a + u) << (8 * u);
      }
      strip[e] = v;
    }
    int start = -1;
    if (have) {
      start = in.idx[i];
      sbest[threadIdx.x] = ((unsigned long long)(unsigned)in.ssd[i] << 32) | (unsigned)start;
    }
    const int b0y = start / B.ncols, b0x = start - b0y * B.ncols;
    // the candidate list: every slot's live candidates, warp counts, one scan, then slot g's
    // entries of warp w follow those of warps < w, after all entries of slots < g
    int cand[kPropSlots];
    unsigned live[kPropSlots];
#pragma unroll
    for (int g = 0; g < kPropSlots; ++g) {
      cand[g] = -1;
      if (have && g < slots) {
        int by = -1, bx = 0;
        if (g < 4) {
          const int ddy = g == 0 ? -1 : g == 1 ? 1 : 0, ddx = g == 2 ? -1 : g == 3 ? 1 : 0;
          const int ny = y + ddy * jump, nx = x + ddx * jump;
          if (ny >= 0 && nx >= 0 && ny < na_rows && nx < A.ncols && !(chg_in && !chg_in[ny * A.ncols + nx])) {
            const int nb = in.idx[ny * A.ncols + nx];
            if (nb >= 0) {
              const int nby = nb / B.ncols;
              by = nby - ddy * jump;
              bx = nb - nby * B.ncols - ddx * jump;
            }
          }
        } else {
          const uint32_t rr = hash3(seed, (uint32_t)i, (uint32_t)(g - 4));
          by = b0y + (int)((rr >> 16) % (2 * radius + 1)) - radius;
          bx = b0x + (int)(rr % (2 * radius + 1)) - radius;
        }
        if (by >= 0 && bx >= 0 && by < nb_rows && bx < B.ncols) {
          const int c = by * B.ncols + bx;
          bool repeat = c == start;
#pragma unroll
          for (int e = 0; e < g; ++e) repeat |= cand[e] == c;
          if (!repeat) cand[g] = c;
        }
      }
      live[g] = __ballot_sync(0xffffffffu, cand[g] >= 0);
      if (lane == 0 && g < slots) swcnt[g][warp] = __popc(live[g]);
    }
    __syncthreads();
    int base = 0;
#pragma unroll
    for (int g = 0; g < kPropSlots; ++g) {
      if (g >= slots) break;
      int off = base, tot = 0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        const int c = swcnt[g][w];
        off += w < warp ? c : 0;
        tot += c;
      }
      if (cand[g] >= 0) {
        const int pos = off + __popc(live[g] & lt_mask);
        sjob[pos] = cand[g];
        sjp[pos] = (unsigned char)threadIdx.x;
      }
      base += tot;
    }
    __syncthreads();
    // the listed candidates, kPropGroup per thread at a time (a warp's are consecutive entries)
    const int njob = base;
    for (int j0 = warp * 32 + lane; j0 < njob; j0 += G * kPropThreads) {
      int cy[G], cx[G], pj[G], lim[G], ssd[G];
#pragma unroll
      for (int u = 0; u < G; ++u) {
        const int j = j0 + u * kPropThreads;
        cy[u] = -1;
        cx[u] = 0;
        pj[u] = 0;
        lim[u] = 0;
        if (j < njob) {
          const int c = sjob[j];
          pj[u] = sjp[j];
          cy[u] = c / B.ncols;
          cx[u] = c - cy[u] * B.ncols;
          // the pixel's best so far (no better than its final best): a candidate whose partial
          // sum passes it cannot win
          lim[u] = (int)(*(volatile unsigned long long*)&sbest[pj[u]] >> 32);
        }
      }
      ssd_jobs<PS, RL, G>(strip, sw, row0, rstep, A.c, pj, B, cy, cx, lim, ssd);
#pragma unroll
      for (int u = 0; u < G; ++u)
        if (cy[u] >= 0 && ssd[u] <= lim[u])
          atomicMin(&sbest[pj[u]], ((unsigned long long)(unsigned)ssd[u] << 32) | (unsigned)(cy[u] * B.ncols + cx[u]));
    }
    __syncthreads();
    if (have) {
      const unsigned long long k = sbest[threadIdx.x];
      const int best = (int)(unsigned)(k & 0xffffffffu);
      out.idx[i] = best;
      out.ssd[i] = (int)(k >> 32);
      if (chg_out) chg_out[i] = best != start;
    }
    __syncthreads();
  }
}

// best of n_cand candidate B indices per A pixel by exact raw SSD (cand [nA][n_cand], -1 = none),
// as a match array seed_out [2 nA] (index, then SSD; -1 / INT_MAX where no candidate is valid)
int seed_matches(const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb, int wb, int c, int psize,
                 const int* cand, int n_cand, int* seed_out, cudaStream_t st) {
  Img A{img_a, ha, wa, c, psize, wa - psize + 1, (long long)ha * wa * c};
  Img B{img_b, hb, wb, c, psize, wb - psize + 1, (long long)hb * wb * c};
  const int nA = (ha - psize + 1) * A.ncols;
  const Match out{seed_out, seed_out + nA};
  const int blocks = (int)std::min<long long>(ceil_div(nA, 256), 32LL * num_sms());
  switch (psize * 100 + psize * c) {
    case 927: fast_init_t_kernel<9, 27><<<blocks, 256, 0, st>>>(A, B, nA, 0, nullptr, nullptr, cand, n_cand, nullptr, out); break;
    case 721: fast_init_t_kernel<7, 21><<<blocks, 256, 0, st>>>(A, B, nA, 0, nullptr, nullptr, cand, n_cand, nullptr, out); break;
    case 515: fast_init_t_kernel<5, 15><<<blocks, 256, 0, st>>>(A, B, nA, 0, nullptr, nullptr, cand, n_cand, nullptr, out); break;
    case 1133: fast_init_t_kernel<11, 33><<<blocks, 256, 0, st>>>(A, B, nA, 0, nullptr, nullptr, cand, n_cand, nullptr, out); break;
    default: fast_init_kernel<<<blocks, 256, 0, st>>>(A, B, nA, 0, nullptr, nullptr, cand, n_cand, nullptr, out);
  }
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

int fast_search(annf_handle* h, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb, int wb, int c,
                int psize, int K, const int* nat_pos, const int* prop, int n_prop, const int* seed_match, int iters,
                uint32_t seed, int rand_samples, int radius0, int* final_idx, float* dist_out, cudaStream_t st) {
  Img A{img_a, ha, wa, c, psize, wa - psize + 1, (long long)ha * wa * c};
  Img B{img_b, hb, wb, c, psize, wb - psize + 1, (long long)hb * wb * c};
  const int nA = (ha - psize + 1) * A.ncols;
  ANNF_ENSURE(h->fast_buf, (size_t)4 * nA * sizeof(int) + (size_t)2 * nA);
  int* base = h->fast_buf.as<int>();
  Match m0{base, base + nA}, m1{base + 2 * (size_t)nA, base + 3 * (size_t)nA};
  // per-pixel "match changed" flags of the previous pass and of this one (none before pass 1:
  // the initial choice tried no neighbour candidates)
  uint8_t* chg[2] = {reinterpret_cast<uint8_t*>(base + 4 * (size_t)nA),
                     reinterpret_cast<uint8_t*>(base + 4 * (size_t)nA) + nA};
  const int blocks = (int)std::min<long long>(ceil_div(nA, 256), 32LL * num_sms());
  // shape-specialised kernels for the common patches, the generic ones otherwise
  const int shape = psize * 100 + psize * c;
  const bool special = shape == 927 || shape == 721 || shape == 515 || shape == 1133;
  // the listing pass holds up to kPropSlots - 4 random offsets per pixel; more go to the generic pass
  const bool listed = special && rand_samples <= kPropSlots - 4;
  const long long prop_tiles = (long long)(ha - psize + 1) * ceil_div(A.ncols, kPropThreads);
  const int prop_blocks = (int)std::min<long long>(prop_tiles, 32LL * num_sms());
#define ANNF_FAST_INIT(PS, RL) fast_init_t_kernel<PS, RL><<<blocks, 256, 0, st>>>(A, B, nA, K, nat_pos, h->perm.as<int>(), prop, n_prop, seed_match, m0)
#define ANNF_FAST_PROP(PS, RL, ...)                                                                     \
  do {                                                                                                  \
    const size_t sm = prop_smem(PS, c, rand_samples);                                    \
    ANNF_CUDA_TRY(cudaFuncSetAttribute(fast_prop_t_kernel<PS, RL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)); \
    fast_prop_t_kernel<PS, RL><<<prop_blocks, kPropThreads, sm, st>>>(__VA_ARGS__);                     \
  } while (0)
  switch (shape) {
    case 927: ANNF_FAST_INIT(9, 27); break;
    case 721: ANNF_FAST_INIT(7, 21); break;
    case 515: ANNF_FAST_INIT(5, 15); break;
    case 1133: ANNF_FAST_INIT(11, 33); break;
    default:
      fast_init_kernel<<<blocks, 256, 0, st>>>(A, B, nA, K, nat_pos, h->perm.as<int>(), prop, n_prop, seed_match, m0);
  }
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "fast_init", st);
  for (int it = 0; it < iters; ++it) {
    const int jump = 1;
    const int radius = std::max(1, radius0 >> it);
    const uint32_t sd = seed * 7919u + (uint32_t)it;
    const uint8_t* cin = it == 0 ? nullptr : chg[(it - 1) & 1];
    uint8_t* cout = chg[it & 1];
    if (listed) {
      switch (shape) {
        case 927: ANNF_FAST_PROP(9, 27, A, B, nA, jump, radius, rand_samples, sd, m0, m1, cin, cout); break;
        case 721: ANNF_FAST_PROP(7, 21, A, B, nA, jump, radius, rand_samples, sd, m0, m1, cin, cout); break;
        case 515: ANNF_FAST_PROP(5, 15, A, B, nA, jump, radius, rand_samples, sd, m0, m1, cin, cout); break;
        default: ANNF_FAST_PROP(11, 33, A, B, nA, jump, radius, rand_samples, sd, m0, m1, cin, cout); break;
      }
    } else {
      fast_prop_kernel<<<blocks, 256, 0, st>>>(A, B, nA, jump, radius, rand_samples, sd, m0, m1, cin, cout);
    }
    ANNF_CHECK_LAUNCH();
    std::swap(m0, m1);
  }
#undef ANNF_FAST_INIT
#undef ANNF_FAST_PROP
  prof_mark(h, "fast_propagate", st);
  fast_final_kernel<<<blocks, 256, 0, st>>>(nA, m0, final_idx, dist_out);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

__global__ void fill_u64_kernel(unsigned long long* a, int n, unsigned long long v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

int raw_nn(const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb, int wb, int c, int psize,
           const int* qpix, int nq, unsigned long long* best, cudaStream_t st) {
  const int rowlen = psize * c, nw = psize * ((rowlen + 3) / 4);
  ANNF_REQUIRE(nw <= kRawMaxWords, "raw nearest neighbour: patch too large");
  Img A{img_a, ha, wa, c, psize, wa - psize + 1, (long long)ha * wa * c};
  Img B{img_b, hb, wb, c, psize, wb - psize + 1, (long long)hb * wb * c};
  fill_u64_kernel<<<ceil_div(nq, 256), 256, 0, st>>>(best, nq, ~0ull);
  ANNF_CHECK_LAUNCH();
  const int qt = ceil_div(nq, kRawQ);
  const int splits = std::max(1, (8 * num_sms()) / std::max(qt, 1));
  const dim3 grid(qt, splits);
  if (nw == 63) raw_nn_kernel<63><<<grid, 256, 0, st>>>(A, B, qpix, nq, splits, best);
  else if (nw == 42) raw_nn_kernel<42><<<grid, 256, 0, st>>>(A, B, qpix, nq, splits, best);
  else if (nw == 20) raw_nn_kernel<20><<<grid, 256, 0, st>>>(A, B, qpix, nq, splits, best);
  else if (nw == 48) raw_nn_kernel<48><<<grid, 256, 0, st>>>(A, B, qpix, nq, splits, best);
  else raw_nn_kernel<0><<<grid, 256, 0, st>>>(A, B, qpix, nq, splits, best);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

}  // namespace annf
