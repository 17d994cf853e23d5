// pca.cu -- PCA fit and patch projection on the GPU (sm_103a).
//
// Fit (annfmp/openmp/base.py:168-191 -> scikit-learn PCA, covariance_eigh solver):
//   G = X^T X and the column sums are integer sums of uint8 products, accumulated EXACTLY: on the
//   tensor cores (gram_tc.cu) where the shape fits, else with dp4a into int32 partials flushed to
//   64-bit integers (gram_kernel); the covariance is then finished in FP64 in the solver's own
//   operation order (mean = sum / n; C = G - (n*mean_i)*mean_j; C /= n-1), so C is bit-identical
//   to the CPU's. Its leading eigenvectors come from the library's FP64 subspace solver (eig.cu,
//   the default), cuSOLVER's full FP64 eigh (on request), or FP32 subspace steps with an FP64
//   Rayleigh-Ritz step (the approximate forms); they are ordered by decreasing eigenvalue and
//   signed so that each component's largest |entry| is positive (sklearn svd_flip with
//   u_based_decision=False).
// Projection (annfmp/openmp/base.py:193-200 -> X @ C^T - mean @ C^T in FP64, cast):
//   each FP64 coefficient is split into 8 signed 7-bit digits (c = 2^-E * sum_k s_k 2^-7k, exact
//   to ~2^-55 of the component's largest entry); every patch . digit-vector product is an exact
//   integer sum over the uint8 patch bytes, read straight from the image (on the tensor cores in
//   proj_tc.cu where the shape fits, else the dp4a project_kernel here); the partial sums are
//   recombined, the mean term subtracted, and the result rounded once to FP32.
#include <cusolverDn.h>

#include <algorithm>

#include "common.cuh"
#include "handle.cuh"
#include "fixed.cuh"

namespace annf {

__device__ __forceinline__ int dp4a_us(unsigned a, int b, int c) {
  int d;
  asm("dp4a.u32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ unsigned dp4a_uu(unsigned a, unsigned b, unsigned c) {
  unsigned d;
  asm("dp4a.u32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// ---------------------------------------------------------------------------------------------
// fit
// ---------------------------------------------------------------------------------------------
// XT[f][s] (feature-major, samples padded to a multiple of 4 with zeros); feature P is a row of
// ones (so that G[i][P] = column sum i and G[P][P] = n), features P+1..F-1 are zero.
__global__ void gather_subset_kernel(const uint8_t* __restrict__ img_a, int wa, const int* __restrict__ pos_a, int n_a,
                                     const uint8_t* __restrict__ img_b, int wb, const int* __restrict__ pos_b, int n_b,
                                     int c, int psize, int F, int ns_pad, uint8_t* __restrict__ XT) {
  const int P = psize * psize * c;
  const long long total = (long long)F * ns_pad;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(e / ns_pad), s = (int)(e - (long long)f * ns_pad);
    uint8_t v = 0;
    if (s < n_a + n_b) {
      if (f < P) {
        const int r = f / (psize * c), rem = f - r * psize * c;
        const int col = rem / c, ch = rem - col * c;
        if (s < n_a) {
          const int y = pos_a[2 * s], x = pos_a[2 * s + 1];
          v = img_a[((long long)(y + r) * wa + (x + col)) * c + ch];
        } else {
          const int t = s - n_a;
          const int y = pos_b[2 * t], x = pos_b[2 * t + 1];
          v = img_b[((long long)(y + r) * wb + (x + col)) * c + ch];
        }
      } else if (f == P) {
        v = 1;
      }
    }
    XT[e] = v;
  }
}

// Same contents, built 64 samples per block: whole patch rows are copied from the image into shared
// memory, then written with coalesced stores (for F <= 1024). blocked = 0: XT [F][ns_pad];
// blocked = 1: [ns_pad / 64][F][64] (each block's feature rows are contiguous 64-byte runs, the
// tensor-core Gram's read order).
constexpr int kGatherS = 64;
__global__ void __launch_bounds__(256) gather_subset_tiled_kernel(
    const uint8_t* __restrict__ img_a, int wa, const int* __restrict__ pos_a, int n_a, const uint8_t* __restrict__ img_b,
    int wb, const int* __restrict__ pos_b, int n_b, int c, int psize, int F, int ns_pad, int blocked,
    uint8_t* __restrict__ XT, unsigned* status) {
  extern __shared__ __align__(16) uint8_t sp[];  // [kGatherS][F]
  if (smem_overrun(sp, sp + (size_t)kGatherS * F, status)) return;
  const int P = psize * psize * c, rowlen = psize * c, ns = n_a + n_b;
  const int s0 = blockIdx.x * kGatherS;
  for (int task = threadIdx.x; task < kGatherS * psize; task += blockDim.x) {
    const int i = task / psize, r = task - i * psize;
    const int s = s0 + i;
    uint8_t* dst = sp + (size_t)i * F + r * rowlen;
    if (s < ns) {
      const uint8_t* src;
      if (s < n_a) {
        src = img_a + ((long long)(pos_a[2 * s] + r) * wa + pos_a[2 * s + 1]) * c;
      } else {
        const int t = s - n_a;
        src = img_b + ((long long)(pos_b[2 * t] + r) * wb + pos_b[2 * t + 1]) * c;
      }
      for (int e = 0; e < rowlen; ++e) dst[e] = src[e];
    } else {
      for (int e = 0; e < rowlen; ++e) dst[e] = 0;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < F * kGatherS; e += blockDim.x) {
    const int f = e / kGatherS, i = e - f * kGatherS;
    const int s = s0 + i;
    if (s >= ns_pad) continue;
    uint8_t v = 0;
    if (f < P) v = sp[(size_t)i * F + f];
    else if (f == P) v = s < ns ? 1 : 0;
    if (blocked)
      XT[((long long)blockIdx.x * F + f) * kGatherS + i] = v;
    else
      XT[(long long)f * ns_pad + s] = v;
  }
}

// G += XT XT^T over a sample-word range; 64x64 output tile per block, 4x4 per thread
constexpr int kGT = 64;       // output tile
constexpr int kGW = 16;       // sample words per smem stage
constexpr int kGramSplitWords = 2048;  // words per split: partials stay far below 2^32; enough blocks to fill the GPU

__global__ void __launch_bounds__(256) gram_kernel(const unsigned* __restrict__ XTw, int F, int nwords,
                                                   unsigned long long* __restrict__ G) {
  __shared__ unsigned sa[kGW][kGT + 1], sb[kGW][kGT + 1];
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (tj < ti) return;  // upper triangle of tiles only; mirrored at the end
  const int w0 = blockIdx.z * kGramSplitWords, w1 = min(nwords, w0 + kGramSplitWords);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  unsigned acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0;
  for (int w = w0; w < w1; w += kGW) {
    for (int e = threadIdx.x; e < kGW * kGT; e += blockDim.x) {
      const int ww = e % kGW, f = e / kGW;
      const int gw = w + ww;
      const int fi = ti * kGT + f, fj = tj * kGT + f;
      sa[ww][f] = (gw < w1 && fi < F) ? XTw[(long long)fi * nwords + gw] : 0u;
      sb[ww][f] = (gw < w1 && fj < F) ? XTw[(long long)fj * nwords + gw] : 0u;
    }
    __syncthreads();
#pragma unroll 4
    for (int ww = 0; ww < kGW; ++ww) {
      unsigned ra[4], rb[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) ra[a] = sa[ww][ty * 4 + a];
#pragma unroll
      for (int b = 0; b < 4; ++b) rb[b] = sb[ww][tx * 4 + b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = dp4a_uu(ra[a], rb[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int i = ti * kGT + ty * 4 + a, j = tj * kGT + tx * 4 + b;
      if (i < F && j < F && acc[a][b]) atomicAdd(&G[(long long)i * F + j], (unsigned long long)acc[a][b]);
    }
}

// covariance in FP64 exactly as the CPU solver computes it; also the mean
__global__ void cov_finish_kernel(const unsigned long long* __restrict__ G, int F, int P, double* __restrict__ C,
                                  double* __restrict__ mean) {
  const unsigned long long n_ll = G[(long long)P * F + P];
  const double n = (double)n_ll;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)P * P; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / P), j = (int)(e - (long long)i * P);
    const int a = min(i, j), b = max(i, j);
    const double g = (double)G[(long long)a * F + b];
    const double mi = __ddiv_rn((double)G[(long long)i * F + P], n);
    const double mj = __ddiv_rn((double)G[(long long)j * F + P], n);
    const double outer = __dmul_rn(__dmul_rn(n, mi), mj);
    C[e] = __ddiv_rn(__dsub_rn(g, outer), n - 1.0);
    if (i == 0) mean[j] = mj;
  }
}

// components: eigenvectors by decreasing eigenvalue, sign of the largest |entry| made positive
__global__ void flip_kernel(const double* __restrict__ V, int P, int ncomp, double* __restrict__ comps) {
  const int c = blockIdx.x;
  const double* v = V + (long long)(P - 1 - c) * P;  // column-major: eigenvector k is column k
  __shared__ double sbest[256];
  __shared__ int sidx[256];
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    const double a = fabs(v[i]);
    if (a > best || (a == best && i < bi)) {
      best = a;
      bi = i;
    }
  }
  sbest[threadIdx.x] = best;
  sidx[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) {
      const double ob = sbest[threadIdx.x + o];
      const int oi = sidx[threadIdx.x + o];
      if (ob > sbest[threadIdx.x] || (ob == sbest[threadIdx.x] && oi < sidx[threadIdx.x])) {
        sbest[threadIdx.x] = ob;
        sidx[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const double piv = v[sidx[0]];
  const double sg = piv > 0 ? 1.0 : (piv < 0 ? -1.0 : 0.0);
  for (int i = threadIdx.x; i < P; i += blockDim.x) comps[(long long)c * P + i] = __dmul_rn(v[i], sg);
}

// ---------------------------------------------------------------------------------------------
// projection
// ---------------------------------------------------------------------------------------------
constexpr int kSlices = 8;  // signed 7-bit digits per coefficient

// digits[j][k][word*4 + byte] laid out over the padded patch (row r occupies rw bytes, rw =
// round_up(psize*c, 4)), total W4 words (multiple of 4). Also scale exponent per component and
// the FP64 mean term m_j = mean . c_j.

__global__ void digits_kernel(const double* __restrict__ comps, const double* __restrict__ mean, int P, int psize,
                              int c, int rw, int W4, int8_t* __restrict__ digits, int* __restrict__ expo,
                              double* __restrict__ mproj, unsigned long long* __restrict__ mfix) {
  const int j = blockIdx.x;
  const double* cj = comps + (long long)j * P;
  __shared__ double smax[256];
  __shared__ double sm[256];
  double mx = 0.0, mm = 0.0;
  for (int i = threadIdx.x; i < P; i += blockDim.x) mx = fmax(mx, fabs(cj[i]));
  smax[threadIdx.x] = mx;
  __syncthreads();
  for (int o = blockDim.x / 2; o; o >>= 1) {
    if ((int)threadIdx.x < o) smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
    __syncthreads();
  }
  mx = smax[0];
  int E = 0;
  if (mx > 0) {
    int e2;
    frexp(mx, &e2);  // mx in [2^(e2-1), 2^e2)
    E = 6 - e2;      // mx * 2^E in [32, 64)
  }
  if (threadIdx.x == 0) expo[j] = E;
  int8_t* dj = digits + (long long)j * kSlices * W4 * 4;
  for (int e = threadIdx.x; e < W4 * 4; e += blockDim.x) {
    const int r = e / rw, within = e - r * rw;
    double v = 0.0;
    if (r < psize && within < psize * c) v = ldexp(cj[r * psize * c + within], E);
#pragma unroll
    for (int k = 0; k < kSlices; ++k) {
      const double s = rint(v);
      dj[(long long)k * W4 * 4 + e] = (int8_t)(int)s;
      v = (v - s) * 128.0;  // exact
    }
  }
  // mean term in FP64 (sequential order)
  if (threadIdx.x == 0) {
    double acc = 0.0;
    for (int i = 0; i < P; ++i) acc = __dadd_rn(acc, __dmul_rn(mean[i], cj[i]));
    mproj[j] = acc;
    const __int128 M = double_to_fixed(acc, 7 * (kSlices - 1) + E);  // the projection's fixed point
    mfix[2 * j] = (unsigned long long)M;
    mfix[2 * j + 1] = (unsigned long long)(M >> 64);
  }
  (void)sm;
  (void)mm;
}

constexpr int kPTW = 32, kPTH = 4;  // projection tile: 32 x 4 pixels, one thread per pixel

__device__ __forceinline__ unsigned load_u32_unaligned_smem(const unsigned* base_words, int byte_off) {
  const int w = byte_off >> 2, sh = (byte_off & 3) * 8;
  const unsigned lo = base_words[w], hi = base_words[w + 1];
  return sh ? __funnelshift_r(lo, hi, sh) : lo;
}

template <typename OutT, int W4>
__global__ void __launch_bounds__(kPTW * kPTH) project_kernel(const uint8_t* __restrict__ img, int H, int W, int c,
                                                               int psize, int rw, int ncomp,
                                                               const int8_t* __restrict__ digits,
                                                               const int* __restrict__ expo,
                                                               const double* __restrict__ mproj,
                                                               const unsigned long long* __restrict__ mfix,
                                                               OutT* __restrict__ out, unsigned* status) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nrows = H - psize + 1, ncols = W - psize + 1;
  const int x0 = blockIdx.x * kPTW, y0 = blockIdx.y * kPTH;
  const int tx = threadIdx.x % kPTW, ty = threadIdx.x / kPTW;
  // digits for all components
  const int dig_words = ncomp * kSlices * W4;
  int* sdig = reinterpret_cast<int*>(smem);
  for (int e = threadIdx.x; e < dig_words; e += blockDim.x) sdig[e] = reinterpret_cast<const int*>(digits)[e];
  // image region
  const int reg_rows = kPTH + psize - 1;
  const int reg_bytes = (kPTW + psize - 1) * c;
  const int reg_stride = ((reg_bytes + 7) / 4 + 1) * 4;  // bytes, word aligned, with slack
  unsigned* sreg = reinterpret_cast<unsigned*>(sdig + dig_words);
  uint8_t* sregb = reinterpret_cast<uint8_t*>(sreg);
  if (smem_overrun(smem, sregb + reg_rows * reg_stride, status)) return;
  for (int e = threadIdx.x; e < reg_rows * reg_stride; e += blockDim.x) {
    const int rr = e / reg_stride, bb = e - rr * reg_stride;
    const int gy = y0 + rr, gxb = x0 * c + bb;
    uint8_t v = 0;
    if (gy < H && bb < reg_bytes && gxb < W * c) v = img[(long long)gy * W * c + gxb];
    sregb[e] = v;
  }
  __syncthreads();
  const int x = x0 + tx, y = y0 + ty;
  if (x >= ncols || y >= nrows) return;
  // this patch's bytes, row by row, each row padded to rw bytes
  unsigned xw[W4];
  const int wpr = rw / 4;
#pragma unroll
  for (int w = 0; w < W4; ++w) {
    const int r = w / wpr, wi = w - r * wpr;
    xw[w] = (r < psize) ? load_u32_unaligned_smem(sreg, (ty + r) * reg_stride + tx * c + wi * 4) : 0u;
  }
  const long long pix = (long long)y * ncols + x;
  for (int j = 0; j < ncomp; ++j) {
    const int4* dj = reinterpret_cast<const int4*>(sdig + j * kSlices * W4);
    int slice[kSlices];
#pragma unroll
    for (int k = 0; k < kSlices; ++k) {
      int s = 0;
#pragma unroll
      for (int w = 0; w < W4; w += 4) {
        const int4 dd = dj[(k * W4 + w) / 4];
        s = dp4a_us(xw[w + 0], dd.x, s);
        s = dp4a_us(xw[w + 1], dd.y, s);
        s = dp4a_us(xw[w + 2], dd.z, s);
        s = dp4a_us(xw[w + 3], dd.w, s);
      }
      slice[k] = s;
    }
    if constexpr (sizeof(OutT) == 4) {
      // exact: X = sum_k slice_k 2^(7(7-k)) = patch.c * 2^(49+E); subtract the mean term as the same
      // fixed-point integer and round once to FP32 -- no FP64 arithmetic on this path
      __int128 X = slice[0];
#pragma unroll
      for (int k = 1; k < kSlices; ++k) X = (X << 7) + slice[k];
      const __int128 M = ((__int128)(long long)__ldg(mfix + 2 * j + 1) << 64) | (unsigned long long)__ldg(mfix + 2 * j);
      out[pix * ncomp + j] = fixed_to_float(X - M, 7 * (kSlices - 1) + __ldg(expo + j));
    } else {
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < kSlices; ++k) acc = __dadd_rn(__dmul_rn(acc, 128.0), (double)slice[k]);  // exact: < 2^53
      const double xc = ldexp(acc, -(7 * (kSlices - 1)) - __ldg(expo + j));
      out[pix * ncomp + j] = (OutT)__dsub_rn(xc, __ldg(mproj + j));
    }
  }
}

static int round_up(int a, int b) { return (a + b - 1) / b * b; }

int subspace_block(int P, int ncomp);
bool gram_tc_supported(int F, int ns_pad);
int gram_tc(const uint8_t* XT, int F, int ns_pad, unsigned long long* G, unsigned* status, cudaStream_t st);
int eig_top_subspace(annf_handle* h, const double* C, int P, int ncomp, int iters, double* comps, cudaStream_t st);
int eig_top_exact(annf_handle* h, const double* C, int P, int ncomp, double* comps, cudaStream_t st);
bool exact_supported(int P, int ncomp);
bool project_rows_exact_supported(int psize, int c, int ncomp);
int project_rows_exact(annf_handle* h, const uint8_t* img, int H, int W, int c, int psize, int ncomp,
                       const int8_t* digits, int rw, int W4, const int* expo, const unsigned long long* mfix,
                       float* out, cudaStream_t st);

// covariance (FP64, in h->cov) and mean of the sampled patches
int pca_covariance(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a,
                   const uint8_t* img_b, int hb, int wb, const int* pos_b, int n_b, int c, int psize, double* mean,
                   cudaStream_t st) {
  (void)ha;
  (void)hb;
  const int P = psize * psize * c;
  const int ns = n_a + n_b;
  ANNF_REQUIRE(ns >= 2, "annf_pca_fit: need at least two samples");
  ANNF_REQUIRE(P + 1 <= 4096, "annf_pca_fit: patch too large");
  const int F = P + 1;
  const int ns_pad = round_up(ns, 64);  // whole 64-sample blocks for the tensor-core Gram
  const int nwords = ns_pad / 4;
  ANNF_ENSURE(h->subset_t, (size_t)F * ns_pad);
  ANNF_ENSURE(h->gram, (size_t)F * F * sizeof(unsigned long long));
  ANNF_ENSURE(h->cov, (size_t)P * P * sizeof(double));
  ANNF_ENSURE(h->eigval, (size_t)P * sizeof(double));
  ANNF_ENSURE(h->solver_info, sizeof(int));
  prof_mark(h, "pca:begin", st);
  const bool tc_gram = gram_tc_supported(F, ns_pad);  // tensor cores (exact, nibble split)
  if (F <= 1024) {
    const size_t gsm = (size_t)kGatherS * F;
    ANNF_CUDA_TRY(cudaFuncSetAttribute(gather_subset_tiled_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsm));
    gather_subset_tiled_kernel<<<ceil_div(ns_pad, kGatherS), 256, gsm, st>>>(
        img_a, wa, pos_a, n_a, img_b, wb, pos_b, n_b, c, psize, F, ns_pad, tc_gram ? 1 : 0,
        h->subset_t.as<uint8_t>(), h->status.as<unsigned>());
  } else {
    gather_subset_kernel<<<std::min(ceil_div((long long)F * ns_pad, 256), 8192), 256, 0, st>>>(
        img_a, wa, pos_a, n_a, img_b, wb, pos_b, n_b, c, psize, F, ns_pad, h->subset_t.as<uint8_t>());
  }
  ANNF_CHECK_LAUNCH();
  ANNF_CUDA_TRY(cudaMemsetAsync(h->gram.p, 0, (size_t)F * F * sizeof(unsigned long long), st));
  if (tc_gram) {  // same integers as the dp4a Gram
    const int rc = gram_tc(h->subset_t.as<uint8_t>(), F, ns_pad, h->gram.as<unsigned long long>(),
                           h->status.as<unsigned>(), st);
    if (rc != ANNF_OK) return rc;
  } else {
    const int tiles = ceil_div(F, kGT);
    dim3 g(tiles, tiles, ceil_div(nwords, kGramSplitWords));
    gram_kernel<<<g, 256, 0, st>>>(reinterpret_cast<const unsigned*>(h->subset_t.p), F, nwords,
                                   h->gram.as<unsigned long long>());
    ANNF_CHECK_LAUNCH();
  }
  prof_mark(h, "pca_gram", st);
  cov_finish_kernel<<<std::min(ceil_div((long long)P * P, 256), 1024), 256, 0, st>>>(
      h->gram.as<unsigned long long>(), F, P, h->cov.as<double>(), mean);
  ANNF_CHECK_LAUNCH();
  h->cov_p = P;
  return ANNF_OK;
}

// the leading ncomp components of the covariance in h->cov (P x P): solver 0 = FP64 subspace
// iteration on all SMs with an FP64 Rayleigh-Ritz step (the drop-in form's result; the library
// solver above 40 components), solver < 0 = full FP64 eigh (cuSOLVER), solver > 0 = FP32
// subspace iteration with that many steps and an FP64 Rayleigh-Ritz step (approximate forms)
int pca_components(annf_handle* h, int P, int ncomp, int solver, double* comps, cudaStream_t st) {
  ANNF_REQUIRE(h->cov_p == P && P >= 1, "annf_pca_components: no covariance of this size on the handle");
  ANNF_REQUIRE(ncomp >= 1 && ncomp <= P, "annf_pca_fit: n_components out of range");
  if (solver > 0 && subspace_block(P, ncomp) > 0) {  // leading components only (approximate forms)
    int rc = eig_top_subspace(h, h->cov.as<double>(), P, ncomp, solver, comps, st);
    prof_mark(h, "pca_eigh", st);
    return rc;
  }
  if (solver == 0 && exact_supported(P, ncomp)) {
    int rc = eig_top_exact(h, h->cov.as<double>(), P, ncomp, comps, st);
    prof_mark(h, "pca_eigh", st);
    return rc;
  }
  if (!h->solver) {
    cusolverDnHandle_t sh;
    if (cusolverDnCreate(&sh) != CUSOLVER_STATUS_SUCCESS) {
      set_error("cusolverDnCreate failed");
      return ANNF_ERR_SOLVER;
    }
    h->solver = reinterpret_cast<cusolverDnContext*>(sh);
  }
  cusolverDnHandle_t sh = reinterpret_cast<cusolverDnHandle_t>(h->solver);
  if (cusolverDnSetStream(sh, st) != CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnSetStream failed");
    return ANNF_ERR_SOLVER;
  }
  int lwork = 0;
  if (cusolverDnDsyevd_bufferSize(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, P, h->cov.as<double>(), P,
                                  h->eigval.as<double>(), &lwork) != CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnDsyevd_bufferSize failed");
    return ANNF_ERR_SOLVER;
  }
  ANNF_ENSURE(h->solver_ws, (size_t)std::max(lwork, 1) * sizeof(double));
  if (cusolverDnDsyevd(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, P, h->cov.as<double>(), P,
                       h->eigval.as<double>(), h->solver_ws.as<double>(), lwork, h->solver_info.as<int>()) !=
      CUSOLVER_STATUS_SUCCESS) {
    set_error("cusolverDnDsyevd failed");
    return ANNF_ERR_SOLVER;
  }
  h->cov_p = 0;  // syevd left the eigenvectors in its place
  prof_mark(h, "pca_eigh", st);
  flip_kernel<<<ncomp, 256, 0, st>>>(h->cov.as<double>(), P, ncomp, comps);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

int pca_fit(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a, const uint8_t* img_b,
            int hb, int wb, const int* pos_b, int n_b, int c, int psize, int ncomp, double* comps, double* mean,
            int solver, cudaStream_t st) {
  const int P = psize * psize * c;
  ANNF_REQUIRE(ncomp >= 1 && ncomp <= P, "annf_pca_fit: n_components out of range");
  int rc = pca_covariance(h, img_a, ha, wa, pos_a, n_a, img_b, hb, wb, pos_b, n_b, c, psize, mean, st);
  if (rc != ANNF_OK) return rc;
  return pca_components(h, P, ncomp, solver, comps, st);
}

#define ANNF_W4_CASES(X) X(8) X(12) X(16) X(20) X(24) X(28) X(32) X(36) X(40) X(44) X(48) X(52) X(56) X(60) X(64)

int project(annf_handle* h, const uint8_t* img, int H, int W, int c, int psize, const double* comps,
            const double* mean, int ncomp, int real_type, void* out, cudaStream_t st) {
  const int P = psize * psize * c;
  const int rw = round_up(psize * c, 4);
  const int W4 = round_up(std::max(psize * rw / 4, 8), 4);
  ANNF_REQUIRE(W4 <= 64, "annf_project: patch rows larger than 256 bytes are not supported");
  ANNF_REQUIRE(ncomp >= 1 && ncomp <= P, "annf_project: n_components out of range");
  ANNF_ENSURE(h->digits, (size_t)ncomp * kSlices * W4 * 4 + (size_t)ncomp * sizeof(int) + 16 +
                             (size_t)ncomp * 2 * sizeof(unsigned long long));
  ANNF_ENSURE(h->meanproj, (size_t)ncomp * sizeof(double));
  prof_mark(h, "project:begin", st);
  int8_t* dig = h->digits.as<int8_t>();
  int* expo = reinterpret_cast<int*>(dig + (size_t)ncomp * kSlices * W4 * 4);
  unsigned long long* mfix = reinterpret_cast<unsigned long long*>(
      (reinterpret_cast<uintptr_t>(expo + ncomp) + 15) & ~uintptr_t(15));
  digits_kernel<<<ncomp, 256, 0, st>>>(comps, mean, P, psize, c, rw, W4, dig, expo, h->meanproj.as<double>(), mfix);
  ANNF_CHECK_LAUNCH();
  // FP32 output of images with at most 4 channels: the slice sums on the tensor cores (the same
  // integers, the same single rounding); otherwise, or when asked, the dp4a kernel below
  if (real_type == ANNF_REAL_F32 && !h->opt_int_projection && project_rows_exact_supported(psize, c, ncomp)) {
    const int rc = project_rows_exact(h, img, H, W, c, psize, ncomp, dig, rw, W4, expo, mfix, (float*)out, st);
    if (rc != ANNF_OK) return rc;
    prof_mark(h, "project", st);
    return ANNF_OK;
  }
  const int nrows = H - psize + 1, ncols = W - psize + 1;
  dim3 grid(ceil_div(ncols, kPTW), ceil_div(nrows, kPTH));
  const int reg_rows = kPTH + psize - 1;
  const int reg_bytes = (kPTW + psize - 1) * c;
  const int reg_stride = ((reg_bytes + 7) / 4 + 1) * 4;
  const size_t smem = (size_t)ncomp * kSlices * W4 * 4 + (size_t)reg_rows * reg_stride + 16;
  ANNF_REQUIRE(smem <= 200 * 1024, "annf_project: too many components for the shared-memory digit table");
#define ANNF_LAUNCH_PROJ(WV)                                                                                     \
  case WV:                                                                                                       \
    if (real_type == ANNF_REAL_F32) {                                                                            \
      ANNF_CUDA_TRY(cudaFuncSetAttribute(project_kernel<float, WV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                         (int)smem));                                                            \
      project_kernel<float, WV><<<grid, kPTW * kPTH, smem, st>>>(img, H, W, c, psize, rw, ncomp, dig, expo,       \
                                                                  h->meanproj.as<double>(), mfix, (float*)out,      \
                                                                  h->status.as<unsigned>());        \
    } else {                                                                                                     \
      ANNF_CUDA_TRY(cudaFuncSetAttribute(project_kernel<double, WV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                         (int)smem));                                                            \
      project_kernel<double, WV><<<grid, kPTW * kPTH, smem, st>>>(img, H, W, c, psize, rw, ncomp, dig, expo,      \
                                                                   h->meanproj.as<double>(), mfix, (double*)out,    \
                                                                   h->status.as<unsigned>());      \
    }                                                                                                            \
    break;
  switch (W4) {
    ANNF_W4_CASES(ANNF_LAUNCH_PROJ)
    default:
      set_error("annf_project: unsupported patch geometry");
      return ANNF_ERR_UNSUPPORTED;
  }
#undef ANNF_LAUNCH_PROJ
  ANNF_CHECK_LAUNCH();
  prof_mark(h, "project", st);
  return ANNF_OK;
}

}  // namespace annf
