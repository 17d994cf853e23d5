// eig.cu -- leading eigenvectors of the patch covariance by subspace iteration (sm_103a).
//
// The full FP64 eigendecomposition of the P x P covariance (P = 243 for 9x9x3 patches) costs
// milliseconds in a library solver, while the NNF only needs the top n_components. This solver:
//   1. simultaneous (subspace) iteration in FP32 on a block of b >= n_components vectors, one CTA:
//      Z = C Q, then column-scaled Cholesky-QR, `iters` times (C kept in FP32 in global memory),
//      from a random block (the first step's Cholesky-QR orthonormalises it); the last step's Q
//      goes on as is, its loss of orthogonality in FP32 being absorbed by the FP64 Gram below;
//   2. Rayleigh-Ritz in FP64 on span(Q): W = C Q, G = Q^T Q, T = Q^T W over many CTAs;
//   3. the b x b generalised problem T y = lambda G y in FP64 on one CTA: W = G^-1/2 by a short
//      binomial series when G is within FP32 rounding of the identity (the usual case; otherwise
//      Cholesky G = R^T R with W = R^-1, dropping columns with a vanishing pivot), T~ = W^T T W,
//      cyclic Jacobi on T~, and coefficients x = W y;
//   4. components = Q x, in decreasing Ritz value, each signed so that its largest |entry| is
//      positive (the sign convention of the exact solver).
// The covariance and the small eigenproblem stay in FP64; only the power steps that find the
// subspace run in FP32. Used by the approximate NNF forms; the plain form runs the FP64 iteration
// further down (subspace_exact_kernel), whose components agree with a full FP64 eigensolver.
#include <algorithm>

#include "common.cuh"
#include "handle.cuh"

namespace annf {

constexpr int kSubThreads = 1024;
constexpr int kMaxBlock = 40;  // three b x b FP64 matrices in static shared memory (<= 48 KB)

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename R>
__device__ __forceinline__ R warp_sum_r(R v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// Orthonormalise the B columns of Z ([P][B] row-major, shared memory) by Cholesky-QR, writing Q
// ([P][B]): every column is scaled to unit norm first (in subspace iteration Z = C Q has nearly
// orthogonal columns, so the scaled Gram matrix is close to the identity and FP32 Cholesky is
// stable), R^-1 is formed explicitly by one warp, and Q = Z D R^-1 is a small product (a row per
// thread). A column whose norm vanishes is replaced by a basis vector. G, Ri: B x B shared
// scratch; d: B shared column scales. Q's contents on entry are overwritten (used as scratch).
template <int B>
__device__ void cholqr_rows(float* Z, float* Q, int P, float* G, float* Ri, float* d) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  // column norms; vanishing columns become basis vectors
  for (int j = warp; j < B; j += nt >> 5) {
    float sq = 0.f;
    for (int i = lane; i < P; i += 32) sq = fmaf(Z[i * B + j], Z[i * B + j], sq);
    sq = warp_sum_f(sq);
    if (!(sq > 1e-30f)) {
      for (int i = lane; i < P; i += 32) Z[i * B + j] = i == (j * 7 + 3) % P ? 1.f : 0.f;
      sq = 1.f;
    }
    if (lane == 0) d[j] = rsqrtf(sq);
  }
  __syncthreads();
  // scaled Gram matrix (upper triangle): a thread per entry and part of the rows (three parts
  // when the rows allow), the partial sums kept in Q (its old contents are dead here) and added
  // in a fixed order
  constexpr int kUpper = B * (B + 1) / 2;
  const int parts = (P >= 3 * B && 3 * kUpper <= nt) ? 3 : 1;
  const int rows = (P + parts - 1) / parts;
  for (int e = tid; e < parts * kUpper; e += nt) {
    const int s = e / kUpper;
    int r = 0, t = e - s * kUpper;
    while (t >= B - r) {
      t -= B - r;
      ++r;
    }
    const int c = r + t;
    float g = 0.f;
    const int i1 = min(P, (s + 1) * rows);
    for (int i = s * rows; i < i1; ++i) g = fmaf(Z[i * B + r], Z[i * B + c], g);
    Q[s * B * B + r * B + c] = g;
  }
  __syncthreads();
  for (int e = tid; e < B * B; e += nt) {
    const int r = e / B, c = e - r * B;
    if (c < r) continue;
    const float g = parts == 3 ? (Q[e] + Q[B * B + e]) + Q[2 * B * B + e] : Q[e];
    G[e] = g * d[r] * d[c];
  }
  __syncthreads();
  if (warp == 0) {
    // Cholesky G = R^T R (upper R in place), lanes over columns
    for (int k = 0; k < B; ++k) {
      const float piv = G[k * B + k];
      const float r = piv > 1e-12f ? sqrtf(piv) : 0.f;
      __syncwarp();
      for (int j = k + lane; j < B; j += 32) G[k * B + j] = r > 0.f ? (j == k ? r : G[k * B + j] / r) : (j == k ? 1.f : 0.f);
      __syncwarp();
      // row k of R in registers first: the column updates then have no load that waits on an
      // earlier store
      float row[B];
#pragma unroll
      for (int u = 0; u < B; ++u) row[u] = k + 1 + u < B ? G[k * B + k + 1 + u] : 0.f;
      for (int j = k + 1 + lane; j < B; j += 32) {
        const float rkj = G[k * B + j];
#pragma unroll
        for (int u = 0; u < B - 1; ++u) {
          const int i = k + 1 + u;
          if (i <= j) G[i * B + j] = fmaf(-row[u], rkj, G[i * B + j]);
        }
      }
      __syncwarp();
    }
    // R^-1 (upper), lanes over columns: back substitution of R x = e_j with the column in
    // registers; each sum runs from the oldest entry of x to the newest, so only its last term
    // waits on the previous step
    for (int j = lane; j < B; j += 32) {
      float x[B];
#pragma unroll
      for (int ii = 0; ii < B; ++ii) {
        const int i = B - 1 - ii;
        float v = i == j ? 1.f : 0.f;
#pragma unroll
        for (int t = B - 1; t > i; --t) v = fmaf(-G[i * B + t], x[t], v);  // x[t] = 0 beyond j
        x[i] = i <= j ? v / G[i * B + i] : 0.f;
      }
#pragma unroll
      for (int i = 0; i < B; ++i) Ri[i * B + j] = x[i];
    }
  }
  __syncthreads();
  // Q = Z D R^-1 (R^-1 upper: column j uses t <= j, summed in increasing t)
  if constexpr (B <= 24) {
    // a row per thread, its outputs in registers: R^-1 is read as broadcasts, and no lane idles
    // on a shorter column than its neighbours'
    for (int i = tid; i < P; i += nt) {
      float q[B];
#pragma unroll
      for (int j = 0; j < B; ++j) q[j] = 0.f;
#pragma unroll
      for (int t = 0; t < B; ++t) {
        const float zt = Z[i * B + t] * d[t];
#pragma unroll
        for (int j = t; j < B; ++j) q[j] = fmaf(zt, Ri[t * B + j], q[j]);
      }
#pragma unroll
      for (int j = 0; j < B; ++j) Q[i * B + j] = q[j];
    }
  } else {
    for (int e = tid; e < P * B; e += nt) {
      const int i = e / B, j = e - i * B;
      float q = 0.f;
      for (int t = 0; t <= j; ++t) q = fmaf(Z[i * B + t] * d[t], Ri[t * B + j], q);
      Q[e] = q;
    }
  }
  __syncthreads();
}

// step 1: one CTA. Z = C Q in FP32 with C (FP32 copy C32, global) read once per step: item
// (i, s) accumulates row i over the s-th of KS slices of k into registers, the KS partial rows
// are summed in a fixed order (deterministic), then Cholesky-QR. Qout [B][P] FP32. (Each
// Cholesky-QR is a chain of dependent steps on one warp, ~33 us at b = 24: it runs once per step.)
template <int B>
__global__ void __launch_bounds__(kSubThreads) subspace_iter_kernel(const double* __restrict__ C, int P, int KS,
                                                                    int iters, float* C32, float* __restrict__ Qout,
                                                                    unsigned* status) {
  extern __shared__ __align__(16) float sm[];
  float* Q = sm;                        // [P][B]
  float* Z = Q + (size_t)P * B;         // [P][B]
  float* part = Z + (size_t)P * B;      // [KS][P][B]
  float* G = part + (size_t)KS * P * B;  // [B][B]
  float* Ri = G + B * B;                 // [B][B]
  float* dsc = Ri + B * B;               // [B]
  if (smem_overrun(sm, dsc + B, status)) return;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (long long e = tid; e < (long long)P * P; e += nt) C32[e] = (float)C[e];
  for (int e = tid; e < B * P; e += nt) {
    const int i = e / B, j = e - i * B;
    Q[e] = (float)(mix32((uint32_t)(j * P + i) * 2654435761u + 12345u) >> 8) * (1.0f / 16777216.0f) - 0.5f;
  }
  __syncthreads();
  const int kper = (P + KS - 1) / KS;
  for (int it = 0; it < iters; ++it) {
    __threadfence_block();
    for (int item = tid; item < P * KS; item += nt) {
      const int s = item / P, i = item - s * P;  // consecutive threads: consecutive rows i
      const int k0 = s * kper, k1 = min(P, k0 + kper);
      float acc[B];
#pragma unroll
      for (int c = 0; c < B; ++c) acc[c] = 0.f;
#pragma unroll 4
      for (int k = k0; k < k1; ++k) {
        const float cv = __ldcg(C32 + (size_t)k * P + i);  // C symmetric: row k read along i
        const float4* q4 = reinterpret_cast<const float4*>(Q + (size_t)k * B);
#pragma unroll
        for (int c4 = 0; c4 < B / 4; ++c4) {
          const float4 q = q4[c4];
          acc[4 * c4] = fmaf(cv, q.x, acc[4 * c4]);
          acc[4 * c4 + 1] = fmaf(cv, q.y, acc[4 * c4 + 1]);
          acc[4 * c4 + 2] = fmaf(cv, q.z, acc[4 * c4 + 2]);
          acc[4 * c4 + 3] = fmaf(cv, q.w, acc[4 * c4 + 3]);
        }
      }
      float4* dst = reinterpret_cast<float4*>(part + ((size_t)s * P + i) * B);
#pragma unroll
      for (int c4 = 0; c4 < B / 4; ++c4)
        dst[c4] = make_float4(acc[4 * c4], acc[4 * c4 + 1], acc[4 * c4 + 2], acc[4 * c4 + 3]);
    }
    __syncthreads();
    for (int e = tid; e < P * B; e += nt) {
      float z = part[e];
      for (int s = 1; s < KS; ++s) z += part[(size_t)s * P * B + e];
      Z[e] = z;
    }
    __syncthreads();
    cholqr_rows<B>(Z, Q, P, G, Ri, dsc);
  }
  for (int e = tid; e < B * P; e += nt) {
    const int j = e / P, i = e - j * P;
    Qout[e] = Q[i * B + j];
  }
}

// step 2a: W[j][i] = sum_k C[i][k] Q[j][k] in FP64, one warp per (j, i)
__global__ void rr_cq_kernel(const double* __restrict__ C, int P, int b, const float* __restrict__ Q,
                             double* __restrict__ W) {
  const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= (long long)b * P) return;
  const int j = (int)(wid / P), i = (int)(wid - (long long)j * P);
  const double* c = C + (size_t)i * P;
  const float* q = Q + (size_t)j * P;
  double s = 0.0;
  for (int k = lane; k < P; k += 32) s = fma(c[k], (double)q[k], s);
  s = warp_sum_d(s);
  if (lane == 0) W[(size_t)j * P + i] = s;
}

// step 2b: G = Q^T Q and T = Q^T W (b x b, FP64), one warp per entry
__global__ void rr_gram_kernel(int P, int b, const float* __restrict__ Q, const double* __restrict__ W,
                               double* __restrict__ G, double* __restrict__ T) {
  const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= 2LL * b * b) return;
  const int which = (int)(wid / (b * b)), e = (int)(wid - (long long)which * b * b);
  const int i = e / b, j = e - i * b;
  const float* qi = Q + (size_t)i * P;
  double s = 0.0;
  if (which == 0) {
    const float* qj = Q + (size_t)j * P;
    for (int k = lane; k < P; k += 32) s = fma((double)qi[k], (double)qj[k], s);
  } else {
    const double* wj = W + (size_t)j * P;
    for (int k = lane; k < P; k += 32) s = fma((double)qi[k], wj[k], s);
  }
  s = warp_sum_d(s);
  if (lane == 0) (which == 0 ? G : T)[e] = s;
}

// Cyclic Jacobi on the symmetric m x m matrix T (row-major, shared), accumulating rotations into
// V (T <- J^T T J, V <- V J), round-robin ordering: each round rotates M/2 disjoint pairs at once
// (M = m rounded up to even; a pair with the phantom index M-1 >= m is skipped). Rotation angles
// are computed by one thread per pair from the matrix before the round, then all row updates,
// then all column updates (disjoint rotations commute). Sweeps stop once the off-diagonal square
// sum is at most tol times the total. FP64: the rotation's tangent is computed in FP32 and cos by
// Newton steps on rsqrt (exactly orthogonal in FP64; an FP32 angle leaves ~1e-7 of apq, removed
// by the next sweep), so the loop has no FP64 division or square root.
template <typename R>
__device__ void jacobi_sweeps(R* T, R* V, int m, int max_sweeps, double tol, R* s_cs, R* s_sn, int* s_p, int* s_q,
                              R* s_off, R* s_tot) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const int M = (m + 1) & ~1, half = M / 2;
  for (int sweep = 0; sweep < max_sweeps && m > 1; ++sweep) {
    if (tid < 32) {
      R off = 0, tot = 0;
      for (int e = tid; e < m * m; e += 32) {
        const R v = T[e] * T[e];
        tot += v;
        if (e / m != e % m) off += v;
      }
      off = warp_sum_r(off);
      tot = warp_sum_r(tot);
      if (tid == 0) {
        *s_off = off;
        *s_tot = tot;
      }
    }
    __syncthreads();
    if (!(*s_off > (R)tol * *s_tot)) break;
    for (int round = 0; round < M - 1; ++round) {
      if (tid < half) {
        auto player = [&](int j) {  // 1 + (j - 1 + round) mod (M - 1), both terms below M - 1
          const int x = j - 1 + round;
          return j == 0 ? 0 : 1 + (x >= M - 1 ? x - (M - 1) : x);
        };
        int p = player(tid), q = player(M - 1 - tid);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        R cs = 1, sn = 0;
        if (q < m) {
          const R apq = T[p * m + q], app = T[p * m + p], aqq = T[q * m + q];
          if (sizeof(R) == 8) {
            if (fabs((double)apq) > 1e-300 && fabs((double)apq) * fabs((double)apq) > 1e-30 * fabs((double)app * aqq)) {
              const float theta = (float)(((double)aqq - app) / (2.0 * apq));
              const float tf = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(fmaf(theta, theta, 1.f)));
              const double t = (double)tf, x = fma(t, t, 1.0);
              double y = (double)rsqrtf((float)x);
              y = y * fma(-0.5 * x, y * y, 1.5);
              y = y * fma(-0.5 * x, y * y, 1.5);
              cs = y;
              sn = t * y;
            }
          } else {
            const float fa = (float)apq;
            if (fabsf(fa) > 1e-30f && fabsf(fa) * fabsf(fa) > 1e-14f * fabsf((float)app * (float)aqq)) {
              // approximate quotients are enough here: the rotation stays orthogonal (c, s from
              // one t), and the FP64 sweeps that follow correct the angles
              const float theta = __fdividef((float)aqq - (float)app, 2.f * fa);
              const float t = __fdividef(theta >= 0.f ? 1.f : -1.f, fabsf(theta) + sqrtf(fmaf(theta, theta, 1.f)));
              const float c = rsqrtf(fmaf(t, t, 1.f));
              cs = c;
              sn = t * c;
            }
          }
        }
        s_p[tid] = p;
        s_q[tid] = q < m ? q : -1;
        s_cs[tid] = cs;
        s_sn[tid] = sn;
      }
      __syncthreads();
      for (int i = warp; i < half; i += nw) {  // rows p, q: a warp per pair, lanes over the columns
        const int p = s_p[i], q = s_q[i];
        const R cs = s_cs[i], sn = s_sn[i];
        if (q < 0 || sn == (R)0) continue;
        for (int k = lane; k < m; k += 32) {
          const R tp = T[p * m + k], tq = T[q * m + k];
          T[p * m + k] = cs * tp - sn * tq;
          T[q * m + k] = sn * tp + cs * tq;
        }
      }
      __syncthreads();
      for (int i = warp; i < half; i += nw) {  // columns p, q and the eigenvectors
        const int p = s_p[i], q = s_q[i];
        const R cs = s_cs[i], sn = s_sn[i];
        if (q < 0 || sn == (R)0) continue;
        for (int k = lane; k < m; k += 32) {
          const R tp = T[k * m + p], tq = T[k * m + q];
          T[k * m + p] = cs * tp - sn * tq;
          T[k * m + q] = sn * tp + cs * tq;
          const R vp = V[k * m + p], vq = V[k * m + q];
          V[k * m + p] = cs * vp - sn * vq;
          V[k * m + q] = sn * vp + cs * vq;
        }
      }
      __syncthreads();
    }
  }
}

// step 3: one CTA, FP64. Writes X [ncomp][b] (coefficients of each component in the Q basis).
constexpr int kRrThreads = 256;  // rr_solve_kernel's block: its register arrays assume it
constexpr double kNearIdentity = 2e-5;  // largest |G - I| entry for the series path

__global__ void __launch_bounds__(kRrThreads) rr_solve_kernel(int b, int ncomp, const double* __restrict__ Gg,
                                                       const double* __restrict__ Tg, double* __restrict__ Xout,
                                                       double* __restrict__ lambda_out) {
  __shared__ double G[kMaxBlock * kMaxBlock], T[kMaxBlock * kMaxBlock], V[kMaxBlock * kMaxBlock];
  __shared__ double lam[kMaxBlock];
  __shared__ int keep[kMaxBlock], order[kMaxBlock];
  __shared__ int s_m;
  __shared__ double s_off, s_tot;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < b * b; e += nt) {
    const int i = e / b, j = e - i * b;
    G[e] = 0.5 * (Gg[i * b + j] + Gg[j * b + i]);
    T[e] = 0.5 * (Tg[i * b + j] + Tg[j * b + i]);
  }
  __syncthreads();
  // G = Q^T Q is within FP32 rounding of the identity when Q comes out of Cholesky-QR. Then
  // W = G^-1/2 comes from the binomial series of (I + E)^-1/2, E = G - I, to the E^4 term (with
  // max |E_ij| <= kNearIdentity the first term left out is below FP64 rounding), T~ = W T W and
  // x = W y: products that all threads share, in place of a serial Cholesky and triangular
  // solves. Otherwise (a degenerate block) Cholesky, dropping the columns with vanishing pivots.
  __shared__ int s_near;
  if (tid < 32) {
    double e = 0.0;
    for (int idx = tid; idx < b * b; idx += 32) e = fmax(e, fabs(G[idx] - (idx / b == idx % b ? 1.0 : 0.0)));
#pragma unroll
    for (int o = 16; o; o >>= 1) e = fmax(e, __shfl_xor_sync(0xffffffffu, e, o));
    if (tid == 0) s_near = e <= kNearIdentity;
  }
  __syncthreads();
  const bool near_identity = s_near != 0;
  int m;
  if (near_identity) {
    m = b;
    for (int k = tid; k < b; k += nt) keep[k] = k;
    constexpr double kC[5] = {1.0, 0.5, 0.375, 0.3125, 0.2734375};  // binom(2n, n) / 4^n
    // G <- F = I - G; V <- S = c4 I; then S <- c_n I + F S for n = 3, 2, 1, 0 (the last is W)
    for (int e = tid; e < b * b; e += nt) {
      const bool dg = e / b == e % b;
      G[e] = (dg ? 1.0 : 0.0) - G[e];
      V[e] = dg ? kC[4] : 0.0;
    }
    __syncthreads();
    double acc[(kMaxBlock * kMaxBlock + kRrThreads - 1) / kRrThreads];
    for (int n = 3; n >= 0; --n) {
      int u = 0;
      for (int e = tid; e < b * b; e += nt) {
        const int i = e / b, j = e - i * b;
        double a = i == j ? kC[n] : 0.0;
        for (int k = 0; k < b; ++k) a = fma(G[i * b + k], V[k * b + j], a);
        acc[u++] = a;
      }
      __syncthreads();
      u = 0;
      for (int e = tid; e < b * b; e += nt) V[e] = acc[u++];
      __syncthreads();
    }
    for (int e = tid; e < b * b; e += nt) G[e] = V[e];  // G <- W (x = W y at the end)
    __syncthreads();
    // T~ = W T W into V (where the other path leaves it): Y = T W, then W Y
    int u = 0;
    for (int e = tid; e < b * b; e += nt) {
      const int i = e / b, j = e - i * b;
      double a = 0.0;
      for (int k = 0; k < b; ++k) a = fma(T[i * b + k], G[k * b + j], a);
      acc[u++] = a;
    }
    __syncthreads();
    u = 0;
    for (int e = tid; e < b * b; e += nt) V[e] = acc[u++];
    __syncthreads();
    u = 0;
    for (int e = tid; e < b * b; e += nt) {
      const int i = e / b, j = e - i * b;
      double a = 0.0;
      for (int k = 0; k < b; ++k) a = fma(G[k * b + i], V[k * b + j], a);  // W symmetric
      acc[u++] = a;
    }
    __syncthreads();
    u = 0;
    for (int e = tid; e < b * b; e += nt) V[e] = acc[u++];
    __syncthreads();
  } else {
    // Cholesky G = R^T R in place, right-looking (upper triangle holds R; the trailing block is
    // updated by all threads); vanishing pivots drop their column
    __shared__ double s_gmax, s_piv;
    if (tid == 0) {
      double gmax = 0.0;
      for (int i = 0; i < b; ++i) gmax = fmax(gmax, G[i * b + i]);
      s_gmax = gmax;
      s_m = 0;
    }
    __syncthreads();
    for (int k = 0; k < b; ++k) {
      if (tid == 0) {
        const double piv = G[k * b + k];
        const bool ok = piv > 1e-10 * s_gmax && piv > 0.0;
        keep[k] = ok ? s_m++ : -1;
        s_piv = ok ? sqrt(piv) : 0.0;
      }
      __syncthreads();
      const double r = s_piv;
      for (int j = k + tid; j < b; j += nt) G[k * b + j] = r > 0.0 ? (j == k ? r : G[k * b + j] / r) : 0.0;
      __syncthreads();
      if (r > 0.0) {
        const int tw = b - k - 1;
        for (int e = tid; e < tw * tw; e += nt) {
          const int i = k + 1 + e / tw, j = k + 1 + e % tw;
          if (j >= i) G[i * b + j] -= G[k * b + i] * G[k * b + j];
        }
      }
      __syncthreads();
    }
    m = s_m;
    // compact the kept columns: R~ (m x m upper), T (m x m); V <- T restricted
    // (kept column k maps to keep[k]); reuse V as scratch for the compacted T
    for (int e = tid; e < b * b; e += nt) {
      const int i = e / b, j = e - i * b;
      if (keep[i] >= 0 && keep[j] >= 0) V[keep[i] * m + keep[j]] = T[e];
    }
    __syncthreads();
    for (int e = tid; e < b * b; e += nt) {
      const int i = e / b, j = e - i * b;
      if (keep[i] >= 0 && keep[j] >= 0) T[keep[i] * m + keep[j]] = (j >= i) ? G[e] : 0.0;  // T now holds R~
    }
    __syncthreads();
    for (int e = tid; e < m * m; e += nt) G[e] = T[e];  // G = R~ (m x m, upper)
    __syncthreads();
    // X = R~^-T Tm : forward substitution per column (R~^T lower)
    for (int c = tid; c < m; c += nt) {
      for (int i = 0; i < m; ++i) {
        double v = V[i * m + c];
        for (int t = 0; t < i; ++t) v -= G[t * m + i] * T[t * m + c];
        T[i * m + c] = v / G[i * m + i];
      }
    }
    __syncthreads();
    // T~ = X R~^-1 : solve T~ R~ = X row by row
    for (int r = tid; r < m; r += nt) {
      for (int j = 0; j < m; ++j) {
        double v = T[r * m + j];
        for (int t = 0; t < j; ++t) v -= V[r * m + t] * G[t * m + j];
        V[r * m + j] = v / G[j * m + j];
      }
    }
    __syncthreads();
  }
  // symmetrise into T, V = I
  for (int e = tid; e < m * m; e += nt) {
    const int i = e / m, j = e - i * m;
    T[e] = 0.5 * (V[i * m + j] + V[j * m + i]);
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) V[e] = (e / m == e % m) ? 1.0 : 0.0;
  __syncthreads();
  // Jacobi in two precisions. FP32 sweeps (cheap on this part) bring T to diagonal within FP32
  // rounding; one Newton-Schulz step makes their eigenvectors orthonormal in FP64; M = V^T T V is
  // then diagonal to ~1e-7 of its norm, and FP64 sweeps on M (quadratic convergence: one or two)
  // finish the small eigenproblem in FP64, accumulating into V.
  __shared__ double s_cs[kMaxBlock / 2], s_sn[kMaxBlock / 2];
  __shared__ float f_cs[kMaxBlock / 2], f_sn[kMaxBlock / 2], f_off, f_tot;  // the FP32 sweeps' own scratch
  __shared__ int s_p[kMaxBlock / 2], s_q[kMaxBlock / 2];
  float* V32 = reinterpret_cast<float*>(V);  // FP32 phase: V32 and T32 share V's storage
  float* T32 = V32 + kMaxBlock * kMaxBlock;
  for (int e = tid; e < m * m; e += nt) {
    T32[e] = (float)T[e];
    V32[e] = (e / m == e % m) ? 1.f : 0.f;
  }
  __syncthreads();
  jacobi_sweeps<float>(T32, V32, m, 16, 1e-12, f_cs, f_sn, s_p, s_q, &f_off, &f_tot);
  {  // V (FP64) <- V32: through registers, the two share storage
    double v[(kMaxBlock * kMaxBlock + kRrThreads - 1) / kRrThreads];
    int u = 0;
    for (int e = tid; e < m * m; e += nt) v[u++] = (double)V32[e];
    __syncthreads();
    u = 0;
    for (int e = tid; e < m * m; e += nt) V[e] = v[u++];
  }
  __syncthreads();
  // Newton-Schulz: V <- V (3 I - V^T V) / 2, with T as scratch (T itself waits in registers;
  // G holds R~ for the back-substitution at the end). The register arrays hold a thread's share
  // of the m x m entries: at most kMaxBlock^2 / 256 with the 256-thread launch.
  {
    double tsave[(kMaxBlock * kMaxBlock + kRrThreads - 1) / kRrThreads];
    int u = 0;
    for (int e = tid; e < m * m; e += nt) tsave[u++] = T[e];
    __syncthreads();
    for (int e = tid; e < m * m; e += nt) {  // T <- W = V^T V
      const int i = e / m, j = e - i * m;
      double w = 0.0;
      for (int k = 0; k < m; ++k) w = fma(V[k * m + i], V[k * m + j], w);
      T[e] = (i == j ? 1.5 : 0.0) - 0.5 * w;
    }
    __syncthreads();
    double vn[(kMaxBlock * kMaxBlock + kRrThreads - 1) / kRrThreads];
    u = 0;
    for (int e = tid; e < m * m; e += nt) {  // V (1.5 I - 0.5 W)
      const int i = e / m, j = e - i * m;
      double a = 0.0;
      for (int k = 0; k < m; ++k) a = fma(V[i * m + k], T[k * m + j], a);
      vn[u++] = a;
    }
    __syncthreads();
    u = 0;
    for (int e = tid; e < m * m; e += nt) {
      V[e] = vn[u];
      T[e] = tsave[u];
      ++u;
    }
    __syncthreads();
    // M = V^T T V: first Y = T V (into registers), then M = V^T Y
    u = 0;
    for (int e = tid; e < m * m; e += nt) {
      const int i = e / m, j = e - i * m;
      double a = 0.0;
      for (int k = 0; k < m; ++k) a = fma(T[i * m + k], V[k * m + j], a);
      vn[u++] = a;
    }
    __syncthreads();
    u = 0;
    for (int e = tid; e < m * m; e += nt) T[e] = vn[u++];  // T <- Y
    __syncthreads();
    u = 0;
    for (int e = tid; e < m * m; e += nt) {
      const int i = e / m, j = e - i * m;
      double a = 0.0;
      for (int k = 0; k < m; ++k) a = fma(V[k * m + i], T[k * m + j], a);
      vn[u++] = a;
    }
    __syncthreads();
    u = 0;
    for (int e = tid; e < m * m; e += nt) T[e] = vn[u++];
    __syncthreads();
    for (int e = tid; e < m * m; e += nt) {  // symmetrise M
      const int i = e / m, j = e - i * m;
      if (i < j) {
        const double a = 0.5 * (T[i * m + j] + T[j * m + i]);
        T[i * m + j] = a;
        T[j * m + i] = a;
      }
    }
    __syncthreads();
  }
  jacobi_sweeps<double>(T, V, m, 8, 1e-20, s_cs, s_sn, s_p, s_q, &s_off, &s_tot);
  for (int i = tid; i < m; i += nt) lam[i] = T[i * m + i];
  __syncthreads();
  // decreasing Ritz value (stable on ties)
  for (int i = tid; i < m; i += nt) {
    int r = 0;
    for (int j = 0; j < m; ++j) r += (lam[j] > lam[i]) || (lam[j] == lam[i] && j < i);
    order[r] = i;
  }
  __syncthreads();
  if (near_identity) {  // x = W y for the selected Ritz vectors, a thread per entry
    for (int e = tid; e < ncomp * b; e += nt) {
      const int c = e / b, k = e - c * b;
      const int col = order[c];
      double a = 0.0;
      for (int j = 0; j < b; ++j) a = fma(G[k * b + j], V[j * m + col], a);
      Xout[(size_t)c * b + k] = a;
    }
    if (lambda_out)
      for (int c = tid; c < ncomp; c += nt) lambda_out[c] = lam[order[c]];
    return;
  }
  // x = R~^-1 y for the selected Ritz vectors, scattered back to the b kept columns
  for (int c = tid; c < ncomp; c += nt) {
    double* x = Xout + (size_t)c * b;
    for (int k = 0; k < b; ++k) x[k] = 0.0;
    if (c >= m) continue;  // fewer independent directions than components: zero component
    const int col = order[c];
    double xs[kMaxBlock];
    for (int i = m - 1; i >= 0; --i) {
      double v = V[i * m + col];
      for (int t = i + 1; t < m; ++t) v -= G[i * m + t] * xs[t];
      xs[i] = v / G[i * m + i];
    }
    for (int k = 0; k < b; ++k)
      if (keep[k] >= 0) x[k] = xs[keep[k]];
    if (lambda_out) lambda_out[c] = lam[col];
  }
}

// step 4: comps[c] = Q x_c (FP64), signed so that the largest |entry| (first on ties) is positive
__global__ void rr_comps_kernel(int P, int b, const float* __restrict__ Q, const double* __restrict__ X,
                                double* __restrict__ comps) {
  const int c = blockIdx.x;
  const double* x = X + (size_t)c * b;
  double* out = comps + (size_t)c * P;
  __shared__ double sbest[256];
  __shared__ int sidx[256];
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < b; ++k) s = fma((double)Q[(size_t)k * P + i], x[k], s);
    out[i] = s;
    const double a = fabs(s);
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
  const double piv = sidx[0] < P ? out[sidx[0]] : 0.0;
  __syncthreads();
  if (piv < 0)
    for (int i = threadIdx.x; i < P; i += blockDim.x) out[i] = -out[i];
}

// ---------------------------------------------------------------------------------------------
// Exact-grade leading eigenvectors (the drop-in form): subspace iteration in FP64 on all SMs.
// A block of b = min(40, P) vectors from a fixed pseudo-random start; kExactSteps power steps
// Z <- C Z M, where M (exact_factor) makes Z M nearly orthonormal: D (I + E)^-1/2 to second
// order once the scaled Gram matrix I + E is near the identity, an FP32 Cholesky factor in the
// first steps from the random start (condition up to ~3e5). Every CTA forms the small M itself;
// the products with M are FP64, so the span is kept to FP64 rounding whatever M's accuracy, and
// the final FP64 Rayleigh-Ritz step (rr_solve_kernel, as the approximate form: G = Q^T Q,
// T = Q^T C Q) absorbs Q's departure from orthonormality; the components are Q x. A Cholesky
// pivot that vanishes drops its column (a covariance of lower rank than the block). The error of
// component j after s steps shrinks like (lambda_{b+1} / lambda_j)^s: 40 steps reach FP64 accuracy
// for ratios up to ~0.45 (measured on the workloads' covariances: 0.10 to 0.29, 12 to 24 steps).
// The phases are separated by a bounded grid barrier; the launch is cooperative, so every CTA is
// resident and the barrier cannot wait on a CTA that has not started.
// ---------------------------------------------------------------------------------------------
constexpr int kExactThreads = 256;
constexpr int kExactSteps = 40;    // power steps in all
constexpr int kExactSteps32 = 24;  // of which the first run their products with C in FP32
constexpr long long kBarrierPolls = 20000000LL;  // ~1 s of polls at 64 ns: then give up, flag it

__device__ __forceinline__ unsigned ld_volatile_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.volatile.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

// bar[0] counts arrivals, bar[1] is the generation (both zero at launch). Returns false once a
// wait ran out (the status bit is then set and later barriers do not wait).
__device__ bool grid_barrier(unsigned* bar, unsigned nblocks, unsigned& gen, unsigned* status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1;
    const unsigned target = gen + 1;
    __threadfence();
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicExch(bar + 1, target);
    } else if (!(ld_volatile_u32(status) & DEV_GRID_TIMEOUT)) {
      long long polls = 0;
      while (ld_volatile_u32(bar + 1) != target) {
        if (++polls > kBarrierPolls) {
          atomicOr(status, DEV_GRID_TIMEOUT);
          s_ok = 0;
          break;
        }
        __nanosleep(64);
      }
    } else {
      s_ok = 0;
    }
    __threadfence();
  }
  gen += 1;
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ double hash_unit(uint32_t i, uint32_t j) {  // deterministic start in [-1, 1)
  const uint32_t h = mix32(i * 0x9E3779B1u + mix32(j + 0x632BE5ABu));
  return (double)h * (2.0 / 4294967296.0) - 1.0;
}

// Work split of a [P][b] product over the grid: CTA c owns outputs [c * opb, (c + 1) * opb), each
// shared by tpo threads (a power of two) that split the sum and meet in shuffles.
struct ExactSplit {
  int opb, tpo;
  __device__ ExactSplit(int P, int b) {
    opb = (P * b + gridDim.x - 1) / gridDim.x;
    tpo = 1;
    while (tpo < 8 && 2 * tpo * opb <= (int)blockDim.x) tpo *= 2;
  }
};

// stage X [P][b] (FP64, global) into shared memory, 16 bytes per load
__device__ void exact_stage(const double* __restrict__ X, int n, double* sX) {
  const int n2 = n >> 1;
  const double2* x2 = reinterpret_cast<const double2*>(X);
  double2* s2 = reinterpret_cast<double2*>(sX);
  for (int e = threadIdx.x; e < n2; e += blockDim.x) s2[e] = x2[e];
  if ((n & 1) && threadIdx.x == 0) sX[n - 1] = X[n - 1];
}

// Y[i][j] = sum_k C[i][k] Z[k][j] for this CTA's outputs, Z staged in shared memory; R: the
// arithmetic (float in the first power steps, double in the last)
template <typename R>
__device__ void exact_cq(const double* __restrict__ C, int P, int b, const double* sZ, double* __restrict__ Y) {
  const ExactSplit sp(P, b);
  const int slot = threadIdx.x / sp.tpo, part = threadIdx.x - slot * sp.tpo;
  const long long o = (long long)blockIdx.x * sp.opb + slot;
  const bool live = slot < sp.opb && o < (long long)P * b;
  R s = 0;
  if (live) {  // four independent partial sums: the FMA latency is hidden within the thread
    const int i = (int)(o / b), j = (int)(o - (long long)i * b);
    const double* c = C + (size_t)i * P;
    R a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    const int st = sp.tpo;
    int k = part;
    for (; k + 3 * st < P; k += 4 * st) {
      a0 = fma((R)__ldg(c + k), (R)sZ[k * b + j], a0);
      a1 = fma((R)__ldg(c + k + st), (R)sZ[(k + st) * b + j], a1);
      a2 = fma((R)__ldg(c + k + 2 * st), (R)sZ[(k + 2 * st) * b + j], a2);
      a3 = fma((R)__ldg(c + k + 3 * st), (R)sZ[(k + 3 * st) * b + j], a3);
    }
    for (; k < P; k += st) a0 = fma((R)__ldg(c + k), (R)sZ[k * b + j], a0);
    s = (a0 + a1) + (a2 + a3);
  }
  for (int m = 1; m < sp.tpo; m <<= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
  if (live && part == 0) Y[o] = (double)s;
}

// out[i][j] = out[j][i] = sum_k X[k][i] Y[k][j] (b x b), a warp per upper-triangular entry, X and
// Y in shared memory
__device__ void exact_gram(int P, int b, const double* sX, const double* sY, double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int nent = b * (b + 1) / 2;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < nent; e += nw) {
    int i = 0, rem = e;  // entry e -> (i, j), i <= j, rows of the upper triangle in order
    while (rem >= b - i) {
      rem -= b - i;
      ++i;
    }
    const int j = i + rem;
    double s = 0.0;
    for (int k = lane; k < P; k += 32) s = fma(sX[k * b + i], sY[k * b + j], s);
    s = warp_sum_d(s);
    if (lane == 0) {
      out[i * b + j] = s;
      out[j * b + i] = s;
    }
  }
}

// The factor that makes Z's columns (nearly) orthonormal, from the Gram matrix G = Z^T Z (FP64,
// global). Every CTA computes the same factor (same inputs, same thread mapping, same
// operations). With D = diag(G)^-1/2 and E = D G D - I: when max |E| <= kNsLimit, the full
// matrix M = D (I - E/2 + 3 E^2 / 8) (the binomial series of (I + E)^-1/2 to second order; returns
// true); otherwise the upper Cholesky factor R of I + E in FP32 (in sE, columns whose pivot
// vanishes dropped: their row of R is zero), applied as Z D R^-1 by exact_apply (returns
// false). The factor's accuracy does not matter: the span of the product is that of Z.
constexpr float kNsLimit = 0.25f;

__device__ bool exact_factor(const double* __restrict__ Gw, int b, double* sM, double* sD, float* sE, int* s_keep,
                             unsigned* s_emax) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  if (tid == 0) *s_emax = 0u;
  for (int e = tid; e < b; e += nt) {
    const double g = Gw[e * b + e];
    sD[e] = g > 0.0 ? 1.0 / sqrt(g) : 0.0;
  }
  __syncthreads();
  float emax = 0.f;
  for (int i = warp; i < b; i += nw)
    for (int j = lane; j < b; j += 32) {
      const bool live = sD[i] > 0.0 && sD[j] > 0.0;
      const float v = live ? (float)(Gw[i * b + j] * sD[i] * sD[j]) - (i == j ? 1.f : 0.f) : 0.f;
      sE[i * b + j] = v;
      emax = fmaxf(emax, fabsf(v));
    }
  atomicMax(s_emax, __float_as_uint(emax));  // non-negative floats order like their bits
  __syncthreads();
  if (__uint_as_float(*s_emax) <= kNsLimit) {
    for (int i = warp; i < b; i += nw)
      for (int j = lane; j < b; j += 32) {
        float e2 = 0.f;
        for (int k = 0; k < b; ++k) e2 = fmaf(sE[i * b + k], sE[k * b + j], e2);
        const float f = (i == j ? 1.f : 0.f) - 0.5f * sE[i * b + j] + 0.375f * e2;
        sM[i * b + j] = sD[i] * (double)f;
      }
    __syncthreads();
    return true;
  }
  // Cholesky of A = I + E, right-looking, one barrier per column: step k reads row k and updates
  // rows k+1.. (A_ij -= A_ki A_kj / A_kk for k < i <= j, warps over rows, lanes over columns);
  // row k of R is then row k of A over sqrt(A_kk)
  for (int e = tid; e < b; e += nt) sE[e * b + e] += 1.f;
  __syncthreads();
  for (int k = 0; k < b; ++k) {
    const float piv = sE[k * b + k];
    const bool keep = sD[k] > 0.0 && piv > 1e-7f;  // (nearly) in the span of the earlier columns: drop
    if (tid == 0) s_keep[k] = keep;
    if (keep) {
      const float inv = 1.f / piv;
      for (int i = k + 1 + warp; i < b; i += nw) {
        const float aki = sE[k * b + i] * inv;
        for (int j = i + lane; j < b; j += 32) sE[i * b + j] -= aki * sE[k * b + j];
      }
    }
    __syncthreads();
  }
  for (int k = warp; k < b; k += nw) {
    const float piv = sE[k * b + k];
    const float r = s_keep[k] ? rsqrtf(piv) : 0.f;
    for (int j = k + lane; j < b; j += 32) sE[k * b + j] *= r;
  }
  __syncthreads();
  return false;
}

// out = in M (ns) or out = (in D) R^-1 (R in sE), in arithmetic R (float in the first power steps,
// double in the last); this CTA's rows, a warp per row
template <typename R>
__device__ void exact_apply(int P, int b, const double* __restrict__ in, bool ns, const double* sM, const double* sD,
                            const float* sE, const int* s_keep, double* __restrict__ out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int rpb = (P + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * rpb, r1 = min(P, r0 + rpb);
  for (int i = r0 + warp; i < r1; i += nw) {
    const double* y = in + (size_t)i * b;
    double* x = out + (size_t)i * b;
    const R y0 = lane < b ? (R)y[lane] : R(0), y1 = lane + 32 < b ? (R)y[lane + 32] : R(0);
    if (ns) {
      R s0 = 0, s1 = 0, t0 = 0, t1 = 0;  // two chains per output
      for (int k = 0; k < b; k += 2) {
        const R yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, k & 31);
        const bool k1 = k + 1 < b;
        const R yk1 = __shfl_sync(0xffffffffu, (k + 1) < 32 ? y0 : y1, (k + 1) & 31);
        if (lane < b) {
          s0 = fma(yk, (R)sM[k * b + lane], s0);
          if (k1) t0 = fma(yk1, (R)sM[(k + 1) * b + lane], t0);
        }
        if (lane + 32 < b) {
          s1 = fma(yk, (R)sM[k * b + lane + 32], s1);
          if (k1) t1 = fma(yk1, (R)sM[(k + 1) * b + lane + 32], t1);
        }
      }
      if (lane < b) x[lane] = (double)(s0 + t0);
      if (lane + 32 < b) x[lane + 32] = (double)(s1 + t1);
      continue;
    }
    // x R = y D by forward substitution: x_j = (y_j D_j - sum_{k<j} x_k R_kj) / R_jj; lane k
    // holds x_k (and x_{k+32}), the sum is a warp reduction
    R x0 = 0, x1 = 0;
    for (int j = 0; j < b; ++j) {
      R part = 0;
      if (lane < j) part = x0 * (R)sE[lane * b + j];
      if (lane + 32 < j) part = fma(x1, (R)sE[(lane + 32) * b + j], part);
#pragma unroll
      for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      const R yj = __shfl_sync(0xffffffffu, j < 32 ? y0 : y1, j & 31);
      const R rjj = (R)sE[j * b + j];
      const R xj = (s_keep[j] && rjj > R(0)) ? (yj * (R)sD[j] - part) / rjj : R(0);
      if (lane == (j & 31)) {
        if (j < 32) x0 = xj; else x1 = xj;
      }
    }
    if (lane < b) x[lane] = (double)x0;
    if (lane + 32 < b) x[lane + 32] = (double)x1;
  }
}

// Z_0 = C Q_0; then per step s: Y = C Z_s and G = Z_s^T Z_s (one phase: both read Z_s only,
// staged in shared memory), M_s from G, Z_{s+1} = Y M_s = C (Z_s M_s). The last step writes
// Q = Z M (the basis) and W = Y M = C Q instead, and the Rayleigh-Ritz Gram matrices
// G = Q^T Q, T = Q^T W follow. The first steps32 products with C run in FP32 arithmetic (they
// only have to find the subspace to FP32 accuracy), the rest in FP64.
__global__ void __launch_bounds__(kExactThreads, 1) subspace_exact_kernel(const double* __restrict__ C, int P, int b,
                                                                          int steps, int steps32,
                                                                          double* __restrict__ Z,
                                                                          double* __restrict__ Y,
                                                                          double* __restrict__ Q,
                                                                          double* __restrict__ W,
                                                                          double* __restrict__ Gw,
                                                                          double* __restrict__ Gout,
                                                                          double* __restrict__ Tout, unsigned* bar,
                                                                          unsigned* status) {
  __shared__ float sE[kMaxBlock * kMaxBlock];
  __shared__ double sM[kMaxBlock * kMaxBlock];
  __shared__ double sD[kMaxBlock];
  __shared__ int s_keep[kMaxBlock];
  __shared__ unsigned s_emax;
  extern __shared__ __align__(16) double dyn[];
  const size_t pb2 = ((size_t)P * b + 1) & ~size_t(1);  // 16-byte aligned regions
  double* sZ = dyn;                                      // [P][b]: the block being multiplied
  double* sRows = dyn + pb2;                             // this CTA's rows for exact_apply, or W
  const int tid = threadIdx.x, nt = blockDim.x;
  unsigned gen = 0;
  const long long nthr = (long long)gridDim.x * nt;
  for (long long o = blockIdx.x * (long long)nt + tid; o < (long long)P * b; o += nthr)
    Q[o] = hash_unit((uint32_t)(o / b), (uint32_t)(o % b));
  if (!grid_barrier(bar, gridDim.x, gen, status)) return;
  exact_stage(Q, P * b, sZ);
  __syncthreads();
  exact_cq<float>(C, P, b, sZ, Z);
  if (!grid_barrier(bar, gridDim.x, gen, status)) return;
  for (int step = 0; step < steps; ++step) {
    exact_stage(Z, P * b, sZ);
    __syncthreads();
    exact_gram(P, b, sZ, sZ, Gw);
    if (step < steps32) {
      exact_cq<float>(C, P, b, sZ, Y);
    } else {
      exact_cq<double>(C, P, b, sZ, Y);
    }
    if (!grid_barrier(bar, gridDim.x, gen, status)) return;
    const bool ns = exact_factor(Gw, b, sM, sD, sE, s_keep, &s_emax);
    if (step + 1 < steps) {
      if (step < steps32) {
        exact_apply<float>(P, b, Y, ns, sM, sD, sE, s_keep, Z);
      } else {
        exact_apply<double>(P, b, Y, ns, sM, sD, sE, s_keep, Z);
      }
    } else {
      exact_apply<double>(P, b, Z, ns, sM, sD, sE, s_keep, Q);
      exact_apply<double>(P, b, Y, ns, sM, sD, sE, s_keep, W);
    }
    if (!grid_barrier(bar, gridDim.x, gen, status)) return;
  }
  exact_stage(Q, P * b, sZ);
  __syncthreads();
  exact_gram(P, b, sZ, sZ, Gout);
  exact_stage(W, P * b, sRows);  // (the rows region has room for a whole block: see the host)
  __syncthreads();
  exact_gram(P, b, sZ, sRows, Tout);  // Q^T W: symmetric up to rounding (rr_solve_kernel averages it)
}

// components [ncomp][P] = Q x (Q [P][b] FP64), signed so that the largest |entry| (first on
// ties) is positive
__global__ void rr_comps_exact_kernel(int P, int b, const double* __restrict__ Q, const double* __restrict__ X,
                                      double* __restrict__ comps) {
  const int c = blockIdx.x;
  const double* x = X + (size_t)c * b;
  double* out = comps + (size_t)c * P;
  __shared__ double sbest[256];
  __shared__ int sidx[256];
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < b; ++k) s = fma(Q[(size_t)i * b + k], x[k], s);
    out[i] = s;
    const double a = fabs(s);
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
  const double piv = sidx[0] < P ? out[sidx[0]] : 0.0;
  __syncthreads();
  if (piv < 0)
    for (int i = threadIdx.x; i < P; i += blockDim.x) out[i] = -out[i];
}

int num_sms();

// the FP64 subspace solver stages two [P][b] blocks in shared memory
bool exact_supported(int P, int ncomp) {
  const int b = std::min(kMaxBlock, P);
  return ncomp >= 1 && ncomp <= b && 2 * ((size_t)P * b + 2) * sizeof(double) <= 196 * 1024;
}

// C [P*P] FP64 covariance (device) -> comps [ncomp*P] FP64, exact-grade (FP64 iteration)
int eig_top_exact(annf_handle* h, const double* C, int P, int ncomp, double* comps, cudaStream_t st) {
  const int b = std::min(kMaxBlock, P);
  ANNF_REQUIRE(ncomp >= 1 && ncomp <= b, "exact subspace eigensolver: n_components above the block size");
  ANNF_REQUIRE(exact_supported(P, ncomp), "exact subspace eigensolver: unsupported size");
  const size_t pb2 = ((size_t)P * b + 1) & ~size_t(1);  // every block 16-byte aligned (staged as double2)
  const size_t f64 = (4 * pb2 + 3 * (size_t)b * b + (size_t)ncomp * b) * sizeof(double);
  ANNF_ENSURE(h->eig_ws, f64 + 256);
  double* Q = h->eig_ws.as<double>();
  double* Z = Q + pb2;
  double* Y = Z + pb2;
  double* Wm = Y + pb2;
  double* Gw = Wm + pb2;
  double* G = Gw + (size_t)b * b;
  double* T = G + (size_t)b * b;
  double* X = T + (size_t)b * b;
  unsigned* bar = reinterpret_cast<unsigned*>(reinterpret_cast<unsigned char*>(h->eig_ws.p) + ((f64 + 15) & ~size_t(15)));
  ANNF_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));
  // two staged [P][b] blocks (the block being multiplied; W, or a CTA's rows of Y) in dynamic
  // shared memory beside the 26 KB of static scratch
  const size_t smem = 2 * (pb2 + 2) * sizeof(double);
  ANNF_CUDA_TRY(cudaFuncSetAttribute(subspace_exact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  ANNF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, subspace_exact_kernel, kExactThreads, smem));
  ANNF_REQUIRE(per_sm >= 1, "exact subspace eigensolver: kernel does not fit an SM");
  const int grid = num_sms();  // one CTA per SM: all resident (cooperative launch)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kExactThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  ANNF_CUDA_TRY(cudaLaunchKernelEx(&cfg, subspace_exact_kernel, C, P, b, kExactSteps, kExactSteps32, Z, Y, Q, Wm, Gw,
                                   G, T, bar, h->status.as<unsigned>()));
  count_launch();
  rr_solve_kernel<<<1, kRrThreads, 0, st>>>(b, ncomp, G, T, X, nullptr);
  ANNF_CHECK_LAUNCH();
  rr_comps_exact_kernel<<<ncomp, 256, 0, st>>>(P, b, Q, X, comps);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

// block size for n components: b >= ncomp + max(8, ncomp / 2), a multiple of 8
int subspace_block(int P, int ncomp) {
  int b = ncomp + std::max(8, ncomp / 2);
  b = (b + 7) / 8 * 8;
  if (b > kMaxBlock || 2 * b > P) return 0;  // the exact solver handles these sizes
  return b;
}

// C [P*P] FP64 covariance (device) -> comps [ncomp*P] FP64
int eig_top_subspace(annf_handle* h, const double* C, int P, int ncomp, int iters, double* comps, cudaStream_t st) {
  const int b = subspace_block(P, ncomp);
  ANNF_REQUIRE(b > 0, "subspace eigensolver: unsupported size");
  // k slices of the C Q product: as many as the threads and shared memory allow (at most 4)
  const size_t fixed = ((size_t)2 * b * P + 2 * (size_t)b * b + b) * sizeof(float);
  int KS = std::max(1, std::min(4, kSubThreads / std::max(P, 1)));
  while (KS > 1 && fixed + (size_t)KS * P * b * sizeof(float) > 220 * 1024) --KS;
  const size_t smem = fixed + (size_t)KS * P * b * sizeof(float);
  ANNF_REQUIRE(smem <= 220 * 1024, "subspace eigensolver: block too large for shared memory");
  const size_t f32_bytes = ((size_t)P * P + (size_t)b * P) * sizeof(float);
  const size_t f64_bytes = ((size_t)b * P + 2 * (size_t)b * b + (size_t)ncomp * b) * sizeof(double);
  ANNF_ENSURE(h->eig_ws, f64_bytes + f32_bytes + 256);
  double* W = h->eig_ws.as<double>();
  double* G = W + (size_t)b * P;
  double* T = G + (size_t)b * b;
  double* X = T + (size_t)b * b;
  float* C32 = reinterpret_cast<float*>(X + (size_t)ncomp * b);
  float* Q = C32 + (size_t)P * P;
  switch (b) {
#define ANNF_SUBSPACE(BB)                                                                                    \
  case BB:                                                                                                   \
    ANNF_CUDA_TRY(cudaFuncSetAttribute(subspace_iter_kernel<BB>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                       (int)smem));                                                          \
    subspace_iter_kernel<BB><<<1, kSubThreads, smem, st>>>(C, P, KS, iters, C32, Q, h->status.as<unsigned>());  \
    break;
    ANNF_SUBSPACE(8)
    ANNF_SUBSPACE(16)
    ANNF_SUBSPACE(24)
    ANNF_SUBSPACE(32)
    ANNF_SUBSPACE(40)
#undef ANNF_SUBSPACE
    default:
      set_error("subspace eigensolver: unsupported block");
      return ANNF_ERR_UNSUPPORTED;
  }
  ANNF_CHECK_LAUNCH();
  rr_cq_kernel<<<ceil_div((long long)b * P * 32, 256), 256, 0, st>>>(C, P, b, Q, W);
  ANNF_CHECK_LAUNCH();
  rr_gram_kernel<<<ceil_div(2LL * b * b * 32, 256), 256, 0, st>>>(P, b, Q, W, G, T);
  ANNF_CHECK_LAUNCH();
  rr_solve_kernel<<<1, kRrThreads, 0, st>>>(b, ncomp, G, T, X, nullptr);
  ANNF_CHECK_LAUNCH();
  rr_comps_kernel<<<ncomp, 256, 0, st>>>(P, b, Q, X, comps);
  ANNF_CHECK_LAUNCH();
  return ANNF_OK;
}

}  // namespace annf
