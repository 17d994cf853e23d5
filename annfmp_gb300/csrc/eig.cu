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
// subspace run in FP32. Used by the approximate NNF forms; the plain form keeps the exact solver.
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
// A block of b = min(40, P) vectors from a fixed pseudo-random start; kExactSteps times
//   Z = C Q                      (FP64, every output split over four threads),
//   G = Z^T Z                    (FP64, a warp per entry),
//   Q = Z D R^-1                 (D = diag(G)^-1/2, R the Cholesky factor of D G D),
// then W = C Q, G = Q^T Q, T = Q^T W for the FP64 Rayleigh-Ritz step (rr_solve_kernel, as the
// approximate form) and the components Q x. Every CTA factors the small scaled Gram matrix in
// FP32 itself (it is well conditioned: at most ~3e5 in the first steps from a random start, then
// near 1); Q = Z (D R^-1) is formed in FP64, so the span of Z is kept to FP64 rounding whatever
// R's accuracy, and the final Rayleigh-Ritz step absorbs Q's departure from orthonormality. A
// pivot that vanishes drops its column (a covariance of lower rank than the block). The error of
// component j after s steps shrinks like (lambda_{b+1} / lambda_j)^s: 40 steps reach FP64 accuracy
// for ratios up to ~0.45 (measured on the workloads' covariances: 0.10 to 0.29, 12 to 24 steps).
// The phases are separated by a bounded grid barrier; the launch is cooperative, so every CTA is
// resident and the barrier cannot wait on a CTA that has not started.
// ---------------------------------------------------------------------------------------------
constexpr int kExactThreads = 256;
constexpr int kExactSteps = 40;
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

// Z[i][j] = sum_k C[i][k] Q[k][j] (Q, Z: [P][b] row-major), four threads per output
__device__ void exact_cq(const double* __restrict__ C, int P, int b, const double* __restrict__ Q, double* __restrict__ Z) {
  const long long total = (long long)P * b * 4;
  const long long nthr = (long long)gridDim.x * blockDim.x;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ((total + 31) / 32) * 32; t += nthr) {
    const long long o = t >> 2;
    const int part = (int)(t & 3);
    double s = 0.0;
    if (o < (long long)P * b) {
      const int i = (int)(o / b), j = (int)(o - (long long)i * b);
      const double* c = C + (size_t)i * P;
      for (int k = part; k < P; k += 4) s = fma(c[k], Q[(size_t)k * b + j], s);
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (part == 0 && o < (long long)P * b) Z[o] = s;
  }
}

// out[i][j] = out[j][i] = sum_k X[k][i] Y[k][j] (b x b), a warp per upper-triangular entry
__device__ void exact_gram(int P, int b, const double* __restrict__ X, const double* __restrict__ Y,
                           double* __restrict__ out) {
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
    for (int k = lane; k < P; k += 32) s = fma(X[(size_t)k * b + i], Y[(size_t)k * b + j], s);
    s = warp_sum_d(s);
    if (lane == 0) {
      out[i * b + j] = s;
      out[j * b + i] = s;
    }
  }
}

__global__ void __launch_bounds__(kExactThreads, 1) subspace_exact_kernel(const double* __restrict__ C, int P, int b,
                                                                          int steps, double* __restrict__ Q,
                                                                          double* __restrict__ Z,
                                                                          double* __restrict__ Gw,
                                                                          double* __restrict__ Gout,
                                                                          double* __restrict__ Tout, unsigned* bar,
                                                                          unsigned* status) {
  __shared__ float sG[kMaxBlock * kMaxBlock];   // scaled Gram, then R (upper)
  __shared__ float sRi[kMaxBlock * kMaxBlock];  // R^-1 (upper)
  __shared__ double sM[kMaxBlock * kMaxBlock];  // D R^-1 in FP64
  __shared__ double sD[kMaxBlock];
  __shared__ float s_piv;
  __shared__ int s_keep[kMaxBlock];
  const int tid = threadIdx.x, nt = blockDim.x;
  unsigned gen = 0;
  const long long nthr = (long long)gridDim.x * nt;
  for (long long o = blockIdx.x * (long long)nt + tid; o < (long long)P * b; o += nthr)
    Q[o] = hash_unit((uint32_t)(o / b), (uint32_t)(o % b));
  bool ok = grid_barrier(bar, gridDim.x, gen, status);
  for (int step = 0; step < steps && ok; ++step) {
    exact_cq(C, P, b, Q, Z);
    ok = grid_barrier(bar, gridDim.x, gen, status);
    if (!ok) break;
    exact_gram(P, b, Z, Z, Gw);
    ok = grid_barrier(bar, gridDim.x, gen, status);
    if (!ok) break;
    // every CTA: D, the Cholesky factor of D G D (FP32, right-looking), R^-1, M = D R^-1
    for (int e = tid; e < b; e += nt) {
      const double g = Gw[e * b + e];
      sD[e] = g > 0.0 ? 1.0 / sqrt(g) : 0.0;
    }
    __syncthreads();
    for (int e = tid; e < b * b; e += nt) {
      const int i = e / b, j = e - i * b;
      sG[e] = (float)(Gw[e] * sD[i] * sD[j]);
    }
    __syncthreads();
    for (int k = 0; k < b; ++k) {
      if (tid == 0) {
        const float piv = sG[k * b + k];
        const bool keep = piv > 1e-7f;  // a column (nearly) in the span of the earlier ones: drop it
        s_keep[k] = keep;
        s_piv = keep ? sqrtf(piv) : 0.f;
      }
      __syncthreads();
      const float r = s_piv;
      for (int j = k + tid; j < b; j += nt) sG[k * b + j] = r > 0.f ? sG[k * b + j] / r : 0.f;
      __syncthreads();
      const int tw = b - k - 1;
      for (int e = tid; e < tw * tw; e += nt) {
        const int i = k + 1 + e / tw, j = k + 1 + e % tw;
        if (j >= i) sG[i * b + j] -= sG[k * b + i] * sG[k * b + j];
      }
      __syncthreads();
    }
    for (int j = tid; j < b; j += nt) {  // column j of R^-1 by back-substitution (dropped pivots: zero)
      for (int i = b - 1; i >= 0; --i) {
        float v = i == j ? 1.f : 0.f;
        if (i > j || !s_keep[i]) {
          sRi[i * b + j] = 0.f;
          continue;
        }
        for (int k = i + 1; k <= j; ++k) v -= sG[i * b + k] * sRi[k * b + j];
        sRi[i * b + j] = v / sG[i * b + i];
      }
    }
    __syncthreads();
    for (int e = tid; e < b * b; e += nt) sM[e] = sD[e / b] * (double)sRi[e];
    __syncthreads();
    for (long long o = blockIdx.x * (long long)nt + tid; o < (long long)P * b; o += nthr) {
      const int i = (int)(o / b), j = (int)(o - (long long)i * b);
      double s = 0.0;
      for (int k = 0; k <= j; ++k) s = fma(Z[(size_t)i * b + k], sM[k * b + j], s);
      Q[o] = s;
    }
    ok = grid_barrier(bar, gridDim.x, gen, status);
  }
  if (!ok) return;
  exact_cq(C, P, b, Q, Z);  // W = C Q
  if (!grid_barrier(bar, gridDim.x, gen, status)) return;
  exact_gram(P, b, Q, Q, Gout);
  exact_gram(P, b, Q, Z, Tout);  // Q^T W: symmetric up to rounding (rr_solve_kernel averages it)
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

int exact_block_max() { return kMaxBlock; }

// C [P*P] FP64 covariance (device) -> comps [ncomp*P] FP64, exact-grade (FP64 iteration)
int eig_top_exact(annf_handle* h, const double* C, int P, int ncomp, double* comps, cudaStream_t st) {
  const int b = std::min(kMaxBlock, P);
  ANNF_REQUIRE(ncomp >= 1 && ncomp <= b, "exact subspace eigensolver: n_components above the block size");
  const size_t f64 = (2 * (size_t)P * b + 3 * (size_t)b * b + (size_t)ncomp * b) * sizeof(double);
  ANNF_ENSURE(h->eig_ws, f64 + 256);
  double* Q = h->eig_ws.as<double>();
  double* Z = Q + (size_t)P * b;
  double* Gw = Z + (size_t)P * b;
  double* G = Gw + (size_t)b * b;
  double* T = G + (size_t)b * b;
  double* X = T + (size_t)b * b;
  unsigned* bar = reinterpret_cast<unsigned*>(reinterpret_cast<unsigned char*>(h->eig_ws.p) + ((f64 + 15) & ~size_t(15)));
  ANNF_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));
  int per_sm = 0;
  ANNF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, subspace_exact_kernel, kExactThreads, 0));
  ANNF_REQUIRE(per_sm >= 1, "exact subspace eigensolver: kernel does not fit an SM");
  const int grid = num_sms();  // one CTA per SM: all resident (cooperative launch)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kExactThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  ANNF_CUDA_TRY(cudaLaunchKernelEx(&cfg, subspace_exact_kernel, C, P, b, kExactSteps, Q, Z, Gw, G, T, bar,
                                   h->status.as<unsigned>()));
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
