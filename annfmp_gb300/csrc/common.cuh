// common.cuh -- shared definitions of the annf_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>
#include <string>

#include "../../include/annf_gb300.h"

namespace annf {

// ------------------------------------------------------------------------------------------
// error plumbing: every entry point returns a status; the message is kept per thread
// ------------------------------------------------------------------------------------------
void set_error(const std::string& msg);

#define ANNF_CUDA_TRY(expr)                                                                  \
  do {                                                                                       \
    cudaError_t e_ = (expr);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      ::annf::set_error(std::string(#expr) + ": " + cudaGetErrorString(e_));                 \
      return ANNF_ERR_CUDA;                                                                  \
    }                                                                                        \
  } while (0)

void count_launch();

// called once after every kernel launch: counts it and reports a launch error
#define ANNF_CHECK_LAUNCH()                                                                  \
  do {                                                                                       \
    ::annf::count_launch();                                                                  \
    cudaError_t e_ = cudaGetLastError();                                                     \
    if (e_ != cudaSuccess) {                                                                 \
      ::annf::set_error(std::string("kernel launch: ") + cudaGetErrorString(e_));            \
      return ANNF_ERR_CUDA;                                                                  \
    }                                                                                        \
  } while (0)

// device buffers that kernels read with 4- or 16-byte loads must start on such a boundary
// (cudaMalloc and torch return 256-byte aligned memory)
#define ANNF_ALIGNED(ptr, a) ((reinterpret_cast<uintptr_t>(ptr) & ((uintptr_t)(a) - 1)) == 0)

#define ANNF_REQUIRE(cond, msg)                                                              \
  do {                                                                                       \
    if (!(cond)) {                                                                           \
      ::annf::set_error(msg);                                                                \
      return ANNF_ERR_INVALID;                                                               \
    }                                                                                        \
  } while (0)

// device-side status bits (bounds checks that skip the access instead of faulting)
enum : unsigned {
  DEV_BAD_INDEX = 1u,
  DEV_BAD_LEAF = 2u,
  DEV_LIST_OVERFLOW = 4u,
  DEV_SMEM_CARVE = 8u,  // a kernel's shared-memory carve exceeded its launch allocation
  DEV_TC_TIMEOUT = 16u, // a tensor-core kernel's bounded wait on its MMA ran out
  DEV_GRID_TIMEOUT = 32u, // a bounded grid-wide barrier gave up waiting for the other CTAs
  DEV_LOOKBACK_TIMEOUT = 64u, // a scatter chunk's bounded wait for its predecessors' counts ran out
};

__device__ __forceinline__ unsigned dyn_smem_size() {
  unsigned r;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
  return r;
}

// true (and the status bit set) when the carve [base, end) does not fit the dynamic allocation;
// the caller returns before touching shared memory
__device__ __forceinline__ bool smem_overrun(const void* base, const void* end, unsigned* status) {
  const size_t used = (size_t)((const unsigned char*)end - (const unsigned char*)base);
  if (used > dyn_smem_size()) {
    if (threadIdx.x == 0 && status) atomicOr(status, DEV_SMEM_CARVE);
    return true;
  }
  return false;
}

// ------------------------------------------------------------------------------------------
// scalar traits
// ------------------------------------------------------------------------------------------
template <typename T> struct real_traits;
template <> struct real_traits<float> {
  static constexpr float big() { return FLT_MAX; }
  __device__ static float sub(float a, float b) { return __fsub_rn(a, b); }
  __device__ static float mul(float a, float b) { return __fmul_rn(a, b); }
  __device__ static float add(float a, float b) { return __fadd_rn(a, b); }
  __device__ static float sqrt_(float a) { return __fsqrt_rn(a); }
};
// Two IEEE round-to-nearest FP32 operations in one instruction (sm_100 and later): each half
// rounds exactly like __fsub_rn / __fmul_rn, so a distance formed with these keeps its bits.
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;"
      : "=l"(r)
      : "l"(((unsigned long long)__float_as_uint(a.y) << 32) | __float_as_uint(a.x)),
        "l"(((unsigned long long)__float_as_uint(b.y) << 32) | __float_as_uint(b.x)));
  return make_float2(__uint_as_float((unsigned)r), __uint_as_float((unsigned)(r >> 32)));
}
__device__ __forceinline__ float2 sq2_rn(float2 t) {  // (t.x * t.x, t.y * t.y)
  unsigned long long r;
  const unsigned long long v = ((unsigned long long)__float_as_uint(t.y) << 32) | __float_as_uint(t.x);
  asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(r) : "l"(v));
  return make_float2(__uint_as_float((unsigned)r), __uint_as_float((unsigned)(r >> 32)));
}
// acc + (w.x - q0)^2 + (w.y - q1)^2 + (w.z - q2)^2 + (w.w - q3)^2, summed in that order with
// every step rounded (the reference's order, no contraction): differences and squares pairwise
__device__ __forceinline__ float dist_step4(float acc, float4 w, float q0, float q1, float q2, float q3) {
  const float2 a = sq2_rn(sub2_rn(make_float2(w.x, w.y), make_float2(q0, q1)));
  const float2 b = sq2_rn(sub2_rn(make_float2(w.z, w.w), make_float2(q2, q3)));
  acc = __fadd_rn(acc, a.x);
  acc = __fadd_rn(acc, a.y);
  acc = __fadd_rn(acc, b.x);
  return __fadd_rn(acc, b.y);
}

template <> struct real_traits<double> {
  static constexpr double big() { return DBL_MAX; }
  __device__ static double sub(double a, double b) { return __dsub_rn(a, b); }
  __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
  __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
  __device__ static double sqrt_(double a) { return __dsqrt_rn(a); }
};

// Order-preserving unsigned image of a float with -0.0 folded onto +0.0, so that key equality is
// IEEE equality and key order is IEEE order (NaN-free inputs).
__device__ __forceinline__ uint32_t ord_key(float f) {
  uint32_t b = __float_as_uint(f);
  if (b == 0x80000000u) b = 0u;
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_to_float(uint32_t k) {
  uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(b);
}
__device__ __forceinline__ unsigned long long ord_key(double f) {
  unsigned long long b = __double_as_longlong(f);
  if (b == 0x8000000000000000ull) b = 0ull;
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_to_real(unsigned long long k) {
  unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double(b);
}

template <typename T> struct key_of;
template <> struct key_of<float> { using type = uint32_t; static constexpr int bits = 32; };
template <> struct key_of<double> { using type = unsigned long long; static constexpr int bits = 64; };

// Sort key of a candidate: the distance's bits (non-negative reals order like their bits), then
// a tie-break that reproduces the reference's visiting order. 64 bits for float distances; for
// double distances the key is a pair.
template <typename T> struct cand_key;
template <> struct cand_key<float> {
  using type = unsigned long long;
  __device__ static type make(float d, uint32_t tie) {
    return ((unsigned long long)__float_as_uint(d) << 32) | tie;
  }
  __device__ static float dist(type k) { return __uint_as_float((uint32_t)(k >> 32)); }
  static constexpr type init_key() { return ((unsigned long long)0x7f7fffffu << 32); }  // FLT_MAX, tie 0
};

struct dkey {  // double distance + tie
  unsigned long long d;
  uint32_t tie;
};
__device__ __forceinline__ bool operator<(const dkey& a, const dkey& b) {
  return a.d < b.d || (a.d == b.d && a.tie < b.tie);
}
template <> struct cand_key<double> {
  using type = dkey;
  __device__ static type make(double d, uint32_t tie) {
    return dkey{(unsigned long long)__double_as_longlong(d), tie};
  }
  __device__ static double dist(type k) { return __longlong_as_double((long long)k.d); }
  __host__ __device__ static type init_key() { return dkey{0x7fefffffffffffffull, 0u}; }  // DBL_MAX
};

__device__ __forceinline__ unsigned long long shfl_xor_u64(unsigned long long v, int m) {
  return __shfl_xor_sync(0xffffffffu, v, m);
}
__device__ __forceinline__ dkey shfl_xor_dk(dkey v, int m) {
  return dkey{__shfl_xor_sync(0xffffffffu, v.d, m), __shfl_xor_sync(0xffffffffu, v.tie, m)};
}
__device__ __forceinline__ unsigned long long shfl_u64(unsigned long long v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

// ------------------------------------------------------------------------------------------
// device tree view (structure of arrays, heap-ordered nodes)
// ------------------------------------------------------------------------------------------
template <typename T>
struct TreeView {
  int n, d, depth;
  int leaf_bits;            // bits needed for an offset inside any leaf
  const T* pts;             // [n*d] tree order
  const int* perm;          // [n] tree position -> original index
  const int* node_axis;     // [2^depth-1]
  const T* node_split;      // [2^depth-1]
  const int* leaf_begin;    // [2^depth+1] (leaf l spans [leaf_begin[l], leaf_begin[l+1]))
  const int* point_leaf;    // [n] original index -> leaf
  unsigned* status;         // device status word (bounds checks)
  const T* leaf_box;        // [2^depth][2][d] per-leaf min / max
};

// Source of raw uint8 patches: an HxWxC image (patch index = y*ncols + x) or a patch array
// ([n*P] bytes, described as psize=1, c=P).
struct PatchSrc {
  const uint8_t* img;  // image (HxWxC) or patch array ([n*P])
  int w, c, psize, ncols;
  bool is_img;
  long long bytes;     // size of the buffer: no load reaches past it
  __device__ __forceinline__ const uint8_t* row(long long idx, int r) const {
    if (is_img) {
      const long long y = idx / ncols, x = idx - y * ncols;
      return img + ((y + r) * w + x) * c;
    }
    return img + idx * (long long)psize * psize * c + (long long)r * psize * c;
  }
};

// bytes [off, off + 4) of a buffer of nbytes bytes (4-byte aligned base), through aligned 32-bit
// loads; within 8 bytes of the end, byte loads (bytes at or past nbytes read as zero)
__device__ __forceinline__ unsigned load_word_bounded(const uint8_t* base, long long off, long long nbytes) {
  const long long a = off & ~3LL;
  const int sh = (int)(off & 3) * 8;
  if (a + 8 <= nbytes) {
    const unsigned* w = reinterpret_cast<const unsigned*>(base + a);
    const unsigned lo = __ldg(w);
    return sh ? __funnelshift_r(lo, __ldg(w + 1), sh) : lo;
  }
  unsigned v = 0;
  for (int u = 0; u < 4; ++u)
    if (off + u < nbytes) v |= (unsigned)__ldg(base + off + u) << (8 * u);
  return v;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace annf
