// handle.cuh -- the opaque annf_handle: device tree, grow-only scratch buffers, solver state.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "common.cuh"

struct cusolverDnContext;

namespace annf {

// counts replacements (free + larger allocation) of every DevBuf in the process: a captured CUDA
// graph holds the buffers' addresses, and stays valid only while this count is unchanged (a first
// allocation moves nothing and is not counted)
void count_realloc();

// grow-only device allocation
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t need) {
    if (need <= bytes) return ANNF_OK;
    if (p) {
      count_realloc();
      cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    size_t sz = need < 256 ? 256 : need;
    cudaError_t e = cudaMalloc(&p, sz);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error(std::string("cudaMalloc(") + std::to_string(sz) + "): " + cudaGetErrorString(e));
      return ANNF_ERR_ALLOC;
    }
    bytes = sz;
    return ANNF_OK;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

#define ANNF_ENSURE(buf, nbytes)                 \
  do {                                           \
    int rc_ = (buf).ensure((size_t)(nbytes));    \
    if (rc_ != ANNF_OK) return rc_;              \
  } while (0)

}  // namespace annf

struct annf_handle {
  int device = 0;
  // ---- current tree ----
  int built = 0;
  int n = 0, d = 0, depth = 0, real_type = ANNF_REAL_F32, leaf_bits = 1, max_leaf = 0;
  annf::DevBuf pts, pts_tmp, perm, perm_tmp, node_axis, node_split, leaf_begin, point_leaf, leaf_box;
  // ---- build scratch ----
  annf::DevBuf bmin, bmax, axis, keys, hist, sel_prefix, sel_rank, sel_nlt, sel_neq, chunk_state,
      off_lt, off_eq, eqpos;
  // ---- query scratch ----
  annf::DevBuf nat_keys, nat_pos, lists, next_range, part_keys, part_pos, leaf_marks;
  // ---- parallel form scratch ----
  annf::DevBuf fast_buf, fast_nat, tc_buf, pj_buf;
  // ---- pca scratch ----
  annf::DevBuf gram, colsum, subset_t, cov, eigval, digits, meanproj, solver_ws, solver_info, eig_ws;
  int cov_p = 0;  // size of the covariance held in cov (0: none)
  // ---- openclopt-semantics tree and lists (openclopt.cu) ----
  int ocl_built = 0, ocl_m = 0, ocl_d = 0, ocl_h = -1, ocl_q = 0, ocl_ppl = 0, ocl_mp = 0;
  annf::DevBuf ocl_pts, ocl_indir, ocl_indir_tmp, ocl_dims, ocl_vals, ocl_clanc, ocl_o2l, ocl_keys, ocl_bounds,
      ocl_sort_ws, ocl_ki, ocl_kd, ocl_nat;
  // ---- options (annf_set_option) ----
  int opt_int_projection = 0;  // 1: the exact projection always runs the dp4a kernel
  cusolverDnContext* solver = nullptr;
  // ---- device status word ----
  annf::DevBuf status;
  // ---- optional stage marks: CUDA events recorded on the launching stream ----
  int prof_on = 0;
  int prof_used = 0;
  static constexpr int kMaxMarks = 64;
  cudaEvent_t prof_ev[kMaxMarks] = {};
  const char* prof_name[kMaxMarks] = {};
};

namespace annf {
// record a named mark on the stream when profiling is enabled (no-op otherwise)
inline void prof_mark(annf_handle* h, const char* name, cudaStream_t st) {
  if (!h->prof_on || h->prof_used >= annf_handle::kMaxMarks) return;
  cudaEvent_t& e = h->prof_ev[h->prof_used];
  if (!e) cudaEventCreate(&e);
  cudaEventRecord(e, st);
  h->prof_name[h->prof_used++] = name;
}
// kernels launched by this library since load (process-wide)
void count_launch();
}  // namespace annf
