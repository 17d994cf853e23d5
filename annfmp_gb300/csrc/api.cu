// api.cu -- the extern "C" entry points declared in include/annf_gb300.h.
#include <cusolverDn.h>

#include <atomic>
#include <string>

#include "common.cuh"
#include "handle.cuh"

namespace annf {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static std::atomic<long long> g_reallocs{0};
void count_realloc() { g_reallocs.fetch_add(1, std::memory_order_relaxed); }

// implemented in tree_build.cu / search.cu / pca.cu
int build_tree(annf_handle* h, const void* points, int n, int d, int real_type, int depth, int splitting,
               cudaStream_t st);
int process_rows_generic(annf_handle* h, int* final_idx, const PatchSrc& A, const PatchSrc& B, const void* ared,
                         int n_rows, int n_cols, int K, int propagate, int select_best, long long max_leaves,
                         int* knn_out, float* dist_out, cudaStream_t st);
int kneighbors_generic(annf_handle* h, const void* Q, int nq, int K, long long max_leaves, void* dist, int* idx,
                       cudaStream_t st);
int kneighbors_noalloc(annf_handle* h, const void* Q, int nq, int K, long long max_leaves, void* dist, int* idx,
                       cudaStream_t st);
int natural_knn_all(annf_handle* h, const void* Q, long long nq, int K, int* out_pos, cudaStream_t st);
int fast_search(annf_handle* h, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb, int wb, int c,
                int psize, int K, const int* nat_pos, const int* prop, int n_prop, const int* seed_match, int iters,
                uint32_t seed, int rand_samples, int radius0, int* final_idx, float* dist_out, cudaStream_t st);
int seed_matches(const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb, int wb, int c, int psize,
                 const int* cand, int n_cand, int* seed_out, cudaStream_t st);
bool leaf_tc_supported(const annf_handle* h, int K);
int ocl_build_tree(annf_handle* h, const float* X, int m, int d, int leaf_size, cudaStream_t st);
int ocl_rows(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb,
             int wb, int ch, int psize, const float* ared, int n_rows, int n_cols, int* knn_out, float* knn_sqdist_out,
             float* dist_out, cudaStream_t st);
int natural_knn_tc(annf_handle* h, const float* Q, long long nq, int K, int prec, int* out_pos, cudaStream_t st);
int tc_tile(const uint16_t* A, const uint16_t* B, int N, int K, float* D, unsigned* status, cudaStream_t st);
int cnn_input(const uint8_t* A, const uint8_t* B, int H, int W, void* X, cudaStream_t st);
int cnn_prep_weights(const float* W, int co, int ci, float* wf, float* wb, cudaStream_t st);
int cnn_conv_forward(const void* X, int nimg, int h, int w, int ci, int co, const float* wf, const float* bias,
                     int relu, void* Y, unsigned* status, cudaStream_t st);
int cnn_prep_weights_tc(const float* W, int co, int ci, uint16_t* wt, cudaStream_t st);
int cnn_conv_forward_tc(const void* X, int nimg, int h, int w, int ci, int co, const uint16_t* wt, const float* bias,
                        int relu, void* Y, unsigned* status, cudaStream_t st);
int cnn_conv_backward_data(const float* G, const void* mask, int nimg, int h, int w, int co, int ci, const float* wb,
                           float* dX, unsigned* status, cudaStream_t st);
int cnn_conv_backward_weights(const void* X, const float* G, const void* mask, int nimg, int h, int w, int ci, int co,
                              float* dW, float* db, unsigned* status, cudaStream_t st);
int cnn_wta_loss(const float* out, const float* tgt, const uint8_t* valid, long long npix, float inv_nv, float* dout,
                 float* loss_sum, cudaStream_t st);
int cnn_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps, int step,
             cudaStream_t st);
int cnn_targets(const int* nnf, int H, int W, int Wb, int psize, float* tgt, uint8_t* valid, cudaStream_t st);
int cnn_proposals(const float* out, int h4, int w4, int H, int W, int Hb, int Wb, int psize, int per_pixel, int* props,
                  cudaStream_t st);
bool project_tc_supported(int psize, int c, int ncomp);
int project_tc(annf_handle* h, const uint8_t* img, int H, int W, int c, int psize, const double* comps,
               const double* mean, int ncomp, float* out, cudaStream_t st);
int raw_nn(const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb, int wb, int c, int psize,
           const int* qpix, int nq, unsigned long long* best, cudaStream_t st);
int pca_covariance(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a,
                   const uint8_t* img_b, int hb, int wb, const int* pos_b, int n_b, int c, int psize, double* mean,
                   cudaStream_t st);
int pca_components(annf_handle* h, int P, int ncomp, int solver, double* comps, cudaStream_t st);
int pca_fit(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a, const uint8_t* img_b,
            int hb, int wb, const int* pos_b, int n_b, int c, int psize, int ncomp, double* comps, double* mean,
            int solver, cudaStream_t st);
int project(annf_handle* h, const uint8_t* img, int H, int W, int c, int psize, const double* comps,
            const double* mean, int ncomp, int real_type, void* out, cudaStream_t st);

}  // namespace annf

using namespace annf;

static constexpr int kMaxK = 32;

#define ANNF_API_HANDLE(h)                                   \
  do {                                                       \
    if (!(h)) {                                              \
      set_error("handle is NULL");                           \
      return ANNF_ERR_INVALID;                               \
    }                                                        \
    cudaError_t e_ = cudaSetDevice((h)->device);             \
    if (e_ != cudaSuccess) {                                 \
      set_error(std::string("cudaSetDevice: ") + cudaGetErrorString(e_)); \
      return ANNF_ERR_CUDA;                                  \
    }                                                        \
  } while (0)

extern "C" {

int annf_version(void) { return 10000; }

const char* annf_last_error(void) { return g_last_error.c_str(); }

int annf_create(annf_handle** out, int device) {
  if (!out) {
    set_error("annf_create: out is NULL");
    return ANNF_ERR_INVALID;
  }
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    set_error(std::string("annf_create: no CUDA device: ") + cudaGetErrorString(e));
    return ANNF_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) {
    set_error("annf_create: device index out of range");
    return ANNF_ERR_INVALID;
  }
  ANNF_CUDA_TRY(cudaSetDevice(device));
  annf_handle* h = new annf_handle();
  h->device = device;
  if (h->status.ensure(sizeof(unsigned)) != ANNF_OK) {
    delete h;
    return ANNF_ERR_ALLOC;
  }
  ANNF_CUDA_TRY(cudaMemset(h->status.p, 0, sizeof(unsigned)));
  *out = h;
  return ANNF_OK;
}

void annf_destroy(annf_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->solver) cusolverDnDestroy(reinterpret_cast<cusolverDnHandle_t>(h->solver));
  DevBuf* bufs[] = {&h->pts, &h->pts_tmp, &h->perm, &h->perm_tmp, &h->node_axis, &h->node_split, &h->leaf_begin,
                    &h->point_leaf, &h->leaf_box, &h->bmin, &h->bmax, &h->axis, &h->keys, &h->hist, &h->sel_prefix,
                    &h->sel_rank, &h->sel_nlt, &h->sel_neq, &h->chunk_state, &h->off_lt, &h->off_eq,
                    &h->eqpos, &h->nat_keys, &h->nat_pos, &h->lists, &h->next_range, &h->part_keys,
                    &h->part_pos, &h->fast_buf, &h->fast_nat, &h->tc_buf, &h->pj_buf, &h->gram, &h->colsum, &h->subset_t, &h->cov, &h->eigval, &h->digits,
                    &h->meanproj, &h->solver_ws, &h->solver_info, &h->eig_ws, &h->status, &h->leaf_marks,
                    &h->ocl_pts, &h->ocl_indir, &h->ocl_indir_tmp, &h->ocl_dims, &h->ocl_vals, &h->ocl_clanc,
                    &h->ocl_o2l, &h->ocl_keys, &h->ocl_bounds, &h->ocl_sort_ws, &h->ocl_ki, &h->ocl_kd, &h->ocl_nat};
  for (DevBuf* b : bufs) b->release();
  for (int i = 0; i < annf_handle::kMaxMarks; ++i)
    if (h->prof_ev[i]) cudaEventDestroy(h->prof_ev[i]);
  delete h;
}

int annf_build_tree(annf_handle* h, const void* points, int n, int d, int real_type, int depth,
                    int splitting_type, void* stream) {
  ANNF_API_HANDLE(h);
  return build_tree(h, points, n, d, real_type, depth, splitting_type, static_cast<cudaStream_t>(stream));
}

int annf_tree_get(const annf_handle* h, annf_tree_view* out) {
  if (!h || !out) {
    set_error("annf_tree_get: NULL argument");
    return ANNF_ERR_INVALID;
  }
  if (!h->built) {
    set_error("annf_tree_get: no tree has been built");
    return ANNF_ERR_STATE;
  }
  out->n = h->n;
  out->d = h->d;
  out->depth = h->depth;
  out->real_type = h->real_type;
  out->n_leaves = 1 << h->depth;
  out->points = h->pts.p;
  out->perm = h->perm.as<int>();
  out->node_axis = h->node_axis.as<int>();
  out->node_split = h->node_split.p;
  out->leaf_begin = h->leaf_begin.as<int>();
  out->point_leaf = h->point_leaf.as<int>();
  out->leaf_box = h->leaf_box.p;
  return ANNF_OK;
}

// max_k: the largest K the entry point's kernels take (kneighbors: the reference's 1000)
static int check_k(const annf_handle* h, int k, long long max_leaves, int max_k = kMaxK) {
  if (!h->built) {
    set_error("no tree has been built (call annf_build_tree first)");
    return ANNF_ERR_STATE;
  }
  if (k < 1 || k > 1000) {  // reference limit, helper.c:32-35
    set_error("k must be in [1, 1000]");
    return ANNF_ERR_INVALID;
  }
  if (k > max_k) {
    set_error("k > 32 is not supported by this entry point's GPU kernels");
    return ANNF_ERR_UNSUPPORTED;
  }
  if (max_leaves < 0) {  // annfmp/openmp/kdtree/base.py:129-130
    set_error("max_leaves must be a positive integer");
    return ANNF_ERR_INVALID;
  }
  return ANNF_OK;
}

int annf_kneighbors(annf_handle* h, const void* queries, int nq, int k, long long max_leaves, void* distances,
                    int* indices, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(queries, 16), "annf_kneighbors: queries must be 16-byte aligned");
  int rc = check_k(h, k, max_leaves, 1000);
  if (rc != ANNF_OK) return rc;
  ANNF_REQUIRE(nq >= 0, "annf_kneighbors: nq < 0");
  if (nq == 0) return ANNF_OK;
  ANNF_REQUIRE(queries && distances && indices, "annf_kneighbors: NULL array");
  return kneighbors_generic(h, queries, nq, k, max_leaves, distances, indices, static_cast<cudaStream_t>(stream));
}

static int rows_common_checks(annf_handle* h, int* final_idx, const void* ared, int n_rows, int n_cols, int k,
                              long long max_leaves) {
  int rc = check_k(h, k, max_leaves);
  if (rc != ANNF_OK) return rc;
  ANNF_REQUIRE(final_idx && ared, "process_rows: NULL output or reduced-patch array");
  ANNF_REQUIRE(n_rows >= 1 && n_cols >= 1, "process_rows: empty patch grid");
  ANNF_REQUIRE((long long)n_rows * n_cols <= 0x7fffffffLL, "process_rows: patch grid too large");
  return ANNF_OK;
}

int annf_process_rows(annf_handle* h, int* final_idx, const uint8_t* patches_a, int n_a, const uint8_t* patches_b,
                      int n_b, int P, const void* ared, int n_rows, int n_cols, int k, int propagate,
                      int select_best, long long max_leaves, int* knn_out, float* dist_out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(patches_a, 4) && ANNF_ALIGNED(patches_b, 4) && ANNF_ALIGNED(ared, 16),
               "annf_process_rows: patch arrays must be 4-byte and reduced patches 16-byte aligned");
  int rc = rows_common_checks(h, final_idx, ared, n_rows, n_cols, k, max_leaves);
  if (rc != ANNF_OK) return rc;
  if (select_best) {
    ANNF_REQUIRE(patches_a && patches_b && P >= 1, "annf_process_rows: select_best needs both patch arrays");
    ANNF_REQUIRE(n_a == n_rows * n_cols, "annf_process_rows: patches_a must have n_rows*n_cols rows");
    ANNF_REQUIRE(n_b == h->n, "annf_process_rows: patches_b must have one row per tree point");
  }
  PatchSrc A{patches_a, 0, P, 1, 0, false, (long long)n_a * P}, B{patches_b, 0, P, 1, 0, false, (long long)n_b * P};
  return process_rows_generic(h, final_idx, A, B, ared, n_rows, n_cols, k, propagate, select_best, max_leaves,
                              knn_out, dist_out, static_cast<cudaStream_t>(stream));
}

int annf_process_rows_img(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b,
                          int hb, int wb, int channels, int psize, const void* ared, int n_rows, int n_cols, int k,
                          int propagate, int select_best, long long max_leaves, int* knn_out, float* dist_out,
                          void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(img_a, 4) && ANNF_ALIGNED(img_b, 4) && ANNF_ALIGNED(ared, 16),
               "annf_process_rows_img: images must be 4-byte and reduced patches 16-byte aligned");
  int rc = rows_common_checks(h, final_idx, ared, n_rows, n_cols, k, max_leaves);
  if (rc != ANNF_OK) return rc;
  if (select_best) {
    ANNF_REQUIRE(img_a && img_b && channels >= 1 && psize >= 1, "annf_process_rows_img: NULL image or bad geometry");
    ANNF_REQUIRE(ha - psize + 1 == n_rows && wa - psize + 1 == n_cols,
                 "annf_process_rows_img: n_rows/n_cols must match image A and psize");
    ANNF_REQUIRE((long long)(hb - psize + 1) * (wb - psize + 1) == h->n,
                 "annf_process_rows_img: the tree must hold every patch of image B");
  }
  PatchSrc A{img_a, wa, channels, psize, wa - psize + 1, true, (long long)ha * wa * channels};
  PatchSrc B{img_b, wb, channels, psize, wb - psize + 1, true, (long long)hb * wb * channels};
  return process_rows_generic(h, final_idx, A, B, ared, n_rows, n_cols, k, propagate, select_best, max_leaves,
                              knn_out, dist_out, static_cast<cudaStream_t>(stream));
}

int annf_pca_fit(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a,
                 const uint8_t* img_b, int hb, int wb, const int* pos_b, int n_b, int channels, int psize,
                 int n_components, double* components_out, double* mean_out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(img_a && img_b && components_out && mean_out, "annf_pca_fit: NULL argument");
  ANNF_REQUIRE((n_a == 0 || pos_a) && (n_b == 0 || pos_b), "annf_pca_fit: NULL positions");
  ANNF_REQUIRE(n_a >= 0 && n_b >= 0 && channels >= 1 && psize >= 1, "annf_pca_fit: bad sizes");
  ANNF_REQUIRE(psize <= ha && psize <= wa && psize <= hb && psize <= wb, "annf_pca_fit: patch larger than image");
  return pca_fit(h, img_a, ha, wa, pos_a, n_a, img_b, hb, wb, pos_b, n_b, channels, psize, n_components,
                 components_out, mean_out, 0, static_cast<cudaStream_t>(stream));
}

int annf_pca_fit_subspace(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a,
                          const uint8_t* img_b, int hb, int wb, const int* pos_b, int n_b, int channels, int psize,
                          int n_components, int iters, double* components_out, double* mean_out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(img_a && img_b && components_out && mean_out, "annf_pca_fit_subspace: NULL argument");
  ANNF_REQUIRE((n_a == 0 || pos_a) && (n_b == 0 || pos_b), "annf_pca_fit_subspace: NULL positions");
  ANNF_REQUIRE(n_a >= 0 && n_b >= 0 && channels >= 1 && psize >= 1, "annf_pca_fit_subspace: bad sizes");
  ANNF_REQUIRE(psize <= ha && psize <= wa && psize <= hb && psize <= wb,
               "annf_pca_fit_subspace: patch larger than image");
  ANNF_REQUIRE(iters >= 1 && iters <= 100, "annf_pca_fit_subspace: iters out of range");
  return pca_fit(h, img_a, ha, wa, pos_a, n_a, img_b, hb, wb, pos_b, n_b, channels, psize, n_components,
                 components_out, mean_out, iters, static_cast<cudaStream_t>(stream));
}

int annf_pca_covariance(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a,
                        const uint8_t* img_b, int hb, int wb, const int* pos_b, int n_b, int channels, int psize,
                        double* mean_out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(img_a && img_b && mean_out, "annf_pca_covariance: NULL argument");
  ANNF_REQUIRE((n_a == 0 || pos_a) && (n_b == 0 || pos_b), "annf_pca_covariance: NULL positions");
  ANNF_REQUIRE(n_a >= 0 && n_b >= 0 && channels >= 1 && psize >= 1, "annf_pca_covariance: bad sizes");
  ANNF_REQUIRE(psize <= ha && psize <= wa && psize <= hb && psize <= wb, "annf_pca_covariance: patch larger than image");
  return pca_covariance(h, img_a, ha, wa, pos_a, n_a, img_b, hb, wb, pos_b, n_b, channels, psize, mean_out,
                        static_cast<cudaStream_t>(stream));
}

int annf_pca_components(annf_handle* h, int P, int n_components, int iters, double* components_out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(components_out, "annf_pca_components: NULL argument");
  ANNF_REQUIRE(iters >= -1 && iters <= 100, "annf_pca_components: iters out of range");
  return pca_components(h, P, n_components, iters, components_out, static_cast<cudaStream_t>(stream));
}

int annf_project(annf_handle* h, const uint8_t* img, int hgt, int wid, int channels, int psize,
                 const double* components, const double* mean, int n_components, int real_type, void* out,
                 void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(img && components && mean && out, "annf_project: NULL argument");
  ANNF_REQUIRE(channels >= 1 && psize >= 1 && psize <= hgt && psize <= wid, "annf_project: bad geometry");
  ANNF_REQUIRE(real_type == ANNF_REAL_F32 || real_type == ANNF_REAL_F64, "annf_project: bad real_type");
  return project(h, img, hgt, wid, channels, psize, components, mean, n_components, real_type, out,
                 static_cast<cudaStream_t>(stream));
}

int annf_ocl_build_tree(annf_handle* h, const float* points, int n, int d, int leaf_size, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(points, "annf_ocl_build_tree: NULL points");
  ANNF_REQUIRE(ANNF_ALIGNED(points, 4), "annf_ocl_build_tree: points must be 4-byte aligned");
  return ocl_build_tree(h, points, n, d, leaf_size, static_cast<cudaStream_t>(stream));
}

int annf_ocl_tree_get(const annf_handle* h, annf_ocl_tree_view* out) {
  if (!h || !out) {
    set_error("annf_ocl_tree_get: NULL argument");
    return ANNF_ERR_INVALID;
  }
  if (!h->ocl_built) {
    set_error("annf_ocl_tree_get: no tree has been built");
    return ANNF_ERR_STATE;
  }
  out->m = h->ocl_m;
  out->d = h->ocl_d;
  out->height = h->ocl_h;
  out->n_nodes = h->ocl_q;
  out->points_per_leaf = h->ocl_ppl;
  out->m_padded = h->ocl_mp;
  out->points = h->ocl_pts.as<float>();
  out->indir = h->ocl_indir.as<int>();
  out->node_dim = h->ocl_dims.as<int>();
  out->node_val = h->ocl_vals.as<float>();
  out->node_same_dim_ancestor = h->ocl_clanc.as<int>();
  out->orig2leaf = h->ocl_o2l.as<int>();
  return ANNF_OK;
}

int annf_ocl_rows(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb,
                  int wb, int channels, int psize, const float* ared, int n_rows, int n_cols, int* knn_out,
                  float* knn_sqdist_out, float* dist_out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(final_idx && img_a && img_b && ared, "annf_ocl_rows: NULL argument");
  ANNF_REQUIRE(channels >= 1 && psize >= 1 && psize <= ha && psize <= wa && psize <= hb && psize <= wb,
               "annf_ocl_rows: bad geometry");
  return ocl_rows(h, final_idx, img_a, ha, wa, img_b, hb, wb, channels, psize, ared, n_rows, n_cols, knn_out,
                  knn_sqdist_out, dist_out, static_cast<cudaStream_t>(stream));
}

int annf_set_option(annf_handle* h, int option, int value) {
  ANNF_API_HANDLE(h);
  switch (option) {
    case ANNF_OPT_INT_PROJECTION:
      ANNF_REQUIRE(value == 0 || value == 1, "annf_set_option: ANNF_OPT_INT_PROJECTION takes 0 or 1");
      h->opt_int_projection = value;
      return ANNF_OK;
    default:
      set_error("annf_set_option: unknown option " + std::to_string(option));
      return ANNF_ERR_INVALID;
  }
}

int annf_device_status(annf_handle* h, void* stream, unsigned* bits_out) {
  ANNF_API_HANDLE(h);
  unsigned bits = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  ANNF_CUDA_TRY(cudaMemcpyAsync(&bits, h->status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  ANNF_CUDA_TRY(cudaStreamSynchronize(st));
  ANNF_CUDA_TRY(cudaMemsetAsync(h->status.p, 0, sizeof(unsigned), st));
  if (bits_out) *bits_out = bits;
  if (bits) {
    set_error("device bounds check tripped (status bits " + std::to_string(bits) + ")");
    return ANNF_ERR_DEVICE;
  }
  return ANNF_OK;
}

int annf_kneighbors_noalloc(annf_handle* h, const void* queries, int nq, int k, long long max_leaves, void* distances,
                            int* indices, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(queries, 16), "annf_kneighbors_noalloc: queries must be 16-byte aligned");
  int rc = check_k(h, k, max_leaves);
  if (rc != ANNF_OK) return rc;
  ANNF_REQUIRE(nq >= 0, "annf_kneighbors_noalloc: nq < 0");
  if (nq == 0) return ANNF_OK;
  ANNF_REQUIRE(queries && distances && indices, "annf_kneighbors_noalloc: NULL array");
  return kneighbors_noalloc(h, queries, nq, k, max_leaves, distances, indices, static_cast<cudaStream_t>(stream));
}

// tensor-core tile precision of natural_knn_tc: 0 BF16 split, 1 FP16, 2 FP8 (E4M3) split
static int leaf_tc_prec(int leaf_precision) {
  return leaf_precision == ANNF_LEAF_FP16 ? 1 : leaf_precision == ANNF_LEAF_FP8 ? 2 : 0;
}

static int parallel_nnf_impl(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa,
                             const uint8_t* img_b, int hb, int wb, int channels, int psize, const void* ared, int k,
                             const int* proposals, int n_prop, const int* seed_match, int iters, unsigned seed,
                             int leaf_precision, int rand_samples, int radius0, float* dist_out, void* stream) {
  ANNF_REQUIRE(ANNF_ALIGNED(img_a, 16) && ANNF_ALIGNED(img_b, 16) && ANNF_ALIGNED(ared, 16),
               "annf_parallel_nnf: images and reduced patches must be 16-byte aligned");
  int rc = check_k(h, k, 2147483640);
  if (rc != ANNF_OK) return rc;
  ANNF_REQUIRE(final_idx && img_a && img_b && ared, "annf_parallel_nnf: NULL argument");
  ANNF_REQUIRE(channels >= 1 && psize >= 1 && psize <= ha && psize <= wa && psize <= hb && psize <= wb,
               "annf_parallel_nnf: bad geometry");
  ANNF_REQUIRE((long long)(hb - psize + 1) * (wb - psize + 1) == h->n,
               "annf_parallel_nnf: the tree must hold every patch of image B");
  ANNF_REQUIRE(n_prop >= 0 && (n_prop == 0 || proposals), "annf_parallel_nnf: bad proposals");
  ANNF_REQUIRE(iters >= 0 && iters <= 64, "annf_parallel_nnf: iters out of range");
  ANNF_REQUIRE(rand_samples >= 0 && rand_samples <= 16 && radius0 >= 1 && radius0 <= 4096,
               "annf_parallel_nnf: bad search schedule");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long nA = (long long)(ha - psize + 1) * (wa - psize + 1);
  ANNF_ENSURE(h->fast_nat, (size_t)nA * k * sizeof(int));
  ANNF_REQUIRE(leaf_precision == ANNF_LEAF_EXACT || leaf_precision == ANNF_LEAF_BF16 ||
                   leaf_precision == ANNF_LEAF_FP16 || leaf_precision == ANNF_LEAF_FP8,
               "annf_parallel_nnf: bad leaf_precision");
  ANNF_REQUIRE(leaf_precision == ANNF_LEAF_EXACT || leaf_tc_supported(h, k),
               "annf_parallel_nnf: tensor-core leaf distances need FP32 points, d <= 32, leaves <= 256, k <= 32");
  prof_mark(h, "parallel:begin", st);
  if (leaf_precision != ANNF_LEAF_EXACT)
    rc = natural_knn_tc(h, static_cast<const float*>(ared), nA, k, leaf_tc_prec(leaf_precision),
                        h->fast_nat.as<int>(), st);
  else
    rc = natural_knn_all(h, ared, nA, k, h->fast_nat.as<int>(), st);
  if (rc != ANNF_OK) return rc;
  prof_mark(h, "natural_knn", st);
  return fast_search(h, img_a, ha, wa, img_b, hb, wb, channels, psize, k, h->fast_nat.as<int>(), proposals, n_prop,
                     seed_match, iters, seed, rand_samples, radius0, final_idx, dist_out, st);
}

int annf_parallel_nnf(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b,
                      int hb, int wb, int channels, int psize, const void* ared, int k, const int* proposals,
                      int n_prop, int iters, unsigned seed, int leaf_precision, int rand_samples, int radius0,
                      float* dist_out, void* stream) {
  ANNF_API_HANDLE(h);
  return parallel_nnf_impl(h, final_idx, img_a, ha, wa, img_b, hb, wb, channels, psize, ared, k, proposals, n_prop,
                           nullptr, iters, seed, leaf_precision, rand_samples, radius0, dist_out, stream);
}

int annf_parallel_nnf_seeded(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa,
                             const uint8_t* img_b, int hb, int wb, int channels, int psize, const void* ared, int k,
                             const int* seed_match, int iters, unsigned seed, int leaf_precision, int rand_samples,
                             int radius0, float* dist_out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(seed_match, "annf_parallel_nnf_seeded: NULL seed");
  return parallel_nnf_impl(h, final_idx, img_a, ha, wa, img_b, hb, wb, channels, psize, ared, k, nullptr, 0,
                           seed_match, iters, seed, leaf_precision, rand_samples, radius0, dist_out, stream);
}

int annf_seed_matches(annf_handle* h, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb, int wb,
                      int channels, int psize, const int* candidates, int n_cand, int* seed_out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(img_a && img_b && seed_out && (n_cand == 0 || candidates), "annf_seed_matches: NULL argument");
  ANNF_REQUIRE(ANNF_ALIGNED(img_a, 16) && ANNF_ALIGNED(img_b, 16), "annf_seed_matches: images must be 16-byte aligned");
  ANNF_REQUIRE(channels >= 1 && psize >= 1 && psize <= ha && psize <= wa && psize <= hb && psize <= wb && n_cand >= 0,
               "annf_seed_matches: bad geometry");
  return seed_matches(img_a, ha, wa, img_b, hb, wb, channels, psize, candidates, n_cand, seed_out,
                      static_cast<cudaStream_t>(stream));
}

int annf_raw_nn(annf_handle* h, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb, int wb,
                int channels, int psize, const int* query_pixels, int nq, unsigned long long* best, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(img_a, 4) && ANNF_ALIGNED(img_b, 4), "annf_raw_nn: images must be 4-byte aligned");
  ANNF_REQUIRE(img_a && img_b && (nq == 0 || (query_pixels && best)), "annf_raw_nn: NULL argument");
  ANNF_REQUIRE(channels >= 1 && psize >= 1 && psize <= ha && psize <= wa && psize <= hb && psize <= wb,
               "annf_raw_nn: bad geometry");
  if (nq == 0) return ANNF_OK;
  return raw_nn(img_a, ha, wa, img_b, hb, wb, channels, psize, query_pixels, nq, best,
                static_cast<cudaStream_t>(stream));
}

int annf_project_f16(annf_handle* h, const uint8_t* img, int hgt, int wid, int channels, int psize,
                      const double* components, const double* mean, int n_components, float* out, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(img, 4), "annf_project_f16: the image must be 4-byte aligned");
  ANNF_REQUIRE(img && components && mean && out, "annf_project_f16: NULL argument");
  ANNF_REQUIRE(channels >= 1 && psize >= 1 && psize <= hgt && psize <= wid, "annf_project_f16: bad geometry");
  if (!project_tc_supported(psize, channels, n_components)) {
    set_error("annf_project_f16: needs psize*psize*channels <= 256 and n_components <= 32");
    return ANNF_ERR_UNSUPPORTED;
  }
  return project_tc(h, img, hgt, wid, channels, psize, components, mean, n_components, out,
                    static_cast<cudaStream_t>(stream));
}

int annf_natural_knn(annf_handle* h, const void* queries, long long nq, int k, int leaf_precision, int* out_pos,
                     void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(queries, 16), "annf_natural_knn: queries must be 16-byte aligned");
  int rc = check_k(h, k, 2147483640);
  if (rc != ANNF_OK) return rc;
  ANNF_REQUIRE(nq >= 0, "annf_natural_knn: nq < 0");
  if (nq == 0) return ANNF_OK;
  ANNF_REQUIRE(queries && out_pos, "annf_natural_knn: NULL argument");
  ANNF_REQUIRE(leaf_precision == ANNF_LEAF_EXACT || leaf_precision == ANNF_LEAF_BF16 ||
                   leaf_precision == ANNF_LEAF_FP16 || leaf_precision == ANNF_LEAF_FP8,
               "annf_natural_knn: bad leaf_precision");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (leaf_precision != ANNF_LEAF_EXACT) {
    ANNF_REQUIRE(leaf_tc_supported(h, k), "annf_natural_knn: tensor-core leaf distances need FP32 points, "
                                          "d <= 32, leaves <= 256, k <= 32");
    return natural_knn_tc(h, static_cast<const float*>(queries), nq, k, leaf_tc_prec(leaf_precision),
                          out_pos, st);
  }
  return natural_knn_all(h, queries, nq, k, out_pos, st);
}

int annf_tc_tile(annf_handle* h, const uint16_t* a, const uint16_t* b, int n, int kdim, float* d, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(a, 16) && ANNF_ALIGNED(b, 16), "annf_tc_tile: a and b must be 16-byte aligned");
  ANNF_REQUIRE(a && b && d, "annf_tc_tile: NULL argument");
  return tc_tile(a, b, n, kdim, d, h->status.as<unsigned>(), static_cast<cudaStream_t>(stream));
}

// ---- offset-proposal network ----
#define ANNF_CNN_DIMS(nimg, h, w) \
  ANNF_REQUIRE((nimg) >= 1 && (h) >= 1 && (w) >= 1, "annf_cnn: bad tensor shape")

int annf_cnn_input(annf_handle* h, const uint8_t* img_a, const uint8_t* img_b, int hgt, int wid, void* x_out,
                   void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(img_a && img_b && x_out, "annf_cnn_input: NULL argument");
  return cnn_input(img_a, img_b, hgt, wid, x_out, static_cast<cudaStream_t>(stream));
}

int annf_cnn_prep_weights(annf_handle* h, const float* w, int co, int ci, float* w_fwd, float* w_bwd, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(w && w_fwd && co >= 1 && ci >= 1, "annf_cnn_prep_weights: bad argument");
  return cnn_prep_weights(w, co, ci, w_fwd, w_bwd, static_cast<cudaStream_t>(stream));
}

int annf_cnn_conv_forward(annf_handle* h, const void* x, int nimg, int hgt, int wid, int ci, int co,
                          const float* w_fwd, const float* bias, int relu, void* y, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(x && w_fwd && bias && y, "annf_cnn_conv_forward: NULL argument");
  ANNF_CNN_DIMS(nimg, hgt, wid);
  return cnn_conv_forward(x, nimg, hgt, wid, ci, co, w_fwd, bias, relu, y, h->status.as<unsigned>(),
                          static_cast<cudaStream_t>(stream));
}

int annf_cnn_prep_weights_tc(annf_handle* h, const float* w, int co, int ci, uint16_t* w_tc, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(w && w_tc, "annf_cnn_prep_weights_tc: NULL argument");
  return cnn_prep_weights_tc(w, co, ci, w_tc, static_cast<cudaStream_t>(stream));
}

int annf_cnn_conv_forward_tc(annf_handle* h, const void* x, int nimg, int hgt, int wid, int ci, int co,
                             const uint16_t* w_tc, const float* bias, int relu, void* y, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(ANNF_ALIGNED(x, 16) && ANNF_ALIGNED(w_tc, 16), "annf_cnn_conv_forward_tc: x and w_tc must be 16-byte aligned");
  ANNF_REQUIRE(x && w_tc && bias && y, "annf_cnn_conv_forward_tc: NULL argument");
  ANNF_CNN_DIMS(nimg, hgt, wid);
  return cnn_conv_forward_tc(x, nimg, hgt, wid, ci, co, w_tc, bias, relu, y, h->status.as<unsigned>(),
                             static_cast<cudaStream_t>(stream));
}

int annf_cnn_conv_backward_data(annf_handle* h, const float* g, const void* mask, int nimg, int hgt, int wid, int co,
                                int ci, const float* w_bwd, float* dx, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(g && w_bwd && dx, "annf_cnn_conv_backward_data: NULL argument");
  ANNF_CNN_DIMS(nimg, hgt, wid);
  return cnn_conv_backward_data(g, mask, nimg, hgt, wid, co, ci, w_bwd, dx, h->status.as<unsigned>(),
                                static_cast<cudaStream_t>(stream));
}

int annf_cnn_conv_backward_weights(annf_handle* h, const void* x, const float* g, const void* mask, int nimg, int hgt,
                                   int wid, int ci, int co, float* dw, float* db, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(x && g && dw && db, "annf_cnn_conv_backward_weights: NULL argument");
  ANNF_CNN_DIMS(nimg, hgt, wid);
  return cnn_conv_backward_weights(x, g, mask, nimg, hgt, wid, ci, co, dw, db, h->status.as<unsigned>(),
                                   static_cast<cudaStream_t>(stream));
}

int annf_cnn_wta_loss(annf_handle* h, const float* out, const float* tgt, const uint8_t* valid, long long npix,
                      float inv_nvalid, float* dout, float* loss_sum, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(out && tgt && valid && dout && loss_sum && npix >= 0, "annf_cnn_wta_loss: bad argument");
  return cnn_wta_loss(out, tgt, valid, npix, inv_nvalid, dout, loss_sum, static_cast<cudaStream_t>(stream));
}

int annf_cnn_adam(annf_handle* h, float* param, const float* grad, float* m, float* v, int n, float lr, float beta1,
                  float beta2, float eps, int step, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(param && grad && m && v && n >= 0 && step >= 1, "annf_cnn_adam: bad argument");
  return cnn_adam(param, grad, m, v, n, lr, beta1, beta2, eps, step, static_cast<cudaStream_t>(stream));
}

int annf_cnn_targets(annf_handle* h, const int* nnf, int ha, int wa, int wb, int psize, float* tgt, uint8_t* valid,
                     void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(nnf && tgt && valid && psize >= 1 && psize <= ha && psize <= wa && ha >= 4 && wa >= 4,
               "annf_cnn_targets: bad argument");
  return cnn_targets(nnf, ha, wa, wb, psize, tgt, valid, static_cast<cudaStream_t>(stream));
}

int annf_cnn_proposals(annf_handle* h, const float* out, int h4, int w4, int ha, int wa, int hb, int wb, int psize,
                       int* props, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(out && props && h4 >= 1 && w4 >= 1 && psize >= 1 && psize <= ha && psize <= wa && psize <= hb &&
                   psize <= wb,
               "annf_cnn_proposals: bad argument");
  return cnn_proposals(out, h4, w4, ha, wa, hb, wb, psize, 4, props, static_cast<cudaStream_t>(stream));
}

int annf_cnn_proposals_per_pixel(annf_handle* h, const float* out, int h4, int w4, int ha, int wa, int hb, int wb,
                                 int psize, int per_pixel, int* props, void* stream) {
  ANNF_API_HANDLE(h);
  ANNF_REQUIRE(out && props && h4 >= 1 && w4 >= 1 && psize >= 1 && psize <= ha && psize <= wa && psize <= hb &&
                   psize <= wb,
               "annf_cnn_proposals_per_pixel: bad argument");
  ANNF_REQUIRE(per_pixel == 1 || per_pixel == 2 || per_pixel == 4, "annf_cnn_proposals_per_pixel: per_pixel must be 1, 2 or 4");
  return cnn_proposals(out, h4, w4, ha, wa, hb, wb, psize, per_pixel, props, static_cast<cudaStream_t>(stream));
}

long long annf_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

long long annf_buffer_epoch(void) { return g_reallocs.load(std::memory_order_relaxed); }

int annf_profile_enable(annf_handle* h, int on) {
  ANNF_API_HANDLE(h);
  h->prof_on = on ? 1 : 0;
  h->prof_used = 0;
  return ANNF_OK;
}

int annf_profile_read(annf_handle* h, void* stream, int cap, float* ms, const char** names) {
  ANNF_API_HANDLE(h);
  ANNF_CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  int n = 0;
  for (int i = 1; i < h->prof_used && n < cap; ++i, ++n) {
    float t = 0.f;
    ANNF_CUDA_TRY(cudaEventElapsedTime(&t, h->prof_ev[i - 1], h->prof_ev[i]));
    if (ms) ms[n] = t;
    if (names) names[n] = h->prof_name[i];
  }
  h->prof_used = 0;
  return n;
}

}  // extern "C"
