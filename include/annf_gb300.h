/*
 * annf_gb300.h -- C ABI of the GB300 (sm_103a) nearest-neighbour-field library.
 *
 * The library replaces the native core of annfmp's OpenMP backend. Each entry point below names
 * the reference interface it stands in for (paths within the annfmp project). All pointers to
 * array data are DEVICE pointers unless a parameter says "host"; the caller owns every input and
 * output buffer. A handle owns the device tree and its scratch memory and frees them in
 * annf_destroy. Calls are asynchronous on the given CUDA stream (NULL = legacy default stream);
 * a handle must not be used from two host threads at once. Images and patch arrays must start on a
 * 4-byte boundary, reduced-patch / query arrays on a 16-byte boundary, and the images of
 * annf_parallel_nnf on a 16-byte boundary (cudaMalloc returns 256-byte aligned memory); a call
 * whose pointers are not aligned returns ANNF_ERR_INVALID. No kernel reads past the end of a
 * buffer.
 *
 * Every function returns ANNF_OK (0) or a negative status; annf_last_error() then describes the
 * failure (thread-local). The reference prints and calls exit() instead
 * (annfmp/openmp/kdtree/src/helper.c:30-52, kdtree.c:403-407).
 */
#ifndef ANNF_GB300_H_
#define ANNF_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ANNF_OK 0
#define ANNF_ERR_INVALID -1     /* bad argument (shape, range, null pointer) */
#define ANNF_ERR_UNSUPPORTED -2 /* valid for the reference, not supported here (e.g. k > 32 in process_rows) */
#define ANNF_ERR_CUDA -3        /* a CUDA runtime call or launch failed */
#define ANNF_ERR_ALLOC -4       /* device allocation failed */
#define ANNF_ERR_STATE -5       /* call order (e.g. query before a tree was built) */
#define ANNF_ERR_DEVICE -6      /* a kernel's own bounds check tripped (see annf_device_status) */
#define ANNF_ERR_SOLVER -7      /* the eigen-solver reported failure */

/* scalar type of reduced patches / tree points (reference FLOAT_TYPE, include/float.h:16-26) */
#define ANNF_REAL_F32 0
#define ANNF_REAL_F64 1

/* split-axis rule (reference SPLITTING_TYPE_*, annfmp/openmp/kdtree/src/include/global.h:18-19) */
#define ANNF_SPLIT_CYCLIC 0  /* axis = node depth mod d */
#define ANNF_SPLIT_LONGEST 1 /* first axis of strictly largest bounding-box width */

/* leaf-distance precision of annf_natural_knn and annf_parallel_nnf* (the row propagation of
 * annf_process_rows* always scans its leaves exactly) */
#define ANNF_LEAF_EXACT 0 /* FP32/FP64 with the reference's summation order */
#define ANNF_LEAF_BF16 1  /* BF16 tensor-core tiles (FP32 accumulate) + exact FP32 re-rank of the survivors */
#define ANNF_LEAF_FP16 2  /* the same with FP16 tiles (tighter bound, fewer survivors) */
#define ANNF_LEAF_FP8 3   /* FP8 (E4M3) hi/lo split tiles with power-of-two scales (wider bound, more survivors) */

/* options (annf_set_option) */
#define ANNF_OPT_INT_PROJECTION 1 /* 1: annf_project always evaluates the exact integer sums with dp4a
                                     (default 0: on the tensor cores where the shape allows; the same
                                     integers, so the same bits) */

typedef struct annf_handle annf_handle;

/* Tree arrays as device pointers (structure-of-arrays form of the reference KD_TREE_RECORD,
 * annfmp/openmp/kdtree/src/include/global.h:40-50). */
typedef struct {
  int n, d, depth, real_type;
  int n_leaves;            /* 2^depth */
  const void* points;      /* [n*d] points in tree order (reference XI float part) */
  const int* perm;         /* [n] tree position -> original index (reference XI index part) */
  const int* node_axis;    /* [2^depth-1] heap order (reference nodes[].axis) */
  const void* node_split;  /* [2^depth-1] (reference nodes[].splitting_value) */
  const int* leaf_begin;   /* [2^depth+1]; leaf l = [leaf_begin[l], leaf_begin[l+1]) (reference leaves[]) */
  const int* point_leaf;   /* [n] original index -> leaf (reference points_leaf_indices) */
  const void* leaf_box;    /* [2^depth][2][d]: per leaf the min, then the max, of each coordinate
                              (no reference counterpart: lower bounds of the exact search) */
} annf_tree_view;

int annf_version(void);
const char* annf_last_error(void);

/* Create / destroy a handle bound to a CUDA device. Stands in for the parameter/record setup of
 * init_extern (annfmp/openmp/kdtree/src/base.c:22-43, include/base.h:36-42). */
int annf_create(annf_handle** out, int device);
void annf_destroy(annf_handle* h);

/* Build the k-d tree over n points of dimension d (row-major device array, real_type scalars) to
 * the given depth: longest-bounding-box axis, split at the order statistic of rank count/2,
 * reference element order. Replaces fit_extern (annfmp/openmp/kdtree/src/base.c:54-69,
 * include/base.h:55-60). Tree depth is chosen by the caller as the reference Python does
 * (annfmp/openmp/kdtree/base.py:260-300). */
int annf_build_tree(annf_handle* h, const void* points, int n, int d, int real_type, int depth,
                    int splitting_type, void* stream);

/* Device pointers of the current tree (valid until the next build or annf_destroy). */
int annf_tree_get(const annf_handle* h, annf_tree_view* out);

/* Exact k nearest neighbours of nq queries ([nq*d], real_type of the tree). distances [nq*k]
 * (Euclidean, i.e. square-rooted) and indices [nq*k] (original point indices), best first.
 * At most max_leaves leaves are scanned, in the reference's depth-first order (exact when
 * max_leaves >= 2^depth; the reference's default is 2147483640). 1 <= k <= 1000 as in the
 * reference (k above 32 runs a kernel with the k-list in shared memory, one CTA per query).
 * Replaces neighbors_extern (annfmp/openmp/kdtree/src/base.c:88-132, include/base.h:67-78). */
int annf_kneighbors(annf_handle* h, const void* queries, int nq, int k, long long max_leaves,
                    void* distances, int* indices, void* stream);

/* No counterpart in the reference. The same exact k nearest neighbours as annf_kneighbors (same
 * results), for callers that must not allocate device memory while they query: serving processes
 * whose device memory is reserved ahead of time, host applications that own all device memory
 * through their own pool, or allocators that refuse to grow. Build the tree first (that
 * allocates); this call then allocates nothing. Its scratch is one static device array shared by
 * all calls, sized for nq * k <= 262144 for both real types (5 MiB: a 16-byte double seed key and
 * a 4-byte position per entry, held by every GPU that loads the library until exit); larger
 * requests fail with ANNF_ERR_INVALID. The first call on each device looks the array's device
 * address up (cudaGetSymbolAddress), so make that first call before any stream capture. Calls that
 * overlap on the GPU (unordered streams) race on the shared scratch. The unbudgeted search always
 * scans every leaf box per query (one warp per query), so many queries on a deep tree run slower
 * here than through annf_kneighbors, which switches to its tiled box scan. */
int annf_kneighbors_noalloc(annf_handle* h, const void* queries, int nq, int k, long long max_leaves,
                            void* distances, int* indices, void* stream);

/* The row-propagation NNF over an n_rows x n_cols grid of A patches (reduced, [n_rows*n_cols*d]
 * real_type, row-major pixels). Raw uint8 patches come as arrays: patches_a [n_a*P],
 * patches_b [n_b*P] (may be NULL when select_best == 0).
 *   final_idx  [n_rows*n_cols]  chosen B index per pixel (output)
 *   knn_out    [n_rows*n_cols*k] optional (NULL): each pixel's k-list as original B indices
 *   dist_out   [n_rows*n_cols]   optional (NULL): raw-patch L2 of the chosen index (select_best)
 * Replaces process_rows_extern (annfmp/openmp/kdtree/src/base.c:150-360, include/base.h:81-98). */
int annf_process_rows(annf_handle* h, int* final_idx, const uint8_t* patches_a, int n_a,
                      const uint8_t* patches_b, int n_b, int P, const void* ared, int n_rows,
                      int n_cols, int k, int propagate, int select_best, long long max_leaves,
                      int* knn_out, float* dist_out, void* stream);

/* As annf_process_rows, but raw patches are read from the images themselves (uint8 HxWxC,
 * row-major, channel fastest; patch (y,x) = rows y..y+psize-1, cols x..x+psize-1), so the
 * 1 GB-scale patch arrays of the reference are never materialised. */
int annf_process_rows_img(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa,
                          const uint8_t* img_b, int hb, int wb, int channels, int psize,
                          const void* ared, int n_rows, int n_cols, int k, int propagate,
                          int select_best, long long max_leaves, int* knn_out, float* dist_out,
                          void* stream);

/* PCA fit on sampled patches of both images (annfmp/openmp/base.py:168-191 with scikit-learn's
 * covariance_eigh solver): Gram matrix accumulated exactly, covariance finished in FP64 in the
 * solver's own operation order, then the leading eigenvectors in FP64 on the GPU (subspace
 * iteration over all SMs on a block of min(40, P) vectors and an FP64 Rayleigh-Ritz step; the
 * library's full eigendecomposition beyond 40 components), sorted by decreasing eigenvalue with
 * the sign convention "largest |entry| positive".
 *   pos_a [n_a*2], pos_b [n_b*2]: (row, col) of the sampled patches (int32, device)
 *   components_out [n_components*P] FP64, mean_out [P] FP64 (device) */
int annf_pca_fit(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a,
                 const uint8_t* img_b, int hb, int wb, const int* pos_b, int n_b, int channels,
                 int psize, int n_components, double* components_out, double* mean_out,
                 void* stream);

/* As annf_pca_fit, but only the leading n_components are computed (an addition for the
 * approximate NNF forms; the reference has no counterpart): the same exact Gram matrix and FP64
 * covariance, then `iters` steps of FP32 subspace iteration on a block of n_components +
 * max(8, n_components/2) vectors, a Rayleigh-Ritz step and the small eigenproblem in FP64, and the
 * same sign convention. Falls back to the full solver when P < 2 * block or the block exceeds 40. */
int annf_pca_fit_subspace(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a,
                          const uint8_t* img_b, int hb, int wb, const int* pos_b, int n_b, int channels,
                          int psize, int n_components, int iters, double* components_out,
                          double* mean_out, void* stream);

/* The two halves of annf_pca_fit / annf_pca_fit_subspace, for callers that want work of their own
 * between them (no reference counterpart): annf_pca_covariance forms the covariance of the sampled
 * patches (kept on the handle) and writes the mean; annf_pca_components then writes the leading
 * components (iters 0: the drop-in result, as annf_pca_fit; iters -1: the full FP64
 * eigendecomposition by the library solver; iters > 0: FP32 subspace iteration with that many
 * steps and an FP64 Rayleigh-Ritz step). P = psize * psize * channels. */
int annf_pca_covariance(annf_handle* h, const uint8_t* img_a, int ha, int wa, const int* pos_a, int n_a,
                        const uint8_t* img_b, int hb, int wb, const int* pos_b, int n_b, int channels,
                        int psize, double* mean_out, void* stream);
int annf_pca_components(annf_handle* h, int P, int n_components, int iters, double* components_out,
                        void* stream);

/* Project every psize x psize patch of an image onto the components
 * (annfmp/openmp/base.py:193-200: X @ C^T - mean @ C^T in FP64, cast to real_type). The
 * product is evaluated exactly in integer arithmetic on split coefficients (each coefficient as
 * 8 signed 7-bit digits; the digit sums on the tensor cores for FP32 output of images with at
 * most 4 channels, else with dp4a), so the result is the FP64 value rounded once.
 * out [(h-psize+1)*(w-psize+1)*n_components], row-major pixels. */
int annf_project(annf_handle* h, const uint8_t* img, int hgt, int wid, int channels, int psize,
                 const double* components, const double* mean, int n_components, int real_type,
                 void* out, void* stream);

/* ---- openclopt semantics: the NNF algorithm of annfmp's GPU backend ---------------------------
 * (annfmp/openclopt/src/futhark/driverKNN.fut and the files it imports, driven by
 * annfmp/openclopt/src/base.c:fit_extern, which the
 * reference runs through Futhark-generated code) as a mode of this library, for comparison with
 * that backend: K is 8 whatever the caller's n_neighbors; the tree has 2^(height+1) leaves of
 * exactly points_per_leaf points (the input padded with +inf rows to m_padded), each node split
 * at the mean of the two middle values of a stable sort of its points by the widest side of its
 * box (lowest dimension on ties); descent goes left on "<="; the first row is searched exactly by
 * the backend's incremental-distance traversal; propagated leaves are deduplicated against the
 * natural leaf, "one row below" clamped to the last row; select best by squared raw-patch
 * distance. FP32 only. */
typedef struct {
  int m, d;                 /* points (before padding), dimension */
  int height;               /* levels of internal nodes minus one (-1: a single leaf) */
  int n_nodes;              /* internal nodes: 2^(height+1) - 1 */
  int points_per_leaf, m_padded;
  const float* points;      /* [m_padded*d] leaf order, +inf pads */
  const int* indir;         /* [m_padded] leaf-order position -> original index (>= m: a pad) */
  const int* node_dim;      /* [n_nodes] heap order */
  const float* node_val;    /* [n_nodes] */
  const int* node_same_dim_ancestor;  /* [n_nodes] closest ancestor splitting the same dim, -1 none */
  const int* orig2leaf;     /* [m_padded] */
} annf_ocl_tree_view;

/* Build the backend's tree over points [n*d] FP32 (device) with leaf_size as the default points
 * per leaf. Replaces the buildKDtree entry (annfmp/openclopt/src/futhark/driverKNN.fut:142-151,
 * buildKDtree.fut:17-157). At most 1024 points per leaf. */
int annf_ocl_build_tree(annf_handle* h, const float* points, int n, int d, int leaf_size, void* stream);
int annf_ocl_tree_get(const annf_handle* h, annf_ocl_tree_view* out);

/* The NNF of image A against the tree over image B's reduced patches, from A's reduced patches
 * ared [n_rows*n_cols*d] FP32: natural-leaf lists (findNaturalLeavesFixK, driverKNN.fut:153-204),
 * the exact first row (exactKnnFixK, :231-290), row propagation (propagateFixK, :305-413), select
 * best (selectBestNN, :90-133). Outputs: final_idx [n] original B indices; optional knn_out [n*8]
 * original indices (-1: none), knn_sqdist_out [n*8] squared reduced distances, dist_out [n]
 * raw-patch L2 of the choice. */
int annf_ocl_rows(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b,
                  int hb, int wb, int channels, int psize, const float* ared, int n_rows, int n_cols,
                  int* knn_out, float* knn_sqdist_out, float* dist_out, void* stream);

/* Set a per-handle option (ANNF_OPT_*). No counterpart in the reference: a knob of this
 * implementation that changes no result. */
int annf_set_option(annf_handle* h, int option, int value);

/* Approximate counterpart of annf_project for the approximate NNF forms (no reference
 * counterpart): the same patches times the components rounded to FP16, FP32 accumulation on the
 * tensor cores (tcgen05), minus the projected mean; out FP32 [(h-psize+1)*(w-psize+1)*n_components].
 * Images of 1 to 4 channels are read by the tensor cores from FP16 copies of their rows (no
 * per-patch expansion); others through an expanded tile. Needs psize*psize*channels <= 256 and
 * n_components <= 32 (else ANNF_ERR_UNSUPPORTED). */
int annf_project_f16(annf_handle* h, const uint8_t* img, int hgt, int wid, int channels, int psize,
                     const double* components, const double* mean, int n_components, float* out, void* stream);

/* The parallel NNF form (an addition beside the reference's row-sequential method, which has no
 * counterpart for it): every pixel's natural-leaf k-list (leaf_precision ANNF_LEAF_EXACT: FP32
 * leaf scan; ANNF_LEAF_BF16 / _FP16 / _FP8: queries grouped by leaf, tensor-core distance tiles,
 * exact FP32 re-rank of every point within the tiles' proven error bound, so the same k-list as
 * the FP32 scan), optional offset proposals
 * (proposals [n_rows*n_cols*n_prop] B patch indices, -1 = none) and `iters` parallel passes of
 * neighbour propagation and random search (rand_samples offsets per pass within radius0 >> pass
 * of the current match, at least 1); every candidate is verified with the exact integer
 * raw-patch SSD. Requires the tree over image B's reduced patches (annf_build_tree). Outputs the
 * chosen B index per pixel and, optionally, its raw-patch L2 distance. */
int annf_parallel_nnf(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa,
                      const uint8_t* img_b, int hb, int wb, int channels, int psize, const void* ared,
                      int k, const int* proposals, int n_prop, int iters, unsigned seed,
                      int leaf_precision, int rand_samples, int radius0, float* dist_out, void* stream);

/* Best of n_cand candidate B patches per A pixel (candidates [n_rows*n_cols*n_cand] B indices, -1 =
 * none) by exact integer raw-patch SSD, as a match array seed_out [2*n_rows*n_cols]: the B index
 * (-1 if no candidate is valid), then the SSD (INT32_MAX if none); ties go to the smaller index.
 * Needs no tree: the caller can run it on a second stream while the PCA fit and the tree run (the
 * learned proposals' candidates are known before them). No reference counterpart. */
int annf_seed_matches(annf_handle* h, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb,
                      int wb, int channels, int psize, const int* candidates, int n_cand, int* seed_out,
                      void* stream);

/* annf_parallel_nnf starting from a seed match (annf_seed_matches' output) instead of proposals:
 * the initial choice is the best of the seed and the natural-leaf k-list, which equals
 * annf_parallel_nnf with the seed's candidates as proposals. No reference counterpart. */
int annf_parallel_nnf_seeded(annf_handle* h, int* final_idx, const uint8_t* img_a, int ha, int wa,
                             const uint8_t* img_b, int hb, int wb, int channels, int psize,
                             const void* ared, int k, const int* seed_match, int iters, unsigned seed,
                             int leaf_precision, int rand_samples, int radius0, float* dist_out,
                             void* stream);

/* Exact raw-patch nearest neighbour (integer SSD over all B patches) of nq sampled A pixels
 * (query_pixels: row-major patch indices). best[i] = ssd << 32 | B index (smallest index on
 * ties). The reference for distance-error measurements; the reference project has no counterpart. */
int annf_raw_nn(annf_handle* h, const uint8_t* img_a, int ha, int wa, const uint8_t* img_b, int hb,
                int wb, int channels, int psize, const int* query_pixels, int nq,
                unsigned long long* best, void* stream);

/* The k nearest points of each query inside the leaf its descent reaches (no backtracking; the
 * reference's traversal with max_leaves = 1, kdtree.c:129-268 with only_leaf_idx). out_pos
 * [nq*k] tree positions (annf_tree_view.perm maps them to original indices), nearest first.
 * ANNF_LEAF_EXACT scans the leaf in FP32 (reference order); ANNF_LEAF_BF16 / _FP16 / _FP8 group
 * the queries by leaf and compute tensor-core distance tiles, re-ranking exactly in FP32 every
 * point within the tiles' proven error bound, so the k-lists equal the FP32 scan's. */
int annf_natural_knn(annf_handle* h, const void* queries, long long nq, int k, int leaf_precision,
                     int* out_pos, void* stream);

/* One 128 x n tile of the tensor-core path, for numerics checks (no counterpart in the reference):
 * d[128][n] = a[128][kdim] . b[n][kdim]^T, a and b BF16 (raw 16-bit, row-major), d FP32, computed by
 * tcgen05.mma from shared-memory core-matrix tiles into tensor memory. n, kdim multiples of 16,
 * n <= 256, kdim <= 256. */
int annf_tc_tile(annf_handle* h, const uint16_t* a, const uint16_t* b, int n, int kdim, float* d,
                 void* stream);

/* ---- offset-proposal network (an addition: the reference's only propagation candidates are the
 * row above, annfmp/openmp/kdtree/src/base.c:255-282). Tensors are NHWC, activations BF16 (raw
 * 16-bit), gradients and weights FP32; six 3x3 layers 8->32, 32->32 x4, 32->8. ---- */

/* x_out [hgt/4][wid/4][8] BF16: 4x4 box means of A.rgb and B.rgb, (v - 127.5) / 64, then 0, 0. */
int annf_cnn_input(annf_handle* h, const uint8_t* img_a, const uint8_t* img_b, int hgt, int wid, void* x_out,
                   void* stream);
/* w [co][3][3][ci] FP32 -> w_fwd [9][ci][co] and (optional) w_bwd [9][co][ci] (flipped taps), both
 * rounded to BF16 values. */
int annf_cnn_prep_weights(annf_handle* h, const float* w, int co, int ci, float* w_fwd, float* w_bwd, void* stream);
/* y = conv3x3(x) + bias (zero padding); relu=1: ReLU, BF16 y; relu=0: FP32 y. (ci, co) in
 * {(8,32), (32,32), (32,8)}. */
int annf_cnn_conv_forward(annf_handle* h, const void* x, int nimg, int hgt, int wid, int ci, int co,
                          const float* w_fwd, const float* bias, int relu, void* y, void* stream);
/* The same forward convolution on the tensor cores (tcgen05 implicit GEMM, M = 128 pixels,
 * K = 9 x ci): w_tc [co padded to 16/32][9*ci padded to 16] BF16 from annf_cnn_prep_weights_tc. */
int annf_cnn_prep_weights_tc(annf_handle* h, const float* w, int co, int ci, uint16_t* w_tc, void* stream);
int annf_cnn_conv_forward_tc(annf_handle* h, const void* x, int nimg, int hgt, int wid, int ci, int co,
                             const uint16_t* w_tc, const float* bias, int relu, void* y, void* stream);
/* dx [nimg,hgt,wid,ci] FP32 = input gradient for upstream g [.., co] FP32, g multiplied by
 * (mask > 0) when mask (BF16 [.., co], the layer's ReLU output) is given. */
int annf_cnn_conv_backward_data(annf_handle* h, const float* g, const void* mask, int nimg, int hgt, int wid, int co,
                                int ci, const float* w_bwd, float* dx, void* stream);
/* dw [co][9][ci] += sum_p g[p][co] x[p + tap][ci]; db [co] += sum_p g[p][co] (accumulates: zero
 * them first). */
int annf_cnn_conv_backward_weights(annf_handle* h, const void* x, const float* g, const void* mask, int nimg,
                                   int hgt, int wid, int ci, int co, float* dw, float* db, void* stream);
/* Relaxed winner-takes-all L1 loss of the 4 hypotheses (x16 px) of each pixel against its 16
 * sub-targets tgt [npix][16][2] (valid [npix][16]): each sub-target's nearest hypothesis weighs 1,
 * the others 0.05, errors truncated at 40 px; dout [npix][8], *loss_sum += loss;
 * inv_nvalid = 1 / number of valid sub-targets. */
int annf_cnn_wta_loss(annf_handle* h, const float* out, const float* tgt, const uint8_t* valid, long long npix,
                      float inv_nvalid, float* dout, float* loss_sum, void* stream);
/* Bias-corrected Adam step (step >= 1) on FP32 parameters, in place. */
int annf_cnn_adam(annf_handle* h, float* param, const float* grad, float* m, float* v, int n, float lr, float beta1,
                  float beta2, float eps, int step, void* stream);
/* Training targets from an NNF of A (ha x wa) into B (width wb): per low-resolution pixel the 16
 * offsets (dx, dy) of the A patches centred in its 4x4 block, tgt [ha/4][wa/4][16][2], valid
 * [ha/4][wa/4][16] (0 where the patch leaves the image). */
int annf_cnn_targets(annf_handle* h, const int* nnf, int ha, int wa, int wb, int psize, float* tgt, uint8_t* valid,
                     void* stream);
/* Proposals [n_A][4] B patch indices from the network output out [h4][w4][8]: each A patch takes
 * the 4 hypotheses of the low-resolution pixel holding its centre, rounded, clamped to B's grid. */
int annf_cnn_proposals(annf_handle* h, const float* out, int h4, int w4, int ha, int wa, int hb, int wb, int psize,
                       int* props, void* stream);
/* The same with per_pixel (1, 2 or 4) hypotheses per A patch, props [n_A][per_pixel]: 4 as above;
 * 2: patches with x + y even take hypotheses 0 and 1, odd ones 2 and 3; 1: patch (y, x) takes
 * hypothesis 2 (y mod 2) + (x mod 2), so every 2 x 2 group of patches verifies all four. */
int annf_cnn_proposals_per_pixel(annf_handle* h, const float* out, int h4, int w4, int ha, int wa, int hb, int wb,
                                 int psize, int per_pixel, int* props, void* stream);

/* Synchronise the stream and report (and clear) the kernels' bounds-check status bits. */
int annf_device_status(annf_handle* h, void* stream, unsigned* bits_out);

/* Instrumentation (no counterpart in the reference, whose only timing is wall-clock per Python
 * stage, annfmp/openmp/base.py:73-126). With profiling on, every call records CUDA events on its
 * stream at stage boundaries; annf_profile_read synchronises the stream and returns the number of
 * intervals (ms[i] = time from the previous mark to mark i, names[i] = the stage that ended there),
 * then clears the marks. annf_launch_count returns the kernels this library has launched. */
int annf_profile_enable(annf_handle* h, int on);
int annf_profile_read(annf_handle* h, void* stream, int cap, float* ms, const char** names);
long long annf_launch_count(void);

/* Graph capture support (no counterpart in the reference). Handles keep grow-only device scratch
 * buffers; a CUDA graph captured around library calls holds their addresses. annf_buffer_epoch
 * returns how many times any handle in the process has replaced a buffer by a larger one (first
 * allocations are not counted): a graph captured at epoch e may be replayed only while
 * annf_buffer_epoch() == e. */
long long annf_buffer_epoch(void);

#ifdef __cplusplus
}
#endif

#endif /* ANNF_GB300_H_ */
