/*
 * annf_oracle.c -- CPU restatement of annfmp's propagation-assisted k-d tree NNF path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker that the CUDA kernels are compared with,
 * and the CPU baseline that bench.py times beside them. Nothing in the product links it.
 *
 * It restates, in its own code, the algorithm of the reference OpenMP backend
 * (annfmp/openmp/kdtree/src/{base,kdtree,helper,util}.c). Each function cites the reference
 * lines it follows. Parity with the reference is pinned in tests against outputs of the
 * reference C core compiled unmodified (oracle/Makefile, target "ref") and against the
 * committed golden fixtures in tests/golden/.
 *
 * Build: oracle/Makefile. REAL is float by default and double with -DORA_DOUBLE=1, mirroring the
 * reference's USE_DOUBLE switch (annfmp/openmp/kdtree/src/include/float.h:16-26). Must be
 * compiled without FMA contraction (-ffp-contract=off): the reference sums squared differences
 * with separate multiplies and adds (helper.c:164-179).
 *
 * Tree layout (structure-of-arrays; the reference keeps an array of {point, index} records):
 *   pts[n*d]          points in tree order (the order the reference's XI array ends up in)
 *   perm[n]           tree position -> original point index (the reference's XI index field)
 *   node_axis[2^D-1]  split axis per internal node, heap order (root 0, children 2i+1, 2i+2)
 *   node_split[2^D-1] split value per internal node
 *   leaf_bounds[2*2^D] {begin, end} tree positions per leaf
 *   point_leaf[n]     leaf of each ORIGINAL point index (reference points_leaf_indices)
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORA_DOUBLE
typedef double REAL;
#define REAL_BIG DBL_MAX
#define REAL_SQRT sqrt
#else
typedef float REAL;
#define REAL_BIG FLT_MAX
#define REAL_SQRT sqrtf
#endif

typedef struct {
    int n;            /* number of points */
    int d;            /* dimension */
    int depth;        /* tree depth (number of internal levels) */
    int splitting;    /* 0: cyclic axis (level mod d), 1: longest bounding-box side */
    REAL *pts;        /* [n*d] */
    int *perm;        /* [n] */
    int *node_axis;   /* [2^depth - 1] */
    REAL *node_split; /* [2^depth - 1] */
    int *leaf_bounds; /* [2 * 2^depth] */
    int *point_leaf;  /* [n] */
} ora_tree;

/* ------------------------------------------------------------------------------------------ */
/* bounded sorted K-list: insertion with strict '<', ties keep the earlier entry             */
/* (reference kdtree.c:502-532)                                                               */
/* ------------------------------------------------------------------------------------------ */
static inline void klist_init(REAL *bd, int *bi, int K) {
    for (int j = 0; j < K; ++j) { bd[j] = REAL_BIG; bi[j] = 0; } /* kdtree.c:141-144 */
}

static inline void klist_offer(REAL dist, int pos, REAL *bd, int *bi, int K) {
    if (!(dist < bd[K - 1])) return;
    int j = K - 1;
    while (j > 0 && dist < bd[j - 1]) {
        bd[j] = bd[j - 1];
        bi[j] = bi[j - 1];
        --j;
    }
    bd[j] = dist;
    bi[j] = pos;
}

/* squared distance, dims in order, separate multiply and add (reference helper.c:164-179) */
static inline REAL sqdist(const REAL *p, const REAL *q, int d) {
    REAL acc = 0;
    for (int j = 0; j < d; ++j) {
        REAL t = p[j] - q[j];
        acc = acc + t * t;
    }
    return acc;
}

/* scan one leaf's tree positions [lo,hi) in order (reference kdtree.c:286-303) */
static inline void scan_leaf(const ora_tree *t, int lo, int hi, const REAL *q, REAL *bd, int *bi,
                             int K) {
    for (int p = lo; p < hi; ++p) klist_offer(sqdist(t->pts + (size_t)p * t->d, q, t->d), p, bd, bi, K);
}

/* ------------------------------------------------------------------------------------------ */
/* build                                                                                      */
/* ------------------------------------------------------------------------------------------ */

/* depth = floor(log2 n) - floor(log2 leaf_size), clamped at 0 (reference kdtree/base.py:260-300).
 * tree_depth >= 0 overrides (clamped to floor(log2 n)). Returns -1 if leaf_size <= 1 and no
 * explicit depth is given. */
int ora_tree_depth(int n, int leaf_size, int tree_depth) {
    int lg = 0;
    while ((2LL << lg) <= (long long)n) ++lg; /* floor(log2 n) */
    if (tree_depth >= 0) return tree_depth > lg ? lg : tree_depth;
    if (leaf_size <= 1) return -1;
    int ls = 0;
    while ((2LL << ls) <= (long long)leaf_size) ++ls;
    return lg - ls < 0 ? 0 : lg - ls;
}

/* axis of the widest bounding-box side: first axis with strictly the largest width, 0 if all
 * widths are 0 (reference kdtree.c:375-417) */
static int widest_axis(const ora_tree *t, int lo, int hi, REAL *mn, REAL *mx) {
    const int d = t->d;
    for (int j = 0; j < d; ++j) { mn[j] = REAL_BIG; mx[j] = -REAL_BIG; }
    for (int p = lo; p < hi; ++p) {
        const REAL *x = t->pts + (size_t)p * d;
        for (int j = 0; j < d; ++j) {
            if (x[j] < mn[j]) mn[j] = x[j];
            if (x[j] > mx[j]) mx[j] = x[j];
        }
    }
    REAL best = 0;
    int axis = 0;
    for (int j = 0; j < d; ++j) {
        REAL w = mx[j] - mn[j];
        if (w > best) { best = w; axis = j; }
    }
    return axis;
}

/* value of rank k (0-based) among v[0..m-1]; v is reordered. Any exact selection returns the same
 * value as the reference's Wirth select (util.c:146-186); this one is an iterative quickselect. */
static REAL select_rank(REAL *v, int m, int k) {
    int lo = 0, hi = m - 1;
    while (lo < hi) {
        /* median of three as pivot value */
        int mid = lo + (hi - lo) / 2;
        REAL a = v[lo], b = v[mid], c = v[hi];
        REAL piv = (a < b) ? ((b < c) ? b : ((a < c) ? c : a)) : ((a < c) ? a : ((b < c) ? c : b));
        /* three-way partition [lo..lt) < piv, [lt..gt] == piv, (gt..hi] > piv */
        int lt = lo, i = lo, gt = hi;
        while (i <= gt) {
            if (v[i] < piv) { REAL s = v[lt]; v[lt] = v[i]; v[i] = s; ++lt; ++i; }
            else if (piv < v[i]) { REAL s = v[gt]; v[gt] = v[i]; v[i] = s; --gt; }
            else ++i;
        }
        if (k < lt) hi = lt - 1;
        else if (k > gt) lo = gt + 1;
        else return piv;
    }
    return v[k];
}

/* Reorder tree positions [lo,hi) around 'piv' on 'axis' exactly as the reference does
 * (helper.c:63-113): elements < piv keep their order at the front; elements >= piv are laid out
 * from the back in reverse visiting order; then one forward pass over that upper block moves the
 * elements equal to piv, in the order met, to the front of the block by swapping. */
static void split_positions(ora_tree *t, int lo, int hi, int axis, REAL piv, REAL *tmp_pts,
                            int *tmp_perm) {
    const int d = t->d, m = hi - lo;
    int front = 0, back = m - 1;
    for (int i = 0; i < m; ++i) {
        const REAL *x = t->pts + (size_t)(lo + i) * d;
        int dst = (x[axis] < piv) ? front++ : back--;
        memcpy(tmp_pts + (size_t)dst * d, x, sizeof(REAL) * d);
        tmp_perm[dst] = t->perm[lo + i];
    }
    int w = back + 1;
    for (int i = back + 1; i < m; ++i) {
        if (tmp_pts[(size_t)i * d + axis] == piv) {
            if (i != w) {
                for (int j = 0; j < d; ++j) {
                    REAL s = tmp_pts[(size_t)i * d + j];
                    tmp_pts[(size_t)i * d + j] = tmp_pts[(size_t)w * d + j];
                    tmp_pts[(size_t)w * d + j] = s;
                }
                int s = tmp_perm[i]; tmp_perm[i] = tmp_perm[w]; tmp_perm[w] = s;
            }
            ++w;
        }
    }
    memcpy(t->pts + (size_t)lo * d, tmp_pts, sizeof(REAL) * (size_t)m * d);
    memcpy(t->perm + lo, tmp_perm, sizeof(int) * m);
}

typedef struct { REAL *mn, *mx, *vals, *tmp_pts; int *tmp_perm; } build_scratch;

/* reference kdtree.c:76-117 (recursion), 463-489 (median split at rank count/2) */
static void build_rec(ora_tree *t, build_scratch *s, int lo, int hi, int node, int level) {
    const int d = t->d;
    if (level == t->depth) {
        int leaf = node - ((1 << t->depth) - 1);
        t->leaf_bounds[2 * leaf] = lo;
        t->leaf_bounds[2 * leaf + 1] = hi;
        for (int p = lo; p < hi; ++p) t->point_leaf[t->perm[p]] = leaf;
        return;
    }
    /* reference kdtree.c:369-371 (cyclic) and 373-417 (longest) */
    int axis = t->splitting == 0 ? level % d : widest_axis(t, lo, hi, s->mn, s->mx);
    int m = hi - lo, half = m / 2;
    for (int i = 0; i < m; ++i) s->vals[i] = t->pts[(size_t)(lo + i) * d + axis];
    REAL piv = select_rank(s->vals, m, half);
    split_positions(t, lo, hi, axis, piv, s->tmp_pts, s->tmp_perm);
    t->node_axis[node] = axis;
    t->node_split[node] = t->pts[(size_t)(lo + half) * d + axis];
    build_rec(t, s, lo, lo + half, 2 * node + 1, level + 1);
    build_rec(t, s, lo + half, hi, 2 * node + 2, level + 1);
}

/* Fill every array of *t (allocated by the caller) from X[n*d]. Returns 0, or -1 on bad input. */
int ora_build(ora_tree *t, const REAL *X) {
    if (!t || !X || t->n < 1 || t->d < 1 || t->depth < 0 || (1LL << t->depth) > t->n) return -1;
    const int n = t->n, d = t->d;
    memcpy(t->pts, X, sizeof(REAL) * (size_t)n * d);
    for (int i = 0; i < n; ++i) t->perm[i] = i;
    build_scratch s;
    s.mn = (REAL *)malloc(sizeof(REAL) * d);
    s.mx = (REAL *)malloc(sizeof(REAL) * d);
    s.vals = (REAL *)malloc(sizeof(REAL) * n);
    s.tmp_pts = (REAL *)malloc(sizeof(REAL) * (size_t)n * d);
    s.tmp_perm = (int *)malloc(sizeof(int) * n);
    if (!s.mn || !s.mx || !s.vals || !s.tmp_pts || !s.tmp_perm) {
        free(s.mn); free(s.mx); free(s.vals); free(s.tmp_pts); free(s.tmp_perm);
        return -1;
    }
    build_rec(t, &s, 0, n, 0, 0);
    free(s.mn); free(s.mx); free(s.vals); free(s.tmp_pts); free(s.tmp_perm);
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* queries                                                                                    */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    const ora_tree *t;
    const REAL *q;
    REAL *bd;
    int *bi;
    int K;
    long long budget; /* leaves that may still be scanned */
    int stop;
} dfs_state;

/* Depth-first search with backtracking: near child first (right when q[axis] - split >= 0), the
 * far child only if (q[axis]-split)^2 <= current K-th distance; stops before the leaf that would
 * exceed the leaf budget (reference kdtree.c:129-268). */
static void dfs(dfs_state *st, int node, int level) {
    const ora_tree *t = st->t;
    if (st->stop) return;
    if (level == t->depth) {
        if (st->budget <= 0) { st->stop = 1; return; }
        st->budget--;
        int leaf = node - ((1 << t->depth) - 1);
        scan_leaf(t, t->leaf_bounds[2 * leaf], t->leaf_bounds[2 * leaf + 1], st->q, st->bd, st->bi,
                  st->K);
        return;
    }
    int axis = t->node_axis[node];
    REAL diff = st->q[axis] - t->node_split[node];
    int near = (diff >= 0) ? 2 * node + 2 : 2 * node + 1;
    int far = (diff >= 0) ? 2 * node + 1 : 2 * node + 2;
    dfs(st, near, level + 1);
    if (st->stop) return;
    if (diff * diff <= st->bd[st->K - 1]) dfs(st, far, level + 1);
}

/* K nearest tree positions of q (exact when max_leaves is large). bd/bi receive squared
 * distances and tree positions, best first. */
void ora_query(const ora_tree *t, const REAL *q, int K, long long max_leaves, REAL *bd, int *bi) {
    klist_init(bd, bi, K);
    dfs_state st = {t, q, bd, bi, K, max_leaves, 0};
    dfs(&st, 0, 0);
}

/* leaf reached by descent alone (reference kdtree.c:171-183 with max_leaves=1, only_leaf_idx=1) */
int ora_natural_leaf(const ora_tree *t, const REAL *q) {
    int node = 0;
    for (int level = 0; level < t->depth; ++level) {
        REAL diff = q[t->node_axis[node]] - t->node_split[node];
        node = (diff >= 0) ? 2 * node + 2 : 2 * node + 1;
    }
    return node - ((1 << t->depth) - 1);
}

/* reference neighbors_extern (base.c:88-132): exact kNN per query, then tree positions mapped to
 * original indices and distances square-rooted */
void ora_kneighbors(const ora_tree *t, const REAL *Q, int nq, int K, long long max_leaves,
                    REAL *dist, int *idx) {
    #pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < nq; ++i) ora_query(t, Q + (size_t)i * t->d, K, max_leaves, dist + (size_t)i * K, idx + (size_t)i * K);
    for (long long i = 0; i < (long long)nq * K; ++i) {
        idx[i] = t->perm[idx[i]];
        dist[i] = REAL_SQRT(dist[i]);
    }
}

/* raw-patch L2 with the reference's REAL accumulation and sqrt (base.c:362-374) */
static inline REAL patch_l2(const uint8_t *a, const uint8_t *b, int P) {
    REAL acc = 0;
    for (int i = 0; i < P; ++i) {
        REAL t = (REAL)a[i] - (REAL)b[i];
        acc = acc + t * t;
    }
    return REAL_SQRT(acc);
}

/* The row-sequential NNF driver (reference process_rows_extern, base.c:150-360).
 *
 *   ared       [n_rows*n_cols*d] reduced A patches, row-major pixel order
 *   pa, pb     raw uint8 patches [nA*P], [nB*P] (pb indexed by original B index)
 *   knn_out    optional [nA*K]: the K-list of each pixel as ORIGINAL B indices
 *   final_out  [nA]: chosen B index per pixel
 *   first_row_max_leaves: leaf budget of the exact first-row search (reference passes its
 *              max_leaves parameter, 2147483640 by default)
 *   ntheads    OpenMP threads (<=0: runtime default)
 */
int ora_process_rows(const ora_tree *t, const REAL *ared, const uint8_t *pa, const uint8_t *pb,
                     int P, int nB, int n_rows, int n_cols, int K, int propagate, int select_best,
                     long long first_row_max_leaves, int *knn_out, int *final_out, int nthreads) {
    if (!t || !ared || n_rows < 1 || n_cols < 1 || K < 1) return -1;
    if (select_best && (!pa || !pb || P < 1)) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const int d = t->d;
    const long long nA = (long long)n_rows * n_cols;
    int *lists = (int *)malloc(sizeof(int) * nA * K); /* K-lists as tree positions */
    REAL *dtmp = (REAL *)malloc(sizeof(REAL) * (size_t)n_cols * K);
    int *leaves = (int *)malloc(sizeof(int) * (size_t)n_cols * (1 + K));
    if (!lists || !dtmp || !leaves) { free(lists); free(dtmp); free(leaves); return -1; }

    /* (I) first row: exact search (base.c:197-215) */
    #pragma omp parallel for schedule(dynamic, 4)
    for (int x = 0; x < n_cols; ++x)
        ora_query(t, ared + (size_t)x * d, K, first_row_max_leaves, dtmp + (size_t)x * K, lists + (size_t)x * K);

    /* (II) later rows, strictly in order (base.c:227-306) */
    for (int y = 1; y < n_rows; ++y) {
        const REAL *row = ared + (size_t)y * n_cols * d;
        #pragma omp parallel for schedule(static)
        for (int x = 0; x < n_cols; ++x) {
            const REAL *q = row + (size_t)x * d;
            int *lv = leaves + (size_t)x * (1 + K);
            lv[0] = ora_natural_leaf(t, q);
            if (propagate) {
                /* (base.c:255-282) the pixel above; its j-th neighbour shifted one row down
                 * unless that leaves A's patch range; then the leaf that point lives in */
                const int *above = lists + ((long long)(y - 1) * n_cols + x) * K;
                for (int j = 0; j < K; ++j) {
                    int b = t->perm[above[j]];
                    if ((long long)b + n_cols < nA) b += n_cols;
                    lv[1 + j] = t->point_leaf[b];
                }
            }
            /* brute force over [natural, propagated...] in that order (kdtree.c:305-352) */
            REAL *bd = dtmp + (size_t)x * K;
            int *bi = lists + ((long long)y * n_cols + x) * K;
            klist_init(bd, bi, K);
            int nleaves = propagate ? 1 + K : 1;
            for (int s = 0; s < nleaves; ++s)
                scan_leaf(t, t->leaf_bounds[2 * lv[s]], t->leaf_bounds[2 * lv[s] + 1], q, bd, bi, K);
        }
    }

    /* (III) tree positions -> original B indices (base.c:309-321) */
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < nA * K; ++i) lists[i] = t->perm[lists[i]];

    /* (IV) pick the final index (base.c:324-353) */
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < nA; ++i) {
        const int *li = lists + i * K;
        if (select_best) {
            int best = -1;
            REAL bestd = REAL_BIG;
            for (int j = 0; j < K; ++j) {
                REAL dd = patch_l2(pa + (size_t)i * P, pb + (size_t)li[j] * P, P);
                if (dd < bestd) { bestd = dd; best = li[j]; }
            }
            final_out[i] = best;
        } else {
            final_out[i] = li[0];
        }
    }
    if (knn_out) memcpy(knn_out, lists, sizeof(int) * nA * K);
    (void)nB;
    free(lists); free(dtmp); free(leaves);
    return 0;
}

/* Uint8 patch gather for an HxWxC image, patch p x p, pixel (y,x) -> row-major index y*nc+x,
 * element ((r*p + c)*C + ch) (sklearn extract_patches_2d as used at annfmp/openmp/base.py:152-166). */
void ora_extract_patches(const uint8_t *img, int H, int W, int C, int p, uint8_t *out) {
    const int nr = H - p + 1, nc = W - p + 1, P = p * p * C;
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < nr; ++y)
        for (int x = 0; x < nc; ++x) {
            uint8_t *o = out + ((size_t)y * nc + x) * P;
            for (int r = 0; r < p; ++r) memcpy(o + (size_t)r * p * C, img + ((size_t)(y + r) * W + x) * C, (size_t)p * C);
        }
}

/* exact raw-patch nearest neighbour over all B patches in FP64 (the distance-error metric's
 * ground truth); returns squared distances and indices for the sampled A pixels */
void ora_exact_raw_nn(const uint8_t *pa, const int *qidx, int nq, const uint8_t *pb, int nB, int P,
                      double *best_d2, int *best_i) {
    #pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < nq; ++i) {
        const uint8_t *a = pa + (size_t)qidx[i] * P;
        long long bestv = -1;
        int bi = -1;
        for (int j = 0; j < nB; ++j) {
            const uint8_t *b = pb + (size_t)j * P;
            long long acc = 0;
            for (int k = 0; k < P; ++k) { int t = (int)a[k] - (int)b[k]; acc += (long long)t * t; }
            if (bestv < 0 || acc < bestv) { bestv = acc; bi = j; }
        }
        best_d2[i] = (double)bestv;
        best_i[i] = bi;
    }
}
