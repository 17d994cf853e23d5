/*
 * ocl_oracle.c -- CPU restatement of the NNF algorithm of annfmp's GPU backend ("openclopt":
 * annfmp/openclopt/src/futhark/{buildKDtree,kd-traverse,brute-force,driverKNN}.fut, orchestrated
 * by annfmp/openclopt/src/base.c:fit_extern).
 *
 * TEST INFRASTRUCTURE ONLY: the checker the CUDA openclopt-semantics mode is compared with.
 * Nothing in the product links it.
 *
 * PARITY UNPINNED: the reference path is Futhark-generated code that cannot be built or run
 * here (no Futhark toolchain; its checked-in CUDA source targets an older architecture through
 * NVRTC), and its tests hold no golden vectors. This file restates the published Futhark
 * programs, function by function, with the lines each follows. Where the Futhark program leaves
 * an order unspecified, this restatement fixes one and the CUDA mode uses the same:
 *   - the longest-spread axis is a commutative reduction whose tie order is unspecified
 *     (buildKDtree.fut:110-114): ties go to the lowest dimension;
 *   - squared distances are sequential sums without contraction into FMA (brute-force.fut:1-3);
 *   - the dimension reduction (driverKNN.fut:47-54, an f32.sum of unspecified order) is not
 *     restated: both sides start from the same reduced patches.
 *
 * Tree (buildKDtree.fut:17-157): 2^(h+1) leaves of exactly ppl points each, the input padded
 * with +inf rows to m' = 2^(h+1) * ppl; per level every node splits its points, sorted stably by
 * the chosen coordinate, into halves; the split value is the mean of the two middle values.
 *   pts[m'*d]     points in leaf order (+inf pads)
 *   indir[m']     leaf-order position -> original index (>= m: a pad)
 *   dims[q], vals[q], clanc[q]  per internal node (heap order): split axis, split value, the
 *                 closest ancestor splitting the same axis (-1: none)
 *   orig2leaf[m'] original index -> leaf
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OCL_K 8 /* the fixed number of neighbours (driverKNN.fut:13) */

typedef struct {
    int m, d;         /* points (before padding), dimension */
    int h;            /* height without the leaves; -1: a single leaf */
    int q;            /* internal nodes: 2^(h+1) - 1 */
    int ppl, mp;      /* points per leaf, padded point count */
    float *pts;       /* [mp*d] */
    int *indir;       /* [mp] */
    int *dims;        /* [q] */
    float *vals;      /* [q] */
    int *clanc;       /* [q] */
    int *orig2leaf;   /* [mp] */
} ocl_tree;

/* nearest power-of-two exponent, ties down (buildKDtree.fut:4-13) */
static int closest_log2(int p) {
    if (p <= 1) return 0;
    int r = 0, x = p;
    while (x > 1) { x >>= 1; ++r; }
    const int down = p - (1 << r), up = (1 << (r + 1)) - p;
    return down <= up ? r : r + 1;
}

/* tree shape from the point count and the default points per leaf (buildKDtree.fut:17-24) */
void ocl_shape(int m, int defppl, int *h, int *q, int *ppl, int *mp) {
    const int def_num_leaves = (m + defppl - 1) / defppl;
    const int hp1 = closest_log2(def_num_leaves);
    if (hp1 <= 0) {
        *h = -1; *q = 0; *ppl = m; *mp = m;
        return;
    }
    const int nl = 1 << hp1;
    *h = hp1 - 1;
    *q = nl - 1;
    *ppl = (m + nl - 1) / nl;
    *mp = nl * *ppl;
}

/* the order of the float radix sort (sign bit flipped, negative values inverted: -0 < +0) */
static uint32_t fkey(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

typedef struct { uint32_t key; int pos; } keyed;
static int cmp_keyed(const void *a, const void *b) {
    const keyed *x = a, *y = b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->pos < y->pos ? -1 : (x->pos > y->pos);  /* stable */
}

static int level_of(int node) { int l = 0; while (node > 0) { node = (node - 1) / 2; ++l; } return l; }

/* mkKDtree (buildKDtree.fut:65-157) and orig2leaf (driverKNN.fut:142-151) */
int ocl_build(ocl_tree *t, const float *X) {
    const int m = t->m, d = t->d, mp = t->mp, q = t->q;
    if (m < 1 || d < 1) return -1;
    float *in = malloc((size_t)mp * d * sizeof(float));
    for (int i = 0; i < mp; ++i)
        for (int j = 0; j < d; ++j) in[(size_t)i * d + j] = i < m ? X[(size_t)i * d + j] : INFINITY;
    float *lub = malloc(2 * (size_t)d * sizeof(float));     /* global bounds (buildKDtree.fut:74-77) */
    for (int j = 0; j < d; ++j) { lub[j] = FLT_MAX; lub[d + j] = -FLT_MAX; }
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < d; ++j) {
            const float v = X[(size_t)i * d + j];
            if (v < lub[j]) lub[j] = v;
            if (v > lub[d + j]) lub[d + j] = v;
        }
    for (int i = 0; i < mp; ++i) t->indir[i] = i;
    for (int i = 0; i < q; ++i) { t->dims[i] = -1; t->vals[i] = 0.f; t->clanc[i] = -1; }
    float *cur = malloc(2 * (size_t)d * sizeof(float));
    keyed *buf = malloc((size_t)mp * sizeof(keyed));
    int *tmp = malloc((size_t)mp * sizeof(int));
    int *ndim = malloc((size_t)(q + 1) * sizeof(int)), *nanc = malloc((size_t)(q + 1) * sizeof(int));
    float *nval = malloc((size_t)(q + 1) * sizeof(float));
    for (int lev = 0; lev <= t->h; ++lev) {
        const int nodes = 1 << lev, ppn = mp / nodes;
        for (int i = 0; i < nodes; ++i) {
            const int node = i + nodes - 1;
            /* bounds: walk from the root (updateBounds, buildKDtree.fut:26-40) */
            memcpy(cur, lub, 2 * (size_t)d * sizeof(float));
            int anc = 0;
            for (int s = 0; s < lev; ++s) {
                const int k = lev - s - 1;
                const int child = (node + 1 - (1 << k)) / (1 << k);
                const int ad = t->dims[anc];
                const int li = (child & 1) == 0 ? ad : d + ad; /* right child: lower bound */
                if (!isinf(t->vals[anc])) cur[li] = t->vals[anc];
                anc = child;
            }
            int best = 0;  /* widest |ub - lb|, lowest dimension on ties (buildKDtree.fut:108-114) */
            float bw = fabsf(cur[d] - cur[0]);
            for (int j = 1; j < d; ++j) {
                const float w = fabsf(cur[d + j] - cur[j]);
                if (w > bw) { bw = w; best = j; }
            }
            int pa = -1;  /* findClosestMed (buildKDtree.fut:42-51) */
            for (int c = node; c != 0 && pa == -1;) {
                const int par = (c - 1) / 2;
                if (t->dims[par] == best) pa = par;
                c = par;
            }
            ndim[i] = best;
            nanc[i] = pa;
            /* stable sort of the node's points by the chosen coordinate, the mean of the two middle
               values (buildKDtree.fut:120-140) */
            int *chunk = t->indir + (size_t)i * ppn;
            for (int r = 0; r < ppn; ++r) {
                buf[r].key = fkey(in[(size_t)chunk[r] * d + best]);
                buf[r].pos = r;
            }
            qsort(buf, ppn, sizeof(keyed), cmp_keyed);
            const int mi = ppn / 2;
            const float a = in[(size_t)chunk[buf[mi].pos] * d + best];
            const float b = in[(size_t)chunk[buf[mi - 1].pos] * d + best];
            nval[i] = (a + b) / 2.0f;
            for (int r = 0; r < ppn; ++r) tmp[r] = chunk[buf[r].pos];
            memcpy(chunk, tmp, (size_t)ppn * sizeof(int));
        }
        for (int i = 0; i < nodes; ++i) {  /* scatter this level's nodes (buildKDtree.fut:142-146) */
            t->dims[i + nodes - 1] = ndim[i];
            t->vals[i + nodes - 1] = nval[i];
            t->clanc[i + nodes - 1] = nanc[i];
        }
    }
    for (int p = 0; p < mp; ++p)
        memcpy(t->pts + (size_t)p * d, in + (size_t)t->indir[p] * d, (size_t)d * sizeof(float));
    for (int p = 0; p < mp; ++p) t->orig2leaf[t->indir[p]] = p / t->ppl;
    free(in); free(lub); free(cur); free(buf); free(tmp); free(ndim); free(nanc); free(nval);
    return 0;
}

/* sumSqrsSeq (brute-force.fut:1-3): sequential, no contraction */
static float sqdist(const float *x, const float *y, int d) {
    float r = 0.f;
    for (int j = 0; j < d; ++j) {
        const float z = x[j] - y[j];
        const float zz = z * z;
        r = r + zz;
    }
    return r;
}

/* findLeaf (kd-traverse.fut:5-14): left when q[dim] <= value */
static int find_leaf(const ocl_tree *t, const float *x) {
    int node = 0;
    while (node < t->q) node = (x[t->dims[node]] <= t->vals[node]) ? 2 * node + 1 : 2 * node + 2;
    return node - t->q;
}

/* bruteForce (brute-force.fut:5-23): sequential insertion, a tie goes behind the entries it ties */
static void brute_seq(const ocl_tree *t, const float *x, int leaf, int *ki, float *kd) {
    for (int i = 0; i < t->ppl; ++i) {
        const int pos = leaf * t->ppl + i;
        float dist = sqdist(x, t->pts + (size_t)pos * t->d, t->d);
        if (dist > kd[OCL_K - 1]) continue;
        int ref = pos;
        for (int j = 0; j < OCL_K; ++j) {
            const float cur = kd[j];
            if (dist >= cur) continue;
            const int ti = ki[j];
            ki[j] = ref;
            kd[j] = dist;
            ref = ti;
            dist = cur;
        }
    }
}

/* bruteForcePar + sortPartSortedSeqs (brute-force.fut:25-66): the leaf's smallest distances
 * (lowest position on ties) replace the list's largest while smaller, then the two sorted runs
 * merge (a tie takes the new entry first) */
static void brute_par(const ocl_tree *t, const float *x, int leaf, int *ki, float *kd, float *dist) {
    const int ppl = t->ppl;
    for (int i = 0; i < ppl; ++i) dist[i] = sqdist(x, t->pts + (size_t)(leaf * ppl + i) * t->d, t->d);
    for (int j = 0; j < OCL_K; ++j) {
        int mi = ppl;
        float mv = INFINITY;
        for (int i = 0; i < ppl; ++i)
            if (dist[i] < mv || (dist[i] == mv && i < mi)) { mv = dist[i]; mi = i; }
        if (!(mv < kd[OCL_K - 1 - j])) break;
        dist[mi] = FLT_MAX;
        ki[OCL_K - 1 - j] = leaf * ppl + mi;
        kd[OCL_K - 1 - j] = mv;
    }
    int si[OCL_K];
    float sd[OCL_K];
    int beg = 0, end = OCL_K - 1;
    for (int i = 0; i < OCL_K; ++i) {
        if (kd[beg] < kd[end]) { si[i] = ki[beg]; sd[i] = kd[beg]; ++beg; }
        else { si[i] = ki[end]; sd[i] = kd[end]; --end; }
    }
    memcpy(ki, si, sizeof si);
    memcpy(kd, sd, sizeof sd);
}

/* natural leaf and its kNN for every query (driverKNN.fut:153-172); positions in leaf order */
void ocl_natural(const ocl_tree *t, const float *Q, int nq, int *ki, float *kd, int *nat) {
    for (int i = 0; i < nq; ++i) {
        const float *x = Q + (size_t)i * t->d;
        nat[i] = t->h < 0 ? 0 : find_leaf(t, x);
        for (int j = 0; j < OCL_K; ++j) { ki[(size_t)i * OCL_K + j] = -1; kd[(size_t)i * OCL_K + j] = FLT_MAX; }
        brute_seq(t, x, nat[i], ki + (size_t)i * OCL_K, kd + (size_t)i * OCL_K);
    }
}

static int stk_get(int s, int i) { return (s >> i) & 1; }
static int stk_set(int s, int i, int v) { return (s & ~(1 << i)) | (v ? (1 << i) : 0); }

/* the first ancestor of node on its chain of same-axis ancestors whose second child was visited
 * contributes its split distance (getAncSameDimContrib, kd-traverse.fut:48-58) */
static float anc_contrib(const ocl_tree *t, float qm, int stack, int node) {
    int idx = node;
    while (idx >= 0) {
        const int anc = t->clanc[idx];
        if (anc == -1) return 0.f;
        if (!stk_get(stack, level_of(anc))) { idx = anc; continue; }
        return t->vals[anc] - qm;
    }
    return 0.f;
}

/* traverseOnce (kd-traverse.fut:23-116): the next leaf to visit (q+1: none), stack and distance */
static int traverse_once(const ocl_tree *t, const float *x, float wnn, int last_leaf, int *stack, float *dist) {
    const int q = t->q, h = t->h;
    if (last_leaf >= q + 1) return q + 1;
    int node = last_leaf + q, count = h, rec = -1;
    int stk = *stack;
    float dd = *dist;
    while (node != 0 && rec < 0) {
        const int parent = (node - 1) / 2;
        const int second = stk_get(stk, count);
        const float qm = x[t->dims[parent]];
        const float cur = t->vals[parent] - qm;
        const float cur2 = cur * cur;
        const float prv = anc_contrib(t, qm, stk, parent);
        const float prv2 = prv * prv;
        const float minu = fabsf((dd - cur2) + prv2);
        const float plus = fabsf((dd - prv2) + cur2);
        if (second) {
            node = parent; count -= 1; dd = minu;
        } else if (!(plus < wnn)) {
            node = parent; count -= 1;
        } else {
            const int fst = node, snd = (fst % 2 == 0) ? fst - 1 : fst + 1;
            stk = stk_set(stk, count, 1);
            node = parent; dd = plus; rec = snd;
        }
    }
    int leaf;
    if (node == 0 && rec == -1) {
        leaf = 2 * q + 1;
    } else {
        int nd = rec, c = count;
        while (nd < q) {
            c += 1;
            stk = stk_set(stk, c, 0);
            nd = (x[t->dims[nd]] <= t->vals[nd]) ? 2 * nd + 1 : 2 * nd + 2;
        }
        leaf = nd;
    }
    *stack = stk;
    *dist = dd;
    return leaf - q;
}

/* exact kNN of the first queries, from their natural-leaf lists (driverKNN.fut:231-266) */
void ocl_exact(const ocl_tree *t, const float *Q, int nq, const int *nat, int *ki, float *kd) {
    float *dist = malloc((size_t)t->ppl * sizeof(float));
    const int nleaves = t->q + 1;
    for (int i = 0; i < nq; ++i) {
        const float *x = Q + (size_t)i * t->d;
        int *li = ki + (size_t)i * OCL_K;
        float *ld = kd + (size_t)i * OCL_K;
        int leaf = nat[i], stack = 0;
        float dd = 0.f;
        if (t->h < 0) continue;
        for (;;) {
            leaf = traverse_once(t, x, ld[OCL_K - 1], leaf, &stack, &dd);
            if (leaf >= nleaves) break;
            brute_par(t, x, leaf, li, ld, dist);
        }
    }
    free(dist);
}

/* the leaf of the patch one row below (the last row clamped) of a tree position's original
 * index (estimateIndex, driverKNN.fut:293-303); -1 outside the grid of B */
static int estimate_leaf(const ocl_tree *t, int n_rows, int n_cols, int pos) {
    const int orig = t->indir[pos];
    const int y = orig / n_cols, x = orig - y * n_cols;
    const int cy = y < n_rows - 1 ? y + 1 : n_rows - 1;
    const long long cand = (long long)cy * n_cols + x;
    if (cand < 0 || cand >= t->mp) return -1;
    return t->orig2leaf[cand];
}

/* row propagation (driverKNN.fut:305-357): each row's lists, from its natural-leaf lists, merge
 * the distinct leaves (not the natural one) below the matches of the pixel above, in order */
int ocl_propagate(const ocl_tree *t, const float *Q, int n_rows, int n_cols, const int *nat, int *ki, float *kd) {
    float *dist = malloc((size_t)t->ppl * sizeof(float));
    int bad = 0;
    for (int r = 1; r < n_rows; ++r) {
        for (int c = 0; c < n_cols; ++c) {
            const long long i = (long long)r * n_cols + c, up = i - n_cols;
            int u[OCL_K], nu = 0;
            for (int j = 0; j < OCL_K; ++j) {
                const int pos = ki[up * OCL_K + j];
                if (pos < 0) continue;
                const int lf = estimate_leaf(t, n_rows, n_cols, pos);
                if (lf < 0) { bad = 1; continue; }
                int found = lf == nat[i];
                for (int z = 0; z < nu && !found; ++z) found = u[z] == lf;
                if (!found) u[nu++] = lf;
            }
            for (int z = 0; z < nu; ++z)
                brute_par(t, Q + (size_t)i * t->d, u[z], ki + i * OCL_K, kd + i * OCL_K, dist);
        }
    }
    free(dist);
    return bad;
}

/* select best (driverKNN.fut:90-133): the list entry (original indices) with the smallest exact
 * squared raw-patch distance, the first on ties; pa, pb: [n*P] uint8 patches */
void ocl_select(const int *knn_orig, long long n, const unsigned char *pa, const unsigned char *pb, int P,
                int *best, float *best_d) {
    for (long long i = 0; i < n; ++i) {
        int bi = -1;
        float bd = INFINITY;
        for (int j = 0; j < OCL_K; ++j) {
            const int o = knn_orig[i * OCL_K + j];
            if (o < 0) continue;
            long long s = 0;
            for (int e = 0; e < P; ++e) {
                const int v = (int)pb[(long long)o * P + e] - (int)pa[i * P + e];
                s += v * v;
            }
            const float f = (float)s;
            if (f < bd) { bd = f; bi = o; }
        }
        best[i] = bi;
        best_d[i] = bd;
    }
}
