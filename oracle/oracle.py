"""CPU oracle for the annfmp NNF path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference arm may import
this module, and only as the checker or the timed CPU baseline. The product path
(``annfmp_gb300``) never imports it.

Contents
--------
* ctypes bindings of ``annf_oracle.c`` (the C restatement, float and double builds);
* a numpy restatement of the PCA the reference fits through scikit-learn
  (annfmp/openmp/base.py:168-200 -> sklearn ``PCA(svd_solver='auto')``, which picks
  ``covariance_eigh`` for these shapes);
* ``oracle_fit``: the whole ``ANNFieldPropKDTreeOpenMP.fit`` pipeline
  (annfmp/openmp/base.py:53-150) on the CPU;
* bindings of the reference C core compiled unmodified into ``oracle/_ref`` (when present), and a
  shim that lets the unmodified reference Python package run on it (``reference_annfmp``).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

_c_int_p = ctypes.POINTER(ctypes.c_int)


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


# ----------------------------------------------------------------------------------------------
# C restatement
# ----------------------------------------------------------------------------------------------
class _OraTree(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int),
        ("d", ctypes.c_int),
        ("depth", ctypes.c_int),
        ("splitting", ctypes.c_int),
        ("pts", ctypes.c_void_p),
        ("perm", ctypes.c_void_p),
        ("node_axis", ctypes.c_void_p),
        ("node_split", ctypes.c_void_p),
        ("leaf_bounds", ctypes.c_void_p),
        ("point_leaf", ctypes.c_void_p),
    ]


_LIBS: dict = {}


def build_oracle(quiet: bool = True) -> None:
    """Compile the C restatement (both float types) with oracle/Makefile."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def _lib(real=np.float32):
    key = np.dtype(real).name
    if key in _LIBS:
        return _LIBS[key]
    name = "libannf_oracle_f32.so" if key == "float32" else "libannf_oracle_f64.so"
    path = os.path.join(HERE, name)
    if not os.path.exists(path):
        build_oracle()
    lib = ctypes.CDLL(path)
    lib.ora_build.restype = ctypes.c_int
    lib.ora_build.argtypes = [ctypes.POINTER(_OraTree), ctypes.c_void_p]
    lib.ora_kneighbors.restype = None
    lib.ora_kneighbors.argtypes = [ctypes.POINTER(_OraTree), ctypes.c_void_p, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p]
    lib.ora_process_rows.restype = ctypes.c_int
    lib.ora_process_rows.argtypes = [ctypes.POINTER(_OraTree), ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    lib.ora_natural_leaf.restype = ctypes.c_int
    lib.ora_natural_leaf.argtypes = [ctypes.POINTER(_OraTree), ctypes.c_void_p]
    lib.ora_extract_patches.restype = None
    lib.ora_extract_patches.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p]
    lib.ora_exact_raw_nn.restype = None
    lib.ora_exact_raw_nn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    _LIBS[key] = lib
    return lib


def tree_depth(n: int, leaf_size: int, tree_depth_param=None) -> int:
    """Reference KDTree._compute_final_tree_depth (annfmp/openmp/kdtree/base.py:260-300)."""
    d = int(math.floor(math.log(n, 2)))
    if tree_depth_param is not None:
        return d if tree_depth_param > d else int(tree_depth_param)
    if not leaf_size > 1:
        raise ValueError("Parameter 'leaf_size' must be larger than 1")
    sub = int(math.floor(math.log(leaf_size, 2)))
    return max(d - sub, 0)


class OracleTree:
    """A k-d tree built by the C restatement; arrays are numpy (see annf_oracle.c header)."""

    def __init__(self, X: np.ndarray, depth: int, splitting: int = 1):
        X = np.ascontiguousarray(X)
        if X.dtype not in (np.float32, np.float64):
            raise TypeError("X must be float32 or float64")
        self.real = X.dtype.type
        n, d = X.shape
        self.n, self.d, self.depth = n, d, depth
        L = 1 << depth
        self.pts = np.empty((n, d), X.dtype)
        self.perm = np.empty(n, np.int32)
        self.node_axis = np.zeros(max(L - 1, 0), np.int32)
        self.node_split = np.zeros(max(L - 1, 0), X.dtype)
        self.leaf_bounds = np.empty(2 * L, np.int32)
        self.point_leaf = np.empty(n, np.int32)
        self._s = _OraTree(n, d, depth, splitting, self.pts.ctypes.data, self.perm.ctypes.data,
                           self.node_axis.ctypes.data if L > 1 else None,
                           self.node_split.ctypes.data if L > 1 else None,
                           self.leaf_bounds.ctypes.data, self.point_leaf.ctypes.data)
        rc = _lib(self.real).ora_build(ctypes.byref(self._s), X.ctypes.data)
        if rc != 0:
            raise ValueError("ora_build rejected its input")

    def kneighbors(self, Q: np.ndarray, K: int, max_leaves: int = 2147483640):
        Q = np.ascontiguousarray(Q, dtype=self.real)
        dist = np.empty((Q.shape[0], K), self.real)
        idx = np.empty((Q.shape[0], K), np.int32)
        _lib(self.real).ora_kneighbors(ctypes.byref(self._s), Q.ctypes.data, Q.shape[0], K, max_leaves,
                                       dist.ctypes.data, idx.ctypes.data)
        return dist, idx

    def natural_leaf(self, q: np.ndarray) -> int:
        q = np.ascontiguousarray(q, dtype=self.real)
        return _lib(self.real).ora_natural_leaf(ctypes.byref(self._s), q.ctypes.data)

    def process_rows(self, ared, pa, pb, n_rows, n_cols, K, propagate=True, select_best=True,
                     max_leaves=2147483640, nthreads=0):
        ared = np.ascontiguousarray(ared, dtype=self.real)
        nA = n_rows * n_cols
        assert ared.shape == (nA, self.d)
        P = 0
        if select_best:
            pa = np.ascontiguousarray(pa, dtype=np.uint8)
            pb = np.ascontiguousarray(pb, dtype=np.uint8)
            P = pa.shape[1]
        final = np.empty(nA, np.int32)
        knn = np.empty((nA, K), np.int32)
        rc = _lib(self.real).ora_process_rows(
            ctypes.byref(self._s), ared.ctypes.data,
            pa.ctypes.data if select_best else None, pb.ctypes.data if select_best else None,
            P, self.n, n_rows, n_cols, K, int(bool(propagate)), int(bool(select_best)), max_leaves,
            knn.ctypes.data, final.ctypes.data, nthreads)
        if rc != 0:
            raise ValueError("ora_process_rows rejected its input")
        return final, knn


def extract_patches(img: np.ndarray, psize: int) -> np.ndarray:
    """All overlapping patches, row-major pixel order (annfmp/openmp/base.py:152-166)."""
    img = np.ascontiguousarray(img, dtype=np.uint8)
    H, W, C = img.shape
    nr, nc = H - psize + 1, W - psize + 1
    out = np.empty((nr * nc, psize * psize * C), np.uint8)
    _lib().ora_extract_patches(img.ctypes.data, H, W, C, psize, out.ctypes.data)
    return out


def exact_raw_nn(pa: np.ndarray, qidx: np.ndarray, pb: np.ndarray):
    """FP64/int64 exact raw-patch NN of the A patches qidx over all of pb (error metric truth)."""
    qidx = np.ascontiguousarray(qidx, dtype=np.int32)
    d2 = np.empty(len(qidx), np.float64)
    bi = np.empty(len(qidx), np.int32)
    _lib().ora_exact_raw_nn(np.ascontiguousarray(pa).ctypes.data, qidx.ctypes.data, len(qidx),
                            np.ascontiguousarray(pb).ctypes.data, pb.shape[0], pb.shape[1],
                            d2.ctypes.data, bi.ctypes.data)
    return d2, bi


# ----------------------------------------------------------------------------------------------
# PCA restatement (numpy): sklearn PCA with svd_solver 'auto' on uint8 patch rows
# ----------------------------------------------------------------------------------------------
def sample_positions(n_h: int, n_w: int, max_patches: int, seed: int):
    """Patch positions sklearn.feature_extraction.image.extract_patches_2d samples for
    max_patches / random_state (legacy RandomState, i then j). Returns None for 'all patches'."""
    total = n_h * n_w
    if not max_patches:
        return None
    if max_patches >= total:
        return None
    rs = np.random.RandomState(seed)
    i_s = rs.randint(n_h, size=max_patches)
    j_s = rs.randint(n_w, size=max_patches)
    return i_s, j_s


def subset_patches(img: np.ndarray, psize: int, max_patches: int, seed: int) -> np.ndarray:
    H, W, C = img.shape
    n_h, n_w = H - psize + 1, W - psize + 1
    pos = sample_positions(n_h, n_w, max_patches, seed)
    if pos is None:
        return extract_patches(img, psize)
    i_s, j_s = pos
    out = np.empty((len(i_s), psize * psize * C), np.uint8)
    for r in range(psize):
        for c in range(psize):
            out[:, (r * psize + c) * C:(r * psize + c + 1) * C] = img[i_s + r, j_s + c, :]
    return out


def pca_fit(image_a, image_b, psize, n_components, n_subset, seed):
    """Fit like annfmp/openmp/base.py:168-191: n_subset/2 sampled patches of A (random_state=seed)
    and of B (seed+1), then sklearn's covariance_eigh PCA restated in numpy. Returns
    (components [d,P] f64, mean [P] f64)."""
    m = int(n_subset / 2)
    X = np.concatenate([subset_patches(image_a, psize, m, seed),
                        subset_patches(image_b, psize, m, seed + 1)], axis=0).astype(np.float64)
    n, P = X.shape
    if not (P <= 1000 and n >= 10 * P):
        raise NotImplementedError("only the covariance_eigh regime of sklearn PCA is restated")
    mean = np.mean(X, axis=0)
    C = X.T @ X
    C -= n * mean.reshape(-1, 1) * mean.reshape(1, -1)
    C /= n - 1
    w, V = np.linalg.eigh(C)
    V = np.flip(V, axis=1)
    Vt = V.T
    rows = np.argmax(np.abs(Vt), axis=1)
    signs = np.sign(Vt[np.arange(Vt.shape[0]), rows])
    Vt = Vt * signs[:, None]
    return np.ascontiguousarray(Vt[:n_components]), mean


def pca_transform(patches: np.ndarray, components: np.ndarray, mean: np.ndarray, real=np.float32):
    """sklearn _BasePCA._transform: X @ C.T - mean @ C.T in float64, then cast."""
    X = patches.astype(np.float64)
    Y = X @ components.T
    Y -= mean.reshape(1, -1) @ components.T
    return Y.astype(real)


def oracle_fit(image_a, image_b, n_neighbors=3, psize=8, dim_reduced=5, n_subset=1000,
               leaf_size=64, propagate=True, select_best_nn=True, float_type="float", seed=0,
               nthreads=0, return_all=False):
    """The ANNFieldPropKDTreeOpenMP.fit pipeline (annfmp/openmp/base.py:53-150) on the CPU."""
    real = np.float32 if float_type == "float" else np.float64
    n_cols = image_a.shape[1] - psize + 1
    n_rows = image_a.shape[0] - psize + 1
    comps, mean = pca_fit(image_a, image_b, psize, dim_reduced, n_subset, seed)
    pa = extract_patches(image_a, psize)
    pb = extract_patches(image_b, psize)
    ared = pca_transform(pa, comps, mean, real)
    bred = pca_transform(pb, comps, mean, real)
    assert leaf_size > n_neighbors
    tree = OracleTree(bred, tree_depth(len(bred), leaf_size))
    final, knn = tree.process_rows(ared, pa, pb, n_rows, n_cols, n_neighbors, propagate,
                                   select_best_nn, nthreads=nthreads)
    if return_all:
        return dict(nn=final, knn=knn, tree=tree, ared=ared, bred=bred, comps=comps, mean=mean,
                    pa=pa, pb=pb, n_rows=n_rows, n_cols=n_cols)
    return final


# ----------------------------------------------------------------------------------------------
# the GPU backend's algorithm (openclopt), restated in ocl_oracle.c (parity unpinned: the
# reference's Futhark path cannot run here)
# ----------------------------------------------------------------------------------------------
OCL_K = 8


class _OclTree(ctypes.Structure):
    _fields_ = [("m", ctypes.c_int), ("d", ctypes.c_int), ("h", ctypes.c_int), ("q", ctypes.c_int),
                ("ppl", ctypes.c_int), ("mp", ctypes.c_int), ("pts", ctypes.c_void_p), ("indir", ctypes.c_void_p),
                ("dims", ctypes.c_void_p), ("vals", ctypes.c_void_p), ("clanc", ctypes.c_void_p),
                ("orig2leaf", ctypes.c_void_p)]


def _ocl_lib():
    if "ocl" in _LIBS:
        return _LIBS["ocl"]
    path = os.path.join(HERE, "libannf_ocl_oracle.so")
    if not os.path.exists(path):
        build_oracle()
    lib = ctypes.CDLL(path)
    vp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)
    lib.ocl_shape.argtypes = [ctypes.c_int, ctypes.c_int, ip, ip, ip, ip]
    lib.ocl_build.argtypes = [ctypes.POINTER(_OclTree), vp]
    lib.ocl_build.restype = ctypes.c_int
    lib.ocl_natural.argtypes = [ctypes.POINTER(_OclTree), vp, ctypes.c_int, vp, vp, vp]
    lib.ocl_exact.argtypes = [ctypes.POINTER(_OclTree), vp, ctypes.c_int, vp, vp, vp]
    lib.ocl_propagate.argtypes = [ctypes.POINTER(_OclTree), vp, ctypes.c_int, ctypes.c_int, vp, vp, vp]
    lib.ocl_propagate.restype = ctypes.c_int
    lib.ocl_select.argtypes = [vp, ctypes.c_longlong, vp, vp, ctypes.c_int, vp, vp]
    _LIBS["ocl"] = lib
    return lib


def ocl_shape(m: int, leaf_size: int):
    """(h, q, ppl, m') of the GPU backend's tree (annfmp/openclopt/src/futhark/buildKDtree.fut:17-25)."""
    v = [ctypes.c_int() for _ in range(4)]
    _ocl_lib().ocl_shape(m, leaf_size, *[ctypes.byref(x) for x in v])
    return tuple(x.value for x in v)


class OclTree:
    """The GPU backend's k-d tree (buildKDtree.fut), built by the C restatement."""

    def __init__(self, X: np.ndarray, leaf_size: int):
        X = np.ascontiguousarray(X, dtype=np.float32)
        m, d = X.shape
        self.h, self.q, self.ppl, self.mp = ocl_shape(m, leaf_size)
        self.m, self.d = m, d
        self.pts = np.empty((self.mp, d), np.float32)
        self.indir = np.empty(self.mp, np.int32)
        self.dims = np.empty(max(self.q, 1), np.int32)
        self.vals = np.empty(max(self.q, 1), np.float32)
        self.clanc = np.empty(max(self.q, 1), np.int32)
        self.orig2leaf = np.empty(self.mp, np.int32)
        self._s = _OclTree(m, d, self.h, self.q, self.ppl, self.mp, self.pts.ctypes.data, self.indir.ctypes.data,
                           self.dims.ctypes.data, self.vals.ctypes.data, self.clanc.ctypes.data,
                           self.orig2leaf.ctypes.data)
        if _ocl_lib().ocl_build(ctypes.byref(self._s), X.ctypes.data) != 0:
            raise ValueError("ocl_build rejected its input")
        self.dims, self.vals, self.clanc = self.dims[:self.q], self.vals[:self.q], self.clanc[:self.q]

    def natural(self, Q):
        """(positions [n, 8], squared distances [n, 8], natural leaf [n])."""
        Q = np.ascontiguousarray(Q, dtype=np.float32)
        n = Q.shape[0]
        ki, kd, nat = np.empty((n, OCL_K), np.int32), np.empty((n, OCL_K), np.float32), np.empty(n, np.int32)
        _ocl_lib().ocl_natural(ctypes.byref(self._s), Q.ctypes.data, n, ki.ctypes.data, kd.ctypes.data, nat.ctypes.data)
        return ki, kd, nat

    def exact(self, Q, nat, ki, kd):
        """Exact lists of the queries Q from their natural-leaf lists (in place)."""
        Q = np.ascontiguousarray(Q, dtype=np.float32)
        _ocl_lib().ocl_exact(ctypes.byref(self._s), Q.ctypes.data, Q.shape[0],
                             np.ascontiguousarray(nat, dtype=np.int32).ctypes.data, ki.ctypes.data, kd.ctypes.data)

    def rows(self, ared, n_rows, n_cols):
        """The lists of every pixel: natural leaf, exact first row, row propagation (positions)."""
        ki, kd, nat = self.natural(ared)
        ki0, kd0 = ki[:n_cols].copy(), kd[:n_cols].copy()
        self.exact(ared[:n_cols], nat[:n_cols], ki0, kd0)
        ki[:n_cols], kd[:n_cols] = ki0, kd0
        bad = _ocl_lib().ocl_propagate(ctypes.byref(self._s), np.ascontiguousarray(ared, np.float32).ctypes.data,
                                       n_rows, n_cols, nat.ctypes.data, ki.ctypes.data, kd.ctypes.data)
        return ki, kd, nat, bool(bad)


def ocl_select(knn_orig, pa, pb):
    """Select best by exact squared raw-patch distance (driverKNN.fut:90-133)."""
    knn_orig = np.ascontiguousarray(knn_orig, dtype=np.int32)
    n = knn_orig.shape[0]
    best, bd = np.empty(n, np.int32), np.empty(n, np.float32)
    _ocl_lib().ocl_select(knn_orig.ctypes.data, n, np.ascontiguousarray(pa).ctypes.data,
                          np.ascontiguousarray(pb).ctypes.data, pa.shape[1], best.ctypes.data, bd.ctypes.data)
    return best, bd


def oracle_fit_openclopt(image_a, image_b, psize=8, dim_reduced=5, n_subset=1000, leaf_size=64, seed=0,
                         return_all=False):
    """ANNFieldPropKDTreeOpenCLOPT.fit (annfmp/openclopt/base.py:46-137, src/base.c:fit_extern):
    the same PCA fit, K = 8 whatever n_neighbors is, the backend's tree, natural-leaf lists, exact
    first row, row propagation, select best. The reduced patches are the plain pipeline's (FP64
    transform rounded once; the backend's own FP32 reduction has no specified order)."""
    comps, mean = pca_fit(image_a, image_b, psize, dim_reduced, n_subset, seed)
    pa, pb = extract_patches(image_a, psize), extract_patches(image_b, psize)
    ared = pca_transform(pa, comps, mean)
    bred = pca_transform(pb, comps, mean)
    n_rows, n_cols = image_a.shape[0] - psize + 1, image_a.shape[1] - psize + 1
    tree = OclTree(bred, leaf_size)
    ki, kd, nat, bad = tree.rows(ared, n_rows, n_cols)
    knn_orig = np.where(ki >= 0, tree.indir[np.maximum(ki, 0)], -1).astype(np.int32)
    nn, nd = ocl_select(knn_orig, pa, pb)
    if return_all:
        return dict(nn=nn, nn_sqdist=nd, knn=knn_orig, knn_pos=ki, knn_sqdist=kd, nat=nat, tree=tree, ared=ared,
                    bred=bred, pa=pa, pb=pb, n_rows=n_rows, n_cols=n_cols, out_of_grid=bad)
    return nn


# ----------------------------------------------------------------------------------------------
# the reference C core, compiled unmodified into oracle/_ref (present only where it was built)
# ----------------------------------------------------------------------------------------------
class KD_TREE_PARAMETERS(ctypes.Structure):
    """Mirror of the reference struct (annfmp/openmp/kdtree/src/include/global.h:22-31)."""
    _fields_ = [("n_neighbors", ctypes.c_int), ("tree_depth", ctypes.c_int),
                ("max_leaves", ctypes.c_int), ("num_threads", ctypes.c_int),
                ("verbosity_level", ctypes.c_int), ("splitting_type", ctypes.c_int)]


def _record_type(real):
    class KD_TREE_RECORD(ctypes.Structure):
        """Mirror of the reference struct (global.h:40-50)."""
        _fields_ = [("Xtrain", ctypes.c_void_p), ("nXtrain", ctypes.c_int), ("dXtrain", ctypes.c_int),
                    ("XI", ctypes.c_void_p), ("nodes", ctypes.c_void_p), ("leaves", ctypes.c_void_p),
                    ("points_leaf_indices", ctypes.c_void_p), ("tree_depth", ctypes.c_int)]
    KD_TREE_RECORD.real = real
    return KD_TREE_RECORD


def reference_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libannfmp_ref_float.so"))


def build_reference(ref_root: str = "/root/reference") -> bool:
    """Compile the reference C core from ref_root into oracle/_ref (False if ref_root is absent)."""
    if not os.path.isdir(ref_root):
        return False
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF={ref_root}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)
    return True


_REF_LIBS: dict = {}


def _ref_lib(real=np.float32):
    key = np.dtype(real).name
    if key not in _REF_LIBS:
        name = "libannfmp_ref_float.so" if key == "float32" else "libannfmp_ref_double.so"
        lib = ctypes.CDLL(os.path.join(REF_DIR, name))
        _REF_LIBS[key] = lib
    return _REF_LIBS[key]


class _SilenceStdout:
    """The reference C core prints progress with printf; keep the test output clean."""

    def __enter__(self):
        sys.stdout.flush()
        self._saved = os.dup(1)
        self._null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self._null, 1)
        return self

    def __exit__(self, *a):
        ctypes.CDLL(None).fflush(None)
        os.dup2(self._saved, 1)
        os.close(self._saved)
        os.close(self._null)


def make_wrapper_module(real=np.float32) -> types.ModuleType:
    """A stand-in for the reference's SWIG module (annfmp/openmp/kdtree/swig/cpu_float.i) that
    forwards numpy buffers to the unmodified reference C core."""
    lib = _ref_lib(real)
    ctreal = ctypes.c_float if np.dtype(real) == np.float32 else ctypes.c_double
    Rec = _record_type(real)
    mod = types.ModuleType("wrapper_cpu_float" if np.dtype(real) == np.float32 else "wrapper_cpu_double")
    mod.KD_TREE_PARAMETERS = KD_TREE_PARAMETERS
    mod.KD_TREE_RECORD = Rec

    def init_extern(k, depth, max_leaves, threads, splitting, verbosity, params):
        lib.init_extern(k, depth, max_leaves, threads, splitting, min(int(verbosity), 1), ctypes.byref(params))

    def fit_extern(X, rec, params):
        assert X.dtype == real and X.flags.c_contiguous
        lib.fit_extern(X.ctypes.data_as(ctypes.POINTER(ctreal)), X.shape[0], X.shape[1],
                       ctypes.byref(rec), ctypes.byref(params))

    def neighbors_extern(X, dist, idx, rec, params):
        with _SilenceStdout():
            lib.neighbors_extern(X.ctypes.data_as(ctypes.POINTER(ctreal)), X.shape[0], X.shape[1],
                                 dist.ctypes.data_as(ctypes.POINTER(ctreal)), dist.shape[0], dist.shape[1],
                                 idx.ctypes.data_as(_c_int_p), idx.shape[0], idx.shape[1],
                                 ctypes.byref(rec), ctypes.byref(params))

    def process_rows_extern(final, pa, pb, ared, n_rows, n_cols, k, propagate, select_best, rec, params):
        with _SilenceStdout():
            lib.process_rows_extern(final.ctypes.data_as(_c_int_p), final.shape[0],
                                    pa.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), pa.shape[0], pa.shape[1],
                                    pb.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), pb.shape[0], pb.shape[1],
                                    ared.ctypes.data_as(ctypes.POINTER(ctreal)), ared.shape[0], ared.shape[1],
                                    n_rows, n_cols, k, propagate, select_best,
                                    ctypes.byref(rec), ctypes.byref(params))

    mod.init_extern = init_extern
    mod.fit_extern = fit_extern
    mod.neighbors_extern = neighbors_extern
    mod.process_rows_extern = process_rows_extern
    mod.free_resources_extern = lambda: None
    return mod


def reference_annfmp(ref_root: str = "/root/reference"):
    """Import the UNMODIFIED reference Python package from ref_root, with the SWIG modules replaced
    by ctypes stand-ins over oracle/_ref. Returns the ``annfmp`` module."""
    if "annfmp" in sys.modules and getattr(sys.modules["annfmp"], "_ora_shim", False):
        return sys.modules["annfmp"]
    sys.dont_write_bytecode = True
    sys.modules["annfmp.openmp.kdtree.wrapper_cpu_float"] = make_wrapper_module(np.float32)
    sys.modules["annfmp.openmp.kdtree.wrapper_cpu_double"] = make_wrapper_module(np.float64)
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    with _SilenceStdout():
        import annfmp  # noqa: E402  (the reference package)
    annfmp._ora_shim = True
    return annfmp


def reference_tree(X: np.ndarray, depth: int):
    """Build a tree with the reference C core (fit_extern) and return its arrays in the oracle's
    structure-of-arrays form: pts, perm, node_axis, node_split, leaf_bounds, point_leaf."""
    X = np.ascontiguousarray(X)
    real = X.dtype.type
    lib = _ref_lib(real)
    ctreal = ctypes.c_float if X.dtype == np.float32 else ctypes.c_double
    params = KD_TREE_PARAMETERS()
    lib.init_extern(1, depth, 2147483640, 1, 1, 0, ctypes.byref(params))
    rec = _record_type(real)()
    lib.fit_extern(X.ctypes.data_as(ctypes.POINTER(ctreal)), X.shape[0], X.shape[1], ctypes.byref(rec),
                   ctypes.byref(params))
    n, d = X.shape
    L = 1 << depth
    esz = X.dtype.itemsize * d + 4
    xi = np.ctypeslib.as_array(ctypes.cast(rec.XI, ctypes.POINTER(ctypes.c_uint8)), shape=(n * esz,)).copy()
    xi = xi.reshape(n, esz)
    pts = xi[:, : X.dtype.itemsize * d].copy().view(X.dtype).reshape(n, d)
    perm = xi[:, X.dtype.itemsize * d:].copy().view(np.int32).reshape(n)
    node_axis = np.zeros(max(L - 1, 0), np.int32)
    node_split = np.zeros(max(L - 1, 0), X.dtype)
    if L > 1:
        if X.dtype == np.float32:
            raw = np.ctypeslib.as_array(ctypes.cast(rec.nodes, ctypes.POINTER(ctypes.c_int32)), shape=(2 * (L - 1),))
            raw = raw.copy()
            node_axis = raw[0::2].copy()
            node_split = raw[1::2].copy().view(np.float32)
        else:  # struct {int axis; double split} -> 16 bytes with padding
            raw = np.ctypeslib.as_array(ctypes.cast(rec.nodes, ctypes.POINTER(ctypes.c_uint8)), shape=(16 * (L - 1),))
            raw = raw.copy().reshape(L - 1, 16)
            node_axis = raw[:, 0:4].copy().view(np.int32).reshape(-1)
            node_split = raw[:, 8:16].copy().view(np.float64).reshape(-1)
    leaves = np.ctypeslib.as_array(ctypes.cast(rec.leaves, _c_int_p), shape=(2 * L,)).copy()
    point_leaf = np.ctypeslib.as_array(ctypes.cast(rec.points_leaf_indices, _c_int_p), shape=(n,)).copy()
    # the reference never frees its record (annfmp/openmp/kdtree/src/base.c:379-381); neither do we
    return dict(pts=pts, perm=perm, node_axis=node_axis, node_split=node_split, leaf_bounds=leaves,
                point_leaf=point_leaf, _rec=rec, _params=params, _X=X)


def reference_process_rows(rt: dict, ared, pa, pb, n_rows, n_cols, K, propagate=True, select_best=True):
    """process_rows_extern of the reference core on a tree from reference_tree (needs the tree
    built with n_neighbors=K; rebuilt here if not)."""
    X = rt["_X"]
    real = X.dtype.type
    lib = _ref_lib(real)
    ctreal = ctypes.c_float if X.dtype == np.float32 else ctypes.c_double
    params = rt["_params"]
    params.n_neighbors = K
    ared = np.ascontiguousarray(ared, dtype=real)
    pa = np.ascontiguousarray(pa, dtype=np.uint8)
    pb = np.ascontiguousarray(pb, dtype=np.uint8)
    final = np.zeros(ared.shape[0], np.int32)
    with _SilenceStdout():
        lib.process_rows_extern(final.ctypes.data_as(_c_int_p), final.shape[0],
                                pa.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), pa.shape[0], pa.shape[1],
                                pb.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), pb.shape[0], pb.shape[1],
                                ared.ctypes.data_as(ctypes.POINTER(ctreal)), ared.shape[0], ared.shape[1],
                                n_rows, n_cols, K, int(propagate), int(select_best),
                                ctypes.byref(rt["_rec"]), ctypes.byref(params))
    return final
