"""KDTree: the reference's k-d tree estimator (annfmp/openmp/kdtree/base.py:18-315) on the GPU.

Same constructor parameters, ``fit`` / ``kneighbors`` / ``process_rows`` entry points and array
outputs as the reference class, backed by the CUDA kernels of libannf_gb300.so. Inputs may be
numpy arrays (results come back as numpy, like the reference) or torch tensors (results stay on
the device).
"""
from __future__ import annotations

import math
import multiprocessing
import warnings

import numpy as np
import torch

from . import _lib
from ._torch import is_numpy, ptr, require_cuda, stream_ptr, to_device


class KDTree(object):
    SPLITTING_TYPE_MAPPINGS = {"cyclic": _lib.ANNF_SPLIT_CYCLIC, "longest": _lib.ANNF_SPLIT_LONGEST}
    ALLOWED_FLOAT_TYPES = ["float", "double"]

    def __init__(self, n_neighbors=5, leaf_size=30, max_leaves=None, tree_depth=None, float_type="double",
                 splitting_type="cyclic", n_jobs=1, verbose=0, device=0):
        self.n_neighbors = n_neighbors
        self.leaf_size = leaf_size
        self.max_leaves = max_leaves
        self.tree_depth = tree_depth
        self.float_type = float_type
        self.splitting_type = splitting_type
        self.n_jobs = n_jobs
        self.verbose = verbose
        self.device = device
        self._handle = None

    def get_params(self):
        return {"n_neighbors": self.n_neighbors, "leaf_size": self.leaf_size, "max_leaves": self.max_leaves,
                "tree_depth": self.tree_depth, "float_type": self.float_type,
                "splitting_type": self.splitting_type, "n_jobs": self.n_jobs, "verbose": self.verbose}

    # -- helpers --------------------------------------------------------------------------------
    def _torch_dtype(self):
        return torch.float32 if self.float_type == "float" else torch.float64

    def _real_type(self):
        return _lib.ANNF_REAL_F32 if self.float_type == "float" else _lib.ANNF_REAL_F64

    def _final_max_leaves(self) -> int:
        # annfmp/openmp/kdtree/base.py:126-131
        if self.max_leaves is None:
            return 2147483640
        if self.max_leaves < 0:
            raise Exception("max_leaves must be a positive integer")
        return int(self.max_leaves)

    def _compute_final_tree_depth(self, n, leaf_size, tree_depth):
        """annfmp/openmp/kdtree/base.py:260-300 (same formula, same warnings)."""
        d = int(math.floor(math.log(n, 2)))
        if tree_depth is not None:
            if tree_depth > d:
                warnings.warn("tree_depth %i too large (using smaller depth): %i.\n" % (tree_depth, d))
                return d
            return tree_depth
        if not self.leaf_size > 1:
            raise Exception("Parameter 'leaf_size' must be larger than 1")
        subtr = int(math.floor(math.log(leaf_size, 2)))
        if d - subtr < 0:
            warnings.warn("tree_depth smaller than 0; setting tree_depth to 0")
            return 0
        return d - subtr

    @property
    def handle(self) -> _lib.Handle:
        if self._handle is None:
            self._dev = require_cuda(self.device)
            self._handle = _lib.Handle(self._dev.index)
        return self._handle

    # -- API ------------------------------------------------------------------------------------
    def fit(self, X):
        assert self.float_type in self.ALLOWED_FLOAT_TYPES
        if self.splitting_type not in self.SPLITTING_TYPE_MAPPINGS:
            raise Exception("Unknown splitting type!")
        if not (1 <= int(self.n_neighbors) <= 1000):  # helper.c:32-35
            raise ValueError("Error: k must be > 0 and <= 1000)")
        h = self.handle
        self._numpy_io = is_numpy(X)
        self.X = to_device(X, self._torch_dtype(), self._dev)
        if self.X.dim() != 2:
            raise ValueError("X must be 2-dimensional")
        n, d = self.X.shape
        self.final_tree_depth_ = self._compute_final_tree_depth(n, self.leaf_size, self.tree_depth)
        if self.verbose > 0:
            print("Final tree depth: " + str(self.final_tree_depth_))
        self._final_max_leaves()
        h.call("annf_build_tree", ptr(self.X), n, d, self._real_type(), self.final_tree_depth_,
               self.SPLITTING_TYPE_MAPPINGS[self.splitting_type], stream_ptr(self._dev))
        return self

    def kneighbors(self, X=None, n_neighbors=None, return_distance=True):
        assert return_distance == True  # noqa: E712  (reference contract)
        if n_neighbors is not None and self.n_neighbors != n_neighbors:
            self.n_neighbors = n_neighbors
            if self.verbose > 0:
                print("\nMODEL MUST BE RETRAINED ...\n")
            self.fit(self.X)
        numpy_out = self._numpy_io if X is None else is_numpy(X)
        Q = self.X if X is None else to_device(X, self._torch_dtype(), self._dev)
        nq = Q.shape[0]
        k = int(self.n_neighbors)
        dist = torch.empty((nq, k), dtype=self._torch_dtype(), device=self._dev)
        idx = torch.empty((nq, k), dtype=torch.int32, device=self._dev)
        self.handle.call("annf_kneighbors", ptr(Q), nq, k, self._final_max_leaves(), ptr(dist), ptr(idx),
                         stream_ptr(self._dev))
        if numpy_out:
            return dist.cpu().numpy(), idx.cpu().numpy()
        return dist, idx

    def natural_kneighbors(self, X, n_neighbors=None, leaf_precision="fp32"):
        """Original indices [nq, k] of each query's k nearest points inside the leaf its descent
        reaches (the reference's traversal with max_leaves=1), nearest first. ``leaf_precision``
        "fp32" scans the leaf exactly; "bf16" / "fp16" compute tensor-core distance tiles and re-rank
        exactly (FP32) every point within the tiles' proven rounding bound, so the result is the
        same."""
        numpy_out = is_numpy(X)
        Q = to_device(X, self._torch_dtype(), self._dev)
        k = int(n_neighbors or self.n_neighbors)
        prec = {"fp32": _lib.ANNF_LEAF_EXACT, "bf16": _lib.ANNF_LEAF_BF16, "fp16": _lib.ANNF_LEAF_FP16,
                "fp8": _lib.ANNF_LEAF_FP8}[leaf_precision]
        pos = torch.empty((Q.shape[0], k), dtype=torch.int32, device=self._dev)
        self.handle.call("annf_natural_knn", ptr(Q), Q.shape[0], k, prec, ptr(pos), stream_ptr(self._dev))
        tv = self.handle.tree_view()
        perm = device_view(tv.perm, (tv.n,), np.int32, self._dev)
        idx = perm[pos.long()]
        return idx.cpu().numpy() if numpy_out else idx

    def process_rows(self, nn_indices, patches_a, patches_b, patchesred, n_rows, n_cols, n_neighbors=None,
                     propagate=True, select_best_nn=True):
        """Row-propagation NNF (annfmp/openmp/kdtree/base.py:210-241); the chosen B index of every
        A pixel is written into ``nn_indices`` (numpy int32 array or int32 tensor) in place."""
        if n_neighbors is not None and self.n_neighbors != n_neighbors:
            self.n_neighbors = n_neighbors
            if self.verbose > 0:
                print("\nMODEL MUST BE RETRAINED ...\n")
            self.fit(self.X)
        dev = self._dev
        k = int(self.n_neighbors)
        ared = to_device(patchesred, self._torch_dtype(), dev)
        nA = ared.shape[0]
        pa = pb = None
        P = 0
        if select_best_nn:
            pa = to_device(patches_a, torch.uint8, dev)
            pb = to_device(patches_b, torch.uint8, dev)
            P = pa.shape[1]
        out = torch.empty(nA, dtype=torch.int32, device=dev)
        self.knn_indices_ = torch.empty((nA, k), dtype=torch.int32, device=dev)
        self.nn_distances_ = torch.empty(nA, dtype=torch.float32, device=dev)
        self.handle.call("annf_process_rows", ptr(out), ptr(pa), nA if pa is not None else 0, ptr(pb),
                         pb.shape[0] if pb is not None else 0, P, ptr(ared), int(n_rows), int(n_cols), k,
                         int(bool(propagate)), int(bool(select_best_nn)), self._final_max_leaves(),
                         ptr(self.knn_indices_), ptr(self.nn_distances_), stream_ptr(dev))
        self.check_device()
        if isinstance(nn_indices, torch.Tensor):
            nn_indices.copy_(out)
        else:
            nn_indices[...] = out.cpu().numpy()
        return nn_indices

    def check_device(self):
        bits = _lib.ctypes.c_uint(0)
        _lib.check(self.handle.lib.annf_device_status(self.handle.h, stream_ptr(self._dev), _lib.ctypes.byref(bits)))

    # -- tree arrays (for parity checks and integration) ----------------------------------------
    def tree_arrays(self) -> dict:
        """Copies of the device tree arrays, in the reference's layout terms:
        points (tree order), perm (tree position -> original index), node_axis, node_split,
        leaves (2 ints per leaf: begin, end), point_leaf (original index -> leaf), leaf_box
        ([leaves, 2, d]: per leaf the minimum, then the maximum, of each coordinate)."""
        tv = self.handle.tree_view()
        torch.cuda.current_stream(self._dev).synchronize()
        real = np.float32 if tv.real_type == _lib.ANNF_REAL_F32 else np.float64
        L = tv.n_leaves

        def fetch(p, count, dtype):
            if count == 0:
                return np.empty(0, dtype)
            return device_view(p, (count,), dtype, self._dev).cpu().numpy().copy()

        lb = fetch(tv.leaf_begin, L + 1, np.int32)
        return dict(points=fetch(tv.points, tv.n * tv.d, real).reshape(tv.n, tv.d),
                    perm=fetch(tv.perm, tv.n, np.int32),
                    node_axis=fetch(tv.node_axis, max(L - 1, 0), np.int32),
                    node_split=fetch(tv.node_split, max(L - 1, 0), real),
                    leaves=np.stack([lb[:-1], lb[1:]], axis=1).reshape(-1).astype(np.int32),
                    point_leaf=fetch(tv.point_leaf, tv.n, np.int32),
                    leaf_box=fetch(tv.leaf_box, 2 * L * tv.d, real).reshape(L, 2, tv.d))

    def __repr__(self):
        return str(self.get_params())


class _DevArray:
    """Zero-copy description of a device buffer for torch.as_tensor."""

    def __init__(self, p: int, shape, dtype):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": np.dtype(dtype).str,
                                         "data": (int(p), False), "version": 2, "strides": None}


def device_view(p: int, shape, dtype, device) -> torch.Tensor:
    """A torch tensor aliasing device memory owned by the library (valid while the tree lives)."""
    return torch.as_tensor(_DevArray(p, shape, dtype), device=device)


def default_n_jobs(n_jobs):
    """annfmp/openmp/kdtree/base.py:133-136 (kept for signature parity; the GPU ignores it)."""
    return multiprocessing.cpu_count() if n_jobs < 1 else n_jobs
