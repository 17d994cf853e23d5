"""ANNFieldPropKDTreeOpenCLOPTGB300: the NNF of annfmp's GPU backend ("openclopt",
annfmp/openclopt/base.py:17-137 driving annfmp/openclopt/src/base.c:fit_extern) on this library's
kernels, for comparison with that backend.

Same constructor parameters and ``fit`` as the reference class. As there, K is 8 whatever
``n_neighbors`` is and ``select_best_nn`` must be True. The PCA fit is the reference's (the same
sampled patches and covariance eigendecomposition as the plain pipeline); the patches are
projected by the exact projection (the FP64 value rounded once; the backend's own FP32 reduction,
driverKNN.fut:47-54, has no specified summation order). Tree, lists and select best follow the
backend's Futhark programs (``annf_ocl_build_tree``, ``annf_ocl_rows``).
"""
from __future__ import annotations

import collections
import ctypes
import time

import numpy
import torch

from . import _lib
from ._torch import is_numpy, ptr, require_cuda, stream_ptr, to_device
from .field import _SUBSETS

K_FIXED = 8  # driverKNN.fut:13


class ANNFieldPropKDTreeOpenCLOPTGB300:
    def __init__(self, n_neighbors=3, psize=8, dim_reduced=5, n_subset=1000, leaf_size=64, n_jobs=-1,
                 select_best_nn=True, verbose=1, seed=0, platform_id=0, device_id=0):
        self.n_neighbors = n_neighbors
        self.psize = psize
        self.dim_reduced = dim_reduced
        self.n_subset = n_subset
        self.leaf_size = leaf_size
        self.n_jobs = n_jobs
        self.select_best_nn = select_best_nn
        self.verbose = verbose
        self.seed = seed
        self.platform_id = platform_id
        self.device_id = device_id
        self._handle = None

    def _get_handle(self, dev):
        if self._handle is None or self._handle.device != dev.index:
            self._handle = _lib.Handle(dev.index)
        return self._handle

    def fit(self, image_a, image_b):
        """Returns the B patch index of every A patch (row-major), numpy for numpy inputs."""
        assert self.select_best_nn == True  # noqa: E712  (annfmp/openclopt/base.py:50)
        self._timers = collections.OrderedDict()
        dev = require_cuda(self.device_id)
        numpy_io = is_numpy(image_a)
        tstart = time.time()
        A = to_device(image_a, torch.uint8, dev)
        B = to_device(image_b, torch.uint8, dev)
        if A.dim() == 2:
            A, B = A.unsqueeze(-1), B.unsqueeze(-1)
        ha, wa, c = A.shape
        hb, wb, _ = B.shape
        p, d = int(self.psize), int(self.dim_reduced)
        P = p * p * c
        h = self._get_handle(dev)
        st = stream_ptr(dev)
        self._n_rows, self._n_cols = ha - p + 1, wa - p + 1
        n_a, n_b = self._n_rows * self._n_cols, (hb - p + 1) * (wb - p + 1)
        # PCA fit (annfmp/openclopt/base.py:201-227): n_subset/2 sampled patches of each image
        m = int(self.n_subset / 2)
        pos_a = _SUBSETS.get(self._n_rows, self._n_cols, m, self.seed, dev)
        pos_b = _SUBSETS.get(hb - p + 1, wb - p + 1, m, self.seed + 1, dev)
        self.components_ = torch.empty((d, P), dtype=torch.float64, device=dev)
        self.mean_ = torch.empty(P, dtype=torch.float64, device=dev)
        h.call("annf_pca_covariance", ptr(A), ha, wa, ptr(pos_a), pos_a.shape[0], ptr(B), hb, wb, ptr(pos_b),
               pos_b.shape[0], c, p, ptr(self.mean_), st)
        h.call("annf_pca_components", P, d, 0, ptr(self.components_), st)
        torch.cuda.synchronize(dev)
        self._timers["pca_fit"] = time.time() - tstart
        tstart = time.time()
        self.patches_a_reduced_ = torch.empty((n_a, d), dtype=torch.float32, device=dev)
        self.patches_b_reduced_ = torch.empty((n_b, d), dtype=torch.float32, device=dev)
        for img, hh, ww, out in ((A, ha, wa, self.patches_a_reduced_), (B, hb, wb, self.patches_b_reduced_)):
            h.call("annf_project", ptr(img), hh, ww, c, p, ptr(self.components_), ptr(self.mean_), d,
                   _lib.ANNF_REAL_F32, ptr(out), st)
        self._timers["python_overhead"] = time.time() - tstart
        tstart = time.time()
        h.call("annf_ocl_build_tree", ptr(self.patches_b_reduced_), n_b, d, int(self.leaf_size), st)
        nn = torch.empty(n_a, dtype=torch.int32, device=dev)
        self.knn_indices_ = torch.empty((n_a, K_FIXED), dtype=torch.int32, device=dev)
        self.knn_sqdist_ = torch.empty((n_a, K_FIXED), dtype=torch.float32, device=dev)
        self.nn_distances_ = torch.empty(n_a, dtype=torch.float32, device=dev)
        h.call("annf_ocl_rows", ptr(nn), ptr(A), ha, wa, ptr(B), hb, wb, c, p, ptr(self.patches_a_reduced_),
               self._n_rows, self._n_cols, ptr(self.knn_indices_), ptr(self.knn_sqdist_), ptr(self.nn_distances_), st)
        h.call("annf_device_status", st, ctypes.byref(ctypes.c_uint()))  # synchronises; raises on a tripped check
        self._timers["futhark"] = time.time() - tstart
        self._A, self._B = A, B
        if self.verbose > 0:
            print("-----------------------------------------")
            print("--------------- RUNTIMES ----------------")
            print("-----------------------------------------")
            print("PCA fit:\t\t{}".format(self._timers["pca_fit"]))
            print("Python overhead:\t{}".format(self._timers["python_overhead"]))
            print("Futhark:\t\t{}".format(self._timers["futhark"]))
            print("Total runtime:\t\t{}".format(sum(self._timers.values())))
            print("-----------------------------------------")
        return nn.cpu().numpy() if numpy_io else nn

    def tree_arrays(self) -> dict:
        """The backend's tree as numpy arrays (for tests)."""
        tv = _lib.OclTreeView()
        _lib.check(self._handle.lib.annf_ocl_tree_get(self._handle.h, ctypes.byref(tv)))
        dev = torch.device("cuda", self._handle.device)

        def arr(p, n, dt):
            from .kdtree import device_view
            return device_view(p, (n,), dt, dev).cpu().numpy()
        return dict(height=tv.height, n_nodes=tv.n_nodes, ppl=tv.points_per_leaf, m_padded=tv.m_padded,
                    points=arr(tv.points, tv.m_padded * tv.d, numpy.float32).reshape(tv.m_padded, tv.d),
                    indir=arr(tv.indir, tv.m_padded, numpy.int32),
                    dims=arr(tv.node_dim, tv.n_nodes, numpy.int32) if tv.n_nodes else numpy.zeros(0, numpy.int32),
                    vals=arr(tv.node_val, tv.n_nodes, numpy.float32) if tv.n_nodes else numpy.zeros(0, numpy.float32),
                    clanc=arr(tv.node_same_dim_ancestor, tv.n_nodes, numpy.int32) if tv.n_nodes else
                    numpy.zeros(0, numpy.int32),
                    orig2leaf=arr(tv.orig2leaf, tv.m_padded, numpy.int32))

    def _create_patches(self, img):
        img = img.cpu().numpy() if isinstance(img, torch.Tensor) else numpy.asarray(img)
        if img.ndim == 2:
            img = img[:, :, None]
        p = self.psize
        win = numpy.lib.stride_tricks.sliding_window_view(img, (p, p, img.shape[2]))[:, :, 0]
        return win.reshape(-1, p * p * img.shape[2]).copy()

    @property
    def patches_a(self):
        return self._create_patches(self._A)

    @property
    def patches_b(self):
        return self._create_patches(self._B)

