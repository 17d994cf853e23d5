"""ANNFieldPropKDTreeGB300: the reference's OpenMP NNF pipeline (annfmp/openmp/base.py:16-218),
re-built for one GB300 GPU.

Same constructor parameters, ``fit(image_a, image_b)`` returning one int32 B-patch index per A
pixel (row-major), ``patches_a`` / ``patches_b`` properties and per-stage ``_timers``. Stages:

1. PCA fit on n_subset/2 sampled patches of A (RandomState(seed)) and of B (seed+1), exactly as
   scikit-learn's extract_patches_2d samples them; exact Gram matrix, FP64 covariance, its leading
   eigenvectors in FP64 (the library's subspace solver; cuSOLVER's full eigh with
   ``pca_solver="full"``), all on the GPU (``annf_pca_covariance`` + ``annf_pca_components``);
2. patch extraction fused into the projection: every patch of A and B is projected straight from
   the image (``annf_project``) -- the reference's 1 GB-scale uint8 patch arrays and 8 GB FP64
   copies never exist;
3. k-d tree over B's reduced patches (``annf_build_tree``, longest-axis splits);
4. exact first row, row propagation, raw-patch re-rank (``annf_process_rows_img``).

Extensions (not in the reference): ``nn_distances_`` (raw-patch L2 of each chosen index),
``knn_indices_`` (each pixel's k-list), torch CUDA tensors accepted as images (results then stay
on the device), repeated fits replayed as one CUDA graph, and ``form="parallel"``: no row chain
(natural-leaf candidates from tensor-core tiles, optional learned proposals, parallel
propagation passes, every candidate verified by its exact raw-patch distance).
"""
from __future__ import annotations

import collections

import numpy
import torch

from . import _lib
from ._torch import is_numpy, ptr, require_cuda, stream_ptr, to_device
from .kdtree import KDTree


class _SubsetCache:
    """Sampled patch positions depend only on (patch grid, count, seed): keep them on the device."""

    def __init__(self):
        self._d = collections.OrderedDict()

    def get(self, n_h, n_w, m, seed, device):
        key = (n_h, n_w, m, seed, str(device))
        if key in self._d:
            self._d.move_to_end(key)
            return self._d[key]
        total = n_h * n_w
        if not m or m >= total:  # sklearn _compute_n_patches: every patch
            yy, xx = torch.meshgrid(torch.arange(n_h, device=device, dtype=torch.int32),
                                    torch.arange(n_w, device=device, dtype=torch.int32), indexing="ij")
            pos = torch.stack([yy.reshape(-1), xx.reshape(-1)], dim=1).contiguous()
        else:
            rs = numpy.random.RandomState(seed)
            i_s = rs.randint(n_h, size=m)
            j_s = rs.randint(n_w, size=m)
            # in image order: the covariance is an exact integer sum over the samples (the same bits
            # in any order), and the gather then walks the images row by row
            order = numpy.lexsort((j_s, i_s))
            pos = torch.from_numpy(numpy.stack([i_s[order], j_s[order]], axis=1).astype(numpy.int32)).to(device)
        self._d[key] = pos
        while len(self._d) > 1024:
            self._d.popitem(last=False)
        return pos


_SUBSETS = _SubsetCache()


class _Marks(dict):
    """Stage events for the timers (no-ops when the call must stay free of host synchronisation)."""

    class _Null:
        def record(self):
            pass

    def __init__(self, timing):
        super().__init__()
        for k in ("t0", "t1", "t2", "t3", "t4"):
            self[k] = torch.cuda.Event(enable_timing=True) if timing else _Marks._Null()


class ANNFieldPropKDTreeGB300:
    FORMS = ("plain", "parallel")

    def __init__(self, n_neighbors=3, psize=8, dim_reduced=5, n_subset=1000, leaf_size=64, n_jobs=-1,
                 propagate=True, select_best_nn=True, float_type="float", verbose=1, seed=0, device=0,
                 form="plain", iters=4, proposal=None, pca_solver=None, pca_iters=6, leaf_precision=None,
                 projection=None, search=(1, 2), graph="auto"):
        """Reference parameters, plus: ``form`` "plain" (the reference's row-sequential method,
        the drop-in) or "parallel" (natural-leaf candidates + proposals + parallel propagation,
        every candidate checked by exact raw-patch distance); ``iters`` propagation passes of the
        parallel form; ``proposal`` an object with ``propose(A, B, psize) -> int32 [n_A, P]`` B
        indices (e.g. ``annfmp_gb300.proposal.ProposalNet``) feeding the parallel form;
        ``pca_solver`` "exact" (the reference's result: the leading eigenvectors in FP64, by
        subspace iteration over all SMs and an FP64 Rayleigh-Ritz step), "full" (the full FP64
        eigendecomposition by cuSOLVER) or "subspace" (FP32 subspace iteration, ``pca_iters``
        steps, with an FP64 Rayleigh-Ritz step); None picks "exact" for the plain form,
        "subspace" otherwise;
        ``leaf_precision`` of the parallel form's natural-leaf distances: "bf16" (tensor-core tiles,
        exact FP32 re-rank of the survivors of a proven BF16 error bound; the default) or "fp32";
        ``projection`` "exact" (the FP64 result rounded once, the reference's) or "fp16" (FP16
        components on the tensor cores, FP32 sums); None picks "exact" for the plain form, "fp16"
        otherwise when the shapes allow it; ``graph``: repeated fits with unchanged shapes and
        parameters replay one captured CUDA graph of the whole NNF ("auto": every form; False:
        never; not with pca_solver "full", whose library solver sizes its workspace on the
        host)."""
        self.graph = graph
        self._graph = None       # captured state: key, epoch, graph, static inputs, outputs
        self._graph_seen = None  # key of the last eager fit (capture happens on the second call)
        self.leaf_precision = leaf_precision
        self.projection = projection
        self.search = search  # parallel form: (random offsets per pass, initial search radius)
        self.pca_solver = pca_solver
        self.pca_iters = pca_iters
        self.form = form
        self.iters = iters
        self.proposal = proposal
        self.n_neighbors = n_neighbors
        self.psize = psize
        self.dim_reduced = dim_reduced
        self.n_subset = n_subset
        self.leaf_size = leaf_size
        self.n_jobs = n_jobs
        self.propagate = propagate
        self.select_best_nn = select_best_nn
        self.float_type = float_type
        self.verbose = verbose
        self.seed = seed
        self.device = device

    def _get_torch_float_type(self):
        if self.float_type == "float":
            return torch.float32
        elif self.float_type == "double":
            return torch.float64
        raise Exception("Unknown float type: {}".format(self.float_type))

    def fit(self, image_a, image_b, sync=True):
        """image_a and image_b have shape (h, w, c), uint8 (numpy or torch). sync=False (device
        tensors only) enqueues the whole NNF on the current stream without any host
        synchronisation, timing or status check, so that it can be captured into a CUDA graph; the
        returned tensor is filled when the stream reaches it.

        With graphs enabled, the first fit of a (shapes, parameters) combination runs eagerly
        (sizing every device buffer), the second captures the NNF into a CUDA graph with static
        input images, and later fits copy the inputs in and replay it: one launch per NNF. The
        graph is dropped when the shapes or parameters change or when any of the library's
        device buffers has been reallocated since the capture."""
        if sync and self._graph_wanted():
            return self._fit_graph(image_a, image_b)
        return self._fit(image_a, image_b, sync)

    # -- CUDA graph replay --------------------------------------------------------------------------
    def _graph_wanted(self):
        full = self.pca_solver == "full"
        if self.graph == "auto":
            return not full
        if self.graph and full:
            raise ValueError("pca_solver 'full' cannot be captured into a CUDA graph (its library solver sizes "
                             "its workspace on the host)")
        return bool(self.graph)

    def _graph_key(self, image_a, image_b, dev):
        shape = lambda x: tuple(x.shape) if hasattr(x, "shape") else tuple(numpy.asarray(x).shape)  # noqa: E731
        return (shape(image_a), shape(image_b), str(dev), self.form, self.n_neighbors, self.psize,
                self.dim_reduced, self.n_subset, self.leaf_size, self.iters, self.seed, self.float_type,
                self.leaf_precision, self.projection, tuple(self.search), self.pca_solver, self.pca_iters,
                id(self.proposal), bool(self.propagate), bool(self.select_best_nn))

    # attributes a fit leaves behind; a replay points them back at the graph's tensors
    _FIT_ATTRS = ("components_", "mean_", "patches_a_reduced_", "patches_b_reduced_", "nn_distances_",
                  "_subset_pos", "_n_rows", "_n_cols", "kdtree", "_A", "_B")

    def _capture(self, image_a, image_b, key, dev):
        from ._torch import to_device as _to
        A_s = _to(image_a, torch.uint8, dev).clone()
        B_s = _to(image_b, torch.uint8, dev).clone()
        epoch = _lib.buffer_epoch()
        cur = torch.cuda.current_stream(dev)
        warm = torch.cuda.Stream(dev)
        warm.wait_stream(cur)
        with torch.cuda.stream(warm):  # warm the capture on a side stream (torch's recommendation)
            self._fit(A_s, B_s, sync=False)
        cur.wait_stream(warm)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        launches = _lib.launch_count()
        with torch.cuda.graph(g, capture_error_mode="relaxed"):
            nn = self._fit(A_s, B_s, sync=False)
        torch.cuda.synchronize(dev)
        launches = _lib.launch_count() - launches
        if _lib.buffer_epoch() != epoch:  # a buffer grew during the capture: its nodes are stale
            return None
        attrs = {a: getattr(self, a) for a in self._FIT_ATTRS if hasattr(self, a)}
        return {"key": key, "epoch": epoch, "graph": g, "A": A_s, "B": B_s, "nn": nn, "attrs": attrs,
                "tree_X": self._tree.X, "kernels": launches}

    def _fit_graph(self, image_a, image_b):
        dev = require_cuda(self.device)
        key = self._graph_key(image_a, image_b, dev)
        g = self._graph
        if g is not None and (g["key"] != key or g["epoch"] != _lib.buffer_epoch()):
            self._graph = g = None
        if g is None:
            if self._graph_seen != key:  # first fit of this combination: eager, sizes every buffer
                nn = self._fit(image_a, image_b, True)
                self._graph_seen = key
                return nn
            self._graph = g = self._capture(image_a, image_b, key, dev)
            if g is None:
                self._graph_seen = None
                return self._fit(image_a, image_b, True)
        numpy_io = is_numpy(image_a)
        self.image_a = image_a
        self.image_b = image_b
        for src, dst in ((image_a, g["A"]), (image_b, g["B"])):
            if isinstance(src, torch.Tensor):
                dst.copy_(src.reshape(dst.shape), non_blocking=True)
            else:
                dst.copy_(torch.from_numpy(numpy.ascontiguousarray(src, dtype=numpy.uint8)).reshape(dst.shape))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g["graph"].replay()
        e1.record()
        for a, v in g["attrs"].items():
            setattr(self, a, v)
        self._tree.X = g["tree_X"]
        self._tree.check_device()  # synchronises and raises if a kernel's bounds check tripped
        self._timers = collections.OrderedDict(graph=e0.elapsed_time(e1) / 1e3)
        if self.verbose > 0:
            print("Graph replay (whole NNF):\t{}".format(self._timers["graph"]))
        if numpy_io:
            return g["nn"].cpu().numpy()
        return g["nn"].clone()

    def _fit(self, image_a, image_b, sync):
        """With proposals, the NNF's own chain runs on a high-priority stream: the side stream's
        proposal kernels then fill idle SMs without holding back the eigensolver (a one-CTA kernel
        that needs a whole SM)."""
        if self.form == "plain" or self.proposal is None:
            return self._fit_chain(image_a, image_b, sync)
        dev = require_cuda(self.device)
        caller = torch.cuda.current_stream(dev)
        hp = getattr(self, "_hp", None)
        if hp is None:
            hp = self._hp = torch.cuda.Stream(dev, priority=-8)  # clamped to the highest priority
        hp.wait_stream(caller)
        with torch.cuda.stream(hp):
            nn = self._fit_chain(image_a, image_b, sync)
        caller.wait_stream(hp)
        if isinstance(nn, torch.Tensor):
            nn.record_stream(caller)
        return nn

    def _fit_chain(self, image_a, image_b, sync):
        numpy.random.seed(self.seed)  # annfmp/openmp/base.py:60
        dev = require_cuda(self.device)
        real = self._get_torch_float_type()
        real_type = _lib.ANNF_REAL_F32 if real == torch.float32 else _lib.ANNF_REAL_F64
        numpy_io = is_numpy(image_a)
        self.image_a = image_a
        self.image_b = image_b
        A = to_device(image_a, torch.uint8, dev)
        B = to_device(image_b, torch.uint8, dev)
        if A.dim() == 2:
            A = A.unsqueeze(-1)
        if B.dim() == 2:
            B = B.unsqueeze(-1)
        if A.shape[2] != B.shape[2]:
            raise ValueError("images must have the same number of channels")
        ha, wa, c = A.shape
        hb, wb, _ = B.shape
        p = int(self.psize)
        if p > min(ha, wa, hb, wb):
            raise ValueError("Height/width of the patch should be less than the height/width of the image.")
        self._n_cols = wa - p + 1
        self._n_rows = ha - p + 1
        n_a = self._n_rows * self._n_cols
        n_b = (hb - p + 1) * (wb - p + 1)
        P = p * p * c
        d = int(self.dim_reduced)
        st = stream_ptr(dev)
        if not hasattr(self, "_tree") or self._tree is None:
            self._tree = KDTree(n_neighbors=self.n_neighbors, leaf_size=self.leaf_size, splitting_type="longest",
                                n_jobs=self.n_jobs, float_type=self.float_type, verbose=0, device=dev.index)
        tree = self._tree
        tree.n_neighbors = self.n_neighbors
        tree.leaf_size = self.leaf_size
        tree.float_type = self.float_type
        h = tree.handle
        ev = _Marks(sync)
        ev["t0"].record()

        # offset proposals depend only on the images: computed on a side stream that starts once
        # the covariance is formed, beside the eigensolver (which keeps one SM busy and leaves the
        # rest idle); joined before the candidates
        prop, side, seeded = None, None, False

        def start_proposals():
            nonlocal prop, side, seeded
            if self.form == "plain" or self.proposal is None:
                return
            side = torch.cuda.Stream(dev) if getattr(self, "_side", None) is None else self._side
            self._side = side
            side.wait_stream(torch.cuda.current_stream(dev))
            with torch.cuda.stream(side):
                prop = self.proposal.propose(A, B, p)
                # their exact distances need no tree: the best proposal of each pixel, here too
                if prop is not None and hasattr(self.proposal, "seed"):
                    prop = self.proposal.seed(A, B, p, prop)
                    seeded = True

        # (1) PCA fit on the sampled subset (annfmp/openmp/base.py:168-191)
        m = int(self.n_subset / 2)
        pos_a = _SUBSETS.get(self._n_rows, self._n_cols, m, self.seed, dev)
        pos_b = _SUBSETS.get(hb - p + 1, wb - p + 1, m, self.seed + 1, dev)
        self._subset_pos = (pos_a, pos_b)  # kept alive while a captured graph reads them
        self.components_ = torch.empty((d, P), dtype=torch.float64, device=dev)
        self.mean_ = torch.empty(P, dtype=torch.float64, device=dev)
        if self.form not in self.FORMS:
            raise ValueError("form must be one of {}".format(self.FORMS))
        solver = self.pca_solver or ("exact" if self.form == "plain" else "subspace")
        if solver in ("exact", "full"):
            h.call("annf_pca_covariance", ptr(A), ha, wa, ptr(pos_a), pos_a.shape[0], ptr(B), hb, wb, ptr(pos_b),
                   pos_b.shape[0], c, p, ptr(self.mean_), st)
            h.call("annf_pca_components", P, d, 0 if solver == "exact" else -1, ptr(self.components_), st)
        elif solver == "subspace":
            h.call("annf_pca_covariance", ptr(A), ha, wa, ptr(pos_a), pos_a.shape[0], ptr(B), hb, wb, ptr(pos_b),
                   pos_b.shape[0], c, p, ptr(self.mean_), st)
            start_proposals()
            h.call("annf_pca_components", P, d, int(self.pca_iters), ptr(self.components_), st)
        else:
            raise ValueError("pca_solver must be 'exact', 'full' or 'subspace'")
        if side is None:
            start_proposals()  # (the exact solver: after the whole fit)
        ev["t1"].record()

        # (2)+(3) patches projected straight from the images (annfmp/openmp/base.py:152-166, 193-200)
        self.patches_a_reduced_ = torch.empty((n_a, d), dtype=real, device=dev)
        self.patches_b_reduced_ = torch.empty((n_b, d), dtype=real, device=dev)
        proj = self.projection
        if proj is None:
            proj = "fp16" if (self.form != "plain" and real == torch.float32 and p * p * c <= 256 and d <= 32) else "exact"
        a_side = None
        if proj == "fp16":
            if real != torch.float32:
                raise ValueError("the FP16 projection needs float_type='float'")
            h.call("annf_project_f16", ptr(B), hb, wb, c, p, ptr(self.components_), ptr(self.mean_), d,
                   ptr(self.patches_b_reduced_), st)
            # A's patches are needed only from the leaf stage on: projected on another stream (with
            # a handle of its own) while the tree over B is built, whose small per-level kernels
            # leave SMs idle
            a_side = self._a_stream if getattr(self, "_a_stream", None) is not None else torch.cuda.Stream(dev)
            self._a_stream = a_side
            if getattr(self, "_a_handle", None) is None:
                self._a_handle = _lib.Handle(dev.index)
            a_side.wait_stream(torch.cuda.current_stream(dev))
            with torch.cuda.stream(a_side):
                self._a_handle.call("annf_project_f16", ptr(A), ha, wa, c, p, ptr(self.components_), ptr(self.mean_),
                                    d, ptr(self.patches_a_reduced_), stream_ptr(dev))
            for t in (A, self.components_, self.mean_, self.patches_a_reduced_):
                t.record_stream(a_side)
        elif proj == "exact":
            h.call("annf_project", ptr(A), ha, wa, c, p, ptr(self.components_), ptr(self.mean_), d, real_type,
                   ptr(self.patches_a_reduced_), st)
            h.call("annf_project", ptr(B), hb, wb, c, p, ptr(self.components_), ptr(self.mean_), d, real_type,
                   ptr(self.patches_b_reduced_), st)
        else:
            raise ValueError("projection must be 'exact' or 'fp16'")
        ev["t2"].record()

        # (4) k-d tree over B (annfmp/openmp/base.py:95-103)
        tree.fit(self.patches_b_reduced_)
        ev["t3"].record()

        if a_side is not None:
            torch.cuda.current_stream(dev).wait_stream(a_side)

        # (5) rows (annfmp/openmp/base.py:113-125)
        assert self.leaf_size > self.n_neighbors
        k = int(self.n_neighbors)
        nn = torch.empty(n_a, dtype=torch.int32, device=dev)
        self.nn_distances_ = torch.empty(n_a, dtype=torch.float32, device=dev)
        if self.form == "plain":
            self.knn_indices_ = torch.empty((n_a, k), dtype=torch.int32, device=dev)
            h.call("annf_process_rows_img", ptr(nn), ptr(A), ha, wa, ptr(B), hb, wb, c, p,
                   ptr(self.patches_a_reduced_), self._n_rows, self._n_cols, k, int(bool(self.propagate)),
                   int(bool(self.select_best_nn)), tree._final_max_leaves(), ptr(self.knn_indices_),
                   ptr(self.nn_distances_), st)
        else:
            if side is not None:
                torch.cuda.current_stream(dev).wait_stream(side)
                if prop is not None:
                    prop.record_stream(torch.cuda.current_stream(dev))
            lp = self.leaf_precision or "bf16"
            if lp not in ("bf16", "fp16", "fp8", "fp32"):
                raise ValueError("leaf_precision must be 'bf16', 'fp16', 'fp8' or 'fp32'")
            if lp != "fp32" and real != torch.float32:
                raise ValueError("tensor-core leaf distances need float_type='float'")
            lpc = {"bf16": _lib.ANNF_LEAF_BF16, "fp16": _lib.ANNF_LEAF_FP16, "fp8": _lib.ANNF_LEAF_FP8,
                   "fp32": _lib.ANNF_LEAF_EXACT}[lp]
            if seeded:  # the proposals' best match, found on the side stream
                h.call("annf_parallel_nnf_seeded", ptr(nn), ptr(A), ha, wa, ptr(B), hb, wb, c, p,
                       ptr(self.patches_a_reduced_), k, ptr(prop), int(self.iters), int(self.seed) & 0xFFFFFFFF, lpc,
                       int(self.search[0]), int(self.search[1]), ptr(self.nn_distances_), st)
            else:
                n_prop = 0 if prop is None else int(prop.shape[1])
                h.call("annf_parallel_nnf", ptr(nn), ptr(A), ha, wa, ptr(B), hb, wb, c, p,
                       ptr(self.patches_a_reduced_), k, ptr(prop), n_prop, int(self.iters),
                       int(self.seed) & 0xFFFFFFFF, lpc, int(self.search[0]), int(self.search[1]),
                       ptr(self.nn_distances_), st)
        ev["t4"].record()
        self.kdtree = tree
        self._A, self._B = A, B
        if not sync:
            return nn
        tree.check_device()  # synchronises and raises if a kernel's bounds check tripped
        self._timers = collections.OrderedDict()
        self._timers["pca_fit"] = ev["t0"].elapsed_time(ev["t1"]) / 1e3
        self._timers["extracting_patches"] = 0.0  # fused into pca_apply
        self._timers["pca_apply"] = ev["t1"].elapsed_time(ev["t2"]) / 1e3
        self._timers["kdtree_fit"] = ev["t2"].elapsed_time(ev["t3"]) / 1e3
        self._timers["remaining_rows"] = ev["t3"].elapsed_time(ev["t4"]) / 1e3
        self.kdtree = tree
        if self.verbose > 0:
            print("-----------------------------------------")
            print("--------------- RUNTIMES ----------------")
            print("-----------------------------------------")
            for name, key in (("Extraction of patches", "extracting_patches"), ("PCA fit", "pca_fit"),
                              ("PCA apply", "pca_apply"), ("K-D Tree (fitting)", "kdtree_fit"),
                              ("Remaining rows", "remaining_rows")):
                print("{}:\t{}".format(name, self._timers[key]))
            print("Total runtime:\t\t{}".format(sum(self._timers.values())))
            print("-----------------------------------------")
        self._A, self._B = A, B
        if numpy_io:
            return nn.cpu().numpy()
        return nn

    # patch arrays as the reference exposes them (annfmp/openmp/base.py:211-218), built on the host
    def _create_patches(self, img):
        img = img.cpu().numpy() if isinstance(img, torch.Tensor) else numpy.asarray(img)
        if img.ndim == 2:
            img = img[:, :, None]
        p = self.psize
        h, w, c = img.shape
        win = numpy.lib.stride_tricks.sliding_window_view(img, (p, p, c))[:, :, 0]
        return numpy.ascontiguousarray(win.reshape((h - p + 1) * (w - p + 1), p * p * c))

    @property
    def patches_a(self):
        return self._create_patches(self.image_a)

    @property
    def patches_b(self):
        return self._create_patches(self.image_b)
