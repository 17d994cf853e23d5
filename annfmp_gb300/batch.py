"""Many image pairs of uneven sizes per CUDA graph launch, with an autotuned leaf size.

The reference computes one pair per call (annfmp/openmp/base.py:55-150); batching is an addition.
``BatchNNF.prepare(pairs)`` takes device-resident uint8 pairs, picks each pair's leaf size and
propagation passes with ``Autotuner`` (per size class, cached), runs every pair once (that run
sizes all device buffers), then captures the parallel-form NNF of every pair, in order, into one
CUDA graph. ``run()`` replays the graph: one launch computes the whole batch. Inputs are read from
the same device tensors on every replay, so a stream of frames copies new images into them and
replays (``BatchNNF.inputs``).

The captured calls are free of host synchronisation and of device allocation (the library's
buffers are already large enough, torch's outputs come from the graph's private pool). A batch
runs the parallel form; a single pair's plain form replays as its own graph
(``ANNFieldPropKDTreeGB300``'s default ``graph="auto"``).
"""
from __future__ import annotations

import json
import os
import time

import numpy as np
import torch

from . import metrics
from ._torch import require_cuda
from .field import ANNFieldPropKDTreeGB300


def _size_class(h: int, w: int) -> int:
    """Pairs are tuned per power-of-two class of their pixel count (A's image)."""
    return int(np.ceil(np.log2(max(h * w, 1))))


class Autotuner:
    """Chooses (leaf_size, iters) for a size class: the fastest candidate whose mean distance-ratio
    error on a probe pair of the class stays within ``max_error`` (else the most accurate one).
    Results are kept per (class, psize, d, k, precision) and optionally in a JSON file."""

    LEAVES = (16, 32, 64)
    ITERS = (1, 2, 3)

    def __init__(self, max_error=0.01, path=None, samples=1024, reps=2):
        self.max_error = max_error
        self.path = path
        self.samples = samples
        self.reps = reps
        self.table = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.table = json.load(f)

    @staticmethod
    def pick(trials, max_error):
        """From (seconds, mean error, leaf, iters) trials: the fastest within ``max_error``, else
        the most accurate (ties broken by the tuple order)."""
        ok = [t for t in trials if t[1] <= max_error]
        return min(ok) if ok else min(trials, key=lambda t: (t[1], t[0], t[2], t[3]))

    def key(self, A, psize, d, k, leaf_precision):
        return f"{_size_class(A.shape[0], A.shape[1])}:{psize}:{d}:{k}:{leaf_precision}"

    def choose(self, A, B, base_kw, leaf_precision="bf16", proposal=None):
        key = self.key(A, base_kw["psize"], base_kw["dim_reduced"], base_kw["n_neighbors"], leaf_precision)
        if key in self.table:
            return tuple(self.table[key]["choice"])
        trials = []
        base_kw = {k: v for k, v in base_kw.items() if k != "leaf_size"}
        for leaf in self.LEAVES:
            if leaf <= base_kw["n_neighbors"]:
                continue
            for it in self.ITERS:
                m = ANNFieldPropKDTreeGB300(form="parallel", iters=it, leaf_size=leaf, proposal=proposal,
                                            leaf_precision=leaf_precision, verbose=0, graph=False, **base_kw)
                nn = m.fit(A, B)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(self.reps):
                    nn = m.fit(A, B)
                torch.cuda.synchronize()
                dt = (time.perf_counter() - t0) / self.reps
                err = metrics.distance_ratio_error(A, B, nn, base_kw["psize"], n_samples=self.samples, seed=17,
                                                   device=A.device)["mean"]
                trials.append((dt, err, leaf, it))
        best = self.pick(trials, self.max_error)
        self.table[key] = {"choice": [best[2], best[3]], "trials": [list(t) for t in trials]}
        if self.path:
            with open(self.path, "w") as f:
                json.dump(self.table, f, indent=1)
        return best[2], best[3]


class BatchNNF:
    """Parallel-form NNFs of a batch of pairs under one CUDA graph.

    Parameters as ``ANNFieldPropKDTreeGB300`` (n_neighbors, psize, dim_reduced, seed, proposal,
    leaf_precision); ``n_subset_frac``: the PCA subset per pair as a fraction of B's patches;
    ``leaf_size`` / ``iters``: fixed values, or "auto" to ask ``tuner``."""

    def __init__(self, n_neighbors=1, psize=7, dim_reduced=8, n_subset_frac=0.1, leaf_size="auto", iters="auto",
                 proposal=None, leaf_precision="bf16", seed=0, device=0, tuner=None):
        self.kw = dict(n_neighbors=n_neighbors, psize=psize, dim_reduced=dim_reduced, seed=seed, device=device)
        self.n_subset_frac = n_subset_frac
        self.leaf_size = leaf_size
        self.iters = iters
        self.proposal = proposal
        self.leaf_precision = leaf_precision
        self.dev = require_cuda(device)
        self.tuner = tuner or Autotuner()
        self.graph = None
        self.models = []
        self.outputs = []
        self.inputs = []

    def _params(self, A, B):
        p = self.kw["psize"]
        n_b = (B.shape[0] - p + 1) * (B.shape[1] - p + 1)
        kw = dict(self.kw, n_subset=int(round(self.n_subset_frac * n_b)))
        leaf, it = self.leaf_size, self.iters
        if leaf == "auto" or it == "auto":
            tl, ti = self.tuner.choose(A, B, kw, self.leaf_precision, self.proposal)
            leaf = tl if leaf == "auto" else leaf
            it = ti if it == "auto" else it
        return kw, int(leaf), int(it)

    def prepare(self, pairs):
        """pairs: [(A, B)] uint8 (h, w, 3) CUDA tensors, kept as the graph's inputs."""
        self.inputs = [(a.contiguous(), b.contiguous()) for a, b in pairs]
        self.models = []
        for A, B in self.inputs:
            kw, leaf, it = self._params(A, B)
            self.models.append(ANNFieldPropKDTreeGB300(form="parallel", iters=it, leaf_size=leaf,
                                                       proposal=self.proposal, leaf_precision=self.leaf_precision,
                                                       verbose=0, graph=False, **kw))
        # one plain run per pair: validates it and sizes every device buffer
        for m, (A, B) in zip(self.models, self.inputs):
            m.fit(A, B)
        torch.cuda.synchronize(self.dev)
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):  # warm the capture stream (torch's recommendation)
            for m, (A, B) in zip(self.models, self.inputs):
                m.fit(A, B, sync=False)
        torch.cuda.current_stream(self.dev).wait_stream(side)
        torch.cuda.synchronize(self.dev)
        self.graph = torch.cuda.CUDAGraph()
        from . import _lib
        before = _lib.launch_count()
        with torch.cuda.graph(self.graph, capture_error_mode="relaxed"):
            self.outputs = [m.fit(A, B, sync=False) for m, (A, B) in zip(self.models, self.inputs)]
        torch.cuda.synchronize(self.dev)
        self.kernels_per_launch = _lib.launch_count() - before  # this library's kernels in the graph
        return self

    def run(self):
        """One graph launch: the NNF of every pair (device int32 tensors, valid after the stream
        reaches them)."""
        if self.graph is None:
            raise RuntimeError("BatchNNF.run before prepare")
        self.graph.replay()
        return self.outputs

    def settings(self):
        return [(m.leaf_size, m.iters) for m in self.models]
