"""ANNField facade (annfmp/base.py:13-142) with the GB300 backend as ``algorithm="gb300"``.

The reference selects its backend with a string in ``fit`` (annfmp/base.py:72-133); the GB300
backend is one more branch of that switch, with the same constructor parameters.
``algorithm="openclopt"`` runs the reference GPU backend's algorithm (annfmp/base.py:100-114) on
this library's kernels (``ANNFieldPropKDTreeOpenCLOPTGB300``).
"""
from __future__ import annotations

from .field import ANNFieldPropKDTreeGB300
from .openclopt import ANNFieldPropKDTreeOpenCLOPTGB300

ALGORITHMS = ["gb300", "openclopt"]


class ANNField:
    def __init__(self, n_neighbors=1, psize=8, dim_reduced=24, n_subset=1000, algorithm="gb300", leaf_size=64,
                 n_jobs=-1, propagate=True, select_best_nn=True, verbose=1, seed=0):
        self.n_neighbors = n_neighbors
        self.psize = psize
        self.dim_reduced = dim_reduced
        self.n_subset = n_subset
        self.algorithm = algorithm
        self.leaf_size = leaf_size
        self.n_jobs = n_jobs
        self.propagate = propagate
        self.select_best_nn = select_best_nn
        self.verbose = verbose
        self.seed = seed

    def get_params(self, deep=True):
        return {"n_neighbors": self.n_neighbors, "psize": self.psize, "dim_reduced": self.dim_reduced,
                "n_subset": self.n_subset, "algorithm": self.algorithm, "leaf_size": self.leaf_size,
                "n_jobs": self.n_jobs, "propagate": self.propagate, "select_best_nn": self.select_best_nn,
                "verbose": self.verbose, "seed": self.seed}

    def set_params(self, **parameters):
        for parameter, value in parameters.items():
            setattr(self, parameter, value)
        return self

    def fit(self, image_a, image_b):
        if self.algorithm not in ALGORITHMS:
            raise Exception("Unknown algorithm '{}'!".format(self.algorithm))
        if self.algorithm == "openclopt":
            self._model = ANNFieldPropKDTreeOpenCLOPTGB300(
                n_neighbors=self.n_neighbors, psize=self.psize, dim_reduced=self.dim_reduced,
                n_subset=self.n_subset, leaf_size=self.leaf_size, n_jobs=self.n_jobs,
                select_best_nn=self.select_best_nn, verbose=self.verbose, seed=self.seed)
            return self._model.fit(image_a, image_b)
        self._model = ANNFieldPropKDTreeGB300(
            n_neighbors=self.n_neighbors, psize=self.psize, dim_reduced=self.dim_reduced, n_subset=self.n_subset,
            leaf_size=self.leaf_size, n_jobs=self.n_jobs, propagate=self.propagate,
            select_best_nn=self.select_best_nn, verbose=self.verbose, seed=self.seed)
        return self._model.fit(image_a, image_b)

    @property
    def patches_a(self):
        return self._model.patches_a

    @property
    def patches_b(self):
        return self._model.patches_b
