"""Generate the golden fixtures in tests/golden/ from the UNMODIFIED reference.

Run in a checkout where the reference tree exists (default /root/reference):

    make -C oracle ref && python tests/golden/make_golden.py [/path/to/reference]

The reference's C core is compiled from its own sources into oracle/_ref (oracle/Makefile) and
its Python package is imported as is, with the SWIG modules replaced by ctypes stand-ins
(oracle/oracle.py: reference_annfmp / reference_tree / reference_process_rows). Every array in
the fixtures is an output of reference code on seeded inputs; inputs are stored beside them so
that no test needs the reference or the generators to reproduce them.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from annfmp_gb300 import gen  # noqa: E402


def ref_tree_cases():
    rng = np.random.default_rng(1234)
    cases = {}
    specs = [  # (n, d, leaf, kind, splitting)
        (1000, 4, 8, "normal", 1), (777, 8, 5, "ties", 1), (2048, 3, 16, "dups", 1), (3000, 16, 32, "normal", 1),
        (513, 5, 4, "negzero", 1), (1500, 6, 10, "normal", 0), (999, 2, 3, "ties", 0), (20000, 8, 32, "normal", 1),
        (4097, 12, 2, "dups", 1), (64, 4, 64, "normal", 1),
    ]
    for ci, (n, d, leaf, kind, split) in enumerate(specs):
        X = rng.standard_normal((n, d)).astype(np.float32) * 10
        if kind == "ties":
            X = np.round(X / 5).astype(np.float32)
        elif kind == "dups":
            X[::4] = X[1]
            X[:, 1] = 0.5
        elif kind == "negzero":
            X = np.round(X / 20).astype(np.float32)
            X[::2] *= -1
        depth = O.tree_depth(n, leaf)
        rt = reference_tree_split(X, depth, split)
        assert np.array_equal(rt["pts"].view(np.uint32), X[rt["perm"]].view(np.uint32))  # pts == X[perm]
        for k in ("perm", "node_axis", "node_split", "leaf_bounds", "point_leaf"):
            cases[f"c{ci}_{k}"] = rt[k]
        cases[f"c{ci}_X"] = X
        cases[f"c{ci}_meta"] = np.array([n, d, depth, split], np.int64)
        # exact kNN queries through neighbors_extern
        K = int(rng.integers(1, 6))
        Q = (rng.standard_normal((40, d)) * 10).astype(np.float32)
        if kind == "ties":
            Q = np.round(Q / 5).astype(np.float32)
        mod = O.make_wrapper_module(np.float32)
        params = O.KD_TREE_PARAMETERS()
        mod.init_extern(K, depth, 2147483640, 2, split, 0, params)
        rec = mod.KD_TREE_RECORD()
        Xc = X.copy()
        mod.fit_extern(Xc, rec, params)
        dist = np.zeros((40, K), np.float32)
        idx = np.zeros((40, K), np.int32)
        mod.neighbors_extern(Q, dist, idx, rec, params)
        cases[f"c{ci}_Q"] = Q
        cases[f"c{ci}_K"] = np.array(K)
        cases[f"c{ci}_knn_dist"] = dist
        cases[f"c{ci}_knn_idx"] = idx
    cases["n_cases"] = np.array(len(specs))
    return cases


def reference_tree_split(X, depth, splitting):
    """reference_tree with a chosen splitting type."""
    import ctypes
    lib = O._ref_lib(np.float32)
    params = O.KD_TREE_PARAMETERS()
    lib.init_extern(1, depth, 2147483640, 1, splitting, 0, ctypes.byref(params))
    rt = O.reference_tree(X, depth) if splitting == 1 else None
    if rt is not None:
        return rt
    # cyclic: rebuild through the wrapper module and read the record back
    Rec = O._record_type(np.float32)
    rec = Rec()
    Xc = np.ascontiguousarray(X)
    lib.fit_extern(Xc.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), X.shape[0], X.shape[1], ctypes.byref(rec),
                   ctypes.byref(params))
    n, d = X.shape
    L = 1 << depth
    esz = 4 * d + 4
    xi = np.ctypeslib.as_array(ctypes.cast(rec.XI, ctypes.POINTER(ctypes.c_uint8)), shape=(n * esz,)).copy().reshape(n, esz)
    raw = np.ctypeslib.as_array(ctypes.cast(rec.nodes, ctypes.POINTER(ctypes.c_int32)), shape=(2 * (L - 1),)).copy()
    return dict(pts=xi[:, :4 * d].copy().view(np.float32).reshape(n, d), perm=xi[:, 4 * d:].copy().view(np.int32).reshape(n),
                node_axis=raw[0::2].copy(), node_split=raw[1::2].copy().view(np.float32),
                leaf_bounds=np.ctypeslib.as_array(ctypes.cast(rec.leaves, ctypes.POINTER(ctypes.c_int)), shape=(2 * L,)).copy(),
                point_leaf=np.ctypeslib.as_array(ctypes.cast(rec.points_leaf_indices, ctypes.POINTER(ctypes.c_int)), shape=(n,)).copy())


def ref_rows_cases():
    rng = np.random.default_rng(99)
    cases = {}
    specs = [  # (n_rows, n_cols, d, P, K, leaf, propagate, select_best, kind)
        (20, 31, 4, 27, 1, 4, True, True, "normal"), (17, 23, 6, 48, 3, 8, True, True, "ties"),
        (40, 40, 8, 75, 4, 16, True, True, "normal"), (25, 19, 3, 12, 2, 5, False, True, "normal"),
        (30, 22, 5, 30, 2, 6, True, False, "ties"), (33, 35, 8, 27, 8, 16, True, True, "normal"),
        (12, 32, 16, 243, 4, 8, True, True, "dupb"),
    ]
    for ci, (nr, nc, d, P, K, leaf, prop, sel, kind) in enumerate(specs):
        nA = nr * nc
        X = (rng.standard_normal((nA, d)) * 10).astype(np.float32)
        Aq = (X + rng.standard_normal((nA, d)).astype(np.float32)).astype(np.float32)
        if kind == "ties":
            X = np.round(X / 4).astype(np.float32)
            Aq = np.round(Aq / 4).astype(np.float32)
        pa = rng.integers(0, 256, (nA, P), dtype=np.uint8)
        pb = rng.integers(0, 256, (nA, P), dtype=np.uint8)
        if kind == "dupb":
            pb[1::3] = pb[0]
        depth = O.tree_depth(nA, leaf)
        rt = O.reference_tree(X, depth)
        final = O.reference_process_rows(rt, Aq, pa, pb, nr, nc, K, prop, sel)
        cases.update({f"r{ci}_X": X, f"r{ci}_A": Aq, f"r{ci}_pa": pa, f"r{ci}_pb": pb, f"r{ci}_final": final,
                      f"r{ci}_meta": np.array([nr, nc, d, P, K, depth, int(prop), int(sel)], np.int64)})
    cases["n_cases"] = np.array(len(specs))
    return cases


def ref_pipeline_case(a, b, **kw):
    ref = O.reference_annfmp()
    m = ref.openmp.ANNFieldPropKDTreeOpenMP(verbose=0, **kw)
    nn = m.fit(a, b)
    pca = m._pca_model
    return dict(a=a, b=b, nn=nn.astype(np.int32), components=pca.components_, mean=pca.mean_,
                params=np.array([kw["n_neighbors"], kw["psize"], kw["dim_reduced"], kw["n_subset"], kw["leaf_size"],
                                 int(kw.get("propagate", True)), int(kw.get("select_best_nn", True)), kw["seed"]],
                                np.int64))


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    if not O.reference_available():
        O.build_reference(ref_root)
    O.reference_annfmp(ref_root)
    np.savez_compressed(os.path.join(HERE, "ref_trees.npz"), **ref_tree_cases())
    np.savez_compressed(os.path.join(HERE, "ref_rows.npz"), **ref_rows_cases())
    # small end-to-end pairs with the workload generators' statistics
    a, b = gen.pair_small(0, 128)
    nb = (128 - 7 + 1) ** 2
    np.savez_compressed(os.path.join(HERE, "ref_pipeline_affine128.npz"),
                        **ref_pipeline_case(a, b, n_neighbors=1, psize=7, dim_reduced=8, n_subset=4000,
                                            leaf_size=32, seed=0))
    a, b = gen.pair_flow(1, 160, magnitude=20.0, sigma=16.0)
    nb = (160 - 9 + 1) ** 2
    np.savez_compressed(os.path.join(HERE, "ref_pipeline_flow160.npz"),
                        **ref_pipeline_case(a, b, n_neighbors=4, psize=9, dim_reduced=16, n_subset=6000,
                                            leaf_size=64, seed=1))
    a, b = gen.pair_small(5, 96)
    np.savez_compressed(os.path.join(HERE, "ref_pipeline_k3_noprop.npz"),
                        **ref_pipeline_case(a, b, n_neighbors=3, psize=5, dim_reduced=6, n_subset=2000, leaf_size=8,
                                            seed=3, propagate=False))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
