"""The CPU oracle pinned to the reference: golden fixtures (made by the unmodified reference, see
tests/golden/make_golden.py) and, where the reference tree is present, live comparisons."""
import os

import numpy as np
import pytest

from conftest import REF_ROOT


def _bits(a):
    return a.view(np.uint32) if a.dtype == np.float32 else a.view(np.uint64)


def test_trees_match_golden(oracle_mod, golden):
    O = oracle_mod
    z = golden("ref_trees.npz")
    for ci in range(int(z["n_cases"])):
        n, d, depth, split = z[f"c{ci}_meta"]
        X = z[f"c{ci}_X"]
        t = O.OracleTree(X, int(depth), int(split))
        assert np.array_equal(t.perm, z[f"c{ci}_perm"]), ci
        assert np.array_equal(_bits(t.pts), _bits(X[z[f"c{ci}_perm"]])), ci
        assert np.array_equal(t.node_axis, z[f"c{ci}_node_axis"]), ci
        assert np.array_equal(_bits(t.node_split), _bits(z[f"c{ci}_node_split"])), ci
        assert np.array_equal(t.leaf_bounds, z[f"c{ci}_leaf_bounds"]), ci
        assert np.array_equal(t.point_leaf, z[f"c{ci}_point_leaf"]), ci


def test_kneighbors_match_golden(oracle_mod, golden):
    O = oracle_mod
    z = golden("ref_trees.npz")
    for ci in range(int(z["n_cases"])):
        n, d, depth, split = z[f"c{ci}_meta"]
        t = O.OracleTree(z[f"c{ci}_X"], int(depth), int(split))
        dist, idx = t.kneighbors(z[f"c{ci}_Q"], int(z[f"c{ci}_K"]))
        assert np.array_equal(idx, z[f"c{ci}_knn_idx"]), ci
        assert np.array_equal(_bits(dist), _bits(z[f"c{ci}_knn_dist"])), ci


def test_process_rows_match_golden(oracle_mod, golden):
    O = oracle_mod
    z = golden("ref_rows.npz")
    for ci in range(int(z["n_cases"])):
        nr, nc, d, P, K, depth, prop, sel = (int(v) for v in z[f"r{ci}_meta"])
        t = O.OracleTree(z[f"r{ci}_X"], depth)
        final, _ = t.process_rows(z[f"r{ci}_A"], z[f"r{ci}_pa"], z[f"r{ci}_pb"], nr, nc, K, bool(prop), bool(sel))
        assert np.array_equal(final, z[f"r{ci}_final"]), ci


@pytest.mark.parametrize("name", ["ref_pipeline_affine128.npz", "ref_pipeline_flow160.npz",
                                  "ref_pipeline_k3_noprop.npz"])
def test_pipeline_matches_golden(oracle_mod, golden, name):
    O = oracle_mod
    z = golden(name)
    k, psize, d, n_subset, leaf, prop, sel, seed = (int(v) for v in z["params"])
    out = O.oracle_fit(z["a"], z["b"], n_neighbors=k, psize=psize, dim_reduced=d, n_subset=n_subset, leaf_size=leaf,
                       propagate=bool(prop), select_best_nn=bool(sel), seed=seed, return_all=True)
    # the numpy PCA restatement equals sklearn's to the last bits on the same LAPACK; allow eigh
    # differences between LAPACK builds (another CPU) at 1e-10
    assert np.allclose(out["comps"], z["components"], rtol=0, atol=1e-10)
    assert np.array_equal(out["mean"], z["mean"])
    agree = (out["nn"] == z["nn"]).mean()
    assert agree >= 0.999, agree


def test_oracle_depth_formula(oracle_mod):
    O = oracle_mod
    assert O.tree_depth(4161600, 64) == 15
    assert O.tree_depth(256036, 32) == 12
    assert O.tree_depth(2061616, 32) == 15
    assert O.tree_depth(100, 1000) == 0
    assert O.tree_depth(1000, 30, tree_depth_param=50) == 9
    with pytest.raises(ValueError):
        O.tree_depth(100, 1)


def test_sampling_matches_sklearn(oracle_mod):
    sk = pytest.importorskip("sklearn.feature_extraction.image")
    O = oracle_mod
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (40, 50, 3), dtype=np.uint8)
    ref = sk.extract_patches_2d(img, (5, 5), max_patches=37, random_state=4).reshape(37, -1)
    assert np.array_equal(O.subset_patches(img, 5, 37, 4), ref)
    full = sk.extract_patches_2d(img, (5, 5)).reshape(-1, 75)
    assert np.array_equal(O.subset_patches(img, 5, 0, 4), full)
    assert np.array_equal(O.subset_patches(img, 5, 10 ** 6, 4), full)


@pytest.mark.skipif(not os.path.isdir(REF_ROOT), reason="reference tree not present")
def test_live_fuzz_against_reference(oracle_mod):
    """Random trees, kNN and row propagation against the reference C core built from source."""
    O = oracle_mod
    if not O.reference_available():
        O.build_reference(REF_ROOT)
    rng = np.random.default_rng(2024)
    for trial in range(25):
        nr, nc = int(rng.integers(1, 25)), int(rng.integers(1, 25))
        d, P, K = int(rng.integers(1, 7)), int(rng.integers(1, 20)), int(rng.integers(1, 5))
        X = rng.standard_normal((nr * nc, d)).astype(np.float32)
        A = rng.standard_normal((nr * nc, d)).astype(np.float32)
        if trial % 2:
            X, A = np.round(X).astype(np.float32), np.round(A).astype(np.float32)
        pa = rng.integers(0, 256, (nr * nc, P), dtype=np.uint8)
        pb = rng.integers(0, 256, (nr * nc, P), dtype=np.uint8)
        depth = O.tree_depth(nr * nc, int(rng.integers(K + 1, K + 9)))
        prop, sel = bool(rng.integers(0, 2)), bool(rng.integers(0, 2))
        rt = O.reference_tree(X, depth)
        ot = O.OracleTree(X, depth)
        for key in ("perm", "node_axis", "leaf_bounds", "point_leaf"):
            assert np.array_equal(rt[key], getattr(ot, key)), (trial, key)
        fr = O.reference_process_rows(rt, A, pa, pb, nr, nc, K, prop, sel)
        fo, _ = ot.process_rows(A, pa, pb, nr, nc, K, prop, sel)
        assert np.array_equal(fr, fo), trial
    # double precision build
    X = rng.standard_normal((3000, 5))
    rt = O.reference_tree(X, O.tree_depth(3000, 8))
    ot = O.OracleTree(X, O.tree_depth(3000, 8))
    assert np.array_equal(rt["perm"], ot.perm) and np.array_equal(rt["node_split"], ot.node_split)


@pytest.mark.skipif(not os.path.isdir(REF_ROOT), reason="reference tree not present")
def test_live_reference_package_pipeline(oracle_mod):
    """The unmodified reference ANNField(algorithm='openmp') and the oracle pipeline agree exactly."""
    O = oracle_mod
    from annfmp_gb300 import gen
    ref = O.reference_annfmp(REF_ROOT)
    a, b = gen.pair_small(3, 80)
    m = ref.ANNField(n_neighbors=2, psize=5, dim_reduced=6, n_subset=1600, algorithm="openmp", leaf_size=8,
                     verbose=0, seed=2, n_jobs=2)
    nn_ref = m.fit(a, b)
    nn_ora = O.oracle_fit(a, b, n_neighbors=2, psize=5, dim_reduced=6, n_subset=1600, leaf_size=8, seed=2)
    assert np.array_equal(nn_ref, nn_ora)


def test_openclopt_oracle_first_row_is_exact(oracle_mod):
    """The openclopt restatement's traversal (kd-traverse.fut:27-116) finds the exact 8 nearest:
    the squared distances equal a brute force over every real point (pads excluded)."""
    O = oracle_mod
    rng = np.random.default_rng(4)
    X = (rng.standard_normal((6000, 8)) * 10).astype(np.float32)
    t = O.OclTree(X, 32)
    assert (t.h, t.q, t.ppl, t.mp) == O.ocl_shape(6000, 32)
    assert t.mp == (t.q + 1) * t.ppl and np.all(t.indir[t.indir >= 6000] >= 6000)
    Q = (rng.standard_normal((200, 8)) * 10).astype(np.float32)
    ki, kd, nat = t.natural(Q)
    t.exact(Q, nat, ki, kd)
    D = ((Q[:, None, :].astype(np.float64) - X[None].astype(np.float64)) ** 2).sum(-1)
    want = np.sort(D, axis=1)[:, :8]
    assert np.allclose(kd, want, rtol=2e-6)
    assert np.all(np.diff(kd, axis=1) >= 0)


def test_openclopt_tree_shape():
    """Leaf count: the power of two nearest m / leaf_size, ties down (buildKDtree.fut:4-24)."""
    from oracle import oracle as O
    O.build_oracle()
    assert O.ocl_shape(1000, 64) == (3, 15, 63, 1008)   # 16 leaves (15.6 -> 16)
    assert O.ocl_shape(100, 64) == (0, 1, 50, 100)      # 2 leaves
    assert O.ocl_shape(1536, 64) == (3, 15, 96, 1536)   # 24 leaves: 16 (tie goes down)
    assert O.ocl_shape(30, 64) == (-1, 0, 30, 30)       # one leaf, no internal node


def test_large_k_against_reference(oracle_mod):
    """The oracle's exact search and row propagation with k above 32 (the reference accepts up to
    1000, helper.c:32-35) against the reference C core built from source."""
    O = oracle_mod
    if not O.reference_available():
        if not os.path.isdir(REF_ROOT):
            pytest.skip("reference tree not present")
        O.build_reference(REF_ROOT)
    rng = np.random.default_rng(77)
    for trial, (nr, nc, d, K) in enumerate([(20, 24, 4, 40), (16, 30, 6, 100), (12, 13, 3, 33)]):
        X = rng.standard_normal((nr * nc, d)).astype(np.float32)
        A = rng.standard_normal((nr * nc, d)).astype(np.float32)
        if trial == 2:
            X, A = np.round(X).astype(np.float32), np.round(A).astype(np.float32)
        pa = rng.integers(0, 256, (nr * nc, 7), dtype=np.uint8)
        pb = rng.integers(0, 256, (nr * nc, 7), dtype=np.uint8)
        depth = O.tree_depth(nr * nc, K + 8)
        rt = O.reference_tree(X, depth)
        ot = O.OracleTree(X, depth)
        fr = O.reference_process_rows(rt, A, pa, pb, nr, nc, K, True, True)
        fo, _ = ot.process_rows(A, pa, pb, nr, nc, K, True, True)
        assert np.array_equal(fr, fo), trial


@pytest.mark.skipif(not os.path.isdir(REF_ROOT), reason="reference tree not present")
def test_kneighbors_tiny_trees_against_reference(oracle_mod):
    """Trees of one to a few leaves and k above the number of points, through the unmodified
    reference KDTree: the oracle fills short lists as the reference does (its initial maximum
    distance, tree position 0 mapped to that point's original index)."""
    O = oracle_mod
    O.reference_annfmp(REF_ROOT)  # the reference package, its C core behind ctypes
    from annfmp.openmp.kdtree.base import KDTree as RefKDTree
    for n in (1, 2, 3, 5, 9, 40):
        for K in (1, 4, 32, 40):
            for dt, ft in ((np.float32, "float"), (np.float64, "double")):
                rng = np.random.default_rng(100 * n + K)
                X = rng.standard_normal((n, 3)).astype(dt)
                Q = np.concatenate([rng.standard_normal((13, 3)).astype(dt), X[:2]])
                depth = O.tree_depth(n, 2)
                do, io = O.OracleTree(X, depth).kneighbors(Q, K)
                rk = RefKDTree(n_neighbors=K, tree_depth=depth, float_type=ft, splitting_type="longest").fit(X)
                dr, ir = rk.kneighbors(Q)
                assert np.array_equal(ir, io), (n, K, ft)
                assert np.array_equal(np.asarray(dr, dt).view(np.uint8), do.view(np.uint8)), (n, K, ft)
