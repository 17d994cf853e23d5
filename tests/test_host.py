"""CPU-only checks of the host side: the C-ABI library builds and exports every declared symbol,
the Python mirror of the reference interface keeps its parameters, and the product fails loudly
without its CUDA library (no CPU fallback)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def _declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "annf_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(annf_[a-z0-9_]+)\s*\(", hdr)))


@pytest.fixture(scope="module")
def built_lib():
    from annfmp_gb300 import build as B
    try:
        B.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    return B.build()


def test_library_exports_every_declared_symbol(built_lib):
    syms = _declared_symbols()
    assert "annf_process_rows" in syms and "annf_build_tree" in syms
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (annf_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(built_lib)  # loads without a GPU
    for s in syms:
        assert hasattr(lib, s)


def test_binding_covers_header(built_lib):
    from annfmp_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == _declared_symbols()
    lib = _lib.load(built_lib)
    assert lib.annf_version() >= 10000


def test_no_cuda_device_is_an_error(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, KDTree
    with pytest.raises(RuntimeError):
        KDTree().fit(np.zeros((10, 2), np.float32))
    with pytest.raises(RuntimeError):
        ANNFieldPropKDTreeGB300(verbose=0).fit(np.zeros((20, 20, 3), np.uint8), np.zeros((20, 20, 3), np.uint8))
    from annfmp_gb300 import _lib
    h = ctypes.c_void_p()
    assert _lib.load().annf_create(ctypes.byref(h), 0) == _lib.ANNF_ERR_CUDA


def test_library_eigensolver_is_never_captured():
    """graph=True asks for a CUDA graph; the library eigensolver (pca_solver "full") sizes its
    workspace on the host and cannot be captured (the default FP64 solver can)."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    img = np.zeros((20, 20, 3), np.uint8)
    with pytest.raises(ValueError, match="full"):
        ANNFieldPropKDTreeGB300(verbose=0, graph=True, pca_solver="full").fit(img, img)
    assert ANNFieldPropKDTreeGB300(verbose=0)._graph_wanted()


def test_null_handle_is_rejected_by_every_entry_point(built_lib):
    """Every status-returning call that takes a handle answers a NULL handle with ANNF_ERR_INVALID
    and an error message, before any CUDA call (the reference prints and exits instead,
    helper.c:30-52); annf_destroy(NULL) is a no-op."""
    from annfmp_gb300 import _lib
    lib = _lib.load(built_lib)
    checked = 0
    for name, (res, args) in sorted(_lib.SIGNATURES.items()):
        if res is not _lib._i or not args or name == "annf_create":
            continue
        vals = [0.0 if a is ctypes.c_float else 0 if a in (_lib._i, _lib._u, _lib._ll, ctypes.c_longlong) else None
                for a in args]
        assert getattr(lib, name)(*vals) == _lib.ANNF_ERR_INVALID, name
        assert "NULL" in lib.annf_last_error().decode(), name
        checked += 1
    assert checked == len(_declared_symbols()) - 6  # all but version, last_error, create, destroy, two counters
    lib.annf_destroy(None)


def test_missing_library_fails_loudly(tmp_path):
    from annfmp_gb300 import _lib
    saved = _lib._lib
    try:
        _lib._lib = None
        with pytest.raises(ImportError):
            _lib.load(str(tmp_path / "nope.so"))
    finally:
        _lib._lib = saved


def test_facade_parameters_mirror_reference():
    from annfmp_gb300 import ANNField, ANNFieldPropKDTreeGB300, KDTree
    f = ANNField()
    assert f.get_params() == {"n_neighbors": 1, "psize": 8, "dim_reduced": 24, "n_subset": 1000,
                              "algorithm": "gb300", "leaf_size": 64, "n_jobs": -1, "propagate": True,
                              "select_best_nn": True, "verbose": 1, "seed": 0}
    f.set_params(algorithm="openmp")
    with pytest.raises(Exception, match="Unknown algorithm 'openmp'!"):
        f.fit(np.zeros((8, 8, 3), np.uint8), np.zeros((8, 8, 3), np.uint8))
    m = ANNFieldPropKDTreeGB300()
    assert (m.n_neighbors, m.psize, m.dim_reduced, m.n_subset, m.leaf_size, m.float_type) == (3, 8, 5, 1000, 64, "float")
    kd = KDTree()
    assert kd.get_params() == {"n_neighbors": 5, "leaf_size": 30, "max_leaves": None, "tree_depth": None,
                               "float_type": "double", "splitting_type": "cyclic", "n_jobs": 1, "verbose": 0}
    assert kd._compute_final_tree_depth(4161600, 64, None) == 15
    with pytest.warns(UserWarning):
        assert kd._compute_final_tree_depth(100, 30, 99) == 6


def test_patch_arrays_match_reference_layout(oracle_mod):
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    rng = np.random.default_rng(1)
    a = rng.integers(0, 256, (23, 31, 3), dtype=np.uint8)
    m = ANNFieldPropKDTreeGB300(psize=5)
    m.image_a = a
    assert np.array_equal(m.patches_a, oracle_mod.extract_patches(a, 5))


def test_subset_positions_match_sklearn_sampling():
    from annfmp_gb300.field import _SubsetCache
    sk = pytest.importorskip("sklearn.feature_extraction.image")
    import torch
    img = np.arange(30 * 40 * 3, dtype=np.int64).reshape(30, 40, 3) % 251
    img = img.astype(np.uint8)
    pos = _SubsetCache().get(26, 36, 50, 7, torch.device("cpu")).numpy()
    ref = sk.extract_patches_2d(img, (5, 5), max_patches=50, random_state=7)
    # sklearn's draws (rows, then columns) give its patches in its order ...
    rs = np.random.RandomState(7)
    i_s, j_s = rs.randint(26, size=50), rs.randint(36, size=50)
    assert np.array_equal(np.stack([img[y:y + 5, x:x + 5] for y, x in zip(i_s, j_s)]), ref)
    # ... and the cache holds the same positions in image order (the covariance is an exact sum)
    order = np.lexsort((j_s, i_s))
    assert np.array_equal(pos, np.stack([i_s[order], j_s[order]], axis=1))


def test_generators_are_seeded():
    from annfmp_gb300 import gen
    a1, b1 = gen.pair_small(0, 64)
    a2, b2 = gen.pair_small(0, 64)
    assert a1.dtype == np.uint8 and a1.shape == (64, 64, 3)
    assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
    a3, _ = gen.pair_small(1, 64)
    assert not np.array_equal(a1, a3)
    a, b = gen.pair_flow(1, 96, sigma=8.0)
    assert a.shape == b.shape == (96, 96, 3)
    assert a.min() == 0 and a.max() == 255


def test_mean_patch_l2_is_the_example_score():
    """metrics.mean_patch_l2 equals the reference example's overall L2 score
    (examples/simple.py:31-36: float32 patch differences, their L2 norms, the mean), restated
    here on the oracle's patch arrays; integer SSDs make ours exact, the example's float32
    norms agree to 1e-6."""
    from annfmp_gb300 import gen, metrics
    from oracle import oracle as O
    O.build_oracle()
    a, b = gen.pair_small(0, 96)
    psize = 5
    n = (96 - psize + 1) ** 2
    nnf = np.random.default_rng(3).integers(0, n, n).astype(np.int32)
    nnf[::4] = np.arange(n)[::4]
    pa, pb = O.extract_patches(a, psize), O.extract_patches(b, psize)
    diff = pa.astype(np.float32) - pb[nnf].astype(np.float32)
    score = np.mean(np.linalg.norm(diff, axis=1))
    assert np.isclose(metrics.mean_patch_l2(a, b, nnf, psize), float(score), rtol=1e-6, atol=0)


def test_parallel_restatement_hash_and_invariants():
    """oracle/parallel.py (the CPU restatement the parallel form's GPU search is checked against):
    its 32-bit hash gives the values of the kernels' C expression, the initial choice is the
    lexicographic minimum of (SSD, index) over the candidates, and passes never worsen a match."""
    import sys
    sys.path.insert(0, ROOT)
    from oracle import parallel as PR
    from oracle.oracle import extract_patches
    # values of the C expression (uint32 arithmetic) for these arguments
    assert list(PR.hash3(np.uint64(7919 * 3), np.arange(3, dtype=np.uint64), np.uint64(0))) == \
        [281888702, 4242423128, 3081578064]
    assert int(PR.hash3(np.uint64(0xFFFFFFFF), np.uint64(4000000000), np.uint64(5))) == 865287707
    rng = np.random.default_rng(5)
    a = rng.integers(0, 256, (20, 23, 3), dtype=np.uint8)
    b = rng.integers(0, 256, (21, 19, 3), dtype=np.uint8)
    ps = 4
    n_a = (20 - ps + 1) * (23 - ps + 1)
    n_b = (21 - ps + 1) * (19 - ps + 1)
    nat = rng.integers(0, n_b, (n_a, 3))
    idx0, ssd0 = PR.parallel_search(a, b, ps, nat, iters=0)
    pa = extract_patches(a, ps).astype(np.int64)
    pb = extract_patches(b, ps).astype(np.int64)
    s = ((pa[:, None, :] - pb[nat]) ** 2).sum(-1)
    best = np.lexsort((nat, s), axis=1)[:, 0]
    assert np.array_equal(idx0, nat[np.arange(n_a), best])
    assert np.array_equal(ssd0, s[np.arange(n_a), best])
    idx3, ssd3 = PR.parallel_search(a, b, ps, nat, iters=3, seed=9)
    assert np.all(ssd3 <= ssd0)
    assert np.array_equal(ssd3, ((pa - pb[idx3]) ** 2).sum(-1))


def test_autotuner_rule_and_cached_choices(tmp_path):
    """The batch autotuner's rule: the fastest (leaf, passes) trial within the error budget, else
    the most accurate; a size class already in its JSON table is answered from the table."""
    from annfmp_gb300.batch import Autotuner
    trials = [(3.0, 0.004, 16, 3), (1.0, 0.02, 16, 1), (2.0, 0.008, 32, 2), (2.5, 0.006, 64, 2)]
    assert Autotuner.pick(trials, 0.01) == (2.0, 0.008, 32, 2)
    assert Autotuner.pick(trials, 0.001) == (3.0, 0.004, 16, 3)
    assert Autotuner.pick(trials, 1.0) == (1.0, 0.02, 16, 1)
    A = np.zeros((300, 500, 3), np.uint8)
    tuner = Autotuner(path=str(tmp_path / "t.json"))
    kw = dict(psize=7, dim_reduced=8, n_neighbors=1)
    key = tuner.key(A, 7, 8, 1, "bf16")
    (tmp_path / "t.json").write_text('{"%s": {"choice": [32, 2], "trials": []}}' % key)
    assert Autotuner(path=str(tmp_path / "t.json")).choose(A, A, kw) == (32, 2)  # no GPU touched
    assert key.startswith("18:")  # 300 x 500 = 150000 pixels -> the 2^18 class
