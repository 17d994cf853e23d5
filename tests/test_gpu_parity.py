"""GPU parity: the CUDA kernels (through the C ABI) against the oracle and the reference's golden
outputs. Integer/index outputs must match bit for bit; the one floating-point tolerance (end to end,
where the GPU fits its own PCA) is stated where it is used."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a.view(np.uint64)


def gpu_tree(X, depth, splitting="longest", K=1):
    from annfmp_gb300 import KDTree
    ft = "float" if X.dtype == np.float32 else "double"
    kd = KDTree(n_neighbors=K, tree_depth=depth, float_type=ft, splitting_type=splitting)
    kd.fit(X)
    return kd


def assert_tree_equal(arrs, perm, node_axis, node_split, leaf_bounds, point_leaf, X, tag=""):
    assert np.array_equal(arrs["perm"], perm), tag
    assert np.array_equal(_bits(arrs["points"]), _bits(X[perm])), tag
    assert np.array_equal(arrs["node_axis"], node_axis), tag
    assert np.array_equal(_bits(arrs["node_split"]), _bits(node_split)), tag
    assert np.array_equal(arrs["leaves"], leaf_bounds), tag
    assert np.array_equal(arrs["point_leaf"], point_leaf), tag
    # per-leaf bounding boxes (the exact search's lower bounds): min / max of each coordinate
    pts = X[perm]
    big = np.finfo(X.dtype).max
    lb = np.asarray(leaf_bounds).reshape(-1, 2)
    box = arrs["leaf_box"]
    for leaf, (b0, b1) in enumerate(lb):
        if b1 > b0:
            want_lo, want_hi = pts[b0:b1].min(axis=0), pts[b0:b1].max(axis=0)
        else:
            want_lo, want_hi = np.full(X.shape[1], big, X.dtype), np.full(X.shape[1], -big, X.dtype)
        assert np.array_equal(box[leaf, 0], want_lo) and np.array_equal(box[leaf, 1], want_hi), (tag, leaf)


# ---------------------------------------------------------------------------------------------
# tree build
# ---------------------------------------------------------------------------------------------
def test_tree_golden(gpu_lib, golden):
    z = golden("ref_trees.npz")
    for ci in range(int(z["n_cases"])):
        n, d, depth, split = (int(v) for v in z[f"c{ci}_meta"])
        X = z[f"c{ci}_X"]
        kd = gpu_tree(X, depth, "longest" if split else "cyclic")
        assert_tree_equal(kd.tree_arrays(), z[f"c{ci}_perm"], z[f"c{ci}_node_axis"], z[f"c{ci}_node_split"],
                          z[f"c{ci}_leaf_bounds"], z[f"c{ci}_point_leaf"], X, f"golden case {ci}")


@pytest.mark.parametrize("n,d,leaf,kind,dtype", [
    (1, 3, 2, "normal", np.float32), (2, 1, 2, "normal", np.float32), (37, 5, 3, "normal", np.float32),
    (5000, 8, 32, "ties", np.float32), (70000, 16, 64, "normal", np.float32), (70000, 8, 16, "dups", np.float32),
    (300000, 16, 64, "normal", np.float32), (131072, 12, 32, "negzero", np.float32),
    (20000, 7, 8, "normal", np.float64), (90000, 16, 64, "ties", np.float64), (40000, 30, 16, "normal", np.float32),
    (10000, 4, 10, "constant", np.float32),
    # leaves too large for the shared-memory finisher: every level global, the points back to rows
    (6000, 16, 1500, "normal", np.float32), (3000, 64, 400, "ties", np.float64),
])
@pytest.mark.parametrize("splitting", ["longest", "cyclic"])
def test_tree_vs_oracle(gpu_lib, oracle_mod, n, d, leaf, kind, dtype, splitting):
    O = oracle_mod
    rng = np.random.default_rng(n * 31 + d)
    X = (rng.standard_normal((n, d)) * 10).astype(dtype)
    if kind == "ties":
        X = np.round(X / 3).astype(dtype)
    elif kind == "dups":
        X[::3] = X[0]
    elif kind == "negzero":
        X = np.round(X / 25).astype(dtype)
        X[::2] *= -1
    elif kind == "constant":
        X[:] = 1.5
    depth = O.tree_depth(n, leaf)
    ot = O.OracleTree(X, depth, 1 if splitting == "longest" else 0)
    kd = gpu_tree(X, depth, splitting)
    assert_tree_equal(kd.tree_arrays(), ot.perm, ot.node_axis, ot.node_split, ot.leaf_bounds, ot.point_leaf, X,
                      f"{n},{d},{kind},{splitting}")


# ---------------------------------------------------------------------------------------------
# exact kNN (reference neighbors_extern)
# ---------------------------------------------------------------------------------------------
def test_kneighbors_golden(gpu_lib, golden):
    z = golden("ref_trees.npz")
    for ci in range(int(z["n_cases"])):
        n, d, depth, split = (int(v) for v in z[f"c{ci}_meta"])
        K = int(z[f"c{ci}_K"])
        kd = gpu_tree(z[f"c{ci}_X"], depth, "longest" if split else "cyclic", K=K)
        dist, idx = kd.kneighbors(z[f"c{ci}_Q"])
        assert np.array_equal(idx, z[f"c{ci}_knn_idx"]), ci
        assert np.array_equal(_bits(dist), _bits(z[f"c{ci}_knn_dist"])), ci


@pytest.mark.parametrize("K", [1, 3, 4, 8, 17, 32])
@pytest.mark.parametrize("dtype,d", [(np.float32, 8), (np.float32, 16), (np.float32, 5), (np.float64, 6)])
def test_kneighbors_vs_oracle(gpu_lib, oracle_mod, K, dtype, d):
    O = oracle_mod
    rng = np.random.default_rng(K * 7 + d)
    n = 30000
    X = (rng.standard_normal((n, d)) * 5).astype(dtype)
    X[::7] = np.round(X[::7])
    Q = (rng.standard_normal((300, d)) * 5).astype(dtype)
    Q[::3] = X[rng.integers(0, n, 100)]  # exact hits -> zero distances and ties
    depth = O.tree_depth(n, 32)
    ot = O.OracleTree(X, depth)
    kd = gpu_tree(X, depth, K=K)
    dg, ig = kd.kneighbors(Q)
    do, io = ot.kneighbors(Q, K)
    assert np.array_equal(ig, io)
    assert np.array_equal(_bits(dg), _bits(do))


@pytest.mark.parametrize("max_leaves", [0, 1, 3, 17, 200])
@pytest.mark.parametrize("K", [1, 4])
def test_kneighbors_leaf_budget_vs_oracle(gpu_lib, oracle_mod, max_leaves, K):
    """A leaf budget cuts the search after the same leaves as the reference's traversal."""
    from annfmp_gb300 import KDTree
    O = oracle_mod
    rng = np.random.default_rng(max_leaves + 11 * K)
    X = (rng.standard_normal((20000, 8)) * 5).astype(np.float32)
    Q = (rng.standard_normal((257, 8)) * 5).astype(np.float32)
    depth = O.tree_depth(20000, 16)
    ot = O.OracleTree(X, depth)
    kd = KDTree(n_neighbors=K, tree_depth=depth, float_type="float", splitting_type="longest",
                max_leaves=max_leaves).fit(X)
    dg, ig = kd.kneighbors(Q)
    do, io = ot.kneighbors(Q, K, max_leaves=max_leaves)
    assert np.array_equal(ig, io)
    assert np.array_equal(_bits(dg), _bits(do))


@pytest.mark.parametrize("K,max_leaves", [(33, 2147483640), (100, 2147483640), (1000, 2147483640), (100, 1),
                                          (100, 7), (257, 0)])
@pytest.mark.parametrize("dtype,d", [(np.float32, 8), (np.float64, 5)])
def test_kneighbors_large_k_vs_oracle(gpu_lib, oracle_mod, K, max_leaves, dtype, d):
    """k above 32 (the reference accepts up to 1000, helper.c:32-35): the shared-memory K-list
    kernel gives the reference traversal's indices and distance bits, with and without a leaf
    budget, including lists longer than the leaves scanned (the (max real, 0) fill)."""
    from annfmp_gb300 import KDTree
    O = oracle_mod
    rng = np.random.default_rng(K + d + max_leaves % 97)
    n = 6000
    X = (rng.standard_normal((n, d)) * 5).astype(dtype)
    X[::5] = np.round(X[::5])
    Q = (rng.standard_normal((150, d)) * 5).astype(dtype)
    Q[::3] = X[rng.integers(0, n, 50)]  # exact hits -> zero distances and ties
    depth = O.tree_depth(n, 32)
    ot = O.OracleTree(X, depth)
    kd = KDTree(n_neighbors=K, tree_depth=depth, float_type="float" if dtype == np.float32 else "double",
                splitting_type="longest", max_leaves=max_leaves).fit(X)
    dg, ig = kd.kneighbors(Q)
    do, io = ot.kneighbors(Q, K, max_leaves=max_leaves)
    assert np.array_equal(ig, io)
    assert np.array_equal(_bits(dg), _bits(do))


# ---------------------------------------------------------------------------------------------
# row propagation (reference process_rows_extern)
# ---------------------------------------------------------------------------------------------
def test_process_rows_golden(gpu_lib, golden):
    z = golden("ref_rows.npz")
    for ci in range(int(z["n_cases"])):
        nr, nc, d, P, K, depth, prop, sel = (int(v) for v in z[f"r{ci}_meta"])
        kd = gpu_tree(z[f"r{ci}_X"], depth, K=K)
        out = np.zeros(nr * nc, np.int32)
        kd.process_rows(out, z[f"r{ci}_pa"], z[f"r{ci}_pb"], z[f"r{ci}_A"], nr, nc, K, bool(prop), bool(sel))
        assert np.array_equal(out, z[f"r{ci}_final"]), ci


@pytest.mark.parametrize("nr,nc,d,K,leaf,prop,sel,dtype", [
    (60, 70, 8, 1, 32, True, True, np.float32), (90, 64, 16, 4, 64, True, True, np.float32),
    (50, 80, 12, 8, 32, True, True, np.float32), (40, 33, 16, 4, 16, False, True, np.float32),
    (45, 51, 8, 2, 8, True, False, np.float32), (40, 40, 6, 3, 8, True, True, np.float64),
    (30, 90, 5, 16, 32, True, True, np.float32), (128, 128, 16, 4, 64, True, True, np.float32),
])
def test_process_rows_vs_oracle(gpu_lib, oracle_mod, nr, nc, d, K, leaf, prop, sel, dtype):
    O = oracle_mod
    rng = np.random.default_rng(nr * nc + K)
    nA = nr * nc
    X = (rng.standard_normal((nA, d)) * 10).astype(dtype)
    # A resembles B shifted by a few pixels, like an image pair, so that propagation matters
    A = np.roll(X.reshape(nr, nc, d), (2, 3), axis=(0, 1)).reshape(nA, d) + rng.standard_normal((nA, d)).astype(dtype)
    A = A.astype(dtype)
    if K == 2:
        X, A = np.round(X / 2).astype(dtype), np.round(A / 2).astype(dtype)
    P = 27
    pa = rng.integers(0, 256, (nA, P), dtype=np.uint8)
    pb = rng.integers(0, 256, (nA, P), dtype=np.uint8)
    depth = O.tree_depth(nA, leaf)
    ot = O.OracleTree(X, depth)
    fo, ko = ot.process_rows(A, pa, pb, nr, nc, K, prop, sel)
    kd = gpu_tree(X, depth, K=K)
    out = np.zeros(nA, np.int32)
    kd.process_rows(out, pa, pb, A, nr, nc, K, prop, sel)
    assert np.array_equal(kd.knn_indices_.cpu().numpy(), ko)
    assert np.array_equal(out, fo)


# ---------------------------------------------------------------------------------------------
# PCA + projection + end to end
# ---------------------------------------------------------------------------------------------
PIPES = ["ref_pipeline_affine128.npz", "ref_pipeline_flow160.npz", "ref_pipeline_k3_noprop.npz"]


def _fit_gpu(z):
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    k, psize, d, n_subset, leaf, prop, sel, seed = (int(v) for v in z["params"])
    m = ANNFieldPropKDTreeGB300(n_neighbors=k, psize=psize, dim_reduced=d, n_subset=n_subset, leaf_size=leaf,
                                propagate=bool(prop), select_best_nn=bool(sel), seed=seed, verbose=0)
    nn = m.fit(z["a"], z["b"])
    return m, nn


@pytest.mark.parametrize("name", PIPES)
def test_pca_fit_vs_reference(gpu_lib, golden, name):
    z = golden(name)
    m, _ = _fit_gpu(z)
    # mean is exact (integer sums, one division); components agree to FP64 eigen-solver accuracy
    assert np.array_equal(m.mean_.cpu().numpy(), z["mean"])
    comps = m.components_.cpu().numpy()
    assert np.allclose(comps, z["components"], rtol=0, atol=1e-9), np.abs(comps - z["components"]).max()


@pytest.mark.parametrize("name", PIPES)
def test_projection_rounds_like_fp64(gpu_lib, oracle_mod, golden, name):
    """GPU projection with the reference's own components vs the FP64 transform rounded to FP32:
    at most 1 ulp apart, and bit-identical on >= 99.99% of the coordinates."""
    O = oracle_mod
    z = golden(name)
    m, _ = _fit_gpu(z)
    from annfmp_gb300 import _lib
    from annfmp_gb300._torch import ptr, stream_ptr
    dev = torch.device("cuda", 0)
    comps = torch.from_numpy(np.ascontiguousarray(z["components"])).to(dev)
    mean = torch.from_numpy(z["mean"]).to(dev)
    psize = int(z["params"][1])
    img = torch.from_numpy(z["a"]).to(dev)
    h, w, c = z["a"].shape
    out = torch.empty(((h - psize + 1) * (w - psize + 1), comps.shape[0]), dtype=torch.float32, device=dev)
    m.kdtree.handle.call("annf_project", ptr(img), h, w, c, psize, ptr(comps), ptr(mean), comps.shape[0],
                         _lib.ANNF_REAL_F32, ptr(out), stream_ptr(dev))
    got = out.cpu().numpy()
    want = O.pca_transform(O.extract_patches(z["a"], psize), z["components"], z["mean"])
    ulps = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
    assert ulps.max() <= 1
    assert (ulps == 0).mean() >= 0.9999


@pytest.mark.parametrize("shape", [(160, 170, 3, 9, 16), (128, 140, 3, 7, 8), (96, 101, 3, 5, 12), (80, 90, 1, 12, 32),
                                   (70, 77, 4, 3, 5), (64, 66, 2, 6, 20)])
def test_exact_projection_tensor_cores_equal_dp4a(gpu_lib, shape):
    """annf_project on the tensor cores (digit-slice sums in FP32 TMEM) and with dp4a (the same
    sums in int32) give identical bits: every slice sum is an integer below 2^24."""
    from annfmp_gb300 import _lib
    from annfmp_gb300._torch import ptr, stream_ptr
    H, W, C, psize, d = shape
    rng = np.random.default_rng(H * W + d)
    dev = torch.device("cuda", 0)
    P = psize * psize * C
    comps = rng.standard_normal((d, P))
    comps /= np.linalg.norm(comps, axis=1, keepdims=True)
    comps[0, :] = np.abs(comps[0, :])  # a component whose digits are all of one sign
    img = torch.from_numpy(rng.integers(0, 256, (H, W, C), dtype=np.uint8)).to(dev)
    img[:8] = 255  # largest products
    C_ = torch.from_numpy(comps).to(dev)
    mean = torch.from_numpy(rng.uniform(0, 255, P)).to(dev)
    outs = []
    for opt in (0, 1):
        h = _lib.Handle(0)
        h.call("annf_set_option", _lib.ANNF_OPT_INT_PROJECTION, opt)
        out = torch.empty(((H - psize + 1) * (W - psize + 1), d), dtype=torch.float32, device=dev)
        h.call("annf_project", ptr(img), H, W, C, psize, ptr(C_), ptr(mean), d, _lib.ANNF_REAL_F32, ptr(out),
               stream_ptr(dev))
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy())
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))


@pytest.mark.parametrize("name", PIPES)
def test_rows_on_reference_reduced_arrays(gpu_lib, oracle_mod, golden, name):
    """Tree + rows on the reference's reduced patches (numpy FP64 transform of the reference's
    components): GPU == oracle bit for bit, and == the reference's NNF."""
    O = oracle_mod
    from annfmp_gb300 import KDTree
    z = golden(name)
    k, psize, d, n_subset, leaf, prop, sel, seed = (int(v) for v in z["params"])
    pa, pb = O.extract_patches(z["a"], psize), O.extract_patches(z["b"], psize)
    ared = O.pca_transform(pa, z["components"], z["mean"])
    bred = O.pca_transform(pb, z["components"], z["mean"])
    nr, nc = z["a"].shape[0] - psize + 1, z["a"].shape[1] - psize + 1
    ot = O.OracleTree(bred, O.tree_depth(len(bred), leaf))
    fo, _ = ot.process_rows(ared, pa, pb, nr, nc, k, bool(prop), bool(sel))
    kd = KDTree(n_neighbors=k, leaf_size=leaf, splitting_type="longest", float_type="float").fit(bred)
    out = np.zeros(nr * nc, np.int32)
    kd.process_rows(out, pa, pb, ared, nr, nc, k, bool(prop), bool(sel))
    assert np.array_equal(out, fo)
    assert (out == z["nn"]).mean() >= 0.999


def _relative_excess(a, b, psize, nn_x, nn_y):
    """raw-patch L2 of A's pixels under two NNFs (int64 exact)."""
    from oracle import oracle as O
    pa, pb = O.extract_patches(a, psize).astype(np.int64), O.extract_patches(b, psize).astype(np.int64)
    dx = np.sqrt(((pa - pb[nn_x]) ** 2).sum(1))
    dy = np.sqrt(((pa - pb[nn_y]) ** 2).sum(1))
    return dx, dy


REL_TOL = 1e-5  # a pixel whose NNF entry differs must match as well as the reference's entry, to 1e-5


def assert_differing_pixels_close(a, b, psize, nn_gpu, nn_ref, rel=REL_TOL):
    """Where the two NNFs differ, the raw-patch L2 of the GPU's match is within `rel` (relative)
    of the reference's: the difference is a tie or a rounding difference, not a worse match.
    Returns the number of differing pixels."""
    from annfmp_gb300.metrics import _patch_ssd
    nn_gpu, nn_ref = np.asarray(nn_gpu), np.asarray(nn_ref)
    diff = np.nonzero(nn_gpu != nn_ref)[0]
    if len(diff) == 0:
        return 0
    dg = np.sqrt(_patch_ssd(a, b, psize, diff, nn_gpu[diff]).astype(np.float64))
    dr = np.sqrt(_patch_ssd(a, b, psize, diff, nn_ref[diff]).astype(np.float64))
    bad = np.abs(dg - dr) > rel * np.maximum(dr, 1e-300)
    bad &= ~((dg == 0) & (dr == 0))
    assert not bad.any(), (f"{int(bad.sum())} of {len(diff)} differing pixels beyond {rel} relative distance",
                           diff[bad][:8], dg[bad][:8], dr[bad][:8])
    return len(diff)


@pytest.mark.parametrize("name", PIPES)
def test_pipeline_vs_reference(gpu_lib, golden, name):
    """End to end from the images (GPU PCA fit, projection, tree, rows, re-rank) vs the reference's
    NNF: identical on >= 99.9% of the pixels."""
    z = golden(name)
    m, nn = _fit_gpu(z)
    agree = (nn == z["nn"]).mean()
    assert agree >= 0.999, agree
    psize = int(z["params"][1])
    dg, dr = _relative_excess(z["a"], z["b"], psize, nn, z["nn"])
    # the per-pixel distance the GPU reports is the raw-patch L2 of its choice
    assert np.allclose(m.nn_distances_.cpu().numpy(), dg, rtol=1e-6)
    # every differing pixel: within 1e-5 relative raw-patch distance of the reference's match
    differ = nn != z["nn"]
    assert np.all(np.abs(dg[differ] - dr[differ]) <= REL_TOL * dr[differ]), np.nonzero(differ)[0][:8]


@pytest.mark.slow
def test_small_pair_workload_vs_oracle(gpu_lib, oracle_mod):
    """The 512x512 workload (psize 7, PCA 8, leaf 32, k 1, n_subset 10%) end to end vs the oracle
    pipeline on the same images: >= 99.9% identical."""
    O = oracle_mod
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen
    a, b = gen.pair_small(0, 512)
    nsub = int(round(0.1 * 506 * 506))
    m = ANNFieldPropKDTreeGB300(n_neighbors=1, psize=7, dim_reduced=8, n_subset=nsub, leaf_size=32, seed=0, verbose=0)
    nn = m.fit(a, b)
    nn_o = O.oracle_fit(a, b, n_neighbors=1, psize=7, dim_reduced=8, n_subset=nsub, leaf_size=32, seed=0)
    agree = (nn == nn_o).mean()
    assert agree >= 0.999, agree
    assert_differing_pixels_close(a, b, 7, nn, nn_o)


def _workload_pair(shape):
    """The image pairs and parameters of the 2048x2048 flow workload (patch 9, PCA 16, leaf 64,
    k 4) and of one 1920x1080 frame pair of the frame stream (patch 5, PCA 12, leaf 32, k 8);
    n_subset is 10% of B's patch count, as in the benchmark."""
    from annfmp_gb300 import gen
    if shape == "flow2048":
        a, b = gen.pair_flow(1, 2048)
        kw = dict(n_neighbors=4, psize=9, dim_reduced=16, leaf_size=64, seed=1)
    else:
        a, b = gen.frame_stream(3, 2, 1080, 1920)[:2]
        kw = dict(n_neighbors=8, psize=5, dim_reduced=12, leaf_size=32, seed=3)
    p = kw["psize"]
    kw["n_subset"] = int(round(0.1 * (b.shape[0] - p + 1) * (b.shape[1] - p + 1)))
    return a, b, kw


@pytest.mark.slow
@pytest.mark.parametrize("shape", ["flow2048", "frame1080"])
def test_plain_form_at_workload_shape_vs_oracle(gpu_lib, oracle_mod, shape):
    """The plain form at the benchmark's own shapes (4.16 M and 2.06 M patches, depth 15) against
    the oracle on the same images. End to end (the GPU fits its own PCA): >= 99.9% identical NNF
    and every differing pixel within 1e-5 relative raw-patch distance. On the oracle's own reduced
    arrays: the tree (permutation, split axes and value bits, leaf bounds, point leaves, leaf
    boxes), the k-lists and the NNF bit for bit."""
    O = oracle_mod
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, KDTree
    a, b, kw = _workload_pair(shape)
    p, k = kw["psize"], kw["n_neighbors"]
    r = O.oracle_fit(a, b, return_all=True, **kw)
    m = ANNFieldPropKDTreeGB300(verbose=0, **kw)
    nn = m.fit(a, b)
    agree = float((nn == r["nn"]).mean())
    assert agree >= 0.999, agree
    assert_differing_pixels_close(a, b, p, nn, r["nn"])
    del m
    ot = r["tree"]
    kd = KDTree(n_neighbors=k, leaf_size=kw["leaf_size"], splitting_type="longest", float_type="float").fit(r["bred"])
    assert kd.final_tree_depth_ == ot.depth
    assert_tree_equal(kd.tree_arrays(), ot.perm, ot.node_axis, ot.node_split, ot.leaf_bounds, ot.point_leaf,
                      r["bred"], shape)
    out = np.zeros(r["n_rows"] * r["n_cols"], np.int32)
    kd.process_rows(out, r["pa"], r["pb"], r["ared"], r["n_rows"], r["n_cols"], k, True, True)
    assert np.array_equal(kd.knn_indices_.cpu().numpy(), r["knn"])
    assert np.array_equal(out, r["nn"])


# ---------------------------------------------------------------------------------------------
# natural-leaf kNN (the reference's traversal with max_leaves=1) in every leaf precision
# ---------------------------------------------------------------------------------------------
def _reduced_pair(O, kind):
    """Reduced patches (oracle PCA and FP64 transform) of a flow pair at the 2048x2048 workload's
    patch settings (patch 9, PCA 16), of a frame pair at the frame stream's (patch 5, PCA 12), or
    the flow pair's coordinates on a coarse grid (many exactly tied distances)."""
    from annfmp_gb300 import gen
    if kind == "frames":
        a, b = gen.frame_stream(3, 2, 360, 640)[:2]
        p, d = 5, 12
    else:
        a, b = gen.pair_flow(1, 512)
        p, d = 9, 16
    nb = (b.shape[0] - p + 1) * (b.shape[1] - p + 1)
    comps, mean = O.pca_fit(a, b, p, d, int(round(0.1 * nb)), 0)
    ared = O.pca_transform(O.extract_patches(a, p), comps, mean)
    bred = O.pca_transform(O.extract_patches(b, p), comps, mean)
    if kind == "grid":
        ared = (np.round(ared / 16) * 16).astype(np.float32)
        bred = (np.round(bred / 16) * 16).astype(np.float32)
    return ared, bred


@pytest.mark.parametrize("kind,leaf,k", [("flow", 64, 4), ("frames", 32, 8), ("grid", 64, 4)])
def test_natural_knn_all_precisions_vs_oracle(gpu_lib, oracle_mod, kind, leaf, k):
    """The k-lists of the natural leaf (the reference's query with max_leaves=1, kdtree.c:179-183)
    from the FP32 leaf scan and from the BF16 / FP16 / FP8 tensor-core tiles with their exact FP32
    re-rank equal the oracle's, index for index (ties broken in the reference's leaf order)."""
    O = oracle_mod
    from annfmp_gb300 import KDTree
    ared, bred = _reduced_pair(O, kind)
    depth = O.tree_depth(len(bred), leaf)
    ot = O.OracleTree(bred, depth)
    _, want = ot.kneighbors(ared, k, max_leaves=1)
    kd = KDTree(n_neighbors=k, leaf_size=leaf, splitting_type="longest", float_type="float").fit(bred)
    for prec in ("fp32", "bf16", "fp16", "fp8"):
        got = kd.natural_kneighbors(ared, k, prec)
        same = (got == want).all(axis=1)
        assert same.all(), (kind, prec, float(same.mean()), np.nonzero(~same)[0][:8])


def test_process_rows_ragged_vs_oracle(gpu_lib, oracle_mod):
    """Ragged and degenerate grids (a single row, a single column, one patch), one- to six-dimensional
    points, patches of 1 to 19 bytes, leaves barely larger than k, every propagate / select_best
    combination: final indices and k-lists equal the oracle's, which the reference's own C core pins
    on the same kind of draws."""
    O = oracle_mod
    rng = np.random.default_rng(4048)
    shapes = [(1, 1), (1, 17), (23, 1), (2, 2)] + [(int(rng.integers(1, 25)), int(rng.integers(1, 25)))
                                                     for _ in range(20)]
    for trial, (nr, nc) in enumerate(shapes):
        d, P, K = int(rng.integers(1, 7)), int(rng.integers(1, 20)), int(rng.integers(1, 5))
        nA = nr * nc
        X = rng.standard_normal((nA, d)).astype(np.float32)
        A = rng.standard_normal((nA, d)).astype(np.float32)
        if trial % 2:
            X, A = np.round(X).astype(np.float32), np.round(A).astype(np.float32)
        pa = rng.integers(0, 256, (nA, P), dtype=np.uint8)
        pb = rng.integers(0, 256, (nA, P), dtype=np.uint8)
        depth = O.tree_depth(nA, int(rng.integers(K + 1, K + 9)))
        prop, sel = bool(rng.integers(0, 2)), bool(rng.integers(0, 2))
        ot = O.OracleTree(X, depth)
        fo, ko = ot.process_rows(A, pa, pb, nr, nc, K, prop, sel)
        kd = gpu_tree(X, depth, K=K)
        out = np.zeros(nA, np.int32)
        kd.process_rows(out, pa, pb, A, nr, nc, K, prop, sel)
        tag = (trial, nr, nc, d, P, K, depth, prop, sel)
        assert np.array_equal(kd.knn_indices_.cpu().numpy(), ko), tag
        assert np.array_equal(out, fo), tag


@pytest.mark.parametrize("n", [1, 2, 3, 5, 9, 40])
@pytest.mark.parametrize("K", [1, 4, 32, 40])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_kneighbors_tiny_trees_vs_oracle(gpu_lib, oracle_mod, n, K, dtype):
    """Trees of one to a few leaves, and k above the number of points: the lists are filled as the
    reference fills them (its initial maximum distance, position 0), indices and distance bits
    equal the oracle's."""
    O = oracle_mod
    rng = np.random.default_rng(100 * n + K)
    X = rng.standard_normal((n, 3)).astype(dtype)
    Q = np.concatenate([rng.standard_normal((13, 3)).astype(dtype), X[:2]])
    depth = O.tree_depth(n, 2)
    ot = O.OracleTree(X, depth)
    kd = gpu_tree(X, depth, K=K)
    dg, ig = kd.kneighbors(Q)
    do, io = ot.kneighbors(Q, K)
    assert np.array_equal(ig, io)
    assert np.array_equal(_bits(dg), _bits(do))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_dimension_limit_vs_oracle(gpu_lib, oracle_mod, dtype):
    """d = 128, the largest dimension the kernels take: tree, exact kNN (k 4 and 40) and row
    propagation equal the oracle's."""
    O = oracle_mod
    rng = np.random.default_rng(128)
    nr, nc, d = 24, 40, 128
    nA = nr * nc
    X = (rng.standard_normal((nA, d)) * 4).astype(dtype)
    X[::6] = np.round(X[::6])
    A = (np.roll(X.reshape(nr, nc, d), (1, 2), axis=(0, 1)).reshape(nA, d)
         + rng.standard_normal((nA, d))).astype(dtype)
    depth = O.tree_depth(nA, 16)
    ot = O.OracleTree(X, depth)
    for K in (4, 40):
        kd = gpu_tree(X, depth, K=K)
        arrs = kd.tree_arrays()
        assert np.array_equal(arrs["perm"], ot.perm) and np.array_equal(arrs["node_axis"], ot.node_axis)
        Q = np.concatenate([A[:200], X[:50]])
        dg, ig = kd.kneighbors(Q)
        do, io = ot.kneighbors(Q, K)
        assert np.array_equal(ig, io), K
        assert np.array_equal(_bits(dg), _bits(do)), K
    K, P = 3, 30
    pa = rng.integers(0, 256, (nA, P), dtype=np.uint8)
    pb = rng.integers(0, 256, (nA, P), dtype=np.uint8)
    fo, ko = ot.process_rows(A, pa, pb, nr, nc, K, True, True)
    kd = gpu_tree(X, depth, K=K)
    out = np.zeros(nA, np.int32)
    kd.process_rows(out, pa, pb, A, nr, nc, K, True, True)
    assert np.array_equal(kd.knn_indices_.cpu().numpy(), ko)
    assert np.array_equal(out, fo)


def test_image_and_array_paths_agree(gpu_lib, golden):
    """annf_process_rows_img (patches read from the images) == annf_process_rows (patch arrays)."""
    from oracle import oracle as O
    from annfmp_gb300 import KDTree
    z = golden("ref_pipeline_flow160.npz")
    m, nn = _fit_gpu(z)
    k, psize = int(z["params"][0]), int(z["params"][1])
    pa, pb = O.extract_patches(z["a"], psize), O.extract_patches(z["b"], psize)
    nr, nc = z["a"].shape[0] - psize + 1, z["a"].shape[1] - psize + 1
    kd = KDTree(n_neighbors=k, leaf_size=int(z["params"][4]), splitting_type="longest", float_type="float")
    kd.fit(m.patches_b_reduced_)
    out = np.zeros(nr * nc, np.int32)
    kd.process_rows(out, pa, pb, m.patches_a_reduced_, nr, nc, k, True, True)
    assert np.array_equal(out, nn)


# ---------------------------------------------------------------------------------------------
# errors are raised, not silently worked around
# ---------------------------------------------------------------------------------------------
def test_errors(gpu_lib):
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, KDTree, _lib
    X = np.random.default_rng(0).standard_normal((1000, 4)).astype(np.float32)
    kd = KDTree(n_neighbors=33, leaf_size=64, float_type="float").fit(X)
    dist, idx = kd.kneighbors(X[:5])  # k up to 1000, as the reference
    assert idx.shape == (5, 33) and dist.shape == (5, 33)
    with pytest.raises(NotImplementedError):  # the row propagation takes k <= 32
        kd.process_rows(np.zeros(4, np.int32), np.zeros((4, 3), np.uint8), np.zeros((1000, 3), np.uint8), X[:4], 2, 2)
    with pytest.raises(Exception, match="max_leaves"):
        KDTree(n_neighbors=2, leaf_size=8, float_type="float", max_leaves=-1).fit(X)
    with pytest.raises(ValueError):
        KDTree(n_neighbors=0).fit(X)
    a = np.zeros((40, 40, 3), np.uint8)
    with pytest.raises(AssertionError):  # annfmp/openmp/base.py:113
        ANNFieldPropKDTreeGB300(n_neighbors=8, leaf_size=8, psize=5, dim_reduced=4, n_subset=2000, verbose=0).fit(a, a)
    h = _lib.Handle(0)
    with pytest.raises(_lib.AnnfError):
        h.call("annf_kneighbors", None, 1, 1, 2147483640, None, None, None)  # no tree yet
