"""The openclopt-semantics mode (annfmp's GPU backend's algorithm on this library's kernels)
against its CPU restatement (oracle/ocl_oracle.c; parity with the Futhark backend itself is
unpinned, it cannot run here). Tree arrays, lists and NNF must match bit for bit on the same
reduced patches; end to end (the GPU fits its own PCA) >= 99.9% identical."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _gpu_tree(X, leaf):
    from annfmp_gb300._torch import ptr, stream_ptr
    from annfmp_gb300.openclopt import ANNFieldPropKDTreeOpenCLOPTGB300
    dev = torch.device("cuda", 0)
    m = ANNFieldPropKDTreeOpenCLOPTGB300(verbose=0)
    h = m._get_handle(dev)
    Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(dev)
    h.call("annf_ocl_build_tree", ptr(Xd), X.shape[0], X.shape[1], leaf, stream_ptr(dev))
    torch.cuda.synchronize()
    return m, h, Xd


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("n,d,leaf,kind", [(5000, 8, 32, "normal"), (70000, 16, 64, "normal"), (20000, 12, 32, "ties"),
                                           (40000, 16, 64, "dups"), (30, 4, 64, "normal"), (9000, 5, 7, "negzero"),
                                           (33333, 3, 50, "normal")])
def test_ocl_tree_vs_oracle(gpu_lib, oracle_mod, n, d, leaf, kind):
    O = oracle_mod
    rng = np.random.default_rng(n + d)
    X = (rng.standard_normal((n, d)) * 10).astype(np.float32)
    if kind == "ties":
        X = np.round(X / 4).astype(np.float32)
    elif kind == "dups":
        X[::3] = X[0]
    elif kind == "negzero":
        X = np.round(X / 25).astype(np.float32)
        X[::2] *= -1
    ot = O.OclTree(X, leaf)
    m, h, _ = _gpu_tree(X, leaf)
    g = m.tree_arrays()
    assert (g["height"], g["n_nodes"], g["ppl"], g["m_padded"]) == (ot.h, ot.q, ot.ppl, ot.mp)
    assert np.array_equal(g["indir"], ot.indir)
    assert np.array_equal(g["dims"], ot.dims)
    assert np.array_equal(_bits(g["vals"]), _bits(ot.vals))
    assert np.array_equal(g["clanc"], ot.clanc)
    assert np.array_equal(g["orig2leaf"], ot.orig2leaf)
    assert np.array_equal(_bits(g["points"]), _bits(ot.pts))


def _reduced(O, a, b, psize, d, n_subset):
    comps, mean = O.pca_fit(a, b, psize, d, n_subset, 0)
    pa, pb = O.extract_patches(a, psize), O.extract_patches(b, psize)
    return O.pca_transform(pa, comps, mean), O.pca_transform(pb, comps, mean), pa, pb


@pytest.mark.parametrize("size,psize,d,leaf", [(160, 7, 8, 32), (200, 9, 16, 64), (128, 5, 12, 16)])
def test_ocl_rows_vs_oracle(gpu_lib, oracle_mod, size, psize, d, leaf):
    """Natural-leaf lists, exact first row, propagation and select best on the oracle's own
    reduced patches: lists (original indices and squared distances) and NNF bit for bit."""
    O = oracle_mod
    from annfmp_gb300 import gen
    from annfmp_gb300._torch import ptr, stream_ptr
    a, b = gen.pair_flow(size, size, magnitude=6.0, sigma=24.0)
    ared, bred, pa, pb = _reduced(O, a, b, psize, d, 4000)
    nr, nc = size - psize + 1, size - psize + 1
    ot = O.OclTree(bred, leaf)
    ki, kd, nat, bad = ot.rows(ared, nr, nc)
    assert not bad
    want_knn = np.where(ki >= 0, ot.indir[np.maximum(ki, 0)], -1)
    want_nn, want_sq = O.ocl_select(want_knn, pa, pb)
    m, h, _ = _gpu_tree(bred, leaf)
    dev = torch.device("cuda", 0)
    A, B = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    Ad = torch.from_numpy(ared).to(dev)
    n = nr * nc
    nn = torch.empty(n, dtype=torch.int32, device=dev)
    knn = torch.empty((n, 8), dtype=torch.int32, device=dev)
    ksq = torch.empty((n, 8), dtype=torch.float32, device=dev)
    dist = torch.empty(n, dtype=torch.float32, device=dev)
    h.call("annf_ocl_rows", ptr(nn), ptr(A), size, size, ptr(B), size, size, 3, psize, ptr(Ad), nr, nc, ptr(knn),
           ptr(ksq), ptr(dist), stream_ptr(dev))
    torch.cuda.synchronize()
    assert np.array_equal(knn.cpu().numpy(), want_knn)
    assert np.array_equal(_bits(ksq.cpu().numpy()), _bits(kd))
    assert np.array_equal(nn.cpu().numpy(), want_nn)
    assert np.allclose(dist.cpu().numpy() ** 2, want_sq, rtol=1e-6)


def test_ocl_pipeline_vs_oracle(gpu_lib, oracle_mod):
    """ANNField(algorithm="openclopt") end to end against the oracle's pipeline on the same
    images: the GPU fits its own PCA (FP64 components agreeing to ~1e-12), so >= 99.9% identical,
    and every differing pixel within 1e-5 relative raw-patch distance."""
    O = oracle_mod
    from annfmp_gb300 import ANNField, gen
    from test_gpu_parity import assert_differing_pixels_close
    a, b = gen.pair_flow(2, 256, magnitude=8.0, sigma=32.0)
    kw = dict(psize=7, dim_reduced=8, n_subset=6000, leaf_size=32, seed=0)
    want = O.oracle_fit_openclopt(a, b, **kw)
    model = ANNField(algorithm="openclopt", n_neighbors=3, verbose=0, **kw)
    got = model.fit(a, b)
    assert (got == want).mean() >= 0.999
    assert_differing_pixels_close(a, b, 7, got, want)
    assert model._model.knn_indices_.shape[1] == 8  # K is 8 whatever n_neighbors says
