"""The parallel form and the distance-error reference on the GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_raw_nn_matches_oracle(gpu_lib, oracle_mod):
    """Exact raw-patch nearest neighbour: GPU integer brute force == CPU int64 brute force."""
    O = oracle_mod
    from annfmp_gb300 import gen, metrics
    for psize, size in ((7, 72), (9, 64), (5, 80)):
        a, b = gen.pair_small(psize, size)
        pa, pb = O.extract_patches(a, psize), O.extract_patches(b, psize)
        q = np.arange(0, len(pa), 37, dtype=np.int32)
        d2, bi = O.exact_raw_nn(pa, q, pb)
        ssd, idx = metrics.exact_nn(a, b, psize, q)
        assert np.array_equal(ssd, d2.astype(np.int64))
        assert np.array_equal(idx, bi.astype(np.int64))  # smallest index on ties, as the oracle


def test_parallel_form_quality(gpu_lib):
    """The parallel form returns real patch distances and, on a smooth warp, lands within a few
    percent of the exact nearest neighbour (and never below it)."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen, metrics
    a, b = gen.pair_flow(11, 192, magnitude=6.0, sigma=24.0)
    kw = dict(n_neighbors=4, psize=7, dim_reduced=8, n_subset=6000, leaf_size=32, seed=0, verbose=0)
    par = ANNFieldPropKDTreeGB300(form="parallel", iters=6, **kw)
    nn_p = par.fit(a, b)
    # the reported distances are the exact raw-patch L2 of the returned indices
    d = np.sqrt(metrics._patch_ssd(a, b, 7, np.arange(len(nn_p)), nn_p).astype(np.float64))
    assert np.allclose(par.nn_distances_.cpu().numpy(), d, rtol=1e-6)
    err_p = metrics.distance_ratio_error(a, b, nn_p, 7, n_samples=2048, seed=3)
    nn_0 = ANNFieldPropKDTreeGB300(**kw).fit(a, b)
    err_0 = metrics.distance_ratio_error(a, b, nn_0, 7, n_samples=2048, seed=3)
    assert err_p["mean"] <= err_0["mean"] + 1e-9, (err_p, err_0)
    assert err_p["mean"] < 0.05, err_p


@pytest.mark.parametrize("leaf_precision", ["fp8", "fp16"])
def test_parallel_form_other_leaf_precisions(gpu_lib, leaf_precision):
    """The natural-leaf k-lists do not depend on the tile precision (exact FP32 re-rank behind each
    tile's proven bound), so the whole NNF equals the BF16 one."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen
    a, b = gen.pair_flow(12, 176, magnitude=6.0, sigma=24.0)
    kw = dict(n_neighbors=4, psize=7, dim_reduced=8, n_subset=6000, leaf_size=32, seed=0, verbose=0,
              form="parallel", iters=2, graph=False)
    ref = ANNFieldPropKDTreeGB300(leaf_precision="bf16", **kw).fit(a, b)
    got = ANNFieldPropKDTreeGB300(leaf_precision=leaf_precision, **kw).fit(a, b)
    assert np.array_equal(ref, got)


class _RandomProposals:
    """Fixed random B indices as offset proposals (some -1 = none), passed in as candidates."""

    def __init__(self, n_prop, rng_seed):
        self.n_prop, self.rng_seed = n_prop, rng_seed
        self.last = None

    def propose(self, A, B, psize):
        import torch
        n_a = (A.shape[0] - psize + 1) * (A.shape[1] - psize + 1)
        n_b = (B.shape[0] - psize + 1) * (B.shape[1] - psize + 1)
        rng = np.random.default_rng(self.rng_seed)
        p = rng.integers(-1, n_b, (n_a, self.n_prop)).astype(np.int32)
        self.last = p
        return torch.from_numpy(p).to(A.device)


@pytest.mark.parametrize("psize,ha,wa,hb,wb,iters,n_prop", [
    (9, 160, 160, 160, 160, 3, 0),    # the headline patch (specialised 9x27-byte kernels)
    (7, 150, 170, 161, 143, 4, 2),    # uneven sizes, proposals in the initial choice
    (6, 120, 128, 128, 120, 3, 1),    # a patch without a specialised kernel (generic kernels)
])
def test_parallel_search_matches_restatement(gpu_lib, psize, ha, wa, hb, wb, iters, n_prop):
    """The parallel form's NNF and distances equal the CPU restatement of its search
    (oracle/parallel.py) started from the same natural-leaf neighbours: the initial choice and
    every propagation / random-search pass, index for index. Candidates the GPU does not load
    (repeats, neighbours unchanged since the previous pass) cannot change this result."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen
    from oracle import parallel as PR
    rng = np.random.default_rng(psize)
    a = gen.spectral_noise(ha, wa, rng)
    b = gen.flow_warp(gen.spectral_noise(max(ha, hb), max(wa, wb), np.random.default_rng(psize))[:hb, :wb],
                      4.0, 16.0, 4.0, rng)
    prop = _RandomProposals(n_prop, 5) if n_prop else None
    k = 4
    m = ANNFieldPropKDTreeGB300(n_neighbors=k, psize=psize, dim_reduced=8, n_subset=4000, leaf_size=32, seed=3,
                                verbose=0, form="parallel", iters=iters, graph=False, proposal=prop)
    nn = m.fit(a, b)
    nat = m.kdtree.natural_kneighbors(m.patches_a_reduced_, k, "bf16").cpu().numpy()
    want, ssd = PR.parallel_search(a, b, psize, nat, proposals=prop.last if prop else None, iters=iters,
                                   seed=3, nrand=m.search[0], radius0=m.search[1])
    assert np.array_equal(nn, want), float((nn == want).mean())
    got_d = m.nn_distances_.cpu().numpy()
    assert np.array_equal(got_d, np.sqrt(ssd.astype(np.float32)))
