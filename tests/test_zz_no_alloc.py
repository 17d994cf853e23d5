"""annf_kneighbors_noalloc: exact kNN for callers that cannot allocate device memory at query time
(a serving process with its device memory reserved up front, or a host application that owns all
device memory through its own pool). It must return what annf_kneighbors returns, call after
call, although its scratch is one static device array shared by every call, and for float and
double trees alike up to its stated limit of n_queries * k = 262144 entries.

This file is collected last on purpose, so that a failure here stops a -x run only after every
other test has run. It also passes on its own in a fresh process."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _query(h, name, Q, k, max_leaves, dtype):
    from annfmp_gb300._torch import ptr, stream_ptr
    dev = Q.device
    dist = torch.empty((Q.shape[0], k), dtype=dtype, device=dev)
    idx = torch.empty((Q.shape[0], k), dtype=torch.int32, device=dev)
    h.call(name, ptr(Q), Q.shape[0], k, max_leaves, ptr(dist), ptr(idx), stream_ptr(dev))
    torch.cuda.synchronize(dev)
    return dist.cpu().numpy(), idx.cpu().numpy()


@pytest.mark.parametrize("dtype,d,k", [(torch.float32, 16, 4), (torch.float32, 8, 1), (torch.float64, 6, 3)])
def test_noalloc_matches_kneighbors_twice(gpu_lib, dtype, d, k):
    from annfmp_gb300 import KDTree, _lib
    rng = np.random.default_rng(d * 10 + k)
    X = (rng.standard_normal((60000, d)) * 5).astype(np.float32 if dtype == torch.float32 else np.float64)
    kd = KDTree(n_neighbors=k, leaf_size=32, splitting_type="longest",
                float_type="float" if dtype == torch.float32 else "double").fit(X)
    h = kd.handle
    dev = torch.device("cuda", 0)
    for trial in range(2):  # the second call sees the first call's leftovers in the shared scratch
        Q = torch.from_numpy((rng.standard_normal((3000, d)) * 5).astype(X.dtype)).to(dev)
        ref_d, ref_i = _query(h, "annf_kneighbors", Q, k, 2147483640, dtype)
        for budget in (2147483640, 7):
            want_d, want_i = (ref_d, ref_i) if budget > 1e6 else _query(h, "annf_kneighbors", Q, k, budget, dtype)
            got_d, got_i = _query(h, "annf_kneighbors_noalloc", Q, k, budget, dtype)
            # same kernels, same order of operations: identical bits (tolerance 0)
            assert np.array_equal(got_i, want_i), (trial, budget)
            assert np.array_equal(got_d, want_d), (trial, budget)


CAP = 262144  # n_queries * k entries the static scratch holds


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_noalloc_at_the_limit_twice(gpu_lib, dtype):
    """Exactly n_queries * k = 262144 entries (65536 queries, k 4): the double seeds are 16 bytes
    each, so this fills the whole key region; results equal annf_kneighbors bit for bit."""
    from annfmp_gb300 import KDTree
    npdt = np.float32 if dtype == torch.float32 else np.float64
    rng = np.random.default_rng(5 if dtype == torch.float32 else 6)
    d, k = 6, 4
    X = (rng.standard_normal((40000, d)) * 5).astype(npdt)
    kd = KDTree(n_neighbors=k, leaf_size=32, splitting_type="longest",
                float_type="float" if dtype == torch.float32 else "double").fit(X)
    dev = torch.device("cuda", 0)
    for trial in range(2):
        Qn = (rng.standard_normal((CAP // k, d)) * 5).astype(npdt)
        Qn[::5] = X[rng.integers(0, len(X), len(Qn[::5]))]  # exact hits: zero distances and ties
        Q = torch.from_numpy(Qn).to(dev)
        want_d, want_i = _query(kd.handle, "annf_kneighbors", Q, k, 2147483640, dtype)
        got_d, got_i = _query(kd.handle, "annf_kneighbors_noalloc", Q, k, 2147483640, dtype)
        assert np.array_equal(got_i, want_i), trial
        assert np.array_equal(got_d, want_d), trial


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_noalloc_rejects_oversized_requests(gpu_lib, dtype):
    from annfmp_gb300 import KDTree, _lib
    npdt = np.float32 if dtype == torch.float32 else np.float64
    X = np.random.default_rng(1).standard_normal((5000, 8)).astype(npdt)
    kd = KDTree(n_neighbors=8, leaf_size=32, splitting_type="longest",
                float_type="float" if dtype == torch.float32 else "double").fit(X)
    Q = torch.zeros((CAP // 8 + 1, 8), dtype=dtype, device="cuda")  # one query past the limit
    with pytest.raises(_lib.AnnfInvalid, match="scratch"):
        _query(kd.handle, "annf_kneighbors_noalloc", Q, 8, 2147483640, dtype)
