"""annf_kneighbors_noalloc: exact kNN for callers that cannot allocate device memory at query time
(for example work captured into a CUDA graph, where cudaMalloc is not allowed, or a serving
process with memory reserved up front). It must return what annf_kneighbors returns, call after
call, although its scratch is one static device array shared by every call.

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


def test_noalloc_rejects_oversized_requests(gpu_lib):
    from annfmp_gb300 import KDTree, _lib
    X = np.random.default_rng(1).standard_normal((5000, 8)).astype(np.float32)
    kd = KDTree(n_neighbors=8, leaf_size=32, splitting_type="longest", float_type="float").fit(X)
    Q = torch.zeros((40000, 8), dtype=torch.float32, device="cuda")  # 40000 * 8 > 262144 entries
    with pytest.raises(_lib.AnnfInvalid, match="scratch"):
        _query(kd.handle, "annf_kneighbors_noalloc", Q, 8, 2147483640, torch.float32)
