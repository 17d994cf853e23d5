"""Components of the approximate NNF forms on the GPU: the subspace eigensolver."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PIPES = ["ref_pipeline_affine128.npz", "ref_pipeline_flow160.npz", "ref_pipeline_k3_noprop.npz"]


def _covariance(O, a, b, psize, n_subset, seed):
    m = int(n_subset / 2)
    X = np.concatenate([O.subset_patches(a, psize, m, seed), O.subset_patches(b, psize, m, seed + 1)]).astype(np.float64)
    mu = X.mean(axis=0)
    C = X.T @ X - len(X) * np.outer(mu, mu)
    return C / (len(X) - 1)


@pytest.mark.parametrize("name", PIPES)
def test_subspace_pca_captures_leading_variance(gpu_lib, oracle_mod, golden, name):
    """Subspace iteration + FP64 Rayleigh-Ritz: orthonormal components in decreasing Ritz value,
    capturing the top-d variance of the exact eigendecomposition to 1e-4, the leading component
    equal to the exact one (same sign convention), the mean exact."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    z = golden(name)
    k, psize, d, n_subset, leaf, prop, sel, seed = (int(v) for v in z["params"])
    m = ANNFieldPropKDTreeGB300(n_neighbors=k, psize=psize, dim_reduced=d, n_subset=n_subset, leaf_size=leaf,
                                seed=seed, verbose=0, form="parallel", pca_solver="subspace")
    m.fit(z["a"], z["b"])
    V = m.components_.cpu().numpy()
    assert np.array_equal(m.mean_.cpu().numpy(), z["mean"])
    assert np.abs(V @ V.T - np.eye(d)).max() < 1e-9
    C = _covariance(oracle_mod, z["a"], z["b"], psize, n_subset, seed)
    w = np.linalg.eigvalsh(C)[::-1]
    ritz = np.einsum("ij,jk,ik->i", V, C, V)
    assert np.all(np.diff(ritz) <= 1e-9 * ritz[0])
    assert ritz.sum() >= w[:d].sum() * (1 - 1e-4), (ritz.sum(), w[:d].sum())
    assert np.dot(V[0], z["components"][0]) > 1 - 1e-6
    j = np.argmax(np.abs(V), axis=1)
    assert np.all(V[np.arange(d), j] > 0)


@pytest.mark.parametrize("name", PIPES)
def test_exact_solver_matches_numpy_eigh(gpu_lib, oracle_mod, golden, name):
    """The drop-in PCA's FP64 subspace solver (annf_pca_components iters 0) and the library's full
    eigendecomposition (iters -1) give the same components as numpy's eigh of the same
    covariance, to 1e-10, with the same sign convention."""
    import torch
    from annfmp_gb300 import _lib
    from annfmp_gb300._torch import ptr, stream_ptr
    O = oracle_mod
    z = golden(name)
    k, psize, d, n_subset, leaf, prop, sel, seed = (int(v) for v in z["params"])
    a, b = z["a"], z["b"]
    C = _covariance(O, a, b, psize, n_subset, seed)
    w, V = np.linalg.eigh(C)
    V = V[:, ::-1][:, :d].T
    j = np.argmax(np.abs(V), axis=1)
    V = V * np.sign(V[np.arange(d), j])[:, None]
    dev = torch.device("cuda", 0)
    m = int(n_subset / 2)
    pa = O.sample_positions(a.shape[0] - psize + 1, a.shape[1] - psize + 1, m, seed)
    pb = O.sample_positions(b.shape[0] - psize + 1, b.shape[1] - psize + 1, m, seed + 1)
    pos_a = torch.from_numpy(np.stack(pa, 1).astype(np.int32)).to(dev)
    pos_b = torch.from_numpy(np.stack(pb, 1).astype(np.int32)).to(dev)
    A, B = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    P = psize * psize * a.shape[2]
    for iters in (0, -1):
        h = _lib.Handle(0)
        mean = torch.empty(P, dtype=torch.float64, device=dev)
        comps = torch.empty((d, P), dtype=torch.float64, device=dev)
        h.call("annf_pca_covariance", ptr(A), a.shape[0], a.shape[1], ptr(pos_a), m, ptr(B), b.shape[0], b.shape[1],
               ptr(pos_b), m, a.shape[2], psize, ptr(mean), stream_ptr(dev))
        h.call("annf_pca_components", P, d, iters, ptr(comps), stream_ptr(dev))
        got = comps.cpu().numpy()
        assert np.abs(got - V).max() < 1e-10, (iters, np.abs(got - V).max())
        assert np.allclose(got, z["components"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("psize,d", [(7, 8), (5, 12), (3, 8)])
def test_exact_solver_rank_deficient_covariance(gpu_lib, oracle_mod, psize, d):
    """The FP64 subspace solver on covariances of lower rank than its block (images u[x] + v[y]:
    2 psize - 1 directions): the dependent columns are dropped, and the leading components are
    orthonormal and capture the variance of numpy's eigh of the same covariance."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    O = oracle_mod
    rng = np.random.default_rng(psize * 10 + d)
    imgs = []
    for _ in range(2):
        u, v = rng.integers(0, 128, 96), rng.integers(0, 128, 96)
        imgs.append(np.repeat((v[:, None] + u[None, :]).astype(np.uint8)[:, :, None], 3, axis=2))
    a, b = imgs
    n_subset = 3000
    C = _covariance(O, a, b, psize, n_subset, 0)
    assert np.linalg.matrix_rank(C) < min(40, C.shape[0])
    m = ANNFieldPropKDTreeGB300(n_neighbors=1, psize=psize, dim_reduced=d, n_subset=n_subset, leaf_size=16, seed=0,
                                verbose=0, graph=False)
    m.fit(a, b)
    Vg = m.components_.cpu().numpy()
    assert np.all(np.isfinite(Vg))
    w = np.linalg.eigvalsh(C)[::-1]
    ritz = np.einsum("ij,jk,ik->i", Vg, C, Vg)
    r = min(d, int(np.linalg.matrix_rank(C)))
    assert np.abs(Vg[:r] @ Vg[:r].T - np.eye(r)).max() < 1e-9
    assert ritz[:r].sum() >= w[:r].sum() * (1 - 1e-10)


def test_subspace_pca_rank_deficient_covariance(gpu_lib, oracle_mod):
    """A covariance of lower rank than the iteration's block (B = d + max(8, d/2) = 16 vectors for
    d = 8): images whose pixels are u[x] + v[y] in all three channels give 7x7 patches spanning
    13 directions, so Cholesky-QR loses columns and Q^T Q is far from the identity. The FP64
    Rayleigh-Ritz step then takes its Cholesky path, dropping the dependent columns. The
    components must still be orthonormal, in decreasing Ritz value, and capture the top-d
    variance of numpy's eigh of the same covariance to the bound the other cases use."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    O = oracle_mod
    rng = np.random.default_rng(17)
    imgs = []
    for _ in range(2):
        u, v = rng.integers(0, 128, 96), rng.integers(0, 128, 96)
        imgs.append(np.repeat((v[:, None] + u[None, :]).astype(np.uint8)[:, :, None], 3, axis=2))
    a, b = imgs
    psize, d, n_subset, seed = 7, 8, 2000, 0
    C = _covariance(O, a, b, psize, n_subset, seed)
    assert np.linalg.matrix_rank(C) < d + max(8, d // 2)  # the block is rank-deficient
    m = ANNFieldPropKDTreeGB300(n_neighbors=1, psize=psize, dim_reduced=d, n_subset=n_subset, leaf_size=16,
                                seed=seed, verbose=0, form="parallel", pca_solver="subspace")
    nn = m.fit(a, b)
    assert nn.shape == (90 * 90,) and nn.min() >= 0 and nn.max() < 90 * 90
    V = m.components_.cpu().numpy()
    assert np.all(np.isfinite(V))
    Xs = np.concatenate([O.subset_patches(a, psize, n_subset // 2, seed),
                         O.subset_patches(b, psize, n_subset // 2, seed + 1)]).astype(np.float64)
    assert np.array_equal(m.mean_.cpu().numpy(), Xs.mean(axis=0))
    assert np.abs(V @ V.T - np.eye(d)).max() < 1e-9
    w = np.linalg.eigvalsh(C)[::-1]
    ritz = np.einsum("ij,jk,ik->i", V, C, V)
    assert np.all(np.diff(ritz) <= 1e-9 * ritz[0])
    assert ritz.sum() >= w[:d].sum() * (1 - 1e-4), (ritz.sum(), w[:d].sum())


# ---------------------------------------------------------------------------------------------
# tensor cores: one tcgen05 tile against a torch FP32 matmul of the same BF16 values
# ---------------------------------------------------------------------------------------------
def _tc_tile(h, A, B):
    import torch
    from annfmp_gb300._torch import ptr, stream_ptr
    dev = A.device
    D = torch.empty((128, B.shape[0]), dtype=torch.float32, device=dev)
    h.call("annf_tc_tile", ptr(A.view(torch.int16)), ptr(B.view(torch.int16)), B.shape[0], A.shape[1], ptr(D),
           stream_ptr(dev))
    return D


@pytest.mark.parametrize("n,kd", [(16, 16), (128, 16), (256, 32), (64, 64), (144, 48), (256, 256)])
def test_tc_tile_exact_on_small_integers(gpu_lib, n, kd):
    """Small integers are exact in BF16 and their dot products exact in FP32: bit-identical."""
    import torch
    from annfmp_gb300 import _lib
    g = torch.Generator().manual_seed(n * 1000 + kd)
    A = torch.randint(-8, 9, (128, kd), generator=g).to(torch.bfloat16).cuda()
    B = torch.randint(-8, 9, (n, kd), generator=g).to(torch.bfloat16).cuda()
    D = _tc_tile(_lib.Handle(0), A, B)
    want = A.float() @ B.float().T
    assert torch.equal(D, want), (D - want).abs().max()


def test_tc_tile_random_bf16(gpu_lib):
    """Random BF16 operands: FP32 accumulation, within 1e-5 of the row/column magnitude scale."""
    import torch
    from annfmp_gb300 import _lib
    g = torch.Generator().manual_seed(7)
    A = torch.randn((128, 32), generator=g).to(torch.bfloat16).cuda()
    B = torch.randn((96, 32), generator=g).to(torch.bfloat16).cuda()
    D = _tc_tile(_lib.Handle(0), A, B)
    want = A.double() @ B.double().T
    scale = A.double().abs() @ B.double().abs().T
    assert ((D.double() - want).abs() <= 1e-5 * scale + 1e-30).all()


# ---------------------------------------------------------------------------------------------
# natural-leaf kNN: BF16 tensor-core tiles + FP32 re-rank vs the exact FP32 leaf scan
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("n,d,leaf,k,quant", [(60000, 16, 64, 4, 0), (40000, 8, 32, 1, 0), (30000, 6, 8, 3, 0),
                                              (50000, 24, 64, 8, 0), (20000, 12, 32, 2, 0), (60000, 16, 64, 4, 8),
                                              (40000, 16, 64, 4, -1)])
def test_natural_knn_bf16_vs_fp32(gpu_lib, n, d, leaf, k, quant):
    """The BF16, FP16 and FP8 tiles only filter: every point within the tiles' proven error bound
    of the k-th best estimate is re-ranked exactly in FP32, so the k-lists equal the FP32 leaf
    scan's. quant > 0: a coarse grid (many exact ties); quant < 0: coordinates from 1e-3 to 1e4
    (FP8's subnormal range)."""
    import torch
    from annfmp_gb300 import KDTree
    rng = np.random.default_rng(n + d)
    # reduced-patch-like data: offset, anisotropic scales
    X = (rng.standard_normal((n, d)) * (300.0 / (1 + np.arange(d))) + 500.0).astype(np.float32)
    Qn = (X[rng.integers(0, n, 8000)] + rng.standard_normal((8000, d)).astype(np.float32) * 3).astype(np.float32)
    if quant > 0:  # coarse grid: many exactly tied distances
        X = (np.round(X / quant) * quant).astype(np.float32)
        Qn = (np.round(Qn / quant) * quant).astype(np.float32)
    elif quant < 0:  # per-dimension scales over seven decades
        sc = (10.0 ** np.linspace(-3, 4, d)).astype(np.float32)
        X = (X * sc / 300.0).astype(np.float32)
        Qn = (Qn * sc / 300.0).astype(np.float32)
    t = KDTree(n_neighbors=k, leaf_size=leaf, float_type="float", splitting_type="longest").fit(torch.from_numpy(X).cuda())
    Q = torch.from_numpy(Qn).cuda()
    i32 = t.natural_kneighbors(Q, k, "fp32").cpu().numpy()
    i16 = t.natural_kneighbors(Q, k, "bf16").cpu().numpy()
    same = (i32 == i16).all(axis=1)
    assert same.all(), (same.mean(), np.nonzero(~same)[0][:10])
    ih = t.natural_kneighbors(Q, k, "fp16").cpu().numpy()
    assert np.array_equal(ih, i32)
    i8 = t.natural_kneighbors(Q, k, "fp8").cpu().numpy()
    same8 = (i8 == i32).all(axis=1)
    assert same8.all(), (same8.mean(), np.nonzero(~same8)[0][:10])

    def d2(idx):
        diff = X[idx].astype(np.float64) - Qn[:, None, :].astype(np.float64)
        return (diff * diff).sum(-1)
    assert np.all(d2(i16)[:, -1] >= d2(i32)[:, -1] * (1 - 1e-6))


# ---------------------------------------------------------------------------------------------
# FP16 tensor-core projection vs the same arithmetic in float64
# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("name", PIPES)
def test_project_f16_matches_f16_components(gpu_lib, oracle_mod, golden, name):
    """out = patches . f16(components)^T - f16(components) . mean: pixel values and FP16
    products are exact, so only FP32 summation order separates the GPU from float64."""
    import torch
    from annfmp_gb300 import _lib
    from annfmp_gb300._torch import ptr, stream_ptr
    z = golden(name)
    psize = int(z["params"][1])
    comps, mean = np.ascontiguousarray(z["components"]), z["mean"]
    dev = torch.device("cuda", 0)
    for img in (z["a"], z["b"]):
        h, w, c = img.shape
        out = torch.empty(((h - psize + 1) * (w - psize + 1), comps.shape[0]), dtype=torch.float32, device=dev)
        # every argument tensor is held by a name until the call returns (a temporary's memory
        # could be handed to the next temporary by the caching allocator before the kernel runs)
        img_d, comps_d, mean_d = (torch.from_numpy(t).to(dev) for t in (img, comps, mean))
        _lib.Handle(0).call("annf_project_f16", ptr(img_d), h, w, c, psize, ptr(comps_d), ptr(mean_d),
                            comps.shape[0], ptr(out), stream_ptr(dev))
        torch.cuda.synchronize()
        cb = comps.astype(np.float32).astype(np.float16).astype(np.float64)
        X = oracle_mod.extract_patches(img, psize).astype(np.float64)
        want = X @ cb.T - cb @ mean
        scale = X @ np.abs(cb).T + np.abs(cb) @ np.abs(mean)
        got = out.cpu().numpy()
        assert np.all(np.abs(got - want) <= 2e-5 * scale + 1e-6), np.abs(got - want).max()


@pytest.mark.parametrize("h,w,psize", [(37, 53, 7), (41, 190, 9), (29, 133, 5)])
def test_project_f16_odd_pitch(gpu_lib, oracle_mod, h, w, psize):
    """Rows whose byte pitch is not a multiple of 4 (odd widths) and tiles narrower than 128."""
    import torch
    from annfmp_gb300 import _lib
    from annfmp_gb300._torch import ptr, stream_ptr
    rng = np.random.default_rng(h * w)
    img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    P = psize * psize * 3
    comps = np.linalg.qr(rng.standard_normal((P, 12)))[0].T.copy()
    mean = rng.random(P) * 255
    dev = torch.device("cuda", 0)
    img_d, comps_d, mean_d = (torch.from_numpy(t).to(dev) for t in (img, comps, mean))
    out = torch.empty(((h - psize + 1) * (w - psize + 1), 12), dtype=torch.float32, device=dev)
    _lib.Handle(0).call("annf_project_f16", ptr(img_d), h, w, 3, psize, ptr(comps_d), ptr(mean_d), 12, ptr(out),
                        stream_ptr(dev))
    torch.cuda.synchronize()
    cb = comps.astype(np.float32).astype(np.float16).astype(np.float64)
    X = oracle_mod.extract_patches(img, psize).astype(np.float64)
    want = X @ cb.T - cb @ mean
    scale = X @ np.abs(cb).T + np.abs(cb) @ np.abs(mean)
    assert np.all(np.abs(out.cpu().numpy() - want) <= 2e-5 * scale + 1e-5)
