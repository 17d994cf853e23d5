"""The offset-proposal network on the GPU: every kernel against the CPU oracle (oracle/cnn.py),
and what the trained network gains in the parallel NNF form."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net(seed=3):
    from annfmp_gb300.proposal import ProposalNet
    net = ProposalNet(None, device=0, seed=seed)
    # non-zero biases so that every ReLU sees both signs
    rng = np.random.default_rng(seed)
    for b in net.b:
        b.copy_(b.new_tensor(rng.standard_normal(b.numel()).astype(np.float32) * 0.05))
    net._dirty = True
    return net


def _bf16_np(t):
    import torch
    return t.float().cpu().numpy() if t.dtype == torch.bfloat16 else t.cpu().numpy()


def test_cnn_input_matches_oracle(gpu_lib):
    import torch
    from oracle import cnn as C
    rng = np.random.default_rng(0)
    a = rng.integers(0, 256, (37, 50, 3), dtype=np.uint8)
    b = rng.integers(0, 256, (37, 50, 3), dtype=np.uint8)
    net = _net()
    x = net.net_input(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    assert np.array_equal(_bf16_np(x), C.net_input(a, b))


@pytest.mark.parametrize("tensor_cores", [True, False])
def test_cnn_forward_backward_match_oracle(gpu_lib, tensor_cores):
    """Layer by layer, each GPU layer equals the oracle fed the GPU's own stored input (BF16
    outputs within 1 BF16 ulp); loss, output gradient and all weight/bias gradients match the
    oracle's within FP32 summation-order tolerance."""
    import torch
    from oracle import cnn as C
    rng = np.random.default_rng(1)
    N, h, w = 2, 19, 23
    x0 = C.bf16_round((rng.standard_normal((N, h, w, 8)) * 0.8).astype(np.float32))
    x0[..., 6:] = 0
    net = _net()
    net.tensor_cores = tensor_cores
    X = torch.from_numpy(x0).to(torch.bfloat16).cuda()
    out, acts = net.forward(X, keep=True)
    params = [(W.cpu().numpy(), b.cpu().numpy()) for W, b in zip(net.W, net.b)]
    acts_np = [_bf16_np(t) for t in acts]
    for li in range(len(params)):
        w_, b_ = params[li]
        y = C.conv3x3(acts_np[li], C.bf16_round(w_), b_)
        if li < len(params) - 1:
            want = C.bf16_round(np.maximum(y, 0).astype(np.float32))
            got = acts_np[li + 1]
            ulp = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64)) >> 16  # BF16 ulps
            assert ulp.max() <= 1 and (ulp == 0).mean() > 0.99, (li, ulp.max(), (ulp == 0).mean())
        else:
            got = out.cpu().numpy()
            assert np.allclose(got, y, rtol=1e-4, atol=1e-4 * np.abs(y).max())
    tgt = (rng.standard_normal((N, h, w, 16, 2)) * 6).astype(np.float32)
    valid = rng.random((N, h, w, 16)) > 0.1
    T = torch.from_numpy(tgt).cuda()
    V = torch.from_numpy(valid.astype(np.uint8)).cuda()
    loss, dout = net.loss(out, T, V)
    loss_o, dout_o = C.wta_loss(out.cpu().numpy(), tgt, valid)
    assert abs(float(loss.item()) - loss_o) <= 1e-5 * max(1.0, abs(loss_o))
    assert np.allclose(dout.cpu().numpy(), dout_o, rtol=1e-6, atol=1e-9)
    grads = net.backward(acts, dout)
    grads_o = C.backward(acts_np, dout.cpu().numpy().astype(np.float64), params)
    for li, ((dW, db), (dWo, dbo)) in enumerate(zip(grads, grads_o)):
        dW, db = dW.cpu().numpy(), db.cpu().numpy()
        sw = np.abs(dWo).max() + 1e-12
        sb = np.abs(dbo).max() + 1e-12
        assert np.abs(dW - dWo).max() <= 1e-4 * sw, (li, np.abs(dW - dWo).max(), sw)
        assert np.abs(db - dbo).max() <= 1e-4 * sb, (li, np.abs(db - dbo).max(), sb)


def test_adam_matches_reference_formula(gpu_lib):
    import torch
    from annfmp_gb300._torch import ptr, stream_ptr
    net = _net()
    rng = np.random.default_rng(5)
    p = rng.standard_normal(1000).astype(np.float32)
    g = rng.standard_normal(1000).astype(np.float32)
    m = rng.standard_normal(1000).astype(np.float32) * 0.1
    v = np.abs(rng.standard_normal(1000)).astype(np.float32) * 0.01
    P, G, M, V = (torch.from_numpy(t.copy()).cuda() for t in (p, g, m, v))
    net.h.call("annf_cnn_adam", ptr(P), ptr(G), ptr(M), ptr(V), 1000, 1e-3, 0.9, 0.999, 1e-8, 7,
               stream_ptr(P.device))
    p, g, m, v = (t.astype(np.float64) for t in (p, g, m, v))
    b1, b2 = float(np.float32(0.9)), float(np.float32(0.999))  # the kernel's FP32 constants
    m2 = b1 * m + float(np.float32(1) - np.float32(b1)) * g
    v2 = b2 * v + float(np.float32(1) - np.float32(b2)) * g * g
    p2 = p - 1e-3 * (m2 / (1 - 0.9 ** 7)) / (np.sqrt(v2 / (1 - 0.999 ** 7)) + 1e-8)
    assert np.allclose(P.cpu().numpy(), p2, rtol=1e-5, atol=1e-6)
    assert np.allclose(M.cpu().numpy(), m2, rtol=1e-5, atol=1e-7)
    assert np.allclose(V.cpu().numpy(), v2, rtol=1e-5, atol=1e-9)


def test_targets_and_proposals_match_oracle(gpu_lib):
    import torch
    from annfmp_gb300._torch import ptr, stream_ptr
    from oracle import cnn as C
    rng = np.random.default_rng(2)
    H, W, p = 45, 61, 7
    n_cols, n_rows = W - p + 1, H - p + 1
    nnf = rng.integers(0, n_rows * n_cols, n_rows * n_cols).astype(np.int32)
    net = _net()
    dev = torch.device("cuda", 0)
    T = torch.empty((H // 4, W // 4, 16, 2), dtype=torch.float32, device=dev)
    V = torch.empty((H // 4, W // 4, 16), dtype=torch.uint8, device=dev)
    nnf_d = torch.from_numpy(nnf).cuda()
    net.h.call("annf_cnn_targets", ptr(nnf_d), H, W, W, p, ptr(T), ptr(V), stream_ptr(dev))
    t_o, v_o = C.targets_from_nnf(nnf, H, W, H, W, p)
    assert np.array_equal(V.cpu().numpy().astype(bool), v_o)
    assert np.array_equal(T.cpu().numpy()[v_o], t_o[v_o])
    out = (rng.standard_normal((H // 4, W // 4, 8)) * 0.7).astype(np.float32)
    props = torch.empty((n_rows * n_cols, 4), dtype=torch.int32, device=dev)
    out_d = torch.from_numpy(out).cuda()
    net.h.call("annf_cnn_proposals", ptr(out_d), H // 4, W // 4, H, W, H, W, p, ptr(props), stream_ptr(dev))
    assert np.array_equal(props.cpu().numpy(), C.proposals(out, H, W, H, W, p))
    for per_pixel in (1, 2, 4):  # a subset of the block's hypotheses per pixel
        sub = torch.empty((n_rows * n_cols, per_pixel), dtype=torch.int32, device=dev)
        net.h.call("annf_cnn_proposals_per_pixel", ptr(out_d), H // 4, W // 4, H, W, H, W, p, per_pixel, ptr(sub),
                   stream_ptr(dev))
        assert np.array_equal(sub.cpu().numpy(), C.proposals(out, H, W, H, W, p, per_pixel))


def test_trained_proposals_gain(gpu_lib):
    """On a held-out flow pair, the same parallel form with the trained network's proposals lands
    closer to the exact nearest neighbour than without them, at one and at two propagation passes.
    The gain is modest: the plain method's matches, the network's targets, sit near the true
    displacement for only a minority of pixels on these images, so the four hypotheses can only
    cover part of them; the tree candidates remain, so proposals never make a pixel worse."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen, metrics
    from annfmp_gb300.proposal import DEFAULT_WEIGHTS, ProposalNet
    if not os.path.exists(DEFAULT_WEIGHTS):
        pytest.skip("no trained weights")
    a, b = gen.pair_flow(424242, 512)
    for per_pixel in (1, 4):  # one hypothesis per pixel (the default) and all four
        net = ProposalNet.pretrained(per_pixel=per_pixel)
        for iters in (1, 2):
            kw = dict(n_neighbors=4, psize=7, dim_reduced=8, n_subset=int(round(0.1 * 506 * 506)), leaf_size=32,
                      seed=0, verbose=0, form="parallel", iters=iters)
            nn0 = ANNFieldPropKDTreeGB300(**kw).fit(a, b)
            nn1 = ANNFieldPropKDTreeGB300(proposal=net, **kw).fit(a, b)
            e0 = metrics.distance_ratio_error(a, b, nn0, 7, n_samples=4096, seed=11)
            e1 = metrics.distance_ratio_error(a, b, nn1, 7, n_samples=4096, seed=11)
            assert e1["mean"] < e0["mean"], (per_pixel, iters, e1, e0)


class _ProposalsOnly:
    """A proposal source without a seed method: the NNF then takes the proposals themselves."""

    def __init__(self, net):
        self.net = net

    def propose(self, A, B, psize):
        return self.net.propose(A, B, psize)


def test_seeded_start_equals_proposals_in_init(gpu_lib):
    """The proposals' best match found beside the PCA fit (annf_seed_matches) and handed to the
    NNF (annf_parallel_nnf_seeded) gives the NNF of the proposals passed in (annf_parallel_nnf):
    the initial choice is the lexicographic minimum of (distance, index) over the same set."""
    import numpy as np
    import torch
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen
    from annfmp_gb300._torch import ptr, stream_ptr
    from annfmp_gb300.proposal import ProposalNet
    # untrained weights (proposals of any quality must give the same NNF), one and four per pixel
    for seed, size, per_pixel in ((5, 160, 1), (6, 203, 4)):
        net = ProposalNet(per_pixel=per_pixel)
        a, b = gen.pair_flow(seed, size, magnitude=6.0, sigma=24.0)
        kw = dict(n_neighbors=4, psize=7, dim_reduced=8, n_subset=3000, leaf_size=32, seed=0, verbose=0,
                  form="parallel", iters=2, graph=False)
        m1 = ANNFieldPropKDTreeGB300(proposal=net, **kw)
        nn1 = m1.fit(a, b)
        m2 = ANNFieldPropKDTreeGB300(proposal=_ProposalsOnly(net), **kw)
        nn2 = m2.fit(a, b)
        assert np.array_equal(nn1, nn2)
        assert torch.equal(m1.nn_distances_, m2.nn_distances_)
    # the seed itself: each pixel's best proposal by exact SSD (checked against the oracle's SSDs)
    from oracle import oracle as O
    A, B = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    props = net.propose(A, B, 7)
    seed = net.seed(A, B, 7, props).cpu().numpy()
    P = props.cpu().numpy().astype(np.int64)
    pa, pb = O.extract_patches(a, 7).astype(np.int64), O.extract_patches(b, 7).astype(np.int64)
    ssd = np.stack([((pa - pb[np.maximum(P[:, j], 0)]) ** 2).sum(axis=1) for j in range(P.shape[1])], axis=1)
    none = np.int64(1) << 40  # above any SSD
    ssd[P < 0] = none
    mins = ssd.min(axis=1)
    best = np.where(ssd == mins[:, None], P, np.iinfo(np.int64).max).min(axis=1)  # smaller index on ties
    assert np.array_equal(seed[0], np.where(mins == none, -1, best))
    assert np.array_equal(seed[1][seed[0] >= 0], mins[seed[0] >= 0])


def test_headline_form_within_one_percent(gpu_lib):
    """The headline form (tensor-core leaf tiles + learned proposals, 3 passes) on the 2048x2048
    flow pair (patch 9, PCA 16, leaf 64, k 4) stays within 1% mean distance-ratio error of the
    exact raw-patch nearest neighbour on 4096 sampled pixels."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen, metrics
    from annfmp_gb300.proposal import DEFAULT_WEIGHTS, ProposalNet
    if not os.path.exists(DEFAULT_WEIGHTS):
        pytest.skip("no trained weights")
    a, b = gen.pair_flow(1, 2048)
    n_b = (2048 - 8) ** 2
    m = ANNFieldPropKDTreeGB300(n_neighbors=4, psize=9, dim_reduced=16, n_subset=int(round(0.1 * n_b)),
                                leaf_size=64, seed=1, verbose=0, form="parallel", iters=3,
                                proposal=ProposalNet.pretrained())
    nn = m.fit(a, b)
    err = metrics.distance_ratio_error(a, b, nn, 9, n_samples=4096, seed=8)
    assert err["mean"] <= 0.01, err
