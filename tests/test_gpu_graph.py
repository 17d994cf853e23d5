"""Repeated fits of the parallel form replay one captured CUDA graph: same NNFs as eager fits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(n_neighbors=4, psize=7, dim_reduced=8, n_subset=6000, leaf_size=32, seed=0, verbose=0)


def _eager(a, b, proposal=None, **extra):
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    m = ANNFieldPropKDTreeGB300(form="parallel", iters=2, proposal=proposal, graph=False, **dict(KW, **extra))
    nn = m.fit(a, b)
    return nn, m.nn_distances_.clone()


@pytest.mark.parametrize("learned", [False, True])
def test_graph_replay_equals_eager(gpu_lib, learned):
    """Third and later fits replay the graph; new images of the same shape give the eager NNF."""
    import torch
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen
    from annfmp_gb300.proposal import ProposalNet
    net = ProposalNet.pretrained() if learned else None
    pairs = [gen.pair_flow(s, 160, magnitude=6.0, sigma=24.0) for s in (21, 22, 23)]
    # eager references first: the replays below must not meet a buffer growth of another handle
    refs = [_eager(a, b, net) for a, b in pairs]
    m = ANNFieldPropKDTreeGB300(form="parallel", iters=2, proposal=net, **KW)
    a, b = pairs[0]
    ref = refs[0][0]
    first = m.fit(a, b)
    assert m._graph is None  # first fit of the combination: eager
    second = m.fit(a, b)
    assert m._graph is not None and m._graph["kernels"] > 0
    graph = m._graph["graph"]
    assert np.array_equal(first, ref) and np.array_equal(second, ref)
    for (a2, b2), (ref2, dref2) in zip(pairs[1:], refs[1:]):
        got = m.fit(a2, b2)  # numpy in, numpy out
        assert m._graph["graph"] is graph  # replayed, not recaptured
        assert np.array_equal(got, ref2)
        assert torch.equal(m.nn_distances_, dref2)
    # device tensors in, device tensor out (a clone: the next replay does not overwrite it)
    A, B = (torch.from_numpy(x).cuda() for x in pairs[0])
    out = m.fit(A, B)
    assert isinstance(out, torch.Tensor) and out.is_cuda
    keep = out.clone()
    m.fit(*(torch.from_numpy(x).cuda() for x in pairs[1]))
    assert torch.equal(out, keep) and np.array_equal(out.cpu().numpy(), ref)


def test_graph_dropped_on_shape_change_and_buffer_growth(gpu_lib):
    import torch
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, _lib, gen
    m = ANNFieldPropKDTreeGB300(form="parallel", iters=2, **KW)
    a, b = gen.pair_flow(31, 128, magnitude=6.0, sigma=24.0)
    c, d = gen.pair_flow(32, 144, magnitude=6.0, sigma=24.0)
    m.fit(a, b)
    m.fit(a, b)
    g0 = m._graph["graph"]
    # another shape: eager (and the old graph is dropped), then captured on its second fit
    assert np.array_equal(m.fit(c, d), _eager(c, d)[0])
    assert m._graph is None
    m.fit(c, d)
    assert m._graph is not None and m._graph["graph"] is not g0
    g1 = m._graph["graph"]
    # a library buffer grows (a much larger query on the same tree): the graph is recaptured
    epoch = _lib.buffer_epoch()
    q = torch.randn(400000, 8, device="cuda")
    m.kdtree.natural_kneighbors(q, 4, "bf16")
    assert _lib.buffer_epoch() > epoch
    got = m.fit(c, d)
    assert m._graph is not None and m._graph["graph"] is not g1
    assert np.array_equal(got, _eager(c, d)[0])
    # a parameter change is a new combination
    m.iters = 1
    assert np.array_equal(m.fit(c, d), _eager_iters(c, d, 1))


def _eager_iters(a, b, iters):
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    return ANNFieldPropKDTreeGB300(form="parallel", iters=iters, graph=False, **KW).fit(a, b)


def test_plain_form_graph_replay_equals_eager(gpu_lib):
    """The plain form (the drop-in) is captured too: its FP64 eigensolver needs no host-side
    workspace query. Replays on new images give the eager NNF, bit for bit."""
    from annfmp_gb300 import ANNFieldPropKDTreeGB300, gen
    kw = dict(KW, n_subset=4000)
    pairs = [gen.pair_flow(s, 144, magnitude=6.0, sigma=24.0) for s in (41, 42, 43)]
    refs = [ANNFieldPropKDTreeGB300(graph=False, **kw).fit(a, b) for a, b in pairs]
    m = ANNFieldPropKDTreeGB300(**kw)  # form "plain", graph "auto"
    assert np.array_equal(m.fit(*pairs[0]), refs[0]) and m._graph is None
    assert np.array_equal(m.fit(*pairs[0]), refs[0]) and m._graph is not None
    graph = m._graph["graph"]
    for (a, b), ref in zip(pairs[1:], refs[1:]):
        assert np.array_equal(m.fit(a, b), ref)
        assert m._graph["graph"] is graph
