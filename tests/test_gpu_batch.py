"""Batched uneven pairs under one CUDA graph, and the autotuner."""
import pytest

pytestmark = pytest.mark.gpu


def _pairs(count, seed=2, lo=96, hi=200):
    import torch
    from annfmp_gb300 import gen
    return [(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
            for a, b in gen.pairs_uneven(seed=seed, count=count, lo=lo, hi=hi)]


def test_batch_graph_equals_single_fits(gpu_lib):
    """One graph launch gives every pair the NNF that a separate fit with the same settings gives;
    replaying after new images are copied into the inputs gives the new pairs' NNFs."""
    import torch
    from annfmp_gb300 import ANNFieldPropKDTreeGB300
    from annfmp_gb300.batch import BatchNNF
    pairs = _pairs(5)
    bt = BatchNNF(n_neighbors=1, psize=7, dim_reduced=8, leaf_size=32, iters=2, seed=0).prepare(pairs)
    outs = [o.clone() for o in bt.run()]
    torch.cuda.synchronize()
    for (A, B), o, m in zip(pairs, outs, bt.models):
        ref = ANNFieldPropKDTreeGB300(form="parallel", iters=2, leaf_size=32, n_neighbors=1, psize=7, dim_reduced=8,
                                      n_subset=m.n_subset, seed=0, verbose=0).fit(A, B)
        assert torch.equal(o, ref)
    # a new batch of the same shapes through the same graph
    new = _pairs(5, seed=2)
    for (A, B), (A2, B2) in zip(bt.inputs, new):
        A.copy_(torch.flip(A2, dims=[0]))
        B.copy_(torch.flip(B2, dims=[0]))
    outs2 = bt.run()
    torch.cuda.synchronize()
    for (A, B), o, m in zip(bt.inputs, outs2, bt.models):
        ref = ANNFieldPropKDTreeGB300(form="parallel", iters=2, leaf_size=32, n_neighbors=1, psize=7, dim_reduced=8,
                                      n_subset=m.n_subset, seed=0, verbose=0).fit(A.clone(), B.clone())
        assert torch.equal(o, ref)


def test_autotuner_picks_a_candidate_within_budget(gpu_lib, tmp_path):
    from annfmp_gb300.batch import Autotuner, BatchNNF
    pairs = _pairs(2, seed=5, lo=150, hi=220)
    tuner = Autotuner(max_error=0.05, path=str(tmp_path / "tune.json"), samples=256, reps=1)
    bt = BatchNNF(n_neighbors=1, psize=7, dim_reduced=8, seed=0, tuner=tuner).prepare(pairs)
    for leaf, it in bt.settings():
        assert leaf in Autotuner.LEAVES and it in Autotuner.ITERS
    assert (tmp_path / "tune.json").exists() and len(tuner.table) >= 1
    for entry in tuner.table.values():
        errs = [t[1] for t in entry["trials"] if t[2] == entry["choice"][0] and t[3] == entry["choice"][1]]
        assert errs and (errs[0] <= 0.05 or errs[0] == min(t[1] for t in entry["trials"]))
    outs = bt.run()
    assert all(o.dtype.is_floating_point is False and o.numel() > 0 for o in outs)
