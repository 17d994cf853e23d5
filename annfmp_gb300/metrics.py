"""Distance error of an NNF against the exact raw-patch nearest neighbour.

For n sampled A pixels (``numpy.random.default_rng(seed)``, without replacement) the exact nearest
B patch is found on the GPU by an integer brute force over every B patch (``annf_raw_nn``); the
NNF's own choice is scored with the same exact integer SSD. The error of a pixel is
``d_found / d_exact - 1`` (L2 distances, FP64); pixels whose exact distance is 0 are excluded and
counted. The reference has no quality metric beyond the mean raw-patch L2 of its example
(examples/simple.py:31-36), which ``mean_patch_l2`` reproduces.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._torch import ptr, require_cuda, stream_ptr, to_device


def _patch_ssd(img_a, img_b, psize, pix_a, pix_b):
    """Exact integer SSD of A patches pix_a against B patches pix_b (host, vectorised)."""
    img_a = np.asarray(img_a).astype(np.int32)
    img_b = np.asarray(img_b).astype(np.int32)
    if img_a.ndim == 2:
        img_a, img_b = img_a[:, :, None], img_b[:, :, None]
    nca = img_a.shape[1] - psize + 1
    ncb = img_b.shape[1] - psize + 1
    ay, ax = np.divmod(np.asarray(pix_a), nca)
    by, bx = np.divmod(np.asarray(pix_b), ncb)
    acc = np.zeros(len(ay), np.int64)
    for r in range(psize):
        for c in range(psize):
            d = img_a[ay + r, ax + c, :] - img_b[by + r, bx + c, :]
            acc += (d * d).sum(axis=1)
    return acc


def exact_nn(img_a, img_b, psize, pixels, device=0):
    """(ssd int64, B index int64) of the exact raw-patch nearest neighbour of the given A pixels."""
    dev = require_cuda(device)
    A = to_device(img_a, torch.uint8, dev)
    B = to_device(img_b, torch.uint8, dev)
    if A.dim() == 2:
        A, B = A.unsqueeze(-1), B.unsqueeze(-1)
    q = torch.as_tensor(np.asarray(pixels, dtype=np.int32), device=dev)
    best = torch.empty(len(q), dtype=torch.int64, device=dev)
    h = _lib.Handle(dev.index)
    h.call("annf_raw_nn", ptr(A), A.shape[0], A.shape[1], ptr(B), B.shape[0], B.shape[1], A.shape[2], int(psize),
           ptr(q), len(q), ptr(best), stream_ptr(dev))
    b = best.cpu().numpy().view(np.uint64)
    return (b >> np.uint64(32)).astype(np.int64), (b & np.uint64(0xFFFFFFFF)).astype(np.int64)


def distance_ratio_error(img_a, img_b, nnf, psize, n_samples=4096, seed=7, device=0):
    """dict(mean, p99, max, n, n_zero): d_found / d_exact - 1 over n_samples sampled A pixels."""
    img_a = img_a.cpu().numpy() if isinstance(img_a, torch.Tensor) else np.asarray(img_a)
    img_b = img_b.cpu().numpy() if isinstance(img_b, torch.Tensor) else np.asarray(img_b)
    nnf = nnf.cpu().numpy() if isinstance(nnf, torch.Tensor) else np.asarray(nnf)
    n_a = (img_a.shape[0] - psize + 1) * (img_a.shape[1] - psize + 1)
    rng = np.random.default_rng(seed)
    pix = np.sort(rng.choice(n_a, size=min(n_samples, n_a), replace=False))
    ssd_exact, _ = exact_nn(img_a, img_b, psize, pix, device)
    ssd_found = _patch_ssd(img_a, img_b, psize, pix, nnf[pix])
    assert np.all(ssd_found >= ssd_exact), "an NNF entry beat the exact nearest neighbour"
    nz = ssd_exact > 0
    ratio = np.sqrt(ssd_found[nz].astype(np.float64)) / np.sqrt(ssd_exact[nz].astype(np.float64)) - 1.0
    return dict(mean=float(ratio.mean()) if ratio.size else 0.0,
                p99=float(np.percentile(ratio, 99)) if ratio.size else 0.0,
                max=float(ratio.max()) if ratio.size else 0.0, n=int(nz.sum()), n_zero=int((~nz).sum()),
                seed=seed)


def mean_patch_l2(img_a, img_b, nnf, psize):
    """Mean over A pixels of the raw-patch L2 of the NNF's match (examples/simple.py:31-36)."""
    img_a = np.asarray(img_a)
    n_a = (img_a.shape[0] - psize + 1) * (img_a.shape[1] - psize + 1)
    pix = np.arange(n_a)
    out = np.empty(n_a)
    step = 1 << 18
    for s in range(0, n_a, step):
        out[s:s + step] = np.sqrt(_patch_ssd(img_a, img_b, psize, pix[s:s + step], np.asarray(nnf)[s:s + step]))
    return float(out.mean())
