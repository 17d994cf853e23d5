"""Learned offset proposals for the parallel NNF form.

A small BF16 CNN looks at the pair at 1/4 resolution and predicts, per low-resolution pixel, four
candidate offsets (dx, dy) from an A patch to its B match. ``ProposalNet.propose`` turns them into
B patch indices, which the parallel form verifies with the exact raw-patch distance beside its
tree candidates (the tree stays the fallback and decides every pixel whose proposals are worse).
By default (``per_pixel=1``) each A pixel verifies one of its block's four hypotheses, 2 (y mod 2)
+ (x mod 2), so every 2x2 group of pixels tries all four and the propagation passes carry the
winners to the neighbours: at 2048x2048 this measured 11.30 ms per NNF at 0.365% mean distance
error, against 11.57 ms at 0.362% when every pixel verifies all four (``per_pixel=4``), in the
same build. The reference has no learned part; its propagation candidates come only from
the row above (annfmp/openmp/kdtree/src/base.c:255-282).

Network: the pair at 1/4 resolution (6 channels + 2 zero), six 3x3 convolutions 8->32, 32->32 x4,
32->8 with ReLU after the first five, BF16 activations and weights, FP32 sums. Every forward,
backward and optimiser step runs in this library's own kernels (``csrc/cnn.cu``); torch only holds
the buffers.

Training (``train``): flow-warped 1024x1024 pairs generated on the GPU with seeds 1000..10999
(the same recipe as ``gen.pair_flow``: 1/f spectral noise, smooth Gaussian-filtered flow of
standard deviation 20 px, bilinear warp, N(0, 4^2) noise), targets = the plain method's NNF of each
pair (patch 7x7, PCA 8, leaf 32, k 1): each low-resolution pixel's four hypotheses learn to cover
the 16 offsets of the A patches centred in its 4x4 block (relaxed winner-takes-all L1, truncated at
40 px), Adam.

    python -m annfmp_gb300.proposal train --out annfmp_gb300/weights/proposal_flow.npz
"""
from __future__ import annotations

import argparse
import math
import os
import time

import numpy as np
import torch

from . import _lib
from ._torch import ptr, require_cuda, stream_ptr, to_device

LAYERS = [(8, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 8)]
WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")
DEFAULT_WEIGHTS = os.path.join(WEIGHTS_DIR, "proposal_flow.npz")
N_HYP = 4  # offset hypotheses per low-resolution pixel (the last layer's 8 outputs)


class ProposalNet:
    """The offset-proposal network. ``weights``: None (random He initialisation from ``seed``), a
    path to an .npz with w0..w5 [co,3,3,ci] and b0..b5 [co], or a dict of such arrays."""

    def __init__(self, weights=None, device=0, seed=0, per_pixel=1):
        if per_pixel not in (1, 2, N_HYP):
            raise ValueError("per_pixel must be 1, 2 or 4")
        self.per_pixel = int(per_pixel)
        self.dev = require_cuda(device)
        self.h = _lib.Handle(self.dev.index)
        if weights is None:
            rs = np.random.RandomState(seed)
            arrs = {}
            for li, (ci, co) in enumerate(LAYERS):
                std = math.sqrt(2.0 / (9 * ci)) if li < len(LAYERS) - 1 else 0.1 * math.sqrt(1.0 / (9 * ci))
                arrs[f"w{li}"] = (rs.standard_normal((co, 3, 3, ci)) * std).astype(np.float32)
                arrs[f"b{li}"] = np.zeros(co, np.float32)
            if True:  # spread the four hypotheses' initial offsets: (0,0), (+-1, +-1) x 16 px / 4
                b = arrs[f"b{len(LAYERS) - 1}"]
                b[:] = np.array([0, 0, 0.25, 0.25, -0.25, 0.25, 0.0, -0.35], np.float32)
        elif isinstance(weights, (str, os.PathLike)):
            z = np.load(weights)
            arrs = {k: z[k] for k in z.files}
        else:
            arrs = dict(weights)
        self.meta = {k: arrs[k] for k in arrs if k.startswith("meta_")}
        self.W, self.b = [], []
        for li, (ci, co) in enumerate(LAYERS):
            w = np.asarray(arrs[f"w{li}"], np.float32)
            if w.shape != (co, 3, 3, ci):
                raise ValueError(f"layer {li}: weight shape {w.shape}, expected {(co, 3, 3, ci)}")
            self.W.append(torch.from_numpy(np.ascontiguousarray(w)).to(self.dev))
            self.b.append(torch.from_numpy(np.asarray(arrs[f"b{li}"], np.float32).copy()).to(self.dev))
        self.wf = [torch.empty(9 * ci * co, dtype=torch.float32, device=self.dev) for ci, co in LAYERS]
        self.wb = [torch.empty(9 * ci * co, dtype=torch.float32, device=self.dev) for ci, co in LAYERS]
        self.wt = [torch.empty(((co + 15) // 16 * 16) * (288 if ci == 32 else 80), dtype=torch.int16, device=self.dev)
                   for ci, co in LAYERS]
        self.tensor_cores = True  # forward convolutions on tcgen05 (False: the CUDA-core kernels)
        self._dirty = True

    @classmethod
    def pretrained(cls, device=0, per_pixel=1):
        return cls(DEFAULT_WEIGHTS, device=device, per_pixel=per_pixel)

    # -- state ------------------------------------------------------------------------------------
    def state(self) -> dict:
        out = {}
        for li in range(len(LAYERS)):
            out[f"w{li}"] = self.W[li].cpu().numpy()
            out[f"b{li}"] = self.b[li].cpu().numpy()
        out.update(self.meta)
        return out

    def save(self, path: str, **meta):
        st = self.state()
        for k, v in meta.items():
            st["meta_" + k] = np.asarray(v)
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez(path, **st)

    def _stream(self):
        return stream_ptr(self.dev)

    def _prep(self):
        if not self._dirty:
            return
        for li, (ci, co) in enumerate(LAYERS):
            self.h.call("annf_cnn_prep_weights", ptr(self.W[li]), co, ci, ptr(self.wf[li]), ptr(self.wb[li]),
                        self._stream())
            self.h.call("annf_cnn_prep_weights_tc", ptr(self.W[li]), co, ci, ptr(self.wt[li]), self._stream())
        self._dirty = False

    # -- forward ----------------------------------------------------------------------------------
    def net_input(self, A: torch.Tensor, B: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """[H/4, W/4, 8] BF16 input of one pair (uint8 HxWx3 device images of the same size)."""
        H, W = A.shape[0], A.shape[1]
        if out is None:
            out = torch.empty((H // 4, W // 4, 8), dtype=torch.bfloat16, device=self.dev)
        self.h.call("annf_cnn_input", ptr(A), ptr(B), H, W, ptr(out), self._stream())
        return out

    def forward(self, X: torch.Tensor, keep=False):
        """X [N, h, w, 8] BF16 -> FP32 output [N, h, w, 8] (and the stored activations if keep)."""
        self._prep()
        n, hh, ww = X.shape[0], X.shape[1], X.shape[2]
        acts = [X]
        x = X
        for li, (ci, co) in enumerate(LAYERS):
            last = li == len(LAYERS) - 1
            y = torch.empty((n, hh, ww, co), dtype=torch.float32 if last else torch.bfloat16, device=self.dev)
            if self.tensor_cores:
                self.h.call("annf_cnn_conv_forward_tc", ptr(x), n, hh, ww, ci, co, ptr(self.wt[li]), ptr(self.b[li]),
                            0 if last else 1, ptr(y), self._stream())
            else:
                self.h.call("annf_cnn_conv_forward", ptr(x), n, hh, ww, ci, co, ptr(self.wf[li]), ptr(self.b[li]),
                            0 if last else 1, ptr(y), self._stream())
            if not last:
                acts.append(y)
            x = y
        return (x, acts) if keep else x

    def propose(self, A, B, psize: int):
        """int32 [n_A, per_pixel] B patch indices for the A patches of the pair (None when A and B
        differ in size or are smaller than 8x8)."""
        A = to_device(A, torch.uint8, self.dev)
        B = to_device(B, torch.uint8, self.dev)
        if A.dim() == 2:
            return None
        if A.shape != B.shape or A.shape[2] != 3 or A.shape[0] < 8 or A.shape[1] < 8:
            return None
        H, W = A.shape[0], A.shape[1]
        X = self.net_input(A, B).unsqueeze(0)
        out = self.forward(X)
        n_a = (H - psize + 1) * (W - psize + 1)
        props = torch.empty((n_a, self.per_pixel), dtype=torch.int32, device=self.dev)
        self.h.call("annf_cnn_proposals_per_pixel", ptr(out), X.shape[1], X.shape[2], H, W, H, W, int(psize),
                    self.per_pixel, ptr(props), self._stream())
        return props

    def seed(self, A, B, psize: int, props: torch.Tensor) -> torch.Tensor:
        """int32 [2, n_A] match array: the best of each A patch's proposals by exact raw SSD (B
        index, then SSD; -1 / INT32_MAX where none is valid). Needs no tree, so it can run beside
        the PCA fit and the tree build (on the caller's current stream)."""
        A = to_device(A, torch.uint8, self.dev)
        B = to_device(B, torch.uint8, self.dev)
        H, W = A.shape[0], A.shape[1]
        c = A.shape[2] if A.dim() == 3 else 1
        n_a = (H - psize + 1) * (W - psize + 1)
        out = torch.empty((2, n_a), dtype=torch.int32, device=self.dev)
        self.h.call("annf_seed_matches", ptr(A), H, W, ptr(B), B.shape[0], B.shape[1], c, int(psize), ptr(props),
                    int(props.shape[1]), ptr(out), self._stream())
        return out

    # -- backward ---------------------------------------------------------------------------------
    def backward(self, acts, dout):
        """Gradients [(dW [co,3,3,ci], db [co]), ...] of every layer for dL/d out = dout."""
        self._prep()
        n, hh, ww = dout.shape[0], dout.shape[1], dout.shape[2]
        grads = [None] * len(LAYERS)
        g = dout
        for li in range(len(LAYERS) - 1, -1, -1):
            ci, co = LAYERS[li]
            mask = None if li == len(LAYERS) - 1 else acts[li + 1]
            dW = torch.zeros((co, 3, 3, ci), dtype=torch.float32, device=self.dev)
            db = torch.zeros(co, dtype=torch.float32, device=self.dev)
            self.h.call("annf_cnn_conv_backward_weights", ptr(acts[li]), ptr(g), ptr(mask), n, hh, ww, ci, co,
                        ptr(dW), ptr(db), self._stream())
            grads[li] = (dW, db)
            if li > 0:
                dx = torch.empty((n, hh, ww, ci), dtype=torch.float32, device=self.dev)
                self.h.call("annf_cnn_conv_backward_data", ptr(g), ptr(mask), n, hh, ww, co, ci, ptr(self.wb[li]),
                            ptr(dx), self._stream())
                g = dx
        return grads

    def loss(self, out, tgt, valid):
        """(loss tensor [1], dL/d out) of the relaxed winner-takes-all L1 loss."""
        npix = out.shape[0] * out.shape[1] * out.shape[2]
        nv = max(int(valid.sum().item()), 1)  # valid sub-targets
        dout = torch.empty_like(out)
        acc = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self.h.call("annf_cnn_wta_loss", ptr(out), ptr(tgt), ptr(valid), npix, 1.0 / nv, ptr(dout), ptr(acc),
                    self._stream())
        return acc, dout


# ---------------------------------------------------------------------------------------------
# training data on the GPU
# ---------------------------------------------------------------------------------------------
def gpu_flow_pair(seed: int, size: int = 1024, magnitude: float = 20.0, sigma: float = 64.0, noise: float = 4.0,
                  device=0, return_flow=False):
    """A flow-warped pair generated on the GPU (the recipe of gen.pair_flow with torch's RNG):
    uint8 (size, size, 3) device tensors A, B (and the flow u [2, size, size], B(p) = A(p + u(p)),
    when return_flow)."""
    dev = require_cuda(device)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    fy = torch.fft.fftfreq(size, device=dev)[:, None]
    fx = torch.fft.rfftfreq(size, device=dev)[None, :]
    f2 = fx * fx + fy * fy
    amp = torch.where(f2 > 0, 1.0 / torch.sqrt(torch.where(f2 > 0, f2, torch.ones_like(f2))), torch.zeros_like(f2))
    white = torch.randn((3, size, size), generator=g, device=dev)
    img = torch.fft.irfft2(torch.fft.rfft2(white) * amp, s=(size, size))
    lo, hi = img.min(), img.max()
    a = torch.clamp(torch.round((img - lo) * (255.0 / torch.clamp(hi - lo, min=1e-12))), 0, 255)
    u = torch.randn((2, size, size), generator=g, device=dev) * magnitude
    gk = torch.exp(-2.0 * (math.pi ** 2) * sigma * sigma * f2)
    u = torch.fft.irfft2(torch.fft.rfft2(u) * gk, s=(size, size))
    u = u * (magnitude / torch.clamp(u.std(dim=(1, 2), keepdim=True), min=1e-12))
    yy, xx = torch.meshgrid(torch.arange(size, device=dev, dtype=torch.float32),
                            torch.arange(size, device=dev, dtype=torch.float32), indexing="ij")
    sy, sx = yy + u[0], xx + u[1]
    grid = torch.stack([sx / (size - 1) * 2 - 1, sy / (size - 1) * 2 - 1], dim=-1)[None]
    warped = torch.nn.functional.grid_sample(a[None], grid, mode="bilinear", padding_mode="reflection",
                                             align_corners=True)[0]
    b = torch.clamp(torch.round(warped + noise * torch.randn(warped.shape, generator=g, device=dev)), 0, 255)
    A, B = a.permute(1, 2, 0).contiguous().to(torch.uint8), b.permute(1, 2, 0).contiguous().to(torch.uint8)
    return (A, B, u) if return_flow else (A, B)


_PLAIN = {}


def plain_nnf(A, B, psize=7, dim_reduced=8, leaf_size=32, seed=0, device=0):
    """The plain method's NNF (k 1) of a pair, on the device (one estimator reused per setting)."""
    from .field import ANNFieldPropKDTreeGB300
    n_b = (B.shape[0] - psize + 1) * (B.shape[1] - psize + 1)
    key = (psize, dim_reduced, leaf_size, n_b, str(device))
    m = _PLAIN.get(key)
    if m is None:
        m = ANNFieldPropKDTreeGB300(n_neighbors=1, psize=psize, dim_reduced=dim_reduced,
                                    n_subset=int(round(0.1 * n_b)), leaf_size=leaf_size, seed=seed, verbose=0,
                                    device=device)
        _PLAIN[key] = m
    m.seed = seed
    return m.fit(A, B)


def train(n_pairs=10000, seed0=1000, size=1024, batch=8, lr=2e-3, lr_min=1e-4, device=0, out_path=None,
          log_every=25, psize=7, init_seed=0, log=print):
    """Train from scratch on n_pairs pairs (seeds seed0 ..), one pass; returns the network."""
    dev = require_cuda(device)
    net = ProposalNet(None, device=dev.index, seed=init_seed)
    h = net.h
    m = [torch.zeros_like(p) for p in net.W + net.b]
    v = [torch.zeros_like(p) for p in net.W + net.b]
    h4 = w4 = size // 4
    X = torch.empty((batch, h4, w4, 8), dtype=torch.bfloat16, device=dev)
    T = torch.empty((batch, h4, w4, 16, 2), dtype=torch.float32, device=dev)
    V = torch.empty((batch, h4, w4, 16), dtype=torch.uint8, device=dev)
    steps = n_pairs // batch
    t0 = time.time()
    hist = []
    for step in range(steps):
        for j in range(batch):
            s = seed0 + step * batch + j
            A, B = gpu_flow_pair(s, size, device=dev)
            nnf = plain_nnf(A, B, psize=psize, seed=s, device=dev)
            net.net_input(A, B, out=X[j])
            h.call("annf_cnn_targets", ptr(nnf), size, size, size, psize, ptr(T[j]), ptr(V[j]), stream_ptr(dev))
        out, acts = net.forward(X, keep=True)
        loss, dout = net.loss(out, T, V)
        grads = net.backward(acts, dout)
        cur_lr = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * step / max(steps - 1, 1)))
        params = net.W + net.b
        gl = [g for g, _ in grads] + [b for _, b in grads]
        for i, (p, gr) in enumerate(zip(params, gl)):
            h.call("annf_cnn_adam", ptr(p), ptr(gr), ptr(m[i]), ptr(v[i]), p.numel(), cur_lr, 0.9, 0.999, 1e-8,
                   step + 1, stream_ptr(dev))
        net._dirty = True
        hist.append(loss)
        if (step + 1) % log_every == 0 or step == steps - 1:
            lv = float(torch.stack(hist).mean().item())
            hist = []
            log(f"step {step + 1}/{steps} pairs {(step + 1) * batch} loss {lv:.4f} lr {cur_lr:.2e} "
                f"{time.time() - t0:.1f}s")
    if out_path:
        net.save(out_path, seeds=np.array([seed0, seed0 + steps * batch - 1]), size=size, batch=batch, steps=steps,
                 lr=lr, psize=psize)
    return net


def evaluate(net, seeds, size=1024, psize=7, device=0):
    """Mean loss and the fraction of valid sub-targets (A patches' plain-method offsets) within 1.5
    px (L1) of one of their block's four hypotheses, over held-out pairs."""
    dev = require_cuda(device)
    h4 = size // 4
    tot, hit, cnt = 0.0, 0, 0
    for s in seeds:
        A, B = gpu_flow_pair(s, size, device=dev)
        nnf = plain_nnf(A, B, psize=psize, seed=s, device=dev)
        X = net.net_input(A, B).unsqueeze(0)
        T = torch.empty((1, h4, h4, 16, 2), dtype=torch.float32, device=dev)
        V = torch.empty((1, h4, h4, 16), dtype=torch.uint8, device=dev)
        net.h.call("annf_cnn_targets", ptr(nnf), size, size, size, psize, ptr(T), ptr(V), stream_ptr(dev))
        out = net.forward(X)
        loss, _ = net.loss(out, T, V)
        o = out.reshape(1, h4, h4, 1, 4, 2) * 16.0
        e = (o - T[..., None, :]).abs().sum(-1).min(-1).values
        vm = V.bool()
        hit += int((e[vm] <= 1.5).sum().item())
        cnt += int(vm.sum().item())
        tot += float(loss.item())
    return dict(loss=tot / max(len(seeds), 1), hit_rate=hit / max(cnt, 1))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    tr = sub.add_parser("train")
    tr.add_argument("--pairs", type=int, default=10000)
    tr.add_argument("--seed0", type=int, default=1000)
    tr.add_argument("--size", type=int, default=1024)
    tr.add_argument("--batch", type=int, default=8)
    tr.add_argument("--lr", type=float, default=2e-3)
    tr.add_argument("--out", default=DEFAULT_WEIGHTS)
    tr.add_argument("--eval-seeds", type=int, default=8)
    args = ap.parse_args(argv)
    if args.cmd == "train":
        net = train(n_pairs=args.pairs, seed0=args.seed0, size=args.size, batch=args.batch, lr=args.lr,
                    out_path=args.out)
        held = list(range(900000, 900000 + args.eval_seeds))
        print("held-out", evaluate(net, held, size=args.size), flush=True)
        print("untrained", evaluate(ProposalNet(None, device=0), held, size=args.size), flush=True)


if __name__ == "__main__":
    main()
