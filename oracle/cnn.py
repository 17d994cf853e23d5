"""CPU oracle of the offset-proposal network (test infrastructure only).

Numpy restatement of what the CUDA kernels of ``annfmp_gb300/csrc/cnn.cu`` compute, used by the
tests to check the forward pass and every gradient. The reference project has no learned component
(its propagation candidates come only from the row above, annfmp/openmp/kdtree/src/base.c:255-282);
the network, its loss and its training are additions of this project, so this oracle follows the
project's own definition:

* input: A and B downsampled 4x4 (box mean), (v - 127.5) / 64, channels A.rgb, B.rgb, 0, 0 (8);
* six 3x3 convolutions, zero padding, NHWC: 8->32, 32->32 (x4), 32->8, bias, ReLU after the first
  five; weights and stored activations rounded to BF16, sums in FP32 or wider;
* output: 4 hypotheses (dx, dy) per low-resolution pixel, in units of OUT_SCALE full-resolution
  pixels;
* loss: relaxed winner-takes-all truncated L1 against each low-resolution pixel's 16 sub-targets
  (the plain method's offsets of the 16 A patches centred in its 4x4 block): for sub-target s,
  e_js = |S o_jx - t_sx| + |S o_jy - t_sy| (pixels, S = OUT_SCALE), c_js = min(e_js, TRUNC),
  loss_s = c_{j*s} + EPS * sum_{j != j*} c_js with j* = argmin_j e_js (first on ties); the loss
  averages loss_s over the valid sub-targets. The four hypotheses thus learn to cover the offsets a
  block's patches take, and no single noisy match dominates the gradient.
"""
from __future__ import annotations

import numpy as np

OUT_SCALE = 16.0
EPS = 0.05
TRUNC = 40.0
CHANNELS = [(8, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 8)]


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def net_input(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """[h4, w4, 8] from two uint8 HxWx3 images of the same size (h4 = H // 4, w4 = W // 4)."""
    h4, w4 = a.shape[0] // 4, a.shape[1] // 4
    out = np.zeros((h4, w4, 8), np.float32)
    for s, img in enumerate((a, b)):
        blk = img[: h4 * 4, : w4 * 4].astype(np.float64).reshape(h4, 4, w4, 4, 3).mean(axis=(1, 3))
        out[:, :, 3 * s: 3 * s + 3] = ((blk - 127.5) / 64.0).astype(np.float32)
    return bf16_round(out)


def _pad(x):
    return np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))


def conv3x3(x: np.ndarray, w: np.ndarray, b: np.ndarray) -> np.ndarray:
    """x [N,h,w,Ci], w [Co,3,3,Ci], b [Co] -> pre-activation [N,h,w,Co] (float64)."""
    n, h, wd, ci = x.shape
    xp = _pad(x.astype(np.float64))
    y = np.zeros((n, h, wd, w.shape[0]), np.float64)
    for ky in range(3):
        for kx in range(3):
            y += xp[:, ky: ky + h, kx: kx + wd, :] @ w[:, ky, kx, :].astype(np.float64).T
    return y + b.astype(np.float64)


def conv3x3_backward(x: np.ndarray, w: np.ndarray, g: np.ndarray):
    """Gradients of conv3x3 for upstream gradient g [N,h,w,Co]: (dx, dw, db)."""
    n, h, wd, ci = x.shape
    xp = _pad(x.astype(np.float64))
    g = g.astype(np.float64)
    dw = np.zeros(w.shape, np.float64)
    dxp = np.zeros(xp.shape, np.float64)
    for ky in range(3):
        for kx in range(3):
            win = xp[:, ky: ky + h, kx: kx + wd, :]
            dw[:, ky, kx, :] = np.einsum("nhwo,nhwi->oi", g, win)
            dxp[:, ky: ky + h, kx: kx + wd, :] += g @ w[:, ky, kx, :].astype(np.float64)
    return dxp[:, 1:-1, 1:-1, :], dw, g.sum(axis=(0, 1, 2))


def forward(x0: np.ndarray, params, exact: bool = False):
    """params: list of (w [Co,3,3,Ci], b [Co]) float32 (master). Returns (acts, out): acts[l] is
    the BF16-rounded input of layer l (acts[0] = x0), out the FP32 last-layer output. exact=True
    keeps everything in float64 (no BF16/FP32 rounding; for finite-difference checks)."""
    rnd = (lambda a: np.asarray(a, np.float64)) if exact else bf16_round
    acts = [x0]
    x = x0
    for li, (w, b) in enumerate(params):
        y = conv3x3(x, rnd(w), b)
        if li < len(params) - 1:
            x = rnd(np.maximum(y, 0.0) if exact else np.maximum(y, 0.0).astype(np.float32))
            acts.append(x)
        else:
            out = y if exact else y.astype(np.float32)
    return acts, out


def wta_loss(out: np.ndarray, tgt: np.ndarray, valid: np.ndarray):
    """out [N,h,w,8], tgt [N,h,w,16,2] (pixels), valid [N,h,w,16] bool -> (loss, d loss / d out)."""
    o = out.astype(np.float64).reshape(out.shape[:-1] + (1, 4, 2)) * OUT_SCALE
    diff = o - tgt.astype(np.float64)[..., :, None, :]  # [N,h,w,16,4,2]
    e = np.abs(diff).sum(-1)  # [N,h,w,16,4]
    jstar = np.argmin(e, axis=-1)
    wgt = np.full(e.shape, EPS)
    np.put_along_axis(wgt, jstar[..., None], 1.0, axis=-1)
    nv = max(int(valid.sum()), 1)
    wgt = wgt * valid[..., None] / nv
    live = e < TRUNC
    loss = float((wgt * np.minimum(e, TRUNC)).sum())
    dout = ((wgt * live)[..., None] * np.sign(diff) * OUT_SCALE).sum(axis=-3).reshape(out.shape)
    return loss, dout


def backward(acts, out_grad, params, exact: bool = False):
    """Gradients of all (w, b) given dL/d out; the ReLU masks come from the stored activations."""
    grads = [None] * len(params)
    g = out_grad.astype(np.float64)
    for li in range(len(params) - 1, -1, -1):
        w, _ = params[li]
        x = acts[li]
        dx, dw, db = conv3x3_backward(x, np.asarray(w, np.float64) if exact else bf16_round(w), g)
        grads[li] = (dw, db)
        if li > 0:
            g = dx * (acts[li] > 0)
    return grads


def targets_from_nnf(nnf: np.ndarray, H: int, W: int, Hb: int, Wb: int, psize: int):
    """Per-low-resolution-pixel sub-targets [h4, w4, 16, 2] (dx, dy) in pixels and validity
    [h4, w4, 16]: the offsets of the 16 A patches centred in the 4x4 block (row-major in the
    block); patches that would leave the image are invalid (offset 0)."""
    n_cols, n_rows = W - psize + 1, H - psize + 1
    ncb = Wb - psize + 1
    h4, w4 = H // 4, W // 4
    tgt = np.zeros((h4, w4, 16, 2), np.float32)
    valid = np.zeros((h4, w4, 16), bool)
    half = psize // 2
    for i in range(h4):
        for j in range(w4):
            for u in range(16):
                y, x = 4 * i + u // 4 - half, 4 * j + u % 4 - half
                if 0 <= y < n_rows and 0 <= x < n_cols:
                    by, bx = divmod(int(nnf[y * n_cols + x]), ncb)
                    tgt[i, j, u] = (bx - x, by - y)
                    valid[i, j, u] = True
    return tgt, valid


def proposals(out: np.ndarray, H: int, W: int, Hb: int, Wb: int, psize: int, per_pixel: int = 4) -> np.ndarray:
    """[n_A, per_pixel] B patch indices: A patch (y, x) takes the hypotheses of the low-resolution
    pixel holding its centre, rounded to the nearest pixel and clamped to B's patch grid; all 4, or
    with per_pixel 2 hypotheses 0, 1 (x + y even) or 2, 3 (odd), or with per_pixel 1 hypothesis
    2 (y mod 2) + (x mod 2)."""
    n_cols, n_rows = W - psize + 1, H - psize + 1
    ncb, nrb = Wb - psize + 1, Hb - psize + 1
    h4, w4 = out.shape[0], out.shape[1]
    half = psize // 2
    y, x = np.divmod(np.arange(n_rows * n_cols), n_cols)
    i = np.minimum((y + half) // 4, h4 - 1)
    j = np.minimum((x + half) // 4, w4 - 1)
    o = out[i, j].astype(np.float32).reshape(-1, 4, 2) * np.float32(OUT_SCALE)
    by = np.clip(y[:, None] + np.rint(o[..., 1]).astype(np.int64), 0, nrb - 1)
    bx = np.clip(x[:, None] + np.rint(o[..., 0]).astype(np.int64), 0, ncb - 1)
    full = (by * ncb + bx).astype(np.int32)
    if per_pixel == 4:
        return full
    j0 = 2 * ((x + y) & 1) if per_pixel == 2 else 2 * (y & 1) + (x & 1)
    cols = j0[:, None] + np.arange(per_pixel)[None, :]
    return np.take_along_axis(full, cols, axis=1)
