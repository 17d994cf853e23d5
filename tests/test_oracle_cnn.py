"""CPU checks of the proposal-network oracle itself (finite differences, shapes, rounding)."""
import numpy as np

from oracle import cnn as C


def test_bf16_round_ties_to_even():
    x = np.array([1.0, 1.00390625, 1.01171875, -2.5, 3.0e38, 0.0], np.float32)
    r = C.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway between 1 and 1+2^-7 rounds to even (1.0)
    assert r[2] == np.float32(1.015625)
    assert r[3] == -2.5 and r[5] == 0.0


def test_conv3x3_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((2, 5, 6, 3))
    w = rng.standard_normal((4, 3, 3, 3))
    b = rng.standard_normal(4)
    g = rng.standard_normal((2, 5, 6, 4))
    f = lambda x_, w_, b_: float((C.conv3x3(x_, w_, b_) * g).sum())  # noqa: E731
    dx, dw, db = C.conv3x3_backward(x, w, g)
    eps = 1e-6
    for idx in [(0, 0, 0, 0), (1, 4, 5, 2), (0, 2, 3, 1)]:
        xp = x.copy(); xp[idx] += eps
        xm = x.copy(); xm[idx] -= eps
        assert abs((f(xp, w, b) - f(xm, w, b)) / (2 * eps) - dx[idx]) < 1e-6
    for idx in [(0, 0, 0, 0), (3, 2, 1, 2), (1, 1, 1, 1)]:
        wp = w.copy(); wp[idx] += eps
        wm = w.copy(); wm[idx] -= eps
        assert abs((f(x, wp, b) - f(x, wm, b)) / (2 * eps) - dw[idx]) < 1e-6
    bp = b.copy(); bp[2] += eps
    bm = b.copy(); bm[2] -= eps
    assert abs((f(x, w, bp) - f(x, w, bm)) / (2 * eps) - db[2]) < 1e-6


def test_wta_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    out = rng.standard_normal((1, 3, 4, 8)).astype(np.float64)
    tgt = rng.standard_normal((1, 3, 4, 16, 2)) * 10
    valid = rng.random((1, 3, 4, 16)) > 0.2
    loss, dout = C.wta_loss(out, tgt, valid)
    eps = 1e-7
    for idx in [(0, 0, 0, 0), (0, 1, 2, 5), (0, 2, 3, 7)]:
        op = out.copy(); op[idx] += eps
        om = out.copy(); om[idx] -= eps
        fd = (C.wta_loss(op, tgt, valid)[0] - C.wta_loss(om, tgt, valid)[0]) / (2 * eps)
        assert abs(fd - dout[idx]) < 1e-5 * max(1.0, abs(fd))


def test_full_backward_matches_finite_differences_without_rounding():
    """With BF16 rounding bypassed, forward + backward of the 6-layer net agree with finite
    differences of the loss (checks the ReLU masks and layer chaining of the oracle)."""
    rng = np.random.default_rng(2)
    params = []
    for ci, co in C.CHANNELS:
        params.append(((rng.standard_normal((co, 3, 3, ci)) * np.sqrt(2.0 / (9 * ci))),
                       rng.standard_normal(co) * 0.1))
    x0 = rng.standard_normal((1, 6, 5, 8))
    tgt = rng.standard_normal((1, 6, 5, 16, 2)) * 8
    valid = np.ones((1, 6, 5, 16), bool)
    def loss_of(ps):
        acts, out = C.forward(x0, ps, exact=True)
        return C.wta_loss(out, tgt, valid)[0]
    acts, out = C.forward(x0, params, exact=True)
    _, dout = C.wta_loss(out, tgt, valid)
    grads = C.backward(acts, dout, params, exact=True)
    eps = 1e-6
    for li, idx in [(0, (3, 1, 1, 2)), (2, (5, 0, 2, 7)), (5, (1, 1, 1, 4)), (4, (7, 2, 0, 30))]:
        w, b = params[li]
        wp = w.copy(); wp[idx] += eps
        wm = w.copy(); wm[idx] -= eps
        pp = list(params); pp[li] = (wp, b)
        pm = list(params); pm[li] = (wm, b)
        fd = (loss_of(pp) - loss_of(pm)) / (2 * eps)
        assert abs(fd - grads[li][0][idx]) < 1e-5 * max(1.0, abs(fd)), (li, fd, grads[li][0][idx])


def test_targets_and_proposals_on_a_pure_shift():
    H = W = 32
    p = 5
    n_cols = W - p + 1
    ys, xs = np.divmod(np.arange((H - p + 1) * n_cols), n_cols)
    by = np.clip(ys + 2, 0, H - p)
    bx = np.clip(xs - 3, 0, W - p)
    nnf = (by * n_cols + bx).astype(np.int32)
    tgt, valid = C.targets_from_nnf(nnf, H, W, H, W, p)
    assert valid[2:5, 2:5].all()
    assert np.allclose(tgt[3, 3], np.tile([-3, 2], (16, 1)))
    out = np.zeros((H // 4, W // 4, 8), np.float32)
    out[..., 0::2] = -3 / 16.0
    out[..., 1::2] = 2 / 16.0
    props = C.proposals(out, H, W, H, W, p)
    assert np.array_equal(props[:, 0], nnf)


def test_proposals_per_pixel_take_their_share_of_the_hypotheses():
    """per_pixel 1: pixel (y, x) takes hypothesis 2 (y mod 2) + (x mod 2), so each 2x2 group of
    pixels covers all four; per_pixel 2: hypotheses 0, 1 for x + y even and 2, 3 for odd; every
    choice is a column of the four-per-pixel proposals."""
    rng = np.random.default_rng(4)
    H, W, p = 29, 38, 5
    n_cols = W - p + 1
    out = (rng.standard_normal((H // 4, W // 4, 8)) * 0.5).astype(np.float32)
    full = C.proposals(out, H, W, H, W, p)
    ys, xs = np.divmod(np.arange(full.shape[0]), n_cols)
    one = C.proposals(out, H, W, H, W, p, per_pixel=1)
    assert one.shape == (full.shape[0], 1)
    assert np.array_equal(one[:, 0], full[np.arange(full.shape[0]), 2 * (ys % 2) + xs % 2])
    two = C.proposals(out, H, W, H, W, p, per_pixel=2)
    j0 = 2 * ((xs + ys) % 2)
    assert np.array_equal(two, np.stack([full[np.arange(full.shape[0]), j0], full[np.arange(full.shape[0]), j0 + 1]], 1))
    assert np.array_equal(C.proposals(out, H, W, H, W, p, per_pixel=4), full)
