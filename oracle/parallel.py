"""CPU restatement of the parallel NNF form's search -- TEST INFRASTRUCTURE ONLY.

The parallel form has no counterpart in the reference (annfmp computes row-sequential
propagation only, annfmp/openmp/kdtree/src/base.c:150-360). This module restates, in numpy, what
the form does after the natural-leaf kNN, so that the GPU's NNF can be checked index for index:

* initial choice: per A pixel, the lexicographic minimum of (exact raw SSD, B index) over an
  optional seed match, the k natural-leaf neighbours and any proposals (B indices, -1 = none;
  candidates whose patch row lies outside B are dropped);
* ``iters`` passes: pass t offers the four neighbours' matches (up, down, left, right) shifted by
  one pixel back onto this pixel, and ``nrand`` random offsets within radius max(1, r0 >> t)
  around the pass's starting match (a 32-bit hash of (seed * 7919 + t, pixel, sample)); a
  candidate equal to the starting match is not tried; the pass keeps the lexicographic minimum.

Only tests import this module.
"""
from __future__ import annotations

import numpy as np

_M32 = np.uint64(0xFFFFFFFF)


def _mul32(a, b):
    return (a * np.uint64(b)) & _M32


def hash3(a, b, c):
    """The 32-bit mixing hash of the random offsets (uint64 arrays holding 32-bit values)."""
    a, b, c = (np.asarray(v, np.uint64) & _M32 for v in (a, b, c))
    h = _mul32(a, 0x9E3779B1) ^ _mul32((b + np.uint64(0x7F4A7C15)) & _M32, 0x85EBCA77) \
        ^ _mul32((c + np.uint64(0x165667B1)) & _M32, 0xC2B2AE3D)
    h ^= h >> np.uint64(15)
    h = _mul32(h, 0x2C1B3C6D)
    h ^= h >> np.uint64(12)
    h = _mul32(h, 0x297A2D39)
    h ^= h >> np.uint64(15)
    return h


class _Patches:
    def __init__(self, a, b, psize):
        from oracle.oracle import extract_patches
        self.pa = extract_patches(a, psize).astype(np.int32)
        self.pb = extract_patches(b, psize).astype(np.int32)
        self.nca = a.shape[1] - psize + 1
        self.nra = a.shape[0] - psize + 1
        self.ncb = b.shape[1] - psize + 1
        self.nrb = b.shape[0] - psize + 1

    def ssd(self, rows, cand):
        """Exact SSD of A patches ``rows`` against B patches ``cand`` (all valid)."""
        d = self.pa[rows] - self.pb[cand]
        return np.einsum("ij,ij->i", d, d).astype(np.int64)


def _lexmin(best, bs, rows, cand, s):
    """Fold candidates (rows, cand, s) into (best, bs) by the lexicographic minimum of (s, index)."""
    key_new = (s << 32) | cand.astype(np.int64)
    key_old = (bs[rows] << 32) | (best[rows].astype(np.int64) & 0xFFFFFFFF)
    order = np.lexsort((key_new, rows))
    rows, key_new = rows[order], key_new[order]
    first = np.ones(len(rows), bool)
    first[1:] = rows[1:] != rows[:-1]
    r, k = rows[first], key_new[first]
    win = k < key_old[first]
    best[r[win]] = (k[win] & 0xFFFFFFFF).astype(np.int32)
    bs[r[win]] = k[win] >> 32


def parallel_search(a, b, psize, nat_idx, proposals=None, seed_match=None, iters=3, seed=0, nrand=1,
                    radius0=2):
    """NNF of the parallel form from the natural-leaf neighbours ``nat_idx`` [nA, k] (B indices).

    Returns (index [nA] int32, exact SSD [nA] int64)."""
    P = _Patches(a, b, psize)
    nA = P.nra * P.nca
    if seed_match is not None:
        best = np.asarray(seed_match[0], np.int32).copy()
        bs = np.asarray(seed_match[1], np.int64).copy()
        bs[best < 0] = 0x7FFFFFFF
    else:
        best = np.full(nA, -1, np.int32)
        bs = np.full(nA, 0x7FFFFFFF, np.int64)
    cands = [np.asarray(nat_idx, np.int64).reshape(nA, -1)]
    if proposals is not None:
        cands.append(np.asarray(proposals, np.int64).reshape(nA, -1))
    C = np.concatenate(cands, axis=1)
    rows = np.repeat(np.arange(nA), C.shape[1])
    c = C.ravel()
    ok = (c >= 0) & (c // P.ncb < P.nrb)
    _lexmin(best, bs, rows[ok], c[ok], P.ssd(rows[ok], c[ok]))

    y, x = np.divmod(np.arange(nA), P.nca)
    for it in range(iters):
        radius = max(1, radius0 >> it)
        sd = (int(seed) * 7919 + it) & 0xFFFFFFFF
        start = best.copy()
        s64 = start.astype(np.int64)
        sy = np.where(s64 < 0, -((-s64) // P.ncb), s64 // P.ncb)  # C division (toward zero)
        sx = s64 - sy * P.ncb
        cy, cx = [], []
        for ddy, ddx in ((-1, 0), (1, 0), (0, -1), (0, 1)):
            ny, nx = y + ddy, x + ddx
            inside = (ny >= 0) & (nx >= 0) & (ny < P.nra) & (nx < P.nca)
            nb = np.where(inside, start[np.clip(ny, 0, P.nra - 1) * P.nca + np.clip(nx, 0, P.nca - 1)], -1)
            nby, nbx = np.divmod(nb.astype(np.int64), P.ncb)
            cy.append(np.where(nb >= 0, nby - ddy, -1))
            cx.append(np.where(nb >= 0, nbx - ddx, -1))
        for t in range(nrand):
            r = hash3(np.uint64(sd), np.arange(nA, dtype=np.uint64), np.uint64(t))
            span = np.uint64(2 * radius + 1)
            cy.append(sy + (((r >> np.uint64(16)) % span).astype(np.int64) - radius))
            cx.append(sx + ((r % span).astype(np.int64) - radius))
        cy, cx = np.stack(cy, 1), np.stack(cx, 1)
        ok = (cy >= 0) & (cx >= 0) & (cy < P.nrb) & (cx < P.ncb)
        cand = cy * P.ncb + cx
        ok &= cand != start[:, None]
        rows = np.repeat(np.arange(nA), cand.shape[1]).reshape(cand.shape)[ok]
        cand = cand[ok]
        _lexmin(best, bs, rows, cand, P.ssd(rows, cand))
    return best, bs
