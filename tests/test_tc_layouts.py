"""The shared-memory operand layouts of two tensor-core kernels, checked on the CPU.

A K-major, no-swizzle tcgen05 operand is read as 8-row x 16-byte core matrices: element (row m,
column k) of an operand whose descriptor starts at `start` sits at byte
start + (m // 8) * SBO + (k // 8) * LBO + (m % 8) * 16 + (k % 8) * 2. These tests build the bytes
the kernels stage (csrc/proj_tc.cu row form, csrc/cnn.cu 32-channel convolution), read them
through that formula with the kernels' descriptors, and compare the products with the oracle's
patches: no GPU is involved, only the addressing that the kernels rely on.
"""
import numpy as np


def _operand(buf_halves, start, lbo, sbo, rows, cols):
    """rows x cols FP16 values read from a half-precision buffer through a K-major descriptor."""
    m = np.arange(rows)[:, None]
    k = np.arange(cols)[None, :]
    byte = start + (m // 8) * sbo + (k // 8) * lbo + (m % 8) * 16 + (k % 8) * 2
    assert byte.max() + 2 <= 2 * buf_halves.size, "descriptor reads past the staged buffer"
    return buf_halves[byte // 2]


def test_row_form_projection_reads_every_second_patch_in_place(oracle_mod):
    rng = np.random.default_rng(7)
    H, W, C, p, d = 14, 300, 3, 9, 16
    img = rng.integers(0, 256, (H, W, C), dtype=np.uint8)
    comps = rng.standard_normal((d, p * p * C))
    cb = comps.astype(np.float32).astype(np.float16).astype(np.float64)
    kr = (4 * p + 15) // 16 * 16          # K per filter row (48 for p = 9)
    pe = 254 + kr // 4                    # pixels per converted copy
    ncols = W - p + 1
    y, x0 = 2, 0
    # B of filter row r: [d][kr], k = 4 s + ch
    B = np.zeros((p, d, kr))
    for r in range(p):
        for s in range(p):
            for ch in range(C):
                B[r, :, 4 * s + ch] = cb[:, (r * p + s) * C + ch]
    got = np.zeros((256, d))
    for half in (0, 1):
        for r in range(p):
            row = np.zeros((pe, 4))
            for q in range(pe):
                X = x0 + half + q
                if X < W:
                    row[q, :C] = img[y + r, X]
            buf = row.reshape(-1)         # the converted copy: 4 FP16 channels per pixel
            for kk in range(kr // 16):
                A = _operand(buf, 32 * kk, 16, 128, 128, 16)
                got[half::2] += A @ B[r, :, 16 * kk:16 * kk + 16].T
    X = oracle_mod.extract_patches(img, p).astype(np.float64)
    want = X[y * ncols + x0: y * ncols + x0 + 256] @ cb.T
    assert np.allclose(got, want, rtol=0, atol=1e-6 * np.abs(want).max())


def test_conv_planes_are_the_taps_of_a_32_channel_convolution():
    rng = np.random.default_rng(8)
    h, w, CI, SPIX = 5, 140, 32, 130
    X = rng.standard_normal((h, w, CI)).astype(np.float32)
    y, x0 = 2, 0
    # staged planes [row ry][channel group c8][pixel px][8 channels], pixel px = image column x0 - 1 + px
    planes = np.zeros((3, CI // 8, SPIX, 8), np.float32)
    for ry in range(3):
        for px in range(SPIX):
            yy, xx = y + ry - 1, x0 + px - 1
            if 0 <= yy < h and 0 <= xx < w:
                planes[ry, :, px, :] = X[yy, xx].reshape(CI // 8, 8)
    buf = planes.reshape(-1)
    plane_bytes = SPIX * 16
    for ky in range(3):
        for kx in range(3):
            for kk in range(CI // 16):
                start = ky * (CI // 8) * plane_bytes + kx * 16 + 2 * kk * plane_bytes
                A = _operand(buf, start, plane_bytes, 128, 128, 16)
                want = np.zeros((128, 16), np.float32)
                for i in range(128):
                    yy, xx = y + ky - 1, x0 + i + kx - 1
                    if 0 <= yy < h and 0 <= xx < w:
                        want[i] = X[yy, xx, 16 * kk:16 * kk + 16]
                assert np.array_equal(A, want), (ky, kx, kk)
