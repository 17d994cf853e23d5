"""Seeded synthetic image pairs with the shapes and statistics of the benchmark workloads.

The reference ships no dataset (its only example reads two JPEGs through OpenCV,
examples/simple.py:8-9), so every workload here is generated. All generators use
``numpy.random.default_rng(seed)`` and return uint8 arrays of shape (H, W, 3).

* spectral noise: per channel, white Gaussian noise shaped in Fourier space to amplitude
  proportional to 1/f (power proportional to 1/f^2), then min-max scaled to [0, 255] and rounded;
* affine pair: B = A translated then rotated about the image centre (bilinear resampling,
  reflected borders), plus N(0, sigma^2) noise, clipped;
* flow pair: B(p) = A(p + u(p)) for a smooth random flow u (per-pixel N(0, s^2) displacements,
  Gaussian-filtered with the given sigma and rescaled back to standard deviation s), bilinear,
  plus N(0, sigma^2) noise, clipped.
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage


def spectral_noise(h: int, w: int, rng: np.random.Generator, channels: int = 3) -> np.ndarray:
    fy = np.fft.fftfreq(h)[:, None]
    fx = np.fft.rfftfreq(w)[None, :]
    f = np.sqrt(fx * fx + fy * fy)
    f[0, 0] = 1.0
    amp = 1.0 / f
    amp[0, 0] = 0.0
    out = np.empty((h, w, channels), np.float64)
    for c in range(channels):
        white = rng.standard_normal((h, w))
        out[:, :, c] = np.fft.irfft2(np.fft.rfft2(white) * amp, s=(h, w))
    lo, hi = out.min(), out.max()
    out = (out - lo) * (255.0 / max(hi - lo, 1e-12))
    return np.clip(np.rint(out), 0, 255).astype(np.uint8)


def _resample(img: np.ndarray, yy: np.ndarray, xx: np.ndarray) -> np.ndarray:
    out = np.empty(img.shape, np.float64)
    for c in range(img.shape[2]):
        out[:, :, c] = ndimage.map_coordinates(img[:, :, c].astype(np.float64), [yy, xx], order=1,
                                               mode="reflect")
    return out


def _add_noise(img: np.ndarray, sigma: float, rng: np.random.Generator) -> np.ndarray:
    if sigma > 0:
        img = img + rng.normal(0.0, sigma, img.shape)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def affine_warp(a: np.ndarray, shift_xy, angle_deg: float, noise_sigma: float,
                rng: np.random.Generator) -> np.ndarray:
    """B = A shifted by shift_xy=(dx, dy) pixels, then rotated by angle_deg about the centre."""
    h, w = a.shape[:2]
    cy, cx = (h - 1) / 2.0, (w - 1) / 2.0
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    th = np.deg2rad(angle_deg)
    # inverse map: output p -> rotate back by -th about the centre -> undo the shift
    ry = (yy - cy) * np.cos(th) - (xx - cx) * np.sin(th) + cy
    rx = (yy - cy) * np.sin(th) + (xx - cx) * np.cos(th) + cx
    src_y = ry - shift_xy[1]
    src_x = rx - shift_xy[0]
    return _add_noise(_resample(a, src_y, src_x), noise_sigma, rng)


def smooth_flow(h: int, w: int, magnitude: float, sigma: float, rng: np.random.Generator):
    fl = []
    for _ in range(2):
        u = ndimage.gaussian_filter(rng.normal(0.0, magnitude, (h, w)), sigma, mode="wrap")
        s = u.std()
        fl.append(u * (magnitude / s) if s > 0 else u)
    return fl[0], fl[1]


def flow_warp(a: np.ndarray, magnitude: float, sigma: float, noise_sigma: float,
              rng: np.random.Generator) -> np.ndarray:
    h, w = a.shape[:2]
    uy, ux = smooth_flow(h, w, magnitude, sigma, rng)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    return _add_noise(_resample(a, yy + uy, xx + ux), noise_sigma, rng)


# --------------------------------------------------------------------------------------------
# the benchmark workloads
# --------------------------------------------------------------------------------------------
def pair_small(seed: int = 0, size: int = 512):
    """512x512 pair: spectral noise; B = A shifted by (13, -7), rotated 15 deg, N(0,4^2) noise."""
    rng = np.random.default_rng(seed)
    a = spectral_noise(size, size, rng)
    b = affine_warp(a, (13.0, -7.0), 15.0, 4.0, rng)
    return a, b


def pair_flow(seed: int = 1, size: int = 2048, magnitude: float = 20.0, sigma: float = 64.0,
              noise: float = 4.0, height: int | None = None):
    """Flow-warped pair (2048x2048 seed 1 is the large-pair workload; 1024x1024 seeds 1000+ are
    the proposal-network training pairs)."""
    rng = np.random.default_rng(seed)
    h = size if height is None else height
    a = spectral_noise(h, size, rng)
    b = flow_warp(a, magnitude, sigma, noise, rng)
    return a, b


def pairs_uneven(seed: int = 2, count: int = 64, lo: int = 256, hi: int = 1536):
    """Uneven pairs: side ~ U(lo, hi) (height), aspect ~ U(0.5, 2) (width = round(side*aspect)),
    random affine warp (rotation U(-20, 20) deg, translation U(-40, 40) px, N(0,4^2) noise)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        side = int(rng.integers(lo, hi + 1))
        aspect = float(rng.uniform(0.5, 2.0))
        h, w = side, max(16, int(round(side * aspect)))
        a = spectral_noise(h, w, rng)
        b = affine_warp(a, (float(rng.uniform(-40, 40)), float(rng.uniform(-40, 40))),
                        float(rng.uniform(-20, 20)), 4.0, rng)
        out.append((a, b))
    return out


def frame_stream(seed: int = 3, frames: int = 120, h: int = 1080, w: int = 1920):
    """Frame sequence: each frame is the previous one warped by a smooth random flow
    (sigma 96 px, magnitude N(0, 6^2)) plus N(0, 3^2) noise, starting from spectral noise."""
    rng = np.random.default_rng(seed)
    f = spectral_noise(h, w, rng)
    out = [f]
    for _ in range(frames - 1):
        f = flow_warp(f, 6.0, 96.0, 3.0, rng)
        out.append(f)
    return out


# --------------------------------------------------------------------------------------------
# the same recipes on the GPU (torch FFT and bilinear sampling; torch's RNG, so not bit-equal to
# the numpy versions above) for workloads too large to synthesise on the host in a benchmark run
# --------------------------------------------------------------------------------------------
def _gpu_spectral(h, w, g, dev):
    import torch
    fy = torch.fft.fftfreq(h, device=dev)[:, None]
    fx = torch.fft.rfftfreq(w, device=dev)[None, :]
    f2 = fx * fx + fy * fy
    amp = torch.where(f2 > 0, 1.0 / torch.sqrt(torch.where(f2 > 0, f2, torch.ones_like(f2))), torch.zeros_like(f2))
    img = torch.fft.irfft2(torch.fft.rfft2(torch.randn((3, h, w), generator=g, device=dev)) * amp, s=(h, w))
    lo, hi = img.min(), img.max()
    return torch.clamp(torch.round((img - lo) * (255.0 / torch.clamp(hi - lo, min=1e-12))), 0, 255)


def _gpu_flow_warp(a, magnitude, sigma, noise, g):
    import math

    import torch
    dev = a.device
    _, h, w = a.shape
    fy = torch.fft.fftfreq(h, device=dev)[:, None]
    fx = torch.fft.rfftfreq(w, device=dev)[None, :]
    gk = torch.exp(-2.0 * (math.pi ** 2) * sigma * sigma * (fx * fx + fy * fy))
    u = torch.randn((2, h, w), generator=g, device=dev) * magnitude
    u = torch.fft.irfft2(torch.fft.rfft2(u) * gk, s=(h, w))
    u = u * (magnitude / torch.clamp(u.std(dim=(1, 2), keepdim=True), min=1e-12))
    yy, xx = torch.meshgrid(torch.arange(h, device=dev, dtype=torch.float32),
                            torch.arange(w, device=dev, dtype=torch.float32), indexing="ij")
    grid = torch.stack([(xx + u[1]) / (w - 1) * 2 - 1, (yy + u[0]) / (h - 1) * 2 - 1], dim=-1)[None]
    warped = torch.nn.functional.grid_sample(a[None], grid, mode="bilinear", padding_mode="reflection",
                                             align_corners=True)[0]
    return torch.clamp(torch.round(warped + noise * torch.randn(warped.shape, generator=g, device=dev)), 0, 255)


def gpu_frame_stream(seed: int = 3, frames: int = 120, h: int = 1080, w: int = 1920, device=0):
    """frame_stream's recipe on the GPU: a list of uint8 (h, w, 3) CUDA tensors."""
    import torch
    dev = torch.device("cuda", device) if isinstance(device, int) else torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    f = _gpu_spectral(h, w, g, dev)
    out = [f]
    for _ in range(frames - 1):
        f = _gpu_flow_warp(f, 6.0, 96.0, 3.0, g)
        out.append(f)
    return [x.permute(1, 2, 0).contiguous().to(torch.uint8) for x in out]


def gpu_pairs_uneven(seed: int = 2, count: int = 64, lo: int = 256, hi: int = 1536, device=0):
    """pairs_uneven's recipe with the image synthesis on the GPU (sizes and affine parameters from
    the same numpy RNG draws): [(A, B)] uint8 CUDA tensors."""
    import math

    import torch
    dev = torch.device("cuda", device) if isinstance(device, int) else torch.device(device)
    rng = np.random.default_rng(seed)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    out = []
    for _ in range(count):
        side = int(rng.integers(lo, hi + 1))
        aspect = float(rng.uniform(0.5, 2.0))
        h, w = side, max(16, int(round(side * aspect)))
        dx, dy, ang = float(rng.uniform(-40, 40)), float(rng.uniform(-40, 40)), float(rng.uniform(-20, 20))
        a = _gpu_spectral(h, w, g, dev)
        cy, cx = (h - 1) / 2.0, (w - 1) / 2.0
        th = math.radians(ang)
        yy, xx = torch.meshgrid(torch.arange(h, device=dev, dtype=torch.float32),
                                torch.arange(w, device=dev, dtype=torch.float32), indexing="ij")
        ry = (yy - cy) * math.cos(th) - (xx - cx) * math.sin(th) + cy - dy
        rx = (yy - cy) * math.sin(th) + (xx - cx) * math.cos(th) + cx - dx
        grid = torch.stack([rx / (w - 1) * 2 - 1, ry / (h - 1) * 2 - 1], dim=-1)[None]
        warped = torch.nn.functional.grid_sample(a[None], grid, mode="bilinear", padding_mode="reflection",
                                                 align_corners=True)[0]
        b = torch.clamp(torch.round(warped + 4.0 * torch.randn(warped.shape, generator=g, device=dev)), 0, 255)
        out.append((a.permute(1, 2, 0).contiguous().to(torch.uint8), b.permute(1, 2, 0).contiguous().to(torch.uint8)))
    return out
