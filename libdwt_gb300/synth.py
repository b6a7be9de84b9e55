"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark workloads (the reference ships no data sets).

image(w, h, seed): a smooth field -- the sum of 64 Gaussian blobs with centres
uniform in the image, sigma uniform in [8, 128] px and amplitudes uniform in
[-1, 1], rescaled to span [0, 255] -- plus N(0, 4) noise, clipped to [0, 255],
rounded to integers and stored as float32.  Each blob is separable, so the
field is a (h x 64) @ (64 x w) product and generation is fast at 16384^2.

ar1_bank(groups, n, lanes, seed): AR(1) signals (rho = 0.95, unit Gaussian
innovations, x0 = 0) laid out as groups x n x lanes float32, i.e. `lanes`
signals interleaved per group with an element stride of lanes * 4 bytes.
"""
from __future__ import annotations

import numpy as np


def image(w: int, h: int, seed: int = 0, blobs: int = 64) -> np.ndarray:
    rng = np.random.default_rng(seed)
    cx = rng.uniform(0, w, blobs)
    cy = rng.uniform(0, h, blobs)
    sig = rng.uniform(8, 128, blobs)
    amp = rng.uniform(-1, 1, blobs)
    xs = np.arange(w, dtype=np.float64)
    ys = np.arange(h, dtype=np.float64)
    gx = np.exp(-((xs[None, :] - cx[:, None]) ** 2) / (2 * sig[:, None] ** 2))  # blobs x w
    gy = np.exp(-((ys[:, None] - cy[None, :]) ** 2) / (2 * sig[None, :] ** 2))  # h x blobs
    field = (gy * amp[None, :]).astype(np.float32) @ gx.astype(np.float32)
    lo, hi = float(field.min()), float(field.max())
    scale = 255.0 / (hi - lo) if hi > lo else 0.0
    field -= lo
    field *= scale
    # noise in row blocks to bound the temporary memory
    block = max(1, (1 << 24) // max(w, 1))
    for y0 in range(0, h, block):
        y1 = min(h, y0 + block)
        field[y0:y1] += rng.standard_normal((y1 - y0, w), dtype=np.float32) * 2.0
    np.clip(field, 0, 255, out=field)
    np.rint(field, out=field)
    return field


def ar1_bank(groups: int, n: int, lanes: int, seed: int = 0, rho: float = 0.95) -> np.ndarray:
    rng = np.random.default_rng(seed)
    eps = rng.standard_normal((groups, n, lanes), dtype=np.float32)
    x = np.empty_like(eps)
    prev = np.zeros((groups, lanes), np.float32)
    x[:, 0, :] = prev
    for i in range(1, n):
        prev = prev * np.float32(rho) + eps[:, i, :]
        x[:, i, :] = prev
    return x


def image_torch(w: int, h: int, seed: int = 0, blobs: int = 64, device: str = "cuda"):
    """The recipe of image() on the GPU with torch (same distribution; values
    are not bit-identical to the numpy version)."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    cx = torch.rand(blobs, generator=g, dtype=torch.float64) * w
    cy = torch.rand(blobs, generator=g, dtype=torch.float64) * h
    sig = 8 + torch.rand(blobs, generator=g, dtype=torch.float64) * 120
    amp = torch.rand(blobs, generator=g, dtype=torch.float64) * 2 - 1
    xs = torch.arange(w, dtype=torch.float64)
    ys = torch.arange(h, dtype=torch.float64)
    gx = torch.exp(-((xs[None, :] - cx[:, None]) ** 2) / (2 * sig[:, None] ** 2)).float().to(device)
    gy = (torch.exp(-((ys[:, None] - cy[None, :]) ** 2) / (2 * sig[None, :] ** 2)) * amp[None, :]).float().to(device)
    field = gy @ gx
    lo, hi = field.min(), field.max()
    field = (field - lo) * (255.0 / torch.clamp(hi - lo, min=1e-20))
    gn = torch.Generator(device=device).manual_seed(seed + 1)
    field += torch.randn(field.shape, generator=gn, device=device) * 2.0
    return torch.round(torch.clamp(field, 0, 255))


def batch_sizes(n: int, lo: int = 33, hi: int = 2048, seed: int = 0):
    """n (w, h) pairs, each side log-uniform in [lo, hi], and a wavelet per
    image (0 = CDF 9/7, 1 = CDF 5/3, 50/50)."""
    rng = np.random.default_rng(seed)
    w = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), n))).astype(int)
    h = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), n))).astype(int)
    wav = rng.integers(0, 2, n)
    return list(zip(w.tolist(), h.tolist(), wav.tolist()))
