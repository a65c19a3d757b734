"""Seeded synthetic image stacks for tests and benchmarks.

Scene: ``n_spots`` Gaussian spots (width ``sigma`` px, peak ``amplitude``) at
uniform random positions, moving by 2D Brownian steps N(0, sqrt(2 D)) per axis
per frame plus a uniform ``drift`` (px/frame), rendered with periodic
(minimum-image) distances on top of ``offset``; every pixel is then a Poisson
draw of its intensity, clipped to the range of ``dtype``.

The rendering is separable: frame = offset + amplitude * Gy^T Gx with
Gx[s, x] = exp(-dx^2 / 2 sigma^2), Gy[s, y] likewise, i.e. one
(H x S) @ (S x W) product per frame.  ``make_stack`` renders on the CPU with
numpy; ``make_stack_torch`` renders on a CUDA device for large stacks.  The two
draw different random numbers; each is deterministic for a given seed.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np


@dataclass(frozen=True)
class Scene:
    length: int
    height: int
    width: int
    n_spots: int
    sigma: float
    amplitude: float
    diffusivity: float
    offset: float
    drift: float = 0.0
    dtype: str = "uint16"
    seed: int = 0


# the configurations of the benchmark suite
CONFIG1 = Scene(64, 128, 128, 200, 2.0, 2000.0, 0.5, 500.0, 0.0, "uint16", 0)
CONFIG2 = Scene(512, 512, 512, 2000, 2.0, 2000.0, 0.2, 500.0, 0.0, "uint16", 0)
# 8-bit large stack: offset and amplitude chosen for the 0..255 range
CONFIG3 = Scene(4000, 1024, 1024, 5000, 1.5, 150.0, 1.0, 20.0, 0.05, "uint8", 0)
# small cases with the kernel configurations of CONFIG3, for profiling:
# the temporal stage (4000 frames, same lags) and the spatial stage (1024 x 1024 frames)
CONFIG3_TALL = Scene(4000, 64, 64, 20, 1.5, 150.0, 1.0, 20.0, 0.05, "uint8", 0)
CONFIG3_WIDE = Scene(64, 1024, 1024, 5000, 1.5, 150.0, 1.0, 20.0, 0.05, "uint8", 0)
# a long series: 20000 frames of 256 x 256 (the split temporal transform, N = 40960)
CONFIG_LONG = Scene(20000, 256, 256, 300, 1.5, 150.0, 1.0, 20.0, 0.05, "uint8", 0)


def _periodic_profile(pos: np.ndarray, n: int, sigma: float) -> np.ndarray:
    grid = np.arange(n, dtype=np.float64)
    d = grid[None, :] - pos[:, None]
    d -= n * np.round(d / n)
    return np.exp(-(d * d) / (2.0 * sigma * sigma))


def make_stack(scene: Scene) -> np.ndarray:
    """Render the stack on the CPU (numpy); shape (length, height, width)."""
    rng = np.random.default_rng(scene.seed)
    T, H, W, S = scene.length, scene.height, scene.width, scene.n_spots
    x = rng.uniform(0, W, S)
    y = rng.uniform(0, H, S)
    step = np.sqrt(2.0 * scene.diffusivity)
    info = np.iinfo(scene.dtype) if np.dtype(scene.dtype).kind in "ui" else None
    out = np.empty((T, H, W), dtype=scene.dtype)
    for t in range(T):
        gx = _periodic_profile(x, W, scene.sigma)
        gy = _periodic_profile(y, H, scene.sigma)
        inten = scene.offset + scene.amplitude * (gy.T @ gx)
        frame = rng.poisson(inten)
        if info is not None:
            frame = np.clip(frame, info.min, info.max)
        out[t] = frame
        x = np.mod(x + rng.normal(0.0, step, S) + scene.drift, W)
        y = np.mod(y + rng.normal(0.0, step, S) + scene.drift, H)
    return out


def make_stack_torch(scene: Scene, device="cuda", batch: int = 32, length: Optional[int] = None):
    """Render the stack on a CUDA device with torch; returns a device tensor."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(scene.seed)
    T = scene.length if length is None else length
    H, W, S = scene.height, scene.width, scene.n_spots
    f64 = torch.float64
    x0 = torch.rand(S, generator=g, device=device, dtype=f64) * W
    y0 = torch.rand(S, generator=g, device=device, dtype=f64) * H
    step = float(np.sqrt(2.0 * scene.diffusivity))
    tdtype = {"uint8": torch.uint8, "uint16": getattr(torch, "uint16", torch.int32), "int16": torch.int16}[scene.dtype]
    hi = float(np.iinfo(scene.dtype).max)
    out = torch.empty((T, H, W), dtype=tdtype, device=device)
    gxs = torch.arange(W, device=device, dtype=f64)
    gys = torch.arange(H, device=device, dtype=f64)

    def prof(pos, grid, n):
        d = grid[None, None, :] - pos[:, :, None]
        d = d - n * torch.round(d / n)
        return torch.exp(-(d * d) / (2.0 * scene.sigma ** 2)).to(torch.float32)

    for t0 in range(0, T, batch):
        nb = min(batch, T - t0)
        # Brownian steps with drift; frame i of the batch sits after i steps
        sx = torch.randn((nb, S), generator=g, device=device, dtype=f64) * step + scene.drift
        sy = torch.randn((nb, S), generator=g, device=device, dtype=f64) * step + scene.drift
        cx = torch.cumsum(sx, dim=0)
        cy = torch.cumsum(sy, dim=0)
        xs = torch.remainder(x0[None] + torch.cat([torch.zeros_like(cx[:1]), cx[:-1]]), W)
        ys = torch.remainder(y0[None] + torch.cat([torch.zeros_like(cy[:1]), cy[:-1]]), H)
        x0 = torch.remainder(x0 + cx[-1], W)
        y0 = torch.remainder(y0 + cy[-1], H)
        inten = scene.offset + scene.amplitude * torch.bmm(prof(ys, gys, H).transpose(1, 2), prof(xs, gxs, W))
        frame = torch.poisson(inten, generator=g).clamp_(0, hi)
        out[t0:t0 + nb] = frame.to(torch.int32).to(tdtype)
    return out


def config4_scenes(n_stacks: int = 96, seed: int = 0):
    """Uneven ROI stacks: side from {64, 96, 128, 192, 256, 384, 512}, T uniform in [100, 2000],
    diffusivity log-uniform in [0.05, 2] px^2/frame, uint16, one spot per ~82 px^2
    (the density of the 64-frame configuration), spot width 2 px, amplitude 2000 on 500."""
    rng = np.random.default_rng(seed)
    sides = [64, 96, 128, 192, 256, 384, 512]
    out = []
    for i in range(n_stacks):
        side = int(rng.choice(sides))
        T = int(rng.integers(100, 2001))
        D = float(np.exp(rng.uniform(np.log(0.05), np.log(2.0))))
        out.append(Scene(T, side, side, max(1, side * side // 82), 2.0, 2000.0, D, 500.0, 0.0, "uint16", seed + i))
    return out
