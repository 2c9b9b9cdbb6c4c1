"""Seeded synthetic Poisson phantoms for the benchmark workloads and the tests.

No public dataset is used by BMND for its Poisson path; these generators stand
in for real count data with the shapes, sizes and value ranges of the
published workloads:

* :func:`shapes_2d` -- background of 5 counts plus 12 random axis-aligned
  rectangles and discs with intensities uniform in [5, 50] counts (256x256 by
  default, smaller sizes scale the shape extents).
* :func:`blobs_2d` -- a sum of 40 Gaussian blobs (sigma uniform 10-80 px) and
  60 rectangles, rescaled so that the peak is log-uniform in [1, 100] counts
  (2048x2048 by default).
* :func:`ellipsoids_3d` -- background of 2 counts plus 30 random ellipsoids
  (semi-axes 10-80 voxels, intensities uniform 5-30 counts), 256^3 by default.
  Passing ``peak`` rescales the clean volume so its maximum equals ``peak``.

Every generator returns ``(clean, noisy)`` as float32 arrays, where
``noisy = np.random.default_rng(seed).poisson(clean)``.  The free choices the
workload descriptions leave open (shape extents, placement, overwrite order)
are fixed here so that a seed determines the volume exactly.
"""

from __future__ import annotations

import numpy as np

__all__ = ["shapes_2d", "blobs_2d", "ellipsoids_3d", "poisson_noise", "psnr"]


def poisson_noise(clean: np.ndarray, seed: int) -> np.ndarray:
    """Poisson counts drawn with ``default_rng(seed).poisson(clean)``."""
    rng = np.random.default_rng(seed)
    return rng.poisson(np.maximum(clean, 0.0)).astype(np.float32)


def shapes_2d(size: int = 256, seed: int = 0, count: int = 12):
    """Background 5 counts + ``count`` rectangles/discs with intensity U[5, 50]."""
    rng = np.random.default_rng(seed)
    clean = np.full((size, size), 5.0, dtype=np.float64)
    yy, xx = np.mgrid[0:size, 0:size]
    scale = size / 256.0
    for _ in range(count):
        intensity = rng.uniform(5.0, 50.0)
        cy, cx = rng.uniform(0, size, size=2)
        if rng.random() < 0.5:
            hy, hx = rng.uniform(8.0, 48.0, size=2) * scale
            mask = (np.abs(yy - cy) <= hy) & (np.abs(xx - cx) <= hx)
        else:
            radius = rng.uniform(6.0, 40.0) * scale
            mask = (yy - cy) ** 2 + (xx - cx) ** 2 <= radius * radius
        clean[mask] = intensity
    clean = clean.astype(np.float32)
    return clean, poisson_noise(clean, seed)


def blobs_2d(size: int = 2048, seed: int = 0, n_blobs: int = 40, n_rects: int = 60):
    """Gaussian blobs plus rectangles, peak log-uniform in [1, 100] counts."""
    rng = np.random.default_rng(seed)
    clean = np.zeros((size, size), dtype=np.float64)
    coords = np.arange(size, dtype=np.float64)
    scale = size / 2048.0
    for _ in range(n_blobs):
        cy, cx = rng.uniform(0, size, size=2)
        sigma = rng.uniform(10.0, 80.0) * scale
        amp = rng.uniform(0.2, 1.0)
        gy = np.exp(-0.5 * ((coords - cy) / sigma) ** 2)
        gx = np.exp(-0.5 * ((coords - cx) / sigma) ** 2)
        clean += amp * np.outer(gy, gx)
    for _ in range(n_rects):
        cy, cx = rng.uniform(0, size, size=2)
        hy, hx = rng.uniform(4.0, 96.0, size=2) * scale
        amp = rng.uniform(0.1, 0.6)
        y0, y1 = int(max(cy - hy, 0)), int(min(cy + hy, size))
        x0, x1 = int(max(cx - hx, 0)), int(min(cx + hx, size))
        clean[y0:y1, x0:x1] += amp
    peak = float(np.exp(rng.uniform(np.log(1.0), np.log(100.0))))
    clean *= peak / max(float(clean.max()), 1e-12)
    clean = clean.astype(np.float32)
    return clean, poisson_noise(clean, seed)


def blobs_2d_window(size: int = 256, seed: int = 0, full: int = 2048, n_blobs: int = 40, n_rects: int = 60):
    """A ``size`` x ``size`` window of a ``full`` x ``full`` phantom of the
    ``blobs_2d`` kind (the same object sizes and counts), at a random offset,
    scaled so that the window's peak is log-uniform in [1, 100] counts.  Only
    the window is evaluated, so thousands of them are cheap."""
    rng = np.random.default_rng(seed)
    oy, ox = rng.integers(0, full - size + 1, size=2)
    ys = np.arange(oy, oy + size, dtype=np.float64)
    xs = np.arange(ox, ox + size, dtype=np.float64)
    clean = np.zeros((size, size), dtype=np.float64)
    for _ in range(n_blobs):
        cy, cx = rng.uniform(0, full, size=2)
        sigma = rng.uniform(10.0, 80.0)
        amp = rng.uniform(0.2, 1.0)
        clean += amp * np.outer(np.exp(-0.5 * ((ys - cy) / sigma) ** 2), np.exp(-0.5 * ((xs - cx) / sigma) ** 2))
    for _ in range(n_rects):
        cy, cx = rng.uniform(0, full, size=2)
        hy, hx = rng.uniform(4.0, 96.0, size=2)
        amp = rng.uniform(0.1, 0.6)
        y0, y1 = int(max(cy - hy - oy, 0)), int(min(cy + hy - oy, size))
        x0, x1 = int(max(cx - hx - ox, 0)), int(min(cx + hx - ox, size))
        if y1 > y0 and x1 > x0:
            clean[y0:y1, x0:x1] += amp
    clean += 1e-3  # a window that misses every object is a flat low-count field
    peak = float(np.exp(rng.uniform(np.log(1.0), np.log(100.0))))
    clean *= peak / float(clean.max())
    clean = clean.astype(np.float32)
    return clean, poisson_noise(clean, seed)


def ellipsoids_3d(
    size: int | tuple[int, int, int] = 256,
    seed: int = 0,
    count: int = 30,
    peak: float | None = None,
):
    """Background 2 counts + ``count`` ellipsoids, semi-axes U[10, 80], intensity U[5, 30]."""
    shape = (size, size, size) if isinstance(size, int) else tuple(int(s) for s in size)
    rng = np.random.default_rng(seed)
    clean = np.full(shape, 2.0, dtype=np.float32)
    scale = min(shape) / 256.0
    axes = [np.arange(n, dtype=np.float32) for n in shape]
    for _ in range(count):
        center = np.array([rng.uniform(0, n) for n in shape], dtype=np.float32)
        semi = rng.uniform(10.0, 80.0, size=3).astype(np.float32) * np.float32(scale)
        semi = np.maximum(semi, 1.5)
        intensity = np.float32(rng.uniform(5.0, 30.0))
        lo = [int(max(np.floor(center[d] - semi[d]), 0)) for d in range(3)]
        hi = [int(min(np.ceil(center[d] + semi[d]) + 1, shape[d])) for d in range(3)]
        if any(h <= l for l, h in zip(lo, hi)):
            continue
        dz = ((axes[0][lo[0]:hi[0]] - center[0]) / semi[0]) ** 2
        dy = ((axes[1][lo[1]:hi[1]] - center[1]) / semi[1]) ** 2
        dx = ((axes[2][lo[2]:hi[2]] - center[2]) / semi[2]) ** 2
        inside = (dz[:, None, None] + dy[None, :, None] + dx[None, None, :]) <= 1.0
        region = clean[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        region[inside] = intensity
    if peak is not None:
        clean *= np.float32(peak) / max(float(clean.max()), 1e-12)
    return clean, poisson_noise(clean, seed)


def psnr(estimate: np.ndarray, clean: np.ndarray, data_range: float | None = None) -> float:
    """Peak signal-to-noise ratio in dB (peak = ``data_range`` or ``clean.max()``)."""
    estimate = np.asarray(estimate, dtype=np.float64)
    clean = np.asarray(clean, dtype=np.float64)
    peak = float(clean.max()) if data_range is None else float(data_range)
    mse = float(np.mean((estimate - clean) ** 2))
    if mse <= 0.0:
        return float("inf")
    return 10.0 * np.log10(peak * peak / mse)
