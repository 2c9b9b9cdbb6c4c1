"""Stationary Gaussian noise: the host-side model behind ``noise_model="gaussian"``.

Restates the reference's PSD handling and the tables its Gaussian path
derives from it, so the GPU kernels receive the same numbers:

* ``resolve_nf``                 -- psd.py:57-98
* ``estimate_global_sigma``      -- sigmaestimation.py:7-45
* ``normalize_sigma_psd``        -- psd.py:100-131 (scalar sigma -> flat PSD)
* ``preprocess_psd``             -- psd.py:154-261 (reduction and blur on the nf grid)
* ``autocovariance_from_psd``    -- psd.py:134-139
* ``GaussianModel``              -- variance.py:452-504 (build_variance_model)
* ``covariance_maps``            -- variance.py:1791-1886: for every spatial
  coefficient c, the covariance of coefficient c between two patches as a
  function of their offset on the periodic nf domain
* ``blockmatch_noise_ssd``       -- variance.py:507-553: the SSD noise bias per
  search offset that HT matching subtracts (times gamma)

Everything here runs once per call on small arrays (the nf domain, the search
window); the per-group work is in ``csrc/groupfilter.cu``.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def resolve_nf(nf, shape: tuple[int, ...]):
    """(domain, conventional): the per-axis local-variance domain (psd.py:57-98)."""
    if nf is None:
        return None, False
    if isinstance(nf, bool):
        raise ValueError(f"nf must be a per-axis integer tuple or zero, got {nf!r}.")
    if isinstance(nf, (int, np.integer)):
        if int(nf) == 0:
            return tuple(min(int(s), 16) for s in shape), True
        raise ValueError(f"nf must be zero or contain one positive integer per volume axis, got {nf!r}.")
    try:
        values = tuple(nf)
    except TypeError as exc:
        raise ValueError(f"nf must be zero or contain one positive integer per volume axis, got {nf!r}.") from exc
    if not values:
        return None, False
    if len(values) != len(shape):
        raise ValueError(f"nf must contain {len(shape)} values for shape {shape}, got {values}.")
    if any(isinstance(v, bool) or not isinstance(v, (int, np.integer)) for v in values):
        raise ValueError(f"nf values must be integers, got {values}.")
    resolved = tuple(int(v) for v in values)
    if any(v < 0 for v in resolved):
        raise ValueError(f"nf values must be non-negative, got {resolved}.")
    if any(v == 0 for v in resolved):
        return tuple(min(int(s), 16) for s in shape), True
    return resolved, False


def estimate_global_sigma(volume, eps: float = 1e-10) -> float:
    """Robust sigma of the values: MAD / 0.6745, then IQR / 1.349, then a
    trimmed standard deviation, then sqrt(eps) (sigmaestimation.py:7-45)."""
    vol = np.asarray(volume, dtype=np.float32)
    finite = np.isfinite(vol)
    nonzero = finite & (vol != 0.0)
    if np.any(nonzero):
        ref = vol[nonzero]
    elif np.any(finite):
        ref = vol[finite]
    else:
        ref = np.array([0.0], dtype=np.float32)
    med = np.median(ref)
    sigma = float(np.median(np.abs(ref - med))) / 0.6745
    if sigma <= 0.0:
        q25, q75 = np.percentile(ref, [25.0, 75.0])
        iqr = float(q75 - q25)
        if iqr > 0.0:
            sigma = iqr / 1.349
    if sigma <= 0.0:
        p5, p95 = np.percentile(ref, [5.0, 95.0])
        trimmed = ref[(ref >= p5) & (ref <= p95)]
        if trimmed.size > 0:
            st = float(np.std(trimmed, dtype=np.float32))
            if st > 0.0:
                sigma = st
    if sigma <= 0.0:
        sigma = float(np.sqrt(eps))
    if not np.isfinite(sigma) or sigma < 0.0:
        return 0.0
    return sigma


def validate_sigma(sigma) -> float:
    if isinstance(sigma, (bool, np.bool_)):
        raise ValueError(f"sigma must be finite and non-negative, got {sigma!r}.")
    try:
        value = float(sigma)
    except (TypeError, ValueError) as exc:
        raise ValueError(f"sigma must be finite and non-negative, got {sigma!r}.") from exc
    if not np.isfinite(value) or value < 0.0:
        raise ValueError(f"sigma must be finite and non-negative, got {sigma!r}.")
    return value


def validate_sigma_psd(shape: tuple[int, ...], sigma_psd) -> np.ndarray:
    try:
        with np.errstate(over="ignore", invalid="ignore"):
            arr = np.asarray(sigma_psd, dtype=np.float32)
    except (TypeError, ValueError) as exc:
        raise ValueError("sigma_psd must contain only finite non-negative values.") from exc
    if not np.all(np.isfinite(arr)) or np.any(arr < 0.0):
        raise ValueError("sigma_psd must contain only finite non-negative values.")
    if arr.ndim != 0 and arr.size != 1 and arr.shape != shape:
        raise ValueError("sigma_psd must either be scalar or have the same shape as volume")
    return arr


def _scalar_psd(shape: tuple[int, ...], sigma: float) -> np.ndarray:
    s = validate_sigma(sigma)
    value = float(np.prod(shape)) * s * s
    if not np.isfinite(value) or value > np.finfo(np.float32).max:
        raise ValueError(f"sigma is too large for a float32 PSD, got {sigma!r}.")
    return np.full(shape, value, dtype=np.float32)


def normalize_sigma_psd(shape, sigma=None, sigma_psd=None):
    if sigma is not None and sigma_psd is not None:
        raise ValueError("sigma and sigma_psd are mutually exclusive.")
    if sigma is None and sigma_psd is None:
        return None
    if sigma_psd is None:
        return _scalar_psd(shape, sigma)
    arr = validate_sigma_psd(shape, sigma_psd)
    if arr.ndim == 0 or arr.size == 1:
        return _scalar_psd(shape, float(np.asarray(arr).reshape(())))
    return arr.astype(np.float32, copy=False)


def _gaussian_kernel(size, sigma_scale) -> np.ndarray:
    axes = []
    for n, sg in zip(size, sigma_scale):
        center = (n - 1) / 2.0
        coords = np.arange(n, dtype=np.float32) - center
        safe = max(float(sg), 1e-6)
        ax = np.exp(-0.5 * (coords / safe) ** 2)
        ax /= np.sum(ax, dtype=np.float32)
        axes.append(ax.astype(np.float32))
    k = axes[0]
    for ax in axes[1:]:
        k = np.multiply.outer(k, ax)
    k = k.astype(np.float32, copy=False)
    k /= np.sum(k, dtype=np.float32)
    return k


def _reduce_and_blur(psd: np.ndarray, nf):
    """(reduced, blurred) PSD on the nf grid (psd.py:199-247): each axis is
    folded by three-tap averages with period 3 while it is more than 16 times
    nf, rescaled, then blurred by a Gaussian of half-width size / (2 nf)."""
    from scipy.ndimage import correlate

    psd = np.array(psd, dtype=np.float32, copy=True)
    if nf is None:
        return psd, psd.copy()
    reduced = psd.copy()
    for axis in range(psd.ndim):
        kshape = [1] * psd.ndim
        kshape[axis] = 3
        k3 = np.ones(tuple(kshape), dtype=np.float32) / np.float32(3.0)
        original_ratio = psd.shape[axis] / float(nf[axis])
        ratio = reduced.shape[axis] / float(nf[axis])
        while ratio > 16.0:
            mid = correlate(reduced, k3, mode="wrap")
            sl = [slice(None)] * psd.ndim
            sl[axis] = slice(1, None, 3)
            reduced = mid[tuple(sl)]
            ratio = reduced.shape[axis] / float(nf[axis])
        reduced *= np.float32(ratio / original_ratio)
    sizes, sigmas = [], []
    for axis in range(reduced.ndim):
        half = np.floor(0.5 * reduced.shape[axis] / nf[axis])
        sizes.append(int(1 + 2 * half))
        sigmas.append(float(1 + 2 * half / 20.0))
    blur = _gaussian_kernel(tuple(sizes), tuple(sigmas))
    blurred = correlate(reduced, blur, mode="wrap").astype(np.float32, copy=False)
    return reduced.astype(np.float32, copy=False), blurred


def autocovariance_from_psd(psd) -> np.ndarray:
    p = np.asarray(psd, dtype=np.float32)
    return np.real(np.fft.ifftn(p) / float(p.size)).astype(np.float32, copy=False)


@dataclass
class GaussianModel:
    """Stationary Gaussian noise of one call (variance.py:452-504)."""

    global_sigma: float
    processed_psd: np.ndarray  # blurred PSD (full volume shape for scalar input)
    autocovariance: np.ndarray
    domain: tuple[int, ...]  # lag domain of the covariance maps
    conventional: bool
    _maps: dict = field(default_factory=dict, repr=False)
    _ssd: dict = field(default_factory=dict, repr=False)


def white_variance(model: GaussianModel) -> float | None:
    """The noise variance when the noise is white, else None
    (variance.py:1459-1470): white means no autocovariance lag but 0 above
    max(1e-12, 1e-6 x the lag-0 variance)."""
    ac = np.asarray(model.autocovariance, dtype=np.float64)
    var0 = float(ac.reshape(-1)[0])
    tol = max(1e-12, 1e-6 * max(var0, 0.0))
    if np.any(np.abs(ac.reshape(-1)[1:]) > tol):
        return None
    return max(var0, 0.0)


def build_model(volume_shape: tuple[int, ...], nf, *, sigma=None, sigma_psd=None, volume=None) -> GaussianModel:
    """The noise model for ``bmnd(volume, profile, sigma=..., sigma_psd=...)``;
    with neither given, sigma is estimated from ``volume``."""
    shape = tuple(int(s) for s in volume_shape)
    if sigma is None and sigma_psd is None:
        sigma = estimate_global_sigma(volume)
    resolved_nf, conventional = resolve_nf(nf, shape)
    psd = normalize_sigma_psd(shape, sigma=sigma, sigma_psd=sigma_psd)
    if sigma is not None:
        scalar = True
    else:
        arr = np.asarray(sigma_psd)
        scalar = arr.ndim == 0 or arr.size == 1
    _, blurred = _reduce_and_blur(psd, None if scalar else resolved_nf)
    size = float(np.prod(shape))
    global_sigma = float(np.sqrt(max(float(np.mean(psd, dtype=np.float32)) / size, 0.0)))
    domain = tuple(int(s) for s in blurred.shape) if resolved_nf is None else tuple(resolved_nf)
    return GaussianModel(max(global_sigma, 0.0), blurred, autocovariance_from_psd(blurred), domain, conventional)


def _separable_matrix(block, spatial_fwd) -> np.ndarray:
    full = np.array([[1.0]], dtype=np.float32)
    for n, m in zip(block, spatial_fwd):
        mat = np.eye(n, dtype=np.float32) if m is None else np.asarray(m, dtype=np.float32)
        full = np.kron(full, mat).astype(np.float32, copy=False)
    return full


def covariance_maps(model: GaussianModel, block: tuple[int, ...], spatial_fwd) -> np.ndarray:
    """[P, *domain] float32: the PSD resampled to the domain (linear, periodic),
    each coefficient's basis folded onto the domain, its power spectrum times
    the PSD transformed back, symmetrised in the lag (variance.py:1791-1886)."""
    key = (tuple(block), tuple(np.asarray(m, dtype=np.float32).tobytes() if m is not None else None
                               for m in spatial_fwd))
    hit = model._maps.get(key)
    if hit is not None:
        return hit
    from scipy.ndimage import map_coordinates

    S = _separable_matrix(block, spatial_fwd)
    psd = np.asarray(model.processed_psd, dtype=np.float32)
    dom = model.domain
    if psd.shape != dom:
        src = tuple(int(s) for s in psd.shape)
        axes = [np.arange(t, dtype=np.float64) * (s / float(t)) for s, t in zip(src, dom)]
        coords = np.stack(np.meshgrid(*axes, indexing="ij"), axis=0)
        psd = map_coordinates(psd, coords, order=1, mode="grid-wrap").astype(np.float32, copy=False)
        psd *= np.float32(np.prod(dom) / float(np.prod(src)))
        psd = np.maximum(psd, 0.0)
    P = int(np.prod(block))
    local = np.stack(np.meshgrid(*[np.arange(b, dtype=np.int64) for b in block], indexing="ij"),
                     axis=-1).reshape(-1, len(block))
    folded_idx = tuple((local[:, a] % dom[a]) for a in range(len(dom)))
    reverse = tuple((-np.arange(n, dtype=np.int64)) % n for n in dom)
    out = np.empty((P,) + dom, dtype=np.float32)
    for c in range(P):
        folded = np.zeros(dom, dtype=np.float32)
        np.add.at(folded, folded_idx, S[c])
        spec = np.fft.fftn(folded)
        cmap = np.real(np.fft.ifftn(psd * (np.abs(spec) ** 2)) / float(psd.size)).astype(np.float32, copy=False)
        out[c] = 0.5 * (cmap + cmap[np.ix_(*reverse)])
    model._maps[key] = out
    return out


def blockmatch_noise_ssd(model: GaussianModel, block: tuple[int, ...], radius: tuple[int, ...]) -> np.ndarray:
    """[2r+1 per axis] float32: 2 P (var - cov(lag)) clipped at 0, with the
    lag covariance averaged over +-lag on the periodic autocovariance, and 0 at
    the reference itself (variance.py:507-553)."""
    key = (tuple(block), tuple(radius))
    hit = model._ssd.get(key)
    if hit is not None:
        return hit
    ac = model.autocovariance
    nd = ac.ndim
    shape_ac = ac.shape
    out_shape = tuple(2 * r + 1 for r in radius)
    out = np.empty(out_shape, dtype=np.float32)
    var = float(ac[(0,) * nd])
    P = float(np.prod(block))
    for idx in np.ndindex(out_shape):
        lag = tuple(idx[a] - radius[a] for a in range(nd))
        pos = tuple(lag[a] % shape_ac[a] for a in range(nd))
        neg = tuple((-lag[a]) % shape_ac[a] for a in range(nd))
        cov = 0.5 * float(ac[pos] + ac[neg])
        out[idx] = np.float32(max(2.0 * P * (var - cov), 0.0))
    out[tuple(radius)] = np.float32(0.0)
    model._ssd[key] = out
    return out
